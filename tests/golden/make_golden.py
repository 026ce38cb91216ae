"""Regenerate tests/golden/oracle_pins.json: SHA-256 pins of the CPU
oracle's residuals and states (and the forces) on small seeded cases, so a
change to the restatement is caught.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle  # noqa: E402
from tests.test_oracle import pins  # noqa: E402

if __name__ == "__main__":
    out = {"generator": "tests/golden/make_golden.py", "pins": pins(oracle)}
    with open(os.path.join(HERE, "oracle_pins.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))
