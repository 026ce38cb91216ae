"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/rans_oracle.cpp + oracle/oracle_capi.cpp into
oracle/_build/liboracle.so with g++ -O3 -DNDEBUG -fopenmp -ffp-contract=off:
the reference's release flags (examples/rans/makefile) without
-march=native, and no FMA contraction, which makes its FP64 results
identical on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["rans_oracle.cpp", "sa_oracle.cpp", "oracle_capi.cpp"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = SOURCES + ["rans_oracle.hpp"]
    return any(os.path.getmtime(os.path.join(HERE, s)) > t for s in deps)


def build(force=False):
    """Compile the oracle library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-DNDEBUG", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB + ".tmp"] + [os.path.join(HERE, s) for s in SOURCES]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
