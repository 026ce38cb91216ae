"""Location of the reference's source tree, for the recipes and fixture
scripts that read it (test infrastructure only).

The tree is read where it lies; nothing is copied from it.  Set
AFX_REFERENCE_DIR to point elsewhere.  Where the tree is absent (a machine
that only runs the product), ``available()`` is False and the tests that
need it skip.
"""
import os

REFERENCE = os.environ.get("AFX_REFERENCE_DIR", "/root/reference")


def path(*parts):
    """Path of a file or folder inside the reference tree."""
    return os.path.join(REFERENCE, *parts)


def available():
    return os.path.isdir(path("src", "rans", "include", "rans"))
