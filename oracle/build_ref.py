"""Recipe for oracle/_ref/libref.so: the reference's own rans code, built from
its unmodified headers where they lie (test infrastructure only).

Compiles oracle/ref_capi.cpp against src/rans/include/rans/*.h,
src/common and libs/headeronly of the reference tree, with the Eigen-API
stand-in of oracle/eigen_api in place of Eigen (not installed here), using
the reference's OpenMP and no FMA contraction (-ffp-contract=off: the
arithmetic of an x86-64 release build of the reference, which has no FMA).
Nothing is copied from the reference tree; the output goes to oracle/_ref/
only.  Where the tree is absent (a machine that only runs the product) the
recipe does nothing and returns None.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from oracle import refsrc  # noqa: E402

OUT_DIR = os.path.join(HERE, "_ref")
EIGEN_API = os.path.join(HERE, "eigen_api")
# variant -> extra compile definitions: the reference's default limiter, and
# its compile-time Michalak switch (solver.h:557-576)
VARIANTS = {"": [], "michalak": ["-DRANS_MICHALAK_LIMITER"]}


def lib_path(variant=""):
    return os.path.join(OUT_DIR, "libref%s.so" % ("_" + variant if variant else ""))


LIB = lib_path()


def _deps():
    deps = [os.path.join(HERE, "ref_capi.cpp"), os.path.join(EIGEN_API, "afx_eigen_api.hpp")]
    inc = refsrc.path("src", "rans", "include", "rans")
    deps += [os.path.join(inc, f) for f in os.listdir(inc)]
    return deps


def build(force=False, variant=""):
    """Compile libref[_variant].so if the reference tree is present and the
    library is missing or older than its inputs; return its path, or None."""
    lib = lib_path(variant)
    if not refsrc.available():
        return lib if os.path.exists(lib) else None
    if not force and os.path.exists(lib):
        t = os.path.getmtime(lib)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return lib
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = lib + ".%d.tmp" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I" + EIGEN_API,
           "-I" + refsrc.path("src", "rans", "include"),
           "-I" + refsrc.path("src", "common"),
           "-I" + refsrc.path("libs", "headeronly")] + VARIANTS[variant] + [
           "-o", tmp, os.path.join(HERE, "ref_capi.cpp")]
    subprocess.check_call(cmd)
    os.replace(tmp, lib)
    return lib


def build_all(force=False):
    """Both variants, compiled in parallel."""
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=len(VARIANTS)) as ex:
        return list(ex.map(lambda v: build(force, v), VARIANTS))


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
