"""Build recipe of libafx_rans.so (in-tree, sm_103a only).

Host C++ (mesh, config, C ABI) is compiled by g++ with -ffp-contract=off so
the FP64 mesh metrics are identical on x86-64 and aarch64; the FP64 kernels
by nvcc with -fmad=false (bit parity with the reference's arithmetic); the
FP32-mixed kernels by nvcc with contraction allowed.  Translation units are
compiled in parallel and linked into aeroflex_gb300/libafx_rans.so.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libafx_rans.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


def _units():
    ch = _cuda_home()
    nvcc = os.path.join(ch, "bin", "nvcc")
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
           "-I" + INCLUDE, "-I" + os.path.join(ch, "include")]
    nv = [nvcc] + ARCH + ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                          "-diag-suppress", "128", "-I" + INCLUDE]
    return [
        (cxx + ["-c"], "afx_mesh.cpp"),
        (cxx + ["-c"], "afx_config.cpp"),
        (cxx + ["-c"], "afx_abi.cpp"),
        (cxx + ["-c"], "afx_vtu.cpp"),
        (nv + ["-fmad=false", "-c"], "afx_kernels_f64.cu"),
        (nv + ["-fmad=false", "-c"], "afx_noalloc.cu"),
        (nv + ["-fmad=false", "-c"], "afx_adjoint.cu"),
        (nv + ["-c"], "afx_implicit.cu"),
        (nv + ["-fmad=false", "-c"], "afx_prolong.cu"),
        (nv + ["-use_fast_math", "-c"], "afx_kernels_f32.cu"),
        (nv + ["-c"], "afx_peak.cu"),
        (nv + ["-c"], "afx_krylov.cu"),
    ], nvcc


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "afx_rans.h")]


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force=False, verbose=False):
    """Compile libafx_rans.so if missing or older than its sources; return its path."""
    if not force and not stale():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    units, nvcc = _units()

    def run(u):
        flags, src = u
        obj = os.path.join(OBJ, src + ".o")
        cmd = flags + [os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(run, units))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
