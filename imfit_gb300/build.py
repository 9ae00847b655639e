"""Build libimfit_gb300.so in-tree (imfit_gb300/_build/) with nvcc for sm_103a.

Each translation unit is compiled in parallel; the plain FP64 kernels are
compiled with --fmad=false so their arithmetic is not contracted into FMAs.
Run: ``python -m imfit_gb300.build`` (or imfit_gb300.build.build()).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libimfit_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + os.path.join(os.path.dirname(HERE), "include")]

UNITS = [
    ("k_plain.cu", ["--fmad=false"]),
    ("k_fft.cu", []),
    ("k_fast.cu", []),
    ("k_cols32.cu", []),
    ("model_object.cpp", ["-x", "cu"]),
    ("k_noalloc.cu", ["--fmad=false"]),
    ("lm.cpp", []),
    ("k_los.cu", ["--fmad=false"]),
    ("k_probe.cu", []),
]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found")
    return exe


def _compile(unit, extra, verbose):
    src = os.path.join(SRC, unit)
    obj = os.path.join(OUT, os.path.splitext(unit)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for root in (SRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(root):
            if os.path.getmtime(os.path.join(root, f)) > t:
                return True
    return False


def build(force=False, verbose=False):
    """Compile the CUDA library; returns the path of the shared object."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
