"""In-tree build of the CUDA library ``libxtrack_gb300.so`` for sm_103a.

The device code is compiled with ``-fmad=false`` (the exact-arithmetic path
must not fuse products into additions; the fast path calls fma()
explicitly) and the host packer with ``-ffp-contract=off`` for the same
reason. Translation units compile in parallel; no cmake.

Run: ``python -m xtrack_gb300._build``.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build_objs")
LIB = os.path.join(PKG, "libxtrack_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler",
              "-fPIC,-ffp-contract=off,-O2", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]

CU_SOURCES = ["xtg_track.cu", "xtg_mlp.cu"]
CXX_SOURCES = ["xtg_lattice.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _defines():
    """Build-time options of the push's register budget (see xtg_track.cu):
    XTG_FAST_MIN_BLOCKS (1 or 2) resident blocks of at most
    XTG_FAST_LB_THREADS (384, the default, or 256) threads each for the fast
    push; XTG_EXACT_LB_THREADS (512, the default, 384 or 256) for the exact
    one; XTG_EMUL (1, the default: the push's stand-alone products on the
    integer pipes, or 0: on the FP64 unit; the results are the same)."""
    out = []
    v = os.environ.get("XTG_FAST_MIN_BLOCKS")
    if v:
        if v not in ("1", "2"):
            raise ValueError("XTG_FAST_MIN_BLOCKS must be 1 or 2")
        out.append(f"-DXTG_FAST_MIN_BLOCKS={v}")
    v = os.environ.get("XTG_EMUL")
    if v:
        if v not in ("0", "1"):
            raise ValueError("XTG_EMUL must be 0 or 1")
        out.append(f"-DXTG_EMUL={v}")
    for name in ("XTG_FAST_LB_THREADS", "XTG_EXACT_LB_THREADS"):
        v = os.environ.get(name)
        if v:
            if v not in ("256", "384", "512"):
                raise ValueError(f"{name} must be 256, 384 or 512")
            out.append(f"-D{name}={v}")
    return out


def build(verbose=False, force=False):
    """Compiles the library if any source is newer than it. Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(PKG, "..", "include", "xtrack_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + _defines() + ["-Xptxas", "-v", "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "--cudart", "static", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
