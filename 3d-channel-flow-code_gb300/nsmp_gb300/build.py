"""Build recipe for libnsmpgpu.so (in-tree, sm_103a only).

Host C++ sources are compiled with g++, CUDA sources with nvcc for
sm_103a, all in parallel, then linked into
3d-channel-flow-code_gb300/lib/libnsmpgpu.so.  The CUDA runtime is linked
statically, so the library loads on a machine without a GPU (host-only entry
points such as the mesh generator run there).
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import subprocess
import sys

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG_ROOT, "_build")
LIBDIR = os.path.join(PKG_ROOT, "lib")
LIB = os.path.join(LIBDIR, "libnsmpgpu.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is built without floating-point contraction (GCC fuses a*b+c by
# default in C++ on targets with FMA, such as aarch64 but not baseline
# x86-64), so the setup gives the same bits on every host and matches the
# oracle, which is built the same way.
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", "-I", INCLUDE,
            "-I", CSRC]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                  "-I", INCLUDE, "-I", CSRC,
                  "--expt-relaxed-constexpr"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cpp"))) + sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(INCLUDE, "*.h")))


def _stamp():
    h = hashlib.sha256()
    for f in _sources() + _headers() + [os.path.abspath(__file__)]:
        with open(f, "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    return h.hexdigest()


# Translation units whose floating-point results must equal the host
# setup's bit for bit: no multiply-add contraction.
NO_FMA = {"setup_gpu.cu"}


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        own = ["-fmad=false"] if os.path.basename(src) in NO_FMA else []
        cmd = [NVCC] + NVFLAGS + own + extra + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp_file = os.path.join(BUILD, "stamp")
    stamp = _stamp()
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as fh:
            if fh.read().strip() == stamp:
                return LIB
    extra = ["-Xptxas", "-v"] if ptxas_v else []
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = [o for o, _ in results]
    if verbose or ptxas_v:
        for _, err in results:
            if err:
                print(err)
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as fh:
        fh.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="-v" in sys.argv))
