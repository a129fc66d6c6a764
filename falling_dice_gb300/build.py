"""Builds libmcg.so in-tree: CUDA sources for sm_103a with nvcc, host C++ with g++.

    python -m falling_dice_gb300.build          # or __graft_entry__.build()

Output: falling_dice_gb300/_build/libmcg.so.  Objects are rebuilt when a source or header
is newer than them; translation units compile in parallel.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libmcg.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC", f"-I{INC}",
                     "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
# Per-unit extra flags.  contact.cu must round like the reference: no FMA contraction.
EXTRA = {"contact.cu": ["-fmad=false"]}
CXX_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             f"-I{CUDA_HOME}/include", f"-I{INC}"]


def _headers():
    return glob.glob(os.path.join(SRC, "*.h")) + glob.glob(os.path.join(SRC, "*.cuh")) + \
        glob.glob(os.path.join(INC, "*.h"))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(src, obj, verbose):
    name = os.path.basename(src)
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + EXTRA.get(name, []) + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {name} failed:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(SRC, "*.cu")) + glob.glob(os.path.join(SRC, "*.cpp")))
    deps = _headers()
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = [ex.submit(_compile, s, o, verbose) for s, o in jobs]
            for f in futs:
                msg = f.result()
                if verbose and msg.strip():
                    print(msg, file=sys.stderr)
    if force or jobs or not os.path.exists(LIB):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fPIC"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking libmcg.so failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
