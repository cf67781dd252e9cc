"""Builds librisltc_gb300.so in-tree: host C (gcc) and CUDA for sm_103a (nvcc).

Translation units compile in parallel.  The exact-numerics kernels get
--fmad=false and IEEE division/square root (bit-identical to the CPU
restatement); the fast kernels allow contraction.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librisltc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["host/light.c", "host/ltc_table.c", "host/bvh.c", "host/quicksave.c", "host/clusters.c"]
EXACT = ["--fmad=false", "-prec-div=true", "-prec-sqrt=true"]
FAST = ["--fmad=true", "-prec-div=true", "-prec-sqrt=true"]
# (source, flags, object): candidate_tiles.cu is built once per numerics mode.
CUDA_SOURCES = [
    ("cuda/shade_exact.cu", EXACT, "shade_exact.o"),
    ("cuda/shade_fast.cu", FAST, "shade_fast.o"),
    ("cuda/candidate_tiles.cu", EXACT + ["-DRISLTC_TILE_FAST=0"], "candidate_tiles_exact.o"),
    ("cuda/candidate_tiles.cu", FAST + ["-DRISLTC_TILE_FAST=1"], "candidate_tiles_fast.o"),
    ("cuda/api.cu", [], "api.o"),
    ("cuda/noalloc.cu", [], "noalloc.o"),
]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _deps():
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files if f.endswith((".c", ".h", ".cu", ".cuh"))]
    inc = os.path.join(REPO, "include")
    out += [os.path.join(inc, f) for f in os.listdir(inc)]
    return out + [os.path.abspath(__file__)]


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), proc.stdout, proc.stderr))
    return proc.stderr


def build(force=False, verbose=False, extra_flags=(), out=None):
    """Compiles the library if any source is newer; returns its path.
    extra_flags go to every nvcc command (e.g. -D tuning macros); out
    redirects the library (and its objects) elsewhere."""
    lib = out or LIB
    build_dir = os.path.join(os.path.dirname(lib), "_build_" + os.path.basename(lib)) if out else BUILD
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(d) for d in _deps())):
        return lib
    os.makedirs(build_dir, exist_ok=True)
    jobs = []
    for src in HOST_SOURCES:
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        jobs.append((["gcc", "-std=c99", "-O3", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                      "-c", os.path.join(CSRC, src), "-o", obj], obj))
    for src, flags, name in CUDA_SOURCES:
        obj = os.path.join(build_dir, name)
        cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "-Xptxas", "-v"] + ARCH + flags + list(extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for log in logs:
            if log:
                print(log)
    objs = [o for _, o in jobs]
    _run([nvcc(), "-shared"] + ARCH + ["-o", lib + ".tmp"] + objs + ["-lm"])
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
