"""Build libmsx.so (the CUDA step kernels, host runtime and C ABI) in-tree.

    python v.1.1_gb300/build.py

Compiles each translation unit for sm_103a with nvcc in parallel and links
v.1.1_gb300/_build/libmsx.so.  msx_exact.cu is compiled with --fmad=false
(reference operation order); the host side is compiled with FP contraction off
so material constants match the reference's expressions bit for bit.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmsx.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = {
    "msx_exact.cu": ["--fmad=false"],
    "msx_fast.cu": [],
    "msx_runtime.cu": [],
    "msx_pool.cu": [],
    "msx_noalloc.cu": ["--fmad=false"],
    "msx_csr.cu": [],
    "msx_deckio.cpp": [],
}
DECK = os.path.join(OUT, "msx_deck")


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
    return obj


def _stale(objs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "msx.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    units = {k: v for k, v in UNITS.items() if os.path.exists(os.path.join(CSRC, k))}
    if not force and not _stale(units):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), units.items()))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    deck = os.path.join(OUT, "msx_deck")
    cxx = shutil.which("g++") or "c++"
    r = subprocess.run([cxx, "-O2", "-std=c++17", os.path.join(CSRC, "msx_deck.cpp"), "-o", deck, "-L" + OUT,
                        "-lmsx", "-Wl,-rpath,$ORIGIN"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("msx_deck build failed:\n" + r.stderr)
    # the FP64 pipe's DFMA rate (the denominator of bench.py's FP64-pipe roofline)
    r = subprocess.run([nvcc(), *ARCH, "-O3", os.path.join(CSRC, "msx_fp64_peak.cu"), "-o", os.path.join(OUT, "msx_fp64_peak")],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("msx_fp64_peak build failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
