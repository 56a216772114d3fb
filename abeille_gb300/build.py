"""In-tree build of the CUDA engine (sm_103a) into abeille_gb300/_lib/.

Thirteen translation units are compiled in parallel with nvcc and linked into one
shared library exposing the C-ABI of include/abeille_gb300.h:

  engine.cu                   host side + bookkeeping kernels     --fmad=false
  transport_fp64.cu           FP64 parity transport kernels        --fmad=false
  transport_fp64_wide.cu      the same, four blocks per SM (large launches)  --fmad=false
  transport_mixed.cu          FP32-tracking kernels, delta tracking       fast div/sqrt, ftz
  transport_mixed_surface.cu  FP32-tracking kernels, surface tracking     fast math
  transport_mixed_variants.cu FP32-tracking kernels, implicit-leakage and Carter tracking   fast div/sqrt
  transport_mixed_branchless.cu FP32-tracking kernels, branchless collisions   fast div/sqrt
  transport_pool_mixed.cu     pooled (event-sorted) FP32 kernels, delta    fast div/sqrt
  transport_pool_mixed_surface.cu pooled FP32 kernels, surface tracking    fast math
  transport_pool_fp64.cu      pooled FP64 parity kernels               --fmad=false
  problem_tables.cpp          host table derivation (problems appended to the pools)
  deck.cpp                    reference-format YAML decks read and flattened natively
  server.cpp                  request loop (host scheduler thread)

Host code is compiled with -ffp-contract=off so derived tables round the same
way on x86-64 and AArch64.  A stamp of the sources and flags skips rebuilds.
"""
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libabeille_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 "-I", os.path.join(REPO, "include")]
# FP32 tracking trades IEEE rounding of single-precision division and square
# root for speed (measured: config 1 +23 %, config 2 +24 %; FP32 denormals
# flushed, +1 % more on config 1 with identical results), and surface
# tracking also takes the fast single-precision log/exp (+30 % on config 2;
# on delta tracking it measured slower than division alone).  FP64 arithmetic
# is unaffected by these flags.
FAST_DIV = ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
FAST_MATH = ["--use_fast_math"]
UNITS = [
    ("engine.cu", ["--fmad=false"]),
    ("transport_fp64.cu", ["--fmad=false"]),
    ("transport_fp64_wide.cu", ["--fmad=false"]),
    ("transport_mixed.cu", FAST_DIV),
    ("transport_mixed_surface.cu", FAST_MATH),
    ("transport_mixed_variants.cu", FAST_DIV),
    ("transport_mixed_branchless.cu", FAST_DIV),
    ("transport_pool_mixed.cu", FAST_DIV),
    ("transport_pool_mixed_surface.cu", FAST_MATH),
    ("transport_pool_fp64.cu", ["--fmad=false"]),
    ("problem_tables.cpp", []),
    ("deck.cpp", []),
    ("server.cpp", []),
]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stamp():
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)):
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode() + fh.read())
    with open(os.path.join(REPO, "include", "abeille_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(repr((COMMON, UNITS)).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    stamp_file = os.path.join(LIBDIR, "stamp")
    stamp = _stamp()
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read().strip() == stamp:
                return LIB
    cc = nvcc()
    objs, procs = [], []
    for src, extra in UNITS:
        obj = os.path.join(LIBDIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"--- {s}\n{o}" for s, o in failed))
    tmp = LIB + ".tmp"
    subprocess.check_call([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
