"""Build recipe for the oracle (test infrastructure): oracle/_build/liboracle.so.

gcc -O2 -ffp-contract=off keeps every double operation separately rounded, as
the reference is on x86-64 (AArch64 GCC would otherwise contract to FMA).
OpenMP parallelises histories for the CPU baseline.
"""
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
FLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    h = hashlib.sha256()
    for f in ("oracle.c", "oracle.h"):
        with open(os.path.join(HERE, f), "rb") as fh:
            h.update(fh.read())
    with open(os.path.join(HERE, "..", "include", "abeille_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(repr(FLAGS).encode() + os.uname().machine.encode())
    stamp = h.hexdigest()
    stamp_file = os.path.join(OUT, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read().strip() == stamp:
                return LIB
    cc = shutil.which("gcc") or "cc"
    tmp = LIB + ".tmp"
    subprocess.check_call([cc] + FLAGS + [src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
