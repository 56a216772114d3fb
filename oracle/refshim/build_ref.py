"""Build recipe for oracle/_ref/abeille_ref: the reference's own multigroup
transport code, compiled from its unmodified sources where they lie in the
reference tree, against the stand-in headers of oracle/refshim/include
(yaml-cpp, PapillonNDL, HighFive, NDArray, Boost.unordered, pcg-cpp from
pyarrow's vendored copy) and oracle/refshim/stubs.cpp (the continuous-energy,
plotting, cancellation and output code the multigroup path never runs),
driven by oracle/refshim/harness.cpp (decks arrive as JSON, oracle/refshim/
yaml_json.cpp).  build_adapter_check() also links the reference-side
transporter binding (include/abeille_gb300_transporter.hpp) against the same
objects and the engine library: oracle/_ref/adapter_check.  Test infrastructure: it checks the
oracle; nothing of the product links it.

Usage: python oracle/refshim/build_ref.py [REFERENCE_ROOT]
(default: the ABEILLE_REFERENCE environment variable, else DEFAULT_REFERENCE).  Builds only where the
reference tree and pyarrow's pcg-cpp are present; prints why not otherwise.
g++ -O2 -ffp-contract=off, no OpenMP (one thread: the bank comes back in the
reference's concatenation order), C++20.
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
EXE = os.path.join(OUT, "abeille_ref")
# translation units outside the multigroup path that need libraries absent
# here (PapillonNDL data, Sobol tables, the GUI, the logo bitmap); stubs.cpp
# stands in for what the others reference of them
SKIP = {"main", "gui_plotter", "logo", "ce_nuclide", "nd_directory", "pctable", "tabulated_energy",
        "basic_exact_mg_cancelator", "exact_mg_cancelator"}
FLAGS = ["-O2", "-std=c++20", "-ffp-contract=off", "-w",
         "-DABEILLE_VERSION_STRING=\"0.4.0\"", "-DABEILLE_GIT_HASH=\"none\"",
         "-DABEILLE_COMPILER_NAME=\"g++\"", "-DABEILLE_COMPILER_VERSION=\"13\""]


def pcg_header():
    try:
        import pyarrow
    except ImportError:
        return None
    h = os.path.join(os.path.dirname(pyarrow.__file__), "include", "arrow", "vendored", "pcg", "pcg_random.hpp")
    return h if os.path.exists(h) else None


# where the reference tree is mounted in the build container
DEFAULT_REFERENCE = "/root/reference"


def build(ref=None, force=False, quiet=False):
    """Returns the path of the driver, or None (with the reason printed)
    where the reference or pcg-cpp is not available."""
    ref = ref or os.environ.get("ABEILLE_REFERENCE") or DEFAULT_REFERENCE
    if quiet:
        global print
        print = lambda *a, **k: None  # noqa: E731,A001
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        print("reference build skipped: no reference tree (pass its path or set ABEILLE_REFERENCE)")
        return None
    pcg = pcg_header()
    if not pcg:
        print("reference build skipped: pyarrow's vendored pcg-cpp is not installed")
        return None
    cxx = shutil.which("g++")
    if not cxx:
        print("reference build skipped: no g++")
        return None
    srcs = sorted(f for f in glob.glob(os.path.join(ref, "src", "*.cpp"))
                  if os.path.splitext(os.path.basename(f))[0] not in SKIP)
    own = [os.path.join(HERE, "harness.cpp"), os.path.join(HERE, "stubs.cpp"), os.path.join(HERE, "yaml_json.cpp")]
    inc = ["-I", os.path.join(ref, "include"), "-I", os.path.join(HERE, "include"),
           f"-DPCG_VENDORED_HEADER=\"{pcg}\""]
    h = hashlib.sha256()
    for f in srcs + own + sorted(glob.glob(os.path.join(HERE, "include", "**", "*"), recursive=True)):
        if os.path.isfile(f):
            h.update(f.encode())
            with open(f, "rb") as fh:
                h.update(fh.read())
    h.update(repr(FLAGS + inc).encode() + os.uname().machine.encode())
    stamp = h.hexdigest()
    stamp_file = os.path.join(OUT, "stamp")
    if not force and os.path.exists(EXE) and os.path.exists(stamp_file) and open(stamp_file).read() == stamp:
        return EXE
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)

    def cc(src):
        obj = os.path.join(OUT, "obj", os.path.basename(os.path.dirname(src)) + "_" +
                           os.path.splitext(os.path.basename(src))[0] + ".o")
        r = subprocess.run([cxx] + FLAGS + inc + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {src}:\n{r.stderr[-4000:]}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs + own))
    tmp = EXE + ".tmp"
    r = subprocess.run([cxx, "-o", tmp] + objs + ["-lm"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-8000:])
    os.replace(tmp, EXE)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return EXE


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force="--force" in sys.argv))


ADAPTER = os.path.join(OUT, "adapter_check")


def build_adapter_check(ref=None):
    """Compile oracle/refshim/adapter_check.cpp -- the reference-side
    GpuTransporter (include/abeille_gb300_transporter.hpp) in a program of
    the reference's own objects -- and link it with libabeille_gb300.so.
    Returns the program's path, or None where the reference build is not
    available."""
    if not build(ref):
        return None
    ref = ref or os.environ.get("ABEILLE_REFERENCE") or DEFAULT_REFERENCE
    repo = os.path.dirname(ORACLE)
    sys.path.insert(0, repo)
    from abeille_gb300 import build as engine_build
    lib = engine_build.build()
    cxx = shutil.which("g++")
    pcg = pcg_header()
    objs = sorted(f for f in glob.glob(os.path.join(OUT, "obj", "*.o")) if not f.endswith("refshim_harness.o"))
    src = os.path.join(HERE, "adapter_check.cpp")
    obj = os.path.join(OUT, "adapter_check.o")
    inc = ["-I", os.path.join(ref, "include"), "-I", os.path.join(HERE, "include"), "-I", os.path.join(repo, "include"),
           f"-DPCG_VENDORED_HEADER=\"{pcg}\""]
    r = subprocess.run([cxx] + FLAGS + inc + ["-c", src, "-o", obj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("adapter check failed to compile:\n" + r.stderr[-4000:])
    libdir = os.path.dirname(lib)
    r = subprocess.run([cxx, "-o", ADAPTER, obj] + objs + ["-L", libdir, "-labeille_gb300", f"-Wl,-rpath,{libdir}",
                                                           "-lpthread", "-lm"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("adapter check failed to link:\n" + r.stderr[-4000:])
    return ADAPTER
