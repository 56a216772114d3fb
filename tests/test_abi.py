"""The C-ABI library: it loads without a GPU, exports every entry point the
header declares, and its structs have the layout ctypes assumes."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from abeille_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "abeille_gb300.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\w[\w\s\*]*?\b(abx_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = abi.load()
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in abi.PROTOTYPES, n


def test_struct_layouts_match_c():
    structs = {"abx_surface": abi.Surface, "abx_cell": abi.Cell, "abx_universe": abi.Universe,
               "abx_material": abi.Material, "abx_mesh_tally": abi.MeshTally, "abx_entropy_mesh": abi.EntropyMesh,
               "abx_source": abi.Source, "abx_settings": abi.Settings, "abx_problem": abi.Problem,
               "abx_particle": abi.Particle, "abx_site": abi.Site, "abx_scores": abi.Scores,
               "abx_run_stats": abi.RunStats, "abx_trace_rec": abi.TraceRec,
               "abx_gen_record": abi.GenRecord, "abx_problem_result": abi.ProblemResult,
               "abx_server_options": abi.ServerOptions, "abx_request_result": abi.RequestResult,
               "abx_server_stats": abi.ServerStats}
    src = '#include <stdio.h>\n#include <stddef.h>\n#include "abeille_gb300.h"\nint main(void){\n'
    for name in structs:
        src += f'printf("%zu\\n", sizeof({name}));\n'
    src += 'printf("%zu %zu %zu\\n", offsetof(abx_problem, entropy), offsetof(abx_problem, sources), ' \
           'offsetof(abx_problem, n_mg_data));\nreturn 0;}\n'
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "s.c"), "w") as f:
            f.write(src)
        subprocess.check_call(["gcc", "-I", os.path.dirname(HEADER), os.path.join(td, "s.c"), "-o",
                               os.path.join(td, "s")])
        out = subprocess.check_output([os.path.join(td, "s")]).decode().split()
    for (name, cls), size in zip(structs.items(), out):
        assert C.sizeof(cls) == int(size), name
    assert [abi.Problem.entropy.offset, abi.Problem.sources.offset, abi.Problem.n_mg_data.offset] == \
        [int(x) for x in out[-3:]]


def test_create_without_gpu_fails_cleanly():
    from abeille_gb300 import decks
    lib = abi.load()
    built = decks.config0(nparticles=10).build()
    ctx = C.c_void_p()
    rc = lib.abx_create(built.ptr, 0, C.byref(ctx))
    if rc == 0:
        lib.abx_destroy(ctx)
        pytest.skip("a GPU is present")
    assert rc == 6 and not ctx.value
    assert b"CUDA" in lib.abx_last_error_string()


def test_fp64_units_keep_ieee_arithmetic():
    """The FP64 parity kernels reproduce the reference per history only if no
    multiply-add is contracted and no approximate division or square root is
    used: every unit that compiles FP64 transport code takes --fmad=false and
    none of the fast FP32 flags; the fast flags go to FP32-tracking units only."""
    from abeille_gb300 import build
    fast = set(build.FAST_DIV) | set(build.FAST_MATH)
    units = dict(build.UNITS)
    for u in ("engine.cu", "transport_fp64.cu", "transport_fp64_wide.cu", "transport_pool_fp64.cu"):
        assert "--fmad=false" in units[u], u
        assert not fast & set(units[u]), u
    for u, flags in units.items():
        if fast & set(flags):
            assert u.startswith("transport_mixed") or u.startswith("transport_pool_mixed"), u
