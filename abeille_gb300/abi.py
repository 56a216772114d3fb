"""ctypes mirror of include/abeille_gb300.h and the loader of the CUDA engine.

The engine is a C-ABI shared library built in-tree (abeille_gb300/_lib).  There
is no CPU fallback: if the library or a CUDA device is missing, every call
raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))

ABX_OK = 0
ERRORS = {
    1: "ABX_ERR_INVALID", 2: "ABX_ERR_LOST_PARTICLE", 3: "ABX_ERR_MAJORANT", 4: "ABX_ERR_OOM",
    5: "ABX_ERR_TIMEOUT", 6: "ABX_ERR_CUDA", 7: "ABX_ERR_CAPACITY", 8: "ABX_ERR_NO_FISSION",
    9: "ABX_ERR_UNSUPPORTED", 10: "ABX_ERR_CANCELLED", 11: "ABX_ERR_BUDGET",
}

SURF = {"xplane": 0, "yplane": 1, "zplane": 2, "plane": 3, "xcylinder": 4, "ycylinder": 5,
        "zcylinder": 6, "sphere": 7}
BC = {"vacuum": 0, "reflective": 1, "normal": 2}
OP_LPAR, OP_RPAR, OP_COMP, OP_INTR, OP_UNIN = 0x7fffffff, 0x7ffffffe, 0x7ffffffd, 0x7ffffffc, 0x7ffffffb
FILL_MATERIAL, FILL_UNIVERSE = 0, 1
UNIV_CELLS, UNIV_RECT_LATTICE = 0, 1
EST = {"collision": 0, "track-length": 1}
QUANTITY = {"flux": 0, "elastic": 1, "absorption": 2, "fission": 3, "total": 4}
SPATIAL = {"point": 0, "box": 1}
DIRECTION = {"isotropic": 0, "mono-directional": 1}
MODE = {"k-eigenvalue": 0, "fixed-source": 1, "branchless-k-eigenvalue": 0}  # the last with BRANCHLESS_ON
BRANCHLESS_ON, BRANCHLESS_MATERIAL, BRANCHLESS_SPLITTING, BRANCHLESS_COMBING = 1, 2, 4, 8
TRACKING = {"delta-tracking": 0, "surface-tracking": 1, "implicit-leakage-delta-tracking": 2,
            "carter-tracking": 3}
PRECISION = {"fp64": 0, "mixed": 1}


class AbxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Surface(C.Structure):
    _fields_ = [("type", C.c_int32), ("bc", C.c_int32), ("id", C.c_uint32), ("reserved", C.c_int32),
                ("c", C.c_double * 4)]


class Cell(C.Structure):
    _fields_ = [("id", C.c_uint32), ("fill_kind", C.c_int32), ("fill", C.c_int32), ("rpn_offset", C.c_int32),
                ("rpn_len", C.c_int32), ("reserved", C.c_int32)]


class Universe(C.Structure):
    _fields_ = [("id", C.c_uint32), ("kind", C.c_int32), ("list_offset", C.c_int32), ("list_len", C.c_int32),
                ("shape", C.c_int32 * 3), ("outer", C.c_int32), ("pitch", C.c_double * 3),
                ("origin", C.c_double * 3)]


class Material(C.Structure):
    _fields_ = [("id", C.c_uint32), ("data_offset", C.c_int32), ("n_legendre", C.c_int32),
                ("n_delayed", C.c_int32)]


class MeshTally(C.Structure):
    _fields_ = [("estimator", C.c_int32), ("quantity", C.c_int32), ("shape", C.c_int32 * 3),
                ("ebounds_offset", C.c_int32), ("n_ebounds", C.c_int32), ("reserved", C.c_int32),
                ("low", C.c_double * 3), ("hi", C.c_double * 3)]


class EntropyMesh(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("shape", C.c_int32 * 3), ("low", C.c_double * 3),
                ("hi", C.c_double * 3)]


class Source(C.Structure):
    _fields_ = [("spatial", C.c_int32), ("direction", C.c_int32), ("energy", C.c_int32),
                ("fissile_only", C.c_int32), ("weight", C.c_double), ("low", C.c_double * 3),
                ("hi", C.c_double * 3), ("dir", C.c_double * 3), ("energy_value", C.c_double)]


class Settings(C.Structure):
    _fields_ = [("mode", C.c_int32), ("tracking", C.c_int32), ("precision", C.c_int32), ("ngroups", C.c_int32),
                ("seed", C.c_uint64), ("stride", C.c_uint64), ("wgt_cutoff", C.c_double),
                ("wgt_survival", C.c_double), ("nparticles", C.c_double), ("block_size", C.c_int32),
                ("reserved", C.c_int32), ("wgt_split", C.c_double), ("branchless", C.c_int32),
                ("global_rng_skip", C.c_int32)]


class Problem(C.Structure):
    _fields_ = [
        ("settings", Settings),
        ("energy_bounds", C.POINTER(C.c_double)),
        ("surfaces", C.POINTER(Surface)), ("n_surfaces", C.c_int32),
        ("cells", C.POINTER(Cell)), ("n_cells", C.c_int32),
        ("rpn", C.POINTER(C.c_int32)), ("n_rpn", C.c_int32),
        ("universes", C.POINTER(Universe)), ("n_universes", C.c_int32),
        ("cell_lists", C.POINTER(C.c_int32)), ("n_cell_lists", C.c_int32),
        ("lattice_elems", C.POINTER(C.c_int32)), ("n_lattice_elems", C.c_int32),
        ("root_universe", C.c_int32),
        ("materials", C.POINTER(Material)), ("n_materials", C.c_int32),
        ("mg_data", C.POINTER(C.c_double)), ("n_mg_data", C.c_int64),
        ("tallies", C.POINTER(MeshTally)), ("n_tallies", C.c_int32),
        ("tally_ebounds", C.POINTER(C.c_double)), ("n_tally_ebounds", C.c_int32),
        ("entropy", EntropyMesh),
        ("sources", C.POINTER(Source)), ("n_sources", C.c_int32),
        ("sampling_xs_ratio", C.POINTER(C.c_double)),
    ]


class Particle(C.Structure):
    _fields_ = [("r", C.c_double * 3), ("u", C.c_double * 3), ("E", C.c_double), ("wgt", C.c_double),
                ("wgt2", C.c_double), ("history_id", C.c_uint64), ("rng_state", C.c_uint64),
                ("family_id", C.c_uint64)]


class Site(C.Structure):
    _fields_ = [("r", C.c_double * 3), ("u", C.c_double * 3), ("E", C.c_double), ("wgt", C.c_double),
                ("wgt2", C.c_double), ("parent_history_id", C.c_uint64), ("parent_daughter_id", C.c_uint64),
                ("family_id", C.c_uint64)]


class Scores(C.Structure):
    _fields_ = [("k_col", C.c_double), ("k_abs", C.c_double), ("k_trk", C.c_double), ("k_tot", C.c_double),
                ("leakage", C.c_double), ("mig_area", C.c_double), ("collisions", C.c_uint64),
                ("flights", C.c_uint64), ("lost", C.c_uint64)]


class RunStats(C.Structure):
    _fields_ = [("generations", C.c_int32), ("active", C.c_int32), ("kcol_avg", C.c_double),
                ("kcol_std", C.c_double), ("ktrk_avg", C.c_double), ("ktrk_std", C.c_double),
                ("leak_avg", C.c_double), ("leak_std", C.c_double), ("mig_avg", C.c_double),
                ("mig_std", C.c_double), ("collisions", C.c_uint64), ("flights", C.c_uint64),
                ("histories", C.c_uint64), ("transport_ms", C.c_double), ("total_ms", C.c_double)]


class TraceRec(C.Structure):
    _fields_ = [("hist", C.c_uint32), ("kind", C.c_int32), ("group", C.c_int32), ("cell", C.c_int32),
                ("rng_state", C.c_uint64), ("r", C.c_double * 3), ("u", C.c_double * 3), ("wgt", C.c_double)]


class GenRecord(C.Structure):
    _fields_ = [("kcol", C.c_double), ("entropy", C.c_double), ("step_ms", C.c_double),
                ("transport_ms", C.c_double), ("collisions", C.c_uint64), ("flights", C.c_uint64),
                ("histories", C.c_uint64), ("sites", C.c_uint64), ("lost", C.c_uint64)]


class ProblemResult(C.Structure):
    _fields_ = [("leak_avg", C.c_double), ("leak_std", C.c_double), ("collisions", C.c_uint64),
                ("flights", C.c_uint64), ("histories", C.c_uint64), ("lost", C.c_uint64), ("batches", C.c_int32),
                ("tally_first", C.c_int32)]


class ServerOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("precision", C.c_int32), ("tracking", C.c_int32), ("nbatches", C.c_int32),
                ("hbm_budget_bytes", C.c_uint64), ("max_round_problems", C.c_int32), ("keep_tallies", C.c_int32),
                ("lanes", C.c_int32), ("history_quantum", C.c_uint32)]


class RequestResult(C.Structure):
    _fields_ = [("request_id", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("round", C.c_int32),
                ("round_problems", C.c_int32), ("n_tallies", C.c_int32), ("n_tally_bins", C.c_uint64),
                ("result", ProblemResult), ("queue_ms", C.c_double), ("latency_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("rounds", C.c_uint64), ("collisions", C.c_uint64), ("flights", C.c_uint64),
                ("histories", C.c_uint64), ("busy_ms", C.c_double), ("transport_ms", C.c_double),
                ("load_ms", C.c_double), ("run_ms", C.c_double), ("readback_ms", C.c_double),
                ("free_ms", C.c_double)]


# every entry point declared in include/abeille_gb300.h, with its argument types
PROTOTYPES = {
    "abx_create": (C.c_int, [C.POINTER(Problem), C.c_int, C.POINTER(C.c_void_p)]),
    "abx_destroy": (C.c_int, [C.c_void_p]),
    "abx_last_error_string": (C.c_char_p, []),
    "abx_version": (C.c_int, [C.POINTER(C.c_int)] * 3),
    "abx_sample_sources": (C.c_int, [C.c_void_p, C.c_uint64, C.c_size_t, C.POINTER(Particle)]),
    "abx_transport": (C.c_int, [C.c_void_p, C.POINTER(Particle), C.c_size_t, C.c_double, C.c_int,
                                C.POINTER(Site), C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(Scores)]),
    "abx_transport_noalloc": (C.c_int, [C.c_void_p, C.POINTER(Particle), C.c_size_t, C.c_double, C.c_int,
                                        C.POINTER(Site), C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(Scores)]),
    "abx_tally_record_generation": (C.c_int, [C.c_void_p, C.c_double]),
    "abx_tally_clear_generation": (C.c_int, [C.c_void_p]),
    "abx_tally_read": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.POINTER(C.c_int)]),
    "abx_tally_size": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]),
    "abx_entropy": (C.c_int, [C.c_void_p, C.POINTER(Site), C.c_size_t, C.POINTER(C.c_double)]),
    "abx_run_power_iteration": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(RunStats), C.c_void_p,
                                          C.c_void_p]),
    "abx_run_power_iteration_ex": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(RunStats),
                                                 C.POINTER(GenRecord)]),
    "abx_run_fixed_source": (C.c_int, [C.c_void_p, C.c_int, C.c_uint64, C.POINTER(RunStats)]),
    "abx_set_trace": (C.c_int, [C.c_void_p, C.c_uint32, C.c_size_t]),
    "abx_get_trace": (C.c_int, [C.c_void_p, C.POINTER(TraceRec), C.c_size_t, C.POINTER(C.c_size_t)]),
    "abx_last_transport_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "abx_set_l2_flush": (C.c_int, [C.c_void_p, C.c_size_t]),
    "abx_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "abx_set_transport_kernel": (C.c_int, [C.c_void_p, C.c_int]),
    "abx_get_transport_kernel": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "abx_set_history_quantum": (C.c_int, [C.c_void_p, C.c_uint32]),
    "abx_deck_read": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.POINTER(Problem))]),
    "abx_deck_free": (C.c_int, [C.c_void_p]),
    "abx_create_from_deck": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "abx_autotune": (C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int),
                               C.POINTER(C.c_double)]),
    "abx_create_batch": (C.c_int, [C.POINTER(Problem), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "abx_run_fixed_source_batch": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(ProblemResult), C.POINTER(RunStats)]),
    "abx_batch_replace": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.c_int]),
    "abx_tally_read_all": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "abx_read_source_bank": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t),
                                       C.POINTER(C.c_double)]),
    "abx_set_source_bank": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "abx_server_create": (C.c_int, [C.POINTER(ServerOptions), C.POINTER(C.c_void_p)]),
    "abx_server_destroy": (C.c_int, [C.c_void_p]),
    "abx_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.c_uint64, C.POINTER(C.c_uint64)]),
    "abx_server_poll": (C.c_int, [C.c_void_p, C.POINTER(RequestResult), C.c_int, C.POINTER(C.c_int), C.c_int]),
    "abx_server_tally": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_size_t]),
    "abx_server_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "abx_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
}

_lib = None


def lib_path():
    return os.path.join(HERE, "_lib", "libabeille_gb300.so")


def load(build_if_missing=True):
    """Load the engine; build it in-tree first when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA engine not built: {path} is missing")
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc, lib=None):
    if rc != ABX_OK:
        lib = lib or load(False)
        raise AbxError(rc, lib.abx_last_error_string().decode(errors="replace"))
