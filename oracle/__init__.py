"""Python binding of the oracle (test infrastructure only).

Mirrors abeille_gb300.engine.Engine on the CPU restatement in oracle.c so
tests can run the same problem through both and compare.
"""
import ctypes as C
import os

import numpy as np

from abeille_gb300 import abi
from abeille_gb300.engine import PARTICLE_DTYPE, SITE_DTYPE, TRACE_DTYPE, scores_dict, stats_dict

from . import build as _build

_lib = None


def load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = C.CDLL(path)
        P = C.POINTER
        protos = {
            "oracle_last_error": (C.c_char_p, []),
            "oracle_create": (C.c_int, [P(abi.Problem), P(C.c_void_p)]),
            "oracle_destroy": (None, [C.c_void_p]),
            "oracle_sample_sources": (C.c_int, [C.c_void_p, C.c_uint64, C.c_size_t, P(abi.Particle)]),
            "oracle_transport": (C.c_int, [C.c_void_p, P(abi.Particle), C.c_size_t, C.c_double, C.c_int,
                                           P(abi.Site), C.c_size_t, P(C.c_size_t), P(abi.Scores), C.c_int]),
            "oracle_tally_record_generation": (C.c_int, [C.c_void_p, C.c_double]),
            "oracle_tally_clear_generation": (C.c_int, [C.c_void_p]),
            "oracle_tally_size": (C.c_int, [C.c_void_p, C.c_int, P(C.c_size_t)]),
            "oracle_tally_read": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                            P(C.c_int)]),
            "oracle_entropy": (C.c_int, [C.c_void_p, P(abi.Site), C.c_size_t, P(C.c_double)]),
            "oracle_run_power_iteration": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, P(abi.RunStats),
                                                     C.c_void_p, C.c_void_p]),
            "oracle_run_fixed_source": (C.c_int, [C.c_void_p, C.c_int, C.c_uint64, C.c_int, P(abi.RunStats)]),
            "oracle_set_source_bank": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
            "oracle_shuffle": (None, [C.c_void_p, C.c_size_t, C.c_size_t, P(C.c_uint64)]),
            "oracle_set_trace": (C.c_int, [C.c_void_p, C.c_uint32, C.c_size_t]),
            "oracle_get_trace": (C.c_int, [C.c_void_p, P(abi.TraceRec), C.c_size_t, P(C.c_size_t)]),
            "oracle_majorant": (C.c_int, [C.c_void_p, P(C.c_double)]),
            "oracle_scatter_cdf": (C.c_int, [C.c_void_p, C.c_int, C.c_int, P(C.c_double)]),
            "oracle_pcg32_seed": (None, [C.c_uint64, P(C.c_uint64)]),
            "oracle_pcg32_next": (C.c_uint32, [P(C.c_uint64)]),
            "oracle_pcg32_advance": (None, [P(C.c_uint64), C.c_uint64]),
            "oracle_canonical": (C.c_double, [P(C.c_uint64)]),
            "oracle_exponential": (C.c_double, [P(C.c_uint64), C.c_double]),
            "oracle_discrete": (C.c_int, [P(C.c_uint64), P(C.c_double), C.c_int]),
        }
        for name, (res, args) in protos.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


class OracleError(RuntimeError):
    pass


class Oracle:
    def __init__(self, built, nthreads=1):
        self.lib = load()
        self.built = built
        self.nthreads = nthreads
        self.ctx = C.c_void_p()
        self._chk(self.lib.oracle_create(built.ptr, C.byref(self.ctx)))

    def _chk(self, rc):
        if rc != 0:
            raise OracleError(f"{abi.ERRORS.get(rc, rc)}: {self.lib.oracle_last_error().decode()}")

    def close(self):
        if self.ctx:
            self.lib.oracle_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sample_sources(self, first, n):
        out = np.zeros(n, PARTICLE_DTYPE)
        self._chk(self.lib.oracle_sample_sources(self.ctx, first, n, out.ctypes.data_as(C.POINTER(abi.Particle))))
        return out

    def transport(self, bank, kcol=1.0, converged=True, site_capacity=None, nthreads=None):
        bank = np.ascontiguousarray(bank, PARTICLE_DTYPE)
        n = bank.size
        cap = site_capacity if site_capacity is not None else 4 * n + 64
        sites = np.zeros(max(cap, 1), SITE_DTYPE)
        ns = C.c_size_t(0)
        sc = abi.Scores()
        self._chk(self.lib.oracle_transport(self.ctx, bank.ctypes.data_as(C.POINTER(abi.Particle)), n, float(kcol),
                                            int(bool(converged)), sites.ctypes.data_as(C.POINTER(abi.Site)), cap,
                                            C.byref(ns), C.byref(sc), nthreads or self.nthreads))
        return sites[: ns.value].copy(), scores_dict(sc)

    def tally(self, tid=0):
        n = C.c_size_t()
        self._chk(self.lib.oracle_tally_size(self.ctx, tid, C.byref(n)))
        gen, avg, var = (np.zeros(n.value) for _ in range(3))
        g = C.c_int()
        self._chk(self.lib.oracle_tally_read(self.ctx, tid, gen.ctypes.data, avg.ctypes.data, var.ctypes.data,
                                             C.byref(g)))
        return {"gen": gen, "avg": avg, "var": var, "generations": g.value}

    def record_generation(self, multiplier=1.0):
        self._chk(self.lib.oracle_tally_record_generation(self.ctx, multiplier))

    def clear_generation(self):
        self._chk(self.lib.oracle_tally_clear_generation(self.ctx))

    def entropy(self, sites):
        sites = np.ascontiguousarray(sites, SITE_DTYPE)
        h = C.c_double()
        self._chk(self.lib.oracle_entropy(self.ctx, sites.ctypes.data_as(C.POINTER(abi.Site)), sites.size,
                                          C.byref(h)))
        return h.value

    def run_power_iteration(self, ngenerations, nignored, nthreads=None):
        st = abi.RunStats()
        k = np.zeros(ngenerations)
        h = np.zeros(ngenerations)
        self._chk(self.lib.oracle_run_power_iteration(self.ctx, ngenerations, nignored, nthreads or self.nthreads,
                                                      C.byref(st), k.ctypes.data, h.ctypes.data))
        return stats_dict(st), k, h

    def set_source_bank(self, source):
        """Restart the next power iteration from rows x y z ux uy uz E wgt wgt2."""
        src = np.ascontiguousarray(source, dtype=np.float64).reshape(-1, 9)
        self._chk(self.lib.oracle_set_source_bank(self.ctx, src.ctypes.data, src.shape[0]))

    def run_fixed_source(self, nbatches, nparticles, nthreads=None):
        st = abi.RunStats()
        self._chk(self.lib.oracle_run_fixed_source(self.ctx, nbatches, nparticles, nthreads or self.nthreads,
                                                   C.byref(st)))
        return stats_dict(st)

    def set_trace(self, n_hist, capacity=1 << 20):
        self._chk(self.lib.oracle_set_trace(self.ctx, n_hist, capacity))

    def get_trace(self):
        n = C.c_size_t()
        self._chk(self.lib.oracle_get_trace(self.ctx, None, 0, C.byref(n)))
        out = np.zeros(n.value, TRACE_DTYPE)
        self._chk(self.lib.oracle_get_trace(self.ctx, out.ctypes.data_as(C.POINTER(abi.TraceRec)), n.value,
                                            C.byref(n)))
        return out

    def majorant(self):
        G = self.built.meta["ngroups"]
        out = np.zeros(G)
        self._chk(self.lib.oracle_majorant(self.ctx, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out


def cores():
    return os.cpu_count() or 1
