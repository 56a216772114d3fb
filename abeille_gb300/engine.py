"""Python face of the C-ABI, shaped like the reference's plugin interface.

``Engine`` owns one abx context (one problem on one GPU).  On top of it:

* ``GpuDeltaTracker`` / ``GpuSurfaceTracker`` mirror ``Transporter::transport``
  (include/simulation/transporter.hpp:78-81): they take a bank of particles and
  return the fission bank in the reference's order;
* ``PowerIterator`` / ``FixedSource`` mirror the drivers
  (src/power_iterator.cpp:305-473, src/fixed_source.cpp:81-173) and run fully
  on the device.
"""
import ctypes as C

import numpy as np

from . import abi

PARTICLE_DTYPE = np.dtype([("r", "<f8", 3), ("u", "<f8", 3), ("E", "<f8"), ("wgt", "<f8"), ("wgt2", "<f8"),
                           ("history_id", "<u8"), ("rng_state", "<u8"), ("family_id", "<u8")])
SITE_DTYPE = np.dtype([("r", "<f8", 3), ("u", "<f8", 3), ("E", "<f8"), ("wgt", "<f8"), ("wgt2", "<f8"),
                       ("parent_history_id", "<u8"), ("parent_daughter_id", "<u8"), ("family_id", "<u8")])
TRACE_DTYPE = np.dtype([("hist", "<u4"), ("kind", "<i4"), ("group", "<i4"), ("cell", "<i4"),
                        ("rng_state", "<u8"), ("r", "<f8", 3), ("u", "<f8", 3), ("wgt", "<f8")])
assert PARTICLE_DTYPE.itemsize == C.sizeof(abi.Particle)
assert SITE_DTYPE.itemsize == C.sizeof(abi.Site)
assert TRACE_DTYPE.itemsize == C.sizeof(abi.TraceRec)


def scores_dict(s):
    return {f: getattr(s, f) for f, _ in abi.Scores._fields_}


def stats_dict(s):
    return {f: getattr(s, f) for f, _ in abi.RunStats._fields_}


class Engine:
    """One problem resident on one GPU."""

    def __init__(self, built, device=0):
        self.lib = abi.load()
        self.built = built
        self.ctx = C.c_void_p()
        abi.check(self.lib.abx_create(built.ptr, device, C.byref(self.ctx)), self.lib)

    def close(self):
        if self.ctx:
            self.lib.abx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        abi.check(rc, self.lib)

    def sample_sources(self, first, n):
        out = np.zeros(n, PARTICLE_DTYPE)
        self._chk(self.lib.abx_sample_sources(self.ctx, first, n, out.ctypes.data_as(C.POINTER(abi.Particle))))
        return out

    def transport(self, bank, kcol=1.0, converged=True, site_capacity=None):
        bank = np.ascontiguousarray(bank, PARTICLE_DTYPE)
        n = bank.size
        cap = site_capacity if site_capacity is not None else 4 * n + 64
        sites = np.zeros(max(cap, 1), SITE_DTYPE)
        ns = C.c_size_t(0)
        sc = abi.Scores()
        self._chk(self.lib.abx_transport(self.ctx, bank.ctypes.data_as(C.POINTER(abi.Particle)), n, float(kcol),
                                         int(bool(converged)), sites.ctypes.data_as(C.POINTER(abi.Site)), cap,
                                         C.byref(ns), C.byref(sc)))
        return sites[: ns.value].copy(), scores_dict(sc)

    def last_transport_ms(self):
        ms = C.c_double()
        self._chk(self.lib.abx_last_transport_ms(self.ctx, C.byref(ms)))
        return ms.value

    def tally(self, tid=0):
        n = C.c_size_t()
        self._chk(self.lib.abx_tally_size(self.ctx, tid, C.byref(n)))
        gen, avg, var = (np.zeros(n.value) for _ in range(3))
        g = C.c_int()
        self._chk(self.lib.abx_tally_read(self.ctx, tid, gen.ctypes.data, avg.ctypes.data, var.ctypes.data,
                                          C.byref(g)))
        return {"gen": gen, "avg": avg, "var": var, "generations": g.value}

    def read_source_bank(self):
        """(bank, kcol): the source bank the next generation would run after
        the last power iteration, and the k_col its transport takes."""
        n, k = C.c_size_t(), C.c_double()
        self._chk(self.lib.abx_read_source_bank(self.ctx, None, 0, C.byref(n), C.byref(k)))
        bank = np.zeros(n.value, PARTICLE_DTYPE)
        self._chk(self.lib.abx_read_source_bank(self.ctx, bank.ctypes.data, n.value, C.byref(n), C.byref(k)))
        return bank, k.value

    def set_source_bank(self, source):
        """Start the next power iterations from a stored source bank: rows
        x y z ux uy uz E wgt wgt2 (the reference's source file layout);
        None or an empty array goes back to sampling the sources."""
        if source is None or len(source) == 0:
            self._chk(self.lib.abx_set_source_bank(self.ctx, None, 0))
            return
        src = np.ascontiguousarray(source, dtype=np.float64).reshape(-1, 9)
        self._chk(self.lib.abx_set_source_bank(self.ctx, src.ctypes.data, src.shape[0]))

    @staticmethod
    def source_rows(bank):
        """Particles (PARTICLE_DTYPE) as source-file rows x y z ux uy uz E wgt wgt2."""
        return np.column_stack([bank["r"], bank["u"], bank["E"], bank["wgt"], bank["wgt2"]])

    def tally_all(self):
        """Average and variance of every tally bin of the context (in a batch
        context: every problem's bins, problem after problem), in one read."""
        n = C.c_size_t()
        self._chk(self.lib.abx_tally_read_all(self.ctx, None, None, 0, C.byref(n)))
        avg, var = np.empty(n.value), np.empty(n.value)
        self._chk(self.lib.abx_tally_read_all(self.ctx, avg.ctypes.data, var.ctypes.data, n.value, C.byref(n)))
        return avg, var

    def record_generation(self, multiplier=1.0):
        self._chk(self.lib.abx_tally_record_generation(self.ctx, multiplier))

    def clear_generation(self):
        self._chk(self.lib.abx_tally_clear_generation(self.ctx))

    def entropy(self, sites):
        sites = np.ascontiguousarray(sites, SITE_DTYPE)
        h = C.c_double()
        self._chk(self.lib.abx_entropy(self.ctx, sites.ctypes.data_as(C.POINTER(abi.Site)), sites.size, C.byref(h)))
        return h.value

    def autotune(self, n_probe):
        """Time the transport launch shapes on `n_probe` source histories and keep
        the fastest; returns (threads per block, blocks, best ms)."""
        b, g, ms = C.c_int(), C.c_int(), C.c_double()
        self._chk(self.lib.abx_autotune(self.ctx, n_probe, C.byref(b), C.byref(g), C.byref(ms)))
        return b.value, g.value, ms.value

    def set_graphs(self, enabled):
        self._chk(self.lib.abx_set_graphs(self.ctx, int(bool(enabled))))

    KERNELS = {"auto": 0, "history": 1, "pool": 2}

    def set_transport_kernel(self, kind):
        """"history": one lane per history; "pool": event-sorted warps over
        pools of 128 histories; "auto": the engine's choice."""
        self._chk(self.lib.abx_set_transport_kernel(self.ctx, self.KERNELS[kind]))

    def transport_kernel(self):
        k = C.c_int()
        self._chk(self.lib.abx_get_transport_kernel(self.ctx, C.byref(k)))
        return {1: "history", 2: "pool"}[k.value]

    def run_power_iteration(self, ngenerations, nignored):
        st = abi.RunStats()
        k = np.zeros(ngenerations)
        h = np.zeros(ngenerations)
        self._chk(self.lib.abx_run_power_iteration(self.ctx, ngenerations, nignored, C.byref(st), k.ctypes.data,
                                                   h.ctypes.data))
        return stats_dict(st), k, h

    def run_power_iteration_records(self, ngenerations, nignored):
        st = abi.RunStats()
        recs = (abi.GenRecord * ngenerations)()
        self._chk(self.lib.abx_run_power_iteration_ex(self.ctx, ngenerations, nignored, C.byref(st), recs))
        rows = [{f: getattr(r, f) for f, _ in abi.GenRecord._fields_} for r in recs]
        return stats_dict(st), rows

    def run_fixed_source(self, nbatches, nparticles):
        st = abi.RunStats()
        self._chk(self.lib.abx_run_fixed_source(self.ctx, nbatches, nparticles, C.byref(st)))
        return stats_dict(st)

    def set_trace(self, n_hist, capacity=1 << 20):
        self._chk(self.lib.abx_set_trace(self.ctx, n_hist, capacity))

    def get_trace(self):
        n = C.c_size_t()
        self._chk(self.lib.abx_get_trace(self.ctx, None, 0, C.byref(n)))
        out = np.zeros(n.value, TRACE_DTYPE)
        self._chk(self.lib.abx_get_trace(self.ctx, out.ctypes.data_as(C.POINTER(abi.TraceRec)), n.value,
                                         C.byref(n)))
        return out


class BatchEngine(Engine):
    """Many fixed-source problems resident on one GPU; batch b of every
    problem is transported in one launch, and each problem's results are those
    of FixedSource::run for it alone."""

    def __init__(self, builts, device=0):
        self.lib = abi.load()
        self.builts = list(builts)
        self.built = self.builts[0]
        arr = (abi.Problem * len(self.builts))(*[b.struct for b in self.builts])
        self._arr = arr
        self.ctx = C.c_void_p()
        abi.check(self.lib.abx_create_batch(arr, len(self.builts), device, C.byref(self.ctx)), self.lib)

    def set_history_quantum(self, histories_per_warp):
        """Warps retire after this many histories so that blocks free their SM
        slots throughout a batch run (0: persistent warps)."""
        abi.check(self.lib.abx_set_history_quantum(self.ctx, int(histories_per_warp)), self.lib)

    def replace(self, builts):
        """Swap in another set of problems, keeping the device buffers."""
        builts = list(builts)
        arr = (abi.Problem * len(builts))(*[b.struct for b in builts])
        self._chk(self.lib.abx_batch_replace(self.ctx, arr, len(builts)))
        self.builts, self.built, self._arr = builts, builts[0], arr

    def run(self, nbatches):
        """Returns (per-problem result dicts, run totals)."""
        res = (abi.ProblemResult * len(self.builts))()
        st = abi.RunStats()
        self._chk(self.lib.abx_run_fixed_source_batch(self.ctx, nbatches, res, C.byref(st)))
        rows = [{f: getattr(r, f) for f, _ in abi.ProblemResult._fields_} for r in res]
        return rows, stats_dict(st)


class Server:
    """The request loop: fixed-source problems submitted one at a time are
    batched by a native scheduler thread under an HBM admission budget."""

    def __init__(self, device=0, precision="mixed", tracking="delta-tracking", nbatches=10, hbm_budget_bytes=0,
                 max_round_problems=0, keep_tallies=True, lanes=0, history_quantum=0):
        self.lib = abi.load()
        o = abi.ServerOptions(device, abi.PRECISION[precision], abi.TRACKING[tracking], nbatches, hbm_budget_bytes,
                              max_round_problems, int(bool(keep_tallies)), lanes, history_quantum)
        self.srv = C.c_void_p()
        abi.check(self.lib.abx_server_create(C.byref(o), C.byref(self.srv)), self.lib)

    def submit(self, built, tag=0):
        rid = C.c_uint64()
        abi.check(self.lib.abx_server_submit(self.srv, built.ptr, tag, C.byref(rid)), self.lib)
        return rid.value

    def poll(self, capacity=256, timeout_ms=0):
        out = (abi.RequestResult * capacity)()
        n = C.c_int()
        abi.check(self.lib.abx_server_poll(self.srv, out, capacity, C.byref(n), timeout_ms), self.lib)
        rows = []
        for r in out[: n.value]:
            d = {f: getattr(r, f) for f, _ in abi.RequestResult._fields_ if f != "result"}
            d.update({f: getattr(r.result, f) for f, _ in abi.ProblemResult._fields_})
            rows.append(d)
        return rows

    def tally(self, request_id, nbins):
        avg, var = np.zeros(nbins), np.zeros(nbins)
        abi.check(self.lib.abx_server_tally(self.srv, request_id, avg.ctypes.data, var.ctypes.data, nbins),
                  self.lib)
        return avg, var

    def release(self, request_id):
        abi.check(self.lib.abx_server_release(self.srv, request_id), self.lib)

    def stats(self):
        st = abi.ServerStats()
        abi.check(self.lib.abx_server_get_stats(self.srv, C.byref(st)), self.lib)
        return {f: getattr(st, f) for f, _ in abi.ServerStats._fields_}

    def close(self):
        if self.srv:
            self.lib.abx_server_destroy(self.srv)
            self.srv = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _GpuTracker:
    """Transporter::transport on the GPU: consumes the bank, returns the
    fission bank in BankedParticle::operator< order."""

    tracking = None

    def __init__(self, engine, tallies=None):
        self.engine = engine
        self.tallies = tallies if tallies is not None else {"kcol": 1.0, "converged": False}
        self.last_scores = None

    def transport(self, bank, noise=False, noise_bank=None, noise_maker=None):
        if noise or noise_bank is not None or noise_maker is not None:
            raise abi.AbxError(9, "noise transport is outside the multigroup transport path")
        sites, scores = self.engine.transport(bank, self.tallies["kcol"], self.tallies["converged"])
        self.last_scores = scores
        return sites


class GpuDeltaTracker(_GpuTracker):
    tracking = "delta-tracking"


class GpuSurfaceTracker(_GpuTracker):
    tracking = "surface-tracking"


class PowerIterator:
    """PowerIterator::run on the device (bank, sort, normalisation, entropy,
    tallies resident in HBM)."""

    def __init__(self, engine, ngenerations, nignored):
        self.engine, self.ngenerations, self.nignored = engine, ngenerations, nignored

    def run(self):
        stats, kcol, entropy = self.engine.run_power_iteration(self.ngenerations, self.nignored)
        self.stats, self.kcol, self.entropy = stats, kcol, entropy
        return stats


class FixedSource:
    def __init__(self, engine, nbatches, nparticles):
        self.engine, self.nbatches, self.nparticles = engine, nbatches, nparticles

    def run(self):
        self.stats = self.engine.run_fixed_source(self.nbatches, self.nparticles)
        return self.stats
