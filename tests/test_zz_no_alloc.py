"""abx_transport_noalloc, the transport step that allocates no device memory.

Some callers cannot allocate device memory while they run: hosts whose every
device allocation goes through their own pool, loops that cannot afford the
device synchronisation of cudaMalloc/cudaFree, processes at their memory
budget.  For them the engine offers a variant of the transport step whose
scratch lives in a fixed device array reserved when the library is loaded.
This test runs it through the C-ABI twice in a row on caller-owned device
buffers and checks both calls against abx_transport, the allocating entry
point, on the same bank (FP64 mode: bank order and ids bit-exact, floating
fields within 1e-12 relative).  It sits in a file that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

from abeille_gb300 import SITE_DTYPE, Engine, abi, decks

pytestmark = pytest.mark.gpu

N = 4096
CAP = 16384


def _call(eng, dev_bank, dev_sites, n, cap):
    ns = C.c_size_t()
    sc = abi.Scores()
    rc = eng.lib.abx_transport_noalloc(eng.ctx, C.cast(dev_bank.data_ptr(), C.POINTER(abi.Particle)), n, 1.1, 1,
                                       C.cast(dev_sites.data_ptr(), C.POINTER(abi.Site)), cap, C.byref(ns),
                                       C.byref(sc))
    return rc, ns.value, sc


def test_noalloc_transport_matches_transport_on_two_calls():
    torch = pytest.importorskip("torch")
    eng = Engine(decks.config0(nparticles=N).build(precision="fp64"), 0)
    bank = eng.sample_sources(0, N)
    ref_sites, ref_sc = eng.transport(bank, 1.1, True, site_capacity=CAP)
    assert len(ref_sites) > 0
    dev_bank = torch.from_numpy(bank.view(np.uint8).copy()).cuda()
    dev_sites = torch.zeros(CAP * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        dev_sites.fill_(0xFF)
        torch.cuda.synchronize()
        rc, ns, sc = _call(eng, dev_bank, dev_sites, N, CAP)
        abi.check(rc, eng.lib)
        torch.cuda.synchronize()
        got = np.frombuffer(dev_sites[: ns * SITE_DTYPE.itemsize].cpu().numpy().tobytes(), dtype=SITE_DTYPE)
        assert ns == len(ref_sites), (call, ns, len(ref_sites))
        for f in ("parent_history_id", "parent_daughter_id", "family_id", "wgt", "E"):
            assert np.array_equal(got[f], ref_sites[f]), (call, f)
        assert np.allclose(got["r"], ref_sites["r"], rtol=1e-12, atol=0)
        assert np.allclose(got["u"], ref_sites["u"], rtol=1e-12, atol=0)
        assert sc.collisions == ref_sc["collisions"] and sc.flights == ref_sc["flights"]
        for k in ("k_col", "k_abs", "leakage", "mig_area"):
            assert abs(getattr(sc, k) - ref_sc[k]) <= 1e-12 * abs(ref_sc[k]), (call, k)
    eng.close()


def test_noalloc_transport_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    eng = Engine(decks.config0(nparticles=64).build(precision="fp64"), 0)
    dev_bank = torch.zeros(16, dtype=torch.uint8, device="cuda")
    dev_sites = torch.zeros(16, dtype=torch.uint8, device="cuda")
    rc, _, _ = _call(eng, dev_bank, dev_sites, 16385, 64)
    assert rc == 7 and b"16384" in eng.lib.abx_last_error_string()
    rc, _, _ = _call(eng, dev_bank, dev_sites, 16, 65537)
    assert rc == 7
    eng.close()
