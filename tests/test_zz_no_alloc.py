"""abx_transport_noalloc, the transport step that allocates no device memory.

Some callers cannot allocate device memory while they run: hosts whose every
device allocation goes through their own pool, loops that cannot afford the
device synchronisation of cudaMalloc/cudaFree, processes at their memory
budget.  For them the engine offers a variant of the transport step whose
scratch lives in a fixed device array reserved when the library is loaded.
These tests run it through the C-ABI twice in a row on caller-owned device
buffers and check both calls against abx_transport, the allocating entry
point, on the same bank: in FP64 mode (bank order and ids bit-exact, floating
fields within 1e-12 relative) and in the FP32-tracking mode (the same kernel
on the same histories: sites bit-exact, FP64 scores within 1e-12 relative,
the order of their atomic additions aside).  The second call must leave the
device's free memory unchanged.  A fission bank larger than the caller's
capacity returns ABX_ERR_CAPACITY.  The file sits where pytest collects it
last.
"""
import ctypes as C

import numpy as np
import pytest

from abeille_gb300 import SITE_DTYPE, Engine, abi, decks

pytestmark = pytest.mark.gpu

N = 4096
CAP = 16384


def _call(eng, dev_bank, dev_sites, n, cap, kcol=1.1):
    ns = C.c_size_t()
    sc = abi.Scores()
    rc = eng.lib.abx_transport_noalloc(eng.ctx, C.cast(dev_bank.data_ptr(), C.POINTER(abi.Particle)), n, kcol, 1,
                                       C.cast(dev_sites.data_ptr(), C.POINTER(abi.Site)), cap, C.byref(ns),
                                       C.byref(sc))
    return rc, ns.value, sc


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_transport_matches_transport_on_two_calls(precision):
    torch = pytest.importorskip("torch")
    eng = Engine(decks.config0(nparticles=N).build(precision=precision), 0)
    bank = eng.sample_sources(0, N)
    ref_sites, ref_sc = eng.transport(bank, 1.1, True, site_capacity=CAP)
    assert len(ref_sites) > 0
    dev_bank = torch.from_numpy(bank.view(np.uint8).copy()).cuda()
    dev_sites = torch.zeros(CAP * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        dev_sites.fill_(0xFF)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc, ns, sc = _call(eng, dev_bank, dev_sites, N, CAP)
        abi.check(rc, eng.lib)
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before, "the second call changed the free device memory"
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


def test_noalloc_transport_reports_a_full_fission_bank():
    torch = pytest.importorskip("torch")
    eng = Engine(decks.config0(nparticles=N).build(precision="fp64"), 0)
    bank = eng.sample_sources(0, N)
    dev_bank = torch.from_numpy(bank.view(np.uint8).copy()).cuda()
    dev_sites = torch.zeros(64 * SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc, ns, _ = _call(eng, dev_bank, dev_sites, N, 64)
    assert rc == 7 and ns > 64
    # the context stays usable
    rc, ns, _ = _call(eng, dev_bank[: 8 * bank.itemsize], dev_sites, 8, 64)
    abi.check(rc, eng.lib)
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
