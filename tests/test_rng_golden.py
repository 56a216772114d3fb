"""The oracle's RNG layer against golden vectors from the real pcg-cpp and
libstdc++ (tests/golden/make_rng_golden.py)."""
import ctypes as C
import json
import os

import oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "rng_golden.json")))
LIB = oracle.load()


def _state(seed):
    s = C.c_uint64()
    LIB.oracle_pcg32_seed(seed, C.byref(s))
    return s


def test_seeding_and_raw_outputs():
    for e in GOLD["seed"]:
        s = _state(e["seed"])
        assert s.value == e["state"]
        assert [LIB.oracle_pcg32_next(C.byref(s)) for _ in e["out"]] == e["out"]


def test_skip_ahead_per_history():
    for e in GOLD["advance"]:
        s = _state(19073486328125)
        LIB.oracle_pcg32_advance(C.byref(s), (152917 * e["id"]) % (1 << 64))
        assert s.value == e["state"]
        assert [LIB.oracle_pcg32_next(C.byref(s)) for _ in e["out"]] == e["out"]


def test_generate_canonical():
    s = _state(19073486328125)
    got = [LIB.oracle_canonical(C.byref(s)) for _ in GOLD["canonical"]]
    assert got == [float.fromhex(h) for h in GOLD["canonical"]]


def test_exponential_distribution():
    for e in GOLD["exponential"]:
        s = _state(e["seed"])
        lam = float.fromhex(e["lambda"])
        got = [LIB.oracle_exponential(C.byref(s), lam) for _ in e["v"]]
        assert got == [float.fromhex(h) for h in e["v"]]


def test_discrete_distribution_and_draw_count():
    for e in GOLD["discrete"]:
        w = [float.fromhex(h) for h in e["w"]]
        arr = (C.c_double * len(w))(*w)
        s = _state(e["seed"])
        got = [LIB.oracle_discrete(C.byref(s), arr, len(w)) for _ in e["idx"]]
        assert got == e["idx"]
        # the next canonical shows how many outputs the samples consumed
        assert LIB.oracle_canonical(C.byref(s)) == float.fromhex(e["next"])
