"""The oracle's RNG layer against golden vectors from the real pcg-cpp and
libstdc++ (tests/golden/make_rng_golden.py)."""
import ctypes as C
import json
import os

import numpy as np

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


def test_default_stream_and_shuffle():
    """settings::rng starts from a default-constructed pcg32; std::shuffle
    over it (the branchless power iteration's combing) draws its swap
    positions by libstdc++'s two paths: the oracle's restatement gives the
    same permutations and leaves the stream in the same state."""
    g = GOLD
    st = C.c_uint64(0)
    oracle.load().oracle_pcg32_seed(0xcafef00dd15ea5e5, C.byref(st))
    assert st.value == g["default_state"]
    lib = oracle.load()
    for case in g["shuffle"]:
        n = case["n"]
        v = np.arange(n, dtype=np.uint32)
        s = C.c_uint64(0)
        lib.oracle_pcg32_seed(case["seed"], C.byref(s))
        lib.oracle_shuffle(v.ctypes.data, n, 4, C.byref(s))
        check = 0
        for x in v.tolist():
            check = (check * 1000003 + x) & ((1 << 64) - 1)
        assert check == case["check"], n
        assert v[:12].tolist() == case["head"], n
        assert lib.oracle_pcg32_next(C.byref(s)) == case["next"], n
