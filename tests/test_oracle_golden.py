"""Pins the oracle: its restatements of the reference's generator pieces
against outputs of the reference's own src/random.cpp (tests/golden/
ref_generator.json, made by tests/golden/make_golden.py from oracle/_ref),
and its seeded workloads / replays against the committed fingerprints."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref_doc():
    return json.load(open(os.path.join(GOLD, "ref_generator.json")))


def test_ref_zipf_tables(oracle_mod, ref_doc):
    L = oracle_mod.lib()
    for t in ref_doc["zipf_tables"]:
        buf = np.zeros(128, np.float64)
        n = L.ltpo_ref_zipf_table(t["n"], t["s"], buf.ctypes.data)
        ref = [float.fromhex(x) for x in t["cdf"]]
        assert n == len(ref)
        assert buf[:n].tolist() == ref, (t["n"], t["s"])


def test_ref_zipf_sampler_replays_reference_draws(oracle_mod, ref_doc):
    """Feeds the oracle's restatement of Random::rand_zipf the same libc
    rand() stream the reference consumed and expects the same ranks."""
    L = oracle_mod.lib()
    for tr in ref_doc["zipf_traces"]:
        buf = np.zeros(128, np.float64)
        ln = L.ltpo_ref_zipf_table(tr["n"], tr["s"], buf.ctypes.data)
        raw, pos = tr["raw"], 0
        b = tr["n"] - 1
        for want in tr["result"]:
            r100 = raw[pos] % 100
            pos += 1
            tail = 0
            u = r100 / 100.0
            if not any(u < buf[i] for i in range(ln)):
                tail = raw[pos] % (b - 100 + 1) + 100
                pos += 1
            got = L.ltpo_ref_zipf_pick(buf.ctypes.data, ln, r100, tail)
            assert got == want


def test_ref_nurand_replays_reference_draws(oracle_mod, ref_doc):
    """NURand(A, x, y) = (U[0,A] | U[x,y]) % (y-x+1) + x; the reference
    evaluates its two uniform draws in one fixed order, found from the trace."""
    L = oracle_mod.lib()
    for tr in ref_doc["nurand_traces"]:
        A, x, y, raw = tr["A"], tr["x"], tr["y"], tr["raw"]
        ok_orders = []
        for first_is_a in (True, False):
            ok = True
            for k, want in enumerate(tr["result"]):
                d1, d2 = raw[2 * k], raw[2 * k + 1]
                ra, rxy = (d1, d2) if first_is_a else (d2, d1)
                got = L.ltpo_ref_nurand(A, x, y, ra % (A + 1), rxy % (y - x + 1) + x)
                if got != want:
                    ok = False
                    break
            ok_orders.append(ok)
        assert any(ok_orders), tr["seed"]


def test_seeded_workload_fingerprints(oracle_mod):
    doc = json.load(open(os.path.join(GOLD, "seeded_workloads.json")))
    O = oracle_mod
    for w in doc["workloads"]:
        p = O.ycsb_params(w["seed"], w["rows"], w["cols"], w["ops_min"], w["ops_max"], w["read_frac"], w["theta"])
        tf, keys, opw = O.gen_ycsb_batch(p, w["batch"], w["txns"])
        assert O.fnv1a(tf) == w["fnv_txn_first"] and O.fnv1a(keys) == w["fnv_keys"] and O.fnv1a(opw) == w["fnv_opw"]
        assert keys[:16].tolist() == w["keys_head"]
        tab = O.table_init(w["seed"], w["rows"], w["cols"])
        assert O.fnv1a(tab) == w["fnv_table_init"]
        for rule in (0, 1):
            t2, commit, out = O.replay(rule, tab, tf, keys, opw)
            e = w[f"r{rule}"]
            assert (O.fnv1a(t2), O.fnv1a(commit), O.fnv1a(out)) == (e["fnv_table"], e["fnv_commit"], e["fnv_out"])


def _py_replay(rule, tab, tf, keys, opw):
    """Pure-Python restatement of the replay for small cases."""
    tab = tab.astype(np.int64).copy()
    n_cols = tab.shape[0]
    n_txns = len(tf) - 1
    out = np.zeros(len(keys), np.int64)
    commit = np.ones(n_txns, np.uint8)
    if rule == 1:
        minw = {}
        for t in range(n_txns):
            for i in range(tf[t], tf[t + 1]):
                if opw[i] & 3:
                    c = (int(keys[i]), (int(opw[i]) >> 2) & 63)
                    minw[c] = min(minw.get(c, t), t)
        for t in range(n_txns):
            for i in range(tf[t], tf[t + 1]):
                c = (int(keys[i]), (int(opw[i]) >> 2) & 63)
                if c in minw and minw[c] < t:
                    commit[t] = 0
    for t in range(n_txns):
        for i in range(tf[t], tf[t + 1]):
            if not commit[t]:
                continue
            col, k = (int(opw[i]) >> 2) & 63, int(keys[i])
            v = int(tab[col, k])
            if opw[i] & 3:
                imm = ((int(opw[i]) >> 12) ^ 0x80000) - 0x80000
                v = ((v + imm + 2 ** 31) % 2 ** 32) - 2 ** 31
                tab[col, k] = v
            out[i] = v
    return tab.astype(np.int32), commit, out.astype(np.int32)


@pytest.mark.parametrize("rule", [0, 1])
def test_c_replay_matches_python_restatement(oracle_mod, rule):
    O = oracle_mod
    for seed, rows, cols, omin, omax, rf, th, n in [(1, 50, 3, 1, 8, 0.5, 1.1, 300), (2, 1000, 10, 10, 10, 0.5, 0.0, 200),
                                                     (3, 40, 1, 1, 20, 0.2, 0.8, 150)]:
        p = O.ycsb_params(seed, rows, cols, omin, omax, rf, th)
        tf, keys, opw = O.gen_ycsb_batch(p, 0, n)
        tab = O.table_init(seed, rows, cols)
        a = O.replay(rule, tab, tf, keys, opw)
        b = _py_replay(rule, tab, tf, keys, opw)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_mt_replay_equals_serial(oracle_mod):
    O = oracle_mod
    p = O.ycsb_params(5, 1 << 12, 10, 1, 32, 0.7, 0.99)
    tf, keys, opw = O.gen_ycsb_batch(p, 1, 5000)
    tab = O.table_init(5, 1 << 12, 10)
    a = O.replay(0, tab, tf, keys, opw)
    b = O.replay(0, tab, tf, keys, opw, threads=7)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_zipf_sampler_distribution(oracle_mod):
    import ctypes
    L = oracle_mod.lib()
    st = ctypes.c_uint64(77)
    n, th, N = 200, 0.99, 100000
    cnt = np.zeros(n + 1)
    for _ in range(N):
        cnt[L.ltpo_zipf_draw(n, th, ctypes.byref(st))] += 1
    w = np.arange(1, n + 1, dtype=float) ** -th
    p = w / w.sum()
    chi2 = (((cnt[1:] - N * p) ** 2) / (N * p)).sum()
    assert chi2 < 300  # 199 degrees of freedom


def test_deterministic_math(oracle_mod):
    import math
    L = oracle_mod.lib()
    for x in [1e-300, 1e-5, 0.3, 1.0, 2.5, 1e5, 1e300]:
        assert abs(L.ltpo_det_log(x) - math.log(x)) <= 4e-16 * max(1, abs(math.log(x)))
    for y in [-700, -1, -1e-9, 0.0, 0.5, 3, 700]:
        assert abs(L.ltpo_det_exp(y) - math.exp(y)) <= 4e-16 * math.exp(y)


def test_feistel_is_a_permutation(oracle_mod):
    L = oracle_mod.lib()
    for n in (1, 2, 3, 100, 1000, 4097):
        vals = {L.ltpo_feistel_perm(9, n, x) for x in range(n)}
        assert vals == set(range(n))
