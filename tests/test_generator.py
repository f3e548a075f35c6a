"""The library's host generator (libltpmg_gb300.so, no GPU needed) against
the oracle's independent restatement and the committed fingerprints."""
import json
import os

import numpy as np
import pytest

import ltpmg_gb300 as G

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "seeded_workloads.json")


@pytest.mark.parametrize("shape", [
    (0x4C54504D47, 1 << 20, 10, 10, 10, 0.5, 0.0, 5000, 0),
    (0x4C54504D47, 1 << 24, 10, 16, 16, 0.8, 0.99, 3000, 5),
    (17, 1 << 24, 10, 1, 32, 0.7, 0.5, 3000, 63),
    (18, 100, 7, 1, 32, 0.3, 1.5, 2000, 2),
])
def test_generator_matches_oracle(lib, oracle_mod, shape):
    seed, rows, cols, omin, omax, rf, th, n, b = shape
    tf, keys, opw = G.gen_ycsb(seed, rows, cols, omin, omax, rf, th, b, n, threads=4)
    p = oracle_mod.ycsb_params(seed, rows, cols, omin, omax, rf, th)
    tf2, k2, w2 = oracle_mod.gen_ycsb_batch(p, b, n)
    assert np.array_equal(tf, tf2) and np.array_equal(keys, k2) and np.array_equal(opw, w2)


def test_generator_thread_invariance(lib):
    args = (3, 1 << 22, 10, 1, 32, 0.7, 0.9, 1, 20000)
    a = G.gen_ycsb(*args, threads=1)
    b = G.gen_ycsb(*args, threads=13)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_generator_fingerprints(lib, oracle_mod):
    for w in json.load(open(GOLD))["workloads"]:
        tf, keys, opw = G.gen_ycsb(w["seed"], w["rows"], w["cols"], w["ops_min"], w["ops_max"], w["read_frac"],
                                   w["theta"], w["batch"], w["txns"])
        assert oracle_mod.fnv1a(keys) == w["fnv_keys"] and oracle_mod.fnv1a(opw) == w["fnv_opw"]


def test_keys_distinct_within_txn_and_in_range(lib):
    tf, keys, opw = G.gen_ycsb(8, 5000, 10, 1, 32, 0.5, 1.2, 0, 4000)
    assert keys.max() < 5000
    for t in range(len(tf) - 1):
        k = keys[tf[t]:tf[t + 1]]
        assert len(set(k.tolist())) == len(k)
    assert ((opw >> 2) & 63).max() < 10


def test_generator_rejects_bad_params(lib):
    with pytest.raises(G.LtpError):
        G.gen_ycsb(1, 5, 10, 1, 8, 0.5, 0.0, 0, 10)  # fewer rows than ops per txn
    with pytest.raises(G.LtpError):
        G.gen_ycsb(1, 100, 65, 1, 8, 0.5, 0.0, 0, 10)  # too many columns


def test_table_value_matches_oracle(lib, oracle_mod):
    for args in [(1, 0, 0, 10), (0x4C54504D47, 12345, 7, 10), (9, 2 ** 23, 63, 64)]:
        assert lib.ltp_table_value(*args) == oracle_mod.lib().ltpo_table_value(*args)
