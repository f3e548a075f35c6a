"""Regenerates the golden fixtures in this folder.

Run from the repository root:  python tests/golden/make_golden.py

ref_generator.json -- outputs of the reference's OWN host generator code
    (src/random.cpp: Random::init_rand_zipf, rand_zipf,
    non_uniform_distribution), compiled from the reference tree into
    oracle/_ref by oracle/build_ref.sh, with libc's rand() seeded by srand().
    The raw rand() stream from the same seed is stored beside each trace so a
    test can replay the draws through the oracle's restatements.
seeded_workloads.json -- fingerprints of small batches of the seeded
    YCSB-style generator and of their serial replays under both rules, as the
    oracle produced them; the library's own generator and the CUDA path are
    checked against these on any machine.
"""
import ctypes
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# Small seeded workloads: (name, seed, rows, cols, ops_min, ops_max, read_frac, theta, txns, batch)
WORKLOADS = [
    ("uniform_c1_small", 0x4C54504D47, 1 << 12, 10, 10, 10, 0.5, 0.0, 256, 0),
    ("zipf99_c2_small", 0x4C54504D47, 1 << 14, 10, 16, 16, 0.8, 0.99, 512, 3),
    ("uneven_c4_small", 0x4C54504D47 ^ 4, 1 << 14, 10, 1, 32, 0.7, 0.75, 300, 7),
    ("hot_tiny_table", 7, 64, 4, 1, 32, 0.3, 1.2, 200, 1),
]


def ref_generator():
    path = O.build_ref()
    if path is None:
        raise SystemExit("reference tree not present: cannot regenerate ref_generator.json")
    R = ctypes.CDLL(path)
    R.ref_zipf_table.restype = ctypes.c_uint32
    R.ref_zipf_table.argtypes = [ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p, ctypes.c_uint32]
    R.ref_zipf_trace.restype = None
    R.ref_zipf_trace.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, ctypes.c_uint32,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
    R.ref_nurand_trace.restype = None
    R.ref_nurand_trace.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
    tables = []
    for n, s in [(100, 0.8), (1000, 0.99), (10 ** 6, 0.5), (10 ** 6, 0.99), (10 ** 7, 0.99), (150, 2.0)]:
        buf = np.zeros(128, np.float64)
        ln = R.ref_zipf_table(n, s, buf.ctypes.data, 128)
        tables.append({"n": n, "s": s, "cdf": [float(v).hex() for v in buf[:ln]]})
    traces = []
    for seed, n, s in [(1, 10 ** 6, 0.99), (12345, 10 ** 6, 0.5), (777, 1000, 0.99)]:
        K = 3000
        res = np.zeros(K, np.uint32)
        raw = np.zeros(2 * K, np.uint32)
        R.ref_zipf_trace(seed, n, s, K, res.ctypes.data, raw.ctypes.data, 2 * K)
        traces.append({"seed": seed, "n": n, "s": s, "result": res.tolist(), "raw": raw.tolist()})
    nurand = []
    for seed, A, x, y in [(3, 8191, 1, 100000), (99, 1023, 1, 3000), (2024, 255, 0, 999)]:
        K = 2000
        res = np.zeros(K, np.uint64)
        raw = np.zeros(2 * K, np.uint32)
        R.ref_nurand_trace(seed, A, x, y, K, res.ctypes.data, raw.ctypes.data, 2 * K)
        nurand.append({"seed": seed, "A": A, "x": x, "y": y, "result": res.tolist(), "raw": raw.tolist()})
    doc = {"source": "reference src/random.cpp compiled by oracle/build_ref.sh; libc rand() after srand(seed)",
           "zipf_tables": tables, "zipf_traces": traces, "nurand_traces": nurand}
    with open(os.path.join(OUT, "ref_generator.json"), "w") as f:
        json.dump(doc, f)


def seeded_workloads():
    docs = []
    for name, seed, rows, cols, omin, omax, rf, th, txns, batch in WORKLOADS:
        p = O.ycsb_params(seed, rows, cols, omin, omax, rf, th)
        tf, keys, opw = O.gen_ycsb_batch(p, batch, txns)
        tab = O.table_init(seed, rows, cols)
        entry = {"name": name, "seed": seed, "rows": rows, "cols": cols, "ops_min": omin, "ops_max": omax,
                 "read_frac": rf, "theta": th, "txns": txns, "batch": batch, "n_ops": int(len(keys)),
                 "fnv_txn_first": O.fnv1a(tf), "fnv_keys": O.fnv1a(keys), "fnv_opw": O.fnv1a(opw),
                 "fnv_table_init": O.fnv1a(tab), "keys_head": keys[:16].tolist(), "opw_head": opw[:16].tolist()}
        for rule in (0, 1):
            t2, commit, out = O.replay(rule, tab, tf, keys, opw)
            entry[f"r{rule}"] = {"fnv_table": O.fnv1a(t2), "fnv_commit": O.fnv1a(commit), "fnv_out": O.fnv1a(out),
                                 "committed": int(commit.sum())}
        docs.append(entry)
    with open(os.path.join(OUT, "seeded_workloads.json"), "w") as f:
        json.dump({"source": "oracle/ltp_oracle.c", "workloads": docs}, f, indent=1)


if __name__ == "__main__":
    O.build()
    ref_generator()
    seeded_workloads()
    print("golden fixtures written to", OUT)
