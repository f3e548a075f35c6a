"""ltp_execute_noalloc: batch execution for callers that cannot allocate.

A caller whose process hands all device memory to its own allocator (or has
reserved it up front) cannot let a library call cudaMalloc.  This entry point
takes every buffer from the caller and keeps its scratch in a fixed array
inside the library; here it is checked, through the C ABI, against the
allocating entry point (ltp_batch_execute) on two calls in a row, bit for
bit, for both rules.  This file is collected last so that a run stopping at
the first failure has already run every other test; it passes alone in a
fresh process as well.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

import ltpmg_gb300 as G
from ltpmg_gb300 import lib as LB


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _oracle():
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import oracle

    return oracle


def _noalloc_call(L, torch, rule, table_t, rows, cols, tf, keys, opw, fixed):
    dev = torch.device("cuda:0")
    k_t = torch.from_numpy(keys.view(np.int64)).to(dev)
    w_t = torch.from_numpy(opw.view(np.int32)).to(dev)
    n_ops, n_txns = len(keys), len(tf) - 1
    out_t = torch.zeros(max(n_ops, 1), dtype=torch.int32, device=dev)
    com_t = torch.zeros(max(n_txns, 1), dtype=torch.uint8, device=dev)
    tf_t = None if fixed else torch.from_numpy(tf.view(np.int32)).to(dev)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.ltp_execute_noalloc(0, rule, _vp(table_t), rows, rows, cols, n_txns, None if tf_t is None else _vp(tf_t),
                               fixed, n_ops, _vp(k_t), _vp(w_t), _vp(out_t), _vp(com_t), ctypes.c_void_p(stream))
    assert rc == 0, rc
    return out_t[:n_ops].cpu().numpy(), com_t[:n_txns].cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("rule", [G.RULE_ORDERED, G.RULE_PRIORITY])
def test_noalloc_matches_allocating_entry_point_twice(rule):
    torch = pytest.importorskip("torch")
    L = G.load()
    rows, cols, seed = 1 << 14, 10, 77
    b0 = G.gen_ycsb(seed, rows, cols, 16, 16, 0.8, 0.99, batch=0, n_txns=8192)
    b1 = G.gen_ycsb(seed, rows, cols, 1, 32, 0.7, 0.9, batch=1, n_txns=6000)

    # reference: the allocating C-ABI path on the same two batches
    with G.Context(device=0, rule=rule) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        tab0 = ctx.download(t)
        ref = []
        b = ctx.batch(8192, 8192 * 32)
        for (tf, keys, opw), fixed in ((b0, 16), (b1, 0)):
            if fixed:
                b.load(None, keys, opw, ops_per_txn=fixed)
            else:
                b.load(tf, keys, opw)
            b.execute()
            commit, vals, _ = b.results()
            ref.append((vals.copy(), commit.copy()))
        ref_final = ctx.download(t)

    table_t = torch.from_numpy(tab0.copy()).to("cuda:0")  # [cols, rows] column-major, caller-owned
    O = _oracle()
    otab = tab0
    for ((tf, keys, opw), fixed), (rvals, rcommit) in zip(((b0, 16), (b1, 0)), ref):
        vals, commit = _noalloc_call(L, torch, rule, table_t, rows, cols, tf, keys, opw, fixed)
        assert np.array_equal(vals, rvals)
        assert np.array_equal(commit, rcommit)
        # and directly against the oracle's serial replay of the same batch
        otab, ocommit, oout = O.replay(rule, otab, tf, keys, opw)
        assert np.array_equal(vals, oout)
        assert np.array_equal(commit, ocommit)
        assert np.array_equal(table_t.cpu().numpy(), otab)
    assert np.array_equal(table_t.cpu().numpy(), ref_final)


def test_noalloc_rejects_oversized_batches():
    L = G.load()
    too_many = int(LB.__dict__.get("NOALLOC_MAX_OPS", 1 << 18)) + 1
    rc = L.ltp_execute_noalloc(0, 0, ctypes.c_void_p(16), 1024, 1024, 4, 1, None, too_many, too_many,
                               ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == LB.LTP_E_CAPACITY
    rc = L.ltp_execute_noalloc(0, 0, ctypes.c_void_p(16), 1 << 22, 1 << 22, 4, 1, None, 4, 4,
                               ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == LB.LTP_E_CAPACITY


@pytest.mark.gpu
def test_noalloc_rejects_malformed_txn_first_on_the_device():
    """txn_first is device memory the host never reads, so the check runs on
    the device: a start other than 0, a decreasing entry, or an end other
    than n_ops makes the call return LTP_E_BADARG, leaves the table as it
    was and writes nothing past the caller's buffers; a valid call after it
    still runs correctly."""
    torch = pytest.importorskip("torch")
    L = G.load()
    rows, cols, seed = 1 << 12, 4, 5
    tf, keys, opw = G.gen_ycsb(seed, rows, cols, 1, 8, 0.5, 0.0, batch=0, n_txns=500)
    n_txns, n_ops = len(tf) - 1, len(keys)
    dev = torch.device("cuda:0")
    with G.Context(device=0) as ctx:
        t = ctx.create_table(rows, cols)
        ctx.fill_seeded(t, seed)
        tab0 = ctx.download(t)
    table_t = torch.from_numpy(tab0.copy()).to(dev)
    k_t = torch.from_numpy(keys.view(np.int64)).to(dev)
    w_t = torch.from_numpy(opw.view(np.int32)).to(dev)
    pad = 4096  # sentinel room after each output buffer
    out_t = torch.full((n_ops + pad,), 0x5A5A5A5A, dtype=torch.int32, device=dev)
    com_t = torch.full((n_txns + pad,), 0xA5, dtype=torch.uint8, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def bad(mutate):
        f = tf.copy()
        mutate(f)
        f_t = torch.from_numpy(f.view(np.int32)).to(dev)
        return L.ltp_execute_noalloc(0, G.RULE_ORDERED, _vp(table_t), rows, rows, cols, n_txns, _vp(f_t), 0, n_ops,
                                     _vp(k_t), _vp(w_t), _vp(out_t), _vp(com_t), stream)

    def set_first(f):
        f[0] = 1

    def decrease(f):
        f[n_txns // 2] = f[n_txns // 2 + 1] + 3

    def short_end(f):
        f[-1] = n_ops - 5

    def long_end(f):
        f[-1] = n_ops + 1000

    for mutate in (set_first, decrease, short_end, long_end):
        assert bad(mutate) == LB.LTP_E_BADARG, mutate.__name__
        assert np.array_equal(table_t.cpu().numpy(), tab0), mutate.__name__
        assert (out_t[n_ops:].cpu().numpy() == 0x5A5A5A5A).all(), mutate.__name__
        assert (com_t[n_txns:].cpu().numpy() == 0xA5).all(), mutate.__name__
    # the array recovers: a valid call equals the oracle's serial replay
    O = _oracle()
    vals, commit = _noalloc_call(L, torch, G.RULE_ORDERED, table_t, rows, cols, tf, keys, opw, 0)
    ref_tab, ref_commit, ref_out = O.replay(0, tab0, tf, keys, opw)
    assert np.array_equal(vals, ref_out)
    assert np.array_equal(commit, ref_commit)
    assert np.array_equal(table_t.cpu().numpy(), ref_tab)
