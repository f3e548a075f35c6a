"""The bench's multi-rank host logic on CPU (gloo, world size 2).

Under torchrun every rank drives an independent replica (no data-path
collective): the only cross-rank steps are a barrier before the timed region
and a max-reduction of the ranks' times.  These tests run those steps on two
gloo ranks, check that each rank draws a different replica of the workload,
and that the reference arm does its work on rank 0 only.
"""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, loc = bench.dist_env()
        bench.barrier(w)
        mx = bench.reduce_max(10.0 + 5.0 * r, w)
        from ltpmg_gb300 import workloads as W

        tf, keys, opw, n, _ = W.generate("plain", 0, rank=r)
        out[r] = (r, w, loc, mx, int(keys[:64].sum() % (1 << 31)), n)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_barrier_reduce_and_replicas():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for r, (rank, w, loc, mx, sig, n) in res.items():
        assert (rank, w, loc) == (r, 2, r)
        assert mx == 15.0  # max over ranks of 10 + 5 * rank
        assert n == 1 << 16
    assert res[0][4] != res[1][4], "ranks must run different replicas"


def _ref_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import contextlib
    import io

    import bench

    class A:
        steps, warmup, gpus = 1, 0, world

    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(A, "plain")
    out[rank] = buf.getvalue()


def test_reference_arm_runs_on_rank_zero_only():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_ref_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    import json

    line = json.loads(res[0].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert res[1].strip() == ""


def test_mixed_pool_is_a_permutation_of_its_sources():
    import ltpmg_gb300 as G
    from ltpmg_gb300 import workloads as W

    g = G.Tpcc(2, seed=4)
    tf_t, k_t, w_t, pay_t, _, _, pf_t = g.gen(0, 400, with_pay_first=True)
    y = G.gen_ycsb(9, 4096, 10, 1, 16, 0.7, 0.99, batch=0, n_txns=400)
    tf, keys, opw, pf, pay, src = W.mixed_pool(y, (tf_t, k_t, w_t, pay_t, pf_t), seed=2)
    assert len(tf) == 801 and src.sum() == 400 and len(pay) == len(pay_t)
    ti = yi = 0
    for j in range(800):
        a, b = int(tf[j]), int(tf[j + 1])
        if src[j]:
            sa, sb = int(tf_t[ti]), int(tf_t[ti + 1])
            assert np.array_equal(opw[a:b], w_t[sa:sb] + (1 << 8))
            ins = (w_t[sa:sb] & 3) == 2
            assert np.array_equal(keys[a:b][~ins], k_t[sa:sb][~ins])
            assert np.array_equal(keys[a:b][ins] - pf[j], k_t[sa:sb][ins] - pf_t[ti])
            assert np.array_equal(pay[pf[j]:pf[j + 1]], pay_t[pf_t[ti]:pf_t[ti + 1]])
            ti += 1
        else:
            sa, sb = int(y[0][yi]), int(y[0][yi + 1])
            assert np.array_equal(keys[a:b], y[1][sa:sb]) and pf[j] == pf[j + 1]
            yi += 1
