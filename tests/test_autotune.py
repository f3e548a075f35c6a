"""Host logic of the autotuner (no GPU): candidate order, the 64-cell word
and pre-check stages, when graph-captured timing is used, and the JSON
round trip.  Timings come from a stand-in for the CUDA-event timer."""
import ltpmg_gb300.autotune as AT
from ltpmg_gb300 import lib as L


class FakeCtx:
    def __init__(self):
        self.tuning = {}
        self.calls = []

    def set_tuning(self, bucket, block, ipt, word_bits=32, flags=0):
        self.tuning[bucket] = (block, ipt, word_bits, flags)
        self.calls.append((bucket, block, ipt, word_bits, flags))


class FakeBatch:
    def __init__(self, n_ops, payload=False):
        self.n_ops = n_ops
        if payload:
            self._keep_payload = [1, 2, 3]

    def execute(self):
        pass

    def finish(self):
        pass


def _fake_timer(cost, seen):
    """cost(block, ipt, word_bits, flags) -> ms; records the copies asked for."""

    def t(ctx, batch, reps, copies=1):
        seen.append(copies)
        return cost(*ctx.tuning[AT.bucket_of(batch.n_ops)])

    return t


def test_tune_tiles_picks_fastest_then_word_width_then_precheck(monkeypatch):
    def cost(block, ipt, wb, flags):
        ms = 1.0 + abs(block - 256) / 1000 + abs(ipt - 2) / 100
        if wb == 64:
            ms -= 0.05 if (block, ipt) == (256, 2) else -0.5
        if flags:
            ms -= 0.01
        return ms

    seen = []
    monkeypatch.setattr(AT, "_time_batch", _fake_timer(cost, seen))
    ctx = FakeCtx()
    ch = AT.tune_tiles(ctx, FakeBatch(1 << 20), reps=1, copies=4)
    assert (ch["block"], ch["ipt"], ch["word_bits"], ch["flags"]) == (256, 2, 64, L.TUNE_MARK_PRECHECK)
    assert ctx.tuning[20] == (256, 2, 64, L.TUNE_MARK_PRECHECK)
    # 64-cell words only for tilings of at most 2048 ops, at most three of them
    w64 = [k for k in ch["candidates"] if k.endswith("w64")]
    assert 1 <= len(w64) <= 3
    for k in w64:
        b, i = (int(x) for x in k[:-3].split("x"))
        assert b * i <= 2048
    assert set(seen) == {4}


def test_tune_tiles_keeps_precheck_off_when_slower(monkeypatch):
    def cost(block, ipt, wb, flags):
        return 1.0 + (0.2 if flags else 0.0) + (0.1 if wb == 64 else 0.0) + (0.0 if (block, ipt) == (512, 4) else 0.3)

    monkeypatch.setattr(AT, "_time_batch", _fake_timer(cost, []))
    ctx = FakeCtx()
    ch = AT.tune_tiles(ctx, FakeBatch(1 << 18), reps=1)
    assert (ch["block"], ch["ipt"], ch["word_bits"], ch["flags"]) == (512, 4, 32, 0)
    assert ctx.tuning[18] == (512, 4, 32, 0)


def test_graph_timing_only_for_small_batches_without_payload(monkeypatch):
    for batch, want in ((FakeBatch(1 << 16), 4), (FakeBatch(1 << 22), 1), (FakeBatch(1 << 16, payload=True), 1)):
        seen = []
        monkeypatch.setattr(AT, "_time_batch", _fake_timer(lambda *a: 1.0, seen))
        AT.tune_tiles(FakeCtx(), batch, reps=1, copies=4)
        assert set(seen) == {want}


def test_tune_buckets_uses_the_largest_batch_of_each_bucket(monkeypatch):
    tuned = []

    def fake_tune(ctx, b, reps, copies=1):
        tuned.append(b.n_ops)
        return {"bucket": AT.bucket_of(b.n_ops), "block": 256, "ipt": 2, "ms": 1.0}

    monkeypatch.setattr(AT, "tune_tiles", fake_tune)
    out = AT.tune_buckets(FakeCtx(), [FakeBatch(n) for n in (1000, 1010, 1 << 20, (1 << 20) + 5, 40)])
    assert sorted(tuned) == [40, 1010, (1 << 20) + 5]  # buckets 5, 9 (512..1023 ops) and 20
    assert sorted(out) == [5, 9, 20]


def test_parse_choice_names():
    assert AT.parse_choice("512x4") == (512, 4, 32, 0)
    assert AT.parse_choice("512x2w64") == (512, 2, 64, 0)
    assert AT.parse_choice("256x8w64+precheck") == (256, 8, 64, L.TUNE_MARK_PRECHECK)
    assert AT.parse_choice("128x1+precheck") == (128, 1, 32, L.TUNE_MARK_PRECHECK)


def test_refine_pipeline_keeps_the_fastest_over_the_batch_list(monkeypatch):
    # single-batch order: 512x2w64+precheck < 512x2w64 < 512x4 < 256x2; the two
    # fastest tilings (512x2w64, 512x4) run with and without the pre-check over
    # the list, where 512x4 with the pre-check wins
    P = L.TUNE_MARK_PRECHECK
    choice = {"bucket": 22, "block": 512, "ipt": 2, "word_bits": 64, "flags": P, "ms": 0.30,
              "candidates": {"512x2w64+precheck": 0.30, "512x2w64": 0.305, "512x4": 0.31, "256x2": 0.33}}
    list_ms = {(512, 2, 64, P): 2.89, (512, 2, 64, 0): 2.90, (512, 4, 32, 0): 2.86, (512, 4, 32, P): 2.82}
    seen = []

    def fake_list(ctx, batches, reps, mode=L.MODE_GRAPH):
        t = ctx.tuning[22]
        seen.append(t)
        return list_ms[t]

    monkeypatch.setattr(AT, "_time_list", fake_list)
    ctx = FakeCtx()
    out = AT.refine_pipeline(ctx, [FakeBatch(1 << 22)] * 4, choice)
    assert sorted(seen) == sorted(list_ms)
    assert (out["block"], out["ipt"], out["word_bits"], out["flags"]) == (512, 4, 32, P)
    assert ctx.tuning[22] == (512, 4, 32, P)
    assert out["pipeline_ms"]["512x4+precheck"] == 2.82


def test_save_and_load_round_trip(tmp_path):
    choices = {14: {"block": 128, "ipt": 1, "word_bits": 32, "flags": 0, "ms": 0.02},
               22: {"block": 512, "ipt": 2, "word_bits": 64, "flags": L.TUNE_MARK_PRECHECK, "ms": 0.3}}
    path = tmp_path / "tuning.json"
    AT.save(str(path), choices, mode=L.MODE_GRAPH)
    ctx = FakeCtx()
    assert AT.load(ctx, str(path)) == L.MODE_GRAPH
    assert ctx.tuning == {14: (128, 1, 32, 0), 22: (512, 2, 64, L.TUNE_MARK_PRECHECK)}
