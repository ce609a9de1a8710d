"""Autotuner host logic with a fake context and timer (no GPU): the fastest
candidates win, configurations that do not fit are skipped, results are
cached per mesh-size class and re-applied from the cache."""
import json

from tahoe_gb300 import autotune, lib


class FakeCtx:
    def __init__(self, nnd=5000, nel=4000):
        self.nnd, self.nel = nnd, nel
        self.cfg = {"tile_blocks": 640, "stages": 2, "tangent_epb": 8, "release": 0, "sym": 0, "sym_tile": 0}
        self.tangents = 0

    def spmv_config(self, t, s):
        if t * s > 3000:
            raise lib.TahoeError(-8, "tg_spmv_config", "does not fit")
        self.last = (t, s)
        self.cfg["tile_blocks"], self.cfg["stages"] = t, s
        self.formed = False  # a new tile layout drops the assembled tangent

    def spmv_release(self, r):
        self.cfg["release"] = r

    def spmv_symmetric(self, on, tile_blocks=0):
        self.cfg["sym"] = on
        if tile_blocks:
            self.cfg["sym_tile"] = tile_blocks

    def tangent_config(self, e):
        self.cfg["tangent_epb"] = e

    def tangent(self, precision):
        self.tangents += 1
        self.formed = True


def fake_timer(ctx, which, reps):
    assert getattr(ctx, "formed", False), "kernel timed without a formed tangent"
    c = ctx.cfg
    if which == autotune.KERNEL_SPMV and c["tile_blocks"] == 1024 and c["stages"] == 2 and c["release"] == 1:
        # a ring that fits the configuration call but not the launch
        raise lib.TahoeError(-8, "tg_time_kernel", "does not fit")
    if which == autotune.KERNEL_SPMV and c["sym"]:
        # symmetric format: faster than every full-storage shape only as mode 2 at 384 blocks per tile
        return 0.5 if (c["sym"], c["sym_tile"]) == (2, 384) else 5.0
    if which == autotune.KERNEL_SPMV:
        return abs(c["tile_blocks"] - 768) / 100.0 + (0.5 if c["stages"] == 3 else 0.0) + 1.0 - 0.1 * c["release"]
    return {2: 3.0, 4: 1.5, 8: 2.0}[c["tangent_epb"]]


def test_picks_fastest_and_caches(tmp_path):
    path = str(tmp_path / "tuning.json")
    t = autotune.Tuner(cache_path=path, reps=4)
    ctx = FakeCtx()
    out = t.tune(ctx, lib.MIXED, lib.TOTAL_LAGRANGIAN, timer=fake_timer)
    assert not out["cached"]
    assert (out["tile_blocks"], out["stages"], out["release"], out["tangent_epb"]) == (768, 2, 1, 4)
    assert (out["sym"], out["sym_tile"]) == (2, 384) and out["spmv_ms"] == 0.5
    assert ctx.cfg == {"tile_blocks": 768, "stages": 2, "tangent_epb": 4, "release": 1, "sym": 2, "sym_tile": 384}
    # 1024x3 and 1536x2/3 do not fit and are skipped, not chosen
    assert out["spmv_sweep"]["1536x2r0"] is None and out["spmv_sweep"]["1024x3r1"] is None
    assert out["spmv_sweep"]["1024x2r1"] is None and out["spmv_sweep"]["1024x2r0"] is not None
    with open(path) as f:
        table = json.load(f)
    assert len(table) == 1
    # a second tuner reads the cache and applies it without timing
    ctx2 = FakeCtx(nnd=5100, nel=4050)  # same size class
    t2 = autotune.Tuner(cache_path=path)
    out2 = t2.tune(ctx2, lib.MIXED, lib.TOTAL_LAGRANGIAN, timer=lambda *a: 1 / 0)
    assert out2["cached"] and ctx2.cfg == {"tile_blocks": 768, "stages": 2, "tangent_epb": 4, "release": 1,
                                           "sym": 2, "sym_tile": 384}
    # another size class or precision is tuned separately
    assert autotune.signature(FakeCtx(nnd=50000), lib.MIXED, 1) != autotune.signature(ctx, lib.MIXED, 1)
    assert autotune.signature(ctx, lib.FP64, 1) != autotune.signature(ctx, lib.MIXED, 1)


def test_pick_ignores_unavailable():
    assert autotune.pick({"a": None, "b": 2.0, "c": 1.0}) == ("c", 1.0)
    assert autotune.pick({"a": None}) == (None, float("inf"))


def test_full_storage_kept_when_symmetric_is_slower(tmp_path):
    def timer(ctx, which, reps):
        if which == autotune.KERNEL_SPMV and ctx.cfg["sym"]:
            return 9.0
        return fake_timer(ctx, which, reps)

    t = autotune.Tuner(cache_path=str(tmp_path / "t.json"), reps=4)
    ctx = FakeCtx()
    out = t.tune(ctx, lib.MIXED, lib.TOTAL_LAGRANGIAN, timer=timer)
    assert out["sym"] == 0 and ctx.cfg["sym"] == 0


class FakePushCtx(FakeCtx):
    """A context whose solve streams the push storage (form 3)."""

    def effective_form(self):
        return 3

    def tuning(self):
        return {"tile_blocks": self.cfg["tile_blocks"], "stages": self.cfg["stages"],
                "tangent_epb": self.cfg["tangent_epb"]}

    def spmv_config(self, t, s):
        raise AssertionError("the push storage's product has no full-storage shape to sweep")

    def spmv_symmetric(self, on, tile_blocks=0):
        raise AssertionError("the push storage's solve is not switched to the symmetric format")


def test_push_storage_tunes_the_tangent_only(tmp_path):
    t = autotune.Tuner(cache_path=str(tmp_path / "tuning.json"), reps=4)
    ctx = FakePushCtx()
    out = t.tune(ctx, lib.MIXED, lib.TOTAL_LAGRANGIAN, timer=fake_timer)
    assert out["push"] and not out["cached"]
    assert (out["tangent_epb"], out["sym"], out["tile_blocks"], out["stages"]) == (4, 0, 640, 2)
    assert ctx.cfg["tangent_epb"] == 4 and ctx.tangents >= 1
    again = t.tune(FakePushCtx(), lib.MIXED, lib.TOTAL_LAGRANGIAN, timer=fake_timer)
    assert again["cached"] and again["tangent_epb"] == 4
    # the key tells the push storage's tuning from the full storage's
    assert autotune.signature(ctx, lib.MIXED, lib.TOTAL_LAGRANGIAN) != \
        autotune.signature(FakeCtx(), lib.MIXED, lib.TOTAL_LAGRANGIAN)

