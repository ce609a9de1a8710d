"""Launch-shape autotuner for the hot kernels.

Two shapes are tuned on the mesh a context holds, by timing the kernels
themselves (CUDA events, tg_time_kernel) on the current state:

  * the streamed PCG product: rows per tile (the unit of the tile-contiguous
    matrix storage, in block nonzeros) x depth of the shared-memory ring x
    stage release (CTA barrier per tile, or per-warp release on an mbarrier),
    then the symmetric stream format (upper blocks only; three launch shapes
    x upper blocks per tile), which replaces the full storage where it is
    faster on the mesh at hand;
  * the element tangent: elements per CTA (one thread per upper node-pair
    block of each element).

When the solve streams the symmetric push storage (tg_pcg_form 3, the
default on meshes of a million block nonzeros and more), the product has
the one launch shape of that storage: the full-storage and symmetric-format
sweeps are skipped (they would time the same product for every candidate)
and only the tangent is tuned.

Results are cached per (GPU, precision, formulation, mesh-size bucket) in a
JSON table, so a serving process tunes once per kind of mesh.  Element
matrices do not depend on the tangent shape (bitwise), and a different tile
size only regroups rows, so tuning changes timings, not results beyond the
rounding order of the Krylov dot products.
"""
import json
import math
import os

from . import lib

SPMV_TILES = (256, 384, 512, 640, 768, 1024, 1536)
SPMV_STAGES = (2, 3)
SPMV_RELEASE = (0, 1)
TANGENT_EPB = (2, 4, 8)
SYM_MODES = (1, 2, 3)
SYM_TILES = (256, 384, 512)
KERNEL_SPMV, KERNEL_TANGENT = 0, 2

_DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "tuning.json")


def signature(ctx, precision, formulation, gpu="gpu0"):
    """Cache key: mesh sizes bucketed to powers of two (shapes are chosen for
    the size class, not the exact mesh), and whether the solve streams the
    push storage."""
    b = lambda x: 1 << max(0, int(math.log2(max(1, x))))
    form = getattr(ctx, "effective_form", None)
    push = "|push" if form is not None and form() == 3 else ""
    return "%s|p%d|f%d|nnd%d|nel%d%s" % (gpu, precision, formulation, b(ctx.nnd), b(ctx.nel), push)


def pick(timings):
    """Fastest candidate of {config: ms}; ties go to the first listed."""
    best, best_ms = None, float("inf")
    for cfg, ms in timings.items():
        if ms is not None and ms < best_ms:
            best, best_ms = cfg, ms
    return best, best_ms


class Tuner:
    def __init__(self, cache_path=_DEFAULT_CACHE, reps=20, tiles=SPMV_TILES, stages=SPMV_STAGES, epbs=TANGENT_EPB,
                 releases=SPMV_RELEASE, sym_modes=SYM_MODES, sym_tiles=SYM_TILES):
        self.cache_path = cache_path
        self.reps = reps
        self.tiles, self.stages, self.epbs, self.releases = tiles, stages, epbs, releases
        self.sym_modes, self.sym_tiles = sym_modes, sym_tiles
        self.table = {}
        if cache_path and os.path.exists(cache_path):
            try:
                with open(cache_path) as f:
                    self.table = json.load(f)
            except (OSError, ValueError):
                self.table = {}

    def save(self):
        if not self.cache_path:
            return
        os.makedirs(os.path.dirname(self.cache_path), exist_ok=True)
        tmp = self.cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.table, f, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    @staticmethod
    def apply(ctx, cfg):
        if cfg.get("push"):  # the push storage's product keeps its one shape
            ctx.tangent_config(cfg["tangent_epb"])
            return
        ctx.spmv_config(cfg["tile_blocks"], cfg["stages"])
        ctx.spmv_release(cfg.get("release", 0))
        ctx.spmv_symmetric(cfg.get("sym", 0), cfg.get("sym_tile", 0))
        ctx.tangent_config(cfg["tangent_epb"])

    def tune(self, ctx, precision, formulation, gpu="gpu0", force=False, timer=None):
        """Tunes (or takes from the cache) and applies the shapes; returns the
        chosen config with the measured timings.  The context must hold a
        mesh and a state on which a tangent can be formed.  `timer(ctx, which,
        reps)` defaults to the library's kernel timer."""
        key = signature(ctx, precision, formulation, gpu)
        if not force and key in self.table:
            cfg = self.table[key]
            self.apply(ctx, cfg)
            return dict(cfg, cached=True)
        timer = timer or (lambda c, which, reps: c.time_kernel(which, reps))
        form = getattr(ctx, "effective_form", None)
        if form is not None and form() == 3:
            return self._tune_tangent_only(ctx, precision, key, timer)
        spmv = {}
        for t in self.tiles:
            for s in self.stages:
                try:
                    ctx.spmv_config(t, s)
                    ctx.tangent(precision)  # assemble into the new tile layout
                except lib.TahoeError as e:
                    if e.code != -8:
                        raise
                    for r in self.releases:
                        spmv[(t, s, r)] = None  # ring does not fit on an SM
                    continue
                for r in self.releases:
                    ctx.spmv_release(r)
                    try:
                        spmv[(t, s, r)] = timer(ctx, KERNEL_SPMV, self.reps)
                    except lib.TahoeError as e:
                        if e.code != -8:  # only "does not fit" is a skipped candidate
                            raise
                        spmv[(t, s, r)] = None
        (tb, st, rl), spmv_ms = pick(spmv)
        ctx.spmv_config(tb, st)
        ctx.spmv_release(rl)
        ctx.tangent(precision)
        # the symmetric stream format, against the best full-storage shape
        sym = {}
        for m in self.sym_modes:
            for t in self.sym_tiles:
                try:
                    ctx.spmv_symmetric(m, t)
                    sym[(m, t)] = timer(ctx, KERNEL_SPMV, self.reps)
                except lib.TahoeError as e:
                    if e.code != -8:
                        raise
                    sym[(m, t)] = None
        best_sym, sym_ms = pick(sym) if sym else (None, float("inf"))
        sm, stile = (best_sym if best_sym is not None and sym_ms < spmv_ms else (0, 0))
        ctx.spmv_symmetric(sm, stile)
        tang = {}
        for e in self.epbs:
            ctx.tangent_config(e)
            tang[e] = timer(ctx, KERNEL_TANGENT, max(3, self.reps // 4))
        epb, tang_ms = pick(tang)
        cfg = {"tile_blocks": tb, "stages": st, "release": rl, "sym": sm, "sym_tile": stile, "tangent_epb": epb,
               "spmv_ms": min(spmv_ms, sym_ms) if sm else spmv_ms, "tangent_ms": tang_ms}
        self.apply(ctx, cfg)
        ctx.tangent(precision)
        self.table[key] = cfg
        self.save()
        out = dict(cfg, cached=False)
        out["spmv_sweep"] = {"%dx%dr%d" % k: v for k, v in spmv.items()}
        out["spmv_sweep"].update({"sym%dx%d" % k: v for k, v in sym.items()})
        out["tangent_sweep"] = {str(k): v for k, v in tang.items()}
        return out

    def _tune_tangent_only(self, ctx, precision, key, timer):
        """The push storage's solve: the product keeps its one shape (timed
        for the record), the tangent's elements per CTA are tuned."""
        cur = ctx.tuning()
        ctx.tangent(precision)
        spmv_ms = timer(ctx, KERNEL_SPMV, self.reps)
        tang = {}
        for e in self.epbs:
            ctx.tangent_config(e)
            tang[e] = timer(ctx, KERNEL_TANGENT, max(3, self.reps // 4))
        epb, tang_ms = pick(tang)
        cfg = {"tile_blocks": cur["tile_blocks"], "stages": cur["stages"], "release": 0, "sym": 0, "sym_tile": 0,
               "tangent_epb": epb, "spmv_ms": spmv_ms, "tangent_ms": tang_ms, "push": True}
        ctx.tangent_config(epb)
        self.table[key] = cfg
        self.save()
        out = dict(cfg, cached=False)
        out["tangent_sweep"] = {str(k): v for k, v in tang.items()}
        return out
