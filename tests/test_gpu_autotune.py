"""Autotuner on the GPU: every tangent shape gives bitwise the same element
matrices and assembled tangent, the tuned product gives the same PCG solution
(to rounding of the dot products), and the tuned shapes are applied."""
import numpy as np
import pytest

from tahoe_gb300 import autotune, lib
from tests.helpers import rel_err
from tahoe_gb300.model import SolidModel
from tahoe_gb300.meshgen import BoxMesh

pytestmark = pytest.mark.gpu


def _ctx(n=10):
    mesh = BoxMesh(n, n, n, jitter=0.2, seed=3)
    m = SolidModel(mesh.X, mesh.conn, "total_lagrangian", {"kind": "fs_simo", "mu": 1.0, "kappa": 10.0})
    for node in mesh.face_nodes(2, 0):
        for d in range(3):
            m.add_kbc(node, d, 0.0, False)
    for node in mesh.face_nodes(2, 1):
        m.add_kbc(node, 2, -0.01, True)
    m.set_schedule([(0.0, 0.0), (1.0, 1.0)])
    m.setup()
    m.apply_step(1.0, (lib.MIXED, 0, 1e-6))
    c = m.ctx
    c.set_iteration(0)
    c.residual(want_vector=False)
    return c


def test_tangent_shapes_bitwise_equal():
    c = _ctx()
    ref = None
    for e in (8, 4, 2):
        c.tangent_config(e)
        c.tangent(lib.MIXED)
        K = c.tangent_csr()
        if ref is None:
            ref = K
        else:
            assert all(np.array_equal(a, b) for a, b in zip(ref, K)), e


def test_tuned_shapes_applied_and_solution_unchanged(tmp_path):
    c = _ctx()
    c.tangent(lib.MIXED)
    R, _ = c.residual()
    du0 = c.pcg(R, rel_tol=1e-7)[0]
    t = autotune.Tuner(cache_path=str(tmp_path / "t.json"), reps=3, tiles=(256, 640, 1024), stages=(2, 3))
    out = t.tune(c, lib.MIXED, lib.TOTAL_LAGRANGIAN)
    assert not out["cached"]
    assert c.tuning() == {k: out[k] for k in ("tile_blocks", "stages", "tangent_epb")}
    # the two stage-release variants of the product give bitwise the same solve
    sols = []
    for r in (0, 1):
        c.spmv_release(r)
        c.tangent(lib.MIXED)
        sols.append(c.pcg(R, rel_tol=1e-7)[:2])
    assert np.array_equal(sols[0][0], sols[1][0]) and sols[0][1] == sols[1][1]
    c.tangent(lib.MIXED)
    du1 = c.pcg(R, rel_tol=1e-7)[0]
    assert rel_err(du1, du0) < 1e-5
    # cached: same shapes re-applied without timing
    out2 = autotune.Tuner(cache_path=str(tmp_path / "t.json")).tune(c, lib.MIXED, lib.TOTAL_LAGRANGIAN)
    assert out2["cached"] and out2["tile_blocks"] == out["tile_blocks"]


def test_push_storage_tunes_the_tangent_only(tmp_path):
    """With the solve on the symmetric push storage the tuner leaves the
    product's storage and shapes alone (no full-storage or symmetric-format
    sweep) and tunes the tangent: the solve after tuning is bitwise the one
    before it."""
    c = _ctx()
    c.pcg_form(3)
    c.tangent(lib.MIXED)
    R, _ = c.residual()
    du0, its0 = c.pcg(R, rel_tol=1e-7)[:2]
    shapes = c.tuning()
    out = autotune.Tuner(cache_path=str(tmp_path / "t.json"), reps=3).tune(c, lib.MIXED, lib.TOTAL_LAGRANGIAN)
    assert out["push"] and out["sym"] == 0 and not out["cached"]
    now = c.tuning()
    assert (now["tile_blocks"], now["stages"]) == (shapes["tile_blocks"], shapes["stages"])
    assert now["tangent_epb"] == out["tangent_epb"]
    assert c.effective_form() == 3 and c.product_kernel() == "pcg_cg_push_kernel"
    c.tangent(lib.MIXED)
    du1, its1 = c.pcg(R, rel_tol=1e-7)[:2]
    assert np.array_equal(du0, du1) and its0 == its1
    c.pcg_form(-1)
