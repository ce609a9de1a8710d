"""Batch meshes composed on the device from resident templates against the
same batch uploaded as one concatenated mesh: equation pattern, residual (FP64
and the mixed form's double-float residual on the templates' pooled geometry
planes) and assembled tangent bit-exact, affine boundary values equal, and the solved
RVE stresses equal; a lane context reused across batches of different size
gives what a fresh context gives."""
import numpy as np
import pytest

from tahoe_gb300 import lib, rve
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

NS = np.array([4, 5, 4, 6])


def _Fs(k, seed=5):
    rng = np.random.default_rng(seed)
    return np.stack([rve.sample_F(rng) for _ in range(k)])


@pytest.fixture(scope="module")
def pair():
    Fs = _Fs(len(NS))
    up = rve.RVEBatch(NS, Fs)
    up.setup()
    res = rve.ResidentRVEs(lib.Context(0))
    res.compose(NS)
    return up, res, Fs


def test_pattern_bit_exact(pair):
    up, res, _ = pair
    for upper in (True, False):
        a = up.ctx.pattern(upper_only=upper)
        b = res.ctx.pattern(upper_only=upper)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert up.ctx.neq == res.ctx.neq and up.ctx.block_nnz == res.ctx.block_nnz


def test_affine_values_and_residual_tangent_bit_exact(pair):
    up, res, Fs = pair
    up.ctx.set_u(np.zeros_like(up.X))
    up.ctx.set_prescribed(up.prescribed_idx, up.prescribed_val)
    res.ctx.set_affine(Fs)
    ua, ub = up.ctx.get_u(), res.ctx.get_u()
    assert rel_err(ub, ua) < 1e-15
    # same displacement on both: everything downstream must agree bitwise
    rng = np.random.default_rng(2)
    u = ua + 1e-3 * rng.standard_normal(ua.shape)
    for c in (up.ctx, res.ctx):
        c.set_u(u)
        c.set_iteration(0)
    Ra = up.ctx.residual()
    Rb = res.ctx.residual()
    assert np.array_equal(Ra[0], Rb[0]) and Ra[1] == Rb[1]
    # the mixed form's double-float residual: the uploaded mesh forms its own
    # geometry planes, the composed one reads its templates' pooled planes
    Ra = up.ctx.residual(precision=lib.MIXED)
    Rb = res.ctx.residual(precision=lib.MIXED)
    assert np.array_equal(Ra[0], Rb[0]) and Ra[1] == Rb[1]
    for prec in (lib.FP64, lib.MIXED):
        up.ctx.tangent(prec)
        res.ctx.tangent(prec)
        ta = up.ctx.tangent_csr(upper_only=False)
        tb = res.ctx.tangent_csr(upper_only=False)
        assert all(np.array_equal(x, y) for x, y in zip(ta, tb))


def test_solved_stress_matches_uploaded_batch(pair):
    up, res, Fs = pair
    rc, rep, rel, Pa = up.solve(precision=lib.MIXED)
    assert rc == 0
    rc, rep, rel, Pb = res.solve(NS, Fs, precision=lib.MIXED)
    assert rc == 0 and rel.max() < 1e-8
    assert rel_err(Pb, Pa) < 1e-10


def test_context_reused_across_batches():
    res = rve.ResidentRVEs(lib.Context(0))
    big, small = np.array([7, 6, 8, 5]), np.array([4, 5])
    Fb, Fsm = _Fs(4, 8), _Fs(2, 9)
    assert res.solve(big, Fb)[0] == 0
    rc, _, _, P1 = res.solve(small, Fsm)
    assert rc == 0
    fresh = rve.ResidentRVEs(lib.Context(0))
    rc, _, _, P2 = fresh.solve(small, Fsm)
    assert rc == 0
    assert np.array_equal(P1, P2)
