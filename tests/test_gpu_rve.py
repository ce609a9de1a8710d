"""Batched FE^2 RVE solves on the GPU against the oracle, per RVE.

Displacements within 1e-8 of the oracle's direct solve, the volume-averaged
first Piola stress within 1e-7 of the oracle's reaction sum
(1/V0) sum_{boundary a} f_a (x) X_a, the mixed form within 1e-6 of FP64, and
an RVE solved alone equal (1e-6) to the same RVE solved inside a batch.
"""
import numpy as np
import pytest

from tahoe_gb300 import lib, rve
from tests.helpers import oracle_rve, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    ns = np.array([4, 5, 4, 6, 5])
    rng = np.random.default_rng(11)
    Fs = np.stack([rve.sample_F(rng) for _ in ns])
    return ns, Fs


def test_batch_matches_oracle_per_rve(batch):
    ns, Fs = batch
    b = rve.RVEBatch(ns, Fs)
    b.setup()
    rc, rep, rel, P = b.solve(precision=lib.FP64, rel_tol=1e-10, lin_rel_tol=1e-12)
    assert rc == 0 and rel.max() < 1e-10
    u = b.ctx.get_u()
    for r, (n, F) in enumerate(zip(ns, Fs)):
        uo, Po = oracle_rve(int(n), F)
        assert rel_err(b.rve_displacement(r, u), uo) < 1e-8, r
        assert rel_err(P[r], Po) < 1e-7, r


def test_mixed_batch_within_1e6_of_fp64(batch):
    ns, Fs = batch
    res = {}
    for prec in (lib.FP64, lib.MIXED):
        b = rve.RVEBatch(ns, Fs)
        b.setup()
        rc, rep, rel, P = b.solve(precision=prec, rel_tol=1e-8, lin_rel_tol=1e-4)
        assert rc == 0 and rel.max() < 1e-8
        res[prec] = P
    assert rel_err(res[lib.MIXED], res[lib.FP64]) < 1e-6


def test_rve_alone_equals_rve_in_batch(batch):
    ns, Fs = batch
    b = rve.RVEBatch(ns, Fs)
    b.setup()
    rc, rep, rel, P = b.solve(precision=lib.MIXED, rel_tol=1e-8)
    assert rc == 0
    for r in (1, 3):
        one = rve.RVEBatch(ns[r:r + 1], Fs[r:r + 1])
        one.setup()
        rc1, rep1, rel1, P1 = one.solve(precision=lib.MIXED, rel_tol=1e-8)
        assert rc1 == 0
        assert rel_err(P1[0], P[r]) < 1e-6, r


def test_macro_tangent_matches_oracle_finite_differences(batch):
    """dP/dF by static condensation on the GPU against central differences of
    the oracle's averaged stress (reaction sum), per RVE; major symmetry of the
    hyperelastic tangent; mixed form against FP64."""
    ns, Fs = batch
    ns, Fs = ns[:2], Fs[:2]
    b = rve.RVEBatch(ns, Fs)
    b.setup()
    rc, rep, rel, P = b.solve(precision=lib.FP64, rel_tol=1e-12, lin_rel_tol=1e-12)
    assert rc == 0
    C64, its = b.ctx.macro_tangent(b.vol0, precision=lib.FP64, lin_rel_tol=1e-12)
    assert its > 0
    h = 1e-5
    for r, (n, F) in enumerate(zip(ns, Fs)):
        Cfd = np.zeros((9, 9))
        for kL in range(9):
            dF = np.zeros(9)
            dF[kL] = h
            Pp = oracle_rve(int(n), F + dF.reshape(3, 3))[1]
            Pm = oracle_rve(int(n), F - dF.reshape(3, 3))[1]
            Cfd[:, kL] = (Pp - Pm).reshape(9) / (2 * h)
        assert rel_err(C64[r], Cfd) < 1e-6, r
        assert rel_err(C64[r], C64[r].T) < 1e-9, r
    Cm, _ = b.ctx.macro_tangent(b.vol0, precision=lib.MIXED, lin_rel_tol=1e-7)
    assert rel_err(Cm, C64) < 1e-5
