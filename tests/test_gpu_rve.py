"""Batched FE^2 RVE solves on the GPU against the oracle, per RVE.

Displacements within 1e-8 of the oracle's direct solve, the volume-averaged
first Piola stress within 1e-7 of the oracle's reaction sum
(1/V0) sum_{boundary a} f_a (x) X_a, the mixed form within 1e-6 of FP64, and
an RVE solved alone bitwise equal to the same RVE solved inside a batch,
a failing RVE reported alone, and the macro tangent in a batch against alone.
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
    """One Krylov solve per RVE (own scaling, alpha, beta, tolerance and
    convergence over the shared matrix stream; converged RVEs frozen): an RVE
    solved alone and inside a batch give bitwise the same displacements and
    averaged stress, in both precision forms."""
    ns, Fs = batch
    for prec in (lib.MIXED, lib.FP64):
        b = rve.RVEBatch(ns, Fs)
        b.setup()
        rc, rep, rel, P = b.solve(precision=prec, rel_tol=1e-8)
        assert rc == 0 and np.all(b.status == 0)
        u = b.ctx.get_u()
        for r in (1, 3):
            one = rve.RVEBatch(ns[r:r + 1], Fs[r:r + 1])
            one.setup()
            rc1, rep1, rel1, P1 = one.solve(precision=prec, rel_tol=1e-8)
            assert rc1 == 0
            assert np.array_equal(P1[0], P[r]), (prec, r)
            assert np.array_equal(one.ctx.get_u(), b.rve_displacement(r, u)), (prec, r)


def test_failing_rve_fails_alone():
    """With one Newton iteration allowed (exact inner solves) some RVEs of a
    batch converge and some do not (an RVE under a tiny deformation starts
    at round-off and cannot gain eight digits; F = I + 0.05 S converges in
    one).  Every RVE's outcome in the batch is its outcome alone, the
    failures are reported per RVE, and every converged RVE's result is its
    own solve, bitwise."""
    rng = np.random.default_rng(5)
    S = [rve.sample_F(rng) - np.eye(3) for _ in range(4)]
    ns = np.array([4, 5, 4, 6])
    Fs = np.stack([np.eye(3) + 2e-5 * S[0], np.eye(3) + S[1], np.eye(3) + 2e-5 * S[2], np.eye(3) + S[3]])
    kw = dict(precision=lib.FP64, rel_tol=1e-8, lin_rel_tol=1e-12, max_iterations=1)
    alone = []
    for r in range(len(ns)):
        one = rve.RVEBatch(ns[r:r + 1], Fs[r:r + 1])
        one.setup()
        rc1, _, _, P1 = one.solve(**kw)
        alone.append((int(one.status[0]), P1[0]))
    b = rve.RVEBatch(ns, Fs)
    b.setup()
    rc, rep, rel, P = b.solve(**kw)
    st = [int(v) for v in b.status]
    assert st == [a[0] for a in alone]
    assert 0 in st and any(v != 0 for v in st)
    assert rc == next(v for v in st if v != 0)
    for r in range(len(ns)):
        if st[r] == 0:
            assert np.array_equal(P[r], alone[r][1]), r


def test_batch_wide_solver_still_selectable(batch):
    """tg_segment_solver(0): one PCG over the whole batch (shared scalars);
    the converged stresses agree with the per-RVE solves within 1e-6."""
    ns, Fs = batch
    res = {}
    for per_rve in (True, False):
        b = rve.RVEBatch(ns, Fs)
        b.setup()
        b.ctx.segment_solver(per_rve)
        rc, rep, rel, P = b.solve(precision=lib.MIXED, rel_tol=1e-8)
        assert rc == 0 and rel.max() < 1e-8
        res[per_rve] = P
    assert rel_err(res[False], res[True]) < 1e-6


def test_macro_tangent_in_batch_against_alone_at_bench_tolerance(batch):
    """The nine condensation solves of the macro tangent run as one
    multi-vector PCG whose tolerance is relative to each right-hand side's
    norm over the whole batch.  At the benchmark's inner tolerance (1e-7,
    mixed) every RVE's tangent in the batch stays within 1e-5 of the same
    RVE's tangent computed alone."""
    ns, Fs = batch
    b = rve.RVEBatch(ns, Fs)
    b.setup()
    rc, rep, rel, P = b.solve(precision=lib.MIXED, rel_tol=1e-8)
    assert rc == 0
    C, _ = b.ctx.macro_tangent(b.vol0, precision=lib.MIXED, lin_rel_tol=1e-7)
    for r in range(len(ns)):
        one = rve.RVEBatch(ns[r:r + 1], Fs[r:r + 1])
        one.setup()
        rc1, _, _, _ = one.solve(precision=lib.MIXED, rel_tol=1e-8)
        assert rc1 == 0
        C1, _ = one.ctx.macro_tangent(one.vol0, precision=lib.MIXED, lin_rel_tol=1e-7)
        assert rel_err(C[r], C1[0]) < 1e-5, r


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


@pytest.mark.parametrize("prec", [lib.MIXED, lib.FP64])
def test_push_and_full_storage_batches_agree(batch, prec):
    """The batch's per-RVE solves on the symmetric push storage (the
    default: upper blocks streamed, transposed products pushed to the lower
    rows and added by the update kernel) and on the full storage (form 1)
    reach the same states to the Newton tolerance, with the same RVE
    statuses; the push product's kernel is the one timed for the batch."""
    ns, Fs = batch
    out = {}
    for form in (-1, 1):
        b = rve.RVEBatch(ns, Fs)
        b.setup()
        b.ctx.pcg_form(form)
        rc, rep, rel, P = b.solve(precision=prec, rel_tol=1e-10, lin_rel_tol=1e-10 if prec == lib.FP64 else 1e-6)
        assert rc == 0 and np.all(b.status == 0) and rel.max() < 1e-10
        out[form] = (P, b.ctx.get_u(), b.ctx.product_kernel())
    assert out[-1][2] == "pcg_seg_push_kernel" and out[1][2] == "pcg_spmv_kernel"
    assert rel_err(out[-1][0], out[1][0]) < 1e-8
    assert rel_err(out[-1][1], out[1][1]) < 1e-8
