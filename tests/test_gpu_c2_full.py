"""The default paths of the mixed form at the full C2 size (64^3 hex8,
274,625 nodes, 7,189,057 block nonzeros, TL Simo), through the C ABI.

* The double-float residual equals the FP64 residual on the step-1
  predictor state to 1e-9 of its largest entry and norm.  That residual is
  nearly equilibrated -- about a thousandth of the element forces it sums --
  and the double-float error scales with the forces (1e-11 of them at random
  displacements, tests/test_gpu_residual_ff.py), so 1e-9 of this residual is
  still ten times below Newton's 1e-8 relative tolerance.
* One Newton iteration on the symmetric push storage (the default at this
  size) and on the full storage (form 1) from the same snapshot, inner PCG
  to 1e-6: the iteration counts agree within 2 %, the displacements within
  1e-3 of the increment, and the new residual norms within 1 %.
"""
import numpy as np
import pytest

from tahoe_gb300 import lib, workloads
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2():
    mesh, model, _ = workloads.c2()
    model.setup()
    model.apply_step(1.0, (lib.MIXED, lib.PRECOND_JACOBI, 1e-4))
    ctx = model.ctx
    ctx.set_iteration(-1)
    return mesh, model, ctx


def test_double_float_residual_at_c2_size(c2):
    mesh, model, ctx = c2
    R64, n64 = ctx.residual()
    Rff, nff = ctx.residual(precision=lib.MIXED)
    assert rel_err(Rff, R64) < 1e-9
    assert abs(nff - n64) <= 1e-9 * n64


def test_push_and_full_storage_newton_iteration_at_c2_size(c2):
    mesh, model, ctx = c2
    assert ctx.effective_form() == 3
    ctx.residual(want_vector=False, precision=lib.MIXED)
    ctx.checkpoint()
    u0 = ctx.get_u()
    out = {}
    for form in (-1, 1):
        ctx.pcg_form(form)
        ctx.rollback()
        ctx.set_iteration(-1)
        nrm, its = ctx.newton_iteration(precision=lib.MIXED, precond=lib.PRECOND_JACOBI, lin_rel_tol=1e-6)
        out[form] = (ctx.get_u(), its, nrm)
    ctx.pcg_form(-1)
    (ua, ia, na), (ub, ib, nb) = out[-1], out[1]
    assert abs(ia - ib) <= max(3, 0.02 * ib), (ia, ib)
    du = ub - u0
    assert np.abs(ua - ub).max() <= 1e-3 * np.abs(du).max()
    assert abs(na - nb) <= 0.01 * nb
