"""The two recurrence forms of the single-vector PCG and the L2 priorities of
the streamed matrix, through the C ABI.

tg_pcg_form selects the textbook recurrences (form 0: product with a
last-block reduction, vector update with a grid barrier) or the single-
reduction recurrences of Chronopoulos & Gear (form 1, the default: the
product writes CTA partials, every CTA of the vector kernel forms the
iteration's scalars from them); form 3 runs form 1 on the symmetric push
storage (upper node blocks streamed, transposed products pushed to the lower
rows' slots and added by the vector kernel).  All solve the same
(block-)Jacobi CG system, so they reach the same solution to the solve's
tolerance; each is bitwise repeatable.  tg_spmv_l2_keep only changes cache
priorities of the bulk copies, so every setting gives bitwise the same
iterates.
"""
import numpy as np
import pytest

from tahoe_gb300 import lib
from tahoe_gb300.meshgen import BoxMesh
from tahoe_gb300.model import SolidModel

pytestmark = pytest.mark.gpu

SIMO = {"kind": "fs_simo", "mu": 1.0, "kappa": 10.0}


def _model(n=12):
    mesh = BoxMesh(n, n, n, jitter=0.2, seed=3)
    m = SolidModel(mesh.X, mesh.conn, "total_lagrangian", SIMO)
    for node in mesh.face_nodes(2, 0):
        for d in range(3):
            m.add_kbc(node, d)
    for node in mesh.face_nodes(2, 1):
        m.add_kbc(node, 2, -0.02, True)
    m.set_schedule([(0.0, 1.0)])
    m.setup()
    return m


def _system(m, precision, precond):
    m.apply_step(1.0, (precision, precond, 1e-8))
    c = m.ctx
    c.set_iteration(-1)
    R, _ = c.residual()
    c.tangent(precision)
    return c, R


@pytest.mark.parametrize("precision", [lib.MIXED, lib.FP64])
@pytest.mark.parametrize("precond", [lib.PRECOND_JACOBI, lib.PRECOND_BLOCK_JACOBI])
def test_forms_reach_the_same_solution(precision, precond):
    m = _model()
    c, R = _system(m, precision, precond)
    tol = 1e-7 if precision == lib.MIXED else 1e-10
    sol = {}
    for form in (0, 1, 3):
        c.pcg_form(form)
        du, its, rr, rc = c.pcg(R, rel_tol=tol, max_it=20000, precond=precond)
        assert rc == 0, form
        assert rr <= tol, (form, rr)
        sol[form] = (du, its)
    scale = np.abs(sol[0][0]).max()
    # all are within the tolerance of the exact solution of the same system
    bound = 2e-4 if precision == lib.MIXED else 1e-6
    for form in (1, 3):
        assert np.abs(sol[form][0] - sol[0][0]).max() <= bound * scale, form
        # the same Krylov method: iteration counts within a few percent
        assert abs(sol[form][1] - sol[0][1]) <= max(3, 0.05 * sol[0][1]), form
    c.pcg_form(1)


@pytest.mark.parametrize("precision", [lib.MIXED, lib.FP64])
def test_programmatic_launch_dependencies_leave_the_iterates_bitwise_unchanged(precision):
    m = _model()
    c, R = _system(m, precision, lib.PRECOND_BLOCK_JACOBI)
    out = []
    for form in (1, 2, 1):
        c.pcg_form(form)
        out.append(c.pcg(R, rel_tol=1e-8, max_it=20000, precond=lib.PRECOND_BLOCK_JACOBI))
    for du, its, rr, rc in out:
        assert rc == 0
        assert its == out[0][1]
        assert np.array_equal(du, out[0][0])
    c.pcg_form(1)


@pytest.mark.parametrize("form", [1, 3])
@pytest.mark.parametrize("precision", [lib.MIXED, lib.FP64])
def test_single_reduction_form_is_bitwise_repeatable(precision, form):
    m = _model()
    c, R = _system(m, precision, lib.PRECOND_JACOBI)
    c.pcg_form(form)
    a = c.pcg(R, rel_tol=1e-8, max_it=20000, precond=lib.PRECOND_JACOBI)
    b = c.pcg(R, rel_tol=1e-8, max_it=20000, precond=lib.PRECOND_JACOBI)
    assert a[3] == 0 and b[3] == 0
    assert a[1] == b[1]
    assert np.array_equal(a[0], b[0])
    c.pcg_form(1)


@pytest.mark.parametrize("precision", [lib.MIXED, lib.FP64])
def test_push_storage_follows_every_assembly(precision):
    """The push storage's values are copied from each new assembly: after a
    second tangent at another state (and a form switch in between), form 3
    solves the new system as form 1 does."""
    m = _model()
    c, R = _system(m, precision, lib.PRECOND_BLOCK_JACOBI)
    c.pcg_form(3)
    c.pcg(R, rel_tol=1e-8, max_it=20000, precond=lib.PRECOND_BLOCK_JACOBI)
    u = c.get_u()
    c.set_u(u * 1.5)
    R2, _ = c.residual()
    c.tangent(precision)
    sol = {}
    for form in (1, 3):
        c.pcg_form(form)
        du, its, rr, rc = c.pcg(R2, rel_tol=1e-9, max_it=20000, precond=lib.PRECOND_BLOCK_JACOBI)
        assert rc == 0
        sol[form] = (du, its)
    scale = np.abs(sol[1][0]).max()
    bound = 2e-4 if precision == lib.MIXED else 1e-6
    assert np.abs(sol[3][0] - sol[1][0]).max() <= bound * scale
    assert abs(sol[3][1] - sol[1][1]) <= max(3, 0.05 * sol[1][1])
    c.pcg_form(1)


@pytest.mark.parametrize("precision", [lib.MIXED, lib.FP64])
def test_symmetric_format_after_a_push_only_tangent(precision):
    """A tangent assembled for the push storage alone (upper blocks; the full
    storage is assembled when something reads it), then the symmetric stream
    format switched on: its values come from this tangent -- the full storage
    still holds an older one -- so its solve equals form 1's."""
    m = _model()
    c, R = _system(m, precision, lib.PRECOND_JACOBI)  # full storage at the first state
    c.set_u(c.get_u() * 1.5)
    R2, _ = c.residual()
    c.pcg_form(3)
    c.tangent(precision)  # upper blocks into the push storage only
    c.spmv_symmetric(1, 512)
    assert c.product_kernel() == "pcg_spmv_sym_kernel"
    tol = 1e-9
    du_s, its_s, rr, rc = c.pcg(R2, rel_tol=tol, max_it=20000, precond=lib.PRECOND_JACOBI)
    assert rc == 0
    c.spmv_symmetric(0, 512)
    c.pcg_form(1)
    du_f, its_f, rr, rc = c.pcg(R2, rel_tol=tol, max_it=20000, precond=lib.PRECOND_JACOBI)
    assert rc == 0
    bound = 2e-4 if precision == lib.MIXED else 1e-6
    assert np.abs(du_s - du_f).max() <= bound * np.abs(du_f).max()
    assert abs(its_s - its_f) <= max(3, 0.05 * its_f)
    c.pcg_form(-1)


def test_l2_priorities_leave_the_iterates_bitwise_unchanged():
    m = _model(16)
    c, R = _system(m, lib.MIXED, lib.PRECOND_JACOBI)
    nbytes = c.block_nnz * 40
    ref = None
    for form in (1, 0, 3):
        c.pcg_form(form)
        ref = None
        for keep in (-1, 0, 1 << 20, nbytes // 3, 4 * nbytes):
            c.spmv_l2_keep(keep)
            du, its, rr, rc = c.pcg(R, rel_tol=1e-8, max_it=20000, precond=lib.PRECOND_JACOBI)
            assert rc == 0
            if ref is None:
                ref = (du, its)
            assert its == ref[1], (form, keep)
            assert np.array_equal(du, ref[0]), (form, keep)
    c.spmv_l2_keep(16 << 20)
    c.pcg_form(1)


def test_single_reduction_form_converges_within_the_first_chunk():
    # a loose tolerance ends the solve inside the first 16-iteration replay:
    # the scalars handed from one vector kernel to the next carry the flag
    m = _model(6)
    c, R = _system(m, lib.MIXED, lib.PRECOND_BLOCK_JACOBI)
    c.pcg_form(1)
    du, its, rr, rc = c.pcg(R, rel_tol=0.3, max_it=20000, precond=lib.PRECOND_BLOCK_JACOBI)
    assert rc == 0
    assert 1 <= its < 16
    assert rr <= 0.3
    c.pcg_form(0)
    du0, its0, rr0, rc0 = c.pcg(R, rel_tol=0.3, max_it=20000, precond=lib.PRECOND_BLOCK_JACOBI)
    assert rc0 == 0 and abs(its0 - its) <= 1


def _iso_C(E=1.0, nu=0.3):
    mu = 0.5 * E / (1.0 + nu)
    lam = 2.0 * mu * nu / (1.0 - 2.0 * nu)
    C = np.zeros((6, 6))
    C[:3, :3] = lam
    C[np.arange(3), np.arange(3)] += 2.0 * mu
    C[np.arange(3, 6), np.arange(3, 6)] = mu
    return C


def _small_strain_system(C, precision):
    mesh = BoxMesh(8, 8, 8, jitter=0.2, seed=7)
    m = SolidModel(mesh.X, mesh.conn, "small_strain", {"kind": "ss_hookean", "C": C.reshape(36)})
    for node in mesh.face_nodes(2, 0):
        for d in range(3):
            m.add_kbc(node, d)
    for node in mesh.face_nodes(2, 1):
        m.add_kbc(node, 2, -0.01, True)
    m.set_schedule([(0.0, 1.0)])
    m.setup()
    c = m.ctx
    u = np.zeros((mesh.nnd, 3))
    u[mesh.face_nodes(2, 1), 2] = -0.01
    c.set_u(u)
    c.set_iteration(-1)
    R, _ = c.residual()
    c.tangent(precision)
    return c, R


@pytest.mark.parametrize("form", [0, 1, 3])
@pytest.mark.parametrize("precision", [lib.MIXED, lib.FP64])
def test_iteration_limit_is_reported_not_raised(form, precision):
    c, R = _small_strain_system(_iso_C(), precision)
    c.pcg_form(form)
    du, its, rr, rc = c.pcg(R, rel_tol=1e-14, max_it=5, precond=lib.PRECOND_JACOBI)
    assert rc == -6  # TG_ERR_NOT_CONVERGED
    assert its == 5
    assert 0.0 < rr < 1.0
    c.pcg_form(1)


@pytest.mark.parametrize("form", [0, 1, 3])
@pytest.mark.parametrize("precision", [lib.MIXED, lib.FP64])
def test_indefinite_operator_breaks_down(form, precision):
    # a negative-definite stiffness: the first curvature p.Ap (u.Au in the
    # single-reduction form) is negative, and both forms stop with it
    c, R = _small_strain_system(-_iso_C(), precision)
    c.pcg_form(form)
    with pytest.raises(lib.TahoeError) as ei:
        c.pcg(R, rel_tol=1e-8, max_it=100, precond=lib.PRECOND_JACOBI)
    assert ei.value.code == -5  # TG_ERR_NAN: breakdown
    assert "indefinite" in str(ei.value)
    c.pcg_form(1)


def test_default_form_follows_mesh_size():
    """The default (-1) runs the push storage on meshes of at least a million
    block nonzeros and the full storage below; an explicit form holds on any
    mesh."""
    small = _model(6)
    c = small.ctx
    assert c.effective_form() == 1
    c.pcg_form(3)
    assert c.effective_form() == 3
    c.pcg_form(2)
    assert c.effective_form() == 2
    c.pcg_form(-1)
    assert c.effective_form() == 1
    big = _model(40)  # 68,921 nodes, about 1.7 M block nonzeros
    assert big.ctx.block_nnz >= 1_000_000
    assert big.ctx.effective_form() == 3
    assert big.ctx.product_kernel() == "pcg_cg_push_kernel"
