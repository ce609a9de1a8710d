"""The mixed form's residual in double-float arithmetic, through the C ABI.

tg_form_residual_precision(TG_MIXED) forms the element forces of a
total-Lagrangian Simo group in pairs of floats (48 significant bits): the
residual must equal the oracle's FP64 residual (TotalLagrangianT::FormKd with
SimoIso3D) to 1e-11 of its largest entry -- the FP64 path reaches 1e-12, a
float residual would be near 1e-6.  Groups it does not cover (other
formulations and materials) keep the FP64 kernel and equal tg_form_residual
bitwise.  The mixed Newton driver, which uses it, converges to solutions whose
FP64 residual meets the same tolerance.
"""
import numpy as np
import pytest

from tahoe_gb300 import lib
from tahoe_gb300.meshgen import BoxMesh
from tahoe_gb300.model import SolidModel
from tests.helpers import cube_case, oracle_for, rel_err

pytestmark = pytest.mark.gpu

SIMO = {"kind": "fs_simo", "mu": 1.0, "kappa": 10.0}
SIMO_MPA = {"kind": "fs_simo", "mu": 76.9e3, "kappa": 166.7e3}  # steel-like moduli in MPa
STV = {"kind": "fs_stvenant", "E": 100.0, "nu": 0.25}
HOOKE = {"kind": "ss_hookean", "E": 200e3, "nu": 0.3}

FF_TOL = 1e-11


def _model(mesh, formulation, material, fixed, blocks=None):
    m = SolidModel(mesh.X, mesh.conn, formulation, material, blocks=blocks)
    for node, d in fixed:
        m.add_kbc(node, d, 0.0, False)
    m.setup()
    return m


def _u(mesh, fixed, scale, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-scale, scale, size=(mesh.nnd, 3))
    for node, d in fixed:
        u[node, d] = 0.0
    return u


@pytest.mark.parametrize("material", [SIMO, SIMO_MPA])
@pytest.mark.parametrize("scale", [1e-3, 0.01, 0.03])
def test_double_float_residual_matches_oracle(material, scale):
    mesh, fixed = cube_case(5, jitter=0.2, seed=4)
    o = oracle_for(mesh, "total_lagrangian", material, fixed)
    g = _model(mesh, "total_lagrangian", material, fixed)
    u = _u(mesh, fixed, scale, 11)
    g.ctx.set_u(u)
    R, nrm = g.ctx.residual(precision=lib.MIXED)
    Ro, _, _ = o.form(u, 1.0, 0)
    err = rel_err(R, Ro)
    assert err < FF_TOL, err
    assert abs(nrm - np.linalg.norm(Ro)) < FF_TOL * np.linalg.norm(Ro)
    R64, _ = g.ctx.residual()
    assert rel_err(R, R64) < FF_TOL


def test_double_float_residual_per_material_block():
    mesh, fixed = cube_case(4, jitter=0.15, seed=6)
    blocks = (np.arange(mesh.nel) % 3 == 0).astype(np.int32)
    mats = [SIMO, {"kind": "fs_simo", "mu": 3.0, "kappa": 40.0}]
    o = oracle_for(mesh, "total_lagrangian", mats, fixed, blocks=blocks)
    g = _model(mesh, "total_lagrangian", mats, fixed, blocks=blocks)
    u = _u(mesh, fixed, 0.05, 3)
    g.ctx.set_u(u)
    R, _ = g.ctx.residual(precision=lib.MIXED)
    Ro, _, _ = o.form(u, 1.0, 0)
    assert rel_err(R, Ro) < FF_TOL


def test_double_float_residual_is_bitwise_repeatable():
    mesh, fixed = cube_case(6, jitter=0.2, seed=1)
    g = _model(mesh, "total_lagrangian", SIMO, fixed)
    g.ctx.set_u(_u(mesh, fixed, 0.05, 5))
    a, na = g.ctx.residual(precision=lib.MIXED)
    b, nb = g.ctx.residual(precision=lib.MIXED)
    assert np.array_equal(a, b) and na == nb


@pytest.mark.parametrize("formulation,material", [("total_lagrangian", STV), ("small_strain", HOOKE),
                                                  ("updated_lagrangian", SIMO)])
def test_groups_outside_the_double_float_kernel_keep_fp64(formulation, material):
    mesh, fixed = cube_case(4, jitter=0.2, seed=2)
    g = _model(mesh, formulation, material, fixed)
    g.ctx.set_u(_u(mesh, fixed, 1e-3 if formulation == "small_strain" else 0.05, 8))
    a, na = g.ctx.residual(precision=lib.MIXED)
    b, nb = g.ctx.residual()
    assert np.array_equal(a, b) and na == nb


def test_inverted_element_reports_bad_jacobian_in_double_float():
    mesh = BoxMesh(2, 2, 2)
    X = mesh.X.copy()
    centre = np.nonzero((mesh.ijk == 1).all(axis=1))[0][0]
    X[centre, 2] = 5.0  # pushes the centre node through the top: inverted elements
    g = SolidModel(X, mesh.conn, "total_lagrangian", SIMO)
    g.add_kbc(0, 0)
    g.setup()
    with pytest.raises(lib.TahoeError) as ei:
        g.ctx.residual(precision=lib.MIXED)
    assert ei.value.code == -4
    # the context stays usable after the error
    g.ctx.set_u(np.zeros((mesh.nnd, 3)))
    with pytest.raises(lib.TahoeError):
        g.ctx.residual()


def test_mixed_newton_converges_on_the_fp64_residual():
    """A compression step of the C2 physics (jittered 8^3 block, Simo): the
    mixed driver's Newton test runs on the double-float residual; the FP64
    residual of its converged state meets the same relative tolerance, and
    the displacements equal the FP64 driver's to 1e-6."""
    mesh = BoxMesh(8, 8, 8, jitter=0.2, seed=0)
    bottom, top = mesh.face_nodes(2, 0), mesh.face_nodes(2, 1)
    out = {}
    for prec in (lib.MIXED, lib.FP64):
        g = SolidModel(mesh.X, mesh.conn, "total_lagrangian", SIMO)
        g.set_schedule([(0.0, 0.0), (1.0, 1.0)])
        for n in bottom:
            for d in range(3):
                g.add_kbc(n, d, 0.0, False)
        for n in top:
            g.add_kbc(n, 2, -0.05, True)
        hist, reps = g.run(1, 1.0, rel_tol=1e-10, abs_tol=0.0, max_iterations=15, precision=prec,
                           lin_rel_tol=1e-6, predictor=True)
        rep = reps[0][-1] if isinstance(reps[0], list) else reps[0]
        assert rep.error <= 1e-10 * rep.error0
        _, n64 = g.ctx.residual()
        assert n64 <= 1e-9 * rep.error0, (n64, rep.error0)
        out[prec] = np.asarray(hist[-1])
    assert rel_err(out[lib.MIXED], out[lib.FP64]) < 1e-6
