"""The CPU oracle against the reference's own golden outputs (regression-suite
.run files extracted into tests/golden).  Pins the oracle before the CUDA path
is tested against it."""
import numpy as np
import pytest

from oracle.pyoracle import J2_PLASTIC, J2_RESET, model_from_fixture
from tests.helpers import (GOLDEN_NAMES, ORACLE_EXTRA_NAMES, SOLVER_CHOICE_NAMES, golden_displacements, load_fixture,
                           rel_err)


@pytest.mark.parametrize("name", GOLDEN_NAMES + ORACLE_EXTRA_NAMES)
def test_oracle_reproduces_golden_displacements(name):
    fx = load_fixture(name)
    m = model_from_fixture(fx)
    sv = fx["solver"]
    status, uh, its = m.run(fx["nsteps"], fx["dt"], sv["rel_tol"], sv["abs_tol"], sv["max_its"], sv["div_tol"], 0)
    assert status == 0
    for step, ref in golden_displacements(fx).items():
        # golden files print 13 significant digits
        assert rel_err(uh[step], ref) < 1e-11, (name, step)


@pytest.mark.parametrize("name", GOLDEN_NAMES + ORACLE_EXTRA_NAMES)
def test_oracle_nodal_stress_matches_golden(name):
    """Output stresses (integration-point Cauchy stress extrapolated to the
    nodes and averaged over elements) against the .run files' s11..s12."""
    fx = load_fixture(name)
    m = model_from_fixture(fx)
    sv = fx["solver"]
    status, uh, its, cuts, sh = m.run_cuts(fx["nsteps"], fx["dt"], sv["rel_tol"], sv["abs_tol"], sv["max_its"],
                                           sv["div_tol"], 0, want_stress=True)
    assert status == 0 and cuts == 0
    for o in fx["outputs"]:
        step = int(round(o["time"] / fx["dt"])) - 1
        ref = np.array(o["rows"])[:, o["labels"].index("s11"):o["labels"].index("s12") + 1]
        assert rel_err(sh[step], ref) < 1e-11, (name, step)


def test_oracle_j2_material_output_matches_golden():
    """alpha, von Mises stress and pressure (J2SSKStV::ComputeOutput),
    extrapolated and averaged, against the J2 deck's .run columns."""
    fx = load_fixture("mat08_j2_cube")
    m = model_from_fixture(fx)
    sv = fx["solver"]
    status, uh, its, cuts, sh = m.run_cuts(fx["nsteps"], fx["dt"], sv["rel_tol"], sv["abs_tol"], sv["max_its"],
                                           sv["div_tol"], 0, want_stress=True)
    assert status == 0
    for o in fx["outputs"]:
        step = int(round(o["time"] / fx["dt"])) - 1
        L = o["labels"]
        ref = np.array(o["rows"])[:, L.index("alpha"):L.index("press") + 1]
        assert rel_err(m.material_output_hist[step], ref) < 1e-11, step


def test_oracle_j2_alpha_matches_golden():
    fx = load_fixture("mat08_j2_cube")
    m = model_from_fixture(fx)
    sv = fx["solver"]
    status, uh, its = m.run(fx["nsteps"], fx["dt"], sv["rel_tol"], sv["abs_tol"], sv["max_its"], sv["div_tol"], 0)
    assert status == 0
    last = fx["outputs"][-1]
    alpha_ref = np.array(last["rows"])[:, last["labels"].index("alpha")]
    flags, alpha, _ = m.j2_state()
    # homogeneous state: every point carries the nodal value
    assert np.allclose(alpha, alpha_ref.mean(), rtol=1e-11)
    # all points yielded in the last step and were closed
    assert np.all(flags == J2_RESET)


def test_oracle_equations_skip_prescribed_node_major():
    fx = load_fixture("mat24_hookean_cube")
    m = model_from_fixture(fx)
    eq, neq = m.equations()
    flat = eq.reshape(-1)
    fixed = {(n * 3 + d) for n, d, _, _ in fx["kbc"]}
    assert neq == flat.size - len(fixed)
    active = [i for i in range(flat.size) if i not in fixed]
    assert np.array_equal(flat[active], np.arange(1, neq + 1))
    assert np.all(flat[sorted(fixed)] == -1)


def test_oracle_pcg_matches_direct_solve():
    fx = load_fixture("beam_newton_totlag")
    m = model_from_fixture(fx)
    u = np.zeros((m.nnd, 3))
    R, val, bindx = m.form(u, 1.0, 0)
    x, it, rr = m.pcg(val, R, 1e-14, 1000)
    assert it > 0
    # check against the symmetric product
    n = m.neq
    A = np.zeros((n, n))
    for r in range(n):
        A[r, r] = val[r]
        for j in range(bindx[r], bindx[r + 1]):
            A[r, bindx[j]] = A[bindx[j], r] = val[j]
    assert np.allclose(A @ x, R, rtol=0, atol=1e-12 * np.abs(R).max())


@pytest.mark.parametrize("name", SOLVER_CHOICE_NAMES)
def test_oracle_newton_reaches_the_field_of_other_solver_choices(name):
    """Decks that select nonlinear PCG (diagonal or profile matrix),
    quasi-Newton or stored shape functions: full Newton reaches the same
    displacements and output stresses, within the deck's own solver tolerance
    (rel 1e-12 on the residual; the golden files print 13 digits)."""
    fx = load_fixture(name)
    sv = fx["solver"]
    assert sv["type"] in ("nonlinear_solver", "PCG_solver") and sv["matrix"] in ("diagonal_matrix", "profile_matrix")
    m = model_from_fixture(fx)
    status, uh, its, cuts, sh = m.run_cuts(fx["nsteps"], fx["dt"], sv["rel_tol"], sv["abs_tol"], 25, sv["div_tol"], 0,
                                           want_stress=True)
    assert status == 0 and cuts == 0
    for step, ref in golden_displacements(fx).items():
        assert rel_err(uh[step], ref) < 1e-10, (name, step)
    for o in fx["outputs"]:
        step = int(round(o["time"] / fx["dt"])) - 1
        ref = np.array(o["rows"])[:, o["labels"].index("s11"):o["labels"].index("s12") + 1]
        assert rel_err(sh[step], ref) < 1e-10, (name, step)
