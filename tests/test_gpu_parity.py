"""Parity of the CUDA path (through the C ABI) with the CPU oracle and the
reference's golden outputs.

Tolerances (FP64 path): element matrices/forces 1e-12 relative to the largest
entry, assembled values 1e-12, converged displacements 1e-9 against the
oracle's direct solve.  Integer work (equations, CSR pattern, J2 active set)
is compared bit-exactly.  The mixed form (FP32 tangent + inner PCG, FP64
residual) must reach 1e-6 relative displacement error against FP64.
"""
import numpy as np
import pytest

from oracle.pyoracle import OracleModel
from tahoe_gb300 import lib, workloads
from tahoe_gb300.meshgen import BoxMesh
from tahoe_gb300.model import SolidModel, model_from_fixture
from tests.helpers import (GOLDEN_NAMES, cube_case, golden_displacements, load_fixture, msr_to_upper_csr,
                           oracle_for, rel_err)

pytestmark = pytest.mark.gpu

HOOKE = {"kind": "ss_hookean", "E": 200e3, "nu": 0.3}
SIMO = {"kind": "fs_simo", "mu": 1.0, "kappa": 10.0}
STV = {"kind": "fs_stvenant", "E": 100.0, "nu": 0.25}
J2 = {"kind": "ss_j2", "E": 200e3, "nu": 0.3, "a": 1000.0, "b": 250.0}


def gpu_model(mesh, formulation, material, fixed, blocks=None, strain_displacement="standard"):
    m = SolidModel(mesh.X, mesh.conn, formulation, material, blocks=blocks, strain_displacement=strain_displacement)
    for node, d in fixed:
        m.add_kbc(node, d, 0.0, False)
    m.setup()
    return m


def random_u(nnd, scale, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-scale, scale, size=(nnd, 3))


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_golden_decks_on_gpu(name):
    """Displacements and the nodal output stresses (extrapolated, averaged;
    written before the step is closed) against the reference's .run files."""
    fx = load_fixture(name)
    m = model_from_fixture(fx)
    sv = fx["solver"]
    stress, matout = {}, {}

    def on_step(step, ctx):
        stress[step - 1] = ctx.nodal_stress()
        matout[step - 1] = ctx.nodal_material_output()

    hist, reps = m.run(fx["nsteps"], fx["dt"], rel_tol=sv["rel_tol"], abs_tol=sv["abs_tol"],
                       max_iterations=sv["max_its"], div_tol=sv["div_tol"], precision=lib.FP64,
                       lin_rel_tol=1e-14, lin_max_it=5000, on_step=on_step)
    for step, ref in golden_displacements(fx).items():
        assert rel_err(hist[step], ref) < 1e-9, (name, step)
    for o in fx["outputs"]:
        step = int(round(o["time"] / fx["dt"])) - 1
        ref = np.array(o["rows"])[:, 3:9]
        assert rel_err(stress[step], ref) < 1e-9, (name, step)
        if "alpha" in o["labels"]:
            L = o["labels"]
            mref = np.array(o["rows"])[:, L.index("alpha"):L.index("press") + 1]
            assert rel_err(matout[step], mref) < 1e-9, (name, step)


@pytest.mark.parametrize("jitter", [0.0, 0.2])
def test_equations_and_pattern_bit_exact(jitter):
    mesh, fixed = cube_case(5, jitter=jitter, seed=7)
    o = oracle_for(mesh, "small_strain", HOOKE, fixed)
    g = gpu_model(mesh, "small_strain", HOOKE, fixed)
    eq_o, neq = o.equations()
    assert np.array_equal(g.eqnos, eq_o)
    assert g.ctx.neq == neq
    bindx = o.msr_pattern(upper=True)
    rp, ci = g.ctx.pattern(upper_only=True)
    rows = msr_to_upper_csr(bindx, neq)
    assert rp[-1] == sum(len(r) for r in rows)
    for r in range(neq):
        assert np.array_equal(ci[rp[r]:rp[r + 1]], rows[r]), r
    # full pattern is the symmetric closure
    bfull = o.msr_pattern(upper=False)
    rpf, cif = g.ctx.pattern(upper_only=False)
    for r in range(0, neq, 7):
        want = np.sort(np.concatenate([[r], bfull[bfull[r]:bfull[r + 1]]]))
        assert np.array_equal(cif[rpf[r]:rpf[r + 1]], want)


@pytest.mark.parametrize("formulation,material,scale", [
    ("small_strain", HOOKE, 1e-3), ("total_lagrangian", SIMO, 0.05), ("total_lagrangian", STV, 0.05),
    ("updated_lagrangian", SIMO, 0.05), ("updated_lagrangian", STV, 0.05)])
def test_element_matrices_match_oracle(formulation, material, scale):
    mesh, fixed = cube_case(3, jitter=0.2, seed=11)
    o = oracle_for(mesh, formulation, material, fixed)
    g = gpu_model(mesh, formulation, material, fixed)
    u = random_u(mesh.nnd, scale, 5)
    g.ctx.set_u(u)
    K, f = g.ctx.element_dump(0, mesh.nel)
    for e in range(mesh.nel):
        Ko, fo = o.element(e, u)
        assert rel_err(K[e], Ko) < 1e-12, e
        assert rel_err(f[e], fo) < 1e-12, e


def test_bbar_element_matrices_and_assembly_match_oracle():
    """B-bar small strain (mean dilatation), nearly incompressible Hooke and
    J2 past yield: element matrices/forces and the assembled system against
    the oracle's explicit B-bar matrices."""
    nearly_incomp = {"kind": "ss_hookean", "E": 100.0, "nu": 0.49}
    mesh, fixed = cube_case(3, jitter=0.2, seed=11)
    for mat, scale in ((nearly_incomp, 1e-3), (J2, 4e-3)):
        o = OracleModel(mesh.X, mesh.conn, "small_strain", [mat], bbar=True)
        for node, d in fixed:
            o.add_kbc(node, d, 0.0, False)
        g = gpu_model(mesh, "small_strain", mat, fixed, strain_displacement="B-bar")
        u = random_u(mesh.nnd, scale, 5)
        for node, d in fixed:
            u[node, d] = 0.0
        g.ctx.set_u(u)
        g.ctx.set_iteration(0)
        R, nrm = g.ctx.residual()
        Ro, val, bindx = o.form(u, 1.0, 0)
        # tangents from the state the residual pass left (both sides)
        Ro, val, bindx = o.form(u, 1.0, 0)
        assert rel_err(R, Ro) < 1e-12
        K, f = g.ctx.element_dump(0, mesh.nel)
        for e in range(mesh.nel):
            Ko, fo = o.element(e, u, 0)
            assert rel_err(K[e], Ko) < 1e-11, e
            assert rel_err(f[e], fo) < 1e-12, e
        for prec, tol in ((lib.FP64, 1e-12), (lib.MIXED, 2e-6)):
            g.ctx.tangent(prec)
            rp, ci, v = g.ctx.tangent_csr(upper_only=True)
            vo = np.concatenate([[val[r]] + list(val[bindx[r]:bindx[r + 1]]) for r in range(o.neq)])
            assert rel_err(v, vo) < tol, prec


@pytest.mark.parametrize("formulation,material,scale", [
    ("small_strain", HOOKE, 1e-3), ("total_lagrangian", SIMO, 0.05), ("updated_lagrangian", SIMO, 0.05)])
@pytest.mark.parametrize("precision", [lib.FP64, lib.MIXED])
def test_assembled_tangent_and_residual(formulation, material, scale, precision):
    mesh, fixed = cube_case(4, jitter=0.2, seed=2)
    o = oracle_for(mesh, formulation, material, fixed)
    g = gpu_model(mesh, formulation, material, fixed)
    u = random_u(mesh.nnd, scale, 9)
    for node, d in fixed:
        u[node, d] = 0.0
    g.ctx.set_u(u)
    R, nrm = g.ctx.residual()
    Ro, val, bindx = o.form(u, 1.0, 0)
    assert rel_err(R, Ro) < 1e-12
    assert abs(nrm - np.linalg.norm(Ro)) < 1e-12 * np.linalg.norm(Ro)
    g.ctx.tangent(precision)
    rp, ci, v = g.ctx.tangent_csr(upper_only=True)
    n = o.neq
    want = np.zeros(len(ci))
    for r in range(n):
        want[rp[r]] = val[r]
        want[rp[r] + 1:rp[r + 1]] = val[bindx[r]:bindx[r + 1]]
    tol = 1e-12 if precision == lib.FP64 else 2e-6
    assert rel_err(v, want) < tol


def test_updated_lagrangian_newton_iterates_match_oracle():
    """The updated-Lagrangian element inside Newton: every iteration's
    residual norm of a finite compression step (large-strain St.Venant, a
    jittered 4^3 block) against the oracle's UL restatement, and the same
    iterates as the total-Lagrangian element (one weak form, two
    evaluations)."""
    mesh = BoxMesh(4, 4, 4, jitter=0.2, seed=5)
    bottom, top = mesh.face_nodes(2, 0), mesh.face_nodes(2, 1)
    norms = {}
    for form in ("updated_lagrangian", "total_lagrangian"):
        o = oracle_for(mesh, form, STV, [])
        g = SolidModel(mesh.X, mesh.conn, form, STV)
        for m in (o, g):
            for n in bottom:
                for d in range(3):
                    m.add_kbc(n, d, 0.0, False)
            for n in top:
                m.add_kbc(n, 2, 0.0, False)
        g.setup()
        eq, _ = o.equations()
        u = np.zeros((mesh.nnd, 3))
        u[top, 2] = -0.01
        o.set_u(u)
        g.ctx.set_u(u)
        g.ctx.set_iteration(-1)
        _, n_g = g.ctx.residual(want_vector=True)
        seq = []
        for it in range(4):
            n_o = o.residual(1.0, it - 1)
            # relative to the step's first residual (late norms sit at round-off)
            assert abs(n_g - n_o) <= 1e-12 * max(seq[0] if seq else n_o, 1e-300), (form, it)
            seq.append(n_g)
            n_g, _ = g.ctx.newton_iteration(precision=lib.FP64, lin_rel_tol=1e-13, lin_max_it=20000)
            o.newton_iteration(1.0, it - 1, 1e-13)
            assert rel_err(g.ctx.get_u(), o.get_u()) < 1e-10, (form, it)
        norms[form] = seq
        g.ctx.close()
    nu, nt = np.array(norms["updated_lagrangian"]), np.array(norms["total_lagrangian"])
    assert np.abs(nu - nt).max() <= 1e-10 * nt[0]


def test_assembly_and_residual_bitwise_repeatable():
    mesh, fixed = cube_case(6, jitter=0.2, seed=4)
    g = gpu_model(mesh, "total_lagrangian", SIMO, fixed)
    g.ctx.set_u(random_u(mesh.nnd, 0.02, 1))
    outs = []
    for _ in range(2):
        R, _ = g.ctx.residual()
        g.ctx.tangent(lib.MIXED)
        _, _, v = g.ctx.tangent_csr(False)
        outs.append((R.copy(), v.copy()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("tile_blocks", [512, 32])
def test_symmetric_product_equals_full_storage(tile_blocks):
    """The single-vector product streaming the symmetric format (upper blocks,
    lower blocks as transposes, output masked at prescribed dofs; all three
    launch shapes) gives the PCG solution of the full block storage: FP64 to
    1e-11, the mixed form to 1e-5, the same iteration count within two; a
    small tile size spreads the rows over many tiles (transposed blocks from
    other tiles)."""
    mesh, fixed = cube_case(6, jitter=0.2, seed=4)
    g = gpu_model(mesh, "total_lagrangian", SIMO, fixed)
    u = random_u(mesh.nnd, 0.002, 3)  # small enough for a positive definite tangent
    for node, d in fixed:
        u[node, d] = 0.0
    g.ctx.set_u(u)
    R, _ = g.ctx.residual()
    for prec, tol, lt in ((lib.FP64, 1e-11, 1e-12), (lib.MIXED, 1e-5, 1e-6)):
        g.ctx.tangent(prec)
        res = {}
        for on in (0, 1, 2, 3):
            g.ctx.spmv_symmetric(on, tile_blocks)
            for pc in (lib.PRECOND_JACOBI, lib.PRECOND_BLOCK_JACOBI):
                du, its, rr, rc = g.ctx.pcg(R, rel_tol=lt, max_it=20000, precond=pc)
                assert rc == 0 and rr < lt
                res[on, pc] = (du, its)
            assert g.ctx.time_kernel(0, 2) > 0.0
        for on in (1, 2, 3):
            for pc in (lib.PRECOND_JACOBI, lib.PRECOND_BLOCK_JACOBI):
                assert rel_err(res[on, pc][0], res[0, pc][0]) < tol, (prec, on, pc)
                assert abs(res[on, pc][1] - res[0, pc][1]) <= 2, (prec, on, pc)
    g.ctx.spmv_symmetric(0, 512)


def test_pcg_solves_oracle_system():
    mesh, fixed = cube_case(6, jitter=0.1, seed=8)
    o = oracle_for(mesh, "small_strain", HOOKE, fixed)
    g = gpu_model(mesh, "small_strain", HOOKE, fixed)
    rng = np.random.default_rng(0)
    b = rng.standard_normal(o.neq)
    u0 = np.zeros((mesh.nnd, 3))
    _, val, _ = o.form(u0, 1.0, 0)
    x_o, it_o, _ = o.pcg(val, b, 1e-13, 20000)
    g.ctx.set_u(u0)
    g.ctx.tangent(lib.FP64)
    for pc in (lib.PRECOND_JACOBI, lib.PRECOND_BLOCK_JACOBI):
        du, its, rr, rc = g.ctx.pcg(b, rel_tol=1e-13, max_it=20000, precond=pc)
        assert rc == 0 and rr < 1e-13
        assert rel_err(du, x_o) < 1e-9


def test_c1_full_size_matches_oracle_and_mixed_within_1e6():
    """configuration 1 at its full size (16^3 hex8, 14,739 dofs, traction
    load, one static step): FP64 against the oracle's Newton with Jacobi CG to
    1e-14 at 1e-9, mixed against FP64 at 1e-6"""
    mesh, o, _ = workloads.c1(add=lambda X, conn, form, mat: OracleModel(X, conn, form, [mat], threads=8))
    st, uh, its = o.run(1, 1.0, 1e-12, 1e-14, 5, 10.0, 1, 1e-14)
    assert st == 0
    res = {}
    for prec in (lib.FP64, lib.MIXED):
        _, g, _ = workloads.c1()
        hist, reps = g.run(1, 1.0, rel_tol=1e-12, abs_tol=1e-14, max_iterations=12, precision=prec,
                           lin_rel_tol=1e-6 if prec == lib.MIXED else 1e-13, lin_max_it=20000)
        res[prec] = hist[-1]
        g.ctx.close()
    assert rel_err(res[lib.FP64], uh[0]) < 1e-9
    assert rel_err(res[lib.MIXED], res[lib.FP64]) < 1e-6


def test_context_pattern_at_c2_size_equals_host_build():
    """the pattern a context builds for the full C2 mesh (tg_pattern_build)
    is the host build's (tg_pattern_build_host, checked against the oracle at
    this size in tests/test_pattern_cpu.py)"""
    mesh, g, _ = workloads.c2()
    g.setup()
    for upper in (True, False):
        rp, ci = g.ctx.pattern(upper_only=upper)
        rph, cih = lib.pattern_host(mesh.conn, g.eqnos, mesh.nnd, upper_only=upper)
        assert np.array_equal(rp, rph) and np.array_equal(ci, cih)
    g.ctx.close()


def test_c2_style_neo_hookean_steps_match_oracle():
    """configuration 2 physics at 4^3 with jitter: 3 compression steps"""
    mesh = BoxMesh(4, 4, 4, jitter=0.2, seed=0)
    bottom, top = mesh.face_nodes(2, 0), mesh.face_nodes(2, 1)
    o = oracle_for(mesh, "total_lagrangian", SIMO, [])
    g = SolidModel(mesh.X, mesh.conn, "total_lagrangian", SIMO)
    for m in (o, g):
        m.set_schedule([(0.0, 0.0), (3.0, 1.0)])
        for n in bottom:
            for d in range(3):
                m.add_kbc(n, d, 0.0, False)
        for n in top:
            m.add_kbc(n, 2, -0.03, True)
    st, uh, its = o.run(3, 1.0, 1e-12, 1e-14, 10, 10.0, 0)
    assert st == 0
    for prec, tol in ((lib.FP64, 1e-9), (lib.MIXED, 1e-6)):
        gg = SolidModel(mesh.X, mesh.conn, "total_lagrangian", SIMO)
        gg.schedule, gg.kbc = g.schedule, g.kbc
        # the GPU path applies each prescribed increment through the linearised
        # predictor; the converged steps equal the oracle's (reference semantics)
        hist, reps = gg.run(3, 1.0, rel_tol=1e-12, abs_tol=1e-14, max_iterations=15, precision=prec,
                            lin_rel_tol=1e-8 if prec == lib.MIXED else 1e-13, predictor=True)
        assert rel_err(hist, uh) < tol, prec


def test_j2_active_set_bit_exact_over_cyclic_steps():
    """configuration 3 physics on a small clamped plate: 8 cyclic steps"""
    mesh = BoxMesh(6, 4, 2, lx=3.0, ly=2.0, lz=1.0, jitter=0.15, seed=3)
    x0, x1 = mesh.face_nodes(0, 0), mesh.face_nodes(0, 1)
    o = oracle_for(mesh, "small_strain", J2, [])
    g = SolidModel(mesh.X, mesh.conn, "small_strain", J2)
    sched = [(0.0, 0.0), (2.0, 1.0), (6.0, -1.0), (8.0, 0.0)]
    for m in (o, g):
        m.set_schedule(sched)
        for n in x0:
            for d in range(3):
                m.add_kbc(n, d, 0.0, False)
        for n in x1:
            m.add_kbc(n, 0, 0.005 * 3.0, True)
            m.add_kbc(n, 1, 0.0, False)
            m.add_kbc(n, 2, 0.0, False)
    flags_g = []
    st, uh_o, its_o = o.run(8, 1.0, 1e-12, 1e-10, 15, 10.0, 0)
    assert st == 0
    fo, ao, eo = o.j2_state()

    def on_step(step, ctx):
        flags_g.append(ctx.active_set().copy())

    hist, reps = g.run(8, 1.0, rel_tol=1e-12, abs_tol=1e-10, max_iterations=15, precision=lib.FP64,
                       lin_rel_tol=1e-14, lin_max_it=20000, on_step=on_step)
    fg = g.ctx.active_set()
    ag, eg = g.ctx.j2_state()
    assert np.array_equal(fg, fo)
    assert rel_err(ag, ao) < 1e-8
    assert rel_err(hist, uh_o) < 1e-8
    assert (fo == 0).sum() + (fo == 3).sum() > 0  # some points yielded


def test_j2_plate_step_cuts_match_oracle():
    """C3-style J2 plate (16 x 16 x 8) with a load step large enough that
    Newton fails: both sides cut the step (TimeManagerT semantics) the same
    number of times, the displacements at the original step ends agree, and
    the active set is bit-exact; the mixed form takes the same cuts."""
    mesh, o, _ = workloads.c3(nx=16, ny=16, nz=8, nsteps=40,
                              add=lambda X, conn, form, mat: OracleModel(X, conn, form, [mat], threads=8))
    st, uh_o, its_o, cuts_o = o.run_cuts(3, 2.0, 1e-8, 1e-10, 25, 1e3, 1, 1e-12, max_cuts=4)
    assert st == 0 and cuts_o >= 1
    fo, ao, eo = o.j2_state()
    res = {}
    for prec in (lib.FP64, lib.MIXED):
        _, g, _ = workloads.c3(nx=16, ny=16, nz=8, nsteps=40)
        hist, reps = g.run(3, 2.0, rel_tol=1e-8, abs_tol=1e-10, max_iterations=25, div_tol=1e3, precision=prec,
                           lin_rel_tol=1e-12 if prec == lib.FP64 else 1e-6, lin_max_it=50000, max_step_cuts=4)
        res[prec] = (hist, g.step_cuts, g.ctx.active_set())
    hist, cuts, fg = res[lib.FP64]
    assert cuts == cuts_o
    assert np.array_equal(fg, fo)
    assert rel_err(hist, uh_o) < 1e-7
    hm, cm, fm = res[lib.MIXED]
    assert cm == cuts_o and np.array_equal(fm, fg)
    assert rel_err(hm, hist) < 1e-6


def test_inverted_element_reports_bad_jacobian():
    mesh = BoxMesh(2, 2, 2)
    X = mesh.X.copy()
    centre = np.nonzero((mesh.ijk == 1).all(axis=1))[0][0]
    X[centre, 2] = 5.0  # pushes the centre node through the top: inverted elements
    g = SolidModel(X, mesh.conn, "small_strain", HOOKE)
    g.add_kbc(0, 0)
    g.setup()
    with pytest.raises(lib.TahoeError) as ei:
        g.ctx.residual()
    assert ei.value.code == -4
    # the context stays usable after the error
    g.ctx.set_u(np.zeros((mesh.nnd, 3)))
    with pytest.raises(lib.TahoeError):
        g.ctx.tangent(lib.FP64)


def test_kernels_launched_and_counted():
    mesh, fixed = cube_case(3)
    g = gpu_model(mesh, "small_strain", HOOKE, fixed)
    n0 = g.ctx.launches
    g.ctx.residual()
    g.ctx.tangent(lib.MIXED)
    assert g.ctx.launches - n0 >= 4
