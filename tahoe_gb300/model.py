"""Host-side mirror of the reference's deck-level plugin surface.

A ``SolidModel`` is what a Tahoe deck with a GPU element group and the GPU
matrix/solver type describes: a hex8 element group (``small_strain`` or
``total_lagrangian``), its material blocks, kinematic/force/traction boundary
conditions with a load schedule, and a Newton solver over the device CSR
matrix with (block-)Jacobi PCG.  ``run`` is the time loop of
FEManagerT::Solve (tahoe/src/main/FEManagerT.cpp:138-262): per step it applies
the prescribed values (FieldT::InitStep, FieldT.cpp:261), sets the schedule
factor, calls the C++ Newton driver (tg_newton_solve) and closes the step
(ContinuumElementT::CloseStep).
"""
import numpy as np

from . import lib
from .meshgen import equations

# XML names registered by the reference factories (ElementListT.cpp:738,752;
# SSSolidMatList3DT.cpp:199-207; FSSolidMatList3DT.cpp:409-415) and what the
# GPU group runs for them.
ELEMENT_GROUPS = {
    "small_strain": lib.SMALL_STRAIN,
    "total_lagrangian": lib.TOTAL_LAGRANGIAN,
    "updated_lagrangian": lib.UPDATED_LAGRANGIAN,
}
STRAIN_DISPLACEMENT = {"standard": lib.STRAIN_STANDARD, "B-bar": lib.STRAIN_BBAR}
MATERIALS = {
    "small_strain_StVenant": lib.MAT_SS_HOOKEAN,
    "small_strain_Hookean": lib.MAT_SS_HOOKEAN,
    "small_strain_StVenant_J2": lib.MAT_SS_J2,
    "Simo_isotropic": lib.MAT_FS_SIMO,
    "large_strain_StVenant": lib.MAT_FS_STVENANT,
}
MATRIX_TYPES = {"GPU_CSR_matrix": (lib.FP64, lib.PRECOND_JACOBI),
                "GPU_CSR_matrix_mixed": (lib.MIXED, lib.PRECOND_JACOBI)}


def material_params(mat):
    """(kind, params) from a material description dict."""
    k = mat["kind"]
    if k == "ss_hookean":
        if "C" in mat:
            return lib.MAT_SS_HOOKEAN, np.asarray(mat["C"], dtype=np.float64).reshape(36)
        return lib.MAT_SS_HOOKEAN, np.array([mat["E"], mat["nu"]])
    if k == "ss_j2":
        return lib.MAT_SS_J2, np.array([mat["E"], mat["nu"], mat["a"], mat["b"], mat.get("elastic_iterations", 0)])
    if k == "fs_simo":
        return lib.MAT_FS_SIMO, np.array([mat["mu"], mat["kappa"]])
    if k == "fs_stvenant":
        return lib.MAT_FS_STVENANT, np.array([mat["E"], mat["nu"]])
    raise ValueError("unknown material kind %r" % k)


def schedule_value(pts, t):
    """PiecewiseLinearT::function (toolbox/src/C1functions/PiecewiseLinearT.cpp:179)"""
    if pts is None or len(pts) == 0:
        return 1.0
    xs = [p[0] for p in pts]
    ys = [p[1] for p in pts]
    if t <= xs[0]:
        return ys[0]
    for i in range(1, len(xs)):
        if t < xs[i]:
            return ys[i - 1] + (t - xs[i - 1]) * (ys[i] - ys[i - 1]) / (xs[i] - xs[i - 1])
    return ys[-1]


class SolidModel:
    def __init__(self, X, conn, formulation, materials, blocks=None, device=0, strain_displacement="standard"):
        self.X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
        # small_strain's strain_displacement option ("standard" | "B-bar")
        self.strain_displacement = STRAIN_DISPLACEMENT[strain_displacement]
        self.conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 8)
        self.formulation = ELEMENT_GROUPS.get(formulation, formulation)
        if isinstance(materials, dict):
            materials = [materials]
        self.materials = materials
        self.blocks = None if blocks is None else np.ascontiguousarray(blocks, dtype=np.int32)
        self.schedule = None
        self.kbc = []       # (node, dof, value, scheduled)
        self.torsions = []  # (axis, rate, point[3], nodes)
        self.forces = []    # (node, dof, value)
        self.tractions = []  # (elem, facet, t3)
        self.device = device
        self.ctx = None

    # boundary conditions -------------------------------------------------
    def set_schedule(self, pts, number=1):
        """Schedule function `number` (1-based, as the deck's schedule ids);
        schedule 1 also scales the external forces and tractions."""
        if not hasattr(self, "schedules"):
            self.schedules = {}
        self.schedules[int(number)] = [tuple(p) for p in pts]
        if int(number) == 1:
            self.schedule = self.schedules[1]

    def add_kbc(self, node, dof, value=0.0, scheduled=False):
        """Prescribed dof: fixed at 0 (scheduled False), or value times
        schedule 1 (True) or schedule n (an int n >= 1) -- KBC_CardT's fixed /
        prescribed codes."""
        n = int(scheduled) if not isinstance(scheduled, bool) else (1 if scheduled else 0)
        self.kbc.append((int(node), int(dof), float(value), n))

    def add_torsion(self, axis, rate, point, nodes):
        """Torsion boundary controller (TorsionKBCT, TorsionKBCT.cpp:39-99,
        148-180): the nodes turn rigidly about coordinate axis `axis` (0..2)
        through `point` by theta = rate * t; the two dofs across the axis are
        prescribed (their values follow the turn of each node's initial
        position), the dof along it stays free."""
        if axis not in (0, 1, 2):
            raise ValueError("torsion axis must be 0, 1 or 2")
        self.torsions.append((int(axis), float(rate), np.asarray(point, dtype=np.float64).reshape(3),
                              np.asarray(nodes, dtype=np.int64).reshape(-1)))

    def _torsion_dofs(self):
        """dof indices (node*3 + dof) the torsion controllers prescribe"""
        across = {0: (1, 2), 1: (2, 0), 2: (0, 1)}
        return [int(n) * 3 + d for (axis, _, _, nodes) in self.torsions for n in nodes for d in across[axis]]

    def _torsion_values(self, t):
        """prescribed values of _torsion_dofs() at time t: the displacement
        that carries each node's initial position through the rigid turn
        (radius vector from the axis rotated by theta; nodes on the axis stay)"""
        across = {0: (1, 2), 1: (2, 0), 2: (0, 1)}
        out = []
        for axis, rate, point, nodes in self.torsions:
            a = np.zeros(3)
            a[axis] = 1.0
            X = self.X[nodes]
            d = X - point
            r = d - np.outer(d @ a, a)
            rad = np.linalg.norm(r, axis=1)
            th = rate * t
            e1 = np.where(rad[:, None] > 1e-12, r / np.maximum(rad, 1e-300)[:, None], 0.0)
            e2 = np.cross(a, e1)
            x = (X - r) + (rad * np.cos(th))[:, None] * e1 + (rad * np.sin(th))[:, None] * e2
            u = np.where(rad[:, None] > 1e-12, x - X, 0.0)
            for k in range(len(nodes)):
                for dd in across[axis]:
                    out.append(u[k, dd])
        return np.array(out)

    def add_force(self, node, dof, value):
        self.forces.append((int(node), int(dof), float(value)))

    def add_traction(self, elem, facet, t):
        self.tractions.append((int(elem), int(facet), [float(x) for x in t]))

    def equations(self):
        idx = [n * 3 + d for (n, d, _, _) in self.kbc] + self._torsion_dofs()
        return equations(self.X.shape[0], idx)

    # set-up ----------------------------------------------------------------
    def setup(self):
        eq = self.equations()
        c = lib.Context(self.device)
        c.upload(self.X, self.conn, eq)
        c.set_formulation(self.formulation)
        c.set_strain_displacement(self.strain_displacement)
        for b, m in enumerate(self.materials):
            kind, p = material_params(m)
            c.set_material(b, kind, p)
        if self.blocks is not None:
            c.set_blocks(self.blocks)
        f = np.zeros((self.X.shape[0], 3))
        for n, d, v in self.forces:
            f[n, d] += v
        if self.tractions:
            e = [t[0] for t in self.tractions]
            fc = [t[1] for t in self.tractions]
            tr = [t[2] for t in self.tractions]
            f += lib.traction_forces(self.X, self.conn, e, fc, tr)
        c.set_fext(f)
        self.ctx = c
        self.eqnos = eq
        self._kbc_idx = np.array([n * 3 + d for (n, d, _, _) in self.kbc], dtype=np.int32)
        self._kbc_val = np.array([v for (_, _, v, _) in self.kbc])
        self._kbc_sch = np.array([s for (_, _, _, s) in self.kbc], dtype=np.int64)
        self._tor_idx = np.array(self._torsion_dofs(), dtype=np.int32)
        return c

    def apply_step(self, t, predictor=None):
        """Prescribed values and load factor of the step at time t.  With
        predictor=(precision, precond, lin_rel_tol) the prescribed increment
        is applied through tg_predict_prescribed instead of directly."""
        sc = schedule_value(self.schedule, t)
        self.ctx.set_load_factor(sc)
        scheds = getattr(self, "schedules", {1: self.schedule})
        factors = np.array([0.0] + [schedule_value(scheds.get(n), t) for n in range(1, max(scheds, default=1) + 1)])
        vals = np.where(self._kbc_sch > 0, factors[np.minimum(self._kbc_sch, len(factors) - 1)] * self._kbc_val, 0.0)
        idx = self._kbc_idx
        if len(self._tor_idx):
            # torsion controllers: values of the rigid turn at time t
            idx = np.concatenate([idx, self._tor_idx]).astype(np.int32)
            vals = np.concatenate([vals, self._torsion_values(t)])
        if predictor is not None:
            prec, pc, tol = predictor
            return self.ctx.predict_prescribed(idx, vals, precision=prec, precond=pc, lin_rel_tol=tol)
        if len(idx):
            self.ctx.set_prescribed(idx, vals)
        return 0

    def run(self, nsteps, dt, rel_tol=1e-12, abs_tol=1e-10, max_iterations=10, div_tol=10.0, precision=lib.FP64,
            precond=lib.PRECOND_JACOBI, lin_rel_tol=1e-12, lin_max_it=20000, on_step=None, predictor=False,
            max_step_cuts=0, quick_solve_iter=6, quick_solve_count=3, first_step=1):
        """The load-step sequence of TimeManagerT around NLSolver (device
        Newton per step).  A step whose Newton iteration fails is reset to the
        last converged state (FEManagerT::ResetStep: displacements from the
        step-start snapshot, J2 flags reset) and retried at half the time step
        while fewer than max_step_cuts halvings are in force
        (TimeManagerT::DecreaseLoadStep / DoDecreaseStep,
        TimeManagerT.cpp:119-136,350-362); after quick_solve_count consecutive
        steps converged with NLSolver's iteration counter below
        quick_solve_iter the step is doubled back at an even step number
        (NLSolver::DoConverged, NLSolver.cpp:517-539; IncreaseLoadStep,
        TimeManagerT.cpp:140-150).  Returns the displacements at the original
        step times k*dt and, per original step, the Newton reports of its
        converged sub-steps; self.step_cuts counts the cuts made.  Raises
        TahoeError when a step fails with no cut left.  first_step > 1 resumes
        a sequence (e.g. from a restart image) at step first_step of nsteps."""
        if self.ctx is None:
            self.setup()
        c = self.ctx
        hist, reports = [], []
        step_num, num_steps, cuts, status, quick = first_step - 1, nsteps, 0, "same", 0
        tstep, t = float(dt), (first_step - 1) * float(dt)
        self.step_cuts = 0
        # Newton iterations per original step, failed attempts included (what
        # the step sequence spends; converged sub-steps alone are in reports)
        self.newton_per_step = []
        spent = 0
        sub = []
        while step_num < num_steps:
            if status == "decrease":
                cuts += 1
                tstep /= 2
                num_steps *= 2
                step_num *= 2
            elif status == "increase":
                cuts -= 1
                tstep *= 2
                num_steps //= 2
                step_num //= 2
            status = "same"
            step_num += 1
            t += tstep
            c.checkpoint()
            self.apply_step(t, (precision, precond, lin_rel_tol) if predictor else None)
            rc, rep = c.newton(rel_tol, abs_tol, div_tol, max_iterations, precision, precond, lin_rel_tol, lin_max_it,
                               check=False)
            spent += rep.iterations
            if rc != lib.TG_OK:
                # bad Jacobian, non-finite values, no convergence, divergence:
                # NLSolver's kFailed, answered by a step cut; anything else
                # (arguments, CUDA, memory) is raised at once
                if rc not in (-4, -5, -6, -7):
                    c._chk(rc, "tg_newton_solve")
                c.rollback()
                c.reset_step()
                t -= tstep
                step_num -= 1
                if cuts >= max_step_cuts:
                    c._chk(rc, "tg_newton_solve (no step cut left)")
                status = "decrease"
                self.step_cuts += 1
                continue
            self.current_time = t
            if on_step is not None:
                on_step(step_num, c)
            c.close_step()
            sub.append(rep)
            if quick_solve_iter > 1 and rep.iterations - 1 < quick_solve_iter:
                quick += 1
                if quick >= quick_solve_count and cuts > 0 and step_num % 2 == 0 and num_steps % 2 == 0 \
                        and step_num < num_steps:
                    status = "increase"
                    quick = 0
            else:
                quick = 0
            k = round(t / dt)
            if k >= 1 and abs(t - k * dt) <= 1e-9 * dt:
                hist.append(c.get_u())
                reports.append(sub[0] if len(sub) == 1 else sub)
                self.newton_per_step.append(spent)
                spent = 0
                sub = []
        return np.array(hist), reports


def model_from_fixture(fx, device=0):
    # the deck's own element group (updated_lagrangian decks run the UL element)
    form = fx.get("reference_element", fx["formulation"])
    m = SolidModel(fx["X"], fx["conn"], form if form in ELEMENT_GROUPS else fx["formulation"], fx["material"],
                   device=device,
                   strain_displacement=fx.get("strain_displacement", "standard"))
    m.set_schedule(fx["schedule"])
    for n, d, v, s in fx["kbc"]:
        m.add_kbc(n, d, v, s)
    for axis, rate, px, py, pz, nodes in fx.get("torsion", []):
        m.add_torsion(axis, rate, [px, py, pz], nodes)
    for n, d, v in fx.get("forces", []):
        m.add_force(n, d, v)
    for row in fx.get("tractions", []):
        m.add_traction(row[0], row[1], row[2:5])
    return m
