"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle library is built by oracle/build.py.  Tests, the smoke check and
the benchmark's CPU-baseline leg are its only users.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

MAT_KINDS = {"ss_hookean": 0, "ss_j2": 1, "fs_simo": 2, "fs_stvenant": 3}
FORMS = {"small_strain": 0, "total_lagrangian": 1, "updated_lagrangian": 2}
J2_PLASTIC, J2_ELASTIC, J2_RESET, J2_UNALLOCATED = 0, 1, 3, 7

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.orc_model_create.restype = ctypes.c_void_p
        L.orc_model_create.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip]
        L.orc_model_free.argtypes = [ctypes.c_void_p]
        for name, args in [
            ("orc_set_formulation", [ctypes.c_int]),
            ("orc_set_bbar", [ctypes.c_int]),
            ("orc_set_material", [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int]),
            ("orc_set_element_blocks", [_ip]),
            ("orc_set_schedule", [ctypes.c_int, _dp, _dp]),
            ("orc_add_kbc", [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]),
            ("orc_add_torsion", [ctypes.c_int, ctypes.c_double, _dp, ctypes.c_int, _ip]),
            ("orc_add_force", [ctypes.c_int, ctypes.c_int, ctypes.c_double]),
            ("orc_add_traction", [ctypes.c_int, ctypes.c_int, _dp]),
            ("orc_set_threads", [ctypes.c_int]),
            ("orc_equations", [_ip]),
            ("orc_element", [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp]),
            ("orc_form", [_dp, ctypes.c_double, ctypes.c_int, _dp, _dp]),
            ("orc_msr_multx", [_dp, _dp, _dp]),
            ("orc_pcg", [_dp, _dp, _dp, ctypes.c_double, ctypes.c_int, _dp]),
            ("orc_run", [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                         ctypes.c_double, ctypes.c_int, ctypes.c_double, _dp, _ip]),
            ("orc_run_cuts", [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                              ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, _dp, _ip, _ip, _dp, _dp]),
            ("orc_nodal_stress", [_dp, ctypes.c_int, _dp]),
            ("orc_nodal_material_output", [_dp, ctypes.c_int, _dp]),
            ("orc_j2_state", [ctypes.c_void_p, _dp, _dp]),
            ("orc_nodal_internal_force", [_dp, ctypes.c_int, _dp]),
            ("orc_get_u", [_dp]),
            ("orc_set_u", [_dp]),
            ("orc_close_step", []),
            ("orc_residual", [ctypes.c_double, ctypes.c_int, _dp]),
            ("orc_newton_iteration", [ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int, _ip, _dp, _dp]),
            ("orc_predict", [ctypes.c_double, ctypes.c_double, ctypes.c_int, _ip]),
        ]:
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.c_void_p] + args
        L.orc_msr_pattern.restype = ctypes.c_longlong
        L.orc_msr_pattern.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, ctypes.c_longlong]
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def material_params(mat):
    """(kind id, parameter vector) for a material dict of the fixtures."""
    k = mat["kind"]
    if k == "ss_hookean":
        if "C" in mat:
            return 0, np.asarray(mat["C"], dtype=np.float64).reshape(36)
        return 0, np.array([mat["E"], mat["nu"]], dtype=np.float64)
    if k == "ss_j2":
        return 1, np.array([mat["E"], mat["nu"], mat["a"], mat["b"], mat.get("elastic_iterations", 0)],
                           dtype=np.float64)
    if k == "fs_simo":
        return 2, np.array([mat["mu"], mat["kappa"]], dtype=np.float64)
    if k == "fs_stvenant":
        return 3, np.array([mat["E"], mat["nu"]], dtype=np.float64)
    raise ValueError(k)


class OracleModel:
    def __init__(self, X, conn, formulation, materials, blocks=None, threads=1, bbar=False):
        L = lib()
        self.X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 8)
        self.nnd, self.nel = self.X.shape[0], self.conn.shape[0]
        self.h = L.orc_model_create(self.nnd, _d(self.X), self.nel, _i(self.conn))
        L.orc_set_formulation(self.h, FORMS[formulation])
        L.orc_set_bbar(self.h, int(bool(bbar)))
        if isinstance(materials, dict):
            materials = [materials]
        for b, m in enumerate(materials):
            kind, p = material_params(m)
            if L.orc_set_material(self.h, b, kind, _d(p), len(p)) != 0:
                raise ValueError("bad material")
        if blocks is not None:
            bl = np.ascontiguousarray(blocks, dtype=np.int32)
            L.orc_set_element_blocks(self.h, _i(bl))
        L.orc_set_threads(self.h, threads)
        self._neq = None

    def __del__(self):
        try:
            if self.h:
                lib().orc_model_free(self.h)
        except Exception:
            pass

    def set_schedule(self, pts):
        pts = np.asarray(pts, dtype=np.float64).reshape(-1, 2)
        x, y = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
        lib().orc_set_schedule(self.h, len(x), _d(x), _d(y))

    def add_kbc(self, node, dof, value=0.0, scheduled=False):
        lib().orc_add_kbc(self.h, int(node), int(dof), float(value), int(bool(scheduled)))

    def add_torsion(self, axis, rate, point, nodes):
        """Rigid turn of `nodes` about coordinate axis `axis` (0..2) through
        `point` by rate * t (the reference's torsion controller)."""
        pt = np.ascontiguousarray(point, dtype=np.float64)
        nd = np.ascontiguousarray(nodes, dtype=np.int32)
        if lib().orc_add_torsion(self.h, int(axis), float(rate), _d(pt), len(nd), _i(nd)) != 0:
            raise ValueError("torsion axis must be 0, 1 or 2")

    def add_force(self, node, dof, value):
        lib().orc_add_force(self.h, int(node), int(dof), float(value))

    def add_traction(self, elem, facet, t):
        t = np.asarray(t, dtype=np.float64)
        lib().orc_add_traction(self.h, int(elem), int(facet), _d(t))

    def equations(self):
        eq = np.zeros(self.nnd * 3, dtype=np.int32)
        self._neq = lib().orc_equations(self.h, _i(eq))
        return eq.reshape(-1, 3), self._neq

    @property
    def neq(self):
        if self._neq is None:
            self.equations()
        return self._neq

    def msr_pattern(self, upper=True):
        L = lib()
        n = L.orc_msr_pattern(self.h, int(upper), None, 0)
        b = np.zeros(n, dtype=np.int32)
        L.orc_msr_pattern(self.h, int(upper), _i(b), n)
        return b

    def element(self, e, u, iteration=0):
        Ke = np.zeros(576)
        f = np.zeros(24)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        s = lib().orc_element(self.h, int(e), _d(u), int(iteration), _d(Ke), _d(f))
        if s:
            raise RuntimeError("oracle element status %d" % s)
        return Ke.reshape(24, 24), f

    def form(self, u, t, iteration=0, want_K=True):
        neq = self.neq
        R = np.zeros(neq)
        bindx = self.msr_pattern(True)
        val = np.zeros(len(bindx)) if want_K else None
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        s = lib().orc_form(self.h, _d(u), float(t), int(iteration), _d(R), _d(val) if want_K else None)
        if s:
            raise RuntimeError("oracle form status %d" % s)
        return R, val, bindx

    def pcg(self, val, b, tol, maxit):
        x = np.zeros(self.neq)
        rr = ctypes.c_double(0)
        it = lib().orc_pcg(self.h, _d(val), _d(np.ascontiguousarray(b)), _d(x), tol, maxit, ctypes.byref(rr))
        return x, it, rr.value

    def run(self, nsteps, dt, rel_tol=1e-12, abs_tol=1e-10, max_its=10, div_tol=10.0, solver=0,
            lin_tol=1e-12):
        uh = np.zeros((nsteps, self.nnd, 3))
        its = np.zeros(nsteps, dtype=np.int32)
        s = lib().orc_run(self.h, nsteps, dt, rel_tol, abs_tol, max_its, div_tol, solver, lin_tol,
                          _d(uh), _i(its))
        return s, uh, its

    def run_cuts(self, nsteps, dt, rel_tol=1e-12, abs_tol=1e-10, max_its=10, div_tol=10.0, solver=0,
                 lin_tol=1e-12, max_cuts=0, quick_iter=6, quick_count=3, want_stress=False):
        """run() inside the reference's step sequence with load-step cuts;
        returns (status, u at the original steps, iterations per original
        step, cuts made) and, with want_stress, the nodal output stresses
        per original step."""
        uh = np.zeros((nsteps, self.nnd, 3))
        its = np.zeros(nsteps, dtype=np.int32)
        sh = np.zeros((nsteps, self.nnd, 6)) if want_stress else None
        mh = np.zeros((nsteps, self.nnd, 3)) if want_stress else None
        cuts = ctypes.c_int(0)
        s = lib().orc_run_cuts(self.h, nsteps, dt, rel_tol, abs_tol, max_its, div_tol, solver, lin_tol, max_cuts,
                               quick_iter, quick_count, _d(uh), _i(its), ctypes.byref(cuts), _d(sh), _d(mh))
        if want_stress:
            self.material_output_hist = mh
            return s, uh, its, cuts.value, sh
        return s, uh, its, cuts.value

    def nodal_stress(self, u, iteration=0):
        out = np.zeros(self.nnd * 6)
        s = lib().orc_nodal_stress(self.h, _d(np.ascontiguousarray(u, dtype=np.float64).reshape(-1)), int(iteration),
                                   _d(out))
        if s:
            raise RuntimeError("oracle nodal stress status %d" % s)
        return out.reshape(-1, 6)

    def j2_state(self):
        fl = np.zeros(self.nel * 8, dtype=np.int8)
        al = np.zeros(self.nel * 8)
        ep = np.zeros(self.nel * 8 * 6)
        lib().orc_j2_state(self.h, fl.ctypes.data_as(ctypes.c_void_p), _d(al), _d(ep))
        return fl.reshape(-1, 8), al.reshape(-1, 8), ep.reshape(-1, 8, 6)

    def nodal_internal_force(self, u, iteration=0):
        f = np.zeros(self.nnd * 3)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        lib().orc_nodal_internal_force(self.h, _d(u), int(iteration), _d(f))
        return f.reshape(-1, 3)

    def get_u(self):
        u = np.zeros(self.nnd * 3)
        lib().orc_get_u(self.h, _d(u))
        return u.reshape(-1, 3)

    def set_u(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        lib().orc_set_u(self.h, _d(u))

    def close_step(self):
        lib().orc_close_step(self.h)

    def residual(self, t, iteration=-1):
        """||R|| at the held displacement; R is kept for newton_iteration."""
        nrm = ctypes.c_double(0)
        if lib().orc_residual(self.h, float(t), int(iteration), ctypes.byref(nrm)):
            raise RuntimeError("oracle residual failed")
        return nrm.value

    def newton_iteration(self, t, iteration, lin_tol, max_it=100000):
        """One Newton iteration from the held state: (CG iterations, new
        ||R||, seconds of [tangent pass, CG, residual pass])."""
        its = ctypes.c_int(0)
        nrm = ctypes.c_double(0)
        tm = np.zeros(3)
        s = lib().orc_newton_iteration(self.h, float(t), int(iteration), float(lin_tol), int(max_it),
                                       ctypes.byref(its), ctypes.byref(nrm), _d(tm))
        if s:
            raise RuntimeError("oracle Newton iteration failed (%d)" % s)
        return its.value, nrm.value, tm

    def predict(self, t, lin_tol, max_it=100000):
        """Prescribed-increment predictor to time t; returns CG iterations."""
        its = ctypes.c_int(0)
        if lib().orc_predict(self.h, float(t), float(lin_tol), int(max_it), ctypes.byref(its)):
            raise RuntimeError("oracle predictor failed")
        return its.value


def model_from_fixture(fx, threads=1):
    # the deck's own element group (updated_lagrangian decks run the UL element)
    form = fx.get("reference_element", fx["formulation"])
    m = OracleModel(fx["X"], fx["conn"], form if form in FORMS else fx["formulation"], fx["material"],
                    threads=threads,
                    bbar=fx.get("strain_displacement") == "B-bar")
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
