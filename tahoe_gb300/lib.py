"""ctypes binding of the tahoe_gb300 C ABI (include/tahoe_gb300.h).

The shared library is built in-tree by tahoe_gb300/build.py.  There is no
CPU fallback: if the library cannot be built or loaded, or no CUDA device is
present, calls raise.
"""
import ctypes
import os

import numpy as np

from . import build as _build

TG_OK = 0
ERRORS = {
    -1: "TG_ERR_ARG", -2: "TG_ERR_CUDA", -3: "TG_ERR_OOM", -4: "TG_ERR_BAD_JACOBIAN", -5: "TG_ERR_NAN",
    -6: "TG_ERR_NOT_CONVERGED", -7: "TG_ERR_DIVERGED", -8: "TG_ERR_CAPACITY",
}
SMALL_STRAIN, TOTAL_LAGRANGIAN, UPDATED_LAGRANGIAN = 0, 1, 2
STRAIN_STANDARD, STRAIN_BBAR = 0, 1
MAT_SS_HOOKEAN, MAT_SS_J2, MAT_FS_SIMO, MAT_FS_STVENANT = 0, 1, 2, 3
FP64, MIXED = 0, 1
PRECOND_JACOBI, PRECOND_BLOCK_JACOBI = 0, 1
J2_PLASTIC, J2_ELASTIC, J2_RESET, J2_UNALLOCATED = 0, 1, 3, 7

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p


class NewtonParams(ctypes.Structure):
    _fields_ = [("rel_tol", ctypes.c_double), ("abs_tol", ctypes.c_double), ("div_tol", ctypes.c_double),
                ("max_iterations", ctypes.c_int), ("precision", ctypes.c_int), ("precond", ctypes.c_int),
                ("lin_rel_tol", ctypes.c_double), ("lin_max_it", ctypes.c_int)]


class NewtonReport(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("pcg_iterations", ctypes.c_int), ("error0", ctypes.c_double),
                ("error", ctypes.c_double), ("ms_residual", ctypes.c_double), ("ms_tangent", ctypes.c_double),
                ("ms_solve", ctypes.c_double)]


# name -> (restype, argtypes); every function takes the context first unless noted
_SIGS = {
    "tg_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int]),
    "tg_destroy": (ctypes.c_int, [_vp]),
    "tg_last_error": (ctypes.c_char_p, [_vp]),
    "tg_launch_count": (ctypes.c_longlong, [_vp]),
    "tg_mesh_upload": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_int, _ip, _ip]),
    "tg_element_set": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_material_set": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int]),
    "tg_element_blocks": (ctypes.c_int, [_vp, _ip]),
    "tg_pattern_build": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _ip, ctypes.POINTER(ctypes.c_longlong)]),
    "tg_sizes": (ctypes.c_int, [_vp, _ip, ctypes.POINTER(ctypes.c_longlong)]),
    "tg_set_displacement": (ctypes.c_int, [_vp, _dp]),
    "tg_get_displacement": (ctypes.c_int, [_vp, _dp]),
    "tg_set_prescribed": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp]),
    "tg_set_external_force": (ctypes.c_int, [_vp, _dp]),
    "tg_set_load_factor": (ctypes.c_int, [_vp, ctypes.c_double]),
    "tg_traction_forces": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _ip, ctypes.c_int, _ip, _ip, _dp, _dp]),
    "tg_pattern_build_host": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _ip, _ip, ctypes.c_int, _ip, _ip,
                                             ctypes.POINTER(ctypes.c_longlong)]),
    "tg_set_iteration": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_form_residual": (ctypes.c_int, [_vp, _dp, _dp]),
    "tg_form_residual_precision": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp]),
    "tg_form_tangent": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_get_tangent_csr": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "tg_element_dump": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "tg_pcg_solve": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, _ip, _dp]),
    "tg_pcg_solve_noalloc": (ctypes.c_int, [_vp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                            ctypes.c_int, _ip, _dp]),
    "tg_apply_update": (ctypes.c_int, [_vp]),
    "tg_close_step": (ctypes.c_int, [_vp]),
    "tg_reset_step": (ctypes.c_int, [_vp]),
    "tg_get_active_set": (ctypes.c_int, [_vp, _vp]),
    "tg_get_j2_state": (ctypes.c_int, [_vp, _dp, _dp]),
    "tg_newton_solve": (ctypes.c_int, [_vp, ctypes.POINTER(NewtonParams), ctypes.POINTER(NewtonReport)]),
    "tg_newton_iteration": (ctypes.c_int, [_vp, ctypes.POINTER(NewtonParams), _dp, _ip]),
    "tg_predict_prescribed": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, ctypes.POINTER(NewtonParams), _ip]),
    "tg_checkpoint": (ctypes.c_int, [_vp]),
    "tg_rollback": (ctypes.c_int, [_vp]),
    "tg_timer_start": (ctypes.c_int, [_vp]),
    "tg_timer_stop": (ctypes.c_int, [_vp, _dp]),
    "tg_time_kernel": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    "tg_spmv_config": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "tg_spmv_symmetric": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "tg_tangent_config": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_element_strain_displacement": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_nodal_stress": (ctypes.c_int, [_vp, _dp]),
    "tg_state_size": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "tg_state_save": (ctypes.c_int, [_vp, _vp, ctypes.c_longlong]),
    "tg_state_load": (ctypes.c_int, [_vp, _vp, ctypes.c_longlong]),
    "tg_nodal_material_output": (ctypes.c_int, [_vp, _dp]),
    "tg_spmv_release": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_spmv_l2_keep": (ctypes.c_int, [_vp, ctypes.c_longlong]),
    "tg_pcg_form": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_pcg_form_get": (ctypes.c_int, [_vp, _ip]),
    "tg_tuning_get": (ctypes.c_int, [_vp, _ip, _ip, _ip]),
    "tg_set_segments": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _ip]),
    "tg_segment_residual_norms": (ctypes.c_int, [_vp, _dp]),
    "tg_segment_average_stress": (ctypes.c_int, [_vp, _dp, _dp]),
    "tg_newton_solve_segmented": (ctypes.c_int, [_vp, ctypes.POINTER(NewtonParams), ctypes.POINTER(NewtonReport),
                                                 _dp, _ip]),
    "tg_segment_solver": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tg_serve_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double]),
    "tg_serve_submit": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_longlong)]),
    "tg_serve_poll": (ctypes.c_int, [_vp, ctypes.c_longlong, _dp, ctypes.POINTER(ctypes.c_int), _dp]),
    "tg_serve_wait": (ctypes.c_int, [_vp]),
    "tg_serve_stats": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
    "tg_serve_error": (ctypes.c_char_p, [_vp]),
    "tg_serve_destroy": (ctypes.c_int, [_vp]),
    "tg_segment_macro_tangent": (ctypes.c_int, [_vp, ctypes.POINTER(NewtonParams), _dp, _dp, _ip]),
    "tg_template_add": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_int, _ip, _ip, _ip, _ip]),
    "tg_mesh_compose": (ctypes.c_int, [_vp, ctypes.c_int, _ip]),
    "tg_set_affine_prescribed": (ctypes.c_int, [_vp, _dp]),
    "tg_predict_affine": (ctypes.c_int, [_vp, _dp, ctypes.POINTER(NewtonParams), _ip]),
}

_lib = None


def library_path():
    return _build.LIB


def load(build=True):
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is None:
        path = _build.build() if build else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError("tahoe_gb300 CUDA library missing: %s" % path)
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


class TahoeError(RuntimeError):
    def __init__(self, code, where, msg):
        self.code = code
        super().__init__("%s failed: %s (%s)" % (where, ERRORS.get(code, code), msg))


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


class Context:
    """One element group + global matrix on one GPU (one CUDA stream)."""

    def __init__(self, device=0):
        self.L = load()
        h = _vp()
        rc = self.L.tg_create(ctypes.byref(h), int(device))
        if rc != TG_OK:
            raise TahoeError(rc, "tg_create", "no CUDA device or driver")
        self.h = h
        self.nnd = self.nel = self.neq = 0
        self.form = -1           # tg_pcg_form default (automatic)
        self.l2_keep = 16 << 20  # tg_spmv_l2_keep default
        self.sym_mode = 0

    def product_kernel(self):
        """Name of the kernel the single-vector solve multiplies with (a
        segmented batch: the kernel of its per-RVE solves)."""
        segmented = getattr(self, "nseg", 0) > 0
        form = self.effective_form()
        if segmented:
            return "pcg_seg_push_kernel" if form == 3 else "pcg_spmv_kernel"
        if self.sym_mode and not getattr(self, "composed", False):
            return "pcg_spmv_sym_kernel"
        if form == 3:
            return "pcg_cg_push_kernel"
        if form in (1, 2):
            return "pcg_cg_spmv_kernel"
        return "pcg_spmv_kernel"

    def close(self):
        if getattr(self, "h", None):
            self.L.tg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, where):
        if rc != TG_OK:
            raise TahoeError(rc, where, self.L.tg_last_error(self.h).decode())
        return rc

    @property
    def launches(self):
        return int(self.L.tg_launch_count(self.h))

    # ---- set-up ----
    def upload(self, X, conn, eqnos):
        X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
        self.nnd = X.shape[0]
        coords = np.ascontiguousarray(X.T).reshape(-1)
        conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 8)
        self.nel = conn.shape[0]
        eq = np.ascontiguousarray(eqnos, dtype=np.int32).reshape(-1)
        self._chk(self.L.tg_mesh_upload(self.h, self.nnd, _d(coords), self.nel, _i(conn), _i(eq)), "tg_mesh_upload")
        n = ctypes.c_int(0)
        nb = ctypes.c_longlong(0)
        self.L.tg_sizes(self.h, ctypes.byref(n), ctypes.byref(nb))
        self.neq, self.block_nnz = n.value, nb.value
        self._coords, self._conn = coords, conn

    def set_formulation(self, form):
        self._chk(self.L.tg_element_set(self.h, int(form)), "tg_element_set")

    def set_material(self, block, kind, params):
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        self._chk(self.L.tg_material_set(self.h, int(block), int(kind), _d(p), len(p)), "tg_material_set")

    def set_blocks(self, blocks):
        b = np.ascontiguousarray(blocks, dtype=np.int32)
        self._chk(self.L.tg_element_blocks(self.h, _i(b)), "tg_element_blocks")

    def pattern(self, upper_only=False):
        nnz = ctypes.c_longlong(0)
        self._chk(self.L.tg_pattern_build(self.h, int(upper_only), None, None, ctypes.byref(nnz)), "tg_pattern_build")
        rp = np.zeros(self.neq + 1, dtype=np.int32)
        ci = np.zeros(nnz.value, dtype=np.int32)
        self._chk(self.L.tg_pattern_build(self.h, int(upper_only), _i(rp), _i(ci), ctypes.byref(nnz)),
                  "tg_pattern_build")
        return rp, ci

    # ---- state ----
    def set_u(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        self._chk(self.L.tg_set_displacement(self.h, _d(u)), "tg_set_displacement")

    def get_u(self, out=None):
        """Displacements (nnd, 3); written into `out` (a contiguous float64
        array of nnd*3 values, e.g. in pinned memory) when given."""
        u = np.zeros(self.nnd * 3) if out is None else out.reshape(-1)
        if u.dtype != np.float64 or u.size != self.nnd * 3 or not u.flags.c_contiguous:
            raise ValueError("get_u: out must be a contiguous float64 array of nnd*3 values")
        self._chk(self.L.tg_get_displacement(self.h, _d(u)), "tg_get_displacement")
        return u.reshape(-1, 3)

    def set_prescribed(self, idx, vals):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self._chk(self.L.tg_set_prescribed(self.h, len(idx), _i(idx), _d(vals)), "tg_set_prescribed")

    def set_fext(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        self._chk(self.L.tg_set_external_force(self.h, _d(f)), "tg_set_external_force")

    def set_load_factor(self, s):
        self._chk(self.L.tg_set_load_factor(self.h, float(s)), "tg_set_load_factor")

    def set_iteration(self, it):
        self._chk(self.L.tg_set_iteration(self.h, int(it)), "tg_set_iteration")

    # ---- element group ----
    def residual(self, want_vector=True, precision=None):
        """R and ||R||: FP64 (tg_form_residual), or in the arithmetic of the
        Newton drivers of `precision` (tg_form_residual_precision)."""
        R = np.zeros(self.neq) if want_vector else None
        nrm = ctypes.c_double(0)
        if precision is None:
            self._chk(self.L.tg_form_residual(self.h, _d(R), ctypes.byref(nrm)), "tg_form_residual")
        else:
            self._chk(self.L.tg_form_residual_precision(self.h, int(precision), _d(R), ctypes.byref(nrm)),
                      "tg_form_residual_precision")
        return R, nrm.value

    def tangent(self, precision):
        self._chk(self.L.tg_form_tangent(self.h, int(precision)), "tg_form_tangent")

    def tangent_csr(self, upper_only=False):
        rp, ci = self.pattern(upper_only)
        v = np.zeros(len(ci))
        self._chk(self.L.tg_get_tangent_csr(self.h, int(upper_only), _d(v)), "tg_get_tangent_csr")
        return rp, ci, v

    def element_dump(self, first, count):
        K = np.zeros(count * 576)
        f = np.zeros(count * 24)
        self._chk(self.L.tg_element_dump(self.h, int(first), int(count), _d(K), _d(f)), "tg_element_dump")
        return K.reshape(count, 24, 24), f.reshape(count, 24)

    def pcg(self, rhs=None, rel_tol=1e-10, max_it=10000, precond=PRECOND_JACOBI, want_du=True):
        its = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        b = None if rhs is None else np.ascontiguousarray(rhs, dtype=np.float64)
        du = np.zeros(self.neq) if want_du else None
        rc = self.L.tg_pcg_solve(self.h, _d(b), _d(du), float(rel_tol), int(max_it), int(precond), ctypes.byref(its),
                                 ctypes.byref(rr))
        if rc not in (TG_OK, -6):
            self._chk(rc, "tg_pcg_solve")
        return du, its.value, rr.value, rc

    def pcg_noalloc(self, rhs_device_ptr, du_device_ptr, rel_tol=1e-10, max_it=10000, precond=PRECOND_JACOBI):
        """tg_pcg_solve_noalloc on caller-owned device buffers (raw pointers);
        returns (iterations, relative residual, status)."""
        its = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        rc = self.L.tg_pcg_solve_noalloc(self.h, ctypes.c_void_p(rhs_device_ptr), ctypes.c_void_p(du_device_ptr),
                                         float(rel_tol), int(max_it), int(precond), ctypes.byref(its),
                                         ctypes.byref(rr))
        if rc not in (TG_OK, -6):
            self._chk(rc, "tg_pcg_solve_noalloc")
        return its.value, rr.value, rc

    def apply_update(self):
        self._chk(self.L.tg_apply_update(self.h), "tg_apply_update")

    def close_step(self):
        self._chk(self.L.tg_close_step(self.h), "tg_close_step")

    def reset_step(self):
        self._chk(self.L.tg_reset_step(self.h), "tg_reset_step")

    def nodal_stress(self):
        out = np.zeros(self.nnd * 6)
        self._chk(self.L.tg_nodal_stress(self.h, _d(out)), "tg_nodal_stress")
        return out.reshape(-1, 6)

    def state_save(self):
        """Restart image of the device state (bytes)."""
        n = ctypes.c_longlong(0)
        self._chk(self.L.tg_state_size(self.h, ctypes.byref(n)), "tg_state_size")
        buf = np.zeros(n.value, dtype=np.uint8)
        self._chk(self.L.tg_state_save(self.h, buf.ctypes.data_as(_vp), n.value), "tg_state_save")
        return buf.tobytes()

    def state_load(self, image):
        buf = np.frombuffer(image, dtype=np.uint8).copy()
        self._chk(self.L.tg_state_load(self.h, buf.ctypes.data_as(_vp), len(buf)), "tg_state_load")

    def nodal_material_output(self):
        out = np.zeros(self.nnd * 3)
        self._chk(self.L.tg_nodal_material_output(self.h, _d(out)), "tg_nodal_material_output")
        return out.reshape(-1, 3)

    def active_set(self):
        f = np.zeros(self.nel * 8, dtype=np.int8)
        self._chk(self.L.tg_get_active_set(self.h, f.ctypes.data_as(_vp)), "tg_get_active_set")
        return f.reshape(-1, 8)

    def j2_state(self):
        a = np.zeros(self.nel * 8)
        e = np.zeros(self.nel * 8 * 6)
        self._chk(self.L.tg_get_j2_state(self.h, _d(a), _d(e)), "tg_get_j2_state")
        return a.reshape(-1, 8), e.reshape(-1, 8, 6)

    def newton(self, rel_tol=1e-12, abs_tol=1e-10, div_tol=10.0, max_iterations=10, precision=FP64,
               precond=PRECOND_JACOBI, lin_rel_tol=1e-12, lin_max_it=20000, check=True):
        P = NewtonParams(rel_tol, abs_tol, div_tol, max_iterations, precision, precond, lin_rel_tol, lin_max_it)
        R = NewtonReport()
        rc = self.L.tg_newton_solve(self.h, ctypes.byref(P), ctypes.byref(R))
        if check:
            self._chk(rc, "tg_newton_solve")
        return rc, R


    def newton_iteration(self, precision=MIXED, precond=PRECOND_JACOBI, lin_rel_tol=1e-6, lin_max_it=20000):
        P = NewtonParams(0.0, 0.0, 1e30, 1 << 30, precision, precond, lin_rel_tol, lin_max_it)
        nrm = ctypes.c_double(0)
        its = ctypes.c_int(0)
        self._chk(self.L.tg_newton_iteration(self.h, ctypes.byref(P), ctypes.byref(nrm), ctypes.byref(its)),
                  "tg_newton_iteration")
        return nrm.value, its.value

    def predict_prescribed(self, idx, vals, precision=MIXED, precond=PRECOND_JACOBI, lin_rel_tol=1e-6,
                           lin_max_it=20000):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        P = NewtonParams(0.0, 0.0, 1e30, 1 << 30, precision, precond, lin_rel_tol, lin_max_it)
        its = ctypes.c_int(0)
        self._chk(self.L.tg_predict_prescribed(self.h, len(idx), _i(idx), _d(vals), ctypes.byref(P),
                                               ctypes.byref(its)), "tg_predict_prescribed")
        return its.value

    def predict_affine(self, F, precision=MIXED, precond=PRECOND_JACOBI, lin_rel_tol=1e-6, lin_max_it=20000):
        F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1)
        if F.size != 9 * self.nseg:
            raise ValueError("need one 3x3 F per segment")
        P = NewtonParams(0.0, 0.0, 1e30, 1 << 30, precision, precond, lin_rel_tol, lin_max_it)
        its = ctypes.c_int(0)
        self._chk(self.L.tg_predict_affine(self.h, _d(F), ctypes.byref(P), ctypes.byref(its)), "tg_predict_affine")
        return its.value

    # ---- resident templates ----
    def template_add(self, X, conn, eqnos, blocks=None):
        X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
        coords = np.ascontiguousarray(X.T).reshape(-1)
        conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 8)
        eq = np.ascontiguousarray(eqnos, dtype=np.int32).reshape(-1)
        b = None if blocks is None else np.ascontiguousarray(blocks, dtype=np.int32)
        tid = ctypes.c_int(-1)
        self._chk(self.L.tg_template_add(self.h, X.shape[0], _d(coords), conn.shape[0], _i(conn), _i(eq), _i(b),
                                         ctypes.byref(tid)), "tg_template_add")
        if not hasattr(self, "_tpl_sizes"):
            self._tpl_sizes = []
        self._tpl_sizes.append((X.shape[0], conn.shape[0]))
        return tid.value

    def compose(self, template_ids):
        ids = np.ascontiguousarray(template_ids, dtype=np.int32)
        self._chk(self.L.tg_mesh_compose(self.h, len(ids), _i(ids)), "tg_mesh_compose")
        sizes = np.asarray(self._tpl_sizes, dtype=np.int64)[ids]
        self.nnd, self.nel = int(sizes[:, 0].sum()), int(sizes[:, 1].sum())
        n = ctypes.c_int(0)
        nb = ctypes.c_longlong(0)
        self.L.tg_sizes(self.h, ctypes.byref(n), ctypes.byref(nb))
        self.neq, self.block_nnz = n.value, nb.value
        self.nseg = len(ids)

    def set_affine(self, F):
        F = np.ascontiguousarray(F, dtype=np.float64).reshape(-1)
        if F.size != 9 * self.nseg:
            raise ValueError("need one 3x3 F per segment")
        self._chk(self.L.tg_set_affine_prescribed(self.h, _d(F)), "tg_set_affine_prescribed")

    def checkpoint(self):
        self._chk(self.L.tg_checkpoint(self.h), "tg_checkpoint")

    def rollback(self):
        self._chk(self.L.tg_rollback(self.h), "tg_rollback")

    def timer_start(self):
        self._chk(self.L.tg_timer_start(self.h), "tg_timer_start")

    def timer_stop(self):
        ms = ctypes.c_double(0)
        self._chk(self.L.tg_timer_stop(self.h, ctypes.byref(ms)), "tg_timer_stop")
        return ms.value

    def set_segments(self, node_off, elem_off):
        no = np.ascontiguousarray(node_off, dtype=np.int32)
        eo = np.ascontiguousarray(elem_off, dtype=np.int32)
        self._chk(self.L.tg_set_segments(self.h, len(no) - 1, _i(no), _i(eo)), "tg_set_segments")
        self.nseg = len(no) - 1

    def segment_norms(self):
        out = np.zeros(self.nseg)
        self._chk(self.L.tg_segment_residual_norms(self.h, _d(out)), "tg_segment_residual_norms")
        return out

    def segment_stress(self, vol0=None):
        P = np.zeros(self.nseg * 9)
        v = None if vol0 is None else np.ascontiguousarray(vol0, dtype=np.float64)
        self._chk(self.L.tg_segment_average_stress(self.h, _d(v), _d(P)), "tg_segment_average_stress")
        return P.reshape(-1, 3, 3)

    def newton_segmented(self, rel_tol=1e-8, abs_tol=0.0, div_tol=1e3, max_iterations=20, precision=MIXED,
                         precond=PRECOND_JACOBI, lin_rel_tol=1e-4, lin_max_it=20000, check=True):
        P = NewtonParams(rel_tol, abs_tol, div_tol, max_iterations, precision, precond, lin_rel_tol, lin_max_it)
        R = NewtonReport()
        rel = np.zeros(self.nseg)
        st = np.zeros(self.nseg, dtype=np.int32)
        rc = self.L.tg_newton_solve_segmented(self.h, ctypes.byref(P), ctypes.byref(R), _d(rel), _i(st))
        # per-RVE status (TG_OK or the RVE's failure code) of the last solve
        self.seg_status = st
        if check:
            self._chk(rc, "tg_newton_solve_segmented")
        return rc, R, rel

    def segment_solver(self, per_rve):
        """One PCG per RVE of a segmented batch (True, default) or one PCG
        over the whole batch (False)."""
        self._chk(self.L.tg_segment_solver(self.h, int(bool(per_rve))), "tg_segment_solver")

    def macro_tangent(self, vol0=None, precision=MIXED, precond=PRECOND_JACOBI, lin_rel_tol=1e-8, lin_max_it=20000):
        """(nseg, 9, 9) consistent macro tangents dP_jJ/dF_kL at the current
        state, and the PCG iterations of the nine solves."""
        P = NewtonParams(0.0, 0.0, 1e30, 1 << 30, precision, precond, lin_rel_tol, lin_max_it)
        C = np.zeros(self.nseg * 81)
        v = None if vol0 is None else np.ascontiguousarray(vol0, dtype=np.float64)
        its = ctypes.c_int(0)
        self._chk(self.L.tg_segment_macro_tangent(self.h, ctypes.byref(P), _d(v), _d(C), ctypes.byref(its)),
                  "tg_segment_macro_tangent")
        return C.reshape(-1, 9, 9), its.value

    def spmv_config(self, tile_blocks, stages):
        self._chk(self.L.tg_spmv_config(self.h, int(tile_blocks), int(stages)), "tg_spmv_config")

    def set_strain_displacement(self, option):
        self._chk(self.L.tg_element_strain_displacement(self.h, int(option)), "tg_element_strain_displacement")

    def spmv_release(self, per_warp):
        self._chk(self.L.tg_spmv_release(self.h, int(per_warp)), "tg_spmv_release")

    def pcg_form(self, form):
        """Recurrences of the single-vector PCG: 3 single-reduction with
        programmatic launch dependencies on the symmetric push storage, 1 the
        same on the full storage, 2 form 1 without programmatic dependencies,
        0 textbook, -1 (default) form 3 on meshes of at least a million block
        nonzeros and form 1 below."""
        self._chk(self.L.tg_pcg_form(self.h, int(form)), "tg_pcg_form")
        self.form = int(form)

    def effective_form(self):
        """The form the next single-vector solve runs on the current mesh."""
        f = ctypes.c_int(0)
        self._chk(self.L.tg_pcg_form_get(self.h, ctypes.byref(f)), "tg_pcg_form_get")
        return f.value

    def spmv_l2_keep(self, nbytes):
        """Matrix bytes the streamed product keeps in the L2 (evict_last;
        the rest streams evict_first); -1 plain copies."""
        self._chk(self.L.tg_spmv_l2_keep(self.h, int(nbytes)), "tg_spmv_l2_keep")
        self.l2_keep = int(nbytes)

    def spmv_symmetric(self, on, tile_blocks=0):
        """Symmetric stream format of the single-vector product (on = 1, 2, 3:
        three launch shapes) or the full block storage (on = 0, default)."""
        self._chk(self.L.tg_spmv_symmetric(self.h, int(on), int(tile_blocks)), "tg_spmv_symmetric")
        self.sym_mode = int(on)

    def tangent_config(self, elems_per_block):
        self._chk(self.L.tg_tangent_config(self.h, int(elems_per_block)), "tg_tangent_config")

    def tuning(self):
        t, s, e = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        self._chk(self.L.tg_tuning_get(self.h, ctypes.byref(t), ctypes.byref(s), ctypes.byref(e)), "tg_tuning_get")
        return {"tile_blocks": t.value, "stages": s.value, "tangent_epb": e.value}

    def time_kernel(self, which, reps):
        ms = ctypes.c_double(0)
        self._chk(self.L.tg_time_kernel(self.h, int(which), int(reps), ctypes.byref(ms)), "tg_time_kernel")
        return ms.value


def traction_forces(X, conn, elems, facets, tractions):
    """Consistent nodal forces of uniform tractions (host helper of the ABI)."""
    L = load()
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    nnd = X.shape[0]
    coords = np.ascontiguousarray(X.T).reshape(-1)
    conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 8)
    e = np.ascontiguousarray(elems, dtype=np.int32)
    fc = np.ascontiguousarray(facets, dtype=np.int32)
    t = np.ascontiguousarray(tractions, dtype=np.float64).reshape(-1)
    f = np.zeros(nnd * 3)
    rc = L.tg_traction_forces(nnd, _d(coords), conn.shape[0], _i(conn), len(e), _i(e), _i(fc), _d(t), _d(f))
    if rc != TG_OK:
        raise TahoeError(rc, "tg_traction_forces", "bad arguments")
    return f.reshape(-1, 3)


def pattern_host(conn, eqnos, nnd, upper_only=False):
    """Scalar CSR (row_ptr, col_idx) of the active equations computed on the
    host from the mesh alone (tg_pattern_build_host; no GPU needed)."""
    L = load()
    conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 8)
    eq = np.ascontiguousarray(eqnos, dtype=np.int32).reshape(-1)
    nnz = ctypes.c_longlong(0)
    rc = L.tg_pattern_build_host(int(nnd), conn.shape[0], _i(conn), _i(eq), int(upper_only), None, None,
                                 ctypes.byref(nnz))
    if rc != TG_OK:
        raise TahoeError(rc, "tg_pattern_build_host", "bad arguments")
    neq = int((eq > 0).sum())
    rp = np.zeros(neq + 1, dtype=np.int32)
    ci = np.zeros(nnz.value, dtype=np.int32)
    rc = L.tg_pattern_build_host(int(nnd), conn.shape[0], _i(conn), _i(eq), int(upper_only), _i(rp), _i(ci),
                                 ctypes.byref(nnz))
    if rc != TG_OK:
        raise TahoeError(rc, "tg_pattern_build_host", "bad arguments")
    return rp, ci
