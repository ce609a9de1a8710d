"""Batched FE^2 micro-solves: seeded RVE batches and their GPU solve.

Configuration 4 of the benchmark set: independent RVEs, each an n x n x n
hex8 unit cube (n drawn from a size set by seed), two-phase compressible
neo-Hookean (matrix mu=1, kappa=10; one centred spherical inclusion of radius
0.3 with 10x stiffer moduli, elements assigned by centroid), affine boundary
displacement u = (F - I) X from a macroscopic F = I + 0.05 S with S symmetric,
entries U(-1, 1).  Each RVE starts from its linearised response to the affine
boundary displacement (the prescribed-increment predictor from the undeformed
state, where the tangent is the positive definite elastic stiffness) and is
solved by Newton to a relative residual of 1e-8 (per RVE).  Starting from the
affine field itself is not used: it over-compresses the stiff inclusion and
leaves an indefinite tangent for a few percent of sampled F (observed: smallest
eigenvalue -0.35 for det F = 0.88), where conjugate gradients break down.
Outputs: the volume-averaged first Piola stress of every RVE.

The whole batch is one disconnected mesh on the device: one tangent, one
matrix stream and one residual per Newton iteration for all RVEs, with one
Krylov solve per RVE over that stream and the exit test applied per RVE
(tg_newton_solve_segmented): an RVE that has converged or failed is frozen and
reported alone (status per RVE), and an RVE's result does not depend on the
batch it is solved in.
"""
import numpy as np

from . import lib
from .meshgen import BoxMesh, equations
from .model import material_params

MATRIX = {"kind": "fs_simo", "mu": 1.0, "kappa": 10.0}
INCLUSION = {"kind": "fs_simo", "mu": 10.0, "kappa": 100.0}
RADIUS = 0.3


class RVETemplate:
    """Mesh, phase blocks and boundary nodes of one RVE size (unit cube)."""

    def __init__(self, n):
        m = BoxMesh(n, n, n)
        self.n = n
        self.X = m.X
        self.conn = m.conn
        centroid = m.element_centroids()
        self.blocks = (np.linalg.norm(centroid - 0.5, axis=1) < RADIUS).astype(np.int32)
        ijk = m.ijk
        self.boundary = np.nonzero(((ijk == 0) | (ijk == n)).any(axis=1))[0].astype(np.int64)
        self.vol = 1.0

    @property
    def nnd(self):
        return self.X.shape[0]

    @property
    def nel(self):
        return self.conn.shape[0]


_templates = {}


def template(n):
    if n not in _templates:
        _templates[n] = RVETemplate(n)
    return _templates[n]


def sample_F(rng):
    """F = I + 0.05 S, S symmetric with entries U(-1, 1)."""
    A = rng.uniform(-1.0, 1.0, size=(3, 3))
    S = np.triu(A) + np.triu(A, 1).T
    return np.eye(3) + 0.05 * S


def sample_batch(count, sizes=range(4, 17), seed=0):
    rng = np.random.default_rng(seed)
    ns = rng.choice(np.asarray(list(sizes)), size=count)
    Fs = np.stack([sample_F(rng) for _ in range(count)])
    return ns, Fs


class RVEBatch:
    """Concatenated device mesh of a batch of RVEs."""

    def __init__(self, ns, Fs):
        self.ns = np.asarray(ns, dtype=np.int64)
        self.Fs = np.asarray(Fs, dtype=np.float64).reshape(-1, 3, 3)
        tpl = [template(int(n)) for n in self.ns]
        nnds = np.array([t.nnd for t in tpl])
        nels = np.array([t.nel for t in tpl])
        self.node_off = np.concatenate([[0], np.cumsum(nnds)]).astype(np.int64)
        self.elem_off = np.concatenate([[0], np.cumsum(nels)]).astype(np.int64)
        self.X = np.concatenate([t.X for t in tpl])
        self.conn = np.concatenate([t.conn + self.node_off[r] for r, t in enumerate(tpl)]).astype(np.int32)
        self.blocks = np.concatenate([t.blocks for t in tpl])
        bnd = [t.boundary + self.node_off[r] for r, t in enumerate(tpl)]
        # affine field on every node (reference) and its boundary values
        U = np.empty_like(self.X)
        for r, t in enumerate(tpl):
            a, b = self.node_off[r], self.node_off[r + 1]
            U[a:b] = self.X[a:b] @ (self.Fs[r] - np.eye(3)).T
        self.u0 = U
        bn = np.concatenate(bnd)
        self.prescribed_idx = (bn[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
        self.prescribed_val = U[bn].reshape(-1)
        self.vol0 = np.array([t.vol for t in tpl])
        self.ctx = None

    @property
    def count(self):
        return len(self.ns)

    @property
    def nnd(self):
        return self.X.shape[0]

    @property
    def nel(self):
        return self.conn.shape[0]

    def setup(self, device=0, ctx=None):
        """Uploads the batch; an existing context (a serving lane's) is
        reused, its previous mesh released into the stream's memory pool."""
        eq = equations(self.nnd, self.prescribed_idx)
        c = ctx if ctx is not None else lib.Context(device)
        c.upload(self.X, self.conn, eq)
        c.set_formulation(lib.TOTAL_LAGRANGIAN)
        for b, m in enumerate((MATRIX, INCLUSION)):
            kind, p = material_params(m)
            c.set_material(b, kind, p)
        c.set_blocks(self.blocks)
        c.set_segments(self.node_off, self.elem_off)
        c.set_fext(np.zeros((self.nnd, 3)))
        self.ctx = c
        return c

    def solve(self, precision=lib.MIXED, rel_tol=1e-8, lin_rel_tol=1e-4, max_iterations=20,
              precond=lib.PRECOND_JACOBI):
        """Predictor from the undeformed state, then Newton to rel_tol per RVE;
        returns (status, report, per-RVE relative residuals, P (count, 3, 3));
        report.pcg_iterations includes the predictor's."""
        c = self.ctx or self.setup()
        c.set_u(np.zeros_like(self.X))
        pred_its = c.predict_prescribed(self.prescribed_idx, self.prescribed_val, precision=precision,
                                        precond=precond, lin_rel_tol=lin_rel_tol)
        rc, rep, rel = c.newton_segmented(rel_tol=rel_tol, abs_tol=0.0, max_iterations=max_iterations,
                                          precision=precision, precond=precond, lin_rel_tol=lin_rel_tol,
                                          check=False)
        rep.pcg_iterations += pred_its
        self.status = c.seg_status.copy()
        P = c.segment_stress(self.vol0)
        return rc, rep, rel, P

    def rve_displacement(self, r, u=None):
        u = self.ctx.get_u() if u is None else u
        return u[self.node_off[r]:self.node_off[r + 1]]


class ResidentRVEs:
    """RVE templates resident on one context: every side length is registered
    once (pattern, contribution map, tiles built one time), and each batch
    mesh is composed on the device from them (tg_mesh_compose), so preparing
    a batch costs O(batch) host work."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.ids = {}
        ctx.set_formulation(lib.TOTAL_LAGRANGIAN)
        for b, m in enumerate((MATRIX, INCLUSION)):
            kind, p = material_params(m)
            ctx.set_material(b, kind, p)

    def template_id(self, n):
        n = int(n)
        if n not in self.ids:
            t = template(n)
            pidx = (t.boundary[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
            self.ids[n] = self.ctx.template_add(t.X, t.conn, equations(t.nnd, pidx), t.blocks)
        return self.ids[n]

    def compose(self, ns):
        self.ctx.compose([self.template_id(n) for n in ns])

    def solve(self, ns, Fs, precision=lib.MIXED, rel_tol=1e-8, lin_rel_tol=1e-4, max_iterations=20,
              precond=lib.PRECOND_BLOCK_JACOBI):
        """Composes the batch, runs the affine predictor from the undeformed
        state and Newton to rel_tol per RVE; same returns as RVEBatch.solve."""
        c = self.ctx
        self.compose(ns)
        Fs = np.asarray(Fs, dtype=np.float64).reshape(-1, 3, 3)
        pred_its = c.predict_affine(Fs, precision=precision, precond=precond, lin_rel_tol=lin_rel_tol)
        rc, rep, rel = c.newton_segmented(rel_tol=rel_tol, abs_tol=0.0, max_iterations=max_iterations,
                                          precision=precision, precond=precond, lin_rel_tol=lin_rel_tol,
                                          check=False)
        rep.pcg_iterations += pred_its
        self.status = c.seg_status.copy()
        P = c.segment_stress(np.array([template(int(n)).vol for n in ns]))
        return rc, rep, rel, P
