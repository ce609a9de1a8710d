"""Seeded synthetic hex8 meshes for the benchmark and parity workloads.

Structured boxes with the reference's hex8 node order (HexahedronT.cpp:23-25):
(-,-,-), (+,-,-), (+,+,-), (-,+,-), then the same on the upper face.  Nodes
are numbered x-fastest, then y, then z.  Optional jitter moves interior nodes
uniformly by +-jitter*h in every direction (seeded).
"""
import numpy as np


class BoxMesh:
    def __init__(self, nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, jitter=0.0, seed=0, origin=(0.0, 0.0, 0.0)):
        self.n = (nx, ny, nz)
        self.L = (lx, ly, lz)
        xs = np.linspace(0.0, lx, nx + 1) + origin[0]
        ys = np.linspace(0.0, ly, ny + 1) + origin[1]
        zs = np.linspace(0.0, lz, nz + 1) + origin[2]
        Z, Y, Xg = np.meshgrid(zs, ys, xs, indexing="ij")
        X = np.stack([Xg.ravel(), Y.ravel(), Z.ravel()], axis=1)
        self.ijk = np.stack(np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij"),
                            axis=-1).reshape(-1, 3)[:, ::-1]  # (i, j, k) per node
        if jitter > 0.0:
            rng = np.random.default_rng(seed)
            h = np.array([lx / nx, ly / ny, lz / nz])
            i, j, k = self.ijk[:, 0], self.ijk[:, 1], self.ijk[:, 2]
            interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
            d = rng.uniform(-jitter, jitter, size=(X.shape[0], 3)) * h
            X = X + d * interior[:, None]
        self.X = X
        self.conn = self._connect(nx, ny, nz)

    @staticmethod
    def _connect(nx, ny, nz):
        def nid(i, j, k):
            return i + (nx + 1) * (j + (ny + 1) * k)

        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        conn = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                         nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)],
                        axis=1)
        return conn.astype(np.int32)

    @property
    def nnd(self):
        return self.X.shape[0]

    @property
    def nel(self):
        return self.conn.shape[0]

    def face_nodes(self, axis, side):
        """nodes on the face axis in {0,1,2}, side 0 (min) / 1 (max)"""
        n = self.n[axis]
        return np.nonzero(self.ijk[:, axis] == (0 if side == 0 else n))[0].astype(np.int32)

    def face_facets(self, axis, side):
        """(elements, facets) on a boundary face; facet numbering of
        HexahedronT::NodesOnFacet: 0 z-, 1 z+, 2 y-, 3 x+, 4 y+, 5 x-"""
        nx, ny, nz = self.n
        e = np.arange(self.nel)
        i = e % nx
        j = (e // nx) % ny
        k = e // (nx * ny)
        coord = (i, j, k)[axis]
        target = 0 if side == 0 else self.n[axis] - 1
        sel = np.nonzero(coord == target)[0].astype(np.int32)
        facet = {(2, 0): 0, (2, 1): 1, (1, 0): 2, (0, 1): 3, (1, 1): 4, (0, 0): 5}[(axis, side)]
        return sel, np.full(len(sel), facet, dtype=np.int32)

    def element_centroids(self):
        return self.X[self.conn].mean(axis=1)


def equations(nnd, prescribed_dofs):
    """Equation numbers of NodeManagerT::SetEquationNumbers: 1-based,
    node-major/dof-minor, prescribed dofs -1."""
    eq = np.zeros(nnd * 3, dtype=np.int64)
    eq[np.asarray(prescribed_dofs, dtype=np.int64)] = -1
    active = eq == 0
    eq[active] = np.arange(1, int(active.sum()) + 1)
    return eq.astype(np.int32).reshape(-1, 3)
