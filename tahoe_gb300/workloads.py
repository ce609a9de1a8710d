"""Synthetic, seeded benchmark workloads (the reference publishes no dataset
for this path; these follow the benchmark configurations' meshes, materials,
boundary conditions and load histories).

  c1: small-strain linear elastic unit cube 16^3 hex8, E=200e3, nu=0.3, z=0
      fully fixed, 1 MPa normal traction on z=1, one static step.
  c2: total-Lagrangian compressible neo-Hookean block 64^3 hex8, mu=1,
      kappa=10, interior nodes jittered +-0.2h (seed 0), bottom fixed, top
      z-displacement to 10% compression in 10 equal steps.
  c3: small-strain J2 (E=200e3, nu=0.3, yield 250, H=1000) plate 96x96x48,
      x=0 face clamped, x=L face gripped (u_y=u_z=0) with u_x cycling to
      +-0.5% strain over 40 steps.
"""
import numpy as np

from .meshgen import BoxMesh
from .model import SolidModel

HOOKE_C1 = {"kind": "ss_hookean", "E": 200e3, "nu": 0.3}
SIMO_C2 = {"kind": "fs_simo", "mu": 1.0, "kappa": 10.0}
J2_C3 = {"kind": "ss_j2", "E": 200e3, "nu": 0.3, "a": 1000.0, "b": 250.0}


def c1(n=16, add=None):
    mesh = BoxMesh(n, n, n)
    m = (add or SolidModel)(mesh.X, mesh.conn, "small_strain", HOOKE_C1)
    for node in mesh.face_nodes(2, 0):
        for d in range(3):
            m.add_kbc(node, d, 0.0, False)
    el, fc = mesh.face_facets(2, 1)
    for e, f in zip(el, fc):
        m.add_traction(e, f, [0.0, 0.0, 1.0])
    m.set_schedule([(0.0, 1.0)])
    return mesh, m, dict(nsteps=1, dt=1.0)


def c2(n=64, jitter=0.2, seed=0, nsteps=10, add=None):
    mesh = BoxMesh(n, n, n, jitter=jitter, seed=seed)
    m = (add or SolidModel)(mesh.X, mesh.conn, "total_lagrangian", SIMO_C2)
    for node in mesh.face_nodes(2, 0):
        for d in range(3):
            m.add_kbc(node, d, 0.0, False)
    for node in mesh.face_nodes(2, 1):
        m.add_kbc(node, 2, -0.1, True)
    m.set_schedule([(0.0, 0.0), (float(nsteps), 1.0)])
    return mesh, m, dict(nsteps=nsteps, dt=1.0)


def c3(nx=96, ny=96, nz=48, nsteps=40, add=None):
    lx, ly, lz = 1.0, 1.0, 0.5
    mesh = BoxMesh(nx, ny, nz, lx=lx, ly=ly, lz=lz)
    m = (add or SolidModel)(mesh.X, mesh.conn, "small_strain", J2_C3)
    for node in mesh.face_nodes(0, 0):
        for d in range(3):
            m.add_kbc(node, d, 0.0, False)
    for node in mesh.face_nodes(0, 1):
        m.add_kbc(node, 0, 0.005 * lx, True)
        m.add_kbc(node, 1, 0.0, False)
        m.add_kbc(node, 2, 0.0, False)
    q = nsteps / 4.0
    m.set_schedule([(0.0, 0.0), (q, 1.0), (3 * q, -1.0), (4 * q, 0.0)])
    return mesh, m, dict(nsteps=nsteps, dt=1.0)


def spmv_bytes(nnzb, nnd, s_val):
    """Algorithmic bytes of one PCG SpMV launch on the node-block CSR: nine
    values + one column index per block, row pointers, the gathered p vector
    once, q written (vectors padded to 4 lanes)."""
    s_vec = 4 * s_val
    return nnzb * (9 * s_val + 4) + (nnd + 1) * 4 + nnd * s_vec + nnd * s_vec


def spmv_bytes_sym(nnzb, nnd, s_val):
    """Algorithmic DRAM bytes of one product streaming the symmetric format:
    the nu = (nnzb + nnd) / 2 upper blocks (nine values + a column index),
    the nl = (nnzb - nnd) / 2 lower entries (column + upper block id; their
    transposed values are re-reads served from L2), upper and lower row
    pointers, the gathered vector once, the product written, the dof mask."""
    s_vec = 4 * s_val
    nu, nl = (nnzb + nnd) // 2, (nnzb - nnd) // 2
    return nu * (9 * s_val + 4) + nl * 8 + 2 * (nnd + 1) * 4 + 2 * nnd * s_vec + nnd


def spmv_bytes_push(nnzb, nnd, s_val):
    """Algorithmic DRAM bytes of one product on the symmetric push storage:
    the nu = (nnzb + nnd) / 2 upper blocks (nine values, a column index, a
    push slot), the row pointers, the gathered vector once and the upper part
    of the product written (vectors padded to 4 lanes).  The transposed
    products it pushes (push_l2_bytes) are an L2 intermediate by design:
    written with evict_last, read by the next kernel and dropped without
    write-back."""
    s_vec = 4 * s_val
    nu = (nnzb + nnd) // 2
    return nu * (9 * s_val + 8) + (nnd + 1) * 4 + 2 * nnd * s_vec


def push_l2_bytes(nnzb, nnd, s_val):
    """Bytes of the nl = (nnzb - nnd) / 2 pushed products, written by the
    product and read by the vector kernel through the L2."""
    return (nnzb - nnd) // 2 * 4 * s_val


def cg_vector_bytes_push(nnzb, nnd, s_val):
    """Algorithmic DRAM bytes of the single-reduction vector kernel on the
    push storage: those of cg_vector_bytes plus the slot pointers and the
    dof mask (the pushed products come from the L2, push_l2_bytes)."""
    return cg_vector_bytes(nnd, s_val) + (nnd + 1) * 4 + nnd


def assembly_bytes(nel, nnzb, nnd, s_val):
    """Algorithmic bytes of one assembly launch: element blocks (36 blocks of
    3 rows padded to 4 values per element) read once, the 64 contribution
    codes per element and their segment pointers, the column indices, the
    block values written once, the preconditioner inverses (two 3x3 blocks
    and Jacobi's diagonal as a padded 4-vector per node) written."""
    return (nel * 36 * 12 * s_val + nel * 64 * 4 + (nnzb + 1) * 4 + nnzb * 9 * s_val + nnzb * 4 +
            nnd * 22 * s_val)


def assembly_bytes_upper(nel, nnzb, nnd, s_val):
    """Algorithmic bytes of one upper-only assembly into the push storage:
    element blocks read once (every upper element block lands in one upper
    global block), 36 contribution codes per element and the upper blocks'
    segment pointers, per row its diagonal position and upper pointer, the
    nu = (nnzb + nnd) / 2 upper block values written, the preconditioner
    inverses written."""
    nu = (nnzb + nnd) // 2
    return nel * 36 * 12 * s_val + nel * 36 * 4 + (nu + nnd) * 4 + nu * 9 * s_val + nnd * 12 + nnd * 22 * s_val


def cg_vector_bytes(nnd, s_val):
    """Algorithmic bytes of one vector kernel of the single-reduction PCG:
    u, w, p, s, x, r and the 3x3 preconditioner block read, p, s, x, r and u
    written (vectors padded to 4 lanes)."""
    s_vec = 4 * s_val
    return nnd * (6 * s_vec + 9 * s_val) + nnd * 5 * s_vec


def update_bytes(nnd, s_val):
    """Algorithmic bytes of one PCG vector update: p, q, x, r and the 3x3
    preconditioner block read, x, r, z and the next p written (vectors padded
    to 4 lanes)."""
    s_vec = 4 * s_val
    return nnd * (4 * s_vec + 9 * s_val) + nnd * 4 * s_vec
