"""Shared builders for the parity tests (oracle and GPU driven from the same
inputs)."""
import json
import os

import numpy as np

from oracle.pyoracle import OracleModel
from tahoe_gb300.meshgen import BoxMesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_NAMES = ["mat08_j2_cube", "mat24_hookean_cube", "mat05_simo_cube", "traction_a_cube",
                "beam_newton_totlag", "beam_newton_updlag", "beam_bbar", "mat01_ssstvenant_cube",
                "mat02_fsstvenant_cube", "mat25_fshookean_cube", "torsion_z", "torsion_y"]
# the beam with the deck's other solver / matrix choices (nonlinear PCG with a
# diagonal or profile matrix, quasi-Newton, stored shape functions): the
# reference's outputs of the same field reached by other algorithms
SOLVER_CHOICE_NAMES = ["beam_pcg_diagonal", "beam_pcg_profile", "beam_quasi_newton", "beam_newton_totlag_store"]
# decks pinned on the oracle only (none at present: large_strain_Hookean with
# an isotropic modulus, read as the St.Venant-Kirchhoff law, and the torsion
# controller's finite rotations run on the GPU path too)
ORACLE_EXTRA_NAMES = []


def load_fixture(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def golden_displacements(fx):
    """{step index (0-based): (nnd,3) displacements} from the golden outputs"""
    out = {}
    for o in fx["outputs"]:
        step = int(round(o["time"] / fx["dt"])) - 1
        out[step] = np.array(o["rows"])[:, :3]
    return out


def msr_to_upper_csr(bindx, n):
    """MSR (diagonal implicit) -> list of sorted upper columns per row incl. diag"""
    rows = []
    for r in range(n):
        rows.append(np.concatenate([[r], bindx[bindx[r]:bindx[r + 1]]]))
    return rows


def cube_case(n=4, jitter=0.0, seed=0, fix="z0"):
    """small box with z=0 fully fixed (and optionally more) for parity"""
    m = BoxMesh(n, n, n, jitter=jitter, seed=seed)
    fixed = []
    for node in m.face_nodes(2, 0):
        for d in range(3):
            fixed.append((int(node), d))
    return m, fixed


def oracle_for(mesh, formulation, material, fixed, blocks=None, threads=1):
    o = OracleModel(mesh.X, mesh.conn, formulation, material, blocks=blocks, threads=threads)
    for node, d in fixed:
        o.add_kbc(node, d, 0.0, False)
    return o


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    s = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / s)


def oracle_rve(n, F):
    """One RVE of side n under the affine boundary displacement (F - I) X,
    solved by the oracle's Newton with its direct solve; returns the
    displacements and the averaged first Piola stress from the reactions,
    (1/V0) sum_{boundary a} f_a (x) X_a."""
    from tahoe_gb300 import rve
    t = rve.template(n)
    o = OracleModel(t.X, t.conn, "total_lagrangian", [rve.MATRIX, rve.INCLUSION], blocks=t.blocks)
    o.set_schedule([(0.0, 1.0)])
    U = t.X @ (F - np.eye(3)).T
    for a in t.boundary:
        for d in range(3):
            o.add_kbc(int(a), d, float(U[a, d]), True)
    st, uh, its = o.run(1, 1.0, 1e-12, 1e-15, 20, 1e3, 0)
    assert st == 0
    u = uh[-1]
    f = o.nodal_internal_force(u)
    P = sum(np.outer(f[a], t.X[a]) for a in t.boundary) / t.vol
    return u, P
