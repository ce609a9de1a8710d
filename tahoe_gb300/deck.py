"""Tahoe input decks on the GPU path: the XML deck and TahoeII geometry
readers, the model they describe, the load-step driver and a writer of the
reference's ``.run`` nodal output layout.

This is the host glue a deck needs to run on the GPU element group: the
geometry reader follows TahoeInputT / the TahoeII ``.geom`` format
(toolbox/src/dataio/input/TahoeInputT.cpp), boundary conditions follow
kinematic_BC / force_BC / natural_bc (KBC_CardT, FieldT::InitStep), the
schedules PiecewiseLinearT, the element group SmallStrainT /
TotalLagrangianT (UpdatedLagrangianT decks run on the total-Lagrangian
element: same converged field), the step loop TimeManagerT + NLSolver
(max_step_cuts, quick_solve_iter, quick_solve_count) and the output the nodal
table of OutputSetT's ``.run`` files (displacements, extrapolated stresses,
material output).
"""
import os
import re
import xml.etree.ElementTree as ET

import numpy as np

from . import lib
from .model import SolidModel

def _tokens(lines):
    for ln in lines:
        ln = ln.split("#", 1)[0].strip()
        if ln:
            for t in ln.split():
                yield t


def read_geom(path):
    """TahoeII .geom reader (toolbox/src/dataio/input/TahoeInputT)."""
    base = os.path.dirname(path)
    with open(path) as f:
        raw = f.read().splitlines()
    # split into *sections
    sections, cur = {}, None
    for ln in raw:
        s = ln.strip()
        if s.startswith("*"):
            cur = s[1:].split()[0]
            sections.setdefault(cur, [])
        elif cur is not None:
            sections[cur].append(ln)
    dims = list(_tokens(sections["dimensions"]))
    it = iter(dims)
    nnd, nsd = int(next(it)), int(next(it))
    nsets = int(next(it))
    eset_dims = [(int(next(it)), int(next(it)), int(next(it))) for _ in range(nsets)]
    nns = int(next(it))
    ns_dims = [(int(next(it)), int(next(it))) for _ in range(nns)]
    nss = int(next(it))
    ss_dims = [(int(next(it)), int(next(it)), int(next(it))) for _ in range(nss)]

    # re-scan raw lines for *set blocks within sections
    def blocks_of(sec):
        out, inside, curb = [], False, None
        for ln in raw:
            s = ln.strip()
            if s.startswith("*") and not s.startswith("*set"):
                if curb is not None:
                    out.append(curb)
                    curb = None
                inside = s[1:].split()[0] == sec
                continue
            if inside and s.startswith("*set"):
                if curb is not None:
                    out.append(curb)
                curb = []
                continue
            if inside and curb is not None:
                curb.append(ln)
        if curb is not None:
            out.append(curb)
        return out

    nodesets = {}
    for (sid, n), blk in zip(ns_dims, blocks_of("nodesets")):
        toks = [int(t) for t in _tokens(blk)]
        cnt = toks[0]
        ids = toks[1:1 + cnt]
        if cnt == 1 and ids == [-1]:
            ids = list(range(1, nnd + 1))
        nodesets[sid] = [i - 1 for i in ids]
    sidesets = {}
    for (sid, blk_id, n), blk in zip(ss_dims, blocks_of("sidesets")):
        toks = [int(t) for t in _tokens(blk)]
        cnt = toks[0]
        pairs = toks[1:1 + 2 * cnt]
        sidesets[sid] = [(pairs[2 * k] - 1, pairs[2 * k + 1] - 1) for k in range(cnt)]

    def read_table(blk_lines, ncols_hint=None):
        toks = list(_tokens(blk_lines))
        if len(toks) == 1 and not re.match(r"^-?\d", toks[0]):
            with open(os.path.join(base, toks[0])) as f:
                toks = list(_tokens(f.read().splitlines()))
        return toks

    eblocks = blocks_of("elements")
    conn = []
    for (eid, nel, nen), blk in zip(eset_dims, eblocks):
        toks = read_table(blk)
        cnt, nen2 = int(toks[0]), int(toks[1])
        vals = [int(t) for t in toks[2:]]
        for k in range(cnt):
            row = vals[k * (nen2 + 1):(k + 1) * (nen2 + 1)]
            conn.append([i - 1 for i in row[1:]])
    ntoks = read_table(sections["nodes"])
    cnt, nsd2 = int(ntoks[0]), int(ntoks[1])
    vals = [float(t) for t in ntoks[2:]]
    X = [None] * cnt
    for k in range(cnt):
        row = vals[k * (nsd2 + 1):(k + 1) * (nsd2 + 1)]
        X[int(row[0]) - 1] = row[1:]
    return X, conn, nodesets, sidesets


def read_run(path):
    """Nodal tables of every output block of a .run file."""
    with open(path) as f:
        lines = f.read().splitlines()
    out, time, i = [], None, 0
    while i < len(lines):
        ln = lines[i]
        if ln.strip().startswith("Time."):
            time = float(ln.split("=")[1])
        if ln.strip().startswith("index") and "node" in ln:
            labels = ln.split()[2:]
            rows = []
            i += 1
            while i < len(lines) and lines[i].strip() and re.match(r"^\s*\d", lines[i]):
                rows.append([float(t) for t in lines[i].split()[2:]])
                i += 1
            out.append({"time": time, "labels": labels, "rows": rows})
            continue
        i += 1
    return out


def _parse_deck(path):
    root = ET.parse(path).getroot()
    d = {"geometry_file": root.get("geometry_file")}
    tm = root.find("time")
    d["nsteps"] = int(tm.get("num_steps"))
    d["dt"] = float(tm.get("time_step"))
    pts = tm.find("schedule_function/piecewise_linear")
    d["schedule"] = [[float(p.get("x")), float(p.get("y"))] for p in pts.findall("OrderedPair")]
    fld = root.find("nodes/field")
    d["kbc"] = [{"dof": int(k.get("dof")) - 1, "set": int(k.get("node_ID")),
                 "value": float(k.get("value", "0.0")),
                 "scheduled": k.get("schedule") is not None}
                for k in fld.findall("kinematic_BC")]
    d["fbc"] = [{"dof": int(k.get("dof")) - 1, "set": int(k.get("node_ID")),
                 "value": float(k.get("value", "0.0"))} for k in fld.findall("force_BC")]
    # torsion controller (TorsionKBCT.cpp:139-160): rigid turn of node sets
    # about a coordinate axis through a point, angle rotation_rate * t
    d["torsion"] = []
    for t in fld.findall("torsion"):
        pt = t.find("point_on_axis")
        d["torsion"].append({"axis": int(t.get("rotation_axis")) - 1, "rate": float(t.get("rotation_rate")),
                             "point": [float(pt.get("x_1")), float(pt.get("x_2")), float(pt.get("x_3"))],
                             "sets": [int(v.get("value")) for v in t.findall("node_ID_list/String")]})
    el = list(root.find("element_list"))[0]
    d["element"] = el.tag
    d["strain_displacement"] = el.get("strain_displacement", "standard")
    d["tractions"] = []
    for nb in el.findall("natural_bc"):
        vals = [float(v.get("value")) for v in nb.findall("DoubleList/Double")]
        d["tractions"].append({"side_set": int(nb.get("side_set_ID")), "t": vals})
    blk = el.find("small_strain_element_block")
    if blk is None:
        blk = el.find("large_strain_element_block")
    mat_holder = list(blk.find("small_strain_material_3D") if blk.find("small_strain_material_3D") is not None
                      else blk.find("large_strain_material_3D"))[0]
    d["material"] = parse_material(mat_holder)
    sol = solver_element(root)
    d["solver"] = {"rel_tol": float(sol.get("rel_tolerance", "1.0e-12")),
                   "abs_tol": float(sol.get("abs_tolerance", "1.0e-12")),
                   "max_its": int(sol.get("max_iterations", "1" if sol.tag.startswith("linear") else "25")),
                   "div_tol": float(sol.get("divergence_tolerance", "1.0e+10")),
                   "type": sol.tag, "matrix": solver_matrix(sol)}
    return d


# Solver names of the reference's solver factory (SolverT_factory.cpp:18-28).
# On the GPU path every one of them is served by the GPU Newton driver with
# the GPU global matrix (block CSR, PCG): the converged field is the same,
# so the deck's tolerances and iteration limits are kept and only the
# algorithm that reaches the field changes.
SOLVER_TYPES = ("linear_solver", "nonlinear_solver", "newton_krylov_solver", "PCG_solver", "nonlinear_solver_LS",
                "linear_solver_RS")


def solver_element(root):
    for name in SOLVER_TYPES:
        el = root.find(name)
        if el is not None:
            return el
    raise ValueError("deck has no solver (one of %s)" % ", ".join(SOLVER_TYPES))


def solver_matrix(sol):
    """Name of the global matrix chosen under the solver (profile_matrix,
    diagonal_matrix, SPOOLES_matrix, ...; SolverT.cpp:577-700), or None."""
    for child in sol:
        if child.tag.endswith("_matrix"):
            return child.tag
    return None


def _modulus_6x6(c):
    """The 6x6 modulus of a modulus_6x6 entry (C_i_j attributes, 1-based,
    mirrored when copy_symmetric is true)."""
    C = [[0.0] * 6 for _ in range(6)]
    for k, v in c.attrib.items():
        mm = re.match(r"C_(\d)_(\d)", k)
        if mm:
            i, j = int(mm.group(1)) - 1, int(mm.group(2)) - 1
            C[i][j] = float(v)
            if c.get("copy_symmetric", "false") == "true":
                C[j][i] = float(v)
    return C


def _e_nu(en):
    """Young's modulus and Poisson's ratio of an E_and_nu entry, rejected as
    IsotropicT::Set_E_nu rejects them (IsotropicT.cpp:32-44): E < 0 or nu
    outside [-1, 0.5]."""
    E, nu = float(en.get("Young_modulus")), float(en.get("Poisson_ratio"))
    if E < 0.0 or nu > 0.5 or nu < -1.0:
        raise ValueError("E_and_nu out of range: E=%g nu=%g" % (E, nu))
    return E, nu


def parse_material(m):
    name = m.tag
    en = m.find("E_and_nu")
    bs = m.find("bulk_and_shear")
    if name == "small_strain_Hookean":
        return {"kind": "ss_hookean", "C": _modulus_6x6(m.find("modulus_6x6"))}
    if name == "small_strain_StVenant":
        E, nu = _e_nu(en)
        return {"kind": "ss_hookean", "E": E, "nu": nu}
    if name == "small_strain_StVenant_J2":
        lf = m.find("linear_function")
        E, nu = _e_nu(en)
        return {"kind": "ss_j2", "E": E, "nu": nu,
                "a": float(lf.get("a")), "b": float(lf.get("b")),
                "elastic_iterations": int(m.get("elastic_iterations", "0"))}
    if name == "Simo_isotropic":
        if en is not None:
            E, nu = _e_nu(en)
            mu = 0.5 * E / (1.0 + nu)
            lam = 2.0 * mu * nu / (1.0 - 2.0 * nu)
            return {"kind": "fs_simo", "mu": mu, "kappa": lam + 2.0 / 3.0 * mu}
        return {"kind": "fs_simo", "mu": float(bs.get("shear_modulus")), "kappa": float(bs.get("bulk_modulus"))}
    if name == "large_strain_StVenant":
        E, nu = _e_nu(en)
        return {"kind": "fs_stvenant", "E": E, "nu": nu}
    if name == "large_strain_Hookean":
        # FDHookeanMatT (FDHookeanMatT.cpp:39-55): S = C : E(Green), pushed
        # forward: the St.Venant-Kirchhoff law; an isotropic modulus is
        # lambda = C_12, mu = C_44
        C = _modulus_6x6(m.find("modulus_6x6"))
        lam, mu = C[0][1], C[3][3]
        iso = [[(lam + 2.0 * mu if i == j else lam) if i < 3 and j < 3 else (mu if i == j else 0.0)
                for j in range(6)] for i in range(6)]
        if any(abs(C[i][j] - iso[i][j]) > 1e-12 * max(abs(lam), abs(mu)) for i in range(6) for j in range(6)):
            raise ValueError("large_strain_Hookean: only an isotropic modulus_6x6 is supported")
        E = mu * (3.0 * lam + 2.0 * mu) / (lam + mu)
        nu = lam / (2.0 * (lam + mu))
        return {"kind": "fs_stvenant", "E": E, "nu": nu}
    raise ValueError("unsupported material " + name)



class Deck:
    """A parsed deck: mesh (0-based connectivity), node and side sets,
    element group, material(s), boundary conditions, schedules, solver and
    time-stepping parameters."""

    def __init__(self, path):
        self.path = path
        d = _parse_deck(path)
        root = ET.parse(path).getroot()
        base = os.path.dirname(os.path.abspath(path))
        X, conn, self.nodesets, self.sidesets = read_geom(os.path.join(base, d["geometry_file"]))
        self.X = np.asarray(X, dtype=np.float64)
        self.conn = np.asarray(conn, dtype=np.int32)
        self.element = d["element"]
        self.strain_displacement = d["strain_displacement"]
        self.material = d["material"]
        self.nsteps, self.dt = d["nsteps"], d["dt"]
        tm = root.find("time")
        self.max_step_cuts = int(tm.get("max_step_cuts", "0"))
        # every schedule function, numbered from 1 in deck order
        self.schedules = {}
        for k, sf in enumerate(tm.findall("schedule_function"), start=1):
            pts = sf.find("piecewise_linear")
            self.schedules[k] = [[float(p.get("x")), float(p.get("y"))] for p in pts.findall("OrderedPair")]
        fld = root.find("nodes/field")
        self.kbc = [(int(k.get("dof")) - 1, int(k.get("node_ID")), float(k.get("value", "0.0")),
                     int(k.get("schedule", "0"))) for k in fld.findall("kinematic_BC")]
        self.fbc = [(int(k.get("dof")) - 1, int(k.get("node_ID")), float(k.get("value", "0.0")),
                     int(k.get("schedule", "1"))) for k in fld.findall("force_BC")]
        self.tractions = d["tractions"]
        self.torsion = d["torsion"]
        self.solver = d["solver"]
        sol = solver_element(root)
        self.quick_solve_iter = int(sol.get("quick_solve_iter", "6"))
        self.quick_solve_count = int(sol.get("quick_solve_count", "3"))

    @property
    def formulation(self):
        # the deck's own element group (ElementListT names)
        if self.element in ("small_strain", "total_lagrangian", "updated_lagrangian"):
            return self.element
        return "total_lagrangian"

    def model(self, device=0):
        """The deck as a GPU SolidModel (not yet set up)."""
        m = SolidModel(self.X, self.conn, self.formulation, self.material, device=device,
                       strain_displacement=self.strain_displacement)
        for k, pts in self.schedules.items():
            m.set_schedule(pts, k)
        for dof, ns, value, sched in self.kbc:
            for n in self.nodesets[ns]:
                m.add_kbc(n, dof, value, sched)
        scheds = {s for (_, _, _, s) in self.fbc}
        if len(scheds - {1}) > 0:
            raise ValueError("external forces follow schedule 1 on the GPU path")
        for dof, ns, value, _ in self.fbc:
            for n in self.nodesets[ns]:
                m.add_force(n, dof, value)
        for t in self.tractions:
            for (e, facet) in self.sidesets[t["side_set"]]:
                m.add_traction(e, facet, t["t"])
        for tc in self.torsion:
            nodes = sorted({n for ns in tc["sets"] for n in self.nodesets[ns]})
            m.add_torsion(tc["axis"], tc["rate"], tc["point"], nodes)
        return m


def run_deck(path, precision=lib.FP64, lin_rel_tol=1e-12, lin_max_it=50000, device=0, material_output=None):
    """Runs a deck through the GPU step loop; returns the deck and, per output
    step, (time, displacements, nodal stresses, nodal material output or
    None).  Output is formed before each step is closed, as the reference
    writes it (FEManagerT::CloseStep, FEManagerT.cpp:625-645)."""
    deck = Deck(path)
    m = deck.model(device)
    sv = deck.solver
    want_mat = (deck.material.get("kind") == "ss_j2") if material_output is None else material_output
    out = []
    at = {}

    def on_step(step, ctx):
        # output at the original step ends only (sub-steps of a cut step are
        # not written)
        k = int(round(m.current_time / deck.dt))
        if k >= 1 and abs(m.current_time - k * deck.dt) <= 1e-9 * deck.dt:
            at[k] = (ctx.nodal_stress(), ctx.nodal_material_output() if want_mat else None)

    hist, reps = m.run(deck.nsteps, deck.dt, rel_tol=sv["rel_tol"], abs_tol=sv["abs_tol"],
                       max_iterations=sv["max_its"], div_tol=sv["div_tol"], precision=precision,
                       lin_rel_tol=lin_rel_tol, lin_max_it=lin_max_it, on_step=on_step,
                       max_step_cuts=deck.max_step_cuts, quick_solve_iter=deck.quick_solve_iter,
                       quick_solve_count=deck.quick_solve_count)
    for k in range(deck.nsteps):
        sig, mat = at[k + 1]
        out.append(((k + 1) * deck.dt, hist[k], sig, mat))
    m.ctx.close()
    return deck, out


def write_run(path, deck, results, labels_mat=("alpha", "VM", "press")):
    """Nodal output in the layout of the reference's ``.run`` files (the
    "O U T P U T   D A T A" blocks: index, node, D_X D_Y D_Z, s11..s12 and
    any material output), one block per output step."""
    labels = ["D_X", "D_Y", "D_Z", "s11", "s22", "s33", "s23", "s13", "s12"]
    if results and results[0][3] is not None:
        labels += list(labels_mat)
    nnd, nel = deck.X.shape[0], deck.conn.shape[0]
    dots = lambda s: (s + " " + ". " * 30)[:48] + "= "
    with open(path, "w") as f:
        f.write("\n S U M M A R Y :\n\n")
        f.write(" %s%d\n" % (dots("Group number."), 1))
        f.write(" %s%d\n" % (dots("Number of nodal values."), len(labels)))
        f.write(" Labels:\n")
        for lb in labels:
            f.write("\t%s\n" % lb)
        f.write(" %s%d\n" % (dots("Number of nodes"), nnd))
        f.write(" %s%d\n\n" % (dots("Number of elements."), nel))
        f.write(" O U T P U T   D A T A :\n\n")
        for step, (t, u, sig, mat) in enumerate(results):
            f.write(" %s%d\n" % (dots("Print Step."), step))
            f.write(" %s%.12e\n\n" % (dots("Time."), t))
            f.write(" Nodal data:\n")
            f.write(" %s%d\n" % (dots("Number of nodal points."), nnd))
            f.write(" %s%d\n\n" % (dots("Number of values."), len(labels)))
            f.write("   index    node" + "".join("%21s" % lb for lb in labels) + "\n")
            for n in range(nnd):
                row = list(u[n]) + list(sig[n]) + (list(mat[n]) if mat is not None else [])
                f.write("%8d%8d" % (n + 1, n + 1) + "".join("%21.12e" % v for v in row) + "\n")
            f.write("\n")
