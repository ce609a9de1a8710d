"""Extract golden parity fixtures from the reference's regression suite.

Runs only where the reference source tree is mounted (it is read, never
modified).  For each selected benchmark deck it records, as compact JSON under
tests/golden/:

  * the mesh (from the deck's TahoeII ``.geom`` file),
  * boundary conditions, load schedule, material and solver tolerances
    (from the XML deck),
  * the nodal results of every output step (from the committed ``.run`` /
    ``.run.psNNNN`` golden files of the reference suite).

Usage:  python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
import json
import os
import re
import sys
import xml.etree.ElementTree as ET

HERE = os.path.dirname(os.path.abspath(__file__))

# (fixture name, deck path relative to benchmark_XML, golden output files)
DECKS = [
    ("mat08_j2_cube", "level.1/material.solid/3D/material.08/mat.8.a.xml",
     ["benchmark/mat.8.a.io0.run.ps0000", "benchmark/mat.8.a.io0.run.ps0001",
      "benchmark/mat.8.a.io0.run.ps0002"]),
    ("mat24_hookean_cube", "level.1/material.solid/3D/material.24/mat.24.a.xml",
     ["benchmark/mat.24.a.io0.run.ps0000", "benchmark/mat.24.a.io0.run.ps0001"]),
    ("mat05_simo_cube", "level.1/material.solid/3D/material.05/mat.5.a.xml",
     ["benchmark/mat.5.a.io0.run"]),
    ("traction_a_cube", "level.0/3D.elastostatic/traction.a.xml",
     ["benchmark/traction.a.io0.run"]),
    ("beam_newton_totlag", "level.0/3D.elastostatic/beam.Newton.TotLag.xml",
     ["benchmark/beam.Newton.TotLag.io0.run"]),
    ("beam_newton_updlag", "level.0/3D.elastostatic/beam.Newton.xml",
     ["benchmark/beam.Newton.io0.run"]),
    ("beam_bbar", "level.0/3D.elastostatic/beam.B_bar.xml",
     ["benchmark/beam.B_bar.io0.run"]),
]


def _tokens(lines):
    for ln in lines:
        ln = ln.split("#", 1)[0].strip()
        if ln:
            for t in ln.split():
                yield t


def parse_geom(path):
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


def parse_run(path):
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


def parse_deck(path):
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
    sol = root.find("nonlinear_solver")
    d["solver"] = {"rel_tol": float(sol.get("rel_tolerance")), "abs_tol": float(sol.get("abs_tolerance")),
                   "max_its": int(sol.get("max_iterations")), "div_tol": float(sol.get("divergence_tolerance"))}
    return d


def parse_material(m):
    name = m.tag
    en = m.find("E_and_nu")
    bs = m.find("bulk_and_shear")
    if name == "small_strain_Hookean":
        c = m.find("modulus_6x6")
        C = [[0.0] * 6 for _ in range(6)]
        for k, v in c.attrib.items():
            mm = re.match(r"C_(\d)_(\d)", k)
            if mm:
                i, j = int(mm.group(1)) - 1, int(mm.group(2)) - 1
                C[i][j] = float(v)
                if c.get("copy_symmetric", "false") == "true":
                    C[j][i] = float(v)
        return {"kind": "ss_hookean", "C": C}
    if name == "small_strain_StVenant":
        return {"kind": "ss_hookean", "E": float(en.get("Young_modulus")), "nu": float(en.get("Poisson_ratio"))}
    if name == "small_strain_StVenant_J2":
        lf = m.find("linear_function")
        return {"kind": "ss_j2", "E": float(en.get("Young_modulus")), "nu": float(en.get("Poisson_ratio")),
                "a": float(lf.get("a")), "b": float(lf.get("b")),
                "elastic_iterations": int(m.get("elastic_iterations", "0"))}
    if name == "Simo_isotropic":
        if en is not None:
            E, nu = float(en.get("Young_modulus")), float(en.get("Poisson_ratio"))
            mu = 0.5 * E / (1.0 + nu)
            lam = 2.0 * mu * nu / (1.0 - 2.0 * nu)
            return {"kind": "fs_simo", "mu": mu, "kappa": lam + 2.0 / 3.0 * mu}
        return {"kind": "fs_simo", "mu": float(bs.get("shear_modulus")), "kappa": float(bs.get("bulk_modulus"))}
    if name == "large_strain_StVenant":
        return {"kind": "fs_stvenant", "E": float(en.get("Young_modulus")), "nu": float(en.get("Poisson_ratio"))}
    raise ValueError("unsupported material " + name)


def make(ref_root):
    bx = os.path.join(ref_root, "benchmark_XML")
    for name, deck_rel, runs in DECKS:
        deck_path = os.path.join(bx, deck_rel)
        deck_dir = os.path.dirname(deck_path)
        d = parse_deck(deck_path)
        X, conn, nodesets, sidesets = parse_geom(os.path.join(deck_dir, d["geometry_file"]))
        kbc = []
        for k in d["kbc"]:
            for n in nodesets[k["set"]]:
                kbc.append([n, k["dof"], k["value"], int(k["scheduled"])])
        forces = []
        for f in d["fbc"]:
            for n in nodesets[f["set"]]:
                forces.append([n, f["dof"], f["value"]])
        tractions = []
        for t in d["tractions"]:
            for (e, facet) in sidesets[t["side_set"]]:
                tractions.append([e, facet] + t["t"])
        outputs = []
        for r in runs:
            outputs.extend(parse_run(os.path.join(deck_dir, r)))
        form = "small_strain" if d["element"] == "small_strain" else "total_lagrangian"
        fx = {
            "name": name,
            "source": "benchmark_XML/" + deck_rel,
            "reference_element": d["element"],
            "strain_displacement": d["strain_displacement"],
            "formulation": form,
            "X": X, "conn": conn,
            "material": d["material"],
            "kbc": kbc, "forces": forces, "tractions": tractions,
            "schedule": d["schedule"], "nsteps": d["nsteps"], "dt": d["dt"],
            "solver": d["solver"],
            "outputs": outputs,
        }
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(fx, f, indent=None, separators=(",", ":"))
        print(name, len(X), "nodes", len(conn), "elements", len(outputs), "outputs")


if __name__ == "__main__":
    make(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
