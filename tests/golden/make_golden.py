"""Extract golden parity fixtures from the reference's regression suite.

Runs only where the reference source tree is mounted (it is read, never
modified).  For each selected benchmark deck it records, as compact JSON under
tests/golden/:

  * the mesh (from the deck's TahoeII ``.geom`` file),
  * boundary conditions, load schedule, material and solver tolerances
    (from the XML deck),
  * the nodal results of every output step (from the committed ``.run`` /
    ``.run.psNNNN`` golden files of the reference suite).

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT   (the reference source tree)
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

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
    ("mat01_ssstvenant_cube", "level.1/material.solid/3D/material.01/mat.1.a.xml",
     ["benchmark/mat.1.a.io0.run"]),
    ("mat02_fsstvenant_cube", "level.1/material.solid/3D/material.02/mat.2.a.xml",
     ["benchmark/mat.2.a.io0.run"]),
    ("mat25_fshookean_cube", "level.1/material.solid/3D/material.25/mat.25.a.xml",
     ["benchmark/mat.25.a.io0.run.ps0000", "benchmark/mat.25.a.io0.run.ps0001"]),
    # the same beam with the other solver / matrix choices of the deck
    ("beam_pcg_diagonal", "level.0/3D.elastostatic/beam.PCG.xml", ["benchmark/beam.PCG.io0.run"]),
    ("beam_pcg_profile", "level.0/3D.elastostatic/beam.PCG.K.xml", ["benchmark/beam.PCG.K.io0.run"]),
    ("beam_quasi_newton", "level.0/3D.elastostatic/beam.quasi-Newton.xml", ["benchmark/beam.quasi-Newton.io0.run"]),
    ("beam_newton_totlag_store", "level.0/3D.elastostatic/beam.Newton.TotLag.store.xml",
     ["benchmark/beam.Newton.TotLag.store.io0.run"]),
    # finite rotations: one end of two stacked cubes turned about z (y) by
    # the torsion controller, the other end pinned
    ("torsion_z", "level.2/torsion/torsion.z.xml", ["benchmark/torsion.z.io0.run"]),
    ("torsion_y", "level.2/torsion/torsion.y.xml", ["benchmark/torsion.y.io0.run"]),
]


from tahoe_gb300.deck import _parse_deck as parse_deck, parse_material, read_geom as parse_geom, \
    read_run as parse_run  # noqa: E402


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
        torsion = []
        for t in d["torsion"]:
            nodes = sorted({n for ns in t["sets"] for n in nodesets[ns]})
            torsion.append([t["axis"], t["rate"]] + t["point"] + [nodes])
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
            "kbc": kbc, "forces": forces, "tractions": tractions, "torsion": torsion,
            "schedule": d["schedule"], "nsteps": d["nsteps"], "dt": d["dt"],
            "solver": d["solver"],
            "outputs": outputs,
        }
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(fx, f, indent=None, separators=(",", ":"))
        print(name, len(X), "nodes", len(conn), "elements", len(outputs), "outputs")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference source tree>")
    make(sys.argv[1])
