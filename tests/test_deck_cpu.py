"""Deck glue on the host (no GPU): the TahoeII geometry and XML deck readers
on the repository's own test decks, the model they describe, and the .run
writer read back by the .run reader."""
import os

import numpy as np

from tahoe_gb300 import deck as dk
from tahoe_gb300.meshgen import BoxMesh

DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks")


def test_geometry_reader():
    X, conn, nodesets, sidesets = dk.read_geom(os.path.join(DECKS, "cube8.geom"))
    m = BoxMesh(2, 2, 2)
    assert np.allclose(X, m.X) and np.array_equal(np.asarray(conn), m.conn)
    assert sorted(nodesets[1]) == sorted(m.face_nodes(2, 0).tolist())
    assert sorted(nodesets[2]) == sorted(m.face_nodes(2, 1).tolist())
    el, fc = m.face_facets(0, 1)
    assert sorted(sidesets[1]) == sorted(zip(el.tolist(), fc.tolist()))


def test_deck_to_model():
    d = dk.Deck(os.path.join(DECKS, "cube8_j2.xml"))
    assert d.formulation == "small_strain" and d.material["kind"] == "ss_j2"
    assert d.nsteps == 3 and d.dt == 1.0 and d.max_step_cuts == 3
    m = d.model()
    # 9 bottom nodes x 3 fixed dofs + 9 top nodes prescribed in z (schedule 1)
    assert len(m.kbc) == 36
    assert sum(1 for k in m.kbc if k[3] == 1) == 9 and all(k[2] == -0.006 for k in m.kbc if k[3] == 1)
    eq = m.equations()
    assert (eq > 0).sum() == 27 * 3 - 36
    t = dk.Deck(os.path.join(DECKS, "cube8_tl_traction.xml"))
    mt = t.model()
    assert mt.formulation == 1 and len(mt.forces) == 9 and len(mt.tractions) == 4


def test_run_file_round_trip(tmp_path):
    d = dk.Deck(os.path.join(DECKS, "cube8_j2.xml"))
    rng = np.random.default_rng(0)
    res = [(float(k + 1), rng.standard_normal((27, 3)), rng.standard_normal((27, 6)), rng.standard_normal((27, 3)))
           for k in range(2)]
    path = str(tmp_path / "out.run")
    dk.write_run(path, d, res)
    back = dk.read_run(path)
    assert len(back) == 2
    for (t, u, s, mo), b in zip(res, back):
        assert b["time"] == t
        assert b["labels"] == ["D_X", "D_Y", "D_Z", "s11", "s22", "s33", "s23", "s13", "s12", "alpha", "VM", "press"]
        assert np.allclose(np.array(b["rows"]), np.hstack([u, s, mo]), rtol=1e-11, atol=1e-300)


def test_every_solver_type_of_the_reference_factory_is_accepted():
    """Each solver name the reference's solver factory registers is read with
    its tolerances and matrix choice; the GPU Newton driver serves them all."""
    import xml.etree.ElementTree as ET
    for name in dk.SOLVER_TYPES:
        root = ET.fromstring('<tahoe><%s abs_tolerance="1e-9" rel_tolerance="1e-11" max_iterations="7" '
                             'divergence_tolerance="5"><SPOOLES_matrix/></%s></tahoe>' % (name, name))
        sol = dk.solver_element(root)
        assert sol.tag == name and dk.solver_matrix(sol) == "SPOOLES_matrix"
    try:
        dk.solver_element(ET.fromstring("<tahoe/>"))
        raise AssertionError("a deck without a solver is rejected")
    except ValueError:
        pass


def test_isotropic_constants_follow_the_reference_unit_tests():
    """The relations the reference's tests/materials/test_IsotropicT.cpp
    checks: mu = E/(2(1+nu)), lambda = 2 mu nu/(1-2nu), E = 9 kappa mu /
    (3 kappa + mu); negative E and nu above 0.5 rejected."""
    import xml.etree.ElementTree as ET
    simo = dk.parse_material(ET.fromstring(
        '<Simo_isotropic><E_and_nu Young_modulus="200.0e9" Poisson_ratio="0.3"/></Simo_isotropic>'))
    mu = 200.0e9 / (2.0 * 1.3)
    lam = 2.0 * mu * 0.3 / (1.0 - 0.6)
    assert abs(simo["mu"] - mu) <= 1.0
    assert abs(simo["kappa"] - (lam + 2.0 / 3.0 * mu)) <= 1.0
    E = 9.0 * simo["kappa"] * simo["mu"] / (3.0 * simo["kappa"] + simo["mu"])
    assert abs(E - 200.0e9) <= 1.0e3
    for E_, nu_ in ((-1.0, 0.3), (100.0, 0.6)):
        try:
            dk.parse_material(ET.fromstring('<small_strain_StVenant><E_and_nu Young_modulus="%g" '
                                            'Poisson_ratio="%g"/></small_strain_StVenant>' % (E_, nu_)))
            raise AssertionError("E=%g nu=%g accepted" % (E_, nu_))
        except ValueError:
            pass


def test_large_strain_hookean_reads_as_st_venant_or_is_rejected():
    """An isotropic modulus_6x6 (C11 = lambda + 2 mu, C12 = lambda, C44 = mu)
    becomes the St.Venant-Kirchhoff material; any other modulus is refused."""
    import xml.etree.ElementTree as ET
    iso = ('<large_strain_Hookean><modulus_6x6 C_1_1="30.0" C_1_2="10.0" C_1_3="10.0" C_2_2="30.0" C_2_3="10.0" '
           'C_3_3="30.0" C_4_4="10.0" C_5_5="10.0" C_6_6="10.0" copy_symmetric="true"/></large_strain_Hookean>')
    m = dk.parse_material(ET.fromstring(iso))
    assert m == {"kind": "fs_stvenant", "E": 25.0, "nu": 0.25}
    try:
        dk.parse_material(ET.fromstring(iso.replace('C_4_4="10.0"', 'C_4_4="12.0"')))
        raise AssertionError("anisotropic modulus accepted")
    except ValueError:
        pass


def test_torsion_controller_is_read_and_mapped_onto_the_model(tmp_path):
    """A deck with the reference's torsion controller: the axis, rate, point
    and node sets are read, and the GPU model prescribes the two dofs across
    the axis of every node of the sets with the rigid turn of its initial
    position (distance to the axis kept, angle rate * t; TorsionKBCT)."""
    import shutil
    with open(os.path.join(DECKS, "cube8_j2.xml")) as f:
        xml = f.read()
    shutil.copy(os.path.join(DECKS, "cube8.geom"), tmp_path / "cube8.geom")
    tors = ('<torsion rotation_axis="3" rotation_rate="0.5"><point_on_axis x_1="0.5" x_2="0.5" x_3="0.0"/>'
            '<node_ID_list><String value="2"/></node_ID_list></torsion>')
    xml = xml.replace("</field>", tors + "</field>", 1)
    path = tmp_path / "torsion.xml"
    path.write_text(xml)
    d = dk.Deck(str(path))
    assert d.torsion == [{"axis": 2, "rate": 0.5, "point": [0.5, 0.5, 0.0], "sets": [2]}]
    m = d.model()
    nodes = sorted(d.nodesets[2])
    assert len(m.torsions) == 1 and list(m.torsions[0][3]) == nodes
    idx = m._torsion_dofs()
    assert idx == [n * 3 + dd for n in nodes for dd in (0, 1)]
    eq = m.equations()
    assert all(eq.reshape(-1)[i] <= 0 for i in idx)  # prescribed
    t = 0.7
    u = m._torsion_values(t).reshape(-1, 2)
    X = d.X[nodes]
    r0 = X[:, :2] - 0.5
    r1 = r0 + u
    assert np.allclose(np.linalg.norm(r1, axis=1), np.linalg.norm(r0, axis=1), atol=1e-14)
    turned = np.linalg.norm(r0, axis=1) > 1e-12
    ang = np.arctan2(r1[:, 1], r1[:, 0]) - np.arctan2(r0[:, 1], r0[:, 0])
    ang = (ang + np.pi) % (2 * np.pi) - np.pi
    assert np.allclose(ang[turned], 0.5 * t, atol=1e-13)
    assert np.all(u[~turned] == 0.0)
