"""CPU-side checks of the product library: it builds for sm_103a, loads, and
exports every entry point the public header declares; host logic (equation
numbering, mesh generation, schedules) against the oracle."""
import ctypes
import os
import re

import numpy as np

from tahoe_gb300 import build, lib
from tahoe_gb300.meshgen import BoxMesh, equations
from tahoe_gb300.model import schedule_value
from tests.helpers import cube_case, load_fixture, oracle_for

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            with open(os.path.join(ROOT, "include", fn)) as f:
                text = f.read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(tg_[a-z0-9_]+)\s*\(", text))
    return syms


def test_library_builds_and_exports_header_symbols():
    path = build.build()
    assert os.path.exists(path)
    L = ctypes.CDLL(path)
    missing = [s for s in sorted(header_symbols()) if not hasattr(L, s)]
    assert not missing, missing
    # the Python binding covers the same set
    assert header_symbols() == set(lib.exported_symbols())


def test_equation_numbering_matches_oracle():
    m, fixed = cube_case(3, jitter=0.1, seed=3)
    o = oracle_for(m, "small_strain", {"kind": "ss_hookean", "E": 1.0, "nu": 0.3}, fixed)
    eq_o, neq = o.equations()
    eq = equations(m.nnd, [n * 3 + d for n, d in fixed])
    assert np.array_equal(eq, eq_o)
    assert eq.max() == neq


def test_meshgen_connectivity_positive_volume():
    m = BoxMesh(3, 2, 4, lx=2.0, ly=1.0, lz=0.5, jitter=0.2, seed=1)
    assert m.nnd == 4 * 3 * 5 and m.nel == 24
    # every element has positive Jacobian at its centre (oracle check)
    o = oracle_for(m, "small_strain", {"kind": "ss_hookean", "E": 1.0, "nu": 0.3}, [])
    for e in range(m.nel):
        o.element(e, np.zeros(m.nnd * 3))


def test_schedule_matches_reference_piecewise_linear():
    pts = [(0.0, 0.0), (2.0, 0.2)]
    assert schedule_value(pts, -1.0) == 0.0
    assert abs(schedule_value(pts, 1.5) - 0.15) < 1e-15
    assert schedule_value(pts, 3.0) == 0.2
    assert schedule_value([(0.0, 1.0)], 5.0) == 1.0


def test_golden_fixture_loads_into_model_driver():
    from tahoe_gb300.model import model_from_fixture
    fx = load_fixture("traction_a_cube")
    m = model_from_fixture(fx)
    eq = m.equations()
    assert eq.shape == (len(fx["X"]), 3)
    assert len(m.tractions) == 4
