"""Decks run on the GPU path end to end (reader -> model -> step loop ->
.run output) against the oracle driven from the same deck: displacements,
nodal stresses and J2 material output at every output step."""
import os

import numpy as np
import pytest

from oracle.pyoracle import OracleModel
from tahoe_gb300 import deck as dk
from tahoe_gb300 import lib
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks")


def oracle_from_deck(d):
    o = OracleModel(d.X, d.conn, d.formulation, [d.material], bbar=d.strain_displacement == "B-bar")
    o.set_schedule(d.schedules[1])
    for dof, ns, value, sched in d.kbc:
        for n in d.nodesets[ns]:
            o.add_kbc(n, dof, value, sched >= 1)
    for dof, ns, value, _ in d.fbc:
        for n in d.nodesets[ns]:
            o.add_force(n, dof, value)
    for t in d.tractions:
        for (e, facet) in d.sidesets[t["side_set"]]:
            o.add_traction(e, facet, t["t"])
    return o


@pytest.mark.parametrize("name", ["cube8_j2.xml", "cube8_tl_traction.xml"])
def test_deck_on_gpu_matches_oracle(name, tmp_path):
    path = os.path.join(DECKS, name)
    d, res = dk.run_deck(path, precision=lib.FP64)
    o = oracle_from_deck(d)
    sv = d.solver
    st, uh, its, cuts, sh = o.run_cuts(d.nsteps, d.dt, sv["rel_tol"], sv["abs_tol"], sv["max_its"], sv["div_tol"], 0,
                                       max_cuts=d.max_step_cuts, quick_iter=d.quick_solve_iter,
                                       quick_count=d.quick_solve_count, want_stress=True)
    assert st == 0
    for k, (t, u, sig, mat) in enumerate(res):
        assert rel_err(u, uh[k]) < 1e-9, k
        assert rel_err(sig, sh[k]) < 1e-9, k
        if mat is not None:
            assert rel_err(mat, o.material_output_hist[k]) < 1e-9, k
    if d.material["kind"] == "ss_j2":
        assert res[-1][3][:, 0].max() > 0.0  # plastic flow happened
    out = str(tmp_path / "gpu.run")
    dk.write_run(out, d, res)
    back = dk.read_run(out)
    assert len(back) == d.nsteps and np.allclose(np.array(back[-1]["rows"])[:, :3], res[-1][1], rtol=1e-11)
