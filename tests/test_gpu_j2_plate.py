"""J2 active set at scale: the 48 x 48 x 24 plate (55,296 elements, 442,368
Gauss points) through the first six steps of the configuration-3 cycle with
load-step cuts, the plain FP64 GPU path against the oracle's committed
results (tests/golden/make_j2_plate.py, same mesh, material, load history and
solver settings):

  * the same number of step cuts and the same Newton iterations per step
    (failed attempts included);
  * the full per-point flag array bit-exact -- plastic, elastic, reset and
    unallocated, so element allocation (which records transient yields of
    intermediate Newton iterates, J2SSC0HardeningT::AllocateElement) is
    compared too;
  * equivalent plastic strain at 4,096 sampled points and the displacements
    at 2,048 sampled nodes after every step within 1e-8.

The mixed form (FP32 tangent and inner PCG) runs the same history: the same
cuts and the same yielding set (points plastic or reset after the last
step); its raw flag array may differ only in allocation, which follows the
iterates it takes."""
import os

import numpy as np
import pytest

from tahoe_gb300 import lib, workloads
from tests.helpers import GOLDEN, rel_err

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(GOLDEN, "j2_plate_48x48x24.npz")


def _run(fx, precision, lin_rel_tol):
    nx, ny, nz, nsched, steps = (int(v) for v in fx["dims"])
    _, g, _ = workloads.c3(nx=nx, ny=ny, nz=nz, nsteps=nsched)
    hist, reps = g.run(steps, 1.0, rel_tol=1e-8, abs_tol=1e-10, max_iterations=25, div_tol=1e3, precision=precision,
                       lin_rel_tol=lin_rel_tol, lin_max_it=50000, max_step_cuts=6, quick_solve_iter=0)
    alpha, _ = g.ctx.j2_state()
    out = dict(hist=hist, cuts=g.step_cuts, newton=list(g.newton_per_step), flags=g.ctx.active_set().reshape(-1),
               alpha=alpha.reshape(-1))
    g.ctx.close()
    return out


@pytest.fixture(scope="module")
def fx():
    return np.load(FIXTURE)


def test_fp64_flags_bit_exact_against_oracle(fx):
    r = _run(fx, lib.FP64, 1e-12)
    assert r["cuts"] == int(fx["cuts"])
    assert r["newton"] == [int(v) for v in fx["newton"]]
    assert np.array_equal(r["flags"], fx["flags"])
    assert rel_err(r["alpha"][fx["sample_points"]], fx["alpha_sample"]) < 1e-8
    assert abs(r["alpha"].sum() - float(fx["alpha_sum"])) <= 1e-8 * float(fx["alpha_sum"])
    assert rel_err(r["hist"][:, fx["sample_nodes"], :], fx["u_sample"]) < 1e-8
    assert rel_err(np.linalg.norm(r["hist"].reshape(len(r["hist"]), -1), axis=1), fx["u_norm"]) < 1e-9


def test_mixed_same_cuts_and_yielding_set(fx):
    r = _run(fx, lib.MIXED, 1e-6)
    assert r["cuts"] == int(fx["cuts"])
    ref = fx["flags"]
    yielding = (r["flags"] == lib.J2_PLASTIC) | (r["flags"] == lib.J2_RESET)
    yielding_ref = (ref == lib.J2_PLASTIC) | (ref == lib.J2_RESET)
    assert np.array_equal(yielding, yielding_ref)
    assert rel_err(r["hist"][:, fx["sample_nodes"], :], fx["u_sample"]) < 1e-6
