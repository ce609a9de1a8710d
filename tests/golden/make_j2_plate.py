"""Oracle fixture of the J2 plate at the active-set parity size.

The configuration-3 physics (small-strain J2, E 200e3, nu 0.3, yield 250,
H 1000; x=0 clamped, x=L gripped with u_x following the 40-step +-0.5 %
strain cycle) on a 48 x 48 x 24 plate, the first six load steps, run by the
CPU oracle through the reference's step sequence with load-step cuts (Newton
to 1e-8, Jacobi CG to 1e-12, at most 6 cuts, no step doubling).  The oracle
takes minutes here, so its results are committed for the GPU test
(tests/test_gpu_j2_plate.py): the full per-point flag array after the last
step (plastic / elastic / reset / unallocated), the number of cuts and the
Newton iterations per step, the equivalent plastic strain and the
displacements at a seeded sample of points and nodes with their norms.

Usage:  python tests/golden/make_j2_plate.py     (about 7 minutes on 8 threads)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.pyoracle import OracleModel  # noqa: E402
from tahoe_gb300 import workloads  # noqa: E402

NX, NY, NZ = 48, 48, 24
SCHEDULE_STEPS = 40     # the 40-step cycle of the benchmark configuration
STEPS = 6               # load steps run
SOLVER = dict(rel_tol=1e-8, abs_tol=1e-10, max_its=25, div_tol=1e3, lin_tol=1e-12, max_cuts=6, quick_iter=0,
              quick_count=3)
OUT = os.path.join(HERE, "j2_plate_48x48x24.npz")


def make(threads=8):
    mesh, o, _ = workloads.c3(nx=NX, ny=NY, nz=NZ, nsteps=SCHEDULE_STEPS,
                              add=lambda X, conn, form, mat: OracleModel(X, conn, form, [mat], threads=threads))
    t0 = time.time()
    st, uh, its, cuts = o.run_cuts(STEPS, 1.0, SOLVER["rel_tol"], SOLVER["abs_tol"], SOLVER["max_its"],
                                   SOLVER["div_tol"], 1, SOLVER["lin_tol"], max_cuts=SOLVER["max_cuts"],
                                   quick_iter=SOLVER["quick_iter"], quick_count=SOLVER["quick_count"])
    if st != 0:
        raise RuntimeError("oracle run failed at step %d" % st)
    flags, alpha, _ = o.j2_state()
    rng = np.random.default_rng(2024)
    pts = np.sort(rng.choice(flags.size, size=4096, replace=False))
    nodes = np.sort(rng.choice(mesh.nnd, size=2048, replace=False))
    np.savez_compressed(
        OUT, flags=flags.reshape(-1).astype(np.int8), cuts=np.int32(cuts), newton=np.asarray(its, np.int32),
        sample_points=pts.astype(np.int64), alpha_sample=alpha.reshape(-1)[pts],
        alpha_sum=np.float64(alpha.sum()), alpha_max=np.float64(alpha.max()),
        sample_nodes=nodes.astype(np.int64), u_sample=uh[:, nodes, :],
        u_norm=np.linalg.norm(uh.reshape(STEPS, -1), axis=1),
        dims=np.array([NX, NY, NZ, SCHEDULE_STEPS, STEPS], np.int32))
    print("cuts", cuts, "newton", list(its), "flags", {k: int((flags == k).sum()) for k in (0, 1, 3, 7)},
          "%.0f s" % (time.time() - t0), "->", OUT)


if __name__ == "__main__":
    make()
