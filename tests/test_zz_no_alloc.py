"""The no-allocation PCG entry point, checked against the allocating one.

tg_pcg_solve_noalloc serves callers that cannot allocate device memory: hosts
that reserve all device memory themselves up front, or whose request path must
not enter the CUDA allocator.  It keeps its work vectors in a fixed static
device array (meshes up to 32,768 nodes) and runs the two-kernel form of the
PCG.  This test calls it through the C ABI on caller-owned device buffers,
twice in a row, and compares each result with tg_pcg_solve in the same form
on the same tangent and right-hand side.  The file name sorts
last so a run that stops at the first failure has run every other test.
"""
import numpy as np
import pytest

from tahoe_gb300 import lib
from tahoe_gb300.meshgen import BoxMesh
from tahoe_gb300.model import SolidModel

pytestmark = pytest.mark.gpu

SIMO = {"kind": "fs_simo", "mu": 1.0, "kappa": 10.0}


def _model():
    mesh = BoxMesh(8, 8, 8, jitter=0.2, seed=5)
    m = SolidModel(mesh.X, mesh.conn, "total_lagrangian", SIMO)
    for n in mesh.face_nodes(2, 0):
        for d in range(3):
            m.add_kbc(n, d)
    for n in mesh.face_nodes(2, 1):
        m.add_kbc(n, 2, -0.01, True)
    m.set_schedule([(0.0, 1.0)])
    m.setup()
    return mesh, m


@pytest.mark.parametrize("precision", [lib.FP64, lib.MIXED])
@pytest.mark.parametrize("precond", [lib.PRECOND_JACOBI, lib.PRECOND_BLOCK_JACOBI])
def test_noalloc_solve_matches_allocating_solve_twice(precision, precond):
    torch = pytest.importorskip("torch")
    mesh, m = _model()
    c = m.ctx
    m.apply_step(1.0, (precision, precond, 1e-8))
    c.set_iteration(-1)
    R, _ = c.residual()
    c.tangent(precision)
    # the scratch solve runs the two-kernel recurrences: compare like with like
    c.pcg_form(0)
    du_ref, its_ref, rr_ref, rc = c.pcg(R, rel_tol=1e-8, max_it=5000, precond=precond)
    assert rc == 0
    d_rhs = torch.tensor(R, dtype=torch.float64, device="cuda:0")
    for call in range(2):
        d_du = torch.full((c.neq,), float("nan"), dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        its, rr, rc = c.pcg_noalloc(d_rhs.data_ptr(), d_du.data_ptr(), rel_tol=1e-8, max_it=5000, precond=precond)
        assert rc == 0, call
        du = d_du.cpu().numpy()
        assert its == its_ref
        scale = np.abs(du_ref).max()
        assert np.abs(du - du_ref).max() <= 1e-12 * scale, call


def test_noalloc_rejects_meshes_above_the_scratch_limit():
    torch = pytest.importorskip("torch")
    mesh = BoxMesh(32, 32, 32)  # 35,937 nodes > 32,768
    m = SolidModel(mesh.X, mesh.conn, "small_strain", {"kind": "ss_hookean", "E": 1.0, "nu": 0.3})
    for n in mesh.face_nodes(2, 0):
        for d in range(3):
            m.add_kbc(n, d)
    m.setup()
    m.ctx.tangent(lib.MIXED)
    d_rhs = torch.zeros(m.ctx.neq, dtype=torch.float64, device="cuda:0")
    d_du = torch.zeros(m.ctx.neq, dtype=torch.float64, device="cuda:0")
    with pytest.raises(lib.TahoeError) as ei:
        m.ctx.pcg_noalloc(d_rhs.data_ptr(), d_du.data_ptr())
    assert ei.value.code == -8
