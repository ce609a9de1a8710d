"""The sparsity pattern against the reference's own code.

oracle/_ref/ref_msr is the reference's MSR structure builder (MSRBuilderT and
the toolbox classes it uses, compiled from the reference's sources by
oracle/build.py) driven as MSRMatrixT drives it (AddGroup with the element
equation sets, SetMSRData for the active rows; MSRMatrixT.cpp:53,633-649).
The library's pattern (tg_pattern_build_host, the code tg_pattern_build runs
on a context) must equal its MSR array bit for bit -- row lengths and every
off-diagonal column -- for the upper (symmetric) and the full pattern, on the
benchmark meshes at full size.  Skipped where the reference tree was not
present when the oracle was built.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import build as ob
from tahoe_gb300 import lib, workloads


def _ref_msr(tmp_path, elem_eq, neq, upper):
    exe = ob.build_ref()
    if exe is None:
        pytest.skip("the reference's MSR builder is not built here (no reference source tree)")
    inp, out = tmp_path / "eq.bin", tmp_path / "msr.bin"
    with open(inp, "wb") as f:
        np.array([int(upper), elem_eq.shape[0], elem_eq.shape[1], neq], dtype=np.int32).tofile(f)
        np.ascontiguousarray(elem_eq, dtype=np.int32).tofile(f)
    subprocess.run([exe, str(inp), str(out)], check=True, timeout=600)
    b = np.fromfile(out, dtype=np.int32)
    os.remove(inp)
    os.remove(out)
    return b[1:1 + b[0]]


@pytest.mark.parametrize("case", ["c2", "c3"])
def test_pattern_equals_the_reference_msr_builder(case, tmp_path):
    mesh, g, _ = {"c2": workloads.c2, "c3": workloads.c3}[case]()
    eq = g.equations()  # nnd x 3, 1-based, < 1 prescribed
    neq = int(eq.max())
    elem_eq = eq[mesh.conn].reshape(mesh.nel, 24)  # node-major, as ElementBaseT::Equations
    for upper in (True, False):
        bindx = _ref_msr(tmp_path, elem_eq, neq, upper)
        assert bindx[0] == neq + 1
        rp, ci = lib.pattern_host(mesh.conn, eq, mesh.nnd, upper_only=upper)
        assert len(rp) == neq + 1
        rows = np.repeat(np.arange(neq, dtype=np.int32), np.diff(rp))
        diag = ci == rows
        assert int(diag.sum()) == neq
        assert np.array_equal(np.diff(rp) - 1, np.diff(bindx[:neq + 1]))
        assert np.array_equal(ci[~diag], bindx[neq + 1:])
        del bindx, rp, ci, rows, diag
