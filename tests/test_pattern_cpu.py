"""Equation numbers and the sparsity pattern at the benchmark meshes' full
sizes, on the host: the package's equation numbering (the mirror of
NodeManagerT::SetEquationNumbers) and the library's pattern builder
(tg_pattern_build_host runs the code tg_pattern_build runs on a context)
against the oracle's restatement of NodeManagerT.cpp:712-760 and
MSRBuilderT::GenerateMSR (MSRBuilderT.cpp:134-175), bit-exactly, for the
upper (symmetric) and the full MSR pattern."""
import numpy as np
import pytest

from oracle.pyoracle import OracleModel
from tahoe_gb300 import lib, workloads


def _oracle_ctor(X, conn, form, mat):
    return OracleModel(X, conn, form, [mat])


def _models(case):
    build = {"c2": workloads.c2, "c3": workloads.c3}[case]
    mesh, o, _ = build(add=_oracle_ctor)
    _, g, _ = build()  # the host-side model: no context is created
    return mesh, o, g


def _msr_from_csr(rp, ci):
    """(row lengths without the diagonal, off-diagonal columns) of a scalar
    CSR whose every row holds its diagonal"""
    n = len(rp) - 1
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(rp))
    diag = ci == rows
    assert int(diag.sum()) == n  # one diagonal entry per row
    return np.diff(rp) - 1, ci[~diag]


@pytest.mark.parametrize("case", ["c2", "c3"])
def test_equations_and_pattern_bit_exact_at_full_size(case):
    mesh, o, g = _models(case)
    eq_o, neq = o.equations()
    eq_g = g.equations()
    assert np.array_equal(eq_g, eq_o)
    for upper in (True, False):
        bindx = o.msr_pattern(upper=upper)
        assert bindx[0] == neq + 1
        rp, ci = lib.pattern_host(mesh.conn, eq_g, mesh.nnd, upper_only=upper)
        assert len(rp) == neq + 1
        lens, off = _msr_from_csr(rp, ci)
        assert np.array_equal(lens, np.diff(bindx[:neq + 1]))
        assert np.array_equal(off, bindx[neq + 1:])
        del bindx, rp, ci, off
