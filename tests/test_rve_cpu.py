"""Host logic of the batched RVE generator (no GPU)."""
import numpy as np

from tahoe_gb300 import rve


def test_template_phases_and_boundary():
    t = rve.template(8)
    assert t.nnd == 9 ** 3 and t.nel == 8 ** 3
    assert len(t.boundary) == 9 ** 3 - 7 ** 3
    c = t.X[t.conn].mean(axis=1)
    inside = np.linalg.norm(c - 0.5, axis=1) < rve.RADIUS
    assert np.array_equal(inside.astype(np.int32), t.blocks)
    assert 0 < t.blocks.sum() < t.nel


def test_sampled_F_symmetric_perturbation():
    ns, Fs = rve.sample_batch(200, seed=3)
    assert ns.min() >= 4 and ns.max() <= 16
    S = (Fs - np.eye(3)) / 0.05
    assert np.allclose(S, np.transpose(S, (0, 2, 1)))
    assert S.min() >= -1.0 and S.max() <= 1.0


def test_batch_concatenation_is_disconnected_and_affine():
    ns, Fs = rve.sample_batch(5, sizes=[4, 5, 6], seed=1)
    b = rve.RVEBatch(ns, Fs)
    assert b.node_off[-1] == b.nnd and b.elem_off[-1] == b.nel
    for r in range(b.count):
        conn = b.conn[b.elem_off[r]:b.elem_off[r + 1]]
        assert conn.min() >= b.node_off[r] and conn.max() < b.node_off[r + 1]
        X = b.X[b.node_off[r]:b.node_off[r + 1]]
        assert np.allclose(b.u0[b.node_off[r]:b.node_off[r + 1]], X @ (Fs[r] - np.eye(3)).T)
    assert len(b.prescribed_idx) == len(b.prescribed_val)
