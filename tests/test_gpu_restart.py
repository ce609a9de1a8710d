"""Restart images: a J2 step sequence saved after step 2 and resumed in a
fresh context gives bitwise the same step 3 as the uninterrupted run; images
that do not match the context are refused."""
import os

import numpy as np
import pytest

from tahoe_gb300 import deck as dk
from tahoe_gb300 import lib

pytestmark = pytest.mark.gpu

DECK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks", "cube8_j2.xml")


def _run(m, d, first, last, on_step=None):
    sv = d.solver
    return m.run(last, d.dt, rel_tol=sv["rel_tol"], abs_tol=sv["abs_tol"], max_iterations=sv["max_its"],
                 div_tol=sv["div_tol"], precision=lib.FP64, lin_rel_tol=1e-13, first_step=first, on_step=on_step)


def test_resume_from_image_is_bitwise():
    d = dk.Deck(DECK)
    full = d.model()
    out = {}
    hist, _ = _run(full, d, 1, 2)
    image = full.ctx.state_save()
    flags2 = full.ctx.active_set()
    hist3, _ = _run(full, d, 3, 3, on_step=lambda s, c: out.setdefault("full", c.nodal_stress()))
    fresh = d.model()
    fresh.setup()
    fresh.ctx.state_load(image)
    assert np.array_equal(fresh.ctx.active_set(), flags2)
    hist3b, _ = _run(fresh, d, 3, 3, on_step=lambda s, c: out.setdefault("fresh", c.nodal_stress()))
    assert np.array_equal(hist3b[-1], hist3[-1])
    assert np.array_equal(out["fresh"], out["full"])
    assert np.array_equal(fresh.ctx.active_set(), full.ctx.active_set())


def test_mismatched_image_refused():
    d = dk.Deck(DECK)
    m = d.model()
    m.setup()
    image = bytearray(m.ctx.state_save())
    other = dk.Deck(os.path.join(os.path.dirname(DECK), "cube8_tl_traction.xml")).model()
    other.setup()
    with pytest.raises(lib.TahoeError) as e:
        other.ctx.state_load(bytes(image))  # no J2 history in this context
    assert e.value.code == -1
    image[0] ^= 0xFF
    with pytest.raises(lib.TahoeError):
        m.ctx.state_load(bytes(image))


def test_rollback_after_load_is_refused():
    """A device snapshot taken before tg_state_load predates the loaded state:
    rolling back to it after the load is refused until a new checkpoint."""
    d = dk.Deck(DECK)
    m = d.model()
    _run(m, d, 1, 1)
    image = m.ctx.state_save()
    m.ctx.checkpoint()
    m.ctx.state_load(image)
    with pytest.raises(lib.TahoeError) as e:
        m.ctx.rollback()
    assert e.value.code == -1
    m.ctx.checkpoint()
    m.ctx.rollback()
