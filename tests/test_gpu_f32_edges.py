"""Edge cases of the FP32 form's brick layout, against the FP64 oracle.

- Ragged bricks: 8 ions per cell in one half of the box, 3 in the other,
  and 2000 in a single cell, so that the passes' CTAs walk from about 190 to
  more than 2000 ions each.  (A cell without ions next to a node leaves the
  node's density at zero, where curlB divides by it: the hybrid model, and
  the reference, need ions everywhere.)
- A brick of more than 65535 ions, past what a tile's 32-bit low words take
  without the carries into the high words: the same sums as the oracle.
"""
import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid, oracle_for

pytestmark = pytest.mark.gpu


def test_ragged_bricks_and_a_crowded_cell():
    h = make_hybrid(cells=(16, 8, 8), ppc=8, seed=41, db=0.02, extra=2100)
    n = int(h.ni_tot[0])
    x0, y0, z0 = h.coords.qx[0], h.coords.qy[0], h.coords.qz[0]
    # the upper half in x keeps 3 of every 8 ions
    upper = h.xp[:n, 0] - x0 > 8.0
    keep = np.nonzero(~upper | (np.arange(n) % 8 < 3))[0]
    for name in ("xp", "vp", "vp1", "mrat", "beta_p"):
        a = getattr(h, name)
        a[: keep.size] = a[keep]
    m = keep.size
    # 2000 ions in one cell of the lower half, nearly at rest
    rng = np.random.default_rng(4)
    h.xp[m : m + 2000] = np.array([x0 + 3.0, y0 + 2.0, z0 + 5.0]) + rng.uniform(0.05, 0.95, (2000, 3))
    h.vp[m : m + 2000] = 0.01 * rng.standard_normal((2000, 3))
    h.vp1[m : m + 2000] = h.vp[m : m + 2000]
    h.mrat[m : m + 2000] = 1.0
    h.beta_p[m : m + 2000] = 1.0
    h.ni_tot[0] = m + 2000
    h.mark_host_dirty()
    o = oracle_for(h)
    h.f32_begin()
    starts = h.f32_key_starts()
    per_brick = np.diff(starts[::64])
    assert per_brick.max() > 2000 and per_brick.min() < 250  # ragged indeed
    h.f32_run(2)
    h.f32_end()
    h.sync_to_host()
    for _ in range(2):
        o.ion_step()
    assert int(h.ni_tot[0]) == int(o.ni_tot[0]) == m + 2000
    assert rel_l2(h.b1, o.b1) < 1e-5
    assert rel_l2(h.np, o.np) < 1e-4
    assert rel_l2(h.up, o.up) < 1e-4
    assert np.all(np.isfinite(h.b1))
    h.close()


def test_a_brick_beyond_65535_ions_sums_exactly():
    # 66000 ions in one 4x4x4-cell brick of an 8^3-cell box, 2 per cell
    # elsewhere: the tile's low words would pass 2^32 without the carries
    g = make_hybrid(cells=(8, 8, 8), ppc=2, seed=6)
    ng = int(g.ni_tot[0])
    g.close()
    N = 66000
    h = make_hybrid(cells=(8, 8, 8), ppc=2, seed=6, extra=N + 16)
    rng = np.random.default_rng(1)
    lo = np.array([h.coords.qx[0], h.coords.qy[0], h.coords.qz[0]])
    sl = slice(ng, ng + N)
    h.xp[sl] = lo + rng.uniform(0.1, 3.9, (N, 3))
    h.vp[sl] = 0.01 * rng.standard_normal((N, 3))
    h.vp1[sl] = h.vp[sl]
    h.mrat[sl] = 1.0
    h.beta_p[sl] = 1.0
    h.ni_tot[0] = ng + N
    h.mark_host_dirty()
    o = oracle_for(h)
    h.f32_begin()
    starts = h.f32_key_starts()
    assert np.diff(starts[::64]).max() > 65535
    h.f32_run(1)
    h.f32_end()
    h.sync_to_host()
    o.ion_step()
    assert rel_l2(h.np, o.np) < 1e-4
    assert rel_l2(h.up, o.up) < 1e-4
    assert rel_l2(h.b1, o.b1) < 1e-5
    h.close()
