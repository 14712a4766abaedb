"""CPU checks of the oracle's per-stage queue model (the checker the GPU queue
tests use): on soups, clipped scenes and odd viewports, at every bin size and
with 1 and 4 samples, every list is in submission order and the exact lists
(entries covering a sample of the cell) are contained in the rule's lists, so
the binning rule is conservative; a tile's rule list only takes entries of its
bin's rule list."""
import numpy as np
import pytest

from conftest import pkg_mod
from oracle import oracle as orc


def _scenes():
    s = pkg_mod("scenes")
    near = s.soup(1500, 256, 200, seed=9, median_px=300.0, sigma=1.2)
    v = near["vertices"].copy()
    v[::5, 2] = -1.5 * v[::5, 3]
    near["vertices"] = v
    return {"soup": s.soup(6000, 200, 136, seed=41, median_px=6.0), "near_clipped": near,
            "odd": s.soup(3000, 173, 91, seed=42, median_px=14.0)}


@pytest.mark.parametrize("samples", [1, 4])
def test_exact_lists_inside_rule_lists(samples):
    for name, sc in _scenes().items():
        p = orc.make_pipe(sc["width"], sc["height"], samples, orc.DEPTH | orc.LERP, "replace", "gouraud", 32)
        for bl in (3, 4, 5):
            q = {k: orc.queue_lists(p, sc["vertices"], sc["indices"], bl, k) for k in orc.QUEUE_KINDS}
            for lvl in ("bin", "tile"):
                eo, ee = q[lvl + "_exact"]
                ro, re_ = q[lvl + "_rule"]
                assert len(eo) == len(ro) and len(ee) > 0
                for c in range(len(eo) - 1):
                    e = ee[eo[c]:eo[c + 1]].astype(np.int64)
                    r = re_[ro[c]:ro[c + 1]].astype(np.int64)
                    assert np.all(np.diff(e) > 0) and np.all(np.diff(r) > 0), (name, bl, lvl, c)
                    assert np.isin(e, r).all(), (name, bl, lvl, c)
            # A tile's rule entries come from its bin's rule list.
            wt = (sc["width"] + 7) >> 3
            side = 1 << bl
            wb = (wt + side - 1) // side
            bo, be = q["bin_rule"]
            to, te = q["tile_rule"]
            for t in range(len(to) - 1):
                b = ((t // wt) >> bl) * wb + ((t % wt) >> bl)
                assert np.isin(te[to[t]:to[t + 1]], be[bo[b]:bo[b + 1]]).all(), (name, bl, t)


def test_queue_entries_name_real_subtriangles():
    sc = _scenes()["near_clipped"]
    p = orc.make_pipe(sc["width"], sc["height"], 1, orc.DEPTH | orc.LERP, "replace", "gouraud", 32)
    sub, _, _, _ = orc.setup(p, sc["vertices"], sc["indices"])
    _, ent = orc.queue_lists(p, sc["vertices"], sc["indices"], 4, "tile_rule")
    t, k = ent >> 3, ent & 7
    n = sub[t].astype(np.int64)
    assert np.all(np.where(k == 7, n == 1, (n > 1) & (k < n)))
    assert (sub > 1).any(), "the scene should have triangles clipped into several subtriangles"
