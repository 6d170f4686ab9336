"""Seeded scene generators: deterministic, non-overlapping where specified, right sizes."""
import numpy as np

from scisim_gb300 import scenes


def test_box_drop_shapes_and_seed():
    a = scenes.box_drop_1024(seed=1)
    b = scenes.box_drop_1024(seed=1)
    assert a["q"].shape == (2048,) and a["r"].shape == (1024,)
    assert np.array_equal(a["q"], b["q"]) and np.array_equal(a["v"], b["v"])
    assert 0.04 <= a["r"].min() and a["r"].max() <= 0.06
    assert np.allclose(a["m"], np.pi * a["r"] ** 2)


def test_dense_pile_fill_small():
    s = scenes.dense_pile(n=4096, seed=5, width=5.0, height=7.5)
    q = s["q"].reshape(-1, 2)
    assert q.shape == (4096, 2)
    assert scenes.min_gap(s["q"], s["r"], s["plane_x"], s["plane_n"]) > 0.0
    frac = (np.pi * s["r"] ** 2).sum() / (5.0 * 7.5)
    assert 0.4 < frac < 0.6
    assert 0.02 <= s["r"].min() and s["r"].max() <= 0.06
