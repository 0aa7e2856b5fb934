"""Rectification oracle against the reference's own RectifyImage (golden vectors; no GPU)."""

import os

import numpy as np
import pytest

from oracle import rectify_oracle as R
from rectify_inputs import RECTIFY_CASES, rectify_input

GOLD = os.path.join(os.path.dirname(__file__), "golden", "rectify_vectors.npz")


@pytest.mark.parametrize("name", sorted(RECTIFY_CASES))
def test_oracle_matches_reference_rectify(name):
    img, kw = rectify_input(name)
    g = np.load(GOLD)[name]
    o = R.rectify_image(img, **kw)
    assert o.shape == g.shape
    assert np.max(np.abs(o - g)) <= 1e-9 * max(1.0, np.max(np.abs(g)))
    assert np.array_equal(np.around(o), np.around(g))


def test_oracle_rejects_even_nnum_and_oversized_cuts():
    img, kw = rectify_input("n5_u8")
    with pytest.raises(ValueError):
        R.rectify_image(img, **dict(kw, Nnum=4))
    with pytest.raises(ValueError):
        R.rectify_image(img, **dict(kw, Crop=True, XcutLeft=10, XcutRight=10))
