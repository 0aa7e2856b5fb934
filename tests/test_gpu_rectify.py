"""GPU rectification (flf_resample_bilinear through rectify.py) against the reference's
RectifyImage golden vectors and the CPU oracle."""

import os

import numpy as np
import pytest

from oracle import rectify_oracle as R
from rectify_inputs import RECTIFY_CASES, rectify_input

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "rectify_vectors.npz")


@pytest.mark.parametrize("name", sorted(RECTIFY_CASES))
def test_rectify_matches_reference_vectors(built_lib, name):
    import rectify
    img, kw = rectify_input(name)
    g = np.load(GOLD)[name]
    out = rectify.RectifyImage(img, **kw)
    assert out.shape == g.shape and out.dtype == np.float64
    assert np.max(np.abs(out - g)) <= 1e-9 * max(1.0, np.max(np.abs(g)))
    assert np.array_equal(np.around(out), np.around(g))


def test_rectify_camera_sized_image_against_oracle(built_lib):
    import rectify
    rng = np.random.default_rng(21)
    img = (rng.random((1200, 1400)) * 60000).astype(np.uint16)
    kw = dict(xCenter_m=701.3, yCenter_m=598.6, dx=14.73, Nnum=15, Crop=True, XcutLeft=2, XcutRight=1,
              YcutUp=1, YcutDown=3)
    out = rectify.RectifyImage(img, **kw)
    o = R.rectify_image(img, **kw)
    assert out.shape == o.shape
    assert np.max(np.abs(out - o)) <= 1e-9 * np.max(np.abs(o))


def test_rectify_files_round_trip(built_lib, tmp_path):
    import rectify
    import tiffio
    img, kw = rectify_input("n9_u16_crop")
    src = str(tmp_path / "raw.tif")
    tiffio.imwrite(src, img)
    args = [src, "-x", str(kw["xCenter_m"]), "-y", str(kw["yCenter_m"]), "-d", str(kw["dx"]), "-n", str(kw["Nnum"]),
            "-c", "-l", str(kw["XcutLeft"]), "-r", str(kw["XcutRight"]), "-t", str(kw["YcutUp"]),
            "-b", str(kw["YcutDown"]), "-o", str(tmp_path / "out")]
    written = rectify.RectifyWithArgList(args)
    assert written == [str(tmp_path / "out" / "raw_N9.tif")]
    got = tiffio.imread(written[0])
    assert got.dtype == np.uint16
    assert np.array_equal(got, np.around(np.load(GOLD)["n9_u16_crop"]).astype(np.uint16))
