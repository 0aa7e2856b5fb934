"""CPU checks of the FP64-oracle fixtures: the inputs the GPU tests rebuild are
the ones the fixtures were computed from, and the fixtures are complete."""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import fp64_inputs as F  # noqa: E402

# integer checksums of the camera images and of the sampled positions (both are
# integer arithmetic, so any machine reproduces them exactly)
CHECKSUMS = {"450px_11planes": (20493378, 111333420460), "450px_21planes": (20475685, 212674765340),
             "1005px_41planes": (103314564, 355292686794)}


@pytest.mark.parametrize("case", list(F.CASES))
def test_fixture_inputs_are_reproducible(case):
    img = F.image(case)
    pos = F.sample_positions(case, len(F.checked_planes(case)))
    assert (int(img.astype(np.int64).sum()), int(pos.sum())) == CHECKSUMS[case]
    assert img.dtype == np.float32 and np.array_equal(img, np.round(img))


@pytest.mark.parametrize("case", list(F.CASES))
def test_fixture_is_complete(case):
    f = F.load_fixture(case)
    assert list(f["planes"]) == F.checked_planes(case)
    assert int(f["iters"]) == F.CASES[case]["iters"]
    for key in ("htf", "x"):
        assert f[key].shape == (F.SAMPLES,) and np.isfinite(f[key]).all()
        assert 0 < float(np.abs(f[key]).max()) <= float(f[key + "_max"]) * (1 + 1e-6)


def test_fixture_psf_shapes_match_the_configurations():
    import synthetic
    assert synthetic.psf_sizes(15, F.z_planes("450px_21planes"), 14) == \
        [421, 391, 361, 301, 271, 211, 181, 151, 91, 61, 61, 61, 91, 151, 181, 211, 271, 301, 361, 391, 421]
    assert max(synthetic.psf_sizes(15, F.z_planes("1005px_41planes"), 28)) == 841
    assert synthetic.psf_sizes(15, F.z_planes("450px_11planes"), 7) == [211, 181, 151, 91, 61, 61, 61, 91, 151, 181,
                                                                         211]
