"""The PSF-generation oracle against the reference's own GeneratePSF outputs.

tests/golden/psf_vectors.npz holds what the reference's generate_psf.py saved
for the cases of tests/golden/psf_inputs.py (make_golden_psf.py).  The oracle
restates that generator with scipy's J0 (the reference links a rational
approximation of J0) and vectorised adaptive quadrature, so the matrices agree
to float32 rounding: 5e-7 of the maximum; CAindex and the set of zeroed
(clipped) entries agree exactly; Hmax to 1e-6 relative.
"""

import os

import numpy as np
import pytest

from oracle import psf_oracle as P

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from psf_inputs import PSF_CASES
    return PSF_CASES, np.load(os.path.join(HERE, "golden", "psf_vectors.npz"))


@pytest.mark.parametrize("name", ["n5_osr3", "n7_z30", "n7_bug"])
def test_psf_oracle_matches_reference_generator(name):
    cases, g = _golden()
    r = P.saved_form(P.generate_psf(cases[name]))
    H, Ht = g[name + "/H"], g[name + "/Ht"]
    assert np.array_equal(r["CAindex"], g[name + "/CAindex"])
    assert abs(r["Hmax"] - g[name + "/Hmax"]) <= 1e-6 * abs(g[name + "/Hmax"])
    assert r["H"].shape == H.shape and r["Ht"].shape == Ht.shape
    assert np.max(np.abs(r["H"] - H)) <= 5e-7 * H.max()
    assert np.max(np.abs(r["Ht"] - Ht)) <= 5e-7 * Ht.max()
    assert np.array_equal(r["H"] == 0, H == 0)


def test_psf_oracle_ht_is_a_rearrangement_of_h():
    """Every Ht entry is an entry of H or zero (the stamping moves values only)."""
    rng = np.random.default_rng(3)
    N, S, Z = 5, 31, 2
    H = rng.random((S, S, 3, 3, Z)).astype(np.float32) + 1
    Ht = P.calc_ht(H, N)
    vals = set(H.ravel().tolist())
    assert all(v == 0 or v in vals for v in Ht.ravel().tolist())
    assert np.count_nonzero(Ht[:, :, 2, 2]) == S * S * Z   # the centre offset needs no shift
