"""CPU tests: the oracle against the reference's golden vectors and its own definitions."""

import numpy as np
import pytest

from golden_inputs import CASES, case_inputs
from oracle import lf_oracle as O

GOLD = None


def gold():
    global GOLD
    if GOLD is None:
        import os
        GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz"))
    return GOLD


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", [n for n in CASES if CASES[n]["kind"] == "project"])
@pytest.mark.parametrize("method", ["special", "direct"])
def test_oracle_projection_matches_reference(name, method):
    c = case_inputs(name)
    dt = np.float32 if method == "special" else np.float64
    bk = O.backward_project(c["Ht"], c["img"], c["Nnum"], method=method, dtype=dt)
    fw = O.forward_project(c["H"], c["vol"], c["Nnum"], method=method, dtype=dt)
    # the reference's own self-test tolerance is 1e-4 absolute on O(1) values
    assert rel(bk, gold()[name + "/backward"]) < 2e-6
    assert rel(fw, gold()[name + "/forward"]) < 2e-6


@pytest.mark.parametrize("name", [n for n in CASES if CASES[n]["kind"] == "rl"])
def test_oracle_rl_matches_reference(name):
    c = case_inputs(name)
    Z = len(c["hs"])
    x0 = None if c["prevedel"] else np.ones((Z,) + c["img"].shape, np.float32)
    r = O.deconv_rl(c["H"], c["Ht"], c["Nnum"], c["iters"], im=c["img"], x0=x0, prevedel=c["prevedel"])
    assert rel(r, gold()[name + "/rl"]) < 1e-5


def test_symmetry_map_properties():
    rng = np.random.default_rng(0)
    N, h = 7, 9
    Hred = rng.random(((N + 1) // 2, (N + 1) // 2, h, h))
    Hf = O.expand_psf_set(Hred, N)
    c = N // 2
    # stored quadrant (upper triangle) is reproduced as is
    for bb in range(c + 1):
        for aa in range(bb, c + 1):
            assert np.array_equal(Hf[bb, aa], Hred[bb, aa])
    # mirror relations between distinct offsets
    for b in range(N):
        for a in range(N):
            if b != c:
                assert np.array_equal(Hf[N - 1 - b, a], Hf[b, a][::-1, :])
            if a != c:
                assert np.array_equal(Hf[b, N - 1 - a], Hf[b, a][:, ::-1])
    # transposed quadrant positions use the transpose of the upper triangle
    for bb in range(c + 1):
        for aa in range(bb + 1, c + 1):
            assert np.array_equal(Hf[aa, bb], Hred[bb, aa].T)


def test_padding_policy_independence():
    """Any FFT size >= the linear-convolution size gives the same 'same' result."""
    c = case_inputs("planes_n7")
    a = O.backward_project(c["Ht"], c["img"], 7, method="special", dtype=np.float64)
    b = O.backward_project(c["Ht"], c["img"], 7, method="special_gpu_pad", dtype=np.float64)
    assert rel(a, b) < 1e-12


def test_convolution_shape_matches_reference_policy():
    # CPU policy pads the quotient to a 7-smooth number (special_fftconvolve.py:122-171)
    fs, full = O.convolution_shape((450, 450), (211, 211), 15, True)
    assert full == (660, 660) and fs == [675, 675]
    fs, full = O.convolution_shape((450, 450), (211, 211), 15, False)
    assert fs == [660, 660]


def test_rl_nan_handling():
    """0/0 in the Prevedel update becomes 0 (lfdeconv.py:118-125)."""
    c = case_inputs("rl_prevedel")
    Z = len(c["hs"])
    img = np.zeros_like(c["img"])
    r = O.deconv_rl(c["H"], c["Ht"], 5, 1, im=img, prevedel=True)
    assert np.all(r == 0) and r.shape == (Z,) + img.shape


@pytest.mark.parametrize("name", [n for n in CASES if CASES[n]["kind"] == "project"])
def test_reference_cpu_algorithm_matches_reference(name):
    """The oracle's restatement of the reference's CPU algorithm (symmetry reuse
    of the stored spectra) against the reference's own outputs, in single
    precision, and in double precision against the FP64 definition."""
    c = case_inputs(name)
    N = c["Nnum"]
    Z = len(c["hs"])
    bk = np.stack([O.project_plane_ref_cpu(c["img"], c["Ht"][z], N) for z in range(Z)])
    fw = sum(O.project_plane_ref_cpu(c["vol"][z], c["H"][z], N) for z in range(Z))
    assert rel(bk, gold()[name + "/backward"]) < 2e-6
    assert rel(fw, gold()[name + "/forward"]) < 2e-6
    bk64 = np.stack([O.project_plane_ref_cpu(c["img"], c["Ht"][z], N, dtype=np.float64) for z in range(Z)])
    ref64 = O.backward_project(c["Ht"], c["img"], N, method="direct", dtype=np.float64)
    assert rel(bk64, ref64) < 1e-12
