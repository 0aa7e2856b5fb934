"""GPU PSF generation (generate_psf.py of this package) against the reference's
generator outputs, the oracle, and full-size properties.

Tolerances: the device integrates the Debye integral by Gauss-Legendre
quadrature with CUDA's FP64 J0 where the reference runs adaptive quad with a
rational-approximation J0, and the matrices are float32: H and Ht agree with
the reference's to 1e-6 of their maximum, CAindex exactly, Hmax to 1e-6
relative, and the set of clipped entries exactly.  Ht is index work: it is
bit-identical to the oracle's stamping applied to the device's own H.
"""

import os
import sys

import numpy as np
import pytest

from oracle import psf_oracle as P

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-6


@pytest.fixture(scope="module")
def gen(built_lib):
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import generate_psf
    from psf_inputs import PSF_CASES
    return generate_psf, PSF_CASES, np.load(os.path.join(HERE, "golden", "psf_vectors.npz"))


def _saved(r):
    """Device result in the reference's saved layout [Z, b, a, y, x]."""
    return (r["H_device"].permute(0, 2, 1, 4, 3).cpu().numpy(), r["Ht_device"].permute(0, 2, 1, 4, 3).cpu().numpy())


@pytest.mark.parametrize("name", ["n5_osr3", "n7_z30", "n7_bug"])
def test_psf_matches_reference_generator(gen, name):
    generate_psf, cases, g = gen
    r = generate_psf.GeneratePSFArrays(**cases[name])
    H, Ht = _saved(r)
    Hg, Htg = g[name + "/H"], g[name + "/Ht"]
    assert np.array_equal(r["CAindex"].T, g[name + "/CAindex"])
    assert abs(r["Hmax"] - float(g[name + "/Hmax"])) <= 1e-6 * float(g[name + "/Hmax"])
    assert H.shape == Hg.shape
    assert np.max(np.abs(H - Hg)) <= TOL * Hg.max()
    assert np.max(np.abs(Ht - Htg)) <= TOL * Htg.max()
    assert np.array_equal(H == 0, Hg == 0)
    # Ht is the reference's stamping of the device's own H, bit for bit
    Href = r["H_device"].permute(3, 4, 1, 2, 0).cpu().numpy()      # [i, j, a, b, z]
    Ht_o = P.calc_ht(Href, cases[name]["Nnum"])
    assert np.array_equal(r["Ht_device"].permute(3, 4, 1, 2, 0).cpu().numpy(), Ht_o)
    # the reduced quadrants are the CAindex crops of the saved arrays
    for z in range(H.shape[0]):
        a0, a1 = r["CAindex"][0, z] - 1, r["CAindex"][1, z]
        assert np.array_equal(r["H"][z], H[z][:, :, a0:a1, a0:a1])
        assert np.array_equal(r["Ht"][z], Ht[z][:, :, a0:a1, a0:a1])


def test_psf_files_load_and_project(gen, tmp_path):
    """GeneratePSFFromFilePath writes the memmap layout; LoadMatrix(createPSF=True)
    finds it and the projector runs on it; an unknown prefix is refused."""
    generate_psf, cases, g = gen
    import lfdeconv
    import projector
    import psfmatrix
    name = "fdnormPSFmatrix_M40NA0.95MLPitch150fml3000from-6to6zspacing3Nnum5lambda520n1.33.mat"
    path = str(tmp_path / name)
    hm = psfmatrix.LoadMatrix(path, createPSF=True)
    assert hm.numZ == 5 and hm.Nnum == 5
    H = np.stack([hm.Hcc(z, False) for z in range(5)])
    Hg = g["n5_osr3/H"]
    assert np.max(np.abs(H - Hg)) <= TOL * Hg.max()
    assert os.path.exists(os.path.join(os.path.splitext(path)[0], "PSFInfo.json"))
    img = np.random.default_rng(0).random((1, 25, 25)).astype(np.float32)
    vol = lfdeconv.BackwardProjectACC(hm, img, planes=None, projector=projector.Projector_gb300(), logPrint=False)
    assert vol.shape == (5, 1, 25, 25) and np.isfinite(vol).all()
    with pytest.raises(ValueError):
        generate_psf.GeneratePSFFromFilePath(str(tmp_path / "PSFmatrix_M40NA0.95.mat"))


def test_psf_full_size_properties(gen):
    """Nnum 15, M40 / NA 0.95, 11 planes at -25..25 um: the reference's PSF sizes
    h_z, unit-sum offsets, mirror symmetry of the centre offset."""
    generate_psf, cases, g = gen
    r = generate_psf.GeneratePSFArrays(M=40, NA=0.95, MLPitch=150e-6, Nnum=15, OSR=3, n=1.33, fml=3000e-6,
                                       lam=520e-9, zmin=-25e-6, zmax=25e-6, zspacing=5e-6)
    assert [h.shape[-1] for h in r["H"]] == [211, 181, 151, 91, 61, 61, 61, 91, 151, 181, 211]
    sums = r["H_device"].double().sum(dim=(3, 4))
    assert float((sums - 1).abs().max()) < 1e-5
    Hc = r["H_device"][:, 7, 7].cpu().numpy()          # centre offset: symmetric under both flips
    assert np.max(np.abs(Hc - Hc[:, ::-1, :])) <= 1e-6 * Hc.max()
    assert np.max(np.abs(Hc - Hc[:, :, ::-1])) <= 1e-6 * Hc.max()
    # z -> -z mirror: the intensity of a point at depth -z matches +z only up to the defocus
    # phase's sign, so only the support sizes agree
    assert r["CAindex"][0, 0] == r["CAindex"][0, -1]


def test_psf_size_limit(gen):
    """The reference's size limit stands by default; a larger limit lets a deep stack through."""
    generate_psf, cases, g = gen
    kw = dict(M=40, NA=0.95, MLPitch=150e-6, Nnum=5, OSR=3, n=1.33, fml=3000e-6, lam=520e-9,
              zmin=-60e-6, zmax=60e-6, zspacing=60e-6)
    with pytest.raises(ValueError, match="exceeds the limit"):
        generate_psf.GeneratePSFArrays(maxPSFLenslets=4, **kw)
    r = generate_psf.GeneratePSFArrays(maxPSFLenslets=60, **kw)
    assert r["IMGSIZE_REF"] > 4
