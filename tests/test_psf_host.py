"""Host logic of the GPU PSF generator that needs no GPU: matrix file names
(generate_psf.py:89-92, 740-775 of the reference) and the quadrature rule."""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "fast-light-field_gb300"))

import generate_psf as G  # noqa: E402


def test_matrix_file_string_round_trip():
    s = G.MatrixFileString(40, 0.95, 150e-6, 3000e-6, -25e-6, 25e-6, 5e-6, 15, 520e-9, 1.33)
    assert s == "M40NA0.95MLPitch150fml3000from-25to25zspacing5Nnum15lambda520n1.33"
    m = G._NAME_RE.match(s)
    assert m is not None and m.group(8) == "15" and float(m.group(5)) == -25.0


@pytest.mark.parametrize("name,err", [
    ("PSFmatrix_M40NA0.95MLPitch150fml3000from-25to25zspacing5Nnum15lambda520n1.33.mat", "Matlab"),
    ("otherPSFmatrix_M40NA0.95MLPitch150fml3000from-25to25zspacing5Nnum15lambda520n1.33.mat", "prefix"),
    ("fdnormPSFmatrix_M40NA0.95MLPitch150fml3000from-25to25zspacing5Nnum15lambda520n1.33.h5", "only generate"),
    ("fdnormPSFmatrix_M40NA0.95.mat", "parse"),
])
def test_file_names_refused_before_any_device_work(name, err, tmp_path):
    with pytest.raises(ValueError, match=err):
        G.GeneratePSFFromFilePath(str(tmp_path / name))


def test_quadrature_integrates_a_known_transform():
    """With u = 0 and J0 weight, the quadrature reproduces a closed form:
    int_0^a J0(v sin t) cos t sin t dt = a-independent form via x = sin t:
    int_0^{sin a} J0(v x) x dx = sin(a) J1(v sin a) / v."""
    import scipy.special
    a = 0.8
    for v in (0.0, 7.0, 300.0, 2000.0):
        st, cw = G._quadrature(a, 0.0, 1.0, v)
        # cw holds sqrt(cos)(1 + cos) sin; divide it back to the test integrand cos sin
        ct = np.sqrt(1 - st ** 2)
        w = cw.real / (np.sqrt(ct) * (1 + ct) * st) * ct * st
        got = np.sum(w * scipy.special.j0(st * v))
        want = 0.5 * np.sin(a) ** 2 if v == 0 else np.sin(a) * scipy.special.j1(v * np.sin(a)) / v
        assert abs(got - want) < 1e-13 * max(1.0, abs(want)) + 1e-15
