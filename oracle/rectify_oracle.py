"""CPU oracle for light-field rectification.

TEST INFRASTRUCTURE ONLY: the checker for fast-light-field_gb300/rectify.py,
which never imports it.  Restates the reference's RectifyImage
(rectify.py:8-81, itself a port of the Prevedel et al. MATLAB code): query
coordinates stepped by dx / Nnum from the given lenslet origin (MATLAB
one-based), bilinear interpolation of the raw image there (the reference's
scipy RectBivariateSpline with kx = ky = 1 is the degree-1 B-spline
interpolant, i.e. bilinear), a crop to whole lenslets, then an optional crop
of XcutLeft / XcutRight / YcutUp / YcutDown lenslets.  Pinned against the
reference's own function by tests/golden/rectify_vectors.npz.
"""

import numpy as np


def _axis(center_m, step, n):
    """The reference's resample axis (rectify.py:41-44): backwards from the origin to 1,
    then forwards to n, both inclusive (the +-1e-10 of its np.arange calls)."""
    down = np.arange(center_m + 1, 1 - 1e-10, -step)[::-1]
    up = np.arange((center_m + 1) + step, n + 1e-10, step)
    return np.append(down, up)


def _bilinear(img, yq, xq):
    """Bilinear interpolation of img at the grid yq x xq (zero-based), float64."""
    H, W = img.shape

    def cell(q, n):
        q = np.clip(q, 0, n - 1)
        i0 = np.minimum(np.floor(q).astype(np.int64), max(n - 2, 0))
        return i0, q - i0, np.minimum(i0 + 1, n - 1)

    y0, fy, y1 = cell(np.asarray(yq, np.float64), H)
    x0, fx, x1 = cell(np.asarray(xq, np.float64), W)
    a = img.astype(np.float64)
    top = (1 - fx)[None, :] * a[y0][:, x0] + fx[None, :] * a[y0][:, x1]
    bot = (1 - fx)[None, :] * a[y1][:, x0] + fx[None, :] * a[y1][:, x1]
    return (1 - fy)[:, None] * top + fy[:, None] * bot


def rectify_image(img, xCenter_m, yCenter_m, dx, Nnum, Crop=False, XcutLeft=0, XcutRight=0, YcutUp=0, YcutDown=0):
    """Rectified image (float64) as the reference's RectifyImage returns it."""
    if Nnum % 2 != 1:
        raise ValueError("Nnum must be an odd integer")
    M, mdiff = Nnum, Nnum // 2
    H, W = img.shape
    Xres = _axis(xCenter_m, dx / M, W)
    Yres = _axis(yCenter_m, dx / M, H)
    xc = int(np.where(Xres == xCenter_m + 1)[0][0]) - mdiff + 1
    yc = int(np.where(Yres == yCenter_m + 1)[0][0]) - mdiff + 1
    xinit = xc - M * (xc // M) + M
    yinit = yc - M * (yc // M) + M
    res = _bilinear(img, Yres[yinit - 1:] - 1, Xres[xinit - 1:] - 1)
    res = res[:M * ((res.shape[0] - yinit) // M), :M * ((res.shape[1] - xinit) // M)]
    if Crop:
        xs, ys = res.shape[1] // M, res.shape[0] // M
        if XcutLeft + XcutRight >= xs or YcutUp + YcutDown >= ys:
            raise ValueError("cut range is larger than the image")
        res = res[YcutUp * M:(ys - YcutDown) * M, XcutLeft * M:(xs - XcutRight) * M]
    return res
