"""CPU oracle for the light-field Richardson-Lucy projection path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: the CUDA path in
``fast-light-field_gb300`` never imports it.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may call it.

It restates, in numpy, the reference's algorithm for the projection hot path
(jmtayloruk/fast-light-field):

* ``expand_psf_set`` - the lenslet-offset symmetry map that turns the stored
  quadrant of PSFs ``H[bb][aa]`` (``aa >= bb`` read, ``0 <= bb,aa < (N+1)/2``)
  into the full ``N x N`` set (projector.py:159-189, py_light_field.cpp:1514-1561,
  1294-1317).
* ``convolution_shape`` - FFT padding policy (special_fftconvolve.py:122-174).
* ``project_plane_special`` - the reference's "special FFT" convolution:
  strided small FFT of each lenslet sub-image, tiled with phase ramps,
  multiplied by the PSF spectrum and accumulated in Fourier space, one
  inverse real FFT per plane, centred crop (special_fftconvolve.py:85-105,
  184-222; projector.py:103-255, 792-796; py_light_field.cpp:303-341,
  1001-1087, 925-950).
* ``project_plane_direct`` - the definition the reference's own strict test
  oracle uses: per offset, mask the input to that lenslet pixel and
  ``fftconvolve(..., 'same')`` with the expanded PSF (projector.py:1084-1126).
  Run in float64 it is the FP64 oracle.
* ``forward_project`` / ``backward_project`` - the plane loops
  (projector.py:806-896: backward keeps each plane, forward sums planes).
* ``deconv_rl`` - the two Richardson-Lucy updates (lfdeconv.py:72-202):
  Prevedel ``x <- x * Htf / (Ht H x)`` (lfdeconv.py:112-149) and standard
  ``x <- x * Ht(y / Hx)`` with an optional trust-mask normaliser
  ``/ Ht m`` (lfdeconv.py:151-183); NaN results are set to 0.

Parity of this restatement is pinned against the reference's own pure-python
projector (``Projector_python``) and RL driver, run in a container that holds
the reference sources; the resulting vectors are committed under
``tests/golden/`` with the script that made them.
"""

import numpy as np
from scipy.signal import fftconvolve

__all__ = [
    "expand_psf_set", "convolution_shape", "better_primes",
    "project_plane_special", "project_plane_direct",
    "forward_project", "backward_project", "deconv_rl",
]


# ---------------------------------------------------------------------------
# Symmetry map (projector.py:159-189; py_light_field.cpp:1514-1561)
# ---------------------------------------------------------------------------

def expand_psf_set(Hred, Nnum):
    """Full ``[N, N, h, h]`` PSF set from the stored ``[n_h, n_h, h, h]`` quadrant.

    Offset ``(b, a)`` (row offset ``b``, column offset ``a`` inside a lenslet)
    uses ``bb = min(b, N-1-b)``, ``aa = min(a, N-1-a)``; the base PSF is
    ``H[bb][aa]`` when ``aa >= bb`` and ``H[aa][bb]`` transposed otherwise
    (the reference's transpose work item, py_light_field.cpp:1526-1541 and
    projector.py:172-181, transposes ``H[bb][aa]`` of the upper triangle).
    The base is flipped along rows when ``b > c`` (the reference's
    ``mirrorX``) and along columns when ``a > c`` (``mirrorY``), ``c = N//2``.
    """
    Hred = np.asarray(Hred)
    N = int(Nnum)
    c = N // 2
    n_h = (N + 1) // 2
    assert Hred.shape[0] == n_h and Hred.shape[1] == n_h, Hred.shape
    h0, h1 = Hred.shape[2], Hred.shape[3]
    assert h0 == h1, "PSFs are square"
    out = np.empty((N, N, h0, h1), dtype=Hred.dtype)
    for b in range(N):
        for a in range(N):
            bb = min(b, N - 1 - b)
            aa = min(a, N - 1 - a)
            P = Hred[bb, aa] if aa >= bb else Hred[aa, bb].T
            if b > c:
                P = P[::-1, :]
            if a > c:
                P = P[:, ::-1]
            out[b, a] = P
    return out


# ---------------------------------------------------------------------------
# Shapes (special_fftconvolve.py:122-174)
# ---------------------------------------------------------------------------

def _prime_factors(n):
    i, f = 2, []
    while i * i <= n:
        if n % i:
            i += 1
        else:
            n //= i
            f.append(i)
    if n > 1:
        f.append(n)
    return f


def better_primes(n, Nnum, max_acceptable=7):
    """Smallest multiple of Nnum >= n whose quotient is 7-smooth (special_fftconvolve.py:122-127)."""
    r = int(n / Nnum)
    while max(_prime_factors(r) or [1]) > max_acceptable:
        r += 1
    return r * Nnum


def convolution_shape(img_shape, psf_shape, Nnum, pad_to_small_primes):
    """``(fshape, full_shape)``: padded FFT shape (multiple of Nnum) and linear-convolution size.

    GPU policy (``pad_to_small_primes=False``): ``ceil(d/N)*N``; CPU policy:
    ``N * (7-smooth quotient)`` (special_fftconvolve.py:142-174).
    """
    s1 = np.array(img_shape[-2:])
    s2 = np.array(psf_shape[-2:])
    full = s1 + s2 - 1
    if not pad_to_small_primes:
        fshape = [int(np.ceil(d / float(Nnum))) * Nnum for d in full]
    else:
        fshape = []
        for d in full:
            q = int(np.ceil(d / float(Nnum)))
            fshape.append(q * Nnum if q < 2 else better_primes(q * Nnum, Nnum))
    return fshape, tuple(int(v) for v in full)


def _centered(arr, newsize):
    """Centre crop of the last two axes (special_fftconvolve.py:71-80)."""
    cur = np.array(arr.shape[-2:])
    new = np.asarray(newsize)
    st = (cur - new) // 2
    return arr[..., st[0]:st[0] + new[0], st[1]:st[1] + new[1]]


# ---------------------------------------------------------------------------
# Per-plane projection: the reference's special-FFT algorithm
# ---------------------------------------------------------------------------

def project_plane_special(src, Hred, Nnum, pad_to_small_primes=True, dtype=np.float32):
    """One z plane of the reference's Fourier-space projection.

    ``src`` is ``[T, Y, X]`` (image for back projection, one volume plane for
    forward projection); ``Hred`` the stored quadrant for that plane and
    direction.  Returns ``[T, Y, X]``.  ``dtype`` float32 follows the
    reference's single-precision arithmetic (complex64 accumulators,
    py_light_field.cpp:1495-1497); float64 gives the same algorithm in
    double precision.
    """
    cdt = np.complex64 if dtype == np.float32 else np.complex128
    src = np.asarray(src, dtype=dtype)
    if src.ndim == 2:
        src = src[np.newaxis]
    T, Y, X = src.shape
    N = int(Nnum)
    Hfull = expand_psf_set(np.asarray(Hred, dtype=dtype), N)
    h = Hfull.shape[-1]
    fshape, full = convolution_shape((Y, X), (h, h), N, pad_to_small_primes)
    FY, FX = fshape
    fy, fx = FY // N, FX // N
    RX = FX // 2 + 1
    accum = np.zeros((T, FY, RX), dtype=cdt)
    ky = np.arange(FY)
    kx = np.arange(RX)
    for b in range(N):
        for a in range(N):
            # strided small FFT of the lenslet sub-image (special_rfftn, special_fftconvolve.py:85-105)
            sub = src[:, b::N, a::N]
            Ssmall = np.fft.fft2(sub, s=(fy, fx), axes=(1, 2)).astype(cdt)
            # tile to the full spectrum with the phase ramps of the (b, a) offset
            ph = (np.exp(-2j * np.pi * b * ky / FY)[:, None]
                  * np.exp(-2j * np.pi * a * kx / FX)[None, :]).astype(cdt)
            Sfull = Ssmall[:, ky % fy][:, :, kx % fx] * ph[None]
            FH = np.fft.fft2(Hfull[b, a], s=(FY, FX)).astype(cdt)[:, :RX]
            accum += Sfull * FH[None]
    full_img = np.fft.irfft2(accum, s=(FY, FX), axes=(1, 2)).astype(dtype)
    full_img = full_img[:, :full[0], :full[1]]
    return _centered(full_img, (Y, X)).astype(dtype)


def project_plane_direct(src, Hred, Nnum, dtype=np.float64):
    """Definition of one plane's projection: per-offset masked ``fftconvolve(..., 'same')``.

    Follows ``ForwardProjectForZ_old`` / ``BackwardProjectForZ_old``
    (projector.py:1084-1126) with the expanded PSF set.  Slow; used in
    float64 as the FP64 oracle on small cases.
    """
    src = np.asarray(src, dtype=dtype)
    if src.ndim == 2:
        src = src[np.newaxis]
    N = int(Nnum)
    Hfull = expand_psf_set(np.asarray(Hred, dtype=dtype), N)
    out = np.zeros(src.shape, dtype=dtype)
    for t in range(src.shape[0]):
        for b in range(N):
            for a in range(N):
                tmp = np.zeros(src.shape[1:], dtype=dtype)
                tmp[b::N, a::N] = src[t, b::N, a::N]
                out[t] += fftconvolve(tmp, Hfull[b, a], "same")
    return out


# ---------------------------------------------------------------------------
# Whole-volume projections (projector.py:806-896)
# ---------------------------------------------------------------------------

def _plane_fn(method):
    if method == "special":
        return lambda s, H, N, dt: project_plane_special(s, H, N, True, dt)
    if method == "special_gpu_pad":
        return lambda s, H, N, dt: project_plane_special(s, H, N, False, dt)
    if method == "direct":
        return lambda s, H, N, dt: project_plane_direct(s, H, N, dt)
    raise ValueError(method)


def backward_project(Ht_planes, img, Nnum, planes=None, method="special", dtype=np.float32):
    """``[Z, T, Y, X]`` back projection of ``img [T, Y, X]`` with per-plane ``Ht`` quadrants."""
    img = np.asarray(img)
    if planes is None:
        planes = range(len(Ht_planes))
    fn = _plane_fn(method)
    out = np.zeros((len(Ht_planes),) + img.shape, dtype=dtype)
    for cc in planes:
        out[cc] = fn(img, Ht_planes[cc], Nnum, dtype)
    return out


def forward_project(H_planes, vol, Nnum, planes=None, method="special", dtype=np.float32):
    """``[T, Y, X]`` forward projection of ``vol [Z, T, Y, X]`` (sum over planes)."""
    vol = np.asarray(vol)
    if planes is None:
        planes = range(len(H_planes))
    fn = _plane_fn(method)
    out = None
    for cc in planes:
        p = fn(vol[cc], H_planes[cc], Nnum, dtype)
        out = p if out is None else out + p
    return out.astype(dtype)


# ---------------------------------------------------------------------------
# Richardson-Lucy (lfdeconv.py:72-202)
# ---------------------------------------------------------------------------

def deconv_rl(H_planes, Ht_planes, Nnum, max_iter, im=None, Htf=None, x0=None,
              prevedel=True, trust_mask=None, method="special", dtype=np.float32):
    """Richardson-Lucy deconvolution as the reference driver runs it.

    ``Htf`` (the back projection of ``im``) is computed when not given and
    ``Xguess`` defaults to a copy of it (lfdeconv.py:84-103).  Prevedel
    variant: ``x *= Htf / Ht(H x)``; standard: ``x *= Ht(im / Hx)``,
    divided by ``Ht(trust_mask)`` when a mask is given.  NaN -> 0 after each
    update (lfdeconv.py:118-125, 151-164).
    """
    if Htf is None and (prevedel or x0 is None):
        Htf = backward_project(Ht_planes, im, Nnum, method=method, dtype=dtype)
    x = (np.array(Htf, dtype=dtype, copy=True) if x0 is None
         else np.array(x0, dtype=dtype, copy=True))
    trust_back = None
    if trust_mask is not None:
        trust_back = backward_project(Ht_planes, np.asarray(trust_mask, dtype=dtype)[np.newaxis],
                                      Nnum, method=method, dtype=dtype)
    with np.errstate(divide="ignore", invalid="ignore"):
        for _ in range(max_iter):
            hx = forward_project(H_planes, x, Nnum, method=method, dtype=dtype)
            if prevedel:
                bp = backward_project(Ht_planes, hx, Nnum, method=method, dtype=dtype)
                x *= (np.asarray(Htf, dtype=dtype) / bp)
            else:
                err = (np.asarray(im, dtype=dtype) / hx).astype(dtype)
                bp = backward_project(Ht_planes, err, Nnum, method=method, dtype=dtype)
                x *= bp
                if trust_back is not None:
                    x /= trust_back
            x[np.isnan(x)] = 0
    return x


# ---------------------------------------------------------------------------
# CPU baseline: the reference's production algorithm with its symmetry reuse
# ---------------------------------------------------------------------------

def project_plane_ref_cpu(src, Hred, Nnum, workers=-1, dtype=np.float32):
    """One plane of the reference's CPU projection, as ``Projector_allC`` computes it.

    Per plane: one real FFT per stored quadrant PSF (``FHWorkItem``,
    py_light_field.cpp:781-812; transposed quadrant positions FFT the
    transposed PSF, :1526-1541), mirrored offsets reuse those spectra with
    an index flip, a conjugate and a phase ramp (``MirrorYArray`` /
    ``CalculateRowMirror``, :284-341; multipliers projector.py:137-151); per
    offset the strided sub-image FFT is tiled with phase ramps and
    multiply-accumulated (``ConvolveWorkItem``, :1001-1087); one inverse real
    FFT and a centred crop finish the plane (:925-950, projector.py:792-796).
    The offsets are visited grouped by the stored spectrum they use, so only one
    spectrum is held at a time.  ``dtype`` float32 is the reference's single
    precision (py_light_field.cpp works in complex<float>); float64 is the same
    algorithm in double precision.  FFTs use scipy with ``workers`` threads
    (the reference's FFTW thread pool).
    """
    import scipy.fft as sfft
    cdt = np.complex64 if dtype == np.float32 else np.complex128
    src = np.asarray(src, dtype=dtype)
    if src.ndim == 2:
        src = src[np.newaxis]
    T, Y, X = src.shape
    N = int(Nnum)
    c = N // 2
    Hred = np.asarray(Hred, dtype=dtype)
    h = Hred.shape[-1]
    (FY, FX), full = convolution_shape((Y, X), (h, h), N, True)
    fy, fx = FY // N, FX // N
    RX = FX // 2 + 1
    ky = np.arange(FY)
    kx = np.arange(RX)
    ph_y = np.exp(-2j * np.pi * ky * (h - 1) / FY).astype(cdt)     # row flip
    ph_x = np.exp(-2j * np.pi * kx * (h - 1) / FX).astype(cdt)     # column flip
    yflip = (-ky) % FY
    accum = np.zeros((T, FY, RX), dtype=cdt)
    groups = {}
    for b in range(N):
        for a in range(N):
            groups.setdefault((min(b, N - 1 - b), min(a, N - 1 - a)), []).append((b, a))
    for (bb, aa), offsets in groups.items():
        P = Hred[bb, aa] if aa >= bb else Hred[aa, bb].T
        Fb = sfft.rfft2(P, s=(FY, FX), workers=workers).astype(cdt)
        for b, a in offsets:
            if b > c and a > c:
                FH = np.conj(Fb) * (ph_y[:, None] * ph_x[None, :])
            elif b > c:
                FH = Fb[yflip] * ph_y[:, None]
            elif a > c:
                FH = np.conj(Fb[yflip]) * ph_x[None, :]
            else:
                FH = Fb
            ey = np.exp(-2j * np.pi * b * ky / FY).astype(cdt)
            ex = np.exp(-2j * np.pi * a * kx / FX).astype(cdt)
            Ss = sfft.fft2(src[:, b::N, a::N], s=(fy, fx), axes=(1, 2), workers=workers).astype(cdt)
            Sx = Ss[:, :, kx % fx] * ex[None, None, :]
            Sf = Sx[:, ky % fy, :] * ey[None, :, None]
            accum += Sf * FH[None]
    img = sfft.irfft2(accum, s=(FY, FX), axes=(1, 2), workers=workers).astype(dtype)
    img = img[:, :full[0], :full[1]]
    return _centered(img, (Y, X)).astype(dtype)
