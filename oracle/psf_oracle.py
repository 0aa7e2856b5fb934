"""ORACLE (test infrastructure only): CPU restatement of the reference's PSF generator.

Follows GeneratePSF in generate_psf.py:63-737 step by step, in numpy/scipy,
for the small optical configurations the tests use:

* the Debye integral of the objective's field (generate_psf.py:96-144 and
  263-315) by adaptive Gauss-Kronrod quadrature (scipy ``quad_vec`` over all
  points of a plane at once, where the reference calls ``quad`` per point)
  with scipy's J0 (the reference links a rational-approximation J0,
  light-field-integrands/bessel.c);
* the PSF size estimate (:156-166), microlens array (:168-205), octant
  fill by flips and rotations (:317-348), Fresnel propagation (:246-261),
  shifts and OSR binning (:456-513), per-offset light-field PSFs (:524-548),
  normalisation and clipping (:560-596), CAindex (:604-612) and the Ht
  rubber-stamping (:624-690).

Only tests/ may import this module.  It is pinned by
tests/golden/psf_vectors.npz, which the reference's own GeneratePSF wrote.
"""

import numpy as np
import scipy.integrate
import scipy.signal
import scipy.special


def optics(M, NA, MLPitch, Nnum, OSR, n, fml, lam, zmin, zmax, zspacing, **_):
    """Derived constants of GeneratePSF (generate_psf.py:77-87, 146-156)."""
    k = 2 * np.pi * n / lam
    ftl = 200e-3
    fobj = ftl / M
    alpha = np.arcsin(NA / n)
    pixelPitch = MLPitch / Nnum
    x3 = np.arange(zmin, zmax + 0.1 * zspacing, zspacing)
    return dict(k=k, k0=2 * np.pi / lam, fobj=fobj, alpha=alpha, pixelPitch=pixelPitch, x3=x3,
                p3max=np.max(np.abs(x3)))


def debye_field(x1, x2, p3, M, lam, n, o, epsrel=1e-12):
    """Koi * I0 at image-side points (x1, x2) for a point source at depth p3
    (generate_psf.py:263-315; the same integral at :96-144)."""
    k, alpha, fobj = o["k"], o["alpha"], o["fobj"]
    xL2normsq = (((np.asarray(x1, np.float64)) ** 2 + (np.asarray(x2, np.float64)) ** 2) ** 0.5) / M
    v = k * xL2normsq * np.sin(alpha)
    u = 4 * k * (p3 * 1) * (np.sin(alpha / 2) ** 2)
    Koi = M / ((fobj * lam) ** 2) * np.exp(-1j * u / (4 * (np.sin(alpha / 2) ** 2)))
    alphaFactor = np.sin(alpha / 2) ** (-2)
    uOver2 = u / 2
    vFactor = np.ravel(v / np.sin(alpha))
    m = vFactor.size

    def f(theta):
        ct, st, s2 = np.cos(theta), np.sin(theta), np.sin(theta / 2)
        common = np.sqrt(ct) * (1 + ct) * st * scipy.special.j0(st * vFactor)
        ph = -uOver2 * (s2 * s2) * alphaFactor
        return np.concatenate([common * np.cos(ph), common * np.sin(ph)])

    I, _ = scipy.integrate.quad_vec(f, 0, alpha, epsabs=0, epsrel=epsrel, norm="max", limit=100000)
    return (Koi * (I[:m] + 1j * I[m:])).reshape(np.shape(v))


def psf_size_ref(case, o, limit_lenslets=20):
    """IMGSIZE_REF (generate_psf.py:156-166)."""
    N, OSR = case["Nnum"], case["OSR"]
    x1test = (o["pixelPitch"] / OSR) * np.arange(0, N * OSR * limit_lenslets + 1)
    line = np.abs(debye_field(x1test, 0.0, o["p3max"], case["M"], case["lam"], case["n"], o, epsrel=1.49e-8) ** 2)
    line = line / np.max(line)
    out = np.where(line < 0.04)[0]
    if len(out) == 0:
        raise ValueError("Estimated PSF size exceeds the limit")
    return int(np.ceil(out[0] / (OSR * N)))


def ml_array(o, case, x1space, x2space):
    """Microlens phase array by convolving lens centres with one lens (generate_psf.py:168-205)."""
    N, OSR = case["Nnum"], case["OSR"]
    d = o["pixelPitch"] / OSR
    xml = d * np.arange(-(N * OSR - 1) / 2, (N * OSR - 1) / 2 + 0.1, 1)
    dist = len(xml)
    c1 = np.where(x1space == 0)[0][0]
    c2 = np.where(x2space == 0)[0][0]
    cen1 = np.append(np.arange(c1, -1, -dist), np.arange(c1 + dist, len(x1space), dist))
    cen2 = np.append(np.arange(c2, -1, -dist), np.arange(c2 + dist, len(x2space), dist))
    lens = np.exp(-1j * o["k0"] / (2 * case["fml"]) * (xml[:, None] ** 2 + xml[None, :] ** 2))
    centres = np.zeros((len(x1space), len(x2space)))
    centres[np.ix_(cen1, cen2)] = 1
    return scipy.signal.fftconvolve(centres.astype(np.complex128), lens, "same")


def psf_wave(p3, o, case, x1space, x2space, centre_area, reproduce_max_bug=False):
    """Objective field on the image grid for one depth: the octant a <= b <= centre
    by quadrature, then mirrored and rotated (generate_psf.py:317-348)."""
    L = len(x1space)
    cpt = int(np.ceil(L / 2))
    a0 = centre_area[0]
    A, B = np.meshgrid(np.arange(a0, cpt), np.arange(a0, cpt), indexing="ij")
    sel = B >= A
    pattern = np.zeros((L, L), np.complex128)
    pattern[A[sel], B[sel]] = debye_field(x1space[A[sel]], x2space[B[sel]], p3, case["M"], case["lam"],
                                          case["n"], o)
    pat3 = np.zeros((L, L, 4), np.complex128)
    pat3[:, :, 0] = pattern
    pat3[:cpt, cpt - 1:, 0] = np.fliplr(pattern[0:cpt, 0:cpt])
    for r in (1, 2, 3):
        pat3[:, :, r] = np.rot90(pat3[:, :, 0], -r)
    if reproduce_max_bug and np.abs(p3) < 1e-10:
        return np.max(pat3, axis=2)
    out = pat3[:, :, 0].copy()
    for r in (1, 2, 3):
        z = out == 0
        out[z] = pat3[:, :, r][z]
    return out


def fresnel2d(f0, dx0, z, lam):
    """Fresnel propagation by FFT (generate_psf.py:246-261)."""
    Nx, Ny = f0.shape
    k = 2 * np.pi / lam
    u = np.append(np.arange(0, np.ceil(Nx / 2)), np.arange(np.ceil(-Nx / 2), 0)) / (Nx * dx0)
    v = np.append(np.arange(0, np.ceil(Ny / 2)), np.arange(np.ceil(-Ny / 2), 0)) / (Ny * dx0)
    H = np.exp(-1j * 2 * np.pi ** 2 * (u[:, None] ** 2 + v[None, :] ** 2) * z / k)
    return np.exp(1j * k * z) * np.fft.ifft2(np.fft.fft2(f0) * H)


def im_shift2(img, sx, sy):
    """Shift with zero fill (generate_psf.py:456-477): out[i, j] = img[i - sx, j - sy]."""
    sx, sy = int(round(sx)), int(round(sy))
    out = np.zeros_like(img)
    X, Y = img.shape[:2]
    out[max(sx, 0):X + min(sx, 0), max(sy, 0):Y + min(sy, 0)] = \
        img[max(-sx, 0):X - max(sx, 0), max(-sy, 0):Y - max(sy, 0)]
    return out


def pixel_binning(simg, OSR):
    """Crop about the centre and sum OSR x OSR blocks (generate_psf.py:479-513)."""
    L1, L2 = simg.shape

    def start(L):
        centre = int((L - 1) / 2 + 1)
        init = centre - int((OSR - 1) / 2)
        init -= int(np.floor(init / OSR) * OSR)
        shift = 0
        if init < 1:
            init += OSR
            shift = 1
        return centre, init, shift

    c1, i1, s1 = start(L1)
    c2, i2, s2 = start(L2)
    hw = c1 - i1
    crop = simg[i1 - 1:c1 + hw, i2 - 1:c2 + hw]
    m, n = crop.shape
    return crop.reshape(m // OSR, OSR, n // OSR, OSR).sum(axis=(1, 3)), s1, s2


def calc_ht(H, Nnum):
    """Ht by stamping the rotated H of every offset (generate_psf.py:624-690)."""
    S, _, half, _, Z = H.shape
    t = int(np.ceil(S / Nnum))
    img = (t + 2) * Nnum if t % 2 == 1 else (t + 3) * Nnum
    imc = int(np.ceil(img / 2))
    imc0 = imc - int(np.ceil(Nnum / 2))
    hc = S // 2
    assert hc % Nnum == 0
    Ht = np.zeros_like(H)
    flipped = H[::-1, ::-1]
    for _aa in range(half):
        for _bb in range(half):
            back = np.zeros((img, img, Z))
            for aa in range(Nnum):
                for bb in range(Nnum):
                    h = flipped[:, :, aa] if aa <= Nnum // 2 else flipped[::-1, :, Nnum - 1 - aa]
                    h = h[:, :, bb] if bb <= Nnum // 2 else h[:, ::-1, Nnum - 1 - bb]
                    a0 = (aa - _aa) % Nnum
                    b0 = (bb - _bb) % Nnum
                    st = h[a0::Nnum, b0::Nnum]
                    r0 = imc0 + _aa - hc + a0
                    c0 = imc0 + _bb - hc + b0
                    back[r0:r0 + st.shape[0] * Nnum:Nnum, c0:c0 + st.shape[1] * Nnum:Nnum] = st
            cut = back[imc - (S - 1) // 2 - 1:imc + (S - 1) // 2, imc - (S - 1) // 2 - 1:imc + (S - 1) // 2]
            for cc in range(Z):
                Ht[:, :, _aa, _bb, cc] = im_shift2(cut[:, :, cc], int(np.ceil(Nnum / 2) - _aa - 1),
                                                   int(np.ceil(Nnum / 2) - _bb - 1))
    return Ht


def generate_psf(case, limit_lenslets=20):
    """H, Ht (reference layout [S, S, a, b, z] float32), CAindex [2, Z] and Hmax."""
    N, OSR = case["Nnum"], case["OSR"]
    o = optics(**case)
    ref = psf_size_ref(case, o, limit_lenslets)
    pp = o["pixelPitch"]
    IMG_HALFWIDTH = np.maximum(N * (ref + 1), 2 * N)
    x1space = (pp / OSR) * np.arange(-IMG_HALFWIDTH * OSR, IMG_HALFWIDTH * OSR + 0.1, 1)
    x2space = x1space.copy()
    L = len(x1space)
    ML = ml_array(o, case, x1space, x2space)
    cpt = int(np.ceil(L / 2))
    halfWidth = N * (ref + 0) * OSR
    x3 = o["x3"]
    waves = []
    for p3 in x3:
        ref_il = np.ceil(ref * (np.abs(p3) / o["p3max"]))
        hw_il = np.maximum(N * (ref_il + 0) * OSR, 2 * N * OSR)
        area = np.arange(np.maximum((cpt - hw_il), 1) - 1, np.minimum((cpt + hw_il), L), dtype=int)
        waves.append(psf_wave(p3, o, case, x1space, x2space, area, case.get("reproduceMaxBug", False)))
    XREF = int(np.ceil(N / 2))
    CP = np.arange((cpt - 1) / OSR - halfWidth / OSR, (cpt - 1) / OSR + halfWidth / OSR + 0.1, 1, dtype=int)
    H = np.zeros((len(CP), len(CP), XREF, XREF, len(x3)), np.float32)
    lo = max(cpt - 1 - halfWidth, 0)
    hi = min(cpt - 1 + halfWidth, L - 1)
    for c in range(len(x3)):
        for a in range(XREF):
            for b in range(XREF):
                sx, sy = OSR * (a + 1 - XREF), OSR * (b + 1 - XREF)
                f1 = fresnel2d(im_shift2(waves[c], sx, sy) * ML, pp / OSR, case["fml"], case["lam"])
                f1 = im_shift2(f1, -sx, -sy)
                ap = np.zeros_like(f1)
                ap[lo:hi + 1, lo:hi + 1] = f1[lo:hi + 1, lo:hi + 1]
                binned, s1, s2 = pixel_binning(np.abs(ap ** 2), OSR)
                H[:, :, a, b, c] = binned[CP - s1, :][:, CP - s2].astype(np.float32)
    Hmax = np.max(H)
    H /= Hmax
    for c in range(H.shape[4]):
        sl = H[:, :, :, :, c]
        sl[sl < (0.005 * np.max(sl))] = 0
    if case.get("normalisePSF", True):
        for c in range(H.shape[4]):
            for b in range(XREF):
                for a in range(XREF):
                    h = H[:, :, a, b, c]
                    h /= np.sum(h, dtype=np.float64)
    else:
        H /= np.max(H)
    centre_cp = np.ceil(len(CP) / 2)
    CA = np.zeros((2, len(x3)), dtype=int)
    for i in range(len(x3)):
        ref_il = np.ceil(ref * (np.abs(x3[i]) / o["p3max"]))
        hw_il = np.maximum(N * (ref_il + 0), 2 * N)
        CA[0, i] = np.maximum(centre_cp - hw_il, 1)
        CA[1, i] = np.minimum(centre_cp + hw_il, H.shape[0])
    Ht = calc_ht(H, N)
    return dict(H=H, Ht=Ht, CAindex=CA, Hmax=Hmax, IMGSIZE_REF=ref)


def saved_form(res):
    """The arrays as the reference's generator saves them (transposed, CAindex as [Z, 2])."""
    return dict(H=res["H"].T, Ht=res["Ht"].T, CAindex=res["CAindex"].T, Hmax=res["Hmax"])
