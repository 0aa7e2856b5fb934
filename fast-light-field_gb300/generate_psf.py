"""Light-field PSF generation on one GB300, with the interface of the reference's generate_psf.py.

``GeneratePSF`` computes the reduced PSF matrices H and Ht of a light-field
microscope (the reference's generate_psf.py:63-737) with the heavy steps on
the GPU:

1. the Debye integral of the objective's field at every image-side point of
   every depth (reference: one adaptive ``quad`` per point and part, on CPU
   threads) -- ``flf_psf_debye``, composite Gauss-Legendre over theta with
   panels sized to the integrand's fastest phase rate, one FP64 J0 per node;
2. for every lenslet offset and depth, the shifted field times the microlens
   array -- ``flf_psf_lf_input``; the Fresnel propagation over the microlens
   focal length as an FFT pair (cuFFT through torch.fft, complex128);
   |field|^2, aperture window, OSR x OSR binning and the lenslet-grid crop --
   ``flf_psf_lf_bin``;
3. the global maximum, per-plane clipping at 0.5 % of the plane maximum and
   per-offset normalisation (torch reductions on the device), CAindex, and Ht
   -- ``flf_psf_ht`` (a gather in place of the reference's stamping).

The result is written in the reference's memmap layout (``<stem>/H{z}.array``,
``Ht{z}.array``, ``HReducedShape.npy``, ``HtReducedShape.npy``), which
``psfmatrix.LoadMatrix`` reads, plus ``PSFInfo.json`` with the optical
parameters, CAindex and Hmax; the reference's HDF5 ``.mat`` needs h5py.

``GeneratePSF(..., maxPSFLenslets=20)`` keeps the reference's size limit
("Estimated PSF size exceeds the limit", generate_psf.py:160-166); a larger
value lets deeper z ranges through.
"""

import json
import os
import re
import time
import warnings

import numpy as np

import _flf
import psfmatrix

try:
    import torch
except ImportError:  # torch is needed for device arrays
    torch = None

__all__ = ["GeneratePSF", "GeneratePSFArrays", "GeneratePSFFromFilePath", "EnsureMatrixFileExists",
           "MatrixFileString"]

# quadrature: Gauss-Legendre order per panel and the largest phase change a panel spans
GL_ORDER = 16
PANEL_RADIANS = 8.0
# device memory for the fields of one batch of lenslet offsets (complex128 L x L each)
FIELD_BATCH_BYTES = 4 << 30


def MatrixFileString(M, NA, MLPitch, fml, zmin, zmax, zspacing, Nnum, lam, n):
    """The parameter part of the reference's matrix file names (generate_psf.py:89-92)."""
    return "M%gNA%gMLPitch%gfml%gfrom%gto%gzspacing%gNnum%glambda%gn%g" % (
        M, NA, MLPitch * 1e6, fml * 1e6, zmin * 1e6, zmax * 1e6, zspacing * 1e6, Nnum, lam * 1e9, n)


def _quadrature(alpha, uOver2, alphaFactor, k_rmax):
    """Nodes (sin theta) and complex weights of the Debye integral over [0, alpha] for one
    depth; the depth's phase exp(-i uOver2 alphaFactor sin^2(theta/2)) and the smooth
    factor sqrt(cos) (1 + cos) sin are folded into the weights."""
    rate = k_rmax + abs(uOver2) * alphaFactor * np.sin(alpha) / 2
    panels = max(8, int(np.ceil(alpha * rate / PANEL_RADIANS)))
    x, w = np.polynomial.legendre.leggauss(GL_ORDER)
    e = np.linspace(0.0, alpha, panels + 1)
    half = (e[1:] - e[:-1])[:, None] / 2
    th = ((e[1:] + e[:-1])[:, None] / 2 + half * x[None, :]).ravel()
    wt = (half * w[None, :]).ravel()
    ct, st, s2 = np.cos(th), np.sin(th), np.sin(th / 2)
    ph = -uOver2 * (s2 * s2) * alphaFactor
    cw = wt * np.sqrt(ct) * (1 + ct) * st * (np.cos(ph) + 1j * np.sin(ph))
    return st, cw


class _Generator:
    def __init__(self, M, NA, MLPitch, Nnum, OSR, n, fml, lam, zmin, zmax, zspacing, device):
        if torch is None:
            raise _flf.FlfError(-4, "PyTorch is required for device arrays")
        assert (Nnum % 2) == 1, "Nnum must be an odd number"
        assert (OSR % 2) == 1, "OSR must be an odd number"
        _flf.load_library()
        self.dev = torch.device("cuda", device)
        self.M, self.NA, self.N, self.OSR, self.n, self.fml, self.lam = M, NA, Nnum, OSR, n, fml, lam
        self.k = 2 * np.pi * n / lam
        self.k0 = 2 * np.pi / lam
        self.fobj = 200e-3 / M
        self.alpha = np.arcsin(NA / n)
        self.pixelPitch = MLPitch / Nnum
        self.dx = self.pixelPitch / OSR
        self.x3 = np.arange(zmin, zmax + 0.1 * zspacing, zspacing)
        assert len(self.x3) > 1
        self.p3max = np.max(np.abs(self.x3))
        self.stream = torch.cuda.current_stream(self.dev).cuda_stream

    def debye(self, p3, mode, count):
        """Koi * I0 at the octant offsets up to count (mode 0) or the line 0..count-1 (mode 1)."""
        alpha, k = self.alpha, self.k
        u = 4 * k * (p3 * 1) * (np.sin(alpha / 2) ** 2)
        Koi = self.M / ((self.fobj * self.lam) ** 2) * np.exp(-1j * u / (4 * (np.sin(alpha / 2) ** 2)))
        alphaFactor = np.sin(alpha / 2) ** (-2)
        far = count * np.sqrt(2.0) if mode == 0 else count
        st, cw = _quadrature(alpha, u / 2, alphaFactor, k * self.dx * far / self.M)
        s_d = torch.as_tensor(st, device=self.dev)
        cw_d = torch.as_tensor(cw, device=self.dev)
        npts = (count + 1) * (count + 2) // 2 if mode == 0 else count
        out = torch.empty(max(npts, 1), dtype=torch.complex128, device=self.dev)
        _flf.psf_debye(out, mode, npts, self.dx, self.M, k, np.sin(alpha), s_d, cw_d, Koi, self.stream)
        return out, len(st)

    def size_ref(self, limit):
        """IMGSIZE_REF: lenslets until the focal-plane intensity at the deepest plane
        falls below 4 % (generate_psf.py:156-166)."""
        npts = self.N * self.OSR * limit + 1
        line, _ = self.debye(self.p3max, 1, npts)
        inten = (line.abs() ** 2).cpu().numpy()
        inten = inten / np.max(inten)
        out = np.where(inten < 0.04)[0]
        if len(out) == 0:
            raise ValueError("Estimated PSF size exceeds the limit")
        return int(np.ceil(out[0] / (self.OSR * self.N)))


def GeneratePSFArrays(M, NA, MLPitch, Nnum, OSR, n, fml, lam, zmin, zmax, zspacing, normalisePSF=True,
                      reproduceMaxBug=False, maxPSFLenslets=20, device=0, verbose=False):
    """Compute the PSF matrices on the GPU without writing files.

    Returns a dict: ``H`` / ``Ht`` (lists, per plane, of the reduced quadrant
    ``[nh, nh, h_z, h_z]`` float32 in the memmap layout psfmatrix reads),
    ``CAindex`` ``[2, Z]`` (1-based, inclusive, as the reference saves it),
    ``Hmax``, ``IMGSIZE_REF``, ``x3objspace``, ``H_device`` / ``Ht_device``
    (``[Z, nh, nh, S, S]`` float32 on the device: ``H_device[z, a, b, i, j]``
    is the reference's ``H[i, j, a, b, z]``) and ``timings``.
    """
    if not normalisePSF:
        warnings.warn("We are not normalising the PSF. It should be normalised for standard deconvolution!")
    t_all = time.time()
    g = _Generator(M, NA, MLPitch, Nnum, OSR, n, fml, lam, zmin, zmax, zspacing, device)
    N, dev = Nnum, g.dev
    timings = {}
    t0 = time.time()
    ref = g.size_ref(maxPSFLenslets)
    timings["size_estimate_s"] = time.time() - t0

    IMG_HALFWIDTH = int(np.maximum(N * (ref + 1), 2 * N))
    L = 2 * IMG_HALFWIDTH * OSR + 1
    c = (L - 1) // 2
    m = N * OSR
    h = (m - 1) // 2
    assert c % m == 0
    # microlens phase (generate_psf.py:168-205): one lens, tiled from the grid centre
    xml = g.dx * np.arange(-(m - 1) / 2, (m - 1) / 2 + 0.1, 1)
    lens = np.exp(-1j * g.k0 / (2 * fml) * (xml[:, None] ** 2 + xml[None, :] ** 2))
    lens_d = torch.as_tensor(np.ascontiguousarray(lens), device=dev)
    # Fresnel transfer function over fml (generate_psf.py:246-261); its constant
    # phase exp(i k z) drops out of |field|^2
    du = 1 / (L * g.dx)
    u = np.append(np.arange(0, np.ceil(L / 2)), np.arange(np.ceil(-L / 2), 0)) * du
    kv = 2 * np.pi / lam
    fres = np.exp(-1j * 2 * np.pi ** 2 * (u[:, None] ** 2 + u[None, :] ** 2) * fml / kv)
    fres_d = torch.as_tensor(fres, device=dev)
    del fres

    cpt = c + 1
    halfWidth = N * ref * OSR
    CP = np.arange((cpt - 1) / OSR - halfWidth / OSR, (cpt - 1) / OSR + halfWidth / OSR + 0.1, 1, dtype=int)
    S = len(CP)
    lo = max(cpt - 1 - halfWidth, 0)
    hi = min(cpt - 1 + halfWidth, L - 1)
    # pixelBinning's crop start (generate_psf.py:479-500); identical in both axes
    ctr = int((L - 1) / 2 + 1)
    init = ctr - int((OSR - 1) / 2)
    init -= int(np.floor(init / OSR) * OSR)
    shift = 0
    if init < 1:
        init += OSR
        shift = 1
    first = (init - 1) + (int(CP[0]) - shift) * OSR
    nh = (N + 1) // 2
    Z = len(g.x3)
    Hd = torch.empty((Z, nh, nh, S, S), dtype=torch.float32, device=dev)
    per = max(1, min(nh * nh, FIELD_BATCH_BYTES // (16 * L * L)))
    field = torch.empty((per, L, L), dtype=torch.complex128, device=dev)
    t_deb = t_lf = 0.0
    nodes_total = 0
    for zi, p3 in enumerate(g.x3):
        ref_il = np.ceil(ref * (np.abs(p3) / g.p3max))
        hw_il = int(np.maximum(N * ref_il * OSR, 2 * N * OSR))
        support = min(hw_il, c)
        torch.cuda.synchronize(dev)
        t0 = time.time()
        wave, nodes = g.debye(p3, 0, support)
        nodes_total += nodes
        bug = bool(reproduceMaxBug and np.abs(p3) < 1e-10)
        if bug:
            warnings.warn("Reproducing matlab bug!")
        torch.cuda.synchronize(dev)
        t_deb += time.time() - t0
        t0 = time.time()
        for q0 in range(0, nh * nh, per):
            nq = min(per, nh * nh - q0)
            f = field[:nq]
            _flf.psf_lf_input(f, wave, support, bug, lens_d, h, L, nh, OSR, q0, nq, g.stream)
            spec = torch.fft.fft2(f)
            spec *= fres_d
            f.copy_(torch.fft.ifft2(spec))
            del spec
            out = Hd[zi].view(nh * nh, S, S)[q0:q0 + nq]
            _flf.psf_lf_bin(out, f, L, S, nh, OSR, q0, nq, lo, hi, first, g.stream)
        torch.cuda.synchronize(dev)
        t_lf += time.time() - t0
        if verbose:
            print("plane %d/%d: support %d, %d nodes" % (zi + 1, Z, support, nodes), flush=True)
        del wave
    del field
    timings["debye_s"] = t_deb
    timings["light_field_s"] = t_lf
    timings["quadrature_nodes"] = nodes_total

    t0 = time.time()
    Hmax = Hd.max()
    Hd /= Hmax
    tol = torch.tensor(0.005, dtype=torch.float32, device=dev)
    for zi in range(Z):
        sl = Hd[zi]
        sl[sl < tol * sl.max()] = 0
    if normalisePSF:
        for zi in range(Z):
            sums = Hd[zi].sum(dim=(2, 3), dtype=torch.float64, keepdim=True)
            Hd[zi].copy_((Hd[zi].double() / sums).float())
    else:
        warnings.warn("Not normalising H properly (as instructed!)")
        Hd /= Hd.max()
    Htd = torch.empty_like(Hd)
    _flf.psf_ht(Htd, Hd, Z, nh, S, N, g.stream)
    # CAindex (generate_psf.py:604-612), 1-based inclusive
    centreCP = np.ceil(S / 2)
    CA = np.zeros((2, Z), dtype=int)
    for i in range(Z):
        ref_il = np.ceil(ref * (np.abs(g.x3[i]) / g.p3max))
        hw_il = np.maximum(N * ref_il, 2 * N)
        CA[0, i] = np.maximum(centreCP - hw_il, 1)
        CA[1, i] = np.minimum(centreCP + hw_il, S)
    Hq, Htq = [], []
    for zi in range(Z):
        a0, a1 = CA[0, zi] - 1, CA[1, zi]
        Hq.append(Hd[zi].permute(1, 0, 3, 2)[:, :, a0:a1, a0:a1].contiguous().cpu().numpy())
        Htq.append(Htd[zi].permute(1, 0, 3, 2)[:, :, a0:a1, a0:a1].contiguous().cpu().numpy())
    timings["normalise_ht_copy_s"] = time.time() - t0
    timings["total_s"] = time.time() - t_all
    return dict(H=Hq, Ht=Htq, CAindex=CA, Hmax=float(Hmax), IMGSIZE_REF=ref, x3objspace=g.x3,
                H_device=Hd, Ht_device=Htd, image_size=L, timings=timings)


def GeneratePSF(M, NA, MLPitch, Nnum, OSR, n, fml, lam, zmin, zmax, zspacing, normalisePSF=True,
                reproduceMaxBug=False, matrixSaveDir="PSFmatrix", verbose=False, maxPSFLenslets=20, device=0,
                matPath=None, saveMat=False):
    """Generate and save the PSF matrices (generate_psf.py:63-737); returns the matrix path.

    The files go to ``<matrixSaveDir>/<prefix>PSFmatrix_<parameters>/`` in the
    memmap layout, where ``<prefix>`` is ``fdnorm`` (normalised), ``reducedBuggy``
    or ``reduced``, as in the reference (or to the folder of ``matPath``);
    ``psfmatrix.LoadMatrix`` opens the returned ``.mat`` path through that folder.
    With ``saveMat`` the ``.mat`` file itself is written too, in the reference's
    HDF5 layout (``psfmatrix.SaveRawMatrixData``), as the reference always does.
    """
    r = GeneratePSFArrays(M, NA, MLPitch, Nnum, OSR, n, fml, lam, zmin, zmax, zspacing, normalisePSF,
                          reproduceMaxBug, maxPSFLenslets, device, verbose)
    if matPath is None:
        prefix = "fdnorm" if normalisePSF else ("reducedBuggy" if reproduceMaxBug else "reduced")
        matPath = os.path.join(matrixSaveDir, "%sPSFmatrix_%s.mat" % (
            prefix, MatrixFileString(M, NA, MLPitch, fml, zmin, zmax, zspacing, Nnum, lam, n)))
    mmapPath, _, _ = psfmatrix.GetPathFormats(matPath)
    psfmatrix.SaveReducedMatrices(mmapPath, r["H"], r["Ht"])
    info = dict(M=M, NA=NA, MLPitch=MLPitch, Nnum=Nnum, OSR=OSR, n=n, fml=fml, **{"lambda": lam},
                zmin=zmin, zmax=zmax, zspacing=zspacing, fobj=200e-3 / M, d=fml,
                x3objspace=[float(v) for v in r["x3objspace"]], pixelPitch=MLPitch / Nnum,
                CAindex=r["CAindex"].T.tolist(), Hmax=r["Hmax"], ReducedMatrix=True,
                IMGSIZE_REF=r["IMGSIZE_REF"])
    with open(os.path.join(mmapPath, "PSFInfo.json"), "w") as f:
        json.dump(info, f, indent=1)
    if saveMat:
        scalars = {k: v for k, v in info.items() if k not in ("CAindex", "ReducedMatrix", "IMGSIZE_REF")}
        psfmatrix.SaveRawMatrixData(matPath, r["H"], r["Ht"], r["CAindex"], scalars)
    if verbose:
        print("PSF matrices written to %s (%.1f s)" % (mmapPath, r["timings"]["total_s"]))
    return matPath


_NAME_RE = re.compile(r"M([-+.\deE]+)NA([-+.\deE]+)MLPitch([-+.\deE]+)fml([-+.\deE]+)from([-+.\deE]+)"
                      r"to([-+.\deE]+)zspacing([-+.\deE]+)Nnum(\d+)lambda([-+.\deE]+)n([-+.\deE]+)$")


def GeneratePSFFromFilePath(filePath, OSR=3, **kw):
    """Generate the matrices a file name describes (generate_psf.py:740-775)."""
    filename = os.path.basename(filePath)
    reproduceMaxBug = False
    if filename.startswith("fdnormPSFmatrix_"):
        normalisePSF = True
    elif filename.startswith("reducedPSFmatrix_"):
        normalisePSF = False
    elif filename.startswith("reducedBuggyPSFmatrix_"):
        normalisePSF = False
        reproduceMaxBug = True
    elif filename.startswith("PSFmatrix_"):
        raise ValueError("We cannot generate filename %s because this filename represents a matrix generated "
                         "from Matlab. We can only generate fdnormPSFmatrix or reducedPSFmatrix." % filename)
    else:
        raise ValueError("Unrecognised matrix file prefix on filename %s" % filename)
    suffix, ext = os.path.splitext(filename[filename.find("PSFmatrix_") + 10:])
    if ext != ".mat":
        raise ValueError("We have been asked to generate filename %s, but can only generate .mat files" % filename)
    mt = _NAME_RE.match(suffix)
    if mt is None:
        raise ValueError("Failed to parse filename %s. Check documentation for correct filename format" % filename)
    M, NA, MLPitch, fml, zmin, zmax, zspacing = (float(mt.group(i)) for i in range(1, 8))
    Nnum = int(mt.group(8))
    lam, n = float(mt.group(9)), float(mt.group(10))
    return GeneratePSF(M, NA, MLPitch * 1e-6, Nnum, OSR, n, fml * 1e-6, lam * 1e-9, zmin * 1e-6, zmax * 1e-6,
                       zspacing * 1e-6, normalisePSF, reproduceMaxBug,
                       matrixSaveDir=os.path.dirname(filePath) or ".", matPath=filePath, **kw)


def EnsureMatrixFileExists(filePath):
    """Generate the matrices of ``filePath`` unless its .mat file or memmap folder exists
    (generate_psf.py:777-781)."""
    mmapPath, _, _ = psfmatrix.GetPathFormats(filePath)
    if os.path.exists(filePath) or os.path.exists(os.path.join(mmapPath, "HReducedShape.npy")):
        return
    print('== Matrix file "%s" needs to be generated from scratch ==' % filePath)
    GeneratePSFFromFilePath(filePath)
