"""PSF matrix store, with the interface of the reference's psfmatrix.py.

``HMatrix`` serves the stored PSF quadrant of each z plane,
``H[bb][aa]`` / ``Ht[bb][aa]`` for ``0 <= bb, aa < (Nnum+1)/2``, each a
``h_z x h_z`` float32 array, from the reference's on-disk memmap layout
(``<mat stem>/H{z:02d}.array``, ``Ht{z:02d}.array`` and ``HReducedShape.npy``;
reference psfmatrix.py:14-98, 164-188).  ``HMatrixArrays`` holds the same data
in memory.  The projector uploads these arrays to the GPU once; the spectra
are precomputed there (reference: recomputed by FHWorkItem on every call).
"""

import os
import warnings

import numpy as np

__all__ = ["HMatrix", "HMatrixArrays", "GetPathFormats", "LoadRawMatrixData", "SaveRawMatrixData", "LoadMatrix",
           "SaveReducedMatrices"]


class HMatrix(object):
    """Memory-mapped reduced PSF matrices (reference psfmatrix.py:14-91)."""

    def __init__(self, HPathFormat, HtPathFormat, HReducedShape, numZ=None, zStart=0,
                 cacheMMap=True, cacheH=False):
        self.HPathFormat = HPathFormat
        self.HtPathFormat = HtPathFormat
        self.HReducedShape = [tuple(int(v) for v in s) for s in HReducedShape]
        self.numZ = int(numZ) if numZ is not None else len(self.HReducedShape)
        self.zStart = int(zStart)
        # Nnum follows from the quadrant size: n_h = (Nnum+1)/2 (psfmatrix.py:26-27)
        self.Nnum = self.HReducedShape[0][0] * 2 - 1
        self.iterableBRange = range(self.HReducedShape[0][0])
        self.cacheH = cacheH
        self.cacheMMap = cacheMMap
        self.mappedH = dict()
        self.mappedHt = dict()
        if self.zStart + self.numZ > len(self.HReducedShape):
            raise ValueError("zStart %d + numZ %d exceeds the %d stored planes"
                             % (self.zStart, self.numZ, len(self.HReducedShape)))

    def Hcc(self, cc, useHt):
        """``[n_h, n_h, h, h]`` float32 PSF quadrant of plane ``cc`` (reference :46-66)."""
        cache = self.mappedHt if useHt else self.mappedH
        key = str(cc)
        if self.cacheMMap and key in cache:
            return cache[key]
        fmt = self.HtPathFormat if useHt else self.HPathFormat
        result = np.memmap(fmt.format(z=cc + self.zStart), dtype="float32", mode="r",
                           shape=tuple(self.HReducedShape[cc + self.zStart]))
        if self.cacheMMap:
            cache[key] = result
        return result

    def UpdateFFTFunc(self, fftFunc):
        """Kept for interface compatibility; spectra are computed on the GPU."""
        return None

    def ClearCache(self):
        self.mappedH.clear()
        self.mappedHt.clear()

    def PSFShape(self, cc):
        s = self.HReducedShape[cc + self.zStart]
        return (s[2], s[3])

    def identity(self):
        """Key under which a projector caches this matrix's GPU transfer matrices."""
        return (self.HPathFormat, self.HtPathFormat, self.zStart, self.numZ)


class HMatrixArrays(HMatrix):
    """In-memory PSF matrices with the HMatrix interface.

    ``H`` and ``Ht`` are sequences (one per plane) of ``[n_h, n_h, h, h]`` arrays.
    """

    _counter = 0

    def __init__(self, H, Ht, numZ=None, zStart=0, name=None):
        H = [np.ascontiguousarray(h, dtype=np.float32) for h in H]
        Ht = [np.ascontiguousarray(h, dtype=np.float32) for h in Ht]
        if len(H) != len(Ht):
            raise ValueError("H and Ht must have the same number of planes")
        for a, b in zip(H, Ht):
            if a.shape != b.shape or a.ndim != 4 or a.shape[0] != a.shape[1] or a.shape[2] != a.shape[3]:
                raise ValueError("each plane must be [n_h, n_h, h, h] for both H and Ht")
        HMatrixArrays._counter += 1
        tag = name or ("arrays#%d" % HMatrixArrays._counter)
        super().__init__("mem:%s/H{z:02d}" % tag, "mem:%s/Ht{z:02d}" % tag,
                         [a.shape for a in H], numZ=numZ, zStart=zStart, cacheMMap=False)
        self._H = H
        self._Ht = Ht

    def Hcc(self, cc, useHt):
        return (self._Ht if useHt else self._H)[cc + self.zStart]


def GetPathFormats(matPath):
    """Memmap folder and path formats for a .mat file (reference psfmatrix.py:93-98)."""
    mmapPath = os.path.splitext(matPath)[0]
    return (mmapPath, mmapPath + "/H{z:02d}.array", mmapPath + "/Ht{z:02d}.array")


def SaveReducedMatrices(mmapPath, H, Ht):
    """Write per-plane quadrants in the reference's memmap layout (psfmatrix.py:134-165)."""
    os.makedirs(mmapPath, exist_ok=True)
    shapes = []
    for z, (h, ht) in enumerate(zip(H, Ht)):
        for name, arr in (("H", h), ("Ht", ht)):
            arr = np.asarray(arr, dtype=np.float32)
            m = np.memmap(os.path.join(mmapPath, "%s%02d.array" % (name, z)), dtype="float32",
                          mode="w+", shape=arr.shape)
            m[...] = arr
            m.flush()
            del m
        shapes.append(np.asarray(h).shape)
    np.save(os.path.join(mmapPath, "HReducedShape.npy"), np.array(shapes))
    np.save(os.path.join(mmapPath, "HtReducedShape.npy"), np.array(shapes))


def SaveRawMatrixData(matPath, H, Ht, CAindex, params=None):
    """Write a PSF .mat (HDF5) file in the reference's layout (generate_psf.py:739-785,
    ``SaveMatrices``): the per-plane quadrants H[z] / Ht[z] ([nh][nh][h][h]) placed at
    their CAindex window (1-based, [2][Z]) in full [Z][nh][nh][L][L] arrays, CAindex
    stored as [Z][2], ``ReducedMatrix`` True, ``Nnum`` and the other scalars of
    ``params``.  LoadRawMatrixData reads it back to the same quadrants.  Written with
    hdf5lite (contiguous datasets, as h5py lays them out by default)."""
    import hdf5lite
    CA = np.asarray(CAindex, dtype=np.int64)
    nz = len(H)
    nh = np.asarray(H[0]).shape[0]
    L = int(CA[1].max())
    items = dict(params or {})
    items["CAindex"] = CA.T.copy()
    items["ReducedMatrix"] = True
    for key, planes in (("H", H), ("Ht", Ht)):
        full = np.zeros((nz, nh, nh, L, L), np.float32)
        for cc in range(nz):
            a, b = int(CA[0, cc]) - 1, int(CA[1, cc])
            full[cc, :, :, a:b, a:b] = planes[cc]
        items[key] = full
    if "Nnum" not in items:
        items["Nnum"] = np.int64(2 * nh - 1)
    hdf5lite.write(matPath, items)


def LoadRawMatrixData(matPath, expectedNnum=None, createPSF=True):
    """Convert a reference PSF .mat (HDF5) file into the memmap layout (psfmatrix.py:100-167).

    Keys read: ``CAindex``, ``Nnum``, ``ReducedMatrix``, ``H``, ``Ht``.  The file is
    opened with h5py where it is installed, else with this package's own HDF5
    reader (hdf5lite: contiguous, compact and chunked/deflate datasets, as h5py
    and MATLAB write them).
    """
    try:
        import h5py
        opener = h5py.File
    except ImportError:
        import hdf5lite
        opener = hdf5lite.File
    if not os.path.exists(matPath):
        raise FileNotFoundError("%s does not exist (LoadMatrix(..., createPSF=True) generates it)" % matPath)
    mmapPath, hPathFormat, htPathFormat = GetPathFormats(matPath)
    os.makedirs(mmapPath, exist_ok=True)
    with opener(matPath, "r") as f:
        CA = f["CAindex"][()].astype("int")
        if CA.shape[1] == 2:
            CA = CA.T
        Nnum = int(f["Nnum"][()])
        if expectedNnum is not None and Nnum != expectedNnum:
            warnings.warn("Nnum={0} from file does not match expected value {1}".format(Nnum, expectedNnum))
        try:
            reduced = bool(f["ReducedMatrix"][()])
        except KeyError:
            reduced = False
        nh = (Nnum + 1) // 2
        Hq, Htq = [], []
        for key, dst in (("H", Hq), ("Ht", Htq)):
            full = f[key][()].astype("float32")
            assert full.shape[2] == (nh if reduced else Nnum)
            for cc in range(full.shape[0]):
                dst.append(np.ascontiguousarray(
                    full[cc, :nh, :nh, CA[0, cc] - 1:CA[1, cc], CA[0, cc] - 1:CA[1, cc]]))
    SaveReducedMatrices(mmapPath, Hq, Htq)
    return (Hq, Htq, CA, hPathFormat, htPathFormat, [h.shape for h in Hq], [h.shape for h in Htq])


def LoadMatrix(matPath, numZ=None, zStart=0, forceRegeneration=False, cacheH=False, createPSF=False):
    """HMatrix for a .mat file, using its memmap folder when present (psfmatrix.py:169-188).

    With ``createPSF`` a matrix that exists neither as .mat nor as memmap folder is
    generated on the GPU from the parameters in its file name (generate_psf.py)."""
    mmapPath, hPathFormat, htPathFormat = GetPathFormats(matPath)
    if createPSF:
        import generate_psf
        generate_psf.EnsureMatrixFileExists(matPath)
    try:
        if forceRegeneration:
            raise FileNotFoundError("forced regeneration")
        hReducedShape = np.load(mmapPath + "/HReducedShape.npy")
    except FileNotFoundError:
        (_, _, _, hPathFormat, htPathFormat, hReducedShape, _) = LoadRawMatrixData(matPath)
    return HMatrix(hPathFormat, htPathFormat, hReducedShape, numZ=numZ, zStart=zStart,
                   cacheH=cacheH, cacheMMap=True)
