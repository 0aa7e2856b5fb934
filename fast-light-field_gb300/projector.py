"""Projector plugins with the interface of the reference's projector.py.

The reference selects its projection backend through the ``projector=``
argument of ``lfdeconv.BackwardProjectACC / ForwardProjectACC / DeconvRL``
(lfdeconv.py:27, 51, 72); every backend implements ``Projector_base``
(projector.py:769-790).  ``Projector_gb300`` is the GB300 backend: it hands
whole volumes to libflf.so (include/flf.h) through ctypes.  The names of the
reference's production classes (``Projector_allC``, ``Projector_gpuHelpers``)
are aliases of it, so code written against the reference picks up the GPU
path unchanged.

There is no CPU fallback: a projector raises ``_flf.FlfError`` when the CUDA
library or a GPU is missing.
"""

import os

import numpy as np

import _flf

try:
    import torch
except ImportError:  # torch is needed for device arrays
    torch = None

__all__ = ["Projector_base", "Projector_gb300", "Projector_allC", "Projector_gpuHelpers",
           "CheckPlanes"]


class Projector_base(object):
    """numpy helpers shared by projectors (reference projector.py:769-790)."""

    def __init__(self):
        super().__init__()
        self.storeVolumesOnGPU = False
        self.cacheFH = False

    def asnative(self, m):
        return np.asarray(m)

    def asnumpy(self, m, out=None):
        if out is not None:
            out[...] = m
            return out
        return np.asarray(m)

    def nativeZeros(self, shape, dtype=float):
        return np.zeros(shape, dtype)

    def nativeDivide(self, a, b, out):
        return np.divide(a, b, out=out)

    def assertNative(self, m):
        assert isinstance(m, np.ndarray)


def CheckPlanes(hMatrix, planes):
    """Normalise a ``planes`` argument to a list of distinct in-range plane ids."""
    if planes is None:
        return list(range(hMatrix.numZ))
    out = [int(p) for p in planes]
    if len(out) == 0:
        raise ValueError("planes must not be empty")
    for p in out:
        if p < 0 or p >= hMatrix.numZ:
            raise IndexError("plane %d out of range for a matrix with %d planes" % (p, hMatrix.numZ))
    if len(set(out)) != len(out):
        raise ValueError("planes lists a plane twice: %s" % (out,))
    return out


class Projector_gb300(Projector_base):
    """Forward / back projection and fused RL iterations on one GB300 GPU.

    Attributes kept from the reference: ``name``, ``storeVolumesOnGPU``
    (results stay as CUDA tensors), ``cacheFH`` (the GPU transfer matrices
    stay resident between calls; they always do here, ``ClearCache`` frees
    them).  GB300-specific: ``device``, ``fft_size`` (0 = automatic lenslet-
    grid transform size), ``fp64_precompute`` (None = double precision when
    the transform fits, else single).
    """

    def __init__(self, device=0):
        super().__init__()
        if torch is None:
            raise _flf.FlfError(-4, "PyTorch is required for device arrays")
        self.name = "GB300 CUDA"
        self.device = int(device)
        self.cacheFH = True
        self.fft_size = 0
        self.fp64_precompute = None
        self._ctx = None
        self._ctx_key = None
        self._shape_key = None
        # RichardsonLucy replays a CUDA graph of the whole loop; the graph runs on
        # staging tensors of its own (one entry per volume shape / iteration count)
        self.useGraphs = True
        self.maxGraphs = 3
        self._graphs = {}

    # -- native array helpers (torch CUDA tensors play cupy's role) ---------
    def _dev(self):
        return torch.device("cuda", self.device)

    def asnative(self, m):
        if isinstance(m, torch.Tensor):
            return m.to(device=self._dev(), dtype=torch.float32).contiguous()
        return torch.as_tensor(np.ascontiguousarray(m, dtype=np.float32), device=self._dev())

    def asnumpy(self, m, out=None):
        """A host copy of m; with ``out`` (a float32 numpy array of m's shape, e.g.
        a view of pinned memory) the copy lands there and ``out`` is returned."""
        if out is not None:
            if not isinstance(out, np.ndarray) or out.dtype != np.float32 or tuple(out.shape) != tuple(m.shape) \
                    or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float32 numpy array of shape %s" % (tuple(m.shape),))
            torch.from_numpy(out).copy_(m if isinstance(m, torch.Tensor) else torch.as_tensor(np.asarray(m)))
            return out
        if isinstance(m, torch.Tensor):
            return m.detach().to("cpu").numpy()
        return np.asarray(m)

    def nativeZeros(self, shape, dtype=float):
        return torch.zeros(tuple(shape), dtype=torch.float32, device=self._dev())

    def nativeDivide(self, a, b, out):
        return torch.div(a, b, out=out)

    def assertNative(self, m):
        assert isinstance(m, torch.Tensor) and m.is_cuda

    def _stream(self):
        return torch.cuda.current_stream(self._dev()).cuda_stream

    # -- context management -------------------------------------------------
    def context(self, hMatrix):
        """libflf context holding ``hMatrix``'s PSFs (uploaded on first use)."""
        key = hMatrix.identity() if hasattr(hMatrix, "identity") else (id(hMatrix),)
        if self._ctx is not None and self._ctx_key == key:
            return self._ctx
        self.ClearCache()
        torch.cuda.init()
        ctx = _flf.Context(hMatrix.Nnum, hMatrix.numZ, self.device)
        for cc in range(hMatrix.numZ):
            ctx.upload_psf(cc, _flf.FLF_DIR_FORWARD, np.asarray(hMatrix.Hcc(cc, False)))
            ctx.upload_psf(cc, _flf.FLF_DIR_BACKWARD, np.asarray(hMatrix.Hcc(cc, True)))
        self._ctx = ctx
        self._ctx_key = key
        self._shape_key = None
        return ctx

    def _auto_fp64(self, hMatrix, Y, X):
        """fp64_precompute=None: the transfer matrices are computed in double
        precision; the library falls back to single precision for transform sizes
        whose double-precision FFT does not fit shared memory (f > 112)."""
        return True

    def _prepare(self, ctx, Y, X, hMatrix=None):
        fp64 = self.fp64_precompute
        key = (Y, X, self.fft_size, fp64)
        if self._shape_key == key:
            return
        if fp64 is None:
            fp64 = self._auto_fp64(hMatrix, Y, X) if hMatrix is not None else False
        ctx.prepare(Y, X, self.fft_size, fp64)
        self._shape_key = key

    def autotune(self, hMatrix, T, Y, X, cache_path=None):
        """Pick the multiply-accumulate launch shape for T frames of Y x X images
        (flf_autotune) and keep it with this image shape's transfer matrices.

        With ``cache_path`` the choice is stored in, and on later calls read back
        from, a JSON file keyed by device, Nnum, plane count, PSF sizes, image
        shape, frames per launch and transform size, so tuning runs once per
        configuration."""
        ctx = self.context(hMatrix)
        self._prepare(ctx, Y, X, hMatrix)
        key = cache = None
        if cache_path:
            import json
            key = "|".join(str(v) for v in (
                torch.cuda.get_device_name(self._dev()), hMatrix.Nnum, hMatrix.numZ,
                tuple(tuple(hMatrix.PSFShape(cc)) for cc in range(hMatrix.numZ)), Y, X,
                min(int(T), 4), self.fft_size, self._shape_key[3]))
            try:
                with open(cache_path) as f:
                    cache = json.load(f)
            except (OSError, ValueError):
                cache = {}
            if key in cache:
                ctx.set_tuned(Y, X, cache[key])
                return dict(cache[key])
        tuned = ctx.autotune(T, Y, X, self._stream())
        if cache_path:
            import json
            cache[key] = tuned
            tmp = cache_path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(cache, f, indent=1)
            os.replace(tmp, cache_path)
        return tuned

    def ClearCache(self):
        self._drop_graphs()
        if self._ctx is not None:
            self._ctx.close()
        self._ctx = None
        self._ctx_key = None
        self._shape_key = None

    def geometry(self):
        return None if self._ctx is None else self._ctx.geometry()

    # -- projections --------------------------------------------------------
    def BackwardProjectACC(self, hMatrix, projection, planes, progress=None, logPrint=False,
                           numjobs=None, rlUpdateFunc=None):
        """``[numZ, T, Y, X]`` back projection of ``projection [T, Y, X]``.

        Planes not listed stay zero, as in the reference
        (projector.py:806-849).  With ``rlUpdateFunc`` the result is passed
        to it as ``rlUpdateFunc(volume, slice(None))`` and None is returned.
        """
        if len(projection.shape) != 3:
            raise ValueError("projection must be [T, Y, X], got shape %s" % (tuple(projection.shape),))
        plist = CheckPlanes(hMatrix, planes)
        ctx = self.context(hMatrix)
        img = self.asnative(projection)
        T, Y, X = img.shape
        self._prepare(ctx, Y, X, hMatrix)
        vol = torch.zeros((hMatrix.numZ, T, Y, X), dtype=torch.float32, device=self._dev())
        ctx.backward(img, vol, T, Y, X, None if len(plist) == hMatrix.numZ else plist,
                     stream=self._stream())
        if rlUpdateFunc is not None:
            rlUpdateFunc(vol, slice(None))
            return None
        if self.storeVolumesOnGPU:
            return vol
        return self.asnumpy(vol)

    def ForwardProjectACC(self, hMatrix, realspace, planes, progress=None, logPrint=False,
                          numjobs=None):
        """``[T, Y, X]`` forward projection of ``realspace [Z, T, Y, X]`` (sum over planes)."""
        if len(realspace.shape) != 4:
            raise ValueError("realspace must be [Z, T, Y, X], got shape %s" % (tuple(realspace.shape),))
        plist = CheckPlanes(hMatrix, planes)
        if realspace.shape[0] != hMatrix.numZ:
            raise ValueError("realspace has %d planes, the matrix %d" % (realspace.shape[0], hMatrix.numZ))
        ctx = self.context(hMatrix)
        vol = self.asnative(realspace)
        _, T, Y, X = vol.shape
        self._prepare(ctx, Y, X, hMatrix)
        img = torch.empty((T, Y, X), dtype=torch.float32, device=self._dev())
        ctx.forward(vol, img, T, Y, X, None if len(plist) == hMatrix.numZ else plist,
                    stream=self._stream())
        if self.storeVolumesOnGPU:
            return img
        return self.asnumpy(img)

    def RichardsonLucy(self, hMatrix, x, ref, iters, prevedel=True, norm=None):
        """Fused RL iterations on device tensors (in place on ``x [Z, T, Y, X]``).

        ``prevedel``: ``ref`` is Htf ``[Z, T, Y, X]``; otherwise ``ref`` is the
        camera image ``[T, Y, X]`` and ``norm`` an optional ``[Z, 1, Y, X]``
        normaliser (the back-projected trust mask).
        """
        ctx = self.context(hMatrix)
        Z, T, Y, X = x.shape
        self._prepare(ctx, Y, X, hMatrix)
        variant = _flf.FLF_RL_PREVEDEL if prevedel else _flf.FLF_RL_STANDARD
        if not self.useGraphs or iters <= 0:
            ctx.rl_iterate(x, ref, norm, variant, iters, T, Y, X, stream=self._stream())
            return x
        key = (Z, T, Y, X, int(iters), variant, norm is not None)
        for attempt in (0, 1):
            ent = self._graphs.pop(key, None)
            if ent is None:
                ent = self._make_rl_graph(ctx, key, ref, norm)
            self._graphs[key] = ent            # most recent last
            gx, gref, gnorm = ent["x"], ent["ref"], ent["norm"]
            if gx.data_ptr() != x.data_ptr():
                gx.copy_(x)
            if gref.data_ptr() != ref.data_ptr():
                gref.copy_(ref)
            if gnorm is not None and gnorm.data_ptr() != norm.data_ptr():
                gnorm.copy_(norm)
            try:
                ent["graph"].launch(self._stream())
                break
            except _flf.FlfError as e:
                # the context freed buffers the graph refers to (new PSFs, larger
                # images, clear_cache): capture it again once
                self._graphs.pop(key)["graph"].close()
                if e.code != -4 or attempt:
                    raise
        if gx.data_ptr() != x.data_ptr():
            x.copy_(gx)
        return x

    def _make_rl_graph(self, ctx, key, ref, norm):
        Z, T, Y, X, iters, variant, _ = key
        while len(self._graphs) >= max(1, self.maxGraphs):
            self._graphs.pop(next(iter(self._graphs)))["graph"].close()
        gx = torch.empty((Z, T, Y, X), dtype=torch.float32, device=self._dev())
        gref = torch.empty(tuple(ref.shape), dtype=torch.float32, device=self._dev())
        gnorm = None if norm is None else torch.empty(tuple(norm.shape), dtype=torch.float32, device=self._dev())
        torch.cuda.current_stream(self._dev()).synchronize()
        g = ctx.rl_graph(gx, gref, gnorm, variant, iters, T, Y, X)
        return {"graph": g, "x": gx, "ref": gref, "norm": gnorm}

    def _drop_graphs(self):
        for ent in self._graphs.values():
            ent["graph"].close()
        self._graphs = {}

    def RichardsonLucyGraph(self, hMatrix, x, ref, iters, prevedel=True, norm=None):
        """RichardsonLucy captured as a CUDA graph on these tensors;
        ``g.launch(stream)`` runs the ``iters`` iterations with one call.  Refill
        ``x`` / ``ref`` in place between launches: the graph keeps their addresses."""
        ctx = self.context(hMatrix)
        Z, T, Y, X = x.shape
        self._prepare(ctx, Y, X, hMatrix)
        variant = _flf.FLF_RL_PREVEDEL if prevedel else _flf.FLF_RL_STANDARD
        torch.cuda.current_stream(self._dev()).synchronize()
        return ctx.rl_graph(x, ref, norm, variant, iters, T, Y, X)


# Reference class names resolve to the GB300 backend (drop-in).
Projector_allC = Projector_gb300
Projector_gpuHelpers = Projector_gb300
