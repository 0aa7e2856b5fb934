"""Richardson-Lucy light-field deconvolution driver (interface of the reference's lfdeconv.py).

``BackwardProjectACC``, ``ForwardProjectACC`` and ``DeconvRL`` keep the
reference's signatures and semantics (lfdeconv.py:27-202).  With the GB300
projector ``DeconvRL`` runs every iteration on the GPU through one C-ABI call
(forward projection, back projection and the fused update).  Other projector
objects that implement the reference interface run the reference's loop.

Deliberate differences from the reference: no ``overall.txt`` side-effect
file; ``progress=None`` is accepted by ``DeconvRL`` (the reference crashes,
lfdeconv.py:185); plane subsets need not start at plane 0.
"""

import time

import numpy as np

import projector as proj

__all__ = ["BackwardProjectACC", "ForwardProjectACC", "DeconvRL"]


def _noProgressBar(work, desc=None, leave=True, **kwargs):
    return work


_default_projector = None


def _projector(p):
    global _default_projector
    if p is not None:
        return p
    if _default_projector is None:
        _default_projector = proj.Projector_gb300()
    return _default_projector


def BackwardProjectACC(hMatrix, projection, planes=None, progress=None, logPrint=True, numjobs=None,
                       projector=None, rlUpdateFunc=None):
    """Back projection ``Ht y``: ``[T, Y, X]`` -> ``[Z, T, Y, X]`` (lfdeconv.py:27-49)."""
    assert len(projection.shape) == 3
    projector = _projector(projector)
    if planes is None:
        planes = range(hMatrix.numZ)
    if progress is None:
        progress = _noProgressBar
    t1 = time.time()
    result = projector.BackwardProjectACC(hMatrix, projection, planes, progress, logPrint, numjobs,
                                          rlUpdateFunc)
    if logPrint:
        print("Backward project: elapsed wallclock time %f" % (time.time() - t1))
    return result


def ForwardProjectACC(hMatrix, realspace, planes=None, progress=None, logPrint=True, numjobs=None,
                      projector=None):
    """Forward projection ``H x``: ``[Z, T, Y, X]`` -> ``[T, Y, X]`` (lfdeconv.py:51-70)."""
    assert len(realspace.shape) == 4
    projector = _projector(projector)
    if planes is None:
        planes = range(hMatrix.numZ)
    if progress is None:
        progress = _noProgressBar
    t1 = time.time()
    result = projector.ForwardProjectACC(hMatrix, realspace, planes, progress, logPrint, numjobs)
    if logPrint:
        print("Forward project: elapsed wallclock time %f" % (time.time() - t1))
    return result


def DeconvRL(hMatrix, Htf, maxIter, Xguess, logPrint=True, numjobs=None, projector=None, im=None,
             progress=None, prevedel=True, trustMask=None, out=None):
    """Richardson-Lucy deconvolution (lfdeconv.py:72-202).

    Htf       the initial back projection of the camera image (or None, with ``im``)
    Xguess    the initial volume (None: a copy of Htf)
    prevedel  True: ``x <- x * Htf / Ht(H x)`` (the default of the reference);
              False: ``x <- x * Ht(im / H x)``, divided by ``Ht(trustMask)``
              when a trust mask is given.  NaN results are set to 0.
    out       optional float32 numpy array ``[Z, T, Y, X]`` (e.g. a view of pinned host
              memory) that receives the volume; it is then the return value.
    Returns the volume as a numpy array ``[Z, T, Y, X]``.
    """
    projector = _projector(projector)
    t1 = time.time()
    fused = hasattr(projector, "RichardsonLucy")
    if Htf is None:
        assert im is not None
        if prevedel or Xguess is None:
            saved = projector.storeVolumesOnGPU
            projector.storeVolumesOnGPU = fused   # keep Htf on the device for the fused path
            try:
                Htf = BackwardProjectACC(hMatrix, im, numjobs=numjobs, progress=None, logPrint=False,
                                         projector=projector)
            finally:
                projector.storeVolumesOnGPU = saved
    if trustMask is not None:
        if prevedel:
            raise ValueError("trustMask is only used by the standard RL update (prevedel=False)")
        tm = np.asarray(trustMask)
        for _im in np.asarray(im):
            if np.sum(_im[tm == 0]) != 0:
                raise ValueError("the image must be 0 where trustMask is 0")

    if fused:
        dev = projector.asnative
        src = Htf if Xguess is None else Xguess
        x = dev(src)
        if hasattr(src, "data_ptr") and x.data_ptr() == src.data_ptr():
            x = x.clone()   # the caller's array is not modified
        if prevedel:
            ref = dev(Htf)
            norm = None
        else:
            ref = dev(im)
            norm = None
            if trustMask is not None:
                saved = projector.storeVolumesOnGPU
                projector.storeVolumesOnGPU = True
                try:
                    norm = projector.BackwardProjectACC(hMatrix, dev(np.asarray(trustMask, np.float32)[np.newaxis]),
                                                        None, None, False, numjobs)
                finally:
                    projector.storeVolumesOnGPU = saved
        if maxIter > 0:
            projector.RichardsonLucy(hMatrix, x, ref, maxIter, prevedel=prevedel, norm=norm)
        result = projector.asnumpy(x, out=out)
    else:
        result = _deconv_rl_generic(hMatrix, Htf, maxIter, Xguess, numjobs, projector, im, prevedel,
                                    trustMask)
        if out is not None:
            out[...] = result
            result = out
    if logPrint:
        print("Deconvolution elapsed wallclock time %f" % (time.time() - t1))
    return result


def _deconv_rl_generic(hMatrix, Htf, maxIter, Xguess, numjobs, projector, im, prevedel, trustMask):
    """The reference loop (lfdeconv.py:185-196) for projectors without a fused RL path."""
    Xguess = (np.array(Htf, dtype=np.float32, copy=True) if Xguess is None
              else np.array(Xguess, dtype=np.float32, copy=True))
    trustBack = None
    if trustMask is not None:
        trustBack = BackwardProjectACC(hMatrix, np.asarray(trustMask, np.float32)[np.newaxis],
                                       numjobs=numjobs, progress=None, logPrint=False, projector=projector)

    def update_prevedel(back, cc):
        with np.errstate(divide="ignore", invalid="ignore"):
            Xguess[cc] *= np.asarray(Htf, np.float32)[cc] / np.asarray(back)
        Xguess[cc][np.isnan(Xguess[cc])] = 0

    def update_standard(back, cc):
        with np.errstate(divide="ignore", invalid="ignore"):
            Xguess[cc] *= np.asarray(back)
            if trustBack is not None:
                Xguess[cc] /= trustBack[cc]
        Xguess[cc][np.isnan(Xguess[cc])] = 0

    for _ in range(maxIter):
        HX = ForwardProjectACC(hMatrix, Xguess, numjobs=numjobs, progress=None, logPrint=False,
                               projector=projector)
        if prevedel:
            BackwardProjectACC(hMatrix, HX, numjobs=numjobs, progress=None, logPrint=False,
                               projector=projector, rlUpdateFunc=update_prevedel)
        else:
            with np.errstate(divide="ignore", invalid="ignore"):
                error = (np.asarray(im, np.float32) / HX).astype(np.float32)
            BackwardProjectACC(hMatrix, error, numjobs=numjobs, progress=None, logPrint=False,
                               projector=projector, rlUpdateFunc=update_standard)
    return Xguess
