"""Deconvolve a time series of rectified light-field images on the GB300.

Command-line and function interface of the reference's
deconvolve_time_series.py:9-85: each camera image (a 2-D TIFF) is back
projected, Richardson-Lucy runs from that back projection (x0 = Htf) for
``--iters`` iterations, and the volume is written as
``<dest>/<name>_deconvolved.tif`` ([Z, Y, X] float32 pages).

Differences from the reference, all in the caller's favour:

* frames of different sizes may be mixed: they are grouped by image shape
  and each group runs in batches of ``--batch-size`` frames (the reference
  exits when a batch mixes sizes);
* back projection, RL and the update stay on the device for the whole batch
  (as with the reference's ``--volumes-on-gpu``); only the camera images go
  up and the finished volumes come down;
* ``--mode`` and ``--cacheFH`` are accepted for compatibility: every mode runs
  the GB300 path, and the transfer matrices always stay resident;
* ``--warm-start NET`` (an addition) starts RL from the learned warm start of
  warmstart.py (weights trained for one image size; frames of other sizes
  start from Htf as usual).
"""

import argparse
import os
import sys
import time

import numpy as np

import _flf
import lfdeconv
import lfimage
import psfmatrix
import projector as proj
import tiffio


def ProcessBatch(projector, hMatrix, timepoints, destDir, maxIter, warm=None):
    """Deconvolve the images `timepoints` (one shape) together and save the volumes
    (deconvolve_time_series.py:9-37).  With `warm` (a warmstart.WarmStart for this
    image size), RL starts from the network's volume instead of Htf."""
    os.makedirs(destDir, exist_ok=True)
    images = [lfimage.LoadLightFieldTiff(t) for t in timepoints]
    if any(im.shape != images[0].shape for im in images):
        raise ValueError("not all images of a batch have the same dimensions")
    images = np.array(images)
    saved = projector.storeVolumesOnGPU
    projector.storeVolumesOnGPU = True      # Htf stays on the device as the RL start and reference
    try:
        Htf = lfdeconv.BackwardProjectACC(hMatrix, images, progress=None, logPrint=False, projector=projector)
        x0 = warm.initial_volume(Htf) if warm is not None else Htf
        result = lfdeconv.DeconvRL(hMatrix, Htf, maxIter=maxIter, Xguess=x0, logPrint=False,
                                   projector=projector)
    finally:
        projector.storeVolumesOnGPU = saved
    if warm is not None:
        _flf.net_status()   # the result is on the host: raise if a network kernel's bounded wait gave up
    paths = []
    for i, t in enumerate(timepoints):
        dest = os.path.join(destDir, "%s_deconvolved.tif" % os.path.splitext(os.path.basename(t))[0])
        tiffio.imwrite(dest, np.ascontiguousarray(result[:, i]))
        paths.append(dest)
    return paths


def GroupByShape(timepoints):
    """Timepoints grouped by image shape, in order of first appearance."""
    groups = {}
    for t in timepoints:
        groups.setdefault(tuple(tiffio.imshape(t)), []).append(t)
    return list(groups.items())


def main(argv, maxIter=8, numParallel=32):
    parser = argparse.ArgumentParser(
        description="Deconvolves a time series of (pre-rectified) light field microscopy images.",
        formatter_class=argparse.ArgumentDefaultsHelpFormatter)
    parser.add_argument("-m", "--mode", dest="platform", metavar="PLATFORM", choices=["cpu", "gpu", "gpubig"],
                        default="gpu", help="accepted for compatibility; every mode runs on the GB300")
    parser.add_argument("-b", "--batch-size", dest="numParallel", metavar="BATCH-SIZE", type=int, default=numParallel,
                        help="number of simultaneous deconvolutions")
    parser.add_argument("-i", "--iters", dest="numIter", metavar="RL-ITERS", type=int, default=maxIter,
                        help="number of iterations of Richardson-Lucy to run")
    parser.add_argument("-v", "--volumes-on-gpu", dest="storeVolumesOnGPU", action="store_true", default=False,
                        help="accepted for compatibility; volumes always stay on the GPU during a batch")
    parser.add_argument("-c", "--cacheFH", dest="cacheFH", action="store_true", default=False,
                        help="accepted for compatibility; the transfer matrices always stay resident")
    parser.add_argument("-d", "--dest", dest="destDir", metavar="DEST-DIR", default=".",
                        help="directory in which deconvolved output will be saved")
    parser.add_argument("-p", "--psf", dest="psfFile", metavar="PSF-FILE", required=True, default=argparse.SUPPRESS,
                        help="path to the PSF .mat file (its memmap folder is used when present)")
    parser.add_argument("-t", "--timepoints", dest="timepoints", metavar="IMG", required=True,
                        default=argparse.SUPPRESS, nargs="+", help="files to deconvolve")
    parser.add_argument("-w", "--warm-start", dest="warmStart", metavar="NET", default=None,
                        help="warm-start network (warmstart.py) for frames of the size it was trained for")
    args = parser.parse_args(argv)
    if args.numParallel < 1:
        raise SystemExit("ERROR: Invalid batch size: %d" % args.numParallel)
    if args.numIter < 1:
        raise SystemExit("ERROR: Invalid number of RL iterations: %d" % args.numIter)

    projector = proj.Projector_gb300()
    projector.cacheFH = args.cacheFH
    hMatrix = psfmatrix.LoadMatrix(args.psfFile, createPSF=True)

    groups = GroupByShape(args.timepoints)
    warm_shape = None
    if args.warmStart:
        import warmstart
        warm_shape = warmstart.WarmStart.trained_shape(args.warmStart)
    total = len(args.timepoints)
    done = 0
    t0 = time.time()
    written = []
    for shape, files in groups:
        warm = None
        if warm_shape is not None and tuple(shape[-2:]) == tuple(warm_shape[1:]):
            warm = warmstart.WarmStart(projector, hMatrix, shape[-2], shape[-1]).load(args.warmStart)
        for b in range(0, len(files), args.numParallel):
            batch = files[b:b + args.numParallel]
            written += ProcessBatch(projector, hMatrix, batch, args.destDir, args.numIter, warm)
            done += len(batch)
            print("Deconvolved %d of %d files (%d x %d px)" % (done, total, shape[0], shape[1]), flush=True)
    print("Deconvolved %d files in %.1f s" % (total, time.time() - t0), flush=True)
    return written


if __name__ == "__main__":
    main(sys.argv[1:])
