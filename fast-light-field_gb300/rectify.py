"""Rectification of raw light-field images on the GB300 (the reference's rectify.py).

RectifyImage resamples a raw camera image so that each lenslet spans exactly
Nnum pixels, then optionally crops whole lenslets from the borders, as the
reference's port of the Prevedel et al. MATLAB code does (rectify.py:8-81).
The query grid is built on the host exactly as the reference builds it (its
np.arange steps of dx / Nnum from the centre lenslet's origin, MATLAB
one-based), and the bilinear resampling runs on the device in double
precision (flf_resample_bilinear).  RectifyImageFiles and the command line
mirror rectify.py:83-140.
"""

import argparse
import glob
import os
import sys

import numpy as np

import tiffio


def rectify_grid(shape, xCenter_m, yCenter_m, dx, Nnum):
    """Zero-based query coordinates (y, x) of the resampled image, before cropping,
    and the row / column counts kept by the reference's first crop."""
    if Nnum - 2 * (Nnum // 2) != 1:
        raise ValueError("Nnum must be an odd integer")
    M = Nnum
    dy = dx
    Mdiff = M // 2
    H, W = shape[-2], shape[-1]
    # the reference steps np.arange up to and including the end points (its +-1e-10)
    Xres = np.append(np.arange(xCenter_m + 1, 1 - 1e-10, -dx / M)[::-1],
                     np.arange((xCenter_m + 1) + dx / M, W + 1e-10, dx / M))
    Yres = np.append(np.arange(yCenter_m + 1, 1 - 1e-10, -dy / M)[::-1],
                     np.arange((yCenter_m + 1) + dy / M, H + 1e-10, dy / M))
    xc = np.where(Xres == (xCenter_m + 1))[0][0] - Mdiff + 1
    xinit = xc - M * (xc // M) + M
    yc = np.where(Yres == (yCenter_m + 1))[0][0] - Mdiff + 1
    yinit = yc - M * (yc // M) + M
    xq = Xres[xinit - 1:] - 1
    yq = Yres[yinit - 1:] - 1
    ny = M * ((len(yq) - yinit) // M)
    nx = M * ((len(xq) - xinit) // M)
    return yq, xq, ny, nx


def RectifyImage(IMG_BW, xCenter_m, yCenter_m, dx, Nnum, Crop, XcutLeft, XcutRight, YcutUp, YcutDown,
                 device=0):
    """Rectified image as float64 (rectify.py:8-81): bilinear resample, crop to whole
    lenslets, then (with Crop) drop XcutLeft / XcutRight / YcutUp / YcutDown lenslets."""
    import torch
    import _flf
    img = np.asarray(IMG_BW)
    if img.ndim != 2:
        raise ValueError("RectifyImage takes a single 2-D image")
    M = Nnum
    yq, xq, ny, nx = rectify_grid(img.shape, xCenter_m, yCenter_m, dx, Nnum)
    if ny <= 0 or nx <= 0:
        return np.zeros((max(ny, 0), max(nx, 0)))
    dev = torch.device("cuda", device)
    yq_d = torch.as_tensor(np.ascontiguousarray(yq[:ny]), dtype=torch.float64, device=dev)
    xq_d = torch.as_tensor(np.ascontiguousarray(xq[:nx]), dtype=torch.float64, device=dev)
    img_d = torch.as_tensor(img.astype(np.float32), device=dev)
    out = torch.empty((ny, nx), dtype=torch.float64, device=dev)
    _flf.resample_bilinear(img_d, yq_d, xq_d, out, torch.cuda.current_stream(dev).cuda_stream)
    res = out.cpu().numpy()
    if Crop:
        XsizeML, YsizeML = res.shape[1] // M, res.shape[0] // M
        if (XcutLeft + XcutRight) >= XsizeML:
            raise ValueError("X-cut range is larger than the x-size of image")
        if (YcutUp + YcutDown) >= YsizeML:
            raise ValueError("Y-cut range is larger than the y-size of image")
        res = res[YcutUp * M:(YsizeML - YcutDown) * M, XcutLeft * M:(XsizeML - XcutRight) * M]
    return res


def RectifyImageFiles(files, outputDir, **kwargs):
    """Rectify the files (glob patterns allowed) into outputDir/<name>_N<Nnum>.tif, rounded
    back to the input's sample type (rectify.py:83-106)."""
    written = []
    for g in files:
        paths = sorted(glob.glob(g))
        if not paths:
            print("WARNING: no file found matching %s" % g)
        for p in paths:
            image = tiffio.imread(p)
            if image.ndim != 2:
                print("  WARNING: SKIPPING FILE %s because it is not a single 2D image" % p)
                continue
            rect = RectifyImage(image, **kwargs)
            fn, ext = os.path.splitext(os.path.basename(p))
            os.makedirs(outputDir, exist_ok=True)
            dest = os.path.join(outputDir, "%s_N%d%s" % (fn, kwargs["Nnum"], ext))
            tiffio.imwrite(dest, np.around(rect).astype(image.dtype))
            written.append(dest)
    return written


def RectifyWithArgList(raw_args):
    """Command line of the reference (rectify.py:108-140)."""
    parser = argparse.ArgumentParser(description="Rectify raw light field images ready for deconvolution",
                                     formatter_class=argparse.ArgumentDefaultsHelpFormatter)
    parser.add_argument("files", nargs="+", help="List of file(s) to rectify (which may contain wildcards)")
    parser.add_argument("-x", "--x-center", dest="xCenter_m", type=float, required=True,
                        help="X origin of center lenslet array (matlab indexing of raw image pixels)")
    parser.add_argument("-y", "--y-center", dest="yCenter_m", type=float, required=True,
                        help="Y origin of center lenslet array (matlab indexing of raw image pixels)")
    parser.add_argument("-d", "--dx", dest="dx", type=float, required=True,
                        help="Period of lenslet array in raw image pixels")
    parser.add_argument("-n", "--Nnum", dest="Nnum", type=int, required=True,
                        help="Resampled period of lenslet array (odd integer)")
    parser.add_argument("-c", "--crop", dest="Crop", action="store_true", help="Crop rectified image")
    parser.add_argument("-l", "--crop-left", dest="XcutLeft", type=int, default=0,
                        help="Number of lenslets to crop from the left boundary of the rectified image")
    parser.add_argument("-r", "--crop-right", dest="XcutRight", type=int, default=0,
                        help="Number of lenslets to crop from the right boundary of the rectified image")
    parser.add_argument("-t", "--crop-top", dest="YcutUp", type=int, default=0,
                        help="Number of lenslets to crop from the top boundary of the rectified image")
    parser.add_argument("-b", "--crop-bottom", dest="YcutDown", type=int, default=0,
                        help="Number of lenslets to crop from the bottom boundary of the rectified image")
    parser.add_argument("-o", "--output-dir", dest="outputDir", default="Data/02_Rectified",
                        help="Directory in which to save rectified images")
    args = vars(parser.parse_args(raw_args))
    files, outputDir = args.pop("files"), args.pop("outputDir")
    return RectifyImageFiles(files, outputDir, **args)


if __name__ == "__main__":
    RectifyWithArgList(sys.argv[1:])
