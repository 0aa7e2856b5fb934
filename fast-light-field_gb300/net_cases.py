"""Timing cases for the warm-start network kernels (CUDA events, no profiler).

    python net_cases.py conv16 [Z Y X] [--kernel tcgen05-all|tcgen05|tcgen05-noswizzle|mma.sync] [--reps N]
    python net_cases.py unet   [Z Y X] [--kernel ...] [--reps N]

``conv16`` runs the 16 -> 16 channel 3x3x3 convolution (flf_conv3d, or
flf_conv3d_tc for the unswizzled tcgen05 variant) on a random BF16 volume
[1][Z][Y][X][16]; ``unet`` runs the U-Net forward with its head.  Both print
the mean time per call after three warm-up calls; the inputs are larger than
L2 at the default 24 x 456 x 456 size.  These are the cases the kernel
profiles are taken on.
"""

import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def _time(torch, fn, reps):
    for _ in range(3):
        fn()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps * 1e3


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("case", choices=["conv16", "unet"])
    ap.add_argument("shape", nargs="*", type=int, default=[24, 456, 456], help="Z Y X")
    ap.add_argument("--kernel", default="tcgen05-all",
                    choices=["tcgen05", "tcgen05-all", "tcgen05-noswizzle", "mma.sync"],
                    help="tcgen05: the 16->16 layers on tcgen05; tcgen05-all (the default): the 32-channel "
                         "layers too")
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args(argv)
    if len(args.shape) != 3:
        ap.error("shape is Z Y X")
    import torch
    import _flf
    _flf.load_library()
    _flf.conv16_tcgen05({"mma.sync": 0, "tcgen05-all": 2}.get(args.kernel, 1))
    Z, Y, X = args.shape
    g = torch.Generator(device="cuda").manual_seed(0)
    if args.case == "conv16":
        x = torch.randn((1, Z, Y, X, 16), generator=g, device="cuda").bfloat16()
        w = (torch.randn((27, 16, 16), generator=g, device="cuda") / 20).bfloat16()
        b = torch.randn(16, generator=g, device="cuda")
        y = torch.empty_like(x)
        if args.kernel == "tcgen05-noswizzle":
            fn = lambda: _flf.conv3d_tc(x, w, b, y, relu=True, rows=0)
        else:
            fn = lambda: _flf.conv3d(x, w, b, y, relu=True)
        flop = 2.0 * Z * Y * X * 27 * 16 * 16
    else:
        import warmstart
        net = warmstart.UNet3D(seed=1)
        x = torch.zeros((1, Z, Y, X, warmstart.CIN), device="cuda").bfloat16()
        x[..., :4] = torch.rand((1, Z, Y, X, 4), generator=g, device="cuda").bfloat16()
        fn = lambda: net.forward(x)
        flop = None
    us = _time(torch, fn, args.reps)
    torch.cuda.synchronize()
    _flf.net_status()
    line = "%s %s %dx%dx%d: %.1f us per call" % (args.case, args.kernel, Z, Y, X, us)
    if flop:
        line += " (%.0f TFLOP/s)" % (flop / us / 1e6)
    print(line, flush=True)


if __name__ == "__main__":
    main()
