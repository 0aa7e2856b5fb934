"""Seeded inputs of the rectification golden cases (shared by the generator and the tests)."""

import numpy as np

RECTIFY_CASES = {
    # name: (image shape, dtype, seed, kwargs of RectifyImage)
    "n5_u8": ((96, 128), "uint8", 1, dict(xCenter_m=64.3, yCenter_m=48.7, dx=7.3, Nnum=5, Crop=False,
                                          XcutLeft=0, XcutRight=0, YcutUp=0, YcutDown=0)),
    "n9_u16_crop": ((120, 110), "uint16", 2, dict(xCenter_m=55.0, yCenter_m=61.0, dx=9.0, Nnum=9, Crop=True,
                                                  XcutLeft=1, XcutRight=2, YcutUp=1, YcutDown=1)),
    "n15_u8_crop": ((137, 151), "uint8", 3, dict(xCenter_m=70.5, yCenter_m=66.25, dx=15.2, Nnum=15, Crop=True,
                                                 XcutLeft=0, XcutRight=1, YcutUp=1, YcutDown=0)),
}


def rectify_input(name):
    shape, dtype, seed, kw = RECTIFY_CASES[name]
    rng = np.random.default_rng(seed)
    hi = 255 if dtype == "uint8" else 60000
    # lenslet-like structure plus noise, so the interpolation sees gradients
    yy, xx = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    base = 0.5 + 0.5 * np.cos(2 * np.pi * xx / kw["dx"]) * np.cos(2 * np.pi * yy / kw["dx"])
    img = np.clip(base * hi * 0.8 + rng.random(shape) * hi * 0.2, 0, hi)
    return np.round(img).astype(dtype), dict(kw)
