"""Generate tests/golden/rectify_vectors.npz by running the reference's RectifyImage.

Runs in a container that holds the reference sources, whose folder is the one
argument (the GPU machines never read them); tifffile, which RectifyImage does not call, is replaced
by an empty stand-in.  Inputs are regenerated from the seeds in rectify_inputs.py;
only the outputs are stored.

Usage:  python tests/golden/make_golden_rectify.py /path/to/reference
"""

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from rectify_inputs import RECTIFY_CASES, rectify_input  # noqa: E402


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    ref_dir = sys.argv[1]
    sys.modules.setdefault("tifffile", types.ModuleType("tifffile"))
    sys.path.insert(0, ref_dir)
    import rectify
    out = {}
    for name in RECTIFY_CASES:
        img, kw = rectify_input(name)
        out[name] = np.asarray(rectify.RectifyImage(img, **kw), np.float64)
        print(name, img.shape, "->", out[name].shape)
    np.savez_compressed(os.path.join(HERE, "rectify_vectors.npz"), **out)


if __name__ == "__main__":
    main()
