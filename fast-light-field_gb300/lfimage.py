"""Light-field image loading with the reference's interface (lfimage.py:4-20)."""

import numpy as np

import tiffio


def LoadLightFieldTiff(imagePath, bigger=(1, 1)):
    """Load a rectified light-field camera image as float32.

    As in the reference, the image is not transposed (the PSF symmetries make
    that unnecessary), and ``bigger`` tiles it up to a larger size for
    performance tests.
    """
    image = tiffio.imread(imagePath)
    if image.ndim != 2:
        raise ValueError("%s: expected a single 2-D image, got shape %s" % (imagePath, image.shape))
    return np.tile(image.astype("float32"), bigger)
