"""Generate tests/golden/psf_vectors.npz by running the reference's GeneratePSF.

Runs in a container that holds the reference sources, whose folder is the one
argument (the GPU machines never read them).  The reference's Cython integrand module
(light-field-integrands: one .pyx plus bessel.c) is compiled into a temporary
folder; h5py, which is not installed, is replaced by a stand-in whose File
object records what GeneratePSF saves.  For every case of psf_inputs.py the
fixture keeps H and Ht (as saved: transposed, [Z, b, a, y, x]), CAindex and
Hmax.

Usage:  python tests/golden/make_golden_psf.py /path/to/reference
"""

import os
import shutil
import subprocess
import sys
import tempfile
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from psf_inputs import PSF_CASES  # noqa: E402

SAVED = {}


class _File(dict):
    """h5py.File stand-in: keeps the datasets assigned to it."""

    def __init__(self, path, mode="r"):
        super().__init__()
        self.path = path

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        SAVED.clear()
        SAVED.update({k: np.array(v) for k, v in self.items()})
        return False


def build_integrands(ref_dir, work):
    src = os.path.join(ref_dir, "light-field-integrands")
    for f in ("light_field_integrands.pyx", "light_field_integrands.pxd", "bessel.c", "bessel.h"):
        shutil.copy(os.path.join(src, f), work)
    with open(os.path.join(work, "build.py"), "w") as f:
        f.write("from setuptools import setup, Extension\n"
                "from Cython.Build import cythonize\n"
                "setup(name='light_field_integrands', script_args=['build_ext', '--inplace'],\n"
                "      ext_modules=cythonize(Extension('light_field_integrands',\n"
                "          sources=['light_field_integrands.pyx', 'bessel.c']), quiet=True))\n")
    subprocess.run([sys.executable, "build.py"], cwd=work, check=True, stdout=subprocess.DEVNULL)
    sys.path.insert(0, work)


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    ref_dir = sys.argv[1]
    work = tempfile.mkdtemp(prefix="flf_psf_golden_")
    build_integrands(ref_dir, work)
    h5 = types.ModuleType("h5py")
    h5.File = _File
    sys.modules["h5py"] = h5
    sys.path.insert(0, ref_dir)
    import generate_psf
    out = {}
    for name, kw in PSF_CASES.items():
        t0 = time.time()
        generate_psf.GeneratePSF(matrixSaveDir=os.path.join(work, name), **kw)
        for key in ("H", "Ht", "CAindex", "Hmax"):
            out["%s/%s" % (name, key)] = SAVED[key]
        print(name, "H", SAVED["H"].shape, "CAindex", SAVED["CAindex"].tolist(), "%.1f s" % (time.time() - t0))
    np.savez_compressed(os.path.join(HERE, "psf_vectors.npz"), **out)
    shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
