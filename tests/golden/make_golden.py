"""Generate tests/golden/reference_vectors.npz by running the reference itself.

Runs in a container that holds the reference sources (jmtayloruk/fast-light-field),
whose folder is the one argument; the GPU test machines never read them.  It imports the
reference's own Python modules and uses its pure-python projector
``Projector_python`` (projector.py:1017) and RL driver ``lfdeconv.DeconvRL``
(lfdeconv.py:72) - the code the reference's self-test trusts as its oracle
(projector.py:1145-1215).  Modules the Python path does not call (the C++
extension ``py_light_field``, h5py, tifffile, the Cython PSF integrands) are
replaced by empty stand-ins so that the imports succeed.

Usage:  python tests/golden/make_golden.py /path/to/reference
"""

import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from golden_inputs import CASES, case_inputs  # noqa: E402


def import_reference(ref_dir):
    for name in ("h5py", "tifffile", "py_light_field", "light_field_integrands"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.path.insert(0, ref_dir)
    import projector
    import lfdeconv
    import psfmatrix
    return projector, lfdeconv, psfmatrix


def make_hmatrix(psfmatrix, H, Ht, tmp):
    shapes = []
    for z, (h, ht) in enumerate(zip(H, Ht)):
        for nm, arr in (("H", h), ("Ht", ht)):
            m = np.memmap(os.path.join(tmp, "%s%02d.array" % (nm, z)), dtype="float32", mode="w+",
                          shape=arr.shape)
            m[...] = arr
            m.flush()
            del m
        shapes.append(h.shape)
    return psfmatrix.HMatrix(os.path.join(tmp, "H{z:02d}.array"), os.path.join(tmp, "Ht{z:02d}.array"),
                             shapes)


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    ref_dir = sys.argv[1]
    projector, lfdeconv, psfmatrix = import_reference(ref_dir)
    out = {}
    noprog = lambda w, desc=None, leave=True, **k: w  # noqa: E731
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)   # the reference writes overall.txt into the working directory
        try:
            for name in CASES:
                c = case_inputs(name)
                hm = make_hmatrix(psfmatrix, c["H"], c["Ht"], tmp + "/" if False else tmp)
                p = projector.Projector_python()
                Z = len(c["hs"])
                if c["kind"] == "project":
                    bk = p.BackwardProjectACC(hm, c["img"], list(range(Z)), noprog, False, 1)
                    fw = p.ForwardProjectACC(hm, c["vol"], list(range(Z)), noprog, False, 1)
                    out[name + "/backward"] = np.asarray(bk, np.float32)
                    out[name + "/forward"] = np.asarray(fw, np.float32)
                else:
                    if c["prevedel"]:
                        res = lfdeconv.DeconvRL(hm, None, c["iters"], None, logPrint=False, numjobs=1,
                                                projector=p, im=c["img"], progress=noprog,
                                                prevedel=True)
                    else:
                        x0 = np.full((Z,) + c["img"].shape, 1.0, np.float32)
                        res = lfdeconv.DeconvRL(hm, None, c["iters"], x0, logPrint=False, numjobs=1,
                                                projector=p, im=c["img"], progress=noprog,
                                                prevedel=False)
                    out[name + "/rl"] = np.asarray(res, np.float32)
                print(name, {k: v.shape for k, v in out.items() if k.startswith(name)})
        finally:
            os.chdir(cwd)
    dst = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
