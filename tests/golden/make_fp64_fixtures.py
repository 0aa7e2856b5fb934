"""Generate tests/golden/fp64_<case>.npz: FP64-oracle outputs at the benchmark sizes.

For every case of fp64_inputs.py this runs the oracle's restatement of the
reference's CPU projection (``oracle.lf_oracle.project_plane_ref_cpu``, which
the oracle tests pin to the reference's own outputs and, in double precision,
to the per-offset FP64 definition) in float64, plane by plane over a process
pool, and the Prevedel RL update ``x <- x * Htf / Ht(H x)`` with NaN -> 0
(lfdeconv.py:112-149) from a uniform start volume.  Stored per case, for the
checked planes:

* ``htf`` / ``x``: the FP64 back projection and RL result at the case's
  SAMPLES hashed positions (float32 storage of the float64 values);
* ``htf_max`` / ``htf_l2`` / ``x_max`` / ``x_l2``: the maximum magnitude and L2
  norm of the full float64 arrays (the error normalisers).

Usage:  python tests/golden/make_fp64_fixtures.py [case ...] [--workers N]
(runs for minutes on a few host cores; the full-field case dominates).
"""

import argparse
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (HERE, ROOT, os.path.join(ROOT, "fast-light-field_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import fp64_inputs as F  # noqa: E402


def _plane(task):
    """FP64 projection of src through plane z of the case's H (forward) or Ht (backward)."""
    case, z, backward, src = task
    from oracle import lf_oracle as O
    H, Ht = F.psf(case, only=[z])
    P = (Ht if backward else H)[z].astype(np.float64)
    return O.project_plane_ref_cpu(src, P, F.CASES[case]["Nnum"], workers=1, dtype=np.float64)


def run_case(case, pool):
    c = F.CASES[case]
    Z = len(F.z_planes(case))
    planes = F.checked_planes(case)
    img = F.image(case).astype(np.float64)
    t0 = time.time()
    # Htf on the planes the RL update touches (all of them for the full runs)
    rl_planes = list(range(Z)) if c["planes"] is None else planes
    htf = dict(zip(rl_planes, pool.map(_plane, [(case, z, True, img) for z in rl_planes])))
    x = {z: np.ones_like(htf[z]) for z in rl_planes}
    for it in range(c["iters"]):
        if c["planes"] is None:
            src = x
        else:
            # only the checked planes are kept; with a uniform start every plane is 1
            assert c["iters"] == 1
            src = {z: np.ones_like(img) for z in range(Z)}
        hx = sum(pool.map(_plane, [(case, z, False, src[z]) for z in range(Z)]))
        bp = dict(zip(rl_planes, pool.map(_plane, [(case, z, True, hx) for z in rl_planes])))
        with np.errstate(divide="ignore", invalid="ignore"):
            for z in rl_planes:
                x[z] = x[z] * (htf[z] / bp[z])
                x[z][np.isnan(x[z])] = 0
        print("  %s: iteration %d done, %.0f s" % (case, it + 1, time.time() - t0), flush=True)
    H_ = np.stack([htf[z][0] for z in planes])
    X_ = np.stack([x[z][0] for z in planes])
    pos = F.sample_positions(case, len(planes))
    return {"htf": H_.ravel()[pos].astype(np.float32), "x": X_.ravel()[pos].astype(np.float32),
            "htf_max": np.float64(np.abs(H_).max()), "htf_l2": np.float64(np.linalg.norm(H_)),
            "x_max": np.float64(np.abs(X_).max()), "x_l2": np.float64(np.linalg.norm(X_)),
            "planes": np.array(planes, np.int32), "iters": np.int32(c["iters"])}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("cases", nargs="*", default=list(F.CASES))
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    with mp.get_context("spawn").Pool(args.workers) as pool:
        for case in args.cases:
            t0 = time.time()
            out = run_case(case, pool)
            dst = os.path.join(HERE, "fp64_%s.npz" % case)
            np.savez_compressed(dst, **out)
            print("wrote %s (%d bytes) in %.0f s" % (dst, os.path.getsize(dst), time.time() - t0), flush=True)


if __name__ == "__main__":
    main()
