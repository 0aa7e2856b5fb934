"""FP32 GPU projections and Richardson-Lucy against FP64-oracle fixtures at the
benchmark sizes (through the C ABI).

The fixtures (tests/golden/fp64_*.npz, made by tests/golden/make_fp64_fixtures.py
with the oracle's double-precision restatement of the reference's CPU
algorithm) hold the FP64 back projection Htf and RL result at 10^5 hashed
positions per case:

* 450 x 450 px, Nnum 15, 11 planes at -25..25 um: Htf and 8 Prevedel
  iterations from a uniform volume;
* 450 x 450 px, 21 planes at -50..50 um (PSF sizes 61..421): the same;
* 1005 x 1005 px, 41 planes at -100..100 um (PSF sizes up to 841): Htf and
  one iteration on 7 planes from the edge to the centre.

Tolerance (the precision statement for FP32 arithmetic): the largest sampled
error is at most 1e-4 of the FP64 array's largest value, and the relative L2
error over the samples at most 1e-4.
"""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import fp64_inputs as F  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 1e-4


def gpu_rl(case):
    """Htf and the RL result of a fixture case on the GPU, [Z, Y, X] numpy each."""
    import torch
    import _flf
    import psfmatrix
    import projector
    c = F.CASES[case]
    H, Ht = F.psf(case)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    p = projector.Projector_gb300()
    ctx = p.context(hm)
    Z, Y, X = len(H), c["Y"], c["X"]
    img = torch.as_tensor(F.image(case), device="cuda")
    htf = torch.empty((Z, 1, Y, X), device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    ctx.backward(img, htf, 1, Y, X, None, stream=s)
    x = torch.ones_like(htf)
    ctx.rl_iterate(x, htf, None, _flf.FLF_RL_PREVEDEL, c["iters"], 1, Y, X, stream=s)
    ctx.synchronize(s)
    out = htf[:, 0].cpu().numpy(), x[:, 0].cpu().numpy()
    ctx.close()
    del p
    torch.cuda.empty_cache()
    return out


@pytest.mark.parametrize("case", list(F.CASES))
def test_fp32_gpu_matches_fp64_oracle(built_lib, case):
    htf, x = gpu_rl(case)
    e = F.compare(case, htf, x)
    print(case, e)
    assert e["htf_max_rel"] < TOL and e["htf_rel_l2"] < TOL, e
    assert e["x_max_rel"] < TOL and e["x_rel_l2"] < TOL, e
