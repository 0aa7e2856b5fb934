"""GPU parity tests: the CUDA path (through the C ABI) against the reference's
golden vectors and the CPU oracle.

Tolerances: projections are FP32 arithmetic; they must agree with the FP64
oracle / the reference's FP32 output to 2e-5 of the output's maximum
(the reference's own self-test accepts 1e-4 absolute on O(1) outputs,
projector.py:1212).  Richardson-Lucy results must agree to 1e-4 relative
(max abs error / max abs value).
"""

import numpy as np
import pytest

from golden_inputs import CASES, case_inputs
from oracle import lf_oracle as O

pytestmark = pytest.mark.gpu

PROJ_TOL = 2e-5
RL_TOL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


@pytest.fixture(scope="module")
def mods(built_lib):
    import lfdeconv
    import projector
    import psfmatrix
    import _flf
    _flf.load_library()
    return projector, lfdeconv, psfmatrix


def gold():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz"))


@pytest.mark.parametrize("name", [n for n in CASES if CASES[n]["kind"] == "project"])
@pytest.mark.parametrize("fp64", [True, False])
def test_projection_matches_reference_vectors(mods, name, fp64):
    projector, lfdeconv, psfmatrix = mods
    c = case_inputs(name)
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    p = projector.Projector_gb300()
    p.fp64_precompute = fp64
    bk = lfdeconv.BackwardProjectACC(hm, c["img"], projector=p, logPrint=False)
    fw = lfdeconv.ForwardProjectACC(hm, c["vol"], projector=p, logPrint=False)
    g = gold()
    assert bk.shape == g[name + "/backward"].shape and bk.dtype == np.float32
    assert fw.shape == g[name + "/forward"].shape and fw.dtype == np.float32
    assert rel(bk, g[name + "/backward"]) < PROJ_TOL
    assert rel(fw, g[name + "/forward"]) < PROJ_TOL


@pytest.mark.parametrize("name", [n for n in CASES if CASES[n]["kind"] == "rl"])
def test_rl_matches_reference_vectors(mods, name):
    projector, lfdeconv, psfmatrix = mods
    c = case_inputs(name)
    Z = len(c["hs"])
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    p = projector.Projector_gb300()
    x0 = None if c["prevedel"] else np.ones((Z,) + c["img"].shape, np.float32)
    r = lfdeconv.DeconvRL(hm, None, c["iters"], x0, logPrint=False, projector=p, im=c["img"],
                          prevedel=c["prevedel"])
    assert rel(r, gold()[name + "/rl"]) < RL_TOL


@pytest.mark.parametrize("N,hs,T,Y,X", [
    (3, [7, 9, 5], 1, 18, 21),
    (5, [21, 11, 31], 3, 40, 35),     # ragged image (not a multiple of Nnum)
    (7, [43, 15], 6, 49, 56),         # T > 4 exercises frame chunking
    (15, [61, 91], 2, 150, 120),
    (19, [77], 1, 95, 114),
    (19, [77, 39], 5, 95, 114),       # Nnum 19 runs 2 frames per pass (shared memory): 2 + 2 + 1
])
def test_projection_matches_fp64_oracle(mods, N, hs, T, Y, X):
    projector, lfdeconv, psfmatrix = mods
    import synthetic
    H, Ht = synthetic.random_psf(N, hs, seed=N * 7 + T)
    rng = np.random.default_rng(N + Y)
    img = rng.random((T, Y, X)).astype(np.float32)
    vol = rng.random((len(hs), T, Y, X)).astype(np.float32)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    p = projector.Projector_gb300()
    bk = p.BackwardProjectACC(hm, img, None)
    fw = p.ForwardProjectACC(hm, vol, None)
    meth = "direct" if N <= 7 else "special"
    bo = O.backward_project(Ht, img, N, method=meth, dtype=np.float64)
    fo = O.forward_project(H, vol, N, method=meth, dtype=np.float64)
    assert rel(bk, bo) < PROJ_TOL
    assert rel(fw, fo) < PROJ_TOL


def test_plane_subsets(mods):
    projector, lfdeconv, psfmatrix = mods
    import synthetic
    N = 5
    H, Ht = synthetic.random_psf(N, [21, 11, 31, 15], seed=3)
    rng = np.random.default_rng(5)
    img = rng.random((2, 30, 35)).astype(np.float32)
    vol = rng.random((4, 2, 30, 35)).astype(np.float32)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    p = projector.Projector_gb300()
    full_bk = O.backward_project(Ht, img, N, method="direct", dtype=np.float64)
    for planes in ([2], [3, 1], [0, 2, 3]):
        bk = p.BackwardProjectACC(hm, img, planes)
        for z in range(4):
            if z in planes:
                assert rel(bk[z], full_bk[z]) < PROJ_TOL
            else:
                assert np.all(bk[z] == 0)
        fw = p.ForwardProjectACC(hm, vol, planes)
        fo = O.forward_project(H, vol, N, planes=planes, method="direct", dtype=np.float64)
        assert rel(fw, fo) < PROJ_TOL


def test_standard_rl_with_trust_mask(mods):
    projector, lfdeconv, psfmatrix = mods
    import synthetic
    N = 5
    H, Ht = synthetic.synthetic_psf(N, [-10, 0, 10], 2)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(9)
    img = (rng.random((1, 40, 40)) * 500 + 100).astype(np.float32)
    mask = np.ones((40, 40), np.float32)
    mask[:5] = 0
    img[:, :5] = 0
    x0 = np.ones((3, 1, 40, 40), np.float32)
    p = projector.Projector_gb300()
    r = lfdeconv.DeconvRL(hm, None, 3, x0, logPrint=False, projector=p, im=img, prevedel=False,
                          trustMask=mask)
    with np.errstate(all="ignore"):
        o = O.deconv_rl(H, Ht, N, 3, im=img, x0=x0, prevedel=False, trust_mask=mask, method="direct",
                        dtype=np.float64)
    assert rel(r, o) < RL_TOL


def test_zero_image_rl_gives_zero(mods):
    projector, lfdeconv, psfmatrix = mods
    c = case_inputs("rl_prevedel")
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    p = projector.Projector_gb300()
    img = np.zeros_like(c["img"])
    r = lfdeconv.DeconvRL(hm, None, 2, None, logPrint=False, projector=p, im=img)
    assert np.all(r == 0)


def test_rl_into_pinned_host_array(mods):
    """DeconvRL with ``out`` (a view of pinned host memory) writes the volume of the
    plain call there and returns that array; a wrong shape or type is refused."""
    import torch
    projector, lfdeconv, psfmatrix = mods
    c = case_inputs("rl_prevedel")
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    p = projector.Projector_gb300()
    want = lfdeconv.DeconvRL(hm, None, 2, None, logPrint=False, projector=p, im=c["img"])
    img = torch.empty(c["img"].shape, dtype=torch.float32, pin_memory=True).numpy()
    img[...] = c["img"]
    out = torch.empty(want.shape, dtype=torch.float32, pin_memory=True).numpy()
    r = lfdeconv.DeconvRL(hm, None, 2, None, logPrint=False, projector=p, im=img, out=out)
    assert r is out and np.array_equal(out, want)
    with pytest.raises(ValueError):
        lfdeconv.DeconvRL(hm, None, 2, None, logPrint=False, projector=p, im=img, out=out[:, :, 1:])
    with pytest.raises(ValueError):
        lfdeconv.DeconvRL(hm, None, 2, None, logPrint=False, projector=p, im=img, out=out.astype(np.float64))


def test_full_size_linearity_and_adjointness(mods):
    """The 450 x 450 px, Nnum 15, 11-plane workload: size-independent properties."""
    projector, lfdeconv, psfmatrix = mods
    import synthetic
    z = np.arange(-25, 26, 5)
    H, Ht = synthetic.synthetic_psf(15, z, 7)
    assert max(h.shape[-1] for h in H) == 211
    hm = psfmatrix.HMatrixArrays(H, Ht)
    p = projector.Projector_gb300()
    rng = np.random.default_rng(1)
    x1 = rng.random((11, 1, 450, 450)).astype(np.float32)
    x2 = rng.random((11, 1, 450, 450)).astype(np.float32)
    y = rng.random((1, 450, 450)).astype(np.float32)
    h1 = p.ForwardProjectACC(hm, x1, None).astype(np.float64)
    h2 = p.ForwardProjectACC(hm, x2, None).astype(np.float64)
    h12 = p.ForwardProjectACC(hm, (2.0 * x1 - 0.5 * x2).astype(np.float32), None).astype(np.float64)
    assert rel(h12, 2.0 * h1 - 0.5 * h2) < 1e-5
    bt = p.BackwardProjectACC(hm, y, None).astype(np.float64)
    lhs = np.sum(h1 * y)
    rhs = np.sum(x1.astype(np.float64) * bt)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    # flux: each forward PSF sums to 1, so far from the border a uniform volume
    # projects to Z per pixel on average over whole lenslet periods
    u = np.ones((11, 1, 450, 450), np.float32)
    hu = p.ForwardProjectACC(hm, u, None).astype(np.float64)
    assert abs(hu[0, 150:300, 150:300].mean() - 11.0) < 1e-4


def test_transform_groups_match_uniform_transform(mods):
    """Per-plane transform sizes (grouped) and one size for all planes agree."""
    projector, lfdeconv, psfmatrix = mods
    import synthetic
    N = 7
    H, Ht = synthetic.random_psf(N, [43, 15, 29, 15, 57], seed=11)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(2)
    img = rng.random((2, 56, 63)).astype(np.float32)
    vol = rng.random((5, 2, 56, 63)).astype(np.float32)
    p = projector.Projector_gb300()
    bk = p.BackwardProjectACC(hm, img, None)
    fw = p.ForwardProjectACC(hm, vol, None)
    geo = p.geometry()
    assert geo["groups"] >= 3
    p.context(hm).set_option("plane_transform_sizes", 0)
    p._shape_key = None
    bku = p.BackwardProjectACC(hm, img, None)
    fwu = p.ForwardProjectACC(hm, vol, None)
    assert p.geometry()["groups"] == 1
    assert rel(bk, bku) < PROJ_TOL and rel(fw, fwu) < PROJ_TOL
    bo = O.backward_project(Ht, img, N, method="direct", dtype=np.float64)
    assert rel(bk, bo) < PROJ_TOL


SIZED_FFT_SIZES = [f for f in range(4, 161, 2)
                   if all(f % p for p in (11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71, 73, 79))]


@pytest.mark.parametrize("f", SIZED_FFT_SIZES)
def test_every_transform_size(mods, f):
    """Each size-specialised transform (every even 7-smooth f in [4, 160]) against
    the oracle, forward and backward, on ragged lenslet grids (odd and even row
    counts, images not a multiple of Nnum)."""
    import torch
    import synthetic
    import _flf
    N = 3
    H, Ht = synthetic.random_psf(N, [3, 5], seed=f)          # kernel radius 1 lenslet
    R = 2
    Ly = max(1, f - R - (f % 3))
    Lx = max(1, f - R - (f % 5) - 1)
    Y, X = N * Ly - 1 if Ly > 1 else N, N * Lx - 2 if Lx > 1 else N
    T = 2
    rng = np.random.default_rng(f)
    img = rng.random((T, Y, X)).astype(np.float32)
    vol = rng.random((2, T, Y, X)).astype(np.float32)
    dev = torch.device("cuda", 0)
    ctx = _flf.Context(N, 2, 0)
    for z in range(2):
        ctx.upload_psf(z, _flf.FLF_DIR_FORWARD, H[z])
        ctx.upload_psf(z, _flf.FLF_DIR_BACKWARD, Ht[z])
    ctx.set_option("plane_transform_sizes", 0)
    ctx.prepare(Y, X, fft_size=f)
    assert ctx.geometry()["f"] == f
    bk = torch.full((2, T, Y, X), float("nan"), device=dev)
    fw = torch.full((T, Y, X), float("nan"), device=dev)
    ctx.backward(torch.as_tensor(img, device=dev), bk, T, Y, X)
    ctx.forward(torch.as_tensor(vol, device=dev), fw, T, Y, X)
    ctx.synchronize()
    ctx.close()
    bo = O.backward_project(Ht, img, N, method="direct", dtype=np.float64)
    fo = O.forward_project(H, vol, N, method="direct", dtype=np.float64)
    assert rel(bk.cpu().numpy(), bo) < PROJ_TOL
    assert rel(fw.cpu().numpy(), fo) < PROJ_TOL


def test_planes_validation(mods):
    projector, lfdeconv, psfmatrix = mods
    c = case_inputs("planes_n7")
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    p = projector.Projector_gb300()
    with pytest.raises(IndexError):
        p.BackwardProjectACC(hm, c["img"], [5])
    with pytest.raises(ValueError):
        p.BackwardProjectACC(hm, c["img"], [1, 1])
    with pytest.raises(ValueError):
        p.BackwardProjectACC(hm, c["img"][0], None)


def test_context_errors(mods):
    import _flf
    with pytest.raises(_flf.FlfError):
        _flf.Context(4, 3)          # even Nnum
    ctx = _flf.Context(5, 2)
    with pytest.raises(_flf.FlfError):
        ctx.upload_psf(0, 0, np.zeros((3, 3, 10, 10), np.float32))   # even h
    with pytest.raises(_flf.FlfError):
        ctx.prepare(30, 30)          # PSFs not uploaded
    ctx.close()


def test_geometry_cache_across_image_shapes(mods):
    """Alternating image shapes in one context: results equal fresh contexts', and a
    shape seen before reuses its parked transfer matrices (no new device memory)."""
    projector, lfdeconv, psfmatrix = mods
    import synthetic
    N = 5
    H, Ht = synthetic.random_psf(N, [21, 11, 31], seed=7)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(3)
    imgs = {s: rng.random((1,) + s).astype(np.float32) for s in [(40, 35), (30, 30), (55, 50)]}
    fresh = {s: projector.Projector_gb300().BackwardProjectACC(hm, im, None) for s, im in imgs.items()}
    p = projector.Projector_gb300()
    mem = []
    for s in [(40, 35), (30, 30), (40, 35), (55, 50), (30, 30)]:
        out = p.BackwardProjectACC(hm, imgs[s], None)
        assert np.array_equal(out, fresh[s]), s
        mem.append(p.context(hm).memory_usage())
    assert mem[2] == mem[1]            # (40, 35) came back from the cache
    assert mem[3] > mem[2]             # a third shape: two parked + one active
    assert mem[4] == mem[3]            # (30, 30) still parked (cache of 2)
    ctx = p.context(hm)
    ctx.set_option("geometry_cache", 0)
    out = p.BackwardProjectACC(hm, imgs[(40, 35)], None)
    assert np.array_equal(out, fresh[(40, 35)])
    assert ctx.memory_usage() < mem[4]


def test_released_psfs_keep_projections_and_refuse_new_shapes(mods):
    """With release_psf the PSF quadrants are freed after the precompute: the
    projections of that image shape are unchanged, the memory count drops by the
    PSF bytes, and another shape is refused until the PSFs are uploaded again."""
    projector, lfdeconv, psfmatrix = mods
    import _flf
    import synthetic
    N = 5
    H, Ht = synthetic.random_psf(N, [21, 11, 31], seed=9)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(4)
    img = rng.random((2, 40, 35)).astype(np.float32)
    want_b = projector.Projector_gb300().BackwardProjectACC(hm, img, None)
    want_f = projector.Projector_gb300().ForwardProjectACC(hm, want_b, None)
    p = projector.Projector_gb300()
    p.BackwardProjectACC(hm, img, None)
    ctx = p.context(hm)
    before = ctx.memory_usage()
    ctx.set_option("release_psf", 1)
    psf_bytes = 2 * sum(h.nbytes for h in H)
    assert ctx.memory_usage() == before - psf_bytes
    assert np.array_equal(p.BackwardProjectACC(hm, img, None), want_b)
    assert np.array_equal(p.ForwardProjectACC(hm, want_b, None), want_f)
    small = img[:, :30, :30].copy()
    with pytest.raises(_flf.FlfError) as e:
        p.BackwardProjectACC(hm, small, None)
    assert e.value.code == -4 and "released" in str(e.value)
    for z in range(len(H)):
        ctx.upload_psf(z, _flf.FLF_DIR_FORWARD, H[z])
        ctx.upload_psf(z, _flf.FLF_DIR_BACKWARD, Ht[z])
    p._shape_key = None
    assert rel(p.BackwardProjectACC(hm, small, None),
               projector.Projector_gb300().BackwardProjectACC(hm, small, None)) == 0.0


def test_autotune_keeps_results_and_caches(mods, tmp_path):
    """flf_autotune picks a launch shape per image shape; results do not change
    beyond rounding, and a cache file brings the choice back without timing."""
    projector, lfdeconv, psfmatrix = mods
    import json
    import synthetic
    N = 7
    H, Ht = synthetic.random_psf(N, [43, 15, 29], seed=5)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(8)
    img = rng.random((2, 56, 63)).astype(np.float32)
    vol = rng.random((3, 2, 56, 63)).astype(np.float32)
    p = projector.Projector_gb300()
    bk0, fw0 = p.BackwardProjectACC(hm, img, None), p.ForwardProjectACC(hm, vol, None)
    cache = str(tmp_path / "tune.json")
    tuned = p.autotune(hm, 2, 56, 63, cache_path=cache)
    assert tuned["stages"] in (2, 3) and tuned["split"] in (1, 2)
    assert tuned["chunk_rows_forward"] in (8, 10, 12, 16, 20) and tuned["chunk_rows_backward"] in (8, 10, 12, 16, 20)
    bk1, fw1 = p.BackwardProjectACC(hm, img, None), p.ForwardProjectACC(hm, vol, None)
    assert rel(bk1, bk0) < PROJ_TOL and rel(fw1, fw0) < PROJ_TOL
    # the choice stays with its image shape across a shape switch
    p.BackwardProjectACC(hm, img[:, :40, :40], None)
    bk2 = p.BackwardProjectACC(hm, img, None)
    assert np.array_equal(bk2, bk1)
    # a fresh projector reads the cache (a planted shape proves no timing ran)
    with open(cache) as f:
        d = json.load(f)
    (k,) = d.keys()
    d[k] = {"stages": 3, "chunk_rows_forward": 10, "chunk_rows_backward": 8, "split": 1}
    with open(cache, "w") as f:
        json.dump(d, f)
    q = projector.Projector_gb300()
    assert q.autotune(hm, 2, 56, 63, cache_path=cache) == d[k]
    assert rel(q.BackwardProjectACC(hm, img, None), bk0) < PROJ_TOL


def test_bounded_wait_gives_up_and_context_recovers(mods):
    """A bulk copy that never arrives (test option test_drop_chunk) makes the
    multiply-accumulate's wait for that ring slot run out after a short limit:
    the kernel sets the error flag and returns, the next synchronize reports
    FLF_E_TIMEOUT, and the context then projects correctly again."""
    projector, lfdeconv, psfmatrix = mods
    import _flf
    import synthetic
    import torch
    N = 5
    H, Ht = synthetic.random_psf(N, [21, 11], seed=12)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(6)
    img = rng.random((1, 40, 35)).astype(np.float32)
    want = projector.Projector_gb300().BackwardProjectACC(hm, img, None)
    p = projector.Projector_gb300()
    p.BackwardProjectACC(hm, img, None)
    ctx = p.context(hm)
    ctx.set_option("mac_wait_limit_us", 2000)
    ctx.set_option("test_drop_chunk", 0)
    img_d = torch.as_tensor(img, device="cuda")
    vol = torch.zeros((2, 1, 40, 35), device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    ctx.backward(img_d, vol, 1, 40, 35, None, stream=s)
    with pytest.raises(_flf.FlfError) as e:
        ctx.synchronize(s)
    assert e.value.code == -5
    ctx.set_option("test_drop_chunk", -1)
    ctx.set_option("mac_wait_limit_us", 1000000)
    ctx.synchronize(s)
    assert np.array_equal(p.BackwardProjectACC(hm, img, None), want)
    with pytest.raises(_flf.FlfError):
        ctx.set_option("mac_wait_limit_us", 10)
