"""CUDA-graph replay of the RL loop (flf_rl_graph_create / flf_graph_launch).

A replay must give bit-identical results to the direct flf_rl_iterate call on
the same inputs (same kernels, same launch shapes), for both RL variants and
for T above the frames one multiply-accumulate pass takes; a graph whose
buffers were freed refuses to launch.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built_lib):
    import torch
    import _flf
    import projector
    import psfmatrix
    import synthetic
    _flf.load_library()
    return torch, _flf, projector, psfmatrix, synthetic


@pytest.mark.parametrize("prevedel,T", [(True, 1), (True, 6), (False, 2)])
def test_graph_replay_matches_direct(env, prevedel, T):
    torch, _flf, projector, psfmatrix, synthetic = env
    N, Y, X, iters = 7, 63, 70, 3
    H, Ht = synthetic.random_psf(N, [43, 15, 29], seed=11)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(4)
    x0 = torch.tensor(rng.random((3, T, Y, X)), dtype=torch.float32, device="cuda")
    if prevedel:
        ref = torch.tensor(rng.random((3, T, Y, X)) + 0.5, dtype=torch.float32, device="cuda")
        norm = None
    else:
        ref = torch.tensor(rng.random((T, Y, X)) * 100 + 10, dtype=torch.float32, device="cuda")
        norm = torch.tensor(rng.random((3, 1, Y, X)) + 0.5, dtype=torch.float32, device="cuda")
    p = projector.Projector_gb300()
    p.useGraphs = False
    direct = x0.clone()
    p.RichardsonLucy(hm, direct, ref, iters, prevedel=prevedel, norm=norm)
    twice = direct.clone()
    p.RichardsonLucy(hm, twice, ref, iters, prevedel=prevedel, norm=norm)

    x = x0.clone()
    g = p.RichardsonLucyGraph(hm, x, ref, iters, prevedel=prevedel, norm=norm)
    assert g.kernels > 0
    assert torch.equal(x, x0)          # capture runs nothing
    g.launch(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(x, direct)
    g.launch(torch.cuda.current_stream().cuda_stream)   # replays continue from x
    torch.cuda.synchronize()
    assert torch.equal(x, twice)
    x.copy_(x0)                        # refilled in place: same result again
    g.launch(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(x, direct)
    g.close()
    # the projector's own graph cache (staging tensors) gives the same volumes
    p.useGraphs = True
    y = x0.clone()
    p.RichardsonLucy(hm, y, ref, iters, prevedel=prevedel, norm=norm)
    assert torch.equal(y, direct)
    p.RichardsonLucy(hm, y, ref, iters, prevedel=prevedel, norm=norm)
    assert torch.equal(y, twice)
    assert len(p._graphs) == 1


def test_graph_refuses_after_buffers_freed(env):
    torch, _flf, projector, psfmatrix, synthetic = env
    N, T, Y, X = 5, 1, 40, 45
    H, Ht = synthetic.random_psf(N, [21, 11], seed=2)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    x = torch.ones((2, T, Y, X), dtype=torch.float32, device="cuda")
    ref = torch.ones((2, T, Y, X), dtype=torch.float32, device="cuda")
    p = projector.Projector_gb300()
    g = p.RichardsonLucyGraph(hm, x, ref, 2)
    g.launch()
    torch.cuda.synchronize()
    p.context(hm).clear_cache()
    with pytest.raises(_flf.FlfError, match="FLF_E_STATE"):
        g.launch()
    g.close()
    # the projector's cached graph is captured again after the buffers changed
    x.fill_(1.0)
    p.RichardsonLucy(hm, x, ref, 2)
    first = x.clone()
    p.context(hm).clear_cache()
    x.fill_(1.0)
    p.RichardsonLucy(hm, x, ref, 2)
    assert torch.equal(x, first)
    p.ClearCache()
    with pytest.raises(_flf.FlfError):
        g.launch()


def test_combined_deconvolution_graph_of_two_sizes(env):
    """flf_deconv_graph_create (back projection, x0 = Htf, Prevedel iterations) for
    two image sizes of one context, combined by flf_graph_combine into one graph:
    one launch gives the volumes of the direct calls, bit for bit."""
    torch, _flf, projector, psfmatrix, synthetic = env
    N, iters, T = 5, 3, 2
    H, Ht = synthetic.random_psf(N, [21, 11, 31], seed=13)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    rng = np.random.default_rng(8)
    sizes = [(40, 35), (55, 50)]
    imgs = [torch.tensor(rng.random((T,) + sz) * 100 + 10, dtype=torch.float32, device="cuda") for sz in sizes]
    p = projector.Projector_gb300()
    ctx = p.context(hm)
    ctx.set_option("geometry_cache", 2)
    s = torch.cuda.current_stream().cuda_stream
    want, bufs = [], []
    for (Y, X), img in zip(sizes, imgs):
        p._prepare(ctx, Y, X, hm)
        htf = torch.empty((3, T, Y, X), device="cuda")
        x = torch.empty_like(htf)
        ctx.backward(img, htf, T, Y, X, None, stream=s)
        x.copy_(htf)
        ctx.rl_iterate(x, htf, None, _flf.FLF_RL_PREVEDEL, iters, T, Y, X, stream=s)
        want.append(x.clone())
        bufs.append((torch.empty_like(htf), torch.zeros_like(htf)))
    torch.cuda.synchronize()
    graphs = []
    for (Y, X), img, (htf, x) in zip(sizes, imgs, bufs):
        p._prepare(ctx, Y, X, hm)
        graphs.append(ctx.deconv_graph(img, htf, x, iters, T, Y, X))
    whole = ctx.combine_graphs(graphs)
    assert whole.kernels == sum(g.kernels for g in graphs) > 0
    for _ in range(2):
        for _, x in bufs:
            x.zero_()
        whole.launch(s)
        ctx.synchronize(s)
        for w, (_, x) in zip(want, bufs):
            assert torch.equal(x, w)
    whole.close()
    for g in graphs:
        g.close()
