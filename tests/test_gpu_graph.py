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
