"""GPU test of flf_backward_noalloc, the back projection that allocates nothing.

Some callers cannot ask the CUDA driver for memory while they run (a
real-time acquisition loop that must never wait on the device allocator, or
a plug-in whose host application owns all device memory).  For them the
library offers one entry point whose intermediate spectra live in a fixed
16 MiB device array inside the library.  This file checks, through the C ABI,
that it returns the same volume as the regular flf_backward on two calls in a
row without changing the device's free memory or the library's own memory
count, and that it refuses what it cannot do without allocating.  It is named
so that pytest collects it last.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PROJ_TOL = 2e-5   # the projection tolerance of the other GPU tests (max abs error / max abs value)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def lib(built_lib):
    import _flf
    _flf.load_library()
    return _flf


def _context(_flf, H, Ht, nnum):
    ctx = _flf.Context(nnum, len(H), 0)
    for z in range(len(H)):
        ctx.upload_psf(z, _flf.FLF_DIR_FORWARD, H[z])
        ctx.upload_psf(z, _flf.FLF_DIR_BACKWARD, Ht[z])
    return ctx


def test_backward_noalloc_matches_backward_twice(lib):
    import torch
    import synthetic
    _flf = lib
    dev = torch.device("cuda", 0)
    H, Ht = synthetic.synthetic_psf(15, np.arange(-25, 26, 5), 7)      # 11 planes, h up to 211
    ctx = _context(_flf, H, Ht, 15)
    T, Y, X = 2, 450, 450
    ctx.prepare(Y, X)
    stream = torch.cuda.current_stream(dev).cuda_stream
    g = torch.Generator(device="cpu").manual_seed(5)
    img = torch.rand((T, Y, X), generator=g).to(dev)
    ref = torch.zeros((11, T, Y, X), device=dev)
    ctx.backward(img, ref, T, Y, X, None, stream=stream)
    ctx.synchronize(stream)
    refh = ref.cpu().numpy()
    out = torch.empty((11, T, Y, X), device=dev)
    # one call at set-up time: under CUDA's lazy loading the first launch of a
    # kernel makes the driver load that kernel's code into device memory
    out.fill_(float("nan"))
    ctx.backward_noalloc(img, out, T, Y, X, stream=stream)
    ctx.synchronize(stream)
    torch.cuda.synchronize()
    # nothing may be allocated by the calls: neither by the library (its own
    # accounting) nor anywhere on the device (driver free memory)
    lib_bytes = ctx.memory_usage()
    free_before = torch.cuda.mem_get_info(dev)[0]
    for _ in range(2):
        out.fill_(float("nan"))
        ctx.backward_noalloc(img, out, T, Y, X, stream=stream)
        ctx.synchronize(stream)
        assert ctx.memory_usage() == lib_bytes
        assert torch.cuda.mem_get_info(dev)[0] == free_before
        assert rel(out.cpu().numpy(), refh) < PROJ_TOL
    ctx.close()


def test_backward_noalloc_needs_prepared_matrices(lib):
    import torch
    import synthetic
    _flf = lib
    H, Ht = synthetic.random_psf(5, [11, 21], seed=2)
    ctx = _context(_flf, H, Ht, 5)
    img = torch.zeros((1, 30, 30), device="cuda")
    vol = torch.zeros((2, 1, 30, 30), device="cuda")
    with pytest.raises(_flf.FlfError) as e:
        ctx.backward_noalloc(img, vol, 1, 30, 30)
    assert e.value.code == -4 and "flf_prepare" in str(e.value)
    ctx.close()


def test_backward_noalloc_rejects_oversize_geometry(lib):
    import torch
    import synthetic
    _flf = lib
    H, Ht = synthetic.random_psf(15, [31], seed=3)
    ctx = _context(_flf, H, Ht, 15)
    ctx.prepare(150, 150, fft_size=100)          # 2 * 225 * 100 * 51 * 8 bytes > 16 MiB
    img = torch.zeros((1, 150, 150), device="cuda")
    vol = torch.zeros((1, 1, 150, 150), device="cuda")
    with pytest.raises(_flf.FlfError) as e:
        ctx.backward_noalloc(img, vol, 1, 150, 150)
    assert e.value.code == -1 and "16777216" in str(e.value)
    ctx.close()
