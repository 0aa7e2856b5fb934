"""ctypes binding of libflf.so (C ABI in include/flf.h).

The GB300 counterpart of the reference's compiled extension ``py_light_field``
(imported as ``plf`` by projector.py / lfdeconv.py).  There is no CPU fallback:
importing works without a GPU, but creating a context raises ``FlfError`` when
the library or a CUDA device is missing.
"""

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libflf.so")

FLF_OK = 0
FLF_DIR_FORWARD = 0
FLF_DIR_BACKWARD = 1
FLF_RL_PREVEDEL = 0
FLF_RL_STANDARD = 1

_ERRNAMES = {-1: "FLF_E_ARG", -2: "FLF_E_CUDA", -3: "FLF_E_NOMEM", -4: "FLF_E_STATE", -5: "FLF_E_TIMEOUT"}

# name -> (restype, argtypes); mirrors include/flf.h
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_F = ctypes.c_float
_SIGS = {
    "flf_ctx_create": (_I, [ctypes.POINTER(_P), _I, _I, _I]),
    "flf_ctx_destroy": (_I, [_P]),
    "flf_last_error": (_I, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "flf_psf_upload": (_I, [_P, _I, _I, _P, _I, _I]),
    "flf_prepare": (_I, [_P, _I, _I, _I, _I]),
    "flf_forward": (_I, [_P, _P, _P, _I, _I, _I, _P, _I, _P]),
    "flf_backward": (_I, [_P, _P, _P, _I, _I, _I, _P, _I, _P]),
    "flf_rl_iterate": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "flf_memory_usage": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "flf_memory_epoch": (_I, [_P, ctypes.POINTER(ctypes.c_ulonglong)]),
    "flf_clear_cache": (_I, [_P]),
    "flf_geometry": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "flf_version": (_I, [ctypes.c_char_p, ctypes.c_size_t]),
    "flf_profile": (_I, [_P, _I]),
    "flf_profile_read": (_I, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "flf_set_option": (_I, [_P, ctypes.c_char_p, ctypes.c_longlong]),
    "flf_synchronize": (_I, [_P, _P]),
    "flf_backward_noalloc": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "flf_resample_bilinear": (_I, [_P, _I, _I, _P, _I, _P, _I, _P, _P]),
    "flf_autotune": (_I, [_P, _I, _I, _I, ctypes.POINTER(ctypes.c_int), _P]),
    "flf_rl_graph_create": (_I, [_P, ctypes.POINTER(_P), _P, _P, _P, _I, _I, _I, _I, _I]),
    "flf_graph_launch": (_I, [_P, _P]),
    "flf_deconv_graph_create": (_I, [_P, ctypes.POINTER(_P), _P, _P, _P, _I, _I, _I, _I]),
    "flf_graph_combine": (_I, [ctypes.POINTER(_P), ctypes.POINTER(_P), _I]),
    "flf_graph_kernels": (_I, [_P]),
    "flf_graph_destroy": (_I, [_P]),
    "flf_set_tuned": (_I, [_P, _I, _I, ctypes.POINTER(ctypes.c_int)]),
    "flf_psf_debye": (_I, [_P, _I, ctypes.c_longlong, _D, _D, _D, _D, _P, _P, _I, _D, _D, _P]),
    "flf_psf_lf_input": (_I, [_P, _P, _I, _I, _P, _I, _I, _I, _I, _I, _I, _P]),
    "flf_psf_lf_bin": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _I, _I, _P]),
    "flf_psf_ht": (_I, [_P, _P, _I, _I, _I, _I, _P]),
    "flf_conv3d": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _P, ctypes.c_longlong, _P, _P]),
    "flf_net_conv_wide_tcgen05": (_I, [_I]),
    "flf_conv3d_wgrad": (_I, [_P, _P, _P, _I, _I, _I, _I, _I, _I, _P, ctypes.c_longlong, _P]),
    "flf_conv3d_tc": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "flf_conv3d_x1": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "flf_net_status": (_I, []),
    "flf_net_conv16_tcgen05": (_I, [_I]),
    "flf_conv3d_pool": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "flf_conv3d_flip": (_I, [_P, _P, _I, _I, _P]),
    "flf_conv3d_pack": (_I, [_P, _P, _I, _I, _P]),
    "flf_bias_grad": (_I, [_P, _P, ctypes.c_longlong, _I, _P, ctypes.c_longlong, _P]),
    "flf_pool2": (_I, [_P, _P, _I, _I, _I, _I, _I, _P]),
    "flf_pool2_bwd": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "flf_up2_add": (_I, [_P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "flf_up2_bwd": (_I, [_P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "flf_mse_grad": (_I, [_P, _P, _P, _P, ctypes.c_longlong, _I, _P]),
    "flf_adam": (_I, [_P, _P, _P, _P, _P, ctypes.c_longlong, _F, _F, _F, _F, _F, _F, _F, _P]),
    "flf_render_blobs": (_I, [_P, _I, _I, _I, _P, _I, _F, _P, _P]),
    "flf_net_launches": (ctypes.c_longlong, []),
    "flf_ws_input": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _F, _F, _P]),
    "flf_ws_head": (_I, [_P, _P, _F, _F, _P, _P, _I, _I, _I, _I, _I, _I, _I, _P]),
}
NOALLOC_SCRATCH_BYTES = 16 * 1024 * 1024
TUNED_KEYS = ("stages", "chunk_rows_forward", "chunk_rows_backward", "split")

_lib = None


class FlfError(RuntimeError):
    """Failure reported by libflf (status code and message)."""

    def __init__(self, code, message):
        super().__init__("%s (%d): %s" % (_ERRNAMES.get(code, "FLF_E?"), code, message))
        self.code = code


def load_library(path=LIB_PATH):
    """Load libflf.so and declare every entry point of include/flf.h."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FlfError(-4, "libflf.so not found at %s: run __graft_entry__.build() or "
                           "python fast-light-field_gb300/build_lib.py" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGS)


def version():
    lib = load_library()
    buf = ctypes.create_string_buffer(256)
    lib.flf_version(buf, 256)
    return buf.value.decode()


def _ptr(x):
    """Raw pointer of a torch tensor / numpy array / int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError("cannot take a pointer of %r" % type(x))


def resample_bilinear(img, yq, xq, out, stream=None):
    """flf_resample_bilinear on device tensors: img float32 [H, W], yq / xq float64,
    out float64 [len(yq), len(xq)]."""
    lib = load_library()
    H, W = int(img.shape[0]), int(img.shape[1])
    rc = lib.flf_resample_bilinear(_ptr(img), H, W, _ptr(yq), int(yq.shape[0]), _ptr(xq), int(xq.shape[0]),
                                   _ptr(out), _ptr(stream))
    if rc != FLF_OK:
        buf = ctypes.create_string_buffer(1024)
        lib.flf_last_error(None, buf, 1024)
        raise FlfError(rc, buf.value.decode(errors="replace"))


def _check_global(rc):
    if rc != FLF_OK:
        buf = ctypes.create_string_buffer(1024)
        _lib.flf_last_error(None, buf, 1024)
        raise FlfError(rc, buf.value.decode(errors="replace"))


def psf_debye(out, mode, npoints, dx, M, k, sin_alpha, s, cw, koi, stream=None):
    """flf_psf_debye on device tensors (out / cw complex128, s float64)."""
    lib = load_library()
    _check_global(lib.flf_psf_debye(_ptr(out), int(mode), int(npoints), float(dx), float(M), float(k),
                                    float(sin_alpha), _ptr(s), _ptr(cw), int(s.shape[0]), float(koi.real),
                                    float(koi.imag), _ptr(stream)))


def psf_lf_input(out, wave, support, max_bug, lens, lens_h, L, nh, osr, q0, nq, stream=None):
    lib = load_library()
    _check_global(lib.flf_psf_lf_input(_ptr(out), _ptr(wave), int(support), int(bool(max_bug)), _ptr(lens),
                                       int(lens_h), int(L), int(nh), int(osr), int(q0), int(nq), _ptr(stream)))


def psf_lf_bin(out, field, L, S, nh, osr, q0, nq, lo, hi, first, stream=None):
    lib = load_library()
    _check_global(lib.flf_psf_lf_bin(_ptr(out), _ptr(field), int(L), int(S), int(nh), int(osr), int(q0), int(nq),
                                     int(lo), int(hi), int(first), _ptr(stream)))


def psf_ht(Ht, H, Z, nh, S, N, stream=None):
    lib = load_library()
    _check_global(lib.flf_psf_ht(_ptr(Ht), _ptr(H), int(Z), int(nh), int(S), int(N), _ptr(stream)))


def _vshape(t):
    """(B, Z, Y, X, C) of a channels-last volume tensor."""
    B, Z, Y, X, C = (int(v) for v in t.shape)
    return B, Z, Y, X, C


def conv3d(x, w, bias, y, relu=False, mask=None, stream=None, ws=None, wp=None):
    """y = [relu](conv3x3x3(x, w) + bias) [* (mask > 0)]; x [B,Z,Y,X,Ci], w [27,Ci,Co], y [B,Z,Y,X,Co] bf16;
    ws: optional float32 workspace for split-K layers (one B*Z*Y*X*Co slice per split, at least two);
    wp: optional packed weights (conv3d_pack of w), with which the wide layers run on tcgen05."""
    lib = load_library()
    B, Z, Y, X, Ci = _vshape(x)
    Co = int(y.shape[-1])
    _check_global(lib.flf_conv3d(_ptr(x), _ptr(w), _ptr(bias), _ptr(mask), _ptr(y), B, Z, Y, X, Ci, Co,
                                 int(bool(relu)), _ptr(ws), int(ws.numel()) if ws is not None else 0, _ptr(wp),
                                 _ptr(stream)))


def conv3d_x1(x, w, bias, y, relu=False, stream=None):
    """y = [relu](3x3x1 convolution over (dz, dy) with the taps dx = 1 of w [27, 16, 16] + bias);
    x, y [B, Z, Y, X, 16] bf16 (the first layer of the warm-start network, whose input
    carries the x neighbours as channels)."""
    lib = load_library()
    B, Z, Y, X, _ = _vshape(x)
    _check_global(lib.flf_conv3d_x1(_ptr(x), _ptr(w), _ptr(bias), _ptr(y), B, Z, Y, X, int(bool(relu)), _ptr(stream)))


def conv3d_pool(x, w, bias, y, pooled, relu=False, stream=None):
    """y = [relu](conv3d(x, w) + bias) for 16 -> 16 channels and pooled = pool2(y)
    (2x2x2 average, [B, Z/2, Y/2, X/2, 16]) from the same launch; x, y [B, Z, Y, X, 16]
    bf16 with Z, Y, X even."""
    lib = load_library()
    B, Z, Y, X, _ = _vshape(x)
    if tuple(pooled.shape) != (B, Z // 2, Y // 2, X // 2, 16):
        raise FlfError(-1, "pooled must be [B, Z/2, Y/2, X/2, 16], got %s" % (tuple(pooled.shape),))
    _check_global(lib.flf_conv3d_pool(_ptr(x), _ptr(w), _ptr(bias), _ptr(y), _ptr(pooled), B, Z, Y, X,
                                      int(bool(relu)), _ptr(stream)))


def conv_wide_tcgen05(mode):
    """Kernel of the wide layers (64 / 128 channels) when packed weights are given:
    0 / False = mma.sync, 1 / True (the default) = tcgen05, 2..5 = tcgen05 with 1..4
    M tiles per work item; returns the previous setting."""
    return int(load_library().flf_net_conv_wide_tcgen05(int(mode)))


def conv3d_pack(w, wp, stream=None):
    """wp = w [27, Ci, Co] bf16 packed as the tcgen05 wide-layer kernel's B blocks (same size)."""
    _, Ci, Co = w.shape
    _check_global(load_library().flf_conv3d_pack(_ptr(w), _ptr(wp), int(Ci), int(Co), _ptr(stream)))


def conv3d_tc(x, w, bias, y, relu=False, mask=None, stream=None, rows=4):
    """conv3d for 16 -> 16 channels on the tcgen05 tensor cores.

    rows = 0: the warp-specialised kernel with TMA-staged input slabs (-1: the
    same with 32-byte swizzled slabs);
    1, 4, 5: single-role kernels with tiles of rows x 128 voxels (5 = 4 rows,
    double-buffered)."""
    lib = load_library()
    B, Z, Y, X, C = _vshape(x)
    if C != 16 or int(y.shape[-1]) != 16:
        raise ValueError("conv3d_tc takes 16 channels in and out")
    _check_global(lib.flf_conv3d_tc(_ptr(x), _ptr(w), _ptr(bias), _ptr(mask), _ptr(y), B, Z, Y, X,
                                    int(bool(relu)), int(rows), _ptr(stream)))


def conv16_tcgen05(mode):
    """Select the kernels conv3d and ws_head use for 16 / 32 -> 16 / 32 channels and
    return the previous mode: 0 or False = mma.sync; 1 = the warp-specialised
    tcgen05 kernel for 16 -> 16, mma.sync for the 32-channel layers; 2 or True
    (the default) = tcgen05 for all of them."""
    if type(mode) is bool:
        mode = 2 if mode else 0
    return int(load_library().flf_net_conv16_tcgen05(int(mode)))


def net_launches():
    """Kernel launches made by the network entry points since the library was loaded."""
    return int(load_library().flf_net_launches())


def net_status():
    """Raise FlfError if a bounded wait in a tensor-core convolution gave up."""
    _check_global(load_library().flf_net_status())


def conv3d_wgrad(x, dy, dw, stream=None, ws=None):
    """dw [27,Ci,Co] float32 += weight gradient of conv3d(x, .) for output gradient dy.

    ws: float32 workspace for the per-chunk partial gradients (27*Ci*Co floats per
    chunk; more chunks spread the voxels over more CTAs), summed in a fixed order."""
    lib = load_library()
    B, Z, Y, X, Ci = _vshape(x)
    _check_global(lib.flf_conv3d_wgrad(_ptr(x), _ptr(dy), _ptr(dw), B, Z, Y, X, Ci, int(dy.shape[-1]),
                                       _ptr(ws), int(ws.numel()) if ws is not None else 0, _ptr(stream)))


def conv3d_flip(w, w2, stream=None):
    lib = load_library()
    _check_global(lib.flf_conv3d_flip(_ptr(w), _ptr(w2), int(w.shape[1]), int(w.shape[2]), _ptr(stream)))


def bias_grad(g, db, stream=None, ws=None):
    """db [C] += sums of g [..., C] over all rows; ws: float32 workspace for the
    per-block sums (C floats per block of 2048 rows), added in block order."""
    lib = load_library()
    C = int(g.shape[-1])
    _check_global(lib.flf_bias_grad(_ptr(g), _ptr(db), int(g.numel() // C), C, _ptr(ws),
                                    int(ws.numel()) if ws is not None else 0, _ptr(stream)))


def pool2(x, out, stream=None):
    lib = load_library()
    _check_global(lib.flf_pool2(_ptr(x), _ptr(out), *_vshape(x), _ptr(stream)))


def pool2_bwd(gpool, gskip, act, gin, stream=None):
    lib = load_library()
    _check_global(lib.flf_pool2_bwd(_ptr(gpool), _ptr(gskip), _ptr(act), _ptr(gin), *_vshape(gin), _ptr(stream)))


def up2_add(low, skip, out, stream=None):
    lib = load_library()
    _check_global(lib.flf_up2_add(_ptr(low), _ptr(skip), _ptr(out), *_vshape(out), _ptr(stream)))


def up2_bwd(g, act, glow, stream=None):
    lib = load_library()
    _check_global(lib.flf_up2_bwd(_ptr(g), _ptr(act), _ptr(glow), *_vshape(g), _ptr(stream)))


def mse_grad(y, target, g, loss, stream=None):
    lib = load_library()
    C = int(y.shape[-1])
    _check_global(lib.flf_mse_grad(_ptr(y), _ptr(target), _ptr(g), _ptr(loss), int(y.numel() // C), C,
                                   _ptr(stream)))


def adam(w, g, m, v, wb, lr, b1, b2, eps, c1, c2, wd, stream=None):
    lib = load_library()
    _check_global(lib.flf_adam(_ptr(w), _ptr(g), _ptr(m), _ptr(v), _ptr(wb), int(w.numel()), lr, b1, b2, eps, c1,
                               c2, wd, _ptr(stream)))


def render_blobs(vol, pts, sigma, stream=None, acc=None):
    """vol [Z,Y,X] float32 += Gaussian blobs at pts [n,4] = (z, y, x, amplitude).

    acc: int64 scratch of Z*Y*X elements; with it the blob terms are summed as
    fixed-point integers, so the volume is the same bits on every run."""
    lib = load_library()
    Z, Y, X = (int(v) for v in vol.shape)
    if acc is not None and acc.numel() < Z * Y * X:
        raise ValueError("render_blobs: acc needs %d elements" % (Z * Y * X))
    _check_global(lib.flf_render_blobs(_ptr(vol), Z, Y, X, _ptr(pts), int(pts.shape[0]), float(sigma),
                                       _ptr(acc), _ptr(stream)))


def ws_input(htf, hth1, ht1, sum_x1, out, c2, c3, stream=None):
    """Warm-start network input [T, Zp, Yp, Xp, 16] from Htf [Z, T, Y, X] (flf_ws_input)."""
    lib = load_library()
    Z, T, Y, X = (int(v) for v in htf.shape)
    Zp, Yp, Xp = (int(v) for v in out.shape[1:4])
    _check_global(lib.flf_ws_input(_ptr(htf), _ptr(hth1), _ptr(ht1), _ptr(sum_x1), _ptr(out), T, Z, Y, X, Zp, Yp,
                                   Xp, float(c2), float(c3), _ptr(stream)))


def ws_head(d, w, bias, floor, sum_x1, x0, stream=None):
    """Start volume x0 [Z, T, Y, X] from the last features d (flf_ws_head)."""
    lib = load_library()
    T, Zp, Yp, Xp = (int(v) for v in d.shape[:4])
    Z, _, Y, X = (int(v) for v in x0.shape)
    _check_global(lib.flf_ws_head(_ptr(d), _ptr(w), float(bias), float(floor), _ptr(sum_x1), _ptr(x0), T, Z, Y, X,
                                  Zp, Yp, Xp, _ptr(stream)))


class RLGraph:
    """A captured RL run; launch() replays it on a stream.  Keeps its tensors alive."""

    def __init__(self, ctx, handle, keep):
        self._ctx, self._h, self._keep = ctx, handle, keep
        self.kernels = ctx._lib.flf_graph_kernels(handle)

    def launch(self, stream=None):
        if not (self._h and self._h.value and self._ctx._h and self._ctx._h.value):
            raise FlfError(-4, "the RL graph or its context was closed")
        self._ctx._check(self._ctx._lib.flf_graph_launch(self._h, _ptr(stream)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._ctx._lib.flf_graph_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One libflf context: PSFs of one Nnum / plane count on one device."""

    def __init__(self, nnum, num_planes, device=0):
        self._lib = load_library()
        self._h = _P()
        rc = self._lib.flf_ctx_create(ctypes.byref(self._h), int(device), int(nnum), int(num_planes))
        if rc != FLF_OK:
            raise FlfError(rc, self._msg(None))
        self.nnum = int(nnum)
        self.num_planes = int(num_planes)
        self.device = int(device)

    def _msg(self, h):
        buf = ctypes.create_string_buffer(1024)
        self._lib.flf_last_error(h, buf, 1024)
        return buf.value.decode(errors="replace")

    def _check(self, rc):
        if rc != FLF_OK:
            if not (self._h and self._h.value):
                raise FlfError(rc, "the context was closed")
            raise FlfError(rc, self._msg(self._h))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.flf_ctx_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_psf(self, plane, direction, H):
        H = np.ascontiguousarray(H, dtype=np.float32)
        if H.ndim != 4 or H.shape[2] != H.shape[3]:
            raise ValueError("PSF array must be [n_h, n_h, h, h], got %s" % (H.shape,))
        self._check(self._lib.flf_psf_upload(self._h, int(plane), int(direction), H.ctypes.data,
                                             int(H.shape[0]), int(H.shape[2])))

    def prepare(self, Y, X, fft_size=0, fp64=False):
        self._check(self._lib.flf_prepare(self._h, int(Y), int(X), int(fft_size), int(bool(fp64))))

    @staticmethod
    def _planes_arg(planes, nz):
        if planes is None:
            return None, nz, None
        arr = np.ascontiguousarray(np.asarray(list(planes), dtype=np.int32))
        return arr.ctypes.data, int(arr.size), arr

    def forward(self, vol, img, T, Y, X, planes=None, stream=None):
        p, n, keep = self._planes_arg(planes, self.num_planes)
        self._check(self._lib.flf_forward(self._h, _ptr(vol), _ptr(img), int(T), int(Y), int(X),
                                          p, n, _ptr(stream)))
        del keep

    def backward(self, img, vol, T, Y, X, planes=None, stream=None):
        p, n, keep = self._planes_arg(planes, self.num_planes)
        self._check(self._lib.flf_backward(self._h, _ptr(img), _ptr(vol), int(T), int(Y), int(X),
                                           p, n, _ptr(stream)))
        del keep

    def backward_noalloc(self, img, vol, T, Y, X, stream=None):
        """Back projection over all planes that allocates no device memory.

        For callers that must not allocate while they run; its scratch is a
        fixed 16 MiB device array set up when the context was created.  The
        call only enqueues work: call ``synchronize`` (which raises on a
        bounded device wait that gave up) before using ``vol``.
        """
        self._check(self._lib.flf_backward_noalloc(self._h, _ptr(img), _ptr(vol), int(T), int(Y), int(X),
                                                   _ptr(stream)))

    def rl_iterate(self, x, ref, norm, variant, iters, T, Y, X, stream=None):
        self._check(self._lib.flf_rl_iterate(self._h, _ptr(x), _ptr(ref), _ptr(norm), int(variant),
                                             int(iters), int(T), int(Y), int(X), _ptr(stream)))

    def memory_usage(self):
        v = ctypes.c_size_t(0)
        self._check(self._lib.flf_memory_usage(self._h, ctypes.byref(v)))
        return int(v.value)

    def memory_epoch(self):
        """Bumped whenever the context frees a buffer: a graph captured around library
        calls stays valid while it is unchanged."""
        v = ctypes.c_ulonglong(0)
        self._check(self._lib.flf_memory_epoch(self._h, ctypes.byref(v)))
        return int(v.value)

    def clear_cache(self):
        self._check(self._lib.flf_clear_cache(self._h))

    def set_option(self, name, value):
        self._check(self._lib.flf_set_option(self._h, name.encode(), int(value)))

    def synchronize(self, stream=None):
        self._check(self._lib.flf_synchronize(self._h, _ptr(stream)))

    def profile(self, enable):
        self._check(self._lib.flf_profile(self._h, int(bool(enable))))

    def profile_read(self):
        """{kernel: {"launches", "ms", "bytes"}} since the last profile() call."""
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._lib.flf_profile_read(self._h, buf, 1 << 16))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms, b = line.split()
            out[name] = {"launches": int(n), "ms": float(ms), "bytes": float(b)}
        return out

    def rl_graph(self, x, ref, norm, variant, iters, T, Y, X):
        """RLGraph replaying `iters` RL iterations on these tensors (flf_rl_graph_create)."""
        h = _P()
        self._check(self._lib.flf_rl_graph_create(self._h, ctypes.byref(h), _ptr(x), _ptr(ref), _ptr(norm),
                                                  int(variant), int(iters), int(T), int(Y), int(X)))
        return RLGraph(self, h, (x, ref, norm))

    def deconv_graph(self, img, htf, x, iters, T, Y, X):
        """RLGraph of the whole deconvolution of T frames (flf_deconv_graph_create):
        Htf = back projection of img, x = Htf, then `iters` Prevedel iterations."""
        h = _P()
        self._check(self._lib.flf_deconv_graph_create(self._h, ctypes.byref(h), _ptr(img), _ptr(htf), _ptr(x),
                                                      int(iters), int(T), int(Y), int(X)))
        return RLGraph(self, h, (img, htf, x))

    def combine_graphs(self, graphs):
        """One RLGraph running `graphs` (of this context) in order (flf_graph_combine)."""
        arr = (_P * len(graphs))(*[g._h for g in graphs])
        h = _P()
        self._check(self._lib.flf_graph_combine(ctypes.byref(h), arr, len(graphs)))
        return RLGraph(self, h, tuple(graphs))

    def autotune(self, T, Y, X, stream=None):
        """Launch shape of the multiply-accumulate for T frames of Y x X images:
        {"stages", "chunk_rows_forward", "chunk_rows_backward", "split"}."""
        out = (ctypes.c_int * 4)()
        self._check(self._lib.flf_autotune(self._h, int(T), int(Y), int(X), out, _ptr(stream)))
        return dict(zip(TUNED_KEYS, list(out)))

    def set_tuned(self, Y, X, tuned):
        arr = (ctypes.c_int * 4)(*[int(tuned[k]) for k in TUNED_KEYS])
        self._check(self._lib.flf_set_tuned(self._h, int(Y), int(X), arr))

    def geometry(self):
        out = (ctypes.c_int * 4)()
        self._check(self._lib.flf_geometry(self._h, out))
        return {"f": out[0], "R": out[1], "fp64": bool(out[2]), "groups": out[3]}
