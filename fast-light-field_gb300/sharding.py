"""Frame-sharded Richardson-Lucy deconvolution over several processes (one GPU each).

Time-series frames are independent (the reference processes a batch of frames
together only to share the PSF spectra, py_light_field.cpp:1299-1303), so
frames shard across ranks with no data exchange inside the projections: each
rank deconvolves its contiguous share of frames with its own projector and the
volumes are gathered along the frame axis at the end.  With one GPU per rank
this is "replicas": the PSF spectra are replicated on every GPU.
"""

import numpy as np

import lfdeconv

__all__ = ["frame_shard", "deconv_rl_sharded"]


def frame_shard(T, rank, world):
    """Contiguous share ``slice`` of ``T`` frames for ``rank`` of ``world`` (sizes differ by <= 1)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank %d out of range for world size %d" % (rank, world))
    base, extra = divmod(int(T), int(world))
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def _dist():
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist
    except ImportError:
        pass
    return None


def deconv_rl_sharded(hMatrix, im, maxIter, projector, prevedel=True, Xguess=None, group=None):
    """Deconvolve ``im [T, Y, X]`` with this rank's share of frames; every rank returns the full volume.

    Without an initialised ``torch.distributed`` process group this is plain
    ``lfdeconv.DeconvRL`` on all frames.
    """
    im = np.asarray(im, dtype=np.float32)
    dist = _dist()
    rank, world = (dist.get_rank(group), dist.get_world_size(group)) if dist else (0, 1)
    sl = frame_shard(im.shape[0], rank, world)
    x0 = None if Xguess is None else np.asarray(Xguess, np.float32)[:, sl]
    local = None
    if sl.stop > sl.start:
        local = lfdeconv.DeconvRL(hMatrix, None, maxIter, x0, logPrint=False, projector=projector,
                                  im=im[sl], prevedel=prevedel)
    if dist is None:
        return local
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    return np.concatenate([p for p in parts if p is not None], axis=1)
