"""Several GPUs: replicas only.  Images are independent (tomography tilts, g-vectors,
precession sets, cells), so N processes, one per GPU, each image their own share of a
batch and no data crosses between them during imaging; the only collectives are the
barrier before a timed region and the reductions of its timing (the slowest rank's time,
the images of all ranks).  The reference spreads one image's pixel patches over MPI ranks
and reduces the images (src/Lib_DynamicalTwoBeamImaging.f90:1714-1760, 1950); that split
stays available through st_geom's pixel window (ix0..iy1) but is not needed on GPUs that
hold whole images."""
import numpy as np


def shard(weights, rank, world):
    """Contiguous share of rank `rank` among `world` of a batch whose images cost
    `weights` (e.g. voxels x precession angles): ranges [lo, hi) with the cumulative cost
    split as evenly as contiguous ranges allow.  Deterministic: every rank computes the same
    split without communicating."""
    w = np.asarray(weights, dtype=np.float64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of %d" % (rank, world))
    if np.any(w < 0):
        raise ValueError("negative image cost")
    n = len(w)
    if n == 0:
        return 0, 0
    c = np.concatenate([[0.0], np.cumsum(w)])
    total = c[-1]
    # boundary k: the first image whose cumulative start reaches k / world of the total
    bounds = [0] + [int(np.searchsorted(c, total * k / world, side="left")) for k in range(1, world)] + [n]
    bounds = np.maximum.accumulate(np.clip(bounds, 0, n))
    return int(bounds[rank]), int(bounds[rank + 1])


def image_cost(geom, n_prec=1):
    """Relative cost of one image: voxels of its window times precession angles."""
    return float(max(geom.ix1 - geom.ix0, 0) * max(geom.iy1 - geom.iy0, 0) * geom.Mz * max(n_prec, 1))


def job_rate(local_ms, local_images, group=None):
    """Whole-job images/s of a timed region: the images of all ranks over the slowest
    rank's time (torch.distributed, any backend; a single process when not initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return 1000.0 * local_images / local_ms, local_ms, local_images
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=dev)
    n = torch.tensor([float(local_images)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    ms, images = float(t.item()), float(n.item())
    return 1000.0 * images / ms, ms, images
