"""The multi-process path on CPU: two gloo ranks on 127.0.0.1 split a tomography batch
(every image once, costs balanced) and reduce a timed region's rate (slowest rank's
time, all ranks' images), as bench.py does under torchrun with one GPU per rank."""
import os
import socket

import numpy as np
import pytest

from simulated_tem_gb300 import replicas

torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def batch_costs():
    """Costs of a 41-tilt x 3-g sweep of a small cell (host geometry only)."""
    from simulated_tem_gb300 import imaging, synth
    cell = synth.small_cell((10, 10, 6), seed=5)
    costs = []
    for g in ((1, 1, 0), (2, 0, 0), (2, 1, 1)):
        for step in range(41):
            t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), g, cell.pos, sg=0.01,
                                             n_tomo=41, tomo_angle=20.0, tomo_step=step)
            G, aa = t.image_geometry(len(x), prec_angle=0.005, n_prec=16)
            costs.append(replicas.image_cost(G, len(aa)))
    return costs


def worker(rank, world, port, costs, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = replicas.shard(costs, rank, world)
        mine = float(np.sum(costs[lo:hi]))
        local_ms = 10.0 + 5.0 * rank  # a slower second rank
        rate, ms, images = replicas.job_rate(local_ms, hi - lo)
        out.put((rank, lo, hi, mine, rate, ms, images))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_and_reduce():
    import torch.multiprocessing as mp
    costs = batch_costs()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, lo0, hi0, c0, rate0, ms0, n0), (r1, lo1, hi1, c1, rate1, ms1, n1) = res
    assert (lo0, hi1) == (0, len(costs)) and hi0 == lo1  # every image exactly once
    assert abs(c0 - c1) <= max(costs)  # balanced to within one image
    assert ms0 == ms1 == 15.0 and n0 == n1 == len(costs)  # slowest rank, all images
    assert rate0 == rate1 == pytest.approx(1000.0 * len(costs) / 15.0)


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shard_covers_once(world):
    rng = np.random.default_rng(world)
    w = rng.uniform(1, 10, size=50)
    spans = [replicas.shard(w, r, world) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == 50
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    parts = [w[lo:hi].sum() for lo, hi in spans]
    assert max(parts) - min(parts) <= 2 * w.max()


def test_single_process_rate():
    rate, ms, n = replicas.job_rate(4.0, 2)
    assert rate == 500.0 and ms == 4.0 and n == 2
