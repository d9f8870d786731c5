"""Benchmark of the d2bi imaging hot path on GB300.

Workload: the 1.2M-atom bcc Fe cell (100 x 100 x 60 cells, screw dislocation
along z through the centre, 20 voids of radius U(5, 15) A, jitter 0.05 A,
seeded), g = [110], k = [001], s_g = 0.01 1/A, M = 4,4, 200 kV: a 566 x 566
image with 240 voxels per column.  One step = one image: link-cell binning
(findGdotR), voxel phase field and column integration, FP32 arithmetic with
FP64 cell assignment and FP64 g.r reduction.

  value  images/s with the atoms resident in HBM (st_image_device), each step
         timed with CUDA events on the launching stream, L2 flushed between
         steps (a 512 MB write), untimed.
  e2e    the same through st_image, the C-ABI call a Fortran or C host makes,
         from pinned host buffers: the H2D copy of the atoms and the D2H copy
         of the image are inside the timed region.
  also   the plain FP64 GPU path (images/s); accuracy of both paths against the
         oracle's whole image (max |dI| and RMS), and FP32 vs FP64.
  roofline  the path roofline of the reference's voxel loop (MUFU, FP32, FP64 and
         HBM work over the measured peaks; the bound is the largest), as a
         fraction of the column kernel's time, and of the whole step; the work
         the kernel executes beside it.
  batched  st_batch_device on (a) the tilt x precession x g sweep of the same
         cell (41 x 16 x 3: 123 images, 1,968 integration passes) and (b) 256
         independent cells of uneven size; images/s, voxel-slices/s, stage
         times of the timed calls, launches, the path roofline, and accuracy
         against the oracle (a row band of one image per g; the largest cell
         whole).  The clock record spans the single-image steps and every leg.

``--impl reference`` times the reference's algorithm on the host cores: the
reference (Fortran) cannot be built here, so the oracle's C restatement runs,
with all host threads, on whole images of the same workload, one per step.
Nothing of the product is imported or loaded in that process.

Under torchrun with N > 1 every rank images its own copy of the workload
(independent images: replicas, no collective on the data path); value is the
total images/s over all ranks.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "images/s at 1.2M atoms: batched FP32 vs plain FP64 GPU at ≤1e-4 max |ΔI|"
WORKLOAD = "bcc Fe 100x100x60 cells (1.2M atoms), screw + 20 voids, g=[110] k=[001] s_g=0.01, M=4,4, 200 kV"


def workload():
    from simulated_tem_gb300 import imaging, synth
    cell = synth.screw_cell_1p2m()
    t, x, aperpx = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.01,
                                          xi0=103.9, xig=207.5, V=200.0, M=(4, 4))
    return cell, t, x, aperpx


def standalone_synth():
    """The seeded cell generator (simulated_tem_gb300/synth.py, numpy only) loaded by its file
    path, without the package: the reference arm must not import or load any product code."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_bench_synth", os.path.join(ROOT, "simulated_tem_gb300",
                                                                               "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def oracle_workload_setup(cell, A0):
    """The oracle's set-up of the 1.2M-atom image (wrapped atoms, geometry, precession)."""
    from oracle import stem_oracle as O
    args = O.make_args(cell.a_super, A0, (0, 0, 1), (1, 1, 0), sg=0.01, xi0=103.9, xig=207.5)
    so, xo, _ = O.setup(args, cell.pos)
    G, aa = O.geometry(so, len(xo))
    return G, aa, xo


def oracle_workload_image(state, threads):
    """The 1.2M-atom image computed whole by the oracle (the C restatement of computeD2BI_img,
    binning included) on `threads` host threads; (image (Mx, My), seconds, stats)."""
    from oracle import stem_oracle as O
    G, aa, xo = state
    t0 = time.perf_counter()
    img, st = O.patch_image(G, aa, xo, nthreads=threads)
    return img, time.perf_counter() - t0, st


def hbm_peak():
    """The measured copy bandwidth of the GB300s (GB/s), else the fallback figure."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback 6.8 TB/s"


# Path roofline of the imaging step (the algorithmic work of the reference's voxel loop,
# counted from the oracle's and the kernel's identical accept counts):
#   MUFU   3 per accepted pair (exp, sin, cos of Lib_DynamicalTwoBeamImaging.f90:1877-1892)
#          + 1 per voxel (the normalisation's rsqrt)
#   FP32   12 per accepted pair + 6 per voxel (normalisation) + 10 per voxel (density, with
#          -density) + 90 per voxel and precession angle (the RK4 double step, :2389-2464)
#   FP64   30 per kept atom (findGdotR's transform, g.r and its reduction)
#   HBM    24 B per atom + 16 B per kept atom + 8 B per pixel
# T_roof = max over the four resources of (work / measured peak); frac = T_roof / time.
def path_roofline(peaks, n_acc, n_kept, n_atoms, voxels, voxel_prec, pixels, density, t_ms):
    if not peaks:
        return None
    hbm_gbs, _ = hbm_peak()
    ex2, sin = peaks["mufu_ex2_gops"] * 1e9, peaks["mufu_sin_gops"] * 1e9
    t_mufu = (n_acc + voxels) / ex2 + 2.0 * n_acc / sin
    w_fp32 = 12.0 * n_acc + (16.0 if density else 6.0) * voxels + 90.0 * voxel_prec
    t_fp32 = w_fp32 / (peaks["fp32_tflops"] * 1e12)
    t_fp64 = 30.0 * n_kept / (peaks["fp64_tflops"] * 1e12)
    w_hbm = 24.0 * n_atoms + 16.0 * n_kept + 8.0 * pixels
    t_hbm = w_hbm / (hbm_gbs * 1e9)
    res = {"mufu": t_mufu, "fp32": t_fp32, "fp64": t_fp64, "hbm": t_hbm}
    bound = max(res, key=res.get)
    t_roof = res[bound]
    t = t_ms * 1e-3
    if bound == "mufu":
        w, peak, unit = t_mufu * ex2, ex2, "Gop/s (MUFU, ex2-equivalent: sin and cos weighted by the ex2/sin rates)"
        scale = 1e9
    elif bound == "fp32":
        w, peak, unit, scale = w_fp32, peaks["fp32_tflops"] * 1e12, "TFLOP/s", 1e12
    elif bound == "fp64":
        w, peak, unit, scale = 30.0 * n_kept, peaks["fp64_tflops"] * 1e12, "TFLOP/s", 1e12
    else:
        w, peak, unit, scale = w_hbm, hbm_gbs * 1e9, "GB/s", 1e9
    return {"bound": bound, "achieved": w / t / scale, "peak": peak / scale, "unit": unit, "frac": t_roof / t,
            "t_roof_ms": t_roof * 1e3, "t_ms": t_ms,
            "per_resource_ms": {k: v * 1e3 for k, v in res.items()},
            "work": {"accepted_pairs": n_acc, "kept_atoms": n_kept, "atoms": n_atoms, "voxels": voxels,
                     "voxel_precession_passes": voxel_prec, "pixels": pixels, "density": bool(density),
                     "mufu_ops": 3.0 * n_acc + voxels, "fp32_flop": w_fp32, "fp64_flop": 30.0 * n_kept,
                     "hbm_bytes": w_hbm}}


SWEEP_G = ((1, 1, 0), (2, 0, 0), (2, 1, 1))
# DRAM bytes (read + write) of one k_column_fp32_v3 launch on the 1.2M-atom image, from an
# ncu capture of `python bench.py --ncu-case fp32` (51.59 MB read + 2.36 MB written)
COLUMN_TRAFFIC_BYTES = 5.395e7


def sweep_specs(cell, n_tomo=41, n_prec=16, gs=SWEEP_G):
    """Tilt series x precession x g on the 1.2M-atom cell: nTomoAngle = 41 tilts over
    +-20 deg, 16 precession angles at 5 mrad, g in {110, 200, 211}.  Returns the
    wrapped positions (shared by every image) and one (geometry, aa) per output image."""
    from simulated_tem_gb300 import imaging, synth
    x0, specs = None, []
    for g in gs:
        for step in range(n_tomo):
            t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), g, cell.pos, sg=0.01,
                                             xi0=103.9, xig=207.5, V=200.0, M=(4, 4), n_tomo=n_tomo,
                                             tomo_angle=20.0, tomo_step=step)
            if x0 is None:
                x0 = x
            elif step == 0 and not np.array_equal(x, x0):
                raise RuntimeError("the sweep's conditions wrap the atoms differently")
            G, aa = t.image_geometry(len(x0), prec_angle=0.005, n_prec=n_prec)
            specs.append((G, aa))
    return x0, specs


def uneven_specs(cells=None):
    """256 independent bcc Fe cells, atom counts log-uniform in [10k, 500k] before voids,
    aspect ratios U(0.5, 2), Poisson(10) voids of radius U(4, 20) A, s_g ~ U(-0.02, 0.02)."""
    from simulated_tem_gb300 import imaging, synth
    out = []
    for cell, sg in (cells if cells is not None else synth.uneven_cells()):
        t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=sg,
                                         xi0=103.9, xig=207.5, V=200.0, M=(4, 4))
        G, aa = t.image_geometry(len(x))
        out.append((G, aa, x))
    return out


def time_batch(ctx, jobs, flags, stream, steps, warmup, flush):
    """CUDA-event time of st_batch_device over `jobs`, L2 flushed before each call; also the
    library's own per-call stage times (binning, columns) of the same timed calls."""
    import torch
    sptr = stream.cuda_stream
    for _ in range(warmup):
        ctx.batch_device(jobs, flags, sptr)
    ms, bins, cols = [], [], []
    for i in range(steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.batch_device(jobs, flags, sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        st = ctx.stats()
        bins.append(st.ms_bin)
        cols.append(st.ms_column)
    time_batch.stages = {"ms_bin": float(np.mean(bins)), "ms_column": float(np.mean(cols)),
                         "note": "mean over the timed calls of the library's CUDA events around the binning "
                                 "(with the image clears) and the column phase (column kernels and epilogues)"}
    return ms


def time_plan(ctx, jobs, flags, stream, steps, warmup, flush):
    """CUDA-event time of st_plan_launch + st_plan_wait (a recorded batch replayed), L2
    flushed before each replay."""
    import torch
    sptr = stream.cuda_stream
    plan = ctx.plan(jobs, flags, sptr)
    ms = []
    try:
        for i in range(warmup + steps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.launch(sptr)
            e1.record(stream)
            plan.wait(sptr)
            if i >= warmup:
                ms.append(e0.elapsed_time(e1))
    finally:
        plan.close()
    return ms


def oracle_band(cell, g, sg, n_prec, rows=None, n_tomo=1, step=0, threads=None):
    """The oracle's image of one condition (the precession average), whole or on a band of
    pixel rows, on all host threads: the checker of the batched legs."""
    from oracle import stem_oracle as O
    from simulated_tem_gb300 import synth
    args = O.make_args(cell.a_super, synth.A0_FE, (0, 0, 1), g, sg=sg, xi0=103.9, xig=207.5, nTomo=n_tomo,
                       tomoAngle=20.0)
    so, xo, _ = O.setup(args, cell.pos, nn=step)
    Go, aao = O.geometry(so, len(xo), nPrec=n_prec, precAngle=0.005)
    img, _ = O.patch_image(Go, aao, xo, rows=rows, nthreads=threads or os.cpu_count() or 1)
    return img / n_prec


def vs_oracle(got, want, rows=None):
    sl = slice(None) if rows is None else slice(rows[0], rows[1])
    d = got[:, sl] - want[:, sl]
    return {"max_abs_dI": float(np.abs(d).max()), "rms_dI": float(np.sqrt((d ** 2).mean())),
            "pixels": int(d.size), "reference": "oracle (FP64 C restatement of computeD2BI_img)"}


def batched_legs(ctx, cell, stream, flush, steps, warmup, peaks=None, cpu=True):
    """The two batched workloads through st_batch_device: the tilt x precession x g sweep on
    the 1.2M-atom cell and the 256-cell uneven batch, FP32 path.  Accuracy against the oracle:
    a band of pixel rows of one mid-series image of each g, and the largest uneven cell whole
    (without host cores for the oracle: against the plain FP64 GPU path)."""
    import torch

    from simulated_tem_gb300 import _lib
    out = {}
    f32 = _lib.ST_FLAG_FP32 | _lib.ST_FLAG_AVERAGE

    def fp64_gpu(G, x_ptr, n, aa):
        ref = torch.empty((G.My, G.Mx), dtype=torch.float64, device="cuda")
        ctx.image_device(G, x_ptr, n, aa, _lib.ST_FLAG_AVERAGE, ref.data_ptr(), stream=stream.cuda_stream)
        torch.cuda.synchronize()
        return ref.cpu().numpy().T

    def roof(st, specs_g, t_col, t_batch, n_atoms):
        vox = sum((G.ix1 - G.ix0) * (G.iy1 - G.iy0) * G.Mz for G in specs_g[0])
        vp = sum((G.ix1 - G.ix0) * (G.iy1 - G.iy0) * G.Mz * n for G, n in zip(*specs_g))
        pix = sum((G.ix1 - G.ix0) * (G.iy1 - G.iy0) for G in specs_g[0])
        r = path_roofline(peaks, st.n_accepted, st.n_kept, n_atoms, vox, vp, pix, False, t_col)
        if r:
            r["kernel"] = "k_column_fp32_v3 (every column launch of the batch)"
            r["frac_batch"] = r["t_roof_ms"] / t_batch
            r["executed"] = {"tests": st.n_tests, "tests_per_voxel": st.n_tests / max(vox, 1)}
        return r

    # tilt x precession x g sweep: set up on the host condition by condition (the atoms
    # wrapped and their extents taken for every image), and on the GPU (wrapped once, the
    # extents of the three g in one pass); the two give the same geometry bit for bit
    from simulated_tem_gb300 import imaging, synth
    t0 = time.perf_counter()
    x, specs_host = sweep_specs(cell)
    setup_host = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d_x, specs, _ = imaging.d2bi_sweep(ctx, cell.a_super, synth.A0_FE, (0, 0, 1), SWEEP_G, cell.pos, n_tomo=41,
                                       tomo_angle=20.0, prec_angle=0.005, n_prec=16, sg=0.01, xi0=103.9, xig=207.5)
    torch.cuda.synchronize()
    setup_dev = time.perf_counter() - t0
    same = all(bytes(a[0]) == bytes(b[0]) and np.array_equal(a[1], b[1]) for a, b in zip(specs, specs_host))
    same = same and bool(np.array_equal(d_x.cpu().numpy(), x))
    imgs = [torch.empty((G.My, G.Mx), dtype=torch.float64, device="cuda") for G, _ in specs]
    jobs = [(G, d_x.data_ptr(), len(x), aa, im.data_ptr()) for (G, aa), im in zip(specs, imgs)]
    time_batch(ctx, jobs, f32 | _lib.ST_FLAG_STATS, stream, 1, 0, flush)  # counts for the roofline
    st = ctx.stats()
    ms = time_batch(ctx, jobs, f32, stream, steps, warmup, flush)
    stages = dict(time_batch.stages)
    launches = ctx.stats().n_launches
    variant = _lib.lib().st_tune_variant_name(ctx.stats().ring_variant).decode()
    slab_atoms = ctx.stats().ring_slab_atoms  # 192 or 256: the larger staging tiers ran
    t = float(np.mean(ms)) * 1e-3
    n_img, n_pass = len(specs), sum(len(aa) for _, aa in specs)
    vs = sum((G.ix1 - G.ix0) * (G.iy1 - G.iy0) * G.Mz * len(aa) for G, aa in specs)
    # one mid-series tilt of each g against the oracle (a band of rows; FP32 bar 1e-4)
    acc = {}
    for gi, g in enumerate(SWEEP_G):
        k = gi * 41 + 20
        G, aa = specs[k]
        got = imgs[k].cpu().numpy().T
        if cpu:
            mid = (G.iy0 + G.iy1) // 2
            rows = (mid - 8, mid + 8)
            want = oracle_band(cell, g, 0.01, 16, rows=rows, n_tomo=41, step=20)
            acc["g%d%d%d" % g] = vs_oracle(got, want, rows)
        else:
            acc["g%d%d%d" % g] = vs_oracle(got, fp64_gpu(G, d_x.data_ptr(), len(x), aa))
            acc["g%d%d%d" % g]["reference"] = "plain FP64 GPU path"
    out["sweep"] = {"workload": "1.2M-atom cell: 41 tilts over +-20 deg x 16 precession angles (5 mrad) x "
                                "g in {110, 200, 211}, FP32, images averaged over precession",
                    "images": n_img, "integration_passes": n_pass, "images_per_s": n_img / t,
                    "passes_per_s": n_pass / t, "voxel_slices_per_s": vs / t, "ms_per_batch": t * 1e3,
                    "steps": steps, "image_sizes": sorted({(G_.Mx, G_.My, G_.Mz) for G_, _ in specs}),
                    "kept_atoms": st.n_kept, "column_kernel": st.column_kernel, "stages": stages,
                    "launches_per_batch": launches, "ring_variant": variant, "ring_slab_atoms": slab_atoms,
                    "roofline": roof(st, ([G_ for G_, _ in specs], [len(aa_) for _, aa_ in specs]),
                                     stages["ms_column"], t * 1e3, len(x) * n_img),
                    "accuracy_tilt20_per_g": acc,
                    "setup": {"host_s": setup_host, "device_s": setup_dev, "same_geometry": same,
                              "images_per_s_with_device_setup": n_img / (t + setup_dev),
                              "note": "set-up of the 123 geometries: host (wrap and extents per image) vs "
                                      "d2bi_sweep (one wrap and one extents pass on the GPU)"}}
    pms = time_plan(ctx, jobs, f32, stream, steps, 1, flush)
    tp = float(np.mean(pms)) * 1e-3
    out["sweep"]["plan"] = {"note": "the same batch recorded once as a CUDA graph (st_plan) and replayed",
                            "ms_per_batch": tp * 1e3, "images_per_s": n_img / tp, "passes_per_s": n_pass / tp}
    del imgs, jobs

    # 256 independent cells of uneven size
    cells = synth.uneven_cells()
    specs = uneven_specs(cells)
    d_xs = [torch.from_numpy(np.ascontiguousarray(x_)).cuda() for _, _, x_ in specs]
    imgs = [torch.empty((G.My, G.Mx), dtype=torch.float64, device="cuda") for G, _, _ in specs]
    jobs = [(G, dx.data_ptr(), len(x_), aa, im.data_ptr()) for (G, aa, x_), dx, im in zip(specs, d_xs, imgs)]
    time_batch(ctx, jobs, f32 | _lib.ST_FLAG_STATS, stream, 1, 0, flush)
    st = ctx.stats()
    ms = time_batch(ctx, jobs, f32, stream, steps, warmup, flush)
    stages = dict(time_batch.stages)
    launches = ctx.stats().n_launches
    variant = _lib.lib().st_tune_variant_name(ctx.stats().ring_variant).decode()
    slab_atoms = ctx.stats().ring_slab_atoms  # 192 or 256: the larger staging tiers ran
    t = float(np.mean(ms)) * 1e-3
    vs = sum((G.ix1 - G.ix0) * (G.iy1 - G.iy0) * G.Mz for G, _, _ in specs)
    k = int(np.argmax([len(x_) for _, _, x_ in specs]))
    G, aa, x_ = specs[k]
    got = imgs[k].cpu().numpy().T
    if cpu:
        cell_k, sg_k = cells[k]
        acc = vs_oracle(got, oracle_band(cell_k, (1, 1, 0), sg_k, 1))
    else:
        acc = vs_oracle(got, fp64_gpu(G, d_xs[k].data_ptr(), len(x_), aa))
        acc["reference"] = "plain FP64 GPU path"
    out["uneven"] = {"workload": "256 bcc Fe cells, atoms log-uniform in [10k, 500k] before voids, aspect U(0.5, 2), "
                                 "Poisson(10) voids of radius U(4, 20) A, s_g U(-0.02, 0.02), FP32",
                     "images": len(specs), "atoms": int(sum(len(x_) for _, _, x_ in specs)),
                     "images_per_s": len(specs) / t, "voxel_slices_per_s": vs / t, "ms_per_batch": t * 1e3,
                     "steps": steps, "kept_atoms": st.n_kept, "column_kernel": st.column_kernel, "stages": stages,
                     "launches_per_batch": launches, "ring_variant": variant, "ring_slab_atoms": slab_atoms,
                     "roofline": roof(st, ([G_ for G_, _, _ in specs], [1] * len(specs)), stages["ms_column"],
                                      t * 1e3, sum(len(x_) for _, _, x_ in specs)),
                     "accuracy_largest_cell": acc}
    return out


def cfg1_leg(ctx, stream, flush, steps, warmup, cpu=True):
    """The 128k-atom void cell (40^3 bcc cells, 8 voids of 10 A), g = 110, s_g = 0, -density,
    M = 4,4: one dark-field image, the bright field 1 - DF, and both blurred at 2.5 A, on the
    plain FP64 path and on the FP32 path; the oracle times the same on the host cores."""
    import torch

    from simulated_tem_gb300 import _lib, imaging, synth
    cell = synth.void_cell_128k()
    t, x, aperpx = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), cell.pos, sg=0.0,
                                          xi0=103.9, xig=207.5, V=200.0, M=(4, 4), density=True)
    G, aa = t.image_geometry(len(x))
    tpx = 2.5 / aperpx
    sp = stream.cuda_stream
    d_x = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    df, bf, dfb, bfb = (torch.empty((G.My, G.Mx), dtype=torch.float64, device="cuda") for _ in range(4))

    def step(flags):
        ctx.image_device(G, d_x.data_ptr(), len(x), aa, flags | _lib.ST_FLAG_AVERAGE, df.data_ptr(), stream=sp)
        torch.neg(df, out=bf)
        bf.add_(1.0)
        ctx.blur_device(df.data_ptr(), G.Mx, G.My, tpx, dfb.data_ptr(), stream=sp)
        ctx.blur_device(bf.data_ptr(), G.Mx, G.My, tpx, bfb.data_ptr(), stream=sp)

    out = {"workload": "bcc Fe 40^3 cells (%d atoms), 8 voids of 10 A, g=[110] k=[001] s_g=0, -density, M=4,4, "
                       "DF + BF, blur 2.5 A (%.3f px)" % (len(x), tpx), "image": [G.Mx, G.My, G.Mz]}
    imgs = {}
    for name, flags in (("gpu_fp64", 0), ("gpu_fp32", _lib.ST_FLAG_FP32)):
        for _ in range(warmup):
            step(flags)
        ms = []
        for i in range(steps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(flags)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        out[name] = {"images_per_s": 1000.0 / float(np.mean(ms)), "ms": float(np.mean(ms)),
                     "note": "one DF + BF pair with both blurs per image"}
        imgs[name] = df.cpu().numpy().T.copy()
    d = imgs["gpu_fp32"] - imgs["gpu_fp64"]
    out["accuracy_fp32_vs_fp64"] = {"max_abs_dI": float(np.abs(d).max()), "rms_dI": float(np.sqrt((d ** 2).mean()))}
    if cpu:
        from oracle import stem_oracle as O
        threads = os.cpu_count() or 1
        args = O.make_args(cell.a_super, synth.A0_FE, (0, 0, 1), (1, 1, 0), sg=0.0, xi0=103.9, xig=207.5,
                           density=True)
        so, xo, _ = O.setup(args, cell.pos)
        Go, aao = O.geometry(so, len(xo))
        t0 = time.perf_counter()
        img, _ = O.patch_image(Go, aao, xo, nthreads=threads)
        O.gaussian_blur(img, tpx)
        O.gaussian_blur(1.0 - img, tpx)
        tc = time.perf_counter() - t0
        dd = imgs["gpu_fp64"] - img
        out["cpu_oracle"] = {"images_per_s": 1.0 / tc, "s": tc, "cores": threads, "kind": "port",
                             "note": "oracle C restatement, whole image + both blurs"}
        out["accuracy_gpu_fp64_vs_oracle"] = {"max_abs_dI": float(np.abs(dd).max())}
    return out


CORRECTOR_WEIGHTS = os.path.join(ROOT, "simulated_tem_gb300", "weights", "corrector_m2_m8.npz")


def cfg5_leg(ctx, stream, flush, steps, warmup, weights=CORRECTOR_WEIGHTS):
    """The learned corrector on the 4.8M-atom cell (200 x 200 x 60 bcc cells, screw
    dislocation, 20 voids of radius U(5, 15) A), s_g = 0.01: the plain M = 8 FP32 solve against
    the M = 2 FP32 solve + corrector + fallback (the fine solve on the flagged tiles), both
    timed with CUDA events; the M = 8 solve judges the corrected image."""
    import torch

    from simulated_tem_gb300 import _lib, corrector as C, synth
    if not os.path.exists(weights):
        return {"unavailable": "no trained corrector weights at %s" % os.path.relpath(weights, ROOT)}
    model = C.UNet().load(weights)
    tau = float(model.meta["tau"])
    cell = synth.make_cell(200, 200, 60, synth.BASE_SEED + 5, n_voids=20, void_radius=(5.0, 15.0), with_screw=True,
                           name="bcc Fe 200x200x60, screw + 20 voids")
    sg = 0.01
    t2, x = C.condition(cell, 2, sg)
    t8, _ = C.condition(cell, 8, sg)
    G8, aa8 = t8.image_geometry(len(x))
    d_x = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    sp = stream.cuda_stream
    fine = torch.empty((G8.My, G8.Mx), dtype=torch.float64, device="cuda")
    imager = C.CorrectedImager(model, ctx, tile=16, tau=tau)

    def fine_step():
        ctx.image_device(G8, d_x.data_ptr(), len(x), aa8, _lib.ST_FLAG_FP32, fine.data_ptr(), stream=sp)

    res = {}

    def corrected_step():
        res["img"], res["nflag"], res["ntiles"] = imager.image(t2, t8, d_x, len(x), sg, stream=sp)

    def timed(fn):
        for _ in range(warmup):
            fn()
        ms = []
        for i in range(steps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.mean(ms))

    ms_fine = timed(fine_step)
    ms_corr = timed(corrected_step)
    stages = {}  # per-stage GPU time of the same call, untimed passes after the timed ones
    for i in range(steps):
        flush.fill_(float(i))
        imager.image(t2, t8, d_x, len(x), sg, stream=sp, times=stages)
    stages = {k: v / steps for k, v in stages.items()}
    ref = fine.cpu().numpy()
    got = res["img"].cpu().numpy()
    # the M = 2 image alone, interpolated (the method without the corrector)
    diag = {}
    plain, _, _ = C.CorrectedImager(model, ctx, tile=16, tau=np.inf).image(t2, t8, d_x, len(x), sg, fallback=False,
                                                                          diag=diag)
    G2, aa2 = t2.image_geometry(len(x))
    img2 = torch.empty((G2.My, G2.Mx), dtype=torch.float64, device="cuda")
    ctx.image_device(G2, d_x.data_ptr(), len(x), aa2, _lib.ST_FLAG_FP32, img2.data_ptr(), stream=sp)
    base = C.coarse_planes(img2, G2, G8, sg)[4, :G8.My, :G8.Mx].cpu().numpy()
    d_c, d_n, d_u = got - ref, plain.cpu().numpy() - ref, base - ref
    return {"workload": "bcc Fe 200x200x60 cells (%d atoms), screw + 20 voids, g=[110] s_g=0.01; M=8 image %dx%dx%d"
                        % (len(x), G8.Mx, G8.My, G8.Mz),
            "m8_fp32": {"images_per_s": 1000.0 / ms_fine, "ms": ms_fine},
            "m2_corrector_fallback": {"images_per_s": 1000.0 / ms_corr, "ms": ms_corr,
                                      "fallback_tiles": res["nflag"], "tiles": res["ntiles"],
                                      "fallback_fraction": res["nflag"] / res["ntiles"], "tau": tau,
                                      "max_abs_dI_vs_m8": float(np.abs(d_c).max()),
                                      "rms_dI_vs_m8": float(np.sqrt((d_c ** 2).mean())),
                                      "stages_ms": stages},
            "m2_corrector_no_fallback": {"max_abs_dI_vs_m8": float(np.abs(d_n).max()),
                                         "rms_dI_vs_m8": float(np.sqrt((d_n ** 2).mean()))},
            "m2_interpolated": {"max_abs_dI_vs_m8": float(np.abs(d_u).max()),
                                "rms_dI_vs_m8": float(np.sqrt((d_u ** 2).mean()))},
            "speedup": ms_fine / ms_corr}


def io_leg(ctx, stream, flush, steps, warmup, cpu=True):
    """d2bi's output files at the M = 8 image size of the 4.8M-atom cell (2263 x 2263,
    synthetic intensities in [0, 0.3)): the '(1000f12.7)' records of the .dat file and the
    16-bit PNG levels on the GPU (device-resident image, CUDA events), the whole
    st_write_dat / st_write_png calls (host image to file), and the oracle's C formatter
    and levels on one host core for the same image."""
    import tempfile

    import torch

    from simulated_tem_gb300 import imaging
    nx = ny = 2263
    n = nx * ny
    rng = np.random.default_rng(20261203 + 7)
    img = np.asfortranarray(rng.random((nx, ny)) * 0.3)
    d_img = torch.from_numpy(img.T.copy()).cuda()
    cap = imaging.lib().st_dat_text_bytes(n)
    d_text = torch.empty(cap, dtype=torch.uint8, device="cuda")
    d_lv = torch.empty(n, dtype=torch.int16, device="cuda")
    sp = stream.cuda_stream

    def timed(fn):
        for _ in range(warmup):
            fn()
        ms = []
        for i in range(steps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    ms_dat = timed(lambda: ctx.format_dat_device(d_img.data_ptr(), n, d_text.data_ptr(), cap, stream=sp))
    ms_png = timed(lambda: ctx.png_levels_device(d_img.data_ptr(), nx, ny, d_lv.data_ptr(), stream=sp))
    hdr = dict(modg=3.97017, sg=0.01, xmax=(811.9, 811.9, 172.2), aperpx=0.3588)
    with tempfile.TemporaryDirectory() as tmp:
        walls = {}
        for name, fn in (("write_dat", lambda: ctx.write_dat(os.path.join(tmp, "i.dat"), hdr, img)),
                         ("write_png", lambda: ctx.write_png(os.path.join(tmp, "i.png"), img, blur_t=6.97))):
            fn()
            t0 = time.perf_counter()
            for _ in range(3):
                fn()
            walls[name] = (time.perf_counter() - t0) / 3 * 1e3
    out = {"workload": "%d x %d image, synthetic intensities in [0, 0.3)" % (nx, ny),
           "dat_records_gpu": {"ms": ms_dat, "MB_per_s": cap / ms_dat / 1e3, "bytes": int(cap)},
           "png_levels_gpu": {"ms": ms_png, "Mpixel_per_s": n / ms_png / 1e3},
           "write_dat_file_ms": walls["write_dat"], "write_png_file_ms": walls["write_png"],
           "note": "write_*_file: host image to file through st_write_dat / st_write_png (the PNG blurred "
                   "at 6.97 px = 2.5 A first); GPU legs device-resident, CUDA events, L2 flushed"}
    if cpu:
        from oracle import stem_oracle as O
        t0 = time.perf_counter()
        O.format_f12_7(img.T.ravel())
        t_dat = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.png_levels(img)
        t_png = time.perf_counter() - t0
        out["cpu_oracle"] = {"dat_records_ms": t_dat * 1e3, "png_levels_ms": t_png * 1e3, "cores": 1,
                             "kind": "port", "note": "oracle C restatement (snprintf per value), one core"}
    return out


def input_leg(ctx, cell, stream, steps, warmup, cpu=True):
    """Reading the 1.2M-atom cell from a LAMMPS data file (written here with shortest
    round-trip coordinates, the layout of LAMMPS' write_data): st_read_lammps end to end
    (file to host positions: read, copy, GPU parse, copy back), the GPU parse alone on the
    resident text (CUDA events), and the oracle's reader (fgets + sscanf, one core)."""
    import tempfile

    import torch

    from simulated_tem_gb300 import imaging, synth
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "cell.lammps")
        synth.write_lammps(path, cell.pos, np.diag(cell.a_super))
        info = imaging.lammps_header(path)
        nb = info.file_bytes - info.data_offset
        walls = []
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            x, _, _ = ctx.read_lammps(path, info)
            if i >= warmup:
                walls.append(time.perf_counter() - t0)
        exact = bool(np.array_equal(x, cell.pos))
        with open(path, "rb") as f:
            f.seek(info.data_offset)
            text = np.frombuffer(f.read(), dtype=np.uint8)
        d_t = torch.from_numpy(text.copy()).cuda()
        d_x = torch.empty((info.n_atoms, 3), dtype=torch.float64, device="cuda")
        sp = stream.cuda_stream
        ms = []
        for i in range(warmup + steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.parse_atoms_device(d_t.data_ptr(), nb, info.n_atoms, d_x.data_ptr(), stream=sp)
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= warmup:
                ms.append(e0.elapsed_time(e1))
        out = {"workload": "LAMMPS data file of the 1.2M-atom cell (%d atoms, %.1f MB of atom lines)"
                           % (info.n_atoms, nb / 1e6),
               "read_file_ms": float(np.median(walls)) * 1e3, "positions_exact": exact,
               "gpu_parse_ms": float(np.median(ms)), "gpu_parse_GB_per_s": nb / float(np.median(ms)) / 1e6,
               "note": "read_file: st_read_lammps, file in the page cache; gpu_parse: text resident in HBM"}
        if cpu:
            from oracle import stem_oracle as O
            t0 = time.perf_counter()
            O.read_lammps_atoms(path, info.data_offset, info.n_atoms)
            out["cpu_oracle"] = {"ms": (time.perf_counter() - t0) * 1e3, "cores": 1, "kind": "port",
                                 "note": "oracle reader: fgets + sscanf per atom line, one core"}
        # the same cell as an extended .xyz file (species, x, y, z; Lattice= on line 2)
        xpath = os.path.join(tmp, "cell.xyz")
        synth.write_xyz(xpath, cell.pos, cell.a_super)
        xi = imaging.xyz_header(xpath)
        xnb = xi.file_bytes - xi.data_offset
        walls = []
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            xx, _, species, _ = ctx.read_xyz(xpath, xi)
            if i >= warmup:
                walls.append(time.perf_counter() - t0)
        with open(xpath, "rb") as f:
            f.seek(xi.data_offset)
            xtext = np.frombuffer(f.read(), dtype=np.uint8)
        d_t = torch.from_numpy(xtext.copy()).cuda()
        d_x3 = torch.empty((xi.n_read, 3), dtype=torch.float64, device="cuda")
        d_ty = torch.empty(xi.n_read, dtype=torch.int32, device="cuda")
        ms = []
        for i in range(warmup + steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.parse_xyz_device(d_t.data_ptr(), xnb, xi.n_read, xi.n_columns, d_x3.data_ptr(), 3, d_ty.data_ptr(),
                                 stream=sp)
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= warmup:
                ms.append(e0.elapsed_time(e1))
        out["xyz"] = {"workload": "extended .xyz file of the same cell (%d atoms, %.1f MB of atom lines)"
                                  % (xi.n_read, xnb / 1e6),
                      "read_file_ms": float(np.median(walls)) * 1e3,
                      "positions_exact": bool(np.array_equal(xx[:, :3], cell.pos)), "species": species,
                      "gpu_parse_ms": float(np.median(ms)), "gpu_parse_GB_per_s": xnb / float(np.median(ms)) / 1e6,
                      "note": "read_file: st_read_xyz (header on the host, atom lines and species on the GPU); "
                              "gpu_parse: st_parse_xyz_device on text resident in HBM, species numbering included"}
        if cpu:
            t0 = time.perf_counter()
            O.read_xyz_atoms(xpath, O.xyz_header(xpath))
            out["xyz"]["cpu_oracle"] = {"ms": (time.perf_counter() - t0) * 1e3, "cores": 1, "kind": "port",
                                        "note": "oracle input0: fgets + strtod per atom line, one core"}
    return out


def tilt_leg(ctx, cell, steps, warmup, cpu=True):
    """The -ng tilt search (setSupercellTilt1a): the testD2BI search itself (27,847 W atoms,
    -k 0,0,1 -g 2,0,0 -ng 1 with its extinction table: 4,000 candidate beam directions x
    2,123 bcc reflections) end to end on the host API with the scores on the GPU, the
    scoring launch alone (CUDA events), and the oracle's scalar search on one core; then
    the same search with the foil thickness from the atoms (-surf) on the 1.2M-atom cell
    (the W table reused: a timing workload for the pass over 27 replicas of every atom)."""
    import torch

    from simulated_tem_gb300 import imaging
    here = os.path.dirname(os.path.abspath(__file__))
    xifile = os.path.join(here, "tests", "golden", "w_xi_V200_T300.dat")
    w = np.load(os.path.join(here, "tests", "golden", "w_loop_input.npz"))
    box = w["box"]
    a_super = np.diag(box[:, 1] - box[:, 0])

    def one(a_sup, a0, g, pos):
        a0 = (a0 + a0 + a0) / 3  # as d2bi forms a0 from -a0 (src/d2bi.f90:787-788)
        xw, a_vox, n = imaging.wrap_pbc(a_sup, (4, 4), a0, pos)
        d = imaging.atom_extents((0, 0, 1), g, a0 * np.eye(3), xw)
        t = imaging.DynamicalTwoBeamImaging(a_vox, n, a0, (0, 0, 1), g, 200.0, 4, 4)
        t.set_conventional_unit_cell(a0 * np.eye(3))
        t.set_voxel_supercell_size(d)
        return t, xw

    t, xw = one(a_super, 3.1652, (2, 0, 0), w["pos"])
    walls, scans = [], []
    for i in range(warmup + steps):
        t, _ = one(a_super, 3.1652, (2, 0, 0), w["pos"])
        t0 = time.perf_counter()
        info = t.set_supercell_tilt_ng(ctx, 1.0, xifile)
        if i >= warmup:
            walls.append(time.perf_counter() - t0)
            scans.append(info["scan_ms"])
    U, R = t.get_rotation()
    pairs = info["nk"] * (info["nn"] - 2)
    scan = float(np.median(scans))
    out = {"workload": "testD2BI -ng 1 search: 27,847 W atoms, k [001], g [200], %d directions x %d reflections"
                       % (info["nk"], info["nn"]),
           "setup_ms": float(np.median(walls)) * 1e3, "scan_ms": scan, "pairs_per_s": pairs / (scan * 1e-3),
           "screen_ms": info["screen_ms"], "n_fp64": info["n_fp64"],
           "n_recheck": info["n_recheck"], "ii_best": info["ii_best"], "RU": (R @ U).tolist(),
           "note": "setup: st_d2bi_set_supercell_tilt1a end to end (reflections, table, directions, FP32 screen "
                   "of every direction, FP64 scores of the n_fp64 it leaves open, exact near-tie re-scoring, "
                   "dark-field golden section, quaternion round trip); scan: the two scoring launches"}
    if cpu:
        from oracle import stem_oracle as O
        args = O.make_args(a_super, 3.1652, (0, 0, 1), (2, 0, 0), V=200.0, M=(4, 4), ng=1.0, xifile=xifile)
        t0 = time.perf_counter()
        so, _, _ = O.setup(args, w["pos"])
        out["cpu_oracle"] = {"ms": (time.perf_counter() - t0) * 1e3, "cores": 1, "kind": "port",
                             "same_rotation": bool(np.array_equal(np.array(list(so.R)).reshape(3, 3).T, R)),
                             "note": "oracle set-up with the -ng search (wrap, extents, search), one core"}
    # -surf on the 1.2M-atom cell: the foil-thickness pass over 27 x 1.2M replicas
    a0 = (2.87 + 2.87 + 2.87) / 3
    xw, a_vox, n = imaging.wrap_pbc(cell.a_super, (4, 4), a0, cell.pos)
    d_x = torch.from_numpy(np.ascontiguousarray(xw)).cuda()
    d = imaging.atom_extents((0, 0, 1), (1, 1, 0), a0 * np.eye(3), xw)
    fms, swall = [], []
    for i in range(warmup + steps):
        ts = imaging.DynamicalTwoBeamImaging(a_vox, n, a0, (0, 0, 1), (1, 1, 0), 200.0, 4, 4)
        ts.set_conventional_unit_cell(a0 * np.eye(3))
        ts.set_voxel_supercell_size(d)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        si = ts.set_supercell_tilt_ng(ctx, 1.0, xifile, d_x=d_x.data_ptr(), n_atoms=len(xw))
        if i >= warmup:
            swall.append(time.perf_counter() - t0)
            fms.append(si["foil_ms"])
    foil = float(np.median(fms))
    out["surf_1p2m"] = {"atoms": len(xw), "setup_ms": float(np.median(swall)) * 1e3, "foil_pass_ms": foil,
                        "replica_atoms_per_s": 27 * len(xw) / (foil * 1e-3), "foil": si["foil"],
                        "foil_sigma": si["foil_sigma"]}
    return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) > 8 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measure_fp32_peak():
    from simulated_tem_gb300 import _lib
    out = (ctypes.c_double * 5)()
    rc = _lib.peaks_lib().stp_measure_peaks(out)
    if rc != 0:
        return None
    # the FP32 peak is the larger of the scalar and the packed FP32x2 FMA rates (the
    # integrator issues FP32x2 instructions)
    return {"fp32_tflops": max(out[0], out[4]), "fp32_scalar_tflops": out[0], "fp32x2_tflops": out[4],
            "fp64_tflops": out[1], "mufu_ex2_gops": out[2], "mufu_sin_gops": out[3]}


def run_gpu(args):
    import torch

    from simulated_tem_gb300 import _lib, imaging, replicas

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cell, t, x, aperpx = workload()
    G, aa = t.image_geometry(len(x))
    n_prec = len(aa)
    ctx = imaging.Context(local)
    # one stream for torch's buffers, the L2 flush, the events and the library's kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    d_x = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    d_img = torch.zeros((G.My, G.Mx), dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    flags = _lib.ST_FLAG_FP32 | _lib.ST_FLAG_AVERAGE

    def step(f=flags):
        ctx.image_device(G, d_x.data_ptr(), len(x), aa, f, d_img.data_ptr(), stream=sptr)

    # counters for the roofline (one untimed image with statistics)
    step(flags | _lib.ST_FLAG_STATS)
    st = ctx.stats()
    n_acc, n_kept, n_tst = st.n_accepted, st.n_kept, st.n_tests
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    col_ms, launches, variant = [], 0, 0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
            st_i = ctx.stats()
            col_ms.append(st_i.ms_column)
            launches += st_i.n_launches
            variant = st_i.ring_variant
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        peaks = measure_fp32_peak()
        batched = None if args.no_batched else batched_legs(ctx, cell, stream, flush, args.batch_steps,
                                                             args.warmup, peaks=peaks,
                                                             cpu=(rank == 0 and not args.no_cpu))
        cfg1 = None if args.no_batched else cfg1_leg(ctx, stream, flush, 5, args.warmup,
                                                      cpu=(rank == 0 and not args.no_cpu))
        cfg5 = None if args.no_batched else cfg5_leg(ctx, stream, flush, 3, args.warmup)
        io = None if args.no_batched else io_leg(ctx, stream, flush, 5, args.warmup,
                                                  cpu=(rank == 0 and not args.no_cpu))
        inp = None if args.no_batched else input_leg(ctx, cell, stream, 3, args.warmup,
                                                     cpu=(rank == 0 and not args.no_cpu))
        tilt = None if args.no_batched else tilt_leg(ctx, cell, 3, args.warmup, cpu=(rank == 0 and not args.no_cpu))
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = float(np.mean(step_ms))
    ms_median = float(np.median(step_ms))
    # replicas: one image per rank per step; the slowest rank's time, all ranks' images
    value, ms, _ = replicas.job_rate(ms, 1)
    img32 = d_img.cpu().numpy().T.copy()

    # end to end through st_image from pinned host memory
    h_x = torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
    h_img = torch.zeros((G.My, G.Mx), dtype=torch.float64).pin_memory()
    geom_ptr = ctypes.byref(G)
    L = _lib.lib()
    aa_c = np.ascontiguousarray(aa)
    x_ptr = ctypes.cast(h_x.data_ptr(), _lib._dp)
    img_ptr = ctypes.cast(h_img.data_ptr(), _lib._dp)

    def e2e_step():
        rc = L.st_image(ctx.handle, geom_ptr, x_ptr, 3, len(x), aa_c.ctypes.data_as(_lib._dp), n_prec, flags, img_ptr)
        _lib.check(rc, ctx.handle)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_ms = []
    for i in range(args.steps):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t1) * 1e3)
    e2e_value, _, _ = replicas.job_rate(float(np.mean(e2e_ms)), 1)

    # the same image recorded as a CUDA graph (st_plan) and replayed
    pms = time_plan(ctx, [(G, d_x.data_ptr(), len(x), aa, d_img.data_ptr())], flags, stream, args.steps,
                    args.warmup, flush)
    plan_value, _, _ = replicas.job_rate(float(np.mean(pms)), 1)

    # plain FP64 GPU path on the same image
    step(_lib.ST_FLAG_AVERAGE)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    step(_lib.ST_FLAG_AVERAGE)
    e1.record(stream)
    torch.cuda.synchronize()
    fp64_ms = e0.elapsed_time(e1)
    img64 = d_img.cpu().numpy().T.copy()
    d = img32 - img64

    V = (G.ix1 - G.ix0) * (G.iy1 - G.iy0) * G.Mz
    col_avg = float(np.mean(col_ms))
    pix = (G.ix1 - G.ix0) * (G.iy1 - G.iy0)
    roof = path_roofline(peaks, n_acc, n_kept, len(x), V, V * n_prec, pix, False, col_avg)
    if roof:
        c_tests = reference_candidate_tests(ctx, G, x)
        roof.update({"kernel": "k_column_fp32_v3",
                     "peak_source": "measured live in this run by the project's pipe microbenchmarks "
                                    "(libstem_peaks.so: FP32 FMA, FP64 FMA, MUFU ex2 and sin); HBM from "
                                    + hbm_peak()[1],
                     "traffic": COLUMN_TRAFFIC_BYTES, "traffic_unit": "bytes per launch",
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_column_fp32_v3 on "
                                       "this image (profiles/k_column_fp32_v3_1p2m_screw.md)",
                     "frac_step": roof["t_roof_ms"] / ms,
                     "executed": {"tests": n_tst, "tests_per_voxel": n_tst / V,
                                  "reference_tests_per_voxel": c_tests / V,
                                  "accepted_per_voxel": n_acc / V,
                                  "ex2_issued": n_tst / 2, "ex2_frac_of_peak":
                                      n_tst / 2 / (col_avg * 1e-3) / (peaks["mufu_ex2_gops"] * 1e9),
                                  "note": "work the kernel executes: tests counts each buffered atom once per "
                                          "column and slice; the in-plane weight is one ex2 per atom and column "
                                          "for both slices of a step (ex2_issued), the depth factor one per atom "
                                          "and slice for the whole warp; the reference's own 27-cell search "
                                          "tests reference_tests_per_voxel candidates per voxel"}})
    acc = {"max_abs_dI_fp32_vs_fp64": float(np.abs(d).max()), "rms_dI_fp32_vs_fp64": float(np.sqrt((d ** 2).mean()))}
    line = {"metric": METRIC, "value": value, "unit": "images/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "ms_per_step_median": ms_median, "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded bcc Fe cell, no dataset)",
            "config": {"workload": WORKLOAD, "atoms": len(x), "image": [G.Mx, G.My, G.Mz], "n_prec": n_prec,
                       "path": "FP32 deposition + integration, FP64 binning and g.r mod 1",
                       "l2": "flushed between steps (512 MB write)", "parallelism": "replicas%d" % ws,
                       "ring_variant": _lib.lib().st_tune_variant_name(variant).decode()},
            "e2e": {"value": e2e_value, "unit": "images/s", "h2d_bytes_per_step": int(x.nbytes),
                    "d2h_bytes_per_step": int(G.Mx * G.My * 8)},
            "fp64": {"value": 1000.0 / fp64_ms, "unit": "images/s", "ms": fp64_ms},
            "plan": {"value": plan_value, "unit": "images/s",
                     "note": "the same step recorded once as a CUDA graph (st_plan) and replayed"},
            "accuracy": acc,
            "gpu_launches": launches,
            "roofline": roof, "peaks": peaks, "wall_s": wall, "clocks": clk.summary(), "batched": batched, "cfg1_128k": cfg1, "cfg5_corrector": cfg5,
            "output_files": io, "input_file": inp, "tilt_search": tilt}
    if rank == 0:
        if ws == 1 and not args.no_cpu:
            from simulated_tem_gb300 import synth
            cb, want = cpu_baseline(cell, synth.A0_FE)
            line["cpu_baseline"] = cb
            for name, img in (("fp32", img32), ("fp64", img64)):
                r = vs_oracle(img, want)
                acc["max_abs_dI_%s_vs_oracle" % name] = r["max_abs_dI"]
                acc["rms_dI_%s_vs_oracle" % name] = r["rms_dI"]
            acc["reference"] = "oracle (FP64 C restatement of computeD2BI_img), whole image, %d pixels" % want.size
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def reference_candidate_tests(ctx, G, x):
    """C_tests of the reference algorithm: every voxel tests every atom of the 27
    link cells around its home cell (Lib_LinkCell3D.f90:1562-1601).  Computed
    from the per-cell atom counts of the binning and the voxels' home cells."""
    # home cells per axis, as the library computes them
    def homes(n, a_vox, lcd, ia, N):
        i = np.arange(n, dtype=np.float64)
        zi = ia * (a_vox * i - lcd)
        return np.mod(np.floor(zi).astype(np.int64) + 16 * N, N)
    hx = homes(G.Mx, G.a_vox[0], G.lc_delta[0], G.ia_col[0], G.Ex)[G.ix0:G.ix1]
    hy = homes(G.My, G.a_vox[4], G.lc_delta[1], G.ia_col[4], G.Ey)[G.iy0:G.iy1]
    hz = homes(G.Mz, G.a_vox[8], G.lc_delta[2], G.ia_col[8], G.Ez)

    def weight(h, N):
        nv = np.bincount(h, minlength=N).astype(np.float64)
        return nv + np.roll(nv, 1) + np.roll(nv, -1)  # voxels whose home is c-1, c or c+1 (periodic)
    wx, wy, wz = weight(hx, G.Ex), weight(hy, G.Ey), weight(hz, G.Ez)
    cnt = _bin_counts(G, x).reshape(G.Ez, G.Ey, G.Ex).astype(np.float64)
    return float(np.einsum("zyx,x,y,z->", cnt, wx, wy, wz))


def _bin_counts(G, x):
    """Per-cell atom counts of findGdotR for geometry G, recounted in numpy for the
    flop accounting (a boundary atom may land in a neighbouring cell here; the
    count is used for the roofline only)."""
    RU = np.array(list(G.RU)).reshape(3, 3, order="F")
    delta = np.array(list(G.delta))
    lcd = np.array(list(G.lc_delta))
    ia = np.array([G.ia_col[0], G.ia_col[4], G.ia_col[8]])
    N = np.array([G.Ex, G.Ey, G.Ez])
    counts = np.zeros(G.Ex * G.Ey * G.Ez, dtype=np.int64)
    for n in range(G.nuvw):
        R = np.array(list(G.Ruvw)[3 * n:3 * n + 3])
        y = (x + R) @ RU.T + delta
        c = (y - lcd) * ia
        ok = np.all((c >= 0) & (c < N), axis=1)
        ci = np.floor(c[ok]).astype(np.int64)
        lin = ci[:, 0] + G.Ex * (ci[:, 1] + G.Ey * ci[:, 2])
        counts += np.bincount(lin, minlength=len(counts))
    return counts


def cpu_baseline(cell, A0, threads=None):
    """The oracle (C restatement of the reference's computeD2BI_img) on all host cores, one
    whole image, binning included; also returns the image (the accuracy reference)."""
    threads = threads or os.cpu_count() or 1
    img, s, st = oracle_workload_image(oracle_workload_setup(cell, A0), threads)
    return {"value": 1.0 / s, "unit": "images/s", "cores": threads, "kind": "port",
            "sample": "one whole 1.2M-atom image (566 x 566 x 240 voxels, binning included) by the oracle's C "
                      "restatement of computeD2BI_img on %d host threads: %.2f s" % (threads, s),
            "seconds_measured": s, "accepted_pairs": st.n_accepted}, img


def run_reference(args):
    """The reference's algorithm on the host cores (the reference's Fortran cannot be built on
    either machine, so the oracle's C restatement of it runs), whole images, all host threads.
    Nothing of the product is imported or loaded: the cell comes from the generator module
    loaded by its file path, the geometry and the image from the oracle."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import stem_oracle as O
    O.build() if not os.path.exists(O.LIB_PATH) else None
    synth = standalone_synth()
    cell = synth.screw_cell_1p2m()
    threads = os.cpu_count() or 1
    state = oracle_workload_setup(cell, synth.A0_FE)
    secs = []
    for i in range(args.warmup + args.steps):
        _, s, _ = oracle_workload_image(state, threads)
        if i >= args.warmup:
            secs.append(s)
    s_per_img = float(np.mean(secs))
    value = 1.0 / s_per_img
    cb = {"value": value, "unit": "images/s", "cores": threads, "kind": "port",
          "sample": "whole 1.2M-atom images (566 x 566 x 240 voxels, binning included), one per step, by the "
                    "oracle's C restatement of computeD2BI_img on %d host threads; min %.2f s, max %.2f s"
                    % (threads, min(secs), max(secs))}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": s_per_img * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded bcc Fe cell)",
            "config": {"workload": WORKLOAD, "atoms": len(cell.pos),
                       "note": "reference Fortran is not buildable here (no Fortran compiler on either machine); "
                               "the oracle C restatement of its algorithm runs on all host cores"},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ncu_case(args):
    """Untimed cases for ncu captures.  fp32 / fp64: two images of the workload through
    st_image, nothing else (binning and column kernels).  cfg1: one warm-up and one step of
    the 128k-atom DF + BF + blur leg on both paths (FP64 column kernel, blur).  corrector:
    one warm-up and one step of the 4.8M-atom corrector leg (convolutions).  io / input: one
    warm-up and one step of the output-file and input-file legs."""
    from simulated_tem_gb300 import _lib, imaging
    if args.ncu_case == "tilt":
        ctx = imaging.Context(0)
        cell, _, _, _ = workload()
        r = tilt_leg(ctx, cell, 1, 1, cpu=False)
        print("ncu case tilt: %s" % json.dumps(r))
        ctx.close()
        return
    if args.ncu_case in ("io", "input"):
        import torch
        stream = torch.cuda.Stream()
        flush = torch.empty(64 << 20, dtype=torch.float64, device="cuda")
        ctx = imaging.Context(0)
        with torch.cuda.stream(stream):
            if args.ncu_case == "io":
                r = io_leg(ctx, stream, flush, 1, 1, cpu=False)
            else:
                cell, _, _, _ = workload()
                r = input_leg(ctx, cell, stream, 1, 1, cpu=False)
        torch.cuda.synchronize()
        print("ncu case %s: %s" % (args.ncu_case, json.dumps(r)))
        ctx.close()
        return
    if args.ncu_case in ("cfg1", "corrector"):
        import torch
        stream = torch.cuda.Stream()
        flush = torch.empty(64 << 20, dtype=torch.float64, device="cuda")
        ctx = imaging.Context(0)
        with torch.cuda.stream(stream):
            if args.ncu_case == "cfg1":
                r = cfg1_leg(ctx, stream, flush, 1, 1, cpu=False)
                print("ncu case cfg1: FP64 %.1f images/s" % r["gpu_fp64"]["images_per_s"])
            else:
                r = cfg5_leg(ctx, stream, flush, 1, 1)
                print("ncu case corrector: %s" % json.dumps(r.get("m2_corrector_fallback", r)))
        torch.cuda.synchronize()
        ctx.close()
        return
    _, t, x, _ = workload()
    G, aa = t.image_geometry(len(x))
    ctx = imaging.Context(0)
    flags = _lib.ST_FLAG_AVERAGE | (0 if args.ncu_case == "fp64" else _lib.ST_FLAG_FP32)
    for _ in range(2):
        img = ctx.image(G, x, aa, flags=flags)
    print("ncu case %s: mean I %.6f, column kernel %d" % (args.ncu_case, img.mean(), ctx.stats().column_kernel))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched sweep and uneven-cell legs")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--ncu-case", choices=["fp32", "fp64", "cfg1", "corrector", "io", "input", "tilt"], default=None,
                    help="run one small untimed case only (for an ncu capture)")
    args = ap.parse_args()
    if args.ncu_case:
        ncu_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
