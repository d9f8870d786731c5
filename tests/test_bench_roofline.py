"""The path roofline that bench.py reports as `roofline.frac`: the reference's algorithmic
work per image (3 MUFU per accepted pair + 1 per voxel; 12 FP32 per accepted pair, 6 per
voxel, 10 more per voxel with density, 90 per voxel and precession angle; 30 FP64 per kept
atom; 24 B per atom, 16 per kept atom, 8 per pixel of HBM), each over its measured peak,
the largest over the measured time.  Checked against the formula written out by hand for
a MUFU-bound single image and an FP32-bound 16-angle sweep, so the reported fractions can
be recomputed from the counts in the bench line."""
import pytest

import bench

PEAKS = {"fp32_tflops": 79.5, "fp64_tflops": 1.05, "mufu_ex2_gops": 9870.0, "mufu_sin_gops": 4965.0}


def _by_hand(n_acc, n_kept, n_atoms, voxels, voxel_prec, pixels, density, hbm_gbs):
    t = {
        "mufu": (n_acc + voxels) / (PEAKS["mufu_ex2_gops"] * 1e9) + 2 * n_acc / (PEAKS["mufu_sin_gops"] * 1e9),
        "fp32": (12 * n_acc + (16 if density else 6) * voxels + 90 * voxel_prec) / (PEAKS["fp32_tflops"] * 1e12),
        "fp64": 30 * n_kept / (PEAKS["fp64_tflops"] * 1e12),
        "hbm": (24 * n_atoms + 16 * n_kept + 8 * pixels) / (hbm_gbs * 1e9),
    }
    return t


def test_single_image_is_mufu_bound():
    # the 1.2M-atom image: 2.16e9 accepted pairs, 566 x 566 x 240 voxels, one angle
    n_acc, n_kept, n_atoms = 2_162_375_050, 2_514_000, 1_193_647
    voxels, pixels = 566 * 566 * 240, 566 * 566
    t_ms = 2.83
    r = bench.path_roofline(PEAKS, n_acc, n_kept, n_atoms, voxels, voxels, pixels, False, t_ms)
    hbm_gbs, _ = bench.hbm_peak()
    want = _by_hand(n_acc, n_kept, n_atoms, voxels, voxels, pixels, False, hbm_gbs)
    assert r["bound"] == "mufu"
    assert r["t_roof_ms"] == pytest.approx(want["mufu"] * 1e3, rel=1e-12)
    assert r["frac"] == pytest.approx(want["mufu"] / (t_ms * 1e-3), rel=1e-12)
    for k in want:
        assert r["per_resource_ms"][k] == pytest.approx(want[k] * 1e3, rel=1e-12)
    # achieved work rate = the bound's work over the measured time, in its unit
    assert r["achieved"] == pytest.approx(r["frac"] * r["peak"], rel=1e-12)
    assert r["work"]["mufu_ops"] == 3 * n_acc + voxels


def test_sixteen_angle_sweep_is_fp32_bound():
    # 16 precession angles per image: the integration's 90 flop per voxel and angle dominate
    n_acc, n_kept, n_atoms = 2.0e9, 2.5e6, 1.2e6
    voxels, pixels = 566 * 566 * 240, 566 * 566
    t_ms = 4.9
    r = bench.path_roofline(PEAKS, n_acc, n_kept, n_atoms, voxels, 16 * voxels, pixels, True, t_ms)
    hbm_gbs, _ = bench.hbm_peak()
    want = _by_hand(n_acc, n_kept, n_atoms, voxels, 16 * voxels, pixels, True, hbm_gbs)
    assert r["bound"] == "fp32"
    assert r["frac"] == pytest.approx(want["fp32"] / (t_ms * 1e-3), rel=1e-12)
    assert r["work"]["fp32_flop"] == pytest.approx(12 * n_acc + 16 * voxels + 90 * 16 * voxels, rel=1e-12)
    assert r["unit"] == "TFLOP/s" and r["peak"] == pytest.approx(PEAKS["fp32_tflops"], rel=1e-12)


def test_no_peaks_no_roofline():
    assert bench.path_roofline(None, 1, 1, 1, 1, 1, 1, False, 1.0) is None
