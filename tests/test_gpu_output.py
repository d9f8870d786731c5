"""d2bi's output files on the GPU: the '(1000f12.7)' records and the 16-bit PNG levels
against the oracle and the reference's shipped .dat and PNG files, and the whole files
written by st_write_dat and st_write_png."""
import os

import numpy as np
import pytest

from oracle import stem_oracle as O
from simulated_tem_gb300 import imaging

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from tests import golden_data
from tests.test_output_formats import MF, dat_text, header_fields


@pytest.fixture(scope="module")
def ctx():
    c = imaging.Context(0)
    yield c
    c.close()


def gpu_records(ctx, values):
    v = torch.from_numpy(np.ascontiguousarray(values, dtype=np.float64).ravel()).cuda()
    n = v.numel()
    cap = imaging.lib().st_dat_text_bytes(n)
    out = torch.zeros(max(cap, 1), dtype=torch.uint8, device="cuda")
    ctx.format_dat_device(v.data_ptr(), n, out.data_ptr(), cap, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return bytes(out.cpu().numpy()[:cap])


def gpu_levels(ctx, img, lo=0.0, hi=0.0):
    img = np.asfortranarray(img, dtype=np.float64)
    d = torch.from_numpy(img.T.copy()).cuda()  # (ny, nx): x fastest, as the image in memory
    lv = torch.zeros(img.size, dtype=torch.int16, device="cuda")
    ctx.png_levels_device(d.data_ptr(), img.shape[0], img.shape[1], lv.data_ptr(), lo, hi,
                          stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return lv.cpu().numpy().view(np.uint16).reshape(img.shape[1], img.shape[0])


def test_records_match_oracle(ctx):
    rng = np.random.default_rng(5)
    v = np.concatenate([
        rng.random(2500), -rng.random(300), rng.random(200) * 1e-8, -rng.random(50) * 1e-8,
        rng.standard_normal(400) * 1000, [0.0, -0.0, 9999.9999999, 9999.99999995, 10000.0, -999.9999999,
                                          -1000.0, 1e300, 5e-8, 4.9999999e-8, 0.12345675, 0.5, 1.0],
        # values whose seventh decimal sits near a rounding boundary
        (np.arange(1000) + 0.5) * 1e-7 + rng.standard_normal(1000) * 1e-15,
    ])
    got = gpu_records(ctx, v)
    assert got == O.format_f12_7(v)


def test_records_reproduce_the_reference_file(ctx):
    d = dat_text()
    img = golden_data.w_loop()["img"]  # the shipped image, column-major (x fastest)
    got = gpu_records(ctx, img.T.ravel())
    lines = got.decode().split("\n")
    assert len(lines) == d["n_records"] + 1 and lines[-1] == ""
    assert lines[0] == d["first_record"] and lines[-2] == d["last_record"]


def test_write_dat_file(ctx, tmp_path):
    d = dat_text()
    img = golden_data.w_loop()["img"]
    path = str(tmp_path / "w.dat")
    ctx.write_dat(path, header_fields(d["header_lines"]), img)
    with open(path) as f:
        lines = f.read().split("\n")
    k = len(d["header_lines"])
    assert lines[:k] == d["header_lines"]
    assert lines[k] == d["first_record"] and lines[-2] == d["last_record"] and lines[-1] == ""
    assert not os.path.exists(path + ".tmp")


@pytest.mark.parametrize("shape", [(94, 94), (300, 7), (1, 1)])
def test_levels_match_oracle(ctx, shape):
    rng = np.random.default_rng(shape[0])
    img = rng.random(shape) * 0.3 + 0.05
    assert np.array_equal(gpu_levels(ctx, img), O.png_levels(img))
    lo, hi = 0.1, 0.25  # the contrast window clamps part of the image
    assert np.array_equal(gpu_levels(ctx, img, lo, hi), O.png_levels_window(img, lo, hi))
    flat = np.full(shape, 0.42)  # no contrast: level 32768 everywhere
    assert np.array_equal(gpu_levels(ctx, flat), O.png_levels(flat))


def test_write_png_reproduces_the_reference_png(ctx, tmp_path):
    """The shipped image blurred at 2.5 A (d2bi's default PNG) and written by st_write_png
    decodes to the oracle's levels exactly and to the shipped PNG's levels within one
    level (the .dat image holds 7 decimals)."""
    g = golden_data.w_loop()
    t = 2.5 / g["header"]["scale (A/px)"][0]
    path = str(tmp_path / "w.png")
    ctx.write_png(path, g["img"], blur_t=t)
    got = MF.decode_png16(path)
    want = O.png_levels(O.gaussian_blur(g["img"], t))
    assert np.array_equal(got, want)
    assert np.abs(got.astype(int) - g["png"].astype(int)).max() <= 1
    # contrast window, no blur
    ctx.write_png(path, g["img"], iso_min=0.05, iso_max=0.2)
    assert np.array_equal(MF.decode_png16(path), O.png_levels_window(g["img"], 0.05, 0.2))
