"""BF16 grid storage (fp32 arithmetic) against the fp32 path and an fp64 oracle.

The fp64 oracle at this size is the fp64 instantiation of the fused kernels (every
sample, weight and sum in fp64), itself pinned to the CPU fp64 oracle by
test_gpu_fused.py (autograd to 1e-10, central differences to 1e-4).

Scene (the precision configuration, reduced to a test-sized ray count): a dense 512^3
grid of 64 Gaussian opacity blobs with uniform RGB, a "model" grid that differs from it
by a realistic training residual, 50 held-out seeded cameras rendered at 64x64 with 512
samples per ray. The bar: PSNR against the fp64 render of the ground truth changes by at
most 0.05 dB between fp32 and BF16 storage."""
import math

import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes

pytestmark = pytest.mark.gpu
DEV = "cuda"
SIDE, BLOBS, S, VIEWS, RES = 512, 64, 512, 50, 64


def _blob_grid(side, n_blobs, seed):
    g = torch.Generator(device=DEV).manual_seed(seed)
    pd = 3.0 / side
    ax = (torch.arange(side, device=DEV, dtype=torch.float32) - math.ceil(side / 2) + 1) * pd
    dens = torch.zeros(side, side, side, device=DEV)
    centres = torch.rand(n_blobs, 3, generator=g, device=DEV) * 2 - 1
    amps = 5 + 15 * torch.rand(n_blobs, generator=g, device=DEV)
    for c, a in zip(centres, amps):
        d2 = ((ax - c[0]) ** 2)[:, None, None] + ((ax - c[1]) ** 2)[None, :, None] + \
            ((ax - c[2]) ** 2)[None, None, :]
        dens += a * torch.exp(-d2 / (2 * 0.3 ** 2))
    rgb = torch.rand(side, side, side, 3, generator=g, device=DEV)
    return torch.cat([rgb, dens.unsqueeze(-1)], -1), g


def _views():
    T = torch.from_numpy(scenes.make_cameras(VIEWS, 900)).to(DEV)
    imgs = torch.zeros(VIEWS, RES, RES, 4, device=DEV)
    d, _ = pg.generate_rays_batched(imgs, RES * RES, T, 0.691, even_spread=True, device=DEV)
    o = torch.repeat_interleave(T[:, :3, 3], RES * RES, 0) + 2.0 * d
    return o.contiguous(), d.contiguous()


def _render(grid, o, d, chunk=65536, transmittance="product"):
    pd = 3.0 / SIDE
    out = []
    for i in range(0, o.shape[0], chunk):
        out.append(pg.render_rays(grid, o[i:i + chunk].to(pg._lib.real_dtype(grid.dtype)),
                                  d[i:i + chunk].to(pg._lib.real_dtype(grid.dtype)),
                                  4.0 / S, S, pd, transmittance=transmittance))
    return torch.cat(out)


def _psnr(x, ref):
    mse = float(((x.double() - ref.double()) ** 2).mean())
    return 10 * math.log10(1.0 / mse)


@pytest.fixture(scope="module")
def scene():
    truth, g = _blob_grid(SIDE, BLOBS, 7)
    # model = truth with a training residual: RGB noise and a damped opacity
    model = truth.clone()
    model[..., :3] += 0.05 * torch.randn(SIDE, SIDE, SIDE, 3, generator=g, device=DEV)
    model[..., 3] *= 0.9
    o, d = _views()
    with torch.no_grad():
        target = _render(truth.double(), o, d)                 # fp64 ground-truth views
    del truth
    return model, o, d, target


def test_bf16_storage_psnr_and_errors_vs_fp64_oracle(scene):
    model, o, d, target = scene
    with torch.no_grad():
        m32 = model
        m16 = model.to(torch.bfloat16)
        r32 = _render(m32, o, d)
        r16 = _render(m16, o, d)
        r64_32 = _render(m32.double(), o, d)                   # fp64 render of the fp32 values
        r64_16 = _render(m16.double(), o, d)                   # fp64 render of the bf16 values
    p32, p16 = _psnr(r32, target), _psnr(r16, target)
    assert 15.0 < p32 < 60.0, f"model residual gives PSNR {p32:.2f} dB"
    assert abs(p16 - p32) <= 0.05, f"PSNR fp32 {p32:.4f} dB vs bf16 {p16:.4f} dB"
    # error of each storage form against fp64 arithmetic on the same cell values. It is
    # dominated by the sample coordinates (fp32 versus fp64 positions move trilinear
    # weights by ~1e-7 of the coordinate), identical for both storage forms; a sample
    # within one fp32 rounding of a box face can land on the other side of the in-bounds
    # test, so the bar is on the 99.99th-percentile ray and the maximum is reported.
    err32 = (r32.double() - r64_32).abs().amax(1)
    err16 = (r16.double() - r64_16).abs().amax(1)
    q32, q16 = float(torch.quantile(err32, 0.9999)), float(torch.quantile(err16, 0.9999))
    e32, e16 = float(err32.max()), float(err16.max())
    assert q32 < 1e-4, (q32, e32)
    assert q16 <= 1.01 * q32 + 1e-7, "BF16 storage must add no arithmetic error"
    assert float(err16.median()) < 1e-5
    # gradient of one view's MSE (fused training step): BF16 storage with fp32
    # accumulation against fp64 on the same values
    sl = slice(0, RES * RES)
    grads = {}
    for name, grid in (("bf16", m16), ("fp64", m16.double())):
        real = pg._lib.real_dtype(grid.dtype)
        step = pg.FusedTrainStep(grid, 3.0 / SIDE, S, 4.0 / S)
        step.step_rays(o[sl].to(real), d[sl].to(real), target[sl].to(real))
        grads[name] = step.grad.double()
        del step
    rel = float((grads["bf16"] - grads["fp64"]).norm() / grads["fp64"].norm())
    # fp32 coordinates move trilinear weights against fp64 ones here as well
    assert rel < 1e-3, f"bf16-storage gradient vs fp64: relative error {rel:.2e}"
    print(f"PSNR fp32 {p32:.4f} dB, bf16 {p16:.4f} dB (delta {p16 - p32:+.4f}); |render - fp64| "
          f"p99.99 fp32 {q32:.2e} bf16 {q16:.2e}, max fp32 {e32:.2e} bf16 {e16:.2e}, median bf16 "
          f"{float(err16.median()):.2e}; gradient relative error {rel:.2e}")


def test_logsum_transmittance_vs_fp64_oracle(scene):
    """The compensated log-sum transmittance (T = exp of a TwoSum-compensated sum of
    log(1 - alpha)) over BF16 and fp32 cells, against fp64 arithmetic with the product form
    on the same cell values: the same per-ray bars as the product form, the same PSNR bar,
    and the BF16-storage gradient within the same relative bar."""
    model, o, d, target = scene
    m16 = model.to(torch.bfloat16)
    with torch.no_grad():
        r64_16 = _render(m16.double(), o, d)
        r64_32 = _render(model.double(), o, d)
        l16 = _render(m16, o, d, transmittance="logsum")
        l32 = _render(model, o, d, transmittance="logsum")
        p32 = _render(model, o, d)
    err_l16 = (l16.double() - r64_16).abs().amax(1)
    err_l32 = (l32.double() - r64_32).abs().amax(1)
    err_p32 = (p32.double() - r64_32).abs().amax(1)
    ql16, ql32, qp32 = (float(torch.quantile(e, 0.9999)) for e in (err_l16, err_l32, err_p32))
    assert ql32 < 1e-4 and ql16 < 1e-4, (ql32, ql16)
    assert float(err_l16.median()) < 1e-5
    psnr_p32, psnr_l16 = _psnr(p32, target), _psnr(l16, target)
    assert abs(psnr_l16 - psnr_p32) <= 0.05, (psnr_p32, psnr_l16)
    sl = slice(0, RES * RES)
    grads = {}
    for name, grid, tr in (("logsum_bf16", m16, "logsum"), ("fp64", m16.double(), "product")):
        real = pg._lib.real_dtype(grid.dtype)
        step = pg.FusedTrainStep(grid, 3.0 / SIDE, S, 4.0 / S, transmittance=tr)
        step.step_rays(o[sl].to(real), d[sl].to(real), target[sl].to(real))
        grads[name] = step.grad.double()
        del step
    rel = float((grads["logsum_bf16"] - grads["fp64"]).norm() / grads["fp64"].norm())
    assert rel < 1e-3, rel
    print(f"log-sum |render - fp64| p99.99 fp32 {ql32:.2e} bf16 {ql16:.2e} (product fp32 {qp32:.2e}); "
          f"PSNR product fp32 {psnr_p32:.4f} dB, log-sum bf16 {psnr_l16:.4f} dB; gradient rel {rel:.2e}")


@pytest.mark.parametrize("mode", ["nearest", "trilinear"])
def test_logsum_transmittance_long_thin_rays(mode):
    """A long ray through a faint medium (8192 samples of alpha ~ 2e-3: T falls to ~1e-7
    over 32 chunks) is where a running fp32 product accumulates the most rounding; the
    log-sum form must track fp64 at least as closely, and its adjoint must match the
    fp64 adjoint."""
    side, n_samples = 64, 8192
    g = torch.Generator(device=DEV).manual_seed(5)
    grid = torch.rand(side, side, side, 4, generator=g, device=DEV)
    grid[..., 3] = 1e-3 + 2e-3 * grid[..., 3]
    pd = 3.0 / side
    R = 512
    o = torch.zeros(R, 3, device=DEV)
    o[:, 0] = -1.49
    o[:, 1:] = (torch.rand(R, 2, generator=g, device=DEV) - 0.5) * 2.0
    d = torch.zeros(R, 3, device=DEV)
    d[:, 0] = 1.0
    delta = 2.98 / n_samples
    with torch.no_grad():
        ref = pg.render_rays(grid.double(), o.double(), d.double(), delta, n_samples, pd, mode=mode)
        prod = pg.render_rays(grid, o, d, delta, n_samples, pd, mode=mode)
        logs = pg.render_rays(grid, o, d, delta, n_samples, pd, mode=mode, transmittance="logsum")
    e_prod = float((prod.double() - ref).abs().max())
    e_log = float((logs.double() - ref).abs().max())
    assert e_log < 1e-5, (e_log, e_prod)
    assert e_log <= 4.0 * e_prod + 1e-6, (e_log, e_prod)
    # adjoint of the log-sum form against the fp64 adjoint
    w = torch.rand(R, 4, generator=g, device=DEV)
    gl = grid.clone().requires_grad_(True)
    (pg.render_rays(gl, o, d, delta, n_samples, pd, mode=mode, transmittance="logsum") * w).sum().backward()
    g64 = grid.double().requires_grad_(True)
    (pg.render_rays(g64, o.double(), d.double(), delta, n_samples, pd, mode=mode) * w.double()).sum().backward()
    rel = float((gl.grad.double() - g64.grad).norm() / g64.grad.norm())
    assert rel < 1e-4, rel
    print(f"{mode}: max |RGBA - fp64| product {e_prod:.2e}, log-sum {e_log:.2e}; adjoint rel {rel:.2e}")


def test_logsum_transmittance_rejects_unclipped_and_fp64():
    grid = torch.rand(8, 8, 8, 4, device=DEV)
    o = torch.zeros(4, 3, device=DEV)
    d = torch.zeros(4, 3, device=DEV)
    d[:, 0] = 1.0
    with pytest.raises(pg._lib.PlenoxelsError):
        pg.render_rays(grid, o, d, 0.1, 16, 3.0 / 8, clip=False, transmittance="logsum")
    with pytest.raises(NotImplementedError):
        pg.render_rays(grid.double(), o.double(), d.double(), 0.1, 16, 3.0 / 8, transmittance="logsum")
    with pytest.raises(ValueError):
        pg.render_rays(grid, o, d, 0.1, 16, 3.0 / 8, transmittance="kahan")
