"""Seeded synthetic smFISH stacks with the shapes of the benchmark
configurations (no public dataset is named for this path).

* PSF: normalised 3-D Gaussian, default 40^3 with sigma_z 2.0, sigma_xy 1.3.
* Hyb colour: Poisson(600) background plus puncta rendered as
  ``A exp(-dz^2/(2 sz^2) - (dx^2+dy^2)/(2 sxy^2))`` over +-4 sigma, positions
  uniform, A lognormal (median 8000, sigma 0.5), rounded and clipped to uint16;
  optionally multiplied by a quadratic flat-field gain ``1 - 0.2 r^2/r_max^2``.
* DAPI: Poisson(600) plus 300 solid ellipsoids (radii 4 x 25 x 25) adding 3000.

``device`` selects torch's generator on that device (fast for full FOVs);
results depend on the device's RNG, so tests that compare against the oracle
generate on the CPU.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def gaussian_psf(shape=(40, 40, 40), sigma_z=2.0, sigma_xy=1.3):
    z, x, y = [np.arange(n, dtype=np.float64) - n // 2 for n in shape]
    g = np.exp(-z[:, None, None] ** 2 / (2 * sigma_z ** 2)
               - (x[None, :, None] ** 2 + y[None, None, :] ** 2) / (2 * sigma_xy ** 2))
    return (g / g.sum()).astype(np.float32)


def flat_gain(X, Y):
    xx = np.arange(X, dtype=np.float64)[:, None] - (X - 1) / 2
    yy = np.arange(Y, dtype=np.float64)[None, :] - (Y - 1) / 2
    r2 = xx ** 2 + yy ** 2
    return (1.0 - 0.2 * r2 / r2.max()).astype(np.float32)


def _gen(seed, device):
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    return g


def hyb_stack(Z, X, Y, n_puncta, seed, device="cpu", sigma_z=1.0, sigma_xy=1.5, gain=None):
    """uint16 (Z, X, Y) colour channel (torch tensor on ``device``)."""
    dev = torch.device(device)
    g = _gen(seed, dev)
    vol = torch.poisson(torch.full((Z, X, Y), 600.0, device=dev), generator=g)
    if n_puncta:
        pos = torch.rand((n_puncta, 3), generator=g, device=dev) * torch.tensor([Z, X, Y], device=dev,
                                                                                   dtype=torch.float32)
        amp = torch.exp(math.log(8000.0) + 0.5 * torch.randn(n_puncta, generator=g, device=dev))
        rz, rxy = int(math.ceil(4 * sigma_z)), int(math.ceil(4 * sigma_xy))
        oz = torch.arange(-rz, rz + 1, device=dev)
        ox = torch.arange(-rxy, rxy + 1, device=dev)
        off = torch.stack(torch.meshgrid(oz, ox, ox, indexing="ij"), -1).reshape(-1, 3)
        chunk = max(1, (1 << 24) // off.shape[0])
        flat_vol = vol.view(-1)
        for s in range(0, n_puncta, chunk):
            p = pos[s:s + chunk]
            c = torch.floor(p).long()
            idx = c[:, None, :] + off[None, :, :]
            d = idx.float() - p[:, None, :]
            val = amp[s:s + chunk, None] * torch.exp(-d[..., 0] ** 2 / (2 * sigma_z ** 2)
                                                      - (d[..., 1] ** 2 + d[..., 2] ** 2) / (2 * sigma_xy ** 2))
            ok = ((idx >= 0) & (idx < torch.tensor([Z, X, Y], device=dev))).all(-1)
            lin = (idx[..., 0] * X + idx[..., 1]) * Y + idx[..., 2]
            flat_vol.index_put_((lin[ok],), val[ok], accumulate=True)
    if gain is not None:
        vol *= torch.as_tensor(gain, device=dev)[None]
    return torch.clamp(torch.round(vol), 0, 65535).to(torch.int32).to(torch.uint16)


def dapi_stack(Z, X, Y, seed, device="cpu", n_nuclei=300, radii=(4.0, 25.0, 25.0), value=3000.0,
               offset=(0.0, 0.0, 0.0), noise_seed=None):
    """uint16 (Z, X, Y) nuclei-like channel.  ``offset`` moves every nucleus
    centre by (dz, dx, dy) before it is rounded to the grid (a drifted round of
    the same field); ``noise_seed`` draws the Poisson background independently
    of the nuclei (default: ``seed``)."""
    dev = torch.device(device)
    g = _gen(seed if noise_seed is None else noise_seed, dev)
    vol = torch.poisson(torch.full((Z, X, Y), 600.0, device=dev), generator=g)
    gc = _gen(seed + 7919, dev)
    cen = torch.rand((n_nuclei, 3), generator=gc, device=dev) * torch.tensor([Z, X, Y], device=dev,
                                                                              dtype=torch.float32)
    cen = cen + torch.tensor(offset, device=dev, dtype=torch.float32)
    rz, rx, ry = radii
    oz = torch.arange(-int(rz), int(rz) + 1, device=dev)
    ox = torch.arange(-int(rx), int(rx) + 1, device=dev)
    oy = torch.arange(-int(ry), int(ry) + 1, device=dev)
    off = torch.stack(torch.meshgrid(oz, ox, oy, indexing="ij"), -1).reshape(-1, 3)
    inside = (off[:, 0] / rz) ** 2 + (off[:, 1] / rx) ** 2 + (off[:, 2] / ry) ** 2 <= 1.0
    off = off[inside]
    mask = torch.zeros(Z * X * Y, dtype=torch.bool, device=dev)
    chunk = max(1, (1 << 24) // off.shape[0])
    for s in range(0, n_nuclei, chunk):
        c = torch.round(cen[s:s + chunk]).long()
        idx = c[:, None, :] + off[None, :, :]
        ok = ((idx >= 0) & (idx < torch.tensor([Z, X, Y], device=dev))).all(-1)
        lin = ((idx[..., 0] * X + idx[..., 1]) * Y + idx[..., 2])[ok]
        mask.index_fill_(0, lin, True)
    vol += value * mask.view(Z, X, Y)
    return torch.clamp(torch.round(vol), 0, 65535).to(torch.int32).to(torch.uint16)
