"""Synthetic scalar fields for benchmarks and tests (seeded, generated with torch).

Every field is returned indexed [x, y, z] with x fastest in memory (a
``permute(2, 1, 0)`` view of a contiguous (nz, ny, nx) tensor), i.e. the
memory layout of a Julia ``Array{T,3}``, sampled on LinRange nodes.

* sphere_sdf       |p| - r on [-1,1]^3                 (64^3 Float64 fixture)
* gyroid           sin x cos y + sin y cos z + sin z cos x on [-3pi,3pi]^3
* sines            sum_k a_k sin(2pi w_k.p + phi_k) on [0,1]^3, 16 seeded terms
* ct_like_u16      N(100,20) background + 3 seeded ellipsoidal shells N(1000,50), UInt16
* primitives_sdf   min-union of 1-8 seeded spheres / boxes on [-1,1]^3
* batch_volumes    many primitives_sdf volumes of uneven seeded shapes
"""
import math

import numpy as np


def _grid(n, a, b, device, dtype):
    import torch
    return torch.linspace(a, b, n, dtype=torch.float64, device=device).to(dtype)


def _julia(t):
    return t.permute(2, 1, 0)


def sphere_sdf(n=64, r=0.4, dtype=None, device='cuda'):
    import torch
    dtype = dtype or torch.float64
    g = _grid(n, -1.0, 1.0, device, torch.float64)
    z, y, x = torch.meshgrid(g, g, g, indexing='ij')
    return _julia((torch.sqrt(x * x + y * y + z * z) - r).to(dtype))


def gyroid(n=256, dtype=None, device='cuda'):
    import torch
    dtype = dtype or torch.float32
    g = _grid(n, -3 * math.pi, 3 * math.pi, device, torch.float32)
    z, y, x = torch.meshgrid(g, g, g, indexing='ij')
    f = torch.sin(x) * torch.cos(y) + torch.sin(y) * torch.cos(z) + torch.sin(z) * torch.cos(x)
    return _julia(f.to(dtype))


def sines_params(seed=0, terms=16):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(terms):
        a = rng.standard_normal()
        mag = rng.uniform(1, 8)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        ph = rng.uniform(0, 2 * np.pi)
        out.append((a, mag * d, ph))
    return out


def sines(n=1024, seed=0, dtype=None, device='cuda', nz=None, z0=0):
    """16-term random plane waves on [0,1]^3 (n^3 nodes); `nz`/`z0` select a z slab."""
    import torch
    dtype = dtype or torch.float32
    nz = n if nz is None else nz
    g = _grid(n, 0.0, 1.0, device, torch.float32)
    gz = g[z0:z0 + nz]
    out = torch.zeros((nz, n, n), dtype=torch.float32, device=device)
    for a, w, ph in sines_params(seed):
        # sin(2pi(w.p) + ph), evaluated per z plane to bound temporaries
        ax = (2 * math.pi * w[0]) * g
        ay = (2 * math.pi * w[1]) * g
        for k in range(nz):
            arg = ax[None, :] + ay[:, None] + float(2 * math.pi * w[2] * gz[k].item() + ph)
            out[k].add_(torch.sin(arg), alpha=float(a))
    return _julia(out.to(dtype))


def ct_like_u16(n=512, seed=0, device='cuda'):
    import torch
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=device).manual_seed(seed)
    f = torch.randn((n, n, n), generator=gen, device=device, dtype=torch.float32) * 20 + 100
    g = torch.arange(n, device=device, dtype=torch.float32)
    z, y, x = g[:, None, None], g[None, :, None], g[None, None, :]
    for _ in range(3):
        c = rng.uniform(0.3, 0.7, 3) * n
        ax = rng.uniform(0.1, 0.4, 3) * n
        val = rng.normal(1000, 50)
        # distance from the ellipsoid surface in voxels, approximately
        q = torch.sqrt(((x - c[0]) / ax[0]) ** 2 + ((y - c[1]) / ax[1]) ** 2 + ((z - c[2]) / ax[2]) ** 2)
        shell = (q - 1).abs() * float(ax.min()) < 2.0
        f = torch.where(shell, torch.full_like(f, float(val)), f)
        del q, shell
    return _julia(f.clamp_(min=0).round_().to(torch.int32).to(torch.uint16))


def primitives_params(rng):
    k = int(rng.integers(1, 9))
    prims = []
    for _ in range(k):
        kind = int(rng.integers(0, 2))
        c = rng.uniform(-0.6, 0.6, 3)
        if kind == 0:
            prims.append(('sphere', c, rng.uniform(0.05, 0.3)))
        else:
            prims.append(('box', c, rng.uniform(0.05, 0.25, 3)))
    return prims


def primitives_sdf(shape, prims, dtype=None, device='cuda'):
    import torch
    dtype = dtype or torch.float32
    nx, ny, nz = shape
    gx, gy, gz = (_grid(n, -1.0, 1.0, device, torch.float32) for n in (nx, ny, nz))
    z, y, x = gz[:, None, None], gy[None, :, None], gx[None, None, :]
    f = None
    for kind, c, s in prims:
        if kind == 'sphere':
            d = torch.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) - float(s)
        else:
            qx, qy, qz = (x - c[0]).abs() - s[0], (y - c[1]).abs() - s[1], (z - c[2]).abs() - s[2]
            outside = torch.sqrt(qx.clamp(min=0) ** 2 + qy.clamp(min=0) ** 2 + qz.clamp(min=0) ** 2)
            inside = torch.maximum(torch.maximum(qx, qy), qz).clamp(max=0)
            d = outside + inside
        f = d if f is None else torch.minimum(f, d)
    return _julia(f.to(dtype).contiguous())


def batch_volumes(n=4096, seed=0, lo=16, hi=128, dtype=None, device='cuda'):
    """`n` volumes, each axis size uniform in lo..hi, each a primitives_sdf of
    1-8 seeded spheres / boxes on [-1,1]^3 (the batched workload)."""
    rng = np.random.default_rng(seed)
    vols = []
    for _ in range(n):
        shape = tuple(int(s) for s in rng.integers(lo, hi + 1, 3))
        vols.append(primitives_sdf(shape, primitives_params(rng), dtype=dtype, device=device))
    return vols
