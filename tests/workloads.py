"""Seeded synthetic inputs of the benchmark configurations.

The reference publishes no benchmark inputs; these stand in for them with
the shapes and value distributions each configuration names:

  config 2 (the bench workload): 4096^2 vertex-centred 2D 9-point masked
    Laplacian. Cell noise N(0,1) (seed 1), gaussian_filter(sigma=32,
    mode='reflect', truncate=4); the lowest 30 % are land. The vertex mask
    follows get_mask_at_corners (test/test_RP.jl:46-54): a vertex is wet iff
    its four cells are. RHS: N(0,1) from the same generator (next draws) on
    wet vertices, wet mean removed.
  config 1: 256^2 cell-centred 5-point, disk of radius 0.45 N, RHS N(0,1)
    (seed 0) on wet cells, mean removed.
"""
from __future__ import annotations

import numpy as np

import fixtures as F


def gaussian_smooth(a, sigma: float, truncate: float = 4.0):
    """scipy.ndimage.gaussian_filter(a, sigma, mode='reflect', truncate) of
    a 2D array, by FFT convolution along each axis: the same sampled and
    normalised kernel and the same half-sample symmetric edges, equal to the
    direct filter to rounding (about 1e-15 relative), at O(n^2 log n)
    instead of O(n^2 sigma) for the wide kernels of large grids."""
    from scipy.signal import fftconvolve

    r = int(truncate * float(sigma) + 0.5)
    t = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (t / sigma) ** 2)
    k /= k.sum()
    out = np.asarray(a, dtype=np.float64)
    for ax in range(out.ndim):
        n = out.shape[ax]
        if r >= n:  # the symmetric padding below must not wrap more than once
            from scipy.ndimage import gaussian_filter1d

            out = gaussian_filter1d(out, sigma, axis=ax, mode="reflect", truncate=truncate)
            continue
        pad = [(0, 0)] * out.ndim
        pad[ax] = (r, r)
        ext = np.pad(out, pad, mode="symmetric")
        shape = [1] * out.ndim
        shape[ax] = 2 * r + 1
        out = fftconvolve(ext, k.reshape(shape), mode="valid", axes=ax)
    return out


def coastline_cells(n: int, seed: int, sigma: float, land: float):
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((n, n))
    sm = gaussian_filter(noise, sigma, mode="reflect", truncate=4.0)
    thr = np.quantile(sm, land)
    return sm > thr, rng


# Deepest hierarchy of the reference's algorithm that converges on the
# config-2 coastline. The coverage-thresholded coarse masks
# (compute_msk_dev, src/gmg_setup.jl:322-366) split the connected ocean
# into many pieces once a coarse cell spans more than ~16 fine cells; with
# 6 levels the F-cycle diverges (x1.18 per cycle), with 10 levels (the
# configuration's own count) by x11 per cycle (CPU oracle, 4096^2).
CONFIG2_LEVELS = 5


def config2(n: int = 4096, nh: int = 3, seed: int = 1, sigma: float = 32.0, land: float = 0.30,
            nlevels: int = CONFIG2_LEVELS):
    """Returns (param dict, level-1 vertex mask, raw RHS noise) for config 2;
    the RHS is masked and mean-removed with the post-setup mask by ``rhs``."""
    wet, rng = coastline_cells(n, seed, sigma * n / 4096.0, land)
    t = n + 2 * nh
    cells = np.zeros((t, t, 1), dtype=np.uint8, order="F")
    cells[nh:nh + n, nh:nh + n, 0] = wet
    vmsk = F.get_mask_at_corners(cells)
    noise = np.asfortranarray(rng.standard_normal((t, t, 1)))
    param = dict(nx=n, ny=n, nz=1, nh=nh, case="twod", location="vertices", operator="laplacian9", cycle="f",
                 nlevels=nlevels, npre=3, npost=3, omega=0.8, ndeepest=20)
    return param, vmsk, noise


def config1(n: int = 256, nh: int = 3, seed: int = 0):
    t = n + 2 * nh
    msk = F.get_circular_domain((t, t, 1), nh=nh, radius=0.45)
    noise = np.asfortranarray(np.random.default_rng(seed).standard_normal((t, t, 1)))
    param = dict(nx=n, ny=n, nz=1, nh=nh, case="twod", location="centers", operator="laplacian", cycle="v",
                 nlevels=6, npre=2, npost=2, omega=0.8, ndeepest=20)
    return param, msk, noise


def rhs(noise, msk_after_setup):
    m = msk_after_setup.astype(np.float64)
    b = np.asfortranarray(noise * m)
    F.subtract_mean(b, m)
    return b


def config4(ninst: int = 2048, seed: int = 3, lo: int = 64, hi: int = 1024, nh: int = 3):
    """Batched config: sizes log-uniform in [lo, hi], rounded to a multiple of
    32; per instance a disk (r = 0.45) or a smoothed-noise coastline mask,
    50/50, and an N(0,1) RHS. Levels go down to a coarsest grid of 8-15
    cells. Returns a list of (n, nlevels, cell mask, rhs noise).

    The noise coastline is smoothed with sigma = N/8 and only its largest
    wet region is kept. With the grid-scale sigma = max(1, 32 N/4096), the
    reference's coverage-thresholded coarsening cannot represent the domain
    and its cell-centred (Neumann) cycles stall near 0.95 per cycle (CPU
    oracle); an isolated wet pocket also makes a global-mean-free RHS
    inconsistent."""
    from concurrent.futures import ThreadPoolExecutor
    import os

    from scipy.ndimage import label

    rng = np.random.default_rng(seed)
    draws = []  # the random stream, in the order it is drawn
    for _ in range(ninst):
        n = int(32 * round(np.exp(rng.uniform(np.log(lo), np.log(hi))) / 32))
        n = max(32, n)
        noise = rng.standard_normal((n, n)) if rng.uniform() >= 0.5 else None
        rhs = np.asfortranarray(rng.standard_normal((n + 2 * nh, n + 2 * nh, 1)))
        draws.append((n, noise, rhs))

    def build(d):
        n, noise, rhs = d
        nlev = int(np.floor(np.log2(n / 8))) + 1
        t = n + 2 * nh
        if noise is None:
            msk = F.get_circular_domain((t, t, 1), nh=nh, radius=0.45)
        else:
            sm = gaussian_smooth(noise, n / 8.0)
            msk = np.zeros((t, t, 1), dtype=np.uint8, order="F")
            msk[nh:nh + n, nh:nh + n, 0] = sm > np.quantile(sm, 0.30)
            lab, nl = label(msk[:, :, 0] > 0)
            if nl > 1:
                keep = 1 + int(np.argmax(np.bincount(lab.ravel())[1:]))
                msk = np.asfortranarray((lab == keep).astype(np.uint8)[:, :, None])
        return (n, nlev, msk, rhs)

    # the FFTs and the labelling release the GIL
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(build, draws))


def config5(ninst: int = 16, n: int = 2048, seed: int = 4, nh: int = 3):
    """Adjoint config: ninst 2D cell-centred variable-coefficient problems,
    div(kappa grad x) = b, kappa = exp(0.5 * gaussian_filter(N(0,1), 16))
    (normalised to unit standard deviation of the smoothed field), disk
    mask r = 0.45, b ~ N(0,1) on wet cells with the mean removed, and a
    target x* ~ N(0,1) (seed 4). Returns (param dict, list of (msk, kappa,
    b, xstar))."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    t = n + 2 * nh
    msk = F.get_circular_domain((t, t, 1), nh=nh, radius=0.45)
    out = []
    for _ in range(ninst):
        g = gaussian_filter(rng.standard_normal((t, t)), 16.0, mode="reflect", truncate=4.0)
        kap = np.asfortranarray(np.exp(0.5 * g / g.std())[:, :, None])
        b = np.asfortranarray(rng.standard_normal((t, t, 1)))
        xs = np.asfortranarray(rng.standard_normal((t, t, 1)))
        out.append((msk, kap, b, xs))
    nlev = int(np.floor(np.log2(n / 8))) + 1
    param = dict(nx=n, ny=n, nz=1, nh=nh, case="twod", location="centers", operator="varcoef", cycle="v", npre=2,
                 npost=2, omega=0.8, ndeepest=20, nlevels=nlev)
    return param, out


def config3(nx: int = 512, ny: int = 512, nz: int = 256, nh: int = 3, seed: int = 2, land: float = 0.30,
            nlevels: int = 8, coast_sigma: float = 32.0, depth_sigma: float = 4.0):
    """3D cell-centred 7-point config: the config-2 coastline recipe at
    nx x ny (smoothed noise, sigma = 32 cells, 30 % land) extruded in z,
    cut by a bottom topography: a column (i, j) is wet for k <= depth(i, j),
    with depth = nz * gaussian_filter(U[0.2, 1], 4 cells). With the
    coastline smoothed at 4 cells instead (32 scaled by 512/4096), the
    reference's V-cycle stalls near 0.9 per cycle (CPU oracle, full size):
    the coverage-thresholded coarse masks cut the narrow channels. Only the largest
    face-connected wet region is kept: the operator is Neumann, and an
    isolated pocket would make a mean-free right-hand side inconsistent.
    RHS N(0,1) on wet cells (the wet mean is removed by ``rhs``). Returns
    (param dict, level-1 mask, raw RHS noise)."""
    from scipy.ndimage import gaussian_filter, label

    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((nx, ny))
    sm = gaussian_filter(noise, coast_sigma, mode="reflect", truncate=4.0)
    coast = sm > np.quantile(sm, land)
    depth = nz * gaussian_filter(rng.uniform(0.2, 1.0, (nx, ny)), depth_sigma, mode="reflect", truncate=4.0)
    k = np.arange(1, nz + 1)
    wet = coast[:, :, None] & (k[None, None, :] <= depth[:, :, None])
    lab, nl = label(wet)
    if nl > 1:
        keep = 1 + int(np.argmax(np.bincount(lab.ravel())[1:]))
        wet = lab == keep
    del lab
    tx, ty, tz = nx + 2 * nh, ny + 2 * nh, nz + 2 * nh
    msk = np.zeros((tx, ty, tz), dtype=np.uint8, order="F")
    msk[nh:nh + nx, nh:nh + ny, nh:nh + nz] = wet
    rhs_noise = np.asfortranarray(rng.standard_normal((tx, ty, tz)))
    param = dict(nx=nx, ny=ny, nz=nz, nh=nh, case="threed", location="centers", operator="laplacian", cycle="v",
                 nlevels=nlevels, npre=2, npost=2, omega=0.8, ndeepest=20)
    return param, msk, rhs_noise
