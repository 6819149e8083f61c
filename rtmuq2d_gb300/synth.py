"""Seeded synthetic inputs for the RTM workloads (numpy/scipy only).

The reference ships no velocity models or seismograms (its Marmousi2 inputs are listed as
missing), so every workload is built here from a seed:

* ``ricker``            800-sample Ricker wavelet (the reference reads 800 float32 samples,
                        SRC/fixed_parameters.h:57, rtm_iso2d.c:72).
* ``grf``               unit-variance Gaussian random field with a given correlation length.
* ``layered_model``     three flat layers times (1 + 0.02 g): the 400 x 200 plain workload.
* ``faulted_model``     water layer over 12-16 folded, faulted layers with a high-velocity
                        ellipse: the 3400 x 700 plain workload.
* ``ensemble_member``   exp(0.03 g_k) perturbation of a model: UQ realizations.
* ``smooth``            Gaussian smoothing (migration velocity from the true model).

Models are returned as float32 [x][z] arrays (x-major, z contiguous) like the
reference's .bin files.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def ricker(f0: float, dt: float, n: int = 800, t0: float | None = None) -> np.ndarray:
    t0 = 1.2 / f0 if t0 is None else t0
    t = np.arange(n, dtype=np.float64) * dt - t0
    a = (np.pi * f0 * t) ** 2
    return ((1.0 - 2.0 * a) * np.exp(-a)).astype(np.float32)


def grf(shape, dx: float, corr_len: float, seed: int) -> np.ndarray:
    """Unit-variance Gaussian random field with Gaussian covariance of length corr_len (m)."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal(shape)
    sigma = max(corr_len / dx / np.sqrt(2.0), 0.5)
    g = ndimage.gaussian_filter(white, sigma=sigma, mode="wrap")
    g -= g.mean()
    sd = g.std()
    return g / sd if sd > 0 else g


def smooth(model: np.ndarray, sigma_m: float, dx: float) -> np.ndarray:
    return ndimage.gaussian_filter(model.astype(np.float64), sigma=sigma_m / dx,
                                   mode="nearest").astype(np.float32)


def layered_model(nx: int, nz: int, dx: float, seed: int,
                  velocities=(1500.0, 2000.0, 2500.0), interfaces=(600.0, 1300.0),
                  perturb: float = 0.02, corr_len: float = 100.0) -> np.ndarray:
    z = np.arange(nz) * dx
    v = np.full(nz, velocities[0])
    for zi, vi in zip(interfaces, velocities[1:]):
        v[z >= zi] = vi
    model = np.broadcast_to(v, (nx, nz)).astype(np.float64)
    g = grf((nx, nz), dx, corr_len, seed)
    return (model * (1.0 + perturb * g)).astype(np.float32)


def faulted_model(nx: int, nz: int, dx: float, seed: int) -> np.ndarray:
    """Water (450 m, 1500 m/s) over 12-16 folded layers cut by 4 normal faults; velocity
    rises with depth from 1600 to 4700 m/s; a 4500 m/s ellipse at 2 km depth."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * dx
    z = np.arange(nz) * dx
    water = 450.0
    n_layers = int(rng.integers(12, 17))
    zmax = z[-1] + dx
    bases = np.sort(rng.uniform(water + 60.0, zmax - 40.0, n_layers - 1))
    # folded interfaces: sums of 3-5 sinusoids, amplitude 20-150 m, wavelength 1-6 km
    tops = np.empty((n_layers - 1, nx))
    for j, b in enumerate(bases):
        k = int(rng.integers(3, 6))
        amp = rng.uniform(20.0, 150.0, k) / k
        lam = rng.uniform(1000.0, 6000.0, k)
        ph = rng.uniform(0, 2 * np.pi, k)
        tops[j] = b + (amp[:, None] * np.sin(2 * np.pi * x[None, :] / lam[:, None] + ph[:, None])).sum(0)
    vel_layers = np.linspace(1600.0, 4700.0, n_layers) * rng.uniform(0.97, 1.03, n_layers)
    vel_layers = np.clip(vel_layers, 1600.0, 4700.0)
    X, Z = np.meshgrid(x, z, indexing="ij")
    # normal faults: planes x = xf + (z - water) / tan(dip); hanging wall shifted down
    shift = np.zeros_like(X)
    for _ in range(4):
        xf = rng.uniform(0.1, 0.9) * x[-1]
        dip = np.deg2rad(rng.uniform(50.0, 70.0))
        throw = rng.uniform(30.0, 120.0)
        side = 1.0 if rng.uniform() < 0.5 else -1.0
        hanging = side * (X - (xf + (Z - water) / np.tan(dip))) > 0
        shift += np.where(hanging & (Z > water), throw, 0.0)
    zs = Z - shift
    layer = np.zeros(X.shape, dtype=np.int64)
    for j in range(n_layers - 1):
        layer += (zs >= tops[j][:, None]).astype(np.int64)
    v = vel_layers[layer]
    v = np.where(Z < water, 1500.0, v)
    # high-velocity ellipse at 2 km depth
    xc = rng.uniform(0.3, 0.7) * x[-1]
    zc = min(2000.0, 0.8 * zmax)
    ax, az = rng.uniform(600.0, 1200.0), rng.uniform(150.0, 300.0)
    inside = ((X - xc) / ax) ** 2 + ((Z - zc) / az) ** 2 <= 1.0
    v = np.where(inside, 4500.0, v)
    return v.astype(np.float32)


def ensemble_member(model: np.ndarray, dx: float, seed: int, sigma: float = 0.03,
                    corr_len: float = 200.0) -> np.ndarray:
    g = grf(model.shape, dx, corr_len, seed)
    return (model.astype(np.float64) * np.exp(sigma * g)).astype(np.float32)


def grf_coarse(shape, dx: float, corr_len: float, seed: int, factor: int = 4) -> np.ndarray:
    """grf() generated on a grid `factor` times coarser and interpolated (linear) back:
    the same covariance to within the interpolation smoothing when corr_len spans many
    cells, at a fraction of the cost on large grids."""
    cs = tuple(max(2, -(-n // factor) + 1) for n in shape)
    g = grf(cs, dx * factor, corr_len, seed)
    zoom = tuple((n - 1) / (c - 1) for n, c in zip(shape, cs))
    out = ndimage.zoom(g, zoom, order=1, mode="nearest", grid_mode=False)[: shape[0], : shape[1]]
    out = out - out.mean()
    sd = out.std()
    return out / sd if sd > 0 else out
