"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference's own geophysical example reads MERRA-2 winds, which are not
available offline; the stand-in is a divergence-free random flow:

  * grid: lon = linspace(-100, 35, 217), lat = linspace(-5, 45, 101),
    t = 3 * arange(121) hours (nt x nlon x nlat = 121 x 217 x 101, float64);
  * streamfunction psi = sum over 256 modes of a_m cos(k_m . (x, y) - w_m t + phi_m)
    with x = R cos(20 deg) lon pi/180, y = R lat pi/180 in km (R = 6371),
    |k| log-uniform in [2 pi/5000, 2 pi/100] 1/km, uniform direction and phase,
    w_m = c_m |k_m| with c_m ~ U(-10, 10) km/h, |a_m| ~ |k|^-2 (energy
    spectrum ~ k^-3), drawn from numpy ``default_rng(seed)``;
  * u = -d psi/dy, v = d psi/dx (km/h), rescaled to an rms speed of 40 km/h
    over the sample grid.
"""
import math

import numpy as np
import torch

R_EARTH = 6371.0


def geo_grid():
    lon = np.linspace(-100.0, 35.0, 217)
    lat = np.linspace(-5.0, 45.0, 101)
    t = 3.0 * np.arange(121, dtype=np.float64)
    return t, lon, lat


def geo_modes(seed=0, nmodes=256):
    rng = np.random.default_rng(seed)
    kmag = np.exp(rng.uniform(math.log(2 * math.pi / 5000.0), math.log(2 * math.pi / 100.0), nmodes))
    theta = rng.uniform(0.0, 2 * math.pi, nmodes)
    phi = rng.uniform(0.0, 2 * math.pi, nmodes)
    c = rng.uniform(-10.0, 10.0, nmodes)
    amp = kmag ** -2.0
    return kmag * np.cos(theta), kmag * np.sin(theta), c * kmag, phi, amp


def geo_velocity(seed=0, device=None, t=None, lon=None, lat=None, nmodes=256):
    """(t, lon, lat, U, V) of the synthetic geophysical flow; U, V (nt, nlon, nlat) km/h.

    Computed with torch on `device` (CUDA when available), returned as numpy.
    """
    if t is None:
        t, lon, lat = geo_grid()
    kx, ky, w, phi, amp = geo_modes(seed, nmodes)
    dev = torch.device(device) if device is not None else (
        torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu"))
    T = torch.as_tensor(t, dtype=torch.float64, device=dev)
    X = torch.as_tensor(R_EARTH * math.cos(math.radians(20.0)) * np.radians(lon), dtype=torch.float64,
                        device=dev)
    Y = torch.as_tensor(R_EARTH * np.radians(lat), dtype=torch.float64, device=dev)
    U = torch.zeros((len(t), len(lon), len(lat)), dtype=torch.float64, device=dev)
    V = torch.zeros_like(U)
    for m in range(len(kx)):
        ph = (kx[m] * X[None, :, None] + ky[m] * Y[None, None, :]) - w[m] * T[:, None, None] + phi[m]
        s = torch.sin(ph)
        # psi = a cos(ph): u = -dpsi/dy = a ky sin(ph), v = dpsi/dx = -a kx sin(ph)
        U += (amp[m] * ky[m]) * s
        V -= (amp[m] * kx[m]) * s
    rms = torch.sqrt(torch.mean(U * U + V * V))
    scale = 40.0 / rms
    U *= scale
    V *= scale
    return t, lon, lat, U.cpu().numpy(), V.cpu().numpy()


def geo_ftle_grid(spacing=0.2):
    """Particle grid of the geophysical FTLE workload (0.2 deg -> 676 x 251)."""
    lonf = np.arange(-100.0, 35.0 + spacing, spacing)
    latf = np.arange(-5.0, 45.0 + spacing, spacing)
    return lonf, latf


# the geophysical FTLE workload: t0 = 180 h, T = -72 h, spherical = 1,
# params = [-1], DOP853 rtol 1e-6 / atol 1e-8, ridge percentile 90
GEO_T0, GEO_T, GEO_PERCENTILE = 180.0, -72.0, 90


def geo_batch_specs(seed=1, nfields=48):
    """The batched time-series workload on the geophysical flow: 48 fields at
    hourly t0 = 168 + k h, T ~ U[-120, -24] h and grid spacing drawn from
    {0.1, 0.2, 0.4} deg (1351x501, 676x251 or 338x126 particles), numpy
    ``default_rng(seed)``.  Returns [(t0, T, spacing)]."""
    rng = np.random.default_rng(seed)
    T = rng.uniform(-120.0, -24.0, nfields)
    sp = rng.choice([0.1, 0.2, 0.4], nfields)
    return [(168.0 + k, float(T[k]), float(sp[k])) for k in range(nfields)]


def bickley_batch_grid(nx=1001, ny=301):
    """Bickley jet particle grid over its domain (0, pi * 6.371) x (-3, 3) Mm."""
    return np.linspace(0.0, np.pi * 6.371, nx), np.linspace(-3.0, 3.0, ny)


# Bickley jet field of the batch: t0 = 0, T = 40 days, default parameters
BICKLEY_T0, BICKLEY_T = 0.0, 40.0


def double_gyre_grid(nx=401, ny=201):
    return np.linspace(0.0, 2.0, nx), np.linspace(0.0, 1.0, ny)
