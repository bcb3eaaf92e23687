"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference ships no data (its inputs lived under a private path,
fwi_files_path.h:1), so models, acquisitions and wavelets are generated here
from fixed seeds:

* ``c1``  201 x 401, dx 10 m, dt 1 ms, nt 2000, CPML 20, layered 1500-4500 m/s
          + depth gradient + 3 Gaussian anomalies (+-300 m/s, sigma 150 m);
          8 surface shots, 10 Hz Ricker, 200 receivers at 2 m depth.
* ``c2``  560 x 1700, dx 10 m, dt 0.8 ms, nt 4000, CPML 20, faulted layered
          model 1500-5500 m/s with 12 dipping layers and 3 normal faults
          (50-150 m throw); 64 shots, 1700 receivers, 8 Hz Ricker.
* ``c3``  600 x 2000, dx 10 m, dt 1 ms, 256 shots with nt ~ U[3000, 6000]
          (rounded to the sampling interval), off-end spreads of 200-1200
          receivers with offsets up to 8 km, 5-12 Hz Ricker.
* ``c4``  2000 x 6000, dx 5 m, dt 0.5 ms, nt 8000, 32 shots.
* ``c5``  800 x 2400, dx 10 m, dt 1 ms, 128 shots.

Grids are given as nz x nx (depth first, like NZ x NX in Mpar.h:13-14).
Starting models are the true models smoothed by a separable triangle filter
(two box passes per axis, the construction of triangle_smooth.c:36-68).
``scale`` shrinks a configuration (grid, shots, time) for quick runs while
keeping its structure.
"""
from __future__ import annotations

import numpy as np

from fwigpu import ShotSpec

CONFIGS = {
    "c1": dict(nz=201, nx=401, dx=10.0, dt=0.001, nt=2000, npml=20, nshots=8, nrec=200, f0=10.0,
               vmin=1500.0, vmax=4500.0, model="layered", seed=1234),
    "c2": dict(nz=560, nx=1700, dx=10.0, dt=0.0008, nt=4000, npml=20, nshots=64, nrec=1700, f0=8.0,
               vmin=1500.0, vmax=5500.0, model="faulted", seed=2024),
    "c3": dict(nz=600, nx=2000, dx=10.0, dt=0.001, nt=(3000, 6000), npml=20, nshots=256, nrec=(200, 1200),
               f0=(5.0, 12.0), vmin=1500.0, vmax=4500.0, model="faulted", seed=3033, offend=8000.0),
    "c4": dict(nz=2000, nx=6000, dx=5.0, dt=0.0005, nt=8000, npml=20, nshots=32, nrec=1200, f0=10.0,
               vmin=1500.0, vmax=4500.0, model="faulted", seed=4044),
    "c5": dict(nz=800, nx=2400, dx=10.0, dt=0.001, nt=4000, npml=20, nshots=128, nrec=800, f0=10.0,
               vmin=1500.0, vmax=4500.0, model="layered", seed=5055),
}


def ricker(nt: int, dt: float, f0: float, t0: float | None = None) -> np.ndarray:
    t0 = 1.2 / f0 if t0 is None else t0
    a = (np.pi * f0 * (np.arange(nt) * dt - t0)) ** 2
    return ((1.0 - 2.0 * a) * np.exp(-a)).astype(np.float32)


def _box(a: np.ndarray, n: int, axis: int) -> np.ndarray:
    """Centred running mean of length n with edge replication."""
    if n <= 1:
        return a
    lo, hi = n // 2, n - 1 - n // 2
    pad = [(0, 0)] * a.ndim
    pad[axis] = (lo + 1, hi)
    c = np.cumsum(np.pad(a, pad, mode="edge"), axis=axis, dtype=np.float64)
    m = a.shape[axis]
    sl_hi = [slice(None)] * a.ndim
    sl_lo = [slice(None)] * a.ndim
    sl_hi[axis] = slice(n, n + m)
    sl_lo[axis] = slice(0, m)
    return (c[tuple(sl_hi)] - c[tuple(sl_lo)]) / n


def triangle_smooth(a: np.ndarray, r: int) -> np.ndarray:
    out = np.asarray(a, np.float64)
    for axis in (0, 1):
        out = _box(_box(out, r, axis), r, axis)
    return out.astype(np.float32)


def layered_model(nz, nx, dx, vmin, vmax, seed, nlayers=6, n_anom=3, anom=300.0, sigma=150.0):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[:, None] * dx
    x = np.arange(nx)[None, :] * dx
    depth = nz * dx
    iface = np.sort(rng.uniform(0.1, 0.9, nlayers - 1)) * depth
    vel_l = np.linspace(vmin, vmax - 600.0, nlayers) + rng.uniform(-100, 100, nlayers)
    v = np.full((nz, nx), vel_l[0])
    for k, zi in enumerate(iface):
        undul = 40.0 * np.sin(2 * np.pi * x / (nx * dx) * (k + 1) + rng.uniform(0, 6.28))
        v = np.where(z >= zi + undul, vel_l[k + 1], v)
    v = v + 600.0 * z / depth                     # linear depth gradient
    for _ in range(n_anom):
        cx, cz = rng.uniform(0.2, 0.8) * nx * dx, rng.uniform(0.25, 0.75) * depth
        s = rng.choice([-1.0, 1.0])
        v = v + s * anom * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * sigma ** 2))
    return np.clip(v, vmin, vmax).astype(np.float32)


def faulted_model(nz, nx, dx, vmin, vmax, seed, nlayers=12, nfaults=3):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[:, None] * dx
    x = np.arange(nx)[None, :] * dx
    depth, length = nz * dx, nx * dx
    base = np.sort(rng.uniform(0.05, 0.95, nlayers)) * depth
    dips = rng.uniform(-0.08, 0.08, nlayers)
    vel_l = np.linspace(vmin, vmax, nlayers + 1)
    # normal faults: a dipping fault plane; the hanging wall (x beyond the plane) drops by the throw
    shift = np.zeros((nz, nx))
    for _ in range(nfaults):
        xf = rng.uniform(0.2, 0.8) * length
        dip = rng.uniform(0.5, 1.5)
        throw = rng.uniform(50.0, 150.0)
        shift = shift + np.where(x > xf + z / np.tan(dip), throw, 0.0)
    zz = z - shift
    v = np.full((nz, nx), vel_l[0])
    for k in range(nlayers):
        v = np.where(zz >= base[k] + dips[k] * (x - 0.5 * length), vel_l[k + 1], v)
    return np.clip(v, vmin, vmax).astype(np.float32)


def _pick(v, rng):
    return rng.uniform(*v) if isinstance(v, tuple) else v


def build(name: str, scale: float = 1.0, nshots: int | None = None, nt: int | None = None,
          jump: int = 1, smooth: int = 30):
    """Returns (config kwargs for fwigpu.make_config, true model, start model, shots)."""
    c = dict(CONFIGS[name])
    rng = np.random.default_rng(c["seed"])
    nz = max(16, int(round(c["nz"] * scale)))
    nx = max(16, int(round(c["nx"] * scale)))
    dx = c["dx"]
    if c["model"] == "layered":
        true = layered_model(nz, nx, dx, c["vmin"], c["vmax"], c["seed"])
    else:
        true = faulted_model(nz, nx, dx, c["vmin"], c["vmax"], c["seed"])
    start = triangle_smooth(true, max(1, int(round(smooth * scale))))
    ns = nshots if nshots is not None else max(1, int(round(c["nshots"] * min(1.0, scale))))
    length = nx * dx
    shots = []
    nt_max = 0
    for s in range(ns):
        if isinstance(c["nt"], tuple):
            n = int(rng.integers(c["nt"][0], c["nt"][1] + 1)) if nt is None else nt
        else:
            n = c["nt"] if nt is None else nt
        n = max(jump + 1, int(round(n * (scale if nt is None else 1.0))))
        n = (n - 1) // jump * jump + 1                 # (nt-1) % jump == 0 (fwi_2d.c:195)
        nt_max = max(nt_max, n)
        f0 = _pick(c["f0"], rng)
        sx = (s + 0.5) / ns * length
        if "offend" in c:                              # off-end spread behind the source
            nr = int(rng.integers(c["nrec"][0], c["nrec"][1] + 1))
            nr = max(2, int(round(nr * scale)))
            span = min(c["offend"] * scale, length - dx)
            side = -1.0 if sx > length / 2 else 1.0
            rx = sx + side * np.linspace(dx, span, nr)
            rx = np.clip(rx, 0.0, length - dx)
        else:
            nr = max(2, int(round(c["nrec"] * scale)))
            rx = np.linspace(0.0, length - dx, nr)
        rec = np.stack([rx, np.full(nr, 2.0)], axis=1)  # receivers at 2 m depth
        shots.append(ShotSpec(sx, 10.0, rec, ricker(n, c["dt"], f0)))
    cfg = dict(nx=nx, nz=nz, dx=dx, dz=dx, dt=c["dt"], nt_max=nt_max, npml=c["npml"], jump=jump)
    return cfg, true, start, shots
