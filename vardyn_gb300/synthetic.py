"""Seeded synthetic inputs standing in for the reference's altimetry example.

The reference's only recorded run uses real along-track altimetry over the
Gulf Stream (mapping/examples/2021a_SSH_mapping_OSE, data not shipped). Its
benchmarks here run on seeded synthetic fields and tracks of the same kind:

- ``kminus3_ssh``: an isotropic SSH field with a k^-3 power spectrum, no power
  at wavelengths shorter than a cutoff, scaled to a target RMS;
- ``satellite_tracks``: straight tracks at random angles crossing the domain,
  one pass time per track (rounded to a model step), points every
  ``spacing_km``, values interpolated from a truth field plus Gaussian noise.

All generators take a ``numpy.random.Generator`` so every input is reproducible
from its seed.
"""
import numpy as np


def kminus3_ssh(ny, nx, dx, dy, rng, rms=0.1, cutoff_km=50.0, slope=-3.0):
    """Random SSH field [m] with |H(k)|^2 ~ k^slope, zero power for
    wavelengths below ``cutoff_km``, zero mean and the given RMS."""
    kx = np.fft.fftfreq(nx, d=dx)
    ky = np.fft.fftfreq(ny, d=dy)
    K = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    amp = np.zeros_like(K)
    nz = K > 0
    amp[nz] = K[nz] ** (slope / 2.0)
    amp[K > 1.0 / (cutoff_km * 1e3)] = 0.0
    spec = amp * (rng.standard_normal(K.shape) + 1j * rng.standard_normal(K.shape))
    field = np.real(np.fft.ifft2(spec))
    field -= field.mean()
    std = field.std()
    if std > 0:
        field *= rms / std
    return field


def satellite_tracks(ny, nx, dx, dy, nstep, n_obs, rng, spacing_km=7.0,
                     points_per_track=None):
    """Straight seeded tracks inside the grid.

    Returns ``(x_km, y_km, step)`` arrays of length ``n_obs``: planar obs
    coordinates measured from grid point (0, 0) and the model step index
    (1..nstep) at which each track is observed. Tracks are laid until
    ``n_obs`` points are placed; each track keeps only points at least two
    cells inside the domain."""
    Lx = (nx - 1) * dx / 1e3
    Ly = (ny - 1) * dy / 1e3
    margin_x = 2 * dx / 1e3
    margin_y = 2 * dy / 1e3
    xs, ys, ts = [], [], []
    total = 0
    while total < n_obs:
        ang = rng.uniform(0, np.pi)
        cx = rng.uniform(0.25 * Lx, 0.75 * Lx)
        cy = rng.uniform(0.25 * Ly, 0.75 * Ly)
        half = np.hypot(Lx, Ly)
        s = np.arange(-half, half, spacing_km)
        px = cx + s * np.cos(ang)
        py = cy + s * np.sin(ang)
        keep = (px >= margin_x) & (px <= Lx - margin_x) & \
            (py >= margin_y) & (py <= Ly - margin_y)
        px, py = px[keep], py[keep]
        if points_per_track is not None:
            px, py = px[:points_per_track], py[:points_per_track]
        if px.size == 0:
            continue
        px, py = px[:n_obs - total], py[:n_obs - total]
        step = int(rng.integers(1, nstep + 1))
        xs.append(px)
        ys.append(py)
        ts.append(np.full(px.size, step, dtype=np.int64))
        total += px.size
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(ts)
