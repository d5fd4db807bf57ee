"""Seeded synthetic STA acquisitions (the workloads' stand-in for recorded RF).

Each A-scan (tx, rx) is the sum over point scatterers s of
  a_s * p(t - (|e_tx - s| + |s - e_rx|) / c)
with p a Gaussian-modulated cosine at fc (fractional bandwidth `bw` at -6 dB,
the convention of scipy.signal.gausspulse), plus N(0, noise_std) noise.
Scatterer draws come first, then noise, from one numpy PCG64 generator.
The numpy path (float64, then rounded to float32) serves tests; the torch
path computes the same sum in float32 on any device (used for the large
benchmark frames).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np


@dataclass
class Scatterers:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    amp: np.ndarray

    def __len__(self) -> int:
        return int(self.x.size)

    @staticmethod
    def concat(*parts: "Scatterers") -> "Scatterers":
        return Scatterers(*(np.concatenate([getattr(p, f) for p in parts]) for f in ("x", "y", "z", "amp")))


def point_scatterers(rng: np.random.Generator, n: int, x_range: Tuple[float, float],
                     z_range: Tuple[float, float], amp_range: Tuple[float, float] = (0.5, 1.0),
                     y_range: Optional[Tuple[float, float]] = None) -> Scatterers:
    x = rng.uniform(x_range[0], x_range[1], n)
    y = rng.uniform(y_range[0], y_range[1], n) if y_range else np.zeros(n)
    z = rng.uniform(z_range[0], z_range[1], n)
    a = rng.uniform(amp_range[0], amp_range[1], n)
    return Scatterers(x, y, z, a)


def speckle(rng: np.random.Generator, n: int, x_range: Tuple[float, float], z_range: Tuple[float, float],
            sigma: float = 0.1) -> Scatterers:
    """Background scatterers with Rayleigh-distributed amplitudes and random sign."""
    x = rng.uniform(x_range[0], x_range[1], n)
    z = rng.uniform(z_range[0], z_range[1], n)
    a = rng.rayleigh(sigma, n) * rng.choice(np.array([-1.0, 1.0]), n)
    return Scatterers(x, np.zeros(n), z, a)


def gauss_coefficient(fc: float, bw: float = 0.6, bwr_db: float = -6.0) -> float:
    """Envelope exp(-a t^2) with a = -(pi fc bw)^2 / (4 ln 10^(bwr/20))."""
    ref = 10.0 ** (bwr_db / 20.0)
    return -(math.pi * fc * bw) ** 2 / (4.0 * math.log(ref))


def _half_width(a: float, fs: float) -> int:
    # exp(-a t^2) < 1e-8 beyond t = sqrt(18.4 / a).
    return int(math.ceil(math.sqrt(18.5 / a) * fs)) + 1


def synth_rf_numpy(tx_xy: np.ndarray, rx_xy: np.ndarray, scat: Scatterers, fs: float, c: float, fc: float,
                   num_samples: int, rng: np.random.Generator, noise_std: float = 0.01,
                   bw: float = 0.6, chunk: int = 64) -> np.ndarray:
    """(num_tx, num_rx, num_samples) float32 RF."""
    tx_xy = np.asarray(tx_xy, np.float64)
    rx_xy = np.asarray(rx_xy, np.float64)
    ntx, nrx = tx_xy.shape[0], rx_xy.shape[0]
    a = gauss_coefficient(fc, bw)
    hw = _half_width(a, fs)
    rf = np.zeros(ntx * nrx * num_samples, np.float64)
    offs = np.arange(-hw, hw + 1)
    base = (np.arange(ntx)[:, None] * nrx + np.arange(nrx)[None, :]) * num_samples  # (ntx, nrx)
    for s0 in range(0, len(scat), chunk):
        sl = slice(s0, min(len(scat), s0 + chunk))
        sx, sy, sz, sa = scat.x[sl], scat.y[sl], scat.z[sl], scat.amp[sl]
        dtx = np.sqrt((sx[None, :] - tx_xy[:, 0:1]) ** 2 + (sy[None, :] - tx_xy[:, 1:2]) ** 2 + sz[None, :] ** 2)
        drx = np.sqrt((sx[None, :] - rx_xy[:, 0:1]) ** 2 + (sy[None, :] - rx_xy[:, 1:2]) ** 2 + sz[None, :] ** 2)
        tau = (dtx[:, None, :] + drx[None, :, :]) / c                     # (ntx, nrx, S)
        n0 = np.floor(tau * fs).astype(np.int64)
        n = n0[..., None] + offs                                          # (ntx, nrx, S, W)
        t = n / fs - tau[..., None]
        v = sa[None, None, :, None] * np.exp(-a * t * t) * np.cos(2.0 * math.pi * fc * t)
        ok = (n >= 0) & (n < num_samples)
        idx = base[:, :, None, None] + n
        np.add.at(rf, idx[ok], v[ok])
    rf = rf.reshape(ntx, nrx, num_samples)
    if noise_std > 0:
        rf += rng.normal(0.0, noise_std, rf.shape)
    return rf.astype(np.float32)


def synth_rf_torch(tx_xy, rx_xy, scat: Scatterers, fs: float, c: float, fc: float, num_samples: int,
                   seed: int, noise_std: float = 0.01, bw: float = 0.6, device="cpu", chunk: int = 128):
    """Same model as synth_rf_numpy, evaluated in float32 with torch on `device`."""
    import torch
    dev = torch.device(device)
    tx = torch.as_tensor(np.asarray(tx_xy, np.float32), device=dev)
    rx = torch.as_tensor(np.asarray(rx_xy, np.float32), device=dev)
    ntx, nrx = tx.shape[0], rx.shape[0]
    a = gauss_coefficient(fc, bw)
    hw = _half_width(a, fs)
    rf = torch.zeros(ntx * nrx * num_samples, dtype=torch.float32, device=dev)
    offs = torch.arange(-hw, hw + 1, device=dev)
    base = ((torch.arange(ntx, device=dev)[:, None] * nrx + torch.arange(nrx, device=dev)[None, :]) * num_samples)
    S = torch.as_tensor(np.stack([scat.x, scat.y, scat.z, scat.amp]).astype(np.float32), device=dev)
    for s0 in range(0, len(scat), chunk):
        sx, sy, sz, sa = S[:, s0:s0 + chunk]
        dtx = torch.sqrt((sx[None] - tx[:, 0:1]) ** 2 + (sy[None] - tx[:, 1:2]) ** 2 + sz[None] ** 2)
        drx = torch.sqrt((sx[None] - rx[:, 0:1]) ** 2 + (sy[None] - rx[:, 1:2]) ** 2 + sz[None] ** 2)
        tau = (dtx[:, None, :] + drx[None, :, :]) / c
        n0 = torch.floor(tau * fs).to(torch.int64)
        n = n0[..., None] + offs
        t = n.to(torch.float32) / fs - tau[..., None]
        v = sa[None, None, :, None] * torch.exp(-a * t * t) * torch.cos(2.0 * math.pi * fc * t)
        ok = (n >= 0) & (n < num_samples)
        idx = (base[:, :, None, None] + n)[ok]
        rf.index_add_(0, idx, v[ok])
    rf = rf.view(ntx, nrx, num_samples)
    if noise_std > 0:
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        rf += noise_std * torch.randn(rf.shape, generator=g, device=dev, dtype=torch.float32)
    return rf


def synth_rf_pairs_torch(tx_xy, rx_xy, scat: Scatterers, fs: float, c: float, fc: float, num_samples: int,
                         seed: int, noise_std: float = 0.01, bw: float = 0.6, device="cpu", chunk: int = 64):
    """(n, num_samples) float32 RF of the n (tx_xy[i], rx_xy[i]) pairs (one
    A-scan per pair: the T1R1 / SAFT acquisition when tx = rx), same echo
    model as synth_rf_numpy."""
    import torch
    dev = torch.device(device)
    tx = torch.as_tensor(np.asarray(tx_xy, np.float32), device=dev)
    rx = torch.as_tensor(np.asarray(rx_xy, np.float32), device=dev)
    n = tx.shape[0]
    a = gauss_coefficient(fc, bw)
    hw = _half_width(a, fs)
    rf = torch.zeros(n * num_samples, dtype=torch.float32, device=dev)
    offs = torch.arange(-hw, hw + 1, device=dev)
    base = torch.arange(n, device=dev)[:, None, None] * num_samples
    S = torch.as_tensor(np.stack([scat.x, scat.y, scat.z, scat.amp]).astype(np.float32), device=dev)
    for s0 in range(0, len(scat), chunk):
        sx, sy, sz, sa = S[:, s0:s0 + chunk]
        dtx = torch.sqrt((sx[None] - tx[:, 0:1]) ** 2 + (sy[None] - tx[:, 1:2]) ** 2 + sz[None] ** 2)
        drx = torch.sqrt((sx[None] - rx[:, 0:1]) ** 2 + (sy[None] - rx[:, 1:2]) ** 2 + sz[None] ** 2)
        tau = (dtx + drx) / c                                            # (n, S)
        nidx = torch.floor(tau * fs).to(torch.int64)[..., None] + offs   # (n, S, W)
        t = nidx.to(torch.float32) / fs - tau[..., None]
        v = sa[None, :, None] * torch.exp(-a * t * t) * torch.cos(2.0 * math.pi * fc * t)
        ok = (nidx >= 0) & (nidx < num_samples)
        rf.index_add_(0, (base + nidx)[ok], v[ok])
    rf = rf.view(n, num_samples)
    if noise_std > 0:
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        rf += noise_std * torch.randn(rf.shape, generator=g, device=dev, dtype=torch.float32)
    return rf


def two_medium_travel_times(elem_x: np.ndarray, interface_xz: np.ndarray, points_xz: np.ndarray, c1: float,
                            c2: float) -> np.ndarray:
    """(num_elements, num_points) one-way travel time from elements at
    (x, 0) in medium 1 to points in medium 2 through the sampled interface:
    the minimum over the interface points (Fermat's principle, brute force)."""
    ex = np.asarray(elem_x, np.float64)[:, None, None]
    ix = np.asarray(interface_xz, np.float64)[None, :, 0:1]
    iz = np.asarray(interface_xz, np.float64)[None, :, 1:2]
    px = np.asarray(points_xz, np.float64)[None, None, :, 0]
    pz = np.asarray(points_xz, np.float64)[None, None, :, 1]
    t = np.sqrt((ix - ex) ** 2 + iz ** 2) / c1 + np.sqrt((px - ix) ** 2 + (pz - iz) ** 2) / c2   # (E, I, P)
    return t.min(axis=1)


def synth_rf_two_medium_numpy(tx_x: np.ndarray, rx_x: np.ndarray, interface_xz: np.ndarray, scat_xz: np.ndarray,
                              amp: np.ndarray, fs: float, c1: float, c2: float, fc: float, num_samples: int,
                              rng: np.random.Generator, noise_std: float = 0.0, bw: float = 0.6,
                              start_offset: int = 0) -> np.ndarray:
    """(num_tx, num_rx, num_samples) float32 RF of point scatterers in medium 2
    seen through the interface; samples before `start_offset` are dropped
    (the dead zone cut of the two-medium method)."""
    ttx = two_medium_travel_times(tx_x, interface_xz, scat_xz, c1, c2)   # (T, S)
    trx = two_medium_travel_times(rx_x, interface_xz, scat_xz, c1, c2)   # (R, S)
    a = gauss_coefficient(fc, bw)
    hw = _half_width(a, fs)
    ntx, nrx = ttx.shape[0], trx.shape[0]
    rf = np.zeros(ntx * nrx * num_samples, np.float64)
    offs = np.arange(-hw, hw + 1)
    base = (np.arange(ntx)[:, None] * nrx + np.arange(nrx)[None, :]) * num_samples
    tau = ttx[:, None, :] + trx[None, :, :] - start_offset / fs                  # (T, R, S)
    n0 = np.floor(tau * fs).astype(np.int64)
    n = n0[..., None] + offs
    t = n / fs - tau[..., None]
    v = np.asarray(amp, np.float64)[None, None, :, None] * np.exp(-a * t * t) * np.cos(2.0 * math.pi * fc * t)
    ok = (n >= 0) & (n < num_samples)
    np.add.at(rf, (base[:, :, None, None] + n)[ok], v[ok])
    rf = rf.reshape(ntx, nrx, num_samples)
    if noise_std > 0:
        rf += rng.normal(0.0, noise_std, rf.shape)
    return rf.astype(np.float32)
