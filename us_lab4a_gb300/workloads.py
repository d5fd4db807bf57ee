"""Seeded STA workloads with the shapes of the benchmark configurations.

  plain2d      32-element linear array, pitch 0.3 mm, fc 5 MHz, fs 40 MHz,
               2048 samples, 8 point scatterers (x U[-4,4] mm, z U[10,40] mm,
               a U[0.5,1]), 4x upsampling, rectangular apodization, no CF,
               128 x 256 grid over x [-5,5] mm, z [5,45] mm.
  cf2d         64 elements, 4096 samples, 32 points + 20 000 Rayleigh speckle
               scatterers (z [5,60] mm), 8x upsampling, Blackman apodization,
               512 x 512 grid over x [-9.6,9.6] mm, z [5,60] mm; CF = PCF/SCF/MF.
  matrix3d     16 x 16 matrix array, pitch 0.3 mm, fc 3 MHz, fs 24 MHz, 1024
               samples, 64 points in x,y [-5,5] mm, z [5,45] mm, 4x upsampling,
               64 x 64 x 128 voxels over the same volume, CF, FP16/BF16 storage.
  mixed        frames drawn from {32,64,96,128} elements x {1024,2048,4096}
               samples x {128x128, 256x256, 512x1024} grids x CF on/off,
               16 scatterers each, 4x upsampling (the mixed-size batch).
  two_medium   linear array in water (c1 1480 m/s) over a cylinder of a
               second medium (c2 2700 m/s, radius 15 mm, top at 15 mm): the
               interface is the upper arc (-170..-10 degrees) sampled every
               lambda2 / 4, a sub-aperture stepped across the array, one
               transmit element or every element per step (STA), scatterers
               inside the cylinder, grid below the top of the cylinder.
Grid extents and upsampling of the mixed frames are not fixed by the
workload descriptions; the values above are this library's choice.
Each workload also has a reduced "small" form for CPU-oracle parity tests.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import List, Optional

import numpy as np

from .config import element_positions_matrix, element_x_centered_2d, window
from .engine import FrameSpec
from . import synth

C_SOUND = 1540.0


@dataclass
class Frame:
    name: str
    spec: FrameSpec
    grid_xyz: np.ndarray                 # (ncols, nrows, 3) float32
    scatterers: synth.Scatterers
    seed: int
    rf: Optional[np.ndarray] = None      # (num_tx, num_rx, num_samples) float32 (host)

    @property
    def npix(self) -> int:
        return int(self.grid_xyz.shape[0] * self.grid_xyz.shape[1])

    def make_rf_numpy(self) -> np.ndarray:
        if self.rf is None:
            s = self.spec
            rng = np.random.default_rng(self.seed + 1)
            self.rf = synth.synth_rf_numpy(s.tx_xy, s.rx_xy, self.scatterers, s.sampling_frequency,
                                           s.propagation_speed, s.center_frequency, s.num_samples, rng)
        return self.rf

    def make_rf_torch(self, device):
        s = self.spec
        return synth.synth_rf_torch(s.tx_xy, s.rx_xy, self.scatterers, s.sampling_frequency, s.propagation_speed,
                                    s.center_frequency, s.num_samples, seed=self.seed + 1, device=device)


def linear_array(n: int, pitch: float = 0.3e-3) -> np.ndarray:
    x = element_x_centered_2d(n, pitch, np.float32)
    return np.stack([x, np.zeros_like(x)], axis=1)


def grid_xz(x0, x1, ncols, z0, z1, nrows) -> np.ndarray:
    xs = np.linspace(x0, x1, ncols, dtype=np.float64).astype(np.float32)
    zs = np.linspace(z0, z1, nrows, dtype=np.float64).astype(np.float32)
    g = np.zeros((ncols, nrows, 3), np.float32)
    g[:, :, 0] = xs[:, None]
    g[:, :, 2] = zs[None, :]
    return g


def grid_xyz3(x0, x1, nx, y0, y1, ny, z0, z1, nz) -> np.ndarray:
    xs = np.linspace(x0, x1, nx).astype(np.float32)
    ys = np.linspace(y0, y1, ny).astype(np.float32)
    zs = np.linspace(z0, z1, nz).astype(np.float32)
    g = np.zeros((nx * ny, nz, 3), np.float32)
    xx, yy = np.meshgrid(xs, ys, indexing="ij")
    g[:, :, 0] = xx.reshape(-1)[:, None]
    g[:, :, 1] = yy.reshape(-1)[:, None]
    g[:, :, 2] = zs[None, :]
    return g


def plain2d(seed: int = 1000, small: bool = False, tiny: bool = False) -> Frame:
    n, ns, ncols, nrows = (32, 2048, 128, 256) if not small else (16, 512, 24, 40)
    if tiny:
        small, (n, ns, ncols, nrows) = True, (12, 320, 16, 24)
    rng = np.random.default_rng(seed)
    zr = (10e-3, 40e-3) if not small else (5e-3, 9e-3)
    scat = synth.point_scatterers(rng, 8, (-4e-3, 4e-3), zr)
    el = linear_array(n)
    spec = FrameSpec(tx_xy=el, rx_xy=el, num_samples=ns, upsampling=4, sampling_frequency=40e6,
                     propagation_speed=C_SOUND, center_frequency=5e6, rx_apod=window("rectangular", n))
    g = grid_xz(-5e-3, 5e-3, ncols, 5e-3, 45e-3, nrows) if not small else grid_xz(-4e-3, 4e-3, ncols, 4e-3, 10e-3, nrows)
    return Frame("plain2d" + ("-small" if small else ""), spec, g, scat, seed)


def cf2d(seed: int = 1001, small: bool = False, coherence: str = "pcf", num_speckle: Optional[int] = None,
         tiny: bool = False) -> Frame:
    n, ns, ncols, nrows, U = (64, 4096, 512, 512, 8) if not small else (16, 640, 32, 32, 8)
    if tiny:
        small, (n, ns, ncols, nrows, U) = True, (12, 400, 20, 20, 8)
    rng = np.random.default_rng(seed)
    if small:
        pts = synth.point_scatterers(rng, 6, (-2e-3, 2e-3), (4e-3, 9e-3))
        spk = synth.speckle(rng, 200 if num_speckle is None else num_speckle, (-3e-3, 3e-3), (3e-3, 11e-3))
        g = grid_xz(-3e-3, 3e-3, ncols, 3e-3, 11e-3, nrows)
    else:
        pts = synth.point_scatterers(rng, 32, (-8e-3, 8e-3), (10e-3, 55e-3))
        spk = synth.speckle(rng, 20000 if num_speckle is None else num_speckle, (-9.6e-3, 9.6e-3), (5e-3, 60e-3))
        g = grid_xz(-9.6e-3, 9.6e-3, ncols, 5e-3, 60e-3, nrows)
    el = linear_array(n)
    spec = FrameSpec(tx_xy=el, rx_xy=el, num_samples=ns, upsampling=U, sampling_frequency=40e6,
                     propagation_speed=C_SOUND, center_frequency=5e6, rx_apod=window("blackman", n),
                     coherence=coherence)
    return Frame("cf2d" + ("-small" if small else ""), spec, g, synth.Scatterers.concat(pts, spk), seed)


def matrix3d(seed: int = 1002, small: bool = False, coherence: str = "pcf", storage: str = "f16",
             tiny: bool = False) -> Frame:
    nx, ns, (gx, gy, gz) = (16, 1024, (64, 64, 128)) if not small else (6, 384, (8, 8, 16))
    if tiny:
        small, nx, ns, (gx, gy, gz) = True, 4, 256, (6, 6, 12)
    rng = np.random.default_rng(seed)
    zr = (5e-3, 45e-3) if not small else (4e-3, 12e-3)
    scat = synth.point_scatterers(rng, 64 if not small else 8, (-5e-3, 5e-3), zr, y_range=(-5e-3, 5e-3))
    el = element_positions_matrix(0.3e-3, nx, 0.0, 0.3e-3, nx, 0.0, np.float32)
    spec = FrameSpec(tx_xy=el, rx_xy=el, num_samples=ns, upsampling=4, sampling_frequency=24e6,
                     propagation_speed=C_SOUND, center_frequency=3e6, rx_apod=np.ones(el.shape[0], np.float32),
                     coherence=coherence, storage=storage)
    g = grid_xyz3(-5e-3, 5e-3, gx, -5e-3, 5e-3, gy, zr[0], zr[1], gz)
    return Frame("matrix3d" + ("-small" if small else ""), spec, g, scat, seed)


MIXED_ELEMENTS = (32, 64, 96, 128)
MIXED_SAMPLES = (1024, 2048, 4096)
MIXED_GRIDS = ((128, 128), (256, 256), (512, 1024))


def mixed(num_frames: int = 48, seed: int = 1003, storage: str = "f16", upsampling: int = 4,
          small: bool = False) -> List[Frame]:
    """Mixed-size frames (element count, samples, grid and CF drawn per frame)."""
    rng = np.random.default_rng(seed)
    frames = []
    for i in range(num_frames):
        if small:
            n = int(rng.choice((8, 12, 16)))
            ns = int(rng.choice((256, 384, 512)))
            ncols, nrows = [(16, 16), (24, 20), (32, 24)][int(rng.integers(3))]
        else:
            n = int(rng.choice(MIXED_ELEMENTS))
            ns = int(rng.choice(MIXED_SAMPLES))
            ncols, nrows = MIXED_GRIDS[int(rng.integers(3))]
        cf_on = bool(rng.integers(2))
        fseed = seed * 1000 + i
        frng = np.random.default_rng(fseed)
        el = linear_array(n)
        half = float(el[-1, 0]) if n > 1 else 1e-3
        depth = (ns / 40e6) * C_SOUND / 2.0
        z1 = min(45e-3, depth * 0.9)
        z0 = min(5e-3, z1 * 0.2)
        scat = synth.point_scatterers(frng, 16, (-0.8 * half, 0.8 * half), (z0 + 0.1 * (z1 - z0), z1))
        spec = FrameSpec(tx_xy=el, rx_xy=el, num_samples=ns, upsampling=upsampling, sampling_frequency=40e6,
                         propagation_speed=C_SOUND, center_frequency=5e6, rx_apod=window("rectangular", n),
                         coherence="pcf" if cf_on else "none", storage=storage)
        frames.append(Frame(f"mixed{i}", spec, grid_xz(-half, half, ncols, z0, z1, nrows), scat, fseed))
    return frames


def large_serving_frame(seed: int = 1004, storage: str = "f16") -> Frame:
    """The 10 % large frames of the serving mix: 128 elements, 4096 samples,
    1024 x 1024 grid, Blackman apodization, 8x upsampling, SCF."""
    rng = np.random.default_rng(seed)
    el = linear_array(128)
    half = float(el[-1, 0])
    scat = synth.point_scatterers(rng, 16, (-0.8 * half, 0.8 * half), (8e-3, 60e-3))
    spec = FrameSpec(tx_xy=el, rx_xy=el, num_samples=4096, upsampling=8, sampling_frequency=40e6,
                     propagation_speed=C_SOUND, center_frequency=5e6, rx_apod=window("blackman", 128),
                     coherence="scf", storage=storage)
    return Frame("large", spec, grid_xz(-half, half, 1024, 5e-3, 60e-3, 1024), scat, seed)


def with_storage(frame: Frame, storage: str) -> Frame:
    return replace(frame, spec=replace(frame.spec, storage=storage))


@dataclass
class TwoMediumScene:
    """Inputs of VectorialCombinedTwoMediumImagingProcessor: configuration
    fields, per-step acquisitions, steps, interface, apodization and grid."""
    num_elements: int
    num_elements_mux: int
    pitch: float
    center_frequency: float
    propagation_speed_1: float
    propagation_speed_2: float
    sampling_frequency: float
    upsampling: int
    steps: np.ndarray            # (num_steps, 4) uint32: baseElemIdx, baseElem, firstTxElem, lastTxElem
    interface_xz: np.ndarray     # (m, 2) float32
    rx_apod: np.ndarray          # (num_elements,) float32
    grid_xz: np.ndarray          # (ncols, nrows, 2) float32
    rf: np.ndarray               # (num_steps, num_tx, num_elements, num_samples) float32
    max_fermat_block_size: float = 2.0
    peak_offset: float = 1.5
    signal_start_offset: int = 0

    @property
    def num_samples(self) -> int:
        return int(self.rf.shape[3])


def two_medium_scene(one_tx: bool, num_elements: int = 32, num_elements_mux: int = 64, num_steps: int = 8,
                     num_samples: int = 2000, upsampling: int = 4, grid=(128, 256), tx_element: int = 0,
                     sampling_frequency: float = 40e6, num_scatterers: int = 24, noise_std: float = 0.01,
                     seed: int = 1005) -> TwoMediumScene:
    pitch, fc, c1, c2, fs = 0.6e-3, 5e6, 1480.0, 2700.0, sampling_frequency
    rng = np.random.default_rng(seed)
    R, cz = 15e-3, 30e-3
    lam2 = c2 / fc
    a1, a2 = np.deg2rad(-170.0), np.deg2rad(-10.0)
    m = int(np.ceil((a2 - a1) / (lam2 / (4 * R)))) + 1
    ang = np.linspace(a1, a2, m)
    ifxz = np.stack([R * np.cos(ang), cz + R * np.sin(ang)], axis=1).astype(np.float32)
    xs = np.linspace(-8e-3, 8e-3, grid[0])
    zs = np.linspace(14e-3, 40e-3, grid[1])
    grid_xz = np.stack(np.meshgrid(xs, zs, indexing="ij"), axis=-1).astype(np.float32)
    base = np.round(np.linspace(0, num_elements_mux - num_elements, num_steps)).astype(np.uint32)
    steps = np.array([[i, b, tx_element, tx_element] if one_tx else [i, b, 0, num_elements - 1]
                      for i, b in enumerate(base)], np.uint32)
    x = (np.arange(num_elements_mux) * pitch - (num_elements_mux - 1) * pitch / 2).astype(np.float64)
    # Scatterers inside the cylinder (a disc of radius 12 mm around the axis).
    rr = 12e-3 * np.sqrt(rng.uniform(0.0, 1.0, num_scatterers))
    th = rng.uniform(0.0, 2 * np.pi, num_scatterers)
    scat = np.stack([rr * np.cos(th), cz + rr * np.sin(th)], axis=1)
    amp = rng.uniform(0.5, 1.0, num_scatterers)
    start = 7
    ntx = 1 if one_tx else num_elements
    rf = np.zeros((num_steps, ntx, num_elements, num_samples), np.float32)
    for i, b in enumerate(base):
        sub = x[b:b + num_elements]
        tx = sub[tx_element:tx_element + 1] if one_tx else sub
        rf[i] = synth.synth_rf_two_medium_numpy(tx, sub, ifxz, scat, amp, fs, c1, c2, fc, num_samples, rng,
                                                noise_std=noise_std, start_offset=start)
    apod = np.hanning(num_elements + 2)[1:-1].astype(np.float32)
    return TwoMediumScene(num_elements=num_elements, num_elements_mux=num_elements_mux, pitch=pitch,
                          center_frequency=fc, propagation_speed_1=c1, propagation_speed_2=c2,
                          sampling_frequency=fs, upsampling=upsampling, steps=steps, interface_xz=ifxz,
                          rx_apod=apod, grid_xz=grid_xz, rf=rf, max_fermat_block_size=2.0, peak_offset=1.5,
                          signal_start_offset=start)
