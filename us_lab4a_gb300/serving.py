"""Continuous-batching serving loop for STA frames on one GPU.

Requests (frames of different array sizes, sample counts, grids and
coherence factors) arrive over time. A request is admitted when a batch slot
is free and its resident device state fits the HBM budget; admitted requests
are launched together as one batch (persistent preparation and
delay-and-sum launches, replayed from a CUDA graph), on one of two streams,
so a new batch is admitted and launched while the previous one is still on
the GPU. Each in-flight frame owns a slot - a context (tables, grid, signal
tensor) plus its RF and output buffers - that stays resident and is recycled
for the next frame of the same class. Latency is measured from arrival to
the image being back in host memory.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

from .batch import Batch, BatchItem
from .engine import FrameSpec, StaEngine


@dataclass
class Request:
    rid: int
    spec: FrameSpec
    grid_xyz: np.ndarray          # (ncols, nrows, 3) float32
    rf: object                    # pinned host torch tensor (num_tx, num_rx, num_samples) float32
    arrival: float                # seconds after the start of the run
    value: Optional[np.ndarray] = None
    factor: Optional[np.ndarray] = None
    done: Optional[float] = None

    @property
    def latency(self) -> Optional[float]:
        return None if self.done is None else self.done - self.arrival


def frame_key(spec: FrameSpec, grid_xyz: np.ndarray) -> Tuple:
    """Frames with the same key can share a resident slot (same parameters,
    same element positions, the same grid array object)."""
    return (spec.num_tx, spec.num_rx, spec.num_samples, spec.upsampling, spec.coherence, spec.storage,
            spec.real_path, spec.sampling_frequency, spec.propagation_speed, spec.center_frequency,
            spec.peak_offset, spec.dead_zone_m, spec.pcf_gamma, spec.scf_p,
            spec.tx_xy.tobytes(), spec.rx_xy.tobytes(),
            None if spec.rx_apod is None else np.asarray(spec.rx_apod, np.float32).tobytes(),
            grid_xyz.shape, id(grid_xyz))


@dataclass
class Slot:
    key: Tuple
    engine: StaEngine
    rf: object
    value: object
    factor: object
    host_value: object
    host_factor: object
    nbytes: int


@dataclass
class _InFlight:
    index: int
    event: object
    work: List[Tuple[Request, Slot]]


class ServingLoop:
    def __init__(self, hbm_budget_bytes: int, max_batch: int = 48, max_elements: int = 128,
                 use_graph: bool = True, device="cuda:0", das_config: Optional[Tuple[int, int, int]] = None,
                 plain: bool = False, per_frame: bool = False):
        """plain=True serves the plain form instead: every admitted frame is
        processed on its own (one preparation launch and one plain
        delay-and-sum launch per frame); per_frame=True also processes every
        admitted frame on its own, but with the context's default (staged,
        autoselected) delay-and-sum kernel. Both are for comparison with the
        batched form."""
        import torch
        self.torch = torch
        self.device = torch.device(device)
        self.budget = int(hbm_budget_bytes)
        self.max_batch = max_batch
        self.use_graph = use_graph
        self.plain = plain
        self.per_frame = plain or per_frame
        self.batches = [Batch(max_batch, max_elements), Batch(max_batch, max_elements)]
        if das_config:
            for b in self.batches:
                if len(das_config) == 4:  # (variant, rows, stage bytes, stages), as Batch.autotune returns
                    b.set_das_config(das_config[1], das_config[2], das_config[3], variant=das_config[0])
                else:                     # (rows, stage bytes, stages)
                    b.set_das_config(*das_config)
        self.streams = [torch.cuda.Stream(device=self.device), torch.cuda.Stream(device=self.device)]
        self.idle: Dict[Tuple, List[Slot]] = {}
        self.used_bytes = 0
        self.peak_bytes = 0
        self.slots_created = 0

    # ------------------------------------------------------------------ slots
    def _slot_bytes(self, spec: FrameSpec, grid_xyz: np.ndarray) -> int:
        L = spec.num_samples * (4 if spec.real_path else spec.upsampling)
        esize = (1 if spec.real_path else 2) * (4 if spec.storage == "f32" else 2)
        npix = grid_xyz.shape[0] * grid_xyz.shape[1]
        rf = spec.num_tx * spec.num_rx * spec.num_samples * 4
        sig = spec.num_tx * spec.num_rx * (((L + 7) // 8) * 8) * esize
        # context RF + our RF + tensor + grid (context copy and ours) + 2 outputs x 2
        return 2 * rf + sig + npix * 4 * (3 + 3 + 4)

    def _acquire(self, req: Request) -> Optional[Slot]:
        key = frame_key(req.spec, req.grid_xyz)
        pool = self.idle.get(key)
        if pool:
            return pool.pop()
        nbytes = self._slot_bytes(req.spec, req.grid_xyz)
        if self.used_bytes + nbytes > self.budget:
            # Free idle slots of other classes to make room.
            for k in list(self.idle):
                while self.idle[k] and self.used_bytes + nbytes > self.budget:
                    self._destroy(self.idle[k].pop())
            if self.used_bytes + nbytes > self.budget:
                return None
        torch = self.torch
        eng = StaEngine(req.spec)
        if self.plain:
            eng.set_das_variant(0)
        g = torch.as_tensor(np.ascontiguousarray(req.grid_xyz, np.float32), device=self.device)
        eng.set_grid_device(g)
        torch.cuda.synchronize(self.device)
        shape = req.grid_xyz.shape[:2]
        slot = Slot(key, eng, torch.empty(req.rf.shape, dtype=torch.float32, device=self.device),
                    torch.empty(shape, dtype=torch.float32, device=self.device),
                    torch.empty(shape, dtype=torch.float32, device=self.device),
                    torch.empty(shape, dtype=torch.float32).pin_memory(),
                    torch.empty(shape, dtype=torch.float32).pin_memory(), nbytes)
        self.used_bytes += nbytes
        self.peak_bytes = max(self.peak_bytes, self.used_bytes)
        self.slots_created += 1
        return slot

    def _release(self, slot: Slot) -> None:
        self.idle.setdefault(slot.key, []).append(slot)

    def _destroy(self, slot: Slot) -> None:
        slot.engine.close()
        self.used_bytes -= slot.nbytes

    def close(self) -> None:
        for pool in self.idle.values():
            for s in pool:
                self._destroy(s)
        self.idle.clear()
        for b in self.batches:
            b.close()

    # ------------------------------------------------------------------- run
    def run(self, requests: List[Request], keep_images: bool = True) -> Dict:
        torch = self.torch
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        queue: deque = deque()
        inflight: List[_InFlight] = []
        free = [0, 1]
        t0 = time.perf_counter()
        launched = 0
        batch_sizes = []
        while pending or queue or inflight:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            # Retire finished batches.
            for fl in list(inflight):
                if fl.event.query():
                    t_done = time.perf_counter() - t0
                    for req, slot in fl.work:
                        req.done = t_done
                        if keep_images:
                            req.value = slot.host_value.numpy().copy()
                            req.factor = slot.host_factor.numpy().copy()
                        self._release(slot)
                    inflight.remove(fl)
                    free.append(fl.index)
            # Admit and launch while a batch object is free.
            if queue and free:
                work: List[Tuple[Request, Slot]] = []
                while queue and len(work) < self.max_batch:
                    slot = self._acquire(queue[0])
                    if slot is None:
                        break  # over budget: wait for a batch to retire
                    work.append((queue.popleft(), slot))
                if work:
                    idx = free.pop(0)
                    stream = self.streams[idx]
                    with torch.cuda.stream(stream):
                        for req, slot in work:
                            slot.rf.copy_(req.rf, non_blocking=True)
                        if self.per_frame:
                            for _, slot in work:
                                slot.engine.set_stream(stream)
                                slot.engine.process_device(slot.rf, slot.value, slot.factor)
                        else:
                            items = [BatchItem(slot.engine, slot.rf, slot.value, slot.factor) for _, slot in work]
                            self.batches[idx].run(items, stream, use_graph=self.use_graph)
                        for _, slot in work:
                            slot.host_value.copy_(slot.value, non_blocking=True)
                            slot.host_factor.copy_(slot.factor, non_blocking=True)
                        ev = torch.cuda.Event()
                        ev.record(stream)
                    inflight.append(_InFlight(idx, ev, work))
                    launched += 1
                    batch_sizes.append(len(work))
                    continue
            if not queue and not inflight and pending:
                time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - t0), 0.001)))
            elif inflight:
                time.sleep(0.00005)
        for b in self.batches:
            b.synchronize()
        wall = time.perf_counter() - t0
        lat = np.array([r.latency for r in requests])
        return {
            "frames": len(requests), "wall_s": wall,
            "frames_per_s": len(requests) / (max(r.done for r in requests) - min(r.arrival for r in requests)),
            "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
            "batches": launched, "mean_batch": float(np.mean(batch_sizes)) if batch_sizes else 0.0,
            "peak_resident_bytes": self.peak_bytes, "slots_created": self.slots_created,
        }


def poisson_arrivals(n: int, rate: float, seed: int) -> np.ndarray:
    """n arrival times (s) of a Poisson process of `rate` frames/s."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n))
