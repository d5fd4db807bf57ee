"""Batched frames: many STA frames of different sizes in two persistent
launches (preparation over every A-scan of every frame, staged delay-and-sum
over every grid tile of every frame), optionally replayed from a captured CUDA
graph. Wraps usgb_batch_* of include/usgb.h."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

from . import native
from .engine import StaEngine


@dataclass
class BatchItem:
    engine: StaEngine   # frame parameters, tables, grid (set_grid_device) and signal tensor
    rf: object          # torch CUDA tensor (num_tx, num_rx, num_samples) float32
    value: object       # torch CUDA tensor (ncols, nrows) float32
    factor: object      # torch CUDA tensor (ncols, nrows) float32


class Batch:
    def __init__(self, max_frames: int, max_elements: int, max_signal_length: int = 0):
        self._lib = native.load()
        h = C.c_void_p()
        rc = self._lib.usgb_batch_create(max_frames, max_elements, max_signal_length, C.byref(h))
        if rc != 0:
            self._raise_create(rc)
        self._h = h
        self.max_frames = max_frames
        self.das_config = None  # library default until set
        self._keep = None

    def _raise_create(self, rc):
        from .errors import from_status
        raise from_status(rc, self._lib.usgb_batch_last_error(None).decode())

    def _check(self, rc: int) -> None:
        if rc != 0:
            from .errors import from_status
            raise from_status(rc, self._lib.usgb_batch_last_error(self._h).decode())

    # (variant, tile rows, stage bytes, stages) tried by autotune(), most likely first;
    # variant 3 is the receiver-group kernel on 64-column tiles.
    CANDIDATES = ((4, 7, 102400, 2), (4, 7, 65536, 2), (4, 4, 102400, 2), (4, 4, 65536, 2), (4, 4, 49152, 2),
                  (4, 8, 102400, 2), (4, 8, 65536, 2),
                  (3, 8, 98304, 2), (3, 8, 65536, 2), (2, 16, 98304, 2),
                  (3, 4, 32768, 2), (3, 4, 49152, 2), (3, 8, 49152, 2), (3, 4, 24576, 3), (2, 8, 24576, 2),
                  (2, 8, 32768, 2), (2, 4, 32768, 2), (2, 4, 24576, 2), (2, 8, 20480, 2),
                  (2, 4, 16384, 2), (1, 8, 24576, 3), (1, 4, 32768, 2), (1, 4, 16384, 2))

    def set_das_config(self, tile_rows: int, stage_bytes: int, stages: int, variant: int = None) -> None:
        """Tile shape of the batched delay-and-sum; variant 2 = receiver-group
        kernel on 32-column tiles, 3 = on 64-column tiles, 4 = on 64 x 2*rows
        tiles with two points per thread (rows 4, 7 or 8), 1 = staged kernel
        (None keeps the current one)."""
        if variant is not None and variant != getattr(self, "_variant", 2):
            # Shrink first so that the variant switch fits, then set the shape.
            self._check(self._lib.usgb_batch_set_das_config(self._h, 4, 8192, 2))
            self._check(self._lib.usgb_batch_set_das_variant(self._h, variant))
            self._variant = variant
        self._check(self._lib.usgb_batch_set_das_config(self._h, tile_rows, stage_bytes, stages))
        self.das_config = (getattr(self, "_variant", 2), tile_rows, stage_bytes, stages)

    def autotune(self, items: Sequence[BatchItem], stream, candidates=None, repeats: int = 1):
        """Time the whole batch (graph replay) under each kernel / tile shape
        that fits and keep the fastest. Returns ((variant, rows, stage_bytes,
        stages), ms)."""
        import torch
        best = None
        for cfg in candidates or self.CANDIDATES:
            try:
                self.set_das_config(cfg[1], cfg[2], cfg[3], variant=cfg[0])
            except Exception:
                continue  # does not fit in shared memory for max_elements
            self.run(items, stream, use_graph=True)  # capture
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(repeats):
                self.run(items, stream, use_graph=True)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / repeats
            if best is None or ms < best[1]:
                best = (cfg, ms)
        if best is None:
            raise RuntimeError("no staged delay-and-sum shape fits this batch")
        v, rows, cap, nst = best[0]
        self.set_das_config(rows, cap, nst, variant=v)
        return best

    def run(self, items: Sequence[BatchItem], stream, use_graph: bool = True) -> None:
        """Enqueue the batch on `stream` (torch.cuda.Stream or raw handle)."""
        arr = (native.BatchItem * len(items))()
        for i, it in enumerate(items):
            arr[i].ctx = it.engine._h
            arr[i].d_rf = it.rf.data_ptr()
            arr[i].d_value = it.value.data_ptr()
            arr[i].d_factor = it.factor.data_ptr()
        self._keep = (arr, list(items))  # tensors stay referenced until the next run
        ptr = getattr(stream, "cuda_stream", stream)
        self._check(self._lib.usgb_batch_run(self._h, arr, len(items), C.c_void_p(ptr), int(use_graph)))

    def synchronize(self) -> None:
        self._check(self._lib.usgb_batch_synchronize(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.usgb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
