"""Image post-processing on the GPU: the envelope along each image column and
the conversion to decibels (the reference's "Envelope - dB" image). Wraps
usgb_post_* of include/usgb.h."""
from __future__ import annotations

import ctypes as C

from . import native


class PostProcessor:
    """For images of `num_samples` rows (grid nrows), column-major as the
    processors write them (value[col][row])."""

    def __init__(self, num_samples: int):
        self._lib = native.load()
        h = C.c_void_p()
        rc = self._lib.usgb_post_create(num_samples, C.byref(h))
        if rc != 0:
            from .errors import from_status
            raise from_status(rc, self._lib.usgb_post_last_error(None).decode())
        self._h = h
        self.num_samples = num_samples

    def _check(self, rc: int) -> None:
        if rc != 0:
            from .errors import from_status
            raise from_status(rc, self._lib.usgb_post_last_error(self._h).decode())

    def envelope(self, image, out=None, stream=None):
        """|analytic signal| of every column of `image` (torch CUDA float32,
        (ncols, nrows)); returns `out` (may be `image`)."""
        import torch
        assert image.is_cuda and image.dtype == torch.float32 and image.is_contiguous()
        assert image.shape[-1] == self.num_samples
        out = torch.empty_like(image) if out is None else out
        s = stream if stream is not None else torch.cuda.current_stream()
        ncols = image.numel() // self.num_samples
        self._check(self._lib.usgb_post_envelope_device(self._h, C.c_void_p(image.data_ptr()), C.c_void_p(out.data_ptr()),
                                                        ncols, C.c_void_p(getattr(s, "cuda_stream", s))))
        return out

    def decibels(self, image, min_db: float, stream=None):
        """In place: image / max|image|, then 20 log10, floored at min_db."""
        import torch
        assert image.is_cuda and image.dtype == torch.float32 and image.is_contiguous()
        s = stream if stream is not None else torch.cuda.current_stream()
        self._check(self._lib.usgb_post_decibels_device(self._h, C.c_void_p(image.data_ptr()), image.numel(),
                                                        float(min_db), C.c_void_p(getattr(s, "cuda_stream", s))))
        return image

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.usgb_post_destroy(self._h)
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
