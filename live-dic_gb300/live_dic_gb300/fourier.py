"""Global-translation initializer (drop-in for live_dic.fourier).

Follows FourierInitializer (fourier.py:16-111): the reference window (at most
1024^2, a power of two) is chosen on the host exactly as there (the centre
window, else the best-textured of nine candidate windows by ROI coverage x
standard deviation); the phase correlation itself -- mean removal, 2x2
averaging, Hann taper, zero-padded float64 FFTs, normalised cross power
spectrum, inverse FFT, peak score, overlap and sample correlation -- runs on
the GPU (csrc/fourier.cu).  The acceptance rule is the reference's: peak score
>= 8, overlap >= 0.25, correlation >= 0.2; an ambiguous target raises
ValueError with the reference's message.
"""

from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _native


class FourierInitializer:
    def __init__(self, reference: np.ndarray, mask: np.ndarray | None = None, *, device: int = 0) -> None:
        if mask is not None:
            mask = np.asarray(mask, dtype=bool)
        reference = np.asarray(reference)
        height, width = reference.shape
        size = 1 << min(10, min(width, height).bit_length() - 1)
        if size < 32:
            raise ValueError("Fourier initialization needs an image of at least 32 pixels per side")
        best = None
        positions = [(0.5, 0.5)] + [(x, y) for y in (0, 0.5, 1) for x in (0, 0.5, 1)]
        for fx, fy in positions:
            x, y = int((width - size) * fx), int((height - size) * fy)
            patch = reference[y: y + size, x: x + size].astype(np.float64)
            allowed = np.ones(patch.shape, bool) if mask is None else mask[y: y + size, x: x + size]
            coverage = float(np.mean(allowed))
            std = float(np.std(patch[allowed])) if allowed.any() else 0.0
            if coverage >= 0.25 and std >= 1.0:
                candidate = (coverage * std, x, y, allowed.copy())
                if best is None or candidate[0] > best[0]:
                    best = candidate
                if fx == fy == 0.5 and coverage >= 0.5:
                    break
        if best is None:
            raise ValueError("Fourier initialization has no sufficiently textured ROI window")
        _, x, y, allowed = best
        self._window = dict(x=x, y=y, size=size, sampleStep=2)
        self.shape = reference.shape
        self.size = size
        self._lib = _native.load()
        window = np.ascontiguousarray(reference[y: y + size, x: x + size], dtype=np.uint8)
        allow = None if mask is None else np.ascontiguousarray(allowed, dtype=np.uint8)
        handle = C.c_void_p()
        code = self._lib.gbdic_fourier_create(int(device), _native.ptr(window), _native.ptr(allow), size, C.byref(handle))
        _native.check(code, self._lib.gbdic_fourier_last_error(None))
        self._handle = handle

    @property
    def window(self) -> dict:
        return dict(self._window)

    def _raw(self, current, *, device_pointer: int | None = None, row_stride: int | None = None) -> np.ndarray:
        out = np.zeros(7, np.float64)
        x, y = self._window["x"], self._window["y"]
        if device_pointer is not None:
            code = self._lib.gbdic_fourier_estimate(self._handle, C.c_void_p(device_pointer), int(row_stride),
                                                    self.shape[0], x, y, 1, _native.ptr(out))
        else:
            frame = np.ascontiguousarray(current, dtype=np.uint8)
            code = self._lib.gbdic_fourier_estimate(self._handle, _native.ptr(frame), frame.strides[0], frame.shape[0],
                                                    x, y, 0, _native.ptr(out))
        _native.check(code, self._lib.gbdic_fourier_last_error(self._handle))
        return out

    def estimate(self, current: np.ndarray) -> dict:
        started = time.perf_counter()
        if current.shape != self.shape:
            raise ValueError("Fourier target dimensions must match the prepared reference")
        r = self._raw(current)
        return self._accept(r, started)

    def estimate_device(self, device_pointer: int, row_stride: int) -> dict:
        """Estimate from a device-resident target (dense or strided rows)."""
        started = time.perf_counter()
        return self._accept(self._raw(None, device_pointer=device_pointer, row_stride=row_stride), started)

    def _accept(self, r: np.ndarray, started: float) -> dict:
        if r[6] < 1.0:
            raise ValueError("Fourier initialization rejected a target window without texture")
        dx, dy, score, overlap, correlation = int(r[0]), int(r[1]), float(r[2]), float(r[3]), float(r[4])
        if score < 8.0 or overlap < 0.25 or correlation < 0.2:
            raise ValueError(
                f"Fourier initialization is ambiguous (peak score {score:.2f}, overlap {overlap:.3f}); "
                "no local field was calculated"
            )
        return dict(dx=dx, dy=dy, peakScore=score, overlap=overlap, correlation=correlation, window=self.window,
                    method="linear-phase-correlation", wallMs=(time.perf_counter() - started) * 1000)

    def close(self) -> None:
        handle, self._handle = getattr(self, "_handle", None), None
        if handle:
            self._lib.gbdic_fourier_destroy(handle)

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass
