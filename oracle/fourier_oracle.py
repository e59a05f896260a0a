"""CPU oracle of the global-translation initializer (TEST INFRASTRUCTURE ONLY).

NumPy float64 restatement of FourierInitializer (fourier.py:16-111 of the
reference): window choice, 2x2 averaging, Hann taper, zero-padded real FFTs,
normalised cross power spectrum, peak score against the background outside
the wrapped 11 x 11 block, even-pixel shift, overlap and sample correlation.
Returns the raw figures; the acceptance rule is applied by the caller.
"""

from __future__ import annotations

import numpy as np


def choose_window(reference: np.ndarray, mask: np.ndarray | None):
    height, width = reference.shape
    size = 1 << min(10, min(width, height).bit_length() - 1)
    best = None
    for fx, fy in [(0.5, 0.5)] + [(x, y) for y in (0, 0.5, 1) for x in (0, 0.5, 1)]:
        x, y = int((width - size) * fx), int((height - size) * fy)
        patch = reference[y:y + size, x:x + size].astype(np.float64)
        allowed = np.ones(patch.shape, bool) if mask is None else mask[y:y + size, x:x + size]
        coverage = float(np.mean(allowed))
        std = float(np.std(patch[allowed])) if allowed.any() else 0.0
        if coverage >= 0.25 and std >= 1.0:
            cand = (coverage * std, x, y, allowed.copy())
            if best is None or cand[0] > best[0]:
                best = cand
            if fx == fy == 0.5 and coverage >= 0.5:
                break
    if best is None:
        raise ValueError("no sufficiently textured ROI window")
    return best[1], best[2], size, best[3]


def estimate(reference: np.ndarray, target: np.ndarray, mask: np.ndarray | None = None) -> dict:
    x, y, size, allowed = choose_window(reference, mask)
    half = size // 2
    hann = np.hanning(half)
    taper = hann[:, None] * hann[None, :]
    patch = reference[y:y + size, x:x + size].astype(np.float64)
    values = (patch - np.mean(patch[allowed])) * allowed
    ref_samples = values.reshape(half, 2, half, 2).mean(axis=(1, 3))
    allowed_samples = allowed.reshape(half, 2, half, 2).all(axis=(1, 3))
    ref_spectrum = np.fft.rfft2(ref_samples * taper, s=(size, size))
    cur = target[y:y + size, x:x + size].astype(np.float64)
    reduced = (cur - np.mean(cur)).reshape(half, 2, half, 2).mean(axis=(1, 3))
    spectrum = np.fft.rfft2(reduced * taper, s=(size, size))
    cross = spectrum * np.conj(ref_spectrum)
    cross /= np.maximum(np.abs(cross), 1e-12)
    corr = np.fft.irfft2(cross, s=(size, size))
    py, px = np.unravel_index(np.argmax(corr), corr.shape)
    peak = float(corr[py, px])
    side = np.ones(corr.shape, bool)
    side[np.ix_(np.arange(py - 5, py + 6) % size, np.arange(px - 5, px + 6) % size)] = False
    background = corr[side]
    score = float((peak - np.mean(background)) / max(float(np.std(background)), 1e-12))
    dx = 2 * int(px if px < half else px - size)
    dy = 2 * int(py if py < half else py - size)
    overlap = max(0, size - abs(dx)) * max(0, size - abs(dy)) / size ** 2
    sx, sy = dx // 2, dy // 2
    ry, rx = slice(max(0, -sy), min(half, half - sy)), slice(max(0, -sx), min(half, half - sx))
    cy, cx = slice(max(0, sy), min(half, half + sy)), slice(max(0, sx), min(half, half + sx))
    keep = allowed_samples[ry, rx]
    a, b = ref_samples[ry, rx][keep], reduced[cy, cx][keep]
    if a.size:
        a, b = a - a.mean(), b - b.mean()
    norm = float(np.linalg.norm(a) * np.linalg.norm(b))
    correlation = float(np.sum(a * b) / norm) if norm > 0 else 0.0
    return dict(dx=dx, dy=dy, peakScore=score, overlap=overlap, correlation=correlation, std=float(np.std(cur)),
                window=(x, y, size))
