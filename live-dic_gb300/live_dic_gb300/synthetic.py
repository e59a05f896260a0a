"""Seeded synthetic speckle pairs with imposed analytic fields and FP64 truth.

Images are sums of Gaussian dots (sigma uniform in [1.5, 3] px, amplitude
uniform in [0.3, 1], 4000 dots per 512^2 px), normalised to [0, 255] with the
reference's range, given independent N(0, 0.5) noise and rounded once to
uint8.  A target is the same continuous texture evaluated at the
inverse-mapped coordinate X of every pixel x, where x = X + u(X) is solved by
fixed-point iteration, so no resampling bias enters the fixture.

The dot sum is evaluated with PyTorch (on the GPU when available) through a
16-pixel cell table: every dot reaches at most 12 px, so a sample only needs
the dots of its 3 x 3 neighbouring cells.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover - torch is part of the runtime image
    torch = None

CELL = 16
DOTS_PER_PIXEL = 4000.0 / (512.0 * 512.0)


@dataclass(frozen=True)
class Speckle:
    """Dot parameters plus the intensity normalisation of the reference."""

    width: int
    height: int
    cx: np.ndarray
    cy: np.ndarray
    sigma: np.ndarray
    amp: np.ndarray
    offset: float = 0.0
    scale: float = 1.0


def make_speckle(width: int, height: int, seed: int, density: float = DOTS_PER_PIXEL) -> Speckle:
    rng = np.random.default_rng(seed)
    margin = 40.0  # dots outside the frame still reach displaced samples
    count = int(round(density * (width + 2 * margin) * (height + 2 * margin)))
    cx = rng.uniform(-margin, width + margin, count)
    cy = rng.uniform(-margin, height + margin, count)
    sigma = rng.uniform(1.5, 3.0, count)
    amp = rng.uniform(0.3, 1.0, count)
    return Speckle(width, height, cx, cy, sigma, amp)


def _device(device: str | None):
    if device is not None:
        return torch.device(device)
    return torch.device("cuda" if torch.cuda.is_available() else "cpu")


class _CellTable:
    def __init__(self, sp: Speckle, device) -> None:
        x0, y0 = -64.0, -64.0
        ncx = int(math.ceil((sp.width + 128.0) / CELL)) + 1
        ncy = int(math.ceil((sp.height + 128.0) / CELL)) + 1
        ix = np.clip(((sp.cx - x0) // CELL).astype(np.int64), 0, ncx - 1)
        iy = np.clip(((sp.cy - y0) // CELL).astype(np.int64), 0, ncy - 1)
        cell = iy * ncx + ix
        order = np.argsort(cell, kind="stable")
        cell_sorted = cell[order]
        counts = np.bincount(cell_sorted, minlength=ncx * ncy)
        k = max(1, int(counts.max()))
        starts = np.concatenate(([0], np.cumsum(counts)[:-1]))
        slot = np.arange(cell_sorted.size) - starts[cell_sorted]
        table = np.zeros((ncx * ncy, k, 4), dtype=np.float64)
        table[..., 2] = 1.0  # sigma of empty slots (amplitude 0)
        table[cell_sorted, slot, 0] = sp.cx[order]
        table[cell_sorted, slot, 1] = sp.cy[order]
        table[cell_sorted, slot, 2] = sp.sigma[order]
        table[cell_sorted, slot, 3] = sp.amp[order]
        self.table = torch.as_tensor(table, device=device)
        self.ncx, self.ncy, self.k, self.x0, self.y0 = ncx, ncy, k, x0, y0

    def evaluate(self, X, Y):
        """Sum of dots at float64 sample coordinates (torch tensors)."""
        out = torch.zeros_like(X)
        cx = torch.clamp(((X - self.x0) // CELL).long(), 1, self.ncx - 2)
        cy = torch.clamp(((Y - self.y0) // CELL).long(), 1, self.ncy - 2)
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                rows = self.table[(cy + dy) * self.ncx + (cx + dx)]  # (..., k, 4)
                ddx = X[..., None] - rows[..., 0]
                ddy = Y[..., None] - rows[..., 1]
                s = rows[..., 2]
                out += (rows[..., 3] * torch.exp(-(ddx * ddx + ddy * ddy) / (2.0 * s * s))).sum(-1)
        return out


def _render(sp: Speckle, X, Y, device):
    table = _CellTable(sp, device)
    values = torch.empty_like(X)
    rows_per_chunk = max(1, 2_000_000 // max(1, X.shape[1]))
    for r in range(0, X.shape[0], rows_per_chunk):
        values[r : r + rows_per_chunk] = table.evaluate(X[r : r + rows_per_chunk], Y[r : r + rows_per_chunk])
    return values


def _quantise(values, sp: Speckle, noise_seed: int, device) -> np.ndarray:
    gen = torch.Generator(device=device)
    gen.manual_seed(int(noise_seed))
    noise = torch.randn(values.shape, generator=gen, device=device, dtype=torch.float64) * 0.5
    img = (values - sp.offset) * sp.scale + noise
    return torch.clamp(torch.round(img), 0, 255).to(torch.uint8).cpu().numpy()


def reference_image(width: int, height: int, seed: int, *, device: str | None = None) -> tuple[np.ndarray, Speckle]:
    """Reference speckle (uint8) and its dot field with normalisation fixed."""
    dev = _device(device)
    sp = make_speckle(width, height, seed)
    y, x = torch.meshgrid(
        torch.arange(height, dtype=torch.float64, device=dev),
        torch.arange(width, dtype=torch.float64, device=dev),
        indexing="ij",
    )
    values = _render(sp, x, y, dev)
    lo, hi = float(values.min()), float(values.max())
    sp = Speckle(sp.width, sp.height, sp.cx, sp.cy, sp.sigma, sp.amp, lo, 255.0 / (hi - lo))
    return _quantise(values, sp, seed + 1, dev), sp


def deformed_image(sp: Speckle, field, *, noise_seed: int, device: str | None = None, iterations: int = 12) -> np.ndarray:
    """Target whose pixel x shows the reference texture at X, x = X + u(X).

    ``field(X, Y)`` returns torch (u, v) for float64 torch coordinates."""
    dev = _device(device)
    y, x = torch.meshgrid(
        torch.arange(sp.height, dtype=torch.float64, device=dev),
        torch.arange(sp.width, dtype=torch.float64, device=dev),
        indexing="ij",
    )
    X, Y = x.clone(), y.clone()
    for _ in range(iterations):
        u, v = field(X, Y)
        X, Y = x - u, y - v
    return _quantise(_render(sp, X, Y, dev), sp, noise_seed, dev)


# ------------------------------------------------------------------ fields
def affine_field(u0: float, ux: float, uy: float, v0: float, vx: float, vy: float):
    """u = u0 + ux x + uy y, v = v0 + vx x + vy y (pixel coordinates)."""

    def field(X, Y):
        return u0 + ux * X + uy * Y, v0 + vx * X + vy * Y

    return field


def affine_truth(params, x, y):
    u0, ux, uy, v0, vx, vy = params
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    return np.stack([u0 + ux * x + uy * y, v0 + vx * x + vy * y], -1)


def sinusoid_field(amp_u=2.0, lu_x=400.0, lu_y=600.0, amp_v=1.5, lv_x=500.0):
    """u = a sin(2 pi x / Lx) cos(2 pi y / Ly), v = b cos(2 pi x / Lvx)."""

    def field(X, Y):
        lib = torch if torch is not None and isinstance(X, torch.Tensor) else np
        u = amp_u * lib.sin(2 * math.pi * X / lu_x) * lib.cos(2 * math.pi * Y / lu_y)
        v = amp_v * lib.cos(2 * math.pi * X / lv_x)
        return u, v

    return field


class KirschField:
    """Plane-strain displacement around a circular hole (radius a, centre
    (cx, cy)) in an infinite plate under uniaxial tension along y, from the
    Kolosov-Muskhelishvili potentials phi = S/4 (z + 2a^2/z) and
    psi = -S/2 (z + a^2/z - a^4/z^3) in a frame whose real axis is the load
    axis: 2 mu (u_1 + i u_2) = kappa phi - z conj(phi') - conj(psi).
    The field is scaled so that max |u| over the image outside the hole equals
    ``peak`` pixels at load factor 1."""

    def __init__(self, width: int, height: int, radius: float, peak: float = 2.0, poisson: float = 0.3) -> None:
        self.cx, self.cy, self.a = 0.5 * width, 0.5 * height, float(radius)
        self.kappa = 3.0 - 4.0 * poisson
        ys, xs = np.mgrid[0:height:8, 0:width:8].astype(np.float64)
        u = self._raw(xs, ys)
        mag = np.hypot(u[..., 0], u[..., 1])
        outside = (xs - self.cx) ** 2 + (ys - self.cy) ** 2 >= self.a**2
        corners = self._raw(np.array([0.0, width - 1.0, 0.0, width - 1.0]), np.array([0.0, 0.0, height - 1.0, height - 1.0]))
        peak_raw = max(float(mag[outside].max()), float(np.hypot(corners[:, 0], corners[:, 1]).max()))
        self.gain = peak / peak_raw

    def _raw(self, x, y):
        # load frame: real axis along image y, imaginary axis along -x
        z = (np.asarray(y, np.float64) - self.cy) - 1j * (np.asarray(x, np.float64) - self.cx)
        r2 = np.abs(z) ** 2
        z = np.where(r2 < (0.25 * self.a) ** 2, 0.25 * self.a + 0j, z)
        a2 = self.a * self.a
        phi = 0.25 * (z + 2 * a2 / z)
        dphi = 0.25 * (1 - 2 * a2 / z**2)
        psi = -0.5 * (z + a2 / z - a2 * a2 / z**3)
        w = self.kappa * phi - z * np.conj(dphi) - np.conj(psi)
        # back to image axes: w = u_load + i u_perp, u_perp along -x
        return np.stack([-w.imag, w.real], -1)

    def truth(self, x, y, load: float = 1.0) -> np.ndarray:
        return load * self.gain * self._raw(x, y)

    def torch_field(self, load: float):
        cx, cy, a, kappa, gain = self.cx, self.cy, self.a, self.kappa, self.gain * load

        def field(X, Y):
            zr = Y - cy
            zi = -(X - cx)
            z = torch.complex(zr, zi)
            small = (zr * zr + zi * zi) < (0.25 * a) ** 2
            z = torch.where(small, torch.full_like(z, 0.25 * a), z)
            a2 = a * a
            phi = 0.25 * (z + 2 * a2 / z)
            dphi = 0.25 * (1 - 2 * a2 / z**2)
            psi = -0.5 * (z + a2 / z - a2 * a2 / z**3)
            w = kappa * phi - z * torch.conj(dphi) - torch.conj(psi)
            return -gain * w.imag, gain * w.real

        return field


def smooth_field(rng: np.random.Generator, width: int, height: int, peak: float):
    """Random affine-plus-sinusoid field whose largest |(u, v)| over the
    image is `peak` px.  Returns (field, params) with field usable on numpy
    arrays and torch tensors."""
    a = [float(x) for x in rng.uniform(-1.0, 1.0, 6)]
    wavelengths = [float(x) for x in rng.uniform(0.6, 1.5, 4) * max(width, height)]
    phases = [float(x) for x in rng.uniform(0.0, 2 * math.pi, 4)]
    amps = [float(x) for x in rng.uniform(0.3, 1.0, 2)]

    def raw(X, Y):
        lib = torch if torch is not None and isinstance(X, torch.Tensor) else np
        xn, yn = X / width - 0.5, Y / height - 0.5
        u = a[0] + a[1] * xn + a[2] * yn + amps[0] * lib.sin(2 * math.pi * X / wavelengths[0] + phases[0]) * lib.cos(
            2 * math.pi * Y / wavelengths[1] + phases[1])
        v = a[3] + a[4] * xn + a[5] * yn + amps[1] * lib.cos(2 * math.pi * X / wavelengths[2] + phases[2]) * lib.sin(
            2 * math.pi * Y / wavelengths[3] + phases[3])
        return u, v

    gy, gx = np.mgrid[0:height:8, 0:width:8].astype(np.float64)
    u, v = raw(gx, gy)
    scale = peak / float(np.sqrt(u * u + v * v).max())

    def field(X, Y):
        u, v = raw(X, Y)
        return scale * u, scale * v

    return field, {"affine": a, "wavelengths": wavelengths, "phases": phases, "amplitudes": amps,
                   "scale": scale, "peak": peak}


def rectangle_roi(rng: np.random.Generator, width: int, height: int, holes: int,
                  radius: tuple[float, float] = (40.0, 200.0)) -> np.ndarray:
    """A rectangle inset 3-10 % from each edge with `holes` circular holes
    (radius drawn from `radius`, capped to an eighth of the smaller side)."""
    x0, x1 = (rng.uniform(0.03, 0.10, 2) * width).astype(int)
    y0, y1 = (rng.uniform(0.03, 0.10, 2) * height).astype(int)
    mask = np.zeros((height, width), dtype=bool)
    mask[y0:height - y1, x0:width - x1] = True
    yy, xx = np.ogrid[:height, :width]
    cap = min(width, height) / 8.0
    for _ in range(holes):
        r = min(rng.uniform(*radius), cap)
        cx = rng.uniform(x0 + r, width - x1 - r)
        cy = rng.uniform(y0 + r, height - y1 - r)
        mask &= (xx - cx) ** 2 + (yy - cy) ** 2 >= r * r
    return mask


def uneven_workload(seed: int, count: int = 16, *, sizes=((640, 480), (1280, 720), (1920, 1080), (3840, 2160)),
                    subsets=(15, 21, 31, 41), quadratic_fraction: float = 0.5, peak=(0.5, 3.0),
                    device: str | None = None) -> list[dict]:
    """Image pairs of uneven size, subset size and shape function: each with
    a rectangle ROI holding 0-3 holes (affine jobs; the quadratic model takes
    no ROI mask) and a random smooth affine-plus-sinusoid field."""
    rng = np.random.default_rng(seed)
    pairs = []
    for k in range(count):
        width, height = sizes[int(rng.integers(len(sizes)))]
        size = int(subsets[int(rng.integers(len(subsets)))])
        model = "quadratic" if rng.uniform() < quadratic_fraction else "affine"
        field, params = smooth_field(rng, width, height, float(rng.uniform(*peak)))
        mask = None if model == "quadratic" else rectangle_roi(rng, width, height, int(rng.integers(0, 4)))
        ref, sp = reference_image(width, height, seed=seed * 1000 + 2 * k, device=device)
        tgt = deformed_image(sp, field, noise_seed=seed * 1000 + 2 * k + 1, device=device)
        pairs.append({"reference": ref, "target": tgt, "motion_model": model, "subset_size": size,
                      "subset_stride": size // 3, "roi_mask": mask, "field": field, "field_params": params})
    return pairs


def hole_mask(width: int, height: int, radius: float) -> np.ndarray:
    y, x = np.ogrid[:height, :width]
    return (x - 0.5 * width) ** 2 + (y - 0.5 * height) ** 2 >= radius**2


def subset_centres(width: int, height: int, size: int, stride: int) -> tuple[np.ndarray, np.ndarray]:
    gw = 1 + (width - size) // stride
    gh = 1 + (height - size) // stride
    y, x = np.indices((gh, gw))
    return x * stride + 0.5 * (size - 1), y * stride + 0.5 * (size - 1)
