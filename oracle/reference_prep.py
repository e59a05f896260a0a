"""Float64 NumPy oracle for reference preparation and the CPU pyramid helpers.

TEST INFRASTRUCTURE ONLY: the product package never imports this module.  It
is the checker for the GPU reference-preparation kernels, the pyramid
reduction and the coarse-to-fine seed transfer, and it is itself pinned to
golden vectors produced by the reference's own NumPy code
(tests/golden/make_golden.py).

Each function restates one reference routine of
DIC/LucasKanadeICGN/python/src/live_dic/wgpu_backend.py:
  fir_weights            -> _fir_weights              (527-541)
  gaussian_sigma_one     -> _gaussian_sigma_one       (544-561)
  bspline_coefficients   -> _spline_filter_axis /
                            _cubic_bspline_prefilter  (564-586)
  reference_arrays       -> _reference_arrays         (589-823)
  reduce_half            -> _reduce_half              (318-334)
  transfer_seed_cpu      -> _transfer_pyramid_seed    (337-454)
"""

from __future__ import annotations

import math

import numpy as np

FIR_HALF_WIDTH = 15
FIR_RUNTIME_HALF_WIDTH = 12
SPLINE_POLE = float(np.sqrt(3.0) - 2.0)


def fir_weights() -> np.ndarray:
    """31 taps: a sigma-one 7-tap Gaussian convolved with the truncated
    (+-12) impulse response sqrt(3) * z^|k| of the inverse cubic B-spline.
    Contributions are added in Gaussian-tap order, in float64."""
    g = np.exp(-0.5 * np.arange(-3.0, 4.0) ** 2)
    g = g / g.sum()
    root3 = np.sqrt(3.0)
    pole = np.sqrt(3.0) - 2.0
    taps = np.zeros(2 * FIR_HALF_WIDTH + 1, dtype=np.float64)
    for gi, offset in enumerate(range(-3, 4)):
        for k in range(-12, 13):
            taps[FIR_HALF_WIDTH + offset + k] += g[gi] * root3 * pole ** abs(k)
    return taps.astype(np.float32)


def runtime_fir_taps() -> np.ndarray:
    """The 25 central float32 taps actually applied per axis."""
    trim = FIR_HALF_WIDTH - FIR_RUNTIME_HALF_WIDTH
    return np.ascontiguousarray(fir_weights()[trim:-trim])


def _reflect_index(n: int, pad: int) -> np.ndarray:
    """Indices of an edge-exclusive reflection padded by `pad` on each side."""
    idx = np.arange(-pad, n + pad)
    idx = np.where(idx < 0, -idx, idx)
    idx = np.where(idx >= n, 2 * n - 2 - idx, idx)
    return idx


def gaussian_sigma_one(image: np.ndarray) -> np.ndarray:
    """Separable mirrored 7-tap sigma-one Gaussian in float64 (x, then y)."""
    g = np.exp(-0.5 * np.arange(-3.0, 4.0) ** 2)
    g = g / g.sum()
    src = np.asarray(image, dtype=np.float64)
    h, w = src.shape
    xi = _reflect_index(w, 3)
    rows = src[:, xi]
    out_x = np.zeros_like(src)
    for k in range(7):
        out_x = out_x + g[k] * rows[:, k : k + w]
    yi = _reflect_index(h, 3)
    cols = out_x[yi, :]
    out = np.zeros_like(src)
    for k in range(7):
        out = out + g[k] * cols[k : k + h, :]
    return out


def _spline_axis_last(values: np.ndarray) -> np.ndarray:
    """Exact causal/anticausal cubic B-spline prefilter along the last axis.

    Gain (1-z)(1-1/z); causal start = sum over a 1e-12 horizon of z^k c[k];
    anticausal start z/(z^2-1) (c+[n-1] + z c+[n-2])."""
    z = SPLINE_POLE
    c = values * ((1.0 - z) * (1.0 - 1.0 / z))
    n = c.shape[-1]
    horizon = min(n, int(math.ceil(math.log(1e-12) / math.log(abs(z)))))
    c[..., 0] = np.sum(c[..., :horizon] * z ** np.arange(horizon, dtype=np.float64), axis=-1)
    for k in range(1, n):
        c[..., k] = c[..., k] + z * c[..., k - 1]
    c[..., n - 1] = (z / (z * z - 1.0)) * (z * c[..., n - 2] + c[..., n - 1])
    for k in range(n - 2, -1, -1):
        c[..., k] = z * (c[..., k + 1] - c[..., k])
    return c


def bspline_coefficients(intensity: np.ndarray) -> np.ndarray:
    """Rows first, then columns."""
    c = np.array(intensity, dtype=np.float64, copy=True)
    c = _spline_axis_last(c)
    c = _spline_axis_last(np.ascontiguousarray(c.T)).T
    return np.ascontiguousarray(c)


def gradients(source: np.ndarray, bspline: bool) -> tuple[np.ndarray, np.ndarray]:
    """Central differences with a one-pixel reflection; for B-spline
    coefficients the difference is smoothed by [1, 4, 1]/6 across the other
    axis (the exact derivative of the interpolant at the nodes)."""
    h, w = source.shape
    p = source[_reflect_index(h, 1)][:, _reflect_index(w, 1)]
    dx = 0.5 * (p[:, 2:] - p[:, :-2])  # shape (h+2, w)
    dy = 0.5 * (p[2:, :] - p[:-2, :])  # shape (h, w+2)
    if not bspline:
        return dx[1:-1, :], dy[:, 1:-1]
    gx = (dx[:-2, :] + 4.0 * dx[1:-1, :] + dx[2:, :]) / 6.0
    gy = (dy[:, :-2] + 4.0 * dy[:, 1:-1] + dy[:, 2:]) / 6.0
    return gx, gy


def grid_shape(width: int, height: int, size: int, stride: int) -> tuple[int, int]:
    if width < size or height < size:
        return 0, 0
    return 1 + (width - size) // stride, 1 + (height - size) // stride


def integration_weights(size: int, weighting: str, sigma: float) -> np.ndarray:
    c = np.arange(size, dtype=np.float64) - 0.5 * (size - 1)
    yy, xx = np.meshgrid(c, c, indexing="ij")
    if weighting == "gaussian":
        return np.exp(-0.5 * (xx * xx + yy * yy) / (sigma * sigma)).ravel()
    return np.ones(size * size, dtype=np.float64)


def reference_arrays(
    image: np.ndarray,
    *,
    interpolation: str = "bspline",
    motion_model: str = "affine",
    subset_size: int = 16,
    subset_stride: int | None = None,
    spatial_weighting: str = "uniform",
    gaussian_sigma: float | None = None,
) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Reference plane (H*W*4 float32), inverse Hessians and metadata.

    Metadata per subset: [sqrt(energy), valid, J^T f (n), sum J (n),
    mean, sum of weights], padded to 16 (n=6) or 28 (n=12) floats."""
    img = np.asarray(image, dtype=np.uint8)
    h, w = img.shape
    size = int(subset_size)
    stride = size if subset_stride is None else int(subset_stride)
    sigma = 0.25 * size if gaussian_sigma is None else float(gaussian_sigma)
    gw, gh = grid_shape(w, h, size, stride)
    if interpolation == "bspline":
        intensity = gaussian_sigma_one(img)
        grad_src = bspline_coefficients(intensity)
    else:
        intensity = img.astype(np.float64)
        grad_src = intensity
    gx, gy = gradients(grad_src, interpolation == "bspline")
    wts = integration_weights(size, spatial_weighting, sigma)
    wsum = float(wts.sum(dtype=np.float64))
    half = 0.5 * (size - 1)
    coords = np.arange(size, dtype=np.float64) - half
    ly, lx = np.meshgrid(coords, coords, indexing="ij")
    lx = lx.ravel()
    ly = ly.ravel()
    model = motion_model
    n = 12 if model == "quadratic" else 6
    meta_stride = 28 if model == "quadratic" else 16
    overlapping = stride != size

    plane = np.zeros((h, w, 4), dtype=np.float32)
    plane[..., 1] = gx
    plane[..., 2] = gy
    centred = intensity
    if overlapping:
        plane[..., 0] = intensity
    else:
        centred = intensity.copy()
        w2d = wts.reshape(size, size)
        for yy in range(gh):
            for xx in range(gw):
                blk = centred[yy * size : (yy + 1) * size, xx * size : (xx + 1) * size]
                blk -= float(np.sum(blk * w2d)) / wsum
        plane[..., 0] = centred

    count = gw * gh
    inverse = np.zeros((count, n * n), dtype=np.float32)
    metadata = np.zeros((count, meta_stride), dtype=np.float32)
    win = np.lib.stride_tricks.sliding_window_view
    for yy in range(gh):
        y0 = yy * stride
        rows_i = win(intensity[y0 : y0 + size], (size, size))[0, ::stride][:gw]
        rows_c = win(centred[y0 : y0 + size], (size, size))[0, ::stride][:gw]
        rows_gx = win(gx[y0 : y0 + size], (size, size))[0, ::stride][:gw]
        rows_gy = win(gy[y0 : y0 + size], (size, size))[0, ::stride][:gw]
        if overlapping:
            raw = rows_i.reshape(gw, -1)
            means = raw @ wts / wsum
            f = raw - means[:, None]
        else:
            f = rows_c.reshape(gw, -1)
            means = np.zeros(gw)
        tgx = rows_gx.reshape(gw, -1)
        tgy = rows_gy.reshape(gw, -1)
        energy = (f * f) @ wts
        if model == "translation":
            hxx = (tgx * tgx) @ wts
            hxy = (tgx * tgy) @ wts
            hyy = (tgy * tgy) @ wts
            det = hxx * hyy - hxy * hxy
            scale = np.maximum(np.abs(hxx * hyy), 1.0)
            valid = np.isfinite(det) & (np.abs(det) > np.finfo(np.float64).eps * scale) & (energy > 1e-12)
            invdet = np.where(valid, 1.0 / np.where(valid, det, 1.0), 0.0)
            inv = np.zeros((gw, 6, 6))
            inv[:, 0, 0] = hyy * invdet
            inv[:, 0, 3] = -hxy * invdet
            inv[:, 3, 0] = -hxy * invdet
            inv[:, 3, 3] = hxx * invdet
            jtf = np.zeros((gw, 6))
            jtf[:, 0] = (tgx * f) @ wts
            jtf[:, 3] = (tgy * f) @ wts
            sj = np.zeros((gw, 6))
            sj[:, 0] = tgx @ wts
            sj[:, 3] = tgy @ wts
        else:
            cols = [tgx, tgx * lx, tgx * ly, tgy, tgy * lx, tgy * ly]
            if model == "quadratic":
                hx2, xy, hy2 = 0.5 * lx * lx, lx * ly, 0.5 * ly * ly
                cols += [tgx * hx2, tgx * xy, tgx * hy2, tgy * hx2, tgy * xy, tgy * hy2]
            jac = np.stack(cols, axis=2)  # (gw, P, n)
            wj = jac * wts[None, :, None]
            hess = np.einsum("gpi,gpj->gij", wj, jac)
            jtf = np.einsum("gpi,gp->gi", wj, f)
            sj = wj.sum(axis=1)
            inv = np.zeros_like(hess)
            valid = np.zeros(gw, dtype=bool)
            for k in range(gw):
                try:
                    inv[k] = np.linalg.inv(hess[k])
                except np.linalg.LinAlgError:
                    continue
                valid[k] = bool(np.isfinite(inv[k]).all()) and energy[k] > 1e-12
        with np.errstate(invalid="ignore"):
            representable = np.max(np.abs(inv), axis=(1, 2)) <= np.finfo(np.float32).max
        valid = valid & representable
        inv[~valid] = 0.0
        sl = slice(yy * gw, (yy + 1) * gw)
        inverse[sl] = inv.reshape(gw, n * n)
        metadata[sl, 0] = np.sqrt(energy)
        metadata[sl, 1] = valid
        metadata[sl, 2 : 2 + n] = jtf
        metadata[sl, 2 + n : 2 + 2 * n] = sj
        metadata[sl, 2 + 2 * n] = means
        metadata[sl, 3 + 2 * n] = wsum
    return plane.ravel(), inverse.ravel(), metadata.ravel()


def reduce_half(image: np.ndarray) -> np.ndarray:
    """Half-resolution level: reflected [1 4 6 4 1]^2 / 256, truncated.
    Computed as an exact integer 5x5 sum (equal to the separable float32 form
    because every partial sum is an exact binary fraction)."""
    img = np.asarray(image, dtype=np.uint8)
    h, w = img.shape
    h2, w2 = h // 2, w // 2
    padded = img.astype(np.int64)[_reflect_index(h, 2)][:, _reflect_index(w, 2)]
    taps = (1, 4, 6, 4, 1)
    total = np.zeros((h2, w2), dtype=np.int64)
    for j, ty in enumerate(taps):
        for i, tx in enumerate(taps):
            total += ty * tx * padded[j : j + 2 * h2 : 2, i : i + 2 * w2 : 2]
    return np.ascontiguousarray((total // 256).astype(np.uint8))


def transfer_seed_cpu(
    parameters: np.ndarray,
    status: np.ndarray,
    *,
    source_available: np.ndarray,
    source_scale: int,
    destination_scale: int,
    destination_grid: tuple[int, int],
    requested: np.ndarray,
    subset_size: int,
    subset_stride: int,
    motion_model: str = "affine",
    permissions: np.ndarray | None = None,
) -> tuple[np.ndarray, np.ndarray]:
    """Bilinear blend of the four coarse warps around each requested fine
    centre, Taylor-recentred, translations scaled by source/destination and
    curvatures by destination/source; float64; ROI fallback neighbour."""
    dw, dh = destination_grid
    ncomp = 12 if motion_model == "quadratic" else 6
    seeds = np.zeros((dh, dw, 16 if motion_model == "quadratic" else 8), dtype=np.float32)
    active = requested.astype(np.uint32)
    sh, sw = status.shape
    if sw < 2 or sh < 2:
        return seeds, active
    dy_i, dx_i = np.nonzero(requested)
    if dy_i.size == 0:
        return seeds, active
    c0 = 0.5 * subset_size
    shift = ((1.0 - destination_scale) - (1.0 - source_scale)) * 0.5
    x = (destination_scale * (c0 + subset_stride * dx_i) + shift) / source_scale
    y = (destination_scale * (c0 + subset_stride * dy_i) + shift) / source_scale
    gxf = (x - c0) / subset_stride
    gyf = (y - c0) / subset_stride
    lx = np.clip(np.floor(gxf), 0, sw - 2).astype(np.intp)
    ly = np.clip(np.floor(gyf), 0, sh - 2).astype(np.intp)
    fx = np.clip(gxf - lx, 0.0, 1.0)
    fy = np.clip(gyf - ly, 0.0, 1.0)
    tscale = source_scale / destination_scale
    cscale = destination_scale / source_scale
    acc = np.zeros((dy_i.size, ncomp))
    wsum = np.zeros(dy_i.size)
    for corner in range(5):
        if corner < 4:
            sx = lx + (corner & 1)
            sy = ly + (corner >> 1)
            ok = (status[sy, sx] >= -0.5) & source_available[sy, sx]
            if permissions is not None:
                ok &= (permissions[dy_i, dx_i] & (1 << corner)) != 0
            wgt = (fx if corner & 1 else 1.0 - fx) * (fy if corner & 2 else 1.0 - fy) * ok
        else:
            if permissions is None:
                break
            fb = (permissions[dy_i, dx_i] >> np.uint32(5)).astype(np.int64)
            idx = np.maximum(fb - 1, 0)
            sx, sy = idx % sw, idx // sw
            ok = (fb != 0) & (wsum == 0) & source_available[sy, sx] & (status[sy, sx] >= 0.5)
            wgt = ok.astype(np.float64)
        p = parameters[sy, sx].astype(np.float64)
        ddx = x - (c0 + subset_stride * sx)
        ddy = y - (c0 + subset_stride * sy)
        q = p.copy()
        q[:, 0] += p[:, 1] * ddx + p[:, 2] * ddy
        q[:, 3] += p[:, 4] * ddx + p[:, 5] * ddy
        if motion_model == "quadratic":
            q[:, 0] += 0.5 * p[:, 6] * ddx * ddx + p[:, 7] * ddx * ddy + 0.5 * p[:, 8] * ddy * ddy
            q[:, 3] += 0.5 * p[:, 9] * ddx * ddx + p[:, 10] * ddx * ddy + 0.5 * p[:, 11] * ddy * ddy
            q[:, 1] += p[:, 6] * ddx + p[:, 7] * ddy
            q[:, 2] += p[:, 7] * ddx + p[:, 8] * ddy
            q[:, 4] += p[:, 9] * ddx + p[:, 10] * ddy
            q[:, 5] += p[:, 10] * ddx + p[:, 11] * ddy
            q[:, 6:12] *= cscale
        q[:, 0] *= tscale
        q[:, 3] *= tscale
        acc += wgt[:, None] * q
        wsum += wgt
    ok = wsum > 0
    seeds[dy_i[ok], dx_i[ok], :ncomp] = acc[ok] / wsum[ok, None]
    return seeds, active
