"""Generate golden vectors from the reference's own NumPy code.

Run from the repository root, in a checkout where the reference sources are
available (they are not needed afterwards):

    python tests/golden/make_golden.py <path of the live-dic checkout>

The reference package imports Pillow and websockets at module level although
none of the routines used here touch them, so both are replaced by empty
stand-ins before the import.  Outputs: tests/golden/*.npz (small, seeded).
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _import_reference(root: Path):
    sys.modules.setdefault("websockets", types.ModuleType("websockets"))
    pil = types.ModuleType("PIL")
    image = types.ModuleType("PIL.Image")
    image.Image = type("Image", (), {})
    pil.Image = image
    sys.modules.setdefault("PIL", pil)
    sys.modules.setdefault("PIL.Image", image)
    python_root = root / "DIC/LucasKanadeICGN/python"
    sys.path.insert(0, str(python_root / "src"))
    sys.path.insert(0, str(python_root / "tests"))
    import live_dic.engine as engine
    import live_dic.roi as roi
    import live_dic.wgpu_backend as backend
    import test_gpu_regressions as regressions

    return backend, engine, roi, regressions


def speckle(rng: np.random.Generator, height: int, width: int, dots: int) -> np.ndarray:
    y, x = np.mgrid[:height, :width].astype(np.float64)
    img = np.zeros((height, width))
    cx = rng.uniform(0, width, dots)
    cy = rng.uniform(0, height, dots)
    sig = rng.uniform(1.5, 3.0, dots)
    amp = rng.uniform(0.3, 1.0, dots)
    for a, b, s, m in zip(cx, cy, sig, amp):
        img += m * np.exp(-((x - a) ** 2 + (y - b) ** 2) / (2 * s * s))
    img = 255.0 * (img - img.min()) / (img.max() - img.min())
    return np.clip(np.rint(img + rng.normal(0, 0.5, img.shape)), 0, 255).astype(np.uint8)


def main(reference_root: str) -> None:
    backend, engine, roi, regressions = _import_reference(Path(reference_root))
    rng = np.random.default_rng(20261203)
    out: dict[str, np.ndarray] = {}

    # FIR taps and the reference's own float32 FIR oracle (test_gpu_regressions._cpu_prefilter).
    out["fir_weights"] = backend._fir_weights()
    img = speckle(rng, 70, 83, 200)
    out["prefilter_image"] = img
    out["prefilter_expected"] = regressions._cpu_prefilter(img)

    # Pyramid reduction: float separable (_reduce_half) and integer oracle.
    for k, (h, w) in enumerate([(32, 48), (37, 53), (64, 64), (17, 16)]):
        src = rng.integers(0, 256, size=(h, w), dtype=np.uint8)
        out[f"reduce_{k}_in"] = src
        out[f"reduce_{k}_half"] = backend._reduce_half(src)
        out[f"reduce_{k}_int"] = regressions._integer_reduction(src)

    # Reference preparation, every model x interpolation, overlapping and
    # tiled grids, uniform and Gaussian weights, plus a flat image.
    cases = []
    ref_img = speckle(rng, 64, 72, 180)
    out["prep_image"] = ref_img
    for model in ("affine", "translation", "quadratic"):
        for interp in ("bspline", "linear", "cubic"):
            cases.append((model, interp, 21, 10, "uniform", None))
    cases += [
        ("affine", "bspline", 16, 16, "uniform", None),
        ("affine", "bspline", 15, 5, "gaussian", 4.0),
        ("quadratic", "bspline", 31, 31, "gaussian", 8.0),
        ("translation", "linear", 8, 8, "uniform", None),
        ("affine", "bspline", 24, 12, "uniform", None),
    ]
    for index, (model, interp, size, stride, weighting, sigma) in enumerate(cases):
        plane, inverse, metadata = backend._reference_arrays(
            ref_img,
            interpolation=interp,
            motion_model=model,
            subset_size=size,
            subset_stride=stride,
            spatial_weighting=weighting,
            gaussian_sigma=sigma,
        )
        out[f"prep_{index}_plane"] = plane
        out[f"prep_{index}_inverse"] = inverse
        out[f"prep_{index}_metadata"] = metadata
    out["prep_cases"] = np.array(
        [f"{m}|{i}|{s}|{t}|{w}|{'' if g is None else g}" for m, i, s, t, w, g in cases]
    )
    flat = np.full((40, 40), 91, dtype=np.uint8)
    plane, inverse, metadata = backend._reference_arrays(flat, subset_size=13, subset_stride=13)
    out["flat_inverse"] = inverse
    out["flat_metadata"] = metadata

    # Seed transfer on a synthetic coarse affine / quadratic field.
    for model in ("affine", "quadratic"):
        n = 12 if model == "quadratic" else 6
        sh, sw = 7, 9
        params = rng.normal(0, 0.5, size=(sh, sw, n)).astype(np.float32)
        params[..., 1:3] *= 0.01
        params[..., 4:6] *= 0.01
        if n == 12:
            params[..., 6:] *= 1e-4
        status = rng.choice(np.array([1.0, 1.0, 1.0, 0.0, -1.0, 2.0], np.float32), size=(sh, sw))
        available = rng.random((sh, sw)) > 0.1
        requested = rng.random((13, 17)) > 0.2
        result = types.SimpleNamespace(
            parameters=params, status=status, config={"motionModel": model}
        )
        seeds, active = backend._transfer_pyramid_seed(
            result,
            source_available=available,
            source_scale=2,
            destination_scale=1,
            destination_grid=(17, 13),
            requested=requested,
            subset_size=21,
            subset_stride=10,
        )
        out[f"transfer_{model}_params"] = params
        out[f"transfer_{model}_status"] = status
        out[f"transfer_{model}_available"] = available
        out[f"transfer_{model}_requested"] = requested
        out[f"transfer_{model}_seeds"] = seeds
        out[f"transfer_{model}_active"] = active

    # ROI planning and pyramid seed permissions for a mask with a hole.
    mask = np.ones((120, 150), dtype=bool)
    yy, xx = np.mgrid[:120, :150]
    mask[(xx - 70) ** 2 + (yy - 55) ** 2 < 23**2] = False
    mask[:, 140:] = False
    out["roi_mask"] = mask
    plan = roi.prepare_roi(mask, 21, 10, policy="full", median_filter_size=3)
    out["roi_selected"] = plan.selected
    out["roi_neighbour_bits"] = plan.neighbour_bits
    plan9 = roi.prepare_roi(mask, 21, 10, policy="full", median_filter_size=9)
    out["roi_median_words"] = plan9.median_neighbour_words
    coarse_mask = roi.reduce_mask(mask)
    out["roi_reduced_mask"] = coarse_mask
    coarse = roi.prepare_roi(coarse_mask, 21, 10, policy="full")
    out["roi_coarse_selected"] = coarse.selected
    out["roi_seed_permissions"] = roi.seed_permissions(
        coarse, plan, source_scale=2, destination_scale=1, size=21, stride=10, reference_mask=mask
    )
    out["roi_temporal_permissions"] = roi.seed_permissions(
        plan, coarse, source_scale=1, destination_scale=2, size=21, stride=10, reference_mask=mask
    )

    # Input normalisation.
    floats = rng.random((20, 24)).astype(np.float32)
    out["gray_float_in"] = floats
    out["gray_float_out"] = engine._as_uint8_gray(floats)
    wide = rng.uniform(0, 300, size=(20, 24))
    out["gray_wide_in"] = wide
    out["gray_wide_out"] = engine._as_uint8_gray(wide)

    np.savez_compressed(HERE / "reference_vectors.npz", **out)
    fourier_vectors(Path(reference_root))
    partial_vectors(Path(reference_root))
    roi_vectors(Path(reference_root))


def roi_vectors(reference_root: Path) -> None:
    """ROI planning on harder masks (several holes, a cut edge, odd and even
    windows, overlapping and tiled grids, every median lattice, both partial
    truncations) and the seed permissions between two pyramid levels."""
    _, _, roi, _ = _import_reference(reference_root)
    rng = np.random.default_rng(2718)
    out: dict[str, np.ndarray] = {}
    cases = [(190, 230, 17, 6), (160, 200, 16, 16), (210, 170, 24, 9)]
    for k, (h, w, size, stride) in enumerate(cases):
        yy, xx = np.mgrid[:h, :w]
        mask = np.ones((h, w), dtype=bool)
        for _ in range(3):
            cx, cy, r = rng.uniform(0, w), rng.uniform(0, h), rng.uniform(8, 30)
            mask &= (xx - cx) ** 2 + (yy - cy) ** 2 >= r * r
        mask[: int(rng.integers(3, 15))] = False
        mask[:, w - int(rng.integers(3, 15)):] = False
        out[f"roi{k}_mask"] = mask
        out[f"roi{k}_geometry"] = np.array([size, stride])
        for median in (3, 5, 7, 9):
            plan = roi.prepare_roi(mask, size, stride, median_filter_size=median)
            if median == 3:
                out[f"roi{k}_selected"] = plan.selected
                out[f"roi{k}_bits"] = plan.neighbour_bits
                out[f"roi{k}_hash"] = np.frombuffer(plan.mask_hash.encode(), np.uint8)
            else:
                out[f"roi{k}_median{median}"] = plan.median_neighbour_words
        for truncation in ("none", "visibility"):
            plan = roi.prepare_roi(mask, size, stride, policy="partial", truncation=truncation)
            for name in ("selected", "partial_indices", "support_words", "support_boxes", "coverage",
                         "neighbour_bits"):
                out[f"roi{k}_partial_{truncation}_{name}"] = getattr(plan, name)
        fine = roi.prepare_roi(mask, size, stride)
        coarse_mask = roi.reduce_mask(mask)
        out[f"roi{k}_reduced"] = coarse_mask
        coarse = roi.prepare_roi(coarse_mask, size, stride)
        out[f"roi{k}_down"] = roi.seed_permissions(coarse, fine, source_scale=2, destination_scale=1, size=size,
                                                   stride=stride, reference_mask=mask)
        out[f"roi{k}_up"] = roi.seed_permissions(fine, coarse, source_scale=1, destination_scale=2, size=size,
                                                 stride=stride, reference_mask=mask)
    np.savez_compressed(HERE / "roi_vectors.npz", **out)


def partial_vectors(reference_root: Path) -> None:
    """Partial-support ROI planning (roi.py, both truncations) and the
    partial reference preparation (partial.py) on a speckle reference."""
    backend, _, roi, _ = _import_reference(reference_root)
    import live_dic.partial as partial

    rng = np.random.default_rng(515)
    ref = speckle(rng, 150, 170, 420)
    yy, xx = np.mgrid[:150, :170]
    mask = ((xx - 80) ** 2 + (yy - 70) ** 2 >= 26 ** 2) & ~((xx > 120) & (yy > 100) & (xx < 130))
    out: dict[str, np.ndarray] = {"partial_ref": ref, "partial_mask": mask}
    for truncation in ("none", "visibility"):
        plan = roi.prepare_roi(mask, 21, 10, policy="partial", truncation=truncation)
        out[f"partial_{truncation}_selected"] = plan.selected
        out[f"partial_{truncation}_indices"] = plan.partial_indices
        out[f"partial_{truncation}_words"] = plan.support_words
        out[f"partial_{truncation}_boxes"] = plan.support_boxes
        out[f"partial_{truncation}_bits"] = plan.neighbour_bits
    plan = roi.prepare_roi(mask, 21, 10, policy="partial", truncation="none")
    plane, inverse, metadata = backend._reference_arrays(ref, subset_size=21, subset_stride=10)
    out["partial_plane"] = plane
    out["partial_metadata_in"] = metadata.copy()
    out["partial_inverse_in"] = inverse.copy()
    updated = partial.prepare_partial_reference(plane, inverse, metadata, plan, width=170, height=150, size=21,
                                                stride=10, motion_model="affine", weighting="uniform", sigma=5.25)
    out["partial_metadata_out"] = metadata
    out["partial_inverse_out"] = inverse
    out["partial_condition"] = updated.support_condition
    out["partial_rank"] = updated.support_rank
    np.savez_compressed(HERE / "partial_vectors.npz", **out)


def fourier_vectors(reference_root: Path) -> None:
    """FourierInitializer (fourier.py) on integer-shifted speckle crops, with
    and without an ROI mask, plus a textured but unrelated target."""
    _import_reference(reference_root)
    import live_dic.fourier as fourier

    rng = np.random.default_rng(4711)
    big = speckle(rng, 360, 420, 900)
    out: dict[str, np.ndarray] = {}
    cases = [((12, -7), None), ((-30, 18), None), ((6, 10), "hole"), ((0, 0), "noise")]
    for k, (shift, kind) in enumerate(cases):
        dx, dy = shift
        ref = np.ascontiguousarray(big[40:296, 50:370])
        tgt = np.ascontiguousarray(big[40 - dy:296 - dy, 50 - dx:370 - dx])
        mask = None
        if kind == "hole":
            yy, xx = np.mgrid[:256, :320]
            mask = (xx - 160) ** 2 + (yy - 128) ** 2 >= 40 ** 2
        if kind == "noise":
            tgt = rng.integers(0, 256, ref.shape, dtype=np.uint8)
        init = fourier.FourierInitializer(ref, mask)
        out[f"fourier_{k}_ref"] = ref
        out[f"fourier_{k}_tgt"] = tgt
        out[f"fourier_{k}_mask"] = np.ones(ref.shape, bool) if mask is None else mask
        out[f"fourier_{k}_has_mask"] = np.array(mask is not None)
        w = init.window
        out[f"fourier_{k}_window"] = np.array([w["x"], w["y"], w["size"]])
        try:
            est = init.estimate(tgt)
            out[f"fourier_{k}_result"] = np.array([est["dx"], est["dy"], est["peakScore"], est["overlap"],
                                                   est["correlation"]])
            out[f"fourier_{k}_accepted"] = np.array(True)
        except ValueError:
            out[f"fourier_{k}_result"] = np.zeros(5)
            out[f"fourier_{k}_accepted"] = np.array(False)
    np.savez_compressed(HERE / "fourier_vectors.npz", **out)
    print(f"wrote {len(out)} arrays to {HERE / 'reference_vectors.npz'}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {sys.argv[0]} <path of the live-dic checkout>")
    main(sys.argv[1])
