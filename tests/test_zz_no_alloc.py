"""The allocation-free registration entry point agrees with gbdic_register.

gbdic_register_noalloc serves callers that cannot allocate GPU memory (code
inside a stream capture, allocation-free real-time loops, plug-ins whose host
framework owns every device allocation): the caller supplies device buffers
for the inputs and the output, and the coefficient scratch is a fixed array
inside the library.  Its result must equal the engine's ordinary entry point
bit for bit (the tolerance every kernel test here uses), on two calls in a
row, since the shared scratch keeps the previous call's contents.

This file is named to be collected last.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, _native, synthetic

pytestmark = pytest.mark.gpu

W, H, S, STRIDE = 192, 160, 21, 10


def _frames():
    ref, sp = synthetic.reference_image(W, H, seed=404, device="cpu")
    a = synthetic.deformed_image(sp, synthetic.affine_field(0.45, 2e-3, 0.0, -0.3, 0.0, 1e-3), noise_seed=405,
                                 device="cpu")
    b = synthetic.deformed_image(sp, synthetic.affine_field(-0.8, 0.0, 1e-3, 0.6, -1e-3, 0.0), noise_seed=406,
                                 device="cpu")
    return ref, a, b


MODELS = {"affine": 0, "translation": 1, "quadratic": 2}
INTERPOLATIONS = {"bspline": 0, "linear": 1, "cubic": 2}


def _roi_mask():
    yy, xx = np.ogrid[:H, :W]
    return (xx - 0.5 * W) ** 2 + (yy - 0.5 * H) ** 2 >= 28.0 ** 2


@pytest.mark.parametrize("model,interpolation,lanes,weighting,roi", [
    ("affine", "bspline", 32, "uniform", False),
    ("affine", "bspline", 16, "uniform", True),
    ("translation", "bspline", 128, "uniform", False),
    ("quadratic", "bspline", 16, "uniform", False),
    ("affine", "linear", 32, "uniform", False),
    ("affine", "cubic", 64, "uniform", False),
    ("affine", "bspline", 16, "gaussian", False),
])
def test_noalloc_matches_register_on_two_calls_in_a_row(model, interpolation, lanes, weighting, roi):
    import torch

    ref, first, second = _frames()
    lib = _native.load()
    stride = 16 if model == "quadratic" else 8
    with ICGNWGPU(subset_size=S, subset_stride=STRIDE, outlier_policy="disabled", solver_workgroup_size=lanes,
                  motion_model=model, interpolation=interpolation, spatial_weighting=weighting) as engine:
        engine.set_reference(ref, roi_mask=_roi_mask() if roi else None)
        plane, inverse, metadata = engine.export_reference()
        weights = engine.export_weights() if weighting == "gaussian" else None
        expected = []
        for frame in (first, second):
            r = engine.register(frame)
            expected.append(np.concatenate([r.parameters, r.status[..., None], r.iterations[..., None]], -1))
    gw, gh = 1 + (W - S) // STRIDE, 1 + (H - S) // STRIDE
    device = torch.device("cuda:0")
    d_plane = torch.from_numpy(plane).to(device)
    d_meta = torch.from_numpy(metadata).to(device)
    d_inv = torch.from_numpy(inverse).to(device)
    d_weights = None if weights is None else torch.from_numpy(weights).to(device)
    d_state = torch.zeros(gw * gh * stride, dtype=torch.float32, device=device)
    for frame, want in zip((first, second), expected, strict=True):
        d_frame = torch.from_numpy(np.ascontiguousarray(frame)).to(device)
        args = _native.NoAllocFrame()
        args.frame, args.plane = d_frame.data_ptr(), d_plane.data_ptr()
        args.metadata, args.inverse = d_meta.data_ptr(), d_inv.data_ptr()
        args.weights = None if d_weights is None else d_weights.data_ptr()
        args.width, args.height = W, H
        args.motion_model, args.interpolation = MODELS[model], INTERPOLATIONS[interpolation]
        args.subset_size, args.subset_stride = S, STRIDE
        args.threads_per_subset, args.roi_enabled = lanes, int(roi)
        args.cfg = _native.SolverCfg(30, 1e-3, 0.8)
        stream = torch.cuda.current_stream(device)
        code = lib.gbdic_register_noalloc(C.byref(args), C.c_void_p(d_state.data_ptr()),
                                          C.c_void_p(stream.cuda_stream))
        _native.check(code, lib.gbdic_last_error(None))
        torch.cuda.synchronize(device)
        got = d_state.view(gh, gw, stride).cpu().numpy()
        n = 12 if model == "quadratic" else 6
        np.testing.assert_array_equal(got[..., : n + 2], want)
        status = got[..., n]
        assert (status == 1).sum() > 0
        if roi:
            assert (status == -3).sum() > 0


def test_noalloc_rejects_frames_beyond_its_scratch():
    lib = _native.load()
    args = _native.NoAllocFrame()
    args.frame = args.plane = args.metadata = args.inverse = 1  # never dereferenced: rejected before any launch
    args.width, args.height = 4096, 4096
    args.motion_model, args.interpolation = 0, 0
    args.subset_size, args.subset_stride = S, STRIDE
    args.threads_per_subset = 32
    args.cfg = _native.SolverCfg(30, 1e-3, 0.8)
    code = lib.gbdic_register_noalloc(C.byref(args), C.c_void_p(1), None)
    assert code == _native.EINVAL
    assert b"exceeds" in lib.gbdic_last_error(None)
