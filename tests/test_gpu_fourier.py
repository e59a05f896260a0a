"""GPU phase correlation (the Fourier initializer) against the reference's
own outputs and the oracle, and the full pyramid seeded by it."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from live_dic_gb300 import ICGNError, ICGNWGPUFullPyramid, synthetic
from live_dic_gb300.fourier import FourierInitializer
from oracle import fourier_oracle

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "fourier_vectors.npz"


@pytest.mark.parametrize("k", range(4))
def test_matches_reference_golden(k):
    with np.load(GOLDEN) as g:
        mask = g[f"fourier_{k}_mask"] if bool(g[f"fourier_{k}_has_mask"]) else None
        init = FourierInitializer(g[f"fourier_{k}_ref"], mask)
        assert [init.window[key] for key in ("x", "y", "size")] == list(g[f"fourier_{k}_window"])
        if bool(g[f"fourier_{k}_accepted"]):
            est = init.estimate(g[f"fourier_{k}_tgt"])
            r = g[f"fourier_{k}_result"]
            assert (est["dx"], est["dy"]) == (int(r[0]), int(r[1]))
            np.testing.assert_allclose([est["peakScore"], est["overlap"], est["correlation"]], r[2:], rtol=1e-7)
        else:
            with pytest.raises(ValueError, match="ambiguous"):
                init.estimate(g[f"fourier_{k}_tgt"])
        init.close()


@pytest.mark.parametrize("shift", [(23.4, -17.7), (-41.0, 9.5), (3.2, 2.9)])
def test_matches_oracle_on_speckle(shift):
    ref, sp = synthetic.reference_image(700, 520, seed=19, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(shift[0], 0.0, 0.0, shift[1], 0.0, 0.0),
                                   noise_seed=20, device="cpu")
    init = FourierInitializer(ref)
    est = init.estimate(tgt)
    expected = fourier_oracle.estimate(ref, tgt)
    assert (est["dx"], est["dy"]) == (expected["dx"], expected["dy"])
    np.testing.assert_allclose([est["peakScore"], est["overlap"], est["correlation"]],
                               [expected["peakScore"], expected["overlap"], expected["correlation"]], rtol=1e-7)
    assert abs(est["dx"] - shift[0]) <= 2.0 and abs(est["dy"] - shift[1]) <= 2.0


def test_fourier_seeds_the_pyramid_beyond_its_capture_range():
    ref, sp = synthetic.reference_image(512, 448, seed=23, device="cpu")
    truth = (47.3, -38.6)
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(truth[0], 0.0, 0.0, truth[1], 0.0, 0.0),
                                   noise_seed=24, device="cpu")
    common = dict(pyramid_levels=2, subset_size=21, subset_stride=10)
    with ICGNWGPUFullPyramid(**common) as plain:
        plain.set_reference(ref)
        zero = plain.register(tgt)
    with ICGNWGPUFullPyramid(initialization="fourier", **common) as engine:
        engine.set_reference(ref)
        result = engine.register(tgt)
        streamed = list(engine.register_stream([tgt, tgt], pipeline_depth=2))
        with pytest.raises(ICGNError, match="ambiguous|texture"):
            engine.register(np.random.default_rng(0).integers(0, 256, ref.shape, dtype=np.uint8))
    est = result.config["globalTranslation"]
    assert abs(est["dx"] - truth[0]) <= 2 and abs(est["dy"] - truth[1]) <= 2
    assert "fourierWallMs" in result.timing
    good = (result.status >= 1) & (np.abs(result.displacement - truth).max(-1) < 0.05)
    good_zero = (zero.status >= 1) & (np.abs(zero.displacement - truth).max(-1) < 0.05)
    assert good.mean() > 0.6 and good_zero.mean() < 0.1
    for r in streamed:
        np.testing.assert_array_equal(r.parameters, result.parameters)


@pytest.mark.parametrize("shift", [(23.4, -17.7), (-41.0, 9.5)])
def test_device_shift_rows_match_host_estimate(shift):
    """The stream-ordered variant leaves the host path's accepted integer shift
    in rows of affine parameters on the device (columns 0 and 3)."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    from live_dic_gb300 import _native

    ref, sp = synthetic.reference_image(700, 520, seed=19, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(shift[0], 0.0, 0.0, shift[1], 0.0, 0.0),
                                   noise_seed=20, device="cpu")
    init = FourierInitializer(ref)
    est = init.estimate(tgt)
    lib = _native.load()
    frame = torch.from_numpy(tgt).cuda()
    rows = torch.full((37, 16), 7.0, device="cuda")
    flat = torch.zeros(520, 700, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for image, accepted in ((frame, True), (flat, False)):
        code = lib.gbdic_fourier_shift_device(init._handle, C.c_void_p(image.data_ptr()), 700, 520, init.window["x"],
                                              init.window["y"], C.c_float(0.5), C.c_void_p(rows.data_ptr()), 37, 16,
                                              C.c_void_p(stream))
        _native.check(code, lib.gbdic_fourier_last_error(init._handle))
        r = rows.cpu().numpy()
        expected = (0.5 * est["dx"], 0.5 * est["dy"]) if accepted else (0.0, 0.0)
        np.testing.assert_array_equal(r[:, 0], np.full(37, expected[0], np.float32))
        np.testing.assert_array_equal(r[:, 3], np.full(37, expected[1], np.float32))
        assert (r[:, [1, 2, 4, 5]] == 7.0).all()
    # the host path still agrees after a device-path call on the same handle
    again = init.estimate(tgt)
    assert (again["dx"], again["dy"], again["peakScore"]) == (est["dx"], est["dy"], est["peakScore"])
    init.close()
