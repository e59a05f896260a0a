"""Batched registration of uneven jobs: every job's field must be
bit-identical to a solo ICGNWGPU.register with the same lanes per subset,
whatever the step mode (one persistent launch per shape-function class over
the work queue, one persistent launch over every job, or one launch per
job), and the resident path must agree with the host path."""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNBatch, ICGNWGPU, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pairs():
    jobs = synthetic.uneven_workload(11, count=6, sizes=((160, 128), (240, 200), (200, 176)), subsets=(15, 21),
                                     peak=(0.3, 1.2), device="cpu")
    ref, sp = synthetic.reference_image(144, 144, seed=5, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(0.6, 0.0, 0.0, -0.4, 0.0, 0.0), noise_seed=6,
                                   device="cpu")
    jobs.append({"reference": ref, "target": tgt, "motion_model": "translation", "subset_size": 17,
                 "subset_stride": 6, "roi_mask": None})
    assert {j["motion_model"] for j in jobs} == {"affine", "quadratic", "translation"}
    return jobs


def _solo(job, lanes):
    with ICGNWGPU(motion_model=job["motion_model"], subset_size=job["subset_size"],
                  subset_stride=job["subset_stride"]) as engine:
        engine.set_solver_variant(lanes, False)
        engine.set_reference(job["reference"], roi_mask=job["roi_mask"])
        r = engine.register(job["target"])
    return np.concatenate([r.parameters, r.status[..., None], r.iterations[..., None]], -1)


def _batch(pairs, **variant):
    batch = ICGNBatch(**variant)
    for job in pairs:
        batch.add(job["reference"], motion_model=job["motion_model"], subset_size=job["subset_size"],
                  subset_stride=job["subset_stride"], roi_mask=job["roi_mask"])
    return batch


def _packed(result):
    return np.concatenate([result.parameters, result.status[..., None], result.iterations[..., None]], -1)


@pytest.mark.parametrize("lanes", [16, 32, 64, 128])
def test_batch_matches_solo_engines(pairs, lanes):
    expected = [_solo(job, lanes) for job in pairs]
    with _batch(pairs, solver_workgroup_size=lanes) as batch:
        assert batch.variant[1] == "single"
        batch.set_variant(lanes, "persistent")
        persistent = batch.register([j["target"] for j in pairs])
        batch.set_variant(lanes, "per-job")
        per_job = batch.register([j["target"] for j in pairs])
        batch.set_variant(lanes, "persistent", 1)
        one_cta = batch.register([j["target"] for j in pairs])
        batch.set_variant(lanes, "single")
        single = batch.register([j["target"] for j in pairs])
        batch.set_variant(lanes, "single", 1)
        single_one_cta = batch.register([j["target"] for j in pairs])
    for k, job in enumerate(pairs):
        np.testing.assert_array_equal(_packed(persistent[k]), expected[k], err_msg=f"job {k} ({job['motion_model']})")
        np.testing.assert_array_equal(_packed(per_job[k]), expected[k])
        np.testing.assert_array_equal(_packed(one_cta[k]), expected[k])
        np.testing.assert_array_equal(_packed(single[k]), expected[k], err_msg=f"job {k} ({job['motion_model']})")
        np.testing.assert_array_equal(_packed(single_one_cta[k]), expected[k])


def test_batch_accuracy_and_roi(pairs):
    with _batch(pairs) as batch:
        results = batch.register([j["target"] for j in pairs])
        infos = batch.jobs
    for job, info, r in zip(pairs, infos, results, strict=True):
        ok = r.status == 1
        inside = r.status != -3
        assert ok[inside].mean() > 0.8, (info, ok[inside].mean())
        if job["roi_mask"] is not None and not job["roi_mask"].all():
            assert (r.status[~info.roi.selected] == -3).all()
        if "field" in job:
            cx, cy = synthetic.subset_centres(info.width, info.height, info.subset_size, info.subset_stride)
            u, v = job["field"](cx, cy)
            err = r.displacement[ok] - np.stack([u, v], -1)[ok]
            assert float(np.sqrt(np.mean(np.sum(err * err, -1)))) < 0.05


def test_resident_path_matches_host_path(pairs):
    torch = pytest.importorskip("torch")
    with _batch(pairs) as batch:
        host = batch.register([j["target"] for j in pairs])
        frames = [torch.from_numpy(j["target"]).cuda() for j in pairs]
        for k, f in enumerate(frames):
            batch.load_device(k, f.data_ptr(), f.stride(0))
        ms = batch.run_device(timed=True)
        assert ms > 0.0
        for k in range(len(pairs)):
            expected = _packed(host[k])
            np.testing.assert_array_equal(batch.export_state(k)[..., :expected.shape[-1]], expected)
        solver_ms = batch.run_device(profile=True)
        assert 0.0 < solver_ms
        for k in range(len(pairs)):
            expected = _packed(host[k])
            np.testing.assert_array_equal(batch.export_state(k)[..., :expected.shape[-1]], expected)


def test_batch_autotuner_keeps_a_valid_variant(pairs):
    with _batch(pairs) as batch:
        best = batch.autotune([j["target"] for j in pairs], repeats=1)
        assert batch.validation[batch.variant_name]["valid"]
        assert best == batch.variant
        # 4 lane counts x (persistent, persistent 2/SM, single, single 2/SM, per-job)
        assert len(batch.tuning_ms) == 20


def test_batch_argument_errors(pairs):
    with ICGNBatch() as batch:
        with pytest.raises(ValueError, match="translation and affine"):
            batch.add(pairs[0]["reference"], motion_model="quadratic", subset_size=15,
                      roi_mask=np.ones(pairs[0]["reference"].shape, bool))
        with pytest.raises(ValueError, match="outlier_policy"):
            batch.add(pairs[0]["reference"], outlier_policy="median")
        from live_dic_gb300 import ICGNError

        with pytest.raises(ICGNError, match="Add at least one job"):
            batch.register([])
        batch.add(pairs[0]["reference"], subset_size=15)
        with pytest.raises(ValueError, match="expected 1 targets"):
            batch.register([])
        with pytest.raises(ValueError, match="does not match"):
            batch.register([np.zeros((32, 32), np.uint8)])
