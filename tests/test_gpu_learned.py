"""The learned seed network on the GPU: forward and backward (tcgen05 BF16
GEMMs) against the CPU oracle with the same BF16 rounding points, training
on engine-generated pairs, and what the trained proposals gain over the
plain pyramid + ZNCC seeding at equal accuracy."""

from __future__ import annotations

import numpy as np
import pytest

from live_dic_gb300 import ICGNWGPU, learned, synthetic
from oracle import cnn_oracle as cnn

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _load_oracle_params(net, weights, biases, w6, b6):
    for i, (w, b) in enumerate(zip(weights, biases, strict=True)):
        net.w[i].zero_()
        net.w[i][:, :w.shape[1]] = torch.as_tensor(w, dtype=torch.float32)
        net.b[i].copy_(torch.as_tensor(b, dtype=torch.float32))
    net.w6.zero_()
    net.w6[:6] = torch.as_tensor(w6, dtype=torch.float32)
    net.b6.zero_()
    net.b6[:6] = torch.as_tensor(b6, dtype=torch.float32)
    net.pack()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_and_backward_match_oracle():
    B = 128
    net = learned.SeedNet(batch=B, seed=1)
    weights, biases, w6, b6 = cnn.init(2)
    _load_oracle_params(net, weights, biases, w6, b6)
    rng = np.random.default_rng(4)
    x0 = cnn.bf16(rng.normal(0, 1, (B, 64, 64, 2)).astype(np.float32))
    target = rng.normal(0, 1, (B, 6)).astype(np.float32)
    net.x0.copy_(torch.as_tensor(x0, dtype=torch.float32).to(torch.bfloat16))
    net.forward()
    net.loss_and_grad(torch.as_tensor(target, device=net.device))
    net.backward()
    torch.cuda.synchronize()
    net.check_device_errors()
    acts, out = cnn.forward(x0, weights, biases, w6, b6, rounded=True)
    got = net.out[:, :6].cpu().numpy()
    assert _rel(got, out) < 1e-2
    assert abs(float(net.loss.item()) - cnn.loss(out, target)) <= 1e-2 * cnn.loss(out, target)
    dws, dbs, dw6, db6 = cnn.backward(acts, out, target, weights, w6, rounded=True)
    for i, (dw, db) in enumerate(zip(dws, dbs, strict=True)):
        g = net.grads[i].cpu().numpy()
        assert _rel(g[:, :dw.shape[1]], dw) < 3e-2, i
        assert np.abs(g[:, dw.shape[1]:]).max(initial=0.0) == 0.0
        assert _rel(net.grads[len(dws) + i].cpu().numpy(), db) < 3e-2, i
    assert _rel(net.grads[2 * len(dws)].cpu().numpy()[:6], dw6) < 3e-2
    assert _rel(net.grads[2 * len(dws) + 1].cpu().numpy()[:6], db6) < 3e-2
    assert np.abs(net.grads[2 * len(dws)].cpu().numpy()[6:]).max() == 0.0


def test_training_and_learned_seeding_gain():
    """What the trained network gains over the method without it, under the
    learned seeding's evaluation conditions (a 3840x2160 frame, a 25 px
    translation, strain and shear of 1-2 %): it reaches the plain path's
    accuracy (the same GPU phase-correlation shift as the Fourier seed of a
    3-level pyramid, an integer ZNCC search centred on it sized to the
    strain residual, IC-GN at every level) in less time."""
    import time

    from live_dic_gb300 import ICGNWGPUFullPyramid

    data = learned.training_pairs(256, size=320, seed=5)
    assert data.size > 250_000
    net = learned.SeedNet(batch=256, seed=0)
    losses = learned.train(net, data, steps=3000, lr=2e-3, log_every=100)
    assert losses[-1] < 0.3 * losses[0], losses

    W, H, S, st = 3840, 2160, 31, 8
    ref, sp = synthetic.reference_image(W, H, seed=901, device="cuda")
    params = (19.5, 0.02, -0.01, -16.3, 0.01, -0.018)
    c = (0.5 * (W - 1), 0.5 * (H - 1))

    def field(X, Y):
        return (params[0] + params[1] * (X - c[0]) + params[2] * (Y - c[1]),
                params[3] + params[4] * (X - c[0]) + params[5] * (Y - c[1]))

    tgt = synthetic.deformed_image(sp, field, noise_seed=902, device="cuda")
    frame = torch.from_numpy(tgt).cuda()
    cx, cy = synthetic.subset_centres(W, H, S, st)
    u, v = field(cx, cy)
    truth = np.stack([u, v], -1)
    inside = (cx - 15 + u > 4) & (cx + 15 + u < W - 5) & (cy - 15 + v > 4) & (cy + 15 + v < H - 5)

    def timed(step, repeats=5):
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        times = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            out = step()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        return float(np.median(times)), out

    def accuracy(state):
        ok = state[..., 6] >= 1
        err = np.linalg.norm(state[..., [0, 3]][ok & inside] - truth[ok & inside], axis=-1)
        return float(ok[inside].mean()), float(np.sqrt(np.mean(err ** 2)))

    # plain: phase-correlation shift -> Fourier seed -> pyramid with a centred search
    residual = abs(params[1]) * c[0] + abs(params[2]) * c[1] + abs(params[4]) * c[0] + abs(params[5]) * c[1]
    radius = int(np.ceil(residual / 4)) + 2
    with ICGNWGPUFullPyramid(pyramid_levels=3, subset_size=S, subset_stride=st, initialization="fourier",
                             seed_search_radius=radius) as plain:
        info = plain.set_reference(ref)
        gw, gh = info.grid
        pstate = torch.zeros(gw * gh * 8, device="cuda")
        shifter = learned.HalfResolutionShift(W, H)
        shifter.set_reference_frame(torch.from_numpy(ref).cuda())
        stream = torch.cuda.Stream()

        def plain_step():
            shift = shifter.shift_of(frame, stream)
            plain.register_device(frame.data_ptr(), pstate.data_ptr(), stream=stream.cuda_stream, translation=shift)
            stream.synchronize()
            return pstate.view(gh, gw, 8).cpu().numpy()

        plain_s, plain_state = timed(plain_step)
        shifter.close()
        fine_iterations, fine_tolerance = plain.iterations_per_level[-1], plain.tolerance_per_level[-1]
    with ICGNWGPU(subset_size=S, subset_stride=st) as engine:
        engine.set_reference(ref, iterations=fine_iterations, tolerance=fine_tolerance)
        seeder = learned.LearnedSeeder(engine, net, step=16)
        seeder.set_reference_image(ref)
        seeder.propose(frame)
        proposals = seeder.seeds.view(engine.grid_height, engine.grid_width, 8).cpu().numpy()

        def learned_step():
            seeder.register_device(frame, counts=False)
            return seeder.state.view(engine.grid_height, engine.grid_width, 8).cpu().numpy()

        learned_s, learned_state = timed(learned_step)
    learned_ok, learned_rmse = accuracy(learned_state)
    plain_ok, plain_rmse = accuracy(plain_state)
    assert learned_ok > 0.95 and plain_ok > 0.9, (learned_ok, plain_ok)
    assert learned_rmse < 0.02 and abs(learned_rmse - plain_rmse) < 0.005, (learned_rmse, plain_rmse)
    proposal_error = np.abs(proposals[..., [0, 3]] - truth)[inside].max(-1)
    assert np.median(proposal_error) < 5.0
    assert learned_s < plain_s, (learned_s, plain_s)


@pytest.mark.parametrize("lw,lh,outliers", [(40, 23, 0.3), (4, 3, 0.0), (12, 9, 0.6)])
def test_device_consensus_matches_host_statement(lw, lh, outliers):
    """gbdic_nn_consensus against fit_consensus on the same tables: an affine
    field through lattice translations with planted outliers and non-finite
    predictions."""
    import ctypes as C

    from live_dic_gb300 import _native

    lib = _native.load()
    rng = np.random.default_rng(lw * 100 + lh)
    n = lw * lh
    gy, gx = np.mgrid[0:lh, 0:lw] * 64.0
    node = np.stack([gx.ravel(), gy.ravel()], -1)
    xy = ((node - node.mean(0)) / 1000.0).astype(np.float32)
    truth = np.stack([12.0 + 8.0 * xy[:, 0] - 5.0 * xy[:, 1], -7.0 + 3.0 * xy[:, 0] + 11.0 * xy[:, 1]], -1)
    t = truth + rng.normal(0.0, 0.4, truth.shape)
    bad = rng.random(n) < outliers
    t[bad] = rng.uniform(-40.0, 40.0, (int(bad.sum()), 2))
    if n > 20:
        t[[3, 17]] = np.nan
    scale = learned.TRANSLATION_SCALE
    pred = np.zeros((n, learned.OUT_PAD), np.float32)
    base = np.zeros((n, learned.OUT_PAD), np.float32)
    split = rng.uniform(-0.3, 0.3, (n, 2)).astype(np.float32)
    base[:, [0, 3]] = split
    pred[:, [0, 3]] = (t / scale - split).astype(np.float32)
    totals = (base[:, [0, 3]].astype(np.float64) + pred[:, [0, 3]].astype(np.float64)) * scale
    tables = learned.consensus_tables(n)
    expected = learned.fit_consensus(totals, xy.astype(np.float64), tables)
    d_pred, d_base = torch.from_numpy(pred).cuda(), torch.from_numpy(base).cuda()
    d_xy = torch.from_numpy(xy).cuda()
    d_tab = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in tables]
    tol = np.array(learned.CONSENSUS_TOLERANCES, np.float32)
    code = lib.gbdic_nn_consensus(C.c_void_p(d_pred.data_ptr()), C.c_void_p(d_base.data_ptr()), learned.OUT_PAD, n,
                                  C.c_void_p(d_xy.data_ptr()), C.c_void_p(d_tab[0].data_ptr()), len(tables[0]),
                                  C.c_void_p(d_tab[1].data_ptr()), len(tables[1]), C.c_void_p(d_tab[2].data_ptr()),
                                  len(tables[2]), tol.ctypes.data_as(C.c_void_p), len(tol), C.c_float(scale), None)
    assert code == 0
    torch.cuda.synchronize()
    got = d_base.cpu().numpy()
    np.testing.assert_allclose(got[:, [0, 3]].astype(np.float64) * scale, expected, atol=1e-3)
    assert (got[:, [1, 2, 4, 5]] == base[:, [1, 2, 4, 5]]).all()
    if outliers <= 0.3:
        np.testing.assert_allclose(expected, truth, atol=0.6)


def test_reseed_selection_and_row_merge():
    import ctypes as C

    from live_dic_gb300 import _native

    lib = _native.load()
    rng = np.random.default_rng(3)
    n = 5000
    state = rng.normal(size=(n, 8)).astype(np.float32)
    state[:, 6] = rng.choice([1.0, 0.0, -1.0, -2.0, 2.0], n)
    usable = (rng.random(n) < 0.9).astype(np.uint8)
    d_state, d_usable = torch.from_numpy(state).cuda(), torch.from_numpy(usable).cuda()
    mask = torch.full((n,), 9, dtype=torch.uint8, device="cuda")
    active = torch.full((n,), 9, dtype=torch.int32, device="cuda")
    counter = torch.full((1,), 123, dtype=torch.int32, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    assert lib.gbdic_nn_reseed_select(P(d_state), 8, P(d_usable), n, P(mask), P(active), P(counter), None) == 0
    expected = ((state[:, 6] == 0.0) | (state[:, 6] == -2.0)) & (usable != 0)
    np.testing.assert_array_equal(mask.cpu().numpy(), expected.astype(np.uint8))
    np.testing.assert_array_equal(active.cpu().numpy(), expected.astype(np.int32))
    assert int(counter.item()) == int(expected.sum())
    src = torch.from_numpy(rng.normal(size=(n, 8)).astype(np.float32)).cuda()
    assert lib.gbdic_nn_merge_rows(P(src), P(mask), n, 8, P(d_state), None) == 0
    merged = d_state.cpu().numpy()
    np.testing.assert_array_equal(merged[expected], src.cpu().numpy()[expected])
    np.testing.assert_array_equal(merged[~expected], state[~expected])


def test_resolve_reuses_the_prefiltered_frame():
    """gbdic_resolve_seeded_device on the frame of the previous seeded
    registration gives the same states as a fresh seeded registration."""
    import ctypes as C

    ref, sp = synthetic.reference_image(320, 256, seed=41, device="cpu")
    tgt = synthetic.deformed_image(sp, synthetic.affine_field(2.3, 0.004, -0.002, -1.6, 0.001, 0.003),
                                   noise_seed=42, device="cpu")
    with ICGNWGPU(subset_size=21, subset_stride=10) as engine:
        engine.set_reference(ref)
        n = engine.grid_width * engine.grid_height
        rng = np.random.default_rng(5)
        seeds = np.zeros((n, 8), np.float32)
        seeds[:, 0] = 2.3 + rng.normal(0, 0.3, n)
        seeds[:, 3] = -1.6 + rng.normal(0, 0.3, n)
        active = (rng.random(n) < 0.3).astype(np.int32)
        d_frame = torch.from_numpy(tgt).cuda()
        d_seed, d_active = torch.from_numpy(seeds).cuda(), torch.from_numpy(active).cuda()
        other = torch.from_numpy(np.ascontiguousarray(tgt[::-1])).cuda()
        a, b = torch.zeros(n * 8, device="cuda"), torch.zeros(n * 8, device="cuda")
        cfg = C.byref(engine._cfg(engine._config))
        P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        lib = engine._lib
        engine._check(lib.gbdic_register_seeded_device(engine._handle, P(d_frame), P(d_seed), P(d_active), cfg, P(a),
                                                       None))
        # prefilter another frame, then the frame of interest, then resolve
        engine._check(lib.gbdic_register_seeded_device(engine._handle, P(other), P(d_seed), P(d_active), cfg, P(b),
                                                       None))
        engine._check(lib.gbdic_register_seeded_device(engine._handle, P(d_frame), P(d_seed), P(d_active), cfg, P(b),
                                                       None))
        b.zero_()
        engine._check(lib.gbdic_resolve_seeded_device(engine._handle, P(d_frame), P(d_seed), P(d_active), cfg, P(b),
                                                      None))
        torch.cuda.synchronize()
        np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
        assert (a.view(-1, 8)[:, 6].cpu().numpy()[active == 1] >= 1).mean() > 0.9


def test_direct_first_layer_matches_the_gemm_path():
    """The inference form of the input layer (direct convolution, weights as
    constant operands) against im2col + tcgen05 GEMM on the same patches:
    identical up to the FP32 summation order before BF16 rounding."""
    gemm = learned.SeedNet(batch=128, seed=3)
    direct = learned.SeedNet(batch=128, seed=3)
    direct.use_direct_first_layer()
    rng = np.random.default_rng(9)
    x = torch.from_numpy(rng.normal(size=(128, 64, 64, 2)).astype(np.float32)).to(torch.bfloat16).cuda()
    gemm.x0.copy_(x)
    direct.x0.copy_(x)
    gemm.forward()
    direct.forward()
    torch.cuda.synchronize()
    y0, y1 = gemm.y[0].float(), direct.y[0].float()
    close = (y0 - y1).abs() <= 1e-2 * y0.abs() + 1e-3
    assert close.float().mean().item() > 0.999
    np.testing.assert_allclose(direct.out[:, :6].cpu().numpy(), gemm.out[:, :6].cpu().numpy(), rtol=2e-2, atol=2e-2)


def test_split_k_forward_matches_the_single_pass_forward():
    """The inference copies' split-K deep layers (FP32 partials, ordered sum,
    bias and ReLU) against the single-pass tcgen05 epilogue on the same
    weights and patches: identical up to the FP32 summation order before
    BF16 rounding."""
    plain = learned.SeedNet(batch=128, seed=3)
    split = learned.SeedNet(batch=128, seed=3, split_forward=True)
    assert max(split.fwd_splits) > 1 and max(plain.fwd_splits) == 1
    rng = np.random.default_rng(10)
    x = torch.from_numpy(rng.normal(size=(128, 64, 64, 2)).astype(np.float32)).to(torch.bfloat16).cuda()
    plain.x0.copy_(x)
    split.x0.copy_(x)
    plain.forward()
    split.forward()
    torch.cuda.synchronize()
    for a, b in zip(plain.y, split.y, strict=True):
        a, b = a.float(), b.float()
        assert ((a - b).abs() <= 1e-2 * a.abs() + 1e-3).float().mean().item() > 0.999
    np.testing.assert_allclose(split.out[:, :6].cpu().numpy(), plain.out[:, :6].cpu().numpy(), rtol=2e-2, atol=2e-2)


def test_learned_seeding_on_a_non_affine_field():
    """Large translation plus sinusoidal deformation (no global affine
    model fits it): the consensus only recentres the second pass, the lattice
    nodes are solved from the network's own proposals and every subset is
    seeded by interpolating them.  The result must match the same solver
    seeded with the exact field (the affine subset's own model error, about
    0.026 px here, is common to both)."""
    data = learned.training_pairs(256, size=320, seed=15)
    net = learned.SeedNet(batch=256, seed=1)
    learned.train(net, data, steps=3000, lr=2e-3, log_every=1000)
    W, H = 1024, 768
    ref, sp = synthetic.reference_image(W, H, seed=907, device="cuda")
    k1, k2 = 2 * np.pi / 300.0, 2 * np.pi / 250.0

    def field(X, Y):
        lib = torch if isinstance(X, torch.Tensor) else np
        return 17.3 + 1.5 * lib.sin(k1 * X), -12.1 + 1.0 * lib.cos(k2 * Y)

    tgt = synthetic.deformed_image(sp, field, noise_seed=908, device="cuda")
    cx, cy = synthetic.subset_centres(W, H, 31, 8)
    u, v = field(cx, cy)
    exact = np.stack([u, 1.5 * k1 * np.cos(k1 * cx), np.zeros_like(u), v, np.zeros_like(v),
                      -1.0 * k2 * np.sin(k2 * cy)], -1).astype(np.float32)
    with ICGNWGPU(subset_size=31, subset_stride=8) as engine:
        engine.set_reference(ref, iterations=16, tolerance=5e-3)
        seeded = engine.register_seeded(tgt, exact, np.ones(u.shape, bool))
        seeder = learned.LearnedSeeder(engine, net, step=4)
        seeder.set_reference_image(ref)
        stats = seeder.register_device(torch.from_numpy(tgt).cuda())
        state = seeder.state.view(engine.grid_height, engine.grid_width, 8).cpu().numpy()
    inside = (cx - 15 + u > 4) & (cx + 15 + u < W - 5) & (cy - 15 + v > 4) & (cy + 15 + v < H - 5)
    ok = state[..., 6] >= 1
    assert ok[inside].mean() > 0.95
    err = np.hypot(state[..., 0] - u, state[..., 3] - v)[ok & inside]
    assert (err >= 0.5).mean() < 0.002
    both = ok & inside & (seeded.status >= 1)
    assert both.sum() > 0.9 * inside.sum()
    gap = np.hypot(state[..., 0] - seeded.displacement[..., 0], state[..., 3] - seeded.displacement[..., 1])[both]
    assert np.percentile(gap, 99) < 0.01, np.percentile(gap, 99)
    assert stats["reseeded"] < 0.1 * inside.sum()


def test_graph_replay_and_listed_solves_match_the_direct_sequence():
    """The learned frame captured as a CUDA graph (frame read from a fixed
    buffer), and the node solve / reseeding run over compact subset lists,
    give the direct masked full-grid sequence's states and reseed counts bit
    for bit, frame after frame, and again after the reference is replaced.
    An untrained network is enough (it leaves many subsets to reseed): what
    is checked is the identity of the paths."""
    net = learned.SeedNet(batch=128, seed=3)
    W, H = 512, 384
    ref, sp = synthetic.reference_image(W, H, seed=31, device="cuda")
    moves = [(3.2, -1.4), (6.1, 2.2), (-4.5, 5.0)]
    frames = [torch.from_numpy(synthetic.deformed_image(sp, synthetic.affine_field(dx, 2e-3, 0.0, dy, 0.0, -1e-3),
                                                        noise_seed=40 + k, device="cuda")).cuda()
              for k, (dx, dy) in enumerate(moves)]
    for lanes in (16, 128):
        _graph_and_list_identity(net, ref, frames, lanes)


def _graph_and_list_identity(net, ref, frames, lanes):
    # masked full-grid solves at the engine's lane count vs listed solves at
    # the same lane count (list_lanes = lanes)
    with ICGNWGPU(subset_size=31, subset_stride=8, solver_workgroup_size=lanes) as engine:
        engine.set_reference(ref, iterations=16, tolerance=5e-3)
        seeders = {(g, l): learned.LearnedSeeder(engine, net, step=4, graph=g, listed=l, list_lanes=lanes)
                   for g, l in ((False, False), (True, True), (False, True))}
        for rnd in range(2):
            for s in seeders.values():
                s.set_reference_image(ref if rnd == 0 else frames[0].cpu().numpy())
            for f in frames:
                out = {}
                for g, s in seeders.items():
                    stats = s.register_device(f)
                    torch.cuda.synchronize()
                    out[g] = (s.state.cpu().numpy().copy(), stats["reseeded"])
                base = out[(False, False)]
                assert base[1] > 0
                for key in ((True, True), (False, True)):
                    np.testing.assert_array_equal(out[key][0], base[0], err_msg=str(key))
                    assert out[key][1] == base[1]
        assert seeders[(True, True)]._graph is not None and seeders[(False, True)]._graph is None
        # the stage breakdown runs the direct sequence: same state again
        seeder = seeders[(False, True)]
        seeder.register_device(frames[-1])
        torch.cuda.synchronize()
        expected = seeder.state.cpu().numpy().copy()
        stages = seeder.stage_times(frames[-1])
        np.testing.assert_array_equal(seeder.state.cpu().numpy(), expected)
        assert {"half frame + shift", "network pass 1", "consensus", "network pass 2", "node solve", "full solve",
                "reseeding"} <= set(stages)
        assert all(v >= 0.0 for v in stages.values())
        assert abs(sum(v for k, v in stages.items() if k != "total") - stages["total"]) <= 1e-3 * stages["total"] + 1e-3
