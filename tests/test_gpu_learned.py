"""The learned seed network on the GPU: forward and backward (tcgen05 BF16
GEMMs) against the CPU oracle with the same BF16 rounding points, training
on engine-generated pairs, and what the trained proposals gain over the
zero-seeded solver."""

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
    data = learned.training_pairs(256, size=320, seed=5)
    assert data.size > 250_000
    net = learned.SeedNet(batch=256, seed=0)
    losses = learned.train(net, data, steps=3000, lr=2e-3, log_every=100)
    assert losses[-1] < 0.3 * losses[0], losses

    ref, sp = synthetic.reference_image(512, 448, seed=901, device="cuda")
    params = (14.5, 0.01, -0.006, -11.3, 0.004, -0.008)
    c = (255.5, 223.5)

    def field(X, Y):
        return (params[0] + params[1] * (X - c[0]) + params[2] * (Y - c[1]),
                params[3] + params[4] * (X - c[0]) + params[5] * (Y - c[1]))

    tgt = synthetic.deformed_image(sp, field, noise_seed=902, device="cuda")
    with ICGNWGPU(subset_size=31, subset_stride=8) as engine:
        engine.set_reference(ref)
        zero = engine.register(tgt)
        seeder = learned.LearnedSeeder(engine, net, step=2)
        seeder.set_reference_image(ref)
        frame = torch.from_numpy(tgt).cuda()
        seeder.propose(frame)
        proposals = seeder.seeds.view(engine.grid_height, engine.grid_width, 8).cpu().numpy()
        stats = seeder.register_device(frame)
        state = seeder.state.view(engine.grid_height, engine.grid_width, 8).cpu().numpy()
    cx, cy = synthetic.subset_centres(512, 448, 31, 8)
    u, v = field(cx, cy)
    truth = np.stack([u, v], -1)
    inside = (cx - 15 + u > 4) & (cx + 15 + u < 507) & (cy - 15 + v > 4) & (cy + 15 + v < 443)
    zero_ok = (zero.status == 1)[inside].mean()
    ok = state[..., 6] >= 1
    assert zero_ok < 0.3
    assert ok[inside].mean() > 0.95
    err = state[..., [0, 3]][ok & inside] - truth[ok & inside]
    assert float(np.sqrt(np.mean(np.sum(err * err, -1)))) < 0.02
    proposal_error = np.abs(proposals[..., [0, 3]] - truth)[inside].max(-1)
    assert np.median(proposal_error) < 5.0
    assert stats["reseeded"] < 0.3 * inside.sum()
