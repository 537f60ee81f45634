"""Learned surrogate: tensor-core GEMM, network inputs, gradients and Adam
against the CPU oracle of the network, training, inference with the traced
audit, checkpoints.

Tolerances (written per test): the GEMM accumulates BF16 products in FP32,
so it must match an FP64 sum of the same BF16 products to 1e-5 relative to
the largest output; gradients are compared with the oracle per layer in
Frobenius norm (3e-2 relative: BF16 activations that round differently after
FP32-vs-FP64 accumulation differ by one BF16 step and move the gradient a
little), and by cosine similarity (> 0.999).
"""
import os
import tempfile
import time

import numpy as np
import pytest

from anacor_public_gb300 import _lib, build, surrogate, synth, tracer
from oracle import surrogate_oracle as so

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()


def _bf(x):
    return so.bf16(x)


@pytest.mark.parametrize("M,N,K,batch,ksplit", [
    (128, 64, 64, 1, 1),
    (128, 128, 128, 2, 1),
    (256, 256, 256, 2, 1),
    (384, 256, 64, 3, 1),
    (256, 256, 1024, 2, 4),
    (256, 64, 2048, 1, 16),
])
def test_tc_gemm_matches_fp64(M, N, K, batch, ksplit):
    rng = np.random.default_rng(M + N + K + batch)
    A = rng.standard_normal((batch, M, K)).astype(np.float32)
    B = rng.standard_normal((batch, N, K)).astype(np.float32)
    C = surrogate.tc_gemm(A, B, ksplit=ksplit)
    ref = np.einsum("zmk,znk->zmn", _bf(A), _bf(B))
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def test_tc_gemm_structured():
    # identity-like operands expose any row / column / K-slice permutation exactly
    M, N, K = 256, 256, 256
    A = np.zeros((M, K), np.float32)
    A[np.arange(M), (np.arange(M) * 37) % K] = 1.0
    B = np.arange(N * K, dtype=np.float32).reshape(N, K) % 251
    C = surrogate.tc_gemm(A, B)[0]
    ref = _bf(A) @ _bf(B).T
    assert np.array_equal(C, ref.astype(np.float32))


def _rotation(axis, w):
    x, y, z = axis
    c, s = np.cos(w), np.sin(w)
    k = 1 - c
    return np.array([[c + x * x * k, x * y * k - z * s, y * s + x * z * k],
                     [z * s + x * y * k, c + y * y * k, -x * s + y * z * k],
                     [-y * s + x * z * k, x * s + y * z * k, c + z * z * k]])


def test_inputs_match_host_rotation(small):
    x7 = surrogate.sample_inputs(small)
    F = small.F.reshape(3, 3)
    for i in range(0, small.n_refl, 37):
        T = (_rotation(small.omega_axis, small.omega[i]) @ F).T
        a = T @ small.xray
        b = T @ small.s1[i]
        want = np.concatenate([[(small.omega[i] / (2 * np.pi)) % 1.0], a / np.linalg.norm(a),
                               b / np.linalg.norm(b)])
        assert np.allclose(x7[i], want, atol=2e-6), i


def _check_grads(g_gpu, g_ref):
    hidden, (o5, ob5) = so.offsets()
    blocks = [(ow, ob) for ow, ob in hidden]
    spans = []
    for l, (ow, ob) in enumerate(blocks):
        spans.append((f"W{l + 1}", ow, ob))
        spans.append((f"b{l + 1}", ob, ob + so.WIDTH))
    spans += [("w5", o5, o5 + so.WIDTH), ("b5", ob5, ob5 + 1)]
    for name, a, b in spans:
        x, y = g_gpu[a:b].astype(np.float64), g_ref[a:b]
        rel = np.linalg.norm(x - y) / np.linalg.norm(y)
        cos = float(x @ y / (np.linalg.norm(x) * np.linalg.norm(y)))
        assert rel < 3e-2 and cos > 0.999, (name, rel, cos)


def test_gradients_match_oracle(small):
    model = surrogate.Surrogate(members=2, seed=3, fourier_scale=1.0)
    try:
        rows = 1024
        rng = np.random.default_rng(5)
        idx = rng.choice(small.n_refl, rows, replace=True)
        x7 = surrogate.sample_inputs(small)[idx]
        target = rng.standard_normal(rows).astype(np.float32)
        # perturb the biases so that every layer's bias gradient path is exercised
        p = model.get_params()
        hidden, (o5, ob5) = so.offsets()
        for ow, ob in hidden:
            p[:, ob:ob + so.WIDTH] = rng.normal(0, 0.1, (2, so.WIDTH))
        p[:, ob5] = 0.3
        model.set_params(p)
        g, y = model.gradients(x7, target)
        X0 = so.features(x7, model.get_fourier())
        for e in range(2):
            loss, y_ref, g_ref = so.loss_and_grads(p[e], X0, target.astype(np.float64))
            assert np.allclose(y[e], y_ref, rtol=0, atol=2e-2 * np.abs(y_ref).max()), e
            _check_grads(g[e], g_ref)
    finally:
        model.close()


def test_first_adam_step_moves_each_weight_by_lr(small):
    # from m = v = 0 the first Adam step is -lr * g / (|g| + eps): every
    # parameter with |g| >> eps moves by lr, whatever the batch
    model = surrogate.Surrogate(members=2, seed=11)
    try:
        x7 = surrogate.sample_inputs(small)
        model.set_data(x7, np.log(np.linspace(0.5, 0.9, small.n_refl)))
        p0 = model.get_params()
        lr = 1e-3
        loss = model.train(1, batch=1024, lr_max=lr, lr_min=lr)
        assert np.isfinite(loss).all()
        d = np.abs(model.get_params().astype(np.float64) - p0)
        moved = d[d > 0]
        assert moved.size > 0.9 * p0.size * (so.PARAM_COUNT - 7) / so.PARAM_COUNT
        # FP32 master arithmetic: the step is lr to FP32 rounding of p
        big = np.abs(p0.astype(np.float64)) < 4.0
        dd = d[(d > 0) & big]
        assert np.median(np.abs(dd - lr)) < 1e-6
    finally:
        model.close()


@pytest.fixture(scope="module")
def trained_small(small):
    s = small
    omega, s1, ah = surrogate.training_set(s, n=16384, seed=21)
    x7 = surrogate.inputs(omega, s1, s.xray, s.omega_axis, s.F)
    model = surrogate.Surrogate(members=4, seed=1, fourier_scale=0.5)
    model.set_data(x7, np.log(ah))
    loss = model.train(1500, batch=2048, lr_max=3e-3, lr_min=3e-5, total_steps=1500)
    yield model, loss
    model.close()


def test_training_reduces_loss(trained_small):
    _, loss = trained_small
    assert np.isfinite(loss).all()
    assert loss[-50:].mean() < 0.02 * loss[:10].mean()


def test_predict_matches_oracle_forward(small, trained_small):
    model, _ = trained_small
    x7 = surrogate.sample_inputs(small)[:256]
    mean, spread, mem = model.predict(x7, members=True)
    p = model.get_params()
    mu, sd = model.scale
    X0 = so.features(x7, model.get_fourier())
    la = []
    for e in range(model.members):
        _, _, y = so.forward(p[e], X0)
        la.append(mu + sd * y)
        assert np.allclose(mem[e], la[-1], atol=5e-3), e
    a = np.exp(np.array(mem, dtype=np.float64))
    assert np.allclose(mean, a.mean(axis=0), rtol=1e-5)
    assert np.allclose(spread, a.std(axis=0) / a.mean(axis=0), atol=1e-5)


def test_fused_inference_matches_layered(small, trained_small):
    """The fused kernel (features, four layers, head and ensemble statistics of
    a 128-row tile on chip) against the layer-by-layer GEMM path on the same
    rows, including a partial last tile: the same arithmetic, so the same
    numbers (compared to 1e-6 relative; reported when bitwise equal)."""
    model, _ = trained_small
    rng = np.random.default_rng(5)
    omega, s1 = synth.reflections(5000, rng, xray=small.xray)
    x7 = surrogate.inputs(omega, s1, small.xray, small.omega_axis, small.F)
    try:
        model.set_inference(False)
        m0, s0, e0 = model.predict(x7, members=True)
        model.set_inference(True)
        m1, s1_, e1 = model.predict(x7, members=True)
    finally:
        model.set_inference(True)
    assert np.all(np.isfinite(m1)) and np.all(np.isfinite(s1_))
    print(f"\nfused vs layered: mean bitwise {np.array_equal(m0, m1)}, members bitwise {np.array_equal(e0, e1)}, "
          f"max rel diff mean {np.max(np.abs(m1 - m0) / np.abs(m0)):.2e}")
    assert np.allclose(m1, m0, rtol=1e-6, atol=0)
    assert np.allclose(e1, e0, rtol=1e-6, atol=1e-7)
    assert np.allclose(s1_, s0, rtol=1e-4, atol=1e-8)


@pytest.mark.parametrize("members", [1, 3])
def test_fused_inference_matches_layered_odd_members(members):
    """The fused kernel runs members two at a time; an odd last member runs
    alone.  Untrained (seeded) weights, rows not a multiple of the tile."""
    rng = np.random.default_rng(members)
    x7 = rng.uniform(-1.0, 1.0, size=(3001, 7)).astype(np.float32)
    model = surrogate.Surrogate(members=members, seed=11, fourier_scale=0.5)
    try:
        model.set_inference(False)
        m0, s0, e0 = model.predict(x7, members=True)
        model.set_inference(True)
        m1, s1, e1 = model.predict(x7, members=True)
    finally:
        model.close()
    assert np.array_equal(e1, e0) and np.array_equal(m1, m0) and np.array_equal(s1, s0)


def test_bounded_wait_reports_and_releases():
    """A tensor-core wait that runs out sets the error word, releases its
    tensor memory and returns; the next tensor-core work runs normally."""
    import ctypes as ct
    L = _lib.load()
    st = ct.c_int32(-1)
    assert L.anacor_wait_guard_check(4096, ct.byref(st)) == 0, _lib.last_error(L)
    assert st.value == 1
    A = np.ones((128, 64), np.float32)
    C = surrogate.tc_gemm(A, A)
    assert np.all(C == 64.0)


def test_audited_absorption_small(small, trained_small):
    model, _ = trained_small
    rng = np.random.default_rng(99)
    omega, s1 = synth.reflections(4000, rng, xray=small.xray)
    plan = tracer.Plan(small.label, small.coords, small.voxel, small.mu)
    try:
        res = surrogate.audited_absorption(model, plan, omega, s1, small.xray, small.omega_axis, small.F,
                                           audit_fraction=0.05, spread_threshold=1e-3, seed=3)
        plan.set_reflections(s1, omega, small.xray, small.omega_axis, small.F)
        plan.run()
        plain = plan.result()
    finally:
        plan.close()
    # traced rows carry the plain kernel's values exactly
    assert np.array_equal(res.ah[res.traced_idx], plain[res.traced_idx])
    # the audit sample is about the requested fraction and its errors are the true errors
    n_audit = int(np.sum(res.flags & 1))
    assert 0.03 * 4000 < n_audit < 0.07 * 4000
    err_all = surrogate.relative_error(res.surrogate, plain)
    q = res.quantiles()
    assert q["q50"] < 1e-2 and np.median(err_all) < 1e-2, (q, np.median(err_all))
    # every reflection whose ensemble spread exceeds the threshold was traced
    assert np.all(res.flags[res.spread > 1e-3] & 2)
    final_err = surrogate.relative_error(res.ah, plain)
    assert np.all(final_err[res.traced_idx] == 0)


def test_surrogate_gain_over_plain(small, trained_small):
    """What the trained network buys: the same reflections at a fraction of
    the plain kernel's time, at the error the audit reports."""
    import torch

    model, _ = trained_small
    n = 65536
    rng = np.random.default_rng(123)
    omega, s1 = synth.reflections(n, rng, xray=small.xray)
    plan = tracer.Plan(small.label, small.coords, small.voxel, small.mu)
    try:
        plan.set_reflections(s1, omega, small.xray, small.omega_axis, small.F)
        plan.run()
        plan.result()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan.run()
        plain = plan.result()
        t_plain = time.perf_counter() - t0
    finally:
        plan.close()
    x7 = surrogate.inputs(omega, s1, small.xray, small.omega_axis, small.F)
    d_x = torch.from_numpy(x7).cuda()
    d_m = torch.empty(n, device="cuda")
    d_s = torch.empty(n, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    model.predict_device(d_x.data_ptr(), n, d_m.data_ptr(), d_s.data_ptr(), stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    model.predict_device(d_x.data_ptr(), n, d_m.data_ptr(), d_s.data_ptr(), stream)
    torch.cuda.synchronize()
    t_sur = time.perf_counter() - t0
    err = surrogate.relative_error(d_m.cpu().numpy(), plain)
    assert t_sur * 5 < t_plain, (t_sur, t_plain)
    assert np.median(err) < 1e-2


def test_checkpoint_round_trip(small, trained_small):
    model, _ = trained_small
    x7 = surrogate.sample_inputs(small)[:512]
    m0, s0 = model.predict(x7)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ens.bin")
        model.save(path)
        other = surrogate.Surrogate(members=4, seed=77)
        try:
            other.load(path)
            m1, s1 = other.predict(x7)
            assert model.scale == other.scale
        finally:
            other.close()
        wrong = surrogate.Surrogate(members=2, seed=77)
        try:
            with pytest.raises(Exception):
                wrong.load(path)
        finally:
            wrong.close()
    assert np.array_equal(m0, m1) and np.array_equal(s0, s1)


def test_audit_flags_rule():
    n = 200000
    rng = np.random.default_rng(8)
    spread = rng.uniform(0, 2e-3, n).astype(np.float32)
    spread[::1000] = np.nan
    f = surrogate.audit_flags_host(spread, seed=4, fraction=0.02, threshold=1e-3)
    assert np.array_equal((f & 2) != 0, ~(spread <= 1e-3))
    frac = np.mean(f & 1)
    assert abs(frac - 0.02) < 5 * np.sqrt(0.02 * 0.98 / n)
    g = surrogate.audit_flags_host(spread, seed=4, fraction=0.02, threshold=1e-3)
    assert np.array_equal(f, g)
    h = surrogate.audit_flags_host(spread, seed=5, fraction=0.02, threshold=1e-3)
    assert not np.array_equal(f & 1, h & 1)


def test_fourier_scale_selection(small):
    omega, s1, ah = surrogate.training_set(small, n=8192, seed=31)
    x7 = surrogate.inputs(omega, s1, small.xray, small.omega_axis, small.F)
    best, scores = surrogate.select_fourier_scale(x7, np.log(ah), candidates=(0.35, 0.5), steps=300,
                                                  batch=1024, members=2, seed=5)
    assert best in (0.35, 0.5) and set(scores) == {0.35, 0.5}
    for fb, med in scores.values():
        assert 0.0 <= fb <= 1.0 and np.isfinite(med) and med < 0.5
    assert scores[best] == min(scores.values())
    with pytest.raises(ValueError):
        surrogate.select_fourier_scale(x7[:1], np.log(ah[:1]))
