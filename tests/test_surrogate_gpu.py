"""Learned morphogen surrogate on the GPU: gradients and tensor-memory inference against the
float64 CPU reference of the network (oracle/mlp_ref.py), training-pair capture, training and
the judged surrogate step.

Tolerances: the GPU and the CPU reference round activations and gradients to bf16 at the same
points; the remaining differences are float32-vs-float64 accumulation and erf ulps, which can
move a bf16 rounding by one unit (2^-8 relative).  Gradients: rtol 3e-2 per element plus an
absolute floor of 1e-3 x the block's largest gradient, cosine similarity > 0.999 per block.
Inference: rtol 2e-2 plus 2e-3 x the largest output.
"""
import numpy as np
import pytest

import mlp_ref
import morphogenesis_gb300 as mg
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo
from morphogenesis_gb300 import surrogate as S

pytestmark = pytest.mark.gpu

BLOCKS = {"W1": (A.P_W1, A.P_B1), "b1": (A.P_B1, A.P_W2), "W2": (A.P_W2, A.P_B2),
          "b2": (A.P_B2, A.P_W3), "W3": (A.P_W3, A.P_B3), "b3": (A.P_B3, A.P_COUNT)}


def random_batch(n, seed):
    r = np.random.default_rng(seed)
    x = np.concatenate([r.random((n, 16)), r.random((n, 16)), (r.random((n, 16)) < 0.5)], 1)
    y = r.normal(0, 0.01, (n, 16))
    return x.astype(np.float32), y.astype(np.float32)


def random_norm(seed):
    r = np.random.default_rng(seed)
    return np.concatenate([r.uniform(0.3, 0.7, 48), r.uniform(1.5, 4.0, 48),
                           r.normal(0, 0.003, 16), r.uniform(50, 200, 16)]).astype(np.float32)


@pytest.fixture(scope="module")
def net(built):
    m = S.Mlp(seed=3)
    m.set_norm(random_norm(4))
    p = m.params()
    p[A.P_B1:A.P_W2] = np.random.default_rng(5).normal(0, 0.1, A.MLP_H)
    p[A.P_B2:A.P_W3] = np.random.default_rng(6).normal(0, 0.1, A.MLP_H)
    m.set_params(p)
    return m


@pytest.mark.parametrize("n", [512, 3000])
def test_gradients_match_cpu_reference(net, n):
    # 3000 rows: a ragged last 128-row tile and five split-K ranges in the weight gradients
    x, y = random_batch(n, 7)
    g, loss = net.gradients(x, y)
    gr, lr = mlp_ref.grads(net.params(), net.norm(), x, y)
    assert abs(loss - lr) <= 1e-4 * abs(lr) + 1e-9
    for name, (a, b) in BLOCKS.items():
        ga, gb = g[a:b].astype(np.float64), gr[a:b]
        scale = np.abs(gb).max()
        assert np.allclose(ga, gb, rtol=3e-2, atol=1e-3 * scale), f"{name}: max |d| {np.abs(ga - gb).max()} of {scale}"
        cos = ga @ gb / (np.linalg.norm(ga) * np.linalg.norm(gb) + 1e-30)
        assert cos > 0.999, f"{name}: cosine {cos}"


def test_tensor_memory_inference_matches_cpu_reference(net):
    x, _ = random_batch(1000, 8)  # not a multiple of the 128-row tile
    y = net.infer(x)
    yr = mlp_ref.infer(net.params(), net.norm(), x)
    scale = np.abs(yr).max()
    assert np.allclose(y, yr, rtol=2e-2, atol=2e-3 * scale), f"max |d| {np.abs(y - yr).max()} of {scale}"


def test_capture_pairs_are_the_plain_step(built):
    d = demo.make_block(12, "R", seed=2)
    fs = mg.FluidSystem(d.params, d.genome, d.n)
    fs.TransferToCL(d.arrays)
    ref = mg.FluidSystem(d.params, d.genome, d.n)
    ref.TransferToCL(d.arrays)
    for f in (fs, ref):
        f.Run(1, 0)  # sort only: the capture step below keeps this order
    pre = fs.download(A.FCONC).astype(np.float64)
    ds = S.Dataset(4 * d.n)
    ds.capture(fs, 0)  # morphogen stage only: positions stay those of the capture
    ref.Run(1, A.STEP_GENES)
    assert len(ds) == d.n
    for b in (A.FPOS, A.FCONC, A.FPARTICLE_ID):
        assert np.array_equal(fs.download(b), ref.download(b)), f"capture step differs from a plain step: {b}"
    x, y = ds.read(0, d.n)
    conc = fs.download(A.FCONC)
    # x[:, :16] is the concentration after diffusion and decay and y the gene reaction's
    # increment, both divided by the particle's scale s = max_t |diffused concentration|
    ref2 = mg.FluidSystem(d.params, d.genome, d.n)
    ref2.TransferToCL(d.arrays)
    ref2.Run(1, 0)
    ref2.ComputeDiffusionCL()
    cd = ref2.download(A.FCONC)
    sc = np.abs(cd).max(1, keepdims=True)
    np.testing.assert_allclose(x[:, :16], cd / sc, rtol=2e-7, atol=0)
    np.testing.assert_allclose(cd + sc * y, conc, rtol=1e-6, atol=1e-7)
    bits = (fs.download(A.FEPIGEN) != 0).T.astype(np.float32)
    assert np.array_equal(x[:, 32:48], bits)
    # neighbour means over the diffusion radius (dsq < (sr/ss)^2), sorted order of that step
    pos = fs.download(A.FPOS)[:, :3]
    r2 = np.float32(np.float32(d.params.psmoothradius) ** 2) / np.float32(np.float32(d.params.psimscale) ** 2)
    for p in range(0, d.n, 37):
        dv = pos[p] - pos
        dsq = (dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1]) + dv[:, 2] * dv[:, 2]
        nb = (dsq < r2) & (dsq > 0)
        want = pre[nb].mean(0) if nb.any() else pre[p]
        np.testing.assert_allclose(x[p, 16:32] * sc[p], want, rtol=1e-5, atol=1e-6)


def _train_small(seed=0):
    ds = S.Dataset(1 << 20)
    for s in range(2):
        d = demo.make_block(24, "R", seed=s)
        fs = mg.FluidSystem(d.params, d.genome, d.n)
        fs.TransferToCL(d.arrays)
        for k in range(8):
            ds.capture(fs, A.STEP_PHYSICS)
            fs.Run(5)
        fs.close()
    m = S.Mlp(seed=seed)
    m.fit_normalization(ds)
    curve = m.train(ds, 400, batch=8192, lr=1e-3, seed=1)
    return m, ds, curve


def test_training_and_judged_surrogate_step(built):
    m, ds, curve = _train_small()
    assert curve[-20:].mean() < 0.1 * curve[:5].mean(), f"loss {curve[:5].mean()} -> {curve[-20:].mean()}"
    # one morphogen stage: surrogate vs plain from the same state
    d = demo.make_block(24, "R", seed=7)
    plain = mg.FluidSystem(d.params, d.genome, d.n)
    sur = mg.FluidSystem(d.params, d.genome, d.n)
    for fs in (plain, sur):
        fs.TransferToCL(d.arrays)
        fs.Run(3)
    S.attach(sur, m, judge_period=1, judge_stride=8, threshold=1e-2)
    c0 = plain.download(A.FCONC)
    plain.Run(1, A.STEP_GENES)
    sur.Run(1, A.STEP_GENES | A.STEP_SURROGATE)
    cp, cs = plain.download(A.FCONC), sur.download(A.FCONC)
    # per particle: largest deviation over the largest plain concentration
    rel = np.abs(cs - cp).max(1) / np.maximum(np.abs(cp).max(1), 1e-30)
    judged, handed, worst = S.stats(sur)
    assert judged == d.n // 8 or judged == (d.n + 7) // 8
    assert handed <= judged
    # particles handed over carry the plain result exactly; the others are within the
    # configuration's 1e-3 (the same network measured 2.7e-4 median on this scene)
    assert np.median(rel) < 1e-3, f"median relative error {np.median(rel)}"
    assert np.isfinite(cs).all()
    _ = c0


def test_handover_takes_the_plain_result(built):
    m = S.Mlp(seed=11)  # untrained: every judged particle is handed over with threshold 0
    d = demo.make_block(10, "R", seed=3)
    plain = mg.FluidSystem(d.params, d.genome, d.n)
    sur = mg.FluidSystem(d.params, d.genome, d.n)
    for fs in (plain, sur):
        fs.TransferToCL(d.arrays)
    S.attach(sur, m, judge_period=1, judge_stride=1, threshold=0.0)
    plain.Run(2)
    sur.Run(2, A.STEP_DEFAULT | A.STEP_SURROGATE)
    judged, handed, _ = S.stats(sur)
    assert judged == d.n and handed == d.n
    assert np.array_equal(plain.download(A.FCONC), sur.download(A.FCONC))
    assert np.array_equal(plain.download(A.FPOS), sur.download(A.FPOS))


def _one_stage_error(m, d):
    """Per-particle relative error of one surrogate morphogen stage against the plain stage from
    the same state (largest deviation over the largest plain concentration)."""
    plain = mg.FluidSystem(d.params, d.genome, d.n)
    sur = mg.FluidSystem(d.params, d.genome, d.n)
    for fs in (plain, sur):
        fs.TransferToCL(d.arrays)
        fs.Run(3)
    S.attach(sur, m, judge_period=0, judge_stride=0, threshold=1e-3)
    plain.Run(1, A.STEP_GENES)
    sur.Run(1, A.STEP_GENES | A.STEP_SURROGATE)
    cp, cs = plain.download(A.FCONC).astype(np.float64), sur.download(A.FCONC).astype(np.float64)
    plain.close()
    sur.close()
    return np.abs(cs - cp).max(1) / np.maximum(np.abs(cp).max(1), 1e-30)


def test_what_the_trained_network_gains(built):
    """What the trained network gains over the method without it, on a 24^3 scene (13,824
    particles): its one-stage accuracy against the same network untrained (the gain of
    training; both with the normalisation fitted on the same pairs), and the morphogen stage's
    cost in both forms inside the full step (step time minus the physics-only step time).  The
    plain stage here is the density pass's fused diffusion + reaction epilogue, and the network
    stands in for the reaction only, so the surrogate form costs more than the plain one: the
    test records the measured ratio and asserts what holds."""
    m, ds, _ = _train_small()
    m0 = S.Mlp(seed=5)
    m0.fit_normalization(ds)
    d = demo.make_block(24, "R", seed=7)
    e_trained, e_untrained = _one_stage_error(m, d), _one_stage_error(m0, d)
    K = 50
    plain = mg.FluidSystem(d.params, d.genome, d.n)
    sur = mg.FluidSystem(d.params, d.genome, d.n)
    for fs in (plain, sur):
        fs.TransferToCL(d.arrays)
        fs.Run(3)
    S.attach(sur, m, judge_period=10, judge_stride=64, threshold=1e-3)
    t_phys = plain.time_steps(K, A.STEP_PHYSICS) / K
    t_plain = plain.time_steps(K, A.STEP_DEFAULT) / K
    t_sur = sur.time_steps(K, A.STEP_DEFAULT | A.STEP_SURROGATE) / K
    stage_plain, stage_sur = t_plain - t_phys, t_sur - t_phys
    print(f"one-stage error, trained: median {np.median(e_trained):.2e} max {e_trained.max():.2e}; "
          f"untrained: median {np.median(e_untrained):.2e}; stage ms plain {stage_plain:.4f} "
          f"surrogate {stage_sur:.4f} (speed ratio {stage_plain / max(stage_sur, 1e-9):.2f})")
    assert np.isfinite(e_trained).all() and np.isfinite(e_untrained).all()
    assert np.median(e_trained) <= 1e-3, f"trained median one-stage error {np.median(e_trained):.2e}"
    # measured on a GB300: trained 2.7e-4, untrained 1.9e-3 (an untrained network's increments
    # are near zero, so its error is about the reaction's own size relative to the
    # concentrations); stage 0.028 ms plain against 0.032 ms surrogate (0.88)
    assert np.median(e_untrained) >= 4 * np.median(e_trained), \
        f"training gained too little: {np.median(e_untrained):.2e} vs {np.median(e_trained):.2e}"
    assert t_phys > 0 and t_plain > 0 and t_sur > 0
    for x in (plain, sur, m, m0, ds):
        x.close()
