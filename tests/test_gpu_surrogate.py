"""The learned field surrogate on the GPU, through the C ABI.

Tolerances (stated per check):
  forward         max|y_gpu - y_oracle| <= 1e-4 max|y|  (FP32 kernels vs FP64 oracle)
  loss            1e-5 relative
  gradient        max|g_gpu - g_oracle| <= 1e-3 max|g| and cosine >= 0.99999 (FP32 sums
                  of 2048 products per weight vs FP64), run to run bit-identical
  trained net     mean field error below the coarse spectral layer's alone on
                  held-out samples (the gain the net brings)
  loop            reaches overflow < 0.10 with the surrogate attached; final
                  HPWL within 2% of the exact-field loop's
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ap():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300

    return aieplace_gb300


def random_params(s, rng, scale=0.15):
    return (scale * rng.standard_normal(s.num_params)).astype(np.float32)


@pytest.mark.parametrize("kernels", [(3, 1, 1, 3), (1, 3, 3, 1), (3, 1, 1, 1), (1, 1, 1, 1)])
def test_forward_and_gradient_match_oracle(ap, oracle_lib, kernels):
    rng = np.random.default_rng(7)
    f, R, B, margin = 2, 32, 2, 2
    with ap.Surrogate(factor=f, kernels=kernels, width=32) as s:
        p = random_params(s, rng)
        s.set_params(p)
        x = rng.standard_normal((B, s.cin, R, R)).astype(np.float32)
        t = rng.standard_normal((B, s.cout, R, R)).astype(np.float32)
        y = s.forward(x)
        yr = oracle_lib.surr_forward(x, p.astype(np.float64), 32, s.cout, kernels)
        assert np.abs(y - yr).max() <= 1e-4 * np.abs(yr).max()
        loss, g = s.gradient(x, t, margin)
        loss2, g2 = s.gradient(x, t, margin)
        np.testing.assert_array_equal(g, g2)  # deterministic reductions
        assert loss == loss2
        lr, gr = oracle_lib.surr_loss_grad(x, t, p.astype(np.float64), 32, kernels, margin)
        assert abs(loss - lr) <= 1e-5 * lr
        assert np.abs(g - gr).max() <= 1e-3 * np.abs(gr).max()
        assert float(g @ gr) / (np.linalg.norm(g) * np.linalg.norm(gr)) >= 0.99999


@pytest.mark.parametrize("kernels,width,f,R", [((3, 1, 1, 1), 32, 4, 64), ((3, 1, 1, 1), 16, 2, 48),
                                                ((1, 1, 1, 1), 24, 1, 32)])
def test_fused_forward_matches_layer_by_layer(ap, kernels, width, f, R):
    """Inference runs (K0, 1, 1, 1) nets as one fused launch; training runs the
    layers one by one (it keeps the hidden maps).  Same arithmetic in the same
    order: with the fused output as the training target, the training
    forward's loss is exactly zero."""
    rng = np.random.default_rng(R)
    with ap.Surrogate(factor=f, kernels=kernels, width=width) as s:
        s.set_params(random_params(s, rng))
        x = rng.standard_normal((2, s.cin, R, R)).astype(np.float32)
        y = s.forward(x)
        loss, _ = s.gradient(x, y, 0)
        assert loss == 0.0


def collect_run(ap, s, n, every, seed):
    """n samples from the exact loop of a 20k-cell netlist on 128^2 bins (coarse 64^2)."""
    nl = ap.synth.generate("c1_small", seed=seed)
    with ap.Placer(nl, bins=128, target_density=0.7) as pl:
        pl.initialize_placement(seed=seed, sigma=1.0)
        assert s.collect(pl, n * every, every) == n


def collected(ap, n_samples=48, every=2, seed=3, held_out=0):
    """n_samples training samples from one seeded run, then `held_out` samples
    spread over the same trials of a run with another seed."""
    s = ap.Surrogate(factor=2)
    s.reserve(n_samples + held_out, 64)
    collect_run(ap, s, n_samples, every, seed)
    if held_out:
        collect_run(ap, s, held_out, n_samples * every // held_out, seed + 100)
    assert s.num_samples == n_samples + held_out
    return s


def test_untrained_net_adds_nothing(ap):
    s = collected(ap, n_samples=8, every=4)
    en, ec = s.validate()
    # the output layer starts at zero: the net's field is the coarse layer's
    np.testing.assert_allclose(en, ec, rtol=1e-6)
    assert np.all(ec > 0) and np.all(ec < 1.5)
    s.close()


def test_training_reduces_field_error_on_held_out_samples(ap):
    train_n = 48
    s = collected(ap, n_samples=train_n, every=2, seed=3, held_out=12)
    losses = s.train(steps=400, batch=8, crop=32, lr=2e-3, seed=11, first=0, count=train_n)
    assert np.all(np.isfinite(losses))
    assert losses[-50:].mean() < 0.7 * losses[:20].mean()
    en, ec = s.validate(first=train_n, count=s.num_samples - train_n)
    # what the trained network gains over the coarse spectral layer alone
    assert en.mean() < 0.9 * ec.mean(), (en, ec)
    s.close()


def test_loop_with_surrogate_reaches_target(ap):
    s = collected(ap, n_samples=64, every=2, seed=3)
    s.train(steps=300, batch=8, crop=32, lr=2e-3, seed=5)
    nl = ap.synth.generate("c1_small", seed=9)
    runs = {}
    for name, attach in (("exact", False), ("surrogate", True)):
        with ap.Placer(nl, bins=128, target_density=0.7, max_iterations=3000, check_interval=16) as pl:
            pl.initialize_placement(seed=9, sigma=1.0)
            if attach:
                pl.attach_surrogate(s, overflow_min=0.3, judge_every=8, max_error=0.05)
            pl.run()
            st = pl.stats()
            runs[name] = (st, pl.surrogate_stats() if attach else None)
    st, ss = runs["surrogate"]
    assert st["overflow"] < 0.10 and st["status"] == 0
    assert ss["judged"] > 0 and ss["used"] > 0
    ref = runs["exact"][0]
    assert abs(st["hpwl"] - ref["hpwl"]) <= 0.02 * ref["hpwl"], (st, ref)
    s.close()
