"""The persistent tensor-core field solve (one launch over the four
contraction stages, row-block dependency counters between them) pinned with
AP_TC_VARIANT, whichever candidate the autotuner would pick:

  parity       against the FP64 oracle, max|dE| <= 1e-4 max|E| (the bound of
               every field test), 128^2 .. 1024^2 bins
  agreement    with the four-launch solve of the same map within 5e-5 of
               max|E|: both sum the same products over K, in one accumulator or
               in split-K partials, and each stage's FP32 result is split into
               BF16 hi/lo again, so each differs from the oracle by ~1e-5 of max
               in its own way (measured 4e-6 .. 1e-5 apart)
  repeatable   repeated solves bit for bit (the counters are reset by the last
               CTA of each launch; a stale count would let a tile read a row
               block before it is written)
  timeout      the load issuer told to issue nothing (ap_debug_inject): the
               bounded waits run out, every CTA leaves, the call reports
               AP_ERR_TIMEOUT, and without the injection the handle solves again
               bit for bit
  loop         the 20k-cell loop on the pinned solver reaches overflow < 0.10
               with HPWL within 1% of the FP32 loop
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

AP_ERR_TIMEOUT = 7
PERSISTENT = (3, 4)


@pytest.fixture(scope="module")
def ap():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300

    return aieplace_gb300


def density_like(m, rng):
    d = (0.8 + 0.1 * rng.standard_normal((m, m))).astype(np.float32)
    d[m // 3: m // 2, m // 4: m // 2] += 2.5
    d[m // 8: m // 5, m // 8: m // 5] = 0.0
    return d


def pinned(ap, monkeypatch, variant, nl, **kw):
    """A Placer whose tensor-core solve is candidate `variant` (read at create)."""
    monkeypatch.setenv("AP_TC_VARIANT", str(variant))
    pl = ap.Placer(nl, **kw)
    monkeypatch.delenv("AP_TC_VARIANT")
    info = pl.solver_info()
    assert info["tc_variant"] == variant, info
    assert info["tc_ms"][variant] > 0.0, info
    return pl


@pytest.mark.parametrize("variant", PERSISTENT)
@pytest.mark.parametrize("m", [128, 256, 512, 1024])
def test_persistent_field_against_oracle(ap, oracle_lib, monkeypatch, variant, m):
    rng = np.random.default_rng(500 + m)
    d = density_like(m, rng)
    nl = ap.synth.generate("c0", seed=1)
    with pinned(ap, monkeypatch, variant, nl, bins=m) as pl:
        ex, ey = pl.compute_electric_fields(d, "bf16x3")
        for _ in range(4):
            ex2, ey2 = pl.compute_electric_fields(d, "bf16x3")
            np.testing.assert_array_equal(ex, ex2)
            np.testing.assert_array_equal(ey, ey2)
    with pinned(ap, monkeypatch, 0, nl, bins=m) as pl:
        fx, fy = pl.compute_electric_fields(d, "bf16x3")
    solve = oracle_lib.field_solve_fft if m >= 512 else oracle_lib.field_solve
    rex, rey = solve(d.astype(np.float64), m)
    for got, four, ref in ((ex, fx, rex), (ey, fy, rey)):
        ref = ref.reshape(got.shape)
        scale = np.abs(ref).max()
        err = np.abs(got - ref).max()
        print(f"variant {variant} m {m}: max|dE| {err / scale:.2e} of max, vs four-launch "
              f"{np.abs(got - four).max() / scale:.2e}")
        assert err <= 1e-4 * scale
        assert np.abs(got - four).max() <= 5e-5 * scale


@pytest.mark.parametrize("variant", PERSISTENT)
@pytest.mark.parametrize("m", [128, 512])
def test_persistent_wait_runs_out_and_reports_timeout(ap, monkeypatch, variant, m):
    from aieplace_gb300 import APError
    from aieplace_gb300._lib import check, lib

    def inject(pl, kind, wait_ns=0):
        check("ap_debug_inject", lib().ap_debug_inject(pl._h, kind, wait_ns))

    rng = np.random.default_rng(9)
    d = density_like(m, rng)
    nl = ap.synth.generate("c1_small", seed=1)
    with pinned(ap, monkeypatch, variant, nl, bins=m, field_solver="bf16x3") as pl:
        pl.initialize_placement(seed=2, sigma=1.0)
        ex0, ey0 = pl.compute_electric_fields(d, "bf16x3")
        inject(pl, 1, 10_000_000)  # AP_FAULT_TC_STALL, 10 ms per wait
        with pytest.raises(APError) as e:
            pl.compute_electric_fields(d, "bf16x3")
        assert e.value.status == AP_ERR_TIMEOUT
        inject(pl, 0)
        inject(pl, 1, 10_000_000)
        with pytest.raises(APError) as e:
            pl.perform_iteration(1)  # the loop's captured trial
        assert e.value.status == AP_ERR_TIMEOUT
        inject(pl, 0)
        ex1, ey1 = pl.compute_electric_fields(d, "bf16x3")
        np.testing.assert_array_equal(ex0, ex1)
        np.testing.assert_array_equal(ey0, ey1)


@pytest.mark.parametrize("variant", PERSISTENT)
def test_persistent_loop_matches_fp32_loop(ap, monkeypatch, variant):
    nl = ap.synth.generate("c1_small", seed=2)
    res = {}
    with ap.Placer(nl, bins=128, field_solver="fp32", max_iterations=3000) as pl:
        pl.initialize_placement(seed=3, sigma=1.0)
        pl.run()
        res["fp32"] = pl.stats()
    with pinned(ap, monkeypatch, variant, nl, bins=128, field_solver="bf16x3", max_iterations=3000) as pl:
        pl.initialize_placement(seed=3, sigma=1.0)
        pl.run()
        res["persistent"] = pl.stats()
    assert res["fp32"]["overflow"] < 0.10 and res["persistent"]["overflow"] < 0.10, res
    assert abs(res["persistent"]["hpwl"] - res["fp32"]["hpwl"]) <= 0.01 * res["fp32"]["hpwl"], res
