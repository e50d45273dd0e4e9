"""Error paths of the library on the GPU, provoked from the host.  Nothing
here faults, traps or hangs a GPU:

  timeout      the tensor-core solve's load issuer is told to issue nothing
               (ap_debug_inject), so the MMA issuer's bounded wait for data runs
               out after 10 ms; every CTA leaves through the abort path with no
               copy in flight, the call returns AP_ERR_TIMEOUT, and after the
               injection is removed the same handle solves again, bit-identical
               to before
  divergence   a host step whose input positions hold a NaN: the loop's step
               control sees a non-finite step length and reports
               AP_ERR_DIVERGED; a new initial placement clears it
  surrogate    weights corrupted from the host (NaN, or scaled by 1e3): every
               judgement falls back to the exact solve, the surrogate field is
               never used, and the loop reaches the same result bit for bit as
               the loop without a surrogate
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

AP_ERR_TIMEOUT = 7
AP_ERR_DIVERGED = 9


@pytest.fixture(scope="module")
def ap():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300

    return aieplace_gb300


def _inject(pl, kind, wait_ns=0):
    from aieplace_gb300._lib import check, lib

    check("ap_debug_inject", lib().ap_debug_inject(pl._h, kind, wait_ns))


def _density(m, seed):
    rng = np.random.default_rng(seed)
    d = (0.8 + 0.1 * rng.standard_normal((m, m))).astype(np.float32)
    d[m // 3: m // 2, m // 4: m // 2] += 2.5
    return d


@pytest.mark.parametrize("m", [128, 512])
def test_tensor_core_wait_runs_out_and_reports_timeout(ap, m):
    from aieplace_gb300 import APError

    nl = ap.synth.generate("c1_small", seed=1)
    d = _density(m, 3)
    with ap.Placer(nl, bins=m, field_solver="bf16x3") as pl:
        pl.initialize_placement(seed=2, sigma=1.0)
        ex0, ey0 = pl.compute_electric_fields(d, "bf16x3")
        _inject(pl, 1, 10_000_000)  # AP_FAULT_TC_STALL, 10 ms per wait
        with pytest.raises(APError) as e:
            pl.compute_electric_fields(d, "bf16x3")
        assert e.value.status == AP_ERR_TIMEOUT
        # the loop's trial (a captured graph) runs out the same way
        _inject(pl, 0)
        _inject(pl, 1, 10_000_000)
        with pytest.raises(APError) as e:
            pl.perform_iteration(1)
        assert e.value.status == AP_ERR_TIMEOUT
        _inject(pl, 0)  # AP_FAULT_NONE: the context and the handle are usable again
        ex1, ey1 = pl.compute_electric_fields(d, "bf16x3")
        np.testing.assert_array_equal(ex0, ex1)
        np.testing.assert_array_equal(ey0, ey1)
        fx, _ = pl.compute_electric_fields(d, "fp32")
        assert np.abs(ex1 - fx).max() <= 1e-4 * np.abs(fx).max()
    # and a fresh handle works
    with ap.Placer(nl, bins=m, field_solver="bf16x3") as pl:
        ex2, _ = pl.compute_electric_fields(d, "bf16x3")
        np.testing.assert_array_equal(ex0, ex2)


def test_nan_positions_report_divergence(ap):
    from aieplace_gb300 import APError

    nl = ap.synth.generate("c0", seed=1)
    with ap.Placer(nl, bins=32) as pl:
        pl.initialize_placement(nl["node_x"], nl["node_y"])
        pl.perform_iteration(5)
        x, y = pl.positions()
        xo, yo = np.zeros_like(x), np.zeros_like(y)
        x[3] = np.nan
        with pytest.raises(APError) as e:
            pl.step_host(x, y, xo, yo)
        assert e.value.status == AP_ERR_DIVERGED
        assert pl.stats()["status"] == AP_ERR_DIVERGED
        with pytest.raises(APError) as e:
            pl.perform_iteration(1)  # the status stays until the optimiser is reset
        assert e.value.status == AP_ERR_DIVERGED
        pl.initialize_placement(nl["node_x"], nl["node_y"])
        pl.perform_iteration(5)
        s = pl.stats()
        assert s["status"] == 0 and s["iteration"] == 5 and np.isfinite(s["hpwl"])


@pytest.mark.parametrize("corruption", ["nan", "scaled"])
def test_corrupted_surrogate_falls_back_to_exact(ap, corruption):
    nl = ap.synth.generate("c1_small", seed=9)
    runs = {}
    for name in ("exact", "corrupted"):
        with ap.Placer(nl, bins=128, target_density=0.7, max_iterations=3000, check_interval=16) as pl:
            pl.initialize_placement(seed=9, sigma=1.0)
            s = None
            if name == "corrupted":
                s = ap.Surrogate(factor=2, kernels=(3, 1, 1, 1))
                p = np.random.default_rng(1).standard_normal(s.num_params).astype(np.float32)
                if corruption == "nan":
                    p[::7] = np.nan
                else:
                    p *= 1e3
                s.set_params(p)
                pl.attach_surrogate(s, overflow_min=0.3, judge_every=4, max_error=0.05)
            it = pl.run()
            runs[name] = (it, pl.stats(), pl.positions(), pl.surrogate_stats() if s else None)
            if s:
                s.close()
    it_e, st_e, (xe, ye), _ = runs["exact"]
    it_c, st_c, (xc, yc), ss = runs["corrupted"]
    assert ss["judged"] > 0 and ss["fallbacks"] == ss["judged"] and ss["used"] == 0, ss
    assert st_c["status"] == 0 and st_c["overflow"] < 0.10
    assert it_c == it_e and st_c["hpwl"] == st_e["hpwl"]
    np.testing.assert_array_equal(xc, xe)
    np.testing.assert_array_equal(yc, ye)
