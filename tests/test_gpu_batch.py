"""The batched form (ap_create_batch).

Both forms -- nine persistent launches over all instances, and every
instance's own launches as parallel graph branches -- give, bit for bit,
what each instance gives when stepped alone with the same parameters (the single-instance loop is
itself checked against the FP64 oracle in test_gpu_parity*.py), with
instances of uneven size and grid, and with filler cells (two scatter records
per instance).  The persistent field launch's dependency waits are bounded:
an injected never-arriving dependency makes the step return AP_ERR_TIMEOUT
within about the limit, with no fault, and the batch works again after the
injection is removed and the instances are re-initialised.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

AP_ERR_TIMEOUT = 7
AP_FAULT_NONE = 0
AP_FAULT_NEVER_ARRIVE = 2


@pytest.fixture(scope="module")
def ap():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300

    return aieplace_gb300


def small_batch(ap, n=3, lo=3000, hi=12000, seed=4):
    specs = ap.synth.batch_specs(n, seed=seed, lo=lo, hi=hi)
    return [ap.synth.generate(s, seed=20 + i) for i, s in enumerate(specs)]


def singles(ap, nls, trials, seed, **kw):
    """Each instance alone, with the batch's grid policy (2048 nodes per block)."""
    out = []
    for i, nl in enumerate(nls):
        with ap.Placer(nl, block_nodes=2048, **kw) as pl:
            pl.initialize_placement(seed=seed + i, sigma=1.0)
            pl.step_async(trials)
            out.append((pl.positions(), pl.stats()))
    return out


@pytest.mark.parametrize("form", ["persistent", "graph"])
def test_batch_matches_single_instances(ap, form):
    nls = small_batch(ap)
    with ap.BatchPlacer(nls) as b:
        assert b.info()["form"] == "persistent"  # the default where it serves every instance
        b.set_form(form)
        b.initialize_placement(seed=100, sigma=1.0)
        b.step(30)
        batch = [(b.positions(i), b.stats(i)) for i in range(len(nls))]
        info = b.info()
    assert info["form"] == form
    for ((bx, by), bs), ((x, y), s) in zip(batch, singles(ap, nls, 30, 100)):
        np.testing.assert_array_equal(bx, x)
        np.testing.assert_array_equal(by, y)
        assert bs["iteration"] == s["iteration"] and bs["hpwl"] == s["hpwl"] and bs["overflow"] == s["overflow"]


def test_persistent_uneven_instances_with_fillers(ap):
    """Instances of 3.6k..124k cells on 128^2 and 256^2 grids, filler cells
    on: every stage's records, the field's 4 x n dependent contractions."""
    nls = small_batch(ap, n=6, lo=2000, hi=150000, seed=10)
    assert len({int(nl["bins"]) for nl in nls}) > 1
    with ap.BatchPlacer(nls, filler_cells=1) as b:
        b.initialize_placement(seed=40, sigma=1.0)
        b.step(25)
        batch = [(b.positions(i), b.stats(i)) for i in range(len(nls))]
        info = b.info()
    assert info["form"] == "persistent" and info["field_tile"] in (32, 64)
    r = info["records"]
    assert r["update"] == r["rho"] == r["wa"] == r["gather"] == 6
    assert r["scatter"] == 12 and r["field"] == 24
    for ((bx, by), bs), ((x, y), s) in zip(batch, singles(ap, nls, 25, 40, filler_cells=1)):
        np.testing.assert_array_equal(bx, x)
        np.testing.assert_array_equal(by, y)
        assert bs["hpwl"] == s["hpwl"] and bs["overflow"] == s["overflow"]


@pytest.mark.parametrize("item_blocks", [3, 64])
def test_persistent_items_of_several_blocks(ap, item_blocks):
    """Work items of several of a record's blocks (3; 64 -- more than most
    records have) give the same results; the stage profile times all six."""
    nls = small_batch(ap, n=4, lo=2000, hi=150000, seed=10)
    with ap.BatchPlacer(nls) as b:
        b.set_item_blocks(item_blocks)
        b.initialize_placement(seed=70, sigma=1.0)
        b.step(12)
        prof = b.profile(3)  # 3 more trial steps
        batch = [(b.positions(i), b.stats(i)) for i in range(len(nls))]
        info = b.info()
    assert all(v > 0 for v in prof.values()), prof
    assert info["item_blocks"]["update"] == item_blocks and info["item_blocks"]["field"] == 1
    for ((bx, by), bs), ((x, y), s) in zip(batch, singles(ap, nls, 15, 70)):
        np.testing.assert_array_equal(bx, x)
        np.testing.assert_array_equal(by, y)
        assert bs["hpwl"] == s["hpwl"]


def test_batch_run_reaches_targets(ap):
    nls = small_batch(ap, n=4)
    with ap.BatchPlacer(nls, max_iterations=3000, check_interval=16) as b:
        b.initialize_placement(seed=7, sigma=1.0)
        its = b.run()
        stats = [b.stats(i) for i in range(len(nls))]
        assert b.info()["active"] == 0
    for s, it in zip(stats, its):
        assert s["overflow"] < 0.10 or it >= 3000
        assert s["status"] == 0
    assert sum(s["overflow"] < 0.10 for s in stats) >= 3


def test_never_arriving_dependency_times_out(ap):
    from aieplace_gb300 import APError
    from aieplace_gb300._lib import check, lib

    nls = small_batch(ap, n=3)
    ref = singles(ap, nls, 10, 60)
    with ap.BatchPlacer(nls) as b:
        b.initialize_placement(seed=60, sigma=1.0)
        check("ap_batch_debug_inject", lib().ap_batch_debug_inject(b._h, AP_FAULT_NEVER_ARRIVE, 20_000_000))
        t0 = time.perf_counter()
        with pytest.raises(APError) as e:
            b.step(1)
        assert e.value.status == AP_ERR_TIMEOUT
        assert time.perf_counter() - t0 < 5.0  # one 20 ms limit, then every later wait gives up at once
        # removed: the context and the batch work again after a re-initialisation
        check("ap_batch_debug_inject", lib().ap_batch_debug_inject(b._h, AP_FAULT_NONE, 0))
        b.initialize_placement(seed=60, sigma=1.0)
        b.step(10)
        batch = [(b.positions(i), b.stats(i)) for i in range(len(nls))]
    for ((bx, by), bs), ((x, y), s) in zip(batch, ref):
        np.testing.assert_array_equal(bx, x)
        np.testing.assert_array_equal(by, y)


def test_injection_arguments(ap):
    from aieplace_gb300._lib import lib

    nls = small_batch(ap, n=2)
    with ap.BatchPlacer(nls) as b:
        assert lib().ap_batch_debug_inject(b._h, AP_FAULT_NEVER_ARRIVE, 10) == 1  # below 1 ms
        assert lib().ap_batch_debug_inject(b._h, 5, 0) == 1
        b.set_form("graph")
        assert lib().ap_batch_debug_inject(b._h, AP_FAULT_NEVER_ARRIVE, 10_000_000) == 6  # persistent only
