"""The batched form (ap_create_batch): instances stepped as parallel branches
of one CUDA graph give, bit for bit, what each gives when stepped alone."""
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


def small_batch(ap, n=3):
    specs = ap.synth.batch_specs(n, seed=4, lo=3000, hi=12000)
    return [ap.synth.generate(s, seed=20 + i) for i, s in enumerate(specs)]


def test_batch_matches_single_instances(ap):
    nls = small_batch(ap)
    with ap.BatchPlacer(nls) as b:
        b.initialize_placement(seed=100, sigma=1.0)
        b.step(30)
        batch = [b.positions(i) for i in range(len(nls))]
        bstats = [b.stats(i) for i in range(len(nls))]
    for i, nl in enumerate(nls):
        with ap.Placer(nl) as pl:
            pl.initialize_placement(seed=100 + i, sigma=1.0)
            pl.step_async(30)
            x, y = pl.positions()
            s = pl.stats()
        np.testing.assert_array_equal(batch[i][0], x)
        np.testing.assert_array_equal(batch[i][1], y)
        assert bstats[i]["iteration"] == s["iteration"] and bstats[i]["hpwl"] == s["hpwl"]


def test_batch_run_reaches_targets(ap):
    nls = small_batch(ap, n=4)
    with ap.BatchPlacer(nls, max_iterations=3000, check_interval=16) as b:
        b.initialize_placement(seed=7, sigma=1.0)
        its = b.run()
        stats = [b.stats(i) for i in range(len(nls))]
    for s, it in zip(stats, its):
        assert s["overflow"] < 0.10 or it >= 3000
        assert s["status"] == 0
    assert sum(s["overflow"] < 0.10 for s in stats) >= 3
