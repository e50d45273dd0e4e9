"""The allocation-free field solve (ap_field_solve_noalloc) against the
handle-based solve (ap_field_solve, FP32), through the C ABI.

Callers of ap_field_solve_noalloc cannot allocate device memory themselves;
here the test plays the host framework that owns the device buffers (torch
allocates them) and checks two calls in a row per grid size -- the second call
reuses the scratch the first one left behind -- within the field tolerance of
the other tests: max|dE| <= 1e-4 * max|E|.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _density(m, seed):
    rng = np.random.default_rng(seed)
    d = (0.8 + 0.1 * rng.standard_normal((m, m))).astype(np.float32)
    d[m // 3: m // 2, m // 4: m // 2] += 2.5
    return d


def test_noalloc_field_matches_handle_solve():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300 as ap
    from aieplace_gb300._lib import lib

    nl = ap.synth.generate("c0", seed=1)
    stream = torch.cuda.current_stream().cuda_stream
    for m in (128, 256, 64):
        for call in range(2):
            d = _density(m, seed=10 * m + call)
            with ap.Placer(nl, bins=m) as pl:
                rex, rey = pl.compute_electric_fields(d, "fp32")
            dd = torch.from_numpy(d.reshape(-1)).cuda()
            ex = torch.full((m * m,), float("nan"), device="cuda")
            ey = torch.full((m * m,), float("nan"), device="cuda")
            st = lib().ap_field_solve_noalloc(C.c_void_p(dd.data_ptr()), C.c_void_p(ex.data_ptr()),
                                              C.c_void_p(ey.data_ptr()), m, 1.0, C.c_void_p(stream))
            assert st == 0
            torch.cuda.synchronize()
            gx, gy = ex.cpu().numpy(), ey.cpu().numpy()
            for got, ref in ((gx, rex), (gy, rey)):
                assert np.isfinite(got).all()
                assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()
    # sizes beyond the static scratch are rejected, nothing is launched
    dummy = torch.zeros(1, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    assert lib().ap_field_solve_noalloc(p, p, p, 512, 1.0, C.c_void_p(stream)) == 1
    assert lib().ap_field_solve_noalloc(p, p, p, 48, 1.0, C.c_void_p(stream)) == 1
