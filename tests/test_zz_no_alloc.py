"""The allocation-free field solve (ap_field_solve_noalloc) through the C ABI.

Callers of ap_field_solve_noalloc cannot allocate device memory themselves
(a host framework that owns every device buffer, a fixed memory budget).
Here the test plays that framework: torch allocates the buffers.  Each grid
size runs two calls in a row -- the second reuses the scratch the first one
left behind -- and each result is checked against the handle-based FP32 solve
(ap_field_solve) and against the FP64 oracle, within the field tolerance of
the other tests: max|dE| <= 1e-4 * max|E|.  A rectangular die (bin height /
bin width = 1.5) checks the y-frequency scaling.  Misaligned or oversized
arguments are rejected before anything is launched.  This file is collected
last.
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


def _setup():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300 as ap
    import oracle

    oracle.build(with_ref=False)
    return torch, ap, oracle


def _noalloc(torch, d, m, ratio, stream):
    from aieplace_gb300._lib import lib

    dd = torch.from_numpy(d.reshape(-1)).cuda()
    ex = torch.full((m * m,), float("nan"), device="cuda")
    ey = torch.full((m * m,), float("nan"), device="cuda")
    st = lib().ap_field_solve_noalloc(C.c_void_p(dd.data_ptr()), C.c_void_p(ex.data_ptr()),
                                      C.c_void_p(ey.data_ptr()), m, C.c_float(ratio), C.c_void_p(stream))
    assert st == 0
    torch.cuda.synchronize()
    return ex.cpu().numpy(), ey.cpu().numpy()


def _close(got, ref):
    assert np.isfinite(got).all()
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


@pytest.mark.parametrize("die_h_over_w", [1.0, 1.5])
def test_noalloc_field_matches_handle_solve_and_oracle(die_h_over_w):
    torch, ap, oracle = _setup()
    nl = dict(ap.synth.generate("c0", seed=1))
    W = float(nl["die"][2])
    nl["die"] = np.array([0.0, 0.0, W, W * die_h_over_w], np.float32)
    stream = torch.cuda.current_stream().cuda_stream
    for m in (128, 256, 64):
        # bin height / bin width, in the float arithmetic of ap_create
        bw = np.float32(nl["die"][2]) / np.float32(m)
        bh = np.float32(nl["die"][3]) / np.float32(m)
        ratio = float(np.float32(bh / bw))
        for call in range(2):
            d = _density(m, seed=10 * m + call)
            with ap.Placer(nl, bins=m) as pl:
                rex, rey = pl.compute_electric_fields(d, "fp32")
            oex, oey = oracle.field_solve(d.astype(np.float64), m, bin_ratio=ratio)
            gx, gy = _noalloc(torch, d, m, ratio, stream)
            for got, ref, orc in ((gx, rex, oex), (gy, rey, oey)):
                _close(got, ref)
                _close(got, orc)


def test_noalloc_rejects_bad_arguments():
    torch, _, _ = _setup()
    from aieplace_gb300._lib import lib

    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    buf = torch.zeros(64 * 64 + 8, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    # sizes beyond the static scratch, or not a multiple of 32
    assert lib().ap_field_solve_noalloc(p, p, p, 512, C.c_float(1.0), stream) == 1
    assert lib().ap_field_solve_noalloc(p, p, p, 48, C.c_float(1.0), stream) == 1
    # a density that does not start on a 16-byte boundary (one float in)
    off = C.c_void_p(buf.data_ptr() + 4)
    assert lib().ap_field_solve_noalloc(off, p, p, 64, C.c_float(1.0), stream) == 1
    # outputs off float alignment, and a non-positive bin ratio
    odd = C.c_void_p(buf.data_ptr() + 2)
    assert lib().ap_field_solve_noalloc(p, odd, p, 64, C.c_float(1.0), stream) == 1
    assert lib().ap_field_solve_noalloc(p, p, p, 64, C.c_float(0.0), stream) == 1
    torch.cuda.synchronize()
