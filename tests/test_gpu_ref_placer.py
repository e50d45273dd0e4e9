"""The CUDA path against the reference's own Placer (vck5000/host/src/
AIEplace.cpp built for the CPU), through the fixture make_golden.py wrote
from it (tests/golden/ref_placer.npz) on inputs rebuilt here bit for bit
(tests/golden/ref_placer_inputs.py).  Per case (576 cells / 32^2 bins, 20k
cells / 128^2 bins; nets of degree 2..8):

  WA partials   computeAllPartials_CPU: per node, the reference's own float
                rounding (ref_placer_inputs.partials_rounding) plus the CUDA
                kernel's 1e-4 of max |g|
  density map   computeOverlaps / getRho: the same bins touched, areas within
                2e-5 of the largest (the reference accumulates in float)
  overflow      computeTotalOverflow: 2e-5 relative
  node force    nudgeNode's force on given fields: 1e-4 of the largest
  HPWL          computeTotalWirelength("HPWL"): 1e-6 relative
  field         the host DCT path (compute_a_uv_DCT / compute_eField_DCT),
                the FP32 solver at both sizes and the tensor-core BF16x3 one
                at 128^2, on the CUDA density map: 1e-4 of the largest, after
                the M^2 / 8 of the reference's unnormalised transforms
"""
import numpy as np
import pytest

from conftest import golden

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


@pytest.mark.parametrize("name", ["c0", "c1_small"])
def test_cuda_path_matches_reference_placer(ap, name):
    import ref_placer_inputs as I

    g = golden("ref_placer.npz")
    nl = I.small_nets(ap.synth.generate(name, seed=I.SEED))
    assert int(g[f"{name}_n_nets"]) == len(nl["net_ptr"]) - 1
    x, y = I.positions(nl)
    W, H, M = float(nl["die"][2]), float(nl["die"][3]), int(g[f"{name}_rho"].shape[0])
    sub = slice(0, None, I.SUBSAMPLE)
    ex, ey = I.field(M)
    fields = {}
    with ap.Placer(nl, bins=M) as pl:
        gx, gy, _, hp = pl.compute_all_partials(x, y, I.GAMMA)
        q = pl.compute_overlaps(x, y)
        fx, fy = pl.compute_node_forces(x, y, ex, ey)
        if f"{name}_dct_ex" in g:
            area = (q / 2.0 ** 32).astype(np.float32)
            for solver in ("fp32", "bf16x3") if M % 128 == 0 else ("fp32",):  # tcgen05 tiles: 128
                fields[solver] = pl.compute_electric_fields(area, solver)
    # WA partials
    rx, ry = g[f"{name}_gx"], g[f"{name}_gy"]
    tol = I.partials_rounding(nl)[sub] + 1e-4 * max(np.abs(rx).max(), np.abs(ry).max())
    assert np.all(np.abs(gx[sub] - rx) <= tol)
    assert np.all(np.abs(gy[sub] - ry) <= tol)
    # HPWL
    ref_hp = float(g[f"{name}_hpwl"])
    assert abs(hp - ref_hp) <= 1e-6 * ref_hp
    # density map and overflow
    rho, ref = (q / 2.0 ** 32).reshape(M, M), g[f"{name}_rho"]
    assert np.array_equal(rho != 0, ref != 0)
    assert np.abs(rho - ref).max() <= 2e-5 * max(1.0, np.abs(ref).max())
    ovf = float(np.maximum(rho - (W / M) * (H / M), 0.0).sum())
    ref_ovf = float(g[f"{name}_overflow"])
    assert abs(ovf - ref_ovf) <= 2e-5 * max(1.0, ref_ovf)
    # nudgeNode's force (movable nodes)
    mov = (nl["node_fixed"] == 0)[sub]
    rfx, rfy = g[f"{name}_fx"], g[f"{name}_fy"]
    scale = max(np.abs(rfx[mov]).max(), np.abs(rfy[mov]).max())
    assert np.abs(fx[sub][mov] - rfx[mov]).max() <= 1e-4 * scale
    assert np.abs(fy[sub][mov] - rfy[mov]).max() <= 1e-4 * scale
    # the field (reference: host DCT path, x M^2 / 8)
    for solver, (cex, cey) in fields.items():
        for ref_e, e in ((g[f"{name}_dct_ex"], cex), (g[f"{name}_dct_ey"], cey)):
            k = M * M / 8.0 * e.reshape(M, M).astype(np.float64)
            assert np.abs(ref_e - k).max() <= 1e-4 * np.abs(ref_e).max(), solver
