"""Parity at the sizes the loop is measured on (200k cells / 512^2 bins and
2M cells / 1024^2 bins), CUDA path against the FP64 oracle through the C ABI.

Tolerances, stated per result:
  field (both solvers)   max|dE| <= 1e-4 * max|E| against the dense FP64
                         solve; per element |dE_b| <= 1e-4 * max|E| is the
                         same bound, and the relative error of bins with
                         |E_b| >= 1e-2 max|E| is reported (-s) as quantiles
  WA gradient            per node |dg_i| <= pins_i * 2^-20 + 1e-4 * max|g|:
                         each pin's term is rounded to 2^-20 before the exact
                         int64 sum, so a node's error grows with its pin count
                         and a per-element relative bound cannot hold for
                         nodes whose terms cancel; quantiles reported
  overflow readout       bit-exact (exact int64 sums, one identical division)
  HPWL readout           1e-7 relative (per-net extents are FP32 differences)
  node force             per node |dF_i| <= 1e-5 * sum_b w_ib |E_b| (the
                         FP32 rounding bound of a sum of weighted terms)
  preconditioned grad    per node |dg_i| <= (pins_i 2^-20 + lambda |dF_i|
                         bound + 1e-6 (|dWA_i| + lambda |F_i|)) / H_i
                         + 1e-5 |g_i|
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_NL = {}


@pytest.fixture(scope="module")
def ap():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300

    return aieplace_gb300


def netlist(ap, preset):
    if preset not in _NL:
        _NL[preset] = ap.synth.generate(preset, seed=1)
    return _NL[preset]


def spread(nl, seed, margin=2.0):
    rng = np.random.default_rng(seed)
    W, H = float(nl["die"][2]), float(nl["die"][3])
    x, y = nl["node_x"].copy(), nl["node_y"].copy()
    mov = nl["node_fixed"] == 0
    x[mov] = rng.uniform(-margin, W + margin, mov.sum()).astype(np.float32)
    y[mov] = rng.uniform(-margin, H + margin, mov.sum()).astype(np.float32)
    return x, y


def clustered(nl, seed, sigma=30.0):
    rng = np.random.default_rng(seed)
    W, H = float(nl["die"][2]), float(nl["die"][3])
    x, y = nl["node_x"].copy(), nl["node_y"].copy()
    mov = nl["node_fixed"] == 0
    x[mov] = (W / 2 + sigma * rng.standard_normal(mov.sum())).astype(np.float32)
    y[mov] = (H / 2 + sigma * rng.standard_normal(mov.sum())).astype(np.float32)
    return x, y


def quantiles(rel):
    if rel.size == 0:
        return {}
    q = np.quantile(rel, [0.5, 0.9, 0.99, 0.999, 1.0])
    return dict(zip(("p50", "p90", "p99", "p99.9", "max"), (float(v) for v in q)))


def oracle_density(oracle_lib, nl, x, y):
    """Solver input of the loop at (x, y): movable map + rho_t * fixed map."""
    m = int(nl["bins"])
    W, H = float(nl["die"][2]), float(nl["die"][3])
    g = oracle_lib.grid(W, H, m)
    fixed = nl["node_fixed"] != 0
    area = (nl["node_w"] * nl["node_h"]) > 0
    mov_q = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], (~fixed & area).astype(np.uint8))
    fix_q = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], (fixed & area).astype(np.uint8))
    # the library holds the target density as a float (ap_params)
    fs_q = oracle_lib.scale_fixed(fix_q, float(np.float32(nl["target_density"])))
    return g, mov_q, fix_q, fs_q, oracle_lib.density_float(g, mov_q, fs_q)


@pytest.mark.parametrize("preset", ["c1", "c2"])
def test_field_solvers_full_size_vs_oracle(ap, oracle_lib, preset):
    """Both solvers on the density map of the netlist at a spread and at a
    clustered placement, against the dense FP64 solve (and the fast FP64
    solve, which must agree with it to rounding)."""
    nl = netlist(ap, preset)
    m = int(nl["bins"])
    with ap.Placer(nl) as pl:
        for x, y in (spread(nl, 3), clustered(nl, 4)):
            _, _, _, _, d = oracle_density(oracle_lib, nl, x, y)
            rex, rey = oracle_lib.field_solve(d.astype(np.float64), m)
            fex, fey = oracle_lib.field_solve_fft(d.astype(np.float64), m)
            assert np.abs(fex - rex).max() <= 1e-11 * np.abs(rex).max()
            for solver in ("fp32", "bf16x3"):
                ex, ey = pl.compute_electric_fields(d, solver)
                for got, ref in ((ex, rex), (ey, rey)):
                    mx = np.abs(ref).max()
                    err = np.abs(got - ref)
                    big = np.abs(ref) >= 1e-2 * mx
                    print(f"\n{preset} field {solver}: max|dE|/max|E| {err.max() / mx:.2e} rel(|E|>=1e-2 max) "
                          f"{quantiles(err[big] / np.abs(ref[big]))}")
                    assert err.max() <= 1e-4 * mx


@pytest.mark.parametrize("preset", ["c1", "c2"])
def test_wirelength_gradient_full_size(ap, oracle_lib, preset):
    nl = netlist(ap, preset)
    n = len(nl["node_w"])
    deg = np.diff(nl["net_ptr"])
    pin_net = np.repeat(np.arange(len(deg)), deg)
    counted = deg[pin_net] >= 2
    pins = np.bincount(nl["pin_node"][counted], minlength=n).astype(np.float64)
    bw = float(nl["die"][2]) / int(nl["bins"])
    with ap.Placer(nl) as pl:
        for (x, y), gamma in ((spread(nl, 5, 0.0), 4 * bw), (clustered(nl, 6), 0.4 * bw),
                              (spread(nl, 7, 0.0), 40 * bw)):
            gx, gy, wa, hp = pl.compute_all_partials(x, y, gamma)
            rx, ry, rwa, rhp = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, gamma)
            scale = max(np.abs(rx).max(), np.abs(ry).max())
            for got, ref in ((gx, rx), (gy, ry)):
                err = np.abs(got - ref)
                bound = pins * 2.0 ** -20 + 1e-4 * scale
                big = np.abs(ref) >= 1e-2 * scale
                print(f"\n{preset} WA gamma {gamma:.3g}: max|dg|/max|g| {err.max() / scale:.2e} "
                      f"max(|dg|/bound) {(err / bound).max():.3f} rel(|g|>=1e-2 max) "
                      f"{quantiles(err[big] / np.abs(ref[big]))}")
                assert (err <= bound).all()
            assert abs(hp - rhp) <= 1e-7 * rhp
            assert abs(wa - rwa) <= 1e-5 * rwa


@pytest.mark.parametrize("preset,start", [("c1", "spread"), ("c2", "spread"), ("c2", "clustered")])
def test_overflow_and_hpwl_readout(ap, oracle_lib, preset, start):
    """ap_overflow / ap_hpwl at the positions given to ap_init_positions
    against the oracle at the same positions: both overflow forms bit-exact,
    HPWL to 1e-7."""
    nl = netlist(ap, preset)
    x, y = spread(nl, 8) if start == "spread" else clustered(nl, 9)
    g, mov_q, fix_q, fs_q, _ = oracle_density(oracle_lib, nl, x, y)
    mov = nl["node_fixed"] == 0
    # llrintf(w * 2^16): the float product is exact, rint rounds half to even
    wq = np.rint(nl["node_w"][mov] * np.float32(65536.0)).astype(np.int64)
    hq = np.rint(nl["node_h"][mov] * np.float32(65536.0)).astype(np.int64)
    area_q = np.cumsum((wq * hq).astype(np.float64))[-1]  # the library's sequential FP64 sum
    tau, tau_abs = oracle_lib.overflow(g, mov_q, fix_q, fs_q, float(np.float32(nl["target_density"])), area_q)
    _, _, _, rhp = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, 1.0)
    from aieplace_gb300._lib import lib
    import ctypes as C

    with ap.Placer(nl) as pl:
        pl.initialize_placement(x, y)
        o, oa, hp = C.c_double(), C.c_double(), C.c_double()
        assert lib().ap_overflow(pl._h, C.byref(o), C.byref(oa)) == 0
        assert lib().ap_hpwl(pl._h, C.byref(hp)) == 0
    print(f"\n{preset} {start}: overflow {o.value!r} vs {tau!r}, abs {oa.value!r} vs {tau_abs!r}, "
          f"hpwl rel {abs(hp.value - rhp) / rhp:.2e}")
    assert o.value == tau
    assert oa.value == tau_abs
    assert abs(hp.value - rhp) <= 1e-7 * rhp


@pytest.mark.parametrize("preset", ["c1_small", "c1", "c2"])
def test_node_force_and_gradient_vs_oracle(ap, oracle_lib, preset):
    """The loop's gather (record path) per node: the overlap-weighted field
    (nudgeNode's force) and the preconditioned gradient, on the exact field
    of the density at the same positions."""
    nl = netlist(ap, preset) if preset != "c1_small" else ap.synth.generate(preset, seed=2)
    m = int(nl["bins"])
    n = len(nl["node_w"])
    mov = nl["node_fixed"] == 0
    for x, y in (spread(nl, 10), clustered(nl, 11, sigma=10.0)):
        g, _, _, _, d = oracle_density(oracle_lib, nl, x, y)
        ex64, ey64 = oracle_lib.field_solve_fft(d.astype(np.float64), m)
        ex, ey = ex64.astype(np.float32), ey64.astype(np.float32)
        rfx, rfy = oracle_lib.node_force(g, x, y, nl["node_w"], nl["node_h"], ex.astype(np.float64),
                                         ey.astype(np.float64), include=mov.astype(np.uint8))
        afx, afy = oracle_lib.node_force(g, x, y, nl["node_w"], nl["node_h"], np.abs(ex).astype(np.float64),
                                         np.abs(ey).astype(np.float64), include=mov.astype(np.uint8))
        bw = float(nl["die"][2]) / m
        gamma = 4 * bw
        rwx, rwy, _, _ = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, gamma)
        # lambda balancing the two terms, as a float (the kernel's type)
        lam = float(np.float32((np.abs(rwx[mov]).sum() + np.abs(rwy[mov]).sum()) /
                               max(np.abs(rfx).sum() + np.abs(rfy).sum(), 1e-30)))
        with ap.Placer(nl) as pl:
            fx, fy, gx, gy = pl.compute_node_forces(x, y, ex, ey, gamma, lam)
            wgx, wgy, _, _ = pl.compute_all_partials(x, y, gamma)
        # sum_b w_ib |E_b| as the error scale; a weight can be a hair below
        # zero where a node edge sits between the float bin edge that picks
        # the bin index and the fixed-point one (both sides use the same
        # integers), hence the absolute value
        afx, afy = np.abs(afx), np.abs(afy)
        for got, ref, scl in ((fx, rfx, afx), (fy, rfy, afy)):
            err = np.abs(got - ref)
            bound = 1e-5 * scl + 1e-30
            print(f"\n{preset} force: max(|dF|/bound) {(err / bound).max():.3f}")
            assert (err <= bound).all()
        deg = np.diff(nl["net_ptr"])
        pin_net = np.repeat(np.arange(len(deg)), deg)
        pins = np.bincount(nl["pin_node"][deg[pin_net] >= 2], minlength=n).astype(np.float64)
        W, H = float(nl["die"][2]), float(nl["die"][3])
        ab = float(np.float32(W) / np.float32(m)) * float(np.float32(H) / np.float32(m))
        charge = nl["node_w"].astype(np.float64) * nl["node_h"] / ab
        hd = np.maximum(1.0, pins + lam * charge)
        for got, wl, f, scl in ((gx, rwx, rfx, afx), (gy, rwy, rfy, afy)):
            ref = (wl - lam * f) / hd
            err = np.abs(got - ref)[mov]
            # quantised WA terms, the force bound, FP32 rounding of the
            # difference of the two terms, and of the preconditioner
            bound = ((pins * 2.0 ** -20 + lam * 1e-5 * scl + 1e-6 * (np.abs(wl) + lam * np.abs(f))) / hd
                     + 1e-5 * np.abs(ref))[mov]
            ratio = err / np.maximum(bound, 1e-300)
            print(f"\n{preset} precond grad (lambda {lam:.3g}): max(|dg|/bound) {ratio.max():.3f} "
                  f"rel {quantiles(err / np.maximum(np.abs(ref[mov]), 1e-30))}")
            if not (err <= bound).all():
                ids = np.flatnonzero(mov)[np.argsort(-ratio)[:5]]
                gw = wgx if got is gx else wgy
                gf = fx if got is gx else fy
                for i in ids:
                    print(f"  node {i}: got {got[i]!r} ref {ref[i]!r} wl {wl[i]!r} gpu-wl {gw[i]!r} F {f[i]!r} "
                          f"gpu-F {gf[i]!r} pins {pins[i]} hd {hd[i]!r} charge {charge[i]!r} "
                          f"from-gpu-parts {(gw[i] - lam * gf[i]) / hd[i]!r} x {x[i]!r} y {y[i]!r}")
            assert (err <= bound).all()
            assert (got[~mov] == 0).all()


_C1_ORACLE = {}


@pytest.mark.parametrize("solver", ["fp32", "bf16x3"])
def test_loop_c1_final_hpwl_and_overflow_match_oracle(ap, oracle_lib, solver):
    """200k cells, 512^2 bins, target density 0.7: from the same seeded start
    (die centre + N(0, 1 site)), both loops run to overflow < 0.10; the GPU
    loop's final HPWL within 0.5% and final overflow within 0.005 of the FP64
    oracle loop's."""
    nl = netlist(ap, "c1")
    x0, y0 = clustered(nl, 1, sigma=1.0)
    if "run" not in _C1_ORACLE:
        ref = oracle_lib.Placer(nl, 512, 0.7)
        ref.init(x0, y0)
        while ref.stats()["overflow"] >= 0.10 and ref.stats()["iteration"] < 4000:
            ref.step(1)
        _C1_ORACLE["run"] = ref.stats()
    rs = _C1_ORACLE["run"]
    with ap.Placer(nl, field_solver=solver, check_interval=1, max_iterations=4000) as pl:
        pl.initialize_placement(x0, y0)
        pl.run()
        s = pl.stats()
    print(f"\nc1 loop {solver}: gpu it {s['iteration']} hpwl {s['hpwl']:.6g} overflow {s['overflow']:.4f}; "
          f"oracle it {rs['iteration']} hpwl {rs['hpwl']:.6g} overflow {rs['overflow']:.4f}")
    assert s["overflow"] < 0.10 and rs["overflow"] < 0.10
    assert abs(s["hpwl"] - rs["hpwl"]) <= 0.005 * rs["hpwl"], (s, rs)
    assert abs(s["overflow"] - rs["overflow"]) <= 0.005, (s, rs)


@pytest.mark.parametrize("preset,iters,fillers", [("c1_small", 3, 0), ("c1_small", 40, 1), ("c2", 5, 0),
                                                  ("c2", 60, 0)])
def test_loop_density_matches_oracle_at_its_positions(ap, oracle_lib, preset, iters, fillers):
    """The loop's own density pass (position update -> bin records -> scatter,
    filler cells in their own map) through its overflow readout: after some
    iterations from the clustered start, both overflow forms equal the
    oracle's at the loop's accepted positions, bit for bit."""
    nl = netlist(ap, preset) if preset == "c2" else ap.synth.generate(preset, seed=3)
    with ap.Placer(nl, filler_cells=fillers) as pl:
        pl.initialize_placement(seed=11, sigma=1.0)
        pl.perform_iteration(iters)
        s = pl.stats()
        x, y = pl.positions()
    g, mov_q, fix_q, fs_q, _ = oracle_density(oracle_lib, nl, x, y)
    mov = nl["node_fixed"] == 0
    wq = np.rint(nl["node_w"][mov] * np.float32(65536.0)).astype(np.int64)
    hq = np.rint(nl["node_h"][mov] * np.float32(65536.0)).astype(np.int64)
    area_q = np.cumsum((wq * hq).astype(np.float64))[-1]
    tau, tau_abs = oracle_lib.overflow(g, mov_q, fix_q, fs_q, float(np.float32(nl["target_density"])), area_q)
    print(f"\n{preset} after {iters}: overflow {s['overflow']!r} vs {tau!r}")
    assert s["overflow"] == tau and s["overflow_abs"] == tau_abs
