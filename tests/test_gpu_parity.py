"""CUDA path against the CPU oracle, through the C ABI.

Tolerances (stated per result, as the comparison is made):
  density map      bit-exact int64 (same fixed-point definition)
  overflow         bit-exact integer sum -> identical double
  WA gradient      |dg| <= 1e-4 * max|g| per node, FP32 kernel vs FP64 oracle
  HPWL / WA        1e-6 / 1e-5 relative
  field (FP32)     max|dE| <= 1e-4 * max|E| vs the FP64 oracle
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


def spread_positions(nl, rng, margin=3.0):
    """Movable cells scattered over (and a little beyond) the die."""
    W, H = float(nl["die"][2]), float(nl["die"][3])
    x = nl["node_x"].copy()
    y = nl["node_y"].copy()
    mov = nl["node_fixed"] == 0
    x[mov] = rng.uniform(-margin, W + margin, mov.sum()).astype(np.float32)
    y[mov] = rng.uniform(-margin, H + margin, mov.sum()).astype(np.float32)
    return x, y


@pytest.mark.parametrize("preset,bins", [("c0", 32), ("c1_small", 128), ("c1_small", 512)])
def test_density_map_bit_exact(ap, oracle_lib, preset, bins):
    nl = ap.synth.generate(preset, seed=4)
    rng = np.random.default_rng(0)
    x, y = spread_positions(nl, rng)
    with ap.Placer(nl, bins=bins) as pl:
        got = pl.compute_overlaps(x, y)
    g = oracle_lib.grid(float(nl["die"][2]), float(nl["die"][3]), bins)
    area = (nl["node_w"] * nl["node_h"]) > 0
    ref = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], area.astype(np.uint8))
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("preset,bins,sigma,outliers,at", [("c1_small", 512, 1.0, 0.0, 0.5),
                                                            ("c1_small", 128, 0.3, 0.0, 0.5),
                                                            ("c0", 32, 0.5, 0.0, 0.5),
                                                            ("c1_small", 512, 4.0, 0.01, 0.5),
                                                            ("c1_small", 128, 2.0, 0.02, 0.0),
                                                            ("c1_small", 512, 1.5, 0.0, 1.0)])
def test_density_map_bit_exact_clustered(ap, oracle_lib, preset, bins, sigma, outliers, at):
    """Nodes packed around one point (the die centre: the initial placement;
    a die corner: the scatter's register tile clamped to the edge, nodes
    partly off the die): the tile's outer products for nodes inside it,
    global adds for the rest and for outliers anywhere on the die."""
    nl = ap.synth.generate(preset, seed=5)
    rng = np.random.default_rng(2)
    W, H = float(nl["die"][2]), float(nl["die"][3])
    x = nl["node_x"].copy()
    y = nl["node_y"].copy()
    mov = nl["node_fixed"] == 0
    x[mov] = (W * at + sigma * rng.standard_normal(mov.sum())).astype(np.float32)
    y[mov] = (H * at + sigma * rng.standard_normal(mov.sum())).astype(np.float32)
    far = np.flatnonzero(mov)[rng.random(mov.sum()) < outliers]
    x[far] = rng.uniform(0, W, far.size).astype(np.float32)
    y[far] = rng.uniform(0, H, far.size).astype(np.float32)
    with ap.Placer(nl, bins=bins) as pl:
        got = pl.compute_overlaps(x, y)
    g = oracle_lib.grid(W, H, bins)
    area = (nl["node_w"] * nl["node_h"]) > 0
    ref = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], area.astype(np.uint8))
    assert np.array_equal(got, ref)


def test_density_map_bit_exact_full_size(ap, oracle_lib):
    """2M cells / 1024^2 bins: the shipped mixed-precision workload."""
    nl = ap.synth.generate("c2", seed=1)
    rng = np.random.default_rng(1)
    x, y = spread_positions(nl, rng, margin=0.0)
    with ap.Placer(nl, bins=1024, target_density=0.8) as pl:
        got = pl.compute_overlaps(x, y)
        got2 = pl.compute_overlaps(x, y)
    assert np.array_equal(got, got2)  # deterministic run to run
    g = oracle_lib.grid(float(nl["die"][2]), float(nl["die"][3]), 1024)
    area = (nl["node_w"] * nl["node_h"]) > 0
    ref = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], area.astype(np.uint8))
    assert np.array_equal(got, ref)
    assert got.sum() == ref.sum()


def test_conversion_helpers_match_hardware(ap):
    """The hot path rounds and converts with integer arithmetic (the FP64 pipe
    that executes conversion instructions is narrow on this part); every helper
    must give the conversion instruction's result bit for bit."""
    from aieplace_gb300._lib import check, lib, ptr

    m = np.zeros(6, np.int32)
    check("ap_selftest_numerics", lib().ap_selftest_numerics(ptr(m), 1 << 26))
    assert m.tolist() == [0, 0, 0, 0, 0, 0]


@pytest.mark.parametrize("preset,gamma", [("c0", 4.0), ("c1_small", 0.7), ("c1_small", 25.0)])
def test_wirelength_gradient(ap, oracle_lib, preset, gamma):
    nl = ap.synth.generate(preset, seed=5)
    rng = np.random.default_rng(2)
    x, y = spread_positions(nl, rng, margin=0.0)
    with ap.Placer(nl, bins=32 if preset == "c0" else 128) as pl:
        gx, gy, wa, hp = pl.compute_all_partials(x, y, gamma)
    rx, ry, rwa, rhp = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, gamma)
    scale = max(np.abs(rx).max(), np.abs(ry).max())
    assert np.abs(gx - rx).max() <= 1e-4 * scale
    assert np.abs(gy - ry).max() <= 1e-4 * scale
    assert abs(hp - rhp) <= 1e-6 * rhp
    assert abs(wa - rwa) <= 1e-5 * rwa


def test_wirelength_gradient_every_degree_bucket(ap, oracle_lib):
    """Nets of degree 2..8 (thread per net), 9..16 (16 lanes), 17..32 and
    33..64 (a warp, pins in registers) and 65..300 (a warp looping): the
    synthetic netlists have none above 64, so these are added here."""
    nl = dict(ap.synth.generate("c0", seed=2))
    rng = np.random.default_rng(8)
    n = len(nl["node_w"])
    ptr = list(nl["net_ptr"])
    pins = list(nl["pin_node"])
    for d in (9, 12, 16, 17, 24, 32, 33, 48, 64, 65, 100, 200, 300):
        pins += list(rng.choice(n, size=min(d, n), replace=False))
        ptr.append(len(pins))
    nl["net_ptr"] = np.array(ptr, np.int32)
    nl["pin_node"] = np.array(pins, np.int32)
    x, y = spread_positions(nl, rng, margin=0.0)
    with ap.Placer(nl, bins=32) as pl:
        gx, gy, wa, hp = pl.compute_all_partials(x, y, 2.0)
    rx, ry, rwa, rhp = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, 2.0)
    scale = max(np.abs(rx).max(), np.abs(ry).max())
    assert np.abs(gx - rx).max() <= 1e-4 * scale
    assert np.abs(gy - ry).max() <= 1e-4 * scale
    assert abs(hp - rhp) <= 1e-6 * rhp
    assert abs(wa - rwa) <= 1e-5 * rwa


def test_nets_below_two_pins_change_nothing(ap, oracle_lib):
    """Nets of 0 and 1 pins interleaved in the CSR.  The reference takes no
    partials from them (computeNetPartials_CPU returns below degree 2,
    AIEplace.cpp:655) and their HPWL is 0: the gradient, HPWL and WA equal
    the oracle's, and the loop is bit-identical to the loop on the netlist
    without them."""
    base = ap.synth.generate("c0", seed=6)
    rng = np.random.default_rng(6)
    n = len(base["node_w"])
    bptr, bpins = base["net_ptr"], base["pin_node"]
    ptr, pins = [0], []
    for e in range(len(bptr) - 1):
        if rng.random() < 0.05:  # an empty net
            ptr.append(len(pins))
        if rng.random() < 0.05:  # a one-pin net
            pins.append(int(rng.integers(n)))
            ptr.append(len(pins))
        pins += [int(p) for p in bpins[bptr[e]:bptr[e + 1]]]
        ptr.append(len(pins))
    nl = dict(base)
    nl["net_ptr"], nl["pin_node"] = np.array(ptr, np.int32), np.array(pins, np.int32)
    assert len(ptr) - 1 > len(bptr) - 1
    x, y = spread_positions(nl, rng, margin=0.0)
    with ap.Placer(nl, bins=32) as pl:
        gx, gy, wa, hp = pl.compute_all_partials(x, y, 2.0)
    rx, ry, rwa, rhp = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, 2.0)
    scale = max(np.abs(rx).max(), np.abs(ry).max())
    assert np.abs(gx - rx).max() <= 1e-4 * scale
    assert np.abs(gy - ry).max() <= 1e-4 * scale
    assert abs(hp - rhp) <= 1e-6 * rhp
    assert abs(wa - rwa) <= 1e-5 * rwa
    with ap.Placer(base, bins=32) as a, ap.Placer(nl, bins=32) as b:
        a.initialize_placement(base["node_x"], base["node_y"])
        b.initialize_placement(base["node_x"], base["node_y"])
        a.perform_iteration(20)
        b.perform_iteration(20)
        (ax, ay), (bx, by) = a.positions(), b.positions()
        np.testing.assert_array_equal(ax, bx)
        np.testing.assert_array_equal(ay, by)
        assert a.stats()["hpwl"] == b.stats()["hpwl"]


@pytest.mark.parametrize("solver", ["fp32", "bf16x3"])
def test_rectangular_die_against_oracle(ap, oracle_lib, solver):
    """A die 1.5 times as wide as high (bins 1.5 times as wide as tall; 20k
    cells, 128^2 bins): the density map bit-exact, the field within 1e-4 of
    the largest against the oracle's solve with the same bin ratio, and the
    per-node force within 1e-5 of the force on |E|."""
    nl = dict(ap.synth.generate("c1_small", seed=9))
    nl["die"] = nl["die"].copy()
    nl["die"][2] *= 1.5
    nl["node_x"] = (nl["node_x"] * np.float32(1.5)).astype(np.float32)
    rng = np.random.default_rng(9)
    x, y = spread_positions(nl, rng, margin=0.0)
    M = 128
    W, H = float(nl["die"][2]), float(nl["die"][3])
    g = oracle_lib.grid(W, H, M)
    mov = nl["node_fixed"] == 0
    area = (nl["node_w"] * nl["node_h"]) > 0
    ref = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], area.astype(np.uint8))
    d = (ref.reshape(M, M) / float(g.bw_q * g.bh_q)).astype(np.float32)
    ratio = float(np.float32(g.bh / g.bw))
    rex, rey = oracle_lib.field_solve(d.astype(np.float64), M, bin_ratio=ratio)
    with ap.Placer(nl, bins=M) as pl:
        got = pl.compute_overlaps(x, y)
        ex, ey = pl.compute_electric_fields(d, solver)
        fx, fy = pl.compute_node_forces(x, y, ex, ey)
    assert np.array_equal(got, ref)
    scale = max(np.abs(rex).max(), np.abs(rey).max())
    assert np.abs(ex - rex).max() <= 1e-4 * scale
    assert np.abs(ey - rey).max() <= 1e-4 * scale
    rfx, rfy = oracle_lib.node_force(g, x, y, nl["node_w"], nl["node_h"], ex.astype(np.float64),
                                     ey.astype(np.float64), include=mov.astype(np.uint8))
    afx, afy = oracle_lib.node_force(g, x, y, nl["node_w"], nl["node_h"], np.abs(ex).astype(np.float64),
                                     np.abs(ey).astype(np.float64), include=mov.astype(np.uint8))
    assert np.all(np.abs(fx[mov] - rfx[mov]) <= 1e-5 * np.abs(afx[mov]) + 1e-12)
    assert np.all(np.abs(fy[mov] - rfy[mov]) <= 1e-5 * np.abs(afy[mov]) + 1e-12)


def test_largest_bin_count(ap, oracle_lib):
    """4096^2 bins, the largest grid ap_create takes (20k cells, each over
    tens of bins: the general overlap path): the density map bit-exact, both
    field solvers within 1e-4 of the largest against the oracle's FP64 fast
    transforms."""
    nl = ap.synth.generate("c1_small", seed=10)
    rng = np.random.default_rng(10)
    x, y = spread_positions(nl, rng, margin=0.0)
    M = 4096
    g = oracle_lib.grid(float(nl["die"][2]), float(nl["die"][3]), M)
    area = (nl["node_w"] * nl["node_h"]) > 0
    ref = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], area.astype(np.uint8))
    d = (ref.reshape(M, M) / float(g.bw_q * g.bh_q)).astype(np.float32)
    rex, rey = oracle_lib.field_solve_fft(d.astype(np.float64), M)
    scale = max(np.abs(rex).max(), np.abs(rey).max())
    with ap.Placer(nl, bins=M) as pl:
        assert np.array_equal(pl.compute_overlaps(x, y), ref)
        for solver in ("fp32", "bf16x3"):
            ex, ey = pl.compute_electric_fields(d, solver)
            assert np.abs(ex - rex).max() <= 1e-4 * scale, solver
            assert np.abs(ey - rey).max() <= 1e-4 * scale, solver


def test_netlist_without_nets(ap):
    """No nets at all: zero gradient, HPWL and WA.  ePlace's initial density
    weight is the ratio of the wirelength and density gradient norms, 0
    here, and the step length of a zero gradient difference is 0: the loop
    runs without error and leaves every cell where it is."""
    nl = dict(ap.synth.generate("c0", seed=7))
    nl["net_ptr"] = np.zeros(1, np.int32)
    nl["pin_node"] = np.zeros(0, np.int32)
    x, y = nl["node_x"], nl["node_y"]
    with ap.Placer(nl, bins=32) as pl:
        gx, gy, wa, hp = pl.compute_all_partials(x, y, 2.0)
        assert not gx.any() and not gy.any() and wa == 0.0 and hp == 0.0
        pl.initialize_placement(seed=3, sigma=1.0)
        tau0 = pl.overflow()[0]
        x0, y0 = pl.positions()
        pl.perform_iteration(30)
        s = pl.stats()
        assert s["status"] == 0 and s["hpwl"] == 0.0 and s["overflow"] == tau0
        x1, y1 = pl.positions()
        np.testing.assert_array_equal(x0, x1)
        np.testing.assert_array_equal(y0, y1)


def with_hub_nodes(ap, seed=3):
    """c0 plus 600 two-pin nets on one movable node and 700 on one fixed node:
    more pins than one packed two-axis accumulator holds (512), so those two
    nodes take the per-axis accumulators."""
    nl = dict(ap.synth.generate("c0", seed=seed))
    rng = np.random.default_rng(seed)
    n = len(nl["node_w"])
    fixed = np.flatnonzero(nl["node_fixed"])
    mov = np.flatnonzero(nl["node_fixed"] == 0)
    hubs = [(int(mov[n // 7 % len(mov)]), 600)] + ([(int(fixed[0]), 700)] if len(fixed) else [])
    ptr = list(nl["net_ptr"])
    pins = list(nl["pin_node"])
    for hub, k in hubs:
        for o in rng.choice(np.setdiff1d(np.arange(n), [hub]), size=k):
            pins += [hub, int(o)]
            ptr.append(len(pins))
    nl["net_ptr"] = np.array(ptr, np.int32)
    nl["pin_node"] = np.array(pins, np.int32)
    return nl, [h for h, _ in hubs]


def test_wirelength_gradient_hub_nodes(ap, oracle_lib):
    nl, hubs = with_hub_nodes(ap)
    rng = np.random.default_rng(4)
    x, y = spread_positions(nl, rng, margin=0.0)
    with ap.Placer(nl, bins=32) as pl:
        gx, gy, wa, hp = pl.compute_all_partials(x, y, 2.0)
    rx, ry, rwa, rhp = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, 2.0)
    scale = max(np.abs(rx).max(), np.abs(ry).max())
    assert np.abs(gx - rx).max() <= 1e-4 * scale
    assert np.abs(gy - ry).max() <= 1e-4 * scale
    for hub in hubs:  # the per-axis accumulators: hundreds of pins in one sum
        assert abs(rx[hub]) + abs(ry[hub]) > 10.0
        assert abs(gx[hub] - rx[hub]) <= 1e-5 * (abs(rx[hub]) + 1.0)
        assert abs(gy[hub] - ry[hub]) <= 1e-5 * (abs(ry[hub]) + 1.0)
    assert abs(hp - rhp) <= 1e-6 * rhp


def test_loop_hub_nodes_first_iterations_like_oracle(ap, oracle_lib):
    """The loop's gather reads the hub's per-axis accumulators: its first
    iterations follow the FP64 oracle loop (positions within 1e-3 of the die)."""
    nl, hubs = with_hub_nodes(ap)
    ref = oracle_lib.Placer(nl, 32, 1.0)
    ref.init(nl["node_x"], nl["node_y"])
    with ap.Placer(nl, bins=32, target_density=1.0) as pl:
        pl.initialize_placement(nl["node_x"], nl["node_y"])
        for _ in range(3):
            pl.perform_iteration(1)
            ref.step(1)
            x, y = pl.positions()
            rx, ry = ref.positions()
            tol = 1e-3 * float(nl["die"][2])
            assert np.abs(x - rx).max() <= tol and np.abs(y - ry).max() <= tol
            assert abs(x[hubs[0]] - rx[hubs[0]]) <= tol and abs(y[hubs[0]] - ry[hubs[0]]) <= tol


@pytest.mark.parametrize("m", [32, 128, 512])
def test_field_fp32_against_oracle(ap, oracle_lib, m):
    rng = np.random.default_rng(m)
    d = rng.random((m, m)).astype(np.float32)
    d[m // 4: m // 2, m // 3: m // 2] += 3.0  # a dense block: strong low frequencies
    nl = ap.synth.generate("c0", seed=1)
    with ap.Placer(nl, bins=m) as pl:
        ex, ey = pl.compute_electric_fields(d, "fp32")
    rex, rey = oracle_lib.field_solve(d.astype(np.float64), m)
    for got, ref in ((ex, rex), (ey, rey)):
        assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def test_field_fp32_matches_reference_fft_golden(ap):
    """replace::FFT::doFFT outputs (fft_replace/fft.cpp), committed fixture."""
    from conftest import golden

    g = golden("replace_field.npz")
    nl = ap.synth.generate("c0", seed=1)
    for case in ("rand32", "rand64"):
        d = g[f"{case}_density"]
        m = d.shape[0]
        with ap.Placer(nl, bins=m) as pl:
            ex, ey = pl.compute_electric_fields(d, "fp32")
        for got, ref in ((ex, g[f"{case}_ex"]), (ey, g[f"{case}_ey"])):
            ref = ref.reshape(-1)
            assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def test_loop_deterministic_and_resumable(ap):
    nl = ap.synth.generate("c1_small", seed=2)
    runs = []
    for _ in range(2):
        with ap.Placer(nl, bins=128) as pl:
            pl.initialize_placement(seed=7, sigma=1.0)
            pl.perform_iteration(40)
            snap = pl.snapshot()
            pl.perform_iteration(25)
            runs.append(pl.positions())
            s = pl.stats()
            pl.restore(snap)
            pl.perform_iteration(25)
            again = pl.positions()
        np.testing.assert_array_equal(runs[-1][0], again[0])
        np.testing.assert_array_equal(runs[-1][1], again[1])
        assert s["iteration"] == 65 and s["evals"] >= 65
    np.testing.assert_array_equal(runs[0][0], runs[1][0])


@pytest.mark.parametrize("use_graph", [1, 0])
def test_caller_stream_matches_own_stream(ap, use_graph):
    """A trial step forks its wirelength launches onto a library stream and
    joins before the gather; on a caller's stream (ap_set_stream), captured in
    a graph or launched eagerly, the loop gives the same bits as on the
    handle's own stream."""
    import torch

    nl = ap.synth.generate("c1_small", seed=4)
    runs = []
    for caller in (False, True):
        with ap.Placer(nl, bins=128, use_graph=use_graph) as pl:
            s = torch.cuda.Stream()
            if caller:
                pl.set_stream(s.cuda_stream)
            pl.initialize_placement(seed=3, sigma=1.0)
            pl.step_async(60)
            if caller:
                ev = torch.cuda.Event()
                ev.record(s)  # everything of the steps precedes an event on the caller's stream
                ev.synchronize()
            runs.append((pl.positions(), pl.stats()))
    (x0, y0), s0 = runs[0]
    (x1, y1), s1 = runs[1]
    np.testing.assert_array_equal(x0, x1)
    np.testing.assert_array_equal(y0, y1)
    assert s0["hpwl"] == s1["hpwl"] and s0["iteration"] == s1["iteration"]


def test_step_host_matches_device_step(ap):
    nl = ap.synth.generate("c0", seed=1)
    with ap.Placer(nl, bins=32) as a, ap.Placer(nl, bins=32) as b:
        a.initialize_placement(nl["node_x"], nl["node_y"])
        b.initialize_placement(nl["node_x"], nl["node_y"])
        x, y = b.positions()
        xo, yo = np.zeros_like(x), np.zeros_like(y)
        for _ in range(10):
            a.perform_iteration(1)
            s = b.step_host(x, y, xo, yo)
            x, y = xo.copy(), yo.copy()
        ax, ay = a.positions()
        np.testing.assert_array_equal(ax, x)
        np.testing.assert_array_equal(ay, y)
        assert s["iteration"] == 10


def test_step_host_output_only_and_in_place(ap):
    # no input (the device state steps on), and one buffer as input and output
    nl = ap.synth.generate("c0", seed=2)
    with ap.Placer(nl, bins=32) as a, ap.Placer(nl, bins=32) as b:
        a.initialize_placement(nl["node_x"], nl["node_y"])
        b.initialize_placement(nl["node_x"], nl["node_y"])
        xo, yo = np.zeros(b.num_nodes, np.float32), np.zeros(b.num_nodes, np.float32)
        for _ in range(3):
            a.perform_iteration(1)
            b.step_host(None, None, xo, yo)
        ax, ay = a.positions()
        np.testing.assert_array_equal(ax, xo)
        np.testing.assert_array_equal(ay, yo)
        x, y = b.positions()
        for _ in range(3):
            a.perform_iteration(1)
            s = b.step_host(x, y, x, y)
        ax, ay = a.positions()
        np.testing.assert_array_equal(ax, x)
        np.testing.assert_array_equal(ay, y)
        assert s["iteration"] == 6


@pytest.mark.parametrize("preset,bins", [("c0", 32), ("c2_small", 512)])
def test_step_host_pinned_buffers_match_eager_host_step(ap, preset, bins):
    """Host steps on pinned buffers (asynchronous copies; 200k cells: the
    input copied in four chunks, each with its own update launch) step
    exactly as the same calls on pageable buffers, with two buffer sets
    alternating, in place, and with pageable calls in between."""
    torch = pytest.importorskip("torch")
    nl = ap.synth.generate(preset, seed=4)
    with ap.Placer(nl, bins=bins) as a, ap.Placer(nl, bins=bins) as b:
        a.initialize_placement(nl["node_x"], nl["node_y"])
        b.initialize_placement(nl["node_x"], nl["node_y"])
        n = b.num_nodes

        def pinned():
            return torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()

        ax, ay = a.positions()
        axo, ayo = np.zeros_like(ax), np.zeros_like(ay)
        ix, iy, ox, oy = pinned(), pinned(), pinned(), pinned()  # input, output
        ix[:], iy[:] = b.positions()
        for k in range(10):
            sa = a.step_host(ax, ay, axo, ayo)
            ax, ay = axo.copy(), ayo.copy()
            if k == 6:  # in place
                ox, oy = ix, iy
            elif k == 7:  # pageable input and output
                ix, iy = ix.copy(), iy.copy()
                ox, oy = ix, iy
            elif k == 8:  # pinned again (new buffers), from the pageable result
                px, py = pinned(), pinned()
                px[:], py[:] = ix, iy
                ix, iy, ox, oy = px, py, pinned(), pinned()
            s = b.step_host(ix, iy, ox, oy)
            np.testing.assert_array_equal(ax, ox)
            np.testing.assert_array_equal(ay, oy)
            assert s["hpwl"] == sa["hpwl"] and s["overflow"] == sa["overflow"]
            if ox is not ix:  # the two buffer sets alternate
                ix, iy, ox, oy = ox, oy, ix, iy
        assert s["iteration"] == 10


def test_errors_are_status_codes(ap):
    from aieplace_gb300 import APError

    nl = ap.synth.generate("c0", seed=1)
    with ap.Placer(nl, bins=32) as pl:
        with pytest.raises(APError) as e:
            pl.perform_iteration(1)  # before any initial placement
        assert e.value.status == 8
        bad = nl["node_x"].copy()
        bad[0] = np.inf
        with pytest.raises(APError) as e:
            pl.initialize_placement(bad, nl["node_y"])
        assert e.value.status == 3


def test_loop_c0_reaches_target_like_oracle(ap, oracle_lib):
    """576-cell case: the GPU loop (FP32, fixed-point density) and the FP64
    oracle loop both reach overflow < 0.10; final HPWL within 0.5%... of each
    other is not implied by a non-convex trajectory, so the bound checked is 3%
    on HPWL and 0.005 on overflow at the first iteration each goes below 0.10."""
    nl = ap.synth.generate("c0", seed=1)
    ref = oracle_lib.Placer(nl, 32, 1.0)
    ref.init(nl["node_x"], nl["node_y"])
    while ref.stats()["overflow"] >= 0.10 and ref.stats()["iteration"] < 3000:
        ref.step(1)
    rs = ref.stats()
    with ap.Placer(nl, bins=32, target_density=1.0, check_interval=1) as pl:
        pl.initialize_placement(nl["node_x"], nl["node_y"])
        pl.run()
        s = pl.stats()
    assert s["overflow"] < 0.10 and rs["overflow"] < 0.10
    assert abs(s["hpwl"] - rs["hpwl"]) <= 0.03 * rs["hpwl"], (s, rs)
    assert abs(s["iteration"] - rs["iteration"]) <= 0.2 * rs["iteration"], (s, rs)


_ORACLE_RUNS = {}


def clustered_start(nl, seed):
    """Movable cells at the die centre plus N(0, 1 site), seeded."""
    rng = np.random.default_rng(seed)
    W, H = float(nl["die"][2]), float(nl["die"][3])
    x0, y0 = nl["node_x"].copy(), nl["node_y"].copy()
    mov = nl["node_fixed"] == 0
    x0[mov] = (W / 2 + rng.standard_normal(mov.sum())).astype(np.float32)
    y0[mov] = (H / 2 + rng.standard_normal(mov.sum())).astype(np.float32)
    return x0, y0


@pytest.mark.parametrize("solver", ["fp32", "bf16x3"])
@pytest.mark.parametrize("seed", [1, 2])
def test_loop_final_hpwl_and_overflow_match_oracle(ap, oracle_lib, solver, seed):
    """20k cells, 128^2 bins, target density 0.7, both loops run to overflow
    < 0.10 from the same seeded start: the GPU loop's final HPWL within 0.5%
    and final overflow within 0.005 of the FP64 oracle loop's (measured
    -0.11% to +0.15%, < 0.001).  The oracle sums in a fixed order, so both
    loops are deterministic and so is the comparison.  On the 576-cell case
    the stopping iteration is too sensitive for this bound (see
    test_loop_c0_reaches_target_like_oracle)."""
    nl = ap.synth.generate("c1_small", seed=seed)
    x0, y0 = clustered_start(nl, seed)
    if seed not in _ORACLE_RUNS:
        ref = oracle_lib.Placer(nl, 128, 0.7)
        ref.init(x0, y0)
        while ref.stats()["overflow"] >= 0.10 and ref.stats()["iteration"] < 4000:
            ref.step(1)
        _ORACLE_RUNS[seed] = ref.stats()
    rs = _ORACLE_RUNS[seed]
    with ap.Placer(nl, bins=128, target_density=0.7, check_interval=1, field_solver=solver) as pl:
        pl.initialize_placement(x0, y0)
        pl.run()
        s = pl.stats()
    assert s["overflow"] < 0.10 and rs["overflow"] < 0.10
    assert abs(s["hpwl"] - rs["hpwl"]) <= 0.005 * rs["hpwl"], (s, rs)
    assert abs(s["overflow"] - rs["overflow"]) <= 0.005, (s, rs)


def density_like(m, rng):
    """A placement-like density: ~0.8 background, a dense cluster, an empty macro."""
    d = (0.8 + 0.1 * rng.standard_normal((m, m))).astype(np.float32)
    d[m // 3: m // 2, m // 4: m // 2] += 2.5
    d[m // 8: m // 5, m // 8: m // 5] = 0.0
    return d


@pytest.mark.parametrize("m", [128, 256, 512])
def test_field_bf16x3_against_oracle(ap, oracle_lib, m):
    """tcgen05 BF16x3 (FP32 accumulate) vs the FP64 oracle: 1e-4 of max."""
    rng = np.random.default_rng(100 + m)
    d = density_like(m, rng)
    nl = ap.synth.generate("c0", seed=1)
    with ap.Placer(nl, bins=m) as pl:
        ex, ey = pl.compute_electric_fields(d, "bf16x3")
        ex2, ey2 = pl.compute_electric_fields(d, "bf16x3")
    np.testing.assert_array_equal(ex, ex2)  # deterministic
    rex, rey = oracle_lib.field_solve(d.astype(np.float64), m)
    for got, ref in ((ex, rex), (ey, rey)):
        assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def test_field_bf16x3_full_size_vs_fp32(ap):
    """1024^2 bins: the tensor-core solve against the FP32 SIMT solve of the
    same map, and linearity of the transform chain (E(2d) = 2 E(d))."""
    rng = np.random.default_rng(7)
    d = density_like(1024, rng)
    nl = ap.synth.generate("c0", seed=1)
    with ap.Placer(nl, bins=1024) as pl:
        ex, ey = pl.compute_electric_fields(d, "bf16x3")
        fx, fy = pl.compute_electric_fields(d, "fp32")
        ex2, ey2 = pl.compute_electric_fields(2.0 * d, "bf16x3")
    for got, ref in ((ex, fx), (ey, fy)):
        assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()
    assert np.abs(ex2 - 2 * ex).max() <= 1e-6 * np.abs(ex).max()


@pytest.mark.parametrize("m", [256, 1024])
def test_field_bf16x3_repeatable(ap, m):
    """The split-K clusters sum their partials in a fixed order through
    distributed shared memory: repeated solves of one map are bit-identical
    (a CTA writing a peer's buffers too early would show up here)."""
    rng = np.random.default_rng(m)
    d = density_like(m, rng)
    nl = ap.synth.generate("c0", seed=1)
    with ap.Placer(nl, bins=m) as pl:
        ex0, ey0 = pl.compute_electric_fields(d, "bf16x3")
        for _ in range(12):
            ex, ey = pl.compute_electric_fields(d, "bf16x3")
            np.testing.assert_array_equal(ex, ex0)
            np.testing.assert_array_equal(ey, ey0)
        fx, fy = pl.compute_electric_fields(d, "fp32")
    assert np.abs(ex0 - fx).max() <= 1e-4 * np.abs(fx).max()
    assert np.abs(ey0 - fy).max() <= 1e-4 * np.abs(fy).max()


def test_loop_bf16x3_matches_fp32_loop(ap):
    """Same netlist, both solvers: the mixed-precision loop reaches the target
    with HPWL within 1% of the plain FP32 loop."""
    nl = ap.synth.generate("c1_small", seed=3)
    res = {}
    for solver in ("fp32", "bf16x3"):
        with ap.Placer(nl, bins=128, field_solver=solver, max_iterations=3000) as pl:
            pl.initialize_placement(seed=5, sigma=1.0)
            pl.run()
            res[solver] = pl.stats()
    assert res["fp32"]["overflow"] < 0.10 and res["bf16x3"]["overflow"] < 0.10, res
    assert abs(res["bf16x3"]["hpwl"] - res["fp32"]["hpwl"]) <= 0.01 * res["fp32"]["hpwl"], res
