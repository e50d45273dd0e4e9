"""The CPU oracle against the reference's own golden vectors and functions.

Pins every restated function before anything is checked against it:
  - WA terms: vck5000/aie/golden_data/partials (bit-exact, fast_exp) and
    python/AIEmath/computeTerm.py on seeded nets (bit-exact);
  - 1-D transforms: customDCT.py outputs (1e-12) and the AIE density goldens
    (printed with 2 decimals, so 6e-3 / 3e-2 absolute);
  - field solve: replace::FFT::doFFT outputs (FP32 reference, 2e-6 of max);
  - density map / overflow / HPWL: Grid.cpp and Net.cpp outputs.
"""
import numpy as np
import pytest

from conftest import golden


def test_fast_exp_matches_python(oracle_lib):
    import math

    for a in (-3.7, -0.25, 0.0, 1.5):
        # computeTerm.fast_exp (computeTerm.py:6-13) in plain Python
        v = 1.0 + a / 2 ** 16
        for _ in range(16):
            v *= v
        assert oracle_lib.fast_exp(a) == v
    assert abs(oracle_lib.fast_exp(-1.0) - math.exp(-1.0)) < 1e-4


def test_aie_partials_golden_bit_exact(oracle_lib):
    g = golden("aie_partials.npz")
    for b in range(4):
        x = g[f"x{b}"]  # row 0 = max pin, row 1 = min pin, 8 nets (lanes)
        for lane in range(8):
            xs = np.array([x[1, lane], x[0, lane]])  # ascending
            ap, am, bc, part = oracle_lib.wa_terms_sorted(xs, 4.0, fast=True)
            assert ap[1] == g[f"a_plus{b}"][0, lane] and ap[0] == g[f"a_plus{b}"][1, lane]
            assert am[1] == g[f"a_minus{b}"][0, lane] and am[0] == g[f"a_minus{b}"][1, lane]
            assert bc[0] == g[f"b_plus{b}"][lane] and bc[1] == g[f"c_plus{b}"][lane]
            assert bc[2] == g[f"b_minus{b}"][lane] and bc[3] == g[f"c_minus{b}"][lane]
            assert part[1] == g[f"partials{b}"][0, lane] and part[0] == g[f"partials{b}"][1, lane]


def test_computeterm_seeded_nets(oracle_lib):
    """a-terms bit-exact; b/c/partials within a few ulps, because the fixture
    was produced under Python >= 3.12 whose built-in sum() (used by
    computeTerm.b_term) is compensated while the oracle sums in order."""
    g = golden("computeterm.npz")
    for k in range(int(g["count"])):
        ap, am, bc, part = oracle_lib.wa_terms_sorted(g[f"x{k}"], 4.0, fast=True)
        np.testing.assert_array_equal(ap, g[f"ap{k}"])
        np.testing.assert_array_equal(am, g[f"am{k}"])
        np.testing.assert_allclose(bc, g[f"bc{k}"], rtol=1e-15, atol=0)
        np.testing.assert_allclose(part, g[f"part{k}"], rtol=1e-12, atol=1e-11)  # formula cancels ~x/gamma


def test_wa_grad_matches_term_formula(oracle_lib):
    """or_wa_grad (AIEplace.cpp:612-673 over a CSR) equals the per-net term
    formula with exp, for nets in any pin order."""
    rng = np.random.default_rng(3)
    n, ne = 50, 30
    x = rng.uniform(0, 40, n).astype(np.float32)
    y = rng.uniform(0, 40, n).astype(np.float32)
    deg = rng.integers(2, 9, ne)
    ptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    pins = np.concatenate([rng.choice(n, d, replace=False) for d in deg]).astype(np.int32)
    gx, gy, wa, hp = oracle_lib.wa_grad(ptr, pins, x, y, 4.0)
    ex, ey = np.zeros(n), np.zeros(n)
    for e in range(ne):
        nodes = pins[ptr[e]:ptr[e + 1]]
        for coord, acc in ((x, ex), (y, ey)):
            order = np.argsort(coord[nodes], kind="stable")
            xs = coord[nodes][order].astype(np.float64)
            _, _, _, part = oracle_lib.wa_terms_sorted(xs, 4.0, fast=False)
            for j, i in enumerate(order):
                acc[nodes[i]] += part[j]
    np.testing.assert_allclose(gx, ex, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(gy, ey, rtol=1e-12, atol=1e-12)


def test_customdct_1d(oracle_lib):
    g = golden("customdct.npz")
    for n in (8, 16, 32):
        v = g[f"in{n}"]
        np.testing.assert_allclose(oracle_lib.dct_1d(v), g[f"dct{n}"], atol=1e-12)
        np.testing.assert_allclose(oracle_lib.idct_1d(v), g[f"idct{n}"], atol=1e-12)
        np.testing.assert_allclose(oracle_lib.idxst_1d(v), g[f"idxst{n}"], atol=1e-12)


def test_aie_dct_goldens(oracle_lib):
    """AIE transform goldens are printed with 2 decimals (createGoldenDCT.py:143-205)."""
    g = golden("aie_dct.npz")
    for r in range(8):
        np.testing.assert_allclose(oracle_lib.dct_1d(g["input_rows0_7"][r]), g["dct_output"][r], atol=6e-3)
    d2 = g["dct_2d_output"]
    for r in range(16):
        np.testing.assert_allclose(oracle_lib.idct_1d(d2[r]), g["idct_output"][r], atol=3e-2)
        np.testing.assert_allclose(oracle_lib.idxst_1d(d2[r]), g["idxst_output"][r], atol=3e-2)


@pytest.mark.parametrize("case", ["run_fft4", "rand16", "rand32", "rand64"])
def test_field_solve_matches_replace_fft(oracle_lib, case):
    g = golden("replace_field.npz")
    d = g[f"{case}_density"].astype(np.float64)
    m = d.shape[0]
    ex, ey, phi = oracle_lib.field_solve(d, m, want_phi=True)
    for mine, ref in ((ex, g[f"{case}_ex"]), (ey, g[f"{case}_ey"]), (phi, g[f"{case}_phi"])):
        ref = ref.reshape(-1).astype(np.float64)
        assert np.abs(mine - ref).max() <= 2e-6 * np.abs(ref).max() + 1e-9


@pytest.mark.parametrize("case", ["run_fft4", "rand16", "rand32", "rand64"])
def test_fast_field_solve_matches_replace_fft(oracle_lib, case):
    """The O(n^2 log n) solve that the oracle loop and the CPU baseline use,
    pinned to the reference's own Ooura solver output like the dense one."""
    g = golden("replace_field.npz")
    d = g[f"{case}_density"].astype(np.float64)
    m = d.shape[0]
    ex, ey, phi = oracle_lib.field_solve_fft(d, m, want_phi=True)
    for mine, ref in ((ex, g[f"{case}_ex"]), (ey, g[f"{case}_ey"]), (phi, g[f"{case}_phi"])):
        ref = ref.reshape(-1).astype(np.float64)
        assert np.abs(mine - ref).max() <= 2e-6 * np.abs(ref).max() + 1e-9


@pytest.mark.parametrize("m,ratio", [(8, 1.0), (64, 1.0), (256, 1.5), (1024, 1.0)])
def test_fast_field_solve_matches_dense(oracle_lib, m, ratio):
    """Fast transforms against the dense FP64 sums (the checker): the same
    sums in another order, so agreement is at FP64 rounding level."""
    rng = np.random.default_rng(m)
    d = rng.random(m * m) + np.where(rng.random(m * m) < 0.01, 5.0, 0.0)
    ex, ey, phi = oracle_lib.field_solve(d, m, ratio, want_phi=True)
    fx, fy, fphi = oracle_lib.field_solve_fft(d, m, ratio, want_phi=True)
    for a, b in ((ex, fx), (ey, fy), (phi, fphi)):
        assert np.abs(a - b).max() <= 1e-11 * np.abs(a).max()


def test_density_matches_reference_grid(oracle_lib):
    g = golden("ref_grid.npz")
    W, M = float(g["die"][0]), int(g["m"])
    grid = oracle_lib.grid(W, W, M)
    q = oracle_lib.density_q(grid, g["x"], g["y"], g["w"], g["h"])
    mine = q / 2.0 ** 32
    ref = g["rho"].astype(np.float64)
    # same bins touched (bin indices are exact), areas within the reference's
    # float accumulation error
    assert np.array_equal(mine != 0, ref != 0)
    assert np.abs(mine - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())
    zero = np.zeros_like(q)
    _, ab = oracle_lib.overflow(grid, q, zero, zero, 1.0, 1.0)
    assert abs(ab - float(g["overflow"])) <= 1e-5 * float(g["overflow"])


def test_hpwl_matches_reference_net(oracle_lib):
    g = golden("ref_grid.npz")
    _, _, _, hp = oracle_lib.wa_grad(g["hp_ptr"], g["hp_pins"], g["hp_x"], g["hp_y"], 4.0)
    assert abs(hp - float(g["hpwl"])) <= 1e-6 * float(g["hpwl"])


def test_reference_lib_live_when_built(oracle_lib):
    """When oracle/_ref exists (reference checkout present), re-run one case live."""
    R = oracle_lib.ref_lib()
    if R is None:
        pytest.skip("reference CPU library not built on this host")
    rng = np.random.default_rng(99)
    d = rng.random((16, 16)).astype(np.float32)
    ex, ey, phi = (np.zeros(256, np.float32) for _ in range(3))
    R.ref_replace_field(16, d.reshape(-1).copy(), phi.ctypes.data, ex, ey)
    mex, mey = oracle_lib.field_solve(d.astype(np.float64), 16)
    assert np.abs(mex - ex).max() <= 2e-6 * np.abs(ex).max()
    assert np.abs(mey - ey).max() <= 2e-6 * np.abs(ey).max()


def test_oracle_matches_reference_placer_fixture(oracle_lib):
    """The reference's own Placer (ref_placer.npz, made by make_golden.py from
    AIEplace.cpp built for the CPU) against the oracle on the same netlists
    and inputs (ref_placer_inputs.py): partials, density map, overflow,
    nudgeNode force, HPWL."""
    import ref_placer_inputs as I
    from aieplace_gb300.presets import PRESETS

    g = golden("ref_placer.npz")
    for name in I.CASES:
        nl = I.small_nets(oracle_lib.synth_generate(PRESETS[name], seed=I.SEED))
        assert int(g[f"{name}_n_nets"]) == len(nl["net_ptr"]) - 1
        x, y = I.positions(nl)
        W, H, M = float(nl["die"][2]), float(nl["die"][3]), nl["bins"]
        sub = slice(0, None, I.SUBSAMPLE)
        ox, oy, _, hp = oracle_lib.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, I.GAMMA)
        tol = (I.partials_rounding(nl) + 1e-6 * max(np.abs(ox).max(), np.abs(oy).max()))[sub]
        assert np.all(np.abs(g[f"{name}_gx"] - ox[sub]) <= tol)
        assert np.all(np.abs(g[f"{name}_gy"] - oy[sub]) <= tol)
        assert abs(hp - float(g[f"{name}_hpwl"])) <= 1e-6 * hp
        grid = oracle_lib.grid(W, H, M)
        q = oracle_lib.density_q(grid, x, y, nl["node_w"], nl["node_h"])
        mine, ref = (q / 2.0 ** 32).reshape(M, M), g[f"{name}_rho"]
        assert np.array_equal(mine != 0, ref != 0)
        assert np.abs(mine - ref).max() <= 2e-5 * max(1.0, np.abs(ref).max())
        zero = np.zeros_like(q)
        _, ab = oracle_lib.overflow(grid, q, zero, zero, 1.0, 1.0)
        assert abs(ab - float(g[f"{name}_overflow"])) <= 2e-5 * max(1.0, ab)
        ex, ey = I.field(M)
        fx, fy = oracle_lib.node_force(grid, x, y, nl["node_w"], nl["node_h"], ex.astype(np.float64),
                                       ey.astype(np.float64))
        mov = (nl["node_fixed"] == 0)[sub]
        scale = max(np.abs(fx).max(), np.abs(fy).max())
        assert np.abs(g[f"{name}_fx"][mov] - fx[sub][mov]).max() <= 1e-4 * scale
        assert np.abs(g[f"{name}_fy"][mov] - fy[sub][mov]).max() <= 1e-4 * scale
        if f"{name}_dct_ex" in g:
            # the host DCT path's field is the spectral solve of the area map
            # times M^2 / 8 (its transforms are unnormalised)
            mex, mey = oracle_lib.field_solve((q / 2.0 ** 32).reshape(M, M), M)
            for ref_e, e in ((g[f"{name}_dct_ex"], mex), (g[f"{name}_dct_ey"], mey)):
                k = M * M / 8.0 * np.asarray(e).reshape(M, M)
                assert np.abs(ref_e - k).max() <= 1e-5 * np.abs(ref_e).max()
