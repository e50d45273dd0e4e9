"""The oracle against the reference's own Placer (vck5000/host/src/AIEplace.cpp)
built for the CPU by oracle/Makefile (refplacer) on the seeded netlists.

These tests run where the reference checkout was present at build time
(oracle/_ref/libref_placer.so exists) and skip elsewhere.  They pin, live:
  * Placer::computeAllPartials_CPU (AIEplace.cpp:574-673) against the oracle's
    WA gradient over nets of degree 2..8;
  * Placer::computeOverlaps (:937-967) and Grid::computeTotalOverflow
    (Grid.cpp:144-151) against the oracle's density map and overflow;
  * Placer::nudgeNode (:1004-1046) against the oracle's node force;
  * DataBase::computeTotalWirelength("HPWL") against the oracle's HPWL;
  * the host DCT field path (compute_a_uv_DCT / compute_eField_DCT,
    :752-934) against the oracle's spectral solve: the same field up to the
    constant M^2/8 of the reference's unnormalised transforms;
  * Placer::run's loop body (:55-76, performIteration :9-40) with use_aie
    false: one pass moves every component by learning_rate min(W, H)
    global_lambda F alone -- nudgeNode reads partials_aie, which
    iterationReset zeroes and only the accelerator path writes, so the CPU
    loop as shipped leaves the wirelength gradient out.
"""
import numpy as np
import pytest

import oracle as O
from aieplace_gb300.presets import PRESETS

pytestmark = pytest.mark.skipif(O.ref_placer_lib() is None,
                                reason="reference placer library not built on this host")

LR, LAMBDA, GAMMA = 1e-3, 1.0, 1.0


def _netlist(name, seed=3, spread=True):
    nl = O.synth_generate(PRESETS[name], seed=seed)
    n, die = len(nl["node_x"]), nl["die"]
    x, y = nl["node_x"].copy(), nl["node_y"].copy()
    if spread:  # uniform positions over the die for the movable nodes
        rng = np.random.default_rng(seed)
        mov = ~nl["node_fixed"].astype(bool)
        x[mov] = (die[2] * rng.random(mov.sum())).astype(np.float32)
        y[mov] = (die[3] * rng.random(mov.sum())).astype(np.float32)
    return nl, n, die, x, y


def _placer(nl, die, x, y, gamma=GAMMA):
    with O.quiet_stdout():
        return O.RefPlacer(nl["net_ptr"], nl["pin_node"], nl["node_w"], nl["node_h"], x, y, nl["node_fixed"],
                           float(die[2]), float(die[3]), nl["bins"], gamma=gamma, learning_rate=LR,
                           global_lambda=LAMBDA)


def _components(nl):
    """The nodes the reference keeps as components (pads become IO pins)."""
    return ~(nl["node_fixed"].astype(bool) & (nl["node_w"] * nl["node_h"] == 0))


@pytest.fixture(scope="module", params=["c0", "c1_small"])
def case(request):
    nl, n, die, x, y = _netlist(request.param)
    rp = _placer(nl, die, x, y)
    yield request.param, nl, n, die, x, y, rp
    rp.close()


@pytest.mark.parametrize("gamma", [1.0, 4.0])
def test_partials_match_oracle_wa_gradient(gamma):
    """computeAllPartials_CPU: float node positions, the net's b/c sums in
    double, each node's term and its sum in float.  (1 + x/gamma) is rounded
    to float before it meets the double sums, so each net term carries up to
    about 2^-24 (1 + |x|/gamma) of absolute error; a node collects that once
    per net of degree 2..8 it is on."""
    nl, n, die, x, y = _netlist("c1_small")
    rp = _placer(nl, die, x, y, gamma=gamma)
    with O.quiet_stdout():
        gx, gy, _ = rp.partials()
    rp.close()
    ox, oy, _, _ = O.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, gamma, min_deg=2, max_deg=8)
    deg = np.diff(nl["net_ptr"])
    k = np.zeros(n)
    for e in np.nonzero((deg >= 2) & (deg <= 8))[0]:
        k[nl["pin_node"][nl["net_ptr"][e]:nl["net_ptr"][e + 1]]] += 1
    span = 1.0 + max(float(die[2]), float(die[3])) / gamma
    tol = 4 * 2.0 ** -24 * span * np.maximum(k, 1) + 1e-6 * max(np.abs(ox).max(), np.abs(oy).max())
    assert np.all(np.abs(gx - ox) <= tol)
    assert np.all(np.abs(gy - oy) <= tol)
    # nodes on no net of degree 2..8 get nothing from either side
    assert np.all(gx[k == 0] == 0) and np.all(ox[k == 0] == 0)


def test_overlaps_and_overflow_match_oracle(case):
    name, nl, n, die, x, y, rp = case
    with O.quiet_stdout():
        rho, ovf, _ = rp.overlaps()
    g = O.grid(float(die[2]), float(die[3]), nl["bins"])
    q = O.density_q(g, x, y, nl["node_w"], nl["node_h"])
    mine = (q / 2.0 ** 32).reshape(rho.shape)
    # the same bins touched; areas within the reference's float accumulation
    assert np.array_equal(mine != 0, rho != 0)
    assert np.abs(mine - rho).max() <= 2e-5 * max(1.0, np.abs(rho).max())
    zero = np.zeros_like(q)
    _, ab = O.overflow(g, q, zero, zero, 1.0, 1.0)
    assert abs(ab - ovf) <= 2e-5 * max(1.0, ab)


def test_hpwl_matches_oracle(case):
    name, nl, n, die, x, y, rp = case
    _, _, _, hp = O.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, GAMMA)
    assert abs(rp.hpwl() - hp) <= 1e-6 * hp


@pytest.mark.parametrize("with_partials", [False, True])
def test_nudge_matches_oracle_node_force(case, with_partials):
    """nudgeNode's move is learning_rate min(W, H) (global_lambda F - p), F the
    overlap-weighted bin field; the reference moves only components."""
    name, nl, n, die, x, y, rp = case
    M = nl["bins"]
    rng = np.random.default_rng(7)
    ex = rng.standard_normal((M, M)).astype(np.float32)
    ey = rng.standard_normal((M, M)).astype(np.float32)
    if with_partials:
        px, py = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    else:
        px = py = np.zeros(n, np.float32)
    with O.quiet_stdout():
        mx, my, _ = rp.nudge(ex, ey, px, py)
    g = O.grid(float(die[2]), float(die[3]), M)
    fx, fy = O.node_force(g, x, y, nl["node_w"], nl["node_h"], ex.astype(np.float64), ey.astype(np.float64))
    coeff = LR * min(float(die[2]), float(die[3]))
    wx, wy = coeff * (LAMBDA * fx - px), coeff * (LAMBDA * fy - py)
    comp = _components(nl)
    scale = max(np.abs(wx).max(), np.abs(wy).max())
    assert np.abs(mx[comp] - wx[comp]).max() <= 1e-4 * scale
    assert np.abs(my[comp] - wy[comp]).max() <= 1e-4 * scale
    assert np.all(mx[~comp] == 0) and np.all(my[~comp] == 0)


def test_host_dct_field_is_oracle_field_times_m2_over_8():
    nl, n, die, x, y = _netlist("c0")
    rp = _placer(nl, die, x, y)
    with O.quiet_stdout():
        rho, _, _ = rp.overlaps()
        ex, ey, _ = rp.fields_dct()
    rp.close()
    M = nl["bins"]
    mex, mey = O.field_solve(rho.astype(np.float64), M)
    k = M * M / 8.0
    for ref, mine in ((ex, mex), (ey, mey)):
        mine = np.asarray(mine).reshape(M, M)
        assert np.abs(ref - k * mine).max() <= 1e-5 * np.abs(ref).max()


def test_cpu_loop_moves_by_density_force_alone():
    nl, n, die, x, y = _netlist("c0")
    rp = _placer(nl, die, x, y)
    M = nl["bins"]
    with O.quiet_stdout():
        ex, ey, _ = rp.fields_naive()  # the loop's own field at the start positions
        rp.iterate(1)                  # iteration 0: learning rate x0.8, lambda x1.01
        x1, y1 = rp.positions()
    rp.close()
    g = O.grid(float(die[2]), float(die[3]), M)
    fx, fy = O.node_force(g, x, y, nl["node_w"], nl["node_h"], ex.astype(np.float64), ey.astype(np.float64))
    coeff = np.float32(LR * 0.8) * min(float(die[2]), float(die[3])) * np.float32(LAMBDA * 1.01)
    comp = _components(nl)
    dx, dy = (x1 - x)[comp], (y1 - y)[comp]
    scale = coeff * max(np.abs(fx).max(), np.abs(fy).max())
    assert np.abs(dx - coeff * fx[comp]).max() <= 1e-3 * scale
    assert np.abs(dy - coeff * fy[comp]).max() <= 1e-3 * scale
    # a wirelength term in the move would have been far outside that
    # tolerance: from these positions it is larger than the density move
    wx, wy, _, _ = O.wa_grad(nl["net_ptr"], nl["pin_node"], x, y, GAMMA, min_deg=2, max_deg=8)
    assert LR * 0.8 * min(float(die[2]), float(die[3])) * np.abs(wx[comp]).max() > scale


def test_timing_script_runs_at_c0(capsys):
    """oracle/time_ref_placer.py (the reference's CPU functions timed) on the
    576-cell case: one JSON object with every function's time."""
    import json
    import os
    import sys

    sys.path.insert(0, os.path.dirname(O.__file__))
    import time_ref_placer

    assert time_ref_placer.main(["--configs", "c0", "--reps", "1", "--loop-iters", "2"]) == 0
    r = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert r["config"] == "c0" and r["threads"] == 1
    for k in ("partials_s", "overlaps_s", "nudge_s", "field_naive_s", "field_dct_s", "loop_s"):
        assert r[k] > 0.0
    assert r["iters_per_s_as_shipped"] > 0.0
