"""Run configuration (ap_run_config_read), the command-line placer
(aieplace_gb300/aieplace), filler cells and the per-trial trajectory log.

CPU: the reference's config keys map as the header states; this placer's
keys; unknown or ill-typed keys are errors that name the key.
GPU: the command-line placer runs a LEF/DEF design directory end to end
(config -> read -> place -> placed DEF + JSONL log); filler cells take the
white space without entering the overflow (the loop's overflow equals the
oracle's of the real cells at the same positions, bit for bit); the
trajectory log holds one record per trial, consistent with the readout.
"""
import ctypes as C
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO

FIX = os.path.join(REPO, "tests", "golden", "lefdef")


@pytest.fixture(scope="module")
def ap():
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300

    return aieplace_gb300


def read_config(path):
    from aieplace_gb300._lib import Params, RunConfig, lib

    p, r = Params(), RunConfig()
    st = lib().ap_run_config_read(str(path).encode(), C.byref(p), C.byref(r))
    return st, p, r, lib().ap_last_error().decode()


def test_reference_keys(ap, tmp_path):
    cfg = {"params": {"use_aie": True, "input_filepath": "designs/blockA", "output_filepath": "out",
                      "wirelength_method": "WA", "bins_per_row": 64, "gamma": 3.5, "max_iterations": 250,
                      "init_learning_rate": 0.05, "init_global_lambda": 0.0}}
    f = tmp_path / "c.json"
    f.write_text(json.dumps(cfg, indent=2))
    st, p, r, _ = read_config(f)
    assert st == 0
    assert (p.bins_x, p.bins_y, p.max_iterations) == (64, 64, 250)
    assert p.gamma_base_bins == np.float32(3.5)
    assert p.init_density_weight == np.float32(8e-5)  # 0 keeps the default
    assert r.input_dir == b"designs/blockA" and r.output_dir == b"out"
    assert r.wirelength_method == 1 and r.use_aie == 1
    assert r.ignored_learning_rate == np.float32(0.05)
    cfg["params"]["init_global_lambda"] = 2e-4
    f.write_text(json.dumps(cfg))
    st, p, _, _ = read_config(f)
    assert st == 0 and p.init_density_weight == np.float32(2e-4)


def test_placer_keys_at_top_level(ap, tmp_path):
    cfg = {"bins_per_row": 256, "target_density": 0.75, "field_solver": "bf16x3", "target_overflow": 0.08,
           "restart_mode": 3, "max_backtracks": 2, "filler_cells": True, "log_path": "t.jsonl", "seed": 9,
           "init_sigma": 2.5, "lef_size_mode": "as_read", "check_interval": 4}
    f = tmp_path / "c.json"
    f.write_text(json.dumps(cfg))
    st, p, r, _ = read_config(f)
    assert st == 0
    assert p.bins_x == 256 and p.target_density == np.float32(0.75) and p.field_solver == 1
    assert p.target_overflow == np.float32(0.08) and p.restart_mode == 3 and p.max_backtracks == 2
    assert p.check_interval == 4
    assert r.filler_cells == 1 and r.log_path == b"t.jsonl" and r.seed == 9 and r.size_mode == 1
    assert r.init_sigma == np.float32(2.5)


@pytest.mark.parametrize("body,needle", [
    ('{"params": {"bins_per_rows": 32}}', 'unknown key "bins_per_rows"'),
    ('{"params": {"gamma": "four"}}', 'key "gamma"'),
    ('{"params": {"field_solver": "fp64"}}', 'key "field_solver"'),
    ('{"params": {"bins_per_row": 32.5}}', 'key "bins_per_row"'),
    ('{"params": {"bins_per_row": 32,}}', "line 1"),
    ('[1, 2]', "not a JSON object"),
])
def test_bad_configs_name_the_problem(ap, tmp_path, body, needle):
    f = tmp_path / "c.json"
    f.write_text(body)
    st, _, _, msg = read_config(f)
    assert st == 1 and needle in msg, msg


@pytest.mark.gpu
def test_command_line_placer_end_to_end(ap, tmp_path):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    design = tmp_path / "design"
    design.mkdir()
    for f in ("tech.lef", "cells.lef", "floorplan.def"):
        shutil.copy(os.path.join(FIX, f), design / f)
    out = tmp_path / "out"
    out.mkdir()
    log = tmp_path / "trajectory.jsonl"
    cfg = {"params": {"use_aie": False, "input_filepath": str(design), "output_filepath": str(out),
                      "wirelength_method": "HPWL", "bins_per_row": 32, "gamma": 4, "max_iterations": 300,
                      "init_learning_rate": 0.02, "init_global_lambda": 0.0, "target_density": 0.9,
                      "log_path": str(log), "seed": 5}}
    (tmp_path / "config.json").write_text(json.dumps(cfg))
    exe = os.path.join(REPO, "aieplace_gb300", "aieplace")
    r = subprocess.run([exe, str(tmp_path / "config.json")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["design"] == "tiny_core" and res["status"] == 0 and res["nodes"] == 16
    assert res["def"] == str(out / "tiny_core.def") and os.path.exists(res["def"])
    with ap.Design.read([os.path.join(FIX, "tech.lef"), os.path.join(FIX, "cells.lef")], res["def"]) as d:
        nl = d.netlist()
    assert np.isfinite(nl["node_x"]).all()
    recs = [json.loads(line) for line in open(log)]
    assert len(recs) == res["evals"] and recs[-1]["iteration"] == res["iterations"]
    assert recs[-1]["hpwl"] == res["hpwl"]


@pytest.mark.gpu
def test_trajectory_log_one_record_per_trial(ap, tmp_path):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    nl = ap.synth.generate("c0", seed=1)
    log = tmp_path / "t.jsonl"
    with ap.Placer(nl, bins=32, check_interval=8) as pl:
        pl.set_log(str(log), capacity=64)  # before the initial placement: installed by it
        pl.initialize_placement(nl["node_x"], nl["node_y"])
        pl.perform_iteration(30)
        pl.run()
        s = pl.stats()
        pl.set_log(None)
    recs = [json.loads(line) for line in open(log)]
    assert len(recs) == s["evals"]
    assert [r["eval"] for r in recs] == list(range(s["evals"]))
    assert all(r["accepted"] is True and r["field"] == "exact" for r in recs)
    assert [r["iteration"] for r in recs] == list(range(1, s["evals"] + 1))
    assert recs[-1]["hpwl"] == s["hpwl"] and recs[-1]["overflow"] == s["overflow"]
    t = [r["t_ms"] for r in recs]
    assert t[0] == 0.0 and all(b >= a for a, b in zip(t, t[1:]))
    # a ring smaller than the trials between two reads loses the oldest and says so
    log2 = tmp_path / "t2.jsonl"
    with ap.Placer(nl, bins=32) as pl:
        pl.initialize_placement(nl["node_x"], nl["node_y"])
        pl.set_log(str(log2), capacity=8)
        pl.step_async(20)
        s = pl.stats()
    lines = [json.loads(line) for line in open(log2)]
    assert lines[0] == {"lost_trials": 12} and len(lines) == 9 and lines[-1]["eval"] == 19


@pytest.mark.gpu
def test_filler_cells_take_white_space_not_overflow(ap, oracle_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aieplace_gb300._lib import lib

    nl = ap.synth.generate("c1_small", seed=6)
    with ap.Placer(nl, bins=128, target_density=0.7, filler_cells=1, max_iterations=3000) as pl:
        n, fw, fh = C.c_int32(), C.c_float(), C.c_float()
        assert lib().ap_get_fillers(pl._h, C.byref(n), C.byref(fw), C.byref(fh)) == 0
        W, H = float(nl["die"][2]), float(nl["die"][3])
        mov = nl["node_fixed"] == 0
        a_mov = float((nl["node_w"][mov].astype(np.float64) * nl["node_h"][mov]).sum())
        fixed = ~mov
        a_fix = float((nl["node_w"][fixed].astype(np.float64) * nl["node_h"][fixed]).sum())
        want = 0.7 * (W * H - a_fix) - a_mov
        assert n.value > 0 and abs(n.value * fw.value * fh.value - want) <= fw.value * fh.value + 1e-6 * want
        pl.initialize_placement(seed=6, sigma=1.0)
        pl.run()
        s = pl.stats()
        x, y = pl.positions()
    assert len(x) == len(nl["node_w"])  # fillers stay internal
    assert s["status"] == 0 and s["overflow"] < 0.10
    # the overflow of the real cells alone, computed by the oracle at the
    # loop's final positions, is the loop's own readout bit for bit
    g = oracle_lib.grid(W, H, 128)
    area = (nl["node_w"] * nl["node_h"]) > 0
    mov_q = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], (mov & area).astype(np.uint8))
    fix_q = oracle_lib.density_q(g, x, y, nl["node_w"], nl["node_h"], (fixed & area).astype(np.uint8))
    rt = float(np.float32(0.7))
    wq = np.rint(nl["node_w"][mov] * np.float32(65536.0)).astype(np.int64)
    hq = np.rint(nl["node_h"][mov] * np.float32(65536.0)).astype(np.int64)
    area_q = np.cumsum((wq * hq).astype(np.float64))[-1]
    tau, tau_abs = oracle_lib.overflow(g, mov_q, fix_q, oracle_lib.scale_fixed(fix_q, rt), rt, area_q)
    assert s["overflow"] == tau and s["overflow_abs"] == tau_abs
