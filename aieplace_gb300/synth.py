"""Seeded synthetic netlists (the generator lives in the C library).

Presets (presets.py) mirror the workload shapes the placer is measured on.
Units: one site wide = one row high = 1.0.  Macro areas are drawn from
U[20, 200] site^2 with aspect ratio in [0.5, 2].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SynthConfig, check, lib, ptr
from .presets import PRESETS


def batch_specs(n: int = 64, seed: int = 1, lo: int = 5_000, hi: int = 150_000) -> list[dict]:
    """The batched workload: cell counts LogUniform[lo, hi], the c1 net and
    macro statistics, bins the power of two at or above sqrt(cells / 4) clamped to
    [128, 512], target density 0.7."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        cells = int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))
        bins = int(2 ** np.ceil(np.log2(np.sqrt(cells / 4.0))))
        bins = min(512, max(128, bins))
        specs.append(dict(num_cells=cells, num_nets=int(round(1.05 * cells)), num_macros=max(1, cells // 50),
                          num_pads=0, unit_cells=0, degree_mix=1, locality=0.8, window=64, target_density=0.7,
                          die_side=0.0, bins=bins))
    return specs


def generate(preset: str | dict, seed: int = 1) -> dict:
    """Returns a dict of numpy arrays: net_ptr, pin_node, node_w/h/x/y, node_fixed,
    die (xl, yl, xh, yh), plus 'bins' and 'target_density' of the preset."""
    spec = dict(PRESETS[preset]) if isinstance(preset, str) else dict(preset)
    bins = spec.pop("bins")
    cfg = SynthConfig(spec["num_cells"], spec["num_nets"], spec["num_macros"], spec["num_pads"],
                      spec["unit_cells"], spec["degree_mix"], spec["locality"], spec["window"],
                      spec.get("macro_area_min", 20.0), spec.get("macro_area_max", 200.0),
                      spec["target_density"], spec["die_side"], seed)
    nn, ne, npins = C.c_int32(), C.c_int32(), C.c_int32()
    check("ap_synth_counts", lib().ap_synth_counts(C.byref(cfg), C.byref(nn), C.byref(ne), C.byref(npins)))
    out = {
        "net_ptr": np.zeros(ne.value + 1, np.int32),
        "pin_node": np.zeros(max(npins.value, 1), np.int32)[: npins.value],
        "node_w": np.zeros(nn.value, np.float32),
        "node_h": np.zeros(nn.value, np.float32),
        "node_x": np.zeros(nn.value, np.float32),
        "node_y": np.zeros(nn.value, np.float32),
        "node_fixed": np.zeros(nn.value, np.uint8),
        "die": np.zeros(4, np.float32),
    }
    check("ap_synth_generate", lib().ap_synth_generate(
        C.byref(cfg), ptr(out["net_ptr"]), ptr(out["pin_node"]), ptr(out["node_w"]), ptr(out["node_h"]),
        ptr(out["node_x"]), ptr(out["node_y"]), ptr(out["node_fixed"]), ptr(out["die"])))
    out["bins"] = bins
    out["target_density"] = spec["target_density"]
    out["seed"] = seed
    return out
