"""Inputs of the reference-Placer fixture (ref_placer.npz), rebuilt the same
way wherever they are needed: by make_golden.py, which runs the reference's
own Placer on them, and by the GPU test that compares the CUDA path with its
results.  Every value comes from exact arithmetic (integer patterns, float64
products and remainders), so the inputs are identical on every machine.

  netlist    the seeded synthetic netlist of a preset, seed 3, keeping the
             nets of degree 2..8 (Placer::computeAllPartials_CPU takes only
             those, AIEplace.cpp:585-588)
  positions  movable nodes on a Weyl sequence over the die (fixed nodes stay)
  field      integer patterns / 8 on the M x M bins (x-major, like getRho)
"""
from __future__ import annotations

import numpy as np

CASES = ("c0", "c1_small")
SEED = 3
GAMMA = 1.0
LEARNING_RATE = 1e-3
GLOBAL_LAMBDA = 1.0
MAX_DEGREE = 8
SUBSAMPLE = 4  # per-node results are kept for every 4th node


def small_nets(nl: dict) -> dict:
    ptr, pins = nl["net_ptr"], nl["pin_node"]
    deg = np.diff(ptr)
    keep = np.flatnonzero((deg >= 2) & (deg <= MAX_DEGREE))
    new_pins = np.concatenate([pins[ptr[e]:ptr[e + 1]] for e in keep]).astype(np.int32)
    new_ptr = np.concatenate([[0], np.cumsum(deg[keep])]).astype(np.int32)
    out = dict(nl)
    out["net_ptr"], out["pin_node"] = new_ptr, new_pins
    return out


def positions(nl: dict):
    n = len(nl["node_x"])
    W, H = float(nl["die"][2]), float(nl["die"][3])
    i = np.arange(n, dtype=np.float64)
    u = np.mod(i * 0.6180339887498949, 1.0)
    v = np.mod(i * 0.7548776662466927, 1.0)
    x, y = nl["node_x"].copy(), nl["node_y"].copy()
    mov = nl["node_fixed"] == 0
    x[mov] = (u[mov] * W).astype(np.float32)
    y[mov] = (v[mov] * H).astype(np.float32)
    return x, y


def field(m: int):
    c = np.arange(m, dtype=np.int64)[:, None]
    r = np.arange(m, dtype=np.int64)[None, :]
    ex = (((7 * c + 13 * r) % 17) - 8).astype(np.float32) / np.float32(8)
    ey = (((11 * c + 5 * r) % 19) - 9).astype(np.float32) / np.float32(8)
    return ex, ey


def partials_rounding(nl: dict) -> np.ndarray:
    """Per node, a bound on the reference partials' own rounding:
    computeNetPartials_CPU rounds (1 +- x/gamma) to float before it meets the
    net's double sums, up to 2^-24 (1 + |x|/gamma) per term, and a node sums
    one term per pin it has on these nets."""
    k = np.zeros(len(nl["node_x"]), np.int64)
    np.add.at(k, nl["pin_node"], 1)
    span = 1.0 + max(float(nl["die"][2]), float(nl["die"][3])) / GAMMA
    return 4 * 2.0 ** -24 * span * np.maximum(k, 1)
