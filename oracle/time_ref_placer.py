"""Times the reference placer's own CPU functions on the seeded synthetic
netlists (c0, c1, c2 of aieplace_gb300/presets.py), single-threaded as the
reference runs them.

TEST INFRASTRUCTURE ONLY: needs oracle/_ref/libref_placer.so (and
libref_placer_O0.so for --opt O0, libref.so for the Ooura field solve), built
from a reference checkout by `make -C oracle REF=<checkout> ref refplacer
refplacer-O0`.  Prints one JSON object per configuration.

What is timed (vck5000/host/src/AIEplace.cpp):
  partials      Placer::computeAllPartials_CPU (:574-673), nets of degree 2..8
  overlaps      Placer::computeOverlaps (:937-967)
  nudge         Placer::nudgeAllNodes (:993-1046)
  field_naive   Placer::computeElectricFields_CPU (:679-750), the field solve
                of the CPU loop as shipped, O(M^4): timed at c0, extrapolated
                by (M/32)^4 elsewhere
  field_dct     compute_a_uv_DCT + compute_eField_DCT (:752-934), the host's
                DCT path (O(M^3) naive transforms): timed at c0
  field_ooura   the RePlAce/Ooura spectral solve the reference ships
                (python/AIEmath/fft_replace, FFT::doFFT through fft.cpp), the
                fastest field solve in the reference, timed at every size
  loop          at c0 only: passes of Placer::run's loop body (performIteration
                with its CPU branches, the learning-rate and lambda schedule)
The per-iteration sum with the Ooura solve is the reference's fastest CPU
iteration; with the naive solve it is the loop as shipped.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, this folder would shadow the oracle package with oracle.py
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, os.path.dirname(HERE))

try:
    from oracle import oracle as O  # noqa: E402  (oracle/ as a package, from the repository root)
except ImportError:
    import oracle as O  # noqa: E402  (oracle/ itself on the path, as the tests have it)
from aieplace_gb300.presets import PRESETS  # noqa: E402


def best_of(fn, reps: int) -> float:
    return min(fn() for _ in range(reps))


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def time_config(name: str, opt: str, seed: int, reps: int, loop_iters: int) -> dict:
    nl = O.synth_generate(PRESETS[name], seed=seed)
    n, die, M = len(nl["node_x"]), nl["die"], nl["bins"]
    x, y = nl["node_x"].copy(), nl["node_y"].copy()
    out = {"config": name, "opt": opt, "seed": seed, "nodes": n, "nets": len(nl["net_ptr"]) - 1, "bins": M,
           "threads": 1, "cpu": cpu_model()}
    t0 = time.perf_counter()
    with O.quiet_stdout():
        rp = O.RefPlacer(nl["net_ptr"], nl["pin_node"], nl["node_w"], nl["node_h"], x, y, nl["node_fixed"],
                         float(die[2]), float(die[3]), M, gamma=1.0, learning_rate=1e-3, global_lambda=1.0,
                         opt=opt)
        out["create_s"] = time.perf_counter() - t0
        out["partials_s"] = best_of(lambda: rp.partials()[2], reps)
        out["overlaps_s"] = best_of(lambda: rp.overlaps()[2], reps)
        rho, _, _ = rp.overlaps()
        ex = np.zeros((M, M), np.float32)
        zero = np.zeros(n, np.float32)
        out["nudge_s"] = best_of(lambda: rp.nudge(ex, ex, zero, zero)[2], reps)
        if M <= 32:
            out["field_naive_s"] = best_of(lambda: rp.fields_naive()[2], reps)
            out["field_dct_s"] = best_of(lambda: rp.fields_dct()[2], reps)
        else:
            c0 = PRESETS["c0"]["bins"]
            out["field_naive_s"] = None
            out["field_naive_extrapolated_s"] = None  # filled by the caller from c0
            out["field_naive_scale_from_c0"] = (M / c0) ** 4
        if name == "c0" and loop_iters > 0:
            h0 = rp.hpwl()
            out["loop_iters"] = loop_iters
            out["loop_s"] = rp.iterate(loop_iters)
            out["loop_hpwl_start"] = h0
            out["loop_hpwl_end"] = rp.hpwl()
            out["loop_overflow_end"] = rp.overlaps()[1]
    R = O.ref_lib()
    if R is not None:
        d = (rho / float(die[2] * die[3] / (M * M))).astype(np.float32).reshape(-1)

        def ooura():
            e1, e2 = np.zeros(M * M, np.float32), np.zeros(M * M, np.float32)
            dd = d.copy()
            t = time.perf_counter()
            R.ref_replace_field(M, dd, None, e1, e2)
            return time.perf_counter() - t

        out["field_ooura_s"] = best_of(ooura, reps)
    rp.close()
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--configs", default="c0,c1,c2")
    ap.add_argument("--opt", default="O2", choices=("O2", "O0"))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--loop-iters", type=int, default=20)
    a = ap.parse_args(argv)
    if O.ref_placer_lib(a.opt) is None:
        print(json.dumps({"unavailable": f"oracle/_ref/libref_placer{'' if a.opt == 'O2' else '_' + a.opt}.so "
                                         "not built (needs the reference checkout)"}))
        return 0
    naive_c0 = None
    for name in a.configs.split(","):
        r = time_config(name, a.opt, a.seed, a.reps, a.loop_iters)
        if r.get("field_naive_s") is not None and r["bins"] == PRESETS["c0"]["bins"]:
            naive_c0 = r["field_naive_s"]
        if r.get("field_naive_s") is None and naive_c0 is not None:
            r["field_naive_extrapolated_s"] = naive_c0 * r["field_naive_scale_from_c0"]
        base = r["partials_s"] + r["overlaps_s"] + r["nudge_s"]
        if r.get("field_ooura_s") is not None:
            r["iter_fastest_s"] = base + r["field_ooura_s"]
            r["iters_per_s_fastest"] = 1.0 / r["iter_fastest_s"]
        naive = r.get("field_naive_s") or r.get("field_naive_extrapolated_s")
        if naive is not None:
            r["iter_as_shipped_s"] = base + naive
            r["iters_per_s_as_shipped"] = 1.0 / r["iter_as_shipped_s"]
        if "loop_s" in r:
            r["loop_iters_per_s"] = r["loop_iters"] / r["loop_s"]
        print(json.dumps(r), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
