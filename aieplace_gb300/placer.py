"""Host-side placer over the C ABI, shaped like the reference's Placer.

Method names follow vck5000/host/src/include/AIEplace.h:21-99 so code written
against the reference loop maps one to one:

  Placer(...)                        Placer::Placer            (AIEplace.cpp:87-138)
  initialize_placement(...)          Placer::initializePlacement (AIEplace.cpp:187-243)
  perform_iteration(n)               Placer::performIteration  (AIEplace.cpp:9-39)
  run()                              Placer::run               (AIEplace.cpp:44-76)
  compute_all_partials(x, y, gamma)  Placer::computeAllPartials_CPU (AIEplace.cpp:574-610)
  compute_overlaps(x, y)             Placer::computeOverlaps + Grid::getRho
  compute_electric_fields(rho)       Placer::computeElectricFields_* / FFT::doFFT
  hpwl(), overflow()                 DataBase::computeTotalWirelength, Grid::computeTotalOverflow

Every call goes to libaieplace_gb300.so on the GPU; errors raise APError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (AP_FIELD_BF16X3, AP_FIELD_FP32, BatchInfo, Netlist, Params, Stats, SurrogatePolicy, SurrogateStats, check,
                   lib, ptr)

SOLVERS = {"fp32": AP_FIELD_FP32, "bf16x3": AP_FIELD_BF16X3}


def default_params() -> Params:
    p = Params()
    check("ap_params_default", lib().ap_params_default(C.byref(p)))
    return p


class Placer:
    def __init__(self, netlist: dict, bins: int | None = None, target_density: float | None = None,
                 field_solver: str = "fp32", **overrides):
        p = default_params()
        p.bins_x = p.bins_y = int(bins if bins is not None else netlist.get("bins", 512))
        p.target_density = float(target_density if target_density is not None
                                 else netlist.get("target_density", 1.0))
        p.field_solver = SOLVERS[field_solver]
        for k, v in overrides.items():
            if not hasattr(p, k):
                raise KeyError(k)
            setattr(p, k, v)
        self.params = p
        self._arrays = {k: np.ascontiguousarray(netlist[k]) for k in
                        ("net_ptr", "pin_node", "node_w", "node_h", "node_x", "node_y", "node_fixed")}
        a = self._arrays
        die = np.asarray(netlist["die"], np.float32)
        self.num_nodes = len(a["node_w"])
        nl = Netlist(self.num_nodes, len(a["net_ptr"]) - 1, len(a["pin_node"]), ptr(a["net_ptr"]),
                     ptr(a["pin_node"]), ptr(a["node_w"]), ptr(a["node_h"]), ptr(a["node_x"]),
                     ptr(a["node_y"]), ptr(a["node_fixed"]), float(die[0]), float(die[1]),
                     float(die[2]), float(die[3]))
        h = C.c_void_p()
        check("ap_create", lib().ap_create(C.byref(nl), C.byref(p), C.byref(h)))
        self._h = h

    # ---- life cycle --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().ap_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- loop --------------------------------------------------------------
    def initialize_placement(self, x=None, y=None, seed: int | None = None, sigma: float = 1.0):
        if x is None:
            check("ap_init_seeded", lib().ap_init_seeded(self._h, int(seed or 0), float(sigma)))
        else:
            x = np.ascontiguousarray(x, np.float32)
            y = np.ascontiguousarray(y, np.float32)
            check("ap_init_positions", lib().ap_init_positions(self._h, ptr(x), ptr(y)))

    def perform_iteration(self, n: int = 1):
        check("ap_step", lib().ap_step(self._h, int(n)))

    def step_async(self, n_trials: int):
        """Enqueue n trial steps on the handle's stream; no host wait."""
        check("ap_step_async", lib().ap_step_async(self._h, int(n_trials)))

    def set_stream(self, stream_handle: int):
        check("ap_set_stream", lib().ap_set_stream(self._h, C.c_void_p(stream_handle)))

    def profile_stages(self, n_trials: int) -> list[float]:
        out = np.zeros(8, np.float32)
        n = C.c_int32()
        check("ap_profile_stages", lib().ap_profile_stages(self._h, int(n_trials), ptr(out), C.byref(n)))
        return [float(v) for v in out[: n.value]]

    def set_log(self, path: str | None, capacity: int = 65536):
        """Per-trial JSON-lines trajectory log (None stops it)."""
        check("ap_set_log", lib().ap_set_log(self._h, None if path is None else str(path).encode(), capacity))

    def solver_info(self) -> dict:
        tv, st = C.c_int32(), C.c_int32()
        tms, sms = np.zeros(5, np.float32), np.zeros(2, np.float32)
        check("ap_solver_info", lib().ap_solver_info(self._h, C.byref(tv), ptr(tms), C.byref(st), ptr(sms)))
        return {"tc_variant": tv.value, "tc_ms": [float(v) for v in tms], "simt_tile": st.value,
                "simt_ms": [float(v) for v in sms]}

    def run(self) -> int:
        done = C.c_int32()
        check("ap_run", lib().ap_run(self._h, C.byref(done)))
        return done.value

    def step_host(self, x_in, y_in, x_out, y_out) -> dict:
        s = Stats()
        check("ap_step_host", lib().ap_step_host(self._h, ptr(x_in), ptr(y_in), ptr(x_out), ptr(y_out),
                                                 C.byref(s)))
        return s.as_dict()

    def positions(self):
        x = np.zeros(self.num_nodes, np.float32)
        y = np.zeros(self.num_nodes, np.float32)
        check("ap_get_positions", lib().ap_get_positions(self._h, ptr(x), ptr(y)))
        return x, y

    def stats(self) -> dict:
        s = Stats()
        check("ap_get_stats", lib().ap_get_stats(self._h, C.byref(s)))
        return s.as_dict()

    def hpwl(self) -> float:
        v = C.c_double()
        check("ap_hpwl", lib().ap_hpwl(self._h, C.byref(v)))
        return v.value

    def overflow(self) -> tuple[float, float]:
        v, a = C.c_double(), C.c_double()
        check("ap_overflow", lib().ap_overflow(self._h, C.byref(v), C.byref(a)))
        return v.value, a.value

    # ---- per-stage entry points -------------------------------------------
    def compute_all_partials(self, x, y, gamma: float):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        gx = np.zeros(self.num_nodes, np.float32)
        gy = np.zeros(self.num_nodes, np.float32)
        wa, hp = C.c_double(), C.c_double()
        check("ap_wirelength_grad", lib().ap_wirelength_grad(self._h, ptr(x), ptr(y), float(gamma), ptr(gx),
                                                             ptr(gy), C.byref(wa), C.byref(hp)))
        return gx, gy, wa.value, hp.value

    def compute_overlaps(self, x, y) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        rho = np.zeros(self.params.bins_x * self.params.bins_y, np.int64)
        check("ap_density_map", lib().ap_density_map(self._h, ptr(x), ptr(y), ptr(rho)))
        return rho

    def compute_electric_fields(self, density, solver: str | None = None):
        d = np.ascontiguousarray(density, np.float32).reshape(-1)
        m = self.params.bins_x
        ex = np.zeros(m * m, np.float32)
        ey = np.zeros(m * m, np.float32)
        sv = -1 if solver is None else SOLVERS[solver]
        check("ap_field_solve", lib().ap_field_solve(self._h, ptr(d), ptr(ex), ptr(ey), sv))
        return ex, ey

    def compute_node_forces(self, x, y, ex, ey, gamma: float | None = None, lam: float | None = None):
        """nudgeNode's per-node force at (x, y) on the field maps (ex, ey),
        and, when gamma and lam are given, the preconditioned gradient
        (dWA - lam F) / max(1, pins + lam area / bin area).  Returns (fx, fy)
        or (fx, fy, gx, gy)."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        ex = np.ascontiguousarray(ex, np.float32).reshape(-1)
        ey = np.ascontiguousarray(ey, np.float32).reshape(-1)
        n = self.num_nodes
        fx, fy = np.zeros(n, np.float32), np.zeros(n, np.float32)
        grad = gamma is not None and lam is not None
        gx = np.zeros(n, np.float32) if grad else None
        gy = np.zeros(n, np.float32) if grad else None
        check("ap_node_force", lib().ap_node_force(
            self._h, ptr(x), ptr(y), ptr(ex), ptr(ey), float(gamma or 0.0), float(lam or 0.0), ptr(fx), ptr(fy),
            ptr(gx) if grad else None, ptr(gy) if grad else None))
        return (fx, fy, gx, gy) if grad else (fx, fy)

    # ---- learned surrogate (no counterpart in the reference) ---------------
    def attach_surrogate(self, surrogate, overflow_min: float = 0.3, judge_every: int = 8,
                         max_error: float = 0.02, use_net: bool = True):
        """The loop takes its field from `surrogate` while the overflow exceeds
        overflow_min; every judge_every-th trial the exact solve runs too and
        the surrogate is dropped until the next judgement if its relative
        field error exceeds max_error.  surrogate=None detaches."""
        self._surrogate = surrogate  # keep it alive while attached
        pol = SurrogatePolicy(float(overflow_min), int(judge_every), float(max_error), int(bool(use_net)))
        sh = None if surrogate is None else surrogate._h
        check("ap_attach_surrogate", lib().ap_attach_surrogate(self._h, sh, C.byref(pol)))

    def surrogate_stats(self) -> dict:
        s = SurrogateStats()
        check("ap_surrogate_get_stats", lib().ap_surrogate_get_stats(self._h, C.byref(s)))
        return {"used": s.used, "judged": s.judged, "fallbacks": s.fallbacks, "last_error": s.last_error}

    # ---- checkpoint / resume ----------------------------------------------
    def snapshot(self) -> bytes:
        n = C.c_size_t()
        check("ap_snapshot_size", lib().ap_snapshot_size(self._h, C.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        check("ap_snapshot", lib().ap_snapshot(self._h, ptr(buf), n.value))
        return buf.tobytes()

    def restore(self, blob: bytes):
        buf = np.frombuffer(blob, np.uint8).copy()
        check("ap_restore", lib().ap_restore(self._h, ptr(buf), len(buf)))


class BatchPlacer:
    """Independent placements stepped together (ap_create_batch): one CUDA
    graph launch advances one trial step of every active instance, as nine
    persistent launches over all instances ("persistent", the default where
    it serves every instance) or as every instance's own launches in
    parallel branches ("graph")."""

    def __init__(self, netlists: list[dict], field_solver: str = "fp32", **overrides):
        n = len(netlists)
        self._keep = []
        nls = (Netlist * n)()
        prms = (Params * n)()
        self.sizes = []
        for i, nl in enumerate(netlists):
            p = default_params()
            p.bins_x = p.bins_y = int(nl["bins"])
            p.target_density = float(nl["target_density"])
            p.field_solver = SOLVERS[field_solver]
            for k, v in overrides.items():
                setattr(p, k, v)
            prms[i] = p
            a = {k: np.ascontiguousarray(nl[k]) for k in
                 ("net_ptr", "pin_node", "node_w", "node_h", "node_x", "node_y", "node_fixed")}
            self._keep.append(a)
            die = np.asarray(nl["die"], np.float32)
            nls[i] = Netlist(len(a["node_w"]), len(a["net_ptr"]) - 1, len(a["pin_node"]), ptr(a["net_ptr"]),
                             ptr(a["pin_node"]), ptr(a["node_w"]), ptr(a["node_h"]), ptr(a["node_x"]),
                             ptr(a["node_y"]), ptr(a["node_fixed"]), float(die[0]), float(die[1]),
                             float(die[2]), float(die[3]))
            self.sizes.append(len(a["node_w"]))
        h = C.c_void_p()
        check("ap_create_batch", lib().ap_create_batch(n, C.cast(nls, C.c_void_p), C.cast(prms, C.c_void_p),
                                                       C.byref(h)))
        self._h = h
        self.n = n

    def close(self):
        if getattr(self, "_h", None):
            lib().ap_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def initialize_placement(self, seed: int = 0, sigma: float = 1.0):
        check("ap_batch_init_seeded", lib().ap_batch_init_seeded(self._h, int(seed), float(sigma)))

    def step(self, n_trials: int):
        check("ap_batch_step", lib().ap_batch_step(self._h, int(n_trials)))

    def run(self) -> list[int]:
        it = np.zeros(self.n, np.int32)
        check("ap_batch_run", lib().ap_batch_run(self._h, ptr(it)))
        return [int(v) for v in it]

    def stats(self, i: int) -> dict:
        s = Stats()
        check("ap_batch_get_stats", lib().ap_batch_get_stats(self._h, int(i), C.byref(s)))
        return s.as_dict()

    def positions(self, i: int):
        x = np.zeros(self.sizes[i], np.float32)
        y = np.zeros(self.sizes[i], np.float32)
        check("ap_batch_get_positions", lib().ap_batch_get_positions(self._h, int(i), ptr(x), ptr(y)))
        return x, y

    def set_form(self, form: str):
        check("ap_batch_set_form", lib().ap_batch_set_form(self._h, {"graph": 0, "persistent": 1}[form]))

    def set_item_blocks(self, blocks: int):
        check("ap_batch_set_item_blocks", lib().ap_batch_set_item_blocks(self._h, int(blocks)))

    def profile(self, n_trials: int = 10) -> dict:
        """Mean ms per persistent launch over n_trials eager trial steps
        (they advance the instances)."""
        ms = np.zeros(6, np.float32)
        check("ap_batch_profile", lib().ap_batch_profile(self._h, int(n_trials), ptr(ms)))
        return dict(zip(("update", "scatter", "rho", "wa", "field", "gather"), [float(v) for v in ms]))

    def info(self) -> dict:
        b = BatchInfo()
        check("ap_batch_get_info", lib().ap_batch_get_info(self._h, C.byref(b)))
        return b.as_dict()
