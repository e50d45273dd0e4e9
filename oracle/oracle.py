"""ctypes front end of the CPU oracle (liboracle.so) and of the reference's own
CPU code (_ref/libref.so, present only where the reference checkout was
available at build time).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py as the checker or the timed CPU baseline.  The product
path (aieplace_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SYNTH_PATH = os.path.join(HERE, "libsynth.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")
REF_PLACER_PATH = os.path.join(HERE, "_ref", "libref_placer.so")
# the reference checkout, where one exists: AP_REFERENCE_DIR, or the
# `ref_dir` argument of build(); there is no default location
REF_SRC = os.environ.get("AP_REFERENCE_DIR", "")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(with_ref: bool | None = None, ref_dir: str | None = None) -> None:
    """Compile liboracle.so and libsynth.so, and _ref/libref.so and
    _ref/libref_placer.so when a reference checkout is named (ref_dir, else
    AP_REFERENCE_DIR) and exists."""
    global REF_SRC
    if ref_dir:
        REF_SRC = ref_dir
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so", "libsynth.so"], check=True)
    if with_ref is None:
        with_ref = bool(REF_SRC) and os.path.isdir(REF_SRC)
    if with_ref:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, f"REF={REF_SRC}", "ref"], check=True)
        # the reference's Placer (test infrastructure for its CPU loop): a
        # failure here leaves only the tests that need it skipped
        r = subprocess.run(["make", "-s", "-j8", "-C", HERE, f"REF={REF_SRC}", "refplacer"])
        if r.returncode != 0:
            print("oracle: the reference placer library did not build; its tests will skip")


class OrGrid(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("die_w", C.c_float), ("die_h", C.c_float),
                ("bw", C.c_float), ("bh", C.c_float), ("small_threshold", C.c_float),
                ("bw_q", C.c_int64), ("bh_q", C.c_int64)]


class OrParams(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("target_density", C.c_double),
                ("gamma_base_bins", C.c_double), ("init_density_weight", C.c_double),
                ("ref_delta_hpwl", C.c_double), ("mu_max", C.c_double), ("mu_min", C.c_double),
                ("init_step_coef", C.c_double), ("restart", C.c_int), ("max_backtracks", C.c_int)]


class OrStats(C.Structure):
    _fields_ = [("iteration", C.c_int), ("hpwl", C.c_double), ("wa", C.c_double),
                ("overflow", C.c_double), ("overflow_abs", C.c_double), ("lambda_", C.c_double),
                ("gamma", C.c_double), ("alpha", C.c_double), ("a_k", C.c_double),
                ("evals", C.c_int), ("norm_wl", C.c_double), ("norm_f", C.c_double),
                ("restarts", C.c_int)]


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        L = C.CDLL(LIB_PATH)
        L.or_fast_exp.restype = C.c_double
        L.or_fast_exp.argtypes = [C.c_double, C.c_int]
        L.or_wa_terms_sorted.argtypes = [C.c_int, _f64p, C.c_double, C.c_int, _f64p, _f64p, _f64p, _f64p]
        L.or_wa_grad.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f32p, _f32p, C.c_double, C.c_int,
                                 C.c_int, _f64p, _f64p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_grid_init.argtypes = [C.POINTER(OrGrid), C.c_float, C.c_float, C.c_int, C.c_int]
        L.or_density_q.argtypes = [C.POINTER(OrGrid), C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_void_p, _i64p]
        L.or_overflow.argtypes = [C.POINTER(OrGrid), _i64p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_node_force.argtypes = [C.POINTER(OrGrid), C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_void_p, _f64p,
                                    _f64p, _f64p, _f64p]
        L.or_scale_fixed.argtypes = [C.c_int, _i64p, C.c_double, _i64p]
        L.or_density_float.argtypes = [C.POINTER(OrGrid), _i64p, C.c_void_p, _f32p]
        L.or_field_solve.argtypes = [C.c_int, C.c_int, C.c_double, _f64p, C.c_void_p, _f64p, _f64p]
        L.or_field_solve_fft.restype = C.c_int
        L.or_field_solve_fft.argtypes = [C.c_int, C.c_int, C.c_double, _f64p, C.c_void_p, _f64p, _f64p]
        for n in ("or_dct_1d", "or_idct_1d", "or_idxst_1d"):
            getattr(L, n).argtypes = [C.c_int, _f64p, _f64p]
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f32p, _f32p, _f32p, _f32p, _u8p,
                                C.c_float, C.c_float, C.POINTER(OrParams)]
        L.or_init.argtypes = [C.c_void_p, _f32p, _f32p]
        L.or_step.argtypes = [C.c_void_p, C.c_int]
        L.or_get_stats.argtypes = [C.c_void_p, C.POINTER(OrStats)]
        L.or_get_positions.argtypes = [C.c_void_p, _f32p, _f32p]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_set_threads.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        L.or_surr_num_params.argtypes = [C.c_int, C.c_int, C.c_int, _i32p]
        L.or_surr_forward.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _f64p, _f64p, _f64p]
        L.or_surr_loss_grad.restype = C.c_double
        L.or_surr_loss_grad.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _f64p, _f64p, _f64p,
                                        C.c_int, _f64p]
        L.or_surr_pool.argtypes = [C.c_int, C.c_int, _f64p, _f64p]
        L.or_surr_combine.argtypes = [C.c_int, C.c_int, _f64p, _f64p, C.c_void_p, C.c_double, _f64p, _f64p]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own CPU functions, or None where they were not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        try:
            R = C.CDLL(REF_PATH)
        except OSError:
            return None
        R.ref_density.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_float, C.c_int,
                                  _f32p, C.POINTER(C.c_double)]
        R.ref_hpwl.restype = C.c_double
        R.ref_hpwl.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f32p, _f32p]
        for n in ("ref_dct", "ref_idct", "ref_idxst"):
            getattr(R, n).argtypes = [C.c_int, _f32p, _f32p]
        R.ref_replace_field.argtypes = [C.c_int, _f32p, C.c_void_p, _f32p, _f32p]
        _ref = R
    return _ref


_refp = {}


def ref_placer_lib(opt: str = "O2"):
    """The reference's Placer built for the CPU (_ref/libref_placer.so at -O2,
    _ref/libref_placer_O0.so at -O0), or None where it was not built."""
    path = REF_PLACER_PATH if opt == "O2" else os.path.join(HERE, "_ref", f"libref_placer_{opt}.so")
    if opt not in _refp and os.path.exists(path):
        try:
            R = C.CDLL(path)
        except OSError:
            return None
        dp = C.POINTER(C.c_double)
        R.ref_placer_create.restype = C.c_void_p
        R.ref_placer_create.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, _u8p, C.c_int, _i32p, _i32p,
                                        C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float,
                                        C.c_char_p]
        R.ref_placer_destroy.argtypes = [C.c_void_p]
        R.ref_placer_set_positions.argtypes = [C.c_void_p, _f32p, _f32p]
        R.ref_placer_partials.argtypes = [C.c_void_p, _f32p, _f32p, dp]
        R.ref_placer_overlaps.argtypes = [C.c_void_p, _f32p, dp, dp]
        R.ref_placer_fields_dct.argtypes = [C.c_void_p, _f32p, _f32p, dp]
        R.ref_placer_nudge.argtypes = [C.c_void_p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, dp]
        R.ref_placer_fields_naive.argtypes = [C.c_void_p, _f32p, _f32p, dp]
        R.ref_placer_iterate.argtypes = [C.c_void_p, C.c_int, dp]
        R.ref_placer_get_positions.argtypes = [C.c_void_p, _f32p, _f32p]
        R.ref_placer_hpwl.restype = C.c_double
        R.ref_placer_hpwl.argtypes = [C.c_void_p]
        _refp[opt] = R
    return _refp.get(opt)


class quiet_stdout:
    """Send file descriptor 1 to /dev/null for the block: the reference's
    placer prints its tables and transform traces there."""

    def __enter__(self):
        import sys
        sys.stdout.flush()
        self._saved = os.dup(1)
        dn = os.open(os.devnull, os.O_WRONLY)
        os.dup2(dn, 1)
        os.close(dn)
        return self

    def __exit__(self, *exc):
        import sys
        try:
            C.CDLL(None).fflush(None)
        except (OSError, AttributeError):
            pass
        sys.stdout.flush()
        os.dup2(self._saved, 1)
        os.close(self._saved)
        return False


class RefPlacer:
    """The reference's own Placer (vck5000/host/src/AIEplace.cpp) on a CSR
    netlist, through ref_placer.cpp.  Every call returns the reference's
    result and the seconds its own function took."""

    def __init__(self, net_ptr, pin_node, w, h, x, y, fixed, die_w, die_h, bins,
                 gamma=1.0, learning_rate=1e-3, global_lambda=1.0, opt="O2"):
        import tempfile
        R = ref_placer_lib(opt)
        if R is None:
            raise RuntimeError("the reference placer library was not built (make refplacer REF=<checkout>)")
        self._R = R
        self.n = len(x)
        self.bins = bins
        self._dir = tempfile.mkdtemp(prefix="ref_placer_")
        self._h = R.ref_placer_create(self.n, _f32(w), _f32(h), _f32(x), _f32(y),
                                      np.ascontiguousarray(fixed, dtype=np.uint8), len(net_ptr) - 1,
                                      _i32(net_ptr), _i32(pin_node), die_w, die_h, bins, gamma,
                                      learning_rate, global_lambda, self._dir.encode())
        if not self._h:
            raise RuntimeError("ref_placer_create failed")

    def close(self):
        import shutil
        if self._h:
            self._R.ref_placer_destroy(self._h)
            self._h = None
            shutil.rmtree(self._dir, ignore_errors=True)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_positions(self, x, y):
        self._R.ref_placer_set_positions(self._h, _f32(x), _f32(y))

    def partials(self):
        gx, gy, t = np.zeros(self.n, np.float32), np.zeros(self.n, np.float32), C.c_double()
        self._R.ref_placer_partials(self._h, gx, gy, C.byref(t))
        return gx, gy, t.value

    def overlaps(self):
        M = self.bins
        rho, ovf, t = np.zeros(M * M, np.float32), C.c_double(), C.c_double()
        self._R.ref_placer_overlaps(self._h, rho, C.byref(ovf), C.byref(t))
        return rho.reshape(M, M), ovf.value, t.value

    def fields_dct(self):
        M = self.bins
        ex, ey, t = np.zeros(M * M, np.float32), np.zeros(M * M, np.float32), C.c_double()
        self._R.ref_placer_fields_dct(self._h, ex, ey, C.byref(t))
        return ex.reshape(M, M), ey.reshape(M, M), t.value

    def fields_naive(self):
        M = self.bins
        ex, ey, t = np.zeros(M * M, np.float32), np.zeros(M * M, np.float32), C.c_double()
        self._R.ref_placer_fields_naive(self._h, ex, ey, C.byref(t))
        return ex.reshape(M, M), ey.reshape(M, M), t.value

    def iterate(self, iters: int) -> float:
        t = C.c_double()
        self._R.ref_placer_iterate(self._h, iters, C.byref(t))
        return t.value

    def positions(self):
        x, y = np.zeros(self.n, np.float32), np.zeros(self.n, np.float32)
        self._R.ref_placer_get_positions(self._h, x, y)
        return x, y

    def nudge(self, ex, ey, px, py):
        mx, my, t = np.zeros(self.n, np.float32), np.zeros(self.n, np.float32), C.c_double()
        self._R.ref_placer_nudge(self._h, _f32(ex), _f32(ey), _f32(px), _f32(py), mx, my, C.byref(t))
        return mx, my, t.value

    def hpwl(self) -> float:
        return self._R.ref_placer_hpwl(self._h)


def set_threads(n: int) -> int:
    return lib().or_set_threads(n)


# ---------------------------------------------------------------- WA terms

def fast_exp(a: float, prec: int = 16) -> float:
    return lib().or_fast_exp(a, prec)


def wa_terms_sorted(xs, gamma: float, fast: bool = False):
    x = np.ascontiguousarray(xs, dtype=np.float64)
    n = len(x)
    ap, am, bc, part = (np.zeros(n), np.zeros(n), np.zeros(4), np.zeros(n))
    lib().or_wa_terms_sorted(n, x, gamma, int(fast), ap, am, bc, part)
    return ap, am, bc, part


def wa_grad(net_ptr, pin_node, x, y, gamma, min_deg=2, max_deg=1 << 30):
    n = len(x)
    gx, gy = np.zeros(n), np.zeros(n)
    wa, hp = C.c_double(), C.c_double()
    lib().or_wa_grad(n, len(net_ptr) - 1, _i32(net_ptr), _i32(pin_node), _f32(x), _f32(y), gamma,
                     min_deg, max_deg, gx, gy, C.byref(wa), C.byref(hp))
    return gx, gy, wa.value, hp.value


# ---------------------------------------------------------------- density

def grid(die_w, die_h, mx, my=None) -> OrGrid:
    g = OrGrid()
    lib().or_grid_init(C.byref(g), die_w, die_h, mx, my or mx)
    return g


def density_q(g: OrGrid, x, y, w, h, include=None):
    rho = np.zeros(g.mx * g.my, dtype=np.int64)
    inc = None if include is None else np.ascontiguousarray(include, dtype=np.uint8)
    lib().or_density_q(C.byref(g), len(x), _f32(x), _f32(y), _f32(w), _f32(h),
                       None if inc is None else inc.ctypes.data, rho)
    return rho


def node_force(g: OrGrid, x, y, w, h, ex, ey, include=None):
    """Per-node overlap-weighted field (FP64), nudgeNode's force."""
    n = len(x)
    fx, fy = np.zeros(n), np.zeros(n)
    inc = None if include is None else np.ascontiguousarray(include, dtype=np.uint8)
    lib().or_node_force(C.byref(g), n, _f32(x), _f32(y), _f32(w), _f32(h), None if inc is None else inc.ctypes.data,
                        np.ascontiguousarray(ex, np.float64).reshape(-1),
                        np.ascontiguousarray(ey, np.float64).reshape(-1), fx, fy)
    return fx, fy


def scale_fixed(fixed_q, rho_t):
    out = np.zeros_like(fixed_q)
    lib().or_scale_fixed(len(fixed_q), np.ascontiguousarray(fixed_q), rho_t, out)
    return out


def overflow(g: OrGrid, mov_q, fixed_q, fixed_scaled_q, rho_t, movable_area_q):
    tau, ab = C.c_double(), C.c_double()
    lib().or_overflow(C.byref(g), mov_q, fixed_q.ctypes.data, fixed_scaled_q.ctypes.data, rho_t,
                      float(movable_area_q), C.byref(tau), C.byref(ab))
    return tau.value, ab.value


def density_float(g: OrGrid, mov_q, fixed_scaled_q):
    d = np.zeros(g.mx * g.my, dtype=np.float32)
    lib().or_density_float(C.byref(g), mov_q, fixed_scaled_q.ctypes.data, d)
    return d


# ---------------------------------------------------------------- spectral

def field_solve(d, m: int, bin_ratio: float = 1.0, want_phi: bool = False):
    d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1)
    ex, ey = np.zeros(m * m), np.zeros(m * m)
    phi = np.zeros(m * m) if want_phi else None
    lib().or_field_solve(m, m, bin_ratio, d, None if phi is None else phi.ctypes.data, ex, ey)
    return (ex, ey, phi) if want_phi else (ex, ey)


def field_solve_fft(d, m: int, bin_ratio: float = 1.0, want_phi: bool = False):
    """The same sums as field_solve through fast transforms (fft_solve.c)."""
    d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1)
    ex, ey = np.zeros(m * m), np.zeros(m * m)
    phi = np.zeros(m * m) if want_phi else None
    rc = lib().or_field_solve_fft(m, m, bin_ratio, d, None if phi is None else phi.ctypes.data, ex, ey)
    if rc != 0:
        raise ValueError(f"or_field_solve_fft: unsupported size {m}")
    return (ex, ey, phi) if want_phi else (ex, ey)


def dct_1d(v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    o = np.zeros_like(v)
    lib().or_dct_1d(len(v), v, o)
    return o


def idct_1d(v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    o = np.zeros_like(v)
    lib().or_idct_1d(len(v), v, o)
    return o


def idxst_1d(v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    o = np.zeros_like(v)
    lib().or_idxst_1d(len(v), v, o)
    return o


# ---------------------------------------------------------------- loop

class Placer:
    """FP64 ePlace loop oracle over a CSR netlist (movable nodes first)."""

    def __init__(self, nl: dict, mx: int, target_density: float, gamma_base_bins=4.0,
                 init_density_weight=8e-5, ref_delta_hpwl=0.0, mu_max=1.05, mu_min=0.95,
                 init_step_coef=0.1, restart=4, max_backtracks=0):
        p = OrParams(mx, mx, target_density, gamma_base_bins, init_density_weight, ref_delta_hpwl,
                     mu_max, mu_min, init_step_coef, restart, max_backtracks)
        self._keep = nl
        die = nl["die"]
        self.h = lib().or_create(len(nl["node_w"]), len(nl["net_ptr"]) - 1, _i32(nl["net_ptr"]),
                                 _i32(nl["pin_node"]), _f32(nl["node_w"]), _f32(nl["node_h"]),
                                 _f32(nl["node_x"]), _f32(nl["node_y"]),
                                 np.ascontiguousarray(nl["node_fixed"], dtype=np.uint8),
                                 float(die[2] - die[0]), float(die[3] - die[1]), C.byref(p))
        self.n = len(nl["node_w"])

    def init(self, x, y):
        lib().or_init(self.h, _f32(x), _f32(y))

    def step(self, n: int = 1):
        lib().or_step(self.h, n)

    def stats(self) -> dict:
        s = OrStats()
        lib().or_get_stats(self.h, C.byref(s))
        return {"iteration": s.iteration, "hpwl": s.hpwl, "wa": s.wa, "overflow": s.overflow,
                "overflow_abs": s.overflow_abs, "lambda": s.lambda_, "gamma": s.gamma,
                "alpha": s.alpha, "a_k": s.a_k, "evals": s.evals,
                "norm_wl": s.norm_wl, "norm_f": s.norm_f, "restarts": s.restarts}

    def positions(self):
        x, y = np.zeros(self.n, np.float32), np.zeros(self.n, np.float32)
        lib().or_get_positions(self.h, x, y)
        return x, y

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# ---- seeded synthetic netlists (libsynth.so) ------------------------------------
# The generator of the product library built on its own, so that CPU-only
# processes (the reference arm of bench.py) draw the same netlists without
# loading the product library.

class SynthConfig(C.Structure):
    _fields_ = [("num_cells", C.c_int32), ("num_nets", C.c_int32), ("num_macros", C.c_int32),
                ("num_pads", C.c_int32), ("unit_cells", C.c_int32), ("degree_mix", C.c_int32),
                ("locality", C.c_float), ("window", C.c_int32), ("macro_area_min", C.c_float),
                ("macro_area_max", C.c_float), ("target_density", C.c_float), ("die_side", C.c_float),
                ("seed", C.c_uint64)]


_synth = None


def synth_lib():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_PATH):
            build(with_ref=False)
        L = C.CDLL(SYNTH_PATH)
        vp = C.c_void_p
        L.ap_synth_counts.argtypes = [C.POINTER(SynthConfig), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32)]
        L.ap_synth_generate.argtypes = [C.POINTER(SynthConfig), vp, vp, vp, vp, vp, vp, vp, vp]
        _synth = L
    return _synth


def synth_generate(spec: dict, seed: int = 1) -> dict:
    """The netlist of a preset spec (aieplace_gb300/presets.py) as numpy
    arrays, identical to aieplace_gb300.synth.generate(spec, seed)."""
    spec = dict(spec)
    bins = spec.pop("bins")
    cfg = SynthConfig(spec["num_cells"], spec["num_nets"], spec["num_macros"], spec["num_pads"],
                      spec["unit_cells"], spec["degree_mix"], spec["locality"], spec["window"],
                      spec.get("macro_area_min", 20.0), spec.get("macro_area_max", 200.0),
                      spec["target_density"], spec["die_side"], seed)
    nn, ne, npins = C.c_int32(), C.c_int32(), C.c_int32()
    L = synth_lib()
    if L.ap_synth_counts(C.byref(cfg), C.byref(nn), C.byref(ne), C.byref(npins)) != 0:
        raise ValueError("ap_synth_counts rejected the spec")
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
    keys = ("net_ptr", "pin_node", "node_w", "node_h", "node_x", "node_y", "node_fixed", "die")
    if L.ap_synth_generate(C.byref(cfg), *[C.c_void_p(out[k].ctypes.data) for k in keys]) != 0:
        raise ValueError("ap_synth_generate failed")
    out["bins"] = bins
    out["target_density"] = spec["target_density"]
    out["seed"] = seed
    return out


# ---- learned surrogate network (surrogate.c) -----------------------------------

def surr_num_params(cin0: int, width: int, cout: int, kernels) -> int:
    k = np.ascontiguousarray(kernels, np.int32)
    return lib().or_surr_num_params(cin0, width, cout, k)


def surr_forward(x, params, width: int, cout: int, kernels):
    """x [B][cin0][R][R] -> y [B][cout][R][R], FP64."""
    x = np.ascontiguousarray(x, np.float64)
    B, cin0, R, _ = x.shape
    y = np.zeros((B, cout, R, R), np.float64)
    lib().or_surr_forward(B, R, cin0, width, cout, np.ascontiguousarray(kernels, np.int32),
                          np.ascontiguousarray(params, np.float64), x, y)
    return y


def surr_loss_grad(x, t, params, width: int, kernels, margin: int):
    x = np.ascontiguousarray(x, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    B, cin0, R, _ = x.shape
    cout = t.shape[1]
    p = np.ascontiguousarray(params, np.float64)
    g = np.zeros_like(p)
    loss = lib().or_surr_loss_grad(B, R, cin0, width, cout, np.ascontiguousarray(kernels, np.int32), p, x, t,
                                   margin, g)
    return loss, g


def surr_pool(d, f: int):
    d = np.ascontiguousarray(d, np.float64)
    M = d.shape[0]
    out = np.zeros((M // f, M // f), np.float64)
    lib().or_surr_pool(M, f, d, out)
    return out


def surr_combine(cex, cey, y, s: float, f: int):
    cex = np.ascontiguousarray(cex, np.float64)
    cey = np.ascontiguousarray(cey, np.float64)
    M = cex.shape[0] * f
    ex = np.zeros((M, M), np.float64)
    ey = np.zeros((M, M), np.float64)
    yp = None if y is None else np.ascontiguousarray(y, np.float64)
    lib().or_surr_combine(M, f, cex, cey, None if yp is None else yp.ctypes.data, float(s), ex, ey)
    return ex, ey
