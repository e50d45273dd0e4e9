"""ctypes bindings of libaieplace_gb300.so (the C ABI in include/aieplace.h).

The library is the only compute path: if it is missing or fails to load,
every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaieplace_gb300.so")

# symbols declared in include/aieplace.h
EXPORTS = [
    "ap_abi_version", "ap_status_string", "ap_params_default", "ap_create", "ap_destroy",
    "ap_set_stream", "ap_init_positions", "ap_init_seeded", "ap_step", "ap_step_async",
    "ap_profile_stages", "ap_solver_info", "ap_run", "ap_step_host",
    "ap_get_positions", "ap_get_stats", "ap_hpwl", "ap_overflow", "ap_wirelength_grad",
    "ap_density_map", "ap_field_solve", "ap_node_force", "ap_debug_inject", "ap_set_log", "ap_get_fillers",
    "ap_run_config_default", "ap_run_config_read", "ap_last_error", "ap_field_solve_noalloc", "ap_selftest_numerics",
    "ap_snapshot_size", "ap_snapshot",
    "ap_restore",
    "ap_synth_counts", "ap_synth_generate",
    "ap_design_read", "ap_design_read_dir", "ap_design_get_info", "ap_design_netlist", "ap_design_name",
    "ap_design_node_name", "ap_design_write_def", "ap_design_destroy",
    "ap_create_batch", "ap_batch_destroy", "ap_batch_init_seeded", "ap_batch_step", "ap_batch_run",
    "ap_batch_get_stats", "ap_batch_get_positions", "ap_batch_set_form", "ap_batch_get_info",
    "ap_batch_debug_inject", "ap_batch_set_item_blocks", "ap_batch_profile",
    "ap_surrogate_config_default", "ap_surrogate_create", "ap_surrogate_destroy", "ap_surrogate_num_params",
    "ap_surrogate_get_params", "ap_surrogate_set_params", "ap_surrogate_forward", "ap_surrogate_gradient",
    "ap_surrogate_reserve", "ap_surrogate_num_samples", "ap_surrogate_collect", "ap_surrogate_train",
    "ap_surrogate_validate", "ap_attach_surrogate", "ap_surrogate_get_stats",
]

AP_OK = 0
AP_FIELD_FP32 = 0
AP_FIELD_BF16X3 = 1


class APError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed: {msg} (status {status})")
        self.status = status


class Netlist(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_nets", C.c_int32), ("num_pins", C.c_int32),
                ("net_ptr", C.c_void_p), ("pin_node", C.c_void_p), ("node_w", C.c_void_p),
                ("node_h", C.c_void_p), ("node_x", C.c_void_p), ("node_y", C.c_void_p),
                ("node_fixed", C.c_void_p), ("die_xl", C.c_float), ("die_yl", C.c_float),
                ("die_xh", C.c_float), ("die_yh", C.c_float)]


class Params(C.Structure):
    _fields_ = [("bins_x", C.c_int32), ("bins_y", C.c_int32), ("target_density", C.c_float),
                ("gamma_base_bins", C.c_float), ("field_solver", C.c_int32),
                ("init_density_weight", C.c_float), ("ref_delta_hpwl", C.c_float),
                ("lambda_mu_max", C.c_float), ("lambda_mu_min", C.c_float),
                ("init_step_coef", C.c_float), ("target_overflow", C.c_float),
                ("max_iterations", C.c_int32), ("check_interval", C.c_int32),
                ("use_graph", C.c_int32), ("max_backtracks", C.c_int32), ("restart_mode", C.c_int32),
                ("filler_cells", C.c_int32), ("block_nodes", C.c_int32)]


STAGES6 = ("update", "scatter", "rho", "wa", "field", "gather")


class BatchInfo(C.Structure):
    _fields_ = [("form", C.c_int32), ("instances", C.c_int32), ("active", C.c_int32), ("field_tile", C.c_int32),
                ("field_tune_ms", C.c_float * 2), ("records", C.c_int32 * 6), ("item_blocks", C.c_int32 * 6),
                ("items", C.c_int32 * 6)]

    def as_dict(self) -> dict:
        return {"form": ("graph", "persistent")[self.form], "instances": self.instances, "active": self.active,
                "field_tile": self.field_tile, "field_tune_ms": list(self.field_tune_ms),
                "records": dict(zip(STAGES6, self.records)), "item_blocks": dict(zip(STAGES6, self.item_blocks)),
                "items": dict(zip(STAGES6, self.items))}


class Stats(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("status", C.c_int32), ("hpwl", C.c_double),
                ("wa_wirelength", C.c_double), ("overflow", C.c_double), ("overflow_abs", C.c_double),
                ("lambda_", C.c_double), ("gamma", C.c_double), ("alpha", C.c_double),
                ("a_k", C.c_double), ("evals", C.c_int32), ("restarts", C.c_int32)]

    def as_dict(self) -> dict:
        return {"iteration": self.iteration, "status": self.status, "hpwl": self.hpwl,
                "wa": self.wa_wirelength, "overflow": self.overflow,
                "overflow_abs": self.overflow_abs, "lambda": self.lambda_, "gamma": self.gamma,
                "alpha": self.alpha, "a_k": self.a_k, "evals": self.evals, "restarts": self.restarts}


class SurrogateConfig(C.Structure):
    _fields_ = [("factor", C.c_int32), ("kernel", C.c_int32 * 4), ("width", C.c_int32), ("seed", C.c_uint64)]


class SurrogatePolicy(C.Structure):
    _fields_ = [("overflow_min", C.c_float), ("judge_every", C.c_int32), ("max_error", C.c_float),
                ("use_net", C.c_int32)]


class SurrogateStats(C.Structure):
    _fields_ = [("used", C.c_int32), ("judged", C.c_int32), ("fallbacks", C.c_int32), ("last_error", C.c_double)]


class RunConfig(C.Structure):
    _fields_ = [("input_dir", C.c_char * 1024), ("output_dir", C.c_char * 1024), ("log_path", C.c_char * 1024),
                ("size_mode", C.c_int32), ("wirelength_method", C.c_int32), ("init_sigma", C.c_float),
                ("seed", C.c_uint64), ("filler_cells", C.c_int32), ("use_aie", C.c_int32),
                ("ignored_learning_rate", C.c_float)]


class DesignInfo(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_nets", C.c_int32), ("num_pins", C.c_int32),
                ("num_components", C.c_int32), ("num_io_pins", C.c_int32), ("units_per_micron", C.c_int32),
                ("die_xl", C.c_float), ("die_yl", C.c_float), ("die_xh", C.c_float), ("die_yh", C.c_float)]


class SynthConfig(C.Structure):
    _fields_ = [("num_cells", C.c_int32), ("num_nets", C.c_int32), ("num_macros", C.c_int32),
                ("num_pads", C.c_int32), ("unit_cells", C.c_int32), ("degree_mix", C.c_int32),
                ("locality", C.c_float), ("window", C.c_int32), ("macro_area_min", C.c_float),
                ("macro_area_max", C.c_float), ("target_density", C.c_float),
                ("die_side", C.c_float), ("seed", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run aieplace_gb300.build.build() first")
        L = C.CDLL(LIB_PATH)
        vp, i32, f32, u64 = C.c_void_p, C.c_int32, C.c_float, C.c_uint64
        L.ap_status_string.restype = C.c_char_p
        L.ap_status_string.argtypes = [C.c_int]
        L.ap_params_default.argtypes = [C.POINTER(Params)]
        L.ap_create.argtypes = [C.POINTER(Netlist), C.POINTER(Params), C.POINTER(vp)]
        L.ap_destroy.argtypes = [vp]
        L.ap_set_stream.argtypes = [vp, vp]
        L.ap_init_positions.argtypes = [vp, vp, vp]
        L.ap_init_seeded.argtypes = [vp, u64, f32]
        L.ap_step.argtypes = [vp, i32]
        L.ap_step_async.argtypes = [vp, i32]
        L.ap_solver_info.argtypes = [vp, C.POINTER(i32), vp, C.POINTER(i32), vp]
        L.ap_profile_stages.argtypes = [vp, i32, vp, C.POINTER(i32)]
        L.ap_run.argtypes = [vp, C.POINTER(i32)]
        L.ap_step_host.argtypes = [vp, vp, vp, vp, vp, C.POINTER(Stats)]
        L.ap_get_positions.argtypes = [vp, vp, vp]
        L.ap_get_stats.argtypes = [vp, C.POINTER(Stats)]
        L.ap_hpwl.argtypes = [vp, C.POINTER(C.c_double)]
        L.ap_overflow.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ap_wirelength_grad.argtypes = [vp, vp, vp, f32, vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ap_node_force.argtypes = [vp, vp, vp, vp, vp, f32, f32, vp, vp, vp, vp]
        L.ap_debug_inject.argtypes = [vp, i32, C.c_int64]
        L.ap_set_log.argtypes = [vp, C.c_char_p, i32]
        L.ap_design_read.argtypes = [C.POINTER(C.c_char_p), i32, C.c_char_p, i32, C.POINTER(vp)]
        L.ap_design_read_dir.argtypes = [C.c_char_p, i32, C.POINTER(vp)]
        L.ap_design_get_info.argtypes = [vp, C.POINTER(DesignInfo)]
        L.ap_design_netlist.argtypes = [vp, C.POINTER(Netlist)]
        L.ap_design_name.restype = C.c_char_p
        L.ap_design_name.argtypes = [vp]
        L.ap_design_node_name.restype = C.c_char_p
        L.ap_design_node_name.argtypes = [vp, i32]
        L.ap_design_write_def.argtypes = [vp, vp, vp, C.c_char_p]
        L.ap_last_error.restype = C.c_char_p
        L.ap_last_error.argtypes = []
        L.ap_get_fillers.argtypes = [vp, C.POINTER(i32), C.POINTER(f32), C.POINTER(f32)]
        L.ap_run_config_default.argtypes = [C.POINTER(Params), C.POINTER(RunConfig)]
        L.ap_run_config_read.argtypes = [C.c_char_p, C.POINTER(Params), C.POINTER(RunConfig)]
        L.ap_design_destroy.argtypes = [vp]
        L.ap_density_map.argtypes = [vp, vp, vp, vp]
        L.ap_field_solve.argtypes = [vp, vp, vp, vp, i32]
        L.ap_field_solve_noalloc.argtypes = [vp, vp, vp, i32, f32, vp]
        L.ap_selftest_numerics.argtypes = [vp, C.c_int64]
        L.ap_snapshot_size.argtypes = [vp, C.POINTER(C.c_size_t)]
        L.ap_snapshot.argtypes = [vp, vp, C.c_size_t]
        L.ap_restore.argtypes = [vp, vp, C.c_size_t]
        L.ap_create_batch.argtypes = [i32, vp, vp, C.POINTER(vp)]
        L.ap_batch_destroy.argtypes = [vp]
        L.ap_batch_init_seeded.argtypes = [vp, u64, f32]
        L.ap_batch_step.argtypes = [vp, i32]
        L.ap_batch_run.argtypes = [vp, vp]
        L.ap_batch_get_stats.argtypes = [vp, i32, C.POINTER(Stats)]
        L.ap_batch_get_positions.argtypes = [vp, i32, vp, vp]
        L.ap_batch_set_form.argtypes = [vp, i32]
        L.ap_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
        L.ap_batch_debug_inject.argtypes = [vp, i32, C.c_int64]
        L.ap_batch_set_item_blocks.argtypes = [vp, i32]
        L.ap_batch_profile.argtypes = [vp, i32, vp]
        L.ap_surrogate_config_default.argtypes = [C.POINTER(SurrogateConfig)]
        L.ap_surrogate_create.argtypes = [C.POINTER(SurrogateConfig), C.POINTER(vp)]
        L.ap_surrogate_destroy.argtypes = [vp]
        L.ap_surrogate_num_params.argtypes = [vp, C.POINTER(i32)]
        L.ap_surrogate_get_params.argtypes = [vp, vp, i32]
        L.ap_surrogate_set_params.argtypes = [vp, vp, i32]
        L.ap_surrogate_forward.argtypes = [vp, vp, i32, i32, vp]
        L.ap_surrogate_gradient.argtypes = [vp, vp, vp, i32, i32, i32, C.POINTER(f32), vp]
        L.ap_surrogate_reserve.argtypes = [vp, i32, i32]
        L.ap_surrogate_num_samples.argtypes = [vp, C.POINTER(i32)]
        L.ap_surrogate_collect.argtypes = [vp, vp, i32, i32, C.POINTER(i32)]
        L.ap_surrogate_train.argtypes = [vp, i32, i32, i32, f32, u64, i32, i32, vp]
        L.ap_surrogate_validate.argtypes = [vp, i32, i32, vp, vp]
        L.ap_attach_surrogate.argtypes = [vp, vp, C.POINTER(SurrogatePolicy)]
        L.ap_surrogate_get_stats.argtypes = [vp, C.POINTER(SurrogateStats)]
        L.ap_synth_counts.argtypes =[C.POINTER(SynthConfig), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]
        L.ap_synth_generate.argtypes = [C.POINTER(SynthConfig), vp, vp, vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def check(fn: str, status: int) -> None:
    if status != AP_OK:
        raise APError(fn, status, lib().ap_status_string(status).decode())


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data
