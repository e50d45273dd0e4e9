"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point include/aieplace.h declares, validates its inputs before
touching a device, and the seeded generator is deterministic."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def lib():
    from aieplace_gb300 import build

    build.build()
    from aieplace_gb300 import _lib

    return _lib


def declared_symbols():
    text = open(os.path.join(REPO, "include", "aieplace.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(ap_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(lib):
    L = lib.lib()
    decl = declared_symbols()
    assert len(decl) >= 20
    for name in decl:
        assert hasattr(L, name), name
    assert sorted(lib.EXPORTS) == sorted(set(lib.EXPORTS))
    assert set(decl) <= set(lib.EXPORTS) | {"ap_abi_version"}


def test_params_default_and_status_strings(lib):
    p = lib.Params()
    assert lib.lib().ap_params_default(C.byref(p)) == 0
    assert p.bins_x == 512 and p.max_backtracks == 0 and p.restart_mode == 4
    assert lib.lib().ap_status_string(2) == b"malformed netlist"


def _netlist(lib, nl, **over):
    a = {k: np.ascontiguousarray(v) for k, v in nl.items() if isinstance(v, np.ndarray)}
    a.update(over)
    die = a["die"]
    n = lib.Netlist(len(a["node_w"]), len(a["net_ptr"]) - 1, len(a["pin_node"]), a["net_ptr"].ctypes.data,
                    a["pin_node"].ctypes.data, a["node_w"].ctypes.data, a["node_h"].ctypes.data,
                    a["node_x"].ctypes.data, a["node_y"].ctypes.data, a["node_fixed"].ctypes.data,
                    float(die[0]), float(die[1]), float(die[2]), float(die[3]))
    return n, a


def _create(lib, nl, **over):
    n, keep = _netlist(lib, nl, **over)
    p = lib.Params()
    lib.lib().ap_params_default(C.byref(p))
    p.bins_x = p.bins_y = 32
    h = C.c_void_p()
    st = lib.lib().ap_create(C.byref(n), C.byref(p), C.byref(h))
    if st == 0:
        lib.lib().ap_destroy(h)
    return st


def test_create_rejects_malformed_csr_before_the_device(lib):
    from aieplace_gb300 import synth

    nl = synth.generate("c0", seed=3)
    bad_pin = nl["pin_node"].copy()
    bad_pin[5] = len(nl["node_w"]) + 7
    assert _create(lib, nl, pin_node=bad_pin) == 2
    bad_ptr = nl["net_ptr"].copy()
    bad_ptr[10] = bad_ptr[11] + 1  # decreasing
    assert _create(lib, nl, net_ptr=bad_ptr) == 2
    bad_x = nl["node_x"].copy()
    bad_x[3] = np.nan
    assert _create(lib, nl, node_x=bad_x) == 3


def test_create_without_gpu_reports_no_device(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from aieplace_gb300 import synth

    assert _create(lib, synth.generate("c0", seed=3)) == 5


def test_generator_deterministic_and_shaped(lib):
    from aieplace_gb300 import synth

    a = synth.generate("c1_small", seed=9)
    b = synth.generate("c1_small", seed=9)
    for k in ("net_ptr", "pin_node", "node_w", "node_x", "node_fixed"):
        np.testing.assert_array_equal(a[k], b[k])
    deg = np.diff(a["net_ptr"])
    assert deg.min() >= 2 and deg.max() <= 64
    frac2 = (deg == 2).mean()
    assert 0.6 < frac2 < 0.7
    fixed = a["node_fixed"].astype(bool)
    assert fixed.sum() == 400
    # fixed macros do not overlap each other and lie inside the die
    x, y, w, h = (a[k][fixed] for k in ("node_x", "node_y", "node_w", "node_h"))
    assert (x >= 0).all() and (x + w <= a["die"][2] + 1e-3).all()
    order = np.argsort(x)
    x, y, w, h = x[order], y[order], w[order], h[order]
    for i in range(len(x)):
        j = i + 1
        while j < len(x) and x[j] < x[i] + w[i]:
            assert not (y[j] < y[i] + h[i] and y[i] < y[j] + h[j])
            j += 1
    c0 = synth.generate("c0", seed=1)
    assert len(c0["node_w"]) == 600 and c0["die"][2] == 24.0


@pytest.mark.parametrize("preset", ["c0", "c1_small"])
def test_standalone_generator_matches_library(lib, preset):
    """oracle/libsynth.so (the generator built on its own, for CPU-only
    processes) draws the same netlists as the product library."""
    import oracle

    import aieplace_gb300 as ap

    oracle.build(with_ref=False)
    a = ap.synth.generate(preset, seed=3)
    b = oracle.synth_generate(ap.synth.PRESETS[preset], seed=3)
    for k in ("net_ptr", "pin_node", "node_w", "node_h", "node_x", "node_y", "node_fixed", "die"):
        assert np.array_equal(a[k], b[k]), k
