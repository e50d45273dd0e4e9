"""LEF/DEF designs through the library's reader and writer (include/aieplace.h
ap_design_*), the ingest and write-back the reference host does in
DataBase.cpp (readLEF/readDEF :42-96, writeDEF :538-655)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import APError, DesignInfo, Netlist, lib

SIZE_DBU = 0       # LEF sizes scaled to DEF database units, rotated orientations swapped
SIZE_AS_READ = 1   # LEF numbers as they are, orientation ignored (the reference host's reading)


def _check(fn: str, st: int):
    if st != 0:
        msg = lib().ap_last_error().decode() or lib().ap_status_string(st).decode()
        raise APError(fn, st, msg)


class Design:
    """A design read from LEF files and a DEF; netlist() gives the arrays
    Placer takes (nodes: components, then IO pins; database units)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def read(cls, lef_paths, def_path: str, size_mode: int = SIZE_DBU) -> "Design":
        paths = [str(p).encode() for p in lef_paths]
        arr = (C.c_char_p * max(len(paths), 1))(*paths)
        h = C.c_void_p()
        _check("ap_design_read", lib().ap_design_read(arr, len(paths), str(def_path).encode(), size_mode, C.byref(h)))
        return cls(h)

    @classmethod
    def read_dir(cls, directory: str, size_mode: int = SIZE_DBU) -> "Design":
        """Every *.lef of the directory and its floorplan.def (the reference's input layout)."""
        h = C.c_void_p()
        _check("ap_design_read_dir", lib().ap_design_read_dir(str(directory).encode(), size_mode, C.byref(h)))
        return cls(h)

    def close(self):
        if self._h:
            lib().ap_design_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def name(self) -> str:
        return lib().ap_design_name(self._h).decode()

    def info(self) -> dict:
        i = DesignInfo()
        _check("ap_design_get_info", lib().ap_design_get_info(self._h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in DesignInfo._fields_}

    def node_name(self, i: int) -> str:
        s = lib().ap_design_node_name(self._h, i)
        if s is None:
            raise IndexError(i)
        return s.decode()

    def netlist(self, bins: int = 512, target_density: float = 1.0) -> dict:
        """Copies of the design's netlist arrays, in the form Placer takes."""
        nl = Netlist()
        _check("ap_design_netlist", lib().ap_design_netlist(self._h, C.byref(nl)))
        n, e, p = nl.num_nodes, nl.num_nets, nl.num_pins

        def arr(ptr_, count, ctype, dtype):
            if count == 0:
                return np.zeros(0, dtype)
            return np.ctypeslib.as_array(C.cast(ptr_, C.POINTER(ctype)), shape=(count,)).astype(dtype)

        return {
            "net_ptr": arr(nl.net_ptr, e + 1, C.c_int32, np.int32),
            "pin_node": arr(nl.pin_node, p, C.c_int32, np.int32),
            "node_w": arr(nl.node_w, n, C.c_float, np.float32),
            "node_h": arr(nl.node_h, n, C.c_float, np.float32),
            "node_x": arr(nl.node_x, n, C.c_float, np.float32),
            "node_y": arr(nl.node_y, n, C.c_float, np.float32),
            "node_fixed": arr(nl.node_fixed, n, C.c_uint8, np.uint8),
            "die": np.array([nl.die_xl, nl.die_yl, nl.die_xh, nl.die_yh], np.float32),
            "bins": bins, "target_density": target_density, "seed": 0,
        }

    def write_def(self, path: str, x, y):
        """DEF with the given node positions (netlist order), rounded to database units."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        _check("ap_design_write_def", lib().ap_design_write_def(self._h, x.ctypes.data, y.ctypes.data,
                                                                str(path).encode()))
