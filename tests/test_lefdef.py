"""LEF/DEF ingest and DEF write-back (ap_design_*), on the hand-written
fixtures in tests/golden/lefdef/.

CPU: the reader keeps what the reference's DataBase callbacks keep
(DataBase.cpp:340-416) and skips the rest; the written DEF reads back to the
same design with the positions rounded to database units; errors name the
file and line.  GPU: read -> place -> write -> re-read gives the placed
positions (rounded), with fixed nodes where they were.
"""
import os
import shutil

import numpy as np
import pytest

from conftest import REPO

FIX = os.path.join(REPO, "tests", "golden", "lefdef")
LEFS = [os.path.join(FIX, "tech.lef"), os.path.join(FIX, "cells.lef")]
DEF = os.path.join(FIX, "floorplan.def")


@pytest.fixture(scope="module")
def ap():
    from aieplace_gb300 import build

    build.build()
    import aieplace_gb300

    return aieplace_gb300


NAMES = ["ram0", "u1", "u2", "u3", "u4", "u5", "u6", "u7", "u8", "u9", "u10", "blk1", "in0", "in1", "clk", "out0"]


def test_reads_the_subset_the_reference_keeps(ap):
    with ap.Design.read(LEFS, DEF) as d:
        assert d.name == "tiny_core"
        info = d.info()
        assert info["units_per_micron"] == 1000
        assert (info["num_components"], info["num_io_pins"], info["num_nets"]) == (12, 4, 9)
        assert (info["die_xh"], info["die_yh"]) == (20000.0, 20000.0)
        assert [d.node_name(i) for i in range(16)] == NAMES
        nl = d.netlist()
    # sizes: LEF microns x 1000; u6 placed E has width and height swapped
    np.testing.assert_array_equal(nl["node_w"][:12], [6000, 380, 380, 570, 570, 3230, 1400, 380, 570, 3230, 380, 6000])
    np.testing.assert_array_equal(nl["node_h"][:12], [4200, 1400, 1400, 1400, 1400, 1400, 3230, 1400, 1400, 1400, 1400,
                                                      4200])
    assert (nl["node_w"][12:] == 0).all() and (nl["node_h"][12:] == 0).all()  # IO pins carry pins only
    # FIXED and COVER components and every IO pin are fixed; u7 is unplaced (0, 0)
    np.testing.assert_array_equal(nl["node_fixed"], [1] + [0] * 10 + [1] * 5)
    assert (nl["node_x"][7], nl["node_y"][7]) == (0.0, 0.0)
    assert (nl["node_x"][4], nl["node_y"][4]) == (4000.0, 2800.0)  # after "+ SOURCE NETLIST"
    np.testing.assert_array_equal(nl["node_x"][12:], [0, 0, 10000, 20000])
    np.testing.assert_array_equal(nl["node_y"][12:], [5000, 10000, 0, 12000])
    # nets in file order, connections in order; routing after '+' ignored;
    # a component on a net twice (u8 A1, A2) is two pins
    idx = {n: i for i, n in enumerate(NAMES)}
    want = [["in0", "u1"], ["in1", "u3", "u4"], ["clk", "u5", "u6", "u9"], ["u1", "u2", "u3"], ["u2", "u4", "u7"],
            ["u3", "u5", "ram0"], ["u4", "u6", "u8", "u8", "u10"], ["u5", "u9"], ["u9", "out0", "u10", "ram0"]]
    ptr = [0]
    pins = []
    for net in want:
        pins += [idx[n] for n in net]
        ptr.append(len(pins))
    np.testing.assert_array_equal(nl["net_ptr"], ptr)
    np.testing.assert_array_equal(nl["pin_node"], pins)


def test_sizes_as_the_reference_reads_them(ap):
    """The reference keeps lefiMacro::sizeX/sizeY (microns) next to DEF
    coordinates in database units and ignores orientation."""
    with ap.Design.read(LEFS, DEF, size_mode=ap.design.SIZE_AS_READ) as d:
        nl = d.netlist()
    np.testing.assert_allclose(nl["node_w"][:7], np.float32([6.0, 0.38, 0.38, 0.57, 0.57, 3.23, 3.23]))
    np.testing.assert_allclose(nl["node_h"][:7], np.float32([4.2, 1.4, 1.4, 1.4, 1.4, 1.4, 1.4]))


def test_written_def_reads_back(ap, tmp_path):
    rng = np.random.default_rng(3)
    with ap.Design.read(LEFS, DEF) as d:
        nl = d.netlist()
        n = len(nl["node_w"])
        x = rng.uniform(0, 19000, n).astype(np.float32)
        y = rng.uniform(0, 19000, n).astype(np.float32)
        out = tmp_path / "placed.def"
        d.write_def(str(out), x, y)
    with ap.Design.read(LEFS, str(out)) as r:
        assert r.name == "tiny_core"
        assert [r.node_name(i) for i in range(16)] == NAMES
        back = r.netlist()
    mov = nl["node_fixed"] == 0
    np.testing.assert_array_equal(back["node_x"][mov], np.rint(x[mov]))
    np.testing.assert_array_equal(back["node_y"][mov], np.rint(y[mov]))
    # fixed components and IO pins stay where they were
    np.testing.assert_array_equal(back["node_x"][~mov], nl["node_x"][~mov])
    np.testing.assert_array_equal(back["node_y"][~mov], nl["node_y"][~mov])
    for k in ("net_ptr", "pin_node", "node_w", "node_h", "node_fixed", "die"):
        np.testing.assert_array_equal(back[k], nl[k])
    # a second round trip changes nothing
    with ap.Design.read(LEFS, str(out)) as r:
        out2 = tmp_path / "again.def"
        r.write_def(str(out2), back["node_x"], back["node_y"])
    assert out.read_text() == out2.read_text()


def test_reads_the_reference_directory_layout(ap, tmp_path):
    for f in ("tech.lef", "cells.lef", "floorplan.def"):
        shutil.copy(os.path.join(FIX, f), tmp_path / f)
    with ap.Design.read_dir(str(tmp_path)) as d:
        assert d.info()["num_nodes"] == 16
    os.remove(tmp_path / "floorplan.def")
    with pytest.raises(ap.APError) as e:
        ap.Design.read_dir(str(tmp_path))
    assert "floorplan.def" in str(e.value)


@pytest.mark.parametrize("edit,needle", [
    (("( u10 A )", "( u99 A )"), "unknown component u99"),
    (("( PIN in0 )", "( PIN nosuch )"), "unknown IO pin nosuch"),
    (("u5 DFF_X1", "u5 NOSUCHCELL"), "model NOSUCHCELL not defined"),
    (("DIEAREA ( 0 0 ) ( 20000 20000 ) ;", "DIEAREA ( 0 0 ) ;"), "DIEAREA"),
    (("END COMPONENTS", "END COMPONENT"), "END COMPONENTS"),
])
def test_errors_name_file_and_line(ap, tmp_path, edit, needle):
    text = open(DEF).read()
    assert edit[0] in text
    bad = tmp_path / "bad.def"
    bad.write_text(text.replace(edit[0], edit[1], 1))
    with pytest.raises(ap.APError) as e:
        ap.Design.read(LEFS, str(bad))
    assert e.value.status == 2 and needle in str(e.value)


def test_lef_macro_without_size_is_an_error(ap, tmp_path):
    bad = tmp_path / "bad.lef"
    bad.write_text(open(LEFS[1]).read().replace("  SIZE 0.57 BY 1.4 ;\n", "", 1))
    with pytest.raises(ap.APError) as e:
        ap.Design.read([LEFS[0], str(bad)], DEF)
    assert "NAND2_X1 has no SIZE" in str(e.value) and "bad.lef:" in str(e.value)


@pytest.mark.gpu
def test_read_place_write_reread(ap, tmp_path):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    with ap.Design.read(LEFS, DEF) as d:
        nl = d.netlist(bins=32, target_density=0.9)
        with ap.Placer(nl, field_solver="fp32") as pl:
            pl.initialize_placement(seed=3, sigma=500.0)
            pl.perform_iteration(50)
            s = pl.stats()
            x, y = pl.positions()
        assert s["status"] == 0 and np.isfinite(s["hpwl"])
        out = tmp_path / "placed.def"
        d.write_def(str(out), x, y)
    with ap.Design.read(LEFS, str(out)) as r:
        back = r.netlist()
    mov = nl["node_fixed"] == 0
    np.testing.assert_array_equal(back["node_x"][mov], np.rint(x[mov]))
    np.testing.assert_array_equal(back["node_y"][mov], np.rint(y[mov]))
    np.testing.assert_array_equal(back["node_x"][~mov], nl["node_x"][~mov])
    # the placer moved the movable cells and kept them on the die
    assert not np.array_equal(back["node_x"][mov], nl["node_x"][mov])
    assert (x[mov] >= 0).all() and (x[mov] + nl["node_w"][mov] <= 20000 + 0.5).all()
