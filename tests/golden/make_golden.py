"""Regenerates the golden fixtures in this folder from the reference checkout.

Run here (not on the GPU machine, which has no reference checkout):

    python tests/golden/make_golden.py <path of the reference checkout>

(it builds oracle/_ref/libref.so and oracle/_ref/libref_placer.so from the
reference sources first, through `make -C oracle ref refplacer REF=<path>`).

Sources of each fixture:
  aie_partials.npz   vck5000/aie/golden_data/partials/*.dat (createGoldenPartials.py:28-132)
  aie_dct.npz        vck5000/aie/golden_data/density/*.dat  (createGoldenDCT.py:103-205)
  computeterm.npz    python/AIEmath/computeTerm.py on seeded nets (fast_exp, gamma 4)
  customdct.npz      python/AIEmath/customDCT.py dct/idct/idxst on seeded vectors
  replace_field.npz  replace::FFT::doFFT (fft_replace/fft.cpp:204-299) via oracle/_ref
  ref_grid.npz       Grid::computeBinOverlaps/getRho/computeTotalOverflow and
                     Net::computeWirelength_HPWL via oracle/_ref
  ref_placer.npz     the reference's own Placer (vck5000/host/src/AIEplace.cpp)
                     via oracle/_ref/libref_placer.so on the inputs of
                     ref_placer_inputs.py: computeAllPartials_CPU partials,
                     computeOverlaps / getRho, computeTotalOverflow, nudgeNode
                     forces, computeTotalWirelength("HPWL"), the host DCT field
                     path (compute_a_uv_DCT / compute_eField_DCT)
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))


def read_dat(path):
    with open(path) as f:
        return np.array([float(t) for t in f.read().split()], dtype=np.float64)


def aie_partials(ref):
    d = os.path.join(ref, "vck5000", "aie", "golden_data", "partials")
    out = {}
    for b in range(4):
        x_in = read_dat(os.path.join(d, f"x_in{b}.dat"))
        out[f"ctrl{b}"] = x_in[:4]
        # after the 4 control words: for pin order [max, min], 8 lanes each
        out[f"x{b}"] = x_in[4:].reshape(2, 8)
        for name in ("a_plus", "a_minus", "partials"):
            out[f"{name}{b}"] = read_dat(os.path.join(d, f"{name}{b}.dat")).reshape(2, 8)
        for name in ("b_plus", "b_minus", "c_plus", "c_minus"):
            out[f"{name}{b}"] = read_dat(os.path.join(d, f"{name}{b}.dat"))
    np.savez_compressed(os.path.join(HERE, "aie_partials.npz"), **out)


def aie_dct(ref):
    d = os.path.join(ref, "vck5000", "aie", "golden_data", "density")
    out = {}
    inp = read_dat(os.path.join(d, "input.dat"))
    # complex pairs; the shipped file stops after 127.5 pairs (rows 0-7 complete)
    n_re = (len(inp) + 1) // 2
    re = inp[0::2][:n_re]
    out["input_rows0_7"] = re[:128].reshape(8, 16)
    for name in ("dct_output", "dct_2d_output", "idct_output", "idxst_output", "idct_2d_output",
                 "idxst_2d_output"):
        v = read_dat(os.path.join(d, f"{name}.dat"))
        out[name] = v[0::2].reshape(16, 16)
    np.savez_compressed(os.path.join(HERE, "aie_dct.npz"), **out)


def computeterm(ref):
    sys.path.insert(0, os.path.join(ref, "python", "AIEmath"))
    import computeTerm  # noqa: E402  (reference module, read-only import)

    rng = np.random.default_rng(20240601)
    out = {}
    k = 0
    for deg in range(2, 9):
        for rep in range(6):
            lo = int(rng.integers(0, 10000))
            xs = sorted(int(v) for v in rng.integers(lo, lo + 30 * deg, size=deg))
            g = 4
            ap = computeTerm.a_plus(xs, g)
            am = computeTerm.a_minus(xs, g)
            bp, bm = computeTerm.b_term(ap), computeTerm.b_term(am)
            cp, cm = computeTerm.c_term(xs, ap), computeTerm.c_term(xs, am)
            part = [computeTerm.WA_partial(xs[i], ap[i], bp, cp, am[i], bm, cm, g) for i in range(deg)]
            out[f"x{k}"] = np.array(xs, dtype=np.float64)
            out[f"ap{k}"] = np.array(ap)
            out[f"am{k}"] = np.array(am)
            out[f"bc{k}"] = np.array([bp, cp, bm, cm])
            out[f"part{k}"] = np.array(part)
            k += 1
    out["count"] = np.array(k)
    np.savez_compressed(os.path.join(HERE, "computeterm.npz"), **out)


def customdct(ref):
    sys.path.insert(0, os.path.join(ref, "python", "AIEmath"))
    import customDCT  # noqa: E402

    rng = np.random.default_rng(7)
    out = {}
    for n in (8, 16, 32):
        v = rng.random(n)
        out[f"in{n}"] = v
        out[f"dct{n}"] = np.array(customDCT.dct(list(v)))
        out[f"idct{n}"] = np.array(customDCT.idct(list(v)))
        out[f"idxst{n}"] = np.array(customDCT.idxst(list(v)))
    np.savez_compressed(os.path.join(HERE, "customdct.npz"), **out)


def replace_field(R):
    out = {}
    cases = {"run_fft4": np.array([[1, 1, 99, 99], [1, 1, 99, 99], [99] * 4, [99] * 4], np.float32)}
    rng = np.random.default_rng(11)
    for m in (16, 32, 64):
        cases[f"rand{m}"] = rng.random((m, m)).astype(np.float32)
    for name, d in cases.items():
        m = d.shape[0]
        ex, ey, phi = (np.zeros(m * m, np.float32) for _ in range(3))
        R.ref_replace_field(m, np.ascontiguousarray(d.reshape(-1)), phi.ctypes.data, ex, ey)
        out[f"{name}_density"] = d
        out[f"{name}_phi"] = phi.reshape(m, m)
        out[f"{name}_ex"] = ex.reshape(m, m)
        out[f"{name}_ey"] = ey.reshape(m, m)
    np.savez_compressed(os.path.join(HERE, "replace_field.npz"), **out)


def ref_grid(R):
    rng = np.random.default_rng(5)
    out = {}
    # nodes straddling the die edge, small (area <= bin/16) and large ones
    n, W, M = 2000, 40.0, 32
    x = rng.uniform(-2.0, W, n).astype(np.float32)
    y = rng.uniform(-2.0, W, n).astype(np.float32)
    w = rng.choice([0.05, 0.2, 0.5, 1.0, 2.5, 6.0], n).astype(np.float32)
    h = rng.choice([0.05, 0.3, 1.0, 1.7], n).astype(np.float32)
    rho = np.zeros(M * M, np.float32)
    ov = C.c_double()
    R.ref_density(n, x, y, w, h, W, W, M, rho, C.byref(ov))
    out.update(x=x, y=y, w=w, h=h, die=np.array([W, W], np.float32), m=np.array(M), rho=rho,
               overflow=np.array(ov.value))
    # HPWL of a small netlist
    nn, ne = 300, 200
    px = rng.uniform(0, 100, nn).astype(np.float32)
    py = rng.uniform(0, 100, nn).astype(np.float32)
    deg = rng.integers(1, 9, ne)
    ptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    pins = np.concatenate([rng.choice(nn, d, replace=False) for d in deg]).astype(np.int32)
    hp = R.ref_hpwl(nn, ne, ptr, pins, px, py)
    out.update(hp_x=px, hp_y=py, hp_ptr=ptr, hp_pins=pins, hpwl=np.array(hp))
    np.savez_compressed(os.path.join(HERE, "ref_grid.npz"), **out)


def ref_placer(ref):
    """Per case: the reference Placer's partials and nudge forces of every
    SUBSAMPLE-th node, its density map and absolute overflow, its HPWL."""
    import oracle
    import ref_placer_inputs as I

    sys.path.insert(0, REPO)
    from aieplace_gb300.presets import PRESETS

    out = {}
    for name in I.CASES:
        nl = I.small_nets(oracle.synth_generate(PRESETS[name], seed=I.SEED))
        x, y = I.positions(nl)
        die, M = nl["die"], nl["bins"]
        with oracle.quiet_stdout():
            rp = oracle.RefPlacer(nl["net_ptr"], nl["pin_node"], nl["node_w"], nl["node_h"], x, y,
                                  nl["node_fixed"], float(die[2]), float(die[3]), M, gamma=I.GAMMA,
                                  learning_rate=I.LEARNING_RATE, global_lambda=I.GLOBAL_LAMBDA)
            gx, gy, _ = rp.partials()
            rho, ovf, _ = rp.overlaps()
            ex, ey = I.field(M)
            zero = np.zeros(len(x), np.float32)
            mx, my, _ = rp.nudge(ex, ey, zero, zero)
            hp = rp.hpwl()
            if M <= 128:  # the host DCT path (naive O(M^3) transforms) at the two small sizes
                dex, dey, _ = rp.fields_dct()
                out.update({f"{name}_dct_ex": dex, f"{name}_dct_ey": dey})
        rp.close()
        # nudgeNode's move is learning_rate min(W, H) global_lambda F (zero partials)
        coeff = np.float32(I.LEARNING_RATE) * np.float32(min(float(die[2]), float(die[3]))) * np.float32(
            I.GLOBAL_LAMBDA)
        sub = slice(0, None, I.SUBSAMPLE)
        out.update({f"{name}_gx": gx[sub], f"{name}_gy": gy[sub], f"{name}_fx": (mx / coeff)[sub],
                    f"{name}_fy": (my / coeff)[sub], f"{name}_rho": rho, f"{name}_overflow": np.array(ovf),
                    f"{name}_hpwl": np.array(hp), f"{name}_n_nets": np.array(len(nl["net_ptr"]) - 1)})
    np.savez_compressed(os.path.join(HERE, "ref_placer.npz"), **out)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AP_REFERENCE_DIR", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py <path of the searsm8/AIEplace checkout> (or set AP_REFERENCE_DIR)")
    import oracle  # noqa: E402

    oracle.build(with_ref=True, ref_dir=ref)
    R = oracle.ref_lib()
    assert R is not None, "oracle/_ref/libref.so did not build"
    assert oracle.ref_placer_lib() is not None, "oracle/_ref/libref_placer.so did not build"
    aie_partials(ref)
    aie_dct(ref)
    computeterm(ref)
    customdct(ref)
    replace_field(R)
    ref_grid(R)
    ref_placer(ref)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
