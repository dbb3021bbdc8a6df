"""Generate the golden fixtures in this directory from the reference itself.

The reference (tmarschall/spherocyls) ships no tests or golden vectors, so the
fixtures are produced here by running the reference's own src/cpp sources,
compiled where they lie by ``oracle/Makefile`` into ``oracle/_ref/`` and driven
through ``oracle/ref_driver.cpp``.  Each fixture stores its inputs and the
reference's outputs (positions, forces, stress/energy, half neighbour lists) so
that the tests can pin the oracle and the CUDA library without the reference
checkout.  Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import RefBox  # noqa: E402
from spherocyls_gb300.box import generate_packing  # noqa: E402


def snapshot(box, prefix: str, out: dict, se: bool = True) -> None:
    x, y, p = box.state()
    fx, fy, t = box.forces()
    out[prefix + "x"], out[prefix + "y"], out[prefix + "phi"] = x, y, p
    out[prefix + "fx"], out[prefix + "fy"], out[prefix + "tau"] = fx, fy, t
    sc = box.scalars()
    out[prefix + "box"] = np.array([sc[k] for k in ("Lx", "Ly", "gamma", "gamma_total", "pad",
                                                    "W", "H", "packing", "rows", "cols")])
    if se:
        out[prefix + "se"] = box.se()


def packing_inputs(n, phi, a_over_r, seed, min_sep=0.1):
    L, x, y, p, R, A = generate_packing(n, phi, a_over_r, seed=seed, min_sep=min_sep)
    return dict(L=np.array(L), x=x, y=y, phi=p, R=R, A=A)


def case_shear(name, n, phi, a_over_r, seed, rate, dt, pad, checkpoints, record_every_step):
    inp = packing_inputs(n, phi, a_over_r, seed)
    out = dict(inp)
    out["params"] = np.array([rate, dt, pad])
    b = RefBox(inp["L"], inp["x"], inp["y"], inp["phi"], inp["A"], inp["R"], pad,
               strain_rate=rate, step=dt)
    out["pairs0"] = b.pairs()
    b.calc_se()
    snapshot(b, "s0_", out)
    done = 0
    se_trace = []
    for cp in checkpoints:
        se = b.run_strain_steps(cp - done, record_se=record_every_step)
        if se is not None:
            se_trace.append(se)
        done = cp
        b.calc_se()
        snapshot(b, f"s{cp}_", out)
    out["checkpoints"] = np.array(checkpoints)
    if se_trace:
        out["se_trace"] = np.concatenate(se_trace)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    b.close()


def case_resize(name, n, phi, a_over_r, seed, rate, dt, pad, shrink, checkpoints):
    inp = packing_inputs(n, phi, a_over_r, seed)
    out = dict(inp)
    out["params"] = np.array([rate, dt, pad, float(shrink)])
    b = RefBox(inp["L"], inp["x"], inp["y"], inp["phi"], inp["A"], inp["R"], pad,
               resize_rate=rate, step=dt)
    b.calc_se()
    snapshot(b, "s0_", out)
    done = 0
    for cp in checkpoints:
        b.run_resize_steps(cp - done, shrink)
        done = cp
        b.calc_se()
        snapshot(b, f"s{cp}_", out)
    out["checkpoints"] = np.array(checkpoints)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    b.close()


def case_gd(name, n, phi, a_over_r, seed, dt, pad, nsteps):
    inp = packing_inputs(n, phi, a_over_r, seed)
    out = dict(inp)
    out["params"] = np.array([dt, pad, float(nsteps)])
    b = RefBox(inp["L"], inp["x"], inp["y"], inp["phi"], inp["A"], inp["R"], pad, step=dt)
    steps, etrace = b.run_gd_steps(nsteps, 0.0)
    out["steps"] = np.array(steps)
    out["e_trace"] = etrace
    b.calc_se()
    snapshot(b, "end_", out)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    b.close()


def case_pairs_geometry(name):
    """Two-particle contacts: parallel, T, end-to-end, across x, across y with shear."""
    L = 8.0
    R = np.array([0.5, 0.5])
    A = np.array([0.5, 0.5])
    cases = {
        # (x0, y0, phi0, x1, y1, phi1, gamma)
        "parallel": (4.0, 4.0, 0.0, 4.3, 4.9, 0.0, 0.0),
        "tee": (4.0, 4.0, 0.0, 4.2, 4.85, np.pi / 2, 0.0),
        "end_to_end": (4.0, 4.0, 0.0, 5.9, 4.05, 0.1, 0.0),
        "crossing_x_boundary": (0.2, 4.0, 0.3, 7.3, 4.2, -0.4, 0.0),
        "crossing_y_boundary_sheared": (4.0, 0.2, 1.0, 4.5, 7.4, 2.0, 0.3),
        "oblique": (4.0, 4.0, 0.7, 4.6, 4.8, 2.2, 0.0),
    }
    out = {"L": np.array(L), "R": R, "A": A, "names": np.array(list(cases.keys()))}
    for key, (x0, y0, p0, x1, y1, p1, g) in cases.items():
        b = RefBox(L, np.array([x0, x1]), np.array([y0, y1]), np.array([p0, p1]), A, R, 0.1,
                   gamma=g)
        b.calc_se()
        out[key + "_in"] = np.array([x0, y0, p0, x1, y1, p1, g])
        out[key + "_f"] = np.array(b.forces())
        out[key + "_se"] = b.se()
        out[key + "_pairs"] = b.pairs()
        b.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def main() -> None:
    import __graft_entry__

    __graft_entry__.ref_env()  # $SPHEROCYLS_REF: the reference checkout to compile
    oracle.build(with_ref=True)
    if not oracle.ref_available():
        raise SystemExit("the reference build oracle/_ref is needed to make the fixtures")
    # config-1 shape (N=1024, phi=0.85, a=R, rate 1e-5, dt 0.02), first 100 steps
    case_shear("shear_n1024_phi085", 1024, 0.85, 1.0, 0, 1e-5, 0.02, 0.1, [1, 10, 100], True)
    # a faster shear that crosses gamma = 0.5 (Lees-Edwards set-back) at step 500
    case_shear("shear_n256_setback", 256, 0.85, 1.0, 7, 0.05, 0.02, 0.1, [1, 250, 520], False)
    # automatic padding (pad = 0), longer shafts
    case_shear("shear_n512_autopad", 512, 0.82, 2.0, 11, 1e-3, 0.02, 0.0, [1, 50], True)
    case_resize("resize_n256_shrink", 256, 0.80, 1.0, 3, 1e-3, 0.02, 0.1, True, [1, 100, 300])
    case_resize("resize_n256_grow", 256, 0.86, 1.0, 5, 1e-3, 0.02, 0.1, False, [1, 100])
    case_gd("gd_n256", 256, 0.85, 1.0, 9, 0.1, 0.1, 150)
    case_pairs_geometry("pair_geometry")
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
