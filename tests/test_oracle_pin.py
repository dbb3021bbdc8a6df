"""Pin the oracle (C restatement of src/cpp) to the reference's own outputs.

The fixtures under tests/golden/ were produced by the reference itself
(tests/golden/make_golden.py runs tmarschall/spherocyls' src/cpp compiled in
oracle/_ref).  The restatement uses the reference's operation order with
-ffp-contract=off, so on the machine that made the fixtures it must agree to
the last bit; on another machine only libm's cos/sin/pow may differ, so the
comparison allows 1e-13 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, periodic_diff

TOL_PIN = 1e-13


def _close(a, b, scale, tol=TOL_PIN):
    a, b = np.asarray(a), np.asarray(b)
    return np.all(np.abs(a - b) <= tol * max(scale, 1e-300))


def _box_from(g, cls, **kw):
    return cls(float(g["L"]), g["x"], g["y"], g["phi"], g["A"], g["R"], **kw)


def _check_snapshot(box, g, prefix, L, se_cols=4):
    x, y, p = box.state()
    assert np.max(np.abs(periodic_diff(x, g[prefix + "x"], L))) <= TOL_PIN * L
    assert np.max(np.abs(periodic_diff(y, g[prefix + "y"], L))) <= TOL_PIN * L
    assert np.max(np.abs(periodic_diff(p, g[prefix + "phi"], 2 * 3.14159265358979))) <= 1e-12
    f = np.array(box.forces())
    fg = np.stack([g[prefix + "fx"], g[prefix + "fy"], g[prefix + "tau"]])
    rms = np.sqrt(np.mean(fg ** 2)) + 1e-300
    assert np.max(np.abs(f - fg)) <= TOL_PIN * rms * 10
    if prefix + "se" in g:
        se = box.se()
        sg = g[prefix + "se"]
        for k in range(se_cols):
            assert abs(se[k] - sg[k]) <= TOL_PIN * max(abs(sg[k]), 1e-3 * abs(sg[0]), 1e-300)


@pytest.mark.parametrize("name", ["shear_n1024_phi085", "shear_n256_setback", "shear_n512_autopad"])
def test_oracle_shear_matches_reference_fixture(oracle_built, name):
    g = load_golden(name)
    rate, dt, pad = g["params"]
    ob = _box_from(g, oracle_built.OracleBox, pad=pad, strain_rate=rate, step=dt)
    pairs = ob.pairs()
    assert np.array_equal(pairs, g["pairs0"])  # same pairs in the same list order
    ob.calc_se()
    L = float(g["L"])
    _check_snapshot(ob, g, "s0_", L, se_cols=5)
    done = 0
    traces = []
    for cp in g["checkpoints"]:
        tr = ob.run_strain_steps(int(cp) - done, record_se="se_trace" in g)
        if tr is not None:
            traces.append(tr)
        done = int(cp)
        ob.calc_se()
        _check_snapshot(ob, g, f"s{int(cp)}_", L)
        sc = ob.scalars()
        bx = g[f"s{int(cp)}_box"]
        assert sc["gamma"] == bx[2] and sc["gamma_total"] == bx[3]
    if traces:
        tr = np.concatenate(traces)
        ref = g["se_trace"]
        scale = np.max(np.abs(ref[:, :4]), axis=0)
        assert np.all(np.abs(tr[:, :4] - ref[:, :4]) <= TOL_PIN * scale)


@pytest.mark.parametrize("name", ["resize_n256_shrink", "resize_n256_grow"])
def test_oracle_resize_matches_reference_fixture(oracle_built, name):
    g = load_golden(name)
    rate, dt, pad, shrink = g["params"]
    ob = _box_from(g, oracle_built.OracleBox, pad=pad, resize_rate=rate, step=dt)
    ob.calc_se()
    done = 0
    for cp in g["checkpoints"]:
        ob.run_resize_steps(int(cp) - done, bool(shrink))
        done = int(cp)
        ob.calc_se()
        bx = g[f"s{int(cp)}_box"]
        sc = ob.scalars()
        assert abs(sc["Lx"] - bx[0]) <= 1e-15 * bx[0]
        _check_snapshot(ob, g, f"s{int(cp)}_", bx[0])


def test_oracle_gd_matches_reference_fixture(oracle_built):
    g = load_golden("gd_n256")
    dt, pad, nsteps = g["params"]
    ob = _box_from(g, oracle_built.OracleBox, pad=pad, step=dt)
    steps, etrace = ob.run_gd_steps(int(nsteps), 0.0)
    assert steps == int(g["steps"])
    assert np.all(np.abs(etrace - g["e_trace"]) <= TOL_PIN * np.max(np.abs(g["e_trace"])))
    ob.calc_se()
    _check_snapshot(ob, g, "end_", float(g["L"]))


def test_oracle_pair_geometry_matches_reference_fixture(oracle_built):
    g = load_golden("pair_geometry")
    for name in g["names"]:
        x0, y0, p0, x1, y1, p1, gam = g[name + "_in"]
        ob = oracle_built.OracleBox(float(g["L"]), [x0, x1], [y0, y1], [p0, p1], g["A"], g["R"], 0.1,
                                    gamma=gam)
        ob.calc_se()
        f = np.array(ob.forces())
        assert np.allclose(f, g[name + "_f"], rtol=0, atol=1e-15), name
        assert np.allclose(ob.se(), g[name + "_se"], rtol=1e-14, atol=1e-18), name
        assert np.array_equal(ob.pairs(), g[name + "_pairs"]), name


def test_oracle_matches_live_reference_when_available(oracle_built):
    """Where the reference checkout is present, compare step by step, bitwise."""
    if not oracle_built.ref_available():
        pytest.skip("reference build oracle/_ref not available here")
    g = load_golden("shear_n256_setback")
    kw = dict(pad=0.1, strain_rate=0.05, step=0.02)
    ob = _box_from(g, oracle_built.OracleBox, **kw)
    rb = _box_from(g, oracle_built.RefBox, **kw)
    for _ in range(6):
        so = ob.run_strain_steps(100, record_se=True)
        sr = rb.run_strain_steps(100, record_se=True)
        assert np.array_equal(so, sr)
        assert np.array_equal(np.array(ob.state()), np.array(rb.state()))
        assert np.array_equal(ob.pairs(), rb.pairs())
    assert ob.scalars() == rb.scalars()


@pytest.mark.parametrize("n,phi,aor,seed", [(2, 0.5, 1.0, 0), (600, 0.84, 1.0, 3),
                                            (5000, 0.86, 0.5, 1), (3000, 0.80, 2.0, 7)])
def test_oracle_generator_equals_library_generator(library, oracle_built, n, phi, aor, seed):
    """The CPU reference arm of the benchmark generates its input packing with the
    oracle's restatement of the library's generator: both give the same packing bit
    for bit, so the two arms run the same workload."""
    import spherocyls_gb300 as sc

    a = oracle_built.generate_packing(n, phi, aor, seed=seed)
    b = sc.generate_packing(n, phi, aor, seed=seed)
    assert a[0] == b[0]
    for u, v in zip(a[1:], b[1:]):
        assert np.array_equal(u, v)
