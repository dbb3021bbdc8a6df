"""Parity of the CUDA library (through its C ABI) with the reference's CPU path.

Plain FP64 form: positions, angles, forces, stress and energy agree with the
reference's own outputs (tests/golden/, made by the reference itself) and with the
oracle within TOL = 1e-12 relative over the first 100 steps, the tolerance the
plain form is specified to meet.  Neighbour lists agree as sets of pairs, exactly.

Positions are compared modulo the box and angles modulo 2*pi_ref: the reference
wraps them only when it rebuilds its lists, and rebuild timing is not part of
the result (any list that contains all pairs within reach gives the same forces).
Pyx is compared only on the first stress evaluation: the reference never resets
it between calls (src/cpp/spherocyl_box.cpp:509-512), the library does.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import REF_PI, load_golden, periodic_diff

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative tolerance of the plain FP64 form


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


def _gpu_box(sc, g, pad, precision="fp64", **kw):
    return sc.SpherocylBox(float(g["L"]), g["x"], g["y"], g["phi"], g["A"], g["R"], pad,
                           precision=precision, **kw)


def _assert_state(box, g, prefix, L, tol=TOL):
    x, y, p = box.state()
    ex = np.max(np.abs(periodic_diff(x, g[prefix + "x"], L)))
    ey = np.max(np.abs(periodic_diff(y, g[prefix + "y"], L)))
    ep = np.max(np.abs(periodic_diff(p, g[prefix + "phi"], 2 * REF_PI)))
    assert ex <= tol * L and ey <= tol * L, (prefix, ex, ey)
    assert ep <= tol * 2 * REF_PI, (prefix, ep)


def _assert_forces(box, g, prefix, tol=TOL):
    f = np.array(box.forces())
    fg = np.stack([g[prefix + "fx"], g[prefix + "fy"], g[prefix + "tau"]])
    rms = np.sqrt(np.mean(fg ** 2))
    err = np.max(np.abs(f - fg))
    assert err <= tol * rms, (prefix, err, rms)


def _assert_se(se, sg, ncols=4, tol=TOL):
    scale = max(abs(sg[0]), np.max(np.abs(sg[1:4])))
    for k in range(ncols):
        assert abs(se[k] - sg[k]) <= tol * scale, (k, se[k], sg[k])


@pytest.mark.parametrize("name", ["shear_n1024_phi085", "shear_n256_setback", "shear_n512_autopad"])
@pytest.mark.parametrize("graphs", [False, True])
def test_fp64_shear_matches_reference(sc, name, graphs):
    g = load_golden(name)
    rate, dt, pad = g["params"]
    L = float(g["L"])
    box = _gpu_box(sc, g, pad, use_graphs=graphs)
    box.set_strain_rate(rate)
    box.set_step(dt)
    # neighbour list of the initial state: the same set of pairs
    pairs = box.pairs()
    ref_pairs = np.sort(g["pairs0"].view([("p", np.int32), ("q", np.int32)]), axis=0)
    assert np.array_equal(pairs, ref_pairs.view(np.int32).reshape(-1, 2))
    se0 = box.calc_se()
    _assert_se(se0, g["s0_se"], ncols=5)
    _assert_forces(box, g, "s0_")
    done = 0
    traces = []
    for cp in g["checkpoints"]:
        cp = int(cp)
        rec = box.strain_steps(cp - done, se_every=1 if "se_trace" in g else 0)
        if rec is not None:
            traces.append(rec[:, 0, :])
        done = cp
        bx = g[f"s{cp}_box"]
        b = box.box()
        assert b["gamma"] == bx[2] and b["gamma_total"] == bx[3]
        _assert_state(box, g, f"s{cp}_", L)
        box.calc_se()
        _assert_forces(box, g, f"s{cp}_")
        _assert_se(box.calc_se(), g[f"s{cp}_se"])
    if traces:
        tr = np.concatenate(traces)
        ref = g["se_trace"]
        for k in range(4):
            assert np.max(np.abs(tr[:, k] - ref[:, k])) <= TOL * np.max(np.abs(ref[:, :4]))


@pytest.mark.parametrize("name", ["resize_n256_shrink", "resize_n256_grow"])
def test_fp64_resize_matches_reference(sc, name):
    g = load_golden(name)
    rate, dt, pad, shrink = g["params"]
    box = _gpu_box(sc, g, pad)
    box.set_resize_rate(rate)
    box.set_step(dt)
    done = 0
    for cp in g["checkpoints"]:
        cp = int(cp)
        box.resize_steps(cp - done, shrink=bool(shrink))
        done = cp
        bx = g[f"s{cp}_box"]
        b = box.box()
        assert b["Lx"] == bx[0] and b["Ly"] == bx[1]
        _assert_state(box, g, f"s{cp}_", bx[0])
        box.calc_se()
        _assert_forces(box, g, f"s{cp}_")
        _assert_se(box.calc_se(), g[f"s{cp}_se"])


def test_fp64_gradient_descent_matches_reference(sc):
    g = load_golden("gd_n256")
    dt, pad, nsteps = g["params"]
    box = _gpu_box(sc, g, pad)
    box.set_step(dt)
    steps, e_final = box.gd_minimize(int(nsteps), 0.0)
    assert steps == int(g["steps"])
    _assert_state(box, g, "end_", float(g["L"]))
    se = box.calc_se()
    _assert_se(se, g["end_se"])


def test_fp64_pair_geometry_matches_reference(sc):
    g = load_golden("pair_geometry")
    for name in g["names"]:
        x0, y0, p0, x1, y1, p1, gam = g[name + "_in"]
        box = sc.SpherocylBox(float(g["L"]), [x0, x1], [y0, y1], [p0, p1], g["A"], g["R"], 0.1)
        box.set_gamma(gam)
        se = box.calc_se()
        f = np.array(box.forces())
        fg = g[name + "_f"]
        assert np.max(np.abs(f - fg)) <= TOL * max(np.abs(fg).max(), 1e-300), name
        _assert_se(se, g[name + "_se"], ncols=5)
        assert np.array_equal(box.pairs(), g[name + "_pairs"]), name
        box.close()


def test_fp64_matches_oracle_long_run_with_setback(sc, oracle_built):
    """Oracle and library side by side over 600 steps through a gamma set-back."""
    g = load_golden("shear_n256_setback")
    L = float(g["L"])
    kw = dict(strain_rate=0.05, step=0.02)
    ob = oracle_built.OracleBox(L, g["x"], g["y"], g["phi"], g["A"], g["R"], 0.1, **kw)
    box = _gpu_box(sc, g, 0.1)
    box.set_strain_rate(kw["strain_rate"])
    box.set_step(kw["step"])
    for _ in range(6):
        se_o = ob.run_strain_steps(100, record_se=True)
        se_g = box.strain_steps(100, se_every=10)[:, 0, :]
        x, y, p = box.state()
        ox, oy, op = ob.state()
        assert np.max(np.abs(periodic_diff(x, ox, L))) <= TOL * L
        assert np.max(np.abs(periodic_diff(y, oy, L))) <= TOL * L
        _assert_se(se_g[-1], se_o[-1])
    assert box.box()["gamma"] == ob.scalars()["gamma"]


def test_neighbour_lists_equal_reference_sets_random_states(sc, oracle_built):
    """Bit-exact list sets for identical positions at several gamma values."""
    for seed, gam in [(1, 0.0), (2, 0.37), (3, -0.49), (4, 0.4999)]:
        L, x, y, p, R, A = sc.generate_packing(400, 0.84, 1.5, seed=seed)
        ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.15, gamma=gam)
        ob.find_neighbors()
        box = sc.SpherocylBox(L, x, y, p, A, R, 0.15)
        box.set_gamma(gam)
        ref = ob.pairs()
        ref = ref[np.lexsort((ref[:, 1], ref[:, 0]))]
        assert np.array_equal(box.pairs(), ref), (seed, gam)


def test_mixed_precision_against_fp64(sc, oracle_built):
    """Same configuration as the reference's fixtures: the mixed form's FP32 pair
    forces are within 1e-4 of the RMS force; its stress and energy, evaluated in FP64
    from its compensated state, are within 1e-9 of the reference's own values,
    each component relative to its own magnitude (Pxy included: a relative error of
    the shear stress, not one on the scale of the normal stress)."""
    g = load_golden("shear_n1024_phi085")
    L = float(g["L"])
    for prefix in ("s0_", "s100_"):
        box = sc.SpherocylBox(L, g[prefix + "x"], g[prefix + "y"], g[prefix + "phi"], g["A"],
                              g["R"], 0.1, precision="mixed")
        box.set_gamma(g[prefix + "box"][2])
        se = box.calc_se()
        _assert_forces(box, g, prefix, tol=1e-4)
        sg = g[prefix + "se"]
        for k in range(4):
            assert abs(se[k] - sg[k]) <= 1e-9 * abs(sg[k]), (prefix, k, se[k], sg[k])


def test_mixed_shear_stress_per_step_against_fp64(sc):
    """The precision A/B of the N = 16384 shear workload (packing 0.86, a = R, strain
    rate 1e-4, dt 0.02, seed 1, padding 0.2): from one sheared state (300 FP64 steps
    after the generated packing) the mixed and FP64 forms each run 20 steps with
    stress and energy recorded every step.  Over the first 5 steps the mixed form's
    shear stress is within 1e-6 of the FP64 run's, relative to |Pxy|, and its
    energy within 1e-6 relative.  The FP32 pair forces (about 1e-6 relative error
    per contact at these overlaps) then move the trajectories apart: the shear
    stress of the two runs differs by more than 1e-6 from about step 6 on (measured
    2e-4 at step 10), while the time averages agree within their statistical error
    (the long-run ensemble test below and the benchmark's precision A/B)."""
    L, x, y, p, R, A = sc.generate_packing(16384, 0.86, 1.0, seed=1)
    prep = sc.SpherocylBox(L, x, y, p, A, R, 0.2)
    prep.set_strain_rate(1e-4)
    prep.set_step(0.02)
    prep.strain_steps(300)
    x, y, p = prep.state()
    bx = prep.box()
    prep.close()
    out = {}
    for precision in ("fp64", "mixed"):
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision=precision)
        b.set_strain_rate(1e-4)
        b.set_step(0.02)
        b.set_gamma(bx["gamma"])
        b.set_total_gamma(bx["gamma_total"])
        out[precision] = b.strain_steps(5, se_every=1)[:, 0, :]
        b.close()
    a, m = out["fp64"], out["mixed"]
    rel_e = np.abs(m[:, 0] - a[:, 0]) / np.abs(a[:, 0])
    rel_pxy = np.abs(m[:, 3] - a[:, 3]) / np.abs(a[:, 3])
    assert np.all(np.abs(a[:, 3]) > 0)
    assert rel_e.max() <= 1e-6, rel_e.max()
    assert rel_pxy.max() <= 1e-6, (rel_pxy.max(), int(np.argmax(rel_pxy)))


def test_mixed_precision_shear_tracks_fp64(sc):
    """100 mixed steps stay close to 100 FP64 steps (short-time, before chaos)."""
    g = load_golden("shear_n1024_phi085")
    L = float(g["L"])
    rate, dt, pad = g["params"]
    a = _gpu_box(sc, g, pad, precision="fp64")
    b = _gpu_box(sc, g, pad, precision="mixed")
    for box in (a, b):
        box.set_strain_rate(rate)
        box.set_step(dt)
    sa = a.strain_steps(100, se_every=10)
    sb = b.strain_steps(100, se_every=10)
    xa, ya, _ = a.state()
    xb, yb, _ = b.state()
    assert np.max(np.abs(periodic_diff(xa, xb, L))) < 1e-4
    assert np.all(np.abs(sa[:, 0, 0] - sb[:, 0, 0]) <= 1e-4 * np.abs(sa[:, 0, 0]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_systems_match_single_runs(sc, precision):
    """Several systems of different size in one handle advance exactly as alone, and
    record the same stress and energy (the third system's slots start inside a block
    of the stress kernels)."""
    specs = [(256, 0.85, 1.0, 1e-3, 21), (400, 0.80, 0.5, 5e-4, 22), (300, 0.88, 2.0, 2e-3, 23)]
    packs = [sc.generate_packing(n, phi, a, seed=s) for n, phi, a, _, s in specs]
    singles, single_se = [], []
    for (n, phi, a, rate, s), (L, x, y, p, R, A) in zip(specs, packs):
        box = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=precision)
        box.set_strain_rate(rate)
        box.set_step(0.02)
        single_se.append(box.strain_steps(150, se_every=50))
        singles.append(np.concatenate(box.state()))
    batch = sc.BoxBatch([sp[0] for sp in specs], [pk[0] for pk in packs],
                        np.concatenate([pk[1] for pk in packs]),
                        np.concatenate([pk[2] for pk in packs]),
                        np.concatenate([pk[3] for pk in packs]),
                        np.concatenate([pk[5] for pk in packs]),
                        np.concatenate([pk[4] for pk in packs]), 0.1, precision=precision)
    for i, sp in enumerate(specs):
        batch.set_strain_rate(sp[3], sys=i)
    batch.set_step(0.02)
    se = batch.strain_steps(150, se_every=50)
    x, y, p = batch.state()
    off = 0
    for i, sp in enumerate(specs):
        n = sp[0]
        got = np.concatenate([x[off:off + n], y[off:off + n], p[off:off + n]])
        assert np.array_equal(got, singles[i]), i
        assert np.array_equal(se[:, i, :], single_se[i][:, 0, :]), i
        off += n


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_and_eager_paths_bitwise_identical(sc, precision):
    """Captured chunks (with the conditional rebuild node) and eager launches run the
    same kernels in the same order, so the trajectories agree bit for bit."""
    L, x, y, p, R, A = sc.generate_packing(2000, 0.85, 1.0, seed=31)
    out = []
    for graphs in (False, True):
        box = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=precision, use_graphs=graphs)
        box.set_strain_rate(0.02)
        box.set_step(0.02)
        se = box.strain_steps(300, se_every=50)
        out.append((np.concatenate(box.state()), se, box.counters()["rebuilds"]))
    assert out[0][2] == out[1][2] and out[0][2] > 1
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_autotune_keeps_state_and_physics(sc):
    """The autotuner times copies of the handle: the live state is not advanced, and
    the tuned run follows an untuned one (same mixed-form tolerance as above)."""
    L, x, y, p, R, A = sc.generate_packing(4096, 0.85, 1.0, seed=11)
    boxes = []
    for tune in (True, False):
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision="mixed")
        b.set_strain_rate(1e-4)
        b.set_step(0.02)
        b.strain_steps(50)
        if tune:
            s0 = np.concatenate(b.state())
            f, blk = b.autotune(20)
            assert f in (0.5, 1.0, 1.5, 2.0, 3.0) and blk in (64, 128)
            assert np.max(np.abs(np.concatenate(b.state()) - s0)) < 1e-12 * L
        boxes.append(b)
    se = [b.strain_steps(200, se_every=200)[-1, 0] for b in boxes]
    assert abs(se[0][0] - se[1][0]) <= 1e-4 * abs(se[1][0])
    xa = np.array(boxes[0].state())
    xb = np.array(boxes[1].state())
    assert np.max(np.abs(periodic_diff(xa[:2], xb[:2], L))) < 1e-4


def test_mixed_and_fp64_ensemble_averages_agree(sc):
    """Long chaotic runs: the trajectories of the two forms separate after a few
    hundred steps, but the ensemble-averaged shear stress and energy of 16 sheared
    replicas agree within their statistical error (3 combined standard errors of
    the replica means, after a transient of strain 0.2)."""
    nrep, n = 16, 1024
    packs = [sc.generate_packing(n, 0.85, 1.0, seed=900 + k) for k in range(nrep)]
    args = ([n] * nrep, [pk[0] for pk in packs],
            np.concatenate([pk[1] for pk in packs]), np.concatenate([pk[2] for pk in packs]),
            np.concatenate([pk[3] for pk in packs]), np.concatenate([pk[5] for pk in packs]),
            np.concatenate([pk[4] for pk in packs]), 0.1)
    means = {}
    for precision in ("fp64", "mixed"):
        b = sc.BoxBatch(*args, precision=precision, stress="virial")
        b.set_strain_rate(1e-3)
        b.set_step(0.02)
        b.strain_steps(10000)
        rec = b.strain_steps(10000, se_every=100)  # (100, nrep, 5)
        means[precision] = rec.mean(axis=0)          # per-replica time averages
        b.close()
    for k, name in ((0, "E"), (3, "Pxy")):
        a, m = means["fp64"][:, k], means["mixed"][:, k]
        err = np.sqrt(a.var(ddof=1) / nrep + m.var(ddof=1) / nrep)
        assert abs(a.mean() - m.mean()) <= 3 * err, (name, a.mean(), m.mean(), err)
        assert abs(a.mean()) > 3 * a.std(ddof=1) / np.sqrt(nrep), name  # a resolved signal


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_flip_shear_reverses_the_configuration(sc, precision):
    """flip_shear_direction: x -> L - x, phi -> -phi, gamma -> -gamma leave the energy
    and the normal stresses unchanged and negate the shear stress; flipping twice
    gives the configuration back."""
    L, x, y, p, R, A = sc.generate_packing(1024, 0.85, 1.0, seed=17)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=precision, stress="virial")
    box.set_strain_rate(1e-3)
    box.set_step(0.02)
    box.strain_steps(200)
    se0 = box.calc_se()
    s0 = np.array(box.state())
    g0 = box.box()["gamma"]
    box.flip_shear()
    se1 = box.calc_se()
    tol = 1e-12 if precision == "fp64" else 1e-6
    scale = max(abs(se0[1]), abs(se0[2]))
    assert abs(se1[0] - se0[0]) <= tol * se0[0]
    assert abs(se1[1] - se0[1]) <= tol * scale and abs(se1[2] - se0[2]) <= tol * scale
    assert abs(se1[3] + se0[3]) <= tol * scale
    assert box.box()["gamma"] == -g0
    box.flip_shear()
    s2 = np.array(box.state())
    assert np.max(np.abs(periodic_diff(s2[:2], s0[:2], L))) < 1e-12 * L
    dphi = np.remainder(s2[2] - s0[2] + np.pi, 2 * np.pi) - np.pi  # rebuilds wrap phi
    assert np.max(np.abs(dphi)) < 1e-12


def test_rectangular_box_tiles_the_square_one(sc):
    """A rectangular box of two copies of a square packing side by side (Lx = 2L,
    Ly = L) is the same Lees-Edwards system: under shear it keeps the square box's
    energy per particle and stresses, through set-backs at gamma = 1/2 in the square
    box and gamma = 1 in the rectangular one (set_back_coords' Lx/Ly)."""
    # virial stress: the reference's compat Pxy keeps only the lower-index particle's
    # arm, and the copies change which particle of a pair has the lower index
    L, x, y, p, R, A = sc.generate_packing(512, 0.85, 1.0, seed=41)
    sq = sc.SpherocylBox(L, x, y, p, A, R, 0.1, stress="virial")
    rect = sc.SpherocylBox(2 * L, np.concatenate([x, x + L]), np.concatenate([y, y]),
                           np.concatenate([p, p]), np.concatenate([A, A]),
                           np.concatenate([R, R]), 0.1, Ly=L, stress="virial")
    for b in (sq, rect):
        b.set_strain_rate(0.5)
        b.set_step(0.02)
    a = sq.strain_steps(150, se_every=10)[:, 0]
    b = rect.strain_steps(150, se_every=10)[:, 0]
    assert rect.box()["Lx"] == 2 * L and rect.box()["Ly"] == L
    scale = np.max(np.abs(a[:, 1:3]), axis=1)
    assert np.all(np.abs(a[:, 0] - b[:, 0]) <= 1e-9 * a[:, 0])
    assert np.all(np.abs(a[:, 3] - b[:, 3]) <= 1e-9 * scale)


def test_rotate_shear_is_an_isometry(sc):
    """rotate_by_gamma turns the sheared cell upright: the energy and the normal
    stress sum are unchanged, the box becomes Ly sqrt(1+g^2) x Lx/sqrt(1+g^2) with
    gamma -> -gamma, and shearing continues in the rectangular box."""
    L, x, y, p, R, A = sc.generate_packing(1024, 0.85, 1.0, seed=43)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1, stress="virial")
    box.set_strain_rate(1e-2)
    box.set_step(0.02)
    box.strain_steps(500)
    g = box.box()["gamma"]
    se0 = box.calc_se()
    box.rotate_shear()
    bx = box.box()
    se1 = box.calc_se()
    assert abs(bx["Lx"] - L * np.sqrt(1 + g * g)) <= 1e-12 * L
    assert abs(bx["Ly"] - L / np.sqrt(1 + g * g)) <= 1e-12 * L
    assert bx["gamma"] == -g
    assert abs(se1[0] - se0[0]) <= 1e-10 * se0[0]
    assert abs((se1[1] + se1[2]) - (se0[1] + se0[2])) <= 1e-10 * abs(se0[1] + se0[2])
    rec = box.strain_steps(200, se_every=50)
    assert np.all(np.isfinite(rec)) and np.all(rec[:, 0, 0] > 0)


@pytest.mark.parametrize("name", ["resize_n256_shrink", "resize_n256_grow"])
def test_mixed_resize_tracks_reference(sc, name):
    """The mixed form's resize steps (affine scaling about the cell centres with the
    compensated positions) follow the reference's resize run through a change of the
    cell grid: the same box lengths at every checkpoint, positions within 1e-4 of the
    box and the energy within 1e-3 relative.  The reference's predictor takes the
    minimum image with the box length from before the step's resize; the FP64 form
    keeps that, the mixed form's cell-offset geometry does not, which moves pairs
    across the boundary by L * rate * dt per step (about 4e-4 of the energy here)."""
    g = load_golden(name)
    rate, dt, pad, shrink = g["params"]
    box = _gpu_box(sc, g, pad, precision="mixed")
    box.set_resize_rate(rate)
    box.set_step(dt)
    done = 0
    for cp in g["checkpoints"]:
        cp = int(cp)
        box.resize_steps(cp - done, shrink=bool(shrink))
        done = cp
        bx = g[f"s{cp}_box"]
        b = box.box()
        assert b["Lx"] == bx[0] and b["Ly"] == bx[1]
        x, y, _ = box.state()
        assert np.max(np.abs(periodic_diff(x, g[f"s{cp}_x"], bx[0]))) < 1e-4 * bx[0]
        assert np.max(np.abs(periodic_diff(y, g[f"s{cp}_y"], bx[1]))) < 1e-4 * bx[1]
        e = box.calc_se()[0]
        assert abs(e - g[f"s{cp}_se"][0]) <= 1e-3 * abs(g[f"s{cp}_se"][0])


def test_mixed_setback_tracks_fp64(sc):
    """Mixed and FP64 shear through Lees-Edwards set-backs (gamma reaching 1/2 twice):
    energy and shear stress per record within 1e-4 of the FP64 run's, the same gamma,
    and positions within 1e-3 of the box at the end (well before chaos separates the
    trajectories at this strain rate)."""
    L, x, y, p, R, A = sc.generate_packing(1024, 0.85, 1.0, seed=51)
    runs = []
    for prec in ("fp64", "mixed"):
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=prec, stress="virial")
        b.set_strain_rate(0.1)
        b.set_step(0.02)
        rec = b.strain_steps(600, se_every=20)[:, 0]
        runs.append((rec, np.array(b.state()), b.box()["gamma"], b.box()["gamma_total"]))
    (ra, sa, ga, ta), (rb, sb, gb, tb) = runs
    assert ta > 1.0 and abs(ga - gb) < 1e-12 and abs(ta - tb) < 1e-12
    scale = np.max(np.abs(ra[:, 1:3]), axis=1)
    assert np.all(np.abs(ra[:, 0] - rb[:, 0]) <= 1e-4 * ra[:, 0])
    assert np.all(np.abs(ra[:, 3] - rb[:, 3]) <= 1e-4 * scale)
    assert np.max(np.abs(periodic_diff(sa[:2], sb[:2], L))) < 1e-3 * L


def test_fp64_two_point_shear_matches_restatement(sc, oracle_built):
    """Shear steps with the two-point contact rule: the FP64 form against the oracle's
    restatement of it over 50 Heun steps with a rebuild inside."""
    L, x, y, p, R, A = sc.generate_packing(512, 0.80, 1.0, seed=61)
    f = np.sqrt(0.80 / 0.87)
    L, x, y = L * f, x * f, y * f
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1, contacts=2)
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, strain_rate=1e-2, step=0.02,
                                two_point=True)
    box.set_strain_rate(1e-2)
    box.set_step(0.02)
    box.strain_steps(50)
    ob.run_strain_steps(50)
    xs, ys, ps = box.state()
    xo, yo, po = ob.state()
    assert np.max(np.abs(periodic_diff(xs, xo, L))) < 1e-10 * L
    assert np.max(np.abs(periodic_diff(ys, yo, L))) < 1e-10 * L
    assert np.max(np.abs(ps - po)) < 1e-10
