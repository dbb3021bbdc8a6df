"""Pure shear: x stretched and y compressed at the strain rate (pure_strain_step_2p,
src/cuda/2point_dynamics.cu:2180-2283; run protocol run_pure_strain_2p :2286-2391;
driver src/cuda/main_pure_shear.cpp).

The reference implements pure shear only in CUDA, which cannot run here, so the
oracle's restatement (orc_pure_step) is pinned by the closed form of the affine flow
on a contact-free box (bit-exact) and by its own invariants; the library's FP64 form
is held to it within TOL = 1e-12 relative (one contact point) through cell-grid
changes and rebuilds, and the mixed form to the FP64 form.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import REF_PI, ROOT, periodic_diff

TOL = 1e-12


def _box_scalars(ob):
    s = ob.scalars()
    return s["Lx"], s["Ly"], int(s["rows"]), int(s["cols"])


def test_oracle_pure_shear_is_the_affine_flow_without_contacts(oracle_built):
    """Contact-free particles follow x <- x + dt e x/2, y <- y - dt e y/2 and
    phi <- phi - dt e RC sin(2 phi)/2 exactly, and the box follows the same map."""
    x = np.array([5.0, 15.0, 25.0, 35.0])
    y = np.array([5.0, 15.0, 5.0, 15.0])
    p = np.array([0.3, -1.0, 1.2, 2.5])
    A = np.array([0.5, 0.7, 0.5, 0.7])
    R = A.copy()
    e, dt = 1e-3, 0.02
    ob = oracle_built.OracleBox(40.0, x, y, p, A, R, 0.2, strain_rate=e, step=dt, Ly=20.0)
    I, RC = ob.consts()
    xs, ys, ps, Lx, Ly = x.copy(), y.copy(), p.copy(), 40.0, 20.0
    for _ in range(50):
        ob.run_pure_steps(1)
        xs = xs + dt * (0.0 + 0.5 * e * xs)
        ys = ys + dt * (0.0 - 0.5 * e * ys)
        ps = ps + dt * (0.0 / I + e * (-0.5 * RC * np.sin(2 * ps)))
        Lx += 0.5 * dt * e * Lx
        Ly -= 0.5 * dt * e * Ly
    X, Y, P = ob.state()
    assert np.array_equal(X, xs) and np.array_equal(Y, ys) and np.array_equal(P, ps)
    s = ob.scalars()
    assert s["Lx"] == Lx and s["Ly"] == Ly and s["gamma"] == 0.0
    assert abs(s["gamma_total"] - 50 * dt * e) < 1e-15


def _regrid_pad(Ly, Rmax, Amax, steps, e, dt):
    """A padding that puts Ly/hmin just above an integer, so that the row count
    drops after about `steps` pure-shear steps."""
    h0 = 2 * (Rmax + Amax) + 0.1
    rows = int(Ly / h0)
    return Ly * (1 - 0.5 * dt * e * steps) / rows - 2 * (Rmax + Amax), rows


def test_oracle_pure_shear_regrids_and_keeps_complete_lists(library, oracle_built):
    """Through a change of the cell grid the oracle's lists stay complete: its forces
    are those of a fresh box built on the same state (summed in another order)."""
    import spherocyls_gb300 as sc

    e, dt = 1e-3, 0.02
    Lx, Ly, x, y, p, R, A = sc.generate_config_rect(400, 0.80, 1.0, 0.5, seed=3)
    pad, rows = _regrid_pad(Ly, R.max(), A.max(), 60, e, dt)
    ob = oracle_built.OracleBox(Lx, x, y, p, A, R, pad, strain_rate=e, step=dt, Ly=Ly)
    assert _box_scalars(ob)[2] == rows
    ob.run_pure_steps(100)
    Lx1, Ly1, rows1, cols1 = _box_scalars(ob)
    assert rows1 == rows - 1
    X, Y, P = ob.state()
    fresh = oracle_built.OracleBox(Lx1, X, Y, P, A, R, pad, Ly=Ly1)
    fa, fb = np.array(ob.forces()), np.array(fresh.forces())
    rms = np.sqrt(np.mean(fb ** 2))
    assert rms > 0 and np.max(np.abs(fa - fb)) <= 1e-12 * rms


def test_generate_config_rect(library):
    """box_aspect = 1 is generate_config's packing bit for bit; other aspects give
    Lx/Ly = box_aspect at the same area and packing fraction, inside the box and
    crossing-free."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_config(300, 0.85, 1.0, seed=9)
    Lx, Ly, x1, y1, p1, R1, A1 = sc.generate_config_rect(300, 0.85, 1.0, 1.0, seed=9)
    assert Lx == L and Ly == L and np.array_equal(x, x1) and np.array_equal(p, p1)
    Lx, Ly, x, y, p, R, A = sc.generate_config_rect(300, 0.85, 1.0, 0.25, seed=9)
    assert abs(Lx / Ly - 0.25) < 1e-14 and abs(Lx * Ly - L * L) < 1e-9 * L * L
    assert np.all((x >= 0) & (x < Lx) & (y >= 0) & (y < Ly))
    s = np.linspace(-1, 1, 41)
    ux, uy = A * np.cos(p), A * np.sin(p)
    worst = np.inf
    for i in range(len(x)):
        dx = x[i] - x
        dy = y[i] - y
        dx -= Lx * np.round(dx / Lx)
        dy -= Ly * np.round(dy / Ly)
        near = np.nonzero((dx ** 2 + dy ** 2 < (2 * A.max() + 0.2) ** 2) & (np.arange(len(x)) != i))[0]
        for j in near:
            ax = dx[j] + s[:, None] * ux[i] - s[None, :] * ux[j]
            ay = dy[j] + s[:, None] * uy[i] - s[None, :] * uy[j]
            worst = min(worst, np.sqrt(ax ** 2 + ay ** 2).min() / (R[i] + R[j]))
    assert worst >= 0.1 - 1e-9
    g = sc.generate_config_rect(300, 0.5, 1.0, 0.5, layout="grid", seed=2)
    assert abs(g[0] / g[1] - 0.5) < 1e-14


# ---- the library on the GPU ----------------------------------------------------


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


def _assert_close_state(box, ob, tol):
    Lx, Ly = ob.scalars()["Lx"], ob.scalars()["Ly"]
    x, y, p = box.state()
    ox, oy, op = ob.state()
    assert np.max(np.abs(periodic_diff(x, ox, Lx))) <= tol * Lx
    assert np.max(np.abs(periodic_diff(y, oy, Ly))) <= tol * Ly
    assert np.max(np.abs(periodic_diff(p, op, 2 * REF_PI))) <= tol * 2 * REF_PI


@pytest.mark.gpu
@pytest.mark.parametrize("graphs", [False, True])
def test_fp64_pure_shear_matches_oracle(sc, oracle_built, graphs):
    """200 FP64 pure-shear steps against the oracle: positions and angles within
    1e-12 of the box, stress and energy records within 1e-12 of their scale, the
    same box lengths and cell grid bit for bit, through a change of the row count."""
    e, dt = 1e-3, 0.02
    Lx, Ly, x, y, p, R, A = sc.generate_config_rect(1024, 0.85, 1.0, 0.5, seed=21)
    pad, rows = _regrid_pad(Ly, R.max(), A.max(), 100, e, dt)
    ob = oracle_built.OracleBox(Lx, x, y, p, A, R, pad, strain_rate=e, step=dt, Ly=Ly)
    box = sc.SpherocylBox(Lx, x, y, p, A, R, pad, Ly=Ly, use_graphs=graphs)
    box.set_strain_rate(e)
    box.set_step(dt)
    for _ in range(10):
        se_o = ob.run_pure_steps(20, record_se=True)
        se_g = box.pure_strain_steps(20, se_every=10)[:, 0, :]
        _assert_close_state(box, ob, TOL)
        for k, r in ((0, 9), (1, 19)):
            scale = max(abs(se_o[r, 0]), np.max(np.abs(se_o[r, 1:3])))
            assert np.max(np.abs(se_g[k, :4] - se_o[r, :4])) <= TOL * scale
        b = box.box()
        oLx, oLy, orows, ocols = _box_scalars(ob)
        assert b["Lx"] == oLx and b["Ly"] == oLy and b["rows"] == orows and b["cols"] == ocols
        assert b["gamma"] == 0.0 and b["gamma_total"] == ob.scalars()["gamma_total"]
    assert _box_scalars(ob)[2] == rows - 1


@pytest.mark.gpu
def test_fp64_two_point_pure_shear_matches_restatement(sc, oracle_built):
    """The same with the two-point contact rule of the src/cuda 2p code, the contact
    model the reference's pure shear uses (tolerance 1e-10, as for shear)."""
    e, dt = 1e-2, 0.02
    Lx, Ly, x, y, p, R, A = sc.generate_config_rect(512, 0.84, 1.0, 0.8, seed=22)
    ob = oracle_built.OracleBox(Lx, x, y, p, A, R, 0.1, strain_rate=e, step=dt, Ly=Ly,
                                two_point=True)
    box = sc.SpherocylBox(Lx, x, y, p, A, R, 0.1, Ly=Ly, contacts=2)
    box.set_strain_rate(e)
    box.set_step(dt)
    box.pure_strain_steps(100)
    ob.run_pure_steps(100)
    _assert_close_state(box, ob, 1e-10)


@pytest.mark.gpu
def test_mixed_pure_shear_tracks_fp64(sc):
    """300 mixed-form pure-shear steps (affine map about the cell centres with
    compensated local positions) stay within 1e-4 of the box of the FP64 run, with
    the energy and the normal-stress difference within 1e-4 of their scale, and the
    same box and grid."""
    e, dt = 2e-3, 0.02
    Lx, Ly, x, y, p, R, A = sc.generate_config_rect(2048, 0.86, 1.0, 0.7, seed=23)
    pad, rows = _regrid_pad(Ly, R.max(), A.max(), 150, e, dt)
    runs = []
    for prec in ("fp64", "mixed"):
        b = sc.SpherocylBox(Lx, x, y, p, A, R, pad, Ly=Ly, precision=prec, stress="virial")
        b.set_strain_rate(e)
        b.set_step(dt)
        rec = b.pure_strain_steps(300, se_every=20)[:, 0]
        runs.append((rec, np.array(b.state()), b.box()))
    (ra, sa, ba), (rb, sb, bb) = runs
    assert ba["Lx"] == bb["Lx"] and ba["Ly"] == bb["Ly"] and ba["rows"] == bb["rows"] == rows - 1
    scale = np.max(np.abs(ra[:, 1:3]), axis=1)
    assert np.all(np.abs(ra[:, 0] - rb[:, 0]) <= 1e-4 * ra[:, 0])
    assert np.all(np.abs((ra[:, 1] - ra[:, 2]) - (rb[:, 1] - rb[:, 2])) <= 1e-4 * scale)
    assert np.max(np.abs(periodic_diff(sa[0], sb[0], ba["Lx"]))) < 1e-4 * ba["Lx"]
    assert np.max(np.abs(periodic_diff(sa[1], sb[1], ba["Ly"]))) < 1e-4 * ba["Ly"]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_pure_shear_matches_single_runs(sc, precision):
    """Two systems with different rates in one handle step exactly as alone."""
    cfg = [sc.generate_config_rect(600, 0.84, 1.0, asp, seed=s) for asp, s in ((0.6, 1), (1.0, 2))]
    rates = (1e-3, 3e-3)
    singles = []
    for (Lx, Ly, x, y, p, R, A), e in zip(cfg, rates):
        b = sc.SpherocylBox(Lx, x, y, p, A, R, 0.1, Ly=Ly, precision=precision)
        b.set_strain_rate(e)
        b.set_step(0.02)
        b.pure_strain_steps(120)
        singles.append(np.array(b.state()))
    n = [c[2].shape[0] for c in cfg]
    cat = lambda k: np.concatenate([c[k] for c in cfg])  # noqa: E731
    bb = sc.BoxBatch(n, [c[0] for c in cfg], cat(2), cat(3), cat(4), cat(6), cat(5), 0.1,
                     Ly=[c[1] for c in cfg], precision=precision)
    for s, e in enumerate(rates):
        bb.set_strain_rate(e, sys=s)
    bb.set_step(0.02)
    bb.pure_strain_steps(120)
    st = np.array(bb.state())
    assert np.array_equal(st[:, : n[0]], singles[0])
    assert np.array_equal(st[:, n[0]:], singles[1])


@pytest.mark.gpu
def test_run_pure_strain_files(sc, tmp_path):
    """The run protocol: position files every pos_save of strain and at the end,
    stress/energy lines labelled with their time unit, the run stopping at the first
    time unit with Lx/Ly at or past the stop aspect."""
    stop = 1.05
    Lx, Ly, x, y, p, R, A = sc.generate_config_rect(256, 0.84, 1.0, 1 / stop, seed=24)
    box = sc.SpherocylBox(Lx, x, y, p, A, R, 0.1, Ly=Ly)
    box.set_strain_rate(1e-2)
    box.set_step(0.02)
    t_end = box.run_pure_strain(str(tmp_path), stop, pos_save=0.02, se_save=1e-3)
    b = box.box()
    assert b["Lx"] / b["Ly"] >= stop
    # one time unit less was not enough
    e, dt = 1e-2, 0.02
    lx, ly = Lx, Ly
    for _ in range((t_end - 1) * 50):
        lx += 0.5 * dt * e * lx
        ly -= 0.5 * dt * e * ly
    assert lx / ly < stop
    assert (tmp_path / f"sd{t_end:010d}.dat").exists()
    assert (tmp_path / "sd0000000000.dat").exists() and (tmp_path / "sd0000000002.dat").exists()
    lines = (tmp_path / "sd_stress_energy.dat").read_text().splitlines()
    labels = [int(s.split()[0]) for s in lines]
    assert labels == sorted(labels) and labels[0] == 0 and labels[-1] == t_end
    # stress every 5 steps: 10 lines per time unit, plus the final state's line
    assert len(lines) == 10 * t_end + 1
    hdr, *_ = sc.read_positions(str(tmp_path / f"sd{t_end:010d}.dat"))
    assert abs(hdr["Lx"] / hdr["Ly"] - b["Lx"] / b["Ly"]) < 1e-12


@pytest.mark.gpu
def test_cli_pure_shear_random_start(library, tmp_path):
    exe = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_pure_shear")
    r = subprocess.run([exe, "r", str(tmp_path), "256", "1e-2", "0.02", "1.04", "0.02", "1e-3",
                        "0.1", "0", "0.84", "1.0", "1.4", "0", "0"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    from spherocyls_gb300 import read_positions

    hdr, *_ = read_positions(str(tmp_path / "sd0000000000.dat"))
    assert abs(hdr["Lx"] / hdr["Ly"] - 1 / 1.04) < 1e-12
    assert (tmp_path / "sd_stress_energy.dat").exists()
