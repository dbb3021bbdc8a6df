"""The quasistatic jamming runs with output: find_jam_2p (sc_run_find_jam) and
compress_qs2p / expand_qs2p (sc_run_qs_compress), and their command-line drivers.

The run writes the reference's files (the start's position file, a stress/energy
line and a position file per resize, the final state as a binary file).  The lines
replay the bisection: every packing fraction follows from the previous one by the
length factor 1 - step (compress) or 1/(1 - step) (expand) of resize_step_2p, the
step growing by 1.1 per resize and restarting at half its last value, the other way,
when the energy per unit area crosses e_jam; the final energy sits at e_jam.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def _lines(path):
    rows = [ln.split() for ln in open(path) if ln.strip()]
    assert all(len(r) == 7 for r in rows)
    return [(int(r[0]),) + tuple(float(v) for v in r[1:]) for r in rows]


def _replay(d0, phi0, rows, e_jam, step0, power=2):
    """The bisection of find_jam_2p / resize_to_energy_2p on the recorded energies:
    the packing fraction each resize must give, from the first direction d0 (+1
    compress, -1 expand: the side of e_jam where the relaxed start lies).  The lines carry 9 digits of the
    energy, so the replay stops at the first energy within 1e-7 of e_jam, where the
    printed value no longer decides the side; returns (packings, last phase step,
    whether every line was replayed).  power: 2 when both lengths change, 1 for y alone."""
    d = d0
    first = nxt = step0
    k = 0
    phi = phi0
    out = []
    for t, _phi, e, *_ in rows:
        f = 1 - nxt if d > 0 else 1 / (1 - nxt)
        phi = phi / f ** power
        out.append(phi)
        if abs(e / e_jam - 1) < 1e-7:
            return np.array(out), first, False
        k += 1
        nxt *= 1.1
        if (d > 0 and not e < e_jam) or (d < 0 and not e > e_jam):
            first = nxt = first * 1.1 ** (k - 1) / 2
            d = 1 if e < e_jam else -1
            k = 0
    return np.array(out), first, True


def test_run_find_jam_files_and_bisection(library, tmp_path):
    """The FP64 form (conjugate-gradient relaxation, as the reference's run); the
    FIRE relaxation of the mixed form is the bisection of sc_find_jam, covered with
    the two-point tests.  A target well above jamming keeps the relaxations short."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(128, 0.80, 1.0, seed=91)
    e_jam, step = 1e-6, 1e-3
    with sc.SpherocylBox(L, x, y, p, A, R, 0.1, contacts=2, precision="fp64") as b:
        phi0 = b.box()["packing"]
        phi, steps = b.run_find_jam(str(tmp_path), e_jam, step, ftol=1e-12)
        se = b.calc_se()
        box = b.box()
        final = np.array(b.state())
    rows = _lines(tmp_path / "sd_stress_energy.dat")
    assert len(rows) == steps > 0
    assert [r[0] for r in rows] == list(range(1, steps + 1))
    for t in (0, steps):
        assert (tmp_path / f"sd{t:010d}.dat").exists()
    # energy column per unit area: E/N x N / 2LxLy
    e_area = se[0] * 128 / (2 * box["Lx"] * box["Ly"])
    assert abs(rows[-1][2] - e_area) <= 1e-8 * e_area
    assert abs(rows[-1][1] - phi) <= 1e-9 and phi > 0
    assert abs(e_area - e_jam) < 0.05 * e_jam, (e_area, e_jam)
    # the recorded packings follow the bisection rule from the recorded energies; the
    # relaxed start's energy (not recorded) sets the first direction, read off the
    # first line
    d0 = 1 if rows[0][1] > phi0 else -1
    want, last, whole = _replay(d0, phi0, rows, e_jam, step)
    got = np.array([r[1] for r in rows[: len(want)]])
    assert len(want) >= 10
    assert np.allclose(got, want, rtol=0, atol=2e-10), np.abs(got - want).max()
    assert last <= 1e-15 or not whole
    hdr, bx, by, bp, *_ = sc.read_positions(str(tmp_path / f"sd{steps:010d}.bin"))
    assert np.array_equal(np.stack([bx, by, bp]), final)
    assert hdr["Lx"] == box["Lx"] and hdr["Ly"] == box["Ly"]


def test_cli_find_jam_random_start(library, tmp_path):
    exe = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_find_jam")
    r = subprocess.run([exe, "r", str(tmp_path), "64", "2e-3", "0.01", "1e-6", "0.01", "0.01",
                        "0.1", "0.80", "1.0", "1.4", "0", "0"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    rows = _lines(tmp_path / "sd_stress_energy.dat")
    steps = rows[-1][0]
    assert (tmp_path / f"sd{steps:010d}.bin").exists()
    assert abs(rows[-1][2] - 1e-6) < 0.05e-6
    assert 0.80 < rows[-1][1] < 0.95


def test_run_y_compress_bisects_in_y_alone(library, tmp_path):
    """y_compress_energy_2p: the bisection of the find-jam run with Ly and the y
    coordinates resized alone (the packing fraction changes by 1/f per resize); Lx
    and every x coordinate stay as they were."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(128, 0.80, 1.0, seed=93)
    e_t, step = 1e-6, 1e-3
    with sc.SpherocylBox(L, x, y, p, A, R, 0.1, contacts=2, precision="fp64") as b:
        phi0 = b.box()["packing"]
        phi, steps = b.run_y_compress(str(tmp_path), e_t, step, ftol=1e-12)
        box = b.box()
        se = b.calc_se()
    assert box["Lx"] == L and box["Ly"] < L
    assert abs(box["packing"] - phi0 * L / box["Ly"]) <= 1e-12
    rows = _lines(tmp_path / "sd_stress_energy.dat")
    assert len(rows) == steps > 0 and phi > 0
    e_area = se[0] * 128 / (2 * box["Lx"] * box["Ly"])
    assert abs(e_area - e_t) < 0.05 * e_t, (e_area, e_t)
    d0 = 1 if rows[0][1] > phi0 else -1
    want, last, whole = _replay(d0, phi0, rows, e_t, step, power=1)
    got = np.array([r[1] for r in rows[: len(want)]])
    assert len(want) >= 10
    assert np.allclose(got, want, rtol=0, atol=2e-10), np.abs(got - want).max()
    assert last <= 1e-14 or not whole
    hdr, *_ = sc.read_positions(str(tmp_path / f"sd{steps:010d}.bin"))
    assert hdr["Lx"] == L and hdr["Ly"] == box["Ly"]


def test_run_qs_compress_and_expand(library, tmp_path):
    """compress_qs2p: the start and every resize give a line and a position file; the
    packing fraction grows by 1/(1 - step)^2 per resize and the run stops at the first
    resize at or above the target; expand_qs2p (a target below) shrinks it by
    (1 - step)^2 per resize.  Energies per unit area, as the find-jam run."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(128, 0.80, 1.0, seed=92)
    step = 5e-3
    with sc.SpherocylBox(L, x, y, p, A, R, 0.1, contacts=2, precision="fp64") as b:
        phi0 = b.box()["packing"]
        up = tmp_path / "up"
        up.mkdir()
        n_up = b.run_qs_compress(str(up), 0.93, step)
        box = b.box()
        e_end = b.calc_se()[0] * 128 / (2 * box["Lx"] * box["Ly"])
        down = tmp_path / "down"
        down.mkdir()
        n_down = b.run_qs_compress(str(down), 0.90, -step)
        phi_end = b.box()["packing"]
    rows = _lines(up / "sd_stress_energy.dat")
    assert [r[0] for r in rows] == list(range(n_up + 1))
    for t in range(n_up + 1):
        assert (up / f"sd{t:010d}.dat").exists()
    want = phi0 / (1 - step) ** (2 * np.arange(n_up + 1))
    got = np.array([r[1] for r in rows])
    assert abs(got[0] - want[0]) < 1e-6 and np.allclose(got[1:], want[1:], rtol=0, atol=2e-9)
    assert want[-1] >= 0.93 > want[-2]
    assert e_end > 0 and abs(rows[-1][2] - e_end) <= 1e-5 * e_end
    rows = _lines(down / "sd_stress_energy.dat")
    assert [r[0] for r in rows] == list(range(n_down + 1))
    want = rows[0][1] * (1 - step) ** (2 * np.arange(n_down + 1))
    assert np.allclose([r[1] for r in rows[1:]], want[1:], rtol=0, atol=2e-6)
    assert phi_end <= 0.90 < phi_end / (1 - step) ** 2


def test_cli_qs_compress_random_start(library, tmp_path):
    exe = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_qs_compress")
    r = subprocess.run([exe, "r", str(tmp_path), "64", "5e-3", "0.01", "0.85", "0.01", "0.01",
                        "0.1", "0.80", "1.0", "1.4", "0", "0"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    rows = _lines(tmp_path / "sd_stress_energy.dat")
    assert rows[0][0] == 0 and rows[-1][1] >= 0.85 > rows[-2][1]
    assert (tmp_path / f"sd{rows[-1][0]:010d}.dat").exists()
