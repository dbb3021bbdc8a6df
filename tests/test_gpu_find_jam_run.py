"""find_jam_2p as a run with output (sc_run_find_jam) and its command-line driver.

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


def _replay(e0, phi0, rows, e_jam, step0):
    """The bisection of find_jam_2p / resize_to_energy_2p on the recorded energies:
    the packing fraction each resize must give.  The lines carry 9 digits of the
    energy, so the replay stops at the first energy within 1e-7 of e_jam, where the
    printed value no longer decides the side; returns (packings, last phase step,
    whether every line was replayed)."""
    d = 1 if e0 < e_jam else -1
    first = nxt = step0
    k = 0
    phi = phi0
    out = []
    for t, _phi, e, *_ in rows:
        f = 1 - nxt if d > 0 else 1 / (1 - nxt)
        phi = phi / (f * f)
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
    # the recorded packings follow the bisection rule from the recorded energies
    # (phi0's minimised energy decides the first direction: below e_jam here)
    want, last, whole = _replay(0.0, phi0, rows, e_jam, step)
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
