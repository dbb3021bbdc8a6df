"""Shear past gamma = 1/2 without set-back (run_strain(dGammaMax),
src/cuda/strain_dynamics.cu:1097-1108), the strain driver's shear-direction change 3
before the box rotation: the FP64 form follows the oracle within 1e-12 (cells widened
to 2 sqrt(1 + gamma_max^2)(R + A) + pad in both), the mixed form the FP64 form, and
the driver runs the whole change."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import REF_PI, ROOT, periodic_diff

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


def test_fp64_strain_to_gamma_matches_oracle(sc, oracle_built):
    L, x, y, p, R, A = sc.generate_packing(1024, 0.85, 1.0, seed=41)
    rate, dt, gmax = 0.25, 0.02, 1.3
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, strain_rate=rate, step=dt)
    with sc.SpherocylBox(L, x, y, p, A, R, 0.1) as b:
        b.set_strain_rate(rate)
        b.set_step(dt)
        k = b.strain_to_gamma(gmax)
        ko = ob.strain_to_gamma(gmax)
        assert k == ko > 0
        s = ob.scalars()
        box = b.box()
        assert box["gamma"] == s["gamma"] >= gmax and box["cols"] == s["cols"]
        X, Y, P = b.state()
        ox, oy, op = ob.state()
        assert np.max(np.abs(periodic_diff(X, ox, L))) <= 1e-12 * L
        assert np.max(np.abs(periodic_diff(Y, oy, L))) <= 1e-12 * L
        assert np.max(np.abs(periodic_diff(P, op, 2 * REF_PI))) <= 1e-12 * 2 * REF_PI


def test_mixed_strain_to_gamma_tracks_fp64(sc):
    L, x, y, p, R, A = sc.generate_packing(2048, 0.85, 1.0, seed=42)
    out = []
    for prec in ("fp64", "mixed"):
        with sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=prec) as b:
            b.set_strain_rate(0.25)
            b.set_step(0.02)
            b.strain_to_gamma(1.1)
            b.rotate_shear()
            b.strain_steps(50)
            out.append((np.array(b.state()), b.box()))
    (sa, ba), (sb, bb) = out
    assert ba["gamma"] == bb["gamma"] and ba["Lx"] == bb["Lx"]
    assert np.max(np.abs(periodic_diff(sa[0], sb[0], ba["Lx"]))) < 1e-4 * ba["Lx"]


def test_cli_strain_change_3(library, tmp_path):
    exe = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_strain")
    r = subprocess.run([exe, "r", str(tmp_path), "256", "1e-2", "0.02", "0.01", "0.01", "1e-3",
                        "0.1", "3", "0.85", "1.0", "1.4", "0", "0", "0.8"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    from spherocyls_gb300 import read_positions

    hdr, *_ = read_positions(str(tmp_path / "sp0000000000.dat"))
    # the rotated box: Lx' = Ly sqrt(1 + g^2), Ly' = Lx / sqrt(1 + g^2), g >= 0.8
    assert hdr["Lx"] / hdr["Ly"] >= 1.64 - 1e-9
