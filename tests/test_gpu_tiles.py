"""The mixed form's two force passes: one thread per particle over its full list
(each pair evaluated twice) and the tile pass (blocks of cells staged in shared
memory, each pair inside a tile evaluated once, the partner's share read back).

Both evaluate the same FP32 pair geometry, so their forces agree to FP32 rounding
and both agree with the FP64 form within the mixed form's tolerance.  The tile pass
is checked at the default tile size, at tiles of a few cells (most pairs cross a
tile edge) and at tiles far larger than shared memory holds (the records and pair
results of the excess go through global memory); its sums are deterministic."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import periodic_diff

pytestmark = pytest.mark.gpu

VARIANTS = [("list", 0), ("tile", 0), ("tile", 16), ("tile", 6000)]


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


@pytest.fixture(scope="module")
def state(sc):
    """A sheared state of 8192 particles (a/R = 1.5) and its FP64 forces."""
    L, x, y, p, R, A = sc.generate_packing(8192, 0.85, 1.5, seed=61)
    b = sc.SpherocylBox(L, x, y, p, A, R, 0.2)
    b.set_strain_rate(1e-3)
    b.set_step(0.02)
    b.strain_steps(200)
    xs, ys, ps = b.state()
    gam = b.box()["gamma"]
    b.calc_forces()
    f64 = np.array(b.forces())
    b.close()
    return L, xs, ys, ps, A, R, gam, f64


@pytest.mark.parametrize("kind,target", VARIANTS)
def test_pass_forces_match_fp64(sc, state, kind, target):
    L, x, y, p, A, R, gam, f64 = state
    b = sc.SpherocylBox(L, x, y, p, A, R, 0.3, precision="mixed", pass_kind=kind,
                        tile_target=target)
    assert b.options()["pass_kind"] == kind
    b.set_gamma(gam)
    b.calc_forces()
    f = np.array(b.forces())
    b.close()
    rms = np.sqrt(np.mean(f64 ** 2))
    assert np.max(np.abs(f - f64)) <= 1e-4 * rms


def test_tile_and_list_passes_agree(sc, state):
    """Same state, same FP32 pair code: the passes differ only in which side of a
    pair evaluates it and in the order of the sums."""
    L, x, y, p, A, R, gam, _ = state
    out = []
    for kind, target in VARIANTS:
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.3, precision="mixed", pass_kind=kind,
                            tile_target=target)
        b.set_gamma(gam)
        b.calc_forces()
        out.append(np.array(b.forces()))
        b.close()
    rms = np.sqrt(np.mean(out[0] ** 2))
    for f in out[1:]:
        # a few FP32 ulps of the largest contact forces (several times the RMS)
        assert np.max(np.abs(f - out[0])) <= 2e-5 * rms


@pytest.mark.parametrize("target", [0, 16, 6000])
def test_tile_pass_trajectories(sc, state, target):
    """100 shear steps with the tile pass track the per-particle pass (FP32-level
    differences only, before chaos amplifies them), and a repeated run is bitwise
    identical (deterministic sums)."""
    L, x, y, p, A, R, gam, _ = state
    runs = []
    for kind, tgt in (("list", 0), ("tile", target), ("tile", target)):
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.3, precision="mixed", pass_kind=kind,
                            tile_target=tgt)
        b.set_gamma(gam)
        b.set_strain_rate(1e-3)
        b.set_step(0.02)
        se = b.strain_steps(100, se_every=20)
        runs.append((np.array(b.state()), se, b.counters()["rebuilds"]))
        b.close()
    (s0, se0, _), (s1, se1, r1), (s2, se2, r2) = runs
    assert np.array_equal(s1, s2) and np.array_equal(se1, se2) and r1 == r2
    assert np.max(np.abs(periodic_diff(s0[:2], s1[:2], L))) < 1e-5 * L
    assert np.all(np.abs(se0[:, 0, 0] - se1[:, 0, 0]) <= 1e-5 * np.abs(se0[:, 0, 0]))


def test_autotune_picks_a_pass(sc, state):
    L, x, y, p, A, R, gam, _ = state
    b = sc.SpherocylBox(L, x, y, p, A, R, 0.3, precision="mixed")
    b.set_gamma(gam)
    b.set_strain_rate(1e-3)
    b.set_step(0.02)
    s0 = np.concatenate(b.state())
    f, blk = b.autotune(10)
    o = b.options()
    assert f in (0.5, 1.0, 1.5, 2.0, 3.0)
    assert o["pass_kind"] in ("list", "tile")
    assert o["pass_kind"] == "list" or o["tile_target"] in (128, 256, 384)
    assert np.max(np.abs(np.concatenate(b.state()) - s0)) < 1e-12 * L
    b.strain_steps(20)
    b.close()
