"""The device placement (sc_generate_packing_device): the host generator's shapes, box
and packing fraction exactly, every spine pair at least min_sep (R_i + R_j) apart,
reproducible for a seed, zero energy with min_sep = 1, and N = 2^20 in well under the
host placement's seconds."""
from __future__ import annotations

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


def _min_separation(L, x, y, p, R, A):
    s = np.linspace(-1, 1, 41)
    ux, uy = A * np.cos(p), A * np.sin(p)
    worst = np.inf
    reach = 2 * A.max() + 2 * R.max()
    for i in range(len(x)):
        dx = x[i] - x
        dy = y[i] - y
        dx -= L * np.round(dx / L)
        dy -= L * np.round(dy / L)
        near = np.nonzero((dx ** 2 + dy ** 2 < reach ** 2) & (np.arange(len(x)) != i))[0]
        for j in near:
            ax = dx[j] + s[:, None] * ux[i] - s[None, :] * ux[j]
            ay = dy[j] + s[:, None] * uy[i] - s[None, :] * uy[j]
            worst = min(worst, np.sqrt(ax ** 2 + ay ** 2).min() / (R[i] + R[j]))
    return worst


def test_device_packing_matches_host_shapes_and_rule(sc):
    L, x, y, p, R, A = sc.generate_packing_device(3000, 0.85, 1.0, seed=11)
    Lh, xh, yh, ph, Rh, Ah = sc.generate_packing(3000, 0.85, 1.0, seed=11)
    assert L == Lh and np.array_equal(R, Rh) and np.array_equal(A, Ah)
    assert not np.array_equal(x, xh)
    assert np.all((x >= 0) & (x < L) & (y >= 0) & (y < L) & (p >= 0) & (p < np.pi))
    assert _min_separation(L, x, y, p, R, A) >= 0.1 - 1e-9
    again = sc.generate_packing_device(3000, 0.85, 1.0, seed=11)
    assert all(np.array_equal(a, b) for a, b in zip((x, y, p), again[1:4]))
    other = sc.generate_packing_device(3000, 0.85, 1.0, seed=12)
    assert not np.array_equal(x, other[1])


def test_device_zero_energy_placement(sc):
    """Contact-free placement (min_sep = 1) below its saturation; near saturation (about
    0.45 for these shapes) a particle needs many tries, one per round here, and the
    sequential host placement is the one to use."""
    L, x, y, p, R, A = sc.generate_packing_device(2000, 0.35, 1.0, seed=13, min_sep=1.0)
    with sc.SpherocylBox(L, x, y, p, A, R, 0.2) as b:
        assert b.calc_se()[0] == 0.0


def test_device_packing_large(sc):
    t = time.perf_counter()
    L, x, y, p, R, A = sc.generate_packing_device(1 << 20, 0.84, 1.0, seed=3)
    dt = time.perf_counter() - t
    assert dt < 2.0, dt
    assert np.all(np.isfinite(x)) and np.all((x >= 0) & (x < L))
    # the packing steps like any other: no crossing spines, so no non-finite force
    with sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision="mixed") as b:
        b.set_strain_rate(1e-4)
        b.set_step(0.02)
        b.strain_steps(20)
        assert np.all(np.isfinite(np.array(b.state())))
