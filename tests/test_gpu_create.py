"""Handle creation: the device-side ingest of the caller's arrays (read in place where
the GPU addresses pageable host memory, else staged through device copies) gives the
same state bit for bit either way and matches the oracle's set_particle; handles of a
size seen before reuse the pooled device memory, and trimming the pool leaves later
handles working."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_staged_and_in_place_ingest_identical(sc, precision):
    L, x, y, p, R, A = sc.generate_packing(3000, 0.84, 1.5, seed=31)
    # positions and angles outside the box and the angle range exercise the wrap
    x = x + L * np.where(np.arange(x.size) % 3 == 0, 1.0, 0.0)
    y = y - L * np.where(np.arange(y.size) % 5 == 0, 2.0, 0.0)
    p = p + 2 * np.pi * np.where(np.arange(p.size) % 7 == 0, 3.0, 0.0)
    out = []
    for staged in (False, True):
        with sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision=precision,
                             stage_inputs=staged) as b:
            s0 = np.array(b.state())
            se = b.calc_se()
            f = np.array(b.forces())
            b.set_strain_rate(1e-3)
            b.set_step(0.02)
            b.strain_steps(50)
            out.append((s0, se, f, np.array(b.state())))
    for a, c in zip(out[0], out[1]):
        assert np.array_equal(a, c)


def test_ingest_matches_oracle_set_particle(sc, oracle_built):
    """Wrapped state and the forces that depend on I and RC through one step agree
    with the oracle's set_particle and strain step (1e-12)."""
    L, x, y, p, R, A = sc.generate_packing(800, 0.85, 1.0, seed=32)
    x = x + 3 * L
    p = p - 4 * np.pi
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, strain_rate=1e-3, step=0.02)
    with sc.SpherocylBox(L, x, y, p, A, R, 0.1) as b:
        X, Y, P = b.state()
        ox, oy, op = ob.state()
        assert np.array_equal(X, ox) and np.array_equal(Y, oy) and np.array_equal(P, op)
        b.set_strain_rate(1e-3)
        b.set_step(0.02)
        b.strain_steps(5)
        ob.run_strain_steps(5)
        X, Y, P = b.state()
        ox, oy, op = ob.state()
        assert np.max(np.abs(X - ox)) <= 1e-12 * L and np.max(np.abs(P - op)) <= 1e-12


def test_pool_reuse_and_trim(sc):
    L, x, y, p, R, A = sc.generate_packing(20000, 0.84, 1.0, seed=33)
    ref = None
    for k in range(3):
        with sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision="mixed") as b:
            b.set_strain_rate(1e-4)
            b.set_step(0.02)
            b.strain_steps(40)
            st = np.array(b.state())
        if ref is None:
            ref = st
        assert np.array_equal(st, ref)
        if k == 1:
            sc.trim_memory(0)
