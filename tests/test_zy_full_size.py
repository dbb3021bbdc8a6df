"""Parity at the benchmark's full size (N = 2^20, packing 0.84, a = R, the shear
workload of the large roofline run): the FP64 form against the oracle for a force
evaluation and three Heun steps, and the mixed form's forces against the FP64 form's.
The oracle runs single-threaded on the host, a few seconds per force evaluation at
this size.  (Collected after the other GPU tests and before the allocation-free
entry point's file.)"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import periodic_diff

pytestmark = pytest.mark.gpu

N = 1 << 20


@pytest.fixture(scope="module")
def big():
    import spherocyls_gb300 as sc

    return sc.generate_packing(N, 0.84, 1.0, seed=3)


def test_fp64_full_size_matches_oracle(library, oracle_built, big):
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = big
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.2)
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.2, strain_rate=1e-4, step=0.02)
    box.set_strain_rate(1e-4)
    box.set_step(0.02)
    box.calc_se()
    ob.calc_se()
    fg = np.array(box.forces())
    fo = np.array(ob.forces())
    rms = np.sqrt(np.mean(fo ** 2))
    assert np.max(np.abs(fg - fo)) <= 1e-12 * rms
    se, so = box.calc_se(), ob.se()
    scale = max(abs(so[0]), np.max(np.abs(so[1:3])))
    assert np.all(np.abs(se[:4] - so[:4]) <= 1e-12 * scale)
    box.strain_steps(3)
    ob.run_strain_steps(3)
    xg, yg, pg = box.state()
    xo, yo, po = ob.state()
    assert np.max(np.abs(periodic_diff(xg, xo, L))) <= 1e-12 * L
    assert np.max(np.abs(periodic_diff(yg, yo, L))) <= 1e-12 * L
    assert np.max(np.abs(pg - po)) <= 1e-12 * np.pi
    ob.close()


def test_mixed_full_size_forces_track_fp64(library, big):
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = big
    f = []
    for prec in ("fp64", "mixed"):
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision=prec)
        se = b.calc_se()
        f.append((np.array(b.forces()), se))
        b.close()
    rms = np.sqrt(np.mean(f[0][0] ** 2))
    assert np.max(np.abs(f[1][0] - f[0][0])) <= 1e-4 * rms
    assert abs(f[1][1][0] - f[0][1][0]) <= 5e-7 * f[0][1][0]
