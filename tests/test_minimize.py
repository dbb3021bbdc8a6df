"""The production minimiser (FIRE, on the device) and quasistatic compression.

Checks against the oracle: after FIRE reports max|F| < ftol, the oracle (the
reference's CPU force routine, restated) evaluated on the returned configuration
agrees that the residual force is below ftol, and the energy went down.  The
packings are either well above jamming (a stable minimum with E > 0 that FIRE
reaches quickly) or well below it (E -> 0); close to jamming the relaxation slows
down critically, which the compression test meets in small systems only.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _max_force(fx, fy, tau, I):
    return max(np.max(np.hypot(fx, fy)), np.max(np.abs(tau) / np.sqrt(I)))


def test_fire_fp64_relaxes_compressed_packing_consistently_with_oracle(library, oracle_built):
    """From a relaxed packing compressed affinely to phi = 0.88, FIRE lowers the
    energy and the residual force; at the state it returns, the library's forces and
    energy are the oracle's (the reference's CPU force routine).

    Relaxation aligns overlapping neighbours, and for nearly parallel spines the
    reference's single contact point sits at one end or the other depending on the
    last bit of cos/sin (its energy has a cusp there).  Torques therefore are not
    compared, and forces only to 1e-6 of the largest: the two ends of a pair that is
    parallel to within an angle eps give distances that differ by about eps times the
    spine length, which moves the energy by parts in 1e-9."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(300, 0.80, 1.0, seed=12)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    it, fmax, done = box.fire_minimize(1e-14, 20000)
    assert done[0]  # below jamming every overlap is removed
    box.affine_scale(np.sqrt(0.80 / 0.88))
    e0 = box.calc_se()[0]
    f0 = np.max(np.abs(np.array(box.forces())))
    it, fmax, done = box.fire_minimize(1e-14, 3000)
    e1 = box.calc_se()[0]
    assert e1 < 0.5 * e0
    assert fmax[0] < f0
    Lc = box.box()["Lx"]
    xs, ys, ps = box.state()
    ob = oracle_built.OracleBox(Lc, xs, ys, ps, A, R, 0.1)
    ob.calc_se()
    fo = np.array(ob.forces())[:2]
    fg = np.array(box.forces())[:2]
    assert np.max(np.abs(fg - fo)) <= 1e-6 * max(np.max(np.abs(fo)), 1e-300)
    assert abs(ob.se()[0] - e1) <= 1e-8 * e1


def test_fire_below_jamming_reaches_zero_energy(library):
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(400, 0.70, 1.0, seed=13)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    it, fmax, done = box.fire_minimize(1e-14, 100000)
    assert done[0]
    assert box.calc_se()[0] < 1e-20


def test_mixed_sweeps_then_fp64_refinement(library, oracle_built):
    """FP32 sweeps to 1e-5, then FP64 refinement of the same state to 1e-14."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(300, 0.78, 1.0, seed=14)
    mixed = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision="mixed")
    it1, fm1, d1 = mixed.fire_minimize(1e-5, 100000)
    assert d1[0]
    xs, ys, ps = mixed.state()
    fine = sc.SpherocylBox(L, xs, ys, ps, A, R, 0.1)
    it2, fm2, d2 = fine.fire_minimize(1e-14, 100000)
    assert d2[0] and fm2[0] < 1e-14
    xf, yf, pf = fine.state()
    ob = oracle_built.OracleBox(L, xf, yf, pf, A, R, 0.1)
    ob.calc_se()
    I, _ = ob.consts()
    assert _max_force(*ob.forces(), I) < 1e-14


def test_batched_fire_matches_single_systems(library):
    import spherocyls_gb300 as sc

    packs = [sc.generate_packing(n, f, a, seed=s) for n, f, a, s in
             [(200, 0.86, 1.0, 41), (300, 0.70, 0.5, 42), (250, 0.84, 2.0, 43)]]
    singles = []
    for L, x, y, p, R, A in packs:
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
        b.fire_minimize(1e-14, 2000)
        singles.append(np.concatenate(b.state()))
    batch = sc.BoxBatch([len(pk[1]) for pk in packs], [pk[0] for pk in packs],
                        np.concatenate([pk[1] for pk in packs]),
                        np.concatenate([pk[2] for pk in packs]),
                        np.concatenate([pk[3] for pk in packs]),
                        np.concatenate([pk[5] for pk in packs]),
                        np.concatenate([pk[4] for pk in packs]), 0.1)
    it, fmax, done = batch.fire_minimize(1e-14, 2000)
    x, y, p = batch.state()
    off = 0
    for k, pk in enumerate(packs):
        n = len(pk[1])
        got = np.concatenate([x[off:off + n], y[off:off + n], p[off:off + n]])
        assert np.array_equal(got, singles[k]), k
        off += n


def test_quasistatic_compression_jams(library):
    import spherocyls_gb300 as sc

    packs = [sc.generate_packing(64, 0.80, 1.0, seed=s) for s in (51, 52)]
    batch = sc.BoxBatch([64, 64], [pk[0] for pk in packs],
                        np.concatenate([pk[1] for pk in packs]),
                        np.concatenate([pk[2] for pk in packs]),
                        np.concatenate([pk[3] for pk in packs]),
                        np.concatenate([pk[5] for pk in packs]),
                        np.concatenate([pk[4] for pk in packs]), 0.1)
    phi_jam, n_inc = batch.quasistatic_compress(1e-2, 1e-10, 1e-10, 30, 20000)
    assert np.all(phi_jam > 0.80) and np.all(phi_jam < 0.95), phi_jam
    se = batch.calc_se()
    assert np.all(se[:, 0] > 1e-10)


def test_fire_graph_and_eager_bitwise_identical(library):
    """FIRE chunks captured in CUDA graphs (with the conditional rebuild node) and
    launched eagerly produce the same trajectory bit for bit."""
    import spherocyls_gb300 as sc

    packs = [sc.generate_packing(n, f, a, seed=s) for n, f, a, s in
             [(200, 0.86, 1.0, 71), (300, 0.80, 0.5, 72)]]
    out = []
    for graphs in (True, False):
        b = sc.BoxBatch([len(pk[1]) for pk in packs], [pk[0] for pk in packs],
                        np.concatenate([pk[1] for pk in packs]),
                        np.concatenate([pk[2] for pk in packs]),
                        np.concatenate([pk[3] for pk in packs]),
                        np.concatenate([pk[5] for pk in packs]),
                        np.concatenate([pk[4] for pk in packs]), 0.1, use_graphs=graphs,
                        contacts=2)
        it, fmax, done = b.fire_minimize(1e-14, 1000)
        out.append((np.concatenate(b.state()), fmax, it))
        b.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]
