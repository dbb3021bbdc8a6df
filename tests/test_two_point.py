"""Two-point contacts (SC_CONTACT_TWO): the contact rule of the reference's CUDA
jamming code (euler_est_2p, src/cuda/2point_dynamics.cu:385-546), which adds a
second contact point for overlapping, nearly parallel spines so that the pair
energy has no cusp at parallel alignment.

The reference has this rule only in CUDA, so the oracle's C restatement
(force_pair2 in oracle/spherocyl_oracle.c) is pinned here by its own invariant
(forces and torques are minus the gradient of the summed contact energies) rather
than by reference output; the GPU kernels are then checked against it.
"""
from __future__ import annotations

import numpy as np
import pytest


def _aligned_rows(seed, ncol=6, nrow=17):
    """Rows of spherocylinders lying along x, stacked so that neighbouring rows
    overlap side by side: exactly parallel, nearly parallel (1e-9 rad) and slightly
    tilted (1e-3 rad) pairs, with random offsets along the rows."""
    rng = np.random.default_rng(seed)
    sx = 3.2
    L = ncol * sx
    sy = L / nrow
    n = ncol * nrow
    R = rng.choice([0.5, 0.7], size=n)
    A = R.copy()
    x = np.empty(n)
    y = np.empty(n)
    for r in range(nrow):
        off = rng.uniform(-1.0, 1.0)
        for c in range(ncol):
            i = r * ncol + c
            x[i] = (c + 0.5) * sx + off
            y[i] = (r + 0.5) * sy
    kind = rng.integers(0, 3, size=n)
    phi = np.where(kind == 0, 0.0,
                   np.where(kind == 1, rng.choice([-1e-9, 1e-9], size=n),
                            rng.uniform(-1e-3, 1e-3, size=n)))
    return L, x % L, y % L, phi, R, A


def test_oracle_two_point_forces_are_energy_gradient(oracle_built):
    """Central differences of the restatement's energy reproduce its forces and
    torques, on the aligned rows and on a random compressed packing."""
    import spherocyls_gb300 as sc

    L1, x1, y1, p1, R1, A1 = _aligned_rows(3, ncol=4, nrow=12)
    L2, x2, y2, p2, R2, A2 = sc.generate_packing(80, 0.80, 1.0, seed=12)
    f = np.sqrt(0.80 / 0.86)
    cases = [(L1, x1, y1, p1, R1, A1), (L2 * f, x2 * f, y2 * f, p2, R2, A2)]
    for L, x, y, p, R, A in cases:
        n = len(x)

        def energy(xx, yy, pp):
            b = oracle_built.OracleBox(L, xx, yy, pp, A, R, 0.1, two_point=True)
            b.calc_se()
            e = b.se()[0] * n
            b.close()
            return e

        b = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, two_point=True)
        b.calc_se()
        F = np.array(b.forces())
        b.close()
        assert np.max(np.abs(F)) > 1e-3  # the configuration is loaded
        h = 1e-6
        rng = np.random.default_rng(1)
        for i in rng.choice(n, size=12, replace=False):
            for k in range(3):
                arrs = [x.copy(), y.copy(), p.copy()]
                arrs[k][i] += h
                ep = energy(*arrs)
                arrs[k][i] -= 2 * h
                em = energy(*arrs)
                g = -(ep - em) / (2 * h)
                assert abs(g - F[k][i]) <= 1e-7 * max(1.0, abs(F[k][i])), (i, k, g, F[k][i])


def test_two_point_rejects_reference_wrapper(oracle_built):
    if not oracle_built.ref_available():
        pytest.skip("reference library not built")
    L, x, y, p, R, A = _aligned_rows(3, ncol=4, nrow=12)
    with pytest.raises(ValueError):
        oracle_built.RefBox(L, x, y, p, A, R, 0.1, two_point=True)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,etol", [("fp64", 1e-10, 1e-12), ("mixed", 1e-4, 2e-6)])
@pytest.mark.parametrize("case", ["aligned", "compressed"])
def test_two_point_forces_match_restatement(library, oracle_built, precision, tol, etol, case):
    """Forces, torques, energy and stress of the two-point rule: FP64 kernels agree
    with the restatement to 1e-10 of the RMS force (the last bits of cos/sin decide
    the branch for exactly parallel spines, where both branches give the same
    contacts to rounding), the mixed form to 1e-4."""
    import spherocyls_gb300 as sc

    if case == "aligned":
        L, x, y, p, R, A = _aligned_rows(7)
    else:
        L, x, y, p, R, A = sc.generate_packing(300, 0.80, 1.0, seed=31)
        f = np.sqrt(0.80 / 0.87)
        L, x, y = L * f, x * f, y * f
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=precision, contacts=2,
                          stress="virial")
    se = box.calc_se()
    fg = np.array(box.forces())
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, two_point=True)
    ob.calc_se()
    fo = np.array(ob.forces())
    so = ob.se()
    rms = np.sqrt(np.mean(fo ** 2))
    assert rms > 1e-3
    assert np.max(np.abs(fg - fo)) <= tol * rms, np.max(np.abs(fg - fo)) / rms
    scale = max(abs(so[0]), np.max(np.abs(so[1:4])))
    for k in range(4):
        assert abs(se[k] - so[k]) <= etol * scale, (k, se[k], so[k])


@pytest.mark.gpu
def test_two_point_differs_from_one_point_only_near_alignment(library):
    """On a random compressed packing (few nearly parallel neighbours) the two
    contact rules give nearly the same energy; on the aligned rows the second
    contacts carry a large share of it."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(300, 0.80, 1.0, seed=31)
    f = np.sqrt(0.80 / 0.87)
    e = [sc.SpherocylBox(L * f, x * f, y * f, p, A, R, 0.1, contacts=c).calc_se()[0]
         for c in (1, 2)]
    assert e[1] >= e[0] and e[1] < 1.5 * e[0]
    L, x, y, p, R, A = _aligned_rows(7)
    e = [sc.SpherocylBox(L, x, y, p, A, R, 0.1, contacts=c).calc_se()[0] for c in (1, 2)]
    assert e[1] > 1.5 * e[0]


@pytest.mark.gpu
def test_fire_two_point_converges_above_jamming(library, oracle_built):
    """Well above jamming (phi = 0.92 at a/R = 1) the two-point energy is smooth at
    alignment, so FIRE reaches a residual force of 1e-12; the restatement confirms
    the residual and the energy at the returned state."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(300, 0.80, 1.0, seed=12)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1, contacts=2)
    it, fmax, done = box.fire_minimize(1e-14, 20000)
    assert done[0]
    box.affine_scale(np.sqrt(0.80 / 0.92))
    e0 = box.calc_se()[0]
    it, fmax, done = box.fire_minimize(1e-12, 200000)
    assert done[0], (it, fmax)
    e1 = box.calc_se()[0]
    assert 1e-8 < e1 < e0  # jammed: a minimum with finite energy
    Lc = box.box()["Lx"]
    xs, ys, ps = box.state()
    ob = oracle_built.OracleBox(Lc, xs, ys, ps, A, R, 0.1, two_point=True)
    ob.calc_se()
    I, _ = ob.consts()
    fo = ob.forces()
    assert max(np.max(np.hypot(fo[0], fo[1])), np.max(np.abs(fo[2]) / np.sqrt(I))) < 1e-11
    assert abs(ob.se()[0] - e1) <= 1e-10 * e1


@pytest.mark.gpu
def test_quasistatic_two_point_jams(library):
    import spherocyls_gb300 as sc

    packs = [sc.generate_packing(128, 0.78, 1.0, seed=s) for s in (61, 62)]
    batch = sc.BoxBatch([128, 128], [pk[0] for pk in packs],
                        np.concatenate([pk[1] for pk in packs]),
                        np.concatenate([pk[2] for pk in packs]),
                        np.concatenate([pk[3] for pk in packs]),
                        np.concatenate([pk[5] for pk in packs]),
                        np.concatenate([pk[4] for pk in packs]), 0.1, contacts=2)
    phi_jam, n_inc = batch.quasistatic_compress(5e-3, 1e-12, 1e-10, 60, 50000)
    assert np.all(phi_jam > 0.80) and np.all(phi_jam < 0.95), phi_jam
    se = batch.calc_se()
    assert np.all(se[:, 0] > 1e-10)


@pytest.mark.gpu
def test_find_jam_bisects_to_target_energy(library):
    """find_jam_2p's bisection: each system ends at a packing fraction whose
    minimised energy per particle sits at e_jam (the final steps are below 1e-7 in
    length, where E/N changes by well under a percent of e_jam)."""
    import spherocyls_gb300 as sc

    packs = [sc.generate_packing(96, 0.80, a, seed=s) for a, s in ((1.0, 81), (0.5, 82))]
    batch = sc.BoxBatch([96, 96], [pk[0] for pk in packs],
                        np.concatenate([pk[1] for pk in packs]),
                        np.concatenate([pk[2] for pk in packs]),
                        np.concatenate([pk[3] for pk in packs]),
                        np.concatenate([pk[5] for pk in packs]),
                        np.concatenate([pk[4] for pk in packs]), 0.1, contacts=2)
    e_jam = 1e-8
    phi, steps = batch.find_jam(e_jam, step=1e-3, min_step=1e-7, ftol=1e-11)
    assert np.all(phi > 0.8) and np.all(phi < 0.95), phi
    e = batch.calc_se()[:, 0]
    assert np.all(np.abs(e - e_jam) < 0.05 * e_jam), e


def _pair(oracle_built, x, y, phi, two):
    R = np.array([0.5, 0.5])
    b = oracle_built.OracleBox(20.0, np.asarray(x, float), np.asarray(y, float),
                               np.asarray(phi, float), R.copy(), R, 0.1, two_point=two)
    b.calc_se()
    e = b.se()[0] * 2
    b.calc_forces()
    f = np.array(b.forces())
    b.close()
    return e, f


def test_one_point_torque_flips_at_parallel_alignment(oracle_built):
    """The one-point rule (src/cpp calc_force_pair) puts the contact at one end of the
    overlapping stretch of two side-by-side spines, and which end flips as the tilt
    passes through zero: the torques jump, so a minimum at parallel alignment is a
    cusp with no zero of the generalised force.  The two-point rule is smooth there."""
    out = {}
    for two in (False, True):
        out[two] = [_pair(oracle_built, [5.0, 5.4], [5.0, 5.95], [t, 0.0], two)[1][2]
                    for t in (-1e-9, 1e-9)]
    (tm, tp) = out[False]
    assert abs(tm[0] - tp[0]) > 0.02  # torque on the tilted spine: +0.005 -> -0.025
    (tm, tp) = out[True]
    assert np.max(np.abs(tm - tp)) < 1e-8


def test_two_point_energy_jumps_where_the_second_contact_ends(oracle_built):
    """The two-point rule (euler_est_2p, src/cuda/2point_dynamics.cu:385-546) drops its
    second contact when the two contact points meet (s1 == s2 or t1 == t2).  Sliding
    two overlapping parallel spines apart along their axis, that happens while the
    second contact still overlaps: the pair energy falls by one contact's share in a
    single step of 5e-4.  Minimisers cannot bring a residual force to zero across such
    a step, which is why FIRE and the reference's CG stall on some jammed states."""
    dxs = np.linspace(0.9, 1.1, 401)
    e = np.array([_pair(oracle_built, [5.0, 5.0 + dx], [5.0, 5.95], [0.0, 0.0], True)[0]
                  for dx in dxs])
    de = np.abs(np.diff(e))
    k = int(np.argmax(de))
    assert abs(dxs[k] - 1.0) < 1e-3  # the spine ends (a = 0.5 each) line up at dx = 2a
    assert de[k] > 0.4 * e[k]  # half of the pair energy (one of two equal contacts)
    rest = np.delete(de, k)
    assert np.max(rest) < 5e-3 * de[k]  # the smooth part changes by 2e-6 per step
