"""The CUDA-only parts of the path against the reference's own CUDA kernels.

tests/golden/ref_cuda_2p.npz holds outputs of tmarschall/spherocyls'
src/cuda/2point_dynamics.cu kernels, compiled where they lie and run on a GPU by
tests/golden/make_golden_cuda.py: the two-point contact forces of calc_fe_2p
(the rule of euler_est_2p, :385-546) on 400 isolated pairs and on a dense packing,
and one pure-shear step (pure_euler_est_2p + pure_heun_corr_2p, :1663-2178, with
the host sequence of pure_strain_step_2p, :2180-2283) with unit drag.

The oracle's restatement (force_pair2 and the pure-shear step in
oracle/spherocyl_oracle.c) is checked here on the CPU; the CUDA library in the
gpu-marked tests.  The kernels are compiled with the reference's default flags
(fused multiply-adds) and use CUDA's cos/sin, so the comparisons allow rounding:
forces within 1e-10 of the RMS force, positions within 1e-12 of the box.  Exactly
or nearly parallel spines are the exception the reference's own case analysis
makes: whether a c - b^2 comes out as zero or as a rounding residue decides its
branch, so those pairs are compared only where both evaluations took the same
branch (the force differs by more than rounding otherwise), and the test counts
how many did.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, periodic_diff

TOL_F = 1e-10


def _case(g, name):
    k = name + "_"
    return (float(g[k + "L"]), g[k + "x"], g[k + "y"], g[k + "phi"], g[k + "R"], g[k + "A"],
            float(g[k + "gamma"]))


def _near_parallel(phi, pair_index):
    """Pairs whose spines are parallel to within 1e-6 rad (either direction)."""
    d = np.abs(np.sin(phi[0::2] - phi[1::2]))
    return d < 1e-6


def _compare_pairs(f, g):
    ref = np.stack([g["pairs_fx"], g["pairs_fy"], g["pairs_tau"]])
    rms = np.sqrt(np.mean(ref ** 2))
    err = np.abs(f - ref).max(axis=0)  # per particle
    per_pair = np.maximum(err[0::2], err[1::2])
    par = _near_parallel(g["pairs_phi"], None)
    assert np.all(per_pair[~par] <= TOL_F * rms), per_pair[~par].max() / rms
    agree = per_pair[par] <= TOL_F * rms
    # most near-parallel pairs take the same branch in both evaluations
    assert agree.sum() >= 0.5 * par.sum(), (agree.sum(), par.sum())
    return int(par.sum()), int(agree.sum())


def test_oracle_two_point_forces_match_reference_cuda(oracle_built):
    g = load_golden("ref_cuda_2p")
    L, x, y, p, R, A, gam = _case(g, "pairs")
    b = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, gamma=gam, two_point=True)
    _compare_pairs(np.array(b.forces()), g)
    b.close()
    L, x, y, p, R, A, gam = _case(g, "dense")
    b = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, gamma=gam, two_point=True)
    f = np.array(b.forces())
    ref = np.stack([g["dense_fx"], g["dense_fy"], g["dense_tau"]])
    assert np.max(np.abs(f - ref)) <= TOL_F * np.sqrt(np.mean(ref ** 2))
    b.close()


def test_oracle_pure_shear_step_matches_reference_cuda(oracle_built):
    g = load_golden("ref_cuda_2p")
    L, x, y, p, R, A, _ = _case(g, "dense")
    b = oracle_built.OracleBox(L, x, y, p, A, R, 0.1, strain_rate=float(g["pure_rate"]),
                               step=float(g["pure_step"]), two_point=True)
    b.run_pure_steps(1)
    xs, ys, ps = b.state()
    sc = b.scalars()
    assert abs(sc["Lx"] - float(g["pure_Lx"])) <= 1e-14 * L
    assert abs(sc["Ly"] - float(g["pure_Ly"])) <= 1e-14 * L
    assert np.max(np.abs(periodic_diff(xs, g["pure_x"], sc["Lx"]))) <= 1e-12 * L
    assert np.max(np.abs(periodic_diff(ys, g["pure_y"], sc["Ly"]))) <= 1e-12 * L
    assert np.max(np.abs(periodic_diff(ps, g["pure_phi"], 2 * np.pi))) <= 1e-12
    b.close()


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_library_two_point_forces_match_reference_cuda(sc, precision):
    g = load_golden("ref_cuda_2p")
    tol = TOL_F if precision == "fp64" else 1e-4
    for name in ("pairs", "dense"):
        L, x, y, p, R, A, gam = _case(g, name)
        b = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=precision, contacts=2)
        b.set_gamma(gam)
        b.calc_forces()
        f = np.array(b.forces())
        b.close()
        if name == "pairs" and precision == "fp64":
            _compare_pairs(f, g)
        else:
            ref = np.stack([g[name + "_fx"], g[name + "_fy"], g[name + "_tau"]])
            err = np.abs(f - ref).max(axis=0)
            rms = np.sqrt(np.mean(ref ** 2))
            if name == "pairs":  # FP32 geometry: the near-parallel branch may differ
                par = np.repeat(_near_parallel(g["pairs_phi"], None), 2)
                err = err[~par]
            assert np.max(err) <= tol * rms


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_library_pure_shear_step_matches_reference_cuda(sc, precision):
    g = load_golden("ref_cuda_2p")
    L, x, y, p, R, A, _ = _case(g, "dense")
    b = sc.SpherocylBox(L, x, y, p, A, R, 0.1, precision=precision, contacts=2)
    b.set_strain_rate(float(g["pure_rate"]))
    b.set_step(float(g["pure_step"]))
    b.pure_strain_steps(1)
    xs, ys, ps = b.state()
    bx = b.box()
    b.close()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert abs(bx["Lx"] - float(g["pure_Lx"])) <= 1e-14 * L
    assert abs(bx["Ly"] - float(g["pure_Ly"])) <= 1e-14 * L
    assert np.max(np.abs(periodic_diff(xs, g["pure_x"], bx["Lx"]))) <= tol * L
    assert np.max(np.abs(periodic_diff(ys, g["pure_y"], bx["Ly"]))) <= tol * L
    assert np.max(np.abs(periodic_diff(ps, g["pure_phi"], 2 * np.pi))) <= tol * 10
