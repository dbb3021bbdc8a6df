"""CPU checks of the C ABI: the library loads, exports every declared entry point,
validates arguments without touching a GPU, and its host-side packing generator
is reproducible and crossing-free."""
from __future__ import annotations

import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared_symbols() -> list[str]:
    hdr = open(os.path.join(ROOT, "include", "spherocyl.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(sc_[a-z0-9_]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol(library):
    names = _declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(library, n), n


def test_binding_covers_header():
    from spherocyls_gb300 import _lib

    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(_declared_symbols()) <= bound


def test_create_rejects_bad_arguments_without_gpu(library):
    import ctypes

    from spherocyls_gb300 import _lib

    h = ctypes.c_void_p()
    n = (ctypes.c_int * 1)(1)
    L = (ctypes.c_double * 1)(10.0)
    a = (ctypes.c_double * 1)(0.5)
    st = library.sc_create(None, 1, n, L, None, a, a, a, a, a, ctypes.byref(h))
    assert st == _lib.SC_E_ARG  # a system needs at least two particles
    assert b"n >= 2" in library.sc_last_error(None)
    n2 = (ctypes.c_int * 1)(2)
    bad = (ctypes.c_double * 2)(float("nan"), 1.0)
    ok = (ctypes.c_double * 2)(0.5, 0.5)
    st = library.sc_create(None, 1, n2, L, None, bad, ok, ok, ok, ok, ctypes.byref(h))
    assert st == _lib.SC_E_NAN
    assert library.sc_status_string(_lib.SC_E_OVERFLOW) == b"capacity exceeded"


def test_create_checks_every_particle_of_large_inputs_without_gpu(library):
    """Above 65536 particles the input checks run on several host threads over
    slices of the arrays: a bad value anywhere, in any system, is still reported
    (non-finite before a bad shape, as for small inputs)."""
    import ctypes

    from spherocyls_gb300 import _lib

    sizes = [70000, 50001, 30000]
    ntot = sum(sizes)
    n = (ctypes.c_int * 3)(*sizes)
    L = (ctypes.c_double * 3)(800.0, 700.0, 600.0)
    dp = ctypes.POINTER(ctypes.c_double)

    def create(arrays):
        h = ctypes.c_void_p()
        ptrs = [a.ctypes.data_as(dp) for a in arrays]
        return library.sc_create(None, 3, n, L, None, *ptrs, ctypes.byref(h))

    base = [np.full(ntot, 1.0), np.full(ntot, 2.0), np.zeros(ntot), np.full(ntot, 0.5),
            np.full(ntot, 0.5)]  # x, y, phi, R, A
    for k, idx, val, want in ((0, ntot - 1, np.nan, _lib.SC_E_NAN),
                              (2, 70000 + 123, np.inf, _lib.SC_E_NAN),
                              (3, 70000 + 50000, -0.5, _lib.SC_E_ARG),
                              (4, 5, -1e-9, _lib.SC_E_ARG),
                              (3, 0, 0.0, _lib.SC_E_ARG)):
        arrays = [a.copy() for a in base]
        arrays[k][idx] = val
        assert create(arrays) == want, (k, idx, val)
    arrays = [a.copy() for a in base]
    arrays[3][100] = -1.0
    arrays[0][140000] = np.nan
    assert create(arrays) == _lib.SC_E_NAN  # the non-finite input is reported first


def test_generator_reproducible_and_crossing_free(library):
    from spherocyls_gb300 import generate_packing

    L1, x1, y1, p1, R1, A1 = generate_packing(300, 0.85, 1.0, seed=5)
    L2, x2, y2, p2, R2, A2 = generate_packing(300, 0.85, 1.0, seed=5)
    assert L1 == L2 and np.array_equal(x1, x2) and np.array_equal(p1, p2)
    _, x3, *_ = generate_packing(300, 0.85, 1.0, seed=6)
    assert not np.array_equal(x1, x3)
    # bidisperse alternation and packing fraction
    assert np.all(R1[0::2] == 0.5) and np.allclose(R1[1::2], 0.7) and np.allclose(A1, R1)
    phi = np.sum(np.pi * R1 ** 2 + 4 * A1 * R1) / L1 ** 2
    assert abs(phi - 0.85) < 1e-12
    assert np.all((x1 >= 0) & (x1 < L1) & (p1 >= 0) & (p1 < np.pi))
    # minimum spine separation >= 0.1 sigma (brute force, sampled segments)
    s = np.linspace(-1, 1, 41)
    ux, uy = A1 * np.cos(p1), A1 * np.sin(p1)
    worst = np.inf
    for i in range(len(x1)):
        dx = x1[i] - x1
        dy = y1[i] - y1
        dx -= L1 * np.round(dx / L1)
        dy -= L1 * np.round(dy / L1)
        near = np.nonzero((dx ** 2 + dy ** 2 < (2 * A1.max() + 0.2) ** 2) & (np.arange(len(x1)) != i))[0]
        for j in near:
            ax = dx[j] + s[:, None] * ux[i] - s[None, :] * ux[j]
            ay = dy[j] + s[:, None] * uy[i] - s[None, :] * uy[j]
            worst = min(worst, np.sqrt(ax ** 2 + ay ** 2).min() / (R1[i] + R1[j]))
    assert worst >= 0.1 - 1e-9


def test_generator_rejects_bad_arguments(library):
    from spherocyls_gb300 import ScError, generate_packing

    with pytest.raises(ScError):
        generate_packing(10, 1.5, 1.0)


def test_generate_config_variants(library, oracle_built):
    """The reference's initial configurations: zero-energy placement has no overlap
    (the oracle's energy is exactly zero), aligned and evenly spaced angles, grid
    layout, Gamma-distributed aspect ratios with the requested mean and spread, the
    steady-shear angle distribution concentrated along the flow, and the packing
    fraction exactly as requested in every case."""
    import spherocyls_gb300 as sc

    def packing(L, R, A):
        return np.sum(np.pi * R * R + 4 * A * R) / L ** 2

    # random sequential placement without overlap jams near 0.55 at a/R = 1
    L, x, y, p, R, A = sc.generate_config(400, 0.45, 1.0, max_overlap=0.0, seed=3)
    assert abs(packing(L, R, A) - 0.45) < 1e-12
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.1)
    ob.calc_se()
    assert ob.se()[0] == 0.0
    ob.close()

    L, x, y, p, R, A = sc.generate_config(300, 0.5, 1.0, angle_range=(0.5, 0.5), seed=4)
    assert np.all(p == 0.0)
    L, x, y, p, R, A = sc.generate_config(300, 0.5, 1.0, angles="even", seed=4)
    d = np.diff(np.sort(p))
    assert np.allclose(d, np.pi / 300, rtol=1e-9)

    L, x, y, p, R, A = sc.generate_config(256, 0.45, 1.0, layout="grid", seed=5)
    assert abs(packing(L, R, A) - 0.45) < 1e-12
    assert np.all((x >= 0) & (x < L) & (y >= 0) & (y < L))
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.1)
    ob.calc_se()
    assert np.isfinite(ob.se()[0])
    ob.close()

    L, x, y, p, R, A = sc.generate_config(4000, 0.5, 1.0, a_sigma=0.3, seed=6)
    alpha = A / R
    assert abs(alpha.mean() - 1.0) < 0.03 and abs(alpha.std() - 0.3) < 0.03
    assert abs(packing(L, R, A) - 0.5) < 1e-12

    L, x, y, p, R, A = sc.generate_config(2000, 0.3, 2.0, shear_angles=True, seed=7)
    assert np.mean(np.cos(2 * p)) > 0.3
    L, x, y, p, R, A = sc.generate_config(2000, 0.3, 2.0, seed=7)
    assert abs(np.mean(np.cos(2 * p))) < 0.1

    with pytest.raises(sc.ScError):
        sc.generate_config(100, 0.5, 1.0, angle_range=(0.6, 0.4))
