"""sc_forces_noalloc: the allocation-free force entry point.

Callers that cannot let a library allocate device memory (a host program that owns
the GPU's memory budget, a loop that must never reach the allocator) pass their own
device buffers to sc_forces_noalloc, which keeps its cell lists in a fixed device
array.  Its forces must equal those of the regular entry point, sc_calc_forces on an
FP64 handle, within the FP64 tolerance of the other parity tests, on two calls in a
row (the second call reuses the scratch the first one left behind).  The cases cover
a small sheared box, a box near the size limit (whose cell grid is coarsened to fit
the fixed array), and a shear offset past gamma = 1/2 (widened cells).

The file is named so that pytest collects it last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

TOL = 1e-12


def _sheared_state(n, seed, rate, steps, gamma_max=None):
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(n, 0.85, 1.0, seed=seed)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    box.set_strain_rate(rate)
    box.set_step(0.02)
    if gamma_max is None:
        box.strain_steps(steps)  # a sheared state with gamma != 0
    else:
        box.strain_to_gamma(gamma_max)  # past 1/2 without set-back, widened cells
    gamma = box.box()["gamma"]
    xs, ys, ps = box.state()
    box.calc_forces()
    ref = np.array(box.forces())
    box.close()
    return L, gamma, (xs, ys, ps, R, A), ref


def _noalloc_twice(L, gamma, arrays, ref):
    torch = pytest.importorskip("torch")
    from spherocyls_gb300 import _lib

    rms = np.sqrt(np.mean(ref ** 2))
    assert rms > 0
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    n = len(arrays[0])
    ins = [torch.tensor(v, dtype=torch.float64, device=dev) for v in arrays]
    outs = [torch.full((n,), float("nan"), dtype=torch.float64, device=dev) for _ in range(3)]
    stream = torch.cuda.current_stream(dev)
    lib = _lib.lib()
    for call in range(2):
        st = lib.sc_forces_noalloc(n, L, gamma, 0.1,
                                   *[ctypes.c_void_p(t.data_ptr()) for t in ins],
                                   *[ctypes.c_void_p(t.data_ptr()) for t in outs],
                                   ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, lib.sc_noalloc_last_error()
        torch.cuda.synchronize()
        got = np.stack([t.cpu().numpy() for t in outs])
        err = np.max(np.abs(got - ref))
        assert err <= TOL * rms, (call, err, rms)


@pytest.mark.gpu
def test_forces_noalloc_matches_calc_forces(library):
    L, gamma, arrays, ref = _sheared_state(3000, 41, 1e-2, 40)
    assert 0 < abs(gamma) < 0.5
    _noalloc_twice(L, gamma, arrays, ref)


@pytest.mark.gpu
def test_forces_noalloc_coarsened_grid_near_the_limit(library):
    # 65536 particles at packing 0.85 need about 135 x 150 cells of the regular
    # width, more than the fixed array's 16384: the grid is coarsened to larger cells
    L, gamma, arrays, ref = _sheared_state(65536, 43, 1e-2, 10)
    _noalloc_twice(L, gamma, arrays, ref)


@pytest.mark.gpu
def test_forces_noalloc_past_half_strain(library):
    L, gamma, arrays, ref = _sheared_state(3000, 47, 5e-1, 0, gamma_max=0.8)
    assert 0.79 < gamma < 0.82
    _noalloc_twice(L, gamma, arrays, ref)


def test_forces_noalloc_rejects_oversize_and_bad_gamma(library):
    from spherocyls_gb300 import _lib

    lib = _lib.lib()
    z = ctypes.c_void_p(0)
    st = lib.sc_forces_noalloc(100000, 10.0, 0.0, 0.1, z, z, z, z, z, z, z, z, z)
    assert st == _lib.SC_E_ARG
    assert b"65536" in lib.sc_noalloc_last_error()
    # rejected before any device work: the pointers are never dereferenced
    buf = (ctypes.c_double * 4)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    for g in (float("nan"), float("inf")):
        st = lib.sc_forces_noalloc(2, 10.0, g, 0.1, p, p, p, p, p, p, p, p, z)
        assert st == _lib.SC_E_ARG
        assert b"gamma" in lib.sc_noalloc_last_error()
