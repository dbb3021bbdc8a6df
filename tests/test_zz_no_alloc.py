"""sc_forces_noalloc: the allocation-free force entry point.

Callers that cannot let a library allocate device memory (a host program that owns
the GPU's memory budget, a loop that must never reach the allocator) pass their own
device buffers to sc_forces_noalloc, which keeps its cell lists in a fixed device
array.  Its forces must equal those of the regular entry point, sc_calc_forces on an
FP64 handle, within the FP64 tolerance of the other parity tests, on two calls in a
row (the second call reuses the scratch the first one left behind).

The file is named so that pytest collects it last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_forces_noalloc_matches_calc_forces(library):
    torch = pytest.importorskip("torch")
    import spherocyls_gb300 as sc
    from spherocyls_gb300 import _lib

    L, x, y, p, R, A = sc.generate_packing(3000, 0.85, 1.0, seed=41)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    box.set_strain_rate(1e-2)
    box.set_step(0.02)
    box.strain_steps(40)  # a sheared state with gamma != 0
    gamma = box.box()["gamma"]
    xs, ys, ps = box.state()
    box.calc_forces()
    ref = np.array(box.forces())
    rms = np.sqrt(np.mean(ref ** 2))
    assert rms > 0

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    ins = [torch.tensor(v, dtype=torch.float64, device=dev) for v in (xs, ys, ps, R, A)]
    outs = [torch.full((len(xs),), float("nan"), dtype=torch.float64, device=dev)
            for _ in range(3)]
    stream = torch.cuda.current_stream(dev)
    lib = _lib.lib()
    for call in range(2):
        st = lib.sc_forces_noalloc(len(xs), L, gamma, 0.1,
                                   *[ctypes.c_void_p(t.data_ptr()) for t in ins],
                                   *[ctypes.c_void_p(t.data_ptr()) for t in outs],
                                   ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, lib.sc_noalloc_last_error()
        torch.cuda.synchronize()
        got = np.stack([t.cpu().numpy() for t in outs])
        err = np.max(np.abs(got - ref))
        assert err <= TOL * rms, (call, err, rms)


def test_forces_noalloc_rejects_oversize(library):
    from spherocyls_gb300 import _lib

    lib = _lib.lib()
    z = ctypes.c_void_p(0)
    st = lib.sc_forces_noalloc(100000, 10.0, 0.0, 0.1, z, z, z, z, z, z, z, z, z)
    assert st == _lib.SC_E_ARG
    assert b"65536" in lib.sc_noalloc_last_error()
