"""Error reporting on the device: capacity and non-finite states come back as status
codes through the C ABI, and the CUDA context stays usable afterwards.

The reference reports neither: its neighbour arrays have a fixed capacity
(nMaxNbrs, src/cuda/spherocyl_box.cpp:352) and a runaway state spins in its wrap
loops (src/cpp/spherocyl_box.cpp:279-290).  The library bounds every list write by
max_nbrs, clamps every cell index and finishes the wrap after 64 periods, so both
failures are safe to provoke.  Nothing here faults the GPU: the failures are a
list capacity that is too small and a time step that throws particles to ~1e306.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


def _packing(sc, n=512, seed=3):
    L, x, y, p, R, A = sc.generate_packing(n, 0.85, 1.0, seed=seed)
    return L, x, y, p, A, R


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_list_capacity_reported(sc, precision):
    from spherocyls_gb300 import _lib

    L, x, y, p, A, R = _packing(sc)
    with pytest.raises(sc.ScError) as ei:
        sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision=precision, max_nbrs=2)
    assert ei.value.status == _lib.SC_E_OVERFLOW
    assert "max_nbrs=2" in str(ei.value)
    # the same packing with room in the lists runs, in the same process
    with sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision=precision) as box:
        box.set_strain_rate(1e-3)
        box.set_step(0.05)
        box.strain_steps(20)
        assert np.all(np.isfinite(np.array(box.state())))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_runaway_state_reported(sc, precision):
    from spherocyls_gb300 import _lib

    L, x, y, p, A, R = _packing(sc, seed=4)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision=precision)
    box.set_strain_rate(1e-3)
    box.set_step(1e306)  # finite, so the setter accepts it; one step throws the particles out
    with pytest.raises(sc.ScError) as ei:
        box.strain_steps(3)
    assert ei.value.status == _lib.SC_E_NAN
    box.close()
    # a new handle on the same device still runs and matches a fresh run bitwise
    outs = []
    for _ in range(2):
        with sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision=precision) as b:
            b.set_strain_rate(1e-3)
            b.set_step(0.05)
            b.strain_steps(10)
            outs.append(np.array(b.state()))
    assert np.array_equal(outs[0], outs[1])
