"""The reference's Polak-Ribiere conjugate-gradient minimiser (cjpr_relax_2p /
cjpr_relax_step_2p / line_search_2p, src/cuda/2point_dynamics.cu:3609-4296).

The reference's CG exists only in CUDA, so the oracle's restatement (orc_cg_minimize)
is checked by what the algorithm guarantees (energies never rise, the stop rules),
and the device form against the oracle: the same iterates within 1e-9 of the box
over the first iterations, where every line-search decision compares energies that
differ far above rounding.  Later iterates part at rounding level (the energies are
summed in different orders), so the full runs are compared by their outcome."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import REF_PI, periodic_diff


def _packing(sc, n=256, phi=0.88, seed=5):
    L, x, y, p, R, A = sc.generate_packing(n, phi, 1.0, seed=seed)
    return L, x, y, p, A, R


def test_oracle_cg_descends_and_stops(library, oracle_built):
    """Energies fall monotonically; with two contact points the unjammed packing
    relaxes to zero energy and the run stops on its energy rule with forces at
    rounding level; with one contact point the energy cusp at parallel alignment
    stops it on the same rule with residual forces (the reason FIRE and the
    reference's jamming code use two points)."""
    import spherocyls_gb300 as sc

    L, x, y, p, A, R = _packing(sc)
    energies = []
    for m in (1, 5, 20, 100):
        ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.2, two_point=True)
        energies.append(ob.cg_minimize(m)[1])
    assert all(b < a for a, b in zip(energies, energies[1:]))
    ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.2, two_point=True)
    it, e, why = ob.cg_minimize(5000)
    fx, fy, tq = ob.forces()
    assert why in (1, 2) and e < 1e-20
    assert np.max(np.hypot(fx, fy)) < 1e-12 and np.max(np.abs(tq)) < 1e-12
    ob1 = oracle_built.OracleBox(L, x, y, p, A, R, 0.2)
    it1, e1, why1 = ob1.cg_minimize(5000)
    assert why1 == 2 and e1 > 1e-7


sc_gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


@sc_gpu
@pytest.mark.parametrize("contacts", [1, 2])
def test_cg_first_iterations_match_oracle(sc, oracle_built, contacts):
    L, x, y, p, A, R = _packing(sc)
    for m in (1, 3, 8):
        ob = oracle_built.OracleBox(L, x, y, p, A, R, 0.2, two_point=contacts == 2)
        oit, oe, _ = ob.cg_minimize(m)
        with sc.SpherocylBox(L, x, y, p, A, R, 0.2, contacts=contacts) as b:
            it, e, why = b.cg_minimize(m)
            assert it[0] == oit == m and why[0] == 4
            assert abs(e[0] - oe) <= 1e-9 * abs(oe)
            X, Y, P = b.state()
            ox, oy, op = ob.state()
            assert np.max(np.abs(periodic_diff(X, ox, L))) <= 1e-9 * L, m
            assert np.max(np.abs(periodic_diff(Y, oy, L))) <= 1e-9 * L, m
            assert np.max(np.abs(periodic_diff(P, op, 2 * REF_PI))) <= 1e-9, m


@sc_gpu
def test_cg_graph_and_eager_identical(sc):
    """The WHILE-node line search and the host-driven one give the same iterates
    bit for bit."""
    L, x, y, p, A, R = _packing(sc, n=400, seed=6)
    out = []
    for graphs in (False, True):
        with sc.SpherocylBox(L, x, y, p, A, R, 0.2, contacts=2, use_graphs=graphs) as b:
            it, e, why = b.cg_minimize(60)
            out.append((it[0], e[0], np.array(b.state())))
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])


@sc_gpu
def test_cg_batched_matches_single(sc):
    cfg = [_packing(sc, n=300, phi=ph, seed=s) for ph, s in ((0.88, 7), (0.9, 8))]
    singles = []
    for L, x, y, p, A, R in cfg:
        with sc.SpherocylBox(L, x, y, p, A, R, 0.2, contacts=2) as b:
            singles.append((b.cg_minimize(150), np.array(b.state())))
    cat = lambda k: np.concatenate([c[k] for c in cfg])  # noqa: E731
    bb = sc.BoxBatch([300, 300], [c[0] for c in cfg], cat(1), cat(2), cat(3), cat(4), cat(5),
                     0.2, contacts=2)
    it, e, why = bb.cg_minimize(150)
    st = np.array(bb.state())
    for k in range(2):
        (sit, se, swhy), sst = singles[k]
        assert it[k] == sit[0] and e[k] == se[0] and why[k] == swhy[0]
        assert np.array_equal(st[:, 300 * k:300 * (k + 1)], sst)


@sc_gpu
def test_cg_converges_with_two_contact_points(sc):
    """The full run stops on the reference's energy rule with forces at rounding
    level, as the oracle's does, and reaches the same zero energy."""
    L, x, y, p, A, R = _packing(sc)
    with sc.SpherocylBox(L, x, y, p, A, R, 0.2, contacts=2) as b:
        it, e, why = b.cg_minimize(5000)
        assert why[0] in (1, 2) and e[0] < 1e-20
        b.calc_forces()
        fx, fy, tq = b.forces()
        assert np.max(np.hypot(fx, fy)) < 1e-12 and np.max(np.abs(tq)) < 1e-12


@sc_gpu
def test_cg_refuses_the_mixed_form(sc):
    L, x, y, p, A, R = _packing(sc, n=64, seed=9)
    with sc.SpherocylBox(L, x, y, p, A, R, 0.2, precision="mixed") as b:
        with pytest.raises(sc.ScError):
            b.cg_minimize(10)


@sc_gpu
@pytest.mark.parametrize("graphs", [True, False])
def test_cg_probe_cap_stops_the_search_with_a_status(sc, graphs):
    """A line search that still wants another energy probe after the handle's probe
    cap (here 2; every search takes at least three probes: the step, twice the
    step or a halving, and the parabola's minimum) ends its system with reason 5
    and sc_cg_minimize returns SC_E_NOCONV, through the graph WHILE node and the
    host-driven loop alike; the handle stays usable."""
    import ctypes

    from spherocyls_gb300 import _lib

    L, x, y, p, A, R = _packing(sc)
    b = sc.BoxBatch([256, 256], [L, L], np.r_[x, x], np.r_[y, y], np.r_[p, p], np.r_[A, A],
                    np.r_[R, R], 0.2, use_graphs=graphs, cg_max_probes=2)
    it = np.zeros(2, dtype=np.int32)
    e = np.zeros(2)
    why = np.zeros(2, dtype=np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    st = _lib.lib().sc_cg_minimize(b.h, 100, it.ctypes.data_as(ip),
                                   e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   why.ctypes.data_as(ip))
    assert st == _lib.SC_E_NOCONV
    assert list(why) == [5, 5] and list(it) == [1, 1]
    assert b"probe cap" in _lib.lib().sc_last_error(b.h)
    b.calc_forces()  # still usable
    assert np.all(np.isfinite(np.array(b.forces())))
    b.close()
