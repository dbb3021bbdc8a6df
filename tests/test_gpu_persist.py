"""The persistent step kernel of the mixed form: runs of shear steps in one
cooperative launch, the corrector and predictor passes separated by grid barriers,
ending at the first step whose corrector asks for a rebuild.

Each particle's forces are summed over its own list in the same order whichever way
the passes are launched, so the persistent path must reproduce the graph and eager
paths bit for bit: states, stress records and rebuild counts, across Lees-Edwards
set-backs, in batches, and with two-point contacts."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


def _run(sc, packs, rates, steps, se_every, **kw):
    b = sc.BoxBatch([len(pk[1]) for pk in packs], [pk[0] for pk in packs],
                    np.concatenate([pk[1] for pk in packs]), np.concatenate([pk[2] for pk in packs]),
                    np.concatenate([pk[3] for pk in packs]), np.concatenate([pk[5] for pk in packs]),
                    np.concatenate([pk[4] for pk in packs]), 0.2, precision="mixed", **kw)
    for s, r in enumerate(rates):
        b.set_strain_rate(r, sys=s)
    b.set_step(0.02)
    se = b.strain_steps(steps, se_every=se_every)
    out = (np.array(b.state()), se, b.counters()["rebuilds"], b.box(0)["gamma"])
    b.close()
    return out


@pytest.mark.parametrize("contacts", [1, 2])
def test_persistent_steps_equal_graph_and_eager(sc, contacts):
    # 600 steps at strain 1e-3 per step: gamma passes 1/2 (a set-back) at step 500
    packs = [sc.generate_packing(5000, 0.85, 1.0, seed=81)]
    ref = _run(sc, packs, [0.05], 600, 50, contacts=contacts)
    assert ref[2] > 2 and ref[3] < 0.2  # rebuilt several times and set back
    for kw in (dict(persist_steps=True), dict(persist_steps=True, use_graphs=False),
               dict(use_graphs=False)):
        got = _run(sc, packs, [0.05], 600, 50, contacts=contacts, **kw)
        assert np.array_equal(got[0], ref[0]), kw
        assert np.array_equal(got[1], ref[1]), kw
        assert got[2] == ref[2] and got[3] == ref[3], kw


def test_persistent_steps_in_a_batch(sc):
    packs = [sc.generate_packing(n, phi, a, seed=s)
             for n, phi, a, s in ((64, 0.8, 0.5, 91), (3000, 0.86, 1.0, 92), (700, 0.84, 2.0, 93))]
    rates = [1e-3, 3e-2, 5e-4]
    ref = _run(sc, packs, rates, 300, 7)
    got = _run(sc, packs, rates, 300, 7, persist_steps=True)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    assert got[2] == ref[2]


def _fire(sc, packs, ftol, iters, **kw):
    b = sc.BoxBatch([len(pk[1]) for pk in packs], [pk[0] * 0.97 for pk in packs],
                    np.concatenate([pk[1] * 0.97 for pk in packs]),
                    np.concatenate([pk[2] * 0.97 for pk in packs]),
                    np.concatenate([pk[3] for pk in packs]), np.concatenate([pk[5] for pk in packs]),
                    np.concatenate([pk[4] for pk in packs]), 0.1, precision="mixed", **kw)
    it, fm, dn = b.fire_minimize(ftol, iters)
    per = b.fire_iterations()
    assert per.max() == it and np.all(per <= iters)
    out = (np.array(b.state()), it, fm, dn, b.counters()["rebuilds"], per)
    b.close()
    return out


@pytest.mark.parametrize("contacts", [1, 2])
def test_persistent_fire_equals_graph_and_eager(sc, contacts):
    """FIRE from affinely compressed packings (3% in length: overlaps to relax, list
    rebuilds on the way); one system converges early and stops taking force passes."""
    packs = [sc.generate_packing(n, phi, a, seed=s)
             for n, phi, a, s in ((3000, 0.80, 1.0, 95), (500, 0.6, 0.5, 96), (1200, 0.84, 2.0, 97))]
    ref = _fire(sc, packs, 1e-6, 3000, contacts=contacts)
    assert ref[4] > 0 and ref[3].any()
    for kw in (dict(persist_steps=True), dict(use_graphs=False)):
        got = _fire(sc, packs, 1e-6, 3000, contacts=contacts, **kw)
        assert np.array_equal(got[0], ref[0]), kw
        assert got[1] == ref[1] and np.array_equal(got[2], ref[2]), kw
        assert np.array_equal(got[3], ref[3]) and got[4] == ref[4], kw
        assert np.array_equal(got[5], ref[5]), kw
