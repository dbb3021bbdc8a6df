"""Ragged batches: systems of 2 to 5000 particles in one handle (the smallest with a
single cell, where the reference's table lists cells twice and the library walks
distinct cells), square and rectangular, each at its own rate, advance and record
stress/energy exactly as they do alone, for shear and for resize."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (n, packing, a/R, rate, seed, Ly/Lx)
SPECS = [(2, 0.30, 1.0, 1e-3, 71, 1.0), (7, 0.60, 0.5, 2e-3, 72, 1.0),
         (64, 0.84, 1.0, 5e-4, 73, 1.0), (5000, 0.85, 1.0, 1e-3, 74, 1.0),
         (300, 0.80, 2.0, 3e-3, 75, 2.0)]


@pytest.fixture(scope="module")
def sc(library):
    import spherocyls_gb300

    return spherocyls_gb300


def _configs(sc):
    out = []
    for n, phi, a, rate, seed, asp in SPECS:
        # crossing-free in its own box (an affine stretch of a square packing is not)
        Lx, Ly, x, y, p, R, A = sc.generate_config_rect(n, phi, a, 1.0 / asp, seed=seed)
        out.append((Lx, Ly, x, y, p, A, R, rate))
    return out


def _run(box, kind, steps, every):
    if kind == "shear":
        return box.strain_steps(steps, se_every=every)
    return box.resize_steps(steps, shrink=True, se_every=every)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["shear", "resize"])
def test_ragged_batch_matches_single_runs(sc, precision, kind):
    cfg = _configs(sc)
    singles = []
    for Lx, Ly, x, y, p, A, R, rate in cfg:
        with sc.SpherocylBox(Lx, x, y, p, A, R, 0.1, Ly=Ly, precision=precision) as b:
            b.set_strain_rate(rate) if kind == "shear" else b.set_resize_rate(rate)
            b.set_step(0.02)
            rec = _run(b, kind, 120, 30)[:, 0, :]
            singles.append((np.array(b.state()), rec, b.box()))
    cat = lambda k: np.concatenate([c[k] for c in cfg])  # noqa: E731
    bb = sc.BoxBatch([len(c[2]) for c in cfg], [c[0] for c in cfg], cat(2), cat(3), cat(4),
                     cat(5), cat(6), 0.1, Ly=[c[1] for c in cfg], precision=precision)
    for s, c in enumerate(cfg):
        bb.set_strain_rate(c[7], sys=s) if kind == "shear" else bb.set_resize_rate(c[7], sys=s)
    bb.set_step(0.02)
    rec = _run(bb, kind, 120, 30)
    st = np.array(bb.state())
    off = 0
    for s, c in enumerate(cfg):
        n = len(c[2])
        sst, srec, sbox = singles[s]
        assert np.array_equal(st[:, off:off + n], sst), (s, n)
        assert np.array_equal(rec[:, s, :], srec), (s, n)
        box = bb.box(s)
        assert box["Lx"] == sbox["Lx"] and box["Ly"] == sbox["Ly"] and box["gamma"] == sbox["gamma"]
        off += n


@pytest.mark.parametrize("shrink", [True, False])
def test_rectangular_resize_through_a_regrid(sc, shrink):
    """A 1 x 2 box shrinks (or grows) through a change of its cell grid: the run ends,
    the grid follows the box, the box lengths are the product of the step factors,
    and the mixed form tracks the FP64 form."""
    Lx, Ly, x, y, p, R, A = sc.generate_config_rect(3000, 0.70, 1.0, 0.5, seed=76)
    rate, dt, steps = 1e-2, 0.02, 400  # lengths change by 8%: several row changes
    out = []
    for prec in ("fp64", "mixed"):
        with sc.SpherocylBox(Lx, x, y, p, A, R, 0.1, Ly=Ly, precision=prec) as b:
            g0 = b.box()
            b.set_resize_rate(rate)
            b.set_step(dt)
            b.resize_steps(steps, shrink=shrink)
            g1 = b.box()
            out.append((np.array(b.state()), g0, g1, b.calc_se()[0]))
    (sa, g0, ga, ea), (sb, _, gb, eb) = out
    f = (1 - rate) ** dt
    lx, ly = Lx, Ly
    for _ in range(steps):
        lx, ly = (lx * f, ly * f) if shrink else (lx / f, ly / f)
    assert ga["Lx"] == gb["Lx"] == lx and ga["Ly"] == gb["Ly"] == ly
    assert (ga["rows"], ga["cols"]) != (g0["rows"], g0["cols"])
    hmin = 2 * (R.max() + A.max()) + ga["pad"]
    assert ga["rows"] == max(int(ga["Ly"] / hmin), 1)
    assert abs(ea - eb) <= 1e-3 * max(abs(ea), 1e-12)
