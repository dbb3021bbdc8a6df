"""Position files, stress/energy files, run protocols with output and the CLIs.

CPU: the reader accepts both header layouts of the reference (src/cpp 7 fields,
src/cuda 8 fields).  GPU: run_strain / resize / minimise write the reference's file
names and line layouts, a continued run rewrites the SE file from the start time,
and the command-line drivers take the input_key.txt argument order.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _write_sp(path, n, L, x, y, p, R, A, gamma=0.0, gt=0.0, rate=1e-3, dt=0.02, packing=0.85):
    with open(path, "w") as f:
        f.write(f"{n} {L!r} {packing} {gamma} {gt} {rate} {dt}\n")
        for k in range(n):
            f.write(f"{float(x[k])!r} {float(y[k])!r} {float(p[k])!r} {float(R[k])} {float(A[k])}\n")


def test_read_positions_both_headers(library, tmp_path):
    from spherocyls_gb300 import read_positions

    rng = np.random.default_rng(0)
    n = 10
    x, y, p = rng.uniform(0, 5, (3, n))
    R = np.full(n, 0.5)
    A = np.full(n, 0.5)
    sp = tmp_path / "sp0000000123.dat"
    _write_sp(sp, n, 5.0, x, y, p, R, A, gamma=0.1, gt=1.1)
    hdr, xx, yy, pp, RR, AA = read_positions(str(sp))
    assert hdr["Lx"] == hdr["Ly"] == 5.0 and hdr["gamma"] == 0.1 and hdr["gamma_total"] == 1.1
    assert np.array_equal(xx, x) and np.array_equal(pp, p) and np.array_equal(AA, A)
    sd = tmp_path / "sd0000000007.dat"
    with open(sd, "w") as f:
        f.write(f"{n} 5.0 6.0 0.850000 0.2 3.5 0.001 0.02\n")
        for k in range(n):
            f.write(f"{float(x[k])!r} {float(y[k])!r} {float(p[k])!r} 0.5 {float(A[k])!r}\n")
    hdr, xx, *_ = read_positions(str(sd))
    assert hdr["Lx"] == 5.0 and hdr["Ly"] == 6.0 and hdr["gamma"] == 0.2 and hdr["dt"] == 0.02
    assert np.array_equal(xx, x)


def test_read_binary_positions(library, tmp_path):
    """The src/cuda binary layout (save_positions_bin): int N, the sd header's seven
    doubles, then x y phi R A per particle, host byte order."""
    import struct

    from spherocyls_gb300 import ScError, read_positions

    rng = np.random.default_rng(1)
    n = 7
    vals = rng.uniform(0, 5, (n, 5))
    head = (5.0, 6.0, 0.85, 0.25, 3.25, 1e-4, 0.02)
    path = tmp_path / "sd0000000042.bin"
    with open(path, "wb") as f:
        f.write(struct.pack("=i7d", n, *head))
        for row in vals:
            f.write(struct.pack("=5d", *row))
    hdr, x, y, p, R, A = read_positions(str(path))
    assert [hdr[k] for k in ("Lx", "Ly", "packing", "gamma", "gamma_total", "rate", "dt")] == \
        list(head)
    assert np.array_equal(np.stack([x, y, p, R, A], axis=1), vals)
    short = tmp_path / "short.bin"
    with open(short, "wb") as f:
        f.write(struct.pack("=i7d", n, *head) + struct.pack("=5d", *vals[0]))
    with pytest.raises(ScError):
        read_positions(str(short))


def test_read_gzip_positions(library, tmp_path):
    """A gzip-compressed position file (GzFileInput, src/cpp/gz_file_input.cpp) reads
    as the plain one; corrupt data is an error, not a short read."""
    import gzip

    from spherocyls_gb300 import ScError, read_positions

    rng = np.random.default_rng(2)
    n = 1000
    x, y, p = rng.uniform(0, 5, (3, n))
    R = np.full(n, 0.5)
    A = np.full(n, 0.25)
    sp = tmp_path / "sp0000000050.dat"
    _write_sp(sp, n, 5.0, x, y, p, R, A, gamma=0.3, gt=2.5)
    gz = tmp_path / "sp0000000050.dat.gz"
    gz.write_bytes(gzip.compress(sp.read_bytes()))
    plain = read_positions(str(sp))
    packed = read_positions(str(gz))
    assert plain[0] == packed[0]
    for a, b in zip(plain[1:], packed[1:]):
        assert np.array_equal(a, b)
    bad = tmp_path / "bad.dat.gz"
    data = gzip.compress(sp.read_bytes())
    bad.write_bytes(data[: len(data) // 2])
    with pytest.raises(ScError):
        read_positions(str(bad))


def test_read_positions_errors(library, tmp_path):
    from spherocyls_gb300 import ScError, read_positions

    bad = tmp_path / "bad.dat"
    bad.write_text("3 4.0 0.8\n1 2 3 4 5\n")
    with pytest.raises(ScError):
        read_positions(str(bad))
    short = tmp_path / "short.dat"
    short.write_text("3 4.0 0.8 0 0 0.001 0.02\n1 2 3 0.5 0.5\n")
    with pytest.raises(ScError):
        read_positions(str(short))
    with pytest.raises(ScError):
        read_positions(str(tmp_path / "missing.dat"))


@pytest.mark.gpu
def test_run_strain_files_and_continue(library, tmp_path):
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(300, 0.85, 1.0, seed=3)
    rate, dt = 1e-2, 0.02
    d1 = tmp_path / "one"
    d1.mkdir()
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    box.set_strain_rate(rate)
    box.set_step(dt)
    t_end = box.run_strain(str(d1), 0.04, 0.02, rate * dt * 10)
    assert t_end == 4
    names = sorted(os.listdir(d1))
    assert names == ["sp0000000000.dat", "sp0000000002.dat", "sp0000000004.dat",
                     "sp_strain_se.dat"]
    lines = (d1 / "sp_strain_se.dat").read_text().splitlines()
    # one line at t=0, 5 records per t (every 10 of 50 steps), plus a repeat per t
    assert len(lines) == 1 + 4 * 6
    assert lines[0].split()[0] == "0" and len(lines[1].split()) == 5
    hdr, xf, yf, pf, *_ = sc.read_positions(str(d1 / "sp0000000004.dat"))
    xs, ys, ps = box.state()
    assert np.allclose(xf, xs, rtol=1e-13, atol=1e-12 * L)
    assert abs(hdr["gamma"] - box.box()["gamma"]) < 1e-15
    # continue from t = 2 in a fresh handle: same SE lines up to t = 2, then new ones
    d2 = tmp_path / "two"
    d2.mkdir()
    import shutil

    shutil.copy(d1 / "sp_strain_se.dat", d2 / "sp_strain_se.dat")
    hdr2, x2, y2, p2, R2, A2 = sc.read_positions(str(d1 / "sp0000000002.dat"))
    b2 = sc.SpherocylBox(hdr2["Lx"], x2, y2, p2, A2, R2, 0.1)
    b2.set_strain_rate(rate)
    b2.set_step(dt)
    b2.set_gamma(hdr2["gamma"])
    b2.set_total_gamma(hdr2["gamma_total"])
    assert b2.run_strain(str(d2), 0.02, 0.02, rate * dt * 10, t_start=2) == 4
    l2 = (d2 / "sp_strain_se.dat").read_text().splitlines()
    # as the reference (strain_dynamics.cpp:257-277): kept up to the first line of
    # t = 2, new lines written after it
    first2 = next(k for k, ln in enumerate(lines) if ln.split()[0] == "2")
    assert l2[: first2 + 1] == lines[: first2 + 1]
    assert len(l2) == first2 + 1 + 2 * 6 and l2[first2 + 1].split()[0] == "3"
    xb, *_ = b2.state()
    # the file holds 14 significant digits; two t-units of dynamics later the
    # positions still agree closely with the uninterrupted run
    assert np.max(np.abs(xb - xs)) < 1e-6


@pytest.mark.gpu
def test_save_positions_all_formats_round_trip(library, tmp_path):
    """sp (precision 14), sd (%.17g) and binary files of the same state read back to
    the state: the binary and sd files bit for bit."""
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(64, 0.80, 1.0, seed=5)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    box.set_strain_rate(1e-3)
    box.set_step(0.02)
    box.strain_steps(10)
    xs, ys, ps = box.state()
    for fmt, name, exact in (("bin", "sd0000000010.bin", True), ("sd", "sd0000000010.dat", True),
                             ("sp", "sp0000000010.dat", False)):
        path = str(tmp_path / name)
        box.save_positions(path, fmt)
        hdr, xx, yy, pp, RR, AA = sc.read_positions(path)
        got = np.stack([xx, yy, pp])
        want = np.stack([xs, ys, ps])
        if exact:
            assert np.array_equal(got, want), fmt
            assert np.array_equal(AA, A)
        else:
            assert np.max(np.abs(got - want)) < 1e-12 * L, fmt
        assert abs(hdr["gamma"] - box.box()["gamma"]) <= 1e-13
        assert hdr["dt"] == 0.02


@pytest.mark.gpu
def test_run_resize_and_minimize_files(library, tmp_path):
    import spherocyls_gb300 as sc

    L, x, y, p, R, A = sc.generate_packing(300, 0.80, 1.0, seed=4)
    box = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    box.set_resize_rate(5e-2)
    box.set_step(0.02)
    t = box.run_resize(str(tmp_path), 0.801, 0.05, 5e-2 * 0.02 * 25)
    b = box.box()
    assert t >= 1 and b["packing"] >= 0.801
    lines = (tmp_path / "sp_resize_se.dat").read_text().splitlines()
    assert len(lines[1].split()) == 6  # t packing E Pxx Pyy Pxy
    assert (tmp_path / f"sp{t:010d}.dat").exists()
    mdir = tmp_path / "m"
    mdir.mkdir()
    box2 = sc.SpherocylBox(L, x, y, p, A, R, 0.1)
    box2.set_step(0.1)
    steps = box2.run_minimize(str(mdir), 30, 0.0, 10)
    assert steps == 30
    se = (mdir / "sr_strain_se.dat").read_text().splitlines()
    assert len(se) == 31 and se[-1].split()[0] == "30"
    assert (mdir / "sr0000000030.dat").exists() and (mdir / "sr0000000010.dat").exists()


@pytest.mark.gpu
def test_cli_strain_new_and_continue(library, tmp_path):
    exe = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_strain")
    out = tmp_path / "run"
    out.mkdir()
    args = [exe, "r", str(out), "256", "1e-2", "0.02", "0.02", "0.01", "1e-3", "0.1", "0",
            "0.85", "1.0", "1.4", "0", "0"]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert (out / "sp0000000002.dat").exists() and (out / "sp_strain_se.dat").exists()
    # continue from the last file, with the arguments on standard input
    stdin = "\n".join([str(out / "sp0000000002.dat"), str(out), "256", "1e-2", "0.02", "0.01",
                       "0.01", "1e-3", "0.1", "0"]) + "\n"
    r = subprocess.run([exe], input=stdin, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert (out / "sp0000000003.dat").exists()
    lines = (out / "sp_strain_se.dat").read_text().splitlines()
    assert lines[-1].split()[0] == "3"
    # reversed shear from a file, and a zero-energy grid start with aligned particles
    r = subprocess.run([exe, str(out / "sp0000000003.dat"), str(out), "256", "1e-2", "0.02",
                        "0.01", "0.01", "1e-3", "0.1", "1"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Change shear direction" in r.stdout
    grid = tmp_path / "grid"
    grid.mkdir()
    r = subprocess.run([exe, "r", str(grid), "256", "1e-2", "0.02", "0.01", "0.01", "1e-3",
                        "0.1", "0", "0.5", "1.0", "1.4", "8", "0"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    from spherocyls_gb300 import read_positions

    hdr, x, y, p, R, A = read_positions(str(grid / "sp0000000000.dat"))
    assert np.all(p == p[0])


@pytest.mark.gpu
def test_cli_strain_rectangular_sd_file(library, tmp_path):
    """An sd file with Lx != Ly (the src/cuda header) runs in a rectangular box and
    the box survives into the output files."""
    import spherocyls_gb300 as sc

    exe = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_strain")
    L, x, y, p, R, A = sc.generate_packing(128, 0.80, 1.0, seed=9)
    n = 2 * len(x)
    src = tmp_path / "sd0000000000.dat"
    with open(src, "w") as f:
        f.write(f"{n} {float(2 * L)!r} {float(L)!r} 0.8 0 0 0.001 0.02\n")
        for xx, yy, pp, RR, AA in zip(np.concatenate([x, x + L]), np.concatenate([y, y]),
                                      np.concatenate([p, p]), np.concatenate([R, R]),
                                      np.concatenate([A, A])):
            f.write(f"{float(xx)!r} {float(yy)!r} {float(pp)!r} {float(RR)} {float(AA)!r}\n")
    out = tmp_path / "out"
    out.mkdir()
    env = dict(os.environ, SC_OUTPUT_FORMAT="sd")
    r = subprocess.run([exe, str(src), str(out), str(n), "1e-3", "0.02", "0.02", "0.01", "1e-3",
                        "0.1", "0"], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    last = sorted(f for f in os.listdir(out) if f.startswith("sd0") and f.endswith(".dat"))[-1]
    assert last != "sd0000000000.dat"
    hdr, *_ = sc.read_positions(str(out / last))
    assert hdr["Lx"] == 2 * L and hdr["Ly"] == L


@pytest.mark.gpu
def test_cli_resize_and_minimize(library, tmp_path):
    rz = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_resize")
    r = subprocess.run([rz, "r", str(tmp_path), "256", "5e-2", "0.02", "0.801", "0.05", "1e-3",
                        "0.1", "0.80", "1.0", "1.4", "0", "0"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "sp_resize_se.dat").exists()
    mz = os.path.join(ROOT, "spherocyls_gb300", "bin", "spherocyl_minimize")
    m = tmp_path / "m"
    m.mkdir()
    r = subprocess.run([mz, "r", str(m), "200", "0.1", "20", "10", "10", "0.1", "0.8", "0.5",
                        "0.5"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert (m / "sr_strain_se.dat").exists()
