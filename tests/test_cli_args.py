"""The jamming drivers' argument handling, which runs before any device call: invalid
numbers and unreadable data files end the driver with status 1 and a message, and a
missing argument is prompted for and read from standard input, as the reference's
drivers do (src/cuda/main_2point_findjam.cpp:17-58)."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT

BIN = os.path.join(ROOT, "spherocyls_gb300", "bin")


def _run(name, args, stdin=subprocess.DEVNULL):
    return subprocess.run([os.path.join(BIN, name)] + [str(a) for a in args], stdin=stdin,
                          capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("name", ["spherocyl_find_jam", "spherocyl_y_compress"])
def test_zero_resize_step_is_refused(library, tmp_path, name):
    r = _run(name, ["r", tmp_path, 64, 0, 0.01, 1e-6, 0.01, 0.01, 0.1, 0.8, 1.0, 1.4])
    assert r.returncode == 1 and "non-zero resize step" in r.stderr


def test_qs_compress_needs_a_positive_packing(library, tmp_path):
    r = _run("spherocyl_qs_compress", ["r", tmp_path, 64, 5e-3, 0.01, 0, 0.01, 0.01, 0.1])
    assert r.returncode == 1 and "final packing fraction" in r.stderr


@pytest.mark.parametrize("name", ["spherocyl_find_jam", "spherocyl_qs_compress",
                                  "spherocyl_y_compress"])
def test_unreadable_data_file_fails_before_the_device(library, tmp_path, name):
    r = _run(name, [tmp_path / "sd0000000000.dat", tmp_path, 64, 1e-3, 0.01, 0.9, 0.01, 0.01,
                    0.1])
    assert r.returncode != 0 and "read" in (r.stdout + r.stderr)


def test_missing_arguments_are_read_from_stdin(library, tmp_path):
    """Arguments past argv come from standard input, one per line; here the resize step
    (0) arrives that way and is refused, and an exhausted input ends the driver."""
    r = _run("spherocyl_find_jam", ["r", tmp_path, 64])
    assert r.returncode == 1 and "missing input" in r.stderr
    r = subprocess.run([os.path.join(BIN, "spherocyl_find_jam"), "r", str(tmp_path), "64"],
                       input="0\n0.01\n1e-6\n0.01\n0.01\n0.1\n", capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and "Resize rate (epsilon): " in r.stdout
    assert "non-zero resize step" in r.stderr
