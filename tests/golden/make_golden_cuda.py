"""Fixtures for the CUDA-only parts of the path, produced by the reference's own CUDA
kernels on a GPU.

The two-point contact rule (euler_est_2p / calc_fe_2p) and the pure-shear step
(pure_euler_est_2p + pure_heun_corr_2p) exist only in tmarschall/spherocyls'
src/cuda/2point_dynamics.cu.  ``oracle/Makefile`` (target ref_cuda, run where the
reference checkout is, by ``__graft_entry__.build()``) compiles that file where it
lies into the device module ``oracle/_ref/ref2p.cubin``; this script, run on a GPU
machine from the repository root, builds ``oracle/ref_cuda_run.cpp`` (a driver-API
loader of that module), runs its kernels on seeded cases and writes
``ref_cuda_2p.npz`` (into the directory given, default this one):

    python tests/golden/make_golden_cuda.py [out_dir]

Cases (every input and output is stored, so the tests need neither the module nor
the checkout):
  pairs  -- 400 isolated pairs of spherocylinders near contact in one box (parallel,
            antiparallel, oblique, tee, end-to-end and random relative placements,
            a/R in {0.25, 1, 2}, R in {0.5, 0.7}) at shear offset 0.27: forces and
            torques of calc_fe_2p<HARMONIC>.  Spines closer than 0.1 (R_i + R_j) are
            redrawn: crossing spines have no contact direction (the pair code's
            0/0), the rule of the library's generator.
  dense  -- a 512-particle packing at packing fraction 0.88 (a = R) at shear offset
            0.13: the same kernel with every pair within reach listed.
  pure   -- one pure-shear step (strain rate 1e-3, dt 0.02) of the dense packing at
            gamma 0 with unit drag (kd = 1, area = 1: the library's convention),
            moment of inertia and rotation coefficient of set_particle.
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

REF_PI = 3.14159265358979  # the reference's pi (src/cpp/spherocyl_box.cpp:12)
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref2p.cubin")
RUNNER = os.path.join(ROOT, "oracle", "_ref", "ref_cuda_run")


def rot_consts(R, A):
    """I and RC of set_particle (src/cpp/spherocyl_box.cpp:188-221)."""
    al = A / R
    C = 3 * REF_PI + 24 * al + 6 * REF_PI * al ** 2 + 8 * al ** 3
    area = R * (REF_PI * R + 4 * A)
    return R ** 4 * C / (6 * area), (8 * al + 6 * REF_PI * al ** 2 + 8 * al ** 3) / C


def full_list(x, y, R, A, Lx, Ly, gamma, extra=0.2):
    """Every pair whose centres are within R_i + A_i + R_j + A_j + extra (sheared
    minimum image), both ways: the kernels test contact themselves."""
    n = len(x)
    reach = R + A
    lists = [[] for _ in range(n)]
    for i in range(n):
        dx = x[i] - x
        dy = y[i] - y
        dx += Lx * ((dx < -0.5 * Lx).astype(float) - (dx > 0.5 * Lx))
        dy += Ly * ((dy < -0.5 * Ly).astype(float) - (dy > 0.5 * Ly))
        dx += gamma * dy
        hit = np.hypot(dx, dy) < reach[i] + reach + extra
        hit[i] = False
        lists[i] = list(np.nonzero(hit)[0])
    m = max(1, max(len(v) for v in lists))
    nbr = np.zeros((m, n), dtype=np.int32)
    nn = np.zeros(n, dtype=np.int32)
    for i, v in enumerate(lists):
        nn[i] = len(v)
        nbr[: len(v), i] = v
    return nn, nbr


def run_case(mode, x, y, phi, R, A, Lx, Ly, gamma, rate=0.0, step=0.02, eps=0.1):
    I, RC = rot_consts(R, A)
    nn, nbr = full_list(x, y, R, A, Lx, Ly, gamma)
    n = len(x)
    with tempfile.TemporaryDirectory() as td:
        cin, cout = os.path.join(td, "case.bin"), os.path.join(td, "out.bin")
        with open(cin, "wb") as f:
            f.write(struct.pack("<3i", mode, n, nbr.shape[0]))
            f.write(np.array([Lx, Ly, gamma, rate, step, eps, 1.0], dtype="<f8").tobytes())
            for v in (x, y, phi, R, A, np.ones(n), I, RC):
                f.write(np.asarray(v, dtype="<f8").tobytes())
            f.write(nn.astype("<i4").tobytes())
            f.write(np.ascontiguousarray(nbr).astype("<i4").tobytes())
        subprocess.run([RUNNER, CUBIN, cin, cout], check=True)
        raw = open(cout, "rb").read()
    d = np.frombuffer(raw[: 8 * (3 * n if mode == 1 else 6 * n)], dtype="<f8")
    if mode == 1:
        e = np.frombuffer(raw[24 * n: 24 * n + 8], dtype="<f8")[0]
        return dict(fx=d[:n].copy(), fy=d[n:2 * n].copy(), tau=d[2 * n:].copy(), energy=e)
    tail = np.frombuffer(raw[48 * n: 48 * n + 16], dtype="<f8")
    return dict(x=d[:n].copy(), y=d[n:2 * n].copy(), phi=d[2 * n:3 * n].copy(),
                fx=d[3 * n:4 * n].copy(), fy=d[4 * n:5 * n].copy(), tau=d[5 * n:].copy(),
                Lx=tail[0], Ly=tail[1])


def seg_dist(ax, ay, ux, uy, bx, by, vx, vy):
    """Distance between the segments a + s u and b + t v, s, t in [-1, 1]: zero when
    they cross, else the least endpoint-to-segment distance."""
    def cross(px, py, qx, qy):
        return px * qy - py * qx

    def pt_seg(px, py, cx, cy, wx, wy):
        ww = wx * wx + wy * wy
        t = 0.0 if ww == 0 else min(max(((px - cx) * wx + (py - cy) * wy) / ww, -1.0), 1.0)
        return np.hypot(px - cx - t * wx, py - cy - t * wy)

    p0, p1 = (ax - ux, ay - uy), (ax + ux, ay + uy)
    q0, q1 = (bx - vx, by - vy), (bx + vx, by + vy)
    d1 = cross(q1[0] - q0[0], q1[1] - q0[1], p0[0] - q0[0], p0[1] - q0[1])
    d2 = cross(q1[0] - q0[0], q1[1] - q0[1], p1[0] - q0[0], p1[1] - q0[1])
    d3 = cross(p1[0] - p0[0], p1[1] - p0[1], q0[0] - p0[0], q0[1] - p0[1])
    d4 = cross(p1[0] - p0[0], p1[1] - p0[1], q1[0] - p0[0], q1[1] - p0[1])
    if d1 * d2 < 0 and d3 * d4 < 0:
        return 0.0
    return min(pt_seg(*p0, bx, by, vx, vy), pt_seg(*p1, bx, by, vx, vy),
               pt_seg(*q0, ax, ay, ux, uy), pt_seg(*q1, ax, ay, ux, uy))


def pairs_case(rng, gamma, npairs=400, spacing=12.0):
    """Pairs placed by their lab-frame displacement; stored in the sheared
    coordinates of shear offset gamma (x_sheared = x_lab - gamma y)."""
    side = int(np.ceil(np.sqrt(npairs)))
    L = side * spacing
    x, y, phi, R, A = (np.zeros(2 * npairs) for _ in range(5))
    kinds = ["parallel", "antiparallel", "oblique", "tee", "end", "random"]
    k = 0
    while k < npairs:
        cx, cy = (k % side + 0.5) * spacing, (k // side + 0.5) * spacing
        r = rng.choice([0.5, 0.7], size=2)
        a = rng.choice([0.25, 1.0, 2.0], size=2) * r
        th = rng.uniform(-np.pi, np.pi)
        kind = kinds[k % len(kinds)]
        if kind == "parallel":
            p2 = th + rng.choice([0.0, 1e-9, -3e-7, 2e-4])
            off = np.array([rng.uniform(-1, 1) * (a[0] + a[1]), (r[0] + r[1]) * rng.uniform(0.8, 0.99)])
        elif kind == "antiparallel":
            p2 = th + np.pi + rng.choice([0.0, 1e-8, -5e-5])
            off = np.array([rng.uniform(-1, 1) * (a[0] + a[1]), (r[0] + r[1]) * rng.uniform(0.8, 0.99)])
        elif kind == "oblique":
            p2 = th + rng.uniform(0.3, np.pi - 0.3)
            off = np.array([rng.uniform(-0.3, 0.3), rng.uniform(0.2, 0.9) * (r[0] + r[1])])
        elif kind == "tee":
            p2 = th + np.pi / 2
            off = np.array([a[0] * rng.uniform(-0.9, 0.9), a[1] + (r[0] + r[1]) * rng.uniform(0.85, 0.99)])
        elif kind == "end":
            p2 = th + rng.choice([0.0, np.pi, 0.05])
            off = np.array([a[0] + a[1] + (r[0] + r[1]) * rng.uniform(0.85, 0.99), rng.uniform(-0.1, 0.1)])
        else:
            p2 = rng.uniform(-np.pi, np.pi)
            off = rng.normal(size=2)
            off *= (a[0] + a[1] + r[0] + r[1]) * rng.uniform(0.3, 1.0) / np.hypot(*off)
        c, s = np.cos(th), np.sin(th)
        d = np.array([c * off[0] - s * off[1], s * off[0] + c * off[1]])
        p2 = (p2 + np.pi) % (2 * np.pi) - np.pi
        if seg_dist(-d[0], -d[1], a[0] * c, a[0] * s, 0.0, 0.0, a[1] * np.cos(p2),
                    a[1] * np.sin(p2)) < 0.1 * (r[0] + r[1]):
            continue  # crossing or nearly crossing spines: redraw
        ds = (d[0] - gamma * d[1], d[1])  # the kernels add gamma dy back
        x[2 * k], y[2 * k] = cx - ds[0] / 2, cy - ds[1] / 2
        x[2 * k + 1], y[2 * k + 1] = cx + ds[0] / 2, cy + ds[1] / 2
        phi[2 * k], phi[2 * k + 1] = th, p2
        R[2 * k: 2 * k + 2], A[2 * k: 2 * k + 2] = r, a
        k += 1
    return L, x, y, phi, R, A


def main() -> None:
    out_dir = sys.argv[1] if len(sys.argv) > 1 else HERE
    if not os.path.exists(CUBIN):
        raise SystemExit("oracle/_ref/ref2p.cubin is missing: build it where the reference "
                         "checkout is (oracle/Makefile, target ref_cuda)")
    oracle.build(with_ref=False)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref_cuda_run"], check=True)
    rng = np.random.default_rng(2024)
    out = {}
    L, x, y, phi, R, A = pairs_case(rng, 0.27)
    r = run_case(1, x, y, phi, R, A, L, L, 0.27)
    out.update({"pairs_L": np.array(L), "pairs_gamma": np.array(0.27), "pairs_x": x, "pairs_y": y,
                "pairs_phi": phi, "pairs_R": R, "pairs_A": A, "pairs_fx": r["fx"],
                "pairs_fy": r["fy"], "pairs_tau": r["tau"], "pairs_energy": np.array(r["energy"])})
    L, x, y, phi, R, A = oracle.generate_packing(512, 0.88, 1.0, seed=17)
    r = run_case(1, x, y, phi, R, A, L, L, 0.13)
    out.update({"dense_L": np.array(L), "dense_gamma": np.array(0.13), "dense_x": x, "dense_y": y,
                "dense_phi": phi, "dense_R": R, "dense_A": A, "dense_fx": r["fx"],
                "dense_fy": r["fy"], "dense_tau": r["tau"], "dense_energy": np.array(r["energy"])})
    r = run_case(2, x, y, phi, R, A, L, L, 0.0, rate=1e-3, step=0.02)
    out.update({"pure_rate": np.array(1e-3), "pure_step": np.array(0.02), "pure_x": r["x"],
                "pure_y": r["y"], "pure_phi": r["phi"], "pure_fx0": r["fx"], "pure_fy0": r["fy"],
                "pure_tau0": r["tau"], "pure_Lx": np.array(r["Lx"]), "pure_Ly": np.array(r["Ly"])})
    path = os.path.join(out_dir, "ref_cuda_2p.npz")
    np.savez_compressed(path, **out)
    print("written", path)


if __name__ == "__main__":
    main()
