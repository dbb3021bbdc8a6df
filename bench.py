"""Benchmark: particle-steps/s of Lees-Edwards shear on one GB300.

Workload (default): N = 1,048,576 bidisperse spherocylinders (R = 0.5 / 0.7
alternating, A = R), packing fraction 0.84, strain rate 1e-4, dt = 0.02, seeded
crossing-free synthetic packing (seed 3).  A "step" is one Heun step (two force
passes) of every particle.  Every arm times the same window of the same run: W
untimed warm-up steps from the generated packing, then K timed steps.

The headline `value` is the mixed-precision form with its state resident on the
device; `value_fp64` is the plain FP64 form over the same window; `e2e` is the
same window through the C ABI from pinned host arrays (handle creation from the
state after the warm-up, K steps, state and stress read back into pinned arrays).  The same JSON line
carries the force-pass roofline, a steady-state figure (after a longer shear), the
CPU baseline (the oracle restatement of the reference's CPU path on the host
cores), the precision A/B of the N = 16384 workload, the 512-system batch and the
minimisation time to tolerance of batched jamming replicas.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]

`--impl reference` runs only the reference's CPU path (the compiled reference in
oracle/_ref when it exists, else the oracle restatement) on the same packing,
generated by the oracle, with no product code loaded.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (N, packing, a/R, strain rate, dt, seed)
    "shear_n1048576_phi084": (1 << 20, 0.84, 1.0, 1e-4, 0.02, 3),
    "shear_n16384_phi086": (16384, 0.86, 1.0, 1e-4, 0.02, 1),
    # 512 independent systems: N log-uniform in [64, 8192] (even), packing U[0.75, 0.90],
    # a/R U[0.2, 2.0], strain rate log-uniform in [1e-6, 1e-3], seed 2
    "batch512": (512, None, None, None, 0.02, 2),
}
PAD = 0.2  # neighbour padding of the workload (the reference's rebuild timing)
METRIC = "particle-steps/s (Lees-Edwards shear, Heun step)"
REF_PI = 3.14159265358979  # the reference's pi (src/cpp/spherocyl_box.cpp:12)


def make_batch(generate, seed=2, nsys=512):
    rng = np.random.default_rng(seed)
    ns = (np.exp(rng.uniform(np.log(64), np.log(8192), nsys)) / 2).round().astype(int) * 2
    phis = rng.uniform(0.75, 0.90, nsys)
    aors = rng.uniform(0.2, 2.0, nsys)
    rates = np.exp(rng.uniform(np.log(1e-6), np.log(1e-3), nsys))
    parts = [generate(int(n), float(f), float(a), seed=int(seed * 100000 + k))
             for k, (n, f, a) in enumerate(zip(ns, phis, aors))]
    return dict(ns=ns, phis=phis, aors=aors, rates=rates, n=int(ns.sum()), dt=0.02, seed=seed,
                L=np.array([pk[0] for pk in parts]),
                x=np.concatenate([pk[1] for pk in parts]), y=np.concatenate([pk[2] for pk in parts]),
                p=np.concatenate([pk[3] for pk in parts]), R=np.concatenate([pk[4] for pk in parts]),
                A=np.concatenate([pk[5] for pk in parts]))


def make_workload(name, generate):
    """The workload's inputs; `generate` is the library's or the oracle's packing
    generator (the same packing bit for bit, tests/test_oracle_pin.py)."""
    if name == "batch512":
        return make_batch(generate)
    n, phi, a, rate, dt, seed = WORKLOADS[name]
    L, x, y, p, R, A = generate(n, phi, a, seed=seed)
    return dict(n=n, phi=phi, a=a, rate=rate, dt=dt, seed=seed, L=L, x=x, y=y, p=p, R=R, A=A)


def config_of(name, world):
    """The workload's definition (identical in both arms)."""
    if name == "batch512":
        return {"workload": name, "systems": 512, "N": "log-uniform [64, 8192], even",
                "packing": "U[0.75, 0.90]", "a_over_r": "U[0.2, 2.0]",
                "strain_rate": "log-uniform [1e-6, 1e-3]", "dt": 0.02, "seed": 2, "pad": PAD,
                "parallelism": "replicas" if world > 1 else "single"}
    n, phi, a, rate, dt, seed = WORKLOADS[name]
    return {"workload": name, "N": n, "packing": phi, "a_over_r": a, "strain_rate": rate,
            "dt": dt, "seed": seed, "pad": PAD,
            "start": "the generated packing; W warm-up steps, then the K timed steps",
            "l2": "inputs larger than L2: a mixed step moves 152 + 8 n B per particle "
                  "(about 200 B, 210 MB at N = 2^20) against 129 MB of L2",
            "parallelism": "replicas" if world > 1 else "single"}


# Algorithmic bytes per particle-step (two force passes plus the state update):
# mixed form 152 + 8 n, plain FP64 form 232 + 8 n, n the mean length of the full
# neighbour list actually used (4 bytes per entry and pass).  Per force pass: half.
def bytes_per_pass(precision: str, nbar: float) -> float:
    return (152.0 if precision == "mixed" else 232.0) / 2 + 4.0 * nbar


# DRAM bytes (read + write) per particle of one mixed force pass, the mean of the
# predictor (113.6 MB) and corrector (172.4 MB) launches in one ncu capture of the
# default workload at the padding the autotuner picks for it, 0.6
# (profiles/k_pass_mixed_n1048576.md).
PASS_DRAM_BYTES_PER_PARTICLE = {"shear_n1048576_phi084": 143.0e6 / (1 << 20)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def __enter__(self):
        cmd = ["nvidia-smi",
               "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler reports (at most 3 s later)
            t0 = time.perf_counter()
            while not self.samples and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            # one more sample after the timed work
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, device=0):
        rows = [s for s in self.samples if s and s[0] == str(device)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if len(r) > 5 + k and r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def max_over_ranks(secs: float, world: int, device: str) -> float:
    """The slowest rank's time (replicas run independently; this all-reduce is the
    only collective, outside the timed region)."""
    if world <= 1:
        return secs
    import torch
    import torch.distributed as dist

    t = torch.tensor([secs], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU (oracle) arm

def cpu_run(w, warmup, steps, threads):
    """The reference's CPU path (the compiled reference when present, else the
    oracle restatement) on `threads` host cores: each core advances its own copy of
    the workload's system (the reference is single-threaded) through `warmup`
    untimed and `steps` timed Heun steps; the timed region spans all copies."""
    import oracle

    oracle.build(with_ref=False)
    kind, cls = ("reference", oracle.RefBox) if oracle.ref_available() else ("port",
                                                                             oracle.OracleBox)
    boxes = [None] * threads
    barrier = threading.Barrier(threads + 1)
    times = [0.0] * threads

    def run(k):
        b = cls(w["L"], w["x"], w["y"], w["p"], w["A"], w["R"], PAD, strain_rate=w["rate"],
                step=w["dt"])
        if warmup:
            b.run_strain_steps(warmup)
        boxes[k] = b
        barrier.wait()
        t = time.perf_counter()
        b.run_strain_steps(steps)
        times[k] = time.perf_counter() - t
        barrier.wait()

    ts = [threading.Thread(target=run, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    barrier.wait()  # every copy built and warmed up
    t0 = time.perf_counter()
    barrier.wait()
    dt = time.perf_counter() - t0
    for t in ts:
        t.join()
    for b in boxes:
        b.close()
    return {"value": threads * w["n"] * steps / dt, "unit": "particle-steps/s", "cores": threads,
            "kind": kind, "seconds": dt,
            "sample": f"{threads} concurrent copies (one per host core) of the N={w['n']} "
                      f"workload, steps {warmup + 1}-{warmup + steps} of the run from the "
                      f"generated packing, {dt:.1f} s"}


def run_reference_arm(args, w, rank, world):
    """The reference's CPU path on every host core over the same window as the GPU
    arm (rank 0 only; the other ranks exit without work)."""
    if rank != 0:
        return
    if w.get("phi") is None:
        print(json.dumps({"impl": "reference", "unavailable":
                          "the CPU arm runs single-system workloads only"}))
        return
    threads = os.cpu_count() or 1
    steps, warmup = min(args.steps, args.ref_max_steps), min(args.warmup, args.ref_max_warmup)
    base = cpu_run(w, warmup, steps, threads)
    line = {"impl": "reference", "metric": METRIC,
            "value": base["value"], "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * base["seconds"] / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded crossing-free packing, oracle generator)",
            "config": config_of(args.workload, world),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU arm helpers

_STREAM = None


def mean_list_length(box):
    """Mean full-list length (2 x half-list pairs / N) of the first system."""
    return 2.0 * len(box.pairs(0)) / int(box.n_per_sys[0])


def time_steps(box, steps, torch):
    """Device time of `steps` steps with CUDA events on the library's stream (a
    dedicated non-default stream shared with torch's events)."""
    global _STREAM
    if _STREAM is None:
        _STREAM = torch.cuda.Stream()
    stream = _STREAM
    box.set_stream(stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    box.strain_steps(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def precision_ab(device, steps_per_step=100, total=100000, every=100, prep_steps=300):
    """The N = 16384 precision workload (packing 0.86, a = R, strain rate 1e-4, dt
    0.02, seed 1): mixed and FP64 from one sheared state (`prep_steps` FP64 steps
    after the generated packing).  Per-step errors of the energy and shear stress of
    the mixed run against the FP64 run over the first `steps_per_step` steps (stress
    recorded every step), then both runs continue to `total` steps with the stress
    recorded every `every` steps for the time averages (block standard errors over 10
    blocks, after the first 10% of the run)."""
    from spherocyls_gb300 import SpherocylBox, generate_packing

    n, phi, a, rate, dt, seed = WORKLOADS["shear_n16384_phi086"]
    L, x, y, p, R, A = generate_packing(n, phi, a, seed=seed)
    prep = SpherocylBox(L, x, y, p, A, R, PAD, device=device)
    prep.set_strain_rate(rate)
    prep.set_step(dt)
    prep.strain_steps(prep_steps)
    x, y, p = prep.state()
    bx = prep.box()
    prep.close()
    first, series, secs = {}, {}, {}
    for precision in ("fp64", "mixed"):
        b = SpherocylBox(L, x, y, p, A, R, PAD, precision=precision, device=device)
        b.set_strain_rate(rate)
        b.set_step(dt)
        b.set_gamma(bx["gamma"])
        b.set_total_gamma(bx["gamma_total"])
        first[precision] = b.strain_steps(steps_per_step, se_every=1)[:, 0, :]
        t = time.perf_counter()
        rest = b.strain_steps(total - steps_per_step, se_every=every)
        secs[precision] = time.perf_counter() - t
        series[precision] = rest[:, 0, :]
        b.close()
    fa, fm = first["fp64"], first["mixed"]
    rel_e = np.abs(fm[:, 0] - fa[:, 0]) / np.abs(fa[:, 0])
    rel_pxy = np.abs(fm[:, 3] - fa[:, 3]) / np.abs(fa[:, 3])
    over = np.nonzero(rel_pxy > 1e-6)[0]

    def avg(v):
        v = v[len(v) // 10:]
        blocks = np.array_split(v, 10)
        means = np.array([bl.mean() for bl in blocks])
        return float(v.mean()), float(means.std(ddof=1) / np.sqrt(len(means)))

    out = {"workload": "shear_n16384_phi086", "steps": total,
           "start": f"{prep_steps} FP64 shear steps after the generated packing",
           "per_step": {"steps": steps_per_step,
                        "energy_rel_err_max": float(rel_e.max()),
                        "pxy_rel_err_max": float(rel_pxy.max()),
                        "pxy_rel_err_max_first10": float(rel_pxy[:10].max()),
                        "pxy_rel_err_max_first50": float(rel_pxy[:50].max()),
                        "first_step_pxy_rel_err_over_1e-6": int(over[0]) + 1 if len(over) else None,
                        "note": "mixed minus FP64 from the same start, each relative to the "
                                "FP64 run's own value (Pxy relative to |Pxy|)"},
           "time_average": {}, "seconds": secs}
    for precision in ("fp64", "mixed"):
        s = series[precision]
        e_m, e_se = avg(s[:, 0])
        p_m, p_se = avg(s[:, 3])
        out["time_average"][precision] = {"energy": e_m, "energy_stderr": e_se, "pxy": p_m,
                                          "pxy_stderr": p_se}
    ta = out["time_average"]
    out["time_average"]["pxy_diff_over_stderr"] = abs(ta["mixed"]["pxy"] - ta["fp64"]["pxy"]) / \
        float(np.hypot(ta["mixed"]["pxy_stderr"], ta["fp64"]["pxy_stderr"]))
    return out


def batched_leg(args, device, torch):
    """The 512-system batch (mixed form): the same warm-up and window as the
    headline, with its force-pass roofline from per-pass CUDA events."""
    from spherocyls_gb300 import BoxBatch, generate_packing

    w = make_batch(generate_packing)

    def new(profile=False, pad=PAD, block=0, **kw):
        b = BoxBatch(w["ns"], w["L"], w["x"], w["y"], w["p"], w["A"], w["R"], pad,
                     precision="mixed", device=device, profile=profile, block=block, **kw)
        for k, r in enumerate(w["rates"]):
            b.set_strain_rate(float(r), sys=k)
        b.set_step(w["dt"])
        return b

    t = new()
    t.strain_steps(args.warmup)
    f, blk = t.autotune(50)
    o = t.options()
    t.close()
    kw = dict(pass_kind=o["pass_kind"], tile_target=o["tile_target"],
              persist_steps=o["persist_steps"])
    b = new(pad=PAD * f, block=blk, **kw)
    b.strain_steps(args.warmup)
    secs = time_steps(b, args.steps, torch)
    b.close()
    pr = new(profile=True, pad=PAD * f, block=blk, **kw)
    pr.strain_steps(args.warmup)
    pr.pass_times()
    pr.strain_steps(max(args.steps, 20))
    pt = pr.pass_times()
    pairs = sum(len(pr.pairs(s)) for s in range(pr.nsys))
    pr.close()
    nbar = 2.0 * pairs / w["n"]
    pass_ms = 0.5 * (pt["corr_ms"] + pt["pred_ms"])
    achieved = bytes_per_pass("mixed", nbar) * w["n"] / (pass_ms / 1e3) / 1e9
    peak, _ = _peaks()
    return {"workload": "batch512", "particles": w["n"], "value": w["n"] * args.steps / secs,
            "unit": "particle-steps/s", "ms_per_step": 1e3 * secs / args.steps,
            "steps": args.steps, "warmup": args.warmup,
            "tuning": {"pad": PAD * f, "block": blk, **kw},
            "pass_ms": pass_ms, "mean_list_length": nbar,
            "roofline_frac": achieved / peak, "achieved_gbs": achieved}


def minimise_leg(replicas=128, n=4096, max_iter=40000, ftol=1e-14, device=0, e_jam=1e-12,
                 dt_max=0.2, cg_iter=2000, over=1e-2, graphs=True, mixed_iter=20000,
                 contacts=2):
    """Minimisation time to tolerance on the jamming workload's shape: replicas of
    N = 4096 with a/R in {0.25, 0.5, 1, 2} (a quarter each), seeds 100 + k, from
    packing 0.70, two-point contacts (the reference's jamming code).  Untimed
    preparation: the mixed form compresses every replica in affine steps of 2e-3 in
    packing fraction (FIRE to 1e-6 after each) until E/N > e_jam = 1e-12 at that
    tolerance.  Incomplete minimisation leaves that much energy below the jamming
    point, so each replica is then compressed by `over` more.  From that same state the
    two timed arms minimise to max|F_i|, |tau_i|/sqrt(I_i) < ftol: (a) mixed FIRE to
    1e-6 (the FP32 pair geometry resolves overlaps to about 1e-7), then FP64 FIRE;
    (b) FP64 FIRE alone; and (c) the reference's conjugate gradient (FP64) on one
    replica of each aspect ratio, stopped by the reference's rules or after cg_iter
    iterations.  Each FIRE stage stops after its iteration cap; a replica that has
    converged takes no further force passes.  A replica is jammed when its final
    E/N > 1e-16.  The two-point rule's energy jumps where a second contact ends, so
    FIRE stalls above ftol on some jammed replicas; the report gives the residuals
    reached, and compares the energies of the replicas jammed in both arms."""
    from spherocyls_gb300 import BoxBatch, generate_packing

    aors = [0.25, 0.5, 1.0, 2.0]
    packs = [generate_packing(n, 0.70, aors[(4 * k) // replicas], seed=100 + k)
             for k in range(replicas)]
    cat = lambda i: np.concatenate([pk[i] for pk in packs])  # noqa: E731
    L0 = np.array([pk[0] for pk in packs])
    R, A = cat(4), cat(5)
    kw = dict(contacts=contacts, device=device, use_graphs=graphs)
    prep = BoxBatch([n] * replicas, L0, cat(1), cat(2), cat(3), A, R, 0.1, precision="mixed",
                    **kw)
    t0 = time.perf_counter()
    prep.fire_minimize(1e-6, 100000)
    phi_j, n_inc = prep.quasistatic_compress(2e-3, 1e-6, e_jam, 1000, 100000)
    t_prep = time.perf_counter() - t0
    Lj = np.array([prep.box(s)["Lx"] for s in range(replicas)])
    xs, ys, ps = prep.state()
    prep.close()
    f = np.sqrt(phi_j / (phi_j + over))
    fp = np.repeat(f, n)
    L1, x1, y1 = Lj * f, xs * fp, ys * fp

    def run(b, tol, cap):
        t = time.perf_counter()
        it, fmax, done = b.fire_minimize(tol, cap, dt_max=dt_max)
        return time.perf_counter() - t, it, fmax, done, b.fire_iterations()

    def iteration_ms(precision, iters):
        # one FIRE iteration of the whole batch, every replica active (from the
        # same start, on a copy)
        b = BoxBatch([n] * replicas, L1, x1, y1, ps, A, R, 0.1, precision=precision, **kw)
        b.fire_minimize(1e-300, 20, dt_max=dt_max)  # graph capture
        t = time.perf_counter()
        b.fire_minimize(1e-300, iters, dt_max=dt_max)
        dt = time.perf_counter() - t
        b.close()
        return 1e3 * dt / iters

    c_mixed, c_fp64 = iteration_ms("mixed", 500), iteration_ms("fp64", 100)
    m = BoxBatch([n] * replicas, L1, x1, y1, ps, A, R, 0.1, precision="mixed", **kw)
    ta, ia, fa, da, pa = run(m, 1e-6, mixed_iter)
    xm, ym, pm = m.state()
    m.close()
    r = BoxBatch([n] * replicas, L1, xm, ym, pm, A, R, 0.1, precision="fp64", **kw)
    tb, ib, fb, db, pb = run(r, ftol, max_iter)
    e_a = r.calc_se()[:, 0]
    r.close()
    p = BoxBatch([n] * replicas, L1, x1, y1, ps, A, R, 0.1, precision="fp64", **kw)
    tc, ic, fc, dc, pc = run(p, ftol, max_iter)
    e_c = p.calc_se()[:, 0]
    p.close()
    sub = sorted({(k * replicas) // 4 for k in range(4)})
    sel = np.concatenate([np.arange(k * n, (k + 1) * n) for k in sub])
    q = BoxBatch([n] * len(sub), L1[sub], x1[sel], y1[sel], ps[sel], A[sel], R[sel], 0.1,
                 precision="fp64", **kw)
    t = time.perf_counter()
    cit, ce, cwhy = q.cg_minimize(cg_iter)
    tcg = time.perf_counter() - t
    q.calc_forces()
    qfx, qfy, qtq = q.forces()
    q.close()
    Rs, As = R[sel], A[sel]
    al = As / Rs
    C = 3 * REF_PI + 24 * al + 6 * REF_PI * al ** 2 + 8 * al ** 3
    inertia = Rs ** 4 * C / (6 * Rs * (REF_PI * Rs + 4 * As))
    res = np.maximum(np.hypot(qfx, qfy), np.abs(qtq) / np.sqrt(inertia)).reshape(len(sub), n)
    cres = res.max(axis=1)
    jam_a, jam_c = e_a > 1e-16, e_c > 1e-16
    jam = jam_a & jam_c
    conv = da & db & dc
    rel = np.abs(e_a - e_c) / np.maximum(e_c, 1e-300)
    levels = (1e-14, 1e-12, 1e-10, 1e-8, 1e-6)

    def below(fm):
        return {f"{v:g}": int((fm < v).sum()) for v in levels}

    def med(v):
        return float(np.median(v)) if len(v) else None

    return {
        "workload": f"jam_{replicas}x{n}", "replicas": replicas, "N": n, "ftol": ftol,
        "contacts": contacts,
        "prep": {"seconds": t_prep, "increments": n_inc, "over_compression": over,
                 "phi_jam_range": [float(phi_j.min()), float(phi_j.max())]},
        "mixed_then_fp64": {"seconds": ta + tb, "mixed_seconds": ta, "mixed_iters": ia,
                            "fp64_iters": ib, "mixed_reached_1e-6": int(da.sum()),
                            "converged": int((da & db).sum()), "max_residual": float(fb.max()),
                            "residual_below": below(fb), "jammed": int(jam_a.sum())},
        "fp64": {"seconds": tc, "iters": ic, "converged": int(dc.sum()),
                 "max_residual": float(fc.max()), "residual_below": below(fc),
                 "jammed": int(jam_c.sum())},
        "iterations_median_converged_both": {
            "mixed": med(pa[conv]), "fp64_after_mixed": med(pb[conv]),
            "fp64_alone": med(pc[conv])},
        "iteration_ms": {"mixed": c_mixed, "fp64": c_fp64,
                         "note": "one FIRE iteration of the 128-replica batch, all active"},
        "time_to_tolerance_speedup_converged_both": (
            {"median": float(np.median(pc[conv] * c_fp64 / (pa[conv] * c_mixed + pb[conv] * c_fp64))),
             "aggregate": float(np.sum(pc[conv]) * c_fp64 /
                                np.sum(pa[conv] * c_mixed + pb[conv] * c_fp64)),
             "replicas": int(conv.sum()),
             "note": "per replica, its iterations in each stage times the batch's cost per "
                     "iteration (modelled: the batch's wall time is set by its slowest replica)"}
            if conv.any() else None),
        "cg_fp64": {"replicas": len(sub), "seconds": tcg, "iters_max": int(cit.max()),
                    "iters_mean": float(cit.mean()),
                    "stop_reasons": {str(k): int((cwhy == k).sum()) for k in (1, 2, 3, 4, 5)},
                    "below_ftol": int((cres < ftol).sum()), "max_residual": float(cres.max())},
        "jammed_both": int(jam.sum()),
        "jammed_energy_rel_diff": {
            "max": float(rel[jam].max()) if jam.any() else None,
            "median": med(rel[jam]),
            "within_1e-10": int((rel[jam] <= 1e-10).sum())},
        "jammed_converged_both": int((conv & jam).sum()),
        "energy_rel_diff_max": (float(rel[conv & jam].max()) if (conv & jam).any() else None),
        "energy_per_particle_range": [float(min(e_a.min(), e_c.min())),
                                      float(max(e_a.max(), e_c.max()))],
        "energy_per_particle_abs_diff_max_unjammed": (
            float(np.max(np.abs(e_a - e_c)[conv & ~jam_a & ~jam_c]))
            if (conv & ~jam_a & ~jam_c).any() else None),
        "speedup": tc / (ta + tb),
    }


# ---------------------------------------------------------------- main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="shear_n1048576_phi084", choices=list(WORKLOADS))
    ap.add_argument("--ref-max-steps", type=int, default=20,
                    help="timed steps of the CPU reference arm at most (a bounded sample)")
    ap.add_argument("--ref-max-warmup", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=2,
                    help="Heun steps of the CPU baseline sample in the GPU arm's line")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", choices=["mixed", "fp64", "minimise"], default=None,
                    help="time one form only, or run the minimisation leg alone "
                         "(for profiler captures)")
    ap.add_argument("--forced-rebuilds", type=int, default=0,
                    help="with --only mixed|fp64: full rebuilds after the timed steps")
    ap.add_argument("--steady-steps", type=int, default=300,
                    help="shear steps before the steady-state window")
    ap.add_argument("--autotune", action=argparse.BooleanOptionalAction, default=True,
                    help="pick the mixed form's padding and block size with sc_autotune")
    ap.add_argument("--legs", default="precision,batched,minimise",
                    help="extra legs of the GPU arm (comma separated, or 'none')")
    ap.add_argument("--min-replicas", type=int, default=128)
    ap.add_argument("--min-iters", type=int, default=40000,
                    help="FP64 FIRE iteration cap of the minimisation leg")
    ap.add_argument("--min-contacts", type=int, default=2, choices=[1, 2],
                    help="contact points per pair in the minimisation leg")
    ap.add_argument("--min-over", type=float, default=1e-2,
                    help="compression past the detected jamming point (minimisation leg)")
    ap.add_argument("--pass-kind", choices=["auto", "list", "tile"], default="auto",
                    help="the mixed form's force pass before autotuning (profiler captures)")
    ap.add_argument("--tile-target", type=int, default=0)
    ap.add_argument("--persist", action="store_true",
                    help="persistent step kernel for the mixed form when not autotuned")
    ap.add_argument("--pad-factor", type=float, default=1.0,
                    help="padding factor of the mixed form when not autotuned")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch eagerly instead of through CUDA graphs (profiler captures: "
                         "kernels inside graphs with conditional nodes cannot be profiled)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    legs = set() if args.legs == "none" else set(args.legs.split(","))

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        # the oracle alone: its own generator, no product code loaded
        import oracle

        run_reference_arm(args, make_workload(args.workload, oracle.generate_packing), rank,
                          world)
        return

    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import __graft_entry__

    __graft_entry__.build()
    from spherocyls_gb300 import BoxBatch, SpherocylBox, generate_packing

    w = make_workload(args.workload, generate_packing)
    n = w["n"]
    tuned = {"pad": PAD * args.pad_factor, "block": 128, "pass_kind": args.pass_kind,
             "tile_target": args.tile_target, "persist_steps": args.persist}

    def new_box(precision, profile=False, state=None, shapes=None):
        # the mixed form runs with the autotuned padding and block size
        pad = tuned["pad"] if precision == "mixed" else PAD
        block = tuned["block"] if precision == "mixed" else 0
        kw = dict(pass_kind=tuned["pass_kind"], tile_target=tuned["tile_target"],
                  persist_steps=tuned["persist_steps"]) if precision == "mixed" else {}
        x, y, p = state[:3] if state is not None else (w["x"], w["y"], w["p"])
        A, R = shapes if shapes is not None else (w["A"], w["R"])
        if args.workload == "batch512":
            b = BoxBatch(w["ns"], w["L"], x, y, p, A, R, pad, precision=precision,
                         device=local, profile=profile, use_graphs=not args.no_graphs,
                         block=block, **kw)
            for k, r in enumerate(w["rates"]):
                b.set_strain_rate(float(r), sys=k)
        else:
            b = SpherocylBox(w["L"], x, y, p, A, R, pad,
                             precision=precision, device=local, profile=profile,
                             use_graphs=not args.no_graphs, block=block, **kw)
            b.set_strain_rate(w["rate"])
        b.set_step(w["dt"])
        if state is not None:
            b.set_gamma(state[3])
            b.set_total_gamma(state[4])
        return b

    if args.autotune and not args.only:
        # sc_autotune on the warmed-up workload picks the mixed form's padding and
        # block size (it times copies; the copies' steps are not timed here)
        t = new_box("mixed")
        t.strain_steps(args.warmup)
        # timed on a window as long as the measured one (candidates run as many
        # steps again first); the copies' steps are not timed here
        f, blk = t.autotune(max(args.steps, 20))
        o = t.options()
        t.close()
        tuned = {"pad": PAD * f, "block": blk, "pass_kind": o["pass_kind"],
                 "tile_target": o["tile_target"], "persist_steps": o["persist_steps"]}

    if args.only == "minimise":
        # the minimisation leg alone (profiler captures: --no-graphs launches eagerly)
        print(json.dumps(minimise_leg(args.min_replicas, 4096, args.min_iters, device=local,
                                      graphs=not args.no_graphs, over=args.min_over,
                                      contacts=args.min_contacts)))
        return
    if args.only:
        b = new_box(args.only)
        b.strain_steps(args.warmup)
        c0 = b.counters()
        secs = time_steps(b, args.steps, torch)
        c1 = b.counters()
        # forced full rebuilds of the sorted state in an NVTX range (profiler captures
        # of the rebuild chain select it with --nvtx-include forced_rebuild/)
        torch.cuda.nvtx.range_push("forced_rebuild")
        for _ in range(args.forced_rebuilds):
            b.find_neighbors()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        # one stress and energy evaluation (profiler captures of the reductions)
        torch.cuda.nvtx.range_push("stress_energy")
        b.calc_se()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        if rank == 0:
            print(json.dumps({"only": args.only, "workload": args.workload, "steps": args.steps,
                              "ms_per_step": 1e3 * secs / args.steps,
                              "value": n * args.steps / secs,
                              "rebuilds": c1["rebuilds"] - c0["rebuilds"],
                              "mean_list_length": mean_list_length(b)}))
        return

    # ---- mixed precision, device-resident: the headline value ----
    box = new_box("mixed")
    box.strain_steps(args.warmup)
    # the state after the warm-up, on the host: the start of the end-to-end run
    bx = box.box(0)
    start = (*box.state(), bx["gamma"], bx["gamma_total"])
    counters0 = box.counters()
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler() as clk:
        secs = time_steps(box, args.steps, torch)
    if world > 1:
        torch.distributed.barrier()
    secs = max_over_ranks(secs, world, "cuda")
    value = world * n * args.steps / secs
    counters = box.counters()
    launches = counters["kernels"] - counters0["kernels"]
    rebuild_chains = counters["rebuilds"] - counters0["rebuilds"]

    # ---- the same run continued: a steady-state window after a longer shear ----
    box.strain_steps(args.steady_steps)
    c2 = box.counters()
    steady_k = 200
    secs_ss = time_steps(box, steady_k, torch)
    c3 = box.counters()
    steady = {"value": n * steady_k / secs_ss, "ms_per_step": 1e3 * secs_ss / steady_k,
              "steps": steady_k, "after_steps": args.warmup + args.steps + args.steady_steps,
              "rebuild_chains": c3["rebuilds"] - c2["rebuilds"]}
    box.close()

    # ---- force-pass timing with per-pass CUDA events (same workload, same window) ----
    prof = new_box("mixed", profile=True)
    prof.strain_steps(args.warmup)
    prof.pass_times()
    prof.strain_steps(max(args.steps, 20))
    pt = prof.pass_times()
    pass_ms = 0.5 * (pt["corr_ms"] + pt["pred_ms"])
    peak, peak_kind = _peaks()
    nbar = mean_list_length(prof)
    bpp = bytes_per_pass("mixed", nbar)
    achieved = bpp * n / (pass_ms / 1e3) / 1e9
    # a forced rebuild of every system (cell sort + list build + ordering), host-timed
    # with a synchronisation per call, so it includes the launches of the chain
    prof.find_neighbors()
    t0 = time.perf_counter()
    for _ in range(10):
        prof.find_neighbors()
    full_rebuild_ms = 1e3 * (time.perf_counter() - t0) / 10
    prof.close()

    # ---- plain FP64 form, same window ----
    b64 = new_box("fp64")
    b64.strain_steps(args.warmup)
    secs64 = time_steps(b64, args.steps, torch)
    value64 = world * n * args.steps / max_over_ranks(secs64, world, "cuda")
    b64.close()

    # ---- end to end through the C ABI with host buffers, same window ----
    # inputs and outputs in pinned host memory (filled before the timed region)
    def pinned(a=None, size=None):
        t = torch.empty(len(a) if a is not None else size, dtype=torch.float64, pin_memory=True)
        v = t.numpy()
        if a is not None:
            v[:] = a
        return v

    h_in = [pinned(a) for a in (start[0], start[1], start[2], w["A"], w["R"])]
    h_out = [pinned(size=len(start[0])) for _ in range(3)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # sc_create copies x, y, phi, A, R in
    e2e_box = new_box("mixed", state=(*h_in[:3], start[3], start[4]), shapes=h_in[3:])
    se = e2e_box.strain_steps(args.steps, se_every=args.steps)
    xs, ys, ps = e2e_box.state(out=h_out)
    torch.cuda.synchronize()
    e2e_secs = time.perf_counter() - t0
    e2e_box.close()
    assert se is not None and np.all(np.isfinite(xs))
    e2e_secs = max_over_ranks(e2e_secs, world, "cuda")
    e2e = {"value": world * n * args.steps / e2e_secs, "unit": "particle-steps/s",
           "h2d_bytes_per_step": 40 * n / args.steps,
           "d2h_bytes_per_step": (24 * n + 40) / args.steps, "steps": args.steps,
           "note": "the same window through the C ABI: handle created from pinned host "
                   "arrays of the state after the warm-up, K steps, stress/energy of the "
                   "last step and positions read back to pinned host arrays"}

    extra = {}
    if rank == 0 and "precision" in legs:
        extra["precision_ab"] = precision_ab(local)
    if rank == 0 and "batched" in legs and args.workload != "batch512":
        extra["batched"] = batched_leg(args, local, torch)
    if rank == 0 and "minimise" in legs:
        extra["minimise"] = minimise_leg(args.min_replicas, 4096, args.min_iters, device=local,
                                         over=args.min_over, contacts=args.min_contacts)

    base = None
    if rank == 0 and not args.no_cpu and w.get("phi") is not None:
        import oracle

        wo = make_workload(args.workload, oracle.generate_packing)
        base = cpu_run(wo, 0, args.cpu_steps, os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64",
            "data": "synthetic (seeded crossing-free packing)",
            "config": config_of(args.workload, world),
            "tuning": {"mixed_pad": tuned["pad"], "mixed_block": tuned["block"],
                       "pass_kind": tuned["pass_kind"], "tile_target": tuned["tile_target"],
                       "persist_steps": tuned["persist_steps"]},
            "value_fp64": value64,
            "plain_fp64": {"value": value64, "unit": "particle-steps/s",
                           "ms_per_step": 1e3 * secs64 / args.steps, "steps": args.steps,
                           "mixed_over_fp64": value / value64},
            "steady_state": steady,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": (PASS_DRAM_BYTES_PER_PARTICLE[args.workload] * n
                                     if args.workload in PASS_DRAM_BYTES_PER_PARTICLE
                                     else None),
                         "traffic_unit": "bytes per launch (ncu capture)",
                         "kernel": ("k_tile_pass" if tuned["pass_kind"] == "tile" else
                                    "k_pass_mixed") + " (corrector/predictor force passes)",
                         "pass_ms": pass_ms, "bytes_per_particle_pass": bpp,
                         "mean_list_length": nbar,
                         "rebuild_body_ms_mean_eager": pt["rebuild_ms"],
                         "full_rebuild_ms": full_rebuild_ms},
            "cpu_baseline": base,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(local),
            "rebuild_chains": rebuild_chains,
            **extra,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
