"""Benchmark of the per-timestep fluid update on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full timestep of the simulation (src/fluid.cpp:298-320 and
src/main.cpp:236-239): velocity advection, divergence, the pressure Jacobi
iteration to relative residual 1e-5 (FP64-checked every 100 sweeps, capped at
2000 sweeps), projection and 3-channel image advection, on a 2048x2048 float32
grid with dt = 0.05 and synthetic seeded inputs (8 Gaussian vortices, 16
Gaussian blobs). Fields stay resident in HBM between steps (a session).

Printed (rank 0, one JSON line): cell-updates/s for the whole job; e2e, the
same metric through the C ABI with pinned host buffers copied in and out
every step; the roofline of the dominant kernel (the fused pressure sweep);
a CPU baseline (the oracle port on this host's cores, bounded sample); the
SM clocks sampled during the timed region; kernel launches in the timed
region.

--impl reference times the reference algorithm on the host cores instead
(the oracle port, bit-pinned to src/fluid.cpp; the reference's own build
cannot be compiled on the GPU host because its sources are not there) on one
core, as the single-threaded reference runs, and prints the same line with
"impl": "reference". A full 2048x2048 step (2000 sweeps) takes about 35 s on
one core, so each step is a bounded sample: the step with 100 pressure sweeps,
extrapolated to the step's sweep count with the per-sweep time measured
against the same step without pressure sweeps (the warm-up steps).

forms.headline is the comparison the metric names: the headline's own states
(2048x2048, dt 0.05, seed 1) stepped to relative residual 1e-5 (FP64-checked)
by every form, two steps each, with cell-updates/s, sweeps and final residual
per step and the ratio to the plain FP32 method that reaches 1e-5.

Several GPUs (torchrun): one independent simulation per rank (seed 1 + rank),
no data exchange; the value is the sum over ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s to residual 1e-5: mixed/batched/warm-start vs plain FP32, 1 GB300"
UNIT = "cell-updates/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "sweep_stream_traffic.json")
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--channels", type=int, default=3)
    ap.add_argument("--dt", type=float, default=0.05)
    ap.add_argument("--tol", type=float, default=1e-5)
    ap.add_argument("--cap", type=int, default=2000)
    ap.add_argument("--check-every", type=int, default=100)
    ap.add_argument("--diffuse-iters", type=int, default=40)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--fuse-depth", type=int, default=0)
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=1, help="0: skip the CPU baseline")
    ap.add_argument("--no-forms", action="store_true", help="skip the precision / batched form measurements")
    ap.add_argument("--form-size", type=int, default=4096)
    ap.add_argument("--form-steps", type=int, default=5)
    ap.add_argument("--form-error-steps", type=int, default=20,
                    help="steps of the per-field error run against the FP64 form (0: skip)")
    ap.add_argument("--members", type=int, default=512)
    ap.add_argument("--ens-steps", type=int, default=50)
    ap.add_argument("--no-headline", action="store_true", help="skip the forms-vs-plain comparison to 1e-5")
    ap.add_argument("--headline-steps", type=int, default=2)
    ap.add_argument("--headline-cap", type=int, default=4_000_000)
    ap.add_argument("--headline-every", type=int, default=500)
    ap.add_argument("--cpu-sample-sweeps", type=int, default=100)
    return ap.parse_args()


def workload(a):
    return (f"{a.size}x{a.size} f32 grid, dt {a.dt}, pressure Jacobi to relative residual {a.tol:g} "
            f"(FP64 check every {a.check_every} sweeps, cap {a.cap}), {a.channels}-channel image, "
            f"viscosity 0 ({a.diffuse_iters} identity diffusion sweeps), {a.steps} steps")


def config(a, extra=None):
    """The workload's configuration, the same dict in both arms."""
    cells = a.size * a.size
    state_mb = cells * 4 * (8 + 2 * a.channels) / 1e6
    c = {"workload": workload(a), "grid": [a.size, a.size], "image_channels": a.channels, "dt": a.dt,
         "tol": a.tol, "max_iters": a.cap, "check_every": a.check_every, "seed": a.seed, "form": "plain-fp32",
         "l2": f"per-step state {state_mb:.0f} MB, larger than the L2 cache; no flush between steps"}
    if extra:
        c.update(extra)
    return c


DATA = "synthetic (seeded Gaussian vortices and blobs; the reference's PNG inputs are not used)"


class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def traffic_per_launch(cells, levels):
    """DRAM bytes per fused-sweep launch from the committed ncu summary (scaled
    by cells when the capture used a smaller grid), or None."""
    try:
        with open(TRAFFIC_FILE) as f:
            t = json.load(f)
    except (OSError, ValueError):
        return None, None
    if t.get("levels") != levels:
        return None, None
    return t["dram_bytes_per_launch"] * cells / t["cells"], t.get("source")


# ---------------------------------------------------------------------------------------------
# CPU side (the oracle port of src/fluid.cpp): our arm's cpu_baseline and the reference arm

def cpu_step(O, state, a, sweeps):
    """One timestep of the workload on the oracle port with `sweeps` pressure
    sweeps (residual checks every check_every, as the workload); returns its
    wall time in seconds."""
    vp, tmp, img, itmp = state
    t0 = time.perf_counter()
    vp, tmp, _ = O.step(vp, tmp, a.dt, 0.0, diffuse_iters=a.diffuse_iters, max_iters=sweeps, tol=a.tol,
                        check_every=a.check_every)
    img, itmp = O.advect_color_step(img, itmp, vp, a.dt)
    el = time.perf_counter() - t0
    state[:] = [vp, tmp, img, itmp]
    return el


def cpu_sampled(a, threads, fixed_steps=1, sampled_steps=1):
    """Per-step time of the workload on the host cores, from a bounded sample:
    steps with no pressure sweep (t_fixed: advection, the identity diffusion
    sweeps, divergence, projection, image) and steps with S = --cpu-sample-sweeps
    pressure sweeps; a full step is t_fixed + (t_S - t_fixed) * cap / S (the
    workload hits the cap every step at this size)."""
    from oracle import oracle as O
    from probabilistic_fluid_simulation_gb300 import synthetic
    used = O.set_threads(threads)
    state = list(synthetic.initial_state(a.size, a.size, a.channels, a.seed))
    S = min(a.cpu_sample_sweeps, a.cap)
    cpu_step(O, state, a, 0)  # untimed: first-touch of the buffers, thread start-up
    t_fixed = [cpu_step(O, state, a, 0) for _ in range(fixed_steps)]
    t_s = [cpu_step(O, state, a, S) for _ in range(sampled_steps)]
    tf, ts = float(np.mean(t_fixed)), float(np.mean(t_s))
    per_step = tf + (ts - tf) * a.cap / S
    return {"value": a.size * a.size / per_step, "unit": UNIT, "cores": used, "s_per_step": per_step,
            "sample": f"{a.size}x{a.size} steps of the workload: {fixed_steps} without pressure sweeps "
                      f"({tf:.2f} s) and {sampled_steps} with {S} sweeps ({ts:.2f} s), extrapolated to "
                      f"{a.cap} sweeps per step; oracle port of src/fluid.cpp (bit-equal to it)",
            "sample_s": round(float(np.sum(t_fixed) + np.sum(t_s)), 2)}


def reference_arm(a, rank):
    """The reference's CPU algorithm (the pinned oracle port) on one core: the
    reference is single-threaded (src/fluid.cpp has no threads), so one core
    is what it can use. W warm-up steps without pressure sweeps (they measure
    the step's fixed part), then K timed steps with --cpu-sample-sweeps sweeps
    each; the rate is for full steps (cap sweeps), extrapolated per sweep. An
    all-core run of the same port (OpenMP over rows) is reported beside it as
    not the reference."""
    if rank != 0:
        return 0
    from oracle import oracle as O
    from probabilistic_fluid_simulation_gb300 import synthetic
    threads = O.set_threads(1)
    state = list(synthetic.initial_state(a.size, a.size, a.channels, a.seed))
    S = min(a.cpu_sample_sweeps, a.cap)
    cpu_step(O, state, a, 0)  # untimed: first-touch of the buffers
    t_fixed = [cpu_step(O, state, a, 0) for _ in range(max(1, a.warmup))]
    t0 = time.perf_counter()
    t_s = [cpu_step(O, state, a, S) for _ in range(a.steps)]
    el = time.perf_counter() - t0
    tf, ts = float(np.mean(t_fixed)), float(np.mean(t_s))
    per_step = tf + (ts - tf) * a.cap / S
    val = a.size * a.size / per_step
    sample = (f"{a.steps} timed steps of the {a.size}x{a.size} workload with {S} pressure sweeps each ({ts:.2f} s "
              f"per step, {el:.1f} s in all) after {len(t_fixed)} warm-up steps without pressure sweeps "
              f"({tf:.2f} s each); per-step rate extrapolated to {a.cap} sweeps; oracle port of src/fluid.cpp, "
              f"bit-equal to it, one core")
    allc = cpu_sampled(a, os.cpu_count() or 1)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": DATA, "config": config(a),
            "runs_on": f"host CPU, {threads} thread (the reference is single-threaded)",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "all_cores_not_the_reference": {k: allc[k] for k in ("value", "cores", "sample")}},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------
# The other forms (precision, batched, warm start), each against the plain path on the same workload

def time_session(fluid, vp, tmp, img, steps, stream, **kw):
    import torch
    h, w, _ = vp.shape
    with fluid.Session(w, h, image_shape=img.shape, stream=stream, **kw) as s:
        s.upload(vp, tmp, img)
        s.step(1)
        s.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            s.step(1)
        e1.record()
        torch.cuda.synchronize()
        st = s.stats()
    ms = e0.elapsed_time(e1) / steps
    return {"value": w * h / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "sweeps_per_step": st["sweeps"],
            "final_rel_residual": st["rel_residual"]}


def precision_forms(a, fluid, synthetic, stream):
    n = a.form_size
    vp, tmp, img, _ = synthetic.initial_state(n, n, a.channels, a.seed)
    kw = dict(dt=a.dt, diffuse_iters=a.diffuse_iters, max_iters=a.cap, tol=a.tol, check_every=a.check_every)
    out = {"workload": f"{n}x{n}, same solver settings as the headline, {a.form_steps} steps"}
    for name, prec in (("plain_f32", fluid.PREC_F32), ("bf16", fluid.PREC_BF16), ("f16", fluid.PREC_F16),
                       ("f32r", fluid.PREC_F32R)):
        out[name] = time_session(fluid, vp, tmp, img, a.form_steps, stream, precision=prec, **kw)
    if a.form_error_steps > 0:
        out["fp64_error"] = precision_errors(a, fluid, vp, tmp, img, stream, kw)
    return out


def precision_errors(a, fluid, vp, tmp, img, stream, kw):
    """Per-field error of each form against the FP64 form (the same method in
    double) after the same number of steps from the same state: max |x - y| /
    max |y| over the grid for u, v, p (the pressure), b (the divergence) and
    the image. Every form runs the same sweep count per step when the cap
    binds (it does at 4096x4096: Jacobi needs millions of sweeps there), so
    the difference is rounding alone."""
    import torch
    n = vp.shape[0]
    steps = a.form_error_steps

    def run(prec):
        vp64 = torch.empty((n, n, 4), dtype=torch.float64, device="cuda")
        im64 = torch.empty(img.shape, dtype=torch.float64, device="cuda")
        t0 = time.perf_counter()
        with fluid.Session(n, n, image_shape=img.shape, stream=stream, precision=prec, **kw) as s:
            s.upload(vp, tmp, img)
            s.step(steps)
            s.download_f64(vp64, im64)
            s.sync()
            st = s.stats()
        return vp64, im64, time.perf_counter() - t0, st

    ref_vp, ref_im, ref_s, ref_st = run(fluid.PREC_F64)
    fields = ("u", "v", "p", "b", "image")
    refs = [ref_vp[..., c] for c in range(4)] + [ref_im]
    out = {"steps": steps, "measure": "max |x - x_fp64| / max |x_fp64| per field; rms: ||x - x_fp64|| / ||x_fp64||",
           "note": "b is a near-cancelling difference of neighbouring velocities (the projected field is nearly "
                   "divergence-free), so its relative error is the velocity error amplified by the cancellation, "
                   "and p solves against b: O(1) for float32 storage too",
           "fp64_run_s": round(ref_s, 2), "fp64_sweeps_last_step": ref_st["sweeps"]}
    for name, prec in (("plain_f32", fluid.PREC_F32), ("bf16", fluid.PREC_BF16), ("f16", fluid.PREC_F16),
                       ("f32r", fluid.PREC_F32R)):
        x_vp, x_im, _, st = run(prec)
        xs = [x_vp[..., c] for c in range(4)] + [x_im]
        e = {}
        for f, x, y in zip(fields, xs, refs):
            m, nrm = float(y.abs().max()), float(y.norm())
            d = x - y
            e[f] = float(d.abs().max()) / m if m > 0 else float(d.abs().max())
            e["rms_" + f] = float(d.norm()) / nrm if nrm > 0 else float(d.norm())
        e["sweeps_last_step"] = st["sweeps"]
        out[name] = e
        del x_vp, x_im, xs
    del ref_vp, ref_im, refs
    torch.cuda.empty_cache()
    return out


def boundary_forms(a, fluid, synthetic, stream):
    """Boundary modes on the headline workload (2048x2048, same solver
    settings), 10 steps each: periodic (the reference), the reference's clamp
    mode, walls."""
    n = a.size
    vp, tmp, img, _ = synthetic.initial_state(n, n, a.channels, a.seed)
    kw = dict(dt=a.dt, diffuse_iters=a.diffuse_iters, max_iters=a.cap, tol=a.tol, check_every=a.check_every)
    out = {"workload": f"{n}x{n}, same solver settings as the headline, 10 steps"}
    for name, bc in (("periodic", fluid.BOUNDARY_PERIODIC), ("clamp", fluid.BOUNDARY_CLAMP),
                     ("walls", fluid.BOUNDARY_WALLS)):
        out[name] = time_session(fluid, vp, tmp, img, 10, stream, boundary=bc, **kw)
    return out


def ensemble_sizes(n, seed):
    from probabilistic_fluid_simulation_gb300 import synthetic
    rng = synthetic.SplitMix64(seed * 7919 + 17)
    sides = (64, 128, 256, 512, 1024)
    return [(sides[int(rng.uniform() * 5)], sides[int(rng.uniform() * 5)]) for _ in range(n)]


def ensemble_member(k, w, h, base, channels, seed):
    from probabilistic_fluid_simulation_gb300 import synthetic as S
    vort = [S.Vortex(v.cx * w / 1024, v.cy * h / 1024, v.radius * (w * h) ** 0.5 / 1024, v.circulation)
            for v in S.perturb_vortices(base, seed=seed, member=k)]
    vp = S.velocity_from_vortices(w, h, vort)
    return vp, np.zeros_like(vp), S.blob_image(w, h, channels, seed=seed * 1000 + k)


def batched_form(a, fluid, synthetic, stream):
    import torch
    from probabilistic_fluid_simulation_gb300 import tune
    sizes = ensemble_sizes(a.members, a.seed)
    base = synthetic.draw_vortices(1024, 1024, seed=a.seed)
    states = [ensemble_member(k, w, h, base, a.channels, a.seed) for k, (w, h) in enumerate(sizes)]
    cells = sum(w * h for w, h in sizes)
    # the ensemble's sweep cap and check interval must be multiples of the fuse depth: 2000 and 200
    every = a.check_every if a.check_every % 8 == 0 else 200
    kw = dict(dt=a.dt, diffuse_iters=a.diffuse_iters, max_iters=a.cap, tol=a.tol, check_every=every)
    out = {"workload": f"{a.members} members, sides uniform in {{64..1024}} (w, h drawn independently), "
                       f"{cells} cells, perturbed vortex fields (+N(0,0.05) circulation, +N(0,2) cells), "
                       f"residual {a.tol:g} checked every {every} sweeps, cap {a.cap}"}
    with fluid.Ensemble(sizes, a.channels, stream=stream, **kw) as ens:
        for k, st in enumerate(states):
            ens.upload(k, *st)
        best, timings = tune.tune_ensemble(ens, steps=1)
        ens.step(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = fluid.kernel_launches()
        e0.record()
        ens.step(a.ens_steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.ens_steps
        launches = (fluid.kernel_launches() - l0) / a.ens_steps
        info = ens.info()
        stats = [ens.stats(k) for k in range(len(sizes))]
        # ensemble statistics of the image over the largest group of members with one grid size
        from collections import Counter
        shape = Counter(sizes).most_common(1)[0][0]
        group = [k for k, sz in enumerate(sizes) if sz == shape]
        md = torch.empty(shape[1], shape[0], a.channels, device="cuda")
        vd = torch.empty_like(md)
        ens.image_stats(group, md, vd)  # warm-up (allocates the member list)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ens.image_stats(group, md, vd)
        stats_ms = 1e3 * (time.perf_counter() - t0)
        ens_mean, ens_var = md.cpu().numpy(), vd.cpu().numpy()
        sample = [0, len(sizes) // 3, 2 * len(sizes) // 3, len(sizes) - 1]
        ens_out = {}
        for k in sample:
            vpo, imo = np.empty_like(states[k][0]), np.empty_like(states[k][2])
            ens.download(k, vpo, imo)
            ens_out[k] = (vpo, imo)
    out["batched"] = {"value": cells / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": a.ens_steps,
                      "launches_per_step": launches, "graph": bool(info["graphs"]), "grid_blocks": info["grid_blocks"],
                      "autotuned": {"fuse_depth": best[0], "chunk_rows": best[1],
                                    "candidates_ms": [[f, c, round(t, 3)] for f, c, t in timings]},
                      "mean_sweeps": float(np.mean([s["sweeps"] for s in stats])),
                      "capped": int(sum(s["capped"] for s in stats))}
    # the sampled members through plain sessions with the same steps (the tuner restores the
    # initial state, then 1 + ens_steps steps ran): fields must be identical
    maxdiff = 0.0
    for k in sample:
        vp, tmp, img = states[k]
        h, w, _ = vp.shape
        with fluid.Session(w, h, image_shape=img.shape, stream=stream, **kw) as s:
            s.upload(vp, tmp, img)
            s.step(1 + a.ens_steps)
            vpo, imo = np.empty_like(vp), np.empty_like(img)
            s.download(vpo, None, imo)
        ev, ei = ens_out[k]
        maxdiff = max(maxdiff, float(np.abs(ev[..., :2] - vpo[..., :2]).max()), float(np.abs(ei - imo).max()))
    # plain-session throughput on the whole ensemble: one step of every member
    sess = []
    for k, (vp, tmp, img) in enumerate(states):
        h, w, _ = vp.shape
        s = fluid.Session(w, h, image_shape=img.shape, stream=stream, **kw)
        s.upload(vp, tmp, img)
        sess.append(s)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in sess:
        s.step(1)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    for s in sess:
        s.close()
    out["plain_sessions"] = {"value": cells / el, "unit": UNIT, "ms_per_step": el * 1e3,
                             "how": "one pfs_session per member, stepped one after another (1 step each)"}
    out["members_checked_vs_sessions"] = {"members": sample, "max_abs_diff": maxdiff}
    # the same statistics from per-instance plain runs of the group's members
    imgs = []
    for k in group:
        vp, tmp, img = states[k]
        h, w, _ = vp.shape
        with fluid.Session(w, h, image_shape=img.shape, stream=stream, **kw) as s:
            s.upload(vp, tmp, img)
            s.step(1 + a.ens_steps)
            imo = np.empty_like(img)
            s.download(None, None, imo)
        imgs.append(imo.astype(np.float64))
    imgs = np.stack(imgs)
    out["to_tolerance"] = batched_to_tolerance(a, fluid, stream, sizes, states)
    out["image_statistics"] = {
        "members": len(group), "grid": list(shape), "ms": stats_ms,
        "how": "pointwise mean and population variance of the image over the members of the most common grid "
               "size (pfs_ensemble_image_stats, FP64 accumulation), against numpy over the same members run as "
               "plain sessions",
        "max_abs_diff_mean": float(np.abs(ens_mean - imgs.mean(axis=0)).max()),
        "max_abs_diff_var": float(np.abs(ens_var - imgs.var(axis=0)).max()),
        "max_var": float(imgs.var(axis=0).max())}
    return out


def batched_to_tolerance(a, fluid, stream, sizes, states, every_nth=8):
    """Every `every_nth` member of the ensemble workload (the same size
    distribution) in the refined float32 form (PFS_PREC_F32R), one step to
    relative residual 1e-5 in one persistent launch, against the same members
    as plain sessions one after another: cells-weighted rates and the
    distribution of the sweeps each member needed (members that converge stop
    taking sweep work)."""
    import torch
    idx = list(range(0, len(sizes), every_nth))
    sub = [sizes[k] for k in idx]
    cells = sum(w * h for w, h in sub)
    kw = dict(dt=a.dt, diffuse_iters=a.diffuse_iters, max_iters=2_000_000, tol=a.tol, check_every=256,
              precision=fluid.PREC_F32R)
    with fluid.Ensemble(sub, a.channels, stream=stream, **kw) as ens:
        for j, k in enumerate(idx):
            ens.upload(j, *states[k])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ens.step(1)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        st = [ens.stats(j) for j in range(len(sub))]
    t_sess = 0.0
    sess_sweeps = []
    for k in idx:
        v, t, im = states[k]
        h, w, _ = v.shape
        with fluid.Session(w, h, image_shape=im.shape, stream=stream, **kw) as sess:
            sess.upload(v, t, im)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            sess.step(1)
            sess.sync()
            t_sess += time.perf_counter() - t1
            sess_sweeps.append(sess.stats()["sweeps"])
    sw = np.array([x["sweeps"] for x in st])
    return {"members": len(sub), "cells": cells, "workload": f"every {every_nth}th member of the ensemble workload, "
                                                           f"PFS_PREC_F32R, one step to relative residual {a.tol:g}",
            "value": cells / el, "ms": 1e3 * el, "sessions_value": cells / t_sess, "sessions_ms": 1e3 * t_sess,
            "ratio_vs_sessions": t_sess / el,
            "converged": int(sum(1 for x in st if x["rel_residual"] <= a.tol)),
            "sweeps_percentiles": {q: int(np.percentile(sw, q)) for q in (0, 25, 50, 75, 100)},
            "sweeps_equal_sessions": int(sum(1 for x, y in zip(sw, sess_sweeps) if x == y))}


def warm_start_form(a, fluid, stream):
    """The learned warm start at the network's training size (256x256, dt 0.1,
    seeds 0 and 1, two steps each, PFS_PREC_F32R to relative residual 1e-5):
    network start against zero start, and the reference's previous-pressure
    start. The 2048x2048 headline states are in forms.headline."""
    from probabilistic_fluid_simulation_gb300 import warmstart as WS
    params, meta = WS.load_default()
    r = WS.evaluate(params, 256, [0, 1], steps=2, check_every=200, starts=((1, 2),), log=lambda *_: None)
    z, n = r["zero"], r["network"]["coarsen1_passes2"]
    return {"workload": "256x256 states of 8-vortex fields (seeds 0, 1; steps 1, 2; dt 0.1), one step each to "
                        "relative residual 1e-5, PFS_PREC_F32R",
            "network": {"trained_on": f"{meta['pairs']} solver pairs at {meta['size']}x{meta['size']}",
                        "held_out_loss": meta["training"]["val_loss"][-1]},
            "zero_start": {"value": z["cell_updates_per_s"], "ms_per_step": z["mean_ms_per_step"],
                           "sweeps_per_step": z["mean_sweeps"]},
            "network_start": {"value": n["cell_updates_per_s"], "ms_per_step": n["mean_ms_per_step"],
                              "sweeps_per_step": n["mean_sweeps"], "fallbacks": n["fallbacks"]},
            "sweeps_saved": n["sweeps_saved"], "time_ratio": n["time_ratio"],
            "previous_start_sweeps": r["previous"]["mean_sweeps"]}


def headline_batched(a, fluid, stream, vp, tmp, img, plain_row, extra=15):
    """The batched form on an ensemble containing the headline state: the
    2048x2048 state and `extra` perturbed members of the ensemble workload's
    generator with sides drawn from {256, 512}, all PFS_PREC_F32R to relative
    residual 1e-5, --headline-steps steps in one persistent launch per step,
    against the same members stepped as plain sessions (the 2048x2048 one is the
    plain row; checks every 512 sweeps here, a multiple of the fuse depth)."""
    import torch
    n, steps = a.size, a.headline_steps
    rng = np.random.default_rng(a.seed)
    sizes = [(n, n)] + [(int(rng.choice((256, 512))), int(rng.choice((256, 512)))) for _ in range(extra)]
    from probabilistic_fluid_simulation_gb300 import synthetic as S
    base = S.draw_vortices(1024, 1024, seed=a.seed)
    states = [(vp, tmp, img)] + [ensemble_member(k, w, h, base, a.channels, a.seed)
                                 for k, (w, h) in enumerate(sizes) if k > 0]
    cells = sum(w * h for w, h in sizes)
    cap = a.headline_cap // 8 * 8
    kw = dict(dt=a.dt, diffuse_iters=a.diffuse_iters, max_iters=cap, tol=a.tol, check_every=512,
              precision=fluid.PREC_F32R)
    with fluid.Ensemble(sizes, a.channels, stream=stream, **kw) as ens:
        for k, st in enumerate(states):
            ens.upload(k, *st)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ens.step(steps)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        stats = [ens.stats(k) for k in range(len(sizes))]
    # the smaller members as plain (F32R) sessions; the headline member's time is the plain row's
    t_small = 0.0
    for k in range(1, len(sizes)):
        v, t, im = states[k]
        h, w, _ = v.shape
        with fluid.Session(w, h, image_shape=im.shape, stream=stream, **kw) as sess:
            sess.upload(v, t, im)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            sess.step(steps)
            sess.sync()
            t_small += time.perf_counter() - t1
    t_sessions = sum(plain_row["ms_per_step"]) / 1e3 + t_small
    value = cells * steps / el
    return {"value": value, "members": len(sizes), "sizes": f"{n}x{n} + {extra} of sides 256/512",
            "ms_per_step": round(1e3 * el / steps, 1), "sweeps_headline_member": stats[0]["sweeps"],
            "sweeps_min_max": [min(x["sweeps"] for x in stats), max(x["sweeps"] for x in stats)],
            "rel_max": float(f"{max(x['rel_residual'] for x in stats):.3g}"),
            "converged": int(sum(1 for x in stats if x["rel_residual"] <= a.tol)),
            "sessions_value": float(f"{cells * steps / t_sessions:.4g}"),
            "ratio_vs_sessions": round(t_sessions / el, 3)}


def headline_forms(a, fluid, synthetic, stream):
    """The comparison the metric names, on the headline's own states: the
    2048x2048 workload (dt 0.05, seed 1, viscosity 0 with 40 identity
    diffusion sweeps, 3-channel image) stepped --headline-steps times by each
    form with the pressure iterated to relative residual 1e-5 (FP64-checked;
    cap --headline-cap sweeps, never reached). Step 2 starts from step 1's
    pressure, as the reference carries it over (src/fluid.cpp:298-305).

    plain_f32  the reference's float32 arithmetic, bit-exact with src/fluid.cpp:
               its float32 pressure cannot represent the solution to 1e-5 at
               this size, so it stops where its residual stops falling (its
               rounding floor), reported with the time to reach it;
    plain      the plain method that reaches 1e-5 (PFS_PREC_F32R): the same
               float32 Jacobi sweeps (the plain form's kernels), with the
               pressure accumulated as a pair of floats (about 48 bits) and
               refined when the float32 correction has run its interval or
               meets the tolerance; the reference's previous-pressure start.
               Every ratio is against this row;
    zero_start the same from zero pressure each step;
    bf16, f16  the precision forms (16-bit storage, FP32 compute, float-pair
               pressure, residual and refinement in error-free float32
               arithmetic), to 1e-5 or to their floor;
    network    the learned warm start (the shipped network on the grid
               coarsened 8x, 8 damped passes), then the plain iteration;
    batched    the ensemble form on the headline state together with smaller
               perturbed members (see the row)."""
    import torch
    n, steps = a.size, a.headline_steps
    vp, tmp, img, _ = synthetic.initial_state(n, n, a.channels, a.seed)
    base = dict(dt=a.dt, diffuse_iters=a.diffuse_iters, max_iters=a.headline_cap, tol=a.tol, stall_sweeps=-1)

    def run(precision, every, start=None, net=None, coarsen=1, passes=1):
        with fluid.Session(n, n, image_shape=img.shape, stream=stream, precision=precision, check_every=every,
                           **base) as s:
            if start is not None:
                s.set_start(start, net, coarsen, passes)
            s.upload(vp, tmp, img)
            ms, sw, rel, kinds = [], [], [], []
            for _ in range(steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s.step(1)
                s.sync()
                ms.append(1e3 * (time.perf_counter() - t0))
                st = s.stats()
                sw.append(st["sweeps"])
                rel.append(st["rel_residual"])
                kinds.append("stalled" if st["stalled"] else "capped" if st["capped"] else "converged")
            fields = np.empty((n, n, 4), np.float64)
            s.download_f64(fields)
        tot = sum(ms) / 1e3
        row = {"value": n * n * steps / tot, "ms_per_step": [round(x, 1) for x in ms], "sweeps": sw,
               "rel": [float(f"{x:.3g}") for x in rel], "end": kinds}
        return row, fields[..., :3]

    out = {"workload": f"{n}x{n}, dt {a.dt}, seed {a.seed}, to relative residual {a.tol:g} (FP64 check), "
                       f"{steps} steps per form, cap {a.headline_cap} sweeps, residual checks every "
                       f"{a.headline_every} sweeps (16-bit forms: refinement every 32)",
           "unit": UNIT}
    rows, fields = {}, {}
    rows["plain_f32"], fields["plain_f32"] = run(fluid.PREC_F32, a.headline_every)
    rows["plain"], fields["plain"] = run(fluid.PREC_F32R, a.headline_every)
    rows["zero_start"], fields["zero_start"] = run(fluid.PREC_F32R, a.headline_every, start=fluid.START_ZERO)
    rows["bf16"], fields["bf16"] = run(fluid.PREC_BF16, 32)
    rows["f16"], fields["f16"] = run(fluid.PREC_F16, 32)
    from probabilistic_fluid_simulation_gb300 import warmstart as WS
    params, _ = WS.load_default()
    net = fluid.UNet((n // 8) ** 2)
    net.set_params(params)
    rows["network"], fields["network"] = run(fluid.PREC_F32R, a.headline_every, start=fluid.START_NETWORK, net=net,
                                             coarsen=8)
    net.close()
    rows["batched"] = headline_batched(a, fluid, stream, vp, tmp, img, rows["plain"])
    plain = rows["plain"]["value"]
    ref = fields["plain"]
    for k, r in rows.items():
        r["ratio_vs_plain"] = round(r["value"] / plain, 3)
        r["value"] = float(f"{r['value']:.4g}")
        if k not in ("plain", "batched"):
            # the answer after the same steps against the plain row's: max |x - x_plain| / max |x_plain|
            # (the pressure with its mean removed: the periodic operator ignores constants)
            e = {}
            for i, c in enumerate(("u", "v", "p")):
                x, y = fields[k][..., i], ref[..., i]
                if c == "p":
                    x, y = x - x.mean(), y - y.mean()
                e[c] = float(f"{np.abs(x - y).max() / np.abs(y).max():.3g}")
            r["err_vs_plain"] = e
    out["note"] = ("16-bit storage rounds u and v by more than their near-cancelling differences, so those forms' "
                   "divergence is mostly rounding noise, which Jacobi removes fast: their residual is relative to "
                   "that noisy b, and err_vs_plain shows how far their answer is from the plain row's")
    out.update(rows)
    return out


def cli_form(a):
    """The command-line driver (same argv as the reference's src/main.cpp) on a
    1024x1024 velocity PNG and image PNG, 20 steps, NUM_JACOBI_ITERS 30: timed
    only, and writing every step's image as a PNG. Rates from the driver's own
    "N timesteps took X us" line."""
    import re
    import tempfile
    from probabilistic_fluid_simulation_gb300 import build as B
    n, steps = 1024, 20
    cli = B.CLI_BIN
    if not os.path.exists(cli):
        return {"unavailable": "driver not built"}
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    out = {"workload": f"{n}x{n} velocity and image PNGs (RGBA, smooth synthetic), {steps} steps, 30 sweeps"}
    with tempfile.TemporaryDirectory() as d:
        for name, ph in (("v.png", 0.3), ("i.png", 1.1)):
            img = np.stack([0.5 + 0.45 * np.sin(2 * np.pi * (k + 1) * xx / n + ph * k) * np.cos(2 * np.pi * yy / n)
                            for k in range(4)], axis=-1)
            rgba = np.clip(np.round(img * 255), 0, 255).astype(np.uint8)
            _write_png(os.path.join(d, name), rgba)
        for mode, extra in (("timed_only", []), ("png_every_step", [os.path.join(d, "out")])):
            r = subprocess.run([cli, str(steps), "0.1", "0.0", os.path.join(d, "i.png"), os.path.join(d, "v.png")]
                               + extra, capture_output=True, text=True, timeout=600)
            m = re.search(r"(\d+) timesteps took (\d+) us", r.stdout)
            if r.returncode != 0 or not m:
                out[mode] = {"failed": (r.stderr or r.stdout)[-300:]}
                continue
            us = int(m.group(2))
            out[mode] = {"value": n * n * steps / (us / 1e6), "unit": UNIT, "ms_per_step": us / 1e3 / steps}
    return out


def _write_png(path, rgba):
    import ctypes as C
    from probabilistic_fluid_simulation_gb300 import build as B
    lib = C.CDLL(B.PNG_LIB)
    lib.pfs_png_encode.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
    lib.pfs_png_free.argtypes = [C.c_void_p]
    p, sz = C.c_void_p(), C.c_size_t()
    rgba = np.ascontiguousarray(rgba)
    assert lib.pfs_png_encode(rgba.ctypes.data, rgba.shape[1], rgba.shape[0], C.byref(p), C.byref(sz)) == 0
    with open(path, "wb") as f:
        f.write(C.string_at(p, sz.value))
    lib.pfs_png_free(p)


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        return reference_arm(a, rank)

    import torch
    from probabilistic_fluid_simulation_gb300 import fluid, synthetic

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream().cuda_stream

    cells = a.size * a.size
    vp, tmp, img, itmp = synthetic.initial_state(a.size, a.size, a.channels, a.seed + rank)
    params = fluid.default_params(dt=a.dt, viscosity=0.0, diffuse_iters=a.diffuse_iters, max_iters=a.cap,
                                  tol=a.tol, check_every=a.check_every, fuse_depth=a.fuse_depth,
                                  chunk_rows=a.chunk)
    sess = fluid.Session(a.size, a.size, image_shape=img.shape, params=params, stream=stream)
    sess.upload(vp, tmp, img)

    for _ in range(a.warmup):
        sess.step(1)
    sess.sync()
    st0 = sess.stats()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)  # let the sampler come up
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = fluid.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    sweeps = []
    for _ in range(a.steps):
        sess.step(1)
        sweeps.append(sess.stats()["sweeps"])
    ev1.record()
    torch.cuda.synchronize()
    launches = fluid.kernel_launches() - launches0
    ms = ev0.elapsed_time(ev1)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    clk = clocks.stop()
    st1 = sess.stats()
    value = cells * a.steps * world / (ms / 1e3)

    # Dominant kernel: the fused pressure sweep, timed alone on this stream
    # (back to back, as a solve launches it; chunk 0 = the library's default).
    levels = a.fuse_depth or 8
    chunk = a.chunk
    ld = (a.size + 31) // 32 * 32
    p = torch.randn(a.size, ld, device="cuda")
    bpl = torch.randn(a.size, ld, device="cuda")
    q = torch.empty_like(p)
    for _ in range(5):
        fluid.pressure_sweeps(p, bpl, q, None, levels, fused=True, chunk_rows=chunk, w=a.size, stream=stream)
    nrep = 200
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    k0.record()
    for i in range(nrep):
        src, dst = (p, q) if i % 2 == 0 else (q, p)
        fluid.pressure_sweeps(src, bpl, dst, None, levels, fused=True, chunk_rows=chunk, w=a.size, stream=stream)
    k1.record()
    torch.cuda.synchronize()
    kms = k0.elapsed_time(k1) / nrep
    peak, peak_src = measured_peak()
    launch_bytes = 12.0 * cells  # p and b read once, p written once per launch, whatever the fused depth
    achieved = launch_bytes / (kms / 1e3) / 1e9
    traffic, tsrc = traffic_per_launch(cells, levels)
    props = torch.cuda.get_device_properties(local)
    sm_mhz = clk["sm_mhz"] if clk else None
    fp32_peak = props.multi_processor_count * 128 * (sm_mhz or 2070.0) * 1e6 / 1e12  # TFLOP/s, 1 op/lane/cycle
    fp32_ops = 5.0 * cells * levels  # per cell and sweep: four adds and a multiply
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": f"k_sweep_stream<float,8,{levels}>", "levels_per_launch": levels,
                "avg_launch_us": kms * 1e3, "algorithmic_bytes_per_launch": launch_bytes,
                "bytes_rule": "12 B per cell per launch: the launch reads p and b once and writes p once for all "
                              f"{levels} fused sweeps",
                "peak_source": f"{peak_src} (hbm_gbs, burst copy)", "traffic_source": tsrc,
                "effective_gbs": 12.0 * cells * levels / (kms / 1e3) / 1e9,
                "effective_note": "12 B per cell per sweep over the launch time: the temporal-blocking figure, not "
                                  "an HBM rate",
                "fp32": {"ops_per_launch": fp32_ops, "tflops": fp32_ops / (kms / 1e3) / 1e12,
                         "peak_tflops": fp32_peak, "frac": fp32_ops / (kms / 1e3) / 1e12 / fp32_peak,
                         "rule": "5 FP32 operations per cell per sweep (useful work; halo recomputation not "
                                 "counted); peak = SMs x 128 lanes x the sampled SM clock"}}
    del p, bpl, q

    # e2e: the same steps through the C ABI, every step's state copied in from pinned host buffers
    # and its result (both velocity buffers and the image) copied back out
    e2e = None
    if not a.no_e2e:
        ne = a.e2e_steps or a.steps

        def pinned(x):
            return torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()
        hin = (pinned(vp), pinned(np.zeros_like(tmp)), pinned(img))
        hout = tuple(pinned(np.zeros_like(x)) for x in hin)

        def timed(fn):
            if dist:
                dist.barrier()
            t0 = time.perf_counter()
            fn()
            el = time.perf_counter() - t0
            if dist:
                t = torch.tensor([el], device="cuda", dtype=torch.float64)
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                el = float(t.item())
            return el

        def serial():  # each call returns once its copy is done
            for _ in range(ne):
                sess.upload(*hin)
                sess.step(1)
                sess.download(*hout)

        def pipelined():  # the next state's upload is queued before each step: copies overlap the steps
            sess.upload_async(*hin)
            for k in range(ne):
                if k + 1 < ne:
                    sess.upload_async(*hin)
                sess.step(1)
                sess.download_async(*hout)
            sess.sync()

        sess.upload(*hin)
        sess.step(1)
        sess.download(*hout)
        el_serial = timed(serial)
        pipelined()
        el = timed(pipelined)
        nbytes = sum(x.nbytes for x in hin)
        e2e = {"value": cells * ne * world / el, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": sum(x.nbytes for x in hout), "steps": ne,
               "api": "pfs_session_upload_async + pfs_session_step(1) + pfs_session_download_async per step, "
                      "pinned host buffers, pfs_session_sync at the end",
               "serial": {"value": cells * ne * world / el_serial,
                          "api": "pfs_session_upload(PFS_HOST) + pfs_session_step(1) + "
                                 "pfs_session_download(PFS_HOST) per step"}}
    sess.close()

    forms = None
    if rank == 0 and not a.no_forms:
        forms = {"precision": precision_forms(a, fluid, synthetic, stream),
                 "batched": batched_form(a, fluid, synthetic, stream),
                 "warm_start_256": warm_start_form(a, fluid, stream),
                 "cli": cli_form(a),
                 "boundary": boundary_forms(a, fluid, synthetic, stream)}
    if rank == 0 and not a.no_headline:
        forms = forms or {}
        forms["headline"] = headline_forms(a, fluid, synthetic, stream)

    cpu = None
    if rank == 0 and not a.no_cpu and a.cpu_steps > 0:
        one = cpu_sampled(a, 1)
        allc = cpu_sampled(a, os.cpu_count() or 1)
        cpu = {"value": one["value"], "unit": UNIT, "cores": 1, "kind": "port", "sample": one["sample"],
               "note": "one core: the reference is single-threaded",
               "all_cores_not_the_reference": {k: allc[k] for k in ("value", "cores", "sample")}}

    if rank == 0:
        mean_sweeps = float(np.mean(sweeps))
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": DATA,
                "config": config(a), "tuning": {"fuse_depth": levels, "chunk_rows": chunk or "default"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk,
                "solver": {"sweeps_per_step": mean_sweeps, "cap_hits": st1["cap_hits"] - st0["cap_hits"],
                           "final_rel_residual": st1["rel_residual"],
                           "cell_sweeps_per_s": cells * mean_sweeps * a.steps * world / (ms / 1e3)},
                "forms": forms}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
