"""Timing and tuning of the fused pressure sweep (k_sweep_stream).

    python -m probabilistic_fluid_simulation_gb300.tune --size 2048 --levels 8 --chunk 32
    python -m probabilistic_fluid_simulation_gb300.tune --size 2048 --scan
    python -m probabilistic_fluid_simulation_gb300.tune --size 2048 --ensemble 1 --ens-sweeps 64

Times back-to-back launches of `levels` fused sweeps on random planar
fields with CUDA events on the launching stream and prints microseconds per
launch and cell-sweeps per second. --scan times every (levels, chunk rows)
candidate and prints the fastest; `best_config` is the same search as a
function (used to pick a session's fuse depth and chunk height).
--ensemble N times the step of the batched form (one persistent launch) on N
grids of that size instead; `tune_ensemble` picks an ensemble's fuse depth
and chunk height.
"""
from __future__ import annotations

import argparse
import json

from . import fluid

LEVELS = (4, 8)
CHUNKS = (16, 24, 32, 48, 64, 96)


def time_sweeps(size: int, levels: int, chunk: int, reps: int = 100, warm: int = 5, height: int = 0) -> float:
    """Microseconds per fused launch of `levels` sweeps on a size x height grid."""
    import torch
    h = height or size
    ld = (size + 31) // 32 * 32
    g = torch.Generator(device="cpu").manual_seed(0)
    p = torch.randn(h, ld, generator=g).cuda()
    b = torch.randn(h, ld, generator=g).cuda()
    q = torch.empty_like(p)
    stream = torch.cuda.current_stream().cuda_stream

    def run(n):
        for i in range(n):
            src, dst = (p, q) if i % 2 == 0 else (q, p)
            fluid.pressure_sweeps(src, b, dst, None, levels, fused=True, chunk_rows=chunk, w=size, stream=stream)

    run(warm)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run(reps)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) * 1e3 / reps


def best_config(size: int, height: int = 0, levels=LEVELS, chunks=CHUNKS, reps: int = 50):
    """(levels, chunk, us_per_sweep) with the lowest time per sweep."""
    best = None
    for lv in levels:
        for ch in chunks:
            us = time_sweeps(size, lv, ch, reps=reps, height=height) / lv
            if best is None or us < best[2]:
                best = (lv, ch, us)
    return best


ENSEMBLE_CANDIDATES = ((8, 16), (8, 24), (8, 32), (8, 48), (4, 16), (4, 32), (4, 64))


def tune_ensemble(ens, steps: int = 1, candidates=ENSEMBLE_CANDIDATES):
    """Pick the ensemble's (fuse depth, chunk rows) by timing `steps` steps
    per candidate, each from the ensemble's current state (snapshot taken
    first, restored before every trial and at the end); leaves the fastest
    configured. Returns (best, timings), timings = [(fuse, chunk, ms/step)]."""
    import torch
    p = ens.params
    timings = []
    ens.snapshot()
    for fuse, chunk in candidates:
        if p.max_iters % fuse or (p.check_every > 0 and p.check_every % fuse):
            continue
        ens.config(fuse, chunk)
        ens.restore()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ens.step(steps)
        e1.record()
        torch.cuda.synchronize()
        timings.append((fuse, chunk, e0.elapsed_time(e1) / steps))
    best = min(timings, key=lambda t: t[2])
    ens.config(best[0], best[1])
    ens.restore()
    return best, timings


def time_ensemble(w: int, h: int, members: int, levels: int, chunk: int, sweeps: int, reps: int = 3) -> float:
    """ms per step of an ensemble of `members` w x h vortex states (float32,
    `sweeps` pressure sweeps per step, no residual checks), CUDA events around
    `reps` steps after one untimed step."""
    import torch
    from probabilistic_fluid_simulation_gb300 import synthetic
    kw = dict(dt=0.05, diffuse_iters=40, max_iters=sweeps, tol=0.0, check_every=0, fuse_depth=levels,
              chunk_rows=chunk or 32)
    with fluid.Ensemble([(w, h)] * members, 3, **kw) as ens:
        for k in range(members):
            vp, tmp, img, _ = synthetic.initial_state(w, h, 3, seed=k)
            ens.upload(k, vp, tmp, img)
        ens.step(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ens.step(reps)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--levels", type=int, default=8)
    ap.add_argument("--chunk", type=int, default=0, help="rows per warp task; 0: the library default for the grid")
    ap.add_argument("--reps", type=int, default=100)
    ap.add_argument("--scan", action="store_true")
    ap.add_argument("--scan-levels", default=",".join(str(x) for x in LEVELS), help="fuse depths for --scan")
    ap.add_argument("--ensemble", type=int, default=0,
                    help="time the step of an ensemble of this many --size grids instead (the batched form)")
    ap.add_argument("--ens-sweeps", type=int, default=2000, help="pressure sweeps per ensemble step")
    a = ap.parse_args()
    cells = a.size * (a.height or a.size)
    if a.ensemble:
        ms = time_ensemble(a.size, a.height or a.size, a.ensemble, a.levels, a.chunk, a.ens_sweeps, a.reps)
        print(json.dumps({"size": a.size, "members": a.ensemble, "levels": a.levels, "sweeps": a.ens_sweeps,
                          "ms_per_step": ms, "cell_sweeps_per_s": cells * a.ensemble * a.ens_sweeps / (ms * 1e-3)}))
    elif a.scan:
        rows = []
        for lv in (int(x) for x in a.scan_levels.split(",")):
            for ch in CHUNKS:
                us = time_sweeps(a.size, lv, ch, reps=a.reps, height=a.height)
                rows.append({"levels": lv, "chunk": ch, "us_per_launch": us,
                             "cell_sweeps_per_s": cells * lv / (us * 1e-6)})
                print(json.dumps(rows[-1]), flush=True)
        best = max(rows, key=lambda r: r["cell_sweeps_per_s"])
        print(json.dumps({"best": best}))
    else:
        us = time_sweeps(a.size, a.levels, a.chunk, reps=a.reps, height=a.height)
        print(json.dumps({"size": a.size, "levels": a.levels, "chunk": a.chunk, "us_per_launch": us,
                          "cell_sweeps_per_s": cells * a.levels / (us * 1e-6)}))


if __name__ == "__main__":
    main()
