"""Learned warm start: training data, training, evaluation.

    python -m probabilistic_fluid_simulation_gb300.warmstart train --pairs 20000 --epochs 4 --out weights.npz
    python -m probabilistic_fluid_simulation_gb300.warmstart eval --weights weights.npz --size 1024 --starts 4x1
    python -m probabilistic_fluid_simulation_gb300.warmstart export --out unet.bin
    python -m probabilistic_fluid_simulation_gb300.warmstart bench-net --size 256 --batch 16

Training pairs come from the solver itself: members of the 256x256 workload
(8 seeded Gaussian vortices, dt 0.1) are stepped by the ensemble solver with
the pressure iterated towards relative residual 1e-5 (the float32 iterate
stops near 1e-4 there, its rounding floor, far below the network's error);
after each step the divergence b and the final pressure p of every member
form a pair, normalised by rms(b) (the pressure equation is linear in b) and
with p's mean removed (the periodic operator ignores constants). The network
(pfs_unet_*, the library's own forward and backward kernels) is trained with
Adam on the mean squared error of the normalised pressure. Evaluation runs
refined-float32 sessions (PFS_PREC_F32R: float32 sweeps, FP64 pressure and
residual) to relative residual 1e-5 with a zero initial pressure and with the
network's prediction (PFS_START_NETWORK) and reports sweeps and wall time.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import time

import numpy as np

from . import fluid, synthetic

SIZE = 256


def _field(args):
    size, seed = args
    return synthetic.vortex_field(size, size, seed)


def vortex_fields(size, seeds, workers=16):
    """Velocity fields for many seeds (host, in a spawn pool: safe after CUDA init)."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(workers, len(seeds))) as pool:
        return pool.map(_field, [(size, s) for s in seeds], chunksize=8)


def make_pairs(n_pairs, size=SIZE, steps_per_member=4, seed0=10_000, batch=256, dt=0.1, tol=1e-5, cap=40_000,
               check_every=400, log=print):
    """(b, p) normalised pairs as two (n_pairs, size, size) float32 CUDA tensors."""
    import torch
    members = math.ceil(n_pairs / steps_per_member)
    B = torch.empty(n_pairs, size, size, device="cuda")
    P = torch.empty(n_pairs, size, size, device="cuda")
    kw = dict(dt=dt, diffuse_iters=2, max_iters=cap, tol=tol, check_every=check_every)
    filled, t0 = 0, time.time()
    sweeps = []
    for start in range(0, members, batch):
        seeds = list(range(seed0 + start, seed0 + min(members, start + batch)))
        fields = vortex_fields(size, seeds)
        zeros = np.zeros_like(fields[0])
        with fluid.Ensemble([(size, size)] * len(seeds), 0, **kw) as ens:
            for k, vp in enumerate(fields):
                ens.upload(k, vp, zeros, None)
            buf = torch.empty(size, size, 4, device="cuda")
            for _ in range(steps_per_member):
                ens.step(1)
                for k in range(len(seeds)):
                    if filled >= n_pairs:
                        break
                    ens.download(k, buf, None)
                    sweeps.append(ens.stats(k)["sweeps"])
                    b = buf[..., 3]
                    s = torch.sqrt((b.double() ** 2).mean()).float().clamp_min(1e-30)
                    p = buf[..., 2] - buf[..., 2].mean()
                    B[filled] = b / s
                    P[filled] = p / s
                    filled += 1
        log(f"pairs {filled}/{n_pairs}  ({time.time() - t0:.1f} s, mean sweeps to tol {np.mean(sweeps):.0f})")
        if filled >= n_pairs:
            break
    return B[:filled], P[:filled], {"mean_sweeps": float(np.mean(sweeps)), "seconds": time.time() - t0}


def init_params(n_params, seed=0):
    """He-normal convolution weights, zero biases, in the library's layout
    (w[cout][9][max(cin,16)] then b[cout] per layer, then the 1x1 head)."""
    convs = [(1, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 64), (64, 64), (128, 64), (64, 64),
             (96, 32), (32, 32), (48, 16), (16, 16)]
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co in convs:
        w = np.zeros((co, 9, max(ci, 16)), np.float32)
        w[:, :, :ci] = rng.standard_normal((co, 9, ci)) * math.sqrt(2.0 / (9 * ci))
        parts += [w.ravel(), np.zeros(co, np.float32)]
    parts += [(rng.standard_normal(16) * math.sqrt(1.0 / 16)).astype(np.float32), np.zeros(1, np.float32)]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == n_params
    return p


def augment(b, p, g):
    """The same random symmetry of the periodic problem applied to a batch of
    (b, p) pairs: a cyclic shift, one of the 8 rotations / reflections of the
    square grid, and a sign (the pressure equation is linear in b and
    commutes with all of them)."""
    import torch
    r = torch.randint(0, 1 << 30, (5,), generator=g).tolist()
    h, w = b.shape[-2:]
    sh = (r[0] % h, r[1] % w)
    b, p = torch.roll(b, sh, (-2, -1)), torch.roll(p, sh, (-2, -1))
    if h == w and r[2] % 4:
        b, p = torch.rot90(b, r[2] % 4, (-2, -1)), torch.rot90(p, r[2] % 4, (-2, -1))
    if r[3] % 2:
        b, p = torch.flip(b, (-1,)), torch.flip(p, (-1,))
    if r[4] % 2:
        b, p = -b, -p
    return b.contiguous(), p.contiguous()


def train(B, P, epochs=4, batch=16, lr=1e-3, lr_min=1e-5, seed=0, holdout=0.05, log=print):
    """Adam on MSE(net(b), p / kappa), kappa the rms of the targets, with
    symmetry augmentation; a held-out share of the pairs gives the validation
    loss. kappa is folded into the linear head afterwards. Returns (params,
    history)."""
    import torch
    n, h, w = B.shape
    nval = int(n * holdout)
    ntr = n - nval
    net = fluid.UNet(batch * h * w)
    net.set_params(init_params(net.n_params, seed))
    kappa = float(torch.sqrt((P[:ntr].double() ** 2).mean()))
    g = torch.Generator(device="cpu").manual_seed(seed)
    steps = epochs * (ntr // batch)
    hist, val, t0, k = [], [], time.time(), 0

    def validate():
        if nval < batch:
            return None
        tot = 0.0
        for i in range(nval // batch):
            sl = slice(ntr + i * batch, ntr + (i + 1) * batch)
            tot += net.forward_backward(B[sl].contiguous(), (P[sl] / kappa).contiguous())  # gradients unused
        return tot / (nval // batch)

    for ep in range(epochs):
        perm = torch.randperm(ntr, generator=g)
        run = 0.0
        for i in range(ntr // batch):
            idx = perm[i * batch:(i + 1) * batch].cuda()
            lr_k = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * k / steps))
            bb, pp = augment(B[idx], P[idx] / kappa, g)
            loss = net.forward_backward(bb, pp)
            net.adam_step(lr_k)
            run += loss
            k += 1
        hist.append(run / (ntr // batch))
        val.append(validate())
        log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.5f}, held-out {val[-1]} ({time.time() - t0:.1f} s)")
    params = net.params()
    head = params.size - 17
    params[head:] *= kappa  # head is linear: predict p / rms(b) directly
    return params, {"loss": hist, "val_loss": val, "kappa": kappa, "seconds": time.time() - t0, "steps": k,
                    "batch": batch, "train_pairs": ntr, "held_out_pairs": nval}


def save(path, params, meta):
    np.savez_compressed(path, params=params, meta=json.dumps(meta))


def load(path):
    z = np.load(path)
    return z["params"], json.loads(str(z["meta"]))


DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet_vortex256.npz")


def load_default():
    """The shipped network: trained on 20k pairs of the 256x256 vortex workload
    by this module's `train` (the command is in the metadata)."""
    return load(DEFAULT_WEIGHTS)


def eval_states(size, seeds, steps, dt=0.1, tol=1e-5, cap=2_000_000, check_every=200):
    """Velocity states at steps 0 .. steps-1 of each seed's simulation, from a
    refined-float32 session with the reference's previous-pressure start, and
    that start's sweeps and wall time per step (steps >= 1)."""
    import torch
    states, sweeps, ms = [], [], []
    for seed in seeds:
        vp = synthetic.vortex_field(size, size, seed)
        zeros = np.zeros_like(vp)
        with fluid.Session(size, size, dt=dt, diffuse_iters=2, max_iters=cap, tol=tol, check_every=check_every,
                           precision=fluid.PREC_F32R) as s:
            s.upload(vp, zeros)
            for k in range(steps):
                states.append(vp.copy())
                if steps == 1:
                    break  # one state per seed: nothing to step for
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s.step(1)
                s.sync()
                if k > 0:
                    ms.append(1e3 * (time.perf_counter() - t0))
                    sweeps.append(s.stats()["sweeps"])
                s.download(vp)
    prev = {"mean_sweeps": float(np.mean(sweeps)) if sweeps else None,
            "mean_ms_per_step": float(np.mean(ms)) if ms else None, "sweeps": sweeps}
    return states, prev


def _measure(size, states, dt, tol, cap, check_every, mode, net=None, coarsen=1, passes=1):
    import torch
    sweeps, ms, kinds, rel0, spasses = [], [], [], [], []
    zeros = np.zeros_like(states[0])
    with fluid.Session(size, size, dt=dt, diffuse_iters=2, max_iters=cap, tol=tol, check_every=check_every,
                       precision=fluid.PREC_F32R) as s:
        s.set_start(mode, net, coarsen, passes)
        for k, vp in enumerate([states[0]] + states):  # the first run warms up (lazy set-up), not recorded
            s.upload(vp, zeros)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.step(1)
            s.sync()
            dt_ms = 1e3 * (time.perf_counter() - t0)
            if k == 0:
                continue
            st = s.stats()
            if st["capped"]:
                raise RuntimeError(f"start mode {mode} hit the cap of {cap} sweeps at {size}x{size}")
            ms.append(dt_ms)
            sweeps.append(st["sweeps"])
            kinds.append(st["start_kind"])
            rel0.append(st["rel_start"])
            spasses.append(st["start_passes"])
    return {"mean_sweeps": float(np.mean(sweeps)), "mean_ms_per_step": float(np.mean(ms)),
            "cell_updates_per_s": size * size / (np.mean(ms) / 1e3), "sweeps": sweeps, "ms": ms,
            "start_kinds": kinds, "rel_start": rel0, "start_passes": spasses}


def evaluate(params, size, seeds, steps=3, dt=0.1, tol=1e-5, cap=4_000_000, check_every=200, starts=((1, 1),),
             log=print):
    """Sweeps and wall time of one step to the residual tol from each state
    (eval_states), zero start against network starts (coarsening, passes),
    in the refined-float32 form (the float32 pressure cannot represent these
    solutions to 1e-5). Each measured step starts from an uploaded state with
    zero pressure, so a network start that falls back continues from zero.
    sweeps_saved counts the damped passes of a network start as sweeps."""
    states, prev = eval_states(size, seeds, steps, dt, tol, cap, check_every)
    out = {"size": size, "tol": tol, "check_every": check_every, "states": len(states), "previous": prev}
    z = out["zero"] = _measure(size, states, dt, tol, cap, check_every, fluid.START_ZERO)
    log(f"{size}x{size} zero: {z['mean_sweeps']:.0f} sweeps/step, {z['mean_ms_per_step']:.2f} ms/step")
    out["network"] = {}
    for coarsen, passes in starts:
        net = fluid.UNet((size // coarsen) ** 2)
        net.set_params(params)
        n = _measure(size, states, dt, tol, cap, check_every, fluid.START_NETWORK, net, coarsen, passes)
        net.close()
        n["coarsen"], n["passes"] = coarsen, passes
        n["sweeps_saved"] = 1.0 - (n["mean_sweeps"] + np.mean(n["start_passes"])) / z["mean_sweeps"]
        n["time_ratio"] = n["mean_ms_per_step"] / z["mean_ms_per_step"]
        n["fallbacks"] = int(sum(k == fluid.START_FALLBACK for k in n["start_kinds"]))
        out["network"][f"coarsen{coarsen}_passes{passes}"] = n
        log(f"{size}x{size} network (coarsen {coarsen}, passes {passes}): {n['mean_sweeps']:.0f} sweeps/step, "
            f"{n['mean_ms_per_step']:.2f} ms/step, saved {n['sweeps_saved']:.3f}, time ratio {n['time_ratio']:.3f}, "
            f"fallbacks {n['fallbacks']}, rel_start {np.mean(n['rel_start']):.3g}")
    return out


# Multiply-adds x 2 per pixel of the network's forward pass, from the layer table
# (3x3 convolutions with the input channels padded to 16, the 1x1 head).
_LAYERS = [(1, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (64, 64, 3), (64, 64, 3),
           (128, 64, 2), (64, 64, 2), (96, 32, 1), (32, 32, 1), (48, 16, 0), (16, 16, 0)]
FORWARD_FLOP_PER_PIXEL = sum(2 * 9 * max(ci, 16) * co / 4 ** lv for ci, co, lv in _LAYERS) + 2 * 16


def bench_network(size=256, batch=16, reps=20, log=print):
    """Time a training step (forward + backward + Adam) on `batch` random
    smooth pairs at size x size and a prediction at size x size; report
    algorithmic TFLOP/s (forward FORWARD_FLOP_PER_PIXEL per pixel, backward
    twice that)."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(0)
    b = torch.randn(batch, size, size, generator=g).cuda()
    p = torch.randn(batch, size, size, generator=g).cuda()
    net = fluid.UNet(batch * size * size)
    net.set_params(init_params(net.n_params))
    out = torch.empty(size, size, device="cuda")
    train = True
    for _ in range(3):
        if train:
            net.forward_backward(b, p)
            net.adam_step(1e-4)
        net.predict(b[0], out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    train_ms = None
    if train:
        e0.record()
        for _ in range(reps):
            net.forward_backward(b, p)
            net.adam_step(1e-4)
        e1.record()
        torch.cuda.synchronize()
        train_ms = e0.elapsed_time(e1) / reps
    e0.record()
    for _ in range(reps):
        net.predict(b[0], out)
    e1.record()
    torch.cuda.synchronize()
    pred_ms = e0.elapsed_time(e1) / reps
    px = batch * size * size
    r = {"size": size, "batch": batch, "forward_flop_per_pixel": FORWARD_FLOP_PER_PIXEL,
         "train_step_ms": train_ms,
         "train_tflops": 3 * FORWARD_FLOP_PER_PIXEL * px / (train_ms / 1e3) / 1e12 if train_ms else None,
         "predict_ms": pred_ms, "predict_tflops": FORWARD_FLOP_PER_PIXEL * size * size / (pred_ms / 1e3) / 1e12}
    log(json.dumps(r))
    return r


def summary(r):
    return {"size": r["size"], "zero_sweeps": r["zero"]["mean_sweeps"],
            **{k: {kk: v[kk] for kk in ("mean_sweeps", "sweeps_saved", "time_ratio", "fallbacks")}
               for k, v in r["network"].items()}}


def _starts(spec):
    """'1x1,4x2' -> ((1, 1), (4, 2)): coarsening x passes."""
    return tuple(tuple(int(x) for x in item.split("x")) for item in spec.split(","))


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=20000)
    t.add_argument("--epochs", type=int, default=4)
    t.add_argument("--batch", type=int, default=16)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--out", required=True)
    t.add_argument("--eval-seeds", type=int, default=4)
    t.add_argument("--eval-steps", type=int, default=3)
    t.add_argument("--eval-sizes", type=int, nargs="*", default=[256])
    t.add_argument("--eval-starts", default="1x1", help="network starts to evaluate: coarsening x passes, ...")
    nb = sub.add_parser("bench-net", help="time the network's training step and prediction")
    nb.add_argument("--size", type=int, default=256)
    nb.add_argument("--batch", type=int, default=16)
    nb.add_argument("--reps", type=int, default=20)
    x = sub.add_parser("export", help="write the shipped parameters as raw little-endian float32")
    x.add_argument("--weights", default=DEFAULT_WEIGHTS)
    x.add_argument("--out", required=True)
    e = sub.add_parser("eval")
    e.add_argument("--weights", required=True)
    e.add_argument("--size", type=int, default=256)
    e.add_argument("--seeds", type=int, default=4)
    e.add_argument("--steps", type=int, default=3)
    e.add_argument("--check-every", type=int, default=200)
    e.add_argument("--starts", default="1x1", help="network starts: coarsening x passes, comma-separated")
    a = ap.parse_args()
    if a.cmd == "train":
        B, P, gen = make_pairs(a.pairs)
        params, hist = train(B, P, epochs=a.epochs, batch=a.batch, lr=a.lr)
        meta = {"pairs": int(B.shape[0]), "size": SIZE, "generation": gen, "training": hist,
                "workload": "8 seeded Gaussian vortices (radius 8-32 cells), dt 0.1, residual 1e-5, "
                            "4 steps per member, seeds from 10000"}
        del B, P
        save(a.out, params, meta)
        print(json.dumps(meta))
        for size in a.eval_sizes:
            r = evaluate(params, size, list(range(a.eval_seeds)), steps=a.eval_steps,
                         check_every=200 if size <= 256 else 500,
                         starts=[st for st in _starts(a.eval_starts) if (size // st[0]) % 128 == 0])
            meta[f"eval_{size}"] = r
            save(a.out, params, meta)
            print(json.dumps(summary(r)))
    elif a.cmd == "bench-net":
        bench_network(a.size, a.batch, a.reps)
    elif a.cmd == "export":
        params, _ = load(a.weights)
        params.astype("<f4").tofile(a.out)
        print(f"{params.size} parameters -> {a.out}")
    else:
        params, _ = load(a.weights)
        r = evaluate(params, a.size, list(range(a.seeds)), steps=a.steps, check_every=a.check_every,
                     starts=_starts(a.starts))
        print(json.dumps(summary(r)))


if __name__ == "__main__":
    main()
