"""Learned-preconditioned LSM on the 2-D dynamic eikonal workload.

Operator: Kirchhoff, ``mode='eikonal'``, ``dynamic=True``, float32;
v(z) = 1500 + 0.6 z m/s on a 256 (z) x 512 (x) grid at 5 m; nt = 1201 at
2 ms with a 15 Hz Ricker; 48 sources and 256 receivers evenly spread on the
surface.  A 4-level, 32-channel BF16 U-Net is trained on pairs
``(K^H K m, m)`` from seeded random models (3-15 dipping layers, 0-3 faults,
spikes at density U[1e-4, 1e-3]) and evaluated on held-out models: LSQR
iterations and wall time to a 1e-2 relative data residual, and model error,
for plain LSQR and the learned variants.

``python -m pylops_gb300.learned.experiment --train 4096 --test 64`` prints
one JSON document.
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np

from .lsm import (LearnedLSM, illumination_diagonal, make_pairs, make_residual_pairs, point_spread_functions,
                  random_reflectivity, train)
from .unet import UNet

__all__ = ["lsm_operator", "run"]


def lsm_operator(dtype: str = "float32", nz: int = 256, nx: int = 512, ns: int = 48, nr: int = 256, nt: int = 1201):
    from ..utils.wavelets import ricker
    from ..waveeqprocessing import Kirchhoff

    dz = dx = 5.0
    dt = 0.002
    z = np.arange(nz) * dz
    x = np.arange(nx) * dx
    t = np.arange(nt) * dt
    vel = 1500.0 + 0.6 * np.broadcast_to(z[None, :], (nx, nz))
    srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.zeros(ns)))
    recs = np.vstack((np.linspace(x[0], x[-1], nr), np.zeros(nr)))
    wav, _, wc = ricker(t[:41], f0=15)
    return Kirchhoff(z, x, t, srcs, recs, np.ascontiguousarray(vel), wav, wc, mode="eikonal", dynamic=True,
                     dtype=dtype)


def _summary(infos, errs):
    its = np.array([i.iterations for i in infos], dtype=float)
    secs = np.array([i.seconds for i in infos])
    res = np.array([i.residual for i in infos])
    return {
        "iterations_median": float(np.median(its)), "iterations_mean": float(its.mean()),
        "operator_pairs_median": float(np.median([i.operator_pairs for i in infos])),
        "seconds_median": float(np.median(secs)), "seconds_mean": float(secs.mean()),
        "residual_max": float(res.max()), "converged": int(np.sum(res <= 1.0001e-2)),
        "model_error_median": float(np.median(errs)), "model_error_mean": float(np.mean(errs)),
        "network_steps_mean": float(np.mean([i.network_steps for i in infos])),
        "network_residual_median": float(np.median([i.network_residual for i in infos])),
    }


def run(n_train: int = 4096, n_test: int = 64, steps: int = 2000, batch: int = 8, lr: float = 1e-3,
        tol: float = 1e-2, niter: int = 600, seed: int = 0, levels: int = 4, base: int = 32,
        variants=("plain", "warm", "learned"), steps_net: int = 4, step_ratio: float = 0.7, log=print,
        op=None, net_state: dict = None, save_net: str = None, return_objects: bool = False,
        stage2_pairs: int = 0, stage2_steps: int = 0):
    import torch

    out = {"config": {"n_train": n_train, "n_test": n_test, "steps": steps, "batch": batch, "lr": lr,
                      "tol": tol, "niter": niter, "seed": seed, "levels": levels, "base": base}}
    t0 = time.perf_counter()
    if op is None:
        op = lsm_operator()
    out["spread_variant_ms"] = op.autotune()
    torch.cuda.synchronize()
    out["setup_seconds"] = time.perf_counter() - t0
    log(f"operator ready in {out['setup_seconds']:.1f} s")

    net = UNet(levels=levels, base=base, seed=seed)
    if net_state is not None:
        net.load_state_dict(net_state)
        log("network loaded")
    else:
        t0 = time.perf_counter()
        X, M = make_pairs(op, n_train, seed=seed)
        torch.cuda.synchronize()
        out["pairs_seconds"] = time.perf_counter() - t0
        log(f"{n_train} training pairs in {out['pairs_seconds']:.1f} s")
        t0 = time.perf_counter()
        losses = train(net, X, M, steps=steps, batch=batch, lr=lr, seed=seed, log_every=max(steps // 10, 1))
        torch.cuda.synchronize()
        out["train_seconds"] = time.perf_counter() - t0
        out["train_loss_first"] = float(np.mean(losses[:20]))
        out["train_loss_last"] = float(np.mean(losses[-20:]))
        log(f"trained {steps} steps in {out['train_seconds']:.1f} s, loss {out['train_loss_first']:.3f} -> "
            f"{out['train_loss_last']:.3f}")
        if stage2_pairs and stage2_steps:
            # second stage: residual pairs after the network's warm start, mixed
            # with the first-stage pairs, training continued at a lower rate
            t0 = time.perf_counter()
            X2, E2 = make_residual_pairs(op, net, stage2_pairs, seed=seed + 1)
            X = torch.cat([X[:stage2_pairs], X2])
            M = torch.cat([M[:stage2_pairs], E2])
            del X2, E2
            torch.cuda.synchronize()
            out["stage2_pairs_seconds"] = time.perf_counter() - t0
            t0 = time.perf_counter()
            losses2 = train(net, X, M, steps=stage2_steps, batch=batch, lr=lr / 3, seed=seed + 1,
                            log_every=max(stage2_steps // 5, 1))
            torch.cuda.synchronize()
            out["stage2_train_seconds"] = time.perf_counter() - t0
            out["stage2_loss_last"] = float(np.mean(losses2[-20:]))
            log(f"stage 2: {stage2_pairs} residual pairs in {out['stage2_pairs_seconds']:.1f} s, "
                f"{stage2_steps} steps in {out['stage2_train_seconds']:.1f} s, loss {out['stage2_loss_last']:.3f}")
        del X, M
        if save_net:
            np.savez(save_net, **net.state_dict())
    # inference time of one image (CUDA events)
    img = torch.randn(op.dims, device="cuda")
    net.forward(img)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        net.forward(img)
    e1.record()
    e1.synchronize()
    out["inference_ms"] = e0.elapsed_time(e1) / 10
    log(f"inference {out['inference_ms']:.2f} ms per image")

    # held-out models (a different seed stream)
    rng = np.random.default_rng(10_000 + seed)
    nx, nz = op.dims
    tests = [random_reflectivity(nx, nz, rng) for _ in range(n_test)]
    diag = illumination_diagonal(op)
    psf_op = None
    if "psf" in variants:
        from ..signalprocessing import NonStationaryConvolve2D

        psfx, psfz = np.arange(16, nx, 32), np.arange(16, nz, 32)
        hs = point_spread_functions(op, psfx, psfz, (31, 31))
        psf_op = NonStationaryConvolve2D(dims=(nx, nz), hs=hs, ihx=psfx, ihz=psfz, dtype="float32")
    solvers = {
        "plain": (LearnedLSM(op), False),
        "diag": (LearnedLSM(op, diag=diag), False),
        "warm": (LearnedLSM(op, net=net, steps=0), True),
        "learned": (LearnedLSM(op, net=net, steps=steps_net, step_ratio=step_ratio), True),
        "learned+diag": (LearnedLSM(op, net=net, diag=diag, steps=steps_net, step_ratio=step_ratio), True),
        "psf": (LearnedLSM(op, psf=psf_op, psf_iters=10), True),
    }
    # warm up every variant once (graph capture, workspaces)
    d = torch.empty(op.shape[0], dtype=torch.float32, device="cuda")
    res = {v: ([], []) for v in variants}
    for k, m in enumerate(tests):
        mt = torch.as_tensor(m.reshape(-1), device="cuda")
        op.apply_into(mt, d)
        mn = float(torch.linalg.norm(mt.double()))
        for v in variants:
            s, use_net = solvers[v]
            if k == 0:
                s.solve(d, tol=tol, niter=5, use_net=use_net)
            x, info = s.solve(d, tol=tol, niter=niter, use_net=use_net)
            err = float(torch.linalg.norm((x - mt).double())) / mn
            res[v][0].append(info)
            res[v][1].append(err)
        if k < 4 or k == n_test - 1:
            log(f"model {k}: " + ", ".join(
                f"{v} {res[v][0][-1].network_steps}+{res[v][0][-1].iterations} it "
                f"{res[v][0][-1].seconds * 1e3:.0f} ms err {res[v][1][-1]:.3f}"
                for v in variants))
    out["variants"] = {v: _summary(*res[v]) for v in variants}
    base_t = out["variants"].get("plain", {}).get("seconds_median")
    for v in variants:
        if base_t:
            out["variants"][v]["speedup_vs_plain_median"] = base_t / out["variants"][v]["seconds_median"]
        out["variants"][v]["gpu_launches_median"] = float(np.median([i.gpu_launches for i in res[v][0]]))
    out["network_flops_per_train_image"] = net.flops(nx, nz, training=True)
    if return_objects:
        return out, {"op": op, "net": net, "tests": tests, "solvers": solvers}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--train", type=int, default=4096)
    ap.add_argument("--test", type=int, default=64)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--niter", type=int, default=600)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--variants", default="plain,warm,learned")
    ap.add_argument("--net-steps", type=int, default=4)
    ap.add_argument("--step-ratio", type=float, default=0.7)
    ap.add_argument("--stage2-pairs", type=int, default=0)
    ap.add_argument("--stage2-steps", type=int, default=0)
    ap.add_argument("--out", default=None)
    ap.add_argument("--save-net", default=None, help="write the trained network (.npz)")
    ap.add_argument("--load-net", default=None, help="skip training, load this network (.npz)")
    a = ap.parse_args(argv)
    r = run(n_train=a.train, n_test=a.test, steps=a.steps, batch=a.batch, lr=a.lr, niter=a.niter, seed=a.seed,
            variants=tuple(a.variants.split(",")), steps_net=a.net_steps, step_ratio=a.step_ratio,
            net_state=dict(np.load(a.load_net)) if a.load_net else None, save_net=a.save_net,
            stage2_pairs=a.stage2_pairs, stage2_steps=a.stage2_steps)
    s = json.dumps(r, indent=1)
    print(s)
    if a.out:
        with open(a.out, "w") as f:
            f.write(s)


if __name__ == "__main__":
    main()
