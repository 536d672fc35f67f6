"""Kirchhoff forward+adjoint throughput on one GB300.

Workload (the headline configuration that fits one GPU): 2-D Kirchhoff,
mode='eikonal', dynamic=True, angleaperture=60 deg, float32; v(z)=1500+0.5 z
m/s plus 5 seeded Gaussian anomalies (+-200 m/s, sigma 40 m); grid nz=300,
nx=800, dz=dx=5 m; nt=1501, dt=2 ms, 15 Hz Ricker; 64 sources and 400
receivers at the surface; reflectivity of 12 random-dip layers plus sparse
spikes.  Synthetic, seeded inputs of those shapes.

A step is one forward (spreading + wavelet) and one adjoint (correlation +
gathering) over the whole data volume.  ``value`` is compulsory GB moved per
step / step time (GB/s), the metric's HBM-roofline view; ``e2e`` is the same
metric through the public API with host numpy buffers (copies inside).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``--impl reference`` times the CPU restatement of the reference's numba loop
nest (oracle/kirch_oracle.c, all host threads) over whole steps of the same
workload, with tables from the oracle's fast-marching restatement.
"""

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

WORKLOAD = "kirchhoff2d_eikonal_dynamic_300x800_64x400_nt1501"
METRIC = "Kirchhoff fwd+adj GB/s vs HBM peak"


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_workload(seed: int = 1, ricker=None):
    """The headline workload's seeded inputs.  ``ricker`` is the wavelet
    function (the package's by default; the reference arm passes the
    oracle's, so that it imports nothing from the package)."""
    if ricker is None:
        from pylops_gb300.utils.wavelets import ricker

    nz, nx, dz, dx = 300, 800, 5.0, 5.0
    nt, dt = 1501, 0.002
    ns, nr = 64, 400
    z = np.arange(nz) * dz
    x = np.arange(nx) * dx
    t = np.arange(nt) * dt
    rng = np.random.default_rng(seed)
    X, Z = np.meshgrid(x, z, indexing="ij")
    vel = 1500.0 + 0.5 * Z
    for _ in range(5):
        cx, cz = rng.uniform(x[0], x[-1]), rng.uniform(z[0] + 200, z[-1])
        amp = rng.choice([-200.0, 200.0])
        vel += amp * np.exp(-((X - cx) ** 2 + (Z - cz) ** 2) / (2 * 40.0 ** 2))
    srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.zeros(ns)))
    recs = np.vstack((np.linspace(x[0], x[-1], nr), np.zeros(nr)))
    wav, _, wc = ricker(t[:41], f0=15)
    refl = np.zeros((nx, nz))
    for _ in range(12):
        z0 = rng.uniform(20, nz - 20)
        dip = np.tan(np.deg2rad(rng.uniform(-15, 15)))
        a = rng.standard_normal()
        for ix in range(nx):
            iz = int(round(z0 + dip * (ix - nx / 2)))
            if 0 <= iz < nz:
                refl[ix, iz] += a
    spikes = rng.random((nx, nz)) < 1e-3
    refl[spikes] += rng.standard_normal(int(spikes.sum()))
    return dict(z=z, x=x, t=t, srcs=srcs, recs=recs, vel=vel, wav=wav, wc=wc, refl=refl,
                ns=ns, nr=nr, nt=nt, nz=nz, nx=nx)


def workload_config(ns, nr, nt, dt, taps):
    """The ``config`` record of the headline workload (both arms)."""
    return {"workload": WORKLOAD, "mode": "eikonal", "dynamic": True, "angleaperture_deg": 60,
            "grid": [800, 300], "spacing_m": 5.0, "ns": int(ns), "nr": int(nr), "nt": int(nt), "dt": float(dt),
            "wavelet_taps": int(taps), "l2": "inputs larger than L2 (tables 1.34 GB, data 154 MB)"}


def compulsory_bytes(ni, ns, nr, nt, s_tab=12):
    """Compulsory HBM bytes of one forward + one adjoint: each table entry,
    the model and the data read or written once per application."""
    return 2 * (s_tab * ni * (ns + nr) + 4 * ni + 4 * ns * nr * nt)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.lines = []
        self.idx = device_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [s.strip() for s in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: C restatement of the numba loop nest on the host cores
# ---------------------------------------------------------------------------
def cpu_baseline(K, m, d, target_s=10.0):
    """Time the oracle on a bounded sample of sources (all host threads) and
    scale to one full forward + adjoint.  Returns the baseline record, the
    number of sampled sources and the oracle's forward rows / adjoint image
    for that sample (for the parity check of the same run)."""
    from oracle.kirch_oracle_c import COracle, build

    build()
    C = COracle(K, _padded_wavelet(K))
    _cpu_step(C, m, d, 0, 1)  # first call: thread start-up, page faults
    # the oracle runs sources in parallel: size the sample from a call with
    # one source per host core
    k = max(1, min(K.ns, os.cpu_count() or 1))
    t0 = time.perf_counter()
    _cpu_step(C, m, d, 0, k)
    tk = time.perf_counter() - t0
    nsamp = int(max(1, min(K.ns, k * max(1, int(target_s / max(tk, 1e-3))))))
    t0 = time.perf_counter()
    yc, xc = _cpu_step(C, m, d, 0, nsamp)
    dt_s = time.perf_counter() - t0
    full_s = dt_s * K.ns / nsamp
    B = compulsory_bytes(K.ni, K.ns, K.nr, K.nt)
    res = {"value": round(B / full_s / 1e9, 4), "unit": "GB/s", "cores": os.cpu_count(), "kind": "port",
           "sample": f"{nsamp} of {K.ns} sources ({nsamp * K.nr} of {K.nsnr} traces), forward+adjoint in "
                     f"float64 with all host threads, {dt_s:.1f} s, scaled by {K.ns / nsamp:.1f} to one full step"}
    return res, nsamp, yc, xc


def _padded_wavelet(K):
    from oracle.kirchhoff_oracle import pad_wavelet

    return pad_wavelet(np.asarray(K.wav), K.wavcenter)


def _cpu_step(C, m, d, s0, s1):
    y = C.spread(m, s0, s1)
    rows = slice(s0 * C.nr, s1 * C.nr)
    yc = np.zeros_like(y)
    yc[rows] = C.conv(y[rows])
    dc = np.zeros((C.ns * C.nr, C.nt))
    dc[rows] = C.conv(np.asarray(d, np.float64).reshape(-1, C.nt)[rows], adjoint=True)
    x = C.gather(dc, s0, s1)
    return yc, x


# ---------------------------------------------------------------------------
def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return rank, ws, dist
    return 0, 1, None


def shard_sources(w, rank, world):
    """This rank's contiguous block of the workload's sources (the operator
    shards by source: its traces and tables; the image is summed over ranks)."""
    from pylops_gb300.distributed import source_shard

    s0, s1 = source_shard(w["ns"], rank, world)
    w = dict(w)
    w["srcs"] = w["srcs"][:, s0:s1]
    w["ns"] = s1 - s0
    return w


def subset_sources(w, ns):
    """Keep ns evenly spaced sources of the workload (small cases for ncu captures)."""
    if ns and ns < w["ns"]:
        idx = np.linspace(0, w["ns"] - 1, ns).round().astype(int)
        w = dict(w)
        w["srcs"] = w["srcs"][:, idx]
        w["ns"] = ns
    return w


def build_operator(w):
    from pylops_gb300.waveeqprocessing import Kirchhoff

    t0 = time.perf_counter()
    K = Kirchhoff(w["z"], w["x"], w["t"], w["srcs"], w["recs"], w["vel"], w["wav"], w["wc"], mode="eikonal",
                  dynamic=True, angleaperture=60.0, engine="cuda", dtype="float32")
    return K, time.perf_counter() - t0


def run_gpu(args):
    import torch

    from pylops_gb300 import _native

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rank, ws, dist = _dist()
    w_full = subset_sources(make_workload(), args.sources)
    w = shard_sources(w_full, rank, ws) if ws > 1 else w_full
    K, t_setup = build_operator(w)
    host_group = dist.new_group(backend="gloo") if dist else None
    L = _native.lib()
    rng = np.random.default_rng(7)
    # dense model and data (an LSQR iterate is dense; a sparse reflectivity
    # would let the forward skip zero image points)
    m_host = rng.standard_normal(K.ni).astype(np.float32)
    d_host = rng.standard_normal(K.nsnr * K.nt).astype(np.float32)
    m = torch.as_tensor(m_host, device="cuda")
    d = torch.as_tensor(d_host, device="cuda")
    y = torch.empty(K.nsnr * K.nt, dtype=torch.float32, device="cuda")
    dcorr = torch.empty_like(y)
    img = torch.empty(K.ni, dtype=torch.float32, device="cuda")
    h = K.native_handle
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def step(evs=None):
        if evs:
            evs[0].record(stream)
        _native.check(L.kgb_kirchhoff_forward(h, m.data_ptr(), y.data_ptr(), sp))
        if evs:
            evs[1].record(stream)
        _native.check(L.kgb_kirchhoff_wavelet(h, d.data_ptr(), dcorr.data_ptr(), 1, sp))
        if evs:
            evs[2].record(stream)
        _native.check(L.kgb_kirchhoff_gather(h, dcorr.data_ptr(), img.data_ptr(), sp))
        if dist:
            dist.all_reduce(img)  # the adjoint image summed over the source shards
        if evs:
            evs[3].record(stream)

    # forward-kernel variants, timed on this workload; the fastest is used
    variant_ms = {}
    for v in ((0, 1, 2, 3) if args.variant < 0 else (args.variant,)):
        K.set_spread_variant(v)
        step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            _native.check(L.kgb_kirchhoff_forward(h, m.data_ptr(), y.data_ptr(), sp))
        e1.record(stream)
        torch.cuda.synchronize()
        variant_ms[v] = e0.elapsed_time(e1) / 2
    best = min(variant_ms, key=variant_ms.get)
    K.set_spread_variant(best)
    # adjoint variants (same image bit for bit); the fastest is used
    adjoint_ms = {}
    for v in ((0, 1, 2) if args.adjoint_variant < 0 else (args.adjoint_variant,)):
        K.set_adjoint_variant(v)
        step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            _native.check(L.kgb_kirchhoff_gather(h, dcorr.data_ptr(), img.data_ptr(), sp))
        e1.record(stream)
        torch.cuda.synchronize()
        adjoint_ms[v] = e0.elapsed_time(e1) / 2
    best_adj = min(adjoint_ms, key=adjoint_ms.get)
    K.set_adjoint_variant(best_adj)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(events[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)
    fwd_ms = [e[0].elapsed_time(e[1]) for e in events]
    cor_ms = [e[1].elapsed_time(e[2]) for e in events]
    gat_ms = [e[2].elapsed_time(e[3]) for e in events]
    ms_step = total_ms / args.steps
    if dist:
        tt = torch.tensor([ms_step], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_step = float(tt.item())

    y_dev = y.cpu().numpy().astype(np.float64)

    # e2e: public API, host numpy buffers (pinned), copies inside the timed region
    if args.no_e2e:
        args.steps_e2e = 0
    m_pin = torch.empty(K.ni, dtype=torch.float32, pin_memory=True).numpy()
    d_pin = torch.empty(K.nsnr * K.nt, dtype=torch.float32, pin_memory=True).numpy()
    m_pin[:] = m_host
    d_pin[:] = d_host
    from pylops_gb300.distributed import DistributedKirchhoff

    # through the public API: this rank's operator (its image summed over the
    # ranks on the host, gloo) or the whole operator on one GPU
    Kp = DistributedKirchhoff(K, group=host_group) if dist else K
    for _ in range(max(1, args.warmup) if args.steps_e2e else 0):
        Kp.matvec(m_pin)
        Kp.rmatvec(d_pin)
    torch.cuda.synchronize()
    te = []
    xx = None
    for _ in range(args.steps_e2e):
        t0 = time.perf_counter()
        Kp.matvec(m_pin)
        xx = Kp.rmatvec(d_pin)
        te.append(time.perf_counter() - t0)
    if dist and te:
        tt = torch.tensor([statistics.median(te)], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX, group=host_group)
        te = [float(tt.item())]
    e2e_s = statistics.median(te) if te else float("nan")

    # the workload's solve: 30 plain LSQR iterations on the data of its
    # reflectivity, float64 reductions and scalars on the device (one graph launch)
    lsqr_rec = None
    if not args.sources and args.lsqr_iters > 0:
        from pylops_gb300.distributed import lsqr as dist_lsqr
        from pylops_gb300.optimization.cls_basic import LSQR

        refl = torch.as_tensor(np.asarray(w["refl"], np.float32).reshape(-1), device="cuda")
        dl = torch.empty(K.nsnr * K.nt, dtype=torch.float32, device="cuda")
        K.apply_into(refl, dl)
        if dist:
            # source-sharded LSQR: one float64 all-reduce per data-space norm,
            # one image all-reduce per adjoint (NCCL)
            Dk = DistributedKirchhoff(K)
            dist_lsqr(Dk, dl, niter=2, atol=0.0, btol=0.0)
            torch.cuda.synchronize()
            dist.barrier()
            tl = time.perf_counter()
            lo = dist_lsqr(Dk, dl, niter=args.lsqr_iters, atol=0.0, btol=0.0)
        else:
            LSQR(K).solve(dl, niter=2, atol=0.0, btol=0.0, calc_var=False)  # capture and workspaces
            torch.cuda.synchronize()
            tl = time.perf_counter()
            lo = LSQR(K).solve(dl, niter=args.lsqr_iters, atol=0.0, btol=0.0, calc_var=False)
        torch.cuda.synchronize()
        t_lsqr = time.perf_counter() - tl
        xl = lo[0]
        dnorm2 = float(torch.linalg.norm(dl.double())) ** 2
        if dist:
            tt = torch.tensor([dnorm2], dtype=torch.float64, device="cuda")
            dist.all_reduce(tt)
            dnorm2 = float(tt.item())
        lsqr_rec = {"iterations": int(lo[2]), "seconds": round(t_lsqr, 4),
                    "ms_per_iteration": round(t_lsqr / max(int(lo[2]), 1) * 1e3, 3),
                    "r1norm_relative": round(float(lo[3]) / np.sqrt(dnorm2), 6),
                    "model_error_relative": round(float(torch.linalg.norm((xl - refl).double()) /
                                                        torch.linalg.norm(refl.double())), 5),
                    "note": ("source-sharded LSQR over %d GPUs (float64 scalars, NCCL all-reduces)" % ws if dist
                             else "device LSQR (float64 dots, norms and rotations), one CUDA-graph launch")}

    # the whole workload's compulsory bytes: with ws ranks each processed
    # its shard of the sources within the (max over ranks) step time
    ns_full = w_full["ns"]
    B = compulsory_bytes(K.ni, ns_full, K.nr, K.nt)
    ngpu = ws
    value = B / (ms_step * 1e-3) / 1e9
    peaks = _peaks()
    hbm = peaks.get("hbm_gbs")
    # dominant kernel: by measured time
    kern = {"spread_fwd_wavelet": statistics.median(fwd_ms), "wavelet_correlate": statistics.median(cor_ms),
            "gather_adj": statistics.median(gat_ms)}
    top = max(kern, key=kern.get)
    tab = 12 * K.ni * (K.ns + K.nr)
    algo = {"spread_fwd_wavelet": tab + 8 * K.ni + 4 * K.nsnr * K.nt,
            "wavelet_correlate": 8 * K.nsnr * K.nt,
            "gather_adj": tab + 8 * K.ni + 4 * K.nsnr * K.nt}
    achieved = algo[top] / (kern[top] * 1e-3) / 1e9
    pairs = K.ni * K.nsnr
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "GB/s",
        "n_gpus": ngpu,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded eikonal velocity with Gaussian anomalies; dense N(0,1) model and data vectors)",
        "config": workload_config(ns_full, K.nr, K.nt, K.dt, len(K.wav)),
        "setup_s": round(t_setup, 2),
        "parallelism": (f"source-sharded over {ws} GPUs ({K.ns} sources per rank), one image all-reduce per "
                        "adjoint" if dist else "one GPU"),
        "traces_per_s": round(ns_full * K.nr / (ms_step * 1e-3), 1),
        "pair_points_per_s": float(f"{2 * K.ni * ns_full * K.nr / (ms_step * 1e-3):.4e}"),
        "hbm_fraction": round(value / hbm, 5) if hbm else None,
        "pair_rate_fraction": _pair_rate(2 * pairs / (ms_step * 1e-3),
                                         {"spread_fwd_wavelet": pairs / (kern["spread_fwd_wavelet"] * 1e-3),
                                          "gather_adj": pairs / (kern["gather_adj"] * 1e-3)}, clk),
        "kernels_ms": {k: round(v, 4) for k, v in kern.items()},
        "spread_variant_ms": {str(k): round(v, 3) for k, v in variant_ms.items()},
        "spread_variant": best,
        "adjoint_variant_ms": {str(k): round(v, 3) for k, v in adjoint_ms.items()},
        "adjoint_variant": best_adj,
        "spread_accumulation": {"split": bool(K.info()["spread_split"]), "max_bin_count": K.info()["max_bin_count"],
                                "note": "split: two fire-and-forget 32-bit shared atomics per contribution, "
                                        "exact while no bin receives more than 65535 contributions"},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": round(achieved, 2), "peak": hbm,
                     "unit": "GB/s", "frac": round(achieved / hbm, 5) if hbm else None,
                     "traffic": _traffic(top, WORKLOAD), "peak_source": "measured" if hbm else "fallback",
                     "note": "compulsory bytes / launch time; the kernel is issue/gather bound, not HBM bound"},
        "gpu_launches": args.steps * (K.info()["kernels_forward"] + 1 + K.info()["kernels_adjoint"] - 1),
        "clocks": clk,
        "e2e": {"value": round(B / e2e_s / 1e9, 3) if te else None, "unit": "GB/s",
                "h2d_bytes_per_step": int(4 * K.ni + 4 * K.nsnr * K.nt),
                "d2h_bytes_per_step": int(4 * K.nsnr * K.nt + 4 * K.ni),
                "ms_per_step": round(e2e_s * 1e3, 3) if te else None},
    }
    if lsqr_rec is not None:
        out["lsqr"] = lsqr_rec
    if rank == 0 and ws == 1 and not args.no_cpu_baseline and not args.sources:
        cb, nsamp, yc, xc = cpu_baseline(K, m_host.astype(np.float64), d_host, target_s=args.cpu_seconds)
        out["cpu_baseline"] = cb
        rows = nsamp * K.nr
        d_mask = d_host.copy()
        d_mask[rows * K.nt:] = 0.0
        x_mask = K.H @ d_mask
        out["parity"] = {
            "oracle": "float64 C restatement of the numba loop nest, identical tables",
            "sample_sources": nsamp,
            "forward_rel_l2": float(np.linalg.norm(y_dev[:rows * K.nt] - yc[:rows].ravel())
                                    / np.linalg.norm(yc[:rows])),
            "adjoint_rel_l2": float(np.linalg.norm(x_mask - xc) / np.linalg.norm(xc)),
        }
    if rank == 0 and ws == 1 and not args.sources and args.subrecords:
        # the other configurations, each with its own roofline and clocks
        del K, m, d, y, dcorr, img
        torch.cuda.empty_cache()
        out["subrecords"] = _subrecords(args)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def _subrecords(args):
    """Records of the 3-D workload (bf16 and float32 weights), the batched
    LSM workload and the learned-vs-plain LSM comparison, measured in the
    same run as the headline line.  A record that fails carries its error."""
    import copy

    import torch

    sub = copy.copy(args)
    sub.steps = max(1, min(args.steps, 10))
    jobs = [("kirchhoff3d_bf16_weights", lambda: kirchhoff3d_record(sub, "bfloat16")),
            ("kirchhoff3d_float32_weights", lambda: kirchhoff3d_record(sub, "float32")),
            ("batched_lsm", lambda: batch_record(sub)),
            ("learned_lsm", lambda: lsm_record(sub, args.lsm_models, ("plain", "warm", "learned"), False))]
    recs = {}
    for name, job in jobs:
        t0 = time.perf_counter()
        try:
            recs[name] = job()
        except Exception as e:  # keep the headline line; the record says what failed
            recs[name] = {"error": f"{type(e).__name__}: {e}"}
        recs[name]["wall_s"] = round(time.perf_counter() - t0, 1)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return recs




def _pair_rate(step_rate, kernel_rates, clk, instr_per_pair=15):
    """The instruction roofline of the pair-point loop: achieved pair-points/s
    over SMs x 128 FP32 lanes x SM clock / the minimum instructions per
    dynamic pair-point (15: time add, index and fraction, two weight FMAs,
    interpolation, accumulation)."""
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    peak = sms * 128 * mhz * 1e6 / instr_per_pair
    rec = {"value": round(step_rate / peak, 4), "peak_pair_points_per_s": float(f"{peak:.4e}"),
           "instr_per_pair_min": instr_per_pair, "sms": sms, "sm_mhz": mhz}
    for k, v in kernel_rates.items():
        rec[k] = round(v / peak, 4)
    return rec


def _traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` on `workload` recorded from an ncu
    capture in profiles/dram_traffic_per_launch.txt, or None."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_per_launch.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for ln in f:
            parts = ln.split()
            if len(parts) == 3 and not ln.startswith("#") and parts[0] == kernel and parts[1] == workload:
                return int(parts[2])
    return None


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def run_reference(args):
    """Reference arm: the C restatement of the reference's numba CPU engine
    (oracle/kirch_oracle.c: prange over sources in the forward, over image
    points in the adjoint, float64) on all host threads, over whole steps of
    the headline workload -- every source and receiver, no sampling or
    extrapolation.  Its tables come from the oracle's own fast-marching
    restatement (oracle/eikonal_oracle.c), so this process loads nothing
    from the package."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.kirch_oracle_c import COracle, build
    from oracle.kirchhoff_oracle import KirchhoffOracle, ricker

    build()
    w = make_workload(ricker=ricker)
    t0 = time.perf_counter()
    K = KirchhoffOracle(w["z"], w["x"], w["t"], w["srcs"], w["recs"], w["vel"], w["wav"], w["wc"],
                        mode="eikonal", dynamic=True, angleaperture=60.0)
    C = COracle(K, K.h)
    t_setup = time.perf_counter() - t0
    rng = np.random.default_rng(7)
    m = rng.standard_normal(K.ni)
    d = rng.standard_normal(K.ns * K.nr * K.nt)
    for _ in range(args.warmup):
        C.matvec(m)
        C.rmatvec(d)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        C.matvec(m)
        C.rmatvec(d)
    total = time.perf_counter() - t0
    ms_step = total / max(args.steps, 1) * 1e3
    B = compulsory_bytes(K.ni, K.ns, K.nr, K.nt)
    v = B / (ms_step * 1e-3) / 1e9
    cores = os.cpu_count()
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded eikonal velocity with Gaussian anomalies; dense N(0,1) model and data vectors)",
        "config": workload_config(K.ns, K.nr, K.nt, K.dt, len(w["wav"])),
        "setup_s": round(t_setup, 2),
        "cpu_baseline": {"value": round(v, 4), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"whole steps: forward (spreading + wavelet) and adjoint (correlation + "
                                   f"gathering) over all {K.ns} x {K.nr} traces, float64, {cores} threads; "
                                   f"{args.steps} timed steps in {total:.1f} s"},
        "e2e": {"value": round(v, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "package_modules_loaded": sorted(k for k in sys.modules if k.split(".")[0] == "pylops_gb300"),
    }))


def run_batch(args):
    print(json.dumps(batch_record(args)))


def batch_record(args):
    """Batched LSM workload (256 independent 2-D kinematic problems of random
    size, 20 CGLS iterations each, one CUDA-graph launch).  A step is one
    batched CGLS solve; value = compulsory GB/s of its 2*20+2 operator
    applications."""
    import torch

    from pylops_gb300.waveeqprocessing.batch import build_batch, random_problems

    t0 = time.perf_counter()
    probs = random_problems(args.batch_problems, seed=3)
    B = build_batch(probs)
    tune = B.autotune(candidates=(2, 4, 8), reps=2)  # forward tile and adjoint shape
    t_setup = time.perf_counter() - t0
    y = torch.cat([torch.as_tensor(K @ p["refl"].ravel().astype(np.float32), device="cuda")
                   for K, p in zip(B.ops, probs)])
    for _ in range(args.warmup):
        B.cgls(y, niter=args.cgls_iters, tol=0.0)
    torch.cuda.synchronize()
    ts = []
    clocks = ClockSampler()
    clocks.start()
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, iiter, kold, cost = B.cgls(y, niter=args.cgls_iters, tol=0.0)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    clk = clocks.stop()
    step = statistics.median(ts)
    napply = 2 * args.cgls_iters + 2
    Bytes = sum(compulsory_bytes(K.ni, K.ns, K.nr, K.nt, s_tab=4) for K in B.ops) / 2 * napply
    rels = [float(c[-1] / c[0]) for c in cost]
    hbm = _peaks().get("hbm_gbs")
    gbs = Bytes / step / 1e9
    return {
        "metric": "batched LSM (CGLS) GB/s and problems/s", "value": round(Bytes / step / 1e9, 3), "unit": "GB/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched_lsm_256x2d_kinematic_nt501", "problems": len(B.ops),
                   "cgls_iterations": args.cgls_iters, "model_total": B.shape[1], "data_total": B.shape[0],
                   "tile_ms": {str(k): round(v, 3) for k, v in tune.items()}, "tile": B.tile,
                   "gather_shape": {"receivers_in_registers": B.gather_shape[0],
                                    "points_per_thread": B.gather_shape[1]},
                   "setup_s": round(t_setup, 2)},
        "problems_per_s": round(len(B.ops) / step, 2),
        "residual_reduction_median": round(float(np.median(rels)), 5),
        "roofline": {"bound": "hbm", "kernel": "batched CGLS iteration (spread, correlation, gather, vector kernels)",
                     "achieved": round(gbs, 2), "peak": hbm, "unit": "GB/s",
                     "frac": round(gbs / hbm, 5) if hbm else None, "traffic": None,
                     "note": "compulsory bytes of the 2 n + 2 operator applications / solve time"},
        "clocks": clk,
    }


def run_single(args):
    """Single traveltime table workload (mode='byot' with trav of shape
    (ni, ns*nr)): the 300 x 800 grid at 5 m with v(z) = 1500 + 0.5 z,
    64 sources x 100 receivers at the surface (6400 traces), nt = 1501 at
    2 ms, 15 Hz Ricker; a 6.1 GB table in HBM.  A step is one forward and one
    adjoint; value = compulsory GB/s (4 bytes per table entry, model and data
    once per application).  The table is read once per application, so this
    is the HBM-bound mode of the operator."""
    import torch

    from oracle.kirchhoff_oracle import conv_same, pad_wavelet, single_table_index, trav_matvec
    from pylops_gb300.utils.wavelets import ricker
    from pylops_gb300.waveeqprocessing import Kirchhoff

    nz, nx, nt, dt = 300, 800, 1501, 0.002
    ns, nr = 64, args.single_receivers
    # the float64 host table is 8 * ni * ns * nr bytes: keep it within a third of free memory
    try:
        free = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_AVPHYS_PAGES")
    except (ValueError, OSError):
        free = 0
    while free and nr > 8 and 3 * 8 * nx * nz * ns * nr > free:
        nr //= 2
    z, x, t = np.arange(nz) * 5.0, np.arange(nx) * 5.0, np.arange(nt) * dt
    srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.zeros(ns)))
    recs = np.vstack((np.linspace(x[0], x[-1], nr), np.zeros(nr)))
    X, Z = np.meshgrid(x, z, indexing="ij")
    v = (1500.0 + 0.5 * Z).ravel()
    t0 = time.perf_counter()
    ts = np.sqrt((X.ravel()[:, None] - srcs[0][None]) ** 2 + Z.ravel()[:, None] ** 2) / v[:, None]
    tr = np.sqrt((X.ravel()[:, None] - recs[0][None]) ** 2 + Z.ravel()[:, None] ** 2) / v[:, None]
    table = (ts[:, :, None] + tr[:, None, :]).reshape(nx * nz, ns * nr)
    wav, _, wc = ricker(t[:41], f0=15)
    K = Kirchhoff(z, x, t, srcs, recs, 1500.0, wav, wc, mode="byot", trav=table, engine="cuda", dtype="float32")
    K.native_handle
    t_setup = time.perf_counter() - t0
    variant_ms = K.autotune()
    g = torch.Generator(device="cuda").manual_seed(0)
    m = torch.randn(K.ni, device="cuda", generator=g)
    d = torch.randn(K.shape[0], device="cuda", generator=g)
    y = torch.empty_like(d)
    img = torch.empty_like(m)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        K.apply_into(m, y)
        K.apply_into(d, img, adjoint=True)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for a, b, c in ev:
        a.record(stream)
        K.apply_into(m, y)
        b.record(stream)
        K.apply_into(d, img, adjoint=True)
        c.record(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    step = e0.elapsed_time(e1) / 1e3 / args.steps
    fwd_ms = statistics.median(a.elapsed_time(b) for a, b, _ in ev)
    adj_ms = statistics.median(b.elapsed_time(c) for _, b, c in ev)
    B = 2 * (4 * K.ni * K.nsnr + 4 * K.ni + 4 * K.nsnr * K.nt)
    table_bytes = 4 * K.ni * K.nsnr
    peaks = _peaks()
    # the gather (adjoint) streams the table once: its bytes / its time
    ach = (table_bytes + 4 * K.ni + 8 * K.nsnr * K.nt) / (adj_ms / 1e3) / 1e9
    # end to end with host buffers
    mh, dh = m.cpu().numpy(), d.cpu().numpy()
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.steps):
        _ = K @ mh
        _ = K.H @ dh
    e2e = (time.perf_counter() - te) / args.steps
    line = {
        "metric": "Kirchhoff single-table fwd+adj GB/s vs HBM peak", "value": round(B / step / 1e9, 2),
        "unit": "GB/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(step * 1e3, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "single_table_2d_300x800_64x%d_nt1501" % nr, "table_gb": round(table_bytes / 1e9, 3),
                   "l2": "table larger than L2", "setup_s": round(t_setup, 1)},
        "kernel_ms": {"forward": round(fwd_ms, 3), "adjoint": round(adj_ms, 3)},
        "spread_variant_ms": {str(k): round(v, 3) for k, v in variant_ms.items()},
        "spread_variant": K.info()["spread_variant"],
        "hbm_fraction": round(B / step / 1e9 / peaks["hbm_gbs"], 4),
        "roofline": {"bound": "hbm", "kernel": "gather1 (adjoint)", "achieved": round(ach, 1),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": round(ach / peaks["hbm_gbs"], 4),
                     "traffic": _traffic("gather1_adjoint", "single_table_2d_300x800_64x%d_nt1501" % nr)},
        "e2e": {"value": round(B / e2e / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": 4 * (K.ni + K.shape[0]),
                "d2h_bytes_per_step": 4 * (K.ni + K.shape[0])},
        "gpu_launches": args.steps * (K.info()["kernels_forward"] + K.info()["kernels_adjoint"]),
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        ntr = 32
        it, w = single_table_index(table[:, :ntr], dt)
        tc = time.perf_counter()
        trav_matvec(mh.astype(np.float64), ntr, nt, K.ni, it, w)
        tcs = time.perf_counter() - tc
        per_step = 2 * tcs * K.nsnr / ntr
        line["cpu_baseline"] = {"value": round(B / per_step / 1e9, 4), "unit": "GB/s", "cores": 1, "kind": "port",
                                "sample": f"NumPy oracle forward spreading of {ntr} of {K.nsnr} traces, "
                                          f"{tcs:.1f} s, x2 for the adjoint, scaled to one step"}
    print(json.dumps(line))


def run_unet(args):
    """U-Net training throughput: the 4-level, 32-channel BF16 network of the
    learned preconditioner on batches of 8 images of 512 x 256 (the learned-LSM
    image size), random inputs and targets.  A step is one training step
    (forward, MSE, backward, Adam).  value = algorithmic TFLOP/s of the
    convolutions (forward + weight and data gradients, 2 flops per MAC)."""
    import torch

    from pylops_gb300.learned.unet import UNet

    B, H, W = 8, 512, 256
    net = UNet(levels=4, base=32, seed=0)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(B, H, W, device="cuda", generator=g)
    t = torch.randn(B, H, W, device="cuda", generator=g)
    for _ in range(args.warmup):
        net.train_step(x, t)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    clocks = ClockSampler()
    clocks.start()
    l0 = net.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        net.train_step(x, t)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = net.launches - l0
    step = e0.elapsed_time(e1) / 1e3 / args.steps
    flops = net.flops(H, W, training=True) * B
    # inference of one image (the solve's use)
    xi = x[:1]
    net.forward(xi)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(20):
        net.forward(xi)
    e1.record(stream)
    torch.cuda.synchronize()
    inf_ms = e0.elapsed_time(e1) / 20
    # end to end: host batch in, loss out
    xh, th = x.cpu().numpy(), t.cpu().numpy()
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.steps):
        xd = torch.from_numpy(xh).pin_memory().to("cuda", non_blocking=True)
        td = torch.from_numpy(th).pin_memory().to("cuda", non_blocking=True)
        float(net.train_step(xd, td))
    e2e = (time.perf_counter() - te) / args.steps
    peaks = _peaks()
    peak = peaks.get("bf16_tflops_sustained") or 1700.0
    ach = flops / step / 1e12
    print(json.dumps({
        "metric": "U-Net (learned preconditioner) training TFLOP/s", "value": round(ach, 2), "unit": "TFLOP/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": "unet4x32_train_batch8_512x256", "flops_per_step": flops,
                   "l2": "activations and unfold buffers larger than L2"},
        "images_per_s": round(B / step, 1), "inference_ms_per_image": round(inf_ms, 3),
        "roofline": {"bound": "tensor", "kernel": "training step (tcgen05 implicit convolutions, weight-gradient GEMMs and helper kernels)",
                     "achieved": round(ach, 2), "peak": peak, "unit": "TFLOP/s", "frac": round(ach / peak, 4),
                     "traffic": None},
        "e2e": {"value": round(flops / e2e / 1e12, 2), "unit": "TFLOP/s", "h2d_bytes_per_step": 2 * x.numel() * 4,
                "d2h_bytes_per_step": 8},
        "gpu_launches": launches, "clocks": clk,
    }))


def run_conv(args):
    """One implicit 3x3 convolution of the U-Net through the C-ABI, on seeded
    bf16 NHWC operands: --conv B,H,W,C,N,flip.  --conv-kind fwd: the
    convolution (flip = 1: its transposed form, the data gradient;
    kgb_conv3x3_bf16, bf16 output, bias-free with ReLU); wgrad: the weight
    gradient (kgb_unet_row_transpose of x and g, then
    kgb_conv3x3_wgrad_bf16).  A step is one such call (with its transposes).
    value = algorithmic TFLOP/s, 2 B H W N 9 C flops per step.  Small cases
    of the network's layers for ncu captures of one kernel."""
    import torch

    from pylops_gb300 import _native

    B, H, W, C, N, flip = (int(v) for v in args.conv.split(","))
    P = B * H * W
    Cp = (C + 63) // 64 * 64
    g = torch.Generator(device="cuda").manual_seed(0)
    L, s = _native.lib(), torch.cuda.current_stream().cuda_stream
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    x = torch.randn(P * C, device="cuda", generator=g).to(torch.bfloat16)
    if args.conv_kind == "fwd":
        w = torch.randn(N * 9 * Cp, device="cuda", generator=g).to(torch.bfloat16)
        y = torch.empty(P * N, dtype=torch.bfloat16, device="cuda")

        def step():
            _native.check(L.kgb_conv3x3_bf16(x.data_ptr(), w.data_ptr(), y.data_ptr(), B, H, W, C, N, flip, None, 3,
                                             err.data_ptr(), s))

        launches, kernel = 1, "conv_halo_kernel / gemm_tn_kernel (implicit convolution)"
    else:
        gy = torch.randn(P * N, device="cuda", generator=g).to(torch.bfloat16)
        xT3 = torch.empty(3 * P * C, dtype=torch.bfloat16, device="cuda")
        gTr = torch.empty(P * N, dtype=torch.bfloat16, device="cuda")
        dW = torch.empty(N * 9 * C, device="cuda")
        work = torch.empty(1 << 23, device="cuda")

        def step():
            _native.check(L.kgb_unet_row_transpose(x.data_ptr(), xT3.data_ptr(), B, H, W, C, 3, s))
            _native.check(L.kgb_unet_row_transpose(gy.data_ptr(), gTr.data_ptr(), B, H, W, N, 1, s))
            _native.check(L.kgb_conv3x3_wgrad_bf16(xT3.data_ptr(), gTr.data_ptr(), dW.data_ptr(), B, H, W, C, N,
                                                   9 * C, work.data_ptr(), work.numel(), err.data_ptr(), s))

        launches, kernel = 4, "gemm_tn_kernel (implicit weight gradient) with its row transposes and slice sum"
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    flops = 2.0 * P * N * 9 * C
    peak = _peaks().get("bf16_tflops") or 1900.0
    ach = flops / (ms * 1e-3) / 1e12
    print(json.dumps({
        "metric": "implicit 3x3 convolution TFLOP/s", "value": round(ach, 2), "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": "conv3x3_%s_b%d_%dx%d_c%d_n%d_flip%d" % (args.conv_kind, B, H, W, C, N, flip)},
        "roofline": {"bound": "tensor", "kernel": kernel, "achieved": round(ach, 2), "peak": peak,
                     "unit": "TFLOP/s", "frac": round(ach / peak, 4), "traffic": None},
        "gpu_launches": launches * args.steps, "device_error": int(err.item()),
    }))


def run_nsconv(args):
    """Image-domain Hessian (NonStationaryConvolve2D): a 512 x 256 image (the
    learned-LSM grid) with 41 x 41 point-spread filters on a 16 x 8 coarse
    grid.  A step is one forward and one adjoint.  value = image points per
    second (both directions); the kernels are FMA-bound gathers (each output
    point reads 41 x 41 inputs from shared memory and interpolates 4 filters)."""
    import torch

    from oracle.nsconv2d_oracle import nsconv2d
    from pylops_gb300.signalprocessing import NonStationaryConvolve2D

    nx, nz, hx = 512, 256, 41
    ihx, ihz = np.arange(16, nx, 32), np.arange(16, nz, 32)
    rng = np.random.default_rng(0)
    hs = rng.standard_normal((len(ihx), len(ihz), hx, hx)).astype(np.float32)
    C = NonStationaryConvolve2D(dims=(nx, nz), hs=hs, ihx=ihx, ihz=ihz, dtype="float32")
    x = torch.randn(nx * nz, device="cuda")
    for _ in range(args.warmup):
        C @ x
        C.H @ x
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    clocks = ClockSampler()
    clocks.start()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    fw, ad = [], []
    for _ in range(args.steps):
        e0.record(stream)
        C @ x
        e1.record(stream)
        C.H @ x
        e2.record(stream)
        torch.cuda.synchronize()
        fw.append(e0.elapsed_time(e1))
        ad.append(e1.elapsed_time(e2))
    clk = clocks.stop()
    step = (statistics.median(fw) + statistics.median(ad)) / 1e3
    xh = x.cpu().numpy()
    te = time.perf_counter()
    for _ in range(args.steps):
        C @ xh
        C.H @ xh
    e2e = (time.perf_counter() - te) / args.steps
    B = 2 * (8 * nx * nz + hs.nbytes)
    peaks = _peaks()
    line = {
        "metric": "NonStationaryConvolve2D fwd+adj image points/s", "value": round(2 * nx * nz / step, 1),
        "unit": "points/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(step * 1e3, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "nsconv2d_512x256_psf41x41_16x8", "l2": "inputs smaller than L2 (re-read per step)"},
        "kernel_ms": {"forward": round(statistics.median(fw), 4), "adjoint": round(statistics.median(ad), 4)},
        "flops_per_step": 2 * 2 * 5 * nx * nz * hx * hx,
        "roofline": {"bound": "hbm", "kernel": "nsconv2d forward", "achieved": round(B / 2 / (statistics.median(fw) / 1e3) / 1e9, 2),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(B / 2 / (statistics.median(fw) / 1e3) / 1e9 / peaks["hbm_gbs"], 5), "traffic": None,
                     "note": "FMA-bound gather; compulsory bytes are tiny"},
        "e2e": {"value": round(2 * nx * nz / e2e, 1), "unit": "points/s", "h2d_bytes_per_step": 8 * nx * nz,
                "d2h_bytes_per_step": 8 * nx * nz},
        "gpu_launches": 2 * args.steps, "clocks": clk,
    }
    if not args.no_cpu_baseline:
        rows = 8
        tc = time.perf_counter()
        nsconv2d(xh.reshape(nx, nz)[:rows + hx], hs[:2], ihx[:2], ihz, adjoint=True)
        tcs = time.perf_counter() - tc
        per = tcs / ((rows + hx) * nz)
        line["cpu_baseline"] = {"value": round(1 / per, 1), "unit": "points/s", "cores": 1, "kind": "port",
                                "sample": f"float64 NumPy oracle adjoint on {rows + hx} x {nz} points, {tcs:.1f} s"}
    print(json.dumps(line))


def run_kirchhoff3d(args):
    print(json.dumps(kirchhoff3d_record(args, args.weights)))


def kirchhoff3d_record(args, weights):
    """The 3-D workload: analytic constant velocity 2500 m/s, dynamic, 100 x 100
    x 120 grid at 10 m, 16 sources on a 4 x 4 and 400 receivers on a 20 x 20
    surface grid, nt = 1001 at 4 ms, 20 Hz Ricker, traveltimes exact and
    amplitude (weight) tables in bf16 (`--weights float32` to keep them in
    float32).  A step is one forward and one adjoint; value = compulsory GB/s
    (8-byte records: traveltime + two bf16 weights).  The line also carries 15
    device LSQR iterations and the error of both directions against the float64
    C oracle on sampled sources."""
    import torch

    from oracle.kirch_oracle_c import COracle, build
    from pylops_gb300.optimization.cls_basic import LSQR
    from pylops_gb300.utils.wavelets import ricker
    from pylops_gb300.waveeqprocessing import Kirchhoff

    ny = nx = 100
    nz = 120
    y, x, z = np.arange(ny) * 10.0, np.arange(nx) * 10.0, np.arange(nz) * 10.0
    t = np.arange(1001) * 0.004
    wav, _, wc = ricker(t[:41], f0=20)
    sy, sx = np.meshgrid(np.linspace(y[0], y[-1], 4), np.linspace(x[0], x[-1], 4), indexing="ij")
    ry, rx = np.meshgrid(np.linspace(y[0], y[-1], 20), np.linspace(x[0], x[-1], 20), indexing="ij")
    srcs = np.vstack((sy.ravel(), sx.ravel(), np.zeros(16)))
    recs = np.vstack((ry.ravel(), rx.ravel(), np.zeros(400)))
    t0 = time.perf_counter()
    K = Kirchhoff(z, x, t, srcs, recs, 2500.0, wav, wc, y=y, mode="analytic", dynamic=True, engine="cuda",
                  dtype="float32")
    K.set_weight_precision(weights)
    t_setup = time.perf_counter() - t0
    variant_ms = K.autotune()
    # reflectivity: 4 planar dipping reflectors with N(0,1) amplitudes
    rng = np.random.default_rng(4)
    refl = np.zeros((ny, nx, nz))
    Y, X = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    for _ in range(4):
        z0, dy_, dx_ = rng.uniform(20, nz - 20), rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2)
        iz = np.round(z0 + dy_ * (Y - ny / 2) + dx_ * (X - nx / 2)).astype(int)
        ok = (iz >= 0) & (iz < nz)
        refl[Y[ok], X[ok], iz[ok]] += rng.standard_normal()
    m = torch.as_tensor(refl.reshape(-1).astype(np.float32), device="cuda")
    d = torch.empty(K.shape[0], device="cuda")
    img = torch.empty(K.ni, device="cuda")
    for _ in range(args.warmup):
        K.apply_into(m, d)
        K.apply_into(d, img, adjoint=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    clocks = ClockSampler()
    clocks.start()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    fw, ad = [], []
    for _ in range(args.steps):
        e0.record(stream)
        K.apply_into(m, d)
        e1.record(stream)
        K.apply_into(d, img, adjoint=True)
        e2.record(stream)
        torch.cuda.synchronize()
        fw.append(e0.elapsed_time(e1))
        ad.append(e1.elapsed_time(e2))
    clk = clocks.stop()
    step = (statistics.median(fw) + statistics.median(ad)) / 1e3
    rec_bytes = 8 if weights == "bfloat16" else 12
    B = 2 * (rec_bytes * K.ni * (K.ns + K.nr) + 8 * K.ni + 4 * K.nsnr * K.nt)
    # 15 LSQR iterations on the device (one graph launch)
    K.apply_into(m, d)
    torch.cuda.synchronize()
    tl = time.perf_counter()
    out = LSQR(K).solve(d, niter=15, atol=0.0, btol=0.0, calc_var=False)
    torch.cuda.synchronize()
    t_lsqr = time.perf_counter() - tl
    xinv = out[0]
    # error against the float64 oracle on sampled sources
    build()
    C = COracle(K, _padded_wavelet(K))
    g = torch.Generator(device="cuda").manual_seed(1)
    mr = torch.randn(K.ni, device="cuda", generator=g)
    dr = torch.randn(K.shape[0], device="cuda", generator=g)
    yg = torch.empty_like(dr)
    K.apply_into(mr, yg)
    mh, dh = mr.cpu().numpy().astype(np.float64), dr.cpu().numpy().astype(np.float64).reshape(K.nsnr, K.nt)
    ef, ea = [], []
    for s_ in (3, 12):
        rows = slice(s_ * K.nr, (s_ + 1) * K.nr)
        yc, xc = _cpu_step(C, mh, dh, s_, s_ + 1)
        ef.append(float(np.linalg.norm(yg.view(K.nsnr, K.nt)[rows].cpu().numpy() - yc[rows]) /
                        np.linalg.norm(yc[rows])))
        dz = torch.zeros(K.nsnr, K.nt, device="cuda")
        dz[rows] = dr.view(K.nsnr, K.nt)[rows]
        xi = torch.empty(K.ni, device="cuda")
        K.apply_into(dz.view(-1), xi, adjoint=True)
        ea.append(float(np.linalg.norm(xi.cpu().numpy() - xc) / np.linalg.norm(xc)))
    peaks = _peaks()
    mh_ = m.cpu().numpy()
    te = time.perf_counter()
    for _ in range(3):
        dd = K @ mh_
        K.H @ dd
    e2e = (time.perf_counter() - te) / 3
    return {
        "metric": "Kirchhoff 3-D fwd+adj GB/s vs HBM peak", "value": round(B / step / 1e9, 2), "unit": "GB/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (weights %s)" % weights, "data": "synthetic",
        "config": {"workload": "kirchhoff3d_analytic_dynamic_100x100x120_16x400_nt1001", "weights": weights,
                   "l2": "tables larger than L2", "setup_s": round(t_setup, 1)},
        "kernel_ms": {"forward": round(statistics.median(fw), 3), "adjoint": round(statistics.median(ad), 3)},
        "spread_variant_ms": {str(k_): round(v_, 3) for k_, v_ in variant_ms.items()},
        "hbm_fraction": round(B / step / 1e9 / peaks["hbm_gbs"], 5),
        "roofline": {"bound": "hbm", "kernel": "spread" if statistics.median(fw) > statistics.median(ad) else "gather",
                     "achieved": round(B / 2 / (max(statistics.median(fw), statistics.median(ad)) / 1e3) / 1e9, 2),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(B / 2 / (max(statistics.median(fw), statistics.median(ad)) / 1e3) / 1e9 /
                                   peaks["hbm_gbs"], 5), "traffic": None},
        "lsqr_15_iterations_s": round(t_lsqr, 3), "lsqr_r1norm_relative": round(float(out[3]) / float(
            torch.linalg.norm(d.double())), 5),
        "error_vs_float64_oracle": {"forward_rel_l2": max(ef), "adjoint_rel_l2": max(ea), "sampled_sources": [3, 12]},
        "e2e": {"value": round(B / e2e / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": 4 * (K.ni + K.shape[0]),
                "d2h_bytes_per_step": 4 * (K.ni + K.shape[0])},
        "gpu_launches": args.steps * (K.info()["kernels_forward"] + K.info()["kernels_adjoint"]),
        "clocks": clk,
    }


def run_lsm(args):
    print(json.dumps(lsm_record(args, args.steps, ("plain", "warm", "learned", "psf"), not args.no_cpu_baseline)))


def lsm_record(args, n_test, variants, with_cpu):
    """Learned-preconditioned LSM workload: 2-D dynamic eikonal Kirchhoff,
    v(z) = 1500 + 0.6 z on 256 x 512 at 5 m, 48 sources, 256 receivers,
    nt = 1201 at 2 ms, 15 Hz Ricker.  The BF16 U-Net is trained on
    --lsm-train pairs that the operator generates from seeded random models;
    a step is one held-out model solved to a 1e-2 relative data residual.
    value = median wall time of the learned solve (plain GPU LSQR beside it)."""
    import torch

    from pylops_gb300.learned import experiment

    clocks = ClockSampler()
    clocks.start()
    out, ctx = experiment.run(n_train=args.lsm_train, n_test=n_test, steps=args.lsm_steps, batch=8,
                              niter=600, variants=variants,
                              stage2_pairs=args.lsm_stage2_pairs, stage2_steps=args.lsm_stage2_steps,
                              steps_net=args.lsm_net_steps,
                              log=lambda *a: print(*a, file=sys.stderr, flush=True), return_objects=True)
    clk = clocks.stop()
    op, tests = ctx["op"], ctx["tests"]
    learned, _ = ctx["solvers"]["learned"]
    v = out["variants"]
    # end to end: host data in, host model out, through LearnedLSM.solve
    e2e_s = []
    for m in tests[:min(8, len(tests))]:
        d = (op @ torch.as_tensor(m.reshape(-1), device="cuda")).cpu().numpy()
        _, info = learned.solve(d, tol=1e-2, niter=600)
        e2e_s.append(info.seconds)
    e2e = statistics.median(e2e_s)
    # tensor-core roofline of a training step (convolution GEMMs)
    step_s = out["train_seconds"] / args.lsm_steps
    achieved = out["network_flops_per_train_image"] * 8 / step_s / 1e12
    peaks = _peaks()
    peak = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops") or 1700.0
    line = {
        "metric": "LSM seconds to 1e-2 relative data residual, learned vs plain GPU LSQR",
        "value": round(v["learned"]["seconds_median"], 4), "unit": "s", "n_gpus": 1, "steps": n_test,
        "warmup": 1, "ms_per_step": round(v["learned"]["seconds_median"] * 1e3, 2), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 operator, bf16 network", "data": "synthetic",
        "config": {"workload": "learned_lsm_2d_eikonal_dyn_256x512_48x256_nt1201", "train_pairs": args.lsm_train,
                   "train_steps": args.lsm_steps, "stage2_residual_pairs": args.lsm_stage2_pairs,
                   "stage2_steps": args.lsm_stage2_steps, "max_network_directions": 1 + args.lsm_net_steps,
                   "batch": 8, "held_out_models": n_test, "tol": 1e-2,
                   "l2": "operator tables (478 MB) larger than L2"},
        "plain_lsqr": v["plain"], "warm_start_only": v["warm"], "learned": v["learned"],
        "psf_image_domain_warm_start": v.get("psf"),
        "speedup_vs_plain_median": round(v["learned"]["speedup_vs_plain_median"], 3),
        "train": {k: out.get(k) for k in ("pairs_seconds", "train_seconds", "train_loss_first", "train_loss_last",
                                          "stage2_pairs_seconds", "stage2_train_seconds", "stage2_loss_last",
                                          "inference_ms")},
        "e2e": {"value": round(e2e, 4), "unit": "s", "h2d_bytes_per_step": int(op.shape[0] * 4),
                "d2h_bytes_per_step": int(op.shape[1] * 4)},
        "roofline": {"bound": "tensor", "kernel": "U-Net training step (tcgen05 implicit convolutions, weight-gradient GEMMs and helper kernels)",
                     "achieved": round(achieved, 2), "peak": peak, "unit": "TFLOP/s",
                     "frac": round(achieved / peak, 4), "traffic": None},
        "gpu_launches": int(v["learned"]["gpu_launches_median"]),
        "clocks": clk,
    }
    if with_cpu:
        m = tests[0].reshape(-1).astype(np.float64)
        dd = np.random.default_rng(0).standard_normal(op.shape[0])
        rec, _, _, _ = cpu_baseline(op, m, dd, target_s=args.cpu_seconds)
        its = v["plain"]["iterations_median"]
        per_it = compulsory_bytes(op.ni, op.ns, op.nr, op.nt) / (rec["value"] * 1e9)
        line["cpu_baseline"] = {"value": round(per_it * its, 2), "unit": "s", "cores": rec["cores"], "kind": "port",
                                "sample": rec["sample"] + f"; x {its:.0f} plain LSQR iterations"}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer (end-to-end) loop")
    ap.add_argument("--sources", type=int, default=0, help="use this many of the 64 sources (small ncu cases)")
    ap.add_argument("--variant", type=int, default=-1, help="force the forward kernel variant (0, 1, 2, 3)")
    ap.add_argument("--adjoint-variant", type=int, default=-1, help="force the adjoint kernel variant (0, 1, 2)")
    ap.add_argument("--workload", default="kirchhoff2d",
                    choices=["kirchhoff2d", "batch", "lsm", "single", "unet", "nsconv", "kirchhoff3d", "conv3x3"],
                    help="kirchhoff2d: the headline fwd+adj workload; batch: 256 batched LSM problems; "
                         "lsm: learned vs plain LSQR time to a 1e-2 data residual (--steps held-out models); "
                         "single: the single-traveltime-table (HBM-streaming) mode; unet: U-Net training; "
                         "nsconv: the non-stationary convolution (image-domain Hessian); kirchhoff3d: the 3-D workload; "
                         "conv3x3: one implicit U-Net convolution or weight gradient (--conv, --conv-kind)")
    ap.add_argument("--conv", default="2,512,256,32,32,0", help="conv3x3 workload: B,H,W,C,N,flip")
    ap.add_argument("--conv-kind", default="fwd", choices=["fwd", "wgrad"])
    ap.add_argument("--weights", default="bfloat16", choices=["bfloat16", "float32"],
                    help="dynamic weight tables of the 3-D workload")
    ap.add_argument("--single-receivers", type=int, default=100)
    ap.add_argument("--lsqr-iters", type=int, default=30, help="LSQR iterations after the timed steps (0: none)")
    ap.add_argument("--lsm-train", type=int, default=4096)
    ap.add_argument("--lsm-steps", type=int, default=3000)
    ap.add_argument("--lsm-stage2-pairs", type=int, default=2048)
    ap.add_argument("--lsm-stage2-steps", type=int, default=1500)
    ap.add_argument("--lsm-net-steps", type=int, default=6, help="at most this many network directions after the warm start")
    ap.add_argument("--lsm-models", type=int, default=32,
                    help="held-out models of the learned-LSM record in the default run")
    ap.add_argument("--no-subrecords", dest="subrecords", action="store_false",
                    help="headline workload only (no 3-D, batched and learned-LSM records)")
    ap.add_argument("--batch-problems", type=int, default=256)
    ap.add_argument("--cgls-iters", type=int, default=20)
    args = ap.parse_args()
    args.steps_e2e = args.steps
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "lsm":
        run_lsm(args)
    elif args.workload == "single":
        run_single(args)
    elif args.workload == "unet":
        run_unet(args)
    elif args.workload == "nsconv":
        run_nsconv(args)
    elif args.workload == "kirchhoff3d":
        run_kirchhoff3d(args)
    elif args.workload == "conv3x3":
        run_conv(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
