"""Benchmark: site-updates/s of one RK4 step of the EWPT lattice at 256^3.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--n 256] [--no-fp32] [--no-e2e] [--no-cpu]

Workload (one step = one classical RK4 step over the whole lattice): the
drop-in FP64 configuration -- 256^3 periodic lattice, dx = 0.25,
dt = dx/10, lambda = 0.129, g = 0.65, g' = 0.35, vev = 1, gp2 = 0.99,
gamma = beta = Jex = 0, 64 seeded tanh bubbles.  The FP32 precision form
(FP32 stencils/fluxes, compensated FP32 hi/lo state) is timed on the same
lattice and reported in the same line.

value    FP64 site-updates/s with the state resident in HBM (CUDA events on
         the library's stream; the 4.8 GB state is larger than L2).
e2e      the same metric through the C ABI with host buffers, as a drop-in
         rk4_step! caller sees it: every step is one ewpt_step_host call
         that uploads the state from pinned host memory, steps once and
         writes the evolved state, the step's result, back into pinned host
         memory, the copies overlapped with stages 1 and 4 over windows of
         z planes.  `sequential_value` is the same round trip as three calls
         (ewpt_set_state_packed, ewpt_step, ewpt_get_state_packed).  The
         snapshot diagnostics are not in the per-step loop: the 256^3
         configuration takes them every 100 steps, and the reference arm's
         steps have none either.
roofline HBM roofline of the stage kernels: algorithmic bytes per
         site-update (3744 B FP64, 2592 B FP32 form) x site-updates/s over
         the measured copy bandwidth.
roofline_compute  the FP64 form's own bound, the FP64 pipe: counted FLOPs
         per site-update x site-updates/s over the FP64 peak measured in
         this run (ewpt_fp64_peak, fused multiply-add chains on every SM).
--impl reference  times the CPU restatement of the reference's routines (the
         oracle) on the host cores on a bounded sample lattice.
With --gpus N > 1 (torchrun), each rank evolves its own replica; value is the
sum over ranks (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "ewpt-gpu_gb300"))

METRIC = "site-updates/s per RK4 step at 256³ (FP64 vs FP32 form), % of HBM peak"
BYTES_FP64 = 3744  # 468 FP64 values per site-update (k-storage RK4)
BYTES_FP32 = 2592  # y in FP64 width, stage rates in FP32
# DRAM bytes per site-update (sum over the 4 stage launches) from one ncu
# capture of the stage kernels (dram__bytes_read.sum + dram__bytes_write.sum):
# FP64 at 80^3, 32x2 threads; FP32 form at 128^3, the tuned paired kernel
# (64x2 pair-threads, <= 168 registers, with its L2 prefetches).  Traffic grows with the site count,
# so a 256^3 launch moves this x S / 4.
TRAFFIC_FP64 = 4383
TRAFFIC_FP32 = 2973
# FP64 operations of one site-update of the FP64 stage kernels (4 stages of
# site_rates + the RK4 epilogue), counted exactly by compiling the kernels'
# own per-site templates with an operator-counting scalar type
# (tests/test_devphys.py checks these figures against that count): FLOPs with
# an FMA as 2, and FP64 pipe instructions with single-use products fused.
FLOPS_FP64 = 7300
FP64_INST_EST = 4976
# FP64 instructions per site-update the stage kernels execute (ncu
# smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum over the 4
# launches at 80^3, per site): 3 x (454 + 126 + 604) + (454 + 126 + 568).
FP64_INST_NCU = 4700
N_BUBBLES = 64


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_params(n, precision):
    import ewpt

    return ewpt.baseline_couplings(N=n, dx=0.25, dt=0.025, precision=precision)


def time_steps(lat, steps, warmup):
    """K steps bracketed by CUDA events on the library's stream."""
    import torch

    st = torch.cuda.ExternalStream(lat.stream)
    lat.step(warmup)
    lat.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    lat.step(steps)
    e1.record(st)
    lat.sync()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    import ewpt

    torch.cuda.set_device(local)
    n = args.n
    p64 = make_params(n, ewpt.FP64)
    p64.device = local
    shape = p64.dims
    S = p64.sites
    y0 = ewpt.ic.bubbles_tanh(shape, p64.dx, N_BUBBLES, seed=1234 + rank)
    hbm, peak_kind = peaks()
    res = {}
    from ewpt import autotune

    tiles = {}
    # ---------------------------------------------------------------- FP64
    with ewpt.Lattice(p64) as lat:
        lat.set_state(y0)
        if not args.no_tune:
            tiles["fp64"] = autotune.tune(lat)
        barrier(ws)
        with Clocks(local) as ck:
            t = time_steps(lat, args.steps, args.warmup)
        t = allmax(ws, t)
        clocks = ck.summary()
        d = lat.diagnostics()
        res["fp64"] = dict(t=t, diag=d.tolist(), peak=ewpt._lib.fp64_peak(local))
        # ------------------------------------------------------------ e2e
        if not args.no_e2e:
            host = torch.empty((36, S), dtype=torch.float64, pin_memory=True)
            host.numpy()[:] = y0
            back = torch.empty((36, S), dtype=torch.float64, pin_memory=True)
            ptr, bptr = host.data_ptr(), back.data_ptr()
            row = np.zeros(20)
            L = lat.L
            import ctypes as C

            def e2e_step():
                ewpt._lib.check(L.ewpt_step_host(lat.h, C.c_void_p(ptr), C.c_void_p(bptr), 1), lat.h)

            def e2e_step_sequential():
                ewpt._lib.check(L.ewpt_set_state_packed(lat.h, C.c_void_p(ptr), 0), lat.h)
                ewpt._lib.check(L.ewpt_step(lat.h, 1), lat.h)
                ewpt._lib.check(L.ewpt_get_state_packed(lat.h, C.c_void_p(bptr), 0), lat.h)

            ke = max(1, args.steps)
            te = {}
            for name, fn in (("sequential", e2e_step_sequential), ("overlapped", e2e_step)):
                for _ in range(max(1, min(args.warmup, 2))):
                    fn()
                barrier(ws)
                t0 = time.perf_counter()
                for _ in range(ke):
                    fn()
                te[name] = allmax(ws, time.perf_counter() - t0)
                # the step's result arrived in host memory: check it is a finite state
                assert np.isfinite(back.numpy()[:, :: max(1, S // 4096)]).all()
            ewpt._lib.check(L.ewpt_diagnostics(lat.h, row.ctypes.data_as(ewpt._lib.DP)), lat.h)  # after the timing
            res["e2e"] = dict(t=te["overlapped"], t_seq=te["sequential"], steps=ke, h2d=36 * S * 8, d2h=36 * S * 8)
    # ---------------------------------------------------------------- FP32
    if not args.no_fp32:
        p32 = make_params(n, ewpt.FP32)
        p32.device = local
        with ewpt.Lattice(p32) as lat:
            lat.set_state(y0)
            if not args.no_tune:
                tiles["fp32"] = autotune.tune(lat)
            barrier(ws)
            k32 = max(args.steps, 10)
            t = allmax(ws, time_steps(lat, k32, args.warmup))
            res["fp32"] = dict(t=t, steps=k32, diag=lat.diagnostics().tolist())
            # the compensated mode (two sites per thread): same lattice, same steps
            if lat.tiling()[3] != 1:
                lat.set_tiling(64, 2, 2, 1)
            lat.set_fp32_compensated(True)
            barrier(ws)
            t = allmax(ws, time_steps(lat, k32, args.warmup))
            res["fp32c"] = dict(t=t, steps=k32, tile=list(lat.tiling()))
    # ------------------------------------------------------------ DF64
    if not args.no_df64:
        pd = make_params(n, ewpt.DF64)
        pd.device = local
        with ewpt.Lattice(pd) as lat:
            lat.set_state(y0)
            if not args.no_tune:
                tiles["df64"] = autotune.tune(lat)
            barrier(ws)
            kd = max(args.steps, 5)
            t = allmax(ws, time_steps(lat, kd, args.warmup))
            res["df64"] = dict(t=t, steps=kd, diag=lat.diagnostics().tolist())
    # ------------------------------------------------------------ ensemble
    if not args.no_ensemble:
        res["ensemble"] = run_ensemble(args, ws)
    # ------------------------------------------------------- CPU baseline
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(budget_s=args.cpu_seconds)
    if rank != 0:
        return
    t64 = res["fp64"]["t"]
    v = ws * S * args.steps / t64
    ach = S * args.steps / t64 * BYTES_FP64 / 1e9
    out = {
        "metric": METRIC,
        "value": v,
        "unit": "site-updates/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t64 / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": f"synthetic: {N_BUBBLES} seeded tanh-profile bubbles (radius 2/sqrt(lambda)), fields at rest",
        "config": {"workload": f"drop-in FP64 RK4 step, {n}^3 periodic lattice, dx=0.25, dt=dx/10, "
                               "lambda=0.129, g=0.65, g'=0.35, vev=1, gp2=0.99, gamma=beta=Jex=0",
                   "lattice": [n, n, n], "form": "FP64",
                   "l2": f"inputs larger than L2 (state {36 * S * 8 / 1e9:.2f} GB per replica)",
                   "parallelism": f"replicas x{ws}",
                   "tiling": {k: list(v) for k, v in tiles.items()}},
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "traffic": TRAFFIC_FP64 * S / 4, "peak_kind": peak_kind,
                     "kernel": "k_stage_fp64 (4 launches/step, the whole step)",
                     "launch_ms": t64 / args.steps / 4 * 1e3,
                     "traffic_source": "ncu dram bytes per site-update at 80^3 x sites / 4",
                     "algorithmic_bytes_per_site_update": BYTES_FP64,
                     "limiter": "the FP64 pipe, not HBM: see roofline_compute"},
        "roofline_compute": {"bound": "fp64", "achieved": S * args.steps / t64 * FLOPS_FP64 / 1e12,
                             "peak": res["fp64"]["peak"] / 1e12, "unit": "TFLOP/s",
                             "frac": S * args.steps / t64 * FLOPS_FP64 / res["fp64"]["peak"],
                             "peak_kind": "measured in this run: ewpt_fp64_peak (DFMA chains on every SM)",
                             "flops_per_site_update": FLOPS_FP64,
                             "flops_source": "exact count of the kernels' per-site source (oracle/devphys.cu), "
                                             "FMA = 2 FLOPs",
                             "pipe": {"fp64_inst_per_site_update": FP64_INST_NCU,
                                      "source": "ncu DADD+DMUL+DFMA thread instructions at 80^3",
                                      "achieved_ginst_s": S * args.steps / t64 * FP64_INST_NCU / 1e9,
                                      "peak_ginst_s": res["fp64"]["peak"] / 2 / 1e9,
                                      "frac": S * args.steps / t64 * FP64_INST_NCU / (res["fp64"]["peak"] / 2)},
                             "note": "FLOP frac < 1 by construction: DADD and DMUL take a pipe slot for 1 FLOP; "
                                     "the pipe frac is the FP64 instruction rate over the probe's",
                             "kernel": "k_stage_fp64 (4 launches/step)"},
        "gpu_launches": 4 * args.steps,
        "clocks": clocks,
    }
    if "e2e" in res:
        e = res["e2e"]
        out["e2e"] = {"value": ws * S * e["steps"] / e["t"], "unit": "site-updates/s",
                      "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"], "steps": e["steps"],
                      "ms_per_step": e["t"] / e["steps"] * 1e3,
                      "path": "ewpt_step_host(pinned host in, pinned host out, 1 step) per step: upload "
                              "overlapped with stage 1, download with stage 4 (windows of z planes)",
                      "sequential_value": ws * S * e["steps"] / e["t_seq"],
                      "sequential_path": "ewpt_set_state_packed(pinned host) + ewpt_step(1) + "
                                         "ewpt_get_state_packed(pinned host) per step"}
    if "fp32" in res:
        f = res["fp32"]
        v32 = ws * S * f["steps"] / f["t"]
        a32 = S * f["steps"] / f["t"] * BYTES_FP32 / 1e9
        out["fp32_form"] = {"value": v32, "unit": "site-updates/s", "ms_per_step": f["t"] / f["steps"] * 1e3,
                            "steps": f["steps"], "dtype": "f32 stencils/fluxes, f32 hi/lo state",
                            "speedup_vs_fp64": v32 / v,
                            "roofline": {"bound": "hbm", "achieved": a32, "peak": hbm, "unit": "GB/s",
                                         "frac": a32 / hbm, "peak_kind": peak_kind,
                                         "traffic": TRAFFIC_FP32 * S / 4,
                                         "traffic_source": "ncu dram bytes per site-update at 128^3 x sites / 4",
                                         "launch_ms": f["t"] / f["steps"] / 4 * 1e3,
                                         "algorithmic_bytes_per_site_update": BYTES_FP32}}
    if "fp32c" in res:
        f = res["fp32c"]
        vc = ws * S * f["steps"] / f["t"]
        ac = S * f["steps"] / f["t"] * BYTES_FP32 / 1e9
        out["fp32c_form"] = {"value": vc, "unit": "site-updates/s", "ms_per_step": f["t"] / f["steps"] * 1e3,
                             "steps": f["steps"], "tiling": f["tile"],
                             "dtype": "f32 stencils/fluxes, the gauge Laplacians and auxiliary gradients "
                                      "compensated (float pairs), f32 hi/lo state",
                             "speedup_vs_fp64": vc / v,
                             "roofline": {"bound": "hbm", "achieved": ac, "peak": hbm, "unit": "GB/s",
                                          "frac": ac / hbm, "peak_kind": peak_kind,
                                          "algorithmic_bytes_per_site_update": BYTES_FP32}}
    if "df64" in res:
        f = res["df64"]
        vd = ws * S * f["steps"] / f["t"]
        ad = S * f["steps"] / f["t"] * BYTES_FP64 / 1e9
        out["df64_form"] = {"value": vd, "unit": "site-updates/s", "ms_per_step": f["t"] / f["steps"] * 1e3,
                            "steps": f["steps"], "dtype": "double-float (float hi + lo, ~2^-47 per operation)",
                            "speedup_vs_fp64": vd / v,
                            "parity": "FP64 bar: 1e-11 relative per field after 100 steps vs the oracle (tested)",
                            "roofline": {"bound": "hbm", "achieved": ad, "peak": hbm, "unit": "GB/s",
                                         "frac": ad / hbm, "peak_kind": peak_kind,
                                         "launch_ms": f["t"] / f["steps"] / 4 * 1e3,
                                         "algorithmic_bytes_per_site_update": BYTES_FP64}}
    if "ensemble" in res:
        out["ensemble"] = res["ensemble"]
    if cpu:
        out["cpu_baseline"] = cpu
    print(json.dumps(out), flush=True)


ENSEMBLE_SIZES = [48] * 32 + [96] * 32 + [128] * 24 + [160] * 8


def run_ensemble(args, ws):
    """Batched-ensemble configuration: 96 independent FP32-form lattices
    (32 x 48^3, 32 x 96^3, 24 x 128^3, 8 x 160^3), alternately seeded bubble
    ICs with 8-40 bubbles and thermal ICs with T in [1, 2] vev (device IC);
    one step of all members is one CUDA graph with a concurrent branch per
    member, each member at the fastest single-lattice shape of its size;
    site-updates/s over all members."""
    import numpy as np
    import torch

    import ewpt

    from ewpt import autotune

    rng = np.random.default_rng(2024)
    ps = [ewpt.baseline_couplings(N=n, dx=0.25, dt=0.025, precision=ewpt.FP32) for n in ENSEMBLE_SIZES]
    # the fastest single-lattice shape per member size (swept before the ensemble exists)
    tiles = None if args.no_tune else autotune.member_tilings(ps)
    with ewpt.Ensemble(ps) as ens:
        if tiles:
            for m, t in enumerate(tiles):
                ens.set_member_tiling(m, *t)
        for m, p in enumerate(ps):
            if m % 2 == 0:  # bubble nucleation: 8-40 tanh bubbles
                R, w = ewpt.ic.tanh_profile_params(p.lam, p.vev)
                nb = int(rng.integers(8, 41))
                ens.init_bubbles(m, ewpt.ic.tanh_bubble_list(p.dims, p.dx, nb, seed=m), "tanh", R, w)
            else:  # thermal: T in [1, 2] vev, device IC
                ens.init_thermal(m, float(rng.uniform(1.0, 2.0)) * p.vev, seed=1000 + m)
        st = torch.cuda.ExternalStream(ens.stream)
        ens.step(args.warmup)
        ens.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k = max(args.steps, 5)
        barrier(ws)
        e0.record(st)
        ens.step(k)
        e1.record(st)
        ens.sync()
        t = allmax(ws, e0.elapsed_time(e1) / 1e3)
        sites = ens.sites
    return {"value": ws * sites * k / t, "unit": "site-updates/s", "ms_per_step": t / k * 1e3, "steps": k,
            "members": len(ps), "sites": sites,
            "workload": "96 FP32-form lattices: 32x48^3 + 32x96^3 + 24x128^3 + 8x160^3, alternately 8-40 tanh "
                        "bubbles and a thermal IC at T in [1, 2] vev; one step of all members is one CUDA graph "
                        "with a concurrent branch per member (its 4 stage launches and 4 ghost refreshes)",
            "gpu_launches": 8 * len(ps) * k,
            "tiling": ({f"{n}^3": list(tiles[ENSEMBLE_SIZES.index(n)]) for n in sorted(set(ENSEMBLE_SIZES))}
                       if tiles else None)}


def cpu_baseline(budget_s=20.0, threads=None):
    """The oracle (CPU restatement of the reference routines) on the host
    cores: config-1 style lattice, seconds-bounded sample."""
    import numpy as np

    import ewpt
    from oracle import oracle as orc

    orc.build()
    if threads:
        orc.set_threads(threads)
    nthr = orc.num_threads()
    p = make_params(64, ewpt.FP64)
    y = ewpt.ic.bubbles_tanh(p.dims, p.dx, 10, seed=7)
    op = orc.params(p.dims, p.dx, p.gw, p.gy, p.gp2, p.lam, p.vev, p.beta_w, p.beta_y, p.theta_w)
    work = np.empty(3 * y.size)
    orc.rk4_step(op, y, p.dt, work=work)  # warm
    steps, t0 = 0, time.perf_counter()
    while True:
        y = orc.rk4_step(op, y, p.dt, work=work)
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or steps >= 200:
            break
    return {"value": p.sites * steps / el, "unit": "site-updates/s", "cores": nthr, "kind": "port",
            "sample": f"64^3 lattice, 10 bubbles, {steps} FP64 RK4 steps ({el:.1f} s) of the oracle "
                      f"(C restatement of rk4_step! + broadcasts, OpenMP {nthr} threads)"}


def run_reference(args, ws, rank):
    """CPU reference arm: the oracle (the C restatement of rk4_step! and its
    RK4 broadcasts) on all host cores.  It runs the full workload lattice
    when W + K steps there fit in --ref-seconds (a 256^3 step takes ~5 s on
    16 Arm cores); otherwise a smaller lattice with the same per-site work
    stands in as the sample."""
    if rank != 0:
        return
    import numpy as np

    import ewpt
    from oracle import oracle as orc

    orc.build()
    nthr = orc.num_threads()
    p = make_params(args.n, ewpt.FP64)
    op = orc.params(p.dims, p.dx, p.gw, p.gy, p.gp2, p.lam, p.vev, p.beta_w, p.beta_y, p.theta_w)
    y = ewpt.ic.bubbles_tanh(p.dims, p.dx, N_BUBBLES, seed=1234)
    work = np.empty(3 * y.size)
    t0 = time.perf_counter()
    y = orc.rk4_step(op, y, p.dt, work=work)  # first warm-up step, at the full workload
    t1 = time.perf_counter() - t0
    n = args.n
    if (args.warmup - 1 + args.steps) * t1 > args.ref_seconds:
        # sample lattice sized so that one step takes ~2 s
        n = int(round((2.0 / t1) ** (1.0 / 3.0) * args.n))
        n = max(32, min(args.n, (n // 8) * 8))
        p = make_params(n, ewpt.FP64)
        op = orc.params(p.dims, p.dx, p.gw, p.gy, p.gp2, p.lam, p.vev, p.beta_w, p.beta_y, p.theta_w)
        y = ewpt.ic.bubbles_tanh(p.dims, p.dx, max(4, N_BUBBLES * n ** 3 // args.n ** 3), seed=1234)
        work = np.empty(3 * y.size)
        y = orc.rk4_step(op, y, p.dt, work=work)
    for _ in range(args.warmup - 1):
        y = orc.rk4_step(op, y, p.dt, work=work)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        y = orc.rk4_step(op, y, p.dt, work=work)
    el = time.perf_counter() - t0
    v = p.sites * args.steps / el
    same = n == args.n
    sample = (f"{n}^3 lattice{' (the full workload)' if same else f' sample with the {args.n}^3 workload per-site work'}"
              f", {N_BUBBLES if same else max(4, N_BUBBLES * n ** 3 // args.n ** 3)} tanh bubbles, {args.steps} "
              f"FP64 RK4 steps of the oracle (C restatement of rk4_step! + RK4 broadcasts), OpenMP {nthr} threads")
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "site-updates/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic: seeded tanh-profile bubbles",
           "config": {"workload": f"drop-in FP64 RK4 step, {args.n}^3 periodic lattice, dx=0.25, dt=dx/10",
                      "lattice": [n, n, n], "form": "FP64", "parallelism": "host cores"},
           "cpu_baseline": {"value": v, "unit": "site-updates/s", "cores": nthr, "kind": "port", "sample": sample},
           "e2e": {"value": v, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=300.0,
                    help="reference arm: largest projected CPU time for W + K steps at the full lattice")
    ap.add_argument("--no-tune", action="store_true", help="keep the default 32x4 tiling")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-df64", action="store_true", help="skip the double-float form")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
