#!/usr/bin/env python3
"""Benchmark of the two hot paths on the 200^3 precision-form workload.

Workload (one "step"): a homogeneous 1 x 1 x 1 cm tissue cube on a 200^3
grid (mua 0.3 /cm, mus 100 /cm, g 0.9, n 1.38 in air), a collimated Gaussian
beam of 1/e^2 radius 0.1 cm with Fresnel faces and Russian roulette at 1e-4:
one MC pass of 1e8 packets (FP32 transport, FP64 tally), then 2 s of heating
at 2 W as 821 fused FP32 + Kahan heat steps (dt = 0.9 x the stability limit,
convective beam face h = 10 W/m^2/K, other faces at 37 C, Arrhenius damage
A = 3.1e98 /s, Ea = 6.28e5 J/mol, optics ablated above 100 C).  Inputs are
synthetic (built from these parameters); the working set (~0.4 GB) is larger
than L2, so no L2 flush is needed between steps.

value   : photons/s of transport + heat (packets per step / step time),
          inputs resident on the device, CUDA events on the library's stream.
e2e     : the same through the C ABI with pinned host buffers: every step
          uploads the material grid and the initial temperature and reads back
          temperature, damage and the absorbed-power field.
roofline: the dominant kernel (transport): 12 B per voxel step (rhokap /
          material read + FP64 tally read-modify-write) against the measured
          HBM copy bandwidth; the stencil's 20 B moved per voxel update
          likewise (and the fixed 36 B definition), on the 200^3 step and on
          a 512^3 cube (roofline_stencil_512, 64 steps; --no-scale skips it).

--impl reference runs the CPU oracle (the C restatement of the reference,
OpenMP on all host cores) on bounded samples of the same workload, scaled to
the same metric, in a fresh process; the GPU arm's cpu_baseline times the same
samples the same way.  Both also time configuration 1 in full.  With --gpus N > 1 every rank runs an independent replica
(the path has no exchange step on one instance).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tissue-ablation-mc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "photons/s & voxel-updates/s, FP32 vs FP64 GPU at stated error; %HBM roofline"
GRID = 200
HALF = 0.5
PACKETS = 100_000_000
POWER = 2.0
SIM_TIME = 2.0
B_TRANSPORT = 12.0   # bytes per voxel step
B_STENCIL32 = 36.0   # bytes per voxel update, FP32 + Kahan
B_STENCIL64 = 56.0   # bytes per voxel update, FP64 plain
B_STENCIL_CLS = 20.0  # bytes the class-table FP32 step moves per update (uniform grid)
SEED = 20251203


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_ctx(tam, precision, grid=GRID, packets=PACKETS, device=0):
    p = tam.default_params(nxg=grid, nyg=grid, nzg=grid, xmax=HALF, ymax=HALF, zmax=HALF, mode=1,
                           precision=precision, nphotons=packets, pulse_type=1, power=POWER,
                           energy_per_pixel=POWER * SIM_TIME * 1e3, total_time=SIM_TIME, loops=1, device=device)
    c = tam.default_config()  # the tissue, beam and boundary values above are the config defaults
    c.retrace_fraction = 0.0  # one MC pass per step (no ablation re-trace inside the timed step)
    return tam.Context(p, c)


def heat_steps_for(ctx):
    dt = ctx.state().delt
    return int(math.ceil(SIM_TIME / dt - 1e-9))


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "0x1", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ GPU arm --
def max_over_ranks(ms: float, dist, device: str) -> float:
    """The largest of the ranks' times (all ranks get it); `dist` None: one rank."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_gpu(args):
    import numpy as np
    import torch

    import tam_gb300 as tam

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    packets = args.packets
    ctx = make_ctx(tam, tam._abi.TAM_FP32, packets=packets, device=local)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    nsteps = args.heat_steps if args.heat_steps > 0 else heat_steps_for(ctx)
    nvox = GRID ** 3

    def one_step(i):
        ctx.init_thermal()                          # device-side reset of the instance
        ctx.mc_pass(packets, seed=SEED, stream=i)   # transport + normalisation
        ctx.heat_steps(nsteps)                      # fused stencil + Arrhenius + ablation

    for i in range(args.warmup):
        one_step(1000 + i)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    l0 = tam.kernel_launches()
    t_tr, t_heat, vsteps, scats = [], [], [], []
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for i in range(args.steps):
            one_step(i)
            tr, hm, _ = ctx.timing()
            t_tr.append(tr)
            t_heat.append(hm)
            tl = ctx.tallies()
            vsteps.append(tl["voxel_steps"])
            scats.append(tl["scatters"])
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = tam.kernel_launches() - l0
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, f"cuda:{local}")
    value = world * packets * args.steps / (ms * 1e-3)
    tr_ms = statistics.mean(t_tr)
    heat_ms = statistics.mean(t_heat)
    vs = statistics.mean(vsteps)
    nsc = statistics.mean(scats)
    hbm, peak_kind = peaks()
    red_peak = tam.tally_atomics_per_second(nvox)

    # ---- end to end through the C ABI with pinned host buffers ----
    mat_h = torch.ones((nvox,), dtype=torch.uint8).pin_memory().numpy()
    temp_h = torch.full(((GRID + 2) ** 3,), 310.15, dtype=torch.float64).pin_memory().numpy()
    out_T = torch.empty(((GRID + 2) ** 3,), dtype=torch.float64).pin_memory().numpy()
    out_O = torch.empty((nvox,), dtype=torch.float64).pin_memory().numpy()
    out_J = torch.empty((nvox,), dtype=torch.float64).pin_memory().numpy()
    import ctypes as C

    L = tam._abi.load()
    h = ctx._h

    def vp(a):
        return a.ctypes.data_as(C.c_void_p)

    def e2e_step(i):
        tam.api.check(L.tam_init_thermal(h, None), h)
        tam.api.check(L.tam_upload(h, tam.TAM_F_MATERIAL, vp(mat_h), mat_h.nbytes), h)
        tam.api.check(L.tam_upload(h, tam.TAM_F_TEMP, vp(temp_h), temp_h.nbytes), h)
        tam.api.check(L.tam_mc_pass(h, packets, SEED, i, None), h)
        tam.api.check(L.tam_heat_steps(h, nsteps, None), h)
        tam.api.check(L.tam_download(h, tam.TAM_F_TEMP, vp(out_T), out_T.nbytes), h)
        tam.api.check(L.tam_download(h, tam.TAM_F_TISSUE, vp(out_O), out_O.nbytes), h)
        tam.api.check(L.tam_download(h, tam.TAM_F_JMEAN_GLOBAL, vp(out_J), out_J.nbytes), h)

    e2e_step(2000)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    w0 = time.perf_counter()
    ev0.record(stream)
    for i in range(args.steps):
        e2e_step(i)
    ev1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = ev0.elapsed_time(ev1)
    e2e_wall = (time.perf_counter() - w0) * 1e3
    e2e_ms = max_over_ranks(max(e2e_ms, e2e_wall), dist, f"cuda:{local}")
    e2e_val = world * packets * args.steps / (e2e_ms * 1e-3)
    h2d = mat_h.nbytes + temp_h.nbytes
    d2h = out_T.nbytes + out_O.nbytes + out_J.nbytes

    # ---- FP64 GPU form on identical Philox streams + stated error ----
    fp64 = None
    if rank == 0 and not args.no_fp64:
        n64 = args.fp64_packets
        c64 = make_ctx(tam, tam._abi.TAM_FP64, packets=n64, device=local)
        c64.set_stream(stream.cuda_stream)
        c64.mc_pass(n64, seed=SEED, stream=7)     # warm-up
        c64.mc_pass(n64, seed=SEED, stream=7)
        tr64, _, _ = c64.timing()
        J64 = c64.download(tam.TAM_F_JMEAN_GLOBAL)
        # the MC noise of a sample this size: the FP64 form on an independent stream
        c64.mc_pass(n64, seed=SEED, stream=8)
        J64b = c64.download(tam.TAM_F_JMEAN_GLOBAL)
        noise = float(np.abs(J64b - J64).sum() / np.abs(J64).sum())
        ctx.init_thermal()
        ctx.mc_pass(n64, seed=SEED, stream=7)
        J32 = ctx.download(tam.TAM_F_JMEAN_GLOBAL)
        fl_err = float(np.abs(J32 - J64).sum() / np.abs(J64).sum())
        # identical source for the heat comparison
        c64.init_thermal()
        c64.upload(tam.TAM_F_JMEAN_GLOBAL, J64)
        c64.heat_steps(nsteps)
        _, heat64_ms, _ = c64.timing()
        T64 = c64.download(tam.TAM_F_TEMP)
        O64 = c64.download(tam.TAM_F_TISSUE)
        ctx.init_thermal()
        ctx.upload(tam.TAM_F_JMEAN_GLOBAL, J64)
        ctx.heat_steps(nsteps)
        T32 = ctx.download(tam.TAM_F_TEMP)
        O32 = ctx.download(tam.TAM_F_TISSUE)
        c64.close()
        t_fp64_step = tr64 * (packets / n64) + heat64_ms
        fp64 = {
            "photons_per_s": packets / (t_fp64_step * 1e-3),
            "transport_photons_per_s": n64 / (tr64 * 1e-3),
            "voxel_updates_per_s": nvox * nsteps / (heat64_ms * 1e-3),
            "sample": f"{n64} packets timed, scaled to {packets}; full {nsteps} heat steps",
            "fp32_speedup": value / (packets / (t_fp64_step * 1e-3)),
            "error_fp32_vs_fp64": {
                "relative_fluence_l1": fl_err,
                "relative_fluence_l1_note": "FP32 and FP64 forms on the same Philox streams; the walks part "
                                            "where their roundings differ",
                "relative_fluence_l1_fp64_independent_streams": noise,
                "max_abs_dT_K": float(np.abs(T32 - T64).max()),
                "max_T_rise_K": float(T64.max() - 310.15),
                "max_abs_dOmega": float(np.abs(O32 - O64).max()),
                "max_Omega": float(O64.max()),
            },
        }

    # ---- configuration 1 in full (1e6 packets on 100^3 + 103 steps), both forms ----
    c1 = None
    if rank == 0 and not args.no_c1:
        from tam_gb300 import workloads

        c1 = {"workload": "configuration 1: 100^3 cube, 1e6 packets + 103 heat steps (1 W for 1 s)"}
        for prec, name in ((tam._abi.TAM_FP64, "fp64"), (tam._abi.TAM_FP32, "fp32")):
            w = workloads.c1()
            w.params.precision = prec
            w.params.device = local
            with w.context() as cc:
                cc.set_stream(stream.cuda_stream)
                cc.mc_pass(w.packets, seed=1, stream=1)  # warm-up
                cc.heat_steps(w.heat_steps)
                cc.init_thermal()
                torch.cuda.synchronize()
                ev0.record(stream)
                cc.mc_pass(w.packets, seed=1, stream=0)
                cc.heat_steps(w.heat_steps)
                ev1.record(stream)
                torch.cuda.synchronize()
                sec = ev0.elapsed_time(ev1) * 1e-3
                c1[name] = {"seconds": sec, "photons_per_s": w.packets / sec, "heat_steps": w.heat_steps}

    # ---- the same stencil kernel at scale: a 512^3 cube (134 M voxels, 2.7 GB moved per step) ----
    big = None
    if rank == 0 and not args.no_scale:
        from tam_gb300 import workloads

        edge, nbig = 512, 64
        w = workloads.homogeneous(edge, 1_000_000, 2.0, 2.0, precision=tam._abi.TAM_FP32)
        w.params.device = local
        with w.context() as cb:
            cb.set_stream(stream.cuda_stream)
            cb.mc_pass(w.packets, seed=SEED, stream=3)
            cb.heat_steps(32)    # warm-up: the chunk graphs are captured here
            cb.heat_steps(nbig)  # replayed from CUDA graphs, timed with the library's CUDA events
            _, hb, _ = cb.timing()
            errs = cb.device_errors()
        vb = edge ** 3
        big = {
            "workload": f"{edge}^3 homogeneous cube (2 W beam, 1e6-packet source), {nbig} heat steps after 32",
            "kernel": "slab_step_kernel<uniform>",
            "us_per_step": hb * 1e3 / nbig,
            "voxel_updates_per_s": vb * nbig / (hb * 1e-3),
            "achieved": B_STENCIL_CLS * vb * nbig / (hb * 1e-3) / 1e9,
            "peak": hbm,
            "unit": "GB/s",
            "frac": B_STENCIL_CLS * vb * nbig / (hb * 1e-3) / 1e9 / hbm,
            "bytes_per_unit": f"{B_STENCIL_CLS:g} B per voxel update moved",
            "device_errors": errs,
        }

    # ---- CPU baseline (oracle port, all host cores, in a fresh process) ----
    cpu = None
    if rank == 0 and not args.no_cpu:
        res = cpu_subprocess(args.cpu_samples, args.cpu_seconds, args.cpu_heat_seconds, c1=not args.no_c1)
        smp = res["samples"]
        cpu = dict(smp[-1])
        cpu["value"] = statistics.mean(r["value"] for r in smp)
        cpu["spread"] = [min(r["value"] for r in smp), max(r["value"] for r in smp)]
        cpu["transport_photons_per_s"] = statistics.mean(r["transport_photons_per_s"] for r in smp)
        cpu["voxel_updates_per_s"] = statistics.mean(r["voxel_updates_per_s"] for r in smp)
        cpu["sample"] = f"mean of {len(smp)} samples; last: " + cpu["sample"]
        cpu["c1_full"] = res.get("c1_full")

    ctx.close()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    clk_s = clk.summary()
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "photons/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 transport + f64 tally; f32+Kahan stencil, float-float Arrhenius exponent + f64 damage sum",
        "data": "synthetic (homogeneous tissue cube built from the workload parameters)",
        "config": workload_config(packets, nsteps, world),
        "voxel_updates_per_s": world * nvox * nsteps / (heat_ms * 1e-3),
        "transport": {
            "photons_per_s": world * packets / (tr_ms * 1e-3),
            "voxel_steps_per_packet": vs / packets,
            "voxel_steps_per_s": world * vs / (tr_ms * 1e-3),
            "kernel_ms": tr_ms,
            # one red.global.add.f64 per voxel step that ends on a face (the
            # steps that end at an interaction carry their deposit onward)
            "l2_atomics": {
                "achieved_per_s": world * (vs - nsc) / (tr_ms * 1e-3),
                "peak_per_s": red_peak,
                "frac": (vs - nsc) / (tr_ms * 1e-3) / red_peak if red_peak else None,
                "peak_kind": "measured in this run: the library's own kernel (tam_measure_tally_atomics) issuing "
                             "red.global.add.f64 at Philox-drawn cells of the 64 MB tally (L2-resident), 4 blocks of "
                             "256 threads per SM as the transport, no index stream",
            },
        },
        "heat": {"ms_per_step_segment": heat_ms, "ms_per_heat_step": heat_ms / nsteps},
        "roofline": {
            "bound": "hbm",
            "kernel": "transport_kernel<float, uniform medium>",
            "achieved": B_TRANSPORT * vs / (tr_ms * 1e-3) / 1e9,
            "peak": hbm,
            "unit": "GB/s",
            "frac": B_TRANSPORT * vs / (tr_ms * 1e-3) / 1e9 / hbm,
            "traffic": None,
            "bytes_per_unit": f"{B_TRANSPORT:g} B per voxel step; {vs / packets:.1f} voxel steps per packet",
            "peak_kind": peak_kind,
            "note": "transport is issue/latency bound (divergent random walks, L2-resident atomics), not HBM bound",
        },
        "roofline_stencil": {
            "bound": "hbm",
            "kernel": "slab_step_kernel<uniform> (FP32 + Kahan, class-table coefficients, slab form)",
            "achieved": B_STENCIL_CLS * nvox * nsteps / (heat_ms * 1e-3) / 1e9,
            "peak": hbm,
            "unit": "GB/s",
            "frac": B_STENCIL_CLS * nvox * nsteps / (heat_ms * 1e-3) / 1e9 / hbm,
            "bytes_per_unit": f"{B_STENCIL_CLS:g} B per voxel update moved (T, Kahan term, J read; T, Kahan term "
                              "written); the thermal properties come from the class table",
            "fixed_definition": {
                "bytes_per_unit": f"{B_STENCIL32:g} B per voxel update (T, Kahan term, k, rho, c, J, Q read; T, "
                                  "Kahan term written)",
                "achieved": B_STENCIL32 * nvox * nsteps / (heat_ms * 1e-3) / 1e9,
                "frac": B_STENCIL32 * nvox * nsteps / (heat_ms * 1e-3) / 1e9 / hbm,
            },
            "peak_kind": peak_kind,
        },
        "roofline_stencil_512": big,
        "e2e": {"value": e2e_val, "unit": "photons/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk_s,
        "fp64": fp64,
        "c1_full": c1,
        "cpu_baseline": cpu,
    }
    traffic = profile_traffic(vs)
    if traffic is not None:
        line["roofline"]["traffic"] = traffic
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def profile_traffic(voxel_steps):
    """DRAM bytes of one full transport launch, scaled from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "transport_kernel_200cube.txt")
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_voxel_step:"):
                return float(ln.split(":")[1]) * voxel_steps
    except OSError:
        pass
    return None


# ------------------------------------------------------- CPU (oracle) --
def workload_config(packets, nsteps, world):
    """The `config` object of both arms' JSON lines."""
    return {
        "workload": f"precision form: {GRID}^3 homogeneous cube 1x1x1 cm, {packets:.0e} packets "
                    f"(Gaussian beam w=0.1 cm, Fresnel, roulette 1e-4) + {nsteps} fused heat steps "
                    f"(2 W for 2 s, Arrhenius, ablation at 100 C)",
        "grid": [GRID, GRID, GRID],
        "packets_per_step": packets,
        "heat_steps_per_step": nsteps,
        "l2": "inputs larger than L2 (working set ~0.4 GB); no flush",
        "parallelism": f"replicas x{world}",
    }


def cpu_nsteps():
    dxm = 2 * HALF * 1e-2 / GRID
    alpha = 0.56 / (1070 * 3400)
    dt = 0.9 * dxm * dxm / (6 * alpha)
    return dt, int(math.ceil(SIM_TIME / dt - 1e-9))


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_samples(nsamples, mc_seconds, heat_seconds, c1=False):
    """The oracle port (C, FP64, OpenMP on every host core) on bounded samples
    of the workload.  Runs in a process of its own (see cpu_subprocess).

    Transport: one oracle call has a fixed cost (per-thread tallies of the
    whole grid are allocated, zeroed and summed, as the reference's per-rank
    tallies and all-reduce), measured with an empty call; each sample times
    about `mc_seconds` of packets (sized from the previous sample's rate), and
    the full pass is that fixed cost plus the sample's per-packet time x 1e8.
    Heat: consecutive fused steps from the initial state, on the sample's own
    normalised tally as the absorbed-power field, for about `heat_seconds`,
    scaled to the full step count."""
    import numpy as np

    import build_oracle

    build_oracle.build()
    import oracle as orc

    ncores = host_cores()
    mats = [(0.0, 0.0, 0.0, 1.0), (0.3, 100.0, 0.9, 1.38)]
    d = orc.mc_desc(GRID, GRID, GRID, HALF, HALF, HALF, materials=mats, source_radius=0.1)
    grid = np.ones((GRID, GRID, GRID), dtype=np.uint8, order="F")
    fix = []
    for _ in range(2):
        t0 = time.perf_counter()
        orc.mc_transport(d, grid, 0, seed=SEED, nthreads=ncores)
        fix.append(time.perf_counter() - t0)
    t_fix = min(fix)
    n = 8000
    while True:
        t0 = time.perf_counter()
        orc.mc_transport(d, grid, n, seed=SEED, stream=99, nthreads=ncores)
        t = time.perf_counter() - t0 - t_fix
        if t >= 0.4 * mc_seconds or n >= 1 << 24:
            break
        n *= 2
    rate = n / max(t, 1e-6)  # packets/s, re-measured by every sample
    dt, nsteps = cpu_nsteps()
    dxm = 2 * HALF * 1e-2 / GRID
    h = orc.heat_desc(GRID, GRID, GRID, dxm, dxm, dxm, dt=dt)
    sh = (GRID, GRID, GRID)
    out = []
    for i in range(nsamples):
        n_mc = max(8000, int(rate * mc_seconds))
        t0 = time.perf_counter()
        jm, tal = orc.mc_transport(d, grid, n_mc, seed=SEED, stream=1 + i, nthreads=ncores)
        t_mc = time.perf_counter() - t0
        per_packet = max(t_mc - t_fix, 1e-9) / n_mc
        rate = 1.0 / per_packet
        t_mc_full = t_fix + per_packet * PACKETS
        J = np.asfortranarray(jm * (1.0 / (n_mc * dxm ** 3)))
        T = np.full(sh, 310.15, order="F")
        k = np.full(sh, 0.56, order="F")
        rho = np.full(sh, 1070.0, order="F")
        c = np.full(sh, 3400.0, order="F")
        Q = np.zeros(sh, order="F")
        om = np.zeros(sh, order="F")
        thr = np.zeros(sh + (3,), order="F")
        mat = np.ones(sh, dtype=np.uint8, order="F")
        t0 = time.perf_counter()
        s = 0
        while s < 2 or ((time.perf_counter() - t0) < heat_seconds and s < nsteps):
            T, _ = orc.fused_step(h, POWER, (s + 1) * h.dt, T, k, rho, c, J, Q, om, thr, mat, nthreads=ncores)
            s += 1
        t_heat = time.perf_counter() - t0
        t_step = t_mc_full + t_heat * (nsteps / s)
        out.append({
            "value": PACKETS / t_step,
            "unit": "photons/s",
            "cores": ncores,
            "kind": "port",
            "sample": f"extrapolated: {n_mc} packets ({t_mc:.2f} s, of which {t_fix:.2f} s is the fixed per-call "
                      f"cost of the per-thread tallies) and {s} of {nsteps} heat steps ({t_heat:.2f} s) of the "
                      f"{GRID}^3 workload, FP64 oracle on {ncores} threads, scaled linearly to {PACKETS:.0e} packets "
                      f"+ {nsteps} steps",
            "transport_photons_per_s": 1.0 / per_packet,
            "voxel_updates_per_s": GRID ** 3 * s / t_heat,
            "voxel_steps_per_packet": tal["voxel_steps"] / n_mc,
        })
    res = {"samples": out}
    if c1:
        res["c1_full"] = cpu_c1_full(orc, ncores)
    return res


def cpu_c1_full(orc, ncores):
    """Configuration 1 in full on the oracle: one pass of 1e6 packets on the
    100^3 cube and its 103 heat steps of 1 s at 1 W (FP64)."""
    import numpy as np

    edge, n, P, secs = 100, 1_000_000, 1.0, 1.0
    mats = [(0.0, 0.0, 0.0, 1.0), (0.3, 100.0, 0.9, 1.38)]
    d = orc.mc_desc(edge, edge, edge, HALF, HALF, HALF, materials=mats, source_radius=0.1)
    grid = np.ones((edge,) * 3, dtype=np.uint8, order="F")
    dxm = 2 * HALF * 1e-2 / edge
    alpha = 0.56 / (1070 * 3400)
    dt = 0.9 * dxm * dxm / (6 * alpha)
    nsteps = int(math.ceil(secs / dt - 1e-9))
    h = orc.heat_desc(edge, edge, edge, dxm, dxm, dxm, dt=dt)
    sh = (edge,) * 3
    t0 = time.perf_counter()
    jm, _ = orc.mc_transport(d, grid, n, seed=1, nthreads=ncores)
    t_mc = time.perf_counter() - t0
    J = np.asfortranarray(jm * (1.0 / (n * dxm ** 3)))
    T = np.full(sh, 310.15, order="F")
    k, rho, c = (np.full(sh, v, order="F") for v in (0.56, 1070.0, 3400.0))
    Q, om = np.zeros(sh, order="F"), np.zeros(sh, order="F")
    thr = np.zeros(sh + (3,), order="F")
    mat = np.ones(sh, dtype=np.uint8, order="F")
    t1 = time.perf_counter()
    for s in range(nsteps):
        T, _ = orc.fused_step(h, P, (s + 1) * dt, T, k, rho, c, J, Q, om, thr, mat, nthreads=ncores)
    t_heat = time.perf_counter() - t1
    return {"workload": f"configuration 1: {edge}^3 cube, {n:.0e} packets + {nsteps} heat steps (FP64)",
            "seconds": t_mc + t_heat, "transport_s": t_mc, "heat_s": t_heat, "photons_per_s": n / (t_mc + t_heat),
            "cores": ncores}


def cpu_subprocess(nsamples, mc_seconds, heat_seconds, c1=False):
    """cpu_samples in a fresh Python process, so that no thread pool or CUDA
    state of the calling process competes with the oracle's threads."""
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-leg", "--cpu-samples", str(nsamples),
           "--cpu-seconds", str(mc_seconds), "--cpu-heat-seconds", str(heat_seconds)]
    if c1:
        cmd.append("--cpu-c1")
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT)
    if r.returncode != 0:
        raise RuntimeError("CPU leg failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    res = cpu_subprocess(args.warmup + args.steps, args.cpu_seconds, args.cpu_heat_seconds, c1=not args.no_c1)
    timed = res["samples"][args.warmup:]
    v = statistics.mean(r["value"] for r in timed)
    last = timed[-1]
    _, nsteps = cpu_nsteps()
    line = {
        "metric": METRIC, "value": v, "unit": "photons/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * PACKETS / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": workload_config(PACKETS, nsteps, int(os.environ.get("WORLD_SIZE", "1"))),
        "cpu_baseline": {"value": v, "unit": "photons/s", "cores": last["cores"], "kind": "port",
                         "sample": last["sample"],
                         "spread": [min(r["value"] for r in timed), max(r["value"] for r in timed)],
                         "transport_photons_per_s": statistics.mean(r["transport_photons_per_s"] for r in timed),
                         "voxel_updates_per_s": statistics.mean(r["voxel_updates_per_s"] for r in timed),
                         "c1_full": res.get("c1_full")},
        "e2e": {"value": v, "unit": "photons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Fortran + MPI and no Fortran compiler exists on either machine; "
                "its C restatement (oracle/) is timed instead; each step is one extrapolated sample",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--packets", type=int, default=PACKETS, help="profiling only: packets per step")
    ap.add_argument("--heat-steps", type=int, default=0, help="profiling only: heat steps per step")
    ap.add_argument("--fp64-packets", type=int, default=2_000_000)
    ap.add_argument("--cpu-seconds", type=float, default=3.0, help="seconds of packets per CPU sample")
    ap.add_argument("--cpu-heat-seconds", type=float, default=1.5, help="seconds of heat steps per CPU sample")
    ap.add_argument("--cpu-samples", type=int, default=3, help="CPU samples of the GPU arm's baseline")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-c1", action="store_true", help="skip the full run of configuration 1")
    ap.add_argument("--no-scale", action="store_true", help="skip the 512^3 stencil measurement")
    ap.add_argument("--cpu-leg", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--cpu-c1", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.cpu_leg:
        print(json.dumps(cpu_samples(args.cpu_samples, args.cpu_seconds, args.cpu_heat_seconds, c1=args.cpu_c1)))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
