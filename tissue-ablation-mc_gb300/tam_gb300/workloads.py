"""Synthetic workloads of the five benchmark configurations, built from seeds.

Each builder returns a ``Workload``: run parameters, the config-mode extension,
an optional per-voxel material grid (u8, Fortran order) and a description.
Sizes default to the full configurations; ``edge``/``scale`` arguments build
smaller copies of the same geometry for tests.

  C1  100^3 homogeneous cube 1x1x1 cm, 1e6 packets, 1 W for 1 s
  C2  200^3 homogeneous cube, 1e8 packets, 2 W for 2 s (FP32 + Kahan)
  C3  256x256x128 three-layer skin slab over 1x1x0.5 cm, 1e8 packets per pass,
      2e4 heat steps at 5 W, MC re-run when 0.1 % of the grid has ablated
  C4  64 instances with edges uniform in [64,192] per axis and per-instance
      optics and laser drawn from a seeded generator; 1e7 packets, 5e3 steps
  C5  512^3 over 2x2x2 cm: dermis with 20 seeded vessel cylinders and 5
      spherical inclusions; 1e9 packets, 10 pulses of 50 ms at 10 W, 1 Hz

Thermal constants that the configurations leave open (the C3 layers, the C5
blood and inclusions) are literature-typical skin values, fixed here:

  epidermis  k 0.21 W/m/K, rho 1200 kg/m^3, c 3590 J/kg/K
  dermis     k 0.37,       rho 1200,        c 3300
  subcutis   k 0.16,       rho 1000,        c 2674
  blood      k 0.52,       rho 1060,        c 3770
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import api

AIR = (0.0, 0.0, 0.0, 1.0, 0.56, 1070.0, 3400.0)  # material 0: optics of air (ablated voxels)
TISSUE = (0.3, 100.0, 0.9, 1.38, 0.56, 1070.0, 3400.0)
EPIDERMIS = (1.0, 200.0, 0.8, 1.4, 0.21, 1200.0, 3590.0)
DERMIS = (0.3, 120.0, 0.9, 1.4, 0.37, 1200.0, 3300.0)
SUBCUTIS = (0.1, 80.0, 0.9, 1.4, 0.16, 1000.0, 2674.0)
BLOOD = (20.0, 300.0, 0.98, 1.4, 0.52, 1060.0, 3770.0)
INCLUSION = (2.0, 120.0, 0.9, 1.4, 0.37, 1200.0, 3300.0)


@dataclass
class Workload:
    name: str
    params: object
    config: object
    grid: np.ndarray | None = None          # u8 material ids, (nx, ny, nz) Fortran order
    packets: int = 0
    heat_steps: int = 0
    info: dict = field(default_factory=dict)

    def context(self):
        """A library context holding this workload (material grid uploaded)."""
        ctx = api.Context(self.params, self.config)
        if self.grid is not None:
            ctx.upload(api._abi.TAM_F_MATERIAL, self.grid)
        return ctx


def _config(mats, **kw):
    c = api.default_config(nmat=len(mats), **kw)
    for i, m in enumerate(mats):
        api.set_material(c, i, *m)
    return c


def _steps(mats_used, d, total_time, factor=0.9):
    amax = max(m[4] / (m[5] * m[6]) for m in mats_used)
    dt = factor / (2.0 * amax * 3.0 / (d * d))
    return int(math.ceil(total_time / dt))


def homogeneous(edge, packets, power, seconds, precision=1):
    """C1 (edge 100, 1e6 packets, 1 W, 1 s) and C2 (edge 200, 1e8, 2 W, 2 s)."""
    p = api.default_params(nxg=edge, nyg=edge, nzg=edge, xmax=0.5, ymax=0.5, zmax=0.5, mode=1, precision=precision,
                           nphotons=packets, pulse_type=1, power=power, energy_per_pixel=power * seconds * 1e3,
                           total_time=seconds, loops=1)
    c = _config([AIR, TISSUE])
    return Workload(f"homogeneous {edge}^3", p, c, None, packets, _steps([TISSUE], 1e-2 / edge, seconds))


def c1():
    return homogeneous(100, 1_000_000, 1.0, 1.0, precision=0)


def c2():
    return homogeneous(200, 100_000_000, 2.0, 2.0, precision=1)


def c3(scale=1.0, packets=100_000_000, steps=20_000):
    """Three-layer skin slab; `scale` shrinks the grid (same physical size)."""
    nx = ny = max(8, int(round(256 * scale)))
    nz = max(8, int(round(128 * scale)))
    dz = 0.5 / nz  # cm
    grid = np.full((nx, ny, nz), 3, dtype=np.uint8, order="F")  # subcutis
    ztop = lambda depth: nz - int(round(depth / dz))  # first z index below `depth` from the top face
    grid[:, :, ztop(0.21):] = 2   # dermis 0.01 .. 0.21 cm
    grid[:, :, ztop(0.01):] = 1   # epidermis, top 0.01 cm (at least one plane)
    grid[:, :, nz - 1] = 1
    mats = [AIR, EPIDERMIS, DERMIS, SUBCUTIS]
    dt_steps = steps
    # the laser stays on for the whole run: 2e4 steps of ~2.45 ms are ~49 s
    # (a 60 s top-hat pulse at 5 W)
    p = api.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=0.5, ymax=0.5, zmax=0.25, mode=1, precision=1,
                           nphotons=packets, pulse_type=1, power=5.0, energy_per_pixel=5.0 * 60.0 * 1e3,
                           total_time=60.0, loops=1)
    c = _config(mats, retrace_fraction=1e-3, retrace_check=50)
    return Workload("C3 three-layer skin slab", p, c, grid, packets, dt_steps,
                    {"grid": (nx, ny, nz), "layers_cm": (0.01, 0.2, 0.29)})


def c4_instances(n=64, seed=4, packets=10_000_000, steps=5_000, edge_range=(64, 192)):
    """Per-instance parameters of the batched form, from a seeded Philox stream."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for i in range(n):
        nx, ny, nz = (int(v) for v in rng.integers(edge_range[0], edge_range[1] + 1, size=3))
        mua = float(math.exp(rng.uniform(math.log(0.05), math.log(5.0))))
        mus = float(math.exp(rng.uniform(math.log(20.0), math.log(300.0))))
        g = float(rng.uniform(0.7, 0.95))
        power = float(rng.uniform(0.5, 5.0))
        radius = float(rng.uniform(0.05, 0.3))
        out.append(dict(edges=(nx, ny, nz), mua=mua, mus=mus, g=g, power=power, radius=radius, packets=packets,
                        steps=steps))
    return out


def c4(n=64, seed=4, packets=10_000_000, steps=5_000, edge_range=(64, 192), precision=1):
    """Workloads of the batched form (50 um voxels, so the cube edge follows the grid)."""
    ws = []
    for k, q in enumerate(c4_instances(n, seed, packets, steps, edge_range)):
        nx, ny, nz = q["edges"]
        h = 0.005  # cm
        mat = (q["mua"], q["mus"], q["g"], 1.38, 0.56, 1070.0, 3400.0)
        p = api.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2, mode=1,
                               precision=precision, nphotons=packets, pulse_type=1, power=q["power"],
                               energy_per_pixel=q["power"] * 1e3, total_time=1.0, loops=1)
        c = _config([AIR, mat], source_radius=q["radius"], retrace_fraction=0.0)
        ws.append(Workload(f"C4 instance {k}", p, c, None, packets, steps, q))
    return ws


def c5(scale=1.0, seed=5, packets=1_000_000_000, steps=100_000):
    """Large heterogeneous instance: dermis, 20 vessels, 5 inclusions; `scale` shrinks the grid."""
    n = max(16, int(round(512 * scale)))
    L = 2.0  # cm
    h = L / n
    rng = np.random.Generator(np.random.Philox(seed))
    cyl = []
    for _ in range(20):
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        cyl.append((rng.uniform(0.0, L, size=3), v, float(rng.uniform(0.01, 0.05))))
    sph = [(rng.uniform(0.1, L - 0.1, size=3), 0.1) for _ in range(5)]
    grid = np.ones((n, n, n), dtype=np.uint8, order="F")  # dermis
    c = (np.arange(n) + 0.5) * h
    X, Y = np.meshgrid(c, c, indexing="ij")
    for k in range(n):
        z = c[k]
        sl = grid[:, :, k]
        for p0, v, r in cyl:
            dx, dy, dz = X - p0[0], Y - p0[1], z - p0[2]
            t = dx * v[0] + dy * v[1] + dz * v[2]
            d2 = dx * dx + dy * dy + dz * dz - t * t
            sl[d2 <= r * r] = 2
        for p0, r in sph:
            d2 = (X - p0[0]) ** 2 + (Y - p0[1]) ** 2 + (z - p0[2]) ** 2
            sl[d2 <= r * r] = 3
    mats = [AIR, DERMIS, BLOOD, INCLUSION]
    total = 10.0  # s: 10 pulses at 1 Hz
    p = api.default_params(nxg=n, nyg=n, nzg=n, xmax=L / 2, ymax=L / 2, zmax=L / 2, mode=1, precision=1,
                           nphotons=packets, pulse_type=1, power=10.0, energy_per_pixel=10.0 * 50.0,
                           repetition_rate_1=1.0, pulses_to_do=10, total_time=total, loops=1)
    # `steps` heat steps span the 10 pulses (1e5 steps: dt = 0.1 ms, 500 steps
    # per 50 ms pulse, well inside the stability limit of the 39 um voxels);
    # the MC pass is re-run when a pulse starts if the previous one ablated
    # voxels (the fraction rule never fires at 1.0), checked every 1000 steps
    # between pulses
    cfg = _config(mats, retrace_fraction=1.0, retrace_check=1000, dt=total / steps)
    return Workload("C5 vessels and inclusions", p, cfg, grid, packets, steps,
                    {"grid": (n, n, n), "cylinders": len(cyl), "spheres": len(sph)})


# ------------------------------------------------------------ command line --
def _run_batch(a) -> None:
    """Configuration 4 at any instance count: one MC pass per instance (all of
    them through tam_batch_mc_pass, timed), warm-up batched heat steps, then
    `steps` batched steps, each part timed on the host clock (each batched call
    returns after the device has finished)."""
    import time

    ws = c4(n=a.instances, packets=a.packets, steps=a.warm + a.steps)
    ctxs = [w.context() for w in ws]
    try:
        nvox = sum(c.nx * c.ny * c.nz for c in ctxs)
        n = len(ctxs)
        forms = [1, 0] if a.compare_mc else [1]
        for on in forms:
            # the instances' MC passes: the batched transport (1) or one launch each (0)
            ctxs[0].set_tuning("batch.transport", on)
            t0 = time.perf_counter()
            api.batch_mc_pass(ctxs, [1] * n, nphotons=[a.packets] * n, streams=[0] * n)
            dt = time.perf_counter() - t0
            print(f"C4 MC ({'batched transport' if on else 'one launch per instance'}): {n} passes of {a.packets} "
                  f"packets in {dt:.3f} s = {n * a.packets / dt:.3e} photons/s", flush=True)
        ctxs[0].set_tuning("batch.transport", 1)
        if a.staged >= 0:
            ctxs[0].set_tuning("batch.staged", a.staged)
        if a.zchunk > 0:
            ctxs[0].set_tuning("batch.zchunk", a.zchunk)
        if a.autotune:
            print("batch autotune:", api.batch_autotune(ctxs, steps=20), flush=True)
        if a.warm:
            api.batch_heat_steps(ctxs, a.warm)
        t0 = time.perf_counter()
        api.batch_heat_steps(ctxs, a.steps)
        dt = time.perf_counter() - t0
        print(f"C4 batch (batch.staged {a.staged}, batch.zchunk {a.zchunk}): {len(ctxs)} instances, {nvox} voxels; "
              f"{a.steps} batched steps "
              f"after {a.warm}: "
              f"{dt * 1e3:.2f} ms = {nvox * a.steps / dt:.3e} voxel updates/s; "
              f"device errors {sum(c.device_errors() for c in ctxs)}", flush=True)
    finally:
        for c in ctxs:
            c.close()


def _run_vessels(a) -> None:
    """Configuration 5's grid at `scale`: a warm-up MC pass, then one pass of
    `packets` timed with the library's CUDA events."""
    w = c5(scale=a.scale, packets=a.packets)
    with w.context() as ctx:
        ctx.set_tuning("transport.tally32", a.tally32)
        ctx.set_tuning("transport.bricks", a.bricks)
        ctx.mc_pass(a.warm_packets, seed=1)
        ctx.mc_pass(a.packets, seed=2)
        tr, _, _ = ctx.timing()
        tl = ctx.tallies()
        n = w.params.nxg
        print(f"C5 grid {n}^3 (FP64 tally {n ** 3 * 8 / 1e6:.0f} MB), transport.tally32={a.tally32}, "
              f"transport.bricks={a.bricks}: "
              f"{a.packets} packets in {tr:.2f} ms = {a.packets / (tr * 1e-3):.3e} photons/s, "
              f"{tl['voxel_steps']:.4e} voxel steps = {tl['voxel_steps'] / (tr * 1e-3):.3e} steps/s; "
              f"device errors {ctx.device_errors()}", flush=True)


def _run_pulsed(a) -> None:
    """Configuration 5's whole coupled run at `scale`: the pulsed laser's MC
    passes (the first, then one at each pulse start after a pulse that
    ablated voxels) and every heat step, through tam_run; timed on the host
    clock, with the library's CUDA-event times of the last pass and the last
    stretch of heat steps."""
    import time

    w = c5(scale=a.scale, packets=a.packets, steps=a.steps)
    with w.context() as ctx:
        n = w.params.nxg
        t0 = time.perf_counter()
        its = ctx.run(seed=a.seed)
        dt = time.perf_counter() - t0
        st = ctx.state()
        tr, hm, hl = ctx.timing()
        T = ctx.download(api._abi.TAM_F_TEMP)
        print(f"C5 pulsed run on {n}^3: {its} outer iterations of one heat step of {st.delt:.3e} s "
              f"(simulated {st.time:.4f} s, {st.pulses_done} pulses), {st.mc_passes} MC passes of {a.packets} packets, "
              f"{st.n_ablated} voxels ablated, max T {T.max():.2f} K; wall {dt:.2f} s; last pass {tr:.1f} ms = "
              f"{a.packets / (tr * 1e-3):.3e} photons/s; device errors {ctx.device_errors()}", flush=True)


def _run_layers(a) -> None:
    """Configuration 3's coupled loop at `scale`: `steps` outer iterations of
    one heat step each, with the MC passes the re-trace rule asks for, timed
    on the host clock (the call returns after the device has finished)."""
    import time

    w = c3(scale=a.scale, packets=a.packets, steps=a.steps)
    with w.context() as ctx:
        ctx.set_tuning("transport.bricks", a.bricks)
        t0 = time.perf_counter()
        ctx.step_coupled(a.steps, seed=a.seed)
        dt = time.perf_counter() - t0
        st = ctx.state()
        T = ctx.download(api._abi.TAM_F_TEMP)
        tr, _, _ = ctx.timing()
        print(f"C3 three-layer slab {w.info['grid']}: {a.steps} heat steps of {st.delt:.3e} s (simulated "
              f"{st.time:.2f} s), {st.mc_passes} MC passes of {a.packets} packets, {st.n_ablated} voxels ablated, "
              f"max T {T.max():.1f} K; wall {dt:.2f} s; last pass {tr:.1f} ms; device errors {ctx.device_errors()}",
              flush=True)


def _run_heat(a) -> None:
    """The heat step of the homogeneous cube (configuration 2 at edge 200), of
    configuration 5's vessel grid (edge 512 at scale 1) or of configuration
    3's three-layer slab (edge 256 at scale 1; both heterogeneous: the
    class-table kernels): one MC pass for the absorbed-power field, then `steps` steps of
    each requested form launched one by one (no graph replay), timed with the
    library's CUDA events; the form used by profiles of the heat kernels."""
    if a.geometry == "vessels":
        w = c5(scale=a.edge / 512.0, packets=a.packets)
    elif a.geometry == "layers":
        w = c3(scale=a.edge / 256.0, packets=a.packets)
    else:
        w = homogeneous(a.edge, a.packets, 2.0, 2.0, precision=1)
    with w.context() as ctx:
        ctx.mc_pass(a.packets, seed=1)
        ctx.set_tuning("heat.graph", 0)
        for form in a.forms.split(","):
            ctx.set_tuning("heat.slab", 1 if form == "slab" else 0)
            ctx.heat_steps(a.steps)
            _, hm, _ = ctx.timing()
            print(f"heat {form}: {a.steps} steps of {a.edge}^3 in {hm:.3f} ms; device errors {ctx.device_errors()}",
                  flush=True)


def parser():
    """The command line of `python -m tam_gb300.workloads`."""
    import argparse

    ap = argparse.ArgumentParser(prog="python -m tam_gb300.workloads",
                                 description="Run parts of the benchmark configurations and print their timings.")
    sub = ap.add_subparsers(dest="cmd", required=True)
    b = sub.add_parser("batch", help="configuration 4: batched heat steps of seeded instances")
    b.add_argument("--instances", type=int, default=64)
    b.add_argument("--packets", type=int, default=100_000, help="packets of each instance's MC pass")
    b.add_argument("--warm", type=int, default=200, help="untimed batched steps first")
    b.add_argument("--steps", type=int, default=200, help="timed batched steps")
    b.add_argument("--autotune", action="store_true")
    b.add_argument("--compare-mc", action="store_true", help="also time the passes with one launch per instance")
    b.add_argument("--staged", type=int, default=-1, choices=[-1, 0, 1, 2, 3, 4],
                   help="batched step form (batch.staged; -1: the library's default)")
    b.add_argument("--zchunk", type=int, default=0, help="z planes per work item (batch.zchunk; 0: default)")
    v = sub.add_parser("vessels", help="configuration 5: MC transport on the vessel grid")
    v.add_argument("--scale", type=float, default=1.0, help="grid edge = 512 * scale")
    v.add_argument("--packets", type=int, default=10_000_000)
    v.add_argument("--warm-packets", type=int, default=1_000_000)
    v.add_argument("--tally32", type=int, default=-1, choices=[-1, 0, 1])
    v.add_argument("--bricks", type=int, default=-1, choices=[-1, 0, 1],
                   help="material lookups through the brick table (transport.bricks)")
    q = sub.add_parser("layers", help="configuration 3: the coupled loop on the three-layer skin slab")
    q.add_argument("--scale", type=float, default=1.0, help="grid 256 x 256 x 128 times scale")
    q.add_argument("--packets", type=int, default=100_000_000, help="packets per MC pass")
    q.add_argument("--steps", type=int, default=20_000, help="outer iterations (one heat step each)")
    q.add_argument("--seed", type=int, default=1)
    q.add_argument("--bricks", type=int, default=-1, choices=[-1, 0, 1],
                   help="material lookups through the brick table (transport.bricks)")
    r = sub.add_parser("pulsed", help="configuration 5: the whole pulsed coupled run on the vessel grid")
    r.add_argument("--scale", type=float, default=1.0, help="grid edge = 512 * scale")
    r.add_argument("--packets", type=int, default=1_000_000_000, help="packets per MC pass")
    r.add_argument("--steps", type=int, default=100_000, help="heat steps over the 10 pulses")
    r.add_argument("--seed", type=int, default=1)
    h = sub.add_parser("heat", help="the FP32 heat step (cube or vessel grid), one launch per step")
    h.add_argument("--edge", type=int, default=200)
    h.add_argument("--packets", type=int, default=1_000_000)
    h.add_argument("--steps", type=int, default=4)
    h.add_argument("--forms", default="slab,pair", help="comma list of slab / pair")
    h.add_argument("--geometry", default="cube", choices=["cube", "vessels", "layers"],
                   help="the homogeneous cube, configuration 5's vessels and inclusions at this edge, or "
                        "configuration 3's three-layer slab (edge x edge x edge / 2)")
    return ap


def main(argv=None) -> None:
    a = parser().parse_args(argv)
    {"batch": _run_batch, "vessels": _run_vessels, "layers": _run_layers, "pulsed": _run_pulsed,
     "heat": _run_heat}[a.cmd](a)


if __name__ == "__main__":
    main()
