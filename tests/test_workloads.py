"""The heterogeneous and pulsed workloads at reduced scale.

CPU: the workload builders (sizes, layer depths, seeded instance draws).
GPU: the three-layer slab (FP32 vs FP64 transport, statistical: >= 99 % of
voxels with signal within 4 combined batch standard errors), the vessel
geometry (FP64 transport vs the oracle on identical Philox streams, 1e-9
relative L1), ablation re-tracing and the pulsed source.
"""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tissue-ablation-mc_gb300"))


def _w():
    from tam_gb300 import workloads
    return workloads


# ------------------------------------------------------------------ CPU --
def test_workload_sizes_and_layers(tam):
    w = _w()
    assert w.c1().heat_steps == 103 and w.c2().heat_steps == 821
    c3 = w.c3()
    assert c3.grid.shape == (256, 256, 128)
    col = c3.grid[0, 0, :]
    # epidermis 0.01 cm, dermis 0.2 cm on a 0.5/128 cm grid, from the top face
    assert int((col == 1).sum()) == 3 and int((col == 2).sum()) == 51 and int((col == 3).sum()) == 74
    assert col[-1] == 1 and col[0] == 3


def test_workload_batched_draws_are_seeded(tam):
    w = _w()
    a, b = w.c4_instances(), w.c4_instances()
    assert a == b and len(a) == 64
    for q in a:
        assert all(64 <= e <= 192 for e in q["edges"])
        assert 0.05 <= q["mua"] <= 5.0 and 20.0 <= q["mus"] <= 300.0 and 0.7 <= q["g"] <= 0.95
        assert 0.5 <= q["power"] <= 5.0 and 0.05 <= q["radius"] <= 0.3
    assert w.c4_instances(seed=5) != a


def test_workload_vessels_geometry(tam):
    w = _w()
    x = w.c5(scale=1 / 16)
    counts = np.bincount(x.grid.ravel(), minlength=4)
    assert x.grid.shape == (32, 32, 32)
    assert counts[0] == 0 and counts[1] > 0.9 * x.grid.size and counts[2] > 0 and counts[3] > 0


def test_workload_command_line(tam):
    p = _w().parser()
    a = p.parse_args(["batch", "--instances", "8", "--warm", "200", "--steps", "4"])
    assert (a.cmd, a.instances, a.warm, a.steps, a.autotune) == ("batch", 8, 200, 4, False)
    a = p.parse_args(["vessels", "--scale", "0.6", "--tally32", "1"])
    assert (a.cmd, a.scale, a.tally32, a.packets) == ("vessels", 0.6, 1, 10_000_000)
    with pytest.raises(SystemExit):
        p.parse_args(["vessels", "--tally32", "2"])
    a = p.parse_args(["vessels", "--bricks", "0"])
    assert (a.bricks, a.tally32) == (0, -1)
    a = p.parse_args(["layers", "--bricks", "1", "--steps", "10"])
    assert (a.cmd, a.bricks, a.steps, a.scale) == ("layers", 1, 10, 1.0)
    a = p.parse_args(["heat", "--edge", "256", "--geometry", "layers", "--forms", "slab,pair"])
    assert (a.edge, a.geometry, a.forms.split(",")) == (256, "layers", ["slab", "pair"])
    assert p.parse_args(["heat"]).geometry == "cube"
    with pytest.raises(SystemExit):
        p.parse_args(["heat", "--geometry", "sphere"])


# ------------------------------------------------------------------ GPU --
def _batches(ctx, F, n, nb, seed, stream0):
    out = []
    for b in range(nb):
        ctx.mc_pass(n, seed=seed, stream=stream0 + b)
        out.append(ctx.download(F.TAM_F_JMEAN) / n)
    return np.array(out)


@pytest.mark.gpu
def test_layered_slab_fp32_vs_fp64(tam):
    w, F = _w(), tam._abi
    res = []
    for prec in (0, 1):
        x = w.c3(scale=0.125, packets=2000)
        x.params.precision = prec
        with x.context() as ctx:
            res.append(_batches(ctx, F, 2000, 16, seed=9, stream0=100 * prec))
    a, b = res
    ma, mb = a.mean(0), b.mean(0)
    se = np.sqrt(a.var(0, ddof=1) / 16 + b.var(0, ddof=1) / 16)
    sig = (np.maximum(ma, mb) > 1e-5) & (se > 0)
    assert sig.sum() > 300
    assert (np.abs(ma - mb)[sig] / se[sig] < 4.0).mean() >= 0.99
    assert abs(ma.sum() - mb.sum()) / mb.sum() < 0.02
    # most of the energy is absorbed in the thin, strongly absorbing epidermis and the dermis
    nz = ma.shape[2]
    assert ma[:, :, nz - 3:].sum() > ma[:, :, : nz // 2].sum()


@pytest.mark.gpu
def test_vessels_fp64_matches_oracle(tam, orc):
    w, F = _w(), tam._abi
    x = w.c5(scale=1 / 16, packets=3000)
    x.params.precision = 0
    mats = [(m.mua, m.mus, m.g, m.n) for m in list(x.config.mat)[: x.config.nmat]]
    n = 3000
    with x.context() as ctx:
        ctx.mc_pass(n, seed=21, stream=3)
        J = ctx.download(F.TAM_F_JMEAN)
    p = x.params
    d = orc.mc_desc(p.nxg, p.nyg, p.nzg, p.xmax, p.ymax, p.zmax, materials=mats, source_radius=x.config.source_radius)
    Jo, _ = orc.mc_transport(d, x.grid, n, seed=21, stream=3, nthreads=0)
    assert np.abs(J - Jo).sum() / np.abs(Jo).sum() < 1e-9
    # the strongly absorbing vessels take a share of the energy out of proportion to their volume
    vessel = x.grid == 2
    assert J[vessel].sum() / J.sum() > 2 * vessel.mean()


@pytest.mark.gpu
def test_ablation_triggers_retrace(tam):
    # a hot beam on a small cube: voxels reach the ablation temperature, their
    # optics turn to air, and the MC pass is re-run once 0.1 % of the grid has ablated
    F = tam._abi
    nx = 24
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=nx, nzg=nx, xmax=half, ymax=half, zmax=half, mode=1, precision=1,
                           nphotons=20000, pulse_type=1, power=40.0, energy_per_pixel=40e3, total_time=1.0, loops=1)
    c = tam.default_config(source_radius=0.01, retrace_fraction=1e-3, retrace_check=10)
    tam.set_material(c, 1, 20.0, 50.0, 0.9, 1.38, 0.56, 1070.0, 3400.0)
    with tam.Context(p, c) as ctx:
        passes = []
        for _ in range(60):
            ctx.step_coupled(10, seed=3)
            passes.append(ctx.state().mc_passes)
        st = ctx.state()
        mat = ctx.download(F.TAM_F_MATERIAL)
        J = ctx.download(F.TAM_F_JMEAN_GLOBAL)
        assert st.n_ablated > 0.001 * nx ** 3
        assert passes[-1] >= 2          # re-traced at least once after the first pass
        assert (mat == 0).sum() == st.n_ablated
        assert np.all(J[mat == 0] == 0.0)
        assert ctx.device_errors() == 0


@pytest.mark.gpu
def test_pulsed_source_turns_off_and_cools(tam):
    # two 20 ms pulses at 1 s period: the laser is on during the pulses only
    F = tam._abi
    nx = 24
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=nx, nzg=nx, xmax=half, ymax=half, zmax=half, mode=1, precision=1,
                           nphotons=20000, pulse_type=1, power=5.0, energy_per_pixel=5.0 * 20.0,
                           repetition_rate_1=1.0, pulses_to_do=2, total_time=1.2, loops=1)
    c = tam.default_config(source_radius=0.02, retrace_fraction=0.0)
    with tam.Context(p, c) as ctx:
        dt = ctx.state().delt
        n_on = int(math.ceil(0.02 / dt))
        ctx.step_coupled(n_on + 2, seed=1)
        hot = ctx.download(F.TAM_F_TEMP).max()
        st = ctx.state()
        assert st.laser_flag == 0 and st.pulses_done == 1
        ctx.step_coupled(int(0.3 / dt), seed=1)
        cooled = ctx.download(F.TAM_F_TEMP).max()
        assert hot > 311.0 and cooled < hot
