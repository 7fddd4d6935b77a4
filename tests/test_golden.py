"""Committed regression vectors (tests/golden/*.npz, made by make_golden.py).

CPU tests: the oracle still reproduces every fixture (catches drift of the
oracle itself).  GPU tests: the CUDA library, FP64, reproduces the fixtures
with no oracle at run time, at the tolerances of the parity tests:
1e-9 relative for transport (tally summation order differs), 1e-10 for the
coupled reference loop, 1e-12 for the fused heat step; Philox bit-exact.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as mg  # noqa: E402


def fixture(name):
    with np.load(os.path.join(HERE, "golden", name + ".npz")) as d:
        return {k: d[k] for k in d.files}


def close(a, b, rtol):
    scale = max(np.abs(b).max(), 1e-300)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=rtol * scale)


# ------------------------------------------------------------ oracle (CPU) --
def test_oracle_reproduces_coupled_fixture(orc):
    g, o = fixture("coupled_ref_16"), mg.coupled(orc)
    for k in ("temp", "jmeanGLOBAL", "tissue", "rhokap", "Q"):
        close(o[k], g[k], 1e-9)
    assert int(o["counter"]) == int(g["counter"]) and float(o["time"]) == pytest.approx(float(g["time"]), rel=1e-12)


def test_oracle_reproduces_layers_fixture(orc):
    g, o = fixture("config_layers"), mg.layers(orc)
    close(o["jmean"], g["jmean"], 1e-9)
    for k in g:
        if k.startswith("tally_"):
            assert float(o[k]) == pytest.approx(float(g[k]), rel=1e-9, abs=1e-9), k


def test_oracle_reproduces_fused_fixture(orc):
    g, o = fixture("fused_24"), mg.fused(orc)
    close(o["T"], g["T"], 1e-12)
    close(o["omega"], g["omega"], 1e-9)
    np.testing.assert_array_equal(o["mat"], g["mat"])


def test_oracle_reproduces_philox_fixture(orc):
    g, o = fixture("philox"), mg.philox_case(orc)
    np.testing.assert_array_equal(o["words"], g["words"])


# ------------------------------------------------------- CUDA library (GPU) --
@pytest.mark.gpu
def test_library_coupled_reference_matches_fixture(tam):
    c, g = mg.COUPLED, fixture("coupled_ref_16")
    F = tam._abi
    p = tam.default_params(nxg=c["nx"], nyg=c["ny"], nzg=c["nz"], precision=0, nphotons=c["nphotons"],
                           power=c["power"], pulse_type=c["pulse_type"])
    with tam.Context(p) as ctx:
        for _ in range(c["iters"]):
            ctx.step_coupled(1, seed=c["seed"])
        close(ctx.download(F.TAM_F_JMEAN_GLOBAL), g["jmeanGLOBAL"], 1e-9)
        close(ctx.download(F.TAM_F_TEMP), g["temp"], 1e-10)
        close(ctx.download(F.TAM_F_RHOKAP), g["rhokap"], 1e-10)
        close(ctx.download(F.TAM_F_TISSUE), g["tissue"], 1e-8)
        close(ctx.download(F.TAM_F_Q), g["Q"], 1e-9)
        assert ctx.state().counter == int(g["counter"])


@pytest.mark.gpu
def test_library_config_layers_matches_fixture(tam):
    c, g = mg.LAYERS, fixture("config_layers")
    F = tam._abi
    p = tam.default_params(nxg=c["nx"], nyg=c["ny"], nzg=c["nz"], xmax=c["half"], ymax=c["half"], zmax=c["half"],
                           mode=1, precision=0, pulse_type=1, power=1.0, energy_per_pixel=1000.0, total_time=1.0)
    cfg = tam.default_config(nmat=len(c["mats"]), source_radius=c["radius"], fresnel=1, roulette=1)
    for i, (mua, mus, gg, nn) in enumerate(c["mats"]):
        tam.set_material(cfg, i, mua, mus, gg, nn, 0.56, 1070.0, 3400.0)
    with tam.Context(p, cfg) as ctx:
        ctx.upload(F.TAM_F_MATERIAL, mg.layers_grid())
        ctx.mc_pass(c["n"], seed=c["seed"], stream=c["stream"])
        J = ctx.download(F.TAM_F_JMEAN)
        assert np.abs(J - g["jmean"]).sum() / np.abs(g["jmean"]).sum() < 1e-9
        t = ctx.tallies()
        for k in ("specular", "reflected", "transmitted", "side"):
            assert t[k] == pytest.approx(float(g["tally_" + k]) / c["n"], rel=1e-9, abs=1e-12), k
        assert t["scatters"] == float(g["tally_scatters"])


@pytest.mark.gpu
def test_library_fused_fp64_matches_fixture(tam):
    c, g = mg.FUSED, fixture("fused_24")
    F = tam._abi
    p = tam.default_params(nxg=c["nx"], nyg=c["ny"], nzg=c["nz"], xmax=c["half"], ymax=c["half"], zmax=c["half"],
                           mode=1, precision=0, pulse_type=1, power=1.0, energy_per_pixel=1e6, total_time=10.0)
    with tam.Context(p, tam.default_config(dt=c["dt"])) as ctx:
        ctx.upload(F.TAM_F_JMEAN_GLOBAL, mg.fused_source())
        T = ctx.heat_steps(c["steps"], want=True)
        close(T[1:-1, 1:-1, 1:-1], g["T"], 1e-12)
        close(ctx.download(F.TAM_F_TISSUE), g["omega"], 1e-9)


@pytest.mark.gpu
def test_library_philox_matches_fixture(tam):
    g = fixture("philox")
    # the self-test kernel takes (ctr[4], key[2]) words per row
    words = np.concatenate([g["ctr"], g["key"]], axis=1).astype(np.uint32)
    mine, _ = tam.selftest_philox(words)
    np.testing.assert_array_equal(mine, g["words"])
