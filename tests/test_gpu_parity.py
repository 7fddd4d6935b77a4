"""Parity of the CUDA library (through its C ABI) with the CPU oracle.

Tolerances, stated per test:
  * reference-mode FP64 heat path: the stencil bit-identical (the kernel
    evaluates the reference's operations in its order with explicit
    round-to-nearest), Arrhenius and the property update 1e-13 relative (the
    device exp, in the damage integral and in air's conductivity, and the C
    library's can differ in the last bit);
  * FP64 transport vs the oracle on identical Philox streams: 1e-9 relative
    per voxel (summation order of the tally differs; the reference's
    absolute-coordinate arithmetic differs from the cell-relative DDA in the
    last bits);
  * FP32 transport vs FP64 / oracle: statistical, |diff| < 4 combined batch
    standard errors for >= 99% of voxels with signal, totals within 4 SE;
  * FP32 + Kahan fused heat vs FP64 fused heat: max |dT| <= 1e-3 K.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F = None  # set by the fixture below


@pytest.fixture(scope="module", autouse=True)
def _fields(tam):
    global F
    F = tam._abi


def ref_pair(tam, orc, nx, ny, nz, precision=0, **kw):
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, precision=precision, **kw)
    okw = {k: v for k, v in kw.items()}
    o = orc.RefOracle(orc.ref_params(nx=nx, ny=ny, nz=nz, **okw))
    return tam.Context(p), o


# ------------------------------------------------------------------ RNG --
def test_philox_matches_curand_and_oracle(tam, orc):
    rng = np.random.default_rng(0)
    w = rng.integers(0, 2 ** 32, size=(4096, 6), dtype=np.uint64).astype(np.uint32)
    w[0] = 0
    w[1] = 0xFFFFFFFF
    mine, ref = tam.selftest_philox(w)
    assert np.array_equal(mine, ref)
    for q in range(0, 4096, 97):
        assert orc.philox(list(map(int, w[q, :4])), list(map(int, w[q, 4:]))) == list(map(int, mine[q]))


# ------------------------------------------------- reference heat path --
def _randomise_ref(o, ctx, rng, hot=True):
    nx, ny, nz = o.nx, o.ny, o.nz
    inter = (slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1))
    T = o.arr("temp")
    T[inter] = rng.uniform(300.0, 380.0 if hot else 360.0, (nx, ny, nz))
    for name, lo, hi in (("kappa", 0.3, 0.7), ("density", 900.0, 1200.0), ("heatcap", 2500.0, 4000.0)):
        a = o.arr(name)
        a[inter] = rng.uniform(lo, hi, (nx, ny, nz))
    o.arr("coeff")[inter] = o.st.delt / (o.arr("density")[inter] * o.arr("heatcap")[inter])
    o.arr("jmeanGLOBAL")[...] = rng.uniform(0.0, 5e9, (nx, ny, nz))
    o.arr("Q")[...] = rng.uniform(0.0, o.st.QVapor * 1.1, (nx, ny, nz))
    for f, name in ((F.TAM_F_TEMP, "temp"), (F.TAM_F_KAPPA, "kappa"), (F.TAM_F_DENSITY, "density"),
                    (F.TAM_F_HEATCAP, "heatcap"), (F.TAM_F_COEFF, "coeff"), (F.TAM_F_JMEAN_GLOBAL, "jmeanGLOBAL"),
                    (F.TAM_F_Q, "Q")):
        ctx.upload(f, o.arr(name))


def test_ref_stencil_fp64_matches_oracle(tam, orc):
    ctx, o = ref_pair(tam, orc, 20, 16, 12)
    rng = np.random.default_rng(1)
    _randomise_ref(o, ctx, rng)
    n = 6
    o.st.p.loops = n
    assert o.heat_sim(nthreads=1) == 0
    T = ctx.heat_steps(n, want=True)
    To = o.arr("temp")
    # bit-identical: both evaluate the Fortran's IEEE operations in its order
    assert np.array_equal(T.view(np.uint64), To.view(np.uint64)), np.mean(T == To)
    assert np.array_equal(ctx.download(F.TAM_F_Q).view(np.uint64), o.arr("Q").view(np.uint64))
    assert (o.arr("Q") > 0).any()
    st = ctx.state()
    assert st.time == o.st.time and st.delt == o.st.delt and st.laser_flag == o.st.laser_flag
    ctx.close()
    o.close()


def _ref_step_numpy(T, K, D, C, coeff, J, Q, st):
    """One FP64 reference heat step (src/3dFD.f90:113-187) in numpy, in the
    kernel's order of operations: float64 arithmetic is IEEE round-to-nearest
    without contraction, so the result is the kernel's, bit for bit."""
    c = (slice(1, -1),) * 3

    def sh(A, ax, o):
        idx = [slice(1, -1)] * 3
        idx[ax] = slice(1 + o, A.shape[ax] - 1 + o)
        return A[tuple(idx)]

    def face(ax, o, id2):
        kh = 0.5 * (K[c] + sh(K, ax, o))
        dh = 0.5 * (D[c] + sh(D, ax, o))
        ch = 0.5 * (C[c] + sh(C, ax, o))
        return (0.5 * (kh / (dh * ch))) * id2

    u = []
    for ax, dd in enumerate((st.dx, st.dy, st.dz)):
        id2 = 1.0 / (dd * dd)
        a, d = face(ax, -1, id2), face(ax, 1, id2)
        b = 0.5 * (a + d)
        u.append(((a * sh(T, ax, -1)) - ((2.0 * b) * T[c])) + (d * sh(T, ax, 1)))
    inc = st.delt * ((u[0] + u[1]) + u[2])
    energy = (((st.laser_on * J) * st.delt) * st.volume_voxel) + ((C[c] * st.mass_voxel) * inc)
    heat = (T[c] + inc) + ((st.laser_on * coeff[c]) * J)
    boil = (T[c] >= 373.0) & (Q < st.qvapor) & (energy > 0.0)
    qn = Q + energy
    Qn = np.where(boil, np.where(qn < st.qvapor, qn, st.qvapor), Q)
    Tn = T.copy()
    Tn[c] = np.where(boil, 373.0, heat)
    return Tn, Qn


def test_ref_stencil_fp64_bitwise_vs_numpy(tam):
    # the FP64 reference step (its exact halvings and compares on the bit
    # pattern included) against a numpy restatement of the same IEEE
    # operations: every voxel bit-identical, boiling branch active
    nx, ny, nz = 20, 16, 12
    ctx = tam.Context(tam.default_params(nxg=nx, nyg=ny, nzg=nz))
    rng = np.random.default_rng(11)
    inter = (slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1))
    f = {}
    for fld, lo, hi in ((F.TAM_F_TEMP, 300.0, 380.0), (F.TAM_F_KAPPA, 0.3, 0.7), (F.TAM_F_DENSITY, 900.0, 1200.0),
                        (F.TAM_F_HEATCAP, 2500.0, 4000.0)):
        A = ctx.download(fld)
        A[inter] = rng.uniform(lo, hi, (nx, ny, nz))
        f[fld] = A
    # a uniform block at 375 K: inside it diffusion is small and the source
    # drives the latent-heat branch (Q grows, T held at 373 K)
    f[F.TAM_F_TEMP][6:14, 5:11, 4:9] = 375.0
    st = ctx.state()
    coeff = ctx.download(F.TAM_F_COEFF)
    coeff[inter] = st.delt / (f[F.TAM_F_DENSITY][inter] * f[F.TAM_F_HEATCAP][inter])
    J = rng.uniform(0.0, 5e9, (nx, ny, nz))
    Q = rng.uniform(0.0, st.qvapor * 1.1, (nx, ny, nz))
    for fld, A in list(f.items()) + [(F.TAM_F_COEFF, coeff), (F.TAM_F_JMEAN_GLOBAL, J), (F.TAM_F_Q, Q)]:
        ctx.upload(fld, A)
    T = ctx.heat_steps(1, want=True)
    assert ctx.state().delt == st.delt and ctx.device_errors() == 0
    Tn, Qn = _ref_step_numpy(f[F.TAM_F_TEMP], f[F.TAM_F_KAPPA], f[F.TAM_F_DENSITY], f[F.TAM_F_HEATCAP], coeff,
                             J, Q, st)
    assert (Qn != Q).any() and (Tn[inter] == 373.0).any()
    assert np.array_equal(T.view(np.uint64), Tn.view(np.uint64)), np.mean(T == Tn)
    assert np.array_equal(ctx.download(F.TAM_F_Q).view(np.uint64), Qn.view(np.uint64))
    ctx.close()


@pytest.mark.parametrize("case,n", [("boiling", 6), ("smooth", 200)])
def test_ref_stencil_fp32_form_within_1mK(tam, orc, case, n):
    # reference mode with FP32 precision: the stencil's arithmetic in FP32 on
    # the FP64 temperatures (neighbour differences and the update in FP64),
    # against the FP64 oracle.  "boiling": random properties, temperatures up
    # to 380 K and Q around QVapor, a few steps (its diffusivity exceeds what
    # delt was set for, so it is not run long).  "smooth": the default
    # properties, 300-340 K and a source of up to 0.04 K per step, 200 steps,
    # all below boiling.  The latent-heat branch is a threshold: a voxel whose
    # FP32 and FP64 temperatures straddle 373 K enters it a step apart, and the
    # two then differ by that step's increment, so the long run is kept off it.
    ctx, o = ref_pair(tam, orc, 20, 16, 12, precision=1)
    rng = np.random.default_rng(1)
    if case == "boiling":
        _randomise_ref(o, ctx, rng)
    else:
        nx, ny, nz = o.nx, o.ny, o.nz
        o.arr("temp")[1:nx + 1, 1:ny + 1, 1:nz + 1] = rng.uniform(300.0, 340.0, (nx, ny, nz))
        o.arr("jmeanGLOBAL")[...] = rng.uniform(0.0, 5e7, (nx, ny, nz))
        for f, name in ((F.TAM_F_TEMP, "temp"), (F.TAM_F_JMEAN_GLOBAL, "jmeanGLOBAL")):
            ctx.upload(f, o.arr(name))
    if case == "smooth":
        # the FP32 copies of the fields are rebuilt after an upload: halfway,
        # a 20 K hot block is written into the temperatures on both sides
        n //= 2
        o.st.p.loops = n
        assert o.heat_sim(nthreads=1) == 0
        ctx.heat_steps(n)
        To = o.arr("temp")
        To[5:10, 4:8, 3:6] += 20.0
        ctx.upload(F.TAM_F_TEMP, To)
    o.st.p.loops = n
    assert o.heat_sim(nthreads=1) == 0
    T = ctx.heat_steps(n, want=True)
    To = o.arr("temp")
    dT = np.abs(T - To).max()
    assert 0.0 < dT <= 1e-3, dT
    assert (To > 373.0).any() if case == "boiling" else To.max() < 373.0
    np.testing.assert_allclose(ctx.download(F.TAM_F_Q), o.arr("Q"), rtol=1e-5, atol=1e-6 * o.arr("Q").max())
    assert ctx.state().time == o.st.time and ctx.device_errors() == 0
    ctx.close()
    o.close()


def test_ref_fp32_coupled_loop_within_mc_noise(tam):
    # the whole FP32 reference loop (FP32 transport, FP32 stencil on the FP32
    # copies, fused FP64 Arrhenius and property update) against the FP64 loop
    # on the reference's own input, 1000 outer iterations.  FP32 draws its
    # uniforms in FP32, so its packets are independent of the FP64 ones: the
    # difference must stay within the seed-to-seed Monte Carlo noise of two
    # FP64 runs plus the FP32 form's 1 mK precision target, with no offset
    def run(prec, seed):
        c = tam.Context(tam.default_params(precision=prec))
        assert c.run(seed=seed, max_iters=1000) == 1000
        T, Om = c.download(F.TAM_F_TEMP), c.download(F.TAM_F_TISSUE)
        assert c.device_errors() == 0
        c.close()
        return T, Om
    (a, oa), (b, ob), (f, of) = run(0, 1), run(0, 2), run(1, 3)
    noise = np.abs(a - b)
    assert noise.max() > 0.0
    d = np.abs(f - a)
    assert d.max() <= 3.0 * noise.max() + 1e-3, (d.max(), noise.max())
    assert d.mean() <= 2.0 * noise.mean() + 1e-4, (d.mean(), noise.mean())
    assert abs(f.mean() - a.mean()) <= 3.0 * abs(a.mean() - b.mean()) + 1e-4
    assert np.abs(of - oa).max() <= 3.0 * np.abs(oa - ob).max() + 1e-9


def test_ref_fp32_form_follows_property_updates(tam):
    # the property update writes the FP32 copies of kappa, density, heatcap
    # and coeff beside the FP64 fields: a random Q lowers the water content,
    # and with it the properties of every voxel, on the first update, and
    # the FP32 form (which reads only the copies) stays within 1 mK of the
    # FP64 form over 100 coupled heat steps and property updates below boiling
    nx, ny, nz = 20, 16, 12
    rng = np.random.default_rng(3)
    ctxs = [tam.Context(tam.default_params(nxg=nx, nyg=ny, nzg=nz, precision=p)) for p in (0, 1)]
    T = ctxs[0].download(F.TAM_F_TEMP)
    T[1:nx + 1, 1:ny + 1, 1:nz + 1] = rng.uniform(300.0, 340.0, (nx, ny, nz))
    J = rng.uniform(0.0, 5e7, (nx, ny, nz))
    Q = rng.uniform(0.0, ctxs[0].state().qvapor, (nx, ny, nz))
    for c in ctxs:
        c.upload(F.TAM_F_TEMP, T)
        c.upload(F.TAM_F_JMEAN_GLOBAL, J)
        c.upload(F.TAM_F_Q, Q)
    k0 = ctxs[0].download(F.TAM_F_KAPPA)
    for _ in range(100):
        for c in ctxs:
            c.heat_steps(1)
            c.update_props(500.0)
    k1 = ctxs[0].download(F.TAM_F_KAPPA)
    assert np.abs(k1 - k0).max() > 0.1 * np.abs(k0).max()  # the properties did change
    T64, T32 = (c.download(F.TAM_F_TEMP) for c in ctxs)
    assert T64.max() < 373.0
    dT = np.abs(T32 - T64).max()
    assert 0.0 < dT <= 1e-3, dT
    assert all(c.device_errors() == 0 for c in ctxs)
    for c in ctxs:
        c.close()


def test_ref_arrhenius_fp64_matches_oracle(tam, orc):
    ctx, o = ref_pair(tam, orc, 11, 9, 7)
    rng = np.random.default_rng(2)
    inter = (slice(1, 12), slice(1, 10), slice(1, 8))
    for it in range(30):
        o.arr("temp")[inter] = rng.uniform(320.0, 372.0, (11, 9, 7))
        ctx.upload(F.TAM_F_TEMP, o.arr("temp"))
        o.st.p.loops = 1
        assert o.heat_sim(nthreads=1) == 0
        ctx.heat_steps(1)
        ctx.upload(F.TAM_F_TEMP, o.arr("temp"))
        o.arrhenius()
        ctx.arrhenius()
    np.testing.assert_allclose(ctx.download(F.TAM_F_TISSUE), o.arr("tissue"), rtol=1e-13, atol=0)
    np.testing.assert_array_equal(ctx.download(F.TAM_F_THRESTIME), o.arr("thres"))
    assert (o.arr("thres")[..., 0] > 0).any()
    ctx.close()
    o.close()


@pytest.mark.parametrize("zero_p", [0.2, 0.6, 0.85])
def test_ref_props_fp64_matches_sequential_sweep(tam, orc, zero_p):
    nx, ny, nz = 13, 10, 9
    ctx, o = ref_pair(tam, orc, nx, ny, nz, ablate_temp=100.0)
    rng = np.random.default_rng(int(zero_p * 100))
    inter = (slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1))
    rk = o.arr("rhokap")
    rk[inter] = np.where(rng.random((nx, ny, nz)) < zero_p, 0.0, rng.uniform(170, 550, (nx, ny, nz)))
    o.arr("temp")[inter] = rng.uniform(300, 400, (nx, ny, nz))
    o.arr("Q")[...] = rng.uniform(0, o.st.QVapor * 1.2, (nx, ny, nz))
    o.arr("water")[...] = rng.uniform(0, 0.75, (nx, ny, nz))
    for f, name in ((F.TAM_F_RHOKAP, "rhokap"), (F.TAM_F_TEMP, "temp"), (F.TAM_F_Q, "Q"), (F.TAM_F_WATER, "water")):
        ctx.upload(f, o.arr(name))
    o.setup_thermal()
    ctx.update_props(100.0)
    np.testing.assert_array_equal(ctx.download(F.TAM_F_RHOKAP) == 0, o.arr("rhokap") == 0)
    for f, name in ((F.TAM_F_RHOKAP, "rhokap"), (F.TAM_F_WATER, "water"), (F.TAM_F_KAPPA, "kappa"),
                    (F.TAM_F_DENSITY, "density"), (F.TAM_F_HEATCAP, "heatcap"), (F.TAM_F_COEFF, "coeff"),
                    (F.TAM_F_ALPHA, "alpha")):
        np.testing.assert_allclose(ctx.download(f), o.arr(name), rtol=1e-13, atol=0, err_msg=name)
    ctx.close()
    o.close()


# --------------------------------------------------- reference transport --
def test_ref_mc_fp64_matches_oracle_same_streams(tam, orc):
    n = 60000
    ctx, o = ref_pair(tam, orc, 80, 80, 80, nphotons=n)  # normalisation divides by nphotons*numproc
    J = ctx.mc_pass(n, seed=12345, stream=3, want=True)
    o.photons(n, seed=12345, stream=3, nthreads=0)
    o.normalise()
    Jo = o.arr("jmeanGLOBAL")
    assert Jo.max() > 0
    np.testing.assert_allclose(J, Jo, rtol=1e-9, atol=1e-9 * Jo.max())
    np.testing.assert_allclose(ctx.download(F.TAM_F_JMEAN), o.arr("jmean"), rtol=1e-9, atol=1e-9 * o.arr("jmean").max())
    t = ctx.tallies()
    assert t["absorbed"] == pytest.approx(o.arr("jmean").sum() / n, rel=1e-12)
    assert t["scatters"] == 0 and t["overflow"] == 0
    ctx.close()
    o.close()


def _batches_gpu(ctx, n, nb, seed, stream0=0, tallies=None):
    out = []
    for b in range(nb):
        ctx.mc_pass(n, seed=seed, stream=stream0 + b)
        out.append(ctx.download(F.TAM_F_JMEAN) / n)
        if tallies is not None:
            tallies.append(ctx.tallies())
    return np.array(out)


def _stat_compare(a, b, thresh=4.0, frac=0.99, min_signal=None):
    ma, mb = a.mean(0), b.mean(0)
    sa = a.std(0, ddof=1) / math.sqrt(a.shape[0])
    sb = b.std(0, ddof=1) / math.sqrt(b.shape[0])
    se = np.sqrt(sa ** 2 + sb ** 2)
    sig = se > 0 if min_signal is None else (np.maximum(ma, mb) > min_signal) & (se > 0)
    z = np.abs(ma - mb)[sig] / se[sig]
    return (z < thresh).mean(), int(sig.sum()), ma, mb


def test_ref_mc_fp32_statistical_vs_oracle(tam, orc):
    ctx, o = ref_pair(tam, orc, 80, 80, 80, precision=1)
    nb, n = 16, 20000
    g = _batches_gpu(ctx, n, nb, seed=77)
    ob = []
    jm = o.arr("jmean")
    for b in range(nb):
        jm[...] = 0.0
        o.photons(n, seed=999, stream=b, nthreads=0)
        ob.append(jm / n)
    ob = np.array(ob)
    ok, nsig, ma, mb = _stat_compare(g, ob, min_signal=1e-4)
    assert nsig > 500
    assert ok >= 0.99, ok
    assert abs(ma.sum() - mb.sum()) / mb.sum() < 0.02
    ctx.close()
    o.close()


# ----------------------------------------------------- config transport --
def cfg_pair(tam, orc, nx, ny, nz, half, precision=0, mats=None, radius=0.1, fresnel=1, roulette=1,
             max_steps=10_000_000):
    mats = mats or [(0.0, 0.0, 0.0, 1.0), (0.3, 100.0, 0.9, 1.38)]
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half, zmax=half, mode=1, precision=precision,
                           pulse_type=1, power=1.0, energy_per_pixel=1000.0, total_time=1.0)
    c = tam.default_config(nmat=len(mats), source_radius=radius, fresnel=fresnel, roulette=roulette,
                           max_steps=max_steps)
    for i, (mua, mus, g, nn) in enumerate(mats):
        tam.set_material(c, i, mua, mus, g, nn, 0.56, 1070.0, 3400.0)
    d = orc.mc_desc(nx, ny, nz, half, half, half, materials=mats, source_radius=radius, fresnel=fresnel,
                    roulette=roulette, max_steps=max_steps)
    return tam.Context(p, c), d


def test_config_mc_fp64_matches_oracle_same_streams(tam, orc):
    ctx, d = cfg_pair(tam, orc, 24, 24, 24, 0.5)
    n = 4000
    ctx.mc_pass(n, seed=31, stream=5)
    J = ctx.download(F.TAM_F_JMEAN)
    grid = np.ones((24, 24, 24), dtype=np.uint8, order="F")
    Jo, to = orc.mc_transport(d, grid, n, seed=31, stream=5, nthreads=0)
    t = ctx.tallies()
    for k in ("specular", "reflected", "transmitted", "side", "roulette_net"):
        assert t[k] == pytest.approx(to[k] / n, rel=1e-9, abs=1e-12), k
    assert t["scatters"] == to["scatters"] and t["voxel_steps"] == to["voxel_steps"]
    rel = np.abs(J - Jo).sum() / np.abs(Jo).sum()
    assert rel < 1e-9, rel
    ctx.close()


def test_config_mc_layers_and_ablated_material(tam, orc):
    # three-layer slab with an ablated (air) pocket: material table + id grid
    mats = [(0.0, 0.0, 0.0, 1.0), (1.0, 200.0, 0.8, 1.4), (0.3, 120.0, 0.9, 1.4), (0.1, 80.0, 0.9, 1.4)]
    nx = ny = 20
    nz = 16
    ctx, d = cfg_pair(tam, orc, nx, ny, nz, 0.25, mats=mats, radius=0.08)
    grid = np.ones((nx, ny, nz), dtype=np.uint8, order="F") * 3
    grid[:, :, nz - 2:] = 1
    grid[:, :, 6:nz - 2] = 2
    grid[8:12, 8:12, nz - 3:] = 0
    ctx.upload(F.TAM_F_MATERIAL, grid)
    n = 3000
    ctx.mc_pass(n, seed=5, stream=1)
    J = ctx.download(F.TAM_F_JMEAN)
    Jo, to = orc.mc_transport(d, grid, n, seed=5, stream=1, nthreads=0)
    assert np.abs(J - Jo).sum() / np.abs(Jo).sum() < 1e-9
    assert J[9, 9, nz - 1] == 0.0  # air absorbs nothing
    rk = ctx.download(F.TAM_F_RHOKAP)
    assert rk[10, 10, nz] == 0.0 and rk[1, 1, nz] == 201.0
    ctx.close()


def test_config_mc_fp32_vs_fp64_statistical(tam, orc):
    c64, _ = cfg_pair(tam, orc, 24, 24, 24, 0.5, precision=0)
    c32, _ = cfg_pair(tam, orc, 24, 24, 24, 0.5, precision=1)
    nb, n = 16, 2000
    ta, tb = [], []
    a = _batches_gpu(c64, n, nb, seed=3, tallies=ta)
    b = _batches_gpu(c32, n, nb, seed=3, stream0=100, tallies=tb)
    ok, nsig, ma, mb = _stat_compare(a, b, min_signal=1e-5)
    assert nsig > 300
    assert ok >= 0.99, ok
    for k in ("absorbed", "reflected", "transmitted", "side"):
        xa = np.array([t[k] for t in ta])
        xb = np.array([t[k] for t in tb])
        se = math.hypot(xa.std(ddof=1), xb.std(ddof=1)) / math.sqrt(nb)
        assert abs(xa.mean() - xb.mean()) < 4 * se + 1e-6, (k, xa.mean(), xb.mean(), se)
    c64.close()
    c32.close()


# --------------------------------------------------------- fused heat ----
def fused_setup(tam, orc, nx, ny, nz, half, precision, dt, rng, jscale):
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half, zmax=half, mode=1, precision=precision,
                           pulse_type=1, power=1.0, energy_per_pixel=1e6, total_time=10.0)
    c = tam.default_config(dt=dt)
    ctx = tam.Context(p, c)
    d = 2 * half * 1e-2 / nx
    h = orc.heat_desc(nx, ny, nz, d, 2 * half * 1e-2 / ny, 2 * half * 1e-2 / nz, dt=dt)
    J = np.asfortranarray(rng.uniform(0, 1, (nx, ny, nz)) ** 2 * jscale)
    ctx.upload(F.TAM_F_JMEAN_GLOBAL, J)
    return ctx, h, J


def test_fused_fp64_matches_oracle(tam, orc):
    nx, ny, nz = 24, 20, 16
    rng = np.random.default_rng(4)
    dt = 2e-3
    ctx, h, J = fused_setup(tam, orc, nx, ny, nz, 0.12, 0, dt, rng, 2e9)
    st = dict(T=np.full((nx, ny, nz), 310.15, order="F"), k=np.full((nx, ny, nz), 0.56, order="F"),
              rho=np.full((nx, ny, nz), 1070.0, order="F"), c=np.full((nx, ny, nz), 3400.0, order="F"),
              Q=np.zeros((nx, ny, nz), order="F"), omega=np.zeros((nx, ny, nz), order="F"),
              thres=np.zeros((nx, ny, nz, 3), order="F"), mat=np.ones((nx, ny, nz), dtype=np.uint8, order="F"))
    Jo = J.copy(order="F")
    T = st["T"]
    nsteps = 40
    for s in range(nsteps):
        T, _ = orc.fused_step(h, 1.0, (s + 1) * dt, T, st["k"], st["rho"], st["c"], Jo, st["Q"], st["omega"],
                              st["thres"], st["mat"])
    Tg = ctx.heat_steps(nsteps, want=True)
    np.testing.assert_allclose(Tg[1:-1, 1:-1, 1:-1], T, rtol=1e-12, atol=0)
    assert T.max() > 320.0
    np.testing.assert_allclose(ctx.download(F.TAM_F_TISSUE), st["omega"], rtol=1e-10, atol=1e-300)
    assert st["omega"].max() > 0
    np.testing.assert_array_equal(ctx.download(F.TAM_F_MATERIAL), st["mat"])
    ctx.close()


def test_fused_fp32_kahan_within_1mK_of_fp64(tam, orc):
    nx = ny = nz = 48
    rng = np.random.default_rng(5)
    half = 0.24
    d = 2 * half * 1e-2 / nx
    alpha = 0.56 / (1070 * 3400)
    dt = 0.9 / (2 * alpha * 3 / d ** 2)
    c64, _, J = fused_setup(tam, orc, nx, ny, nz, half, 0, dt, rng, 1e8)
    c32, _, _ = fused_setup(tam, orc, nx, ny, nz, half, 1, dt, np.random.default_rng(5), 1e8)
    nsteps = 400
    T64 = c64.heat_steps(nsteps, want=True)
    T32 = c32.heat_steps(nsteps, want=True)
    rise = (T64 - 310.15).max()
    assert rise > 20.0, rise
    err = np.abs(T32 - T64).max()
    assert err <= 1e-3, err
    om64, om32 = c64.download(F.TAM_F_TISSUE), c32.download(F.TAM_F_TISSUE)
    assert np.abs(om32 - om64).max() <= 1e-3 * max(om64.max(), 1e-30) + 1e-30
    c64.close()
    c32.close()


# ------------------------------------------------------- coupled driver --
def test_coupled_reference_matches_oracle(tam, orc):
    # tophat at 8 W heats the beam column to the 100 C latent-heat clamp within a
    # few iterations, so Q, water content, rhokap and the MC source all feed back
    kw = dict(nphotons=3000, power=8.0, pulse_type=1)
    ctx, o = ref_pair(tam, orc, 16, 16, 16, **kw)
    for it in range(12):
        ctx.step_coupled(1, seed=2024)
        assert o.outer_iteration(2024, nthreads=0) == 0
    np.testing.assert_allclose(ctx.download(F.TAM_F_JMEAN_GLOBAL), o.arr("jmeanGLOBAL"), rtol=1e-9,
                               atol=1e-9 * o.arr("jmeanGLOBAL").max())
    To = o.arr("temp")
    np.testing.assert_allclose(ctx.download(F.TAM_F_TEMP), To, rtol=1e-10, atol=0)
    np.testing.assert_allclose(ctx.download(F.TAM_F_TISSUE), o.arr("tissue"), rtol=1e-8, atol=1e-300)
    np.testing.assert_array_equal(ctx.download(F.TAM_F_RHOKAP) == 0, o.arr("rhokap") == 0)
    np.testing.assert_allclose(ctx.download(F.TAM_F_RHOKAP), o.arr("rhokap"), rtol=1e-10)
    np.testing.assert_allclose(ctx.download(F.TAM_F_Q), o.arr("Q"), rtol=1e-9, atol=1e-9 * o.st.QVapor)
    assert o.arr("Q").max() > 0 and o.arr("temp").max() >= 373.0
    st = ctx.state()
    assert st.counter == o.st.counter and st.time == o.st.time
    ctx.close()
    o.close()


# --------------------------------------------------------- error paths --
def test_error_paths_and_recovery(tam, orc):
    ctx, d = cfg_pair(tam, orc, 12, 12, 12, 0.3, max_steps=3)
    with pytest.raises(tam.TamError) as e:
        ctx.mc_pass(500, seed=1)
    assert e.value.code == F.TAM_E_DEVICE
    assert ctx.device_errors() & F.TAM_DEVERR_STEP_CAP
    assert ctx.tallies()["overflow"] > 0
    with pytest.raises(tam.TamError) as e:
        ctx.arrhenius()
    assert e.value.code == F.TAM_E_STATE
    with pytest.raises(tam.TamError) as e:
        ctx.download(F.TAM_F_WATER)
    assert e.value.code == F.TAM_E_STATE
    # the context stays usable after a device-reported error
    ctx.heat_steps(2)
    ctx.close()
    p = tam.default_params(nxg=8, nyg=8, nzg=8)
    with tam.Context(p) as c2:
        bad = np.ones((10, 10, 10), order="F")
        bad[3, 3, 3] = -1.0
        with pytest.raises(tam.TamError) as e:
            c2.upload(F.TAM_F_RHOKAP, bad)
        assert e.value.code == F.TAM_E_INVALID
        import ctypes as C

        buf = np.zeros(5)
        rc = c2._lib.tam_download(c2._h, F.TAM_F_TEMP, buf.ctypes.data_as(C.c_void_p), buf.nbytes)
        assert rc == F.TAM_E_INVALID


def test_writer_files(tam, orc, tmp_path):
    p = tam.default_params(nxg=8, nyg=8, nzg=8)
    with tam.Context(p) as ctx:
        ctx.step_coupled(2, seed=1)
        ctx.finalize()
        ctx.write_output(str(tmp_path))
    names = sorted(x.name for x in tmp_path.iterdir())
    tail = "70w-8-500-400-0.030-0.030-0.060.dat"
    want = sorted([f"{k}-t{tail}" for k in ("jmean", "rhokap", "temp", "water", "tissue")] +
                  [f"time-t-{q}-{tail}" for q in (1, 2, 3)])
    assert names == want
    assert (tmp_path / f"temp-t{tail}").stat().st_size == 10 ** 3 * 8
    assert (tmp_path / f"jmean-t{tail}").stat().st_size == 8 ** 3 * 8
    t = np.fromfile(tmp_path / f"temp-t{tail}").reshape((10, 10, 10), order="F")
    assert t[0, 5, 5] == 5.0 and t[5, 5, 0] == 25.0


# ------------------------------------------- class-table fused heat step --
def _layered_heat_ctx(tam, nx, ny, nz, precision, cls, dt, J, grid, mats, rows=2, tma=1, slab=0):
    half = 0.0025 * nx  # cm: 50 um voxels
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half * ny / nx, zmax=half * nz / nx, mode=1,
                           precision=precision, pulse_type=1, power=1.0, energy_per_pixel=1e6, total_time=10.0)
    c = tam.default_config(nmat=len(mats), dt=dt)
    for i, (k, rho, cp) in enumerate(mats):
        tam.set_material(c, i, 0.3, 10.0, 0.9, 1.4, k, rho, cp)
    ctx = tam.Context(p, c)
    ctx.set_tuning("heat.cls", cls)
    ctx.set_tuning("heat.cls_rows", rows)
    ctx.set_tuning("heat.tma", tma)
    ctx.set_tuning("heat.slab", slab)
    ctx.upload(F.TAM_F_MATERIAL, grid)
    ctx.upload(F.TAM_F_JMEAN_GLOBAL, J)
    return ctx


@pytest.mark.parametrize("nx", [44, 45, 48])
def test_fused_class_table_matches_coefficient_arrays(tam, nx):
    # three thermal materials in slabs plus an inclusion; the class-table step
    # (face coefficients looked up per class pair) against the per-voxel
    # coefficient arrays (same FP32 + Kahan arithmetic up to the rounding of
    # the coefficients) and against FP64.  Rows of 45 voxels are not 16-byte
    # aligned, so every class-table case there runs the cp.async-staged step;
    # "stg" runs that step on every size (TMA off).
    ny, nz = 40, 36
    mats = [(0.026, 1.2, 1005.0), (0.56, 1070.0, 3400.0), (0.21, 911.0, 2348.0), (0.47, 1090.0, 3421.0)]
    grid = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
    grid[:, :, 12:24] = 2
    grid[:, :, :12] = 3
    grid[10:20, 8:30, 20:30] = 3
    rng = np.random.default_rng(11)
    J = np.asfortranarray(rng.uniform(0, 1, (nx, ny, nz)) ** 2 * 5e8)
    d = 5e-5  # voxel spacing, m
    alpha = max(k / (r * c) for k, r, c in mats[1:])
    dt = 0.9 / (2 * alpha * 3 / d ** 2)
    out = {}
    for name, prec, cls, rows, tma, slab in (("cls", 1, 1, 2, 1, 0), ("cls1", 1, 1, 1, 1, 0), ("cls0", 1, 1, 0, 1, 0),
                                             ("arr", 1, 0, 1, 1, 0), ("f64", 0, 1, 1, 1, 0), ("stg", 1, 1, 0, 0, 0),
                                             ("slab", 1, 1, 0, 1, 1)):
        ctx = _layered_heat_ctx(tam, nx, ny, nz, prec, cls, dt, J, grid, mats, rows, tma, slab)
        T = ctx.heat_steps(300, want=True)
        out[name] = (T, ctx.download(F.TAM_F_TISSUE), ctx.device_errors())
        ctx.close()
    rise = (out["f64"][0] - 310.15).max()
    assert rise > 5.0, rise
    assert out["cls"][2] == 0 and out["arr"][2] == 0
    assert np.abs(out["cls"][0] - out["arr"][0]).max() <= 1e-4
    assert np.abs(out["cls1"][0] - out["cls"][0]).max() <= 1e-5
    assert np.abs(out["cls0"][0] - out["cls1"][0]).max() <= 1e-5 and out["cls0"][2] == 0
    assert np.abs(out["cls"][0] - out["f64"][0]).max() <= 1e-3
    assert np.abs(out["stg"][0] - out["cls"][0]).max() <= 1e-4 and out["stg"][2] == 0
    assert np.abs(out["stg"][1] - out["cls"][1]).max() <= 1e-4 * max(out["cls"][1].max(), 1e-30)
    # the slab form (rows of 44 and 48: TMA; 45: not 16-byte aligned, the staged step runs)
    assert out["slab"][2] == 0
    assert np.abs(out["slab"][0] - out["cls"][0]).max() <= 1e-4
    assert np.abs(out["slab"][0] - out["f64"][0]).max() <= 1e-3
    assert np.abs(out["slab"][1] - out["f64"][1]).max() <= 1e-3 * max(out["f64"][1].max(), 1e-30)


@pytest.mark.parametrize("nx,layered", [(40, False), (96, False), (64, False), (40, True), (96, True), (64, True)])
def test_slab_step_matches_pair_step_and_fp64(tam, nx, layered):
    # the slab form of the class-table step (tiles of 32 x 8, so nx = 40 and 96
    # leave a partly filled last tile), uniform and layered grids, against the
    # voxel-pair form (1e-4 K) and the FP64 step (1e-3 K), 300 steps with a hot
    # spot at the convective top face that boils and ablates
    ny, nz = 24, 20
    mats = [(0.026, 1.2, 1005.0), (0.56, 1070.0, 3400.0), (0.21, 911.0, 2348.0)]
    grid = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
    if layered:
        grid[:, :, :8] = 2
        grid[5:15, 3:12, 10:16] = 2
    rng = np.random.default_rng(nx)
    J = np.asfortranarray(rng.uniform(0, 1, (nx, ny, nz)) ** 2 * 5e8)
    J[nx // 2 - 2:nx // 2 + 2, 10:14, nz - 4:] = 5e10
    d = 5e-5
    alpha = max(k / (r * c) for k, r, c in mats[1:])
    dt = 0.9 / (2 * alpha * 3 / d ** 2)
    out = {}
    for name, prec, rows, slab in (("slab", 1, 0, 1), ("pair", 1, 0, 0), ("f64", 0, 1, 0)):
        ctx = _layered_heat_ctx(tam, nx, ny, nz, prec, 1, dt, J, grid, mats, rows, 1, slab)
        T = ctx.heat_steps(300, want=True)
        out[name] = (T, ctx.download(F.TAM_F_TISSUE), ctx.device_errors(), ctx.download(F.TAM_F_Q),
                     ctx.download(F.TAM_F_MATERIAL))
        ctx.close()
    assert out["slab"][2] == 0 and out["pair"][2] == 0
    # the latent-heat branch ran and the hot spot ablated (its source then stops, so it cools again)
    assert (out["f64"][3] > 0).any() and (out["f64"][4] == 0).any()
    np.testing.assert_array_equal(out["slab"][4], out["f64"][4])
    hot = out["f64"][0] - 373.15
    away = np.abs(hot) > 0.05  # voxels straddling the boiling threshold enter the clamp a step apart
    assert np.abs(out["slab"][0] - out["pair"][0])[away].max() <= 1e-4
    assert np.abs(out["slab"][0] - out["f64"][0])[away].max() <= 1e-3
    om = out["f64"][1]
    assert np.abs(out["slab"][1] - om).max() <= 1e-3 * max(om.max(), 1e-30)


def test_slab_one_class_blocks_follow_material_changes(tam, tmp_path):
    # blocks whose tile, rim and planes hold one class take the one-class
    # update, decided from per-(tile, plane) flags of the class grid: after a
    # new material grid is uploaded, and after a state file with another grid
    # is loaded, the flags must describe the new grid.  The slab form (flags)
    # against the voxel-pair form (no flags) on the same steps, 1e-4 K; a
    # stale flag would apply one class's coefficients across an interface.
    nx, ny, nz = 64, 40, 36
    mats = [(0.026, 1.2, 1005.0), (0.56, 1070.0, 3400.0), (0.21, 911.0, 2348.0), (0.47, 1090.0, 3421.0)]
    ga = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
    ga[:, :, 12:24] = 2
    gb = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
    gb[:, 20:, :] = 3
    gb[40:50, :12, 5:30] = 2
    rng = np.random.default_rng(5)
    J = np.asfortranarray(rng.uniform(0, 1, (nx, ny, nz)) ** 2 * 2e9)
    d = 5e-5
    alpha = max(k / (r * c) for k, r, c in mats[1:])
    dt = 0.9 / (2 * alpha * 3 / d ** 2)
    ckpt = str(tmp_path / "a.state")
    out = {}
    for name, slab, rows in (("slab", 1, 0), ("pair", 0, 0)):
        ctx = _layered_heat_ctx(tam, nx, ny, nz, 1, 1, dt, J, ga, mats, rows, 1, slab)
        ctx.heat_steps(40)
        if name == "slab":
            ctx.save_state(ckpt)          # grid A
        ctx.upload(F.TAM_F_MATERIAL, gb)  # grid B: other interfaces
        ctx.upload(F.TAM_F_JMEAN_GLOBAL, J)
        tb = ctx.heat_steps(40, want=True)
        out[name] = (tb, ctx.device_errors())
        ctx.close()
    assert out["slab"][1] == 0 and out["pair"][1] == 0
    assert np.abs(out["slab"][0] - out["pair"][0]).max() <= 1e-4
    # a context holding grid B loads the state of grid A: its steps must equal
    # those of a context that never left grid A
    res = []
    for src in ("loaded", "straight"):
        ctx = _layered_heat_ctx(tam, nx, ny, nz, 1, 1, dt, J, gb if src == "loaded" else ga, mats, 0, 1, 1)
        if src == "loaded":
            ctx.heat_steps(3)
            ctx.load_state(ckpt)
        else:
            ctx.heat_steps(40)
        res.append((ctx.heat_steps(40, want=True), ctx.device_errors()))
        ctx.close()
    assert res[0][1] == 0 and res[1][1] == 0
    np.testing.assert_array_equal(res[0][0], res[1][0])


def test_fused_class_table_off_after_per_voxel_properties(tam):
    # uploading k per voxel switches the FP32 step to the coefficient arrays
    nx, ny, nz = 32, 24, 20
    mats = [(0.026, 1.2, 1005.0), (0.56, 1070.0, 3400.0)]
    grid = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
    J = np.asfortranarray(np.full((nx, ny, nz), 2e8))
    dt = 1e-3
    res = []
    for cls in (1, 0):
        ctx = _layered_heat_ctx(tam, nx, ny, nz, 1, cls, dt, J, grid, mats)
        kap = ctx.download(F.TAM_F_KAPPA)
        kap[1:-1, 1:-1, 1:nz // 2] = 0.3
        ctx.upload(F.TAM_F_KAPPA, kap)
        res.append(ctx.heat_steps(100, want=True))
        ctx.close()
    np.testing.assert_array_equal(res[0], res[1])


def test_fused_fp32_arrhenius_float_float_vs_fp64_exponent(tam, orc):
    # the FP32 step's damage integral with the float-float exponent against the
    # FP64 exponent on the same temperatures: relative 1e-6 of the largest Omega
    nx = ny = nz = 32
    half = 0.16
    d = 2 * half * 1e-2 / nx
    alpha = 0.56 / (1070 * 3400)
    dt = 0.9 / (2 * alpha * 3 / d ** 2)
    om = []
    for fp64 in (0, 1):
        ctx, _, _ = fused_setup(tam, orc, nx, ny, nz, half, 1, dt, np.random.default_rng(8), 5e7)
        ctx.set_tuning("heat.arrhenius_fp64", fp64)
        ctx.heat_steps(300)
        om.append(ctx.download(F.TAM_F_TISSUE))
        ctx.close()
    assert om[1].max() > 1e-6, om[1].max()
    assert np.abs(om[0] - om[1]).max() <= 1e-6 * om[1].max()


def test_autotune_restores_state(tam):
    # the autotuner times trial passes and steps, keeps the fastest settings and
    # leaves fields, clock and pulse state as they were
    nx = 40
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=nx, nzg=nx, xmax=half, ymax=half, zmax=half, mode=1, precision=1,
                           nphotons=20000, pulse_type=1, power=2.0, energy_per_pixel=2e3, total_time=1.0)
    with tam.Context(p, tam.default_config(source_radius=0.03)) as ctx:
        ctx.step_coupled(5, seed=2)
        before = {f: ctx.download(f) for f in (F.TAM_F_TEMP, F.TAM_F_JMEAN_GLOBAL, F.TAM_F_TISSUE, F.TAM_F_MATERIAL)}
        st0 = ctx.state()
        t0, passes0 = st0.time, st0.mc_passes
        chosen = ctx.autotune(packets=50000, steps=10)
        assert chosen["transport.scat_min"] in (12, 16, 20, 24, 28)
        assert chosen["heat.zchunk"] in (2, 3, 4, 5, 8, 16) and chosen["heat.cls_rows"] in (0, 1)
        assert chosen["heat.slab"] in (0, 1)
        for f, arr in before.items():
            np.testing.assert_array_equal(ctx.download(f), arr)
        st = ctx.state()
        assert st.time == t0 and st.mc_passes == passes0
        ctx.step_coupled(2, seed=2)  # the tuned context keeps running
        assert ctx.device_errors() == 0


@pytest.mark.parametrize("layered,box", [(False, 0), (True, 0), (False, 20 * 20 * 16), (True, 20 * 20 * 16)])
def test_fp32_tally_flushed_matches_fp64_tally(tam, layered, box):
    # FP32 transport with deposits into the FP32 tally, flushed into the FP64
    # jmean every 30000 packets (four flushes), against FP64 deposits on the
    # same Philox streams: only the rounding of the accumulation differs.
    # Uniform medium and a per-voxel material grid (two kernel forms); the
    # tally either covers the grid or is a 20 x 20 x 16 box below the beam,
    # the deposits outside it going to the FP64 jmean directly.
    nx = 40
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=nx, nzg=nx, xmax=half, ymax=half, zmax=half, mode=1, precision=1,
                           nphotons=100000)
    c = tam.default_config(source_radius=0.03, nmat=3)
    tam.set_material(c, 1, 0.3, 100.0, 0.9, 1.38, 0.56, 1070.0, 3400.0)
    tam.set_material(c, 2, 3.0, 200.0, 0.8, 1.40, 0.52, 1060.0, 3770.0)
    grid = np.ones((nx, nx, nx), dtype=np.uint8, order="F")
    if layered:
        grid[:, :, nx - 6:] = 2
        grid[10:25, 12:30, 5:20] = 2
    out = []
    for t32 in (0, 1):
        with tam.Context(p, c) as ctx:
            ctx.upload(F.TAM_F_MATERIAL, grid)
            ctx.set_tuning("transport.tally32", t32)
            ctx.set_tuning("transport.tally32_chunk", 30000)
            if box:
                ctx.set_tuning("transport.tally32_box", box)
            J = ctx.mc_pass(100000, seed=4, stream=1, want=True)
            out.append((J, ctx.tallies(), ctx.device_errors()))
    (Ja, ta, ea), (Jb, tb, eb) = out
    assert ea == eb == 0
    assert ta["voxel_steps"] == tb["voxel_steps"] and ta["scatters"] == tb["scatters"]
    assert np.abs(Ja - Jb).sum() / np.abs(Ja).sum() < 1e-6
    sig = Ja > 1e-3 * Ja.max()
    assert (np.abs(Ja - Jb)[sig] / Ja[sig]).max() < 1e-4
    if box:
        # a sizeable share of the deposits on either side of the box: both paths ran
        inside = np.zeros(Ja.shape, dtype=bool)
        inside[10:30, 10:30, nx - 16:] = True
        assert Ja[~inside].sum() > 0.1 * Ja.sum() and Ja[inside].sum() > 0.1 * Ja.sum()


def _brick_grid(nx, ny, nz):
    # one-material bricks (background, a layer), mixed bricks (a tilted
    # cylinder, layer edges off the brick boundaries), partial bricks at the
    # grid's far faces (edges not multiples of 8)
    g = np.full((nx, ny, nz), 3, dtype=np.uint8, order="F")
    g[:, :, nz - 5:] = 1
    g[:, :, 9:nz - 5] = 2
    X, Y, Z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    g[((X - 0.6 * Z - 6) ** 2 + (Y - ny / 2) ** 2) < 9.0] = 1
    return g


def test_brick_table_fp64_transport_matches_oracle(tam, orc):
    # the transport's material lookups through the 8^3 brick table (forced on
    # for a small grid) against the oracle, which reads the grid cell by cell,
    # on the same Philox streams: identical walks
    mats = [(0.0, 0.0, 0.0, 1.0), (1.0, 200.0, 0.8, 1.4), (0.3, 120.0, 0.9, 1.4), (0.1, 80.0, 0.9, 1.4)]
    nx, ny, nz = 36, 30, 28
    ctx, d = cfg_pair(tam, orc, nx, ny, nz, 0.2, mats=mats, radius=0.06)
    grid = _brick_grid(nx, ny, nz)
    ctx.upload(F.TAM_F_MATERIAL, grid)
    ctx.set_tuning("transport.bricks", 1)
    npk = 20000
    ctx.mc_pass(npk, seed=9, stream=4)
    J = ctx.download(F.TAM_F_JMEAN)
    t = ctx.tallies()
    Jo, to = orc.mc_transport(d, grid, npk, seed=9, stream=4, nthreads=0)
    assert ctx.device_errors() == 0
    assert t["scatters"] == to["scatters"] and t["voxel_steps"] == to["voxel_steps"]
    assert np.abs(J - Jo).sum() / np.abs(Jo).sum() < 1e-9
    ctx.close()


def test_brick_table_follows_material_changes(tam):
    # FP32 transport with the brick table on and off, same streams: the same
    # walks (step and scatter counts equal, tallies to the order of the FP64
    # atomic sums), on a grid with ids beyond the material table (read as 0,
    # a whole brick of id 255 included), then again after the grid changed
    # (the table is rebuilt for every pass)
    nx, ny, nz = 44, 40, 34
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half * ny / nx, zmax=half * nz / nx, mode=1,
                           precision=1, nphotons=50000)
    c = tam.default_config(source_radius=0.03, nmat=4)
    tam.set_material(c, 1, 1.0, 200.0, 0.8, 1.4, 0.56, 1070.0, 3400.0)
    tam.set_material(c, 2, 0.3, 120.0, 0.9, 1.4, 0.56, 1070.0, 3400.0)
    tam.set_material(c, 3, 0.1, 80.0, 0.9, 1.4, 0.56, 1070.0, 3400.0)
    g1 = _brick_grid(nx, ny, nz)
    g1[16:24, 8:16, 8:16] = 255
    g1[3, 30, 20] = 200
    g2 = g1.copy()
    g2[10:30, 5:35, nz - 8:] = 0  # a crater at the top, as ablation leaves it
    out = []
    for bricks in (0, 1):
        with tam.Context(p, c) as ctx:
            ctx.set_tuning("transport.bricks", bricks)
            res = []
            for g, seed in ((g1, 3), (g2, 4)):
                ctx.upload(F.TAM_F_MATERIAL, g)
                J = ctx.mc_pass(50000, seed=seed, stream=1, want=True)
                res.append((J, ctx.tallies(), ctx.device_errors()))
            out.append(res)
    for (Ja, ta, ea), (Jb, tb, eb) in zip(*out):
        assert ea == eb == 0
        assert ta["voxel_steps"] == tb["voxel_steps"] and ta["scatters"] == tb["scatters"]
        assert np.abs(Ja - Jb).sum() / np.abs(Ja).sum() < 1e-9


def test_box_tally_fp64_transport_matches_oracle(tam, orc):
    # the FP32 box tally on the FP64 transport (a 16 x 16 x 12 box under the
    # beam of a 32^3 layered grid) against the oracle on the same Philox
    # streams: paths identical, deposits summed in FP32 inside the box
    # (flushed every 5000 packets) and in FP64 outside it
    mats = [(0.0, 0.0, 0.0, 1.0), (1.0, 200.0, 0.8, 1.4), (0.3, 120.0, 0.9, 1.4), (0.1, 80.0, 0.9, 1.4)]
    n = 32
    ctx, d = cfg_pair(tam, orc, n, n, n, 0.2, mats=mats, radius=0.06)
    grid = np.full((n, n, n), 3, dtype=np.uint8, order="F")
    grid[:, :, n - 4:] = 1
    grid[:, :, 12:n - 4] = 2
    ctx.upload(F.TAM_F_MATERIAL, grid)
    ctx.set_tuning("transport.tally32", 1)
    ctx.set_tuning("transport.tally32_box", 16 * 16 * 12)
    ctx.set_tuning("transport.tally32_chunk", 5000)
    npk = 20000
    ctx.mc_pass(npk, seed=8, stream=2)
    J = ctx.download(F.TAM_F_JMEAN)
    t = ctx.tallies()
    Jo, to = orc.mc_transport(d, grid, npk, seed=8, stream=2, nthreads=0)
    assert t["scatters"] == to["scatters"] and t["voxel_steps"] == to["voxel_steps"]
    assert np.abs(J - Jo).sum() / np.abs(Jo).sum() < 1e-6
    sig = Jo > 1e-3 * Jo.max()
    assert (np.abs(J - Jo)[sig] / Jo[sig]).max() < 1e-4
    inside = np.zeros(J.shape, dtype=bool)
    inside[8:24, 8:24, n - 12:] = True
    assert Jo[~inside].sum() > 0 and Jo[inside].sum() > 0.5 * Jo.sum()
    ctx.close()


@pytest.mark.parametrize("precision,check", [(1, 5), (1, 50), (0, 50)])
def test_heat_graph_replay_matches_plain_launches(tam, precision, check):
    # heat steps replayed from CUDA graphs (chunks of 16 whose step values come
    # from a device table) against one launch per step: bit-identical fields,
    # clock and pulse state, with a pulsed source switching on and off inside
    # the run and re-trace checks every `check` steps
    nx = 32
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=nx, nzg=nx, xmax=half, ymax=half, zmax=half, mode=1, precision=precision,
                           nphotons=20000, pulse_type=1, power=20.0, energy_per_pixel=20.0 * 20.0,
                           repetition_rate_1=0.1, pulses_to_do=3, total_time=10.0, loops=1)
    # one absorbed-power field for both runs (an MC pass in FP64 sums its
    # tally with atomics, so two passes differ in the last bits)
    rng = np.random.default_rng(12)
    J = np.asfortranarray(rng.uniform(0, 1, (nx, nx, nx)) ** 4 * 2e7)
    out = []
    for graph in (0, 1):
        c = tam.default_config(source_radius=0.03, retrace_fraction=1e-3, retrace_check=check)
        with tam.Context(p, c) as ctx:
            ctx.set_tuning("heat.graph", graph)
            ctx.upload(F.TAM_F_JMEAN_GLOBAL, J)
            ctx.heat_steps(3)
            ctx.heat_steps(197)
            st = ctx.state()
            out.append((ctx.download(F.TAM_F_TEMP), ctx.download(F.TAM_F_TISSUE), st.time, st.pulses_done,
                        st.laser_flag, ctx.device_errors()))
    (Ta, Oa, ta, pa, la, ea), (Tb, Ob, tb, pb, lb, eb) = out
    assert ea == eb == 0
    assert (Ta - 310.15).max() > 0.5
    np.testing.assert_array_equal(Ta, Tb)
    np.testing.assert_array_equal(Oa, Ob)
    assert (ta, pa, la) == (tb, pb, lb) and pa >= 1


def test_ref_props_reuse_matches_full_update(tam, tmp_path):
    # a property update that keeps the skin properties of voxels whose water
    # content did not change since the previous update, against a full
    # update from the same state (restored from a checkpoint): bit-identical
    nx, ny, nz = 20, 16, 12
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, precision=0)
    rng = np.random.default_rng(4)
    T = np.full((nx + 2, ny + 2, nz + 2), 310.15, order="F")
    T[1:-1, 1:-1, 1:-1] = rng.uniform(300.0, 380.0, (nx, ny, nz))
    fields = (F.TAM_F_KAPPA, F.TAM_F_DENSITY, F.TAM_F_HEATCAP, F.TAM_F_COEFF, F.TAM_F_ALPHA, F.TAM_F_RHOKAP,
              F.TAM_F_WATER)
    with tam.Context(p) as a:
        qv = a.state().qvapor
        a.upload(F.TAM_F_TEMP, T)
        a.upload(F.TAM_F_Q, np.asfortranarray(rng.uniform(0.0, 1.1 * qv, (nx, ny, nz))))
        a.update_props(80.0)  # ablation at 80 C: the hottest voxels take air properties
        a.save_state(str(tmp_path / "state"))
        a.update_props(80.0)  # water contents unchanged: the skin properties are kept
        got = [a.download(f) for f in fields]
        assert a.device_errors() == 0
    with tam.Context(p) as b:
        b.load_state(str(tmp_path / "state"))
        b.update_props(80.0)  # every voxel recomputed
        want = [b.download(f) for f in fields]
    assert (want[5][1:-1, 1:-1, 1:-1] == 0).any() and (want[5][1:-1, 1:-1, 1:-1] > 0).any()
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


@pytest.mark.parametrize("precision", [0, 1])
def test_isolation_rule_on_cratered_slab(tam, orc, precision):
    # config.isolation = 1: after every heat step, tissue whose six neighbours
    # are air (outside the grid counts as air) turns to air and loses its
    # source (src/3dFD.f90:347-349).  A crater open to the top face holds
    # single tissue voxels (removed, one of them on the top face) and a pair
    # (kept); against the oracle's step + sequential sweep, FP64 to 1e-12 and
    # FP32 (slab form) to 1e-3 K, the material grids equal
    nx, ny, nz = 24, 20, 16
    half = 0.12
    dt = 2e-3
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half, zmax=half, mode=1, precision=precision,
                           pulse_type=1, power=1.0, energy_per_pixel=1e6, total_time=10.0)
    c = tam.default_config(dt=dt, nmat=2, isolation=1)
    tam.set_material(c, 0, 0.0, 0.0, 0.0, 1.0, 0.56, 1070.0, 3400.0)
    tam.set_material(c, 1, 0.3, 100.0, 0.9, 1.38, 0.56, 1070.0, 3400.0)
    grid = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
    grid[6:18, 5:15, 8:] = 0
    grid[10, 9, 12] = 1
    grid[14, 11, 10] = 1
    grid[12, 10, nz - 1] = 1
    grid[8, 8, 13] = grid[9, 8, 13] = 1
    rng = np.random.default_rng(31)
    J = np.asfortranarray(rng.uniform(0, 1, (nx, ny, nz)) ** 2 * 2e9)
    nsteps = 6
    with tam.Context(p, c) as ctx:
        ctx.upload(F.TAM_F_MATERIAL, grid)
        ctx.upload(F.TAM_F_JMEAN_GLOBAL, J)
        T = ctx.heat_steps(nsteps, want=True)
        mat = ctx.download(F.TAM_F_MATERIAL)
        Jg = ctx.download(F.TAM_F_JMEAN_GLOBAL)
        assert ctx.device_errors() == 0
    h = orc.heat_desc(nx, ny, nz, 2 * half * 1e-2 / nx, 2 * half * 1e-2 / ny, 2 * half * 1e-2 / nz, dt=dt)
    sh = (nx, ny, nz)
    To = np.full(sh, 310.15, order="F")
    k, rho, cc = (np.full(sh, v, order="F") for v in (0.56, 1070.0, 3400.0))
    Q, om = np.zeros(sh, order="F"), np.zeros(sh, order="F")
    thres = np.zeros(sh + (3,), order="F")
    mo = grid.copy(order="F")
    Jo = J.copy(order="F")
    removed = 0
    for s in range(nsteps):
        To, _ = orc.fused_step(h, 1.0, (s + 1) * dt, To, k, rho, cc, Jo, Q, om, thres, mo)
        removed += orc.isolate(mo, Jo)
    assert removed == 3
    assert mo[10, 9, 12] == mo[14, 11, 10] == mo[12, 10, nz - 1] == 0 and mo[8, 8, 13] == mo[9, 8, 13] == 1
    np.testing.assert_array_equal(mat, mo)
    np.testing.assert_array_equal(Jg == 0, Jo == 0)
    if precision == 0:
        np.testing.assert_allclose(T[1:-1, 1:-1, 1:-1], To, rtol=1e-12, atol=0)
    else:
        assert np.abs(T[1:-1, 1:-1, 1:-1] - To).max() <= 1e-3


def _coupled_cfg(tam, retrace, check, precision=1):
    nx = 32
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=nx, nzg=nx, xmax=half, ymax=half, zmax=half, mode=1, precision=precision,
                           nphotons=20000, pulse_type=1, power=30.0, energy_per_pixel=30.0 * 40.0,
                           repetition_rate_1=0.1, pulses_to_do=3, total_time=0.35, loops=1)
    c = tam.default_config(source_radius=0.03, retrace_fraction=retrace, retrace_check=check)
    return p, c


def test_coupled_config_loop_batched_matches_one_iteration_at_a_time(tam):
    # tam_run's config-mode loop runs the iterations between MC passes as one
    # heat-step call (steps replayed from CUDA graphs); against one iteration
    # per call with every step launched on its own: bit-identical fields,
    # clock, pulse state and counters (pulsed source switching on and off, no
    # re-trace, so no MC pass after the first and nothing summed atomically)
    out = []
    p, c = _coupled_cfg(tam, 0.0, 0)
    with tam.Context(p, c) as ctx:
        ctx.mc_pass(20000, seed=5)
        J = ctx.download(F.TAM_F_JMEAN_GLOBAL)
    for batched in (1, 0):
        p, c = _coupled_cfg(tam, 0.0, 0)
        with tam.Context(p, c) as ctx:
            ctx.upload(F.TAM_F_JMEAN_GLOBAL, J)  # no MC pass inside the loop
            if batched:
                iters = ctx.run(seed=7)
            else:
                ctx.set_tuning("heat.graph", 0)
                iters = 0
                while ctx.state().time <= ctx.state().total_time:
                    ctx.step_coupled(1, seed=7)
                    iters += 1
            st = ctx.state()
            out.append((iters, ctx.download(F.TAM_F_TEMP), ctx.download(F.TAM_F_TISSUE), st.time, st.counter,
                        st.pulses_done, st.mc_passes, ctx.device_errors()))
    (ia, Ta, Oa, ta, ca, pa, ma, ea), (ib, Tb, Ob, tb, cb, pb, mb, eb) = out
    assert ea == eb == 0 and ia == ib > 100 and pa == pb >= 2
    np.testing.assert_array_equal(Ta, Tb)
    np.testing.assert_array_equal(Oa, Ob)
    assert (ta, ca, ma) == (tb, cb, mb)


def test_coupled_config_loop_retrace_batched(tam):
    # with ablation re-traces (a check every 10 steps) the batched loop stops
    # its heat-step call after the check that asks for a new MC pass, as the
    # one-iteration loop does: the same MC passes at the same iterations (the
    # FP64 tally's atomic sums may differ in their last bits, so fields to 1e-4 K)
    out = []
    for batched in (1, 0):
        p, c = _coupled_cfg(tam, 1e-4, 10)
        c.T_abl = 320.0
        with tam.Context(p, c) as ctx:
            if not batched:
                ctx.set_tuning("heat.graph", 0)
            for _ in range(150 if not batched else 6):
                ctx.step_coupled(1 if not batched else 25, seed=9)
            st = ctx.state()
            out.append((ctx.download(F.TAM_F_TEMP), st.mc_passes, st.n_ablated, st.counter, ctx.device_errors()))
    (Ta, ma, na, ca, ea), (Tb, mb, nb, cb, eb) = out
    assert ea == eb == 0 and ca == cb
    assert ma == mb >= 3, (ma, mb)
    assert abs(na - nb) <= 2 and na > 0
    assert np.abs(Ta - Tb).max() <= 1e-4


@pytest.mark.parametrize("precision", [0, 1])
def test_reference_loop_graph_replay_matches_launches(tam, precision):
    # reference mode on the reference's own input (80^3, 125k packets per
    # pass): outer iterations replayed from CUDA graphs in runs of 16 (MC pass,
    # normalisation, heat step, damage and property update; per-iteration
    # stream, normalisation, laserOn and clock from a device table) against
    # every kernel launched: the same clock, counters and pulse state, and the
    # same fields up to the order of the tally's atomic sums (1e-12 relative)
    out = []
    for graph in (1, 0):
        p = tam.default_params(precision=precision)
        with tam.Context(p) as ctx:
            ctx.set_tuning("heat.graph", graph)
            l0 = tam.kernel_launches()
            ctx.step_coupled(96, seed=11)
            launches = tam.kernel_launches() - l0
            st = ctx.state()
            out.append(({f: ctx.download(f) for f in (F.TAM_F_TEMP, F.TAM_F_JMEAN_GLOBAL, F.TAM_F_Q, F.TAM_F_TISSUE,
                                                         F.TAM_F_RHOKAP)},
                        (st.time, st.counter, st.pulses_done, st.laser_flag, st.mc_passes), launches,
                        ctx.device_errors()))
    (fa, sa, la, ea), (fb, sb, lb, eb) = out
    assert ea == eb == 0
    assert sa == sb and sa[1] == 96 and sa[4] == 96
    assert la == lb  # the same kernels, counted whether replayed or launched
    for f in fa:
        np.testing.assert_allclose(fa[f], fb[f], rtol=1e-12, atol=1e-12 * max(np.abs(fb[f]).max(), 1e-300),
                                   err_msg=str(f))
    assert fa[F.TAM_F_JMEAN_GLOBAL].max() > 0 and fa[F.TAM_F_TEMP][1:-1, 1:-1, 1:-1].max() > 279.0
