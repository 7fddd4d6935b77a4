"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden vectors and cannot be compiled here
(no Fortran compiler), so the oracle is pinned by closed-form answers that
follow from the reference's own equations:
  * Beer-Lambert depth profile of the single-flight pure absorber
    (src/sourceph.f90:7-49 + src/inttau2.f90:7-72, kappa from src/ch_opt.f90:15-22)
  * the discrete sine-mode decay of the reference's halved stencil
    (src/3dFD.f90:119-177) and of the config-mode full operator
  * the constant-temperature Arrhenius integral and its threshold chain
    (src/3dFD.f90:424-466)
  * HG mean cosine of src/stokes.f90, Fresnel at normal incidence
  * energy balance of the config-mode transport
  * the generic (cell-relative) transport reproducing the statement-by-
    statement restatement on the reference's own geometry
  * the parallel form of setupThermalCoeff (used by the GPU) reproducing the
    sequential sweep of src/3dFD.f90:330-360.
"""
import math

import numpy as np
import pytest


# ------------------------------------------------------------------ RNG --
def test_philox_uniform_and_independent(orc):
    # uniforms in (0,1), stream/packet/event counters give distinct blocks
    seen = set()
    vals = []
    for pid in range(200):
        for ev in range(5):
            u = orc.uniforms(1234, pid, 3, ev)
            assert all(0.0 < x < 1.0 for x in u)
            seen.add(tuple(u))
            vals.extend(u)
    assert len(seen) == 1000
    v = np.array(vals)
    # chi-square on 20 bins, 4000 samples
    h, _ = np.histogram(v, bins=20, range=(0, 1))
    chi2 = ((h - 200.0) ** 2 / 200.0).sum()
    assert chi2 < 45.0  # p ~ 1e-3 for 19 dof
    assert orc.uniforms(1, 2, 3, 4) == orc.uniforms(1, 2, 3, 4)
    assert orc.uniforms(1, 2, 3, 4) != orc.uniforms(2, 2, 3, 4)


def test_philox_round_structure(orc):
    # zero key and counter do not give a zero block; one-bit changes diffuse
    a = orc.philox([0, 0, 0, 0], [0, 0])
    b = orc.philox([1, 0, 0, 0], [0, 0])
    assert a != [0, 0, 0, 0]
    flips = sum(bin(x ^ y).count("1") for x, y in zip(a, b))
    assert 40 < flips < 88


# ------------------------------------------------- Beer-Lambert (mode R) --
def test_beer_lambert_depth_profile(orc):
    p = orc.ref_params()
    o = orc.RefOracle(p)
    kappa = o.st.kappa_opt
    assert kappa == 680.0
    nb, per = 16, 12500
    jm = o.arr("jmean")
    layers = []
    for b in range(nb):
        jm[...] = 0.0
        o.photons(per, seed=99, stream=0, p0=b * per, nthreads=4)
        layers.append(jm.sum(axis=(0, 1)) / per)
    layers = np.array(layers)
    mean = layers.mean(axis=0)
    se = layers.std(axis=0, ddof=1) / math.sqrt(nb)
    nz = p.nz
    zf = np.array([(i - 1) * 2.0 * p.zmax / nz for i in range(1, nz + 2)])
    z0 = 2 * p.zmax - 1e-8 * (2 * p.zmax / nz)
    exp_ = np.zeros(nz)
    for k in range(nz):
        s_top = max(z0 - zf[k + 1], 0.0)
        s_bot = z0 - zf[k]
        exp_[k] = math.exp(-kappa * s_top) - math.exp(-kappa * s_bot)
    sig = exp_ > 1e-4
    assert sig.sum() >= 6
    z = np.abs(mean[sig] - exp_[sig]) / np.maximum(se[sig], 1e-12)
    assert z.max() < 5.0, (mean[sig], exp_[sig], se[sig])
    tot = layers.sum(axis=1)  # per packet the whole optical depth tau ~ Exp(1) is deposited
    se_tot = tot.std(ddof=1) / math.sqrt(nb)
    assert abs(tot.mean() - (1 - math.exp(-kappa * z0))) < 5 * se_tot
    o.close()


# ------------------------------------------- stencil eigen-decay (mode R) --
def test_reference_stencil_sine_mode_decay(orc):
    N = 12
    p = orc.ref_params(nx=N, ny=N, nz=N, loops=7)
    o = orc.RefOracle(p)
    kin = o.arr("kappa")[1, 1, 1]
    o.arr("kappa")[...] = kin  # homogeneous, including the halo
    Tb, A = 300.0, 2.5
    T = o.arr("temp")
    T[...] = Tb
    i = np.arange(1, N + 1)
    s = np.sin(np.pi * i / (N + 1))
    mode = s[:, None, None] * s[None, :, None] * s[None, None, :]
    T[1:N + 1, 1:N + 1, 1:N + 1] = Tb + A * mode
    o.arr("jmeanGLOBAL")[...] = 0.0
    st = o.st
    alpha = kin / (o.arr("density")[1, 1, 1] * o.arr("heatcap")[1, 1, 1])
    lam = 4 * math.sin(math.pi / (2 * (N + 1))) ** 2
    # the reference's face coefficient a = 0.5 * alpha / d^2 (src/3dFD.f90:128-129)
    rate = sum(0.5 * alpha / d ** 2 * lam for d in (st.dx, st.dy, st.dz))
    g = 1.0 - st.delt * rate
    assert o.heat_sim(nthreads=1) == 0
    got = (o.arr("temp")[1:N + 1, 1:N + 1, 1:N + 1] - Tb) / mode
    np.testing.assert_allclose(got, A * g ** 7, rtol=1e-9)
    assert abs(st.time - 7 * st.delt) < 1e-15
    o.close()


def test_reference_init_values(orc):
    o = orc.RefOracle(orc.ref_params())
    st = o.st
    # delt = 1/(alpha * sum 1/d^2) with d = 2 max 1e-2 / (N+2)  (src/3dFD.f90:249-281)
    assert abs(st.delt - 1.628e-4) / 1.628e-4 < 1e-3
    assert st.pulseLength == pytest.approx(400e-3 * 81 / 70, rel=1e-15)
    # gaussian override of total_time (src/mcpolar.f90:134-137)
    assert st.p.total_time == pytest.approx(2 * st.pulseLength * 2 * math.sqrt(2 * math.log(2)), rel=1e-15)
    T = o.arr("temp")
    assert T[0, 5, 5] == 278.0 and T[5, 5, 0] == 298.0 and T[5, 5, 81] == 298.0 and T[40, 40, 40] == 278.0
    rk = o.arr("rhokap")
    assert rk[0, 3, 3] == 0.0 and rk[3, 3, 3] == 680.0
    assert o.arr("kappa")[0, 1, 1] == pytest.approx(orc.load().orc_air_thermal_cond(298.0))
    o.close()


# ------------------------------------------------- Arrhenius (mode R) ----
def test_arrhenius_constant_temperature(orc):
    p = orc.ref_params(nx=6, ny=5, nz=4)
    o = orc.RefOracle(p)
    T = o.arr("temp")
    rng = np.random.default_rng(3)
    Tint = rng.choice([300.0, 316.0, 330.0, 350.0, 372.9, 373.0, 400.0], size=(6, 5, 4))
    T[1:7, 1:6, 1:5] = Tint
    st = o.st
    A, dE, R = 3.1e98, 6.3e5, 8.314
    om = np.zeros((6, 5, 4))
    thr = np.zeros((6, 5, 4, 3))
    for n in range(40):
        st.time = st.time + st.delt
        o.arrhenius()
        for idx in np.ndindex(6, 5, 4):
            t = Tint[idx]
            if 316.0 <= t < 373.0:
                om[idx] = om[idx] + st.delt * A * math.exp(-(dE / (R * t)))
            if thr[idx + (0,)] == 0.0 and om[idx] >= 0.53:
                thr[idx + (0,)] = st.time
            elif thr[idx + (1,)] == 0.0 and om[idx] >= 1.0:
                thr[idx + (1,)] = st.time
            elif thr[idx + (2,)] == 0.0 and om[idx] >= 1e4:
                thr[idx + (2,)] = st.time
    assert np.array_equal(o.arr("tissue"), om)
    assert np.array_equal(o.arr("thres"), thr)
    assert (thr[..., 0] > 0).any() and (thr[..., 1] > 0).any()
    o.close()


# ------------------------------------------------------ stokes / Fresnel --
@pytest.mark.parametrize("g", [0.0, 0.5, 0.9])
def test_hg_mean_cosine(orc, g):
    rng = np.random.default_rng(11)
    n = 40000
    dots = np.empty(n)
    for q in range(n):
        ct = rng.uniform(-0.999, 0.999)
        st_ = math.sqrt(1 - ct * ct)
        ph = rng.uniform(0, 2 * math.pi)
        d = [ct, st_, ph, math.cos(ph), math.sin(ph)]
        old = np.array([st_ * d[3], st_ * d[4], ct])
        u0, u1 = rng.random(2)
        r = orc.stokes(g, g * g, u0, u1, d)
        new = np.array([r[1] * r[3], r[1] * r[4], r[0]])
        dots[q] = old @ new
    se = dots.std() / math.sqrt(n)
    assert abs(dots.mean() - g) < 4.5 * se + 2e-6
    if g == 0.0:
        assert abs((dots ** 2).mean() - 1 / 3) < 0.01


def test_fresnel(orc):
    assert orc.fresnel(1.0, 1.38, 1.0) == pytest.approx(((1 - 1.38) / 2.38) ** 2, rel=1e-14)
    assert orc.fresnel(1.38, 1.0, 1.0) == pytest.approx(((1 - 1.38) / 2.38) ** 2, rel=1e-14)
    assert orc.fresnel(1.4, 1.4, 0.3) == 0.0
    # total internal reflection beyond the critical angle
    assert orc.fresnel(1.4, 1.0, 0.5) == 1.0
    assert 0.0 < orc.fresnel(1.4, 1.0, 0.9) < 1.0


# ------------------------------------------------ generic vs reference ---
def test_generic_transport_matches_reference_restatement(orc):
    p = orc.ref_params()
    o = orc.RefOracle(p)
    n = 20000
    o.photons(n, seed=5, stream=2, nthreads=1)
    jr = o.arr("jmean").copy()
    d = orc.mc_desc(p.nx, p.ny, p.nz, p.xmax, p.ymax, p.zmax, medium=orc.ORC_MED_RHOKAP, source=orc.ORC_SRC_DISK,
                    source_radius=250e-4 / 2, fresnel=0, roulette=0, rhokap_n=1.38, n_ambient=1.0,
                    nudge=o.st.delta)
    jg, tal = orc.mc_transport(d, o.arr("rhokap").copy(), n, seed=5, stream=2, nthreads=1)
    assert abs(jg.sum() - jr.sum()) / jr.sum() < 1e-12
    assert np.abs(jg - jr).max() / jr.max() < 1e-10
    assert tal["scatters"] == 0
    o.close()


# --------------------------------------------- config-mode energy balance --
def test_config_transport_energy_balance(orc):
    mats = [(0.0, 0.0, 0.0, 1.0), (1.0, 20.0, 0.8, 1.4)]
    d = orc.mc_desc(20, 20, 20, 0.5, 0.5, 0.5, materials=mats, source_radius=0.1)
    grid = np.ones((20, 20, 20), dtype=np.uint8, order="F")
    tot = []
    for b in range(8):
        jm, t = orc.mc_transport(d, grid, 2500, seed=21, stream=0, p0=b * 2500, nthreads=4)
        s = (t["absorbed"] + t["specular"] + t["reflected"] + t["transmitted"] + t["side"] + t["missed"]
             - t["roulette_net"]) / 2500
        tot.append(s)
        assert t["specular"] / 2500 == pytest.approx(((1 - 1.4) / 2.4) ** 2, rel=1e-12)
        assert t["overflow"] == 0
    tot = np.array(tot)
    se = tot.std(ddof=1) / math.sqrt(len(tot))
    assert abs(tot.mean() - 1.0) < 5 * se + 1e-3


def test_config_transport_sharding_is_exact(orc):
    # packet-id keyed streams: two disjoint ranges sum to the single run
    mats = [(0.0, 0.0, 0.0, 1.0), (0.5, 30.0, 0.9, 1.4)]
    d = orc.mc_desc(12, 12, 12, 0.3, 0.3, 0.3, materials=mats, source_radius=0.05)
    grid = np.ones((12, 12, 12), dtype=np.uint8, order="F")
    j_all, _ = orc.mc_transport(d, grid, 3000, seed=8, nthreads=1)
    j_a, _ = orc.mc_transport(d, grid, 1700, seed=8, p0=0, nthreads=1)
    j_b, _ = orc.mc_transport(d, grid, 1300, seed=8, p0=1700, nthreads=1)
    np.testing.assert_allclose(j_a + j_b, j_all, rtol=1e-12, atol=1e-15)


# ------------------------------------ parallel setupThermalCoeff == sweep --
def parallel_props(rk, T, water, Q, qv, ablate, delt, mw, mp, dens, hcap, kap, coeff, alpha):
    """The GPU's parallel map (heat.cu ref_props_kernel) written in numpy."""
    nx, ny, nz = rk.shape[0] - 2, rk.shape[1] - 2, rk.shape[2] - 2
    w = np.maximum(np.minimum(np.minimum(0.75 - 0.75 * (Q / qv), 0.75), water), 0.0)
    abl_T = ablate + 273.0
    abl = T >= abl_T
    z_old = ~(rk > 0.0)
    c = (slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1))
    back_ok = np.ones((nx, ny, nz), dtype=bool)
    for ax in range(3):
        sl = [slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1)]
        sl[ax] = slice(0, rk.shape[ax] - 2)
        sl = tuple(sl)
        zb = z_old[sl].copy()
        interior = np.ones_like(zb)
        idx = [slice(None)] * 3
        idx[ax] = 0
        interior[tuple(idx)] = False  # ghost backward neighbour: its own value only
        zb = zb | (abl[sl] & interior)
        back_ok &= zb
        slf = [slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1)]
        slf[ax] = slice(2, rk.shape[ax])
        back_ok &= z_old[tuple(slf)]
    zero = abl[c] | z_old[c] | back_ok
    rk_new = rk.copy()
    out = {}
    dn = 1000.0 / (w + 0.649 * 0.25)
    hc = 1000.0 * (4.2 * w + 1.09 * 0.25)
    kk = dn * (6.28e-4 * w + 1.17e-4 * 0.25)
    Tc = T[c]
    adn = 101.325e3 / (287.058 * Tc)
    ak = -0.188521 * np.exp(-(0.000367259 * (Tc - 273.15))) + 0.212453
    rk_new[c] = np.where(zero, 0.0, w * mw + mp)
    out["density"] = np.where(zero, adn, dn)
    out["heatcap"] = np.where(zero, 1.006e3, hc)
    out["kappa"] = np.where(zero, ak, kk)
    out["coeff"] = np.where(zero, delt / (adn * 1.006e3), delt / (dn * hc))
    out["alpha"] = np.where(zero, ak / (adn * 1.006e3), alpha[c])
    return rk_new, w, out


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_parallel_props_equals_sequential_sweep(orc, seed):
    nx, ny, nz = 9, 7, 6
    o = orc.RefOracle(orc.ref_params(nx=nx, ny=ny, nz=nz, ablate_temp=100.0))
    rng = np.random.default_rng(seed)
    rk = o.arr("rhokap")
    T = o.arr("temp")
    inter = (slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1))
    zero_p = [0.3, 0.6, 0.8, 0.9][seed]
    rk[inter] = np.where(rng.random((nx, ny, nz)) < zero_p, 0.0, rng.uniform(170, 550, (nx, ny, nz)))
    T[inter] = rng.uniform(300, 400, (nx, ny, nz))
    o.arr("Q")[...] = rng.uniform(0, o.st.QVapor * 1.2, (nx, ny, nz))
    o.arr("water")[...] = rng.uniform(0, 0.75, (nx, ny, nz))
    args = dict(rk=rk.copy(), T=T.copy(), water=o.arr("water").copy(), Q=o.arr("Q").copy(), qv=o.st.QVapor,
                ablate=100.0, delt=o.st.delt, mw=510.0, mp=170.0, dens=None, hcap=None, kap=None, coeff=None,
                alpha=o.arr("alpha").copy())
    rk_new, w, out = parallel_props(**args)
    o.setup_thermal()
    assert np.array_equal(o.arr("rhokap") == 0.0, rk_new == 0.0)
    np.testing.assert_allclose(o.arr("rhokap"), rk_new, rtol=1e-15, atol=0)
    np.testing.assert_allclose(o.arr("water"), w, rtol=1e-15, atol=0)
    for name, v in out.items():
        np.testing.assert_allclose(o.arr(name)[inter], v, rtol=1e-13, atol=0, err_msg=name)
    o.close()


# ------------------------------------------------ config-mode fused step --
def _homog(nx, ny, nz, T0=310.15, k=0.56, rho=1070.0, c=3400.0):
    sh = (nx, ny, nz)
    f = lambda v: np.full(sh, v, order="F")  # noqa: E731
    return dict(T=f(T0), k=f(k), rho=f(rho), c=f(c), J=f(0.0), Q=f(0.0), omega=f(0.0),
                thres=np.zeros(sh + (3,), order="F"), mat=np.ones(sh, dtype=np.uint8, order="F"))


def test_fused_steady_state_and_sine_decay(orc):
    N = 10
    d = 1e-4
    h = orc.heat_desc(N, N, N, d, d, d, dt=1.0, bc_type=(0,) * 6, bc_h=(0,) * 6)
    alpha = 0.56 / (1070 * 3400)
    h.dt = orc.load().orc_stable_dt(h, alpha) * 0.9
    st = _homog(N, N, N)
    Tn, nab = orc.fused_step(h, 0.0, h.dt, st["T"], st["k"], st["rho"], st["c"], st["J"], st["Q"], st["omega"],
                             st["thres"], st["mat"])
    assert nab == 0 and np.array_equal(Tn, st["T"])
    i = np.arange(1, N + 1)
    s = np.sin(np.pi * i / (N + 1))
    mode = s[:, None, None] * s[None, :, None] * s[None, None, :]
    T = np.asfortranarray(310.15 + 3.0 * mode)
    lam = 4 * math.sin(math.pi / (2 * (N + 1))) ** 2
    g = 1.0 - h.dt * 3 * alpha / d ** 2 * lam
    for n in range(5):
        T, _ = orc.fused_step(h, 0.0, h.dt * (n + 1), T, st["k"], st["rho"], st["c"], st["J"], st["Q"], st["omega"],
                              st["thres"], st["mat"])
    np.testing.assert_allclose((T - 310.15) / mode, 3.0 * g ** 5, rtol=1e-9)


def test_fused_arrhenius_and_ablation(orc):
    N = 4
    h = orc.heat_desc(N, N, N, 1e-4, 1e-4, 1e-4, dt=1e-3, bc_type=(0,) * 6, bc_h=(0,) * 6, bc_T=(340.0,) * 6,
                      boil=0, T_abl=373.15)
    st = _homog(N, N, N, T0=340.0)
    T = st["T"]
    for n in range(25):
        T, nab = orc.fused_step(h, 0.0, (n + 1) * 1e-3, T, st["k"], st["rho"], st["c"], st["J"], st["Q"],
                                st["omega"], st["thres"], st["mat"])
        assert nab == 0
    want = 25 * 1e-3 * math.exp(math.log(3.1e98) - 6.28e5 / (8.314 * 340.0))
    np.testing.assert_allclose(st["omega"], want, rtol=1e-12)
    # a voxel pushed over the ablation temperature loses its optics and source
    T2 = T.copy(order="F")
    T2[1, 2, 3] = 380.0
    st["J"][...] = 5.0
    _, nab = orc.fused_step(h, 0.0, 1.0, T2, st["k"], st["rho"], st["c"], st["J"], st["Q"], st["omega"],
                            st["thres"], st["mat"])
    assert nab >= 1 and st["mat"][1, 2, 3] == 0 and st["J"][1, 2, 3] == 0.0
    assert st["mat"].sum() == N ** 3 - nab


def test_isolation_sweep_equals_parallel_rule(orc):
    # src/3dFD.f90:347-349 sweeps k, j, i in place; the library applies the rule
    # to every voxel at once from the old grid.  The two agree because a voxel
    # that turns to air has only air around it, so no other test depends on it.
    rng = np.random.default_rng(21)
    for frac in (0.05, 0.2, 0.5):
        mat = np.asfortranarray((rng.random((13, 11, 9)) < frac).astype(np.uint8) * rng.integers(1, 4, (13, 11, 9),
                                                                                                 dtype=np.uint8))
        J = np.asfortranarray(rng.random(mat.shape))
        P = np.pad(mat, 1)  # outside the grid counts as air
        nb = (P[:-2, 1:-1, 1:-1] | P[2:, 1:-1, 1:-1] | P[1:-1, :-2, 1:-1] | P[1:-1, 2:, 1:-1] |
              P[1:-1, 1:-1, :-2] | P[1:-1, 1:-1, 2:])
        want = (mat != 0) & (nb == 0)
        m2, J2 = mat.copy(order="F"), J.copy(order="F")
        n = orc.isolate(m2, J2)
        assert n == want.sum() and want.sum() > 0
        np.testing.assert_array_equal(m2, np.where(want, 0, mat))
        np.testing.assert_array_equal(J2, np.where(want, 0.0, J))
