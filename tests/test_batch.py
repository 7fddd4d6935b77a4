"""Batches of independent instances (tam_batch_step_coupled / tam_batch_run).

Each instance of a batch must end in the state it reaches when run alone:
FP64, same seeds, compared at 1e-9 relative (only the order of the FP64
tally atomics differs between runs).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instance(tam, edge, mua, mus, g, power, radius):
    half = 0.005 * edge / 2  # 50 um voxels
    p = tam.default_params(nxg=edge, nyg=edge, nzg=edge // 2, xmax=half, ymax=half, zmax=half / 2, mode=1,
                           precision=0, nphotons=20000, pulse_type=1, power=power,
                           energy_per_pixel=power * 0.05 * 1e3, total_time=0.05, loops=5)
    c = tam.default_config(source_radius=radius, retrace_fraction=0.0)
    tam.set_material(c, 1, mua, mus, g, 1.38, 0.56, 1070.0, 3400.0)
    return tam.Context(p, c)


CASES = [(32, 0.3, 100.0, 0.9, 1.0, 0.05), (48, 2.0, 50.0, 0.8, 3.0, 0.03), (40, 0.1, 200.0, 0.95, 2.0, 0.08)]
SEEDS = [11, 22, 33]


def _state(tam, ctx):
    F = tam._abi
    return ctx.download(F.TAM_F_TEMP), ctx.download(F.TAM_F_JMEAN_GLOBAL), ctx.download(F.TAM_F_TISSUE)


def test_batch_step_coupled_matches_single_runs(tam):
    alone = []
    for case, seed in zip(CASES, SEEDS):
        with _instance(tam, *case) as ctx:
            ctx.step_coupled(3, seed=seed)
            alone.append(_state(tam, ctx))
    ctxs = [_instance(tam, *case) for case in CASES]
    try:
        tam.batch_step_coupled(ctxs, 3, SEEDS)
        for ctx, want in zip(ctxs, alone):
            got = _state(tam, ctx)
            for a, b in zip(got, want):
                np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * max(np.abs(b).max(), 1e-300))
            assert got[0].max() > 310.2  # heated
    finally:
        for c in ctxs:
            c.close()


def test_batch_run_counts_and_rejects_duplicates(tam):
    ctxs = [_instance(tam, *case) for case in CASES[:2]]
    try:
        its = tam.batch_run(ctxs, SEEDS[:2], max_iters=4)
        assert its == [4, 4]
        with pytest.raises(tam.TamError):
            tam.batch_run([ctxs[0], ctxs[0]], [1, 2], max_iters=1)
    finally:
        for c in ctxs:
            c.close()


# ------------------------------------------- device-batched FP32 heat steps --
def _fp32_instance(tam, nx, ny, nz, layered, power):
    half = 0.0025 * nx  # cm: 50 um voxels
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half * ny / nx, zmax=half * nz / nx, mode=1,
                           precision=1, nphotons=20000, pulse_type=1, power=power, energy_per_pixel=power * 1e3,
                           total_time=1.0, loops=1)
    mats = [(0.0, 0.0, 0.0, 1.0, 0.026, 1.2, 1005.0), (0.3, 100.0, 0.9, 1.38, 0.56, 1070.0, 3400.0),
            (1.0, 200.0, 0.8, 1.4, 0.21, 1200.0, 3590.0)]
    c = tam.default_config(nmat=3, retrace_fraction=0.0, source_radius=0.05)
    for i, m in enumerate(mats):
        tam.set_material(c, i, *m)
    ctx = tam.Context(p, c)
    if layered:
        g = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
        g[:, :, nz - 3:] = 2
        g[nx // 3: nx // 2, :, : nz // 2] = 2
        ctx.upload(tam._abi.TAM_F_MATERIAL, g)
    rng = np.random.default_rng(nx * 1000 + ny)
    ctx.upload(tam._abi.TAM_F_JMEAN_GLOBAL, np.asfortranarray(rng.uniform(0, 1, (nx, ny, nz)) ** 2 * 4e8))
    return ctx


SHAPES = [(37, 29, 23, True, 1.0), (48, 40, 36, False, 2.0), (64, 20, 18, True, 3.0)]


@pytest.mark.parametrize("streams,staged", [(0, 2), (1, 2), (0, 3), (0, 4)])
def test_batch_heat_steps_matches_single_contexts(tam, streams, staged):
    # streams 0: the batched kernels (staged 2: 4-byte cp.async copies; 3:
    # the slab form in one cooperative launch; 4: the slab form one launch per
    # step with the rare voxels in a kernel of their own); 1: each instance's
    # own single-context steps on its stream, issued round-robin
    # (bit-identical to the single runs, so held to the same bound here)
    F = tam._abi
    want = []
    for shp in SHAPES:
        with _fp32_instance(tam, *shp) as ctx:
            ctx.heat_steps(300)
            want.append((ctx.download(F.TAM_F_TEMP), ctx.download(F.TAM_F_TISSUE), ctx.state().time))
    ctxs = [_fp32_instance(tam, *shp) for shp in SHAPES]
    try:
        ctxs[0].set_tuning("batch.streams", streams)
        ctxs[0].set_tuning("batch.staged", staged)
        tam.batch_heat_steps(ctxs, 300)
        if streams:
            for ctx, (T, _, _) in zip(ctxs, want):
                assert np.array_equal(ctx.download(F.TAM_F_TEMP), T)
        for ctx, (T, om, t) in zip(ctxs, want):
            assert ctx.device_errors() == 0
            got_T = ctx.download(F.TAM_F_TEMP)
            assert (T - 310.15).max() > 1.0
            assert np.abs(got_T - T).max() <= 1e-4
            assert np.abs(ctx.download(F.TAM_F_TISSUE) - om).max() <= 1e-4 * max(om.max(), 1e-30)
            assert ctx.state().time == pytest.approx(t, rel=1e-12)
    finally:
        for c in ctxs:
            c.close()


def test_batch_coupled_fp32_matches_single_runs(tam):
    F = tam._abi
    seeds = [5, 6, 7]
    want = []
    for shp, sd in zip(SHAPES, seeds):
        with _fp32_instance(tam, *shp) as ctx:
            ctx.step_coupled(40, seed=sd)
            want.append(ctx.download(F.TAM_F_TEMP))
    ctxs = [_fp32_instance(tam, *shp) for shp in SHAPES]
    try:
        tam.batch_step_coupled(ctxs, 40, seeds)
        for ctx, T in zip(ctxs, want):
            assert np.abs(ctx.download(F.TAM_F_TEMP) - T).max() <= 1e-4
        its = tam.batch_run(ctxs, seeds, max_iters=45)
        assert its == [45, 45, 45]
    finally:
        for c in ctxs:
            c.close()


def test_batch_device_path_with_mc_passes(tam):
    # FP32 instances that start without a source: the batched loop runs each
    # instance's MC pass (overlapped on the instances' streams), then the
    # batched heat steps; every instance ends where it ends when run alone
    F = tam._abi

    def make(shp):
        nx, ny, nz, layered, power = shp
        half = 0.0025 * nx
        p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half * ny / nx, zmax=half * nz / nx, mode=1,
                               precision=1, nphotons=20000, pulse_type=1, power=power, energy_per_pixel=power * 1e3,
                               total_time=1.0, loops=1)
        c = tam.default_config(retrace_fraction=0.0, source_radius=0.05)
        return tam.Context(p, c)

    seeds = [3, 4, 5]
    want = []
    for shp, sd in zip(SHAPES, seeds):
        with make(shp) as ctx:
            ctx.step_coupled(20, seed=sd)
            want.append((ctx.download(F.TAM_F_TEMP), ctx.download(F.TAM_F_JMEAN_GLOBAL), ctx.state().mc_passes))
    ctxs = [make(shp) for shp in SHAPES]
    try:
        tam.batch_step_coupled(ctxs, 20, seeds)
        for ctx, (T, J, passes) in zip(ctxs, want):
            assert ctx.state().mc_passes == passes == 1
            np.testing.assert_allclose(ctx.download(F.TAM_F_JMEAN_GLOBAL), J, rtol=1e-6, atol=1e-9 * J.max())
            assert np.abs(ctx.download(F.TAM_F_TEMP) - T).max() <= 1e-4
            assert (T - 310.15).max() > 0.01
    finally:
        for c in ctxs:
            c.close()


@pytest.mark.parametrize("zchunk", [0, 1, 7])
def test_batch_staged_matches_cached_loads(tam, zchunk):
    # the four forms of the batched step (neighbours by cached global loads;
    # planes staged in shared memory by cp.async, one voxel or a pair of
    # voxels per thread; the slab form) on odd, layered and uniform
    # instances, with z-chunks of one plane, a ragged last chunk and the
    # default
    F = tam._abi
    res = []
    for staged in (0, 1, 2, 3, 4):
        ctxs = [_fp32_instance(tam, *shp) for shp in SHAPES]
        try:
            for c in ctxs:
                c.set_tuning("batch.staged", staged)
                c.set_tuning("heat.zchunk", zchunk)
            tam.batch_heat_steps(ctxs, 60)
            res.append([(c.download(F.TAM_F_TEMP), c.download(F.TAM_F_TISSUE), c.device_errors()) for c in ctxs])
        finally:
            for c in ctxs:
                c.close()
    for form in res[1:]:
        for (Ta, Oa, ea), (Tb, Ob, eb) in zip(res[0], form):
            assert ea == eb == 0
            assert (Tb - 310.15).max() > 0.5
            assert np.abs(Ta - Tb).max() <= 1e-4
            assert np.abs(Oa - Ob).max() <= 1e-4 * max(Ob.max(), 1e-30)


def test_batch_autotune_restores_state(tam):
    # the batch autotuner times forms and z-chunks (and the streams form) on
    # the instances, keeps the fastest and leaves every instance's fields and
    # clock as they were
    F = tam._abi
    ctxs = [_fp32_instance(tam, *shp) for shp in SHAPES]
    try:
        tam.batch_heat_steps(ctxs, 5)
        before = [(c.download(F.TAM_F_TEMP), c.download(F.TAM_F_TISSUE), c.state().time) for c in ctxs]
        chosen = tam.batch_autotune(ctxs, steps=8)
        assert (chosen["batch.staged"], chosen["batch.zchunk"]) in [(4, 16), (4, 32), (4, 64), (3, 8), (3, 16), (3, 32),
                                                                    (2, 8), (2, 16), (2, 32), (2, 64), (1, 16), (1, 32)]
        assert chosen["batch.streams"] in (0, 1)
        for c, (T, om, t) in zip(ctxs, before):
            np.testing.assert_array_equal(c.download(F.TAM_F_TEMP), T)
            np.testing.assert_array_equal(c.download(F.TAM_F_TISSUE), om)
            assert c.state().time == t
        tam.batch_heat_steps(ctxs, 5)  # the tuned batch keeps running
        assert all(c.device_errors() == 0 for c in ctxs)
    finally:
        for c in ctxs:
            c.close()


def test_batch_run_uneven_lengths_matches_single_runs(tam):
    # instances whose loops end after different numbers of iterations: the
    # batched launches keep stepping the live ones while the finished ones
    # stay put; each ends where it ends when run alone
    F = tam._abi

    def make(shp, total_time):
        nx, ny, nz, layered, power = shp
        half = 0.0025 * nx
        p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half * ny / nx, zmax=half * nz / nx, mode=1,
                               precision=1, nphotons=20000, pulse_type=1, power=power, energy_per_pixel=power * 1e3,
                               total_time=total_time, loops=1)
        return tam.Context(p, tam.default_config(retrace_fraction=0.0, source_radius=0.05))

    times = [0.05, 0.12, 0.08]
    seeds = [7, 8, 9]
    want = []
    for shp, tt, sd in zip(SHAPES, times, seeds):
        with make(shp, tt) as ctx:
            its = ctx.run(seed=sd)
            want.append((its, ctx.download(F.TAM_F_TEMP), ctx.state().time))
    ctxs = [make(shp, tt) for shp, tt in zip(SHAPES, times)]
    try:
        its = tam.batch_run(ctxs, seeds)
        assert len(set(its)) == 3  # three different loop lengths
        for ctx, n, (its1, T, t) in zip(ctxs, its, want):
            assert n == its1
            assert ctx.state().time == pytest.approx(t, rel=1e-12)
            assert np.abs(ctx.download(F.TAM_F_TEMP) - T).max() <= 1e-4
            assert ctx.device_errors() == 0
    finally:
        for c in ctxs:
            c.close()


# ------------------------------------------------- batched MC transport --
def _c4_like(tam, n, packets, edge_range, seed=4):
    from tam_gb300 import workloads

    return [w.context() for w in workloads.c4(n=n, seed=seed, packets=packets, steps=1, edge_range=edge_range)]


def _single_pass(tam, ctx, n, seed, stream):
    F = tam._abi
    ctx.mc_pass(n, seed=seed, stream=stream)
    return ctx.download(F.TAM_F_JMEAN), ctx.download(F.TAM_F_JMEAN_GLOBAL), ctx.tallies()


EXACT_TALLIES = ("voxel_steps", "scatters", "missed", "overflow")


def _check_same_pass(got, want):
    (Jm, Jg, tl), (Jm0, Jg0, tl0) = got, want
    assert Jm0.max() > 0
    np.testing.assert_allclose(Jm, Jm0, rtol=1e-9, atol=1e-9 * Jm0.max())
    np.testing.assert_allclose(Jg, Jg0, rtol=1e-6, atol=1e-7 * Jg0.max())
    for k, v in tl0.items():
        if k in EXACT_TALLIES:
            assert tl[k] == v, k
        else:
            assert tl[k] == pytest.approx(v, rel=1e-9, abs=1e-12), k


def test_batch_mc_pass_matches_single_passes(tam):
    # uneven uniform-medium instances (edges 24..56, the batched form's
    # per-instance optics) in one launch of the batched transport, plus a
    # layered instance and an FP64 one, whose passes run alone: every
    # instance's tally equals its own pass's on the same Philox streams up to
    # the order of the FP64 atomic sums
    F = tam._abi
    N = 30000
    seeds = [101, 102, 103, 104, 105, 106, 107]
    streams = [3, 0, 7, 1, 2, 9, 4]

    def make():
        ctxs = _c4_like(tam, 5, N, (24, 56))
        ctxs.append(_fp32_instance(tam, 37, 29, 23, True, 1.0))
        p = tam.default_params(nxg=24, nyg=24, nzg=20, xmax=0.06, ymax=0.06, zmax=0.05, mode=1, precision=0,
                               nphotons=N, pulse_type=1, power=1.0, energy_per_pixel=1e3, total_time=1.0, loops=1)
        ctxs.append(tam.Context(p, tam.default_config(retrace_fraction=0.0, source_radius=0.03)))
        return ctxs

    want = []
    for i, c in enumerate(make()):
        with c:
            want.append(_single_pass(tam, c, N, seeds[i], streams[i]))
    ctxs = make()
    try:
        l0 = tam.kernel_launches()
        tam.batch_mc_pass(ctxs, seeds, nphotons=[N] * len(ctxs), streams=streams)
        # one batched transport for the five uniform instances, a transport
        # each for the other two, and a normalisation per instance
        assert tam.kernel_launches() - l0 == 1 + 2 + len(ctxs)
        for c, w in zip(ctxs, want):
            assert c.device_errors() == 0
            assert c.state().mc_passes == 1
            _check_same_pass((c.download(F.TAM_F_JMEAN), c.download(F.TAM_F_JMEAN_GLOBAL), c.tallies()), w)
    finally:
        for c in ctxs:
            c.close()


def test_batch_mc_pass_more_instances_than_one_launch(tam):
    # 70 small instances: two launches of the batched transport (64 + 6), the
    # instances' own streams (their pass counts) and per-instance packet counts
    F = tam._abi
    n = 70
    packets = [2000 + 37 * i for i in range(n)]
    seeds = [1000 + i for i in range(n)]
    want = []
    for i, c in enumerate(_c4_like(tam, n, 2000, (12, 20), seed=9)):
        with c:
            want.append(_single_pass(tam, c, packets[i], seeds[i], 0))
    ctxs = _c4_like(tam, n, 2000, (12, 20), seed=9)
    try:
        l0 = tam.kernel_launches()
        tam.batch_mc_pass(ctxs, seeds, nphotons=packets)
        assert tam.kernel_launches() - l0 == 2 + n
        for c, w in zip(ctxs, want):
            assert c.device_errors() == 0
            _check_same_pass((c.download(F.TAM_F_JMEAN), c.download(F.TAM_F_JMEAN_GLOBAL), c.tallies()), w)
    finally:
        for c in ctxs:
            c.close()


def test_batch_loop_transport_switch(tam):
    # the batched coupled loop's passes through the batched transport and
    # through one launch per instance ("batch.transport" 0) agree
    F = tam._abi
    seeds = [21, 22, 23, 24]
    res = []
    for on in (1, 0):
        ctxs = _c4_like(tam, 4, 20000, (24, 40), seed=11)
        try:
            ctxs[0].set_tuning("batch.transport", on)
            tam.batch_step_coupled(ctxs, 3, seeds)
            res.append([(c.download(F.TAM_F_JMEAN), c.download(F.TAM_F_TEMP), c.state().mc_passes) for c in ctxs])
            assert all(c.device_errors() == 0 for c in ctxs)
        finally:
            for c in ctxs:
                c.close()
    for (Ja, Ta, pa), (Jb, Tb, pb) in zip(*res):
        assert pa == pb == 1
        np.testing.assert_allclose(Ja, Jb, rtol=1e-9, atol=1e-9 * Jb.max())
        assert np.abs(Ta - Tb).max() <= 1e-4


# ------------------------------------------- slab form through the rare paths --
HOT = [(45, 24, 20, True), (37, 29, 21, False), (64, 20, 18, False)]


def _hot_ctx(tam, nx, ny, nz, layered, precision):
    # three thermal classes (air, tissue, a second tissue), random sources
    # plus a hot spot at the convective top face that boils and ablates
    mats = [(0.026, 1.2, 1005.0), (0.56, 1070.0, 3400.0), (0.21, 911.0, 2348.0)]
    d = 5e-5  # voxel spacing, m
    alpha = max(k / (r * c) for k, r, c in mats[1:])
    half = 0.0025 * nx  # cm
    p = tam.default_params(nxg=nx, nyg=ny, nzg=nz, xmax=half, ymax=half * ny / nx, zmax=half * nz / nx, mode=1,
                           precision=precision, pulse_type=1, power=1.0, energy_per_pixel=1e6, total_time=10.0)
    c = tam.default_config(nmat=3, dt=0.9 / (2 * alpha * 3 / d ** 2))
    for i, (k, rho, cp) in enumerate(mats):
        tam.set_material(c, i, 0.3, 10.0, 0.9, 1.4, k, rho, cp)
    ctx = tam.Context(p, c)
    grid = np.ones((nx, ny, nz), dtype=np.uint8, order="F")
    if layered:
        grid[:, :, :8] = 2
        grid[5:15, 3:12, 10:16] = 2
    ctx.upload(tam._abi.TAM_F_MATERIAL, grid)
    rng = np.random.default_rng(nx)
    J = np.asfortranarray(rng.uniform(0, 1, (nx, ny, nz)) ** 2 * 5e8)
    J[nx // 2 - 2:nx // 2 + 2, 10:14, nz - 4:] = 5e10
    ctx.upload(tam._abi.TAM_F_JMEAN_GLOBAL, J)
    return ctx


@pytest.mark.parametrize("staged", [3, 4])
@pytest.mark.parametrize("which", ["mixed", "uniform"])
def test_batch_slab_form_boils_and_ablates_like_fp64(tam, which, staged):
    # the slab form of the batched step (rows of 45, 37 and 64 voxels: odd
    # rows leave a half pair at the x+ face) through boiling and ablation,
    # against each instance's own FP64 steps: the same ablated voxels, 1e-3 K
    # away from the boiling threshold; "uniform" runs the batch's
    # one-class kernel, "mixed" the class-table one
    F = tam._abi
    shapes = HOT if which == "mixed" else [h for h in HOT if not h[3]]
    want = []
    for shp in shapes:
        with _hot_ctx(tam, *shp, 0) as ctx:
            T = ctx.heat_steps(300, want=True)
            want.append((T, ctx.download(F.TAM_F_TISSUE), ctx.download(F.TAM_F_Q), ctx.download(F.TAM_F_MATERIAL)))
    ctxs = [_hot_ctx(tam, *shp, 1) for shp in shapes]
    try:
        ctxs[0].set_tuning("batch.staged", staged)
        tam.batch_heat_steps(ctxs, 300)
        for ctx, (T, om, Q, mat) in zip(ctxs, want):
            assert ctx.device_errors() == 0
            # the latent-heat branch ran and the hot spot ablated
            assert (Q > 0).any() and (mat == 0).any()
            np.testing.assert_array_equal(ctx.download(F.TAM_F_MATERIAL), mat)
            got = ctx.download(F.TAM_F_TEMP)
            away = np.abs(T - 373.15) > 0.05  # voxels straddling the threshold enter the clamp a step apart
            assert np.abs(got - T)[away].max() <= 1e-3
            assert np.abs(ctx.download(F.TAM_F_TISSUE) - om).max() <= 1e-3 * max(om.max(), 1e-30)
    finally:
        for c in ctxs:
            c.close()
