"""ctypes binding of the CPU oracle liboracle.so (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and the CPU legs of bench.py use this
module, and only to check results / as the CPU baseline: the product library never
imports it.  See tam_oracle.h for what the oracle restates and how it is
pinned.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

ORC_PULSE_GAUSSIAN, ORC_PULSE_TOPHAT, ORC_PULSE_TRIANGULAR = 0, 1, 2
ORC_SRC_DISK, ORC_SRC_GAUSSIAN = 0, 1
ORC_MED_RHOKAP, ORC_MED_MATERIAL = 0, 1
ORC_BC_DIRICHLET, ORC_BC_ROBIN = 0, 1
TALLY_NAMES = ("absorbed", "specular", "reflected", "transmitted", "side", "roulette_net", "missed",
               "voxel_steps", "scatters", "overflow")
NTALLY = len(TALLY_NAMES)
MAX_MAT = 16


class RefParams(C.Structure):
    _fields_ = [
        ("nphotons", C.c_int64),
        ("xmax", C.c_double), ("ymax", C.c_double), ("zmax", C.c_double),
        ("n1", C.c_double), ("n2", C.c_double),
        ("total_time", C.c_double),
        ("loops", C.c_int32),
        ("repetition_rate_1", C.c_double),
        ("power", C.c_double),
        ("energy_per_pixel", C.c_double),
        ("ablate_temp", C.c_double),
        ("pulses_to_do", C.c_int32),
        ("pulse_type", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("numproc", C.c_int32),
    ]


_DP = C.POINTER(C.c_double)


class RefState(C.Structure):
    _fields_ = [("p", RefParams)] + [(n, C.c_double) for n in (
        "hgg", "g2", "mua", "mus", "kappa_opt", "albedo", "mu_water", "mu_protein", "delta",
        "delt", "dx", "dy", "dz", "volumeVoxel", "massVoxel", "QVapor", "pulseLength", "realPulseLength",
        "time", "pulseCount", "repetitionCount", "laserOn")] + [
        ("laser_flag", C.c_int32), ("pulseFlag", C.c_int32), ("pulsesDone", C.c_int32), ("loops_left", C.c_int32),
        ("counter", C.c_int32), ("skinDensityInit", C.c_double), ("error", C.c_int32)] + [
        (n, _DP) for n in ("xface", "yface", "zface", "rhokap", "jmean", "jmeanGLOBAL", "temp", "tissue", "thres",
                           "kappa", "density", "heatcap", "coeff", "alpha", "Q", "water")]


class OptMat(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("mua", "mus", "g", "n")]


class McDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("xmax", C.c_double), ("ymax", C.c_double), ("zmax", C.c_double),
        ("medium", C.c_int32), ("nmat", C.c_int32), ("mat", OptMat * MAX_MAT),
        ("n_ambient", C.c_double), ("source", C.c_int32), ("source_radius", C.c_double),
        ("fresnel", C.c_int32), ("roulette", C.c_int32), ("roulette_w", C.c_double), ("roulette_m", C.c_double),
        ("rhokap_n", C.c_double), ("max_steps", C.c_int64), ("nudge", C.c_double),
    ]


class HeatDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("opscale", C.c_double), ("dt", C.c_double), ("vvox", C.c_double),
        ("boil", C.c_int32), ("T_boil", C.c_double), ("lw", C.c_double), ("T_abl", C.c_double),
        ("arrhenius", C.c_int32), ("lnA", C.c_double), ("Ea", C.c_double), ("Rgas", C.c_double),
        ("T_lo", C.c_double), ("T_hi", C.c_double), ("thr", C.c_double * 3),
        ("bc_type", C.c_int32 * 6), ("bc_T", C.c_double * 6), ("bc_h", C.c_double * 6), ("bc_Tamb", C.c_double * 6),
    ]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        from build_oracle import build  # noqa: E402  (same directory)
        build()
    L = C.CDLL(LIB)
    P = C.c_void_p
    L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.orc_philox_uniform4.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, _DP]
    L.orc_ref_create.restype = C.POINTER(RefState)
    L.orc_ref_create.argtypes = [C.POINTER(RefParams)]
    L.orc_ref_free.argtypes = [C.POINTER(RefState)]
    L.orc_ref_photons.argtypes = [C.POINTER(RefState), C.c_int64, C.c_int64, C.c_uint64, C.c_uint32, C.c_int]
    L.orc_ref_normalise.argtypes = [C.POINTER(RefState)]
    L.orc_ref_get_pwr.restype = C.c_double
    L.orc_ref_get_pwr.argtypes = [C.POINTER(RefState)]
    L.orc_ref_heat_sim.argtypes = [C.POINTER(RefState), C.c_int]
    L.orc_ref_arrhenius.argtypes = [C.POINTER(RefState)]
    L.orc_ref_setup_thermal.argtypes = [C.POINTER(RefState)]
    L.orc_ref_outer_iteration.argtypes = [C.POINTER(RefState), C.c_uint64, C.c_int]
    L.orc_ref_run.restype = C.c_int64
    L.orc_ref_run.argtypes = [C.POINTER(RefState), C.c_uint64, C.c_int64, C.c_int]
    L.orc_ref_finalize.argtypes = [C.POINTER(RefState)]
    for f in ("orc_air_thermal_cond", "orc_air_density", "orc_skin_density", "orc_skin_heat_cap"):
        getattr(L, f).restype = C.c_double
        getattr(L, f).argtypes = [C.c_double]
    L.orc_skin_thermal_cond.restype = C.c_double
    L.orc_skin_thermal_cond.argtypes = [C.c_double, C.c_double]
    L.orc_water_content.restype = C.c_double
    L.orc_water_content.argtypes = [C.c_double, C.c_double, C.c_double]
    L.orc_stokes.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, _DP]
    L.orc_mc_transport.argtypes = [C.POINTER(McDesc), P, C.c_int64, C.c_int64, C.c_uint64, C.c_uint32, C.c_int,
                                   _DP, _DP]
    L.orc_fresnel.restype = C.c_double
    L.orc_fresnel.argtypes = [C.c_double, C.c_double, C.c_double]
    L.orc_fused_step.restype = C.c_int64
    L.orc_fused_step.argtypes = [C.POINTER(HeatDesc), C.c_double, C.c_double, _DP, _DP, _DP, _DP, _DP, _DP, _DP,
                                 _DP, _DP, C.POINTER(C.c_uint8), C.c_int]
    L.orc_isolate.restype = C.c_int64
    L.orc_isolate.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint8), _DP]
    L.orc_stable_dt.restype = C.c_double
    L.orc_stable_dt.argtypes = [C.POINTER(HeatDesc), C.c_double]
    _lib = L
    return L


def dp(a: np.ndarray):
    # grids are Fortran-ordered (x fastest) like the reference's arrays
    if a.dtype != np.float64 or not a.flags.f_contiguous:
        raise ValueError("oracle arrays must be float64 and Fortran-ordered")
    return a.ctypes.data_as(_DP)


def philox(ctr, key):
    L = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    L.orc_philox4x32_10(c, k, o)
    return list(o)


def uniforms(seed: int, pid: int, stream: int, ev: int):
    u = (C.c_double * 4)()
    load().orc_philox_uniform4(seed, pid, stream, ev, u)
    return list(u)


def ref_params(**kw) -> RefParams:
    """The shipped res/input.params on the 80^3 grid (src/constants.f90:12)."""
    p = RefParams(nphotons=125000, xmax=0.03, ymax=0.03, zmax=0.06, n1=1.0, n2=1.38, total_time=2.0, loops=1,
                  repetition_rate_1=1e7, power=70.0, energy_per_pixel=400.0, ablate_temp=500.0, pulses_to_do=1,
                  pulse_type=ORC_PULSE_GAUSSIAN, nx=80, ny=80, nz=80, numproc=1)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class RefOracle:
    """Reference-mode state (module globals of the Fortran) owned by C."""

    def __init__(self, p: RefParams):
        self.L = load()
        self.p = p
        self.s = self.L.orc_ref_create(C.byref(p))
        if not self.s:
            raise RuntimeError("orc_ref_create failed")
        self.nx, self.ny, self.nz = p.nx, p.ny, p.nz

    def close(self):
        if self.s:
            self.L.orc_ref_free(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def st(self) -> RefState:
        return self.s.contents

    def arr(self, name: str) -> np.ndarray:
        """Live numpy view (Fortran order) of a module array."""
        halo = name in ("rhokap", "temp", "kappa", "density", "heatcap", "coeff", "alpha")
        if halo:
            shape = (self.nx + 2, self.ny + 2, self.nz + 2)
        elif name == "thres":
            shape = (self.nx, self.ny, self.nz, 3)
        else:
            shape = (self.nx, self.ny, self.nz)
        n = int(np.prod(shape))
        ptr = getattr(self.st, name)
        return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(shape, order="F")

    def photons(self, n, seed, stream=0, p0=0, nthreads=0):
        self.L.orc_ref_photons(self.s, p0, n, seed, stream, nthreads)

    def normalise(self):
        self.L.orc_ref_normalise(self.s)

    def heat_sim(self, nthreads=0):
        return self.L.orc_ref_heat_sim(self.s, nthreads)

    def arrhenius(self):
        self.L.orc_ref_arrhenius(self.s)

    def setup_thermal(self):
        self.L.orc_ref_setup_thermal(self.s)

    def outer_iteration(self, seed, nthreads=0):
        return self.L.orc_ref_outer_iteration(self.s, seed, nthreads)

    def run(self, seed, max_iters=0, nthreads=0):
        return self.L.orc_ref_run(self.s, seed, max_iters, nthreads)

    def finalize(self):
        self.L.orc_ref_finalize(self.s)


def mc_desc(nx, ny, nz, xmax, ymax, zmax, materials=None, medium=ORC_MED_MATERIAL, n_ambient=1.0,
            source=ORC_SRC_GAUSSIAN, source_radius=0.1, fresnel=1, roulette=1, roulette_w=1e-4, roulette_m=10.0,
            rhokap_n=1.38, max_steps=10_000_000, nudge=0.0) -> McDesc:
    d = McDesc(nx=nx, ny=ny, nz=nz, xmax=xmax, ymax=ymax, zmax=zmax, medium=medium, n_ambient=n_ambient,
               source=source, source_radius=source_radius, fresnel=fresnel, roulette=roulette,
               roulette_w=roulette_w, roulette_m=roulette_m, rhokap_n=rhokap_n, max_steps=max_steps, nudge=nudge)
    mats = materials or [(0.0, 0.0, 0.0, 1.0)]
    d.nmat = len(mats)
    for i, (mua, mus, g, n) in enumerate(mats):
        d.mat[i] = OptMat(mua, mus, g, n)
    return d


def mc_transport(desc: McDesc, grid: np.ndarray, n: int, seed: int, stream: int = 0, p0: int = 0, nthreads: int = 0):
    """Returns (jmean interior F-order in packet units, tallies dict of raw sums)."""
    L = load()
    jm = np.zeros((desc.nx, desc.ny, desc.nz), order="F")
    tal = np.zeros(NTALLY)
    g = np.asfortranarray(grid)
    L.orc_mc_transport(C.byref(desc), g.ctypes.data_as(C.c_void_p), p0, n, seed, stream, nthreads, dp(jm), dp(tal))
    return jm, dict(zip(TALLY_NAMES, tal.tolist()))


def stokes(hgg, g2, u0, u1, d5):
    a = (C.c_double * 5)(*d5)
    load().orc_stokes(hgg, g2, u0, u1, a)
    return list(a)


def fresnel(n1, n2, cosi):
    return load().orc_fresnel(n1, n2, cosi)


def heat_desc(nx, ny, nz, dx, dy, dz, dt, opscale=1.0, boil=1, T_boil=373.15, lw=2256e3, T_abl=373.15,
              arrhenius=1, A=3.1e98, Ea=6.28e5, Rgas=8.314, T_lo=316.15, T_hi=373.15, thr=(0.53, 1.0, 1e4),
              bc_type=(0, 0, 0, 0, 0, 1), bc_T=(310.15,) * 6, bc_h=(0, 0, 0, 0, 0, 10.0),
              bc_Tamb=(298.15,) * 6) -> HeatDesc:
    h = HeatDesc(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, opscale=opscale, dt=dt, vvox=dx * dy * dz, boil=boil,
                 T_boil=T_boil, lw=lw, T_abl=T_abl, arrhenius=arrhenius, lnA=float(np.log(A)), Ea=Ea, Rgas=Rgas,
                 T_lo=T_lo, T_hi=T_hi)
    for i in range(3):
        h.thr[i] = thr[i]
    for f in range(6):
        h.bc_type[f] = bc_type[f]
        h.bc_T[f] = bc_T[f]
        h.bc_h[f] = bc_h[f]
        h.bc_Tamb[f] = bc_Tamb[f]
    return h


def fused_step(h: HeatDesc, P, t_new, T, k, rho, c, J, Q, omega, thres, mat, nthreads=0):
    """One config-mode step; returns (Tn, n_ablated). Q, omega, thres, mat, J updated in place."""
    L = load()
    if not mat.flags.f_contiguous or mat.dtype != np.uint8:
        raise ValueError("mat must be uint8 and Fortran-ordered")
    Tn = np.empty_like(T, order="F")
    n = L.orc_fused_step(C.byref(h), P, t_new, dp(T), dp(Tn), dp(k), dp(rho), dp(c), dp(J), dp(Q), dp(omega),
                         dp(thres), mat.ctypes.data_as(C.POINTER(C.c_uint8)), nthreads)
    return Tn, n


def isolate(mat, J):
    """The isolation rule (src/3dFD.f90:347-349) in place on a u8 material
    grid and its FP64 source field (both Fortran order); returns the count."""
    L = load()
    if not mat.flags.f_contiguous or mat.dtype != np.uint8:
        raise ValueError("mat must be uint8 and Fortran-ordered")
    nx, ny, nz = mat.shape
    return L.orc_isolate(nx, ny, nz, mat.ctypes.data_as(C.POINTER(C.c_uint8)), dp(J))
