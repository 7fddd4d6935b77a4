"""Python wrapper over the C ABI of libtam.so.

Mirrors the reference's subroutine surface (src/mcpolar.f90 driver calls)
through ``Context`` methods; arrays come back as numpy arrays in the
reference layout (Fortran order, halo where the reference has one).
Every call goes through libtam.so: there is no CPU path here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import Config, Params, State

HALO_FIELDS = {_abi.TAM_F_TEMP, _abi.TAM_F_RHOKAP, _abi.TAM_F_KAPPA, _abi.TAM_F_DENSITY, _abi.TAM_F_HEATCAP,
               _abi.TAM_F_COEFF, _abi.TAM_F_ALPHA}


class TamError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib():
    return _abi.load()


def check(code: int, ctx=None) -> None:
    if code != _abi.TAM_OK:
        L = lib()
        msg = L.tam_last_error(ctx)
        raise TamError(code, msg.decode() if msg else "")


def default_params(**kw) -> Params:
    p = Params()
    check(lib().tam_params_default(C.byref(p)))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def default_config(**kw) -> Config:
    c = Config()
    check(lib().tam_config_default(C.byref(c)))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def set_material(cfg: Config, i: int, mua, mus, g, n, k, rho, c) -> None:
    m = cfg.mat[i]
    m.mua, m.mus, m.g, m.n, m.k, m.rho, m.c = mua, mus, g, n, k, rho, c


def read_input_params(path: str, base: Params | None = None) -> Params:
    p = base if base is not None else default_params()
    check(lib().tam_read_input_params(path.encode(), C.byref(p)))
    return p


def read_config(path: str, base: Config | None = None) -> Config:
    """A config-mode extension file (tam_read_config) over `base` (default:
    the library's defaults)."""
    c = base if base is not None else default_config()
    check(lib().tam_read_config(path.encode(), C.byref(c)))
    return c


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Context:
    """One device-resident instance (``struct tam_ctx``)."""

    def __init__(self, params: Params, config: Config | None = None):
        self._lib = lib()
        self.params = params
        self.config = config
        h = C.c_void_p()
        check(self._lib.tam_create(C.byref(params), C.byref(config) if config is not None else None, C.byref(h)))
        self._h = h
        self.nx, self.ny, self.nz = params.nxg, params.nyg, params.nzg

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.tam_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, code: int) -> None:
        check(code, self._h)

    # -- shapes -------------------------------------------------------------
    def field_shape(self, field: int):
        if field in HALO_FIELDS:
            return (self.nx + 2, self.ny + 2, self.nz + 2)
        if field == _abi.TAM_F_THRESTIME:
            return (self.nx, self.ny, self.nz, 3)
        return (self.nx, self.ny, self.nz)

    def download(self, field: int) -> np.ndarray:
        dtype = np.uint8 if field == _abi.TAM_F_MATERIAL else np.float64
        out = np.empty(self.field_shape(field), dtype=dtype, order="F")
        self._ck(self._lib.tam_download(self._h, field, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def upload(self, field: int, arr) -> None:
        dtype = np.uint8 if field == _abi.TAM_F_MATERIAL else np.float64
        a = np.asfortranarray(np.asarray(arr, dtype=dtype).reshape(self.field_shape(field), order="F"))
        self._ck(self._lib.tam_upload(self._h, field, a.ctypes.data_as(C.c_void_p), a.nbytes))

    # -- hot path -----------------------------------------------------------
    def set_stream(self, stream_handle: int | None) -> None:
        self._ck(self._lib.tam_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None))

    def mc_pass(self, nphotons: int, seed: int, stream: int = 0, want: bool = False):
        out = np.empty((self.nx, self.ny, self.nz), order="F") if want else None
        self._ck(self._lib.tam_mc_pass(self._h, int(nphotons), int(seed), int(stream),
                                       _dptr(out) if want else None))
        return out

    def heat_steps(self, n: int, want: bool = False):
        out = np.empty((self.nx + 2, self.ny + 2, self.nz + 2), order="F") if want else None
        self._ck(self._lib.tam_heat_steps(self._h, int(n), _dptr(out) if want else None))
        return out

    def arrhenius(self) -> None:
        self._ck(self._lib.tam_arrhenius(self._h))

    def update_props(self, ablate_temp: float) -> None:
        self._ck(self._lib.tam_update_props(self._h, float(ablate_temp)))

    def step_coupled(self, n: int, seed: int) -> None:
        self._ck(self._lib.tam_step_coupled(self._h, int(n), int(seed)))

    def run(self, seed: int, max_iters: int = 0) -> int:
        it = C.c_int64(0)
        self._ck(self._lib.tam_run(self._h, int(seed), int(max_iters), C.byref(it)))
        return it.value

    def finalize(self) -> None:
        self._ck(self._lib.tam_finalize(self._h))

    def init_thermal(self) -> float:
        d = C.c_double(0)
        self._ck(self._lib.tam_init_thermal(self._h, C.byref(d)))
        return d.value

    def gridset(self, xmax, ymax, zmax) -> None:
        self._ck(self._lib.tam_gridset(self._h, xmax, ymax, zmax))

    def tallies(self) -> dict:
        out = (C.c_double * len(_abi.TALLY_NAMES))()
        self._ck(self._lib.tam_get_tallies_ex(self._h, out, len(_abi.TALLY_NAMES)))
        return dict(zip(_abi.TALLY_NAMES, list(out)))

    def state(self) -> State:
        s = State()
        self._ck(self._lib.tam_get_state(self._h, C.byref(s)))
        return s

    def device_errors(self) -> int:
        b = C.c_uint32(0)
        self._ck(self._lib.tam_device_errors(self._h, C.byref(b)))
        return b.value

    def set_tuning(self, key: str, value: int) -> None:
        self._ck(self._lib.tam_set_tuning(self._h, key.encode(), int(value)))

    def timing(self):
        t = C.c_double(0)
        h = C.c_double(0)
        n = C.c_int64(0)
        self._ck(self._lib.tam_get_timing(self._h, C.byref(t), C.byref(h), C.byref(n)))
        return t.value, h.value, n.value

    def save_state(self, path: str) -> None:
        self._ck(self._lib.tam_save_state(self._h, str(path).encode()))

    def load_state(self, path: str) -> None:
        self._ck(self._lib.tam_load_state(self._h, str(path).encode()))

    def autotune(self, packets: int = 1_000_000, steps: int = 20) -> dict:
        """Pick the fastest kernel settings on this context's workload; state is restored."""
        out = (C.c_int64 * 4)()
        self._ck(self._lib.tam_autotune(self._h, int(packets), int(steps), out, 4))
        return {"transport.scat_min": out[0], "heat.zchunk": out[1], "heat.cls_rows": out[2], "heat.slab": out[3]}

    def write_output(self, directory: str) -> None:
        self._ck(self._lib.tam_write_output(self._h, directory.encode()))


def _batch_args(contexts, seeds):
    n = len(contexts)
    if len(seeds) != n:
        raise ValueError("one seed per context")
    hs = (_abi._P * n)(*[c._h for c in contexts])
    sd = (C.c_uint64 * n)(*[int(x) for x in seeds])
    return n, hs, sd


def batch_step_coupled(contexts, iters: int, seeds) -> None:
    """`iters` outer iterations on every context, the instances running concurrently."""
    n, hs, sd = _batch_args(contexts, seeds)
    check(lib().tam_batch_step_coupled(hs, n, int(iters), sd))


def batch_run(contexts, seeds, max_iters: int = 0):
    """Each context's whole coupled loop (as Context.run), concurrently; returns iteration counts."""
    n, hs, sd = _batch_args(contexts, seeds)
    it = (C.c_int64 * n)()
    check(lib().tam_batch_run(hs, n, sd, int(max_iters), it))
    return list(it)


def batch_mc_pass(contexts, seeds, nphotons=None, streams=None) -> None:
    """One MC pass of every context (tam_batch_mc_pass): the FP32 uniform-medium
    instances' passes in shared launches of the batched transport, each packet
    on its instance's own Philox stream.  nphotons / streams: one per context,
    or None for each context's nphotons x numproc / its count of passes."""
    n, hs, sd = _batch_args(contexts, seeds)
    if (nphotons is not None and len(nphotons) != n) or (streams is not None and len(streams) != n):
        raise ValueError("one value per context")
    np_ = None if nphotons is None else (C.c_int64 * n)(*[int(x) for x in nphotons])
    st = None if streams is None else (C.c_uint32 * n)(*[int(x) for x in streams])
    check(lib().tam_batch_mc_pass(hs, n, np_, sd, st))


def batch_heat_steps(contexts, nsteps: int) -> None:
    """`nsteps` FP32 heat steps of every context in persistent batched launches."""
    n = len(contexts)
    hs = (_abi._P * n)(*[c._h for c in contexts])
    check(lib().tam_batch_heat_steps(hs, n, int(nsteps)))


def batch_autotune(contexts, steps: int = 20) -> dict:
    """Pick the fastest batched-step form (cooperative kernel form and z-chunk,
    or each instance's own steps on its stream) on these contexts; their
    state is restored."""
    n = len(contexts)
    hs = (_abi._P * n)(*[c._h for c in contexts])
    out = (C.c_int64 * 3)()
    check(lib().tam_batch_autotune(hs, n, int(steps), out, 3))
    return {"batch.staged": out[0], "batch.zchunk": out[1], "batch.streams": out[2]}


def tally_atomics_per_second(cells: int, fp32: bool = False) -> float:
    """Rate of the device's atomic adds into a tally of `cells` entries (the
    transport's tally-update ceiling; tam_measure_tally_atomics)."""
    v = C.c_double(0)
    check(lib().tam_measure_tally_atomics(int(cells), 1 if fp32 else 0, C.byref(v)))
    return v.value


def kernel_launches() -> int:
    return int(lib().tam_kernel_launches())


def selftest_philox(words: np.ndarray):
    """words: (n, 6) uint32 {c0,c1,c2,c3,k0,k1} -> (mine, curand) each (n, 4)."""
    w = np.ascontiguousarray(words, dtype=np.uint32)
    n = w.shape[0]
    a = np.empty((n, 4), dtype=np.uint32)
    b = np.empty((n, 4), dtype=np.uint32)
    u = C.POINTER(C.c_uint32)
    check(lib().tam_selftest_philox(w.ctypes.data_as(u), a.ctypes.data_as(u), b.ctypes.data_as(u), n))
    return a, b
