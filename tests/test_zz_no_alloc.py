"""The allocation-free MC pass (tam_mc_pass_noalloc).

tam_mc_pass_noalloc serves callers that cannot let the library allocate
device memory (device arrays owned by another runtime, such as a Fortran host
using OpenACC or CUDA Fortran, or a fixed device-memory budget): they pass
rhokap and jmeanGLOBAL as device pointers and the pass keeps its scratch in
one static device array.  Two calls in a row must each reproduce

  * the pass of the context-based entry point on the same Philox streams, in
    the same precision, within 1e-9 relative (the same transport kernel; only
    the order of the atomic tally sums differs), and
  * the oracle on the same streams: 1e-9 relative per voxel for the FP64
    transport, as the other same-stream transport tests; the FP32 transport
    follows the same straight single-flight paths of the reference medium
    with FP32 positions, so only packets whose launch point or exit lies
    within FP32 rounding of a cell face change cells: 1e-4 relative L1 and
    1e-5 on the total absorbed weight.

This file is collected last so that a failure here cannot stop the rest of the
suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 20000
EDGE = 40
SEED, STREAM, POWER = 4242, 9, 70.0


@pytest.fixture(scope="module")
def oracle_pass(orc):
    # tophat pulse: getPwr() is the configured power while the laser is on
    o = orc.RefOracle(orc.ref_params(nx=EDGE, ny=EDGE, nz=EDGE, nphotons=N, power=POWER, pulse_type=1))
    o.photons(N, seed=SEED, stream=STREAM, nthreads=0)
    o.normalise()
    J = o.arr("jmeanGLOBAL").copy()
    o.close()
    return J


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_context_pass_and_oracle_twice(tam, oracle_pass, precision):
    torch = pytest.importorskip("torch")
    F = tam._abi
    lib = F.load()
    p = tam.default_params(nxg=EDGE, nyg=EDGE, nzg=EDGE, pulse_type=1, power=POWER, nphotons=N, precision=precision)
    with tam.Context(p) as ctx:
        rk = ctx.download(F.TAM_F_RHOKAP)
        want = ctx.mc_pass(N, seed=SEED, stream=STREAM, want=True)
    assert want.max() > 0
    Jo = oracle_pass
    rk_dev = torch.from_numpy(np.ascontiguousarray(rk.ravel(order="F"))).cuda()
    for call in range(2):
        out = torch.full((EDGE ** 3,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.tam_mc_pass_noalloc(C.byref(p), C.c_void_p(rk_dev.data_ptr()), C.c_void_p(out.data_ptr()), N, SEED,
                                     STREAM, POWER, None)
        assert rc == F.TAM_OK, lib.tam_last_error(None)
        got = out.cpu().numpy().reshape((EDGE,) * 3, order="F")
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * want.max(), err_msg=f"call {call}")
        if precision == 0:
            np.testing.assert_allclose(got, Jo, rtol=1e-9, atol=1e-9 * Jo.max(), err_msg=f"oracle, call {call}")
        else:
            l1 = np.abs(got - Jo).sum() / np.abs(Jo).sum()
            assert l1 < 1e-4, (call, l1)
            assert abs(got.sum() - Jo.sum()) <= 1e-5 * Jo.sum(), call


def test_noalloc_rejects_oversized_grid(tam):
    F = tam._abi
    lib = F.load()
    p = tam.default_params(nxg=200, nyg=200, nzg=200)
    rc = lib.tam_mc_pass_noalloc(C.byref(p), C.c_void_p(16), C.c_void_p(16), 10, 1, 0, 1.0, None)
    assert rc == F.TAM_E_INVALID
    assert b"allocation-free limit" in lib.tam_last_error(None)


def test_noalloc_rejects_other_device(tam):
    # the pass runs on the caller's current device; a p->device naming another
    # one is refused before anything touches a device pointer
    F = tam._abi
    lib = F.load()
    p = tam.default_params(nxg=8, nyg=8, nzg=8, device=7)
    rc = lib.tam_mc_pass_noalloc(C.byref(p), C.c_void_p(16), C.c_void_p(16), 10, 1, 0, 1.0, None)
    assert rc == F.TAM_E_INVALID
    assert b"not the current device" in lib.tam_last_error(None)
