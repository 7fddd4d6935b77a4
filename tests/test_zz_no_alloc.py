"""The allocation-free MC pass (tam_mc_pass_noalloc) against tam_mc_pass.

tam_mc_pass_noalloc serves callers that cannot let the library allocate
device memory (device arrays owned by another runtime, a fixed device-memory
budget, no allocation inside a capture or real-time loop): they pass rhokap
and jmeanGLOBAL as device pointers and the pass keeps its scratch in one
static device array.  Two calls in a row must each reproduce the pass of the
context-based entry point on the same Philox streams, within the 1e-9
relative tolerance of the other same-stream transport tests.  This file is
collected last so that a failure here cannot stop the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_context_pass_twice(tam):
    torch = pytest.importorskip("torch")
    F = tam._abi
    lib = F.load()
    n = 20000
    # tophat pulse: getPwr() is the configured power while the laser is on
    p = tam.default_params(nxg=40, nyg=40, nzg=40, pulse_type=1, power=70.0, nphotons=n)
    with tam.Context(p) as ctx:
        rk = ctx.download(F.TAM_F_RHOKAP)
        want = ctx.mc_pass(n, seed=4242, stream=9, want=True)
    assert want.max() > 0
    rk_dev = torch.from_numpy(np.ascontiguousarray(rk.ravel(order="F"))).cuda()
    for call in range(2):
        out = torch.full((40 * 40 * 40,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.tam_mc_pass_noalloc(C.byref(p), C.c_void_p(rk_dev.data_ptr()), C.c_void_p(out.data_ptr()), n, 4242,
                                     9, 70.0, None)
        assert rc == F.TAM_OK, lib.tam_last_error(None)
        got = out.cpu().numpy().reshape((40, 40, 40), order="F")
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * want.max(), err_msg=f"call {call}")


def test_noalloc_rejects_oversized_grid(tam):
    F = tam._abi
    lib = F.load()
    p = tam.default_params(nxg=200, nyg=200, nzg=200)
    rc = lib.tam_mc_pass_noalloc(C.byref(p), C.c_void_p(16), C.c_void_p(16), 10, 1, 0, 1.0, None)
    assert rc == F.TAM_E_INVALID
    assert b"allocation-free limit" in lib.tam_last_error(None)
