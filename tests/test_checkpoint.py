"""Checkpoint / resume: a context restored from tam_save_state continues bit
for bit (FP64 reference mode, FP32 config mode), and a state file written by a
context with other parameters is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref(tam):
    return tam.Context(tam.default_params(nxg=16, nyg=16, nzg=16, nphotons=3000, power=8.0, pulse_type=1))


def _cfg(tam):
    nx = 32
    half = 0.0025 * nx
    p = tam.default_params(nxg=nx, nyg=nx, nzg=nx, xmax=half, ymax=half, zmax=half, mode=1, precision=1,
                           nphotons=20000, pulse_type=1, power=3.0, energy_per_pixel=3e3, total_time=1.0)
    return tam.Context(p, tam.default_config(source_radius=0.03, retrace_check=5))


@pytest.mark.parametrize("make", [_ref, _cfg], ids=["reference-fp64", "config-fp32"])
def test_resume_continues_bit_for_bit(tam, tmp_path, make):
    F = tam._abi
    path = str(tmp_path / "state.bin")
    fields = (F.TAM_F_TEMP, F.TAM_F_TISSUE, F.TAM_F_JMEAN_GLOBAL, F.TAM_F_RHOKAP)
    with make(tam) as a:
        a.step_coupled(4, seed=11)
        a.save_state(path)
        a.step_coupled(3, seed=11)
        want = [a.download(f) for f in fields]
        st_a = a.state()
    with make(tam) as b:
        b.load_state(path)
        b.step_coupled(3, seed=11)
        got = [b.download(f) for f in fields]
        st_b = b.state()
    assert st_a.time == st_b.time and st_a.mc_passes == st_b.mc_passes and st_a.counter == st_b.counter
    for x, y in zip(got, want):
        # the FP64 tally sums in atomic order, so an MC pass after the restore agrees to rounding
        np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-12 * max(np.abs(y).max(), 1e-300))


def test_state_file_of_other_parameters_is_refused(tam, tmp_path):
    path = str(tmp_path / "state.bin")
    with _ref(tam) as a:
        a.save_state(path)
    p = tam.default_params(nxg=16, nyg=16, nzg=16, nphotons=3000, power=9.0, pulse_type=1)
    with tam.Context(p) as b:
        with pytest.raises(tam.TamError):
            b.load_state(path)
