"""C ABI checks that need no GPU: the library loads, exports every entry
point declared in include/tam.h, its struct layouts match the binding, the
res/input.params reader follows Fortran list-directed rules
(src/mcpolar.f90:79-94), and creating a context without a GPU fails loudly
(no CPU fallback)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "tam.h")
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tam_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(tam):
    lib = tam._abi.load()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in tam._abi.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


def test_struct_layouts_match(tam):
    lib = tam._abi.load()
    assert lib.tam_struct_size(0) == C.sizeof(tam.Params)
    assert lib.tam_struct_size(1) == C.sizeof(tam.Config)
    assert lib.tam_struct_size(2) == C.sizeof(tam.State)
    assert lib.tam_struct_size(3) == C.sizeof(tam._abi.Material)
    assert lib.tam_struct_size(9) == -1
    assert lib.tam_abi_version() == 2
    assert b"sm_103a" in lib.tam_version()


def test_params_default_is_shipped_input(tam):
    p = tam.default_params()
    assert (p.nphotons, p.xmax, p.ymax, p.zmax, p.n1, p.n2) == (125000, 0.03, 0.03, 0.06, 1.0, 1.38)
    assert (p.total_time, p.loops, p.repetition_rate_1, p.power) == (2.0, 1, 1e7, 70.0)
    assert (p.energy_per_pixel, p.ablate_temp, p.pulses_to_do, p.pulse_type) == (400.0, 500.0, 1, 0)
    assert (p.nxg, p.nyg, p.nzg, p.numproc) == (80, 80, 80, 1)
    c = tam.default_config()
    assert c.nmat == 2 and c.mat[1].mus == 100.0 and c.bc_type[5] == 1 and c.bc_h[5] == 10.0


def test_read_input_params_fixture(tam):
    p = tam.Params()
    p.nxg = 7
    got = tam.read_input_params(os.path.join(GOLD, "input.params"), p)
    d = tam.default_params()
    for name, _ in tam.Params._fields_:
        if name == "nxg":
            assert got.nxg == 7  # not in the file: untouched
            continue
        if name in ("nyg", "nzg", "numproc", "mode", "precision", "device"):
            continue
        assert getattr(got, name) == getattr(d, name), name


def _write(tmp_path, lines):
    f = tmp_path / "input.params"
    f.write_text("\n".join(lines) + "\n")
    return str(f)


def test_read_input_params_list_directed_rules(tam, tmp_path):
    lines = ["  1000 , packets", "0.5d0", "", "5.D-1", "2.5e-1 x", "1.0", "1.4", "1.", "3", "1.0/2.", "10",
             "1000", "100.", "10", "'tophat' quoted"]
    p = tam.read_input_params(_write(tmp_path, lines))
    assert p.nphotons == 1000 and p.xmax == 0.5 and p.ymax == 0.5 and p.zmax == 0.25
    assert p.loops == 3 and p.repetition_rate_1 == 1.0 and p.pulses_to_do == 10
    assert p.pulse_type == tam._abi.TAM_PULSE_TOPHAT


def test_read_input_params_errors(tam, tmp_path):
    with pytest.raises(tam.TamError) as e:
        tam.read_input_params(str(tmp_path / "missing.params"))
    assert e.value.code == tam._abi.TAM_E_IO
    lines = open(os.path.join(GOLD, "input.params")).read().splitlines()
    bad = list(lines)
    bad[13] = "sawtooth"
    with pytest.raises(tam.TamError) as e:
        tam.read_input_params(_write(tmp_path, bad))
    assert e.value.code == tam._abi.TAM_E_PARSE
    bad = list(lines)
    bad[7] = "1.5"  # integer field
    with pytest.raises(tam.TamError) as e:
        tam.read_input_params(_write(tmp_path, bad))
    assert e.value.code == tam._abi.TAM_E_PARSE
    with pytest.raises(tam.TamError) as e:
        tam.read_input_params(_write(tmp_path, lines[:10]))
    assert e.value.code == tam._abi.TAM_E_PARSE


def test_create_rejects_bad_params(tam):
    p = tam.default_params(nxg=0)
    with pytest.raises(tam.TamError) as e:
        tam.Context(p)
    assert e.value.code == tam._abi.TAM_E_INVALID
    p = tam.default_params(mode=1)
    with pytest.raises(tam.TamError) as e:
        tam.Context(p)  # config mode without a tam_config
    assert e.value.code == tam._abi.TAM_E_INVALID


def _has_gpu(tam):
    lib = tam._abi.load()
    h = C.c_void_p()
    p = tam.default_params(nxg=2, nyg=2, nzg=2)
    rc = lib.tam_create(C.byref(p), None, C.byref(h))
    if rc == 0:
        lib.tam_destroy(h)
    return rc != tam._abi.TAM_E_NODEV


def test_no_cpu_fallback_without_gpu(tam):
    if _has_gpu(tam):
        pytest.skip("a GPU is present")
    with pytest.raises(tam.TamError) as e:
        tam.Context(tam.default_params(nxg=8, nyg=8, nzg=8))
    assert e.value.code == tam._abi.TAM_E_NODEV
    a, b = None, None
    with pytest.raises(tam.TamError) as e:
        import numpy as np

        a, b = tam.selftest_philox(np.zeros((4, 6), dtype=np.uint32))
    assert e.value.code == tam._abi.TAM_E_NODEV


def test_fortran_module_matches_header(tam):
    # include/tam.f90 (not compiled here: no Fortran compiler) binds names the
    # library exports, with the header's enum values and struct field order
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = open(os.path.join(root, "include", "tam.f90")).read()
    lib = tam._abi.load()
    names = re.findall(r"function (tam_\w+)\(", src)
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    params = dict((k, int(v)) for k, v in re.findall(r"(TAM_\w+) = (\d+)", src))
    for k, v in params.items():
        if hasattr(tam._abi, k):
            assert getattr(tam._abi, k) == v, k
    # bind(C) tam_params: the ctypes mirror's field order
    block = src[src.index("type, bind(C) :: tam_params"): src.index("end type")].split("\n", 1)[1]
    fields = [f.strip() for line in re.findall(r"::\s*(.*)", block) for f in line.split(",")]
    assert fields == [f[0] for f in tam._abi.Params._fields_]
