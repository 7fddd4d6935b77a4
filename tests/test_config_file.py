"""The config-mode extension file (tam_read_config): the parameters that
res/input.params (src/mcpolar.f90:79-94) has no slot for -- materials, beam,
boundaries, Arrhenius constants -- read from a file beside it.  Host-side
parsing only: no GPU needed."""
import math

import numpy as np
import pytest

SKIN = """
# three-layer skin slab: air for ablated voxels, epidermis, dermis, subcutis
nmat 4
material 0  0.0 0.0   0.0  1.0  0.026 1.2  1005.0   # air
material 1  1.0 200.0 0.8  1.4  0.21  1200 3590     # epidermis
material 2  0.3 120.0 0.9  1.4  0.37  1200 3300
material 3  0.1 80.0  0.9  1.4  0.16  1000 2674
source gaussian
source_radius 0.05
n_ambient 1.0
fresnel 1
roulette 1
roulette_w 1e-4
roulette_m 10
max_steps 1000000
bc z+ robin h=10 Tamb=298.15
bc z- dirichlet T=310.15
T0 310.15
dt_factor 0.9
dt 0
opscale 1
boil 1
T_boil 373.15
lw 2.257e6
T_abl 373.15
arrhenius 1
A 3.1e98
Ea 6.28e5
Rgas 8.314
T_lo 316.15
T_hi 373.15
thr 0.53 1.0 4.6
retrace_fraction 1e-3
retrace_check 50
isolation 1
"""


def _write(tmp_path, text, name="tissue.params"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_config_file_sets_every_key(tam, tmp_path):
    c = tam.read_config(_write(tmp_path, SKIN))
    assert c.nmat == 4
    m1, m3 = c.mat[1], c.mat[3]
    assert (m1.mua, m1.mus, m1.g, m1.n, m1.k, m1.rho, m1.c) == (1.0, 200.0, 0.8, 1.4, 0.21, 1200.0, 3590.0)
    assert (m3.mua, m3.mus, m3.k, m3.rho, m3.c) == (0.1, 80.0, 0.16, 1000.0, 2674.0)
    assert c.source == tam._abi.TAM_SRC_GAUSSIAN and c.source_radius == 0.05
    assert c.max_steps == 1000000 and c.isolation == 1
    assert c.bc_type[5] == tam._abi.TAM_BC_ROBIN and c.bc_h[5] == 10.0 and c.bc_Tamb[5] == 298.15
    assert c.bc_type[4] == tam._abi.TAM_BC_DIRICHLET and c.bc_T[4] == 310.15
    assert list(c.thr) == [0.53, 1.0, 4.6]
    assert c.A == 3.1e98 and c.Ea == 6.28e5 and c.T_lo == 316.15 and c.retrace_check == 50


def test_config_file_keeps_what_it_leaves_out(tam, tmp_path):
    base = tam.default_config()
    base.T0 = 300.0
    base.fresnel = 0
    c = tam.read_config(_write(tmp_path, "material 5 2.0 50 0.7 1.33 0.5 1000 4000\nsource disk\n"), base)
    assert c.nmat == 6  # raised to hold material 5
    assert c.mat[5].mua == 2.0 and c.source == tam._abi.TAM_SRC_DISK
    assert c.T0 == 300.0 and c.fresnel == 0  # untouched
    assert math.isclose(c.mat[1].mus, tam.default_config().mat[1].mus)


@pytest.mark.parametrize("text,what", [
    ("colour blue\n", "unknown setting 'colour'"),
    ("T0 hot\n", "malformed value for T0"),
    ("T0 nan\n", "malformed value for T0"),
    ("material 2 0.3 inf 0.9 1.4 0.37 1200 3300\n", "malformed material value 'inf'"),
    ("material 16 0 0 0 1 1 1 1\n", "material takes an id"),
    ("material 2 0.3 100\n", "material takes an id"),
    ("bc top robin h=10\n", "bc takes a face"),
    ("bc z+ robin k=10\n", "bc value 'k'"),
    ("thr 0.5 1\n", "thr takes three"),
    ("fresnel 1.5\n", "malformed integer for fresnel"),
    ("nmat 0\n", "nmat takes one count"),
])
def test_config_file_errors_name_the_line(tam, tmp_path, text, what):
    F = tam._abi
    path = _write(tmp_path, "# header\n\n" + text)
    base = tam.default_config()
    before = bytes(base)
    with pytest.raises(tam.TamError) as e:
        tam.read_config(path, base)
    assert e.value.code == F.TAM_E_PARSE
    assert f"{path}:3: {what}" in str(e.value)
    assert bytes(base) == before  # left unchanged


def test_config_file_crlf_tabs_and_comments(tam, tmp_path):
    # a file saved on Windows with tabs between fields reads like the plain one
    plain = tam.read_config(_write(tmp_path, SKIN))
    dos = SKIN.replace(" ", "\t").replace("\n", "\r\n")
    c = tam.read_config(_write(tmp_path, "   # leading comment\r\n" + dos, "dos.params"))
    assert bytes(c) == bytes(plain)


def test_config_file_missing(tam, tmp_path):
    with pytest.raises(tam.TamError) as e:
        tam.read_config(str(tmp_path / "absent.params"))
    assert e.value.code == tam._abi.TAM_E_IO


@pytest.mark.gpu
def test_config_file_drives_a_run_like_the_same_struct(tam, tmp_path):
    # a context built from the file runs exactly as one built from the same
    # settings made in code (same Philox streams, same kernels)
    F = tam._abi
    text = ("nmat 3\nmaterial 1 1.0 200 0.8 1.4 0.21 1200 3590\nmaterial 2 0.3 120 0.9 1.4 0.37 1200 3300\n"
            "source_radius 0.03\nbc z+ robin h=20 Tamb=295\nretrace_fraction 0\n")
    c_file = tam.read_config(_write(tmp_path, text))
    c_code = tam.default_config(nmat=3, source_radius=0.03, retrace_fraction=0.0)
    tam.set_material(c_code, 1, 1.0, 200.0, 0.8, 1.4, 0.21, 1200.0, 3590.0)
    tam.set_material(c_code, 2, 0.3, 120.0, 0.9, 1.4, 0.37, 1200.0, 3300.0)
    c_code.bc_h[5], c_code.bc_Tamb[5] = 20.0, 295.0
    assert bytes(c_file) == bytes(c_code)
    out = []
    for c in (c_file, c_code):
        p = tam.default_params(nxg=24, nyg=24, nzg=16, xmax=0.06, ymax=0.06, zmax=0.04, mode=1, precision=0,
                               nphotons=5000, pulse_type=1, power=2.0, energy_per_pixel=2e3, total_time=1.0, loops=1)
        with tam.Context(p, c) as ctx:
            grid = np.ones((24, 24, 16), dtype=np.uint8, order="F")
            grid[:, :, 12:] = 2
            ctx.upload(F.TAM_F_MATERIAL, grid)
            ctx.step_coupled(20, seed=3)
            out.append((ctx.download(F.TAM_F_TEMP), ctx.download(F.TAM_F_JMEAN), ctx.device_errors()))
    (Ta, Ja, ea), (Tb, Jb, eb) = out
    assert ea == eb == 0 and Ja.max() > 0
    np.testing.assert_allclose(Ja, Jb, rtol=1e-9, atol=1e-9 * Jb.max())
    np.testing.assert_allclose(Ta, Tb, rtol=1e-12)
