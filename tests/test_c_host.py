"""The C ABI from a C host: tests/c_host/host.c, compiled as strict C99
against include/tam.h and linked against libtam.so, reads the reference's
input.params fixture and a config-mode extension file, checks the header's
struct layouts against the library's and creates a context (on a machine
without a CUDA device the creation must fail with TAM_E_NODEV)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c99_host_builds_links_and_runs(tam, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = tam._abi.LIB_PATH
    exe = str(tmp_path / "host")
    cmd = [cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_host", "host.c"), "-o", exe, "-L", os.path.dirname(lib), "-ltam",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ext = tmp_path / "tissue.params"
    ext.write_text("nmat 3\nmaterial 2 0.3 120 0.9 1.4 0.37 1200 3300\nT0 309.0\n")
    r = subprocess.run([exe, os.path.join(ROOT, "tests", "golden", "input.params"), str(ext)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "config: 3 materials, T0 309 K" in r.stdout
    assert "no CUDA device" in r.stdout or "absorbed" in r.stdout
