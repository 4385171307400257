"""The C-ABI library builds for sm_103a, loads, and exports every function
declared in include/life_gb300.h. Nothing here launches GPU work."""
import ctypes
import os
import re

import pytest

from life_gb300 import build as B
from life_gb300.case import parse_geometry_config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def libpath():
    return B.build()


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(life_\w+)\s*\(", text))
    # helpers defined inline in life_params_pack.h are not library exports
    return sorted(n for n in names if not n.startswith(("life_pack_", "life_print_")))


def test_exports_every_declared_function(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(declared_functions()) >= 17


def test_abi_version_and_error_string(libpath):
    from life_gb300.lib import lib
    L = lib()
    assert L.life_abi_version() == 1
    assert isinstance(L.life_last_error(), bytes)


def test_parse_geometry_matches_reference_rules(libpath):
    from life_gb300.lib import parse_geometry
    text = ("# comment line\n# another\n"
            "CIRCLE 2 7 0.2 0.2 0.1 0.0 0.05\n"
            "FILAMENT 3 10 0.25 0.2 0.0 0.05 0.35 0.02 15.0 FLEXIBLE CONFORMING SUPPORTED 10000.0 1.4e6\n"
            "FILAMENT 1 20 0.5 0.2 0.0 0.0 0.1 0.01 0.0 RIGID 20 CLAMPED 1.0 2.0\n")
    got = parse_geometry(text)
    py = parse_geometry_config(text)
    assert len(got) == len(py) == 3
    assert (got[0].kind, got[0].number, got[0].id, got[0].radius) == (0, 2, 7, 0.05)
    assert (got[1].kind, got[1].flexible, got[1].n_elements, got[1].clamped) == (1, 1, 0, 0)
    assert got[1].angle_deg == py[1].angle_deg == 15.0
    assert (got[2].flexible, got[2].n_elements, got[2].clamped, got[2].E) == (0, 20, 1, 2.0)


def test_parse_geometry_rejects_unknown_keyword(libpath):
    from life_gb300.lib import LifeError, parse_geometry
    with pytest.raises(LifeError):
        parse_geometry("SQUARE 1 0 0 0 0 0 1\n")


C_CLIENT = r"""
#include <stdio.h>
#include "life_gb300.h"
int main(void) {
    LifeBodyDesc b[4];
    int32_t n = 0;
    const char* text = "# comment\nCIRCLE 1 0 20.0 20.0 0.0 0.0 5.0\n";
    const int rc = life_parse_geometry(text, b, 4, &n);
    printf("abi %d rc %d n %d\n", life_abi_version(), rc, (int)n);
    return (life_abi_version() == 1 && rc == 0 && n == 1 && b[0].radius == 5.0) ? 0 : 1;
}
"""


def test_header_is_plain_c(libpath, tmp_path):
    """The public header compiles as strict C11 (no C++ in a C-ABI) and a C
    program links against the library and calls it (host-only calls)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    libdir = os.path.dirname(libpath)
    res = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I",
                          os.path.join(ROOT, "include"), str(src), "-L", libdir, "-llife_gb300",
                          f"-Wl,-rpath,{libdir}", "-o", str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "abi 1 rc 0 n 1" in run.stdout
