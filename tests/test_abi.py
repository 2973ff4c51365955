"""The C ABI boundary without a GPU: exported symbols, struct layout, config validation."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "tp_wcsph.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tp_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "tp_kick" in names and "tp_integrate_ck2n54" in names
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib._name)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (tp_[a-z0-9_]+)$", out, flags=re.M))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_python_prototypes_cover_header(pkg):
    from importlib import import_module  # noqa: F401

    protos = {p[0] for p in pkg._abi.PROTOTYPES}
    assert set(declared_functions()) == protos


def test_config_struct_layout(pkg, tmp_path):
    fields = [f[0] for f in pkg.TpConfig._fields_]
    src = tmp_path / "layout.c"
    body = "\n".join(f'printf("{f} %zu\\n", offsetof(tp_config, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "tp_wcsph.h"\n'
                   f'int main(void){{ {body} printf("size %zu\\n", sizeof(tp_config)); return 0; }}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    c_off = {l.split()[0]: int(l.split()[1]) for l in out if l}
    for f in fields:
        assert getattr(pkg.TpConfig, f).offset == c_off[f], f
    assert ctypes.sizeof(pkg.TpConfig) == c_off["size"]


def test_config_default_matches(lib, pkg):
    c = pkg.TpConfig()
    lib.tp_config_default(ctypes.byref(c))
    d = pkg.default_config()
    for f, _ in pkg.TpConfig._fields_:
        a, b = getattr(c, f), getattr(d, f)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), f
        else:
            assert a == b, f
    assert lib.tp_abi_version() == 1


def good_config(pkg):
    c = pkg.default_config()
    c.ndims = 2
    c.n_fluid = 10
    c.n_wall = 10
    c.smoothing_length = 0.1
    c.sound_speed = 10.0
    c.max_corner[0] = c.max_corner[1] = 1.0
    return c


@pytest.mark.parametrize("field,value,status", [
    ("ndims", 4, 1), ("precision", 7, 1), ("n_fluid", -1, 1), ("smoothing_length", 0.0, 1),
    ("smoothing_length", float("nan"), 1), ("sound_speed", -1.0, 1), ("exponent", 0.0, 1),
    ("viscosity_model", 9, 5), ("density_diffusion_model", 9, 5),
])
def test_create_rejects_bad_config(lib, pkg, field, value, status):
    c = good_config(pkg)
    setattr(c, field, value)
    h = ctypes.c_void_p()
    st = lib.tp_create(ctypes.byref(c), ctypes.byref(h))
    assert st == status
    assert h.value is None
    assert lib.tp_last_error(None)


def test_create_rejects_inverted_bounds(lib, pkg):
    c = good_config(pkg)
    c.min_corner[0] = 2.0
    h = ctypes.c_void_p()
    assert lib.tp_create(ctypes.byref(c), ctypes.byref(h)) == 1
    assert b"bounds" in lib.tp_last_error(None)


def test_null_handle_is_an_argument_error(lib):
    assert lib.tp_kick(None, None, None, None, 0.0) == 1
    assert lib.tp_sync(None) == 1
    assert lib.tp_destroy(None) == 0
