"""The C-ABI library builds, loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(augur_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from augur_gb300 import build as B

    path = B.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("augur_pm_plan_create", "augur_pm_force", "augur_pm_step", "augur_pm_run",
                 "augur_direct_sum_fp64", "augur_energy_fp64"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    from augur_gb300 import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_status_strings_without_gpu(lib):
    lib.augur_status_string.restype = ctypes.c_char_p
    assert lib.augur_status_string(0) == b"ok"
    assert b"invalid" in lib.augur_status_string(-22)
    assert lib.augur_version() >= 0x000100


def test_plan_rejects_bad_geometry_without_gpu(lib):
    p = ctypes.c_void_p()
    f = lib.augur_pm_plan_create
    f.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int,
                  ctypes.c_double, ctypes.c_double, ctypes.c_double]
    assert f(ctypes.byref(p), 3, 250, 10, 0, 1.0, 0.0, 1.0) == -22  # G not a multiple of 16
    assert f(ctypes.byref(p), 2, 64, 10, 0, 1.0, 0.0, 1.0) == -22  # periodic mode is 3D
    assert f(ctypes.byref(p), 3, 64, 0, 0, 1.0, 0.0, 1.0) == -22  # no bodies
    assert not p.value


def test_product_rejects_cpu_tensors():
    import torch

    from augur_gb300.pm import _need

    with pytest.raises(ValueError, match="CUDA"):
        _need(torch.zeros(4, 3), "pos")


def test_unet2d_param_count_matches_reference_layout(golden):
    """augur_unet2d_param_count equals the reference UNet's parameter count (levels 5, width 32,
    6 inputs, 1 output: the net.* tensors of tests/golden/field2d.npz)."""
    from augur_gb300 import _lib

    g = golden["field2d"]
    n = sum(int(np.prod(g["w_" + k].shape)) for k in g["names"] if k.startswith("net."))
    assert _lib.load().augur_unet2d_param_count(6, 1, 32, 5) == n


@pytest.mark.parametrize("lang", ("c", "c++"))
def test_headers_compile_as_c_and_cxx(tmp_path, lang):
    """include/*.h is the C ABI a C, C++ or FFI caller binds: every header compiles on its own
    as C99 and as C++17 (no torch or CUDA types in the signatures)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip(f"no {lang} compiler")
    heads = sorted(p.name for p in (ROOT / "include").glob("*.h"))
    src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    src.write_text("".join(f'#include "{h}"\n' for h in heads) + "int main(void) { return 0; }\n")
    std = ["-std=c99", "-pedantic"] if lang == "c" else ["-std=c++17"]
    r = subprocess.run([cc, *std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
