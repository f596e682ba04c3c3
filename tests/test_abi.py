"""The C-ABI boundary, checked without a GPU.

- every function declared in include/*.h is exported by libtopefft.so;
- the headers compile as C and C++ and the ctypes mirror's struct layouts
  match the C compiler's;
- a C caller written like the reference's drivers compiles and links;
- without a usable GPU the library reports errors instead of crashing or
  falling back to the CPU.
"""
import ctypes
import re
import subprocess

import pytest

from conftest import ROOT

INCLUDE = ROOT / "include"
HEADERS = [INCLUDE / "topefft.h", INCLUDE / "topefft_ext.h"]


def declared_functions():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(\w+)\s*\([^;{]*\)\s*;", text, re.M):
            names.append(m.group(1))
    return sorted(set(names) - {"assert"})


def test_every_declared_symbol_is_exported(T):
    names = declared_functions()
    assert len(names) >= 35
    lib = ctypes.CDLL(str(T.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    mirrored = {s[0] for s in T.SIGNATURES}
    assert set(names) <= mirrored, set(names) - mirrored


@pytest.mark.parametrize("compiler", ["gcc -x c -std=c99", "g++ -x c++ -std=c++11"])
def test_headers_compile(tmp_path, compiler):
    src = tmp_path / "h.c"
    src.write_text('#include "topefft.h"\n#include "topefft_ext.h"\nint main(void){return 0;}\n')
    cmd = compiler.split() + ["-Wall", "-Werror", "-Wno-dollar-in-identifier-extension",
                              f"-I{INCLUDE}", str(src), "-o", str(tmp_path / "h")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode and "dollar" in r.stderr:
        r = subprocess.run([c for c in cmd if "dollar" not in c], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_struct_layout_matches_mirror(T, tmp_path):
    structs = {"topeFFT": T.TopeFFT, "topePlan1D": T.TopePlan1D, "topePlan2D": T.TopePlan2D,
               "topePlan3D": T.TopePlan3D, "topeBatch": T.TopeBatch}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "topefft.h"',
             '#include "topefft_ext.h"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof(struct {cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof(struct {cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{INCLUDE}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for line in filter(None, out):
        cname, field, val = line.split()
        py = structs[cname]
        want = ctypes.sizeof(py) if field == "size" else getattr(py, field).offset
        assert int(val) == want, (cname, field, val, want)


@pytest.mark.parametrize("driver", ["tope_driver", "ext_driver"])
def test_c_drivers_link(T, tmp_path, driver):
    """The reference-style caller and the caller of the whole extension
    surface compile without warnings against include/ and link against the
    built library."""
    exe = tmp_path / driver
    r = subprocess.run(["gcc", "-O2", "-Wall", "-Werror", f"-I{INCLUDE}",
                        str(ROOT / "tests" / "drivers" / f"{driver}.c"),
                        "-o", str(exe), f"-L{T.LIB_PATH.parent}", "-ltopefft",
                        f"-Wl,-rpath,{T.LIB_PATH.parent}", "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _gpu_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu_present(), reason="checks the no-GPU error path")
def test_no_gpu_reports_error_not_fallback(T):
    import numpy as np
    f = T.TopeFFT()
    T.topeFFTInit(f)
    assert f.error == T.TOPE_ERR_CUDA
    assert T.topeGetLastError() == T.TOPE_ERR_CUDA
    assert T.topeGetLastError() == T.TOPE_SUCCESS  # reading resets
    t = T.TopePlan1D()
    d = np.zeros(16)
    T.tope1DPlanInit(f, t, 8, T.C2C, d)
    assert f.error != T.TOPE_SUCCESS and t.impl is None
    T.tope1DExec(f, t, d, T.FORWARD)
    assert f.error == T.TOPE_ERR_DESTROYED
    T.tope1DDestroy(f, t)
    assert f.error == T.TOPE_ERR_DESTROYED


def test_error_strings(T):
    for st in range(0, 9):
        assert T.topeErrorString(st)
    assert T.topeErrorString(999) == "unknown status"


def test_null_arguments_are_rejected(T):
    import numpy as np
    f = T.TopeFFT()
    t = T.TopePlan2D()
    # framework never initialised: PlanInit must fail cleanly, not crash
    T.lib.tope2DPlanInit(ctypes.byref(f), None, 4, 4, T.C2C, None)
    assert f.error == T.TOPE_ERR_INVALID_ARG
    T.tope2DPlanInit(f, t, 34, 4, T.C2C, np.zeros(272))  # 34 = 2 * 17
    assert f.error == T.TOPE_ERR_INVALID_SIZE
    T.tope2DPlanInit(f, t, 4, 4, 5, np.zeros(32))  # neither C2C nor R2C
    assert f.error == T.TOPE_ERR_UNSUPPORTED
