"""The C ABI library loads, exports every declared symbol, and its struct layout
matches the header (checked with the host C compiler). No GPU calls."""
import ctypes
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from volumefluxes_sm103 import _native as N

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(vf_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    return N.load(build_if_missing=True)


def test_library_exports_every_declared_symbol(lib):
    decl = declared_functions()
    assert decl, "no declarations found"
    missing = [n for n in decl if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(N.EXPORTED_SYMBOLS) == decl


@pytest.mark.parametrize("ctype,cname", [(N.VfConfig, "vf_config"), (N.VfBatchOptions, "vf_batch_options")])
def test_struct_layouts_match_header(tmp_path, ctype, cname):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in ctype._fields_]
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "volumefluxes_sm103.h"', "int main(void){",
           f'printf("%zu\\n", sizeof({cname}));']
    src += [f'printf("%zu\\n", offsetof({cname}, {f}));' for f in fields]
    src += ["return 0;}"]
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run([cc, f"-I{ROOT / 'include'}", str(c), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert out[0] == ctypes.sizeof(ctype)
    assert out[1:] == [getattr(ctype, f).offset for f in fields]


def _cfg(**kw):
    c = N.VfConfig()
    c.abi_version = N.VF_ABI_VERSION
    c.nx, c.ny, c.gc = 16, 16, 2
    for i, v in enumerate((0.0, 1.0, 0.0, 1.0)):
        c.extent[i] = v
    c.real_bytes = 8
    c.g, c.rho, c.depth_cutoff, c.desingularizing_kappa = 9.81, 1.0, 1e-5, 1e-5
    c.reconstruction, c.theta = N.VF_REC_LINEAR, 1.2
    c.stepper, c.bc, c.cfl = N.VF_STEPPER_RK2, N.VF_BC_WALL, 0.25
    c.bottom_is_constant = 1
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("bad", [
    {"gc": 1}, {"nx": 1}, {"real_bytes": 2}, {"stepper": 7}, {"bc": 4}, {"reconstruction": 0}, {"friction": 9},
    {"abi_version": 99}, {"cfl": 0.0}, {"bottom_constant": 1.0}, {"desingularizing_kappa": 0.0},
])
def test_create_rejects_invalid_configurations_without_touching_the_gpu(lib, bad):
    h = ctypes.c_void_p()
    rc = lib.vf_create(ctypes.byref(_cfg(**bad)), ctypes.byref(h))
    assert rc == N.VF_EINVAL
    assert not h.value
    assert lib.vf_last_error(None)


def test_nonzero_constant_bottom_needs_bottom_source(lib):
    h = ctypes.c_void_p()
    assert lib.vf_create(ctypes.byref(_cfg(bottom_constant=2.0)), ctypes.byref(h)) == N.VF_EINVAL
    assert b"source term" in lib.vf_last_error(None)


def test_null_handles_are_rejected(lib):
    assert lib.vf_step(None, 1.0, 0.0, None) == N.VF_EINVAL
    assert lib.vf_water_volume(None, None) == N.VF_EINVAL
    assert lib.vf_launch_count(None) == 0


def test_batch_rejects_bad_arguments_without_touching_the_gpu(lib):
    b = ctypes.c_void_p()
    t = (ctypes.c_double * 1)(0.0)
    assert lib.vf_batch_launch(None, 1, t, t, 1, -1.0, 0, None, ctypes.byref(b)) == N.VF_EINVAL
    hs = (ctypes.c_void_p * 1)(None)
    assert lib.vf_batch_launch(hs, 1, t, t, 1, -1.0, 0, None, ctypes.byref(b)) == N.VF_EINVAL
    assert b"NULL handle" in lib.vf_batch_last_error(None)
    assert lib.vf_batch_launch(hs, 0, t, t, 1, -1.0, 0, None, ctypes.byref(b)) == N.VF_EINVAL
    assert not b.value
    assert lib.vf_batch_poll(None, None) == N.VF_EINVAL
    assert lib.vf_batch_free(None) == N.VF_OK


def test_server_rejects_requests_without_touching_the_gpu(lib):
    s = ctypes.c_void_p()
    assert lib.vf_server_create(0, 0, None, 0, ctypes.byref(s)) == N.VF_EINVAL
    assert lib.vf_server_create(0, 1 << 20, None, 0, ctypes.byref(s)) == N.VF_OK
    import numpy as np
    w = np.zeros((16, 16))
    tk = ctypes.c_int64()
    big = _cfg(nx=1024, ny=1024)
    rc = lib.vf_server_submit(s, ctypes.byref(big), None, w.ctypes.data, w.ctypes.data, w.ctypes.data, 0.0, 1.0,
                              None, None, None, ctypes.byref(tk))
    assert rc == N.VF_ENOMEM and b"budget" in lib.vf_server_last_error(s)
    tab = _cfg(n_sources=1)
    tab.source_kind[0] = N.VF_SRC_TIME_RAIN
    rc = lib.vf_server_submit(s, ctypes.byref(tab), None, w.ctypes.data, w.ctypes.data, w.ctypes.data, 0.0, 1.0,
                              None, None, None, ctypes.byref(tk))
    assert rc == N.VF_EINVAL
    assert lib.vf_server_result(s, 12345, None, None, None, None) == N.VF_EINVAL
    assert lib.vf_server_destroy(s) == N.VF_OK
