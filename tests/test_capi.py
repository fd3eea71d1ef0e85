"""The C ABI: the library loads without a GPU and exports every function the header declares."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from asteroid_gb300 import api, capi

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(ast_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(built):
    lib = capi.load()
    names = header_functions()
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(built):
    names = header_functions()
    assert names <= set(capi.SIGNATURES), sorted(names - set(capi.SIGNATURES))


def test_prepare_without_device_fails_cleanly(built):
    """No GPU here: ast_prepare returns a status instead of aborting the process."""
    from tests.conftest import _gpu_available

    if _gpu_available():
        return
    m = api.make_model("TORQUE,P_PSI,ACC")
    n = 40
    o = api.Obs(np.arange(n) * 0.01, np.zeros(n), np.ones(n), np.zeros(n, np.int32),
                np.tile([1.0, 0, 0], n), np.tile([0, 1.0, 0], n))
    cobs = o.as_c()
    ctx = C.c_void_p()
    rc = capi.load().ast_prepare(C.byref(m), C.byref(cobs), -1, C.byref(ctx))
    assert rc in (-9, -3)  # AST_E_NODEVICE or AST_E_CUDA
    assert not ctx


def test_version_and_errors(built):
    lib = capi.load()
    assert b"sm_103a" in lib.ast_version()
    rc = lib.ast_model_init(None, 0, 1e-2, 2.0, 4800.0)
    assert rc == -1 and lib.ast_last_error()
