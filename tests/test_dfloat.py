"""The mixed-precision arithmetic on the CPU: the product's double-float operations, the
double-float magnitude of the NUDGE candidates and chi2_mixed, compiled for the host
(tests/host/mixed_harness.cu) and checked against 120-bit mpmath, the FP64 magnitude and the
oracle's FP64 chi^2."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import api, build

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def harness(built, tmp_path_factory):
    out = tmp_path_factory.mktemp("harness") / "libmixed_harness.so"
    cmd = [build._nvcc(), "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off", "-O2", "-std=c++17",
           f"-I{build.PKG / 'csrc'}", f"-I{build.INCLUDE}", str(ROOT / "tests" / "host" / "mixed_harness.cu"),
           "-o", str(out), f"-L{build.BUILD}", "-lasteroid_gb300", f"-Xlinker=-rpath={build.BUILD}"]
    subprocess.run(cmd, check=True, capture_output=True)
    lib = C.CDLL(str(out))
    lib.h_vmod_diff.restype = C.c_double
    lib.h_chi2_mixed.restype = C.c_double
    return lib


def _split(v):
    hi = np.float32(v)
    return float(hi), float(np.float32(v - np.float64(hi)))


def _run(lib, op, xs, ys):
    x = np.array([_split(v) for v in xs]).ravel()
    y = np.array([_split(v) for v in ys]).ravel()
    out = np.zeros(2 * len(xs))
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    lib.h_df_op(op, len(xs), P(x), P(y), P(out))
    return x, y, out


def _mp(a, i):
    import mpmath as mp

    return mp.mpf(a[2 * i]) + mp.mpf(a[2 * i + 1])


U2 = 2.0 ** -48  # u^2 for u = 2^-24


# Bounds: relative error for the arithmetic (Joldes, Muller & Popescu 2017: AccurateDWPlusDW 3u^2,
# DWTimesDW3 4u^2; the quotient with two corrections a few u^2), relative to max(|log|, 1) for the
# logarithm, absolute error for the angle functions (the e^3/6 term of sin e is carried in FP32).
@pytest.mark.parametrize("op,name,xr,yr,tol,relative", [
    (0, "add", (-1e3, 1e3), (-1e3, 1e3), 3.5 * U2, True),
    (2, "mul", (-1e3, 1e3), (-1e3, 1e3), 4.5 * U2, True),
    (4, "div", (-1e3, 1e3), (0.5, 1e3), 10 * U2, True),
    (5, "div_fast", (-1e3, 1e3), (0.5, 1e3), 30 * U2, True),
    (6, "sqrt", (1e-3, 1e6), (0, 1), 4 * U2, True),
    (7, "log", (1e-6, 1e6), (0, 1), 3e-14, "max1"),
    (8, "atan2", (-5, 5), (-5, 5), 1e-13, False),
    (9, "sin", (-7e4, 7e4), (0, 1), 2e-13, False),
    (10, "cos", (-3.5, 3.5), (0, 1), 2e-13, False),
])
def test_double_float_operations(harness, op, name, xr, yr, tol, relative):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 120
    rng = np.random.default_rng(op)
    xs, ys = rng.uniform(*xr, 600), rng.uniform(*yr, 600)
    x, y, out = _run(harness, op, xs, ys)
    ref = {0: lambda a, b: a + b, 2: lambda a, b: a * b, 4: lambda a, b: a / b, 5: lambda a, b: a / b,
           6: lambda a, b: mp.sqrt(a), 7: lambda a, b: mp.log(a), 8: lambda a, b: mp.atan2(a, b),
           9: lambda a, b: mp.sin(a), 10: lambda a, b: mp.cos(a)}[op]
    worst = 0.0
    for i in range(len(xs)):
        r = ref(_mp(x, i), _mp(y, i))
        err = abs(_mp(out, i) - r)
        scale = abs(r) if relative is True else (max(abs(r), mp.mpf(1)) if relative == "max1" else 1)
        worst = max(worst, float(err / scale))
    assert worst <= tol, f"{name}: {worst:.3e} > {tol:.3e}"


@pytest.mark.parametrize("name,flags", [("c0acc", None), ("c1bc", None), ("c0acc", "TORQUE,BW_BALL,ACC")])
def test_double_float_magnitude_matches_fp64(harness, synth_objects, name, flags):
    s = synth_objects(name)
    m = s.model if flags is None else api.make_model(flags, s.model.time_step, (2.0, 4800.0))
    rng = np.random.default_rng(3)
    P = []
    while len(P) < 4:
        p = api.x2params(m, rng.uniform(0, 1, m.n_params), reopt=1)
        if p is not None:
            P.append(p)
    cobs = s.obs.as_c()
    for p in P:
        A = np.ascontiguousarray(np.column_stack([rng.uniform(-np.pi, np.pi, 8), rng.uniform(0.05, 3.1, 8),
                                                  rng.uniform(-np.pi, np.pi, 8)]))
        p = np.ascontiguousarray(p)
        d = harness.h_vmod_diff(C.byref(m), C.byref(cobs), p.ctypes.data_as(C.c_void_p),
                                A.ctypes.data_as(C.c_void_p), 8)
        assert d <= 1e-10, d


def test_chi2_mixed_on_the_host_within_1e6_of_the_oracle(harness, oracle_mod, synth_objects):
    from tests.test_gpu_eval import well_conditioned

    s = synth_objects("c0acc")
    m, obs = s.model, s.obs
    rng = np.random.default_rng(5)
    iL = api.param_names(m).index("L")
    P = [s.params_true]
    while len(P) < 24:
        p = api.x2params(m, rng.uniform(0, 1, m.n_params), reopt=0)
        if p is not None and p[iL] * m.time_step <= 0.5:
            P.append(p)
    P = np.array(P)
    ref, _ = oracle_mod.chi2_batch(m, obs, P)
    good = well_conditioned(oracle_mod, m, obs, P)
    cobs = obs.as_c()
    dv = np.zeros(obs.n_filters)
    got = np.array([harness.h_chi2_mixed(C.byref(m), C.byref(cobs), np.ascontiguousarray(p).ctypes.data_as(C.c_void_p),
                                         dv.ctypes.data_as(C.c_void_p)) for p in P])
    ok = good & np.isfinite(ref) & (ref < 1e29)
    rel = np.abs(got[ok] - ref[ok]) / np.abs(ref[ok])
    assert ok.sum() >= 12 and np.all(rel <= 1e-6), rel.max()
