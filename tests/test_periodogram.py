"""Periodogram of model minima of -plot mode (minima(), misc.c:65-276): the oracle pinned to the
reference's own build and to its golden vectors (CPU), and the CUDA interval count against both
(GPU), bit for bit: the counts are integers, the normalisation follows the reference's order."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import api, capi

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = json.loads((ROOT / "tests" / "golden" / "minima_ref.json").read_text())["cases"]
REF_LIB = ROOT / "oracle" / "_ref" / "libref_minima.so"


def case_inputs(c):
    t = np.arange(c["n"]) * c["h"]
    vm = np.asarray(c["vm_scaled"], dtype=np.int64).astype(np.float64) / c["scale"]
    return t, vm


def same(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray([np.nan if x is None else x for x in b], dtype=float)
    return np.array_equal(a, b, equal_nan=True)


def noisy_curve(n, span, seed, period=0.4, noise=0.05):
    rng = np.random.default_rng(seed)
    t = np.arange(n) * (span / (n - 1))
    return t, 0.3 * np.sin(2 * np.pi * t / period) + noise * rng.standard_normal(n)


@pytest.mark.parametrize("c", GOLDEN, ids=[c["kind"] for c in GOLDEN])
def test_oracle_matches_reference_golden(built, oracle_mod, c):
    t, vm = case_inputs(c)
    fr, h, counts, n = oracle_mod.minima(t, vm)
    assert n == c["n_minima"]
    assert same(fr, c["cl_fr"]) and same(h, c["cl_H"]), (fr, h, c["cl_fr"], c["cl_H"])
    assert counts.sum() <= 10000 * n * (n - 1) // 2


@pytest.mark.skipif(not REF_LIB.exists(), reason="reference build oracle/_ref/libref_minima.so not present")
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_oracle_matches_reference_build(built, oracle_mod, seed):
    import ctypes as C
    lib = C.CDLL(str(REF_LIB))
    lib.refm_minima.restype = C.c_int
    rng = np.random.default_rng(seed)
    t, vm = noisy_curve(int(rng.integers(1000, 4000)), float(rng.uniform(2, 20)), seed,
                        period=float(rng.uniform(0.1, 1.0)), noise=float(rng.uniform(0, 0.1)))
    fr, h = np.zeros(5), np.zeros(5)
    n_ref = lib.refm_minima(t.ctypes.data_as(C.c_void_p), vm.ctypes.data_as(C.c_void_p), t.size,
                            fr.ctypes.data_as(C.c_void_p), h.ctypes.data_as(C.c_void_p))
    ofr, oh, _, n = oracle_mod.minima(t, vm)
    assert n == n_ref
    assert np.array_equal(fr, ofr, equal_nan=True) and np.array_equal(h, oh, equal_nan=True)


def test_oracle_refuses_too_many_minima(built, oracle_mod):
    n = 20006
    t = np.arange(n) * 1e-4
    vm = np.where(np.arange(n) % 2 == 1, 1.0, 0.0)   # 10002 minima
    with pytest.raises(ValueError):
        oracle_mod.minima(t, vm)


@pytest.mark.gpu
@pytest.mark.parametrize("c", GOLDEN, ids=[c["kind"] for c in GOLDEN])
def test_gpu_matches_reference_golden(gpu, c):
    t, vm = case_inputs(c)
    r = api.minima(t, vm)
    assert r.n_minima == c["n_minima"] and r.n_intervals == r.n_minima * (r.n_minima - 1) // 2
    assert same(r.cl_fr, c["cl_fr"]) and same(r.cl_H, c["cl_H"]), (r.cl_fr, r.cl_H, c["cl_fr"], c["cl_H"])
    assert r.n_clusters == sum(1 for x in c["cl_fr"] if x != -1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("n,span,seed,period,noise", [(6000, 20.0, 21, 0.37, 0.05), (20000, 60.0, 22, 0.21, 0.02),
                                                      (4000, 3.0, 23, 0.05, 0.0)])
def test_gpu_counts_equal_oracle(gpu, oracle_mod, n, span, seed, period, noise):
    """Every one of the 10000 counts, over up to 2e10 interval tests, equals the oracle's."""
    t, vm = noisy_curve(n, span, seed, period, noise)
    fr, h, counts, n_min = oracle_mod.minima(t, vm)
    r = api.minima(t, vm)
    assert r.n_minima == n_min
    assert np.array_equal(r.counts, counts)
    assert np.array_equal(r.cl_fr, fr) and np.array_equal(r.cl_H, h)


@pytest.mark.gpu
def test_gpu_refused_inputs(gpu):
    t = np.arange(100) * 0.01
    with pytest.raises(capi.AstError, match="increase"):
        api.minima(t[::-1].copy(), np.sin(t))
    n = 20006
    t = np.arange(n) * 1e-4
    vm = np.where(np.arange(n) % 2 == 1, 1.0, 0.0)
    with pytest.raises(capi.AstError, match="NMIN_MAX"):
        api.minima(t, vm)
    r = api.minima(t[:2], vm[:2])     # too short for a minimum
    assert r.n_minima == 0 and list(r.cl_fr) == [-1.0] * 5


@pytest.mark.gpu
def test_gpu_plot_curve_periodogram(gpu, oracle_mod, synth_objects):
    """The -plot sequence: model curve on the plot grid shifted by delta_V[0], then minima()."""
    s = synth_objects("c0acc")
    t, e, u = api.plot_grid(s.dir / "lc.dat", s.dir, 20000)
    with api.Engine(s.model, s.obs) as eng:
        _, dv = eng.eval(np.asarray(s.params_true)[None, :])
        vm = eng.model_curve_at(s.params_true, t, e, u) + dv[0, 0]
    fr, h, counts, n_min = oracle_mod.minima(t, vm)
    r = api.minima(t, vm)
    assert r.n_minima == n_min >= 2
    assert np.array_equal(r.counts, counts) and np.array_equal(r.cl_fr, fr) and np.array_equal(r.cl_H, h)
