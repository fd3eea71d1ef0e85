"""Pin of the oracle against the reference's own chi^2 code.

tests/golden/ref_<variant>.json hold outputs of the reference's chi2one / x2params / params2x,
compiled from its sources (oracle/build_ref.sh) and run on the fixture's inputs
(tests/golden/make_golden.py).  The oracle must reproduce them bit for bit on x86-64, where they
were generated; on another architecture the host libm may round differently, so there the bar
is a tight relative tolerance.  When oracle/_ref is built (here, with the reference checkout),
random vectors are compared against it directly as well.
"""
import json
import platform
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import api

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("ref_*.json"))
EXACT = platform.machine() in ("x86_64", "AMD64")


def load_fixture(path):
    fx = json.loads(path.read_text())
    m = api.make_model(fx["flags"], fx["time_step"], tuple(fx["ppsi_hours"]))
    o = fx["obs"]
    obs = api.Obs(np.array(o["mjd"]), np.array(o["v"]), np.array(o["w"]), np.array(o["filt"]),
                  np.array(o["e_unit"]), np.array(o["s_unit"]), np.array(o["eph_e"]), np.array(o["eph_s"]),
                  np.array(o["eph_mjd0"]), np.array(o["t_min"]), np.array(o["v_min"]))
    return fx, m, obs


def same(a, b, rtol=1e-12):
    a, b = np.asarray(a, float), np.asarray(b, float)
    if EXACT:
        return np.array_equal(a, b, equal_nan=True)
    return np.allclose(a, b, rtol=rtol, atol=0, equal_nan=True)


def test_fixtures_present():
    assert len(FIXTURES) >= 8


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_chi2_matches_reference(built, oracle_mod, path):
    fx, m, obs = load_fixture(path)
    for p, c_ref, dv_ref in zip(fx["params"], fx["chi2"], fx["delta_v"]):
        c, dv = oracle_mod.chi2(m, obs, np.array(p))
        assert same([c], [c_ref]), (c, c_ref)
        assert same(dv, dv_ref), (dv, dv_ref)


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_maps_match_reference(built, oracle_mod, path):
    fx, m, obs = load_fixture(path)
    for reopt in (0, 1):
        for x, p_ref in zip(fx["x"], fx["x2params"][str(reopt)]):
            p = oracle_mod.x2params(m, np.array(x), reopt=reopt)
            assert (p is None) == (p_ref is None)
            if p is not None:
                assert same(p, p_ref), (p, p_ref)
    for p, x_ref in zip(fx["params"], fx["params2x"]):
        assert same(oracle_mod.params2x(m, np.array(p)), x_ref)


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_engine_host_maps_match_reference(built, path):
    """The engine's x2params/params2x (the code the kernels run, compiled for the host)."""
    fx, m, obs = load_fixture(path)
    for reopt in (0, 1):
        for x, p_ref in zip(fx["x"], fx["x2params"][str(reopt)]):
            p = api.x2params(m, np.array(x), reopt=reopt)
            assert (p is None) == (p_ref is None)
            if p is not None:
                assert np.allclose(p, p_ref, rtol=1e-14, atol=0)


REF_DIR = Path(__file__).resolve().parents[1] / "oracle" / "_ref"


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_random_vectors_against_reference_build(built, oracle_mod, path):
    fx, m, obs = load_fixture(path)
    lib = REF_DIR / f"libref_{fx['variant']}.so"
    if not lib.exists() or not EXACT:
        pytest.skip("reference host build not present (it is built where the reference checkout exists)")
    ref = oracle_mod.RefHost(fx["variant"])
    rng = np.random.default_rng(11)
    n = 0
    for _ in range(60):
        x = rng.uniform(0, 1, m.n_params)
        for reopt in (0, 1):
            p = oracle_mod.x2params(m, x, reopt=reopt)
            q = ref.x2params(m, x, reopt=reopt)
            assert (p is None) == (q is None)
            if p is None:
                continue
            assert np.array_equal(p, q)
            c1, d1 = oracle_mod.chi2(m, obs, p)
            c2, d2 = ref.chi2(m, obs, p)
            assert np.array_equal([c1], [c2], equal_nan=True)
            assert np.array_equal(d1, d2[: obs.n_filters], equal_nan=True)
            n += 1
    assert n > 20


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_model_curve_matches_reference_plot_branch(built, oracle_mod, path):
    """The model curve (chi2one with Nplot > 0, the branch chi2_plot and the -plot mode use,
    cuda.c:699-704) from the reference's host build equals the oracle's, bit for bit, for every
    fixture parameter vector (the reference does not support the branch under NUDGE)."""
    fx, m, obs = load_fixture(path)
    lib = REF_DIR / f"libref_{fx['variant']}.so"
    if not lib.exists() or not EXACT:
        pytest.skip("reference host build not present (it is built where the reference checkout exists)")
    if "NUDGE" in fx["flags"]:
        pytest.skip("the reference's plot branch is not defined under NUDGE")
    ref = oracle_mod.RefHost(fx["variant"])
    for p in fx["params"]:
        a = ref.model_curve(m, obs, np.array(p))
        b = oracle_mod.model_curve(m, obs, np.array(p))
        assert np.array_equal(a, b, equal_nan=True)
