"""Pin of the oracle's simplex driver and RMSD sampler against the reference's own kernels.

oracle/build_ref.sh compiles the reference's chi2_gpu (cuda.c:1326-1833) and, in -DRMSD builds,
chi2_gpu_rms (cuda.c:2148-2389) from its sources as host code (libref_nm_<variant>.so): a block's
threads run as host threads with a barrier for __syncthreads, and its cuRAND draws are the
engine's Philox stream, the only substitution, so that both sides draw the same points.
Everything else is the reference's code.

Simplex: the random start rules, the simplex steps, the block's serial argmin, the P_PSI
re-meaning of x at the stage hand-off, the final x2params and delta_V.  The oracle
(oracle/nm_oracle_*.h, whose chains the GPU fit kernel follows in tests/test_gpu_fit.py) must give
the same block results bit for bit: two stages of a block of 256 chains of N_STEPS = 100 (the
reference's -DTIMING value), random and -reopt starts, on the fixture objects of eight variants
(every non-RMSD fixture: P_PSI, TORQUE, INTERP, BC, BW_BALL, free rotation; CHI_FLOAT double and
float) and on a 400-point NUDGE object (the fixture's 120 points give no admissible minima: every chain would
end at the 1e30 penalty).

RMSD: the normal-draw perturbation with its hard-limit clamps, x2params, the one-sigma RMSD test,
the periodic-angle and SPHERICAL_K conversions and the float min/max reductions.  The oracle
(oracle/rmsd_oracle*.h, which the GPU sampler matches in tests/test_rmsd.py) must give the same
f0, f1, sample counts and parameter ranges bit for bit, for two launch indices of the host loop.

tests/golden/drivers_ref.json (tests/golden/make_driver_golden.py) keeps the reference builds'
results for the fixture objects, so the oracle is checked against them where the reference is
absent too (bit for bit on x86-64, where they were generated; to 1e-12 elsewhere).
"""
from pathlib import Path

import numpy as np
import pytest

import json

from tests.test_oracle_pin import EXACT, GOLDEN, load_fixture, same

REF_DIR = Path(__file__).resolve().parents[1] / "oracle" / "_ref"


def _compare(oracle_mod, variant, m, obs, reopt, p0):
    ref = oracle_mod.RefNM(variant)
    a = ref.fit(m, obs, seed=5, n_blocks=1, n_stages=2, reopt=reopt, params0=p0)
    b = oracle_mod.fit(m, obs, seed=5, n_chains=ref.block_size, group_size=ref.block_size, n_stages=2,
                       reopt=reopt, params0=p0, steps_cap=ref.n_steps)
    print(variant, "reopt" if reopt else "random", "block best chi2", a["best_f"])
    assert np.all(a["best_f"] < 1e29)
    assert np.array_equal(a["best_f"], b["best_f"])
    assert np.array_equal(a["best_params"], b["best_params"])
    assert np.array_equal(a["best_dv"], b["best_dv"])


def _need(variant):
    if not (REF_DIR / f"libref_nm_{variant}.so").exists() or not EXACT:
        pytest.skip("reference simplex host build not present (it is built where the reference checkout exists)")


@pytest.mark.parametrize("variant", ["ppsi_torque_acc", "ppsi_torque_sp", "torque_interp_acc", "bc_interp_acc",
                                     "bw_torque_acc", "bc_torque_ppsi_acc", "free_acc", "bc_interp_sp"])
@pytest.mark.parametrize("reopt", [False, True], ids=["random", "reopt"])
def test_oracle_simplex_equals_reference_chi2_gpu(built, oracle_mod, variant, reopt):
    _need(variant)
    fx, m, obs = load_fixture(GOLDEN / f"ref_{variant}.json")
    _compare(oracle_mod, variant, m, obs, reopt, np.array(fx["params"][0]) if reopt else None)


def test_oracle_simplex_equals_reference_chi2_gpu_nudge(built, oracle_mod, tmp_path):
    _need("c2_nudge_acc")
    from asteroid_gb300 import synth

    cfg = synth.SynthConfig("nudge400", "TORQUE,P_PSI,INTERP,ACC,NUDGE", 5e-3, 400, 2, 10, 5, seed=1007,
                            n_minima=3, filter_chars="RV", dv_range=0.5, ppsi_hours=(20.0, 4800.0))
    s = synth.generate(cfg, tmp_path / "nudge400", vmod_fn=lambda m, o, p: oracle_mod.model_curve(m, o, p))
    _compare(oracle_mod, "c2_nudge_acc", s.model, s.obs, True, s.params_true)


@pytest.mark.parametrize("variant,fixture,spherical", [("rmsd_ppsi_torque_acc", "rmsd_ppsi_torque_acc", False),
                                                       ("rmsd_sph_ppsi_torque_acc", "rmsd_ppsi_torque_acc", True),
                                                       ("rmsd_bc_interp_sp", "rmsd_bc_interp_sp", False)])
def test_oracle_rmsd_equals_reference_chi2_gpu_rms(built, oracle_mod, variant, fixture, spherical):
    _need(variant)
    fx, m, obs = load_fixture(GOLDEN / f"ref_{fixture}.json")
    ref = oracle_mod.RefNM(variant)
    p0 = np.array(fx["params"][0])
    for call in (0, 3):
        a = ref.rmsd(m, obs, p0, seed=9, call=call, n_blocks=2, samples=8, dx=2e-5)
        b = oracle_mod.rmsd(m, obs, p0, seed=9, call=call, n_streams=2 * ref.block_size, samples=8, dx=2e-5, reopt=1,
                            spherical=spherical)
        print(variant, call, "points", a["n_tot"], "rejected", a["n_bad"])
        assert a["n_tot"] == b["n_tot"] and a["n_bad"] == b["n_bad"]
        assert a["n_tot"] - a["n_bad"] > 100  # enough accepted points for the ranges to mean something
        assert np.float32(b["f0"]) == np.float32(a["f0"]) and np.float32(b["f1"]) == np.float32(a["f1"])
        assert np.array_equal(np.float32(b["par_min"]), a["par_min"])
        assert np.array_equal(np.float32(b["par_max"]), a["par_max"])


DRIVERS = json.loads((GOLDEN / "drivers_ref.json").read_text())


@pytest.mark.parametrize("case", DRIVERS["simplex"],
                         ids=[f"{c.get('fixture', 'nudge400')}-{'reopt' if c['reopt'] else 'random'}"
                              for c in DRIVERS["simplex"]])
def test_oracle_simplex_matches_reference_golden(built, oracle_mod, case, tmp_path):
    if "synth" in case:
        from asteroid_gb300 import synth

        cfg = synth.SynthConfig(**{k: tuple(v) if isinstance(v, list) else v for k, v in case["synth"].items()})
        s = synth.generate(cfg, tmp_path / cfg.name, vmod_fn=lambda m, o, p: oracle_mod.model_curve(m, o, p))
        m, obs, p0 = s.model, s.obs, s.params_true
    else:
        fx, m, obs = load_fixture(GOLDEN / f"ref_{case['fixture']}.json")
        p0 = None if case["params0"] is None else np.array(case["params0"])
    b = oracle_mod.fit(m, obs, seed=case["seed"], n_chains=case["n_chains"], group_size=case["n_chains"],
                       n_stages=case["n_stages"], reopt=case["reopt"], params0=p0, steps_cap=case["steps_cap"])
    assert same(b["best_f"], case["best_f"])
    assert same(b["best_params"], case["best_params"])
    assert same(b["best_dv"], case["best_dv"])


@pytest.mark.parametrize("case", DRIVERS["rmsd"], ids=[f"{c['build']}-call{c['call']}" for c in DRIVERS["rmsd"]])
def test_oracle_rmsd_matches_reference_golden(built, oracle_mod, case):
    fx, m, obs = load_fixture(GOLDEN / f"ref_{case['fixture']}.json")
    b = oracle_mod.rmsd(m, obs, np.array(case["params0"]), seed=case["seed"], call=case["call"],
                        n_streams=case["n_streams"], samples=case["samples"], dx=case["dx"], reopt=1,
                        spherical=case["spherical"])
    f32 = lambda v: np.float32(np.asarray(v, dtype=np.float64)).astype(np.float64)
    assert same(f32([b["f0"], b["f1"]]), [case["f0"], case["f1"]])
    assert same(f32(b["par_min"]), case["par_min"]) and same(f32(b["par_max"]), case["par_max"])
    if EXACT:
        assert (b["n_tot"], b["n_bad"]) == (case["n_tot"], case["n_bad"])
