"""Pin of the oracle's simplex driver against the reference's own chi2_gpu.

oracle/build_ref.sh compiles the reference's chi2_gpu kernel (cuda.c:1326-1833) from its
sources as host code (libref_nm_<variant>.so): a block's threads run as host threads with a
barrier for __syncthreads, and its cuRAND draws are the engine's Philox stream, the only
substitution, so that both sides start their chains from the same points.  Everything else --
the random start rules, the simplex steps, the block's serial argmin, the P_PSI re-meaning of x
at the stage hand-off, the final x2params and delta_V -- is the reference's code.  The oracle
(oracle/nm_oracle_*.h, whose chains the GPU fit kernel follows in tests/test_gpu_fit.py) must
give the same block results bit for bit: two stages of 2 x 256 chains of N_STEPS = 100 (the
reference's -DTIMING value), random and -reopt starts, on the fixture objects of two variants and
on a 400-point NUDGE object (the fixture's 120 points give no admissible minima: every chain
would end at the 1e30 penalty).
"""
from pathlib import Path

import numpy as np
import pytest

from tests.test_oracle_pin import EXACT, GOLDEN, load_fixture

REF_DIR = Path(__file__).resolve().parents[1] / "oracle" / "_ref"


def _compare(oracle_mod, variant, m, obs, reopt, p0):
    ref = oracle_mod.RefNM(variant)
    a = ref.fit(m, obs, seed=5, n_blocks=2, n_stages=2, reopt=reopt, params0=p0)
    b = oracle_mod.fit(m, obs, seed=5, n_chains=2 * ref.block_size, group_size=ref.block_size, n_stages=2,
                       reopt=reopt, params0=p0, steps_cap=ref.n_steps)
    print(variant, "reopt" if reopt else "random", "block best chi2", a["best_f"])
    assert np.all(a["best_f"] < 1e29)
    assert np.array_equal(a["best_f"], b["best_f"])
    assert np.array_equal(a["best_params"], b["best_params"])
    assert np.array_equal(a["best_dv"], b["best_dv"])


def _need(variant):
    if not (REF_DIR / f"libref_nm_{variant}.so").exists() or not EXACT:
        pytest.skip("reference simplex host build not present (it is built where the reference checkout exists)")


@pytest.mark.parametrize("variant", ["ppsi_torque_acc", "bc_interp_sp"])
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
