"""Device-side failure paths, exercised without a fault.

Every spin-wait in the kernels has an iteration limit.  The fit kernel's wait for the bulk
copy that stages the observations in shared memory takes its limit from the context
(ast_set_stage_wait); with 0 polls every CTA gives up at once, records the error word, reads the
observations from global memory instead and, before it exits, waits (with the full limit) for the
copy it issued.  The host then reports AST_E_TIMEOUT for the step, the step is still complete,
and the results must equal those of the staged run.  The context must stay usable afterwards.
"""
import ctypes as C

import numpy as np
import pytest

from asteroid_gb300 import api, capi

pytestmark = pytest.mark.gpu

CFG = dict(n_chains=1024, group_size=256, n_stages=2, seed=5, evals_cap=40, precision=api.PREC_MIXED)


def _run_steps(eng, polls):
    """fit_begin, then ast_fit_step until done (codes collected), then fit_end."""
    lib = capi.load()
    assert lib.ast_set_stage_wait(eng.ctx, int(polls)) == 0
    eng.fit_begin(**CFG, stage_obs=1)
    launch = eng.fit_launch()
    codes = []
    done = C.c_int32(0)
    for _ in range(64):
        codes.append(lib.ast_fit_step(eng.ctx, 0, C.byref(done), None))
        if done.value:
            break
    assert done.value == 1
    return launch, codes, eng.fit_end()


def test_staging_wait_timeout_is_reported_and_harmless(gpu, synth_objects):
    s = synth_objects("c0acc")  # 300 points: the observation block fits in shared memory
    with api.Engine(s.model, s.obs) as eng:
        launch, codes, ref = _run_steps(eng, 1 << 22)
        assert launch["smem"] > 0, "the block is not staged: the timeout path would not be taken"
        assert codes == [0] * len(codes)
        launch0, codes0, got = _run_steps(eng, 0)
        assert launch0["smem"] == launch["smem"]
        assert codes0 and all(c == -7 for c in codes0), codes0           # AST_E_TIMEOUT every launch
        assert b"staging wait ran out" in capi.load().ast_last_error()
        assert np.array_equal(got.best_f, ref.best_f)
        assert np.array_equal(got.best_params, ref.best_params)
        assert np.array_equal(got.best_dv, ref.best_dv)
        assert got.n_evals == ref.n_evals
        # ast_fit reports the timeout after completing the fit with the same results.
        with pytest.raises(capi.AstError) as ei:
            eng.fit(**CFG, stage_obs=1)
        assert ei.value.code == -7
        # The context is still usable: a normal fit and an evaluation afterwards.
        assert capi.load().ast_set_stage_wait(eng.ctx, 1 << 22) == 0
        again = eng.fit(**CFG, stage_obs=1)
        assert np.array_equal(again.best_f, ref.best_f)
        c, _ = eng.eval(ref.best_params[:2], api.PREC_FP64)
        assert np.all(np.isfinite(c))


def test_stage_wait_rejects_a_negative_limit(gpu, synth_objects):
    s = synth_objects("c0acc")
    with api.Engine(s.model, s.obs) as eng:
        assert capi.load().ast_set_stage_wait(eng.ctx, -1) == -1
