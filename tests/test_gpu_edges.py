"""Edge cases of the evaluation and the fit: the largest object (AST_MAX_DATA observations in
AST_MAX_FILTERS filters), frozen parameters, the NUDGE "more than M_MAX minima" rejection, a
rotation phase beyond the double-float fast sin/cos range within one observation gap, and inputs
the entry points must refuse."""
import ctypes as C

import numpy as np
import pytest

from asteroid_gb300 import api, capi

pytestmark = pytest.mark.gpu


def _resolved(model, n, seed, reopt=0):
    """Parameter vectors from the prior that the fixed-step RK4 resolves (h L <= 0.5)."""
    rng = np.random.default_rng(seed)
    iL = api.param_names(model).index("L")
    out = []
    while len(out) < n:
        p = api.x2params(model, rng.uniform(0, 1, model.n_params), reopt=reopt)
        if p is not None and p[iL] * model.time_step <= 0.5:
            out.append(p)
    return np.array(out)


def _geometry(n, seed):
    """Unit asteroid->Earth and asteroid->Sun vectors, slowly varying, phase angle ~35 deg."""
    rng = np.random.default_rng(seed)
    a = 0.2 + 0.05 * np.linspace(0, 1, n) + 1e-3 * rng.standard_normal(n)
    e = np.column_stack([np.cos(a), np.sin(a), 0.1 * np.ones(n)])
    s = np.column_stack([np.cos(a + 0.6), np.sin(a + 0.6), 0.05 * np.ones(n)])
    return e / np.linalg.norm(e, axis=1)[:, None], s / np.linalg.norm(s, axis=1)[:, None]


def test_largest_object_matches_oracle(gpu, oracle_mod):
    from tests.test_gpu_eval import well_conditioned

    n, nf = 16384, 8
    rng = np.random.default_rng(77)
    t = np.sort(rng.uniform(0.0, 2.0, n))
    e, sv = _geometry(n, 77)
    filt = np.arange(n, dtype=np.int32) % nf
    obs = api.Obs(t, rng.normal(0.0, 0.3, n), np.full(n, 100.0), filt, e, sv)
    m = api.make_model("TORQUE,ACC", 1e-2)
    P = _resolved(m, 8, 5, reopt=1)
    ref, rdv = oracle_mod.chi2_batch(m, obs, P)
    good = well_conditioned(oracle_mod, m, obs, P)
    with api.Engine(m, obs) as eng:
        got, dv = eng.eval(P, api.PREC_FP64)
        mix, _ = eng.eval(P, api.PREC_MIXED)
        res = eng.fit(n_chains=256, group_size=128, seed=3, evals_cap=20, precision=api.PREC_MIXED)
    ok = good & np.isfinite(ref) & (ref < 1e29)
    assert ok.sum() >= 4
    assert np.all(np.abs(got[ok] - ref[ok]) <= 1e-9 * np.abs(ref[ok]))
    assert np.all(np.abs(dv[ok] - rdv[ok]) <= 1e-9 * np.maximum(np.abs(rdv[ok]), 1))
    assert np.all(np.abs(mix[ok] - got[ok]) <= 1e-6 * np.abs(got[ok]))
    assert res.best_dv.shape == (2, nf) and np.all(np.isfinite(res.best_f))


def test_frozen_parameters_stay_at_their_value(gpu, oracle_mod, synth_objects):
    s = synth_objects("c0acc")
    m = api.make_model("TORQUE,P_PSI,ACC", s.model.time_step, (2.0, 4800.0))
    lib = capi.load()
    assert lib.ast_model_freeze(C.byref(m), m.ids.Ti, 0.25) == 0
    assert lib.ast_model_freeze(C.byref(m), m.ids.theta_M, 1.1) == 0
    iTi, iTh = api.param_names(m).index("Ti"), api.param_names(m).index("theta_M")
    for prec in (api.PREC_FP64, api.PREC_MIXED):
        with api.Engine(m, s.obs) as eng:
            res = eng.fit(n_chains=128, group_size=64, seed=9, evals_cap=40, precision=prec)
        ok = res.best_f < 1e29
        assert ok.any()
        assert np.all(res.best_params[ok, iTi] == 0.25) and np.all(res.best_params[ok, iTh] == 1.1)
    # and chain by chain like the CPU driver (most chains; see test_fit_matches_oracle_chains)
    with api.Engine(m, s.obs) as eng:
        res = eng.fit(n_chains=128, group_size=64, seed=9, evals_cap=40)
    ref = oracle_mod.fit(m, s.obs, seed=9, n_chains=128, group_size=64, evals_cap=40)
    a, b = res.chain_f, ref["chain_f"]
    fin = np.isfinite(a) & np.isfinite(b) & (a < 1e29) & (b < 1e29)
    assert np.mean(np.abs(a[fin] - b[fin]) <= 1e-6 * np.abs(b[fin])) > 0.8


def test_nudge_rejects_models_with_too_many_minima(gpu, oracle_mod, synth_objects):
    """Random starts on the NUDGE object often produce more than M_MAX model minima near the
    observed ones; the reference then returns 1e30 (cuda.c:737-742), and so must both paths."""
    s = synth_objects("c2")
    P = _resolved(s.model, 48, 21, reopt=1)
    ref, _ = oracle_mod.chi2_batch(s.model, s.obs, P)
    rejected = ref >= 1e29
    assert rejected.sum() >= 3
    with api.Engine(s.model, s.obs) as eng:
        got, _ = eng.eval(P, api.PREC_FP64)
        mix, _ = eng.eval(P, api.PREC_MIXED)
    assert np.all(got[rejected] >= 1e29) and np.all(mix[rejected] >= 1e29)
    assert np.all(got[~rejected] < 1e29)


def test_phase_beyond_the_fast_sincos_range_in_one_gap(gpu, oracle_mod):
    """Two nights 118 days apart and L ~ 700 rad/day: the rotation phase grows by ~8e4 rad within
    one observation gap, past the double-float sin/cos fast range (|angle| <= 65 536), where the
    mixed path reduces the angle by 2 pi first."""
    from tests.test_gpu_eval import well_conditioned

    rng = np.random.default_rng(88)
    t = np.sort(np.concatenate([rng.uniform(0.0, 0.12, 30), 118.0 + rng.uniform(0.0, 0.12, 30)]))
    n = t.size
    e, sv = _geometry(n, 88)
    obs = api.Obs(t, np.full(n, 0.3), np.full(n, 100.0), np.zeros(n, np.int32), e, sv)
    m = api.make_model("TORQUE,ACC", 5e-4)
    names = api.param_names(m)
    P = _resolved(m, 6, 12, reopt=1)
    P[:, names.index("L")] = np.linspace(650.0, 720.0, len(P))
    with api.Engine(m, obs) as eng:
        got, _ = eng.eval(P, api.PREC_FP64)
        mix, _ = eng.eval(P, api.PREC_MIXED)
        a64 = eng.model_angles(P[0], api.PREC_FP64)
        a32 = eng.model_angles(P[0], api.PREC_MIXED)
    assert np.abs(a64).max() > 65536 + 10
    drift = np.abs((a32 - a64 + np.pi) % (2 * np.pi) - np.pi).max()
    assert drift < 1e-6, drift
    # 236 000 RK4 steps of a torqued tumbler: some vectors are chaotic (their FP64 chi^2 moves
    # under a one-ulp change of the parameters); only the well-conditioned ones are compared.
    good = well_conditioned(oracle_mod, m, obs, P)
    fin = good & np.isfinite(got) & (got < 1e29)
    assert fin.sum() >= 2
    assert np.all(np.abs(mix[fin] - got[fin]) <= 1e-6 * np.abs(got[fin])), np.abs(mix[fin] - got[fin]) / got[fin]


def test_entry_points_refuse_bad_inputs(gpu, synth_objects):
    s = synth_objects("c0acc")
    lib = capi.load()
    ctx = C.c_void_p()
    o = s.obs
    n = 5  # fewer observations than parameters + filters
    small = api.Obs(o.mjd[:n].copy(), o.v[:n].copy(), o.w[:n].copy(), o.filt[:n].copy(), o.e_unit[:n].copy(),
                    o.s_unit[:n].copy())
    cobs = small.as_c()
    assert lib.ast_prepare(C.byref(s.model), C.byref(cobs), -1, C.byref(ctx)) < 0 and not ctx
    with api.Engine(s.model, s.obs) as eng:
        with pytest.raises(capi.AstError):
            eng.fit(n_chains=100, group_size=64)  # not a multiple of the group size
        cfg = capi.FitCfg()
        cfg.seed, cfg.n_chains, cfg.group_size, cfg.n_stages, cfg.reopt = 1, 64, 64, 1, 1  # reopt, no params0
        assert lib.ast_fit_begin(eng.ctx, C.byref(cfg)) < 0 and b"params0" in lib.ast_last_error()
