"""chi^2 batch evaluation on the GPU (FP64 plain path) against the oracle.

Tolerances: the oracle is compiled without fused multiply-adds and with the host libm, the
kernel with nvcc's contractions and CUDA's libm, so the two differ by rounding only.  Rounding
differences stay at that level for well-conditioned vectors and are amplified without bound where
the fixed-step RK4 is unstable (fast or torque-spun-up rotation, Euler-angle poles).  Each
vector's conditioning is measured on the oracle itself: chi^2 before and after moving every
parameter by one ulp.  Vectors whose chi^2 moves by more than COND_LIMIT are ill-conditioned
(a few percent) and are left out; all others must agree to RTOL_FP64.  The 1e-12 bar is against the reference's
own kernel (tests/test_ref_kernel.py), which shares the compiler and libm.
"""
import numpy as np
import pytest

from asteroid_gb300 import api, capi

pytestmark = pytest.mark.gpu

RTOL_FP64 = 1e-9
COND_LIMIT = 1e-10


def well_conditioned(oracle_mod, model, obs, P, return_cond=False):
    """Mask of vectors whose oracle chi^2 (in FP64, CHI_FLOAT = double) moves by at most
    COND_LIMIT when every parameter is moved by one ulp, for three random sign patterns
    (and, with return_cond, that largest relative move per vector)."""
    acc_model = model
    if not model.flags & api.ACC:
        acc_model = api.make_model(model.flags | api.ACC, model.time_step, (2.0, 4800.0))
        acc_model.ppsi1, acc_model.ppsi2 = model.ppsi1, model.ppsi2
    a, _ = oracle_mod.chi2_batch(acc_model, obs, P)
    rng = np.random.default_rng(0)
    worst = np.zeros(len(P))
    for _ in range(3):
        Q = P * (1 + rng.choice([-1.0, 1.0], size=P.shape) * 2.3e-16)
        b, _ = oracle_mod.chi2_batch(acc_model, obs, Q)
        with np.errstate(invalid="ignore", divide="ignore"):
            worst = np.maximum(worst, np.abs(a - b) / np.abs(a))
    mask = np.isfinite(a) & np.isfinite(worst) & (worst <= COND_LIMIT)
    return (mask, worst) if return_cond else mask


def _vectors(model, n, seed, reopt=0, resolved=True):
    rng = np.random.default_rng(seed)
    names = api.param_names(model)
    iL = names.index("L")
    out = []
    while len(out) < n:
        x = rng.uniform(0, 1, model.n_params)
        p = api.x2params(model, x, reopt=reopt)
        if p is None:
            continue
        if resolved and not p[iL] * model.time_step <= 0.5:
            continue
        out.append(p)
    return np.array(out)


@pytest.mark.parametrize("name", ["c0acc", "c1", "c1bc", "c2"])
def test_fp64_matches_oracle(gpu, oracle_mod, synth_objects, name):
    s = synth_objects(name)
    P = _vectors(s.model, 200, seed=3)
    P = np.vstack([P, s.params_true[None, :]])
    with api.Engine(s.model, s.obs) as eng:
        chi2, dv = eng.eval(P)
    ref, ref_dv = oracle_mod.chi2_batch(s.model, s.obs, P)
    good = well_conditioned(oracle_mod, s.model, s.obs, P)
    assert good.sum() >= 0.5 * len(P), f"only {good.sum()} well-conditioned vectors"
    assert good[-1], "the true model must be well conditioned"
    assert np.all(np.isfinite(chi2[good]))
    fin = good
    acc = bool(s.model.flags & api.ACC)
    rtol = RTOL_FP64 if acc else 2e-6  # without ACC chi2 is rounded to float (CHI_FLOAT)
    if s.model.flags & api.NUDGE:
        rtol = max(rtol, 5e-6)  # the NUDGE merit is float arithmetic with powf
    rel = np.abs(chi2[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-300)
    assert rel.max() <= rtol, f"max rel chi2 diff {rel.max():.3e}"
    dvrel = np.abs(dv[fin] - ref_dv[fin]) / np.maximum(np.abs(ref_dv[fin]), 1e-12)
    assert dvrel.max() <= max(rtol, 1e-9)


def test_true_model_chi2_near_one(gpu, synth_objects):
    """The generating model fits its own noisy data: reduced chi^2 ~ 1 (sigma = 0.1)."""
    s = synth_objects("c0acc")
    with api.Engine(s.model, s.obs) as eng:
        chi2, dv = eng.eval(s.params_true[None, :])
    assert 0.7 < chi2[0] < 1.4
    assert abs(dv[0, 0] - s.dv_true[0]) < 0.05


def test_model_curve_matches_oracle(gpu, oracle_mod, synth_objects):
    s = synth_objects("c1")
    with api.Engine(s.model, s.obs) as eng:
        v = eng.model_curve(s.params_true)
    ref = oracle_mod.model_curve(s.model, s.obs, s.params_true)
    assert np.max(np.abs(v - ref)) < 1e-9


def test_unresolved_vectors_agree_on_finiteness(gpu, oracle_mod, synth_objects):
    s = synth_objects("c0acc")
    P = _vectors(s.model, 100, seed=9, reopt=1, resolved=False)
    with api.Engine(s.model, s.obs) as eng:
        chi2, _ = eng.eval(P)
    ref, _ = oracle_mod.chi2_batch(s.model, s.obs, P)
    # Vectors whose RK4 diverges to NaN on one side diverge on the other too, almost always.
    agree = np.mean(np.isnan(chi2) == np.isnan(ref))
    assert agree > 0.9


def test_eval_rejects_bad_precision(gpu, synth_objects):
    s = synth_objects("c0acc")
    with api.Engine(s.model, s.obs) as eng:
        with pytest.raises(Exception):
            eng.eval(s.params_true[None, :], precision=7)


def test_empty_batch(gpu, synth_objects):
    s = synth_objects("c0acc")
    with api.Engine(s.model, s.obs) as eng:
        chi2, dv = eng.eval(np.zeros((0, s.model.n_params)))
    assert chi2.shape == (0,)


@pytest.mark.parametrize("name", ["c0acc", "c1"])
def test_model_curve_at_grid_matches_oracle(gpu, oracle_mod, synth_objects, name):
    """-plot model curve (chi2one with Nplot > 0, cuda.c:1949-1950): at the data times it is the
    data's model curve bit for bit; on the fine plot grid it is the oracle's curve there (under
    INTERP both interpolate E and S from the ephemeris)."""
    s = synth_objects(name)
    interp = bool(s.model.flags & api.INTERP)
    t, e, u = api.plot_grid(s.dir / "lc.dat", s.dir, 3 * s.obs.n_data, interp=interp)
    with api.Engine(s.model, s.obs) as eng:
        at_data = eng.model_curve_at(s.params_true, s.obs.mjd, s.obs.e_unit, s.obs.s_unit)
        assert np.array_equal(at_data, eng.model_curve(s.params_true))
        fine = eng.model_curve_at(s.params_true, t, e, u)
        with pytest.raises(capi.AstError, match="increase"):
            eng.model_curve_at(s.params_true, t[::-1], e, u)
    grid = api.Obs(mjd=t, v=np.zeros(t.size), w=np.ones(t.size), filt=np.zeros(t.size), e_unit=e, s_unit=u,
                   eph_e=s.obs.eph_e, eph_s=s.obs.eph_s, eph_mjd0=s.obs.eph_mjd0, hmjd0=s.obs.hmjd0)
    ref = oracle_mod.model_curve(s.model, grid, s.params_true)
    assert np.max(np.abs(fine - ref)) < 1e-9
