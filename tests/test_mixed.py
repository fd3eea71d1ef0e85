"""Mixed-precision path (double-float RK4 on the FP32 pipe, FP32 brightness) against FP64.

The accuracy target of the mixed path is |dchi2|/chi2 <= 1e-6 against the FP64 result.  It is asserted
on well-conditioned vectors (tests/test_gpu_eval.py::well_conditioned), where the FP64 result
itself is stable to rounding; the ill-conditioned few percent, where any change of rounding
moves chi^2, are reported but not held to it.  Under NUDGE the count of model minima is a
discontinuous function of the model magnitudes, so a near-tie decided differently in FP32
changes the merit factor; such flips are counted and must stay rare.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import api, build
from tests.test_gpu_eval import _vectors, well_conditioned

pytestmark = pytest.mark.gpu

BAR = 1e-6


@pytest.mark.parametrize("name", ["c0acc", "c1", "c1bc", "c2"])
def test_mixed_within_1e6_of_fp64(gpu, oracle_mod, synth_objects, name):
    s = synth_objects(name)
    P = np.vstack([_vectors(s.model, 300, seed=13), s.params_true[None, :]])
    good = well_conditioned(oracle_mod, s.model, s.obs, P)
    with api.Engine(s.model, s.obs) as eng:
        c64, d64 = eng.eval(P, api.PREC_FP64)
        c32, d32 = eng.eval(P, api.PREC_MIXED)
    ok = good & np.isfinite(c64) & (c64 < 1e29)
    both = ok & (c32 < 1e29)
    flips = np.sum(ok & (c32 >= 1e29))
    rel = np.abs(c32[both] - c64[both]) / np.abs(c64[both])
    acc = bool(s.model.flags & api.ACC)
    bar = BAR if acc else 2e-6  # CHI_FLOAT = float rounds both results to 6e-8
    frac = np.mean(rel <= bar)
    print(f"{name}: {both.sum()} vectors, median {np.median(rel):.2e}, p99 {np.quantile(rel, 0.99):.2e}, "
          f"max {rel.max():.2e}, <= {bar}: {frac:.4f}, NUDGE flips {flips}")
    assert rel[-1] <= bar, f"true model: {rel[-1]:.3e}"
    assert frac >= 0.99, f"only {frac:.4f} within {bar}"
    assert flips <= 0.01 * ok.sum()
    assert np.median(rel) <= 2e-7


def test_mixed_fit_finds_same_minimum(gpu, synth_objects):
    """Re-optimisation from the truth lands on the same chi^2 in both precisions."""
    s = synth_objects("c0acc")
    with api.Engine(s.model, s.obs) as eng:
        a = eng.fit(n_chains=256, group_size=256, seed=3, reopt=True, params0=s.params_true, evals_cap=300)
        b = eng.fit(n_chains=256, group_size=256, seed=3, reopt=True, params0=s.params_true, evals_cap=300,
                    precision=api.PREC_MIXED)
        f64, _ = eng.eval(b.best_params, api.PREC_FP64)
    assert abs(a.best_f[0] - b.best_f[0]) / a.best_f[0] < 1e-3
    # The mixed fit's reported chi^2 is what FP64 gives at its parameters, within the bar.
    assert abs(f64[0] - b.best_f[0]) / f64[0] <= BAR


def test_packed_step_equals_scalar_step(gpu, tmp_path):
    """The RK4 step on packed FP32x2 pairs gives the scalar double-float step's bits.

    tests/host/packed_step_check.cu restates the step lane by lane with scalar operations and
    compares sin/cos, both right-hand sides and both steps on 1M random states per configuration
    (angles up to 2^20 rad, rates up to 2^17 rad/day), on the GPU.  A packed product that the
    compiler fused into the next packed add, or a lane mix-up, shows up as mismatches."""
    exe = tmp_path / "packed_step_check"
    src = Path(__file__).resolve().parent / "host" / "packed_step_check.cu"
    subprocess.run([build._nvcc(), *build.GENCODE, "-O3", "-std=c++17", f"-I{build.PKG / 'csrc'}",
                    f"-I{build.INCLUDE}", f"-I{build.PKG / 'host'}", str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe), str(1 << 20)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
