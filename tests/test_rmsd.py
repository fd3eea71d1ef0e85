"""RMSD confidence intervals (chi2_gpu_rms, cuda.c:2148-2389; host loop asteroid.c:690-725).

The RMSD figure itself is pinned to the reference's -DRMSD builds by the golden vectors
(tests/golden/ref_rmsd_*.json, test_oracle_pin.py).  Here: the sampler and bookkeeping of the
oracle (CPU), and the CUDA path against the oracle on the points the device drew (GPU): the same
points, RMSDs within the FP64 tolerance, the same good/bad split and the same ranges."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import api, build, capi
from tests.test_gpu_eval import well_conditioned


def rmsd_model(s, extra=0):
    return api.make_model(s.model.flags | capi.RMSD | extra, s.model.time_step, ppsi_hours=s.cfg.ppsi_hours)


def test_oracle_normals_are_standard(built, oracle_mod):
    import ctypes as C
    lib = oracle_mod.load()
    lib.orc_normal4.restype = None
    z = np.zeros(4, np.float32)
    out = []
    for k in range(20000):
        lib.orc_normal4(C.c_uint64(7), C.c_uint64(3), C.c_uint32(0x80000000), C.c_uint32(k), z.ctypes.data_as(C.c_void_p))
        out.extend(z.tolist())
    out = np.array(out)
    assert abs(out.mean()) < 0.01 and abs(out.std() - 1) < 0.01
    assert abs(np.mean(np.abs(out) < 1.0) - 0.6827) < 0.01


def test_oracle_zero_shift_keeps_the_model(built, oracle_mod, synth_objects):
    """dx = 0: every draw is x0, every model is good, the ranges collapse onto the round trip
    x2params(params2x(m)) of the -m model."""
    s = synth_objects("c0acc")
    m = rmsd_model(s)
    r = oracle_mod.rmsd(m, s.obs, s.params_true, seed=1, call=0, n_streams=3, samples=2, dx=0.0, reopt=1)
    p = oracle_mod.x2params(m, oracle_mod.params2x(m, s.params_true), reopt=1)
    assert r["n_tot"] == 6 and r["n_bad"] == 0 and r["f1"] > r["f0"] > 0
    assert np.allclose(r["par_min"], p, rtol=1e-12, atol=1e-12) and np.allclose(r["par_max"], p, rtol=1e-12, atol=1e-12)


def test_oracle_counts_and_angle_rule(built, oracle_mod, synth_objects):
    s = synth_objects("c0acc")
    m = rmsd_model(s)
    r = oracle_mod.rmsd(m, s.obs, s.params_true, seed=5, call=0, n_streams=8, samples=4, dx=1e-4, reopt=1,
                        trace=True)
    ok = ~np.isnan(r["trace_f"])
    assert r["n_tot"] == ok.sum() and r["n_bad"] == np.sum(~(r["trace_f"][ok] < r["f1"]))
    assert 0 < r["n_bad"] < r["n_tot"]
    names = api.param_names(m)
    for nm in ("phi_M", "phi_0"):   # the reference's replacement keeps them within pi of the -m model
        i = names.index(nm)
        assert r["par_max"][i] <= s.params_true[i] + np.pi + 1e-9 or r["par_max"][i] == s.params_true[i] + 2 * np.pi


@pytest.mark.gpu
@pytest.mark.parametrize("name,dx,spherical,extra", [("c0acc", 1e-4, False, 0), ("c0acc", 3e-5, True, 0),
                                                     ("c1", 1e-3, False, capi.ACC), ("c1", 1e-3, False, 0)])
def test_gpu_rmsd_matches_oracle(gpu, oracle_mod, synth_objects, name, dx, spherical, extra):
    """With CHI_FLOAT = float (c1 without ACC) x2params rounds parameters to float, where the
    device's contracted multiply-adds and the oracle's separate roundings can differ by an ulp;
    the RMSD comparison is then made only with CHI_FLOAT = double, the split and ranges always."""
    s = synth_objects(name)
    m = rmsd_model(s, extra)
    streams, samples = 512, 3
    with api.Engine(m, s.obs) as eng:
        g = eng.rmsd(s.params_true, dx, n_streams=streams, samples=samples, seed=11, call=2, spherical_k=spherical,
                     trace=True)
    own = oracle_mod.rmsd(m, s.obs, s.params_true, seed=11, call=2, n_streams=streams, samples=samples, dx=dx,
                          reopt=1, spherical=spherical, trace=True)
    acc = bool(m.flags & capi.ACC)
    # The same draws up to the float Box-Muller (device and host logf / sin / cos), and under
    # float CHI_FLOAT one rounding of x.
    assert np.max(np.abs(g["trace_x"] - own["trace_x"])) < 1e-5 * dx + (0 if acc else 2e-7)
    # The device's own points through the oracle: same RMSDs, split and ranges.
    o = oracle_mod.rmsd(m, s.obs, s.params_true, seed=11, call=2, n_streams=streams, samples=samples, dx=dx,
                        reopt=1, spherical=spherical, x_in=g["trace_x"], trace=True)
    tol = 1e-9 if acc else 2.5e-7   # the FP64 tolerance against the oracle (its libm is glibc); one float ulp where CHI_FLOAT is float
    assert abs(g["f0"] - o["f0"]) <= tol * o["f0"] and abs(g["f1"] - o["f1"]) <= tol * o["f1"]
    gf, of = g["trace_f"], o["trace_f"]
    assert np.array_equal(np.isnan(gf), np.isnan(of))
    ok = ~np.isnan(of)
    assert g["n_tot"] == o["n_tot"] == ok.sum()
    if acc:
        # RMSDs agree on every well-conditioned model (the oracle's own figure moves by <= 1e-10
        # under one-ulp parameter changes); chaotic ones are left out as in the chi^2 parity tests.
        P = np.array([oracle_mod.x2params(m, x, reopt=1) for x in g["trace_x"][ok]])
        cond = well_conditioned(oracle_mod, m, s.obs, P)
        assert cond.sum() >= 0.5 * ok.sum(), f"{cond.sum()} of {ok.sum()} well conditioned"
        rel = np.abs(gf[ok] - of[ok]) / np.abs(of[ok])
        assert np.max(rel[cond]) < tol, np.max(rel[cond])
    # The bookkeeping on the device's own RMSDs: counts exact, ranges equal after the float rounding.
    b = oracle_mod.rmsd(m, s.obs, s.params_true, seed=11, call=2, n_streams=streams, samples=samples, dx=dx,
                        reopt=1, spherical=spherical, x_in=g["trace_x"], f_in=gf)
    assert g["n_tot"] == b["n_tot"] and g["n_bad"] == b["n_bad"]
    # (with CHI_FLOAT = float, x2params itself rounds to float on both sides: a few ulps apart)
    rr = 2.5e-7 if acc else 2e-6
    assert np.allclose(g["par_min"], b["par_min"].astype(np.float32), rtol=rr, atol=0)
    assert np.allclose(g["par_max"], b["par_max"].astype(np.float32), rtol=rr, atol=0)
    assert 0 < g["n_bad"] < g["n_tot"]


@pytest.mark.gpu
def test_gpu_rmsd_mixed_close_to_fp64(gpu, synth_objects):
    s = synth_objects("c0acc")
    m = rmsd_model(s)
    with api.Engine(m, s.obs) as eng:
        a = eng.rmsd(s.params_true, 1e-4, n_streams=1024, samples=2, seed=3, trace=True)
        b = eng.rmsd(s.params_true, 1e-4, n_streams=1024, samples=2, seed=3, precision=api.PREC_MIXED, trace=True)
    assert np.array_equal(a["trace_x"], b["trace_x"])
    ok = ~np.isnan(a["trace_f"])
    rel = np.abs(a["trace_f"][ok] - b["trace_f"][ok]) / a["trace_f"][ok]
    # the mixed path's own accuracy (chaotic models, a few percent, amplify its rounding)
    assert np.median(rel) < 1e-6 and np.mean(rel < 1e-5) >= 0.9
    assert a["n_tot"] == b["n_tot"]
    assert abs(a["n_bad"] - b["n_bad"]) <= 0.02 * a["n_tot"]


@pytest.mark.gpu
def test_gpu_rmsd_independent_of_geometry_and_refuses(gpu, synth_objects):
    """A stream's draws depend on (seed, call, stream, draw) only; refused inputs fail cleanly."""
    s = synth_objects("c0acc")
    m = rmsd_model(s)
    with api.Engine(m, s.obs) as eng:
        a = eng.rmsd(s.params_true, 1e-4, n_streams=300, samples=2, seed=9, trace=True)
        b = eng.rmsd(s.params_true, 1e-4, n_streams=600, samples=2, seed=9, trace=True)
        assert np.array_equal(a["trace_x"], b["trace_x"][:600])
        assert np.array_equal(a["trace_f"], b["trace_f"][:600], equal_nan=True)
        c = eng.rmsd(s.params_true, 1e-4, n_streams=300, samples=2, seed=9, call=1, trace=True)
        assert not np.array_equal(a["trace_x"], c["trace_x"])
        with pytest.raises(capi.AstError, match="positive"):
            eng.rmsd(s.params_true, 1e-4, n_streams=0)
    with api.Engine(s.model, s.obs) as eng:
        with pytest.raises(capi.AstError, match="RMSD"):
            eng.rmsd(s.params_true, 1e-4, n_streams=10)


@pytest.mark.gpu
def test_cli_rmsd_run(gpu, synth_objects, tmp_path):
    """asteroid.c:690-725: 'f0=..., f1=...', then per loop the bad fraction and the cumulative
    '%13.6e %13.6e ; ' ranges (stdout) and the ranges alone (output file)."""
    s = synth_objects("c0acc")
    m = [f"{v:.12f}" for v in s.params_true]
    cli = Path(build.BUILD) / "asteroid"
    r = subprocess.run([str(cli), "-variant", "TORQUE,P_PSI,ACC,RMSD", "-Nblocks", "2", "-bsize", "64", "-Nstages", "2",
                        "-N", "3", "-seed", "4", "-dx", "1e-4", "-reopt", "-i", str(s.dir / "lc.dat"), "-eph",
                        str(s.dir), "-o", str(tmp_path / "ci.dat"), "-Ppsi", "2", "4800", "-m", *m],
                       cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    lines = r.stdout.splitlines()
    assert any(l.startswith("f0=") and ", f1=" in l for l in lines)
    rows = [l for l in lines if l.count(";") == 11]
    assert len(rows) == 3
    frac = float(rows[-1].split()[0])
    assert 0 <= frac < 1
    file_rows = (tmp_path / "ci.dat").read_text().splitlines()
    assert len(file_rows) == 3
    groups = [g.split() for g in file_rows[-1].split(";") if g.strip()]
    assert len(groups) == 11
    lo = np.array([float(a) for a, b in groups])
    hi = np.array([float(b) for a, b in groups])
    assert np.all(lo <= hi)
    # cumulative: every loop's ranges contain the previous loop's
    prev = [[float(x) for x in g.split()] for g in file_rows[0].split(";") if g.strip()]
    assert all(lo[i] <= prev[i][0] and hi[i] >= prev[i][1] for i in range(11))
