"""Pin of the engine's C reader against the reference's own host readers.

oracle/build_ref.sh compiles the reference's read_data.c and misc.c from its sources as host code
(oracle/_ref/libref_read_<variant>.so, harness oracle/ref_harness_read_data.cu: cudaMallocHost as
malloc, cudaMemcpyToSymbol into the symbol's host copy).  On a light curve with all four filter
kinds (W: no correction; D: magnitude correction only; R, V: magnitude and light-time
corrections), a twelve-point HORIZONS ephemeris (the reader's three-point window slides along it)
and an observed.min with minima inside and outside the data, the engine's reader
(host/read_data.c through ast_read_data, ast_read_minima and ast_plot_grid) must give the same
numbers bit for bit as read_data() (read_data.c:6-377) and prepare_chi2_params() (misc.c:279-323):
times, magnitudes, weights, filters, hMJD0, the ephemeris window, the unit E and S vectors, the
-plot grid and the observed minima, without INTERP, with INTERP and with INTERP + NUDGE.
"""
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import api, synth
from tests.test_oracle_pin import EXACT

REF_DIR = Path(__file__).resolve().parents[1] / "oracle" / "_ref"
NPLOT = 500


def _files(d: Path, n=150, seed=4, n_eph=12):
    rng = np.random.default_rng(seed)
    mjd0 = 58050.0 + np.arange(n_eph, dtype=float)
    ast, earth, sun = synth._positions(mjd0, mjd0[n_eph // 2])
    jd = mjd0 + 2400000.5
    synth._write_eph(d / "asteroid.eph", "asteroid", jd, ast)
    synth._write_eph(d / "earth.eph", "earth", jd, earth)
    synth._write_eph(d / "sun.eph", "sun", jd, sun)
    t = np.sort(rng.uniform(mjd0[0] + 0.3, mjd0[-1] - 0.3, n))
    chars = [("W", "R", "D", "V")[i] for i in rng.integers(0, 4, n)]
    synth._write_lc(d / "lc.dat", chars, t, rng.uniform(20, 22, n), rng.uniform(0.05, 0.2, n))
    mins = np.concatenate([[mjd0[0] - 2.0], np.sort(rng.uniform(t[0], t[-1], 4)), [mjd0[-1] + 3.0]])
    (d / "observed.min").write_text("".join(f"{m:.6f} {rng.uniform(20, 22):.4f}\n" for m in mins))


@pytest.mark.parametrize("variant,interp,nudge", [("plain", False, False), ("interp", True, False),
                                                  ("interp_nudge", True, True)])
def test_reader_matches_reference_read_data(built, oracle_mod, tmp_path, variant, interp, nudge):
    if not (REF_DIR / f"libref_read_{variant}.so").exists() or not EXACT:
        pytest.skip("reference reader build not present (it is built where the reference checkout exists)")
    _files(tmp_path)
    ref = oracle_mod.RefRead(variant)
    r = ref.read(tmp_path, "lc.dat", nplot=NPLOT)
    o = api.read_data(tmp_path / "lc.dat", tmp_path, interp=interp,
                      minima_path=(tmp_path / "observed.min") if nudge else None)
    t, e, s = api.plot_grid(tmp_path / "lc.dat", tmp_path, n_plot=NPLOT, interp=interp)
    assert r["filters"] == o.filters == "VRWD"
    for key in ("mjd", "v", "w", "filt"):
        assert np.array_equal(r[key], getattr(o, key)), key
    assert r["hmjd0"] == o.hmjd0
    assert np.array_equal(r["eph_e"], o.eph_e) and np.array_equal(r["eph_s"], o.eph_s)
    assert np.array_equal(r["plot_t"], t)
    if interp:
        assert np.array_equal(r["eph_mjd0"], o.eph_mjd0)
    else:
        # Without INTERP the reference moves its ephemeris times to hMJD0 only inside its plot
        # block (read_data.c:316-319), where nothing reads them; with Nplot = 0 they are the
        # reader's.
        assert np.array_equal(ref.read(tmp_path, "lc.dat", nplot=0)["eph_mjd0"], o.eph_mjd0)
        assert np.array_equal(r["e_unit"], o.e_unit.ravel()) and np.array_equal(r["s_unit"], o.s_unit.ravel())
        assert np.array_equal(r["plot_e"], e) and np.array_equal(r["plot_s"], s)
    if nudge:
        assert len(r["t_min"]) == 4
        assert np.array_equal(r["t_min"], o.t_min) and np.array_equal(r["v_min"], o.v_min)
