"""Host side (C): variant tables, file readers and conversions, output format.  No GPU."""
import math
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import api, capi, synth

# Property order and __COUNTER__ type numbering of the reference (asteroid.c:86-125,
# asteroid.h:137-178), for the variants of the benchmark set.
EXPECTED_ORDER = {
    "TORQUE,P_PSI": ["theta_M", "phi_M", "phi_0", "Ti", "Ts", "Tl", "c_tumb", "b_tumb", "Es", "L", "psi_0"],
    "BC": ["theta_M", "phi_M", "phi_0", "c_tumb", "b_tumb", "Es", "L", "psi_0", "c", "b"],
    "BW_BALL,TORQUE": ["theta_M", "phi_M", "phi_0", "Ti", "Ts", "Tl", "c_tumb", "b_tumb", "Es", "L", "psi_0",
                       "theta_R", "phi_R", "kappa"],
    "": ["theta_M", "phi_M", "phi_0", "c_tumb", "b_tumb", "Es", "L", "psi_0"],
}


@pytest.mark.parametrize("flags,names", list(EXPECTED_ORDER.items()))
def test_property_order(built, flags, names):
    m = api.make_model(flags or 0)
    assert api.param_names(m) == names
    assert m.n_params == len(names)


def test_type_ids_follow_counter_order(built):
    m = api.make_model("TORQUE,BC,BW_BALL")
    t = m.ids
    assert (t.theta_M, t.phi_M, t.phi_0, t.L, t.Ti, t.Ts, t.Tl, t.c_tumb, t.b_tumb, t.Es, t.psi_0, t.c, t.b,
            t.theta_R, t.phi_R, t.kappa, t.n_types) == tuple(range(16)) + (16,)
    m2 = api.make_model("P_PSI")
    assert (m2.ids.c_tumb, m2.ids.psi_0, m2.ids.n_types, m2.ids.Ti) == (4, 7, 8, -1)


def test_limits_float_rounding_and_ppsi(built):
    m = api.make_model("TORQUE,P_PSI", ppsi_hours=(2.0, 4800.0))
    lim = np.ctypeslib.as_array(m.limits)
    t = m.ids
    assert lim[0][t.c_tumb] == float(np.float32(math.log(0.01)))   # CHI_FLOAT = float
    assert lim[1][t.L] == float(np.float32(48 * math.pi / 0.1))
    assert m.ppsi1 == np.float32(24.0 / 4800.0) and m.ppsi2 == np.float32(24.0 / 2.0)
    ma = api.make_model("TORQUE,P_PSI,ACC")
    assert np.ctypeslib.as_array(ma.limits)[0][ma.ids.c_tumb] == math.log(0.01)


def test_freeze_limits_and_random_switches(built):
    lib = capi.load()
    import ctypes as C
    m = api.make_model("TORQUE,ACC")
    assert lib.ast_model_freeze(C.byref(m), m.ids.Ti, 0.5) == 0
    i = api.param_names(m).index("Ti")
    assert m.property[i][capi.AST_N_COLUMNS - 4] == 1  # P_frozen
    assert lib.ast_model_set_limits(C.byref(m), m.ids.L, 10.0, 20.0) == 0
    assert np.ctypeslib.as_array(m.limits)[1][m.ids.L] == 20.0
    assert lib.ast_model_set_free_random(C.byref(m), 0) == 0 and m.property[0][2] == -1
    assert lib.ast_model_freeze(C.byref(m), 99, 0.0) < 0


def write_lc(path, rows):
    Path(path).write_text("".join(f"{c} {t:.8f} {v:.5f} {s:.3f} x\n" for c, t, v, s in rows))


def eph_files(d, t0, t1):
    synth._write_eph(Path(d) / "asteroid.eph", "a", [t0 + 2400000.5, (t0 + t1) / 2 + 2400000.5, t1 + 2400000.5],
                     np.array([[1.0, 0.5, 0.0], [1.01, 0.51, 0.0], [1.02, 0.52, 0.0]]))
    synth._write_eph(Path(d) / "earth.eph", "e", [t0 + 2400000.5, (t0 + t1) / 2 + 2400000.5, t1 + 2400000.5],
                     np.array([[1.0, 0.0, 0.0], [1.0, 0.01, 0.0], [1.0, 0.02, 0.0]]))
    synth._write_eph(Path(d) / "sun.eph", "s", [t0 + 2400000.5, (t0 + t1) / 2 + 2400000.5, t1 + 2400000.5],
                     np.zeros((3, 3)))


def test_read_data_conversions(built, tmp_path):
    """W rows: no corrections; other filters: +5 log10(1/(E S)) and minus light time; D: no light time."""
    eph_files(tmp_path, 58000.0, 58002.0)
    rows = [("W", 58000.5, 20.0, 0.1), ("R", 58000.7, 21.0, 0.2), ("D", 58001.1, 22.0, 0.1), ("R", 58001.5, 21.5, 0.1)]
    write_lc(tmp_path / "lc", rows)
    o = api.read_data(tmp_path / "lc", tmp_path)
    assert o.filters == "WRD" and list(o.filt) == [0, 1, 2, 1]
    assert o.w[1] == np.float32(1 / 0.04)
    mjd0 = np.array([58000.0, 58001.0, 58002.0])
    a = np.array([[1.0, 0.5, 0.0], [1.01, 0.51, 0.0], [1.02, 0.52, 0.0]])
    e = np.array([[1.0, 0.0, 0.0], [1.0, 0.01, 0.0], [1.0, 0.02, 0.0]]) - a
    s = -a
    tt = np.array([r[1] for r in rows])
    E = synth._interp_vec(tt, mjd0, e)
    S = synth._interp_vec(tt, mjd0, s)
    En, Sn = np.linalg.norm(E, axis=1), np.linalg.norm(S, axis=1)
    assert o.v[0] == np.float32(20.0)
    assert abs(o.v[1] - (21.0 + 5 * math.log10(1 / En[1] / Sn[1]))) < 1e-5
    t_ast = tt - np.array([0, En[1], 0, En[3]]) / synth.LIGHT_SPEED
    assert np.allclose(o.mjd, t_ast - t_ast[0], rtol=0, atol=1e-12)
    assert np.allclose(o.e_unit.reshape(-1, 3), E / En[:, None], atol=1e-12)


def test_read_data_errors(built, tmp_path):
    eph_files(tmp_path, 58000.0, 58002.0)
    write_lc(tmp_path / "unsorted", [("W", 58001.0, 20, 0.1), ("W", 58000.9, 20, 0.1)])
    with pytest.raises(capi.AstError, match="sorted"):
        api.read_data(tmp_path / "unsorted", tmp_path)
    write_lc(tmp_path / "outside", [("W", 58000.5, 20, 0.1), ("W", 58003.0, 20, 0.1)])
    with pytest.raises(capi.AstError, match="bracket"):
        api.read_data(tmp_path / "outside", tmp_path)
    write_lc(tmp_path / "many", [(c, 58000.1 + 0.1 * k, 20, 0.1) for k, c in enumerate("ABC")])
    with pytest.raises(capi.AstError, match="filters"):
        api.read_data(tmp_path / "many", tmp_path, max_filters=2)
    with pytest.raises(capi.AstError, match="does not exist"):
        api.read_data(tmp_path / "missing", tmp_path)
    write_lc(tmp_path / "ok", [("W", 58000.5, 20, 0.1)])
    with pytest.raises(capi.AstError, match="ephemeris"):
        api.read_data(tmp_path / "ok", tmp_path / "nowhere")


def test_observed_minima_window(built, tmp_path):
    eph_files(tmp_path, 58000.0, 58002.0)
    write_lc(tmp_path / "lc", [("W", 58000.5, 20, 0.1), ("W", 58001.5, 20, 0.1)])
    (tmp_path / "observed.min").write_text("58000.46 25.0\n58000.40 24.0\n58001.54 25.5\n58001.6 26\n")
    o = api.read_data(tmp_path / "lc", tmp_path, minima_path=tmp_path / "observed.min")
    # kept: within [first - 0.05, last + 0.05] (misc.c:294), times as float minus hMJD0
    assert o.t_min.size == 2
    assert o.t_min[0] == np.float32(np.float32(58000.46) - 58000.5)
    (tmp_path / "none.min").write_text("57000 1\n")
    with pytest.raises(capi.AstError, match="No local minima"):
        api.read_data(tmp_path / "lc", tmp_path, minima_path=tmp_path / "none.min")


def test_format_result_line(built):
    line = api.format_result(1.5, [0.25, -0.5], [1.0, 2.5, -3.25])
    assert line == "%13.6e %13.6e %13.6e %15.11f %15.11f %15.11f \n" % (1.5, 0.25, -0.5, 1.0, 2.5, -3.25)


def test_quadratic_interpolation_exact_on_quadratics(built):
    import ctypes as C
    lib = capi.load()
    mjd0 = (C.c_double * 3)(0.0, 1.0, 3.0)
    f = lambda t: 2 * t * t - t + 0.5
    e = ((C.c_double * 3) * 3)()
    s = ((C.c_double * 3) * 3)()
    for k in range(3):
        for j, t in enumerate((0.0, 1.0, 3.0)):
            e[k][j] = f(t) * (k + 1)
            s[k][j] = -f(t)
    oe, os_ = (C.c_double * 3)(), (C.c_double * 3)()
    lib.ast_quadratic_interpolation(mjd0, C.cast(e, C.POINTER(C.c_double)), C.cast(s, C.POINTER(C.c_double)),
                                    1.7, oe, os_)
    assert abs(oe[1] - 2 * f(1.7)) < 1e-12 and abs(os_[0] + f(1.7)) < 1e-12


def test_synthetic_generator_files(built, oracle_mod, tmp_path):
    s = synth.generate("c0acc", tmp_path, vmod_fn=lambda m, o, p: oracle_mod.model_curve(m, o, p))
    lines = (tmp_path / "lc.dat").read_text().splitlines()
    assert len(lines) == 300 and all(l.startswith("W ") for l in lines)
    assert (tmp_path / "asteroid.eph").read_text().count("$$SOE") == 1
    assert s.obs.n_data == 300 and np.all(np.diff(s.obs.mjd) > 0)
    c, dv = oracle_mod.chi2(s.model, s.obs, s.params_true)
    assert 0.7 < c < 1.4


@pytest.mark.parametrize("interp", [False, True])
def test_plot_grid_follows_read_data(built, tmp_path, interp):
    """-plot grid (read_data.c:309-370): ends = first/last observation, interior evenly spaced
    with E, S interpolated in the last ephemeris window and normalised."""
    eph_files(tmp_path, 58000.0, 58002.0)
    rows = [("W", 58000.2, 20.0, 0.1), ("R", 58000.7, 21.0, 0.2), ("R", 58001.9, 21.5, 0.1)]
    write_lc(tmp_path / "lc", rows)
    o = api.read_data(tmp_path / "lc", tmp_path, interp=interp)
    n_plot = 9
    t, e, s = api.plot_grid(tmp_path / "lc", tmp_path, n_plot, interp=interp)
    assert t[0] == o.mjd[0] == 0.0 and t[-1] == o.mjd[-1]
    assert np.array_equal(e[0], o.e_unit[0]) and np.array_equal(s[-1], o.s_unit[-1])
    h = o.mjd[-1] / (n_plot - 1)
    assert np.array_equal(t[1:-1], np.arange(1, n_plot - 1) * h)
    mjd0 = np.array([58000.0, 58001.0, 58002.0])
    a = np.array([[1.0, 0.5, 0.0], [1.01, 0.51, 0.0], [1.02, 0.52, 0.0]])
    E = synth._interp_vec(t[1:-1] + o.hmjd0, mjd0, np.array([[1.0, 0.0, 0.0], [1.0, 0.01, 0.0], [1.0, 0.02, 0.0]]) - a)
    S = synth._interp_vec(t[1:-1] + o.hmjd0, mjd0, -a)
    assert np.allclose(e[1:-1], E / np.linalg.norm(E, axis=1)[:, None], rtol=0, atol=1e-10)
    assert np.allclose(s[1:-1], S / np.linalg.norm(S, axis=1)[:, None], rtol=0, atol=1e-10)
    assert np.allclose(np.linalg.norm(e, axis=1), 1.0, atol=1e-14)


def test_cli_usage_and_argument_errors_without_a_gpu(built, tmp_path):
    """The command line's own checks run before any device call (asteroid.c:173-445)."""
    import subprocess
    from asteroid_gb300 import build

    cli = str(Path(build.BUILD) / "asteroid")
    r = subprocess.run([cli], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=60)
    assert r.returncode == 0
    for sw in ("-best", "-i name", "-m param1", "-Nstages", "-Ppsi", "-plot", "-dx", "-i1", "-i2", "-animate"):
        assert sw in r.stdout, sw
    def run(*args):
        r = subprocess.run([cli, *args], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                           timeout=60)
        return r.returncode, r.stdout
    assert run("-o", "x") == (1, "-i parameter is missing!\n")
    rc, out = run("-i", "lc", "-plot")
    assert rc == 1 and "require -m" in out
    rc, out = run("-i", "lc", "-m", "1", "2")
    assert rc == 1 and "-m can only be used together with -reopt or -plot" in out
    rc, out = run("-i", "lc", "-bogus")
    assert rc == 1 and "Bad arguments" in out
    rc, out = run("-i", "lc", "-plot", "-Nplot", "1", "-m", "1")
    assert rc == 1 and "Bad arguments" in out
