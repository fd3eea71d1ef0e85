"""The asteroid command-line drop-in: switches, output files and lines (asteroid.c:655-825)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from asteroid_gb300 import build

pytestmark = pytest.mark.gpu

CLI = Path(build.BUILD) / "asteroid"


def run(args, cwd):
    r = subprocess.run([str(CLI), *args], cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    return r.returncode, r.stdout


@pytest.fixture(scope="module")
def data(synth_objects):
    return synth_objects("c0acc")


def parse(path, n_filters, n_params):
    rows = [l.split() for l in Path(path).read_text().splitlines() if l.strip()]
    for r in rows:
        assert len(r) == 1 + n_filters + n_params
    return np.array(rows, dtype=float)


def test_random_search_writes_all_blocks(gpu, data, tmp_path):
    d = data.dir
    rc, out = run(["-variant", "TORQUE,P_PSI,ACC", "-Nblocks", "4", "-bsize", "64", "-evals", "40", "-seed", "5",
                   "-N", "2", "-i", str(d / "lc.dat"), "-eph", str(d), "-o", str(tmp_path / "out.dat"),
                   "-Ppsi", "2", "4800"], tmp_path)
    assert rc == 0, out
    assert "Simplex optimization" in out and "N_threads = 256" in out
    rows = parse(tmp_path / "out.dat", 1, 11)
    assert rows.shape[0] == 4  # without -keep the file holds the current best of every block
    best_lines = [l for l in out.splitlines() if l.strip() and l.strip()[0].isdigit() and "e" in l.split()[0]]
    assert len(best_lines) == 2  # one stdout line per loop (-N 2)
    # the last stdout line is the best block of the file
    assert abs(float(best_lines[-1].split()[0]) - rows[:, 0].min()) <= 1e-6 * rows[:, 0].min()


def test_keep_appends_and_best_writes_one_line(gpu, data, tmp_path):
    d = data.dir
    args = ["-variant", "TORQUE,P_PSI,ACC", "-Nblocks", "2", "-bsize", "32", "-evals", "30", "-seed", "9", "-N", "3",
            "-i", str(d / "lc.dat"), "-eph", str(d), "-Ppsi", "2", "4800"]
    rc, out = run(args + ["-keep", "-o", str(tmp_path / "keep.dat")], tmp_path)
    assert rc == 0, out
    assert parse(tmp_path / "keep.dat", 1, 11).shape[0] == 6
    rc, out = run(args + ["-best", "-o", str(tmp_path / "best.dat")], tmp_path)
    assert rc == 0, out
    assert parse(tmp_path / "best.dat", 1, 11).shape[0] == 1


def test_reopt_from_true_model(gpu, data, tmp_path):
    d = data.dir
    m = [f"{v:.12f}" for v in data.params_true]
    rc, out = run(["-variant", "TORQUE,P_PSI,ACC", "-Nblocks", "1", "-bsize", "64", "-evals", "100", "-seed", "3",
                   "-N", "1", "-reopt", "-best", "-i", str(d / "lc.dat"), "-eph", str(d), "-o",
                   str(tmp_path / "re.dat"), "-Ppsi", "2", "4800", "-m", *m], tmp_path)
    assert rc == 0, out
    row = parse(tmp_path / "re.dat", 1, 11)[0]
    assert row[0] < 1.2


def test_bad_arguments(gpu, data, tmp_path):
    rc, out = run(["-o", "x"], tmp_path)
    assert rc == 1 and "-i parameter is missing" in out
    rc, out = run(["-i", str(data.dir / "lc.dat"), "-reopt", "-o", "x"], tmp_path)
    assert rc == 1 and "require -m" in out
    rc, out = run(["-i", str(data.dir / "lc.dat"), "-plot"], tmp_path)
    assert rc == 1 and "require -m" in out


def test_plot_mode_files(gpu, data, tmp_path):
    """-plot (asteroid.c:834-1060): delta_V, model_params.dat without the torque parameters,
    model.dat on the Nplot grid shifted by delta_V[0], data.dat converted to the first filter."""
    from asteroid_gb300 import api

    d = data.dir
    m = [f"{v:.12f}" for v in data.params_true]
    rc, out = run(["-variant", "TORQUE,P_PSI,ACC", "-plot", "-Nplot", "500", "-i", str(d / "lc.dat"), "-eph", str(d),
                   "-Ppsi", "2", "4800", "-m", *m], tmp_path)
    assert rc == 0, out
    assert "*** Plotting ***" in out
    line = [l for l in out.splitlines() if l.startswith("chi2_plot = ")]
    assert len(line) == 1
    with api.Engine(data.model, data.obs) as eng:
        chi2, dv = eng.eval(np.asarray(data.params_true)[None, :])
        t, e, s = api.plot_grid(d / "lc.dat", d, 500)
        vm = eng.model_curve_at(data.params_true, t, e, s)
    assert float(line[0].split()[2].rstrip(",")) == float("%13.6e" % chi2[0])
    # the periodogram line (asteroid.c:974-980): cl_fr then cl_H, "%f " each, of the curve + delta_V[0]
    pg = api.minima(t, vm + dv[0, 0])
    expect = "".join("%f " % x for x in list(pg.cl_fr) + list(pg.cl_H))
    assert expect.strip() in [l.strip() for l in out.splitlines()]
    assert float((tmp_path / "delta_V").read_text().split()[0]) == float("%8.4f" % dv[0, 0])
    mp = (tmp_path / "model_params.dat").read_text().split()
    ids = data.model.ids
    keep = [j for j in range(data.model.n_params) if data.model.property[j][0] not in (ids.Ti, ids.Ts, ids.Tl)]
    assert len(mp) == len(keep) == data.model.n_params - 3
    assert np.allclose([float(x) for x in mp], np.asarray(data.params_true)[keep], rtol=0, atol=1e-10)
    model = np.loadtxt(tmp_path / "model.dat")
    assert model.shape == (500, 2)
    assert np.allclose(model[:, 0], data.obs.hmjd0 + t, rtol=0, atol=1e-7)
    assert np.allclose(model[:, 1], vm + dv[0, 0], rtol=1e-6, atol=0)
    rows = [l.split() for l in (tmp_path / "data.dat").read_text().splitlines()]
    assert len(rows) == data.obs.n_data and all(r[3] == "w" for r in rows)
    dd = np.array([[float(x) for x in r[:3]] for r in rows])
    assert np.allclose(dd[:, 1], data.obs.v - dv[0, data.obs.filt] + dv[0, 0], rtol=1e-6, atol=0)
    assert np.allclose(dd[:, 2], 1 / np.sqrt(data.obs.w), rtol=1e-6, atol=0)
