"""Seeded synthetic light curves in the reference's file formats.

The reference ships no data (its 'Oumuamua light curve and HORIZONS files are not public in
its repository), so every workload here is synthetic, with the shapes of the benchmark
configurations:

  c0  LS + TORQUE + P_PSI, 1 filter 'W', 300 points in 5 nightly 6 h windows over 5 days,
      TIME_STEP 1e-2, sigma 0.1 mag
  c1  same generator, 480 points over 8 days, 2 filters with offsets U(-0.5, 0.5); INTERP
  c2  3 filters, 2000 points clustered in nightly windows over 60 days, TIME_STEP 5e-3,
      ACC + NUDGE + INTERP, 5 observed minima taken from the true model

Files written (formats of README.md:11-41 and read_data.c / misc.c):
  lc.dat          "filter MJD V sgm aux" per line
  asteroid.eph, earth.eph, sun.eph   HORIZONS VECTORS: "$$SOE", JD line, "X Y Z" line, ..., "$$EOE"
  observed.min    "MJD_min V_min" per line (NUDGE)
  truth.json      the true dimensionless point, physical parameters and offsets

The true model's magnitudes come from ``vmod_fn(model, obs, params)``; by default the CUDA
engine's model curve (``Engine.model_curve``).  Tests on a machine without a GPU pass the
oracle's model curve instead.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field, asdict
from pathlib import Path

import numpy as np

from . import api

LIGHT_SPEED = 173.144632674  # au/day (asteroid.h:287)


@dataclass
class SynthConfig:
    name: str
    flags: str
    time_step: float
    n_points: int
    n_filters: int
    span_days: int
    n_nights: int
    window_hours: float = 6.0
    sigma: float = 0.1
    seed: int = 1000
    n_minima: int = 0
    filter_chars: str = "W"
    dv_range: float = 0.0
    ppsi_hours: tuple = (2.0, 4800.0)
    base_mag: float = 22.0


CONFIGS = {
    "c0": SynthConfig("c0", "TORQUE,P_PSI", 1e-2, 300, 1, 5, 5, seed=1000, filter_chars="W"),
    "c0acc": SynthConfig("c0acc", "TORQUE,P_PSI,ACC", 1e-2, 300, 1, 5, 5, seed=1000, filter_chars="W"),
    "c1": SynthConfig("c1", "TORQUE,INTERP", 1e-2, 480, 2, 8, 8, seed=1001, filter_chars="RV", dv_range=0.5),
    "c1bc": SynthConfig("c1bc", "BC,INTERP", 1e-2, 480, 2, 8, 8, seed=1001, filter_chars="RV", dv_range=0.5),
    "c2": SynthConfig("c2", "TORQUE,P_PSI,INTERP,ACC,NUDGE", 5e-3, 2000, 3, 60, 20, seed=1002, n_minima=5,
                      filter_chars="RVB", dv_range=0.5, ppsi_hours=(20.0, 4800.0)),
}


@dataclass
class Synth:
    cfg: SynthConfig
    dir: Path
    model: object
    obs: "api.Obs"
    x_true: np.ndarray
    params_true: np.ndarray
    dv_true: np.ndarray
    files: dict = field(default_factory=dict)


def _times(rng, cfg: SynthConfig, t0: float) -> np.ndarray:
    """Uniform random times inside nightly windows, strictly increasing."""
    if cfg.n_nights >= cfg.span_days:
        nights = np.arange(cfg.n_nights, dtype=float)
    else:
        nights = np.sort(rng.choice(cfg.span_days, size=cfg.n_nights, replace=False)).astype(float)
    win = cfg.window_hours / 24.0
    while True:
        k = rng.integers(0, cfg.n_nights, size=cfg.n_points)
        t = np.sort(t0 + nights[k] + rng.uniform(0.0, win, size=cfg.n_points))
        if np.all(np.diff(t) > 1e-6):
            return t


def _positions(t, t_mid):
    """Sun at the origin; Earth and asteroid on linear tracks near 1 and 1.2 au."""
    dt = np.asarray(t) - t_mid
    earth = np.stack([1.0 + 0 * dt, 0.0172 * dt, 0 * dt], axis=-1)
    ang = np.deg2rad(30.0)
    ast = np.stack([1.2 * np.cos(ang) - 0.010 * dt, 1.2 * np.sin(ang) + 0.015 * dt, 0.05 + 0.002 * dt], axis=-1)
    sun = np.zeros_like(earth)
    return ast, earth, sun


def _write_eph(path: Path, name: str, jd, xyz):
    lines = [f"Synthetic ephemeris ({name}), HORIZONS VECTORS layout, type 1 (x,y,z), labels off",
             "Coordinate Origin: Solar System Barycenter (SSB)", "$$SOE"]
    for j, p in zip(jd, xyz):
        lines.append(f"{j:.9f} = A.D. synthetic TDB")
        lines.append(f" {p[0]: .15E} {p[1]: .15E} {p[2]: .15E}")
    lines.append("$$EOE")
    lines.append("End of synthetic ephemeris")
    path.write_text("\n".join(lines) + "\n")


def _interp_vec(t, mjd0, vals):
    """Second-order Lagrange interpolation (misc.c:20-35 formula)."""
    rr0 = (t - mjd0[1]) * (t - mjd0[2]) / (mjd0[0] - mjd0[1]) / (mjd0[0] - mjd0[2])
    rr1 = (t - mjd0[0]) * (t - mjd0[2]) / (mjd0[1] - mjd0[0]) / (mjd0[1] - mjd0[2])
    rr2 = (t - mjd0[0]) * (t - mjd0[1]) / (mjd0[2] - mjd0[0]) / (mjd0[2] - mjd0[1])
    return vals[0] * rr0[..., None] + vals[1] * rr1[..., None] + vals[2] * rr2[..., None]


def _model_minima(vmod) -> np.ndarray:
    """Indices of brightness minima (V maxima) over three consecutive points (cuda.c:725)."""
    i = np.arange(1, vmod.size - 1)
    return i[(vmod[i] > vmod[i - 1]) & (vmod[i] >= vmod[i + 1])]


def _write_lc(path: Path, chars, mjd_obs, v, sgm):
    with open(path, "w") as f:
        for c, t, vv, s in zip(chars, mjd_obs, v, sgm):
            f.write(f"{c} {t:.10f} {vv:.7f} {s:.4f} x\n")


def engine_vmod(model, obs, params):
    eng = api.Engine(model, obs)
    try:
        return eng.model_curve(params)
    finally:
        eng.close()


def generate(cfg: SynthConfig | str, outdir, vmod_fn=None) -> Synth:
    """Write one synthetic object under outdir and return it read back through the C reader."""
    if isinstance(cfg, str):
        cfg = CONFIGS[cfg]
    vmod_fn = vmod_fn or engine_vmod
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(cfg.seed)
    flags = api.flags_from_names(cfg.flags)
    model = api.make_model(flags, cfg.time_step, cfg.ppsi_hours)
    interp = bool(flags & api.INTERP)

    t0 = 58051.0
    t_ast = _times(rng, cfg, t0)
    fidx = rng.integers(0, cfg.n_filters, size=cfg.n_points).astype(np.int32)
    fidx[: cfg.n_filters] = np.arange(cfg.n_filters)  # every filter appears, first in order
    order_chars = [cfg.filter_chars[i] for i in range(cfg.n_filters)]
    chars = [order_chars[i] for i in fidx]

    # Three ephemeris points strictly bracketing the data (read_data.c:208).
    t_mid = 0.5 * (t_ast[0] + t_ast[-1])
    mjd0 = np.array([t_ast[0] - 1.0, t_mid, t_ast[-1] + 1.0])
    jd = mjd0 + 2400000.5
    ast_p, earth_p, sun_p = _positions(mjd0, t_mid)
    _write_eph(out / "asteroid.eph", "asteroid", jd, ast_p)
    _write_eph(out / "earth.eph", "earth", jd, earth_p)
    _write_eph(out / "sun.eph", "sun", jd, sun_p)
    e_pts = earth_p - ast_p
    s_pts = sun_p - ast_p

    # Observer times: 'W' data are already light-time corrected; others get MJD = t + E/c.
    mjd_obs = t_ast.copy()
    for _ in range(6):
        e = _interp_vec(mjd_obs, mjd0, e_pts)
        delay = np.linalg.norm(e, axis=-1) / LIGHT_SPEED
        corr_t = np.array([0.0 if c in "WD" else 1.0 for c in chars])
        mjd_obs = t_ast + corr_t * delay

    sgm = np.full(cfg.n_points, cfg.sigma)
    _write_lc(out / "lc.dat", chars, mjd_obs, np.zeros(cfg.n_points), sgm)
    obs0 = api.read_data(out / "lc.dat", out, interp=interp)
    geom = obs0.v.astype(np.float64)  # V=0 in the file: what the reader adds (0 for 'W')

    # True parameters: x ~ U(0,1) in the free coordinates mapped by x2params with the fit's
    # own meaning of x (under P_PSI, L from the Ppsi range), redrawn until the model is
    # resolved by the fixed-step RK4: a finite light curve and h * L <= 0.5.  (Uniform L up
    # to 48*pi/0.1 rad/day with h = 5e-3 d gives h*L ~ 7, where RK4 diverges to NaN.)
    obs_model = obs0
    if flags & api.NUDGE:
        obs_model = api.Obs(obs0.mjd, obs0.v, obs0.w, obs0.filt, obs0.e_unit, obs0.s_unit, obs0.eph_e, obs0.eph_s,
                            obs0.eph_mjd0, np.zeros(1, np.float32), np.zeros(1, np.float32), obs0.hmjd0, obs0.filters)
    reopt_truth = 0 if flags & api.P_PSI else 1
    i_L = api.param_names(model).index("L")
    for _ in range(10000):
        x_true = rng.uniform(0.0, 1.0, size=model.n_params)
        p_true = api.x2params(model, x_true, reopt=reopt_truth)
        if p_true is None or not np.all(np.isfinite(p_true)) or p_true[i_L] * cfg.time_step > 0.5:
            continue
        vmod = np.asarray(vmod_fn(model, obs_model, p_true), dtype=np.float64)
        if not (np.all(np.isfinite(vmod)) and np.ptp(vmod) < 6.0):
            continue
        if cfg.n_minima > 0:
            peaks = _model_minima(vmod)
            if peaks.size < cfg.n_minima:
                continue
            pick = peaks[np.linspace(0, peaks.size - 1, cfg.n_minima).round().astype(int)]
            # NUDGE fails a model with more than M_MAX minima near the observed ones
            # (cuda.c:737-742); keep the truth well inside (M_MAX2 = 20).
            near = sum(np.any(np.abs(obs0.mjd[peaks][:, None] - obs0.mjd[pick][None, :]) < 0.18, axis=1))
            if near > 20:
                continue
        break
    else:
        raise RuntimeError("no resolvable true model found")
    x_true = api.params2x(model, p_true)
    dv = rng.uniform(-cfg.dv_range, cfg.dv_range, size=cfg.n_filters) if cfg.dv_range > 0 else np.zeros(cfg.n_filters)
    v_target = vmod + cfg.base_mag + dv[fidx] + rng.normal(0.0, cfg.sigma, size=cfg.n_points)
    _write_lc(out / "lc.dat", chars, mjd_obs, v_target - geom, sgm)

    files = {"lc": out / "lc.dat", "eph_dir": out}
    t_min = v_min = np.zeros(0)
    if cfg.n_minima > 0:
        # Brightness minima (model V maxima) of the true curve at the data points.
        peaks = _model_minima(vmod)
        pick = np.unique(peaks[np.linspace(0, peaks.size - 1, cfg.n_minima).round().astype(int)])
        t_min = obs0.mjd[pick] + obs0.hmjd0
        v_min = vmod[pick] + cfg.base_mag + dv[0]
        with open(out / "observed.min", "w") as f:
            for a, b in zip(t_min, v_min):
                f.write(f"{a:.6f} {b:.4f}\n")
        files["minima"] = out / "observed.min"
    obs = api.read_data(out / "lc.dat", out, interp=interp, minima_path=files.get("minima"))
    truth = {"config": asdict(cfg), "x_true": x_true.tolist(), "params_true": p_true.tolist(),
             "dv_true": (dv + cfg.base_mag).tolist(), "param_names": api.param_names(model)}
    (out / "truth.json").write_text(json.dumps(truth, indent=1))
    return Synth(cfg, out, model, obs, x_true, p_true, dv + cfg.base_mag, files)


# Variants of the batched workload (config 3), drawn evenly: LS + TORQUE, BC, BW_BALL, all with
# ACC so that one batch (one simplex precision) holds them.
BATCH_VARIANTS = ("TORQUE,ACC", "BC,ACC", "BW_BALL,ACC")


def batch_config(i: int, seed: int = 1003) -> SynthConfig:
    """Object i of the batched workload: log-uniform 50-2000 points, 1-4 filters, a span of
    3-60 days in nightly 6 h windows, the variant BATCH_VARIANTS[i % 3]."""
    rng = np.random.default_rng([seed, i])
    n_points = int(round(np.exp(rng.uniform(np.log(50.0), np.log(2000.0)))))
    n_filters = int(rng.integers(1, 5))
    span = int(rng.integers(3, 61))
    n_nights = span if span <= 10 else int(rng.integers(max(3, span // 4), span + 1))
    chars = "RVBI"[:n_filters]
    return SynthConfig(f"c3_{i}", BATCH_VARIANTS[i % 3], 1e-2, n_points, n_filters, span, n_nights, seed=seed * 100003 + i,
                       filter_chars=chars, dv_range=0.5 if n_filters > 1 else 0.0)


def generate_batch(n_objects: int, outdir, seed: int = 1003, vmod_fn=None) -> list:
    """n_objects objects of the batched workload under outdir/<i>."""
    out = Path(outdir)
    return [generate(batch_config(i, seed), out / f"{i:04d}", vmod_fn) for i in range(n_objects)]
