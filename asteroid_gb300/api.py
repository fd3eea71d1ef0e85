"""Python host API over the C ABI (include/asteroid_gb300.h).

Mirrors the reference's host flow (asteroid.c:main): build the variant tables
(``make_model`` ~ asteroid.c:86-169,473-601), read the light curve and ephemerides
(``read_data`` ~ read_data.c), upload (``Engine`` ~ gpu_prepare.c + cudaMemcpyToSymbol), evaluate
chi^2 (``Engine.eval`` ~ chi2one) and run the simplex search (``Engine.fit`` ~ setup_kernel +
chi2_gpu + the host argmin, asteroid.c:626-759).  Every call goes to the CUDA engine; there is no
CPU fallback: without the built library or a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import capi
from .capi import (ACC, BC, BW_BALL, INTERP, NUDGE, P_PSI, PREC_FP64, PREC_MIXED, PREC_MIXED_RHS32, TORQUE, check,
                   dptr, fptr, iptr)


def flags_from_names(names) -> int:
    """"TORQUE,P_PSI" or ["TORQUE", "P_PSI"] -> flag bits (the reference's -D macros)."""
    if isinstance(names, int):
        return names
    if isinstance(names, str):
        names = [n for n in names.replace("+", ",").split(",") if n.strip()]
    f = 0
    for n in names:
        n = n.strip().upper().lstrip("-D")
        if n not in capi.FLAG_NAMES:
            raise ValueError(f"unknown variant macro {n!r}")
        f |= capi.FLAG_NAMES[n]
    return f


def flag_names(flags: int) -> str:
    return ",".join(n for n, b in capi.FLAG_NAMES.items() if flags & b) or "LS"


def make_model(flags, time_step: float = 1e-2, ppsi_hours=(2.0, 4800.0)) -> capi.Model:
    """Variant tables exactly as the reference builds them (asteroid.c:86-169,473-601)."""
    lib = capi.load()
    m = capi.Model()
    check(lib.ast_model_init(C.byref(m), flags_from_names(flags), float(time_step),
                             float(ppsi_hours[0]), float(ppsi_hours[1])), "ast_model_init")
    return m


def param_names(m: capi.Model) -> list[str]:
    lib = capi.load()
    return [lib.ast_param_name(C.byref(m), i).decode() for i in range(m.n_params)]


def x2params(m: capi.Model, x, reopt: int = 1):
    """Dimensionless x -> physical parameters; None when x leaves a hard limit."""
    lib = capi.load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    p = np.zeros(m.n_params)
    rc = check(lib.ast_x2params(C.byref(m), int(reopt), dptr(x), dptr(p)), "ast_x2params")
    return None if rc else p


def params2x(m: capi.Model, params):
    lib = capi.load()
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.zeros(m.n_params)
    check(lib.ast_params2x(C.byref(m), dptr(p), dptr(x)), "ast_params2x")
    return x


@dataclass
class Obs:
    """One object's light curve in the converted frame the model uses (read_data.c:243-302)."""
    mjd: np.ndarray                      # asteroid time minus hMJD0 (days)
    v: np.ndarray                        # float32 magnitudes
    w: np.ndarray                        # float32 1/sgm^2
    filt: np.ndarray                     # int32 filter index
    e_unit: np.ndarray                   # (n,3) unit asteroid->Earth
    s_unit: np.ndarray                   # (n,3) unit asteroid->Sun
    eph_e: np.ndarray = field(default_factory=lambda: np.zeros((3, 3)))   # [component][point]
    eph_s: np.ndarray = field(default_factory=lambda: np.zeros((3, 3)))
    eph_mjd0: np.ndarray = field(default_factory=lambda: np.zeros(3))
    t_min: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v_min: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    hmjd0: float = 0.0
    filters: str = "W"

    def __post_init__(self):
        self.mjd = np.ascontiguousarray(self.mjd, dtype=np.float64)
        self.v = np.ascontiguousarray(self.v, dtype=np.float32)
        self.w = np.ascontiguousarray(self.w, dtype=np.float32)
        self.filt = np.ascontiguousarray(self.filt, dtype=np.int32)
        self.e_unit = np.ascontiguousarray(np.asarray(self.e_unit, dtype=np.float64).reshape(-1, 3))
        self.s_unit = np.ascontiguousarray(np.asarray(self.s_unit, dtype=np.float64).reshape(-1, 3))
        self.eph_e = np.asarray(self.eph_e, dtype=np.float64).reshape(3, 3)
        self.eph_s = np.asarray(self.eph_s, dtype=np.float64).reshape(3, 3)
        self.eph_mjd0 = np.asarray(self.eph_mjd0, dtype=np.float64).reshape(3)
        self.t_min = np.asarray(self.t_min, dtype=np.float32).reshape(-1)
        self.v_min = np.asarray(self.v_min, dtype=np.float32).reshape(-1)

    @property
    def n_data(self) -> int:
        return int(self.mjd.shape[0])

    @property
    def n_filters(self) -> int:
        return int(self.filt.max()) + 1 if self.filt.size else 0

    def as_c(self) -> capi.ObsSet:
        """ObsSet pointing into this object's arrays (keep self alive while it is used)."""
        o = capi.ObsSet()
        o.n_data = self.n_data
        o.n_filters = self.n_filters
        o.mjd = dptr(self.mjd)
        o.v = fptr(self.v)
        o.w = fptr(self.w)
        o.filter = iptr(self.filt)
        o.e_unit = dptr(self.e_unit)
        o.s_unit = dptr(self.s_unit)
        for k in range(3):
            for j in range(3):
                o.eph_e[k][j] = self.eph_e[k, j]
                o.eph_s[k][j] = self.eph_s[k, j]
            o.eph_mjd0[k] = self.eph_mjd0[k]
        o.n_minima = int(self.t_min.size)
        for k in range(min(self.t_min.size, capi.AST_NOBS_MAX)):
            o.t_min[k] = self.t_min[k]
            o.v_min[k] = self.v_min[k]
        return o

    def with_minima(self, t_min, v_min) -> "Obs":
        self.t_min = np.asarray(t_min, np.float32).reshape(-1)
        self.v_min = np.asarray(v_min, np.float32).reshape(-1)
        return self


def read_data(lc_path, eph_dir=".", interp: bool = False, minima_path=None, max_filters: int = 8) -> Obs:
    """read_data.c + prepare_chi2_params (misc.c:279-323), through the C host reader."""
    lib = capi.load()
    hd = C.POINTER(capi.HostData)()
    check(lib.ast_read_data(str(lc_path).encode(), str(eph_dir).encode(), int(bool(interp)), int(max_filters),
                            C.byref(hd)), "ast_read_data")
    try:
        if minima_path is not None:
            check(lib.ast_read_minima(str(minima_path).encode(), hd), "ast_read_minima")
        h = hd.contents
        n = h.obs.n_data
        o = Obs(
            mjd=np.ctypeslib.as_array(h.mjd, (n,)).copy(),
            v=np.ctypeslib.as_array(h.v, (n,)).copy(),
            w=np.ctypeslib.as_array(h.w, (n,)).copy(),
            filt=np.ctypeslib.as_array(h.filter, (n,)).copy(),
            e_unit=np.ctypeslib.as_array(h.e_unit, (n * 3,)).copy(),
            s_unit=np.ctypeslib.as_array(h.s_unit, (n * 3,)).copy(),
            eph_e=np.array([[h.obs.eph_e[k][j] for j in range(3)] for k in range(3)]),
            eph_s=np.array([[h.obs.eph_s[k][j] for j in range(3)] for k in range(3)]),
            eph_mjd0=np.array([h.obs.eph_mjd0[k] for k in range(3)]),
            t_min=np.array([h.obs.t_min[k] for k in range(h.obs.n_minima)], np.float32),
            v_min=np.array([h.obs.v_min[k] for k in range(h.obs.n_minima)], np.float32),
            hmjd0=h.hmjd0,
            filters=bytes(h.filters[: h.obs.n_filters]).decode(errors="replace"),
        )
        return o
    finally:
        lib.ast_free_host_data(hd)


def plot_grid(lc_path, eph_dir=".", n_plot: int = 20000, interp: bool = False):
    """The -plot grid (read_data.c:309-370): times relative to hMJD0 and unit E, S vectors
    [n_plot, 3] from the light curve's last ephemeris window, through the C host."""
    lib = capi.load()
    hd = C.POINTER(capi.HostData)()
    check(lib.ast_read_data(str(lc_path).encode(), str(eph_dir).encode(), int(bool(interp)), 8, C.byref(hd)),
          "ast_read_data")
    try:
        t = np.zeros(n_plot)
        e = np.zeros((n_plot, 3))
        s = np.zeros((n_plot, 3))
        check(lib.ast_plot_grid(hd, int(bool(interp)), int(n_plot), dptr(t), dptr(e), dptr(s)), "ast_plot_grid")
        return t, e, s
    finally:
        lib.ast_free_host_data(hd)


@dataclass
class PeriodogramResult:
    cl_fr: np.ndarray       # [5] cluster frequencies (1/day), -1 where none
    cl_H: np.ndarray        # [5] normalised counts there, 0 where none
    counts: np.ndarray      # [10000] raw count of each frequency bin
    n_minima: int
    n_clusters: int
    n_intervals: int
    n_distinct: int
    kernel_ms: float
    count_ms: float


def minima(t, vm, device: int = -1) -> PeriodogramResult:
    """Periodogram of the minima of a model curve (misc.c:65-276), on the GPU."""
    lib = capi.load()
    t = np.ascontiguousarray(t, dtype=np.float64)
    vm = np.ascontiguousarray(vm, dtype=np.float64)
    if t.shape != vm.shape:
        raise ValueError("t and vm differ in length")
    out = capi.Periodogram()
    counts = np.zeros(capi.MINIMA_BINS, np.int32)
    check(lib.ast_minima(int(device), int(t.size), dptr(t), dptr(vm), C.byref(out), iptr(counts)), "ast_minima")
    return PeriodogramResult(np.array(out.cl_fr[:]), np.array(out.cl_H[:]), counts, out.n_minima, out.n_clusters,
                             out.n_intervals, out.n_distinct, out.kernel_ms,
                             out.count_ms)


def render_frames(geo, size_pix: int = 1080, device: int = -1):
    """ANIMATE frames [n, size_pix, size_pix, 3] (uint8) from their geometry, and the device ms."""
    lib = capi.load()
    g = np.ascontiguousarray(geo, dtype=np.float64).reshape(-1, capi.AST_GEO)
    rgb = np.zeros((g.shape[0], size_pix, size_pix, 3), np.uint8)
    ms = C.c_double(0)
    check(lib.ast_render_frames(int(device), dptr(g), int(g.shape[0]), int(size_pix),
                                rgb.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(ms)), "ast_render_frames")
    return rgb, ms.value


def write_png(path, rgb) -> None:
    """One 8-bit RGB PNG from an [height, width, 3] uint8 array."""
    lib = capi.load()
    a = np.ascontiguousarray(rgb, dtype=np.uint8)
    check(lib.ast_write_png(str(path).encode(), a.ctypes.data_as(C.POINTER(C.c_uint8)), int(a.shape[1]),
                            int(a.shape[0])), "ast_write_png")


def format_result(chi2, dv, params) -> str:
    """One output line in the reference's format (asteroid.c:798-811)."""
    lib = capi.load()
    dv = np.ascontiguousarray(dv, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    buf = C.create_string_buffer(4096)
    check(lib.ast_format_result(buf, 4096, float(chi2), dptr(dv), int(dv.size), dptr(p), int(p.size)),
          "ast_format_result")
    return buf.value.decode()


@dataclass
class FitResult:
    best_f: np.ndarray        # [groups]
    best_params: np.ndarray   # [groups, n_params]
    best_dv: np.ndarray       # [groups, n_filters]
    chain_f: np.ndarray       # [chains]
    n_evals: int
    n_fits: int
    kernel_ms: float

    @property
    def best(self) -> int:
        """Host argmin over groups (asteroid.c:741-759): first minimum."""
        return int(np.argmin(self.best_f))


class Engine:
    """One object on the GPU: observations staged in HBM, tables uploaded."""

    def __init__(self, model: capi.Model, obs: Obs, device: int = -1):
        self.lib = capi.load()
        self.model = model
        self.obs = obs
        self._cobs = obs.as_c()
        self.ctx = C.c_void_p()
        check(self.lib.ast_prepare(C.byref(model), C.byref(self._cobs), int(device), C.byref(self.ctx)), "ast_prepare")
        self.n_params = model.n_params
        self.n_filters = obs.n_filters

    def close(self):
        if self.ctx:
            self.lib.ast_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_tables(self, model: capi.Model):
        check(self.lib.ast_set_tables(self.ctx, C.byref(model)), "ast_set_tables")
        self.model = model

    @property
    def stream(self) -> int:
        return self.lib.ast_stream(self.ctx) or 0

    def eval(self, params, precision: int = PREC_FP64, chi2_out=None, dv_out=None):
        """chi2one on each row of params [n, n_params] -> (chi2 [n], delta_V [n, n_filters]).
        chi2_out / dv_out: optional float64 host arrays of those shapes to write into (for
        example views of page-locked buffers)."""
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        if p.shape[1] != self.n_params:
            raise ValueError(f"params must have {self.n_params} columns")
        n = p.shape[0]
        chi2 = np.zeros(n) if chi2_out is None else chi2_out
        dv = np.zeros((n, self.n_filters)) if dv_out is None else dv_out
        if chi2.shape != (n,) or dv.shape != (n, self.n_filters) or chi2.dtype != np.float64 or \
                dv.dtype != np.float64 or not (chi2.flags.c_contiguous and dv.flags.c_contiguous):
            raise ValueError("chi2_out / dv_out must be contiguous float64 arrays of shapes (n,), (n, n_filters)")
        check(self.lib.ast_eval_batch(self.ctx, int(precision), dptr(p), n, dptr(chi2), dptr(dv)), "ast_eval_batch")
        return chi2, dv

    def eval_device(self, d_params: int, n: int, d_chi2: int, d_dv: int, stream: int = 0,
                    precision: int = PREC_FP64):
        """Stream-ordered evaluation on device buffers (raw pointers)."""
        check(self.lib.ast_eval_batch_device(self.ctx, int(precision), C.c_void_p(d_params), int(n), C.c_void_p(d_chi2),
                                             C.c_void_p(d_dv) if d_dv else None, C.c_void_p(stream) if stream else None),
              "ast_eval_batch_device")

    def model_curve(self, params) -> np.ndarray:
        p = np.ascontiguousarray(params, dtype=np.float64)
        out = np.zeros(self.obs.n_data)
        check(self.lib.ast_model_curve(self.ctx, dptr(p), dptr(out)), "ast_model_curve")
        return out

    def model_curve_at(self, params, t, e_unit=None, s_unit=None) -> np.ndarray:
        """Model magnitudes at increasing times t (relative to hMJD0) with unit E, S [n, 3]
        (unused under INTERP): the -plot model curve."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        e = None if e_unit is None else np.ascontiguousarray(e_unit, dtype=np.float64).reshape(-1, 3)
        s = None if s_unit is None else np.ascontiguousarray(s_unit, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(t.size)
        check(self.lib.ast_model_curve_at(self.ctx, dptr(p), int(t.size), dptr(t), dptr(e) if e is not None else None,
                                          dptr(s) if s is not None else None, dptr(out)), "ast_model_curve_at")
        return out

    def rmsd(self, params0, dx: float, n_streams: int = 116736, samples: int = 1, seed: int = 1, call: int = 0,
             precision: int = PREC_FP64, reopt: bool = True, spherical_k: bool = False, trace: bool = False) -> dict:
        """One chi2_gpu_rms call (cuda.c:2148-2389): RMSD confidence intervals of params0 over
        n_streams x samples random models (the ctx model must carry RMSD)."""
        p0 = np.ascontiguousarray(params0, dtype=np.float64)
        N = self.model.n_params
        rows = int(n_streams) * int(samples)
        cfg = capi.RmsdCfg()
        cfg.seed = int(seed) & ((1 << 64) - 1)
        cfg.n_streams = int(n_streams)
        cfg.samples = int(samples)
        cfg.precision = int(precision)
        cfg.dx = float(dx)
        cfg.reopt = int(bool(reopt))
        cfg.spherical_k = int(bool(spherical_k))
        cfg.call = int(call)
        cfg.params0 = dptr(p0)
        tx = np.zeros((rows, N)) if trace else None
        tf = np.zeros(rows) if trace else None
        if trace:
            cfg.trace_x = dptr(tx)
            cfg.trace_f = dptr(tf)
        out = capi.RmsdOut()
        check(self.lib.ast_rmsd(self.ctx, C.byref(cfg), C.byref(out)), "ast_rmsd")
        r = {"f0": out.f0, "f1": out.f1, "n_tot": out.n_tot, "n_bad": out.n_bad,
             "par_min": np.array(out.par_min[:N]), "par_max": np.array(out.par_max[:N]), "kernel_ms": out.kernel_ms}
        if trace:
            r["trace_x"], r["trace_f"] = tx, tf
        return r

    def model_geometry(self, params, t, e_unit=None, s_unit=None) -> np.ndarray:
        """compute_rgb's inputs [n, 20] at increasing times t (the ANIMATE snapshots)."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        e = None if e_unit is None else np.ascontiguousarray(e_unit, dtype=np.float64).reshape(-1, 3)
        s = None if s_unit is None else np.ascontiguousarray(s_unit, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((t.size, capi.AST_GEO))
        check(self.lib.ast_model_geometry(self.ctx, dptr(p), int(t.size), dptr(t), dptr(e) if e is not None else None,
                                          dptr(s) if s is not None else None, dptr(out)), "ast_model_geometry")
        return out

    def model_angles(self, params, precision: int = PREC_FP64) -> np.ndarray:
        """Euler angles [n_data, 3] along the FP64 or the mixed-precision integration."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        out = np.zeros((self.obs.n_data, 3))
        check(self.lib.ast_model_angles(self.ctx, int(precision), dptr(p), dptr(out)), "ast_model_angles")
        return out

    def _cfg(self, n_chains, group_size, n_stages, seed, reopt, params0, precision, evals_cap, steps_cap, tpb,
             min_ctas_per_sm=0, stage_obs=0, fp64_result=False):
        cfg = capi.FitCfg()
        cfg.seed = int(seed) & ((1 << 64) - 1)
        cfg.n_chains = int(n_chains)
        cfg.group_size = int(group_size)
        cfg.n_stages = int(n_stages)
        cfg.reopt = int(bool(reopt))
        cfg.precision = int(precision)
        cfg.evals_cap = int(evals_cap)
        cfg.steps_cap = int(steps_cap)
        cfg.tpb = int(tpb)
        cfg.min_ctas_per_sm = int(min_ctas_per_sm)
        cfg.stage_obs = int(stage_obs)
        cfg.fp64_result = int(bool(fp64_result))
        self._p0 = None
        if reopt:
            self._p0 = np.ascontiguousarray(params0, dtype=np.float64)
            cfg.params0 = dptr(self._p0)
        return cfg

    def fit_begin(self, n_chains=56 * 256, group_size=256, n_stages=1, seed=1, reopt=False, params0=None,
                  precision=PREC_FP64, evals_cap=0, steps_cap=0, tpb=0, min_ctas_per_sm=0, stage_obs=0,
                  fp64_result=False):
        self._fitcfg = self._cfg(n_chains, group_size, n_stages, seed, reopt, params0, precision, evals_cap,
                                 steps_cap, tpb, min_ctas_per_sm, stage_obs, fp64_result)
        check(self.lib.ast_fit_begin(self.ctx, C.byref(self._fitcfg)), "ast_fit_begin")

    def fit_step(self, evals_per_slot: int = 0, stream: int = 0) -> bool:
        done = C.c_int32(0)
        check(self.lib.ast_fit_step(self.ctx, int(evals_per_slot), C.byref(done),
                                    C.c_void_p(stream) if stream else None), "ast_fit_step")
        return bool(done.value)

    def fit_counters(self):
        ne, nf = C.c_int64(0), C.c_int64(0)
        check(self.lib.ast_fit_counters(self.ctx, C.byref(ne), C.byref(nf)), "ast_fit_counters")
        return ne.value, nf.value

    def fit_slots(self) -> int:
        return int(self.lib.ast_fit_slots(self.ctx))

    def fit_launch(self) -> dict:
        """Launch geometry of the current fit: CTA size, CTAs, register budget, shared bytes."""
        v = [C.c_int32(0) for _ in range(4)]
        check(self.lib.ast_fit_launch(self.ctx, *[C.byref(x) for x in v]), "ast_fit_launch")
        return dict(tpb=v[0].value, ctas=v[1].value, min_ctas_per_sm=v[2].value, smem=v[3].value)

    def fit_end(self) -> FitResult:
        cfg = self._fitcfg
        G = cfg.n_chains // cfg.group_size
        res = FitResult(np.zeros(G), np.zeros((G, self.n_params)), np.zeros((G, self.n_filters)),
                        np.zeros(cfg.n_chains), 0, 0, 0.0)
        out = capi.FitOut()
        out.best_f = dptr(res.best_f)
        out.best_params = dptr(res.best_params)
        out.best_dv = dptr(res.best_dv)
        out.chain_f = dptr(res.chain_f)
        check(self.lib.ast_fit_end(self.ctx, C.byref(out)), "ast_fit_end")
        res.n_evals, res.n_fits, res.kernel_ms = out.n_evals, out.n_fits, out.kernel_ms
        return res

    def fit(self, n_chains=56 * 256, group_size=256, n_stages=1, seed=1, reopt=False, params0=None,
            precision=PREC_FP64, evals_cap=0, steps_cap=0, tpb=0, min_ctas_per_sm=0, stage_obs=0,
            fp64_result=False) -> FitResult:
        """setup_kernel + chi2_gpu + result copies for one pass (asteroid.c:626-759)."""
        self.fit_begin(n_chains, group_size, n_stages, seed, reopt, params0, precision, evals_cap, steps_cap, tpb,
                       min_ctas_per_sm, stage_obs, fp64_result)
        while not self.fit_step(0):
            pass
        return self.fit_end()


def probe_peak(kind: str = "fp64", device: int = -1) -> float:
    """Measured FMA throughput in GFLOP/s (kind 'fp64' or 'fp32')."""
    lib = capi.load()
    g = C.c_double(0)
    check(lib.ast_probe_peak(int(device), 0 if kind == "fp64" else 1, C.byref(g)), "ast_probe_peak")
    return g.value


def fit_cfg(n_chains=1024, group_size=256, seed=1, reopt=False, params0=None, precision=PREC_FP64, evals_cap=0,
            steps_cap=0, n_stages=1, tpb=0, fp64_result=False):
    """An ast_fit_cfg; the returned tuple keeps params0 alive while the struct is in use."""
    cfg = capi.FitCfg()
    cfg.seed = int(seed) & ((1 << 64) - 1)
    cfg.n_chains = int(n_chains)
    cfg.group_size = int(group_size)
    cfg.n_stages = int(n_stages)
    cfg.reopt = int(bool(reopt))
    cfg.precision = int(precision)
    cfg.evals_cap = int(evals_cap)
    cfg.steps_cap = int(steps_cap)
    cfg.tpb = int(tpb)
    cfg.fp64_result = int(bool(fp64_result))
    keep = None
    if reopt:
        keep = np.ascontiguousarray(params0, dtype=np.float64)
        cfg.params0 = dptr(keep)
    return cfg, keep


def _result(n_chains, group_size, n_params, n_filters):
    """An empty FitResult for one object and the ast_fit_out that points into it."""
    G = n_chains // group_size
    res = FitResult(np.zeros(G), np.zeros((G, n_params)), np.zeros((G, n_filters)), np.zeros(0), 0, n_chains, 0.0)
    out = capi.FitOut()
    out.best_f = dptr(res.best_f)
    out.best_params = dptr(res.best_params)
    out.best_dv = dptr(res.best_dv)
    return res, out


class Batch:
    """Many objects fitted by one persistent, graph-captured launch (ast_batch_*)."""

    def __init__(self, precision=PREC_MIXED, acc=True, n_slots=0, device=-1):
        self.lib = capi.load()
        h = C.c_void_p()
        check(self.lib.ast_batch_create(int(device), int(precision), int(bool(acc)), int(n_slots), C.byref(h)),
              "ast_batch_create")
        self.h = h
        self.precision = precision
        self.items = []

    def add(self, model, obs: Obs, **cfg_kw) -> int:
        cfg, keep = fit_cfg(precision=self.precision, **cfg_kw)
        idx = C.c_int32(-1)
        cobs = obs.as_c()
        check(self.lib.ast_batch_add(self.h, C.byref(model), C.byref(cobs), C.byref(cfg), C.byref(idx)), "ast_batch_add")
        self.items.append((cfg.n_chains, cfg.group_size, model.n_params, obs.n_filters))
        return idx.value

    def tune(self, evals_per_slot=4) -> dict:
        t = capi.BatchTune()
        check(self.lib.ast_batch_tune(self.h, int(evals_per_slot), C.byref(t)), "ast_batch_tune")
        return dict(tpb=t.tpb, refill=t.refill, ctas=t.ctas, evals_per_s=t.evals_per_s, tile=t.tile)

    def run(self, tpb=0, refill=0, tile=0) -> float:
        """Every chain to completion in one graph-captured launch; tpb / refill / tile set the
        geometry (0: the tuned or default one).  Returns the device milliseconds."""
        ms = C.c_double(0)
        t = None
        if tpb:
            t = capi.BatchTune()
            t.tpb, t.refill, t.tile = int(tpb), int(refill or 1), int(tile)
        check(self.lib.ast_batch_run(self.h, C.byref(t) if t is not None else None, C.byref(ms)), "ast_batch_run")
        return ms.value

    def set_geometry(self, tpb, refill=1, tile=0):
        """The launch geometry of the following step() calls (ast_batch_set_geometry)."""
        t = capi.BatchTune()
        t.tpb, t.refill, t.tile = int(tpb), int(refill), int(tile)
        check(self.lib.ast_batch_set_geometry(self.h, C.byref(t)), "ast_batch_set_geometry")

    def step(self, evals_per_slot: int) -> tuple:
        """One bounded launch: (done, kernel ms)."""
        done, ms = C.c_int32(0), C.c_double(0)
        check(self.lib.ast_batch_step(self.h, int(evals_per_slot), C.byref(done), C.byref(ms)), "ast_batch_step")
        return bool(done.value), ms.value

    def result(self, index) -> FitResult:
        n_chains, group, n_params, n_filters = self.items[index]
        res, out = _result(n_chains, group, n_params, n_filters)
        check(self.lib.ast_batch_result(self.h, int(index), C.byref(out)), "ast_batch_result")
        return res

    def counters(self) -> dict:
        ne, nf = C.c_int64(0), C.c_int64(0)
        tpb, refill, ctas = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        check(self.lib.ast_batch_counters(self.h, C.byref(ne), C.byref(nf), C.byref(tpb), C.byref(refill),
                                          C.byref(ctas)), "ast_batch_counters")
        g = capi.BatchTune()
        check(self.lib.ast_batch_geometry(self.h, C.byref(g)), "ast_batch_geometry")
        return dict(n_evals=ne.value, n_fits=nf.value, tpb=tpb.value, refill=refill.value, ctas=ctas.value,
                    tile=g.tile)

    def close(self):
        if self.h:
            self.lib.ast_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Server:
    """Continuous batching of fit requests (ast_server_*, ast_submit, ast_poll)."""

    def __init__(self, precision=PREC_MIXED, acc=True, n_slots=0, hbm_budget=0, device=-1, lanes=1):
        self.lib = capi.load()
        h = C.c_void_p()
        check(self.lib.ast_server_create(int(device), int(precision), int(bool(acc)), int(n_slots), int(hbm_budget),
                                         C.byref(h)), "ast_server_create")
        self.h = h
        if lanes != 1:
            check(self.lib.ast_server_set_lanes(self.h, int(lanes)), "ast_server_set_lanes")
        self.precision = precision
        self.items = {}

    def submit(self, model, obs: Obs, **cfg_kw) -> int:
        cfg, keep = fit_cfg(precision=self.precision, **cfg_kw)
        rid = C.c_int64(-1)
        cobs = obs.as_c()
        check(self.lib.ast_submit(self.h, C.byref(model), C.byref(cobs), C.byref(cfg), C.byref(rid)), "ast_submit")
        self.items[rid.value] = (cfg.n_chains, cfg.group_size, model.n_params, obs.n_filters)
        return rid.value

    def step(self, evals_per_slot=16):
        r, q = C.c_int32(0), C.c_int32(0)
        check(self.lib.ast_server_step(self.h, int(evals_per_slot), C.byref(r), C.byref(q)), "ast_server_step")
        return r.value, q.value

    def poll(self, request):
        """(FitResult, latency seconds) once done, else None; raises AstError (AST_E_CANCELLED)
        for a cancelled request."""
        n_chains, group, n_params, n_filters = self.items[request]
        res, out = _result(n_chains, group, n_params, n_filters)
        lat = C.c_double(0)
        rc = check(self.lib.ast_poll(self.h, int(request), C.byref(out), C.byref(lat)), "ast_poll")
        return (res, lat.value) if rc == 1 else None

    def cancel(self, request) -> bool:
        """Cancel a queued or running request (ast_cancel); False if it had already finished."""
        return check(self.lib.ast_cancel(self.h, int(request)), "ast_cancel") == 0

    def request_bytes(self, request) -> int:
        return int(self.lib.ast_request_bytes(self.h, int(request)))

    def stats(self) -> dict:
        ne, used, budget = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        ms = C.c_double(0)
        check(self.lib.ast_server_stats(self.h, C.byref(ne), C.byref(ms), C.byref(used), C.byref(budget)),
              "ast_server_stats")
        return dict(n_evals=ne.value, kernel_ms=ms.value, hbm_used=used.value, hbm_budget=budget.value)

    def close(self):
        if self.h:
            self.lib.ast_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
