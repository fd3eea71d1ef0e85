"""THE ORACLE (Python side).  TEST INFRASTRUCTURE ONLY.

ctypes access to oracle/_build/liboracle.so (the CPU restatement in chi2_oracle.c) and to the
reference's own host build in oracle/_ref/libref_<variant>.so (oracle/build_ref.sh).  Only the
tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_DIR = HERE / "_ref"

_lib = None


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            import sys
            sys.path.insert(0, str(HERE.parent))
            from asteroid_gb300 import build
            build.build_oracle()
        lib = C.CDLL(str(LIB_PATH))
        V = C.c_void_p
        lib.orc_chi2.restype = C.c_double
        lib.orc_chi2.argtypes = [V, V, V, V]
        lib.orc_chi2_batch.restype = None
        lib.orc_chi2_batch.argtypes = [V, V, V, C.c_int64, V, V, C.c_int]
        lib.orc_model_curve.restype = None
        lib.orc_model_curve.argtypes = [V, V, V, V]
        lib.orc_x2params.restype = C.c_int
        lib.orc_x2params.argtypes = [V, C.c_int, V, V]
        lib.orc_params2x.restype = None
        lib.orc_params2x.argtypes = [V, V, V]
        lib.orc_uniform.restype = C.c_float
        lib.orc_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32]
        lib.orc_philox4x32_10.restype = None
        lib.orc_philox4x32_10.argtypes = [V, V, V]
        lib.orc_max_threads.restype = C.c_int
        lib.orc_minima.restype = C.c_int
        lib.orc_minima.argtypes = [V, V, C.c_int, C.c_int, V, V, V, V]
        lib.orc_render.restype = None
        lib.orc_render.argtypes = [V, C.c_int, C.c_int, V]
        lib.orc_model_geometry.restype = None
        lib.orc_model_geometry.argtypes = [V, V, V, V]
        lib.orc_rmsd.restype = C.c_int
        lib.orc_rmsd.argtypes = [V, V, V, C.c_uint64, C.c_uint32, C.c_int64, C.c_int32, C.c_float, C.c_int, C.c_int,
                                 V, V, V, V, V, V, V, V]
        lib.orc_fit.restype = None
        lib.orc_fit.argtypes = [V, V, C.c_uint64, C.c_int64, C.c_int32, C.c_int32, C.c_int32, V, C.c_int64, C.c_int32,
                                V, V, V, V, V]
        _lib = lib
    return _lib


def _ptrs(model, obs):
    """(model*, obs*) plus the objects that keep the ctypes structures alive."""
    cobs = obs.as_c()
    return C.cast(C.byref(model), C.c_void_p), C.cast(C.byref(cobs), C.c_void_p), cobs


def chi2(model, obs, params):
    lib = load()
    mp, op, keep = _ptrs(model, obs)
    p = np.ascontiguousarray(params, dtype=np.float64)
    dv = np.zeros(obs.n_filters)
    r = lib.orc_chi2(mp, op, p.ctypes.data, dv.ctypes.data)
    return r, dv


def chi2_batch(model, obs, params, threads: int = 0):
    lib = load()
    mp, op, keep = _ptrs(model, obs)
    p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
    n = p.shape[0]
    out = np.zeros(n)
    dv = np.zeros((n, obs.n_filters))
    lib.orc_chi2_batch(mp, op, p.ctypes.data, n, out.ctypes.data, dv.ctypes.data, int(threads))
    return out, dv


def model_curve(model, obs, params):
    lib = load()
    mp, op, keep = _ptrs(model, obs)
    p = np.ascontiguousarray(params, dtype=np.float64)
    out = np.zeros(obs.n_data)
    lib.orc_model_curve(mp, op, p.ctypes.data, out.ctypes.data)
    return out


def minima(t, vm, threads: int = 0):
    """Periodogram of model minima (misc.c:65-276): (cl_fr[5], cl_H[5], counts[10000], n_minima)."""
    lib = load()
    t = np.ascontiguousarray(t, dtype=np.float64)
    vm = np.ascontiguousarray(vm, dtype=np.float64)
    fr = np.zeros(5)
    h = np.zeros(5)
    counts = np.zeros(10000, np.int32)
    n = np.zeros(1, np.int32)
    rc = lib.orc_minima(t.ctypes.data, vm.ctypes.data, int(t.size), int(threads or max_threads()), fr.ctypes.data,
                        h.ctypes.data, counts.ctypes.data, n.ctypes.data)
    if rc < 0:
        raise ValueError("more than 10000 minima")
    return fr, h, counts, int(n[0])


def rmsd(model, obs, params0, seed, call, n_streams, samples, dx, reopt=1, spherical=False, x_in=None,
         f_in=None, trace=False):
    """RMSD confidence intervals of chi2_gpu_rms (cuda.c:2148-2389), one call.  Returns a dict with
    f0, f1, n_tot, n_bad, par_min, par_max (double) and, with trace, the drawn points and RMSDs."""
    lib = load()
    mp, op, keep = _ptrs(model, obs)
    p0 = np.ascontiguousarray(params0, dtype=np.float64)
    N = model.n_params
    rows = int(n_streams) * int(samples)
    f01 = np.zeros(2)
    counts = np.zeros(2, np.int64)
    pmin = np.zeros(N)
    pmax = np.zeros(N)
    tx = np.zeros((rows, N)) if trace else None
    tf = np.zeros(rows) if trace else None
    xi = None if x_in is None else np.ascontiguousarray(x_in, dtype=np.float64).reshape(rows, N)
    fi = None if f_in is None else np.ascontiguousarray(f_in, dtype=np.float64).reshape(rows)
    lib.orc_rmsd(mp, op, p0.ctypes.data, int(seed) & ((1 << 64) - 1), int(call), int(n_streams), int(samples),
                 float(dx), int(reopt), int(bool(spherical)), None if xi is None else xi.ctypes.data,
                 None if fi is None else fi.ctypes.data, f01.ctypes.data, counts.ctypes.data, pmin.ctypes.data, pmax.ctypes.data,
                 None if tx is None else tx.ctypes.data, None if tf is None else tf.ctypes.data)
    out = {"f0": f01[0], "f1": f01[1], "n_tot": int(counts[0]), "n_bad": int(counts[1]), "par_min": pmin,
           "par_max": pmax}
    if trace:
        out["trace_x"], out["trace_f"] = tx, tf
    return out


def model_geometry(model, obs, params):
    """compute_rgb's 20 inputs at every observation of obs, [n, 20]."""
    lib = load()
    mp, op, keep = _ptrs(model, obs)
    p = np.ascontiguousarray(params, dtype=np.float64)
    geo = np.zeros((obs.n_data, 20))
    lib.orc_model_geometry(mp, op, p.ctypes.data, geo.ctypes.data)
    return geo


def render(geo, size_pix):
    """compute_rgb frames [n_frames, size_pix, size_pix, 3] (uint8) from their geometry."""
    lib = load()
    g = np.ascontiguousarray(geo, dtype=np.float64).reshape(-1, 20)
    rgb = np.zeros((g.shape[0], size_pix, size_pix, 3), np.uint8)
    lib.orc_render(g.ctypes.data, int(g.shape[0]), int(size_pix), rgb.ctypes.data)
    return rgb


def x2params(model, x, reopt=1):
    lib = load()
    xx = np.ascontiguousarray(x, dtype=np.float64)
    p = np.zeros(model.n_params)
    rc = lib.orc_x2params(C.cast(C.byref(model), C.c_void_p), int(reopt), xx.ctypes.data, p.ctypes.data)
    return None if rc else p


def params2x(model, params):
    lib = load()
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.zeros(model.n_params)
    lib.orc_params2x(C.cast(C.byref(model), C.c_void_p), p.ctypes.data, x.ctypes.data)
    return x


def uniform(seed, chain, stage, k):
    return load().orc_uniform(seed, chain, stage, k)


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    load().orc_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out


def fit(model, obs, seed, n_chains, group_size, n_stages=1, reopt=False, params0=None, evals_cap=0, steps_cap=0):
    """Group/stage simplex driver on the CPU (small cases)."""
    lib = load()
    mp, op, keep = _ptrs(model, obs)
    G = n_chains // group_size
    bf = np.zeros(G)
    bp = np.zeros((G, model.n_params))
    bdv = np.zeros((G, obs.n_filters))
    cf = np.zeros(n_chains)
    ne = C.c_int64(0)
    p0 = np.ascontiguousarray(params0 if params0 is not None else np.zeros(model.n_params), dtype=np.float64)
    lib.orc_fit(mp, op, int(seed), int(n_chains), int(group_size), int(n_stages), int(bool(reopt)), p0.ctypes.data,
                int(evals_cap), int(steps_cap), bf.ctypes.data, bp.ctypes.data, bdv.ctypes.data, cf.ctypes.data,
                C.cast(C.byref(ne), C.c_void_p))
    return {"best_f": bf, "best_params": bp, "best_dv": bdv, "chain_f": cf, "n_evals": ne.value}


def max_threads() -> int:
    return int(load().orc_max_threads())


# ---------------------------------------------------------------- the reference's host build

class RefHost:
    """The reference's own chi2one / x2params / params2x, built from its sources."""

    def __init__(self, variant: str):
        path = REF_DIR / f"libref_{variant}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        lib = C.CDLL(str(path))
        V = C.c_void_p
        I = C.c_int
        lib.refh_chi2.restype = I
        lib.refh_chi2.argtypes = [V, I, V, I, V, I, I, I, V, V, V, V, V, V, V, V, V, I, V, V, V, V, V]
        lib.refh_x2params.restype = I
        lib.refh_x2params.argtypes = [V, I, V, I, V, I, C.c_float, C.c_float, I, V, V]
        lib.refh_params2x.restype = I
        lib.refh_params2x.argtypes = [V, I, V, I, V, I, V, V]
        for n in ("refh_n_params", "refh_n_types", "refh_chi_float_bytes", "refh_max_filters"):
            getattr(lib, n).restype = I
        lib.refh_time_step.restype = C.c_double
        self.lib = lib
        self.n_params = lib.refh_n_params()
        self.n_types = lib.refh_n_types()
        self.time_step = lib.refh_time_step()

    def _tables(self, m):
        prop = np.ctypeslib.as_array(m.property).reshape(-1, 6)[: m.n_params].astype(np.int32).copy()
        types = np.ctypeslib.as_array(m.types)[: m.n_types].astype(np.int32).copy()
        lim = np.ctypeslib.as_array(m.limits).reshape(2, -1).astype(np.float64).copy()
        return prop, types, lim

    def chi2(self, m, obs, params):
        prop, types, lim = self._tables(m)
        p = np.ascontiguousarray(params, dtype=np.float64)
        out = np.zeros(1)
        dv = np.zeros(max(obs.n_filters, 1))
        cobs = obs  # arrays
        rc = self.lib.refh_chi2(prop.ctypes.data, m.n_params, types.ctypes.data, m.n_types, lim.ctypes.data,
                                lim.shape[1], obs.n_data, obs.n_filters, obs.mjd.ctypes.data, obs.v.ctypes.data,
                                obs.w.ctypes.data, obs.filt.ctypes.data, obs.e_unit.ctypes.data,
                                obs.s_unit.ctypes.data, np.ascontiguousarray(obs.eph_e).ctypes.data,
                                np.ascontiguousarray(obs.eph_s).ctypes.data,
                                np.ascontiguousarray(obs.eph_mjd0).ctypes.data, int(obs.t_min.size),
                                obs.t_min.ctypes.data, obs.v_min.ctypes.data, p.ctypes.data, out.ctypes.data,
                                dv.ctypes.data)
        del cobs
        if rc:
            raise RuntimeError(f"refh_chi2 failed ({rc}): tables do not match the reference build")
        return out[0], dv

    def model_curve(self, m, obs, params):
        """chi2one with Nplot > 0 (the plot branch, cuda.c:699-704): the model magnitude at every
        observation, without the delta_V shift.  Not available in -DNUDGE builds."""
        prop, types, lim = self._tables(m)
        p = np.ascontiguousarray(params, dtype=np.float64)
        out = np.zeros(obs.n_data)
        V, I = C.c_void_p, C.c_int
        f = self.lib.refh_model_curve
        f.restype = I
        f.argtypes = [V, I, V, I, V, I, I, I, V, V, V, V, V, V, V, V, V, V, V]
        rc = f(prop.ctypes.data, m.n_params, types.ctypes.data, m.n_types, lim.ctypes.data, lim.shape[1], obs.n_data,
               obs.n_filters, obs.mjd.ctypes.data, obs.v.ctypes.data, obs.w.ctypes.data, obs.filt.ctypes.data,
               obs.e_unit.ctypes.data, obs.s_unit.ctypes.data, np.ascontiguousarray(obs.eph_e).ctypes.data,
               np.ascontiguousarray(obs.eph_s).ctypes.data, np.ascontiguousarray(obs.eph_mjd0).ctypes.data,
               p.ctypes.data, out.ctypes.data)
        if rc:
            raise RuntimeError(f"refh_model_curve failed ({rc})")
        return out

    def x2params(self, m, x, reopt=1):
        prop, types, lim = self._tables(m)
        xx = np.ascontiguousarray(x, dtype=np.float64)
        p = np.zeros(m.n_params)
        rc = self.lib.refh_x2params(prop.ctypes.data, m.n_params, types.ctypes.data, m.n_types, lim.ctypes.data,
                                    lim.shape[1], m.ppsi1, m.ppsi2, int(reopt), xx.ctypes.data, p.ctypes.data)
        if rc < 0:
            raise RuntimeError("refh_x2params: tables do not match the reference build")
        return None if rc else p

    def params2x(self, m, params):
        prop, types, lim = self._tables(m)
        p = np.ascontiguousarray(params, dtype=np.float64)
        x = np.zeros(m.n_params)
        rc = self.lib.refh_params2x(prop.ctypes.data, m.n_params, types.ctypes.data, m.n_types, lim.ctypes.data,
                                    lim.shape[1], p.ctypes.data, x.ctypes.data)
        if rc:
            raise RuntimeError("refh_params2x: tables do not match the reference build")
        return x


class RefNM(RefHost):
    """The reference's own chi2_gpu simplex driver (cuda.c:1326-1833) run on the host
    (oracle/_ref/libref_nm_<variant>.so: the block's threads as host threads, cuRAND replaced by
    the engine's Philox stream, N_STEPS = 100 by the reference's -DTIMING switch)."""

    def __init__(self, variant: str):
        path = REF_DIR / f"libref_nm_{variant}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        lib = C.CDLL(str(path))
        V, I = C.c_void_p, C.c_int
        if hasattr(lib, "refnm_fit"):  # the -DRMSD builds hold refnm_rmsd instead
            lib.refnm_fit.restype = I
            lib.refnm_fit.argtypes = [V, I, V, I, V, I, C.c_float, C.c_float, I, I, V, V, V, V, V, V, V, V, V, I, V,
                                      V, I, V, I, I, C.c_ulonglong, V, V, V]
        for n in ("refnm_block_size", "refnm_n_params", "refh_n_params", "refh_n_types"):
            getattr(lib, n).restype = I
        lib.refnm_n_steps.restype = C.c_uint
        self.lib = lib
        self.n_params = lib.refh_n_params()
        self.n_types = lib.refh_n_types()
        self.block_size = lib.refnm_block_size()
        self.n_steps = lib.refnm_n_steps()

    def fit(self, m, obs, seed, n_blocks, n_stages=1, reopt=False, params0=None):
        """One chi2_gpu launch of n_blocks blocks: each block's best chi^2, parameters, delta_V."""
        prop, types, lim = self._tables(m)
        eph = [np.ascontiguousarray(a, dtype=np.float64) for a in (obs.eph_e, obs.eph_s, obs.eph_mjd0)]
        p0 = np.ascontiguousarray(params0 if params0 is not None else np.zeros(m.n_params), dtype=np.float64)
        bf = np.zeros(n_blocks)
        bp = np.zeros((n_blocks, m.n_params))
        bdv = np.zeros((n_blocks, obs.n_filters))
        rc = self.lib.refnm_fit(prop.ctypes.data, m.n_params, types.ctypes.data, m.n_types, lim.ctypes.data,
                                lim.shape[1], m.ppsi1, m.ppsi2, obs.n_data, obs.n_filters, obs.mjd.ctypes.data,
                                obs.v.ctypes.data, obs.w.ctypes.data, obs.filt.ctypes.data, obs.e_unit.ctypes.data,
                                obs.s_unit.ctypes.data, eph[0].ctypes.data, eph[1].ctypes.data, eph[2].ctypes.data,
                                int(obs.t_min.size), obs.t_min.ctypes.data, obs.v_min.ctypes.data, int(bool(reopt)),
                                p0.ctypes.data, int(n_blocks), int(n_stages), int(seed), bf.ctypes.data,
                                bp.ctypes.data, bdv.ctypes.data)
        if rc:
            raise RuntimeError(f"refnm_fit failed ({rc}): tables or sizes do not match the reference build")
        return {"best_f": bf, "best_params": bp, "best_dv": bdv}

    def rmsd(self, m, obs, params0, seed, call, n_blocks, samples, dx, reopt=1):
        """One chi2_gpu_rms launch (-DRMSD builds): f0 and f1 (float, as d_f0 / d_f1), the counts
        of evaluated and rejected points, and the parameter ranges over all blocks (float)."""
        lib = self.lib
        if not hasattr(lib, "refnm_rmsd"):
            raise RuntimeError("not a -DRMSD build")
        V, I = C.c_void_p, C.c_int
        lib.refnm_rmsd.restype = I
        lib.refnm_rmsd.argtypes = [V, I, V, I, V, I, I, I, V, V, V, V, V, V, V, V, V, I, V, I, I, C.c_float,
                                   C.c_ulonglong, C.c_uint, V, V, V, V]
        prop, types, lim = self._tables(m)
        eph = [np.ascontiguousarray(a, dtype=np.float64) for a in (obs.eph_e, obs.eph_s, obs.eph_mjd0)]
        p0 = np.ascontiguousarray(params0, dtype=np.float64)
        f01 = np.zeros(2)
        counts = np.zeros(2, np.int64)
        pmin = np.zeros(m.n_params, np.float32)
        pmax = np.zeros(m.n_params, np.float32)
        rc = lib.refnm_rmsd(prop.ctypes.data, m.n_params, types.ctypes.data, m.n_types, lim.ctypes.data, lim.shape[1],
                            obs.n_data, obs.n_filters, obs.mjd.ctypes.data, obs.v.ctypes.data, obs.w.ctypes.data,
                            obs.filt.ctypes.data, obs.e_unit.ctypes.data, obs.s_unit.ctypes.data, eph[0].ctypes.data,
                            eph[1].ctypes.data, eph[2].ctypes.data, int(reopt), p0.ctypes.data, int(n_blocks),
                            int(samples), float(dx), int(seed), int(call), f01.ctypes.data, counts.ctypes.data,
                            pmin.ctypes.data, pmax.ctypes.data)
        if rc:
            raise RuntimeError(f"refnm_rmsd failed ({rc}): tables or sizes do not match the reference build")
        return {"f0": f01[0], "f1": f01[1], "n_tot": int(counts[0]), "n_bad": int(counts[1]), "par_min": pmin,
                "par_max": pmax}


class RefRead:
    """The reference's own host readers, read_data() (read_data.c:6-377) and, under NUDGE,
    prepare_chi2_params() (misc.c:279-323), built from its sources
    (oracle/_ref/libref_read_<variant>.so: plain, interp, interp_nudge)."""

    def __init__(self, variant: str):
        path = REF_DIR / f"libref_read_{variant}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        self.lib = C.CDLL(str(path))
        self.lib.refr_read.restype = C.c_int
        self.lib.refr_read.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int] + [C.c_void_p] * 17

    def read(self, directory, lc_file: str, nplot: int = 0, n_max: int = 16384):
        """Everything read_data (and prepare_chi2_params) leave behind, run in `directory`."""
        n = np.zeros(2, np.int32)
        filters = C.create_string_buffer(16)
        mjd, e, s = np.zeros(n_max), np.zeros(3 * n_max), np.zeros(3 * n_max)
        v, w = np.zeros(n_max, np.float32), np.zeros(n_max, np.float32)
        filt = np.zeros(n_max, np.int32)
        hmjd0 = np.zeros(1)
        eph = np.zeros(21)
        pt, pe, ps = np.zeros(max(nplot, 1)), np.zeros(3 * max(nplot, 1)), np.zeros(3 * max(nplot, 1))
        n_min = np.zeros(1, np.int32)
        t_min, v_min = np.zeros(16, np.float32), np.zeros(16, np.float32)
        rc = self.lib.refr_read(str(directory).encode(), lc_file.encode(), int(n_max), int(nplot),
                                n[0:].ctypes.data, n[1:].ctypes.data, C.cast(filters, C.c_void_p), mjd.ctypes.data,
                                v.ctypes.data, w.ctypes.data, filt.ctypes.data, e.ctypes.data, s.ctypes.data,
                                hmjd0.ctypes.data, eph.ctypes.data, pt.ctypes.data, pe.ctypes.data, ps.ctypes.data,
                                n_min.ctypes.data, t_min.ctypes.data, v_min.ctypes.data)
        if rc:
            raise RuntimeError(f"refr_read failed ({rc})")
        nd, nf = int(n[0]), int(n[1])
        return {"mjd": mjd[:nd], "v": v[:nd], "w": w[:nd], "filt": filt[:nd], "e_unit": e[: 3 * nd],
                "s_unit": s[: 3 * nd], "filters": filters.raw[:nf].decode(), "hmjd0": float(hmjd0[0]),
                "eph_e": eph[0:9].reshape(3, 3), "eph_s": eph[9:18].reshape(3, 3), "eph_mjd0": eph[18:21],
                "plot_t": pt[:nplot], "plot_e": pe[: 3 * nplot].reshape(-1, 3), "plot_s": ps[: 3 * nplot].reshape(-1, 3),
                "t_min": t_min[: int(n_min[0])], "v_min": v_min[: int(n_min[0])]}


def ref_render(geo):
    """The reference's own compute_rgb on the GPU (oracle/_ref/ref_animate.cubin), 1080 x 1080."""
    cubin = REF_DIR / "ref_animate.cubin"
    if not cubin.exists():
        raise FileNotFoundError(cubin)
    lib = C.CDLL(str(HERE / "_build" / "libref_gpu_loader.so"))
    lib.refk_render.restype = C.c_int
    lib.refk_last_error.restype = C.c_char_p
    g = np.ascontiguousarray(geo, dtype=np.float64).reshape(-1, 20)
    rgb = np.zeros((g.shape[0], 1080, 1080, 3), np.uint8)
    rc = lib.refk_render(str(cubin).encode(), C.c_void_p(g.ctypes.data), int(g.shape[0]), C.c_void_p(rgb.ctypes.data))
    if rc:
        raise RuntimeError(lib.refk_last_error().decode())
    return rgb


class RefKernel:
    """The reference's own chi2one on the GPU (oracle/_ref/ref_<variant>.cubin, sm_100)."""

    def __init__(self, variant: str):
        self.cubin = REF_DIR / f"ref_{variant}.cubin"
        if not self.cubin.exists():
            raise FileNotFoundError(self.cubin)
        lib = C.CDLL(str(HERE / "_build" / "libref_gpu_loader.so"))
        lib.refk_eval_batch.restype = C.c_int
        lib.refk_last_error.restype = C.c_char_p
        self.lib = lib

    def chi2_batch(self, model, obs, params):
        from asteroid_gb300 import capi
        P = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        n = P.shape[0]
        types = np.ctypeslib.as_array(model.types)[: model.n_types].astype(np.int32).copy()
        eph = np.concatenate([np.asarray(obs.eph_e).ravel(), np.asarray(obs.eph_s).ravel(),
                              np.asarray(obs.eph_mjd0).ravel()]).astype(np.float64)
        obs_bytes = 24 if model.flags & capi.INTERP else 72
        chi2 = np.zeros(n)
        dv = np.zeros((n, obs.n_filters))
        V = C.c_void_p
        ms = C.c_double(0)
        rc = self.lib.refk_eval_batch(
            str(self.cubin).encode(), obs_bytes, model.n_params, V(P.ctypes.data), n, V(types.ctypes.data),
            model.n_types, obs.n_data, obs.n_filters, V(obs.mjd.ctypes.data), V(obs.v.ctypes.data),
            V(obs.w.ctypes.data), V(obs.filt.ctypes.data), V(obs.e_unit.ctypes.data), V(obs.s_unit.ctypes.data),
            V(eph.ctypes.data), int(obs.t_min.size), V(obs.t_min.ctypes.data), V(obs.v_min.ctypes.data),
            V(chi2.ctypes.data), V(dv.ctypes.data), C.byref(ms))
        if rc:
            raise RuntimeError(self.lib.refk_last_error().decode())
        self.last_ms = ms.value  # device time of the evaluation launch
        return chi2, dv
