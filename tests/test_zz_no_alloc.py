"""ast_fit_noalloc: the fit for callers that cannot allocate device memory.

Some callers of this library may not call cudaMalloc: a host framework that hands out every
device allocation from its own pool, or a service that reserves its device memory at start-up
and must not grow it.  For them ast_fit_noalloc takes device inputs and outputs from the caller
and keeps its working state in a fixed device array inside the library.  This test calls it
through the C ABI twice in a row (the array keeps the previous call's contents, so the second
call checks that the entry point re-initialises what it must) and requires both results to equal
those of ast_fit, which allocates its own buffers, to the tolerance the other fit tests use.
"""
import ctypes as C

import numpy as np
import pytest

from asteroid_gb300 import api, capi

pytestmark = pytest.mark.gpu


def _cfg(n_chains, group, stages, seed, cap, precision=api.PREC_FP64):
    cfg = capi.FitCfg()
    cfg.seed = seed
    cfg.n_chains = n_chains
    cfg.group_size = group
    cfg.n_stages = stages
    cfg.reopt = 0
    cfg.precision = precision
    cfg.evals_cap = cap
    cfg.steps_cap = 0
    cfg.tpb = 0
    return cfg


def test_noalloc_fit_matches_fit_on_two_calls(gpu, synth_objects):
    import torch

    s = synth_objects("c0acc")
    n_chains, group, stages, seed, cap = 1024, 256, 2, 21, 60
    with api.Engine(s.model, s.obs) as eng:
        ref = eng.fit(n_chains=n_chains, group_size=group, n_stages=stages, seed=seed, evals_cap=cap)
    dev = torch.device("cuda:0")
    o = s.obs
    d_mjd = torch.from_numpy(o.mjd).to(dev)
    d_v = torch.from_numpy(o.v).to(dev)
    d_w = torch.from_numpy(o.w).to(dev)
    d_f = torch.from_numpy(o.filt).to(dev)
    d_e = torch.from_numpy(o.e_unit.ravel().copy()).to(dev)
    d_s = torch.from_numpy(o.s_unit.ravel().copy()).to(dev)
    G, N, NF = n_chains // group, s.model.n_params, o.n_filters
    lib = capi.load()
    cobs = o.as_c()
    cfg = _cfg(n_chains, group, stages, seed, cap)
    for call in range(2):
        bf = torch.full((G,), float("nan"), dtype=torch.float64, device=dev)
        bp = torch.full((G, N), float("nan"), dtype=torch.float64, device=dev)
        bdv = torch.full((G, NF), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = lib.ast_fit_noalloc(C.byref(s.model), C.byref(cobs), d_mjd.data_ptr(), d_v.data_ptr(), d_w.data_ptr(),
                                 d_f.data_ptr(), d_e.data_ptr(), d_s.data_ptr(), C.byref(cfg), bf.data_ptr(),
                                 bp.data_ptr(), bdv.data_ptr(), None)
        assert rc == 0, lib.ast_last_error()
        torch.cuda.synchronize()
        got_f, got_p, got_dv = bf.cpu().numpy(), bp.cpu().numpy(), bdv.cpu().numpy()
        assert np.allclose(got_f, ref.best_f, rtol=1e-12, atol=0), (call, got_f, ref.best_f)
        assert np.allclose(got_p, ref.best_params, rtol=1e-12, atol=1e-300), call
        assert np.allclose(got_dv, ref.best_dv, rtol=1e-12, atol=1e-300), call


def test_noalloc_rejects_sizes_beyond_its_array(gpu, synth_objects):
    s = synth_objects("c0acc")
    lib = capi.load()
    cobs = s.obs.as_c()
    cfg = _cfg(8192, 256, 1, 1, 10)
    rc = lib.ast_fit_noalloc(C.byref(s.model), C.byref(cobs), 1, 1, 1, 1, 1, 1, C.byref(cfg), 1, 1, 1, None)
    assert rc == -5 and b"n_chains" in lib.ast_last_error()
