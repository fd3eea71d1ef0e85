"""ast_fit_noalloc: the fit for callers that cannot allocate device memory.

Some callers of this library may not call cudaMalloc: a host framework that hands out every
device allocation from its own pool, or a service that reserves its device memory at start-up
and must not grow it.  For them ast_fit_noalloc takes device inputs and outputs from the caller
and keeps its working state in a fixed device array inside the library.  These tests call it
through the C ABI twice in a row (the array keeps the previous call's contents, so the second
call checks that the entry point re-initialises what it must) and require both results to equal
those of ast_fit, which allocates its own buffers, to 1e-12 relative (the launch geometry is the
same, so in practice the results are equal bit for bit).

Covered: both precisions, random starts and -reopt starts from a model, the mixed search with
FP64 results, an INTERP + NUDGE object, observation blocks staged in shared memory above 48 KB
(480 points), blocks too large to stage (2000 points) and the array's largest object (4096
points, E/S vectors from the caller).  The last three run in a fresh process whose first fit is
ast_fit_noalloc, so nothing set up by an earlier ast_fit can hide a missing launch attribute.
"""
import ctypes as C
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if __name__ == "__main__":
    for p in (str(ROOT), str(ROOT / "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)

from asteroid_gb300 import api, capi  # noqa: E402

RTOL = 1e-12


def _noalloc(s, n_chains, group, stages, seed, cap, precision, reopt=False, fp64_result=False):
    """One ast_fit_noalloc call on the object `s` with torch device buffers; host results."""
    import torch

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
    cfg, _keep = api.fit_cfg(n_chains=n_chains, group_size=group, seed=seed, reopt=reopt,
                             params0=s.params_true if reopt else None, precision=precision, evals_cap=cap,
                             n_stages=stages, fp64_result=fp64_result)
    bf = torch.full((G,), float("nan"), dtype=torch.float64, device=dev)
    bp = torch.full((G, N), float("nan"), dtype=torch.float64, device=dev)
    bdv = torch.full((G, NF), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.ast_fit_noalloc(C.byref(s.model), C.byref(cobs), d_mjd.data_ptr(), d_v.data_ptr(), d_w.data_ptr(),
                             d_f.data_ptr(), d_e.data_ptr(), d_s.data_ptr(), C.byref(cfg), bf.data_ptr(),
                             bp.data_ptr(), bdv.data_ptr(), None)
    assert rc == 0, lib.ast_last_error()
    torch.cuda.synchronize()
    return bf.cpu().numpy(), bp.cpu().numpy(), bdv.cpu().numpy()


def _fit(s, n_chains, group, stages, seed, cap, precision, reopt=False, fp64_result=False):
    with api.Engine(s.model, s.obs) as eng:
        return eng.fit(n_chains=n_chains, group_size=group, n_stages=stages, seed=seed, evals_cap=cap,
                       precision=precision, reopt=reopt, params0=s.params_true if reopt else None,
                       fp64_result=fp64_result)


def _same(got, ref, what):
    f, p, dv = got
    assert np.allclose(f, ref.best_f, rtol=RTOL, atol=0), (what, f, ref.best_f)
    assert np.allclose(p, ref.best_params, rtol=RTOL, atol=1e-300), what
    assert np.allclose(dv, ref.best_dv, rtol=RTOL, atol=1e-300), what


CASES = [
    # (object, chains, group, stages, seed, evals cap, precision, reopt, fp64_result)
    ("c0acc", 1024, 256, 2, 21, 60, api.PREC_FP64, False, False),
    ("c0acc", 1024, 256, 2, 22, 60, api.PREC_MIXED, False, False),
    ("c0acc", 512, 128, 1, 23, 60, api.PREC_FP64, True, False),
    ("c0acc", 512, 128, 2, 24, 60, api.PREC_MIXED, True, True),
    ("c2", 256, 128, 2, 25, 12, api.PREC_MIXED, False, True),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{'mixed' if c[6] == api.PREC_MIXED else 'fp64'}"
                                             f"-reopt{int(c[7])}-fp64res{int(c[8])}" for c in CASES])
def test_noalloc_fit_matches_fit_on_two_calls(gpu, synth_objects, case):
    name, n_chains, group, stages, seed, cap, prec, reopt, fp64_res = case
    s = synth_objects(name)
    ref = _fit(s, n_chains, group, stages, seed, cap, prec, reopt, fp64_res)
    for call in range(2):
        _same(_noalloc(s, n_chains, group, stages, seed, cap, prec, reopt, fp64_res), ref, (name, call))


@pytest.mark.gpu
def test_noalloc_first_call_in_a_fresh_process(gpu):
    """480 points (block staged in shared memory, 65 KB), 2000 points with INTERP + NUDGE (read
    through L1) and 4096 points (the array's maximum): ast_fit_noalloc is the process's first fit."""
    r = subprocess.run([sys.executable, str(Path(__file__).resolve()), "fresh"], cwd=str(ROOT),
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=900)
    print(r.stdout[-4000:])
    assert r.returncode == 0, r.stdout[-4000:]


@pytest.mark.gpu
def test_noalloc_rejects_sizes_beyond_its_array(gpu, synth_objects):
    s = synth_objects("c0acc")
    lib = capi.load()
    cobs = s.obs.as_c()
    cfg, _ = api.fit_cfg(n_chains=8192, group_size=256, seed=1, evals_cap=10)
    rc = lib.ast_fit_noalloc(C.byref(s.model), C.byref(cobs), 1, 1, 1, 1, 1, 1, C.byref(cfg), 1, 1, 1, None)
    assert rc == -5 and b"n_chains" in lib.ast_last_error()


def _fresh_process_main() -> int:
    import oracle
    from asteroid_gb300 import synth

    oracle.load()
    big = synth.SynthConfig("n4096", "TORQUE,P_PSI,ACC", 1e-2, 4096, 2, 6, 6, seed=1005, filter_chars="RV",
                            dv_range=0.5)
    runs = [("c1", api.PREC_FP64, False), ("c1", api.PREC_MIXED, True), ("c2", api.PREC_MIXED, True),
            (big, api.PREC_FP64, False)]
    with tempfile.TemporaryDirectory() as d:
        objs = {}
        for cfg, prec, fp64_res in runs:
            key = cfg if isinstance(cfg, str) else cfg.name
            if key not in objs:
                objs[key] = synth.generate(cfg, Path(d) / key, vmod_fn=lambda m, o, p: oracle.model_curve(m, o, p))
            s = objs[key]
            n_chains, group, stages, seed, cap = 256, 128, 2, 31, 10
            first = _noalloc(s, n_chains, group, stages, seed, cap, prec, False, fp64_res)
            ref = _fit(s, n_chains, group, stages, seed, cap, prec, False, fp64_res)
            second = _noalloc(s, n_chains, group, stages, seed, cap, prec, False, fp64_res)
            _same(first, ref, (key, "first"))
            _same(second, ref, (key, "second"))
            print(f"{key} ({s.obs.n_data} points, {'mixed' if prec == api.PREC_MIXED else 'fp64'}): "
                  f"best {ref.best_f.min():.6f}, equal to ast_fit on two calls")
    return 0


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "fresh":
    sys.exit(_fresh_process_main())
