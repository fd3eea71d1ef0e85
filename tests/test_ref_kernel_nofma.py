"""FP64 parity with the reference kernel when neither side contracts multiply-adds.

The default builds of both the engine and the reference's cuda.c let nvcc fuse a*b + c into one
rounding wherever it likes, and the two programs' choices differ, so their FP64 chi^2 differ in
the last bits (tests/test_ref_kernel.py bounds that by each vector's own rounding sensitivity).
Built with nvcc -fmad=false -- the engine's evaluation kernels (build.build_parity_engine) and
the reference's cuda.c for every fixture variant (oracle/_ref/ref_<variant>_nofma.cubin) -- both
sides round every product and sum separately in the reference's operation order, with the same
CUDA libm.  Then every well-conditioned vector must agree within 1e-12 relative chi^2; the
bit-identical fraction is printed.  Besides the resolved-rotation sample (h*L <= 0.5) each
variant gets an unresolved one (h*L up to 7, the rest of the L prior at asteroid.c:479-480):
finite and non-finite results must coincide, and where both are finite and well conditioned
the 1e-12 bar holds too.

The parity library is loaded in a child process (AST_ENGINE_LIB), so that it never shares a
process with the default build.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
REF = ROOT / "oracle" / "_ref"
RTOL = 1e-12
N_RESOLVED = 256
N_UNRESOLVED = 128


@pytest.mark.gpu
def test_fp64_without_contraction_matches_reference_kernel(gpu):
    from asteroid_gb300 import build

    if not list(REF.glob("ref_*_nofma.cubin")):
        pytest.skip("ref_*_nofma.cubin not built (needs the reference checkout where the tree was prepared)")
    lib = build.build_parity_engine()
    env = dict(os.environ, AST_ENGINE_LIB=str(lib))
    r = subprocess.run([sys.executable, str(Path(__file__).resolve()), "run"], cwd=str(ROOT), env=env,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=1200)
    print(r.stdout[-6000:])
    assert r.returncode == 0, r.stdout[-6000:]
    stats = json.loads(r.stdout.strip().splitlines()[-1])
    assert len(stats) >= 8
    for variant, st in stats.items():
        for sample in ("resolved", "unresolved"):
            s = st[sample]
            assert s["finite_mismatch"] == 0, (variant, sample, s)
            assert s["max_rel"] <= RTOL, (variant, sample, s)
        assert st["resolved"]["compared"] >= 0.5 * N_RESOLVED, (variant, st)


def _child() -> int:
    sys.path[:0] = [str(ROOT), str(ROOT / "oracle")]
    import oracle

    from asteroid_gb300 import api, capi
    from tests.test_gpu_eval import well_conditioned
    from tests.test_oracle_pin import load_fixture

    oracle.load()
    assert str(capi.lib_path()) == os.environ["AST_ENGINE_LIB"]
    out = {}
    for path in sorted(GOLDEN.glob("ref_*.json")):
        fx, m, obs = load_fixture(path)
        variant = fx["variant"]
        cubin = REF / f"ref_{variant}_nofma.cubin"
        if not cubin.exists():
            continue
        rk = oracle.RefKernel(f"{variant}_nofma")
        iL = api.param_names(m).index("L")
        rng = np.random.default_rng(29)
        res, unres = [np.array(p) for p in fx["params"]], []
        while len(res) < N_RESOLVED or len(unres) < N_UNRESOLVED:
            p = api.x2params(m, rng.uniform(0, 1, m.n_params), reopt=0)
            if p is None:
                continue
            hl = p[iL] * m.time_step
            if hl <= 0.5 and len(res) < N_RESOLVED:
                res.append(p)
            elif 0.5 < hl <= 7.0 and len(unres) < N_UNRESOLVED:
                unres.append(p)
        st = {}
        with api.Engine(m, obs) as eng:
            for name, P in (("resolved", np.array(res)), ("unresolved", np.array(unres))):
                ref, ref_dv = rk.chi2_batch(m, obs, P)
                got, dv = eng.eval(P, api.PREC_FP64)
                good = well_conditioned(oracle, m, obs, P)
                fin_r, fin_g = np.isfinite(ref) & (ref < 1e29), np.isfinite(got) & (got < 1e29)
                both = good & fin_r & fin_g
                rel = np.abs(got[both] - ref[both]) / np.abs(ref[both])
                dv_rel = (np.abs(dv[both] - ref_dv[both]) / np.maximum(np.abs(ref_dv[both]), 1e-300)).max() \
                    if both.any() else 0.0
                st[name] = {"vectors": len(P), "compared": int(both.sum()),
                            "finite_mismatch": int(np.sum(fin_r != fin_g)),
                            "max_rel": float(rel.max()) if rel.size else 0.0,
                            "frac_le_1e-12": float(np.mean(rel <= RTOL)) if rel.size else 1.0,
                            "bit_identical": float(np.mean((got == ref) | (np.isnan(got) & np.isnan(ref)))),
                            "max_rel_dv": float(dv_rel)}
                print(f"{variant} {name}: {st[name]}", flush=True)
        out[variant] = st
    print(json.dumps(out))
    return 0


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "run":
    sys.exit(_child())
