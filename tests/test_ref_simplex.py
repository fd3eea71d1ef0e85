"""The simplex search against the reference's own chi2_gpu, by best-chi^2 distributions.

oracle/_ref/ref_nm_ppsi_torque_acc.cubin is the reference's cuda.c (-DP_PSI -DTORQUE -DACC)
compiled for sm_100 from its sources (oracle/build_ref.sh).  oracle/ref_gpu_loader.cpp runs its
setup_kernel + chi2_gpu (cuda.c:2039, cuda.c:1326) unmodified but for three hooks: N_STEPS set
per run, a per-thread count of chi2one calls, and every chain's final chi^2.  ast_fit runs the
same object (config 0: 300 points, LS + TORQUE + P_PSI, FP64 simplex) with the same chain count,
the same group size and the same iteration cap.

The two draw their random starts from different generators (cuRAND XORWOW there, Philox here)
and their chi^2 differ in the last bits, so trajectories diverge; what must agree is the
distribution of outcomes.  At each seed, on 4096 chains per side, the test requires
  * two-sample Kolmogorov-Smirnov p > 1e-3 for the chains' final chi^2 (failed chains, 1e30,
    compared separately: their fractions within 4 standard errors);
  * the 10/50/90% quantiles of one side to sit at the same quantile of the other side within
    4 standard errors of an empirical quantile, sqrt(p(1-p)(1/n1 + 1/n2));
  * KS p > 1e-3 for the group bests (the reference's block bests; groups of 4 chains);
  * evaluations per chain within 5% of each other.
The same checks are pooled over the seeds at the end.

Sizes.  4096 chains, the config-0 chain count.  With one stage a chain's outcome does not
depend on its block, so the reference's chains run as 1024 blocks of 4 threads and the groups
(block bests) here are groups of 4: one FP64 warp per SM is latency-bound on this GPU (about
200 ms per reference chi2one of this object with a single warp), and the reference kernel's 30 KB
of static shared memory allows at most 7 blocks per SM, so small blocks are what spreads its
chains over the SMs.  The iteration cap is N_STEPS = 100 (about 160 evaluations per chain):
config 0's 2000 evaluations per chain take the reference kernel about two minutes per seed even
so.  AST_REF_SIMPLEX_STEPS sets another cap for a longer run.
"""
import os

import numpy as np
import pytest

from asteroid_gb300 import api

pytestmark = pytest.mark.gpu

N_CHAINS = 4096
BLOCK = 4
N_STEPS = int(os.environ.get("AST_REF_SIMPLEX_STEPS", "100"))  # simplex iterations per chain
SEEDS = (101, 202)
P_MIN = 1e-3
FAILED = 1e29


def _ks(a, b):
    from scipy.stats import ks_2samp

    return ks_2samp(a, b).pvalue


def _quantiles_agree(a, b, qs=(0.1, 0.5, 0.9), k=4.0):
    """Every q-quantile of a sits at the q-quantile of b (and vice versa) within k standard
    errors of an empirical quantile, measured in probability."""
    out = []
    for q in qs:
        se = np.sqrt(q * (1 - q) * (1 / len(a) + 1 / len(b)))
        qa, qb = np.quantile(a, q), np.quantile(b, q)
        fa, fb = np.mean(b <= qa), np.mean(a <= qb)
        out.append((q, qa, qb, abs(fa - q) <= k * se and abs(fb - q) <= k * se))
    return out


def _compare(label, ours_chain, ref_chain, ours_best, ref_best, ours_evals, ref_evals):
    ok_o, ok_r = ours_chain < FAILED, ref_chain < FAILED
    fo, fr = 1 - ok_o.mean(), 1 - ok_r.mean()
    se = np.sqrt(max(fo * (1 - fo), fr * (1 - fr), 1e-6) * (1 / ok_o.size + 1 / ok_r.size))
    p_chain = _ks(ours_chain[ok_o], ref_chain[ok_r])
    p_best = _ks(ours_best[ours_best < FAILED], ref_best[ref_best < FAILED])
    qs = _quantiles_agree(ours_chain[ok_o], ref_chain[ok_r])
    print(f"{label}: chains KS p={p_chain:.3g}, group bests KS p={p_best:.3g}, failed {fo:.4f} vs {fr:.4f}, "
          "quantiles " + ", ".join(f"{int(q * 100)}%: {a:.4f} vs {b:.4f}" for q, a, b, _ in qs)
          + f"; evals/chain {ours_evals:.1f} vs {ref_evals:.1f}; best {ours_best.min():.5f} vs {ref_best.min():.5f}")
    assert abs(fo - fr) <= 4 * se, (label, fo, fr)
    assert p_chain > P_MIN, (label, p_chain)
    assert p_best > P_MIN, (label, p_best)
    assert all(q[3] for q in qs), (label, qs)
    assert abs(ours_evals / ref_evals - 1) < 0.05, (label, ours_evals, ref_evals)


def test_simplex_distribution_matches_reference_chi2_gpu(gpu, oracle_mod, synth_objects):
    s = synth_objects("c0acc")
    try:
        ref = oracle_mod.RefSimplex("ppsi_torque_acc")
    except FileNotFoundError as e:
        pytest.skip(f"{e} not built (needs the reference checkout where the tree was prepared)")
    pooled = {k: [] for k in ("oc", "rc", "ob", "rb")}
    ev_o = ev_r = 0.0
    with api.Engine(s.model, s.obs) as eng:
        for seed in SEEDS:
            r = ref.fit(s.model, s.obs, seed=seed, n_blocks=N_CHAINS // BLOCK, block=BLOCK, n_stages=1,
                        n_steps=N_STEPS)
            o = eng.fit(n_chains=N_CHAINS, group_size=BLOCK, n_stages=1, seed=seed, steps_cap=N_STEPS,
                        precision=api.PREC_FP64)
            # The reference's block best is its chains' minimum (cuda.c:1770-1782, 1810-1823).
            assert np.array_equal(r["best_f"], np.minimum(r["chain_f"][0].reshape(-1, BLOCK).min(axis=1), 1e30))
            assert np.array_equal(o.best_f, np.minimum(o.chain_f.reshape(-1, BLOCK).min(axis=1), 1e30))
            ref_evals = r["evals"].mean()
            print(f"seed {seed}: reference chi2_gpu {r['kernel_ms'] / 1e3:.2f} s, ast_fit {o.kernel_ms / 1e3:.3f} s; "
                  f"iterations at the cap: {np.mean(r['chain_l'][0] > N_STEPS):.3f} of the reference's chains")
            _compare(f"seed {seed}", o.chain_f, r["chain_f"][0], o.best_f, r["best_f"], o.n_evals / N_CHAINS,
                     ref_evals)
            pooled["oc"].append(o.chain_f)
            pooled["rc"].append(r["chain_f"][0])
            pooled["ob"].append(o.best_f)
            pooled["rb"].append(r["best_f"])
            ev_o += o.n_evals / N_CHAINS / len(SEEDS)
            ev_r += ref_evals / len(SEEDS)
    _compare("pooled", *(np.concatenate(pooled[k]) for k in ("oc", "rc", "ob", "rb")), ev_o, ev_r)
