"""Philox4x32-10 known answers and the simplex driver's semantics on the CPU oracle."""
import numpy as np
import pytest

# Published known-answer vectors of Philox4x32-10 (Salmon et al. 2011, Random123 kat_vectors).
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,out", KAT)
def test_philox_known_answers(oracle_mod, ctr, key, out):
    assert list(oracle_mod.philox(ctr, key)) == out


def test_uniform_open_interval_and_mean(oracle_mod):
    u = np.array([oracle_mod.uniform(5, c, 0, k) for c in range(64) for k in range(64)])
    assert u.min() > 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.02
    # distinct streams per chain and stage
    assert oracle_mod.uniform(5, 1, 0, 0) != oracle_mod.uniform(5, 2, 0, 0)
    assert oracle_mod.uniform(5, 1, 0, 0) != oracle_mod.uniform(5, 1, 1, 0)


def test_group_best_and_ties(oracle_mod, synth_objects):
    s = synth_objects("c0acc")
    r = oracle_mod.fit(s.model, s.obs, seed=3, n_chains=64, group_size=16, evals_cap=30)
    cf = r["chain_f"].reshape(4, 16)
    assert np.array_equal(r["best_f"], np.min(np.where(np.isfinite(cf), cf, np.inf), axis=1))
    assert r["n_evals"] >= 64 * 12


def test_stage_handoff_improves_or_keeps(oracle_mod, synth_objects):
    s = synth_objects("c0acc")
    one = oracle_mod.fit(s.model, s.obs, seed=4, n_chains=32, group_size=32, n_stages=1, evals_cap=40)
    two = oracle_mod.fit(s.model, s.obs, seed=4, n_chains=32, group_size=32, n_stages=2, evals_cap=40)
    # Stage 2 restarts every chain near the stage-1 best (DX_RAND jitter): it cannot be far worse.
    assert two["best_f"][0] <= one["best_f"][0] * 1.5


def test_reopt_from_truth_stays_near_truth(oracle_mod, synth_objects):
    s = synth_objects("c0acc")
    r = oracle_mod.fit(s.model, s.obs, seed=5, n_chains=16, group_size=16, reopt=True, params0=s.params_true,
                       evals_cap=100)
    c_true, _ = oracle_mod.chi2(s.model, s.obs, s.params_true)
    assert r["best_f"][0] <= c_true * 1.05
    assert np.allclose(r["best_params"][0][:3], s.params_true[:3], atol=0.05)
