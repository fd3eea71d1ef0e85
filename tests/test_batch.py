"""Batched fits (ast_batch_*) and served fits (ast_server_*, ast_submit, ast_poll).

Every object of a batch, and every request of a server, must come out exactly as a
single-object ast_fit with the same model, observations and configuration: the chain's random
draws are keyed by the object's seed and the chain's index within the object, and the
evaluation is the same code, so neither the other objects in flight, nor the slot a chain runs
on, nor the refill mapping may change a result.
"""
import numpy as np
import pytest

from asteroid_gb300 import api

pytestmark = pytest.mark.gpu

OBJECTS = ["c3_0", "c3_1", "c3_2", "c3_3", "c0acc"]
CFG = dict(n_chains=256, group_size=64, seed=7, evals_cap=40)


def single(s, precision, seed):
    with api.Engine(s.model, s.obs) as eng:
        return eng.fit(n_chains=CFG["n_chains"], group_size=CFG["group_size"], n_stages=1, seed=seed,
                       evals_cap=CFG["evals_cap"], precision=precision)


def same(a, b):
    assert np.array_equal(a.best_f, b.best_f), (a.best_f, b.best_f)
    assert np.array_equal(a.best_params, b.best_params)
    assert np.array_equal(a.best_dv, b.best_dv)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_batch_objects_equal_single_fits(gpu, synth_objects, precision):
    objs = [synth_objects(n) for n in OBJECTS]
    with api.Batch(precision=precision, acc=True, n_slots=152 * 64) as b:
        idx = [b.add(s.model, s.obs, **dict(CFG, seed=CFG["seed"] + k)) for k, s in enumerate(objs)]
        b.run()
        got = [b.result(i) for i in idx]
        c = b.counters()
        assert c["n_fits"] == len(objs) * CFG["n_chains"]
    for k, s in enumerate(objs):
        same(got[k], single(s, precision, CFG["seed"] + k))


def test_batch_refill_and_geometry_do_not_change_results(gpu, synth_objects):
    objs = [synth_objects(n) for n in OBJECTS[:4]]
    res = []
    for tpb, refill in ((256, 1), (64, 32), (128, 32)):
        with api.Batch(precision=api.PREC_MIXED, acc=True, n_slots=152 * 32) as b:
            for k, s in enumerate(objs):
                b.add(s.model, s.obs, **dict(CFG, seed=3 + k))
            b.run(tpb=tpb, refill=refill)
            assert b.counters()["refill"] == refill
            res.append([b.result(i) for i in range(len(objs))])
    for r in res[1:]:
        for a, b_ in zip(res[0], r):
            same(a, b_)


def test_batch_tuner_picks_a_measured_candidate(gpu, synth_objects):
    objs = [synth_objects(n) for n in OBJECTS[:3]]
    with api.Batch(precision=api.PREC_MIXED, acc=True) as b:
        for k, s in enumerate(objs):
            b.add(s.model, s.obs, **dict(CFG, seed=11 + k))
        t = b.tune(evals_per_slot=2)
        assert t["tpb"] in (64, 128, 256) and t["refill"] in (1, 32) and t["evals_per_s"] > 0
        b.run()
        assert all(np.all(np.isfinite(b.result(i).best_f)) for i in range(3))


def test_server_request_alone_equals_request_in_mix(gpu, synth_objects):
    a, others = synth_objects("c3_3"), [synth_objects(n) for n in ("c3_0", "c3_1", "c3_2")]
    cfg_a = dict(CFG, seed=99)
    with api.Server(precision=api.PREC_MIXED, acc=True, n_slots=152 * 64) as srv:
        r = srv.submit(a.model, a.obs, **cfg_a)
        while srv.poll(r) is None:
            srv.step(8)
        alone, _ = srv.poll(r)
    with api.Server(precision=api.PREC_MIXED, acc=True, n_slots=152 * 64) as srv:
        ids = [srv.submit(s.model, s.obs, **dict(CFG, seed=20 + k)) for k, s in enumerate(others)]
        srv.step(4)
        srv.step(4)
        r = srv.submit(a.model, a.obs, **cfg_a)  # arrives while the others run
        while any(srv.poll(i) is None for i in ids + [r]):
            srv.step(8)
        mixed, lat = srv.poll(r)
        assert lat > 0
        in_mix_others = [srv.poll(i)[0] for i in ids]
    same(alone, mixed)
    same(alone, single(a, api.PREC_MIXED, 99))
    for k, s in enumerate(others):
        with api.Engine(s.model, s.obs) as eng:
            ref = eng.fit(n_chains=CFG["n_chains"], group_size=CFG["group_size"], seed=20 + k,
                          evals_cap=CFG["evals_cap"], precision=api.PREC_MIXED)
        same(in_mix_others[k], ref)


def test_server_admits_by_hbm_budget(gpu, synth_objects):
    s = synth_objects("c3_1")
    with api.Server(precision=api.PREC_FP64, acc=True, n_slots=152 * 32, hbm_budget=1) as srv:
        with pytest.raises(api.capi.AstError):
            srv.submit(s.model, s.obs, **CFG)  # larger than the whole budget
    # Three requests of the same footprint; the budget holds one and a half: one runs at a time
    # and the others wait in arrival order.
    with api.Server(precision=api.PREC_FP64, acc=True, n_slots=152 * 32, hbm_budget=1 << 40) as probe:
        need = probe.request_bytes(probe.submit(s.model, s.obs, **CFG))
    budget = need + need // 2
    with api.Server(precision=api.PREC_FP64, acc=True, n_slots=152 * 32, hbm_budget=budget) as srv:
        ids = [srv.submit(s.model, s.obs, **dict(CFG, seed=5 + k)) for k in range(3)]
        running, queued = srv.step(4)
        assert running == 1 and queued == 2
        peak = 0
        while any(srv.poll(i) is None for i in ids):
            running, queued = srv.step(16)
            st = srv.stats()
            peak = max(peak, st["hbm_used"])
            assert st["hbm_used"] <= st["hbm_budget"] and running <= 1
        for k, i in enumerate(ids):
            same(srv.poll(i)[0], single(s, api.PREC_FP64, 5 + k))


def test_fp64_results_of_a_mixed_fit(gpu, synth_objects):
    """fp64_result: each group's reported chi^2 is the plain path's chi^2 at the group's best
    parameters, the same alone (ast_fit) and in a batch, and the search stays the mixed one."""
    objs = [synth_objects(n) for n in ("c3_0", "c3_2")]
    with api.Batch(precision=api.PREC_MIXED, acc=True, n_slots=152 * 32) as b:
        for k, s in enumerate(objs):
            b.add(s.model, s.obs, **dict(CFG, seed=40 + k), fp64_result=True)
        b.run()
        got = [b.result(i) for i in range(len(objs))]
    for k, s in enumerate(objs):
        with api.Engine(s.model, s.obs) as eng:
            plain = eng.fit(n_chains=CFG["n_chains"], group_size=CFG["group_size"], seed=40 + k,
                            evals_cap=CFG["evals_cap"], precision=api.PREC_MIXED)
            pol = eng.fit(n_chains=CFG["n_chains"], group_size=CFG["group_size"], seed=40 + k,
                          evals_cap=CFG["evals_cap"], precision=api.PREC_MIXED, fp64_result=True)
            c64, _ = eng.eval(pol.best_params, api.PREC_FP64)
        same(got[k], pol)
        assert np.array_equal(pol.best_params, plain.best_params)  # same search
        ok = pol.best_f < 1e29
        assert ok.any() and np.allclose(pol.best_f[ok], c64[ok], rtol=1e-12, atol=0)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_cooperative_chains_equal_single_fits(gpu, synth_objects, precision):
    """Four lanes per chain (ast_server_set_lanes) evaluate the candidate points of each simplex
    move side by side; the chain's path and result are those of the one-lane chain, bit for bit."""
    objs = [synth_objects(n) for n in ("c3_0", "c3_1", "c0acc")]
    with api.Server(precision=precision, acc=True, n_slots=152 * 64, lanes=4) as srv:
        ids = [srv.submit(s.model, s.obs, **dict(CFG, seed=60 + k)) for k, s in enumerate(objs)]
        while any(srv.poll(i) is None for i in ids):
            srv.step(8)
        got = [srv.poll(i)[0] for i in ids]
        evals = srv.stats()["n_evals"]
    total = 0
    for k, s in enumerate(objs):
        ref = single(s, precision, 60 + k)
        same(got[k], ref)
        total += ref.n_evals
    assert evals == total  # only the evaluations the one-lane chains make are counted


@pytest.mark.parametrize("lanes", [1, 4])
def test_server_cancel_queued_and_running(gpu, synth_objects, lanes):
    """ast_cancel on a queued request removes it before admission; on a running request the next
    step drops its chains, its memory returns to the HBM budget, and ast_poll reports
    AST_E_CANCELLED.  The other requests' results are those of their single fits, bit for bit."""
    objs = [synth_objects(n) for n in ("c3_0", "c3_1", "c3_2", "c3_3")]
    cfg = dict(CFG, evals_cap=200)
    with api.Server(precision=api.PREC_MIXED, acc=True, n_slots=152 * 64, lanes=lanes) as srv:
        ids = [srv.submit(s.model, s.obs, **dict(cfg, seed=80 + k)) for k, s in enumerate(objs)]
        assert srv.cancel(ids[3])                      # still queued: never admitted
        srv.step(4)                                    # admits 0..2, which start to run
        used_before = srv.stats()["hbm_used"]
        assert used_before >= sum(srv.request_bytes(i) for i in ids[:3])
        assert srv.cancel(ids[1])                      # running
        srv.step(4)
        assert srv.stats()["hbm_used"] <= used_before - srv.request_bytes(ids[1])
        for i in (ids[1], ids[3]):
            with pytest.raises(api.capi.AstError) as ei:
                srv.poll(i)
            assert ei.value.code == -10
        while any(srv.poll(i) is None for i in (ids[0], ids[2])):
            srv.step(16)
        got = {i: srv.poll(i)[0] for i in (ids[0], ids[2])}
        assert not srv.cancel(ids[0])                  # finished: the result stays
        assert srv.stats()["hbm_used"] == 0
    for k in (0, 2):
        s = objs[k]
        with api.Engine(s.model, s.obs) as eng:
            ref = eng.fit(n_chains=cfg["n_chains"], group_size=cfg["group_size"], seed=80 + k,
                          evals_cap=cfg["evals_cap"], precision=api.PREC_MIXED)
        same(got[ids[k]], ref)


@pytest.mark.parametrize("tile", [8, 16, 32])
def test_warp_tiled_mapping_equals_single_fits(gpu, synth_objects, tile):
    """Warp per model with observation tiles (ast_batch_launch.tile): the warp's 32 chains are
    integrated one per lane through T observations, the tile's magnitudes are spread over the
    lanes, each lane sums its own residuals.  The arithmetic is the thread path's, so every
    object equals its single fit bit for bit; the NUDGE object (c2) takes the lane-by-lane
    evaluation inside the same kernel."""
    objs = [synth_objects(n) for n in OBJECTS + ["c2"]]
    with api.Batch(precision=api.PREC_MIXED, acc=True, n_slots=152 * 32) as b:
        for k, s in enumerate(objs):
            b.add(s.model, s.obs, **dict(CFG, seed=90 + k))
        b.run(tpb=64, refill=32, tile=tile)
        c = b.counters()
        assert c["tile"] == tile and c["refill"] == 32
        got = [b.result(i) for i in range(len(objs))]
    for k, s in enumerate(objs):
        same(got[k], single(s, api.PREC_MIXED, 90 + k))
