"""The multi-GPU form (replicas with distinct seeds, host argmin) as world_size-2 gloo ranks on
the CPU: each rank runs the oracle's simplex driver with its replica seed, gather_best merges over
the process group, and the merged best equals the argmin over both ranks' results computed in
one process."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from asteroid_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, obj_dir, out):
    import sys

    from tests.conftest import ROOT

    for p in (str(ROOT), str(ROOT / "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import oracle as O

    from asteroid_gb300 import api

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    model = api.make_model("TORQUE,P_PSI,ACC", 1e-2, (2.0, 4800.0))
    obs = api.read_data(os.path.join(obj_dir, "lc.dat"), obj_dir)
    res = O.fit(model, obs, replicas.replica_seed(41, rank), n_chains=32, group_size=16, evals_cap=30)
    merged = replicas.gather_best(res, dist)
    out[rank] = (replicas.best_of(res), merged)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_merge_to_the_host_argmin(synth_objects):
    s = synth_objects("c0acc")
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, world, port, str(s.dir), out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=300)
            assert p.exitcode == 0
        bests = [out[r][0] for r in range(world)]
        merged = [out[r][1] for r in range(world)]
    assert merged[0] == merged[1]
    expect = replicas.merge(bests)
    assert merged[0]["chi2"] == expect["chi2"] and merged[0]["rank"] == expect["rank"]
    assert merged[0]["chi2"] == min(b["chi2"] for b in bests)
    # Distinct seeds: the replicas are different searches.
    assert bests[0]["params"] != bests[1]["params"]


def test_replica_seeds_are_distinct_and_rank0_keeps_the_seed():
    seeds = {replicas.replica_seed(7, r) for r in range(64)}
    assert len(seeds) == 64 and replicas.replica_seed(7, 0) == 7


def test_merge_breaks_ties_by_rank():
    a = {"chi2": 1.0, "group": 3, "params": [1], "dv": [0]}
    b = {"chi2": 1.0, "group": 0, "params": [2], "dv": [0]}
    assert replicas.merge([a, b])["rank"] == 0
    assert replicas.merge([{"chi2": 2.0, "group": 0, "params": [0], "dv": [0]}, b])["rank"] == 1
