"""Generate tests/golden/drivers_ref.json from the reference's own chi2_gpu and chi2_gpu_rms.

Run here, where the reference checkout exists:  bash oracle/build_ref.sh nm && python
tests/golden/make_driver_golden.py.  For every host build of the reference's simplex driver and
RMSD sampler in oracle/_ref (libref_nm_<variant>.so, oracle/build_ref.sh), on the object of the
matching tests/golden/ref_<variant>.json fixture, it stores what the reference computes:

  simplex  one launch of one block of 256 chains, two stages, seed 5, random starts and -reopt
           starts from the fixture's first parameter vector: the block's best chi^2, parameters
           and delta_V; the same on a 400-point NUDGE object (-reopt from its true parameters);
  rmsd     one chi2_gpu_rms launch of two blocks, 8 samples per thread, dx 2e-5, seed 9, launch
           indices 0 and 3 around the fixture's first parameter vector: f0, f1, the counts of
           evaluated and rejected points and the float parameter ranges.

The builds draw their random numbers from the engine's Philox stream instead of cuRAND (see
oracle/ref_nm_shim.h); everything else is the reference's code.  The fixture lets the oracle be
checked against these results where the reference is absent.
"""
from __future__ import annotations

import dataclasses
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as O  # noqa: E402
from asteroid_gb300 import synth  # noqa: E402
from tests.test_oracle_pin import load_fixture  # noqa: E402

GOLDEN = Path(__file__).resolve().parent
SIMPLEX = ["ppsi_torque_acc", "ppsi_torque_sp", "torque_interp_acc", "bc_interp_acc", "bw_torque_acc",
           "bc_torque_ppsi_acc", "free_acc", "bc_interp_sp"]
# The NUDGE case: the fixture's 120 points give no admissible minima, so a 400-point object made
# by the synthetic generator (seeded; its true curve from the oracle) stands in; the test
# regenerates it from this configuration.
NUDGE_CFG = synth.SynthConfig("nudge400", "TORQUE,P_PSI,INTERP,ACC,NUDGE", 5e-3, 400, 2, 10, 5, seed=1007,
                              n_minima=3, filter_chars="RV", dv_range=0.5, ppsi_hours=(20.0, 4800.0))
# build -> (fixture, SPHERICAL_K)
RMSD = {"rmsd_ppsi_torque_acc": ("rmsd_ppsi_torque_acc", False),
        "rmsd_sph_ppsi_torque_acc": ("rmsd_ppsi_torque_acc", True),
        "rmsd_bc_interp_sp": ("rmsd_bc_interp_sp", False)}


def main() -> int:
    out = {"generator": "tests/golden/make_driver_golden.py", "simplex": [], "rmsd": []}
    for variant in SIMPLEX:
        fx, m, obs = load_fixture(GOLDEN / f"ref_{variant}.json")
        ref = O.RefNM(variant)
        for reopt in (False, True):
            p0 = np.array(fx["params"][0]) if reopt else None
            r = ref.fit(m, obs, seed=5, n_blocks=1, n_stages=2, reopt=reopt, params0=p0)
            out["simplex"].append({"fixture": variant, "seed": 5, "n_chains": ref.block_size, "n_stages": 2,
                                   "steps_cap": int(ref.n_steps), "reopt": reopt,
                                   "params0": None if p0 is None else p0.tolist(),
                                   "best_f": r["best_f"].tolist(), "best_params": r["best_params"].tolist(),
                                   "best_dv": r["best_dv"].tolist()})
            print(variant, "reopt" if reopt else "random", r["best_f"])
    with tempfile.TemporaryDirectory() as d:
        sn = synth.generate(NUDGE_CFG, Path(d) / "nudge400", vmod_fn=lambda m, o, p: O.model_curve(m, o, p))
        ref = O.RefNM("c2_nudge_acc")
        for reopt in (False, True):
            r = ref.fit(sn.model, sn.obs, seed=5, n_blocks=1, n_stages=2, reopt=reopt, params0=sn.params_true)
            out["simplex"].append({"synth": dataclasses.asdict(NUDGE_CFG), "seed": 5, "n_chains": ref.block_size,
                                   "n_stages": 2, "steps_cap": int(ref.n_steps), "reopt": reopt, "params0": "truth",
                                   "best_f": r["best_f"].tolist(), "best_params": r["best_params"].tolist(),
                                   "best_dv": r["best_dv"].tolist()})
            print("nudge400", "reopt" if reopt else "random", r["best_f"])
    for build, (fixture, spherical) in RMSD.items():
        fx, m, obs = load_fixture(GOLDEN / f"ref_{fixture}.json")
        ref = O.RefNM(build)
        p0 = np.array(fx["params"][0])
        for call in (0, 3):
            r = ref.rmsd(m, obs, p0, seed=9, call=call, n_blocks=2, samples=8, dx=2e-5)
            out["rmsd"].append({"fixture": fixture, "build": build, "spherical": spherical, "seed": 9, "call": call,
                                "n_streams": 2 * ref.block_size, "samples": 8, "dx": 2e-5, "params0": p0.tolist(),
                                "f0": float(r["f0"]), "f1": float(r["f1"]), "n_tot": r["n_tot"], "n_bad": r["n_bad"],
                                "par_min": [float(v) for v in r["par_min"]],
                                "par_max": [float(v) for v in r["par_max"]]})
            print(build, call, r["n_tot"], r["n_bad"])
    (GOLDEN / "drivers_ref.json").write_text(json.dumps(out, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
