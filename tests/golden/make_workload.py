"""Writes tests/golden/workload_c2.npz: the config-2 object of the benchmark (2000 points,
3 filters, 60 days, TORQUE + P_PSI + INTERP + ACC + NUDGE, TIME_STEP 5e-3) as the synthetic
generator makes it, with the oracle's model curve for the true magnitudes.

bench.py --impl reference times the CPU implementation of the path on this object without
loading the engine library: the model tables are stored as the bytes of the ast_model
structure, the observations as the converted arrays of ast_obs_set, and the true parameters.
Run from the repository root: python tests/golden/make_workload.py
"""
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "oracle")]


def main(name="c2"):
    import oracle

    from asteroid_gb300 import build, synth

    build.build()
    oracle.load()
    with tempfile.TemporaryDirectory() as d:
        s = synth.generate(name, d, vmod_fn=lambda m, o, p: oracle.model_curve(m, o, p))
        o = s.obs
        np.savez_compressed(ROOT / "tests" / "golden" / f"workload_{name}.npz", model=np.frombuffer(bytes(s.model), np.uint8),
                            mjd=o.mjd, v=o.v, w=o.w, filt=o.filt, e_unit=o.e_unit, s_unit=o.s_unit, eph_e=o.eph_e,
                            eph_s=o.eph_s, eph_mjd0=o.eph_mjd0, t_min=o.t_min, v_min=o.v_min,
                            params_true=s.params_true, hmjd0=np.array([o.hmjd0]))


if __name__ == "__main__":
    main(*sys.argv[1:])
