"""Generate tests/golden/ref_<variant>.json from the reference's own chi^2 code.

Run here, where the reference checkout exists:  bash oracle/build_ref.sh host && python
tests/golden/make_golden.py.  For every reference build in oracle/_ref (one per variant of
oracle/build_ref.sh) it writes a small synthetic object and the reference's outputs for it:
chi2one and delta_V on a set of parameter vectors, x2params on dimensionless points (reopt 0 and
1) and params2x.  The inputs are stored with them, so the fixtures need neither the reference
nor the generator at test time.  The reference computes every expected value; the oracle is used
only to give the synthetic object a true-model light curve.
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
from asteroid_gb300 import api, build, synth  # noqa: E402

# reference build -> (variant macros, time step, points, filters, filter chars, minima)
VARIANTS = {
    "ppsi_torque_acc": ("TORQUE,P_PSI,ACC", 1e-2, 120, 1, "W", 0),
    "ppsi_torque_sp": ("TORQUE,P_PSI", 1e-2, 120, 1, "W", 0),
    "torque_interp_acc": ("TORQUE,INTERP,ACC", 1e-2, 120, 2, "RV", 0),
    "bc_interp_acc": ("BC,INTERP,ACC", 1e-2, 120, 2, "RV", 0),
    "bw_torque_acc": ("BW_BALL,TORQUE,ACC", 1e-2, 120, 1, "W", 0),
    "c2_nudge_acc": ("TORQUE,P_PSI,INTERP,ACC,NUDGE", 5e-3, 300, 3, "RVB", 3),
    "bc_torque_ppsi_acc": ("BC,TORQUE,P_PSI,ACC", 1e-2, 120, 1, "W", 0),
    "free_acc": ("ACC", 1e-2, 120, 1, "W", 0),
    "bc_interp_sp": ("BC,INTERP", 1e-2, 120, 2, "RV", 0),
    "rmsd_ppsi_torque_acc": ("TORQUE,P_PSI,ACC,RMSD", 1e-2, 120, 1, "W", 0),
    "rmsd_bc_interp_sp": ("BC,INTERP,RMSD", 1e-2, 120, 2, "RV", 0),
}


def main():
    build.build()
    out_dir = Path(__file__).resolve().parent
    for k, (variant, (flags, ts, npts, nf, chars, nmin)) in enumerate(VARIANTS.items()):
        ref = O.RefHost(variant)
        cfg = synth.SynthConfig(f"golden_{variant}", flags, ts, npts, nf, 6, 6, seed=2000 + k, n_minima=nmin,
                                filter_chars=chars, dv_range=0.5 if nf > 1 else 0.0,
                                ppsi_hours=(20.0, 4800.0) if "NUDGE" in flags else (2.0, 4800.0))
        with tempfile.TemporaryDirectory() as d:
            s = synth.generate(cfg, d, vmod_fn=lambda m, o, p: O.model_curve(m, o, p))
        m, obs = s.model, s.obs
        assert ref.n_params == m.n_params and abs(ref.time_step - ts) < 1e-15
        rng = np.random.default_rng(3000 + k)
        iL = api.param_names(m).index("L")
        P = [s.params_true]
        for reopt in (0, 1):
            for _ in range(40):
                x = rng.uniform(0, 1, m.n_params)
                p = ref.x2params(m, x, reopt=reopt)
                if p is not None and (p[iL] * ts <= 0.5 or len(P) < 3):
                    P.append(p)
                if len(P) >= 4 + 3 * reopt:
                    break
        chi2, dv = zip(*(ref.chi2(m, obs, p) for p in P))
        X = rng.uniform(-0.05, 1.05, size=(10, m.n_params))
        x2p = {str(r): [None if (q := ref.x2params(m, x, reopt=r)) is None else q.tolist() for x in X] for r in (0, 1)}
        p2x = [ref.params2x(m, p).tolist() for p in P]
        fx = {
            "variant": variant, "flags": flags, "time_step": ts, "ppsi_hours": list(cfg.ppsi_hours),
            "obs": {"mjd": obs.mjd.tolist(), "v": obs.v.astype(float).tolist(), "w": obs.w.astype(float).tolist(),
                    "filt": obs.filt.tolist(), "e_unit": obs.e_unit.ravel().tolist(),
                    "s_unit": obs.s_unit.ravel().tolist(), "eph_e": obs.eph_e.tolist(), "eph_s": obs.eph_s.tolist(),
                    "eph_mjd0": obs.eph_mjd0.tolist(), "t_min": obs.t_min.astype(float).tolist(),
                    "v_min": obs.v_min.astype(float).tolist()},
            "params": [p.tolist() for p in P],
            "chi2": [float(c) for c in chi2],
            "delta_v": [d[: obs.n_filters].tolist() for d in dv],
            "x": X.tolist(), "x2params": x2p, "params2x": p2x,
            "generator": "tests/golden/make_golden.py from the reference host build oracle/_ref/libref_%s.so" % variant,
        }
        (out_dir / f"ref_{variant}.json").write_text(json.dumps(fx))
        print(variant, "chi2:", ["%.6g" % c for c in chi2])


if __name__ == "__main__":
    main()
