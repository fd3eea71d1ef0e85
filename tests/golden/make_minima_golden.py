"""Generate tests/golden/minima_ref.json from the reference's own minima() (misc.c:65-276).

Run here, where the reference checkout exists:  bash oracle/build_ref.sh minima && python
tests/golden/make_minima_golden.py.  Each case is a curve on a plot-style grid t[i] = i * h,
with magnitudes that are multiples of 2^-20 (stored as integers, so the fixture holds them
exactly); the expected cl_fr, cl_H and number of minima come from oracle/_ref/libref_minima.so.
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
SCALE = 2.0 ** 20


def curve(kind: str, n: int, span: float, seed: int):
    h = span / (n - 1)
    t = np.arange(n) * h
    rng = np.random.default_rng(seed)
    if kind == "double_wave":      # a tumbler's two minima per rotation, two periods beating
        v = 0.6 * np.sin(2 * np.pi * t / 0.31) + 0.25 * np.sin(2 * np.pi * t / 0.137 + 1.0)
    elif kind == "noisy":          # a few hundred minima from noise on a slow wave
        v = 0.3 * np.sin(2 * np.pi * t / 0.5) + 0.05 * rng.standard_normal(n)
    elif kind == "plateaus":       # equal neighbours: V[i] >= V[i+1] counts, V[i] > V[i-1] does not
        v = np.round(2 * np.sin(2 * np.pi * t / 0.23), 1)
    elif kind == "one_minimum":    # a single minimum: no intervals
        v = -((t - span / 2) ** 2)
    elif kind == "flat":           # no minimum at all
        v = np.zeros(n)
    else:
        raise ValueError(kind)
    q = np.round(v * SCALE).astype(np.int64)
    return h, q


CASES = [("double_wave", 4000, 9.0, 1), ("noisy", 3000, 6.0, 2), ("plateaus", 2000, 5.0, 3),
         ("one_minimum", 500, 2.0, 4), ("flat", 300, 1.0, 5)]


def main():
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libref_minima.so"))
    lib.refm_minima.restype = C.c_int
    out = []
    for kind, n, span, seed in CASES:
        h, q = curve(kind, n, span, seed)
        t = np.arange(n) * h
        vm = q.astype(np.float64) / SCALE
        fr = np.zeros(5)
        H = np.zeros(5)
        nmin = lib.refm_minima(t.ctypes.data_as(C.c_void_p), vm.ctypes.data_as(C.c_void_p), n,
                               fr.ctypes.data_as(C.c_void_p), H.ctypes.data_as(C.c_void_p))
        assert nmin >= 0
        out.append({"kind": kind, "n": n, "h": h, "vm_scaled": q.tolist(), "scale": SCALE, "n_minima": nmin,
                    "cl_fr": fr.tolist(), "cl_H": [None if np.isnan(x) else x for x in H]})
        print(kind, nmin, fr, H)
    doc = {"generator": "tests/golden/make_minima_golden.py from the reference host build oracle/_ref/libref_minima.so",
           "cases": out}
    (Path(__file__).resolve().parent / "minima_ref.json").write_text(json.dumps(doc))


if __name__ == "__main__":
    main()
