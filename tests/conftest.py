"""Shared fixtures: the built libraries, synthetic objects, GPU availability."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT), str(ROOT / "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    from asteroid_gb300 import build

    build.build()
    return True


@pytest.fixture(scope="session")
def oracle_mod(built):
    import oracle

    oracle.load()
    return oracle


def _gpu_available() -> bool:
    try:
        import ctypes

        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(built):
    if not _gpu_available():
        pytest.fail("a -m gpu test ran without a visible CUDA device")
    return True


_SYNTH_CACHE: dict = {}


@pytest.fixture(scope="session")
def synth_objects(built, oracle_mod, tmp_path_factory):
    """Synthetic objects of the benchmark configurations ("c0" ... "c2", or "c3_<i>" for object i
    of the batched workload), with oracle true-model curves."""
    from asteroid_gb300 import synth

    def get(name: str):
        if name not in _SYNTH_CACHE:
            d = tmp_path_factory.mktemp(f"synth_{name}")
            cfg = synth.batch_config(int(name[3:])) if name.startswith("c3_") else name
            _SYNTH_CACHE[name] = synth.generate(cfg, d, vmod_fn=lambda m, o, p: oracle_mod.model_curve(m, o, p))
        return _SYNTH_CACHE[name]

    return get
