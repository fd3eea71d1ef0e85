"""In-tree build of the engine (CUDA, sm_103a), the C command-line tool and the oracle.

Everything is compiled with plain nvcc / gcc command lines, in parallel, into ``_build/``
directories next to the sources (git-ignored).  No cmake, no pip install: the library that the
tests and the bench load is the one built here, in the tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"

ARCH = os.environ.get("AST_CUDA_ARCH", "sm_103a")
GENCODE = [f"-gencode=arch=compute_{ARCH[3:]},code={ARCH}"]
CU_SOURCES = ["csrc/engine.cu", "csrc/fit.cu", "csrc/batch.cu", "csrc/periodogram.cu", "csrc/rmsd.cu",
              "csrc/animate.cu"]
C_SOURCES = ["host/tables.c", "host/read_data.c", "host/misc.c", "host/errors.c", "host/png.c"]
CLI_SOURCES = ["host/asteroid.c"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir() -> Path:
    nvcc = Path(_nvcc()).resolve()
    for cand in (nvcc.parent.parent / "lib64", nvcc.parent.parent / "targets" / "sbsa-linux" / "lib",
                 nvcc.parent.parent / "targets" / "x86_64-linux" / "lib"):
        if (cand / "libcudart.so").exists() or (cand / "libcudart_static.a").exists():
            return cand
    return nvcc.parent.parent / "lib64"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")
    if os.environ.get("AST_BUILD_VERBOSE") and r.stdout.strip():
        print(r.stdout, file=sys.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(list(PKG.glob("csrc/*.cuh")) + list(PKG.glob("host/*.h")) + list(INCLUDE.glob("*.h")))


_ZLIB = None


def _zlib() -> tuple[list[str], list[str]]:
    """(-D flags, link flags) for zlib when this machine can compile and link against it; the
    PNG writer falls back to stored deflate blocks otherwise."""
    global _ZLIB
    if _ZLIB is None:
        _ZLIB = ([], [])
        src = "#include <zlib.h>\nint main(void){uLongf n=64;unsigned char a[64],b[1]={0};return compress2(a,&n,b,1,6);}\n"
        BUILD.mkdir(exist_ok=True)
        for lib in ("-lz", "-l:libz.so.1"):
            r = subprocess.run(["gcc", "-x", "c", "-", "-o", str(BUILD / "zlib_probe"), lib], input=src, text=True,
                               stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if r.returncode == 0:
                _ZLIB = (["-DAST_HAVE_ZLIB"], [lib])
                break
    return _ZLIB


def build_engine(force: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compile libasteroid_gb300.so (CUDA engine + C host code) and the asteroid CLI."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    objs: list[Path] = []
    jobs = []
    for src in CU_SOURCES:
        s = PKG / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nvcc, *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
                   f"-I{INCLUDE}", f"-I{PKG / 'host'}", "-c", str(s), "-o", str(o)]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in C_SOURCES:
        s = PKG / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["gcc", "-O2", "-fPIC", "-std=c11", "-Wall", "-ffp-contract=off", *_zlib()[0], f"-I{INCLUDE}",
                         f"-I{PKG / 'host'}",
                         "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=max(4, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs))
    lib = BUILD / "libasteroid_gb300.so"
    if force or jobs or not lib.exists():
        _run([nvcc, *GENCODE, "-shared", "-o", str(lib), *map(str, objs), "-lcudart", *_zlib()[1]])
    cli = BUILD / "asteroid"
    cli_src = [PKG / s for s in CLI_SOURCES if (PKG / s).exists()]
    if cli_src and (force or _stale(cli, cli_src + hdrs + [lib])):
        _run(["gcc", "-O2", "-std=c11", "-Wall", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{PKG / 'host'}", *map(str, cli_src),
              "-o", str(cli), f"-L{BUILD}", "-lasteroid_gb300", f"-Wl,-rpath,{BUILD}", "-lm"])
    return lib


PARITY = BUILD / "parity"


def build_parity_engine(force: bool = False) -> Path:
    """The engine with engine.cu -- the evaluation kernels behind ast_eval_batch -- compiled
    without fused multiply-adds (nvcc -fmad=false), linked with the other objects of the main
    build into _build/parity/libasteroid_gb300.so.  Test infrastructure for the FP64 parity
    check against the reference kernel compiled the same way (oracle/build_ref.sh nofma): both
    sides then round every product and sum separately, so only the order of operations and
    CUDA's libm are left to differ.  Loaded in a child process through AST_ENGINE_LIB."""
    build_engine()
    PARITY.mkdir(exist_ok=True)
    nvcc = _nvcc()
    src = PKG / "csrc" / "engine.cu"
    obj = PARITY / "engine.o"
    if force or _stale(obj, [src] + _headers()):
        _run([nvcc, *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-Xcompiler",
              "-fPIC,-O2,-ffp-contract=off", f"-I{INCLUDE}", f"-I{PKG / 'host'}", "-c", str(src), "-o", str(obj)])
    objs = [obj] + [BUILD / (Path(s).stem + ".o") for s in CU_SOURCES if Path(s).stem != "engine"]
    objs += [BUILD / (Path(s).stem + ".o") for s in C_SOURCES]
    lib = PARITY / "libasteroid_gb300.so"
    if force or _stale(lib, objs):
        _run([nvcc, *GENCODE, "-shared", "-o", str(lib), *map(str, objs), "-lcudart", *_zlib()[1]])
    return lib


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) with OpenMP and without fused multiply-adds."""
    ORACLE_BUILD.mkdir(exist_ok=True)
    src = ORACLE / "chi2_oracle.c"
    deps = [src] + sorted(ORACLE.glob("*.h")) + [INCLUDE / "asteroid_gb300.h"]
    lib = ORACLE_BUILD / "liboracle.so"
    if force or _stale(lib, deps):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp", f"-I{INCLUDE}",
              str(src), "-o", str(lib), "-lm"])
    # Driver-API loader for the reference kernel cubins (oracle/_ref/ref_*.cubin).
    loader_src = ORACLE / "ref_gpu_loader.cpp"
    loader = ORACLE_BUILD / "libref_gpu_loader.so"
    if loader_src.exists() and (force or _stale(loader, [loader_src])):
        cuda = Path(_nvcc()).resolve().parent.parent
        libdirs = [p for p in (cuda / "lib64" / "stubs", cuda / "lib64", cuda / "targets" / "sbsa-linux" / "lib" / "stubs")
                   if p.exists()]
        _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", f"-I{cuda / 'include'}", str(loader_src), "-o", str(loader),
              *[f"-L{d}" for d in libdirs], "-lcuda"])
    return lib


def build_reference_oracle() -> None:
    """Where the reference checkout is present, build its own chi^2 code (oracle/_ref)."""
    script = ORACLE / "build_ref.sh"
    ref = Path(os.environ.get("AST_REFERENCE_DIR", str(ROOT.parent / "reference")))
    if script.exists() and (ref / "cuda.c").exists():
        R = ORACLE / "_ref"
        have = list(R.glob("libref_*.so")) if R.exists() else []
        if not have:
            _run(["bash", str(script)])
            return
        if not (R / "libref_minima.so").exists():
            _run(["bash", str(script), "minima"])
        if not (R / "ref_ppsi_torque_acc_nofma.cubin").exists():
            _run(["bash", str(script), "nofma"])
        if any(_stale(R / f"libref_read_{v}.so", [ORACLE / "ref_harness_read_data.cu"])
               for v in ("plain", "interp", "interp_nudge")):
            _run(["bash", str(script), "read"])
        # The host builds again when their harness is newer than them (new entry points).
        if _stale(R / "libref_ppsi_torque_acc.so", [ORACLE / "ref_harness_host.cu", script]):
            _run(["bash", str(script), "host"])  # also the simplex / RMSD drivers
        elif any(_stale(R / f"libref_nm_{v}.so", [ORACLE / "ref_nm_shim.h", ORACLE / "ref_harness_nm.cu"])
                 for v in ("ppsi_torque_acc", "ppsi_torque_sp", "torque_interp_acc", "bc_interp_acc", "bw_torque_acc",
                           "bc_torque_ppsi_acc", "free_acc", "bc_interp_sp", "c2_nudge_acc", "rmsd_ppsi_torque_acc",
                           "rmsd_bc_interp_sp", "rmsd_sph_ppsi_torque_acc")):
            _run(["bash", str(script), "nm"])


def build(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_engine, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", BUILD / "libasteroid_gb300.so")
