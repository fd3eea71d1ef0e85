#!/usr/bin/env bash
# build_ref.sh -- TEST INFRASTRUCTURE ONLY.  Builds the reference's own chi^2 code from its
# sources, where they lie, into oracle/_ref/ (git-ignored):
#
#   libref_<variant>.so  host build of chi2one / x2params / params2x / ODE_func (cuda.c:13-1319)
#                        with oracle/ref_harness_host.cu as entry points; used here to pin the
#                        oracle and to generate tests/golden/.
#   ref_<variant>.cubin  device build (sm_100) of the same functions plus
#                        oracle/ref_harness_kernel.cu; loaded on the GPU by
#                        oracle/ref_gpu_loader.cpp to check the CUDA path at 1e-12.
#   libref_minima.so     host build of minima() (misc.c:65-276, default macros) with
#                        oracle/ref_harness_minima.cu; pins the periodogram oracle.
#   ref_animate.cubin    device build (sm_100) of cuda.c with -DANIMATE plus
#                        oracle/ref_harness_animate.cu: the reference's compute_rgb on the GPU.
#   ref_<variant>_nofma.cubin  the same device build with nvcc -fmad=false (no multiply-add
#                        contraction), for the parity check against the engine built the same way.
#   libref_nm_<variant>.so  the host build above plus the reference's chi2_gpu simplex driver
#                        (cuda.c:1326-1833) cut from cuda.c and compiled as host code between
#                        oracle/ref_nm_shim.h and oracle/ref_harness_nm.cu (the block's threads as
#                        host threads, cuRAND as the engine's Philox stream); -DTIMING, the
#                        reference's own switch, sets N_STEPS = 100.  Pins the oracle's simplex.
#   libref_read_<variant>.so  the reference's host readers, read_data.c and misc.c, with
#                        oracle/ref_harness_read_data.cu (cudaMallocHost as malloc); pins the
#                        engine's C reader (host/read_data.c, host/misc.c).
#
# The reference's asteroid.h and cuda.c are streamed through sed into nvcc's standard input:
# the four device functions become __host__ __device__ (host build only), N_FILTERS becomes 8
# and TIME_STEP the variant's step.  The variant macros are the reference's own (-DTORQUE ...).
# Nothing of the reference is written to disk.  Needs the reference checkout ($AST_REFERENCE_DIR,
# by default the directory "reference" beside the repository); without it the script does
# nothing.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${AST_REFERENCE_DIR:-$(cd "$here/../.." && pwd)/reference}"
OUT="$here/_ref"
if [[ ! -f "$REF/cuda.c" || ! -f "$REF/asteroid.h" ]]; then
    echo "build_ref.sh: no reference checkout at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"

# name  time_step  macros...
VARIANTS=(
  "ppsi_torque_acc 1e-2 -DP_PSI -DTORQUE -DACC"
  "ppsi_torque_sp 1e-2 -DP_PSI -DTORQUE"
  "torque_interp_acc 1e-2 -DTORQUE -DINTERP -DACC"
  "bc_interp_acc 1e-2 -DBC -DINTERP -DACC"
  "bw_torque_acc 1e-2 -DBW_BALL -DTORQUE -DACC"
  "c2_nudge_acc 5e-3 -DP_PSI -DTORQUE -DINTERP -DACC -DNUDGE"
  "bc_torque_ppsi_acc 1e-2 -DBC -DTORQUE -DP_PSI -DACC"
  "free_acc 1e-2 -DACC"
  "bc_interp_sp 1e-2 -DBC -DINTERP"
  "rmsd_ppsi_torque_acc 1e-2 -DP_PSI -DTORQUE -DACC -DRMSD"
  "rmsd_bc_interp_sp 1e-2 -DBC -DINTERP -DRMSD"
)

stream_source() {  # $1 = time step, $2 = 1 for the host build
    local ts="$1" host="$2"
    sed -e 's/^const int N_FILTERS = 1;/const int N_FILTERS = 8;/' \
        -e "s/^const double TIME_STEP = 1e-2;.*/const double TIME_STEP = $ts;/" "$REF/asteroid.h"
    if [[ "$host" == 1 ]]; then
        sed -e 's/^#include "asteroid.h"//' \
            -e 's/^__device__ void ODE_func/__host__ __device__ void ODE_func/' \
            -e 's/^__device__ CHI_FLOAT chi2one/__host__ __device__ CHI_FLOAT chi2one/' \
            -e 's/^__device__ void params2x/__host__ __device__ void params2x/' \
            -e 's/^__device__ int x2params/__host__ __device__ int x2params/' "$REF/cuda.c"
        cat "$here/ref_harness_host.cu"
    else
        sed -e 's/^#include "asteroid.h"//' "$REF/cuda.c"
        cat "$here/ref_harness_kernel.cu"
    fi
}

pids=()
if [[ -f "$REF/misc.c" && ( "${1:-all}" == "all" || "${1:-all}" == "host" || "${1:-all}" == "minima" ) ]]; then
    ( { sed -e 's/^const int N_FILTERS = 1;/const int N_FILTERS = 8;/' "$REF/asteroid.h"
        sed -e 's/^#include "asteroid.h"//' "$REF/misc.c"
        cat "$here/ref_harness_minima.cu"; } |
      nvcc -x cu -arch=sm_100 -O2 -DMAIN -I"$REF" -Xcompiler -fPIC,-ffp-contract=off -shared -w \
           -o "$OUT/libref_minima.so" - ) &
    pids+=($!)
fi
if [[ "${1:-all}" == "all" || "${1:-all}" == "cubin" || "${1:-all}" == "animate" ]]; then
    ( { sed -e 's/^const int N_FILTERS = 1;/const int N_FILTERS = 8;/' -e 's|^ *#include <png.h>||' "$REF/asteroid.h"
        sed -e 's/^#include "asteroid.h"//' "$REF/cuda.c"
        cat "$here/ref_harness_animate.cu"; } |
      nvcc -x cu -cubin -arch=sm_100 -O3 -DMAIN -DANIMATE -I"$REF" -w -o "$OUT/ref_animate.cubin" - ) &
    pids+=($!)
fi
if [[ "${1:-all}" == "all" || "${1:-all}" == "cubin" || "${1:-all}" == "nofma" ]]; then
    for v in "${VARIANTS[@]}"; do
        read -r name ts macros <<<"$v"
        ( stream_source "$ts" 0 | nvcc -x cu -cubin -arch=sm_100 -O3 -fmad=false -DMAIN $macros -I"$REF" -w \
              -o "$OUT/ref_${name}_nofma.cubin" - ) &
        pids+=($!)
    done
fi
# name  time_step  macros...  (the simplex driver on the host)
# (the -DRMSD variants take chi2_gpu_rms, the others chi2_gpu)
NM_VARIANTS=(
  "ppsi_torque_acc 1e-2 -DP_PSI -DTORQUE -DACC"
  "ppsi_torque_sp 1e-2 -DP_PSI -DTORQUE"
  "torque_interp_acc 1e-2 -DTORQUE -DINTERP -DACC"
  "bc_interp_acc 1e-2 -DBC -DINTERP -DACC"
  "bw_torque_acc 1e-2 -DBW_BALL -DTORQUE -DACC"
  "bc_torque_ppsi_acc 1e-2 -DBC -DTORQUE -DP_PSI -DACC"
  "free_acc 1e-2 -DACC"
  "bc_interp_sp 1e-2 -DBC -DINTERP"
  "c2_nudge_acc 5e-3 -DP_PSI -DTORQUE -DINTERP -DACC -DNUDGE"
  "rmsd_ppsi_torque_acc 1e-2 -DP_PSI -DTORQUE -DACC -DRMSD"
  "rmsd_sph_ppsi_torque_acc 1e-2 -DP_PSI -DTORQUE -DACC -DRMSD -DSPHERICAL_K"
  "rmsd_bc_interp_sp 1e-2 -DBC -DINTERP -DRMSD"
)
if [[ "${1:-all}" == "all" || "${1:-all}" == "host" || "${1:-all}" == "nm" ]]; then
    for v in "${NM_VARIANTS[@]}"; do
        read -r name ts macros <<<"$v"
        kernel=chi2_gpu
        [[ "$macros" == *-DRMSD* ]] && kernel=chi2_gpu_rms
        ( { stream_source "$ts" 1
            cat "$here/ref_nm_shim.h"
            # from the kernel's first line to its closing brace (chi2_gpu_rms: the line before its
            # "#endif //RMSD", the brace being indented there)
            awk -v k="$kernel" '$0 ~ "^__global__ void " k " \\(" {p=1}
                                p && k == "chi2_gpu_rms" && /^ *#endif *\/\/ *RMSD/ {exit}
                                p {print}
                                p && k == "chi2_gpu" && /^}/ {exit}' "$REF/cuda.c"
            cat "$here/ref_harness_nm.cu"; } |
          nvcc -x cu -arch=sm_100 -O2 -DMAIN -DTIMING $macros -I"$REF" -I"$here" -I"$here/../asteroid_gb300/csrc" \
               -Xcompiler -fPIC,-ffp-contract=off,-ftrivial-auto-var-init=zero,-pthread -shared -w \
               -o "$OUT/libref_nm_$name.so" - ) &
        pids+=($!)
    done
fi
# name  macros...  (the host readers: read_data.c and misc.c)
READ_VARIANTS=(
  "plain"
  "interp -DINTERP"
  "interp_nudge -DINTERP -DNUDGE"
)
if [[ -f "$REF/read_data.c" && -f "$REF/misc.c" && ( "${1:-all}" == "all" || "${1:-all}" == "host" || "${1:-all}" == "read" ) ]]; then
    for v in "${READ_VARIANTS[@]}"; do
        read -r name macros <<<"$v"
        ( { sed -e 's/^const int N_FILTERS = 1;/const int N_FILTERS = 8;/' "$REF/asteroid.h"
            cat "$here/ref_harness_read_data.cu"
            sed -e 's/^#include "asteroid.h"//' "$REF/read_data.c"
            sed -e 's/^#include "asteroid.h"//' "$REF/misc.c"
            echo "#define REFR_TAIL 1"
            cat "$here/ref_harness_read_data.cu"; } |
          nvcc -x cu -arch=sm_100 -O2 -DMAIN $macros -I"$REF" -Xcompiler -fPIC,-ffp-contract=off -shared -w \
               -o "$OUT/libref_read_$name.so" - ) &
        pids+=($!)
    done
fi
[[ "${1:-all}" == "minima" || "${1:-all}" == "animate" || "${1:-all}" == "nofma" || "${1:-all}" == "nm" || "${1:-all}" == "read" ]] && VARIANTS=()
for v in "${VARIANTS[@]}"; do
    read -r name ts macros <<<"$v"
    if [[ "${1:-all}" == "all" || "${1:-all}" == "host" ]]; then
        ( stream_source "$ts" 1 | nvcc -x cu -arch=sm_100 -O2 -DMAIN $macros -I"$REF" \
              -Xcompiler -fPIC,-ffp-contract=off -shared -w -o "$OUT/libref_$name.so" - ) &
        pids+=($!)
    fi
    if [[ -f "$here/ref_harness_kernel.cu" && ( "${1:-all}" == "all" || "${1:-all}" == "cubin" ) ]]; then
        ( stream_source "$ts" 0 | nvcc -x cu -cubin -arch=sm_100 -O3 -DMAIN $macros -I"$REF" -w \
              -o "$OUT/ref_$name.cubin" - ) &
        pids+=($!)
    fi
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
