// engine.cuh -- the context object behind the C ABI and the helpers the kernels share.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>
#include "asteroid_gb300.h"
#include "model.cuh"

extern "C" int ast_set_error(int code, const char* fmt, ...);

#define AST_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return ast_set_error(AST_E_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,       \
                                 cudaGetErrorString(e_));                                     \
    } while (0)

namespace ast {

// Device error word: kernels record a wait that ran out of iterations here instead of
// trapping, so the context stays usable and the host returns AST_E_TIMEOUT.
enum : int32_t { kErrNone = 0, kErrStageTimeout = 1 };

struct FitBuffers {
    int64_t slots = 0, slots_pad = 0, chains = 0, groups = 0;
    int32_t n_params = 0, n_filters = 0, cf_bytes = 0;
    void* x = nullptr;        // CF [(N+1)*N][S]
    void* f = nullptr;        // CF [N+1][S]
    uint8_t* ind = nullptr;   // [N+1][S]
    void* x0 = nullptr;       // CF [N][S]
    void* xr = nullptr;       // CF [N][S]
    void* fr = nullptr;       // CF [S]
    int32_t* st = nullptr;    // [S] phase | j << 8 | bad << 16
    int32_t* it = nullptr;    // [S] simplex iterations l
    int32_t* ev = nullptr;    // [S] evaluations of the current chain-stage
    int64_t* chain = nullptr; // [S] chain on the slot, -1 if none
    double* dv = nullptr;     // [NF][S] last delta_V of the slot's chain
    double* chain_f = nullptr;  // [C]
    void* chain_x = nullptr;    // CF [C][N] best vertex
    double* chain_dv = nullptr; // [C][NF]
    void* group_x = nullptr;    // CF [G][N] next stage start
    double* out_f = nullptr;    // [G]
    double* out_p = nullptr;    // [G][N]
    double* out_dv = nullptr;   // [G][NF]
    unsigned long long* ctr = nullptr;  // [0] next chain, [1] finished chains, [2] evals, [3] fits, [4] err
    size_t bytes = 0;
    void* base = nullptr;
};

struct FitRun {
    bool active = false;
    ast_fit_cfg cfg{};
    int32_t stage = 0;
    int32_t reopt = 0;          // reopt of the current stage
    int64_t n_evals = 0, n_fits = 0;
    double kernel_ms = 0;
    int tpb = 256, ctas = 0;
    size_t smem = 0;   // dynamic shared memory of the launch (the observation block, or 0)
    int minb = 1;      // register budget variant of fit_kernel
};

}  // namespace ast

struct ast_ctx {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ast_model model{};
    ast::DevModel dm{};
    int32_t n_data = 0, n_filters = 0;
    ast::ObsLayout layout{};
    void* d_obs = nullptr;
    // evaluation scratch
    double* d_params = nullptr;
    double* d_chi2 = nullptr;
    double* d_dv = nullptr;
    int64_t eval_cap = 0;
    // fit
    ast::FitBuffers fb;
    ast::FitRun run;
    int32_t stage_wait = 1 << 22;  // polls of the fit kernel's shared-memory staging wait
};

namespace ast {
// Dynamic shared memory for staging an observation block of `bytes` in one CTA of `kern`: the
// block's size when it fits beside the kernel's static shared memory (the double-float trig
// table, the staging barrier) under the per-CTA opt-in limit `optin`, else 0 -- the kernel then
// reads the block from global memory through L1.  When it is staged, the kernel's dynamic
// shared-memory limit is raised to the block's size (needed above 48 KB; allocates nothing).
template <class K>
inline int obs_smem_for(K kern, size_t bytes, size_t optin, size_t* smem)
{
    *smem = 0;
    if (!bytes) return AST_OK;
    cudaFuncAttributes a;
    AST_CUDA(cudaFuncGetAttributes(&a, kern));
    if (bytes + a.sharedSizeBytes > optin) return AST_OK;
    AST_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    *smem = bytes;
    return AST_OK;
}

int build_dev_model(const ast_model* m, const ast_obs_set* obs, DevModel* dm);
int set_device(int device);
void obs_image(const ast_model* model, const ast_obs_set* obs, const ObsLayout& L, std::vector<unsigned char>& img);
int launch_prep(const DevModel& dm, char* d_block, const ObsLayout& L, int64_t n, cudaStream_t s);
}  // namespace ast
