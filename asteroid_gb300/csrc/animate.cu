// animate.cu -- frames of the ANIMATE build (compute_rgb, cuda.c:2394-2540 of the reference).
//
// The reference runs chi2_plot<<<ceil(SIZE_PIX^2 / BSIZE), BSIZE>>> in which every thread
// integrates the whole model over the plot grid (one RK4 recursion per pixel) and, at each
// snapshot, shades its own pixel: four lines of sight through the pixel's corners intersected with
// the triaxial ellipsoid, Lambert-like shading between terminator, shadow and sunlit colours, a
// red spot around the end of the b axis.  Here the recursion runs once (ast_model_geometry: one
// thread, the fit's FP64 evaluation) and render_kernel shades every pixel of every frame from
// that geometry: one CTA per 32 x 8 tile of a frame, frames on the grid's y dimension, the frame's
// 20 doubles in shared memory, each line of sight through a pixel corner evaluated once and shared
// by the four pixels that meet there.  The arithmetic is the reference's, in FP64, with every
// rounding explicit (no contracted multiply-adds) so that the CPU restatement reproduces each byte.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>

#include "asteroid_gb300.h"
#include "dfloat.cuh"
#include "engine.cuh"

namespace ast {
namespace {

constexpr int kRenderTpb = 256;
// Colours (asteroid.h:300-313): deepest shadow, terminator, brightest sunlit element.
constexpr float kSminR = 6, kSminG = 8, kSminB = 10;
constexpr float kSmaxR = 30, kSmaxG = 41, kSmaxB = 53;
constexpr float kImaxR = 255, kImaxG = 191, kImaxB = 144;
constexpr float kSpotRad = 0.04f;  // SPOT_RAD (asteroid.h:315), a float: its square is rounded to float

#define M_(a, b) DD_MUL(a, b)
#define A_(a, b) DD_ADD(a, b)
#define S_(a, b) DD_SUB(a, b)

// One CTA shades a kTileX x kTileY tile of one frame.  The four corners of a pixel are shared
// with its neighbours, so the CTA first evaluates the (kTileX+1) x (kTileY+1) corner lines of
// sight of its tile once each (hit, red spot, I), then every thread accumulates its pixel's four
// corners in the reference's order (jz outer, jy inner) -- the same values, combined in the same
// float steps, as four evaluations per pixel would give.
// Float pre-test of a corner line of sight.  Most lines of sight miss the ellipsoid; the
// reference settles them with the FP64 discriminant D = B^2 - 4AC < 0.  Here D is first formed in
// float together with a running bound on its error (each product x*y adds |x| e(y) + |y| e(x) +
// u|xy|, each sum e(x) + e(y) + u|x+y|, u = 2^-24, the inputs carrying one rounding each).  When
// D + 2 e(D) + 1e-12 M < 0 (M the sum of the magnitudes of D's terms, far above FP64's own
// rounding of them), the FP64 D is negative too and the corner is background; every other corner
// takes the reference's FP64 expressions, so the frame is the same byte for byte.
struct ScreenF {
    float Y1x, Y1y, Y1z, Z1x, Z1z;
    float ax[9];  // body axes b, c, a in inertial coordinates
    float Epb, Epc, Epa, ibb, icc, A;
};

__device__ __forceinline__ bool screen_background(const ScreenF& F, int cz, int cy, int S)
{
    constexpr float u = 5.9604645e-8f;  // 2^-24
    const float fS = (float)S;
    const float z1 = (2.4f * (float)(cz - S / 2)) / fS;
    const float y1 = (2.4f * (float)(cy - S / 2)) / fS;
    const float ez1 = 4.f * u * fabsf(z1), ey1 = 4.f * u * fabsf(y1);  // 2.4f, product, quotient
    // products and sums with their error bounds
#define PM(x, ex, y, ey, z, ez) \
    const float z = (x) * (y); \
    const float ez = fabsf(x) * (ey) + fabsf(y) * (ex) + u * fabsf(z);
#define PS(x, ex, y, ey, z, ez) \
    const float z = (x) + (y); \
    const float ez = (ex) + (ey) + u * fabsf(z);
    const float eY1x = u * fabsf(F.Y1x), eY1y = u * fabsf(F.Y1y), eY1z = u * fabsf(F.Y1z);
    const float eZ1x = u * fabsf(F.Z1x), eZ1z = u * fabsf(F.Z1z);
    PM(y1, ey1, F.Y1x, eY1x, yx, eyx) PM(z1, ez1, F.Z1x, eZ1x, zx, ezx) PS(yx, eyx, zx, ezx, px, epx)
    PM(y1, ey1, F.Y1y, eY1y, py, epy)
    PM(y1, ey1, F.Y1z, eY1z, yz, eyz) PM(z1, ez1, F.Z1z, eZ1z, zz, ezz) PS(yz, eyz, zz, ezz, pz, epz)
    float pbca[3], epbca[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const float a0 = F.ax[3 * r], a1 = F.ax[3 * r + 1], a2 = F.ax[3 * r + 2];
        PM(a0, u * fabsf(a0), px, epx, t0, et0) PM(a1, u * fabsf(a1), py, epy, t1, et1)
        PM(a2, u * fabsf(a2), pz, epz, t2, et2) PS(t0, et0, t1, et1, s01, es01) PS(s01, es01, t2, et2, sr, esr)
        pbca[r] = sr;
        epbca[r] = esr;
    }
    const float pb = pbca[0], pc = pbca[1], pa = pbca[2], epb = epbca[0], epc = epbca[1], epa = epbca[2];
    const float eEpb = u * fabsf(F.Epb), eEpc = u * fabsf(F.Epc), eEpa = u * fabsf(F.Epa);
    const float eibb = u * F.ibb, eicc = u * F.icc, eA = u * fabsf(F.A);
    // B = 2 (pb Epb / b^2 + pc Epc / c^2 + pa Epa)
    PM(pb, epb, F.Epb, eEpb, b1, eb1) PM(b1, eb1, F.ibb, eibb, tb, etb)
    PM(pc, epc, F.Epc, eEpc, c1, ec1) PM(c1, ec1, F.icc, eicc, tc, etc_)
    PM(pa, epa, F.Epa, eEpa, ta, eta) PS(tb, etb, tc, etc_, s1, es1) PS(s1, es1, ta, eta, s2, es2)
    const float B = 2.f * s2, eB = 2.f * es2;
    const float Babs = 2.f * (fabsf(tb) + fabsf(tc) + fabsf(ta));
    // C = pb^2 / b^2 + pc^2 / c^2 + pa^2 - 1
    PM(pb, epb, pb, epb, q1, eq1) PM(q1, eq1, F.ibb, eibb, qb, eqb)
    PM(pc, epc, pc, epc, q2, eq2) PM(q2, eq2, F.icc, eicc, qc, eqc)
    PM(pa, epa, pa, epa, qa, eqa) PS(qb, eqb, qc, eqc, r1, er1) PS(r1, er1, qa, eqa, r2, er2)
    PS(r2, er2, -1.f, 0.f, C, eC)
    const float Cabs = qb + qc + qa + 1.f;
    // D = B^2 - 4 A C
    PM(B, eB, B, eB, BB, eBB) PM(F.A, eA, C, eC, AC, eAC) PS(BB, eBB, -4.f * AC, 4.f * eAC, D, eD)
#undef PM
#undef PS
    const float M = Babs * Babs + 4.f * fabsf(F.A) * Cabs;
    return D + 2.f * eD + 1e-12f * M < 0.f;
}

constexpr int kTileX = 32, kTileY = 8;
constexpr int kCorners = (kTileX + 1) * (kTileY + 1);
static_assert(kTileX * kTileY == kRenderTpb, "one thread per pixel of the tile");

__global__ void __launch_bounds__(kRenderTpb, 3) render_kernel(const double* __restrict__ geo, int n_frames, int S,
                                                            uint8_t* __restrict__ rgb)
{
    __shared__ double g[kAstGeo];
    __shared__ double Z1x, Z1z, Y1x, Y1y, Y1z, A_s;
    __shared__ ScreenF F;
    __shared__ double cI[kCorners];
    __shared__ uint8_t cF[kCorners];  // bit 0: the line of sight hits the ellipsoid; bit 1: red spot
    __shared__ int16_t todo[kCorners];  // corners the float pre-test leaves to FP64
    __shared__ int n_todo;
    const int f = blockIdx.y;
    const int tiles_x = (S + kTileX - 1) / kTileX;
    const int y0 = (blockIdx.x % tiles_x) * kTileX;  // first pixel column (iy) of the tile
    const int z0 = (blockIdx.x / tiles_x) * kTileY;  // first pixel row (iz)
    if (threadIdx.x < kAstGeo) g[threadIdx.x] = geo[(int64_t)kAstGeo * f + threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        // Image axes: X1 toward the observer (E), Z1 = [E x y], Y1 = [Z1 x X1] (cuda.c:2418-2427).
        const double Ex = g[2], Ey = g[3], Ez = g[4];
        const double scale = 1.0 / sqrt(A_(M_(Ex, Ex), M_(Ez, Ez)));
        Z1x = M_(-Ez, scale);
        Z1z = M_(Ex, scale);
        Y1x = M_(M_(-Ex, Ey), scale);
        Y1y = M_(A_(M_(Ex, Ex), M_(Ez, Ez)), scale);
        Y1z = M_(M_(-Ey, Ez), scale);
        // The quadratic's A depends on the frame only (cuda.c:2454).
        const double Epb = g[5], Epc = g[6], Epa = g[7], bb = M_(g[0], g[0]), cc = M_(g[1], g[1]);
        A_s = A_(A_(M_(Epb, Epb) / bb, M_(Epc, Epc) / cc), M_(Epa, Epa));
        F.Y1x = (float)Y1x; F.Y1y = (float)Y1y; F.Y1z = (float)Y1z; F.Z1x = (float)Z1x; F.Z1z = (float)Z1z;
        for (int r = 0; r < 9; r++) F.ax[r] = (float)g[11 + r];
        F.Epb = (float)Epb; F.Epc = (float)Epc; F.Epa = (float)Epa;
        F.ibb = (float)(1.0 / bb); F.icc = (float)(1.0 / cc); F.A = (float)A_s;
    }
    __syncthreads();
    {
        const double b = g[0], c = g[1];
        const double Epb = g[5], Epc = g[6], Epa = g[7], Spb = g[8], Spc = g[9], Spa = g[10];
        const double bb = M_(b, b), cc = M_(c, c), A = A_s;
        // Pass 1: the float pre-test of every corner; the undecided ones are listed.  Pass 2: the
        // CTA's threads share the listed corners evenly, so the FP64 work (clustered on the
        // asteroid's disc and silhouette) keeps whole warps busy instead of a few lanes.
        if (threadIdx.x == 0) n_todo = 0;
        __syncthreads();
        for (int k = threadIdx.x; k < kCorners; k += kRenderTpb) {
            const int cz = z0 + k / (kTileX + 1), cy = y0 + k % (kTileX + 1);  // corner (iz + jz, iy + jy)
            if (screen_background(F, cz, cy, S)) {
                cI[k] = 0.0;
                cF[k] = 0;
            } else {
                todo[atomicAdd(&n_todo, 1)] = (int16_t)k;
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < n_todo; e += kRenderTpb) {
            const int k = todo[e];
            const int cz = z0 + k / (kTileX + 1), cy = y0 + k % (kTileX + 1);
            const double z1 = 2.4 * (double)(cz - S / 2) / (double)S;
            const double y1 = 2.4 * (double)(cy - S / 2) / (double)S;
            const double p_x = A_(M_(y1, Y1x), M_(z1, Z1x));
            const double p_y = A_(M_(y1, Y1y), M_(z1, 0.0));
            const double p_z = A_(M_(y1, Y1z), M_(z1, Z1z));
            const double p_b = A_(A_(M_(g[11], p_x), M_(g[12], p_y)), M_(g[13], p_z));
            const double p_c = A_(A_(M_(g[14], p_x), M_(g[15], p_y)), M_(g[16], p_z));
            const double p_a = A_(A_(M_(g[17], p_x), M_(g[18], p_y)), M_(g[19], p_z));
            // Line of sight p + lambda E' against the ellipsoid (b, c, 1) (cuda.c:2453-2460).
            const double B = M_(2.0, A_(A_(M_(p_b, Epb) / bb, M_(p_c, Epc) / cc), M_(p_a, Epa)));
            const double C = S_(A_(A_(M_(p_b, p_b) / bb, M_(p_c, p_c) / cc), M_(p_a, p_a)), 1.0);
            const double D = S_(M_(B, B), M_(M_(4.0, A), C));
            double I = 0.0;
            uint8_t fl = 0;
            if (D >= 0.0) {
                const double sD = sqrt(D);
                double lambda = S_(-B, sD) / M_(2.0, A);
                const double lambda1 = A_(-B, sD) / M_(2.0, A);
                if (lambda1 > lambda) lambda = lambda1;
                const double ri_b = A_(p_b, M_(lambda, Epb));
                const double ri_c = A_(p_c, M_(lambda, Epc));
                const double ri_a = A_(p_a, M_(lambda, Epa));
                const bool red_spot = A_(M_(ri_c, ri_c), M_(ri_a, ri_a)) < (double)(kSpotRad * kSpotRad) && ri_b > 0.0;
                double ni_b = ri_b / bb, ni_c = ri_c / cc, ni_a = ri_a;
                const double scale = 1.0 / sqrt(A_(A_(M_(ni_b, ni_b), M_(ni_c, ni_c)), M_(ni_a, ni_a)));
                ni_b = M_(ni_b, scale);
                ni_c = M_(ni_c, scale);
                ni_a = M_(ni_a, scale);
                I = A_(A_(M_(ni_b, Spb), M_(ni_c, Spc)), M_(ni_a, Spa));
                fl = red_spot ? 3 : 1;
            }
            cI[k] = I;
            cF[k] = fl;
        }
    }
    __syncthreads();
    const int ty = threadIdx.x % kTileX, tz = threadIdx.x / kTileX;
    const int iy = y0 + ty, iz = z0 + tz;
    if (iy >= S || iz >= S) return;
    float br[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int jz = 0; jz < 2; jz++)
#pragma unroll
        for (int jy = 0; jy < 2; jy++) {
            const int k = (tz + jz) * (kTileX + 1) + ty + jy;
            const uint8_t fl = cF[k];
            if (!(fl & 1)) continue;
            const double I = cI[k];
            const bool red_spot = (fl & 2) != 0;
            // float + float + double*float, rounded back to float (cuda.c:2500-2525).
            if (I >= 0.0) {
                br[0] = (float)A_((double)(br[0] + kSmaxR), M_(I, (double)(kImaxR - kSmaxR)));
                if (!red_spot) {
                    br[1] = (float)A_((double)(br[1] + kSmaxG), M_(I, (double)(kImaxG - kSmaxG)));
                    br[2] = (float)A_((double)(br[2] + kSmaxB), M_(I, (double)(kImaxB - kSmaxB)));
                }
            } else {
                br[0] = (float)A_((double)(br[0] + kSmaxR), M_(I, (double)(kSmaxR - kSminR)));
                if (!red_spot) {
                    br[1] = (float)A_((double)(br[1] + kSmaxG), M_(I, (double)(kSmaxG - kSminG)));
                    // The reference adds to br[1] here, not br[2] (cuda.c:2523).
                    br[2] = (float)A_((double)(br[1] + kSmaxB), M_(I, (double)(kSmaxB - kSminB)));
                }
            }
        }
    uint8_t* out = rgb + 3 * ((int64_t)iy + (int64_t)S * ((int64_t)iz + (int64_t)S * f));
#pragma unroll
    for (int ic = 0; ic < 3; ic++) {
        int v = (int)((double)br[ic] / 4.0);
        v = v > 255 ? 255 : (v < 0 ? 0 : v);
        out[ic] = (uint8_t)v;
    }
}

#undef M_
#undef A_
#undef S_

struct RenderScratch {
    double* geo = nullptr;
    uint8_t* rgb = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~RenderScratch()
    {
        cudaFree(geo);
        cudaFree(rgb);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (s) cudaStreamDestroy(s);
    }
};

}  // namespace
}  // namespace ast

using namespace ast;

extern "C" int ast_render_frames(int32_t device, const double* geo, int32_t n_frames, int32_t size_pix, uint8_t* rgb,
                                 double* kernel_ms)
{
    if (!geo || !rgb || n_frames < 0 || size_pix < 2 || size_pix > 8192 || (size_pix & 1))
        return ast_set_error(AST_E_INVALID, "ast_render_frames: bad argument");
    if (kernel_ms) *kernel_ms = 0;
    if (n_frames == 0) return AST_OK;
    int rc = set_device(device);
    if (rc) return rc;
    const int64_t frame_bytes = 3ll * size_pix * size_pix;
    // Frames per launch: at most 2 GB of pixels on the device at once (the reference uses dNPLOT),
    // and at most 65 535 (the grid's y dimension).
    const int64_t chunk =
        std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(n_frames, 65535), (2ll << 30) / frame_bytes));
    RenderScratch d;
    if (cudaMalloc(&d.geo, sizeof(double) * kAstGeo * chunk) != cudaSuccess ||
        cudaMalloc(&d.rgb, (size_t)(frame_bytes * chunk)) != cudaSuccess) {
        cudaGetLastError();
        return ast_set_error(AST_E_NOMEM, "ast_render_frames: cudaMalloc failed");
    }
    AST_CUDA(cudaStreamCreateWithFlags(&d.s, cudaStreamNonBlocking));
    AST_CUDA(cudaEventCreate(&d.e0));
    AST_CUDA(cudaEventCreate(&d.e1));
    const unsigned blocks = (unsigned)(((size_pix + kTileX - 1) / kTileX) * ((size_pix + kTileY - 1) / kTileY));
    double total = 0;
    for (int64_t f0 = 0; f0 < n_frames; f0 += chunk) {
        const int64_t nf = std::min<int64_t>(chunk, n_frames - f0);
        AST_CUDA(cudaMemcpyAsync(d.geo, geo + kAstGeo * f0, sizeof(double) * kAstGeo * nf, cudaMemcpyHostToDevice, d.s));
        AST_CUDA(cudaEventRecord(d.e0, d.s));
        render_kernel<<<dim3(blocks, (unsigned)nf), kRenderTpb, 0, d.s>>>(d.geo, (int)nf, size_pix, d.rgb);
        AST_CUDA(cudaGetLastError());
        AST_CUDA(cudaEventRecord(d.e1, d.s));
        AST_CUDA(cudaMemcpyAsync(rgb + frame_bytes * f0, d.rgb, (size_t)(frame_bytes * nf), cudaMemcpyDeviceToHost, d.s));
        AST_CUDA(cudaStreamSynchronize(d.s));
        float ms = 0;
        AST_CUDA(cudaEventElapsedTime(&ms, d.e0, d.e1));
        total += ms;
    }
    if (kernel_ms) *kernel_ms = total;
    return AST_OK;
}
