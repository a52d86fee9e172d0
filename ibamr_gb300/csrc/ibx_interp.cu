// ibx_interp.cu -- interpolation of the plan pipeline (mixed precision).
//
// Markers are taken in home-tile order (the counting sort keeps consecutive
// markers of a warp together, so markers along a fibre stay adjacent).  Each
// thread handles a short chunk of consecutive markers for one component and
// keeps the W^d grid values of the current stencil in registers: markers of
// a run (same stencil base) reuse them and only evaluate their weights and
// the FP32 multiply-adds.  Sum order: V = sum_z w_z sum_y w_y sum_x w_x u,
// the separable form of the reference's w(i0,i1,i2) * u (F3D:1309-1328).

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
constexpr int INTERP_THREADS = 256;
constexpr int CHUNK = 8; // markers per thread

template <int DIM, int K>
__global__ void __launch_bounds__(INTERP_THREADS) interp_home_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int NF = DIM == 3 ? W * W * W : W * W;
    constexpr bool CACHE = NF <= 64;
    // Adjacent threads take the components of one chunk, so that the
    // chunk's records are read from DRAM once.
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int c = (int)(tid % D.max_ncomp);
    const long long total = D.hcount[D.n_tiles];
    const long long m0 = (tid / D.max_ncomp) * CHUNK;
    if (m0 >= total) return;
    const long long m1 = min(m0 + CHUNK, total);
    float u[CACHE ? NF : 1];
    int cur[3] = { -100000, -100000, -100000 };
    int curp = -1;
    for (long long m = m0; m < m1; ++m)
    {
        const int g = D.home_list[m];
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.marker_offs, D.n_probs, (long long)g);
        const PlanProb& P = D.probs[p];
        if (c >= P.ncomp) continue;
        const Rec R = D.hrec[m];
        int b[3] = { 0, 0, 0 };
        float w[3][W];
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            if (d >= DIM)
            {
                w[d][0] = 1.f;
                continue;
            }
            const bool stag = P.side && d == c;
            b[d] = stag ? R.bs(d) : R.bc(d);
            weights_f32<K>(stag ? R.rs[d] : R.rc[d], w[d]);
        }
        const float* q = static_cast<const float*>(P.qi[c]);
        const long long n0 = P.N[0], n01 = (long long)P.N[0] * P.N[1];
        const bool same = CACHE && p == curp && b[0] == cur[0] && b[1] == cur[1] && (DIM == 2 || b[2] == cur[2]);
        float V = 0.f;
        if (CACHE)
        {
            if (!same)
            {
                int co[3][W];
#pragma unroll
                for (int d = 0; d < DIM; ++d)
#pragma unroll
                    for (int i = 0; i < W; ++i) co[d][i] = wrap_cell(b[d] + i, P.N[d]);
#pragma unroll
                for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
                    {
                        const float* row = q + (DIM == 3 ? co[2][i2] * n01 : 0) + co[1][i1] * n0;
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0) u[(i2 * W + i1) * W + i0] = __ldg(row + co[0][i0]);
                    }
                cur[0] = b[0];
                cur[1] = b[1];
                cur[2] = b[2];
                curp = p;
            }
#pragma unroll
            for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
            {
                float vy = 0.f;
#pragma unroll
                for (int i1 = 0; i1 < W; ++i1)
                {
                    float vx = 0.f;
#pragma unroll
                    for (int i0 = 0; i0 < W; ++i0) vx = fmaf(w[0][i0], u[(i2 * W + i1) * W + i0], vx);
                    vy = fmaf(w[1][i1], vx, vy);
                }
                V = fmaf(DIM == 3 ? w[2][i2] : 1.f, vy, V);
            }
        }
        else
        {
            int co[3][W];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
#pragma unroll
                for (int i = 0; i < W; ++i) co[d][i] = wrap_cell(b[d] + i, P.N[d]);
#pragma unroll
            for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
            {
                float vy = 0.f;
#pragma unroll
                for (int i1 = 0; i1 < W; ++i1)
                {
                    const float* row = q + (DIM == 3 ? co[2][i2] * n01 : 0) + co[1][i1] * n0;
                    float vx = 0.f;
#pragma unroll
                    for (int i0 = 0; i0 < W; ++i0) vx = fmaf(w[0][i0], __ldg(row + co[0][i0]), vx);
                    vy = fmaf(w[1][i1], vx, vy);
                }
                V = fmaf(DIM == 3 ? w[2][i2] : 1.f, vy, V);
            }
        }
        static_cast<float*>(P.Qi)[(long long)P.Q_depth * (g - P.marker0) + c] = V;
    }
}
} // namespace

int
launch_interp(int dim, int kernel, const DevPlan& D, cudaStream_t s)
{
    const long long chunks = (D.n_markers + CHUNK - 1) / CHUNK;
    const unsigned bx = (unsigned)((chunks * D.max_ncomp + INTERP_THREADS - 1) / INTERP_THREADS);
    if (bx == 0) return IBX_OK;
    const dim3 grid(bx, 1);
#define IBX_INTERP_CASE(DD, KK)                                                                                      \
    if (dim == DD && kernel == KK)                                                                                   \
    {                                                                                                                \
        interp_home_mixed<DD, KK><<<grid, INTERP_THREADS, 0, s>>>(D);                                                \
        note_launches(1);                                                                                            \
        return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;                                             \
    }
    IBX_INTERP_CASE(2, K_PL) IBX_INTERP_CASE(2, K_PCUBIC) IBX_INTERP_CASE(2, K_IB3) IBX_INTERP_CASE(2, K_IB4)
    IBX_INTERP_CASE(2, K_IB6) IBX_INTERP_CASE(2, K_BSPL4) IBX_INTERP_CASE(3, K_PL) IBX_INTERP_CASE(3, K_PCUBIC)
    IBX_INTERP_CASE(3, K_IB3) IBX_INTERP_CASE(3, K_IB4) IBX_INTERP_CASE(3, K_IB6) IBX_INTERP_CASE(3, K_BSPL4)
#undef IBX_INTERP_CASE
    return IBX_E_BAD_KERNEL;
}

} // namespace ibx
