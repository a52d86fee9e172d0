// ibx_interp.cu -- interpolation of the plan pipeline (mixed precision).
//
// Two kernels, both in home-tile order:
//  - dense home tiles (more than dense_min markers): the work items of the
//    dense spread (item_units home units of one tile); one thread per (unit,
//    component) loads the unit's stencil values once and sums every marker
//    of the unit from registers;
//  - the other markers: each thread handles a short chunk of consecutive
//    markers for one component and keeps the W^d grid values of the current
//    stencil in registers, so markers of a run (same stencil base) reuse
//    them and only evaluate their weights and the FP32 multiply-adds.
// Sum order in both: V = sum_z w_z sum_y w_y sum_x w_x u, the separable form
// of the reference's w(i0,i1,i2) * u (F3D:1309-1328).

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
constexpr int INTERP_THREADS = 256;
constexpr int CHUNK = 8; // markers per thread

// Markers of dense home tiles, by home unit (a run of markers sharing every
// stencil base): one thread per (unit, component) of a work item loads the
// unit's W^d grid values once into registers and sums every marker of the
// unit from them, so the threads of a warp load together and then compute
// together, without divergence between cached and uncached markers.
template <int DIM, int K>
__global__ void __launch_bounds__(INTERP_THREADS) interp_units_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int NF = DIM == 3 ? W * W * W : W * W;
    constexpr bool CACHE = NF <= 64;
    if (!CACHE) return; // wider footprints are interpolated in chunks
    const int n_items = min(D.items[D.n_tiles], D.n_item_cap);
    for (int item = blockIdx.x; item < n_items; item += gridDim.x)
    {
        const int t = D.item_tile[item];
        const int k = item - D.items[t];
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        const int ncomp = P.ncomp;
        const int c = threadIdx.x % ncomp;
        const int ustep = blockDim.x / ncomp;
        if ((int)threadIdx.x >= ustep * ncomp) continue;
        const float* q = static_cast<const float*>(P.qi[c]);
        float* Qi = static_cast<float*>(P.Qi);
        const long long n0 = P.N[0], n01 = (long long)P.N[0] * P.N[1];
        for (int ul = threadIdx.x / ncomp; ul < D.item_units; ul += ustep)
        {
            const int u = D.hucount[t] + k * D.item_units + ul;
            if (u >= D.hucount[t + 1]) break;
            const int2 un = D.home_units[u];
            if (un.y <= 0) continue;
            int co[3][W];
            {
                const Rec R0 = D.hrec[un.x];
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                {
                    const int b = (P.side && d == c) ? R0.bs(d) : R0.bc(d);
#pragma unroll
                    for (int i = 0; i < W; ++i) co[d][i] = wrap_cell(b + i, P.N[d]);
                }
            }
            float uv[CACHE ? NF : 1];
            if (CACHE)
            {
#pragma unroll
                for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
                    {
                        const float* row = q + (DIM == 3 ? co[2][i2] * n01 : 0) + co[1][i1] * n0;
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0) uv[(i2 * W + i1) * W + i0] = __ldg(row + co[0][i0]);
                    }
            }
            for (int v = un.x; v < un.x + un.y; ++v)
            {
                const Rec R = D.hrec[v];
                const int g = D.home_list[v];
                float w[3][W];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                {
                    if (d >= DIM)
                    {
                        w[d][0] = 1.f;
                        continue;
                    }
                    weights_f32<K>((P.side && d == c) ? R.rs[d] : R.rc[d], w[d]);
                }
                float V = 0.f;
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
                        for (int i0 = 0; i0 < W; ++i0)
                            vx = fmaf(w[0][i0], CACHE ? uv[(i2 * W + i1) * W + i0] : __ldg(row + co[0][i0]), vx);
                        vy = fmaf(w[1][i1], vx, vy);
                    }
                    V = fmaf(DIM == 3 ? w[2][i2] : 1.f, vy, V);
                }
                Qi[(long long)P.Q_depth * (g - P.marker0) + c] = V;
            }
        }
    }
}

// The W = 4 values of a stencil row starting at cell x0 (x0 in [0, N), N a
// multiple of 4, the row 16-byte aligned): the aligned group holding x0 and,
// unless x0 is its first cell, the next group (periodically), read as two
// float4 and selected without dynamic indexing.
__device__ __forceinline__ void
row4(const float* row, int x0, int N, float* v)
{
    const int a = x0 & ~3, o = x0 & 3;
    const float4 A = __ldg(reinterpret_cast<const float4*>(row + a));
    float4 B = A;
    if (o) B = __ldg(reinterpret_cast<const float4*>(row + (a + 4 == N ? 0 : a + 4)));
    v[0] = o == 0 ? A.x : o == 1 ? A.y : o == 2 ? A.z : A.w;
    v[1] = o == 0 ? A.y : o == 1 ? A.z : o == 2 ? A.w : B.x;
    v[2] = o == 0 ? A.z : o == 1 ? A.w : o == 2 ? B.x : B.y;
    v[3] = o == 0 ? A.w : o == 1 ? B.x : o == 2 ? B.y : B.z;
}

// Markers in chunks of consecutive home-order markers: every marker, or with
// skip_dense only those of sparse home tiles.  RUNS keeps the stencil values
// of the last marker in registers for the next markers of its run (worth it
// where runs are long, i.e. when dense-homed markers are included).
template <int DIM, int K, bool RUNS>
__global__ void __launch_bounds__(INTERP_THREADS) interp_home_mixed(const DevPlan D, int skip_dense)
{
    constexpr int W = KT<K>::W;
    constexpr int NF = DIM == 3 ? W * W * W : W * W;
    constexpr bool CACHE = RUNS && NF <= 64;
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
        if (skip_dense)
        {
            const int ht = D.home_tile[g];
            if (D.hcount[ht + 1] - D.hcount[ht] > D.dense_min) continue;
        }
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
            const bool rv = W == 4 && P.vec4i;
#pragma unroll
            for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
            {
                float vy = 0.f;
#pragma unroll
                for (int i1 = 0; i1 < W; ++i1)
                {
                    const float* row = q + (DIM == 3 ? co[2][i2] * n01 : 0) + co[1][i1] * n0;
                    float vx = 0.f;
                    if (W == 4 && rv)
                    {
                        float v4[4];
                        row4(row, co[0][0], P.N[0], v4);
#pragma unroll
                        for (int i0 = 0; i0 < 4; ++i0) vx = fmaf(w[0][i0], v4[i0], vx);
                    }
                    else
                    {
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0) vx = fmaf(w[0][i0], __ldg(row + co[0][i0]), vx);
                    }
                    vy = fmaf(w[1][i1], vx, vy);
                }
                V = fmaf(DIM == 3 ? w[2][i2] : 1.f, vy, V);
            }
        }
        static_cast<float*>(P.Qi)[(long long)P.Q_depth * (g - P.marker0) + c] = V;
    }
}
} // namespace

namespace
{
template <int DIM, int K>
int
launch_interp_k(const DevPlan& D, cudaStream_t s)
{
    constexpr int NF = DIM == 3 ? KT<K>::W * KT<K>::W * KT<K>::W : KT<K>::W * KT<K>::W;
    const int skip_dense = (D.dense_interp && NF <= 64) ? 1 : 0;
    if (skip_dense)
    {
        int dev = 0, sms = 152, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, interp_units_mixed<DIM, K>, INTERP_THREADS, 0);
        if (per_sm < 1) per_sm = 1;
        const unsigned blocks = (unsigned)(D.n_item_cap < per_sm * sms ? D.n_item_cap : per_sm * sms);
        if (blocks > 0)
        {
            interp_units_mixed<DIM, K><<<blocks, INTERP_THREADS, 0, s>>>(D);
            note_launches(1);
            if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;
        }
    }
    const long long chunks = (D.n_markers + CHUNK - 1) / CHUNK;
    const unsigned bx = (unsigned)((chunks * D.max_ncomp + INTERP_THREADS - 1) / INTERP_THREADS);
    if (bx == 0) return IBX_OK;
    if (skip_dense)
        interp_home_mixed<DIM, K, false><<<bx, INTERP_THREADS, 0, s>>>(D, 1);
    else
        interp_home_mixed<DIM, K, true><<<bx, INTERP_THREADS, 0, s>>>(D, 0);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}
} // namespace

int
launch_interp(int dim, int kernel, const DevPlan& D, cudaStream_t s)
{
#define IBX_INTERP_CASE(DD, KK)                                                                                      \
    if (dim == DD && kernel == KK) return launch_interp_k<DD, KK>(D, s);
    IBX_INTERP_CASE(2, K_PL) IBX_INTERP_CASE(2, K_PCUBIC) IBX_INTERP_CASE(2, K_IB3) IBX_INTERP_CASE(2, K_IB4)
    IBX_INTERP_CASE(2, K_IB6) IBX_INTERP_CASE(2, K_BSPL4) IBX_INTERP_CASE(3, K_PL) IBX_INTERP_CASE(3, K_PCUBIC)
    IBX_INTERP_CASE(3, K_IB3) IBX_INTERP_CASE(3, K_IB4) IBX_INTERP_CASE(3, K_IB6) IBX_INTERP_CASE(3, K_BSPL4)
#undef IBX_INTERP_CASE
    return IBX_E_BAD_KERNEL;
}

} // namespace ibx
