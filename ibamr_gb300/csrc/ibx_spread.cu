// ibx_spread.cu -- tiled spreading of the plan pipeline (mixed precision).
//
// One CTA per work item (a tile's visit list, split into items of at most
// item_visits visits).  The CTA owns the tile's grid values in shared memory
// as double-FP32 pairs (hi, lo).  Each thread walks a contiguous chunk of
// the item's visits; consecutive visits with the same stencil base (a "run":
// markers of a fibre that share a half-cell) are summed in FP32 registers
// over the whole W^d footprint, and each run is merged into the tile with
// compensated shared atomics (Knuth TwoSum on the returned old value).  The
// flush adds hi + lo to the grid in FP64 with one coalesced read-modify-
// write per owned value, rounded once to FP32; tiles split into several
// items merge their partial sums with FP32 atomics instead.
//
// Product order per contribution: w0 * (w1 * (w2 * (Q/vol))), as in the
// reference's tensor-product kernels (F3D:1436-1468).

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
constexpr int SPREAD_THREADS = 256;
constexpr int SPARSE_MAX = 96;     // tiles with at most this many visits take the warp-per-tile kernel
constexpr int SPARSE_WARPS = 8;    // tiles (warps) per CTA of the sparse kernel

template <int DIM, int W>
struct Foot
{
    static constexpr int n = DIM == 3 ? W * W * W : W * W;
    // Footprints up to 4^3 points are accumulated in registers.
    static constexpr bool regs = n <= 64;
};

// Merge one run (footprint accumulator acc at base b) into the tile.
template <int DIM, int W>
__device__ __forceinline__ void
flush_run(const float* acc, const int* b, const int* org, const int* N, float* hi, float* lo)
{
    constexpr int E = TileT<DIM>::E;
    int li[3][W];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        if (d >= DIM) continue;
#pragma unroll
        for (int i = 0; i < W; ++i)
        {
            const int l = wrap_cell(b[d] + i, N[d]) - org[d];
            li[d][i] = (l >= 0 && l < E) ? l : -1;
        }
    }
#pragma unroll
    for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
    {
        if (DIM == 3 && li[2][i2] < 0) continue;
        const int zo = DIM == 3 ? li[2][i2] * E * E : 0;
#pragma unroll
        for (int i1 = 0; i1 < W; ++i1)
        {
            if (li[1][i1] < 0) continue;
            const int row = zo + li[1][i1] * E;
#pragma unroll
            for (int i0 = 0; i0 < W; ++i0)
            {
                if (li[0][i0] < 0) continue;
                const float v = acc[(i2 * W + i1) * W + i0];
                if (v != 0.f) acc2(hi + row + li[0][i0], lo + row + li[0][i0], v);
            }
        }
    }
}

template <int DIM, int K>
__global__ void __launch_bounds__(SPREAD_THREADS, 2) spread_items_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int E = TileT<DIM>::E;
    constexpr int PTS = TileT<DIM>::PTS;
    constexpr int NF = Foot<DIM, W>::n;
    extern __shared__ float sm[]; // [ncomp][hi, lo][PTS]
    const int item = blockIdx.x;
    if (item >= D.items[D.n_tiles] || item >= D.n_item_cap) return;
    const int t = D.item_tile[item];
    if (D.vcount[t + 1] - D.vcount[t] <= SPARSE_MAX) return; // warp-per-tile kernel
    const int k = item - D.items[t];
    const bool split = D.items[t + 1] - D.items[t] > 1;
    const int vbeg = D.vcount[t] + k * D.item_visits;
    const int vend = min(vbeg + D.item_visits, D.vcount[t + 1]);
    const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
    const PlanProb& P = D.probs[p];
    const int lt = t - P.tile0;
    const int org[3] = { (lt % P.ntile[0]) * E, ((lt / P.ntile[0]) % P.ntile[1]) * E,
                         DIM == 3 ? (lt / (P.ntile[0] * P.ntile[1])) * E : 0 };
    const int ncomp = P.ncomp;
    for (int i = threadIdx.x; i < ncomp * 2 * PTS; i += blockDim.x) sm[i] = 0.f;
    __syncthreads();
    const float* Qf = static_cast<const float*>(P.Q);
    const int n = vend - vbeg;
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int my0 = vbeg + threadIdx.x * per;
    const int my1 = min(my0 + per, vend);
    for (int c = 0; c < ncomp; ++c)
    {
        float* hi = sm + (2 * c) * PTS;
        float* lo = hi + PTS;
        float acc[NF];
        int cur[3] = { -100000, -100000, -100000 };
        bool have = false;
        for (int v = my0; v < my1; ++v)
        {
            const int g = D.visit_list[v];
            const Rec R = D.rec[g];
            int b[3] = { 0, 0, 0 };
            float w[3][W];
#pragma unroll
            for (int d = 0; d < 3; ++d)
            {
                if (d >= DIM) continue;
                const bool stag = P.side && d == c;
                b[d] = stag ? R.bs[d] : R.bc[d];
                weights_f32<K>(stag ? R.rs[d] : R.rc[d], w[d]);
            }
            const float V = Qf[(long long)P.Q_depth * (g - P.marker0) + c] * P.inv_vol;
            if (Foot<DIM, W>::regs)
            {
                const bool same = have && b[0] == cur[0] && b[1] == cur[1] && (DIM == 2 || b[2] == cur[2]);
                if (!same)
                {
                    if (have) flush_run<DIM, W>(acc, cur, org, P.N, hi, lo);
#pragma unroll
                    for (int i = 0; i < NF; ++i) acc[i] = 0.f;
                    cur[0] = b[0];
                    cur[1] = b[1];
                    cur[2] = b[2];
                    have = true;
                }
#pragma unroll
                for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
                {
                    const float wz = DIM == 3 ? w[2][i2] * V : V;
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
                    {
                        const float wyz = w[1][i1] * wz;
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0) acc[(i2 * W + i1) * W + i0] = fmaf(w[0][i0], wyz, acc[(i2 * W + i1) * W + i0]);
                    }
                }
            }
            else
            {
                // Wide footprints: per-contribution compensated merge.
                int li[3][W];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                {
                    if (d >= DIM) continue;
#pragma unroll
                    for (int i = 0; i < W; ++i)
                    {
                        const int l = wrap_cell(b[d] + i, P.N[d]) - org[d];
                        li[d][i] = (l >= 0 && l < E) ? l : -1;
                    }
                }
#pragma unroll
                for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
                {
                    if (DIM == 3 && li[2][i2] < 0) continue;
                    const float wz = DIM == 3 ? w[2][i2] * V : V;
                    const int zo = DIM == 3 ? li[2][i2] * E * E : 0;
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
                    {
                        if (li[1][i1] < 0) continue;
                        const float wyz = w[1][i1] * wz;
                        const int row = zo + li[1][i1] * E;
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0)
                        {
                            if (li[0][i0] < 0) continue;
                            acc2(hi + row + li[0][i0], lo + row + li[0][i0], w[0][i0] * wyz);
                        }
                    }
                }
            }
        }
        if (Foot<DIM, W>::regs && have) flush_run<DIM, W>(acc, cur, org, P.N, hi, lo);
    }
    __syncthreads();
    // Owner flush.
    for (int c = 0; c < ncomp; ++c)
    {
        float* q = static_cast<float*>(P.q[c]);
        const float* hi = sm + (2 * c) * PTS;
        const float* lo = hi + PTS;
        for (int i = threadIdx.x; i < PTS; i += blockDim.x)
        {
            const int x = org[0] + i % E;
            const int y = org[1] + (i / E) % E;
            const int z = DIM == 3 ? org[2] + i / (E * E) : 0;
            if (x >= P.N[0] || y >= P.N[1] || (DIM == 3 && z >= P.N[2])) continue;
            const float h = hi[i], l = lo[i];
            if (h == 0.f && l == 0.f) continue;
            const long long o = x + (long long)P.N[0] * (y + (long long)P.N[1] * z);
            if (split)
                atomicAdd(q + o, (float)((double)h + (double)l));
            else
                q[o] = (float)((double)q[o] + ((double)h + (double)l));
        }
    }
}
// Sparse tiles: one warp per tile, components one after another.  The warp
// owns a private double-FP32 accumulator for one component of its tile;
// lanes take visits and merge every contribution with compensated shared
// atomics (lanes whose footprints overlap are serialised by the atomics);
// the warp then adds the component to the grid with coalesced FP64 RMWs.
template <int DIM, int K>
__global__ void __launch_bounds__(32 * SPARSE_WARPS) spread_sparse_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int E = TileT<DIM>::E;
    constexpr int PTS = TileT<DIM>::PTS;
    extern __shared__ float sm[]; // [SPARSE_WARPS][hi, lo][PTS]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * SPARSE_WARPS + warp;
    if (t >= D.n_tiles) return;
    const int vbeg = D.vcount[t], vend = D.vcount[t + 1];
    if (vend == vbeg || vend - vbeg > SPARSE_MAX) return;
    const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
    const PlanProb& P = D.probs[p];
    const int lt = t - P.tile0;
    const int org[3] = { (lt % P.ntile[0]) * E, ((lt / P.ntile[0]) % P.ntile[1]) * E,
                         DIM == 3 ? (lt / (P.ntile[0] * P.ntile[1])) * E : 0 };
    float* hi = sm + warp * 2 * PTS;
    float* lo = hi + PTS;
    const float* Qf = static_cast<const float*>(P.Q);
    for (int c = 0; c < P.ncomp; ++c)
    {
        for (int i = lane; i < 2 * PTS; i += 32) hi[i] = 0.f;
        __syncwarp();
        for (int v = vbeg + lane; v < vend; v += 32)
        {
            const int g = D.visit_list[v];
            const Rec R = D.rec[g];
            float w[3][W];
            int li[3][W];
#pragma unroll
            for (int d = 0; d < 3; ++d)
            {
                if (d >= DIM) continue;
                const bool stag = P.side && d == c;
                const int b = stag ? R.bs[d] : R.bc[d];
                weights_f32<K>(stag ? R.rs[d] : R.rc[d], w[d]);
#pragma unroll
                for (int i = 0; i < W; ++i)
                {
                    const int l = wrap_cell(b + i, P.N[d]) - org[d];
                    li[d][i] = (l >= 0 && l < E) ? l : -1;
                }
            }
            const float V = Qf[(long long)P.Q_depth * (g - P.marker0) + c] * P.inv_vol;
#pragma unroll
            for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
            {
                if (DIM == 3 && li[2][i2] < 0) continue;
                const float wz = DIM == 3 ? w[2][i2] * V : V;
                const int zo = DIM == 3 ? li[2][i2] * E * E : 0;
#pragma unroll
                for (int i1 = 0; i1 < W; ++i1)
                {
                    if (li[1][i1] < 0) continue;
                    const float wyz = w[1][i1] * wz;
                    const int row = zo + li[1][i1] * E;
#pragma unroll
                    for (int i0 = 0; i0 < W; ++i0)
                    {
                        if (li[0][i0] < 0) continue;
                        acc2(hi + row + li[0][i0], lo + row + li[0][i0], w[0][i0] * wyz);
                    }
                }
            }
        }
        __syncwarp();
        float* q = static_cast<float*>(P.q[c]);
        for (int i = lane; i < PTS; i += 32)
        {
            const float h = hi[i], l = lo[i];
            if (h == 0.f && l == 0.f) continue;
            const int x = org[0] + i % E;
            const int y = org[1] + (i / E) % E;
            const int z = DIM == 3 ? org[2] + i / (E * E) : 0;
            if (x >= P.N[0] || y >= P.N[1] || (DIM == 3 && z >= P.N[2])) continue;
            const long long o = x + (long long)P.N[0] * (y + (long long)P.N[1] * z);
            q[o] = (float)((double)q[o] + ((double)h + (double)l));
        }
        __syncwarp();
    }
}
} // namespace

int
launch_spread(int dim, int kernel, const DevPlan& D, int max_ncomp, cudaStream_t s)
{
    if (D.n_tiles == 0 || D.n_item_cap == 0) return IBX_OK;
    const int pts = dim == 3 ? TileT<3>::PTS : TileT<2>::PTS;
    const size_t smem = sizeof(float) * 2 * pts * max_ncomp;
    const size_t smem_sparse = sizeof(float) * 2 * pts * SPARSE_WARPS;
    const unsigned sparse_blocks = (unsigned)((D.n_tiles + SPARSE_WARPS - 1) / SPARSE_WARPS);
#define IBX_SPREAD_CASE(DD, KK)                                                                                      \
    if (dim == DD && kernel == KK)                                                                                   \
    {                                                                                                                \
        spread_items_mixed<DD, KK><<<D.n_item_cap, SPREAD_THREADS, smem, s>>>(D);                                    \
        if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;                                                   \
        if (smem_sparse > 48 * 1024 &&                                                                               \
            cudaFuncSetAttribute(spread_sparse_mixed<DD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                 (int)smem_sparse) != cudaSuccess)                                                   \
            return IBX_E_CUDA;                                                                                       \
        spread_sparse_mixed<DD, KK><<<sparse_blocks, 32 * SPARSE_WARPS, smem_sparse, s>>>(D);                        \
        return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;                                             \
    }
    IBX_SPREAD_CASE(2, K_PL) IBX_SPREAD_CASE(2, K_PCUBIC) IBX_SPREAD_CASE(2, K_IB3) IBX_SPREAD_CASE(2, K_IB4)
    IBX_SPREAD_CASE(2, K_IB6) IBX_SPREAD_CASE(2, K_BSPL4) IBX_SPREAD_CASE(3, K_PL) IBX_SPREAD_CASE(3, K_PCUBIC)
    IBX_SPREAD_CASE(3, K_IB3) IBX_SPREAD_CASE(3, K_IB4) IBX_SPREAD_CASE(3, K_IB6) IBX_SPREAD_CASE(3, K_BSPL4)
#undef IBX_SPREAD_CASE
    return IBX_E_BAD_KERNEL;
}

} // namespace ibx
