// ibx_spread.cu -- tiled spreading of the plan pipeline (mixed precision).
//
// Every tile's grid values are owned by exactly one CTA (or one warp), which
// accumulates the clipped footprints of all markers visiting the tile in
// shared memory as double-FP32 pairs (hi, lo) and then adds hi + lo to the
// grid with one coalesced read-modify-write per value (compensated FP32
// merge, within one FP32 ulp of the exact sum).  No global atomics and no halo exchange between CTAs, except that
// tiles split into several work items merge their partial sums with FP32
// atomics.
//
// Two kernels:
//  - dense tiles (more than SPARSE_MAX_VISITS visits): one thread per unit
//    (a run of visits sharing every stencil base, typically consecutive
//    markers of a fibre); the unit's contributions are summed in FP32
//    registers over the whole W^d footprint and merged into the tile once,
//    with compensated shared atomics (Knuth TwoSum on the returned old
//    value).  Work items of item_units units, grid-stride over items.
//  - sparse tiles: one warp per tile, lanes take visits and merge each
//    contribution with compensated shared atomics.
//
// Product order per contribution: w0 * (w1 * (w2 * (Q/vol))), the
// association of the reference's tensor-product kernels (F3D:1436-1468).

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
constexpr int UNIT_THREADS = 256;  // threads (units) per dense work item
constexpr int SPARSE_WARPS = 8;    // tiles (warps) per CTA of the sparse kernel

template <int DIM, int W>
struct Foot
{
    static constexpr int n = DIM == 3 ? W * W * W : W * W;
    // Footprints up to 4^3 points are accumulated in registers, two
    // z-planes per pass in 3D.
    static constexpr bool regs = n <= 64;
    static constexpr int NZ = DIM == 3 ? (W % 2 == 0 ? W / 2 : W) : 1;
    static constexpr int passes = DIM == 3 ? W / NZ : 1;
    static constexpr int nacc = NZ * W * W;
};

__device__ __forceinline__ void
tile_origin(const PlanProb& P, int lt, int E, int dim, int* org)
{
    org[0] = (lt % P.ntile[0]) * E;
    org[1] = ((lt / P.ntile[0]) % P.ntile[1]) * E;
    org[2] = dim == 3 ? (lt / (P.ntile[0] * P.ntile[1])) * E : 0;
}

// Local tile index of stencil point i along each dim, or -1 outside the tile.
template <int DIM, int W, int E>
__device__ __forceinline__ void
local_index(const int* b, const int* org, const int* N, int (*li)[W])
{
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
        for (int i = 0; i < W; ++i)
        {
            const int l = wrap_cell(b[d] + i, N[d]) - org[d];
            li[d][i] = (l >= 0 && l < E) ? l : -1;
        }
}

// q + hi + lo rounded to FP32 without FP64 arithmetic (GB300 runs FP64 at a
// small fraction of the FP32 rate): s + e = q + hi exactly (Knuth TwoSum),
// then s + (e + lo); the result is within one FP32 ulp of the exact sum.
__device__ __forceinline__ float
merge3(float q, float h, float l)
{
    const float s = q + h;
    const float bp = s - q;
    const float e = (q - (s - bp)) + (h - bp);
    return s + (e + l);
}

// q += hi + lo for every owned value of one component.
template <int DIM, int E, int PTS>
__device__ __forceinline__ void
owner_flush(const PlanProb& P, const int* org, int c, const float* hi, const float* lo, bool split, int tid, int nthr)
{
    float* q = static_cast<float*>(P.q[c]);
    for (int i = tid; i < PTS; i += nthr)
    {
        const float h = hi[i], l = lo[i];
        if (h == 0.f && l == 0.f) continue;
        const int x = org[0] + i % E;
        const int y = org[1] + (i / E) % E;
        const int z = DIM == 3 ? org[2] + i / (E * E) : 0;
        if (x >= P.N[0] || y >= P.N[1] || (DIM == 3 && z >= P.N[2])) continue;
        const long long o = x + (long long)P.N[0] * (y + (long long)P.N[1] * z);
        if (split)
            atomicAdd(q + o, h + l);
        else
            q[o] = merge3(q[o], h, l);
    }
}

template <int DIM, int K>
__global__ void __launch_bounds__(UNIT_THREADS) spread_units_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int E = TileT<DIM>::E;
    constexpr int PTS = TileT<DIM>::PTS;
    constexpr int NZ = Foot<DIM, W>::NZ;
    constexpr int NA = Foot<DIM, W>::nacc;
    extern __shared__ float sm[]; // [ncomp][hi, lo][PTS]
    const int n_items = D.items[D.n_tiles];
    for (int item = blockIdx.x; item < n_items && item < D.n_item_cap; item += gridDim.x)
    {
        const int t = D.item_tile[item];
        const int k = item - D.items[t];
        const bool split = D.items[t + 1] - D.items[t] > 1;
        const int u0 = D.ucount[t] + k * D.item_units;
        const int u1 = min(u0 + D.item_units, D.ucount[t + 1]);
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin(P, t - P.tile0, E, DIM, org);
        const int ncomp = P.ncomp;
        for (int i = threadIdx.x; i < ncomp * 2 * PTS; i += blockDim.x) sm[i] = 0.f;
        __syncthreads();
        const float* Qf = static_cast<const float*>(P.Q);
        const int u = u0 + threadIdx.x;
        const int2 un = u < u1 ? D.units[u] : make_int2(0, 0);
        int bc[3] = { 0, 0, 0 }, bs[3] = { 0, 0, 0 };
        if (un.y > 0)
        {
            const Rec R0 = D.rec[D.visit_list[un.x]];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
            {
                bc[d] = R0.bc[d];
                bs[d] = R0.bs[d];
            }
        }
        for (int c = 0; c < ncomp; ++c)
        {
            float* hi = sm + (2 * c) * PTS;
            float* lo = hi + PTS;
            int b[3] = { 0, 0, 0 };
#pragma unroll
            for (int d = 0; d < DIM; ++d) b[d] = (P.side && d == c) ? bs[d] : bc[d];
            int li[3][W];
            local_index<DIM, W, E>(b, org, P.N, li);
#pragma unroll
            for (int pass = 0; pass < Foot<DIM, W>::passes; ++pass)
            {
                const int z0 = pass * NZ;
                float acc[NA];
#pragma unroll
                for (int i = 0; i < NA; ++i) acc[i] = 0.f;
                for (int v = un.x; v < un.x + un.y; ++v)
                {
                    const int g = D.visit_list[v];
                    const Rec R = D.rec[g];
                    float w[3][W];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        weights_f32<K>((P.side && d == c) ? R.rs[d] : R.rc[d], w[d]);
                    const float V = Qf[(long long)P.Q_depth * (g - P.marker0) + c] * P.inv_vol;
#pragma unroll
                    for (int j2 = 0; j2 < NZ; ++j2)
                    {
                        const float wz = DIM == 3 ? w[2][z0 + j2] * V : V;
#pragma unroll
                        for (int i1 = 0; i1 < W; ++i1)
                        {
                            const float wyz = w[1][i1] * wz;
#pragma unroll
                            for (int i0 = 0; i0 < W; ++i0)
                                acc[(j2 * W + i1) * W + i0] = fmaf(w[0][i0], wyz, acc[(j2 * W + i1) * W + i0]);
                        }
                    }
                }
                if (un.y > 0)
                {
#pragma unroll
                    for (int j2 = 0; j2 < NZ; ++j2)
                    {
                        const int i2 = z0 + j2;
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
                                const float a = acc[(j2 * W + i1) * W + i0];
                                if (a != 0.f) acc2(hi + row + li[0][i0], lo + row + li[0][i0], a);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
        for (int c = 0; c < ncomp; ++c)
            owner_flush<DIM, E, PTS>(P, org, c, sm + (2 * c) * PTS, sm + (2 * c + 1) * PTS, split, threadIdx.x,
                                     blockDim.x);
        __syncthreads();
    }
}

// Footprints wider than the register accumulator (IB_6 in 3D): one thread
// per visit of the dense tile, every contribution merged with a compensated
// shared atomic.
template <int DIM, int K>
__global__ void __launch_bounds__(UNIT_THREADS) spread_visits_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int E = TileT<DIM>::E;
    constexpr int PTS = TileT<DIM>::PTS;
    extern __shared__ float sm[];
    const int n_items = D.items[D.n_tiles];
    for (int item = blockIdx.x; item < n_items && item < D.n_item_cap; item += gridDim.x)
    {
        const int t = D.item_tile[item];
        const int k = item - D.items[t];
        const bool split = D.items[t + 1] - D.items[t] > 1;
        const int u0 = D.ucount[t] + k * D.item_units;
        const int u1 = min(u0 + D.item_units, D.ucount[t + 1]);
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin(P, t - P.tile0, E, DIM, org);
        const int ncomp = P.ncomp;
        for (int i = threadIdx.x; i < ncomp * 2 * PTS; i += blockDim.x) sm[i] = 0.f;
        __syncthreads();
        const float* Qf = static_cast<const float*>(P.Q);
        // This item's share of the tile's visit range.
        const int ni = D.items[t + 1] - D.items[t];
        const long long nv = D.vcount[t + 1] - D.vcount[t];
        const int vb = D.vcount[t] + (int)(nv * k / ni);
        const int ve = D.vcount[t] + (int)(nv * (k + 1) / ni);
        (void)u0;
        (void)u1;
        {
            for (int v = vb + threadIdx.x; v < ve; v += blockDim.x)
            {
                const int g = D.visit_list[v];
                const Rec R = D.rec[g];
                for (int c = 0; c < ncomp; ++c)
                {
                    float* hi = sm + (2 * c) * PTS;
                    float* lo = hi + PTS;
                    int b[3] = { 0, 0, 0 };
                    float w[3][W];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        const bool stag = P.side && d == c;
                        b[d] = stag ? R.bs[d] : R.bc[d];
                        weights_f32<K>(stag ? R.rs[d] : R.rc[d], w[d]);
                    }
                    int li[3][W];
                    local_index<DIM, W, E>(b, org, P.N, li);
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
            }
        }
        __syncthreads();
        for (int c = 0; c < ncomp; ++c)
            owner_flush<DIM, E, PTS>(P, org, c, sm + (2 * c) * PTS, sm + (2 * c + 1) * PTS, split, threadIdx.x,
                                     blockDim.x);
        __syncthreads();
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
    if (vend == vbeg || vend - vbeg > SPARSE_MAX_VISITS) return;
    const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
    const PlanProb& P = D.probs[p];
    int org[3];
    tile_origin(P, t - P.tile0, E, DIM, org);
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
            int b[3] = { 0, 0, 0 };
#pragma unroll
            for (int d = 0; d < DIM; ++d)
            {
                const bool stag = P.side && d == c;
                b[d] = stag ? R.bs[d] : R.bc[d];
                weights_f32<K>(stag ? R.rs[d] : R.rc[d], w[d]);
            }
            int li[3][W];
            local_index<DIM, W, E>(b, org, P.N, li);
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
        owner_flush<DIM, E, PTS>(P, org, c, hi, lo, false, lane, 32);
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
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned dense_blocks = (unsigned)(D.n_item_cap < 4 * sms ? D.n_item_cap : 4 * sms);
#define IBX_SPREAD_CASE(DD, KK)                                                                                      \
    if (dim == DD && kernel == KK)                                                                                   \
    {                                                                                                                \
        if (Foot<DD, KT<KK>::W>::regs)                                                                               \
            spread_units_mixed<DD, KK><<<dense_blocks, UNIT_THREADS, smem, s>>>(D);                                  \
        else                                                                                                         \
            spread_visits_mixed<DD, KK><<<dense_blocks, UNIT_THREADS, smem, s>>>(D);                                 \
        note_launches(1);                                                                                            \
        if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;                                                   \
        if (smem_sparse > 48 * 1024 &&                                                                               \
            cudaFuncSetAttribute(spread_sparse_mixed<DD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                 (int)smem_sparse) != cudaSuccess)                                                   \
            return IBX_E_CUDA;                                                                                       \
        spread_sparse_mixed<DD, KK><<<sparse_blocks, 32 * SPARSE_WARPS, smem_sparse, s>>>(D);                        \
        note_launches(1);                                                                                            \
        return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;                                             \
    }
    IBX_SPREAD_CASE(2, K_PL) IBX_SPREAD_CASE(2, K_PCUBIC) IBX_SPREAD_CASE(2, K_IB3) IBX_SPREAD_CASE(2, K_IB4)
    IBX_SPREAD_CASE(2, K_IB6) IBX_SPREAD_CASE(2, K_BSPL4) IBX_SPREAD_CASE(3, K_PL) IBX_SPREAD_CASE(3, K_PCUBIC)
    IBX_SPREAD_CASE(3, K_IB3) IBX_SPREAD_CASE(3, K_IB4) IBX_SPREAD_CASE(3, K_IB6) IBX_SPREAD_CASE(3, K_BSPL4)
#undef IBX_SPREAD_CASE
    return IBX_E_BAD_KERNEL;
}

} // namespace ibx
