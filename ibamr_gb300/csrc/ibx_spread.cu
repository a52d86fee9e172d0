// ibx_spread.cu -- tiled spreading of the plan pipeline (mixed precision).
//
// Two kernels, run in this order:
//  - dense home tiles (more than dense_min markers): one CTA per work item
//    (item_units home units of one tile, one thread per unit and component;
//    a unit is a run of markers sharing every stencil base, typically
//    consecutive markers of a fibre).  A unit's contributions are summed in FP32
//    registers over its whole W^d footprint and merged once, with
//    compensated shared atomics (Knuth TwoSum on the returned old value),
//    into a double-FP32 region covering the tile and its stencil halo; the
//    region is then added to the grid with FP32 global atomics (each grid
//    value receives at most 2^d region sums).  Every dense-homed marker is
//    processed exactly once.
//  - every tile visited by sparse-homed markers: one warp per tile; lanes
//    take visits and merge each in-tile contribution with compensated shared
//    atomics, then the warp adds the tile's double-FP32 sums to the grid with
//    one coalesced read-modify-write per value (compensated FP32 merge,
//    within one FP32 ulp of the exact sum).  The warp owns its tile's values;
//    the dense kernel's atomics have completed before it starts.
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
constexpr int SPARSE_WARPS = 8;    // tiles (warps) per CTA of the visit kernel

// Region of a dense home tile: the tile plus the stencil halo of every
// marker homed in it, (E + W)^d values per component.  The cell-centred
// footprint of a marker homed in the tile starts at region offset
// (home cell - tile origin) along each dim, the staggered one 0 or 1 later.
template <int DIM, int W>
struct Region
{
    static constexpr int E = TileT<DIM>::E;
    static constexpr int RE = E + W;
    static constexpr int RP = DIM == 3 ? RE * RE * RE : RE * RE;
    static constexpr int NF = DIM == 3 ? W * W * W : W * W;
    // Footprints up to 4^3 points are accumulated in registers per unit.
    static constexpr bool regs = NF <= 64;
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

// q += hi + lo for every owned value of one component of a tile: lanes take
// groups of four consecutive x values; rows lying wholly inside the grid
// are read and written as float4 when the array allows it.
template <int DIM, int E, int PTS>
__device__ __forceinline__ void
owner_flush(const PlanProb& P, const int* org, int c, const float* hi, const float* lo, int tid, int nthr)
{
    constexpr int G = PTS / 4;  // groups of 4 values
    constexpr int GR = E / 4;   // groups per row
    float* q = static_cast<float*>(P.q[c]);
    const bool row_vec = P.vec4 && org[0] + E <= P.N[0];
    for (int j = tid; j < G; j += nthr)
    {
        const float4 h = reinterpret_cast<const float4*>(hi)[j];
        const float4 l = reinterpret_cast<const float4*>(lo)[j];
        if (h.x == 0.f && h.y == 0.f && h.z == 0.f && h.w == 0.f && l.x == 0.f && l.y == 0.f && l.z == 0.f &&
            l.w == 0.f)
            continue;
        const int r = j / GR;
        const int x = org[0] + 4 * (j % GR);
        const int y = org[1] + (DIM == 3 ? r % E : r);
        const int z = DIM == 3 ? org[2] + r / E : 0;
        if (y >= P.N[1] || (DIM == 3 && z >= P.N[2])) continue;
        const long long o = x + (long long)P.N[0] * (y + (long long)P.N[1] * z);
        if (row_vec)
        {
            float4 v = *reinterpret_cast<float4*>(q + o);
            v.x = merge3(v.x, h.x, l.x);
            v.y = merge3(v.y, h.y, l.y);
            v.z = merge3(v.z, h.z, l.z);
            v.w = merge3(v.w, h.w, l.w);
            *reinterpret_cast<float4*>(q + o) = v;
        }
        else
        {
            const float hh[4] = { h.x, h.y, h.z, h.w }, ll[4] = { l.x, l.y, l.z, l.w };
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (x + e < P.N[0] && (hh[e] != 0.f || ll[e] != 0.f)) q[o + e] = merge3(q[o + e], hh[e], ll[e]);
        }
    }
}

// Region sums of one component added to the grid with FP32 atomics.
template <int DIM, int W>
__device__ __forceinline__ void
region_flush(const PlanProb& P, const int* org, int c, const float* hi, const float* lo, int tid, int nthr)
{
    using RG = Region<DIM, W>;
    float* q = static_cast<float*>(P.q[c]);
    for (int i = tid; i < RG::RP; i += nthr)
    {
        const float h = hi[i], l = lo[i];
        if (h == 0.f && l == 0.f) continue;
        const int lx = i % RG::RE;
        const int ly = (i / RG::RE) % RG::RE;
        const int lz = DIM == 3 ? i / (RG::RE * RG::RE) : 0;
        const int x = wrap_cell(org[0] - (W - 1) / 2 + lx, P.N[0]);
        const int y = wrap_cell(org[1] - (W - 1) / 2 + ly, P.N[1]);
        const int z = DIM == 3 ? wrap_cell(org[2] - (W - 1) / 2 + lz, P.N[2]) : 0;
        atomicAdd(q + x + (long long)P.N[0] * (y + (long long)P.N[1] * z), h + l);
    }
}

template <int DIM, int K>
__global__ void __launch_bounds__(UNIT_THREADS, 2) spread_home_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int E = TileT<DIM>::E;
    using RG = Region<DIM, W>;
    constexpr int RE = RG::RE;
    constexpr int RP = RG::RP;
    constexpr int NF = RG::NF;
    extern __shared__ float sm[]; // [ncomp][hi, lo][RP]
    const int n_items = D.items[D.n_tiles];
    for (int item = blockIdx.x; item < n_items && item < D.n_item_cap; item += gridDim.x)
    {
        const int t = D.item_tile[item];
        const int k = item - D.items[t];
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin(P, t - P.tile0, E, DIM, org);
        const int ncomp = P.ncomp;
        for (int i = threadIdx.x; i < ncomp * 2 * RP; i += blockDim.x) sm[i] = 0.f;
        __syncthreads();
        const float* Qf = static_cast<const float*>(P.Q);
        if (RG::regs)
        {
            // Thread -> (unit, component): the components of a unit sit in
            // adjacent lanes and read the same records.
            const int c = threadIdx.x % ncomp;
            const int ul = threadIdx.x / ncomp;
            const int u = D.hucount[t] + k * D.item_units + ul;
            const bool mine = ul < D.item_units && u < D.hucount[t + 1];
            const int2 un = mine ? D.home_units[u] : make_int2(0, 0);
            float acc[NF];
#pragma unroll
            for (int i = 0; i < NF; ++i) acc[i] = 0.f;
            int s0[3] = { 0, 0, 0 };
            if (un.y > 0)
            {
                const Rec R0 = D.hrec[un.x];
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                {
                    const int st = (P.side && d == c) ? min(max(R0.bs[d] - R0.bc[d], 0), 1) : 0; // 0 or 1
                    s0[d] = wrap_cell(R0.bc[d] + (W - 1) / 2, P.N[d]) - org[d] + st;
                }
            }
            // Markers of the unit, the next one's loads issued before the
            // current one's arithmetic.
            const int vend = un.x + un.y;
            Rec Rn;
            int gn = 0;
            if (un.y > 0)
            {
                Rn = D.hrec[un.x];
                gn = D.home_list[un.x];
            }
            for (int v = un.x; v < vend; ++v)
            {
                const Rec R = Rn;
                const int g = gn;
                const float Qv = Qf[(long long)P.Q_depth * (g - P.marker0) + c];
                if (v + 1 < vend)
                {
                    Rn = D.hrec[v + 1];
                    gn = D.home_list[v + 1];
                }
                float w[3][W];
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    weights_f32<K>((P.side && d == c) ? R.rs[d] : R.rc[d], w[d]);
                const float V = Qv * P.inv_vol;
#pragma unroll
                for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
                {
                    const float wz = DIM == 3 ? w[2][i2] * V : V;
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
                    {
                        const float wyz = w[1][i1] * wz;
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0)
                            acc[(i2 * W + i1) * W + i0] = fmaf(w[0][i0], wyz, acc[(i2 * W + i1) * W + i0]);
                    }
                }
            }
            if (un.y > 0)
            {
                float* hi = sm + (2 * c) * RP;
                float* lo = hi + RP;
#pragma unroll
                for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
                    {
                        const int row = (s0[1] + i1) * RE + (DIM == 3 ? (s0[2] + i2) * RE * RE : 0) + s0[0];
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0)
                        {
                            const float a = acc[(i2 * W + i1) * W + i0];
                            if (a != 0.f) acc2(hi + row + i0, lo + row + i0, a);
                        }
                    }
            }
        }
        else
        {
            // Wide footprints: this item's share of the tile's home markers,
            // one thread per marker, every contribution merged directly.
            const int ni = D.items[t + 1] - D.items[t];
            const long long nh = D.hcount[t + 1] - D.hcount[t];
            const int mb = D.hcount[t] + (int)(nh * k / ni);
            const int me = D.hcount[t] + (int)(nh * (k + 1) / ni);
            for (int v = mb + threadIdx.x; v < me; v += blockDim.x)
            {
                const Rec R = D.hrec[v];
                const int g = D.home_list[v];
                for (int c = 0; c < ncomp; ++c)
                {
                    float* hi = sm + (2 * c) * RP;
                    float* lo = hi + RP;
                    int s0[3] = { 0, 0, 0 };
                    float w[3][W];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        const bool st = P.side && d == c;
                        s0[d] = wrap_cell(R.bc[d] + (W - 1) / 2, P.N[d]) - org[d] +
                                (st ? min(max(R.bs[d] - R.bc[d], 0), 1) : 0);
                        weights_f32<K>(st ? R.rs[d] : R.rc[d], w[d]);
                    }
                    const float V = Qf[(long long)P.Q_depth * (g - P.marker0) + c] * P.inv_vol;
#pragma unroll
                    for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
                    {
                        const float wz = DIM == 3 ? w[2][i2] * V : V;
#pragma unroll
                        for (int i1 = 0; i1 < W; ++i1)
                        {
                            const float wyz = w[1][i1] * wz;
                            const int row = (s0[1] + i1) * RE + (DIM == 3 ? (s0[2] + i2) * RE * RE : 0) + s0[0];
#pragma unroll
                            for (int i0 = 0; i0 < W; ++i0) acc2(hi + row + i0, lo + row + i0, w[0][i0] * wyz);
                        }
                    }
                }
            }
        }
        __syncthreads();
        for (int c = 0; c < ncomp; ++c)
            region_flush<DIM, W>(P, org, c, sm + (2 * c) * RP, sm + (2 * c + 1) * RP, threadIdx.x, blockDim.x);
        __syncthreads();
    }
}

// Visits of sparse-homed markers: one warp per tile, components one after another.  The warp
// owns a private double-FP32 accumulator for one component of its tile;
// lanes take visits and merge every contribution with compensated shared
// atomics (lanes whose footprints overlap are serialised by the atomics);
// the warp then adds the component to the grid with coalesced FP64 RMWs.
template <int DIM, int K>
__global__ void __launch_bounds__(32 * SPARSE_WARPS) spread_visits_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    constexpr int E = TileT<DIM>::E;
    constexpr int PTS = TileT<DIM>::PTS;
    extern __shared__ float sm[]; // [SPARSE_WARPS][hi, lo][PTS]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * SPARSE_WARPS + warp;
    if (t >= D.n_tiles) return;
    const int vbeg = D.vcount[t];
    const int vend = (long long)D.vcount[t + 1] < D.n_visit_cap ? D.vcount[t + 1] : (int)D.n_visit_cap;
    if (vend <= vbeg) return;
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
        owner_flush<DIM, E, PTS>(P, org, c, hi, lo, lane, 32);
        __syncwarp();
    }
}
} // namespace

int
launch_spread(int dim, int kernel, const DevPlan& D, int max_ncomp, cudaStream_t s)
{
    if (D.n_tiles == 0) return IBX_OK;
    const int pts = dim == 3 ? TileT<3>::PTS : TileT<2>::PTS;
    const size_t smem_sparse = sizeof(float) * 2 * pts * SPARSE_WARPS;
    const unsigned sparse_blocks = (unsigned)((D.n_tiles + SPARSE_WARPS - 1) / SPARSE_WARPS);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = D.dense_blocks_per_sm > 0 ? D.dense_blocks_per_sm : 2;
    const unsigned dense_blocks = (unsigned)(D.n_item_cap < per_sm * sms ? D.n_item_cap : per_sm * sms);
#define IBX_SPREAD_CASE(DD, KK)                                                                                      \
    if (dim == DD && kernel == KK)                                                                                   \
    {                                                                                                                \
        const size_t smem = sizeof(float) * 2 * Region<DD, KT<KK>::W>::RP * max_ncomp;                               \
        if (smem > 48 * 1024 &&                                                                                      \
            cudaFuncSetAttribute(spread_home_mixed<DD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,             \
                                 (int)smem) != cudaSuccess)                                                          \
            return IBX_E_CUDA;                                                                                       \
        if (dense_blocks > 0)                                                                                        \
        {                                                                                                            \
            spread_home_mixed<DD, KK><<<dense_blocks, UNIT_THREADS, smem, s>>>(D);                                   \
            note_launches(1);                                                                                        \
            if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;                                               \
        }                                                                                                            \
        if (smem_sparse > 48 * 1024 &&                                                                               \
            cudaFuncSetAttribute(spread_visits_mixed<DD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                 (int)smem_sparse) != cudaSuccess)                                                   \
            return IBX_E_CUDA;                                                                                       \
        spread_visits_mixed<DD, KK><<<sparse_blocks, 32 * SPARSE_WARPS, smem_sparse, s>>>(D);                        \
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
