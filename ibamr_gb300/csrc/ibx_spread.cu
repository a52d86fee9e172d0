// ibx_spread.cu -- tiled spreading of the plan pipeline (mixed precision).
//
// Two kernels, run in this order:
//  - dense home tiles (more than dense_min markers): one CTA per work item
//    (item_units home units of one tile, sorted by length; one thread per
//    unit, component and z-slice of the footprint; a unit is a run of
//    markers sharing every stencil base, typically consecutive markers of a
//    fibre).  A unit's contributions are summed in FP32 registers over its
//    footprint and merged once, with compensated shared atomics (Knuth
//    TwoSum on the returned old value), into a double-FP32 region covering
//    the tile and its stencil halo; the region is then added to the grid
//    with FP32 global atomics (each grid value receives at most 2^d region
//    sums).  Every dense-homed marker is processed exactly once.
//  - every tile visited by sparse-homed markers: one warp per tile, in one
//    of three forms (ibx_plan_set_visit_kernel): the tile gathered in
//    registers from the visits' separable weights (form 2), or the visits'
//    in-tile points merged with compensated shared atomics (forms 0 and 1).
//    The warp then adds the tile's double-FP32 sums to the grid with one
//    coalesced read-modify-write per value (compensated FP32 merge, within
//    one FP32 ulp of the exact sum).  The warp owns its tile's values; the
//    dense kernel's atomics have completed before it starts.
//
// Product order per contribution: w0 * (w1 * (w2 * (Q/vol))), the
// association of the reference's tensor-product kernels (F3D:1436-1468).

#include "ibx_interp_body.cuh" // the interpolation bodies the fused step kernel runs
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
constexpr int UNIT_THREADS = 256;  // threads (units) per dense work item
constexpr int MAX_ITEM_UNITS = 256; // largest item_units ibx_plan_set_tuning accepts
constexpr int SPARSE_WARPS = 8;    // tiles (warps) per CTA of the visit kernel

// Two FP32 lanes in one 64-bit register: {lo, hi} = {first, second}.
__device__ __forceinline__ unsigned long long
pack2(float a, float b)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ void
unpack2(unsigned long long r, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}

// d = a * b + c on both FP32 lanes, each rounded once (as fmaf).
__device__ __forceinline__ unsigned long long
fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Smallest v >= n with v = r (mod m).
__host__ __device__ constexpr int
pad_to(int n, int m, int r)
{
    return n + ((r - n % m) % m + m) % m;
}

// Region of a dense home tile: the tile plus the stencil halo of every
// marker homed in it, (E_d + W) values along each dim per component.  The
// cell-centred footprint of a marker homed in the tile starts at region
// offset (home cell - tile origin) along each dim, the staggered one 0 or 1
// later.
template <int DIM, int W, int SH>
struct Region
{
    using T = TileT<DIM, SH>;
    static constexpr int R0 = T::E0 + W;
    static constexpr int R1 = T::E1 + W;
    static constexpr int R2 = DIM == 3 ? T::E2 + W : 1;
    static constexpr int RP = R0 * R1 * R2;
    static constexpr int NF = DIM == 3 ? W * W * W : W * W;
    // A unit's footprint is accumulated in registers, split over ZS threads
    // along z, when a thread's share is at most 64 points (every kernel).
    static constexpr int ZS = dense_zsplit(DIM, W);
    static constexpr int NZ = (DIM == 3 ? W : 1) / ZS; // z-planes per thread
    static constexpr int NA = NZ * W * W;              // accumulators per thread
    static constexpr bool regs = NA <= 64;
    // Padded shared-memory layout: x + R0*y + PSR*z within a component;
    // the threads of one unit (its components and z-halves) start 4 banks
    // apart per z-half (with NZ = 2: PSR = 2 mod 32) and 8 banks apart per
    // component (CSTR = 8 mod 32), so their atomics do not collide.
    static constexpr int PSR = (DIM == 3 && ZS == 2) ? pad_to(R0 * R1, 32, 2) : R0 * R1;
    static constexpr int PAD = R2 * PSR;                 // words of one hi (or lo) block
    static constexpr int CSTR = pad_to(2 * PAD, 32, 8);  // words per component (hi, lo)
};

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

// Region sums of one component added to the grid with FP32 atomics.
template <int DIM, int W, int SH>
__device__ __forceinline__ void
region_flush(const PlanProb& P, const int* org, int c, const float* hi, const float* lo, int tid, int nthr)
{
    using RG = Region<DIM, W, SH>;
    float* q = static_cast<float*>(P.q[c]);
    for (int i = tid; i < RG::RP; i += nthr)
    {
        const int lx = i % RG::R0;
        const int ly = (i / RG::R0) % RG::R1;
        const int lz = DIM == 3 ? i / (RG::R0 * RG::R1) : 0;
        const int so = lx + RG::R0 * ly + RG::PSR * lz;
        const float h = hi[so], l = lo[so];
        if (h == 0.f && l == 0.f) continue;
        const int x = wrap_cell(org[0] - (W - 1) / 2 + lx, P.N[0]);
        const int y = wrap_cell(org[1] - (W - 1) / 2 + ly, P.N[1]);
        const int z = DIM == 3 ? wrap_cell(org[2] - (W - 1) / 2 + lz, P.N[2]) : 0;
        atomicAdd(q + x + (long long)P.N[0] * (y + (long long)P.N[1] * z), h + l);
    }
}

// CTAs per SM the register budget is cut for: 3D footprints hold 32
// accumulators per thread, 2D ones 16.
template <int DIM>
struct HomeOccupancy
{
    static constexpr int value = DIM == 3 ? 3 : 4;
};

// One dense work item, by every thread of a CTA of UNIT_THREADS (it holds
// CTA barriers and ends with one): sm is the CTA's region buffer
// ([ncomp][hi, lo][PAD], components CSTR apart).
template <int DIM, int K, int SH>
__device__ __forceinline__ void
dense_item(const DevPlan& D, int item, float* sm)
{
    constexpr int W = KT<K>::W;
    using RG = Region<DIM, W, SH>;
    constexpr int R0 = RG::R0;
    constexpr int R01 = RG::PSR; // padded plane stride
    constexpr int PAD = RG::PAD;
    constexpr int CSTR = RG::CSTR;
    constexpr int NF = RG::NF;
    {
        const int t = D.item_tile[item];
        const int k = item - D.items[t];
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin<DIM, SH>(P, t - P.tile0, org);
        const int ncomp = P.ncomp;
        for (int i = threadIdx.x; i < ncomp * CSTR / 4; i += blockDim.x)
            reinterpret_cast<float4*>(sm)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int i = ncomp * CSTR / 4 * 4 + threadIdx.x; i < ncomp * CSTR; i += blockDim.x) sm[i] = 0.f;
        // The item's units, longest first (a counting sort by length in
        // shared memory), so that the threads of a warp take units of
        // similar length and finish together.
        __shared__ int s_order[MAX_ITEM_UNITS];
        __shared__ int s_start[33];
        int u0, nu;
        item_unit_range(D, t, k, u0, nu);
        if (RG::regs)
        {
            if (threadIdx.x < 33) s_start[threadIdx.x] = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < nu; i += blockDim.x)
                atomicAdd(&s_start[32 - min(D.home_units[u0 + i].y, 32)], 1);
            __syncthreads();
            if (threadIdx.x == 0)
            {
                int run = 0;
                for (int b = 0; b < 33; ++b)
                {
                    const int v = s_start[b];
                    s_start[b] = run;
                    run += v;
                }
            }
            __syncthreads();
            for (int i = threadIdx.x; i < nu; i += blockDim.x)
                s_order[atomicAdd(&s_start[32 - min(D.home_units[u0 + i].y, 32)], 1)] = i;
        }
        __syncthreads();
        const float* Qf = static_cast<const float*>(P.Q);
        if (RG::regs)
        {
            // Thread -> (unit, z-half, component): the threads of a unit sit
            // in adjacent lanes and read the same records.  A CTA holds
            // blockDim / (ncomp * ZS) units at a time and loops over the
            // item's units in steps of that.
            constexpr int ZS = RG::ZS, NZ = RG::NZ, NA = RG::NA;
            const int c = threadIdx.x % ncomp;
            const int zh = (threadIdx.x / ncomp) % ZS;
            const int ustep = blockDim.x / (ncomp * ZS);
            for (int ul = threadIdx.x / (ncomp * ZS); ul < nu; ul += ustep)
            {
                if (threadIdx.x >= ustep * ncomp * ZS) break;
                const int u = u0 + s_order[ul];
                const int2 un = D.home_units[u];
                // Even widths accumulate x-pairs with packed FP32x2
                // multiply-adds (each lane rounded once, as fmaf).
                constexpr bool PACK = W % 2 == 0;
                constexpr int WP = W / 2;
                float acc[PACK ? 1 : NA];
                unsigned long long accp[PACK ? NA / 2 : 1];
#pragma unroll
                for (int i = 0; i < (PACK ? NA / 2 : NA); ++i)
                {
                    if (PACK)
                        accp[i] = 0ull;
                    else
                        acc[i] = 0.f;
                }
                int s0[3] = { 0, 0, 0 };
                if (un.y > 0)
                {
                    const Rec R0 = D.hrec[un.x];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        const int st = (P.side && d == c) ? R0.stagger(d) : 0; // 0 or 1
                        s0[d] = wrap_from_base(R0.bc(d) + (W - 1) / 2, P.N[d]) - org[d] + st;
                    }
                }
                // Markers of the unit, software-pipelined: the next marker's
                // record and value and the id of the one after it are loaded
                // before the current marker's arithmetic.
                const int vend = un.x + un.y;
                const long long qstride = P.Q_depth;
                const float* Qc = Qf + c - qstride * P.marker0;
                Rec Rn;
                float Qn = 0.f;
                int gnn = 0;
                if (un.y > 0)
                {
                    Rn = D.hrec[un.x];
                    Qn = Qc[qstride * D.home_list[un.x]];
                    if (un.y > 1) gnn = D.home_list[un.x + 1];
                }
                for (int v = un.x; v < vend; ++v)
                {
                    const Rec R = Rn;
                    const float Qv = Qn;
                    if (v + 1 < vend)
                    {
                        Rn = D.hrec[v + 1];
                        Qn = Qc[qstride * gnn];
                        if (v + 2 < vend) gnn = D.home_list[v + 2];
                    }
                    float w[3][W];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        weights_f32<K>((P.side && d == c) ? R.rs[d] : R.rc[d], w[d]);
                    const float V = Qv * P.inv_vol;
                    // this thread's z-planes (selected without dynamic indexing)
                    float wzv[NZ];
#pragma unroll
                    for (int j2 = 0; j2 < NZ; ++j2)
                    {
                        float wz = DIM == 3 ? w[2][j2] : 1.f;
#pragma unroll
                        for (int h = 1; h < ZS; ++h)
                            if (zh == h) wz = w[2][h * NZ + j2];
                        wzv[j2] = wz * V;
                    }
                    unsigned long long w0p[PACK ? WP : 1];
                    if (PACK)
                    {
#pragma unroll
                        for (int q = 0; q < WP; ++q) w0p[q] = pack2(w[0][2 * q], w[0][2 * q + 1]);
                    }
#pragma unroll
                    for (int j2 = 0; j2 < NZ; ++j2)
                    {
#pragma unroll
                        for (int i1 = 0; i1 < W; ++i1)
                        {
                            const float wyz = w[1][i1] * wzv[j2];
                            if (PACK)
                            {
                                const unsigned long long aa = pack2(wyz, wyz);
#pragma unroll
                                for (int q = 0; q < WP; ++q)
                                    accp[(j2 * W + i1) * WP + q] = fma2(w0p[q], aa, accp[(j2 * W + i1) * WP + q]);
                            }
                            else
                            {
#pragma unroll
                                for (int i0 = 0; i0 < W; ++i0)
                                    acc[(j2 * W + i1) * W + i0] = fmaf(w[0][i0], wyz, acc[(j2 * W + i1) * W + i0]);
                            }
                        }
                    }
                }
                if (un.y > 0)
                {
                    float* hi = sm + c * CSTR;
                    float* lo = hi + PAD;
#pragma unroll
                    for (int j2 = 0; j2 < NZ; ++j2)
#pragma unroll
                        for (int i1 = 0; i1 < W; ++i1)
                        {
                            const int row =
                                (s0[1] + i1) * R0 + (DIM == 3 ? (s0[2] + zh * NZ + j2) * R01 : 0) + s0[0];
#pragma unroll
                            for (int i0 = 0; i0 < W; ++i0)
                            {
                                float a;
                                if (PACK)
                                {
                                    float e0, e1;
                                    unpack2(accp[(j2 * W + i1) * WP + i0 / 2], e0, e1);
                                    a = (i0 & 1) ? e1 : e0;
                                }
                                else
                                    a = acc[(j2 * W + i1) * W + i0];
                                if (a != 0.f) acc2(hi + row + i0, lo + row + i0, a);
                            }
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
                    float* hi = sm + c * CSTR;
                    float* lo = hi + PAD;
                    int s0[3] = { 0, 0, 0 };
                    float w[3][W];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        const bool st = P.side && d == c;
                        s0[d] = wrap_from_base(R.bc(d) + (W - 1) / 2, P.N[d]) - org[d] + (st ? R.stagger(d) : 0);
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
                            const int row = (s0[1] + i1) * R0 + (DIM == 3 ? (s0[2] + i2) * R01 : 0) + s0[0];
#pragma unroll
                            for (int i0 = 0; i0 < W; ++i0) acc2(hi + row + i0, lo + row + i0, w[0][i0] * wyz);
                        }
                    }
                }
            }
        }
        __syncthreads();
        for (int c = 0; c < ncomp; ++c)
            region_flush<DIM, W, SH>(P, org, c, sm + c * CSTR, sm + c * CSTR + PAD, threadIdx.x, blockDim.x);
        __syncthreads();
    }
    (void)NF;
}

template <int DIM, int K, int SH>
__global__ void __launch_bounds__(UNIT_THREADS, HomeOccupancy<DIM>::value) spread_home_mixed(const DevPlan D)
{
    extern __shared__ float sm[]; // [ncomp][hi, lo][PAD], components CSTR apart
    __shared__ int s_item;
    const int n_items = min(D.items[D.n_tiles], D.n_item_cap);
    // Work items are taken from a counter, so that CTAs that become resident
    // late (beside other kernels, or in a second wave) do not leave a tail.
    for (;;)
    {
        if (threadIdx.x == 0) s_item = atomicAdd(&D.work[0], 1);
        __syncthreads();
        const int item = s_item;
        if (item >= n_items) break;
        dense_item<DIM, K, SH>(D, item, sm);
    }
}

// Visits of sparse-homed markers: one warp per tile, components one after
// another.  The warp owns a private double-FP32 accumulator for one
// component of its tile, laid out with padded strides so that the 4x4x4 (or
// 4x4) stencil blocks of a visit fall into distinct shared-memory banks.
// Batches of 32 visits are prepared lane-parallel: each lane finds the
// stencil points of its visit that fall inside the tile, and the non-empty
// visits write their weights and local offsets, compacted per dimension,
// into consecutive shared-memory slots.  The in-tile points of the batch are
// numbered consecutively (warp prefix sum) and the lanes take them 32 at a
// time; a lane finds its visit from one ballot (visits starting at or before
// the chunk) and one OR-reduction (visits starting inside it), and merges
// its contribution with a compensated shared atomic.  Finally the warp adds
// the component to the grid with coalesced read-modify-writes.
// Padded accumulator layout of a tile: row and plane strides chosen so that
// a 4 x 4 block of rows of two consecutive planes falls into distinct banks.
template <int DIM, int SH>
struct TileLayout
{
    using T = TileT<DIM, SH>;
    static constexpr int RS = DIM == 3 ? (SH == 0 ? 8 : 20) : (SH == 0 ? 20 : 36); // row stride (words)
    static constexpr int PS = DIM == 3 ? (SH == 0 ? 68 : 176) : 0;                 // plane stride (words)
    static constexpr int SZ = DIM == 3 ? T::E2 * PS : T::E1 * RS;                   // words per accumulator
    static_assert(RS >= T::E0 && (DIM == 2 || PS >= T::E1 * RS), "padded strides hold a tile");
};

template <int DIM, int W, int SH>
struct VisitSlots
{
    static constexpr int SS = DIM * W + 1; // words per visit slot (odd: no bank conflicts)
    // per warp: hi, lo, slots (weights, local offsets), counts, magics, first points, values
    static constexpr int words = 2 * TileLayout<DIM, SH>::SZ + 2 * 32 * SS + 7 * 32;
};

// floor(j / n) = (j * magic(n)) >> 16 for 0 <= j < 4096 and 1 <= n <= 6
// (exact: the error of the fixed-point reciprocal stays below 1/n, the
// smallest gap between j/n and the next integer).
__device__ __forceinline__ int
div_magic(int n)
{
    return n == 1 ? 65537 : n == 2 ? 32769 : n == 3 ? 21846 : n == 4 ? 16385 : n == 5 ? 13108 : 10923;
}

// q += hi + lo for one component of a tile from the padded accumulator.
template <int DIM, int SH>
__device__ __forceinline__ void
tile_flush(const PlanProb& P, const int* org, int c, const float* hi, const float* lo, int lane)
{
    using TL = TileLayout<DIM, SH>;
    using T = TileT<DIM, SH>;
    constexpr int GR = T::E0 / 4; // groups of 4 values per row
    constexpr int G = T::E1 * T::E2 * GR;
    float* q = static_cast<float*>(P.q[c]);
    const bool row_vec = P.vec4 && org[0] + T::E0 <= P.N[0];
    for (int j = lane; j < G; j += 32)
    {
        const int r = j / GR;
        const int xo = 4 * (j % GR);
        const int yl = r % T::E1;
        const int zl = r / T::E1;
        const int so = xo + yl * TL::RS + zl * TL::PS;
        const float4 h = *reinterpret_cast<const float4*>(hi + so);
        const float4 l = *reinterpret_cast<const float4*>(lo + so);
        if (h.x == 0.f && h.y == 0.f && h.z == 0.f && h.w == 0.f && l.x == 0.f && l.y == 0.f && l.z == 0.f &&
            l.w == 0.f)
            continue;
        const int x = org[0] + xo, y = org[1] + yl, z = org[2] + zl;
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

template <int DIM, int K, int SH>
__global__ void __launch_bounds__(32 * SPARSE_WARPS, 3) spread_visits_mixed(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    using T = TileT<DIM, SH>;
    using TL = TileLayout<DIM, SH>;
    using VS = VisitSlots<DIM, W, SH>;
    constexpr int SS = VS::SS;
    extern __shared__ float sm[]; // [SPARSE_WARPS][VS::words]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const unsigned le_mask = lane == 31 ? 0xffffffffu : (2u << lane) - 1u;
    float* hi = sm + warp * VS::words;
    float* lo = hi + TL::SZ;
    float* wv = lo + TL::SZ;                          // [32][SS] in-tile weights per dim
    int* lv = reinterpret_cast<int*>(wv + 32 * SS);  // [32][SS] their offsets in the accumulator
    int* nn = lv + 32 * SS;                           // [3][32] in-tile points per dim
    int* mg = nn + 3 * 32;                            // [2][32] division magics of n0, n1
    int* pf = mg + 2 * 32;                            // [32] first point of each slot
    float* Vs = reinterpret_cast<float*>(pf + 32);    // [32] Q / vol
    // Persistent: each warp walks tiles with a grid-wide stride.
    for (int t = blockIdx.x * SPARSE_WARPS + warp; t < D.n_tiles; t += gridDim.x * SPARSE_WARPS)
    {
        const int vbeg = D.vcount[t];
        const int vend = (long long)D.vcount[t + 1] < D.n_visit_cap ? D.vcount[t + 1] : (int)D.n_visit_cap;
        if (vend <= vbeg) continue;
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin<DIM, SH>(P, t - P.tile0, org);
        const float* Qf = static_cast<const float*>(P.Q);
        for (int c = 0; c < P.ncomp; ++c)
        {
            for (int i = lane; i < 2 * TL::SZ / 4; i += 32)
                reinterpret_cast<float4*>(hi)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int b0 = vbeg; b0 < vend; b0 += 32)
            {
                // -- lane-parallel preparation of visit b0 + lane ----------
                const int v = b0 + lane;
                int cnt[3] = { 1, 1, 1 };
                unsigned inmask[3] = { 0u, 0u, 0u }; // in-tile stencil points per dim
                int lof[3][W];
                float w[3][W];
                int g = 0;
                if (v < vend)
                {
                    g = D.visit_list[v];
                    const Rec R = D.rec[g];
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        const bool stag = P.side && d == c;
                        const int b = stag ? R.bs(d) : R.bc(d);
                        weights_f32<K>(stag ? R.rs[d] : R.rc[d], w[d]);
                        const int stride = d == 0 ? 1 : d == 1 ? TL::RS : TL::PS;
                        int n = 0;
#pragma unroll
                        for (int i = 0; i < W; ++i)
                        {
                            const int l = wrap_from_base(b + i, P.N[d]) - org[d];
                            const bool in = l >= 0 && l < T::edge(d);
                            inmask[d] |= in ? (1u << i) : 0u;
                            n += in ? 1 : 0;
                            lof[d][i] = l * stride;
                        }
                        cnt[d] = n;
                    }
                }
                const int npts = v < vend ? cnt[0] * cnt[1] * (DIM == 3 ? cnt[2] : 1) : 0;
                const bool has = npts > 0;
                const unsigned hm = __ballot_sync(0xffffffffu, has);
                const int slot = __popc(hm & lt_mask); // compact slot of this visit
                int incl = npts;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1)
                {
                    const int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                const int first = incl - npts;
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                if (has)
                {
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        int n = 0;
#pragma unroll
                        for (int i = 0; i < W; ++i)
                            if (inmask[d] & (1u << i))
                            {
                                wv[slot * SS + d * W + n] = w[d][i];
                                lv[slot * SS + d * W + n] = lof[d][i];
                                ++n;
                            }
                        nn[d * 32 + slot] = cnt[d];
                        if (d < 2) mg[d * 32 + slot] = div_magic(cnt[d]);
                    }
                    pf[slot] = first;
                    Vs[slot] = Qf[(long long)P.Q_depth * (g - P.marker0) + c] * P.inv_vol;
                }
                __syncwarp();
                // -- the batch's in-tile points, 32 at a time ---------------
                for (int base = 0; base < total; base += 32)
                {
                    // slot of point base + lane: the non-empty visits that
                    // start at or before base, plus those starting in
                    // (base, base + lane]
                    const int kb = __popc(__ballot_sync(0xffffffffu, has && first <= base)) - 1;
                    const unsigned starts = __reduce_or_sync(
                        0xffffffffu, (has && first > base && first < base + 32) ? 1u << (first - base) : 0u);
                    const int kk = kb + __popc(starts & le_mask);
                    const int j = base + lane;
                    if (j < total)
                    {
                        const int jj = j - pf[kk];
                        const int n0 = nn[kk];
                        const int q1 = (jj * mg[kk]) >> 16;
                        const int j0 = jj - q1 * n0;
                        int j1 = q1, j2 = 0;
                        if (DIM == 3)
                        {
                            const int n1 = nn[32 + kk];
                            j2 = (q1 * mg[32 + kk]) >> 16;
                            j1 = q1 - j2 * n1;
                        }
                        const float* ws = wv + kk * SS;
                        const int* ls = lv + kk * SS;
                        const float V = Vs[kk];
                        const float wyz = DIM == 3 ? ws[W + j1] * (ws[2 * W + j2] * V) : ws[W + j1] * V;
                        const int idx = ls[j0] + ls[W + j1] + (DIM == 3 ? ls[2 * W + j2] : 0);
                        acc2(hi + idx, lo + idx, ws[j0] * wyz);
                    }
                }
                __syncwarp();
            }
            tile_flush<DIM, SH>(P, org, c, hi, lo, lane);
            __syncwarp();
        }
    }
}
// Visits of sparse-homed markers, second form: one lane per (visit,
// component) work item, all components of the tile accumulated at once.
// The lane keeps its visit's weights and accumulator offsets in registers
// and runs the whole W^d footprint unrolled; points outside the tile are
// masked by a negative offset and their atomics predicated off, so the warp
// does not diverge.  Chosen by the autotuner when it is faster.
constexpr int LANE_WARPS = 4; // tiles (warps) per CTA of this form

__device__ __forceinline__ void
acc2_always(float* hi, float* lo, float v)
{
    const float old = atomicAdd(hi, v);
    const float s = old + v;
    const float bp = s - old;
    atomicAdd(lo, (old - (s - bp)) + (v - bp));
}

template <int DIM, int K, int SH>
__global__ void __launch_bounds__(32 * LANE_WARPS, 4) spread_visits_lanes(const DevPlan D, int ncomp_max)
{
    constexpr int W = KT<K>::W;
    using T = TileT<DIM, SH>;
    using TL = TileLayout<DIM, SH>;
    extern __shared__ float sm[]; // [LANE_WARPS][ncomp_max][hi, lo][SZ]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* acc = sm + warp * (2 * TL::SZ * ncomp_max);
    for (int t = blockIdx.x * LANE_WARPS + warp; t < D.n_tiles; t += gridDim.x * LANE_WARPS)
    {
        const int vbeg = D.vcount[t];
        const int vend = (long long)D.vcount[t + 1] < D.n_visit_cap ? D.vcount[t + 1] : (int)D.n_visit_cap;
        if (vend <= vbeg) continue;
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin<DIM, SH>(P, t - P.tile0, org);
        const int ncomp = P.ncomp;
        for (int i = lane; i < ncomp * 2 * TL::SZ / 4; i += 32)
            reinterpret_cast<float4*>(acc)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncwarp();
        const float* Qf = static_cast<const float*>(P.Q);
        const int nitems = (vend - vbeg) * ncomp;
        for (int b0 = 0; b0 < nitems; b0 += 32)
        {
            const int it = b0 + lane;
            if (it >= nitems) continue;
            const int v = vbeg + it / ncomp;
            const int c = it % ncomp;
            const int g = D.visit_list[v];
            const Rec R = D.rec[g];
            float w[3][W];
            int off[3][W];
#pragma unroll
            for (int d = 0; d < 3; ++d)
            {
                if (d >= DIM)
                {
#pragma unroll
                    for (int i = 0; i < W; ++i)
                    {
                        w[d][i] = 1.f;
                        off[d][i] = 0;
                    }
                    continue;
                }
                const bool stag = P.side && d == c;
                const int b = stag ? R.bs(d) : R.bc(d);
                weights_f32<K>(stag ? R.rs[d] : R.rc[d], w[d]);
                const int stride = d == 0 ? 1 : d == 1 ? TL::RS : TL::PS;
#pragma unroll
                for (int i = 0; i < W; ++i)
                {
                    const int l = wrap_from_base(b + i, P.N[d]) - org[d];
                    off[d][i] = (l >= 0 && l < T::edge(d)) ? l * stride : -(1 << 20);
                }
            }
            const float V = Qf[(long long)P.Q_depth * (g - P.marker0) + c] * P.inv_vol;
            float* hi = acc + c * 2 * TL::SZ;
            float* lo = hi + TL::SZ;
#pragma unroll
            for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
            {
                const float wz = DIM == 3 ? w[2][i2] * V : V;
                const int oz = DIM == 3 ? off[2][i2] : 0;
#pragma unroll
                for (int i1 = 0; i1 < W; ++i1)
                {
                    const float wyz = w[1][i1] * wz;
                    const int oyz = off[1][i1] + oz;
#pragma unroll
                    for (int i0 = 0; i0 < W; ++i0)
                    {
                        const int idx = off[0][i0] + oyz;
                        if (idx >= 0) acc2_always(hi + idx, lo + idx, w[0][i0] * wyz);
                    }
                }
            }
        }
        __syncwarp();
        for (int c = 0; c < ncomp; ++c)
            tile_flush<DIM, SH>(P, org, c, acc + c * 2 * TL::SZ, acc + c * 2 * TL::SZ + TL::SZ, lane);
        __syncwarp();
    }
}


// Visits of sparse-homed markers, third form: the tile gathered rather than
// scattered.  A visit's contribution to one component of a tile is the outer
// product of its separable weights restricted to the tile, w0(x) w1(y)
// w2(z) Q/vol, so the tile's sum over its visits is a small contraction:
// lane l owns CPL values of the tile (NR rows of SX consecutive x) in
// registers, and for every visit adds a(row) * b(x) with a(row) = w1(y) *
// (w2(z) * Q/vol) and b(x) = w0(x), reading the visit's tile-restricted
// weight vectors (zero outside its stencil) from shared memory.  No atomics:
// every lane updates only its own values, all lanes run every visit, and the
// warp then adds the tile to the grid with coalesced read-modify-writes.
// Sums over batches of 32 visits are folded into a double-FP32 pair with
// Knuth TwoSum, so the error bound is that of 32-term FP32 sums.
template <int DIM, int SH>
struct GatherLayout
{
    using T = TileT<DIM, SH>;
    static constexpr int CPL = T::PTS / 32;                  // values per lane
    static constexpr int SX = CPL < T::E0 ? CPL : T::E0;     // consecutive x per lane row
    static constexpr int NR = CPL / SX;                      // rows per lane
    static constexpr int VW = T::E0 + T::E1 + T::E2;         // weight vector words of a visit
    static constexpr int SS = ((VW + 3) / 8) * 8 + 4;        // slot stride: = 4 mod 8 (float4-aligned)
    static_assert(CPL * 32 == T::PTS && SX % 4 == 0 && NR * SX == CPL, "lane layout covers the tile");
};

constexpr int GATHER_WARPS = 8; // tiles (warps) per CTA of the gather form

// CTAs per SM the register budget is cut for: 4 x (256 threads) with 16
// values per lane (64 registers: more warps to hide the record loads beat
// the few spilled values), 1 with 32 (3D tiles of 16 x 8 x 8).
template <int DIM, int SH>
struct GatherOccupancy
{
    static constexpr int value = GatherLayout<DIM, SH>::CPL > 16 ? 1 : 4;
};

// The W weights of a stencil with base b, restricted to the E cells of a tile
// starting at org (zero elsewhere), into dst.  PREP 0: dst was zeroed, the
// in-tile weights are stored one by one (added when a grid narrower than the
// stencil wraps two points onto one cell); PREP 1: the E values are formed in
// registers and written with 16-byte stores.
template <int W, int E, int PREP>
__device__ __forceinline__ void
put_weights(float* dst, const float* w, int b, int N, int org)
{
    if (PREP == 0)
    {
        const bool distinct = N >= W; // the stencil's points on distinct cells
#pragma unroll
        for (int i = 0; i < W; ++i)
        {
            const int l = wrap_from_base(b + i, N) - org;
            if (l >= 0 && l < E) dst[l] = distinct ? w[i] : dst[l] + w[i];
        }
    }
    else
    {
        float vec[E];
#pragma unroll
        for (int j = 0; j < E; ++j) vec[j] = 0.f;
#pragma unroll
        for (int i = 0; i < W; ++i)
        {
            const int l = wrap_from_base(b + i, N) - org;
#pragma unroll
            for (int j = 0; j < E; ++j) vec[j] = l == j ? vec[j] + w[i] : vec[j];
        }
        if (E % 4 == 0)
        {
#pragma unroll
            for (int j = 0; j < E; j += 4)
                *reinterpret_cast<float4*>(dst + j) = make_float4(vec[j], vec[j + 1], vec[j + 2], vec[j + 3]);
        }
        else
        {
#pragma unroll
            for (int j = 0; j < E; ++j) dst[j] = vec[j];
        }
    }
}

// Tile t's visits gathered by one warp (every lane); slots: the warp's 32
// visit slots of SS floats.  PREP: how a lane writes its visit's
// tile-restricted weight vectors into its slot -- 0: the slot is zeroed with
// 16-byte stores and the in-tile weights stored one by one (added when a
// grid narrower than the stencil wraps two points onto one cell); 1: each
// vector is assembled in registers (a compare and select per tile position
// and stencil point) and written with 16-byte stores, no zeroing (form 3:
// fewer shared-memory wavefronts, more arithmetic).  L2ONLY: the grid values
// are read past L1 (the fused step, where atomics of the same launch wrote
// them).
template <int DIM, int K, int SH, int PREP, bool L2ONLY = false>
__device__ __forceinline__ void
gather_tile(const DevPlan& D, int t, float* slots, int lane)
{
    constexpr int W = KT<K>::W;
    using T = TileT<DIM, SH>;
    using GL = GatherLayout<DIM, SH>;
    constexpr int CPL = GL::CPL, SX = GL::SX, NR = GL::NR, SS = GL::SS;
    constexpr int SP = SX / 2; // value pairs per lane row
    float* mine = slots + lane * SS;
    // This lane's values: NR consecutive rows y0 .. y0 + NR - 1 of plane z
    // (rows are y + E1 * z; NR and E1 are even or NR is 1), x in [xs, xs + SX).
    const int first = lane * CPL;
    const int r0 = first / T::E0;
    const int xs = first % T::E0;
    const int y0 = r0 % T::E1;
    const int z0 = r0 / T::E1;
    static_assert(NR == 1 || (NR == 2 && T::E1 % 2 == 0), "a lane's rows share their plane");
    {
        const int vbeg = D.vcount[t];
        const int vend = (long long)D.vcount[t + 1] < D.n_visit_cap ? D.vcount[t + 1] : (int)D.n_visit_cap;
        if (vend <= vbeg) return;
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin<DIM, SH>(P, t - P.tile0, org);
        const float* Qf = static_cast<const float*>(P.Q);
        for (int c = 0; c < P.ncomp; ++c)
        {
            float hi[CPL], lo[CPL];
#pragma unroll
            for (int i = 0; i < CPL; ++i) hi[i] = lo[i] = 0.f;
            for (int b0 = vbeg; b0 < vend; b0 += 32)
            {
                const int nb = min(32, vend - b0);
                // -- this lane's visit: its weight vectors restricted to the tile
                //    (only the slots of the batch's visits are read)
                if (PREP == 0)
                {
#pragma unroll
                    for (int i = 0; i < SS / 4; ++i)
                        reinterpret_cast<float4*>(mine)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                if (lane < nb)
                {
                    const int g = D.visit_list[b0 + lane];
                    const Rec R = D.rec[g];
                    const float V = Qf[(long long)P.Q_depth * (g - P.marker0) + c] * P.inv_vol;
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                    {
                        const bool stag = P.side && d == c;
                        const int b = stag ? R.bs(d) : R.bc(d);
                        float w[W];
                        weights_f32<K>(stag ? R.rs[d] : R.rc[d], w);
                        const int off = d == 0 ? 0 : d == 1 ? T::E0 : T::E0 + T::E1;
                        // Q/vol rides on the last dimension's weights
                        if (d == DIM - 1)
                        {
#pragma unroll
                            for (int i = 0; i < W; ++i) w[i] *= V;
                        }
                        if (d == 0)
                            put_weights<W, T::E0, PREP>(mine + off, w, b, P.N[d], org[d]);
                        else if (d == 1)
                            put_weights<W, T::E1, PREP>(mine + off, w, b, P.N[d], org[d]);
                        else
                            put_weights<W, T::E2, PREP>(mine + off, w, b, P.N[d], org[d]);
                    }
                }
                __syncwarp();
                // -- the batch's contraction into this lane's values, two
                //    x-values per packed multiply-add
                unsigned long long acc[NR][SP];
#pragma unroll
                for (int k = 0; k < NR; ++k)
#pragma unroll
                    for (int j = 0; j < SP; ++j) acc[k][j] = 0ull;
                for (int m = 0; m < nb; ++m)
                {
                    const float* sv = slots + m * SS;
                    unsigned long long bx[SP];
#pragma unroll
                    for (int j = 0; j < SP / 2; ++j)
                    {
                        const ulonglong2 q2 = *reinterpret_cast<const ulonglong2*>(sv + xs + 4 * j);
                        bx[2 * j] = q2.x;
                        bx[2 * j + 1] = q2.y;
                    }
                    float ay[NR];
                    if (NR == 2)
                    {
                        const float2 y2 = *reinterpret_cast<const float2*>(sv + T::E0 + y0);
                        ay[0] = y2.x;
                        ay[NR - 1] = y2.y;
                    }
                    else
                        ay[0] = sv[T::E0 + y0];
                    const float az = DIM == 3 ? sv[T::E0 + T::E1 + z0] : 1.f;
#pragma unroll
                    for (int k = 0; k < NR; ++k)
                    {
                        const float a = DIM == 3 ? ay[k] * az : ay[k];
                        const unsigned long long aa = pack2(a, a);
#pragma unroll
                        for (int j = 0; j < SP; ++j) acc[k][j] = fma2(bx[j], aa, acc[k][j]);
                    }
                }
                // -- fold the batch sums into the double-FP32 pair
#pragma unroll
                for (int k = 0; k < NR; ++k)
#pragma unroll
                    for (int j = 0; j < SP; ++j)
                    {
                        float av[2];
                        unpack2(acc[k][j], av[0], av[1]);
#pragma unroll
                        for (int e = 0; e < 2; ++e)
                        {
                            const int i = k * SX + 2 * j + e;
                            const float s2 = hi[i] + av[e];
                            const float bp = s2 - hi[i];
                            lo[i] += (hi[i] - (s2 - bp)) + (av[e] - bp);
                            hi[i] = s2;
                        }
                    }
                __syncwarp();
            }
            // -- q += hi + lo for this lane's values
            float* q = static_cast<float*>(P.q[c]);
#pragma unroll
            for (int k = 0; k < NR; ++k)
            {
                const int y = org[1] + y0 + k;
                const int z = DIM == 3 ? org[2] + z0 : 0;
                if (y >= P.N[1] || (DIM == 3 && z >= P.N[2])) continue;
                const int x0 = org[0] + xs;
                const long long o = x0 + (long long)P.N[0] * (y + (long long)P.N[1] * z);
                const bool vec = P.vec4 && x0 + SX <= P.N[0];
#pragma unroll
                for (int i = 0; i < SX; i += 4)
                {
                    const float* h = hi + k * SX + i;
                    const float* l = lo + k * SX + i;
                    if (h[0] == 0.f && h[1] == 0.f && h[2] == 0.f && h[3] == 0.f && l[0] == 0.f && l[1] == 0.f &&
                        l[2] == 0.f && l[3] == 0.f)
                        continue;
                    if (vec)
                    {
                        float4 v = L2ONLY ? __ldcg(reinterpret_cast<const float4*>(q + o + i))
                                          : *reinterpret_cast<const float4*>(q + o + i);
                        v.x = merge3(v.x, h[0], l[0]);
                        v.y = merge3(v.y, h[1], l[1]);
                        v.z = merge3(v.z, h[2], l[2]);
                        v.w = merge3(v.w, h[3], l[3]);
                        *reinterpret_cast<float4*>(q + o + i) = v;
                    }
                    else
                    {
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (x0 + i + e < P.N[0] && (h[e] != 0.f || l[e] != 0.f))
                                q[o + i + e] = merge3(L2ONLY ? __ldcg(q + o + i + e) : q[o + i + e], h[e], l[e]);
                    }
                }
            }
        }
    }
}

// OCC: CTAs per SM the register budget is cut for (GatherOccupancy: 64
// registers for 3D tiles of 8^3).
template <int DIM, int K, int SH, int OCC, int PREP>
__global__ void __launch_bounds__(32 * GATHER_WARPS, OCC) spread_visits_gather(const DevPlan D)
{
    using GL = GatherLayout<DIM, SH>;
    extern __shared__ float sm[]; // [GATHER_WARPS][32][SS]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* slots = sm + warp * 32 * GL::SS;
    // each warp takes its next tile from a counter (no tail from late CTAs)
    for (;;)
    {
        int t = 0;
        if (lane == 0) t = atomicAdd(&D.work[1], 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= D.n_tiles) break;
        gather_tile<DIM, K, SH, PREP>(D, t, slots, lane);
    }
}

// ---- the post-binning step in one persistent launch ------------------------
// Every CTA takes work from one device counter, in this order: the dense
// spread's work items (dense_item), the per-unit interpolation of the same
// items (units_item), the chunked interpolation of the sparse-homed markers
// (chunk_body, no register cache; every marker where the per-unit form does
// not apply), and groups of GATHER_WARPS tiles of the
// per-visit gather spread (gather_tile, one warp per tile).  The gather adds
// into tiles that the dense items' region atomics also reach, so a gather
// group first waits until every dense item has finished -- a counter the
// dense items raise after a device-wide fence.  Every dense item was claimed
// before any gather group (counter order) by a CTA that is running, so the
// wait ends; it is bounded all the same (about a second), reported through
// bit 2 of the status word.  One launch for the spread and the interpolation
// of every problem of the plan; the phases share the SMs as their work
// arrives instead of partitioning them between two streams.
constexpr int FUSED_THREADS = 256;
constexpr int DONE_SPINS = 1 << 22;
static_assert(FUSED_THREADS == UNIT_THREADS && FUSED_THREADS == INTERP_THREADS &&
                  FUSED_THREADS == 32 * GATHER_WARPS,
              "one CTA shape for every phase");

template <int DIM, int K, int SH, int PREP>
__global__ void __launch_bounds__(FUSED_THREADS, 3) step_fused(const DevPlan D)
{
    using GL = GatherLayout<DIM, SH>;
    extern __shared__ float sm[]; // the dense region buffer, or the warps' visit slots
    __shared__ int s_item;
    __shared__ int s_order[256];
    __shared__ int s_start[33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nD = min(D.items[D.n_tiles], D.n_item_cap);
    const long long chunk_threads = (D.n_markers + CHUNK - 1) / CHUNK * D.max_ncomp;
    const int nC = (int)((chunk_threads + FUSED_THREADS - 1) / FUSED_THREADS);
    const int nG = (D.n_tiles + GATHER_WARPS - 1) / GATHER_WARPS;
    // the per-unit interpolation holds a unit's stencil values in registers
    // only up to 64 per lane; beyond that the chunks take every marker
    constexpr bool UNITS = UnitSplit<DIM, KT<K>::W>::NC <= 64;
    const int nU = UNITS ? nD : 0;
    const int total = nD + nU + nC + nG;
    for (;;)
    {
        __syncthreads(); // the previous piece of work is done with s_item, s_order and sm
        if (threadIdx.x == 0) s_item = atomicAdd(&D.work[0], 1);
        __syncthreads();
        const int w = s_item;
        if (w >= total) break;
        if (w < nD)
        {
            dense_item<DIM, K, SH>(D, w, sm);
            __threadfence(); // this thread's region atomics, visible device-wide
            __syncthreads();
            if (threadIdx.x == 0) atomicAdd(&D.work[1], 1);
        }
        else if (w < nD + nU)
            units_item<DIM, K>(D, w - nD, s_order, s_start);
        else if (w < nD + nU + nC)
            chunk_body<DIM, K, false>(D, (long long)(w - nD - nU) * FUSED_THREADS + threadIdx.x,
                                      UNITS ? SEL_SPARSE : SEL_ALL, 0);
        else
        {
            if (threadIdx.x == 0)
            {
                for (int spins = 0; atomicAdd(&D.work[1], 0) < nD; ++spins)
                {
                    if (spins >= DONE_SPINS)
                    {
                        atomicOr(D.status, 4);
                        break;
                    }
                    __nanosleep(256);
                }
                __threadfence();
            }
            __syncthreads();
            const int t = (w - nD - nU - nC) * GATHER_WARPS + warp;
            if (t < D.n_tiles) gather_tile<DIM, K, SH, PREP, true>(D, t, sm + warp * 32 * GL::SS, lane);
        }
    }
}

template <int DIM, int K, int SH, int PREP>
int
launch_fused_k(const DevPlan& D, int max_ncomp, cudaStream_t s, int sms)
{
    constexpr int W = KT<K>::W;
    const size_t smem_d = sizeof(float) * Region<DIM, W, SH>::CSTR * max_ncomp;
    const size_t smem_g = sizeof(float) * 32 * GatherLayout<DIM, SH>::SS * GATHER_WARPS;
    const size_t smem = smem_d > smem_g ? smem_d : smem_g;
    if (cudaFuncSetAttribute(step_fused<DIM, K, SH, PREP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return IBX_E_CUDA;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_fused<DIM, K, SH, PREP>, FUSED_THREADS, smem);
    if (per_sm < 1) per_sm = 1;
    step_fused<DIM, K, SH, PREP><<<(unsigned)(per_sm * sms), FUSED_THREADS, smem, s>>>(D);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

} // namespace

namespace
{
template <int DIM, int K, int SH, int OCC, int PREP>
int
launch_gather(const DevPlan& D, cudaStream_t s, int sms)
{
    using GL = GatherLayout<DIM, SH>;
    const size_t smem_g = sizeof(float) * 32 * GL::SS * GATHER_WARPS;
    if (smem_g > 48 * 1024 &&
        cudaFuncSetAttribute(spread_visits_gather<DIM, K, SH, OCC, PREP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_g) != cudaSuccess)
        return IBX_E_CUDA;
    int per_sm_g = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_g, spread_visits_gather<DIM, K, SH, OCC, PREP>, 32 * GATHER_WARPS,
                                                  smem_g);
    if (per_sm_g < 1) per_sm_g = 1;
    const unsigned need_g = (unsigned)((D.n_tiles + GATHER_WARPS - 1) / GATHER_WARPS);
    const unsigned blocks_g = need_g < (unsigned)(per_sm_g * sms) ? need_g : (unsigned)(per_sm_g * sms);
    spread_visits_gather<DIM, K, SH, OCC, PREP><<<blocks_g, 32 * GATHER_WARPS, smem_g, s>>>(D);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

template <int DIM, int K, int SH>
int
launch_spread_k(const DevPlan& D, int max_ncomp, cudaStream_t s, int sms, cudaEvent_t visits_done)
{
    constexpr int W = KT<K>::W;
    const int per_sm = D.dense_blocks_per_sm > 0 ? D.dense_blocks_per_sm : 2;
    const unsigned dense_blocks = (unsigned)(D.n_item_cap < per_sm * sms ? D.n_item_cap : per_sm * sms);
    const size_t smem = sizeof(float) * Region<DIM, W, SH>::CSTR * max_ncomp;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(spread_home_mixed<DIM, K, SH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return IBX_E_CUDA;
    if (dense_blocks > 0)
    {
        spread_home_mixed<DIM, K, SH><<<dense_blocks, UNIT_THREADS, smem, s>>>(D);
        note_launches(1);
        if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;
    }
    if (visits_done && cudaStreamWaitEvent(s, visits_done, 0) != cudaSuccess) return IBX_E_CUDA;
    if (D.visit_kernel == 2 || D.visit_kernel == 3)
    {
        constexpr int OCC = GatherOccupancy<DIM, SH>::value;
        return D.visit_kernel == 2 ? launch_gather<DIM, K, SH, OCC, 0>(D, s, sms)
                                   : launch_gather<DIM, K, SH, OCC, 1>(D, s, sms);
    }
    if (D.visit_kernel == 1)
    {
        const size_t smem_l = sizeof(float) * 2 * TileLayout<DIM, SH>::SZ * max_ncomp * LANE_WARPS;
        if (smem_l > 48 * 1024 &&
            cudaFuncSetAttribute(spread_visits_lanes<DIM, K, SH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem_l) != cudaSuccess)
            return IBX_E_CUDA;
        int per_sm_l = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_l, spread_visits_lanes<DIM, K, SH>, 32 * LANE_WARPS,
                                                      smem_l);
        if (per_sm_l < 1) per_sm_l = 1;
        const unsigned need_l = (unsigned)((D.n_tiles + LANE_WARPS - 1) / LANE_WARPS);
        const unsigned blocks_l = need_l < (unsigned)(per_sm_l * sms) ? need_l : (unsigned)(per_sm_l * sms);
        spread_visits_lanes<DIM, K, SH><<<blocks_l, 32 * LANE_WARPS, smem_l, s>>>(D, max_ncomp);
        note_launches(1);
        return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
    }
    const size_t smem_sparse = sizeof(float) * VisitSlots<DIM, W, SH>::words * SPARSE_WARPS;
    if (smem_sparse > 48 * 1024 &&
        cudaFuncSetAttribute(spread_visits_mixed<DIM, K, SH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_sparse) != cudaSuccess)
        return IBX_E_CUDA;
    int per_sm_v = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_v, spread_visits_mixed<DIM, K, SH>, 32 * SPARSE_WARPS,
                                                  smem_sparse);
    if (per_sm_v < 1) per_sm_v = 1;
    const unsigned need = (unsigned)((D.n_tiles + SPARSE_WARPS - 1) / SPARSE_WARPS);
    const unsigned sparse_blocks = need < (unsigned)(per_sm_v * sms) ? need : (unsigned)(per_sm_v * sms);
    spread_visits_mixed<DIM, K, SH><<<sparse_blocks, 32 * SPARSE_WARPS, smem_sparse, s>>>(D);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}
} // namespace

int
launch_fused(int dim, int kernel, const DevPlan& D, int max_ncomp, cudaStream_t s)
{
    if (D.n_tiles == 0) return IBX_OK;
    if (cudaMemsetAsync(D.work, 0, 2 * sizeof(int), s) != cudaSuccess) return IBX_E_CUDA;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // the gather phase in its plain form (visit forms 2 and 3 give the same sums)
    const int sh = D.tile_shape;
#define IBX_FUSED_CASE(DD, KK)                                                                                       \
    if (dim == DD && kernel == KK)                                                                                   \
        return sh == 0 ? launch_fused_k<DD, KK, 0, 0>(D, max_ncomp, s, sms) : launch_fused_k<DD, KK, 1, 0>(D, max_ncomp, s, sms);
    IBX_FUSED_CASE(2, K_PL) IBX_FUSED_CASE(2, K_PCUBIC) IBX_FUSED_CASE(2, K_IB3) IBX_FUSED_CASE(2, K_IB4)
    IBX_FUSED_CASE(2, K_IB6) IBX_FUSED_CASE(2, K_BSPL4) IBX_FUSED_CASE(3, K_PL) IBX_FUSED_CASE(3, K_PCUBIC)
    IBX_FUSED_CASE(3, K_IB3) IBX_FUSED_CASE(3, K_IB4) IBX_FUSED_CASE(3, K_IB6) IBX_FUSED_CASE(3, K_BSPL4)
#undef IBX_FUSED_CASE
    return IBX_E_BAD_KERNEL;
}

int
launch_spread(int dim, int kernel, const DevPlan& D, int max_ncomp, cudaStream_t s, cudaEvent_t visits_done)
{
    if (D.n_tiles == 0) return IBX_OK;
    if (cudaMemsetAsync(D.work, 0, 2 * sizeof(int), s) != cudaSuccess) return IBX_E_CUDA;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int sh = D.tile_shape;
#define IBX_SPREAD_CASE(DD, KK)                                                                                      \
    if (dim == DD && kernel == KK)                                                                                   \
        return sh == 0 ? launch_spread_k<DD, KK, 0>(D, max_ncomp, s, sms, visits_done)                             \
                       : launch_spread_k<DD, KK, 1>(D, max_ncomp, s, sms, visits_done);
    IBX_SPREAD_CASE(2, K_PL) IBX_SPREAD_CASE(2, K_PCUBIC) IBX_SPREAD_CASE(2, K_IB3) IBX_SPREAD_CASE(2, K_IB4)
    IBX_SPREAD_CASE(2, K_IB6) IBX_SPREAD_CASE(2, K_BSPL4) IBX_SPREAD_CASE(3, K_PL) IBX_SPREAD_CASE(3, K_PCUBIC)
    IBX_SPREAD_CASE(3, K_IB3) IBX_SPREAD_CASE(3, K_IB4) IBX_SPREAD_CASE(3, K_IB6) IBX_SPREAD_CASE(3, K_BSPL4)
#undef IBX_SPREAD_CASE
    return IBX_E_BAD_KERNEL;
}

} // namespace ibx
