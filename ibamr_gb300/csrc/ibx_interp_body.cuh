// ibx_interp_body.cuh -- device bodies of the chunked and the per-unit
// interpolation of the plan pipeline (mixed precision), shared by their own
// kernels (ibx_interp.cu) and the fused step kernel (ibx_spread.cu).
//
// Sum order everywhere: V = sum_z w_z sum_y w_y sum_x w_x u, the separable
// form of the reference's w(i0,i1,i2) * u (F3D:1309-1328), so every form
// gives bit-identical results.
#pragma once

#include "ibx_plan.cuh"

namespace ibx
{
namespace
{
constexpr int INTERP_THREADS = 256;
constexpr int CHUNK = 4;      // markers per thread of interp_chunks

// Which markers a kernel takes.
enum Select
{
    SEL_ALL = 0,
    SEL_SPARSE = 1, // markers of home tiles with at most dense_min markers
    SEL_DENSE = 2
};

__device__ __forceinline__ bool
tile_dense(const DevPlan& D, int t)
{
    return D.hcount[t + 1] - D.hcount[t] > D.dense_min;
}

// V = sum_z w2 sum_y w1 sum_x w0 u(x, y, z), u(i0, i1, i2) = at(i0, i1, i2).
template <int DIM, int W, typename At>
__device__ __forceinline__ float
separable_sum(const float (&w)[3][W], At at)
{
    float V = 0.f;
#pragma unroll
    for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
    {
        float vy = 0.f;
#pragma unroll
        for (int i1 = 0; i1 < W; ++i1)
        {
            float vx = 0.f;
#pragma unroll
            for (int i0 = 0; i0 < W; ++i0) vx = fmaf(w[0][i0], at(i0, i1, i2), vx);
            vy = fmaf(w[1][i1], vx, vy);
        }
        V = fmaf(DIM == 3 ? w[2][i2] : 1.f, vy, V);
    }
    return V;
}

// separable_sum over rows read as aligned 8-byte pairs: q0 points at the
// even value at or before the stencil's first x (odd: the first x is the
// pair's second value); the rows' cells along y and z are co[1], co[2].  The
// same FP32 operations in the same order as separable_sum.
template <int DIM, int W>
__device__ __forceinline__ float
separable_sum_pairs(const float (&w)[3][W], const float* q0, int odd, const int (&co)[3][W], long long n0,
                    long long n01)
{
    constexpr int NP = W / 2 + 1; // pairs covering W values from an odd start
    float V = 0.f;
#pragma unroll
    for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
    {
        float vy = 0.f;
#pragma unroll
        for (int i1 = 0; i1 < W; ++i1)
        {
            const float2* row = reinterpret_cast<const float2*>(q0 + (DIM == 3 ? co[2][i2] * n01 : 0) + co[1][i1] * n0);
            float f[2 * NP];
#pragma unroll
            for (int j = 0; j < NP; ++j)
            {
                // the last pair only when it holds a stencil value (an odd
                // start, or an odd width)
                float2 v = make_float2(0.f, 0.f);
                if (j < NP - 1 || odd || (W & 1)) v = __ldg(row + j);
                f[2 * j] = v.x;
                f[2 * j + 1] = v.y;
            }
            float vx = 0.f;
#pragma unroll
            for (int i0 = 0; i0 < W; ++i0) vx = fmaf(w[0][i0], odd ? f[i0 + 1] : f[i0], vx);
            vy = fmaf(w[1][i1], vx, vy);
        }
        V = fmaf(DIM == 3 ? w[2][i2] : 1.f, vy, V);
    }
    return V;
}

// Kernel weights of component c of a record (w[d][0] = 1 beyond DIM).
template <int DIM, int K>
__device__ __forceinline__ void
record_weights(const PlanProb& P, const Rec& R, int c, float (&w)[3][KT<K>::W])
{
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
}

// Periodic cells of the stencil of component c of a record.
template <int DIM, int W>
__device__ __forceinline__ void
stencil_cells(const PlanProb& P, const Rec& R, int c, int (&co)[3][W])
{
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        if (d >= DIM)
        {
            co[d][0] = 0;
            continue;
        }
        const int b = (P.side && d == c) ? R.bs(d) : R.bc(d);
#pragma unroll
        for (int i = 0; i < W; ++i) co[d][i] = wrap_from_base(b + i, P.N[d]);
    }
}

// Chunks of consecutive home-order markers, one component per thread
// (adjacent threads take the components of one chunk, so that the chunk's
// records are read from DRAM once).
// CACHE_OK: the W^d stencil values may be cached in registers across markers
// sharing a stencil (interp_chunks); off where registers are scarce (the
// fused step kernel takes only sparse-homed markers this way, which rarely
// share stencils).  PAIRS: uncached six-value rows that do not wrap are read
// as aligned 8-byte pairs (separable_sum_pairs).
template <int DIM, int K, bool CACHE_OK, bool PAIRS = false>
__device__ __forceinline__ void
chunk_body(const DevPlan& D, long long tid, int select, int marker_order)
{
    constexpr int W = KT<K>::W;
    constexpr int NF = DIM == 3 ? W * W * W : W * W;
    constexpr bool CACHE = NF <= 64 && CACHE_OK;
    const int c = (int)(tid % D.max_ncomp);
    // home order: the binned markers; marker order: every marker (those
    // without a record, non-finite positions, are skipped)
    const long long total = marker_order ? D.n_markers : (long long)D.hcount[D.n_tiles];
    const long long m0 = (tid / D.max_ncomp) * CHUNK;
    if (m0 >= total) return;
    const long long m1 = min(m0 + CHUNK, total);
    float u[CACHE ? NF : 1];
    int cur[3] = { -100000, -100000, -100000 };
    int curp = -1;
    int lastp = 0; // the previous marker's problem: consecutive markers mostly share it
    for (long long m = m0; m < m1; ++m)
    {
        const int g = marker_order ? (int)m : D.home_list[m];
        if (marker_order && D.home_tile[g] < 0) continue;
        if (select != SEL_ALL && tile_dense(D, D.home_tile[g]) != (select == SEL_DENSE)) continue;
        int p = 0;
        if (D.n_probs > 1)
        {
            p = (g >= D.marker_offs[lastp] && g < D.marker_offs[lastp + 1])
                    ? lastp
                    : find_in_offsets(D.marker_offs, D.n_probs, (long long)g);
            lastp = p;
        }
        const PlanProb& P = D.probs[p];
        if (c >= P.ncomp) continue;
        const Rec R = marker_order ? D.rec[g] : D.hrec[m];
        float w[3][W];
        record_weights<DIM, K>(P, R, c, w);
        const float* q = static_cast<const float*>(P.qi[c]);
        const long long n0 = P.N[0], n01 = (long long)P.N[0] * P.N[1];
        float V;
        if (CACHE)
        {
            int b[3] = { 0, 0, 0 };
#pragma unroll
            for (int d = 0; d < DIM; ++d) b[d] = (P.side && d == c) ? R.bs(d) : R.bc(d);
            const bool same = p == curp && b[0] == cur[0] && b[1] == cur[1] && (DIM == 2 || b[2] == cur[2]);
            if (!same)
            {
                int co[3][W];
                stencil_cells<DIM, W>(P, R, c, co);
#pragma unroll
                for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0)
                            u[(i2 * W + i1) * W + i0] =
                                __ldg(q + (DIM == 3 ? co[2][i2] * n01 : 0) + co[1][i1] * n0 + co[0][i0]);
                cur[0] = b[0];
                cur[1] = b[1];
                cur[2] = b[2];
                curp = p;
            }
            V = separable_sum<DIM, W>(w, [&](int i0, int i1, int i2) { return u[(i2 * W + i1) * W + i0]; });
        }
        else
        {
            int co[3][W];
            stencil_cells<DIM, W>(P, R, c, co);
            const int bx = (P.side && c == 0) ? R.bs(0) : R.bc(0);
            // six-value rows that do not wrap, in a grid whose rows start
            // 8-byte aligned: read as aligned pairs (three or four loads per
            // row instead of six), the values picked by the row's parity; the
            // same sums.  (For four-value rows the pairs measured slower in
            // the concurrent step: they take more of the L1 the gather spread
            // shares.)
            if (PAIRS && W == 6 && bx + W <= P.N[0] && (P.N[0] & 1) == 0 &&
                (reinterpret_cast<unsigned long long>(q) & 7ull) == 0)
                V = separable_sum_pairs<DIM, W>(w, q + (bx & ~1), bx & 1, co, n0, n01);
            else
                V = separable_sum<DIM, W>(w, [&](int i0, int i1, int i2) {
                    return __ldg(q + (DIM == 3 ? co[2][i2] * n01 : 0) + co[1][i1] * n0 + co[0][i0]);
                });
        }
        static_cast<float*>(P.Qi)[(long long)P.Q_depth * (g - P.marker0) + c] = V;
    }
}

// Lanes per (home unit, component) of interp_units: the footprint's z-planes
// are split over ZS adjacent lanes (dense_zsplit, as for the dense spread),
// each caching NZ planes of W x W values.
template <int DIM, int W>
struct UnitSplit
{
    static constexpr int ZS = dense_zsplit(DIM, W);
    static constexpr int NZ = (DIM == 3 ? W : 1) / ZS;
    static constexpr int NC = NZ * W * W; // cached values per lane
    static constexpr int GPW = 32 / ZS;   // lane groups per warp
};

// Dense-homed markers by home unit: a group of ZS lanes per (unit,
// component) of a dense work item loads the unit's W^d grid values once
// (NZ planes per lane) and sums every marker of the unit from registers.
// Each lane forms sum_y w_y sum_x w_x u for its planes; the first lane of
// the group gathers the plane sums with shuffles and adds them in z order,
// so the sum order is the chunked form's.
// One dense work item (item_units home units of one tile), by every thread
// of a CTA of INTERP_THREADS (it holds CTA barriers; the caller has finished
// with s_order / s_start of the previous item).
template <int DIM, int K>
__device__ __forceinline__ void
units_item(const DevPlan& D, int item, int* s_order, int* s_start)
{
    constexpr int W = KT<K>::W;
    using US = UnitSplit<DIM, W>;
    constexpr int ZS = US::ZS, NZ = US::NZ, NC = US::NC;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = lane < US::GPW * ZS;       // lanes beyond the last full group idle
    const int zh = lane % ZS;                       // this lane's planes: zh * NZ ...
    const int lead = lane - zh;                     // first lane of the group
    const unsigned gmask = ((1u << ZS) - 1u) << lead; // the group's lanes
    const int group = warp * US::GPW + lane / ZS;
    const int n_groups = (INTERP_THREADS / 32) * US::GPW;
    {
        const int t = D.item_tile[item];
        const int k = item - D.items[t];
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        const int ncomp = P.ncomp;
        int u0, nu;
        item_unit_range(D, t, k, u0, nu);
        float* Qi = static_cast<float*>(P.Qi);
        const long long n0 = P.N[0], n01 = (long long)P.N[0] * P.N[1];
        // the item's units, longest first, as in the dense spread
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
        __syncthreads();
        if (!active) return;
        for (int pair = group; pair < nu * ncomp; pair += n_groups)
        {
            const int c = pair % ncomp;
            const int2 un = D.home_units[u0 + s_order[pair / ncomp]];
            if (un.y <= 0) continue;
            const float* q = static_cast<const float*>(P.qi[c]);
            float uv[NC];
            {
                int co[3][W];
                stencil_cells<DIM, W>(P, D.hrec[un.x], c, co);
#pragma unroll
                for (int j2 = 0; j2 < NZ; ++j2)
                {
                    // plane zh * NZ + j2, selected without dynamic indexing
                    int cz = co[2][j2];
#pragma unroll
                    for (int h = 1; h < ZS; ++h)
                        if (zh == h) cz = co[2][h * NZ + j2];
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0)
                            uv[(j2 * W + i1) * W + i0] =
                                __ldg(q + (DIM == 3 ? cz * n01 : 0) + co[1][i1] * n0 + co[0][i0]);
                }
            }
            // Markers of the unit, software-pipelined: the next marker's
            // record and id are loaded before the current marker's arithmetic.
            const int vend = un.x + un.y;
            Rec Rn = D.hrec[un.x];
            int gn = D.home_list[un.x];
            for (int v = un.x; v < vend; ++v)
            {
                const Rec R = Rn;
                const int g = gn;
                if (v + 1 < vend)
                {
                    Rn = D.hrec[v + 1];
                    gn = D.home_list[v + 1];
                }
                float w[3][W];
                record_weights<DIM, K>(P, R, c, w);
                float vy[NZ];
#pragma unroll
                for (int j2 = 0; j2 < NZ; ++j2)
                {
                    float acc = 0.f;
#pragma unroll
                    for (int i1 = 0; i1 < W; ++i1)
                    {
                        float vx = 0.f;
#pragma unroll
                        for (int i0 = 0; i0 < W; ++i0) vx = fmaf(w[0][i0], uv[(j2 * W + i1) * W + i0], vx);
                        acc = fmaf(w[1][i1], vx, acc);
                    }
                    vy[j2] = acc;
                }
                float V = 0.f;
#pragma unroll
                for (int z = 0; z < (DIM == 3 ? W : 1); ++z)
                {
                    const float vz = ZS == 1 ? vy[z % NZ] : __shfl_sync(gmask, vy[z % NZ], lead + z / NZ);
                    V = fmaf(DIM == 3 ? w[2][z] : 1.f, vz, V);
                }
                if (zh == 0) Qi[(long long)P.Q_depth * (g - P.marker0) + c] = V;
            }
        }
    }
}

} // namespace
} // namespace ibx
