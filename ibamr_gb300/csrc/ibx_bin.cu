// ibx_bin.cu -- marker binning of the plan pipeline: exact stencil indices,
// integer counting sort by tile, work items of the tiled spread.
//
// Index arithmetic.  The reference computes t = (X + Xshift - x_lower)/dx in
// FP64 and takes NINT(t) (IB_4, IB_6), floor(t) (IB_3, PIECEWISE_CUBIC,
// BSPLINE_4) or NINT(t - 1/2) plus a half-cell test (PIECEWISE_LINEAR)
// (F3D:1265-1293, 2244-2330, 808-840, 305-330).  GB300 executes FP64 at
// about 1/70 of the FP32 rate, so t is formed here in 64-bit fixed point on
// the integer pipe: Xf = floor(X*2^sx) from the bits of X, D = Xf - xlo_f,
// T = mulhi(D, inv_f), t = T/2^F with |t - t_real| < 2^-44.  The FP64 value
// the reference rounds differs from t_real by a few ulps of t, so every
// decision (integer and half-integer crossings) is taken from T unless T
// lies within a margin of 16 ulps of the largest t of the problem from a
// decision boundary; those rare markers (and any position outside the
// fixed-point range) are recomputed with the reference's FP64 expressions.
// Either way the stencil indices are bit-identical to the reference's.

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
// floor(x * 2^S) for |x| * 2^S < 2^62; ok = false otherwise (or non-finite).
__device__ __forceinline__ long long
to_fixed(double x, int S, bool& ok)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    ok = false;
    if (e == 0x7FF) return 0;
    unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    int ee = e;
    if (e)
        m |= 1ull << 52;
    else
        ee = 1;
    const int sh = ee - 1075 + S; // x*2^S = m * 2^sh
    unsigned long long v;
    bool exact;
    if (sh >= 0)
    {
        if (sh > 9) return 0; // |x|*2^S >= 2^62
        v = m << sh;
        exact = true;
    }
    else
    {
        const int r = -sh;
        if (r >= 64)
        {
            v = 0;
            exact = m == 0;
        }
        else
        {
            v = m >> r;
            exact = (m & ((1ull << r) - 1)) == 0;
        }
    }
    long long out = (long long)v;
    if (b >> 63) out = -out - (exact ? 0 : 1);
    ok = true;
    return out;
}

// Exact stencil base and r_first by the reference's FP64 expressions (the
// fallback; see stencil_fp64 in ibx_device.cuh for the per-kernel rules).
template <int K>
__device__ __noinline__ void
base_r_fp64(double X, double xlo, double dx, double inv_dx, int pow2, int& base, float& rfirst)
{
    const double v = __dsub_rn(X, xlo);
    const double t = clamp_index_arg(pow2 ? __dmul_rn(v, inv_dx) : __ddiv_rn(v, dx));
    if (K == K_IB4)
        base = nint_exact(t) - 2;
    else if (K == K_IB6)
        base = nint_exact(t) - 3;
    else if (K == K_PL)
    {
        const int icc = nint_exact(__dsub_rn(t, 0.5));
        base = (X < cell_center(icc, xlo, dx)) ? icc - 1 : icc;
    }
    else
    {
        const int icc = (int)floor(t);
        if (K == K_IB3)
            base = icc - 1;
        else
            base = (X < cell_center(icc, xlo, dx)) ? icc - 2 : icc - 1;
    }
    rfirst = (float)(t - ((double)base + 0.5));
}

// Base and r_first from the fixed-point t; returns false when t is within
// the margin of a decision boundary.
template <int K>
__device__ __forceinline__ bool
base_r_fixed(long long Xf, long long xlo_f, long long inv_f, int F, int dshift, int& base, float& rfirst)
{
    const long long D = Xf - xlo_f;
    const long long T = __mul64hi(D, inv_f);
    const long long one = 1ll << F;
    const long long half = one >> 1;
    const long long fr = T & (one - 1);
    const long long dl = 1ll << dshift;
    if (fr < dl || fr > one - dl || (fr > half - dl && fr < half + dl)) return false;
    const int ip = (int)(T >> F);
    const bool up = fr >= half;
    if (K == K_IB4)
        base = ip + (up ? 1 : 0) - 2;
    else if (K == K_IB6)
        base = ip + (up ? 1 : 0) - 3;
    else if (K == K_PL)
        base = up ? ip : ip - 1;
    else if (K == K_IB3)
        base = ip - 1;
    else
        base = up ? ip - 1 : ip - 2;
    const long long rf = T - ((long long)base << F) - half;
    rfirst = __ll2float_rn(rf) * __int_as_float((127 - F) << 23);
    return true;
}

// Warp-aggregated counter increment (no result is read back, so the add
// compiles to a reduction): one atomic per group of lanes with equal keys.
__device__ __forceinline__ void
agg_count(int* counters, int key, bool valid)
{
    const unsigned act = __ballot_sync(__activemask(), valid);
    if (valid)
    {
        const unsigned grp = __match_any_sync(act, key);
        if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&counters[key], __popc(grp));
    }
}

// Distinct tiles (along one dim, at most 4, in order of first appearance)
// holding the cells (b+i) mod N, i in [0, span), span <= MAXSPAN; unrolled,
// with the list in registers (no dynamic indexing).
template <int MAXSPAN, int E>
__device__ __forceinline__ int
tiles_1d(int b, int span, int N, int* out)
{
    int o0 = 0, o1 = 0, o2 = 0, o3 = 0, n = 0;
#pragma unroll
    for (int i = 0; i < MAXSPAN; ++i)
    {
        if (i >= span) break;
        const int tile = wrap_from_base(b + i, N) / E;
        const bool seen = (n > 0 && o0 == tile) || (n > 1 && o1 == tile) || (n > 2 && o2 == tile) ||
                          (n > 3 && o3 == tile);
        if (!seen && n < 4)
        {
            o0 = n == 0 ? tile : o0;
            o1 = n == 1 ? tile : o1;
            o2 = n == 2 ? tile : o2;
            o3 = n == 3 ? tile : o3;
            ++n;
        }
    }
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
    out[3] = o3;
    return n;
}

template <int DIM, int K, int SH>
__device__ __forceinline__ int
visit_tiles(const PlanProb& P, const Rec& R, int (*tl)[4], int* nt)
{
    constexpr int W = KT<K>::W;
    int total = 1;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        if (d >= DIM)
        {
            nt[d] = 1;
            tl[d][0] = tl[d][1] = tl[d][2] = tl[d][3] = 0;
            continue;
        }
        const int lo = R.bc(d);
        const int span = (P.side ? R.stagger(d) : 0) + W;
        nt[d] = d == 0   ? tiles_1d<W + 1, TileT<DIM, SH>::E0>(lo, span, P.N[d], tl[d])
                : d == 1 ? tiles_1d<W + 1, TileT<DIM, SH>::E1>(lo, span, P.N[d], tl[d])
                         : tiles_1d<W + 1, TileT<DIM, SH>::E2>(lo, span, P.N[d], tl[d]);
        total *= nt[d];
    }
    return total;
}

__device__ __forceinline__ int
pick4(const int* a, int i)
{
    return i == 0 ? a[0] : i == 1 ? a[1] : i == 2 ? a[2] : a[3];
}

// The tile of the visit whose per-dim tile digits are c (c[0] fastest).
template <int DIM>
__device__ __forceinline__ int
visit_tile_at(const PlanProb& P, int (*tl)[4], const int* c)
{
    return P.tile0 + pick4(tl[0], c[0]) +
           P.ntile[0] * (pick4(tl[1], c[1]) + (DIM == 3 ? P.ntile[1] * pick4(tl[2], c[2]) : 0));
}

// The next visit's digits: a mixed-radix counter over nt (no divisions).
__device__ __forceinline__ void
visit_next(int* c, const int* nt)
{
    if (++c[0] == nt[0])
    {
        c[0] = 0;
        if (++c[1] == nt[1])
        {
            c[1] = 0;
            ++c[2];
        }
    }
}

// The stencil bases of a record as one 64-bit key: markers with equal keys
// share the stencil of every component.
__device__ __forceinline__ unsigned long long
base_key(const Rec& R)
{
    return R.key;
}

// Lanes of the active set that share both the tile and the stencil key,
// split into groups of at most cap lanes (by rank within the group).
__device__ __forceinline__ unsigned
unit_group(unsigned act, int tile, unsigned long long key, int cap = 32)
{
    const unsigned grp = __match_any_sync(act, tile) & __match_any_sync(act, key);
    if (cap >= 32) return grp;
    const int sub = __popc(grp & ((1u << (threadIdx.x & 31)) - 1)) / cap;
    return grp & __match_any_sync(act, sub);
}

// Phase 0: one thread per marker derives the record (exact stencil bases
// and kernel arguments of the cell-centred and staggered positions) and its
// home tile, and counts the marker and its unit (warp-local run of markers
// with equal stencil bases) into the home tile.
template <int DIM, int K, int SH>
__global__ void __launch_bounds__(256) bin_kernel(const DevPlan D)
{
    constexpr int W = KT<K>::W;
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    bool valid = g < D.n_markers;
    const int p = (!valid || D.n_probs == 1) ? 0 : find_in_offsets(D.marker_offs, D.n_probs, g);
    const PlanProb& P = D.probs[p];
    Rec R;
    int home[3] = { 0, 0, 0 };
    if (valid)
    {
        const long long s = g - P.marker0;
        bool finite = true;
        unsigned long long rkey = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            if (d >= DIM)
            {
                R.rc[d] = R.rs[d] = 0.f;
                continue;
            }
            double X;
            if (D.x_src)
            {
                X = D.x_src[DIM * g + d];
                D.x_dst[DIM * g + d] = X;
            }
            else
                X = P.X[DIM * s + d];
            finite = finite && isfinite(X);
            const FixedDim& fx = P.fx[d];
            int bc, bs;
            float rc, rs;
            bool ok = P.fixed_ok != 0;
            long long Xf = 0;
            if (ok) Xf = to_fixed(X, fx.sx, ok);
            if (!(ok && base_r_fixed<K>(Xf, fx.xlo_c_f, fx.inv_f, fx.F, fx.dshift, bc, rc)))
                base_r_fp64<K>(X, P.xlo_c[d], P.dx[d], P.inv_dx[d], P.dx_pow2[d], bc, rc);
            if (!(ok && base_r_fixed<K>(Xf, fx.xlo_s_f, fx.inv_f, fx.F, fx.dshift, bs, rs)))
                base_r_fp64<K>(X, P.xlo_s[d], P.dx[d], P.inv_dx[d], P.dx_pow2[d], bs, rs);
            // Periodic domain: move both bases by the multiple of N that puts bc in [0, N).
            const int N = P.N[d];
            // (no division for markers within one period of the box)
            const int shift = (bc >= 0 && bc < N)   ? 0
                              : (bc >= N && bc < 2 * N) ? N
                              : (bc < 0 && bc >= -N)    ? -N
                              : (bc >= 0 ? bc / N : -((-bc + N - 1) / N)) * N;
            bc -= shift;
            bs -= shift;
            rkey |= (unsigned long long)(unsigned short)bc << (16 * d);
            rkey |= (unsigned long long)(bs - bc == 1) << (48 + d);
            finite = finite && (bs - bc == 0 || bs - bc == 1);
            R.rc[d] = rc;
            R.rs[d] = rs;
            home[d] = wrap_from_base(bc + (W - 1) / 2, N) / TileT<DIM, SH>::edge(d);
        }
        R.key = rkey;
        if (!finite)
        {
            // Reported through the plan's status word; the marker is skipped.
            atomicOr(D.status, 1);
            D.home_tile[g] = -1;
            valid = false;
        }
    }
    int ht = 0;
    unsigned long long key = 0;
    if (valid)
    {
        D.rec[g] = R;
        ht = P.tile0 + home[0] + P.ntile[0] * (home[1] + (DIM == 3 ? P.ntile[1] * home[2] : 0));
        D.home_tile[g] = ht;
        key = base_key(R);
    }
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    bool lead = false;
    if (valid)
    {
        const unsigned grp = unit_group(act, ht, key, D.unit_cap);
        lead = (threadIdx.x & 31) == __ffs(grp) - 1;
    }
    agg_count(D.hcount, ht, valid);
    agg_count(D.hucount, ht, lead);
}

// Places a home unit group: its leader reserves a contiguous range of the
// list and one unit record; returns the lane's slot in the list.
__device__ __forceinline__ int
place_group(unsigned grp, int tile, int* cursor, const int* start, int* ucursor, const int* ustart, int2* units)
{
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (lane == leader)
    {
        const int n = __popc(grp);
        base = start[tile] + atomicAdd(&cursor[tile], n);
        const int u = ustart[tile] + atomicAdd(&ucursor[tile], 1);
        units[u] = make_int2(base, n);
    }
    base = __shfl_sync(grp, base, leader);
    return base + __popc(grp & ((1u << lane) - 1));
}

__device__ __forceinline__ bool
dense_home(const DevPlan& D, int ht)
{
    return D.hcount[ht + 1] - D.hcount[ht] > D.dense_min;
}

// Phase 1: counting sort by home tile (home list, home units and the records
// in home order); markers of sparse home tiles count their visits.
template <int DIM, int K, int SH>
__global__ void __launch_bounds__(256) scatter_home_kernel(const DevPlan D)
{
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    // Dense-tile spread work items: a home tile with more than dense_min
    // markers and u home units gets ceil(u / item_units) items.
    for (long long t = g; t < D.n_tiles; t += (long long)gridDim.x * blockDim.x)
    {
        const int u = D.hucount[t + 1] - D.hucount[t];
        D.items[t] = dense_home(D, (int)t) ? (u + D.item_units - 1) / D.item_units : 0;
    }
    bool valid = g < D.n_markers;
    const int ht = valid ? D.home_tile[g] : -1;
    valid = valid && ht >= 0;
    const int p = (!valid || D.n_probs == 1) ? 0 : find_in_offsets(D.marker_offs, D.n_probs, g);
    const PlanProb& P = D.probs[p];
    Rec R;
    unsigned long long key = 0;
    int tl[3][4], nt[3] = { 0, 0, 0 }, nvis = 0;
    if (valid)
    {
        R = D.rec[g];
        key = base_key(R);
    }
    {
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (valid)
        {
            const unsigned grp = unit_group(act, ht, key, D.unit_cap);
            const int pos = place_group(grp, ht, D.hcursor, D.hcount, D.hucursor, D.hucount, D.home_units);
            D.home_list[pos] = (int)g;
            D.hrec[pos] = R;
            if (!dense_home(D, ht)) nvis = visit_tiles<DIM, K, SH>(P, R, tl, nt);
        }
    }
    int cd[3] = { 0, 0, 0 };
    for (int k = 0; __any_sync(0xffffffffu, k < nvis); ++k)
    {
        const bool v = k < nvis;
        agg_count(D.vcount, v ? visit_tile_at<DIM>(P, tl, cd) : 0, v);
        if (v) visit_next(cd, nt);
    }
}

// Phase 2: counting sort of the visits of sparse-homed markers by visited tile.
template <int DIM, int K, int SH>
__global__ void __launch_bounds__(256) scatter_visits_kernel(const DevPlan D)
{
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    bool valid = g < D.n_markers;
    const int ht = valid ? D.home_tile[g] : -1;
    valid = valid && ht >= 0 && !dense_home(D, ht);
    const int p = (!valid || D.n_probs == 1) ? 0 : find_in_offsets(D.marker_offs, D.n_probs, g);
    const PlanProb& P = D.probs[p];
    int tl[3][4], nt[3] = { 0, 0, 0 }, nvis = 0;
    if (valid) nvis = visit_tiles<DIM, K, SH>(P, D.rec[g], tl, nt);
    int cd[3] = { 0, 0, 0 };
    for (int k = 0; __any_sync(0xffffffffu, k < nvis); ++k)
    {
        const bool v = k < nvis;
        const int t = v ? visit_tile_at<DIM>(P, tl, cd) : 0;
        if (v) visit_next(cd, nt);
        const unsigned act = __ballot_sync(0xffffffffu, v);
        if (v)
        {
            // lanes visiting the same tile share one reservation
            const unsigned grp = __match_any_sync(act, t);
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(grp) - 1;
            int base = 0;
            if (lane == leader) base = D.vcount[t] + atomicAdd(&D.vcursor[t], __popc(grp));
            const int pos = __shfl_sync(grp, base, leader) + __popc(grp & ((1u << lane) - 1));
            if (pos < D.n_visit_cap)
                D.visit_list[pos] = (int)g;
            else
                atomicOr(D.status, 2);
        }
    }
}

// ---- exclusive scan (two levels, exact integer) ---------------------------
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 2048; // elements per block

// Block-level Blelloch scan of array blockIdx.y (arrays of n ints, stride n).
__global__ void __launch_bounds__(SCAN_BLOCK) scan_blocks(int* data, int n, int* block_sums, int nb)
{
    __shared__ int s[SCAN_ITEMS];
    int* a = data + (long long)blockIdx.y * n;
    const int base = blockIdx.x * SCAN_ITEMS;
    for (int i = threadIdx.x; i < SCAN_ITEMS; i += SCAN_BLOCK) s[i] = (base + i < n) ? a[base + i] : 0;
    int offset = 1;
    for (int d = SCAN_ITEMS >> 1; d > 0; d >>= 1)
    {
        __syncthreads();
        if (threadIdx.x < d)
        {
            const int ai = offset * (2 * threadIdx.x + 1) - 1;
            const int bi = offset * (2 * threadIdx.x + 2) - 1;
            s[bi] += s[ai];
        }
        offset <<= 1;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        if (block_sums) block_sums[blockIdx.y * nb + blockIdx.x] = s[SCAN_ITEMS - 1];
        s[SCAN_ITEMS - 1] = 0;
    }
    for (int d = 1; d < SCAN_ITEMS; d <<= 1)
    {
        offset >>= 1;
        __syncthreads();
        if (threadIdx.x < d)
        {
            const int ai = offset * (2 * threadIdx.x + 1) - 1;
            const int bi = offset * (2 * threadIdx.x + 2) - 1;
            const int t = s[ai];
            s[ai] = s[bi];
            s[bi] += t;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < SCAN_ITEMS; i += SCAN_BLOCK)
        if (base + i < n) a[base + i] = s[i];
}

__global__ void scan_add(int* data, int n, const int* block_offsets, int nb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[(long long)blockIdx.y * n + i] += block_offsets[blockIdx.y * nb + i / SCAN_ITEMS];
}

__global__ void items_fill(const DevPlan D)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0 && D.items[D.n_tiles] > D.n_item_cap) atomicOr(D.status, 2);
    if (t >= D.n_tiles) return;
    for (int k = D.items[t]; k < D.items[t + 1] && k < D.n_item_cap; ++k) D.item_tile[k] = t;
}
} // namespace

// Exclusive scan of array blockIdx.x (n ints, arrays n apart) by one CTA:
// each thread sums a contiguous segment of at most SINGLE_PER values, the
// segment totals are scanned across the block with warp shuffles, and each
// thread rewrites its segment.  One launch for up to 1024 * SINGLE_PER values
// (beyond that the three-launch scan is faster: the single CTA's serial
// segments are latency-bound).
constexpr int SINGLE_PER = 8;

__global__ void __launch_bounds__(SCAN_BLOCK) scan_single(int* data, int n)
{
    __shared__ int warp_tot[SCAN_BLOCK / 32];
    int* a = data + (long long)blockIdx.x * n;
    const int per = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    const int b = min((int)threadIdx.x * per, n), e = min(b + per, n);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int sum = 0;
    for (int i = b; i < e; ++i) sum += a[i];
    int x = sum; // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        int t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    int run = x - sum + (warp ? warp_tot[warp - 1] : 0);
    for (int i = b; i < e; ++i)
    {
        const int v = a[i];
        a[i] = run;
        run += v;
    }
}

int
exclusive_scan(int* data, int n, int count, int* tmp, cudaStream_t s)
{
    if (n <= SCAN_BLOCK * SINGLE_PER)
    {
        scan_single<<<count, SCAN_BLOCK, 0, s>>>(data, n);
        note_launches(1);
        return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
    }
    const int nb = (n + SCAN_ITEMS - 1) / SCAN_ITEMS;
    if (nb > SCAN_ITEMS || (long long)nb * count > SCAN_TMP_INTS) return IBX_E_TOO_LARGE; // more than 4M entries
    scan_blocks<<<dim3(nb, count), SCAN_BLOCK, 0, s>>>(data, n, tmp, nb);
    if (nb > 1)
    {
        // tmp[a * nb + b]: block sums of array a, scanned per array.
        scan_blocks<<<dim3(1, count), SCAN_BLOCK, 0, s>>>(tmp, nb, nullptr, 1);
        scan_add<<<dim3((n + 255) / 256, count), 256, 0, s>>>(data, n, tmp, nb);
    }
    note_launches(nb > 1 ? 3 : 1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

int
launch_items_fill(const DevPlan& D, cudaStream_t s)
{
    const int blocks = (D.n_tiles + 255) / 256;
    items_fill<<<blocks, 256, 0, s>>>(D);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

namespace
{
template <int DIM, int K, int SH>
void
launch_bin_k(const DevPlan& D, cudaStream_t s, int phase, unsigned blocks)
{
    if (phase == 0)
        bin_kernel<DIM, K, SH><<<blocks, 256, 0, s>>>(D);
    else if (phase == 1)
        scatter_home_kernel<DIM, K, SH><<<blocks, 256, 0, s>>>(D);
    else
        scatter_visits_kernel<DIM, K, SH><<<blocks, 256, 0, s>>>(D);
    note_launches(1);
}
} // namespace

int
launch_bin(int dim, int kernel, const DevPlan& D, cudaStream_t s, int phase)
{
    const unsigned blocks = (unsigned)((D.n_markers + 255) / 256);
    if (blocks == 0) return IBX_OK;
    const int sh = D.tile_shape;
#define IBX_BIN_CASE(DD, KK)                                                                                         \
    if (dim == DD && kernel == KK)                                                                                   \
    {                                                                                                                \
        if (sh == 0)                                                                                                 \
            launch_bin_k<DD, KK, 0>(D, s, phase, blocks);                                                            \
        else                                                                                                         \
            launch_bin_k<DD, KK, 1>(D, s, phase, blocks);                                                            \
        return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;                                             \
    }
    IBX_BIN_CASE(2, K_PL) IBX_BIN_CASE(2, K_PCUBIC) IBX_BIN_CASE(2, K_IB3) IBX_BIN_CASE(2, K_IB4)
    IBX_BIN_CASE(2, K_IB6) IBX_BIN_CASE(2, K_BSPL4) IBX_BIN_CASE(3, K_PL) IBX_BIN_CASE(3, K_PCUBIC)
    IBX_BIN_CASE(3, K_IB3) IBX_BIN_CASE(3, K_IB4) IBX_BIN_CASE(3, K_IB6) IBX_BIN_CASE(3, K_BSPL4)
#undef IBX_BIN_CASE
    return IBX_E_BAD_KERNEL;
}

int
launch_visits(int dim, int kernel, const DevPlan& D, cudaStream_t s)
{
    return launch_bin(dim, kernel, D, s, 2);
}

int
bin_sequence(int dim, int kernel, const DevPlan& D, int* scan_tmp, cudaStream_t s, cudaEvent_t records_done,
             cudaEvent_t records_done2, bool defer_visits)
{
    const int nt = D.n_tiles;
    // Counters, cursors and item counts are contiguous: one memset.
    if (cudaMemsetAsync(D.hcount, 0, sizeof(int) * counter_ints(nt), s) != cudaSuccess) return IBX_E_CUDA;
    int rc = launch_bin(dim, kernel, D, s, 0);
    if (!rc && records_done && cudaEventRecord(records_done, s) != cudaSuccess) rc = IBX_E_CUDA;
    if (!rc && records_done2 && cudaEventRecord(records_done2, s) != cudaSuccess) rc = IBX_E_CUDA;
    if (!rc) rc = exclusive_scan(D.hcount, nt + 1, 2, scan_tmp, s); // hcount, hucount
    if (!rc) rc = launch_bin(dim, kernel, D, s, 1);                 // also counts the work items
    if (!rc) rc = exclusive_scan(D.vcount, nt + 1, 2, scan_tmp, s); // vcount, items
    if (!rc) rc = launch_items_fill(D, s);
    if (!rc && !defer_visits) rc = launch_bin(dim, kernel, D, s, 2);
    return rc;
}

} // namespace ibx
