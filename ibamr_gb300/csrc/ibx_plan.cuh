// ibx_plan.cuh -- data structures and device helpers of the binned plan
// pipeline (bin -> scan -> scatter -> spread / interpolate).
#pragma once

#include "ibx_internal.h"

#include <cuda.h> // CUtensorMap

namespace ibx
{
// Tile shapes (cells per dimension), chosen per plan:
//   shape 0: 8 x 8 x 8 in 3D, 16 x 16 in 2D;
//   shape 1: 16 x 8 x 8 in 3D, 32 x 16 in 2D (longer x rows, fewer tiles
//            visited per marker, larger dense-tile regions).
constexpr int N_TILE_SHAPES = 2;

template <int DIM, int SH>
struct TileT
{
    static constexpr int E0 = DIM == 3 ? (SH == 0 ? 8 : 16) : (SH == 0 ? 16 : 32);
    static constexpr int E1 = DIM == 3 ? 8 : 16;
    static constexpr int E2 = DIM == 3 ? 8 : 1;
    static constexpr int PTS = E0 * E1 * E2;
    __host__ __device__ static constexpr int
    edge(int d)
    {
        return d == 0 ? E0 : d == 1 ? E1 : E2;
    }
};

// Threads per (unit, component) of the dense-tile spread: a 4 x 4 x 4
// footprint is split into two z-halves held by adjacent threads (32
// accumulators each), a 6 x 6 x 6 one into six z-planes (36 each), other
// footprints are held by one thread.
__host__ __device__ constexpr int
dense_zsplit(int dim, int width)
{
    return dim == 3 && width == 4 ? 2 : dim == 3 && width == 6 ? 6 : 1;
}

// Stencil width of a kernel id (host side).
inline int
kernel_width(int kernel)
{
    return kernel == K_PL ? 2 : kernel == K_IB3 ? 3 : kernel == K_IB6 ? 6 : 4;
}

// Tile edges of a shape at run time (host side).
inline void
tile_edges(int dim, int shape, int* e)
{
    e[0] = dim == 3 ? (shape == 0 ? 8 : 16) : (shape == 0 ? 16 : 32);
    e[1] = dim == 3 ? 8 : 16;
    e[2] = dim == 3 ? 8 : 1;
}

// Per-marker stencil record (32 bytes: one DRAM sector).  For every
// dimension: the stencil base (relative to the box's lower index, shifted by
// a multiple of N into [0, N) for the cell-centred one) of the cell-centred
// and of the staggered (side-normal) position, and r_first = t - (base +
// 1/2), the distance in cells of the marker from the first stencil point,
// computed exactly and rounded once to FP32.  The staggered position is half
// a cell above the cell-centred one, so its base is the cell-centred base or
// the next cell: the bases pack into one word, 16 bits of cell-centred base
// per dimension and one bit per dimension for the staggered step.  Markers
// with equal words share the stencils of every component.
struct __align__(16) Rec
{
    float rc[3];
    float rs[3];
    unsigned long long key;

    __host__ __device__ __forceinline__ int bc(int d) const { return (short)(unsigned short)(key >> (16 * d)); }
    __host__ __device__ __forceinline__ int bs(int d) const { return bc(d) + (int)((key >> (48 + d)) & 1u); }
    __host__ __device__ __forceinline__ int stagger(int d) const { return (int)((key >> (48 + d)) & 1u); }
};
static_assert(sizeof(Rec) == 32, "one record per 32-byte sector");

// Exact fixed-point description of t = (X - x_lower)/dx for one dimension
// (see ibx_bin.cu): Xf = floor(X*2^sx), D = Xf - xlo_f, T = mulhi(D, inv_f),
// t = T / 2^F up to 2^-40 cells.
struct FixedDim
{
    long long xlo_c_f, xlo_s_f; // x_lower and x_lower - dx/2 in units of 2^-sx
    long long inv_f;            // 1/dx in units of 2^-si
    int sx, F;                  // F = sx + si - 64
    int dshift;                 // decision margin: 2^dshift units of 2^-F
};

// Per-problem data (device side).
struct PlanProb
{
    int dim, ncomp, side, Q_depth;
    int N[3];          // cells per dim
    int ntile[3];      // tiles per dim
    int tile0;         // first global tile id of this problem
    long long marker0; // first global marker id of this problem
    double dx[3], inv_dx[3];
    double xlo_c[3], xlo_s[3];
    int dx_pow2[3];
    int fixed_ok;      // the fixed-point index path is valid for this problem
    FixedDim fx[3];
    float inv_vol;     // 1/(dx0*dx1[*dx2]) rounded to FP32
    int vec4;          // N[0] % 4 == 0 and every spread target 16-byte aligned
    int tma;           // interior tile regions of the interpolation sources load by TMA
    const double* X;
    void* Q;           // spread source
    void* q[3];        // spread target, one array per component (side axis or cell depth)
    void* Qi;          // interpolation target
    void* qi[3];       // interpolation source
};

// Device view of a plan.  Markers whose home tile holds more than dense_min
// markers ("dense-homed") are spread once each, by their home tile, into a
// shared-memory region covering the tile and its stencil halo; every other
// marker is listed once per tile its footprint touches ("visits") and spread
// by the owner of each visited tile.
struct DevPlan
{
    const PlanProb* probs;
    const long long* marker_offs; // [n_probs+1]
    const int* tile_offs;         // [n_probs+1]
    int n_probs;
    long long n_markers;
    int n_tiles;
    Rec* rec;         // [n_markers], original marker order
    Rec* hrec;        // [n_markers], home-tile order (same order as home_list)
    int* home_tile;   // [n_markers]
    // Counters (zeroed together each step; the *count arrays are scanned in
    // place into start offsets; hcount/hucount and vcount/items are
    // adjacent so that each pair is scanned by one launch).
    int* hcount;      // [n_tiles+1] markers per home tile
    int* hucount;     // [n_tiles+1] home units per tile
    int* vcount;      // [n_tiles+1] visits per tile (sparse-homed markers only)
    int* items;       // [n_tiles+1] dense-tile spread work items, scanned into offsets
    int* hcursor;     // [n_tiles]
    int* hucursor;    // [n_tiles]
    int* vcursor;     // [n_tiles]
    int* home_list;   // [n_markers] global marker ids grouped by home tile
    int* visit_list;  // [n_visit_cap] global marker ids grouped by visited tile
    long long n_visit_cap;
    // A home unit is a run of consecutive home-list entries that share the
    // tile and every stencil base: (start in the list, length).
    int2* home_units; // [n_markers]
    int* item_tile;   // [n_item_cap] tile of each work item
    int n_item_cap;
    int item_units;   // home units per dense work item (one per thread, <= 256)
    int dense_min;    // a home tile with more markers than this is dense
    int dense_blocks_per_sm; // CTAs per SM of the dense spread grid
    int max_ncomp;    // largest component count over the problems
    int zsplit;       // dense_zsplit(dim, kernel width)
    int visit_kernel; // 0: points of 32 visits flattened over lanes; 1: lane per (visit, component); 2: tile gathered
    int interp_form;  // 0: chunks in home order; 1: dense-homed per home unit; 2: chunks in marker order;
                      // 3: every marker from TMA-staged tile regions; 4: dense-homed from staged regions
    int unit_cap;     // most markers per home unit (1..32)
    int tile_shape;   // TileT shape id of every tile of the plan
    int* status;      // error word: bit 0 non-finite position, bit 1 visit overflow, bit 2 wait timeout
    int* work;        // [3] work counters (dense spread items, visited tiles, dense interpolation items),
                      // zeroed before each launch that takes from them
    // Tensor maps of the interpolation sources, 3 per problem (one per
    // component), valid where the problem's tma flag is set.
    const CUtensorMap* tmaps;
    // Positions of this step read from page-locked host memory by the
    // binning (x_src, dim values per marker in global marker order) and
    // stored on the way into the plan's position array (x_dst); null: the
    // binning reads the problems' X.  Set only in the copy of the plan passed
    // to one step's binning (ibx_plan_step_io).
    const double* x_src;
    double* x_dst;
};

// Region of an interpolation source staged for the markers homed in one
// tile: every cell of their stencils, for both the cell-centred and the
// staggered position.  The markers' cell-centred bases lie in [org - H,
// org + E - 1 - H] (H = (W - 1) / 2 below the home cell), the staggered ones
// one cell higher at most, so E + W cells per dimension cover them; along x
// the region starts at org - 4, a 16-byte boundary (tile origins are
// multiples of 8), and spans E + 8 cells.  CS: floats per component in
// shared memory (a multiple of 32 so that every component starts on a
// 128-byte boundary).
template <int DIM, int W, int SH>
struct IBox
{
    using T = TileT<DIM, SH>;
    static constexpr int H = (W - 1) / 2;
    static constexpr int X0 = 4; // region x origin = org - X0
    static constexpr int BX = T::E0 + 8;
    static constexpr int BY = T::E1 + W;
    static constexpr int BZ = DIM == 3 ? T::E2 + W : 1;
    static constexpr int PTS = BX * BY * BZ;
    static constexpr int CS = (PTS + 31) / 32 * 32;
    // highest x index: (E0 - 1) + 1 (stagger) + (W - 1) + (X0 - H) <= BX - 1
    static_assert(W - H <= 4, "the x extent covers every stencil");
    static_assert((BX * 4) % 16 == 0 && BX <= 256 && BY <= 256 && BZ <= 256, "TMA box rules");
};

// Host side: encodes the tensor maps of every problem's interpolation
// sources (maps[3 * p + c]) and sets each problem's tma flag; problems whose
// layout TMA cannot address (x extent not a multiple of 4 values, a grid
// smaller than the box, a misaligned base) keep the flag clear and load
// their regions with plain loads.
void encode_interp_maps(int dim, int kernel, int tile_shape, PlanProb* probs, int n_probs, CUtensorMap* maps);

// Block sums of the exclusive scans: up to 2 arrays of up to 2048 blocks.
constexpr int SCAN_TMP_INTS = 2 * 2048;

// Number of ints of the counter block starting at hcount: hcount, hucount,
// vcount and items ([n_tiles + 1] each; the pairs hcount/hucount and
// vcount/items are adjacent so that each pair scans in one launch), then the
// three cursors ([n_tiles] each).
__host__ __device__ inline size_t
counter_ints(int n_tiles)
{
    return 7 * (size_t)n_tiles + 4;
}

// Buffer layout of a plan for the given sizes; with base == nullptr only the
// byte count is computed.  The problem table, marker and tile offsets are at
// the returned offsets (to be filled by the caller).
struct PlanSizes
{
    int tile_shape;
    int n_probs;
    long long n_markers;
    int n_tiles;
    long long visit_cap;
    long long item_cap;
};
struct PlanCarve
{
    size_t bytes, o_probs, o_moffs, o_toffs, o_status, o_tmaps;
    int* scan_tmp;
};
PlanCarve carve_plan(const PlanSizes& z, char* base, DevPlan& D);

// Constants of the exact fixed-point index path for one dimension; false
// when the problem's coordinate range does not fit it.
bool fixed_dim(double x_lower, double x_upper, double dx, FixedDim& fx);

// The binning sequence of one step (counters zeroed, bin, scans, home
// placement, dense work items, visit placement) on stream s; records_done
// and records_done2 (optional) are recorded once the stencil records and
// home tiles exist (before the counting sort).  defer_visits: the visit
// placement is left out, for the caller to launch (launch_visits) beside the
// kernels that do not read the visits (the dense-tile spread, the
// interpolation).
int bin_sequence(int dim, int kernel, const DevPlan& D, int* scan_tmp, cudaStream_t s,
                 cudaEvent_t records_done = nullptr, cudaEvent_t records_done2 = nullptr,
                 bool defer_visits = false);

// Home units [u0, u0 + nu) of dense work item k of tile t: the tile's units
// split evenly over its items (ceil(units / item_units) items, so at most
// item_units each), which keeps the longest item short.
__device__ __forceinline__ void
item_unit_range(const DevPlan& D, int t, int k, int& u0, int& nu)
{
    const int ub = D.hucount[t], ut = D.hucount[t + 1] - ub;
    const int ni = D.items[t + 1] - D.items[t];
    const int a = (int)((long long)ut * k / ni), b = (int)((long long)ut * (k + 1) / ni);
    u0 = ub + a;
    nu = b - a;
}

template <typename T>
__device__ __forceinline__ int
find_in_offsets(const T* offs, int n, T g)
{
    int lo = 0, hi = n - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (offs[mid] <= g)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int
wrap_cell(int c, int N)
{
    while (c >= N) c -= N;
    while (c < 0) c += N;
    return c;
}

// First cell of local tile lt of a problem.
template <int DIM, int SH>
__device__ __forceinline__ void
tile_origin(const PlanProb& P, int lt, int* org)
{
    using T = TileT<DIM, SH>;
    org[0] = (lt % P.ntile[0]) * T::E0;
    org[1] = ((lt / P.ntile[0]) % P.ntile[1]) * T::E1;
    org[2] = DIM == 3 ? (lt / (P.ntile[0] * P.ntile[1])) * T::E2 : 0;
}

// Cell x = b + i of a stencil whose base b lies in [0, N] (the bases of a
// plan's records), wrapped into [0, N): one conditional subtraction unless
// the grid is narrower than the stencil.
__device__ __forceinline__ int
wrap_from_base(int x, int N)
{
    if (x >= N) x -= N;
    return x < N ? x : wrap_cell(x, N);
}

// ---- FP32 weights (mixed form) --------------------------------------------
// sqrt(a) rounded to nearest for a > 0 (the IEEE square root of CUDA's
// __fsqrt_rn), 0 for a <= 0.
__device__ __forceinline__ float
sqrt_f32(float a)
{
    return a > 0.f ? __fsqrt_rn(a) : 0.f;
}

__device__ __forceinline__ float
pcubic_f(float r)
{
    r = fabsf(r);
    if (r < 1.f) return 1.f - 0.5f * r - r * r + 0.5f * r * r * r;
    if (r < 2.f) return 1.f - (11.f / 6.f) * r + r * r - (1.f / 6.f) * r * r * r;
    return 0.f;
}
__device__ __forceinline__ float
ib3_f(float r)
{
    r = fabsf(r);
    if (r < 0.5f) return 0.333333333333333f * (1.f + sqrt_f32(1.f - 3.f * r * r));
    if (r < 1.5f) return 0.16666666666667f * (5.f - 3.f * r - sqrt_f32(1.f - 3.f * (1.f - r) * (1.f - r)));
    return 0.f;
}
// The cubic B-spline of FDELTA:268-294 in the same pieces (|x| <= 1,
// |x| <= 2), written in |x| itself: the reference's polynomials in
// r = |x| + 2 (FP64 path, ibx_device.cuh) expand to (4 - 6 x^2 + 3 |x|^3) / 6
// and (2 - |x|)^3 / 6, which FP32 evaluates without the cancellation of terms
// of size ~200 that the r form suffers.
__device__ __forceinline__ float
bspline4_f(float x)
{
    const float m = fabsf(x);
    if (m <= 1.f) return (2.f / 3.f) - m * m + 0.5f * (m * m * m);
    if (m <= 2.f)
    {
        const float t = 2.f - m;
        return (1.f / 6.f) * (t * t * t);
    }
    return 0.f;
}

// The W weights of one dimension from r_first; the formulas of the FP64
// path (ibx_device.cuh) evaluated in FP32 (the B-spline in an equal,
// better-conditioned form).
template <int K>
__device__ __forceinline__ void
weights_f32(float rf, float* w)
{
    if (K == K_IB4)
    {
        const float r = rf - 1.f;
        const float q = sqrt_f32(1.f + 4.f * r * (1.f - r));
        w[0] = 0.125f * (3.f - 2.f * r - q);
        w[1] = 0.125f * (3.f - 2.f * r + q);
        w[2] = 0.125f * (1.f + 2.f * r + q);
        w[3] = 0.125f * (1.f + 2.f * r - q);
    }
    else if (K == K_IB6)
    {
        // The IB_6 quadratic-root weights (ib6_weights) in FP32.
        const float r = 3.f - rf;
        const float Kc = 0.714075092976608f;
        const float r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r6 = r3 * r3;
        const float beta = (9.f / 4.f) - (3.f / 2.f) * (Kc + r2) + ((22.f / 3.f) - 7.f * Kc) * r - (7.f / 3.f) * r3;
        const float gamma = 0.25f * (((161.f / 36.f) - (59.f / 6.f) * Kc + 5.f * Kc * Kc) * 0.5f * r2 +
                                     (-(109.f / 24.f) + 5.f * Kc) * (1.f / 3.f) * r4 + (5.f / 18.f) * r6);
        const float discr = beta * beta - 112.f * gamma;
        const float pm3 = (-beta + sqrt_f32(discr)) * (1.f / 56.f);
        w[0] = pm3;
        w[1] = -(3.f * pm3) - (1.f / 16.f) + 0.125f * (Kc + r2) + (1.f / 12.f) * (3.f * Kc - 1.f) * r + (1.f / 12.f) * r3;
        w[2] = 2.f * pm3 + 0.25f + (1.f / 6.f) * (4.f - 3.f * Kc) * r - (1.f / 6.f) * r3;
        w[3] = 2.f * pm3 + (5.f / 8.f) - 0.25f * (Kc + r2);
        w[4] = -(3.f * pm3) + 0.25f - (1.f / 6.f) * (4.f - 3.f * Kc) * r + (1.f / 6.f) * r3;
        w[5] = pm3 - (1.f / 16.f) + 0.125f * (Kc + r2) - (1.f / 12.f) * (3.f * Kc - 1.f) * r - (1.f / 12.f) * r3;
    }
    else if (K == K_PL)
    {
        w[0] = 1.f - rf;
        w[1] = rf;
    }
    else
    {
#pragma unroll
        for (int i = 0; i < KT<K>::W; ++i)
        {
            const float a = rf - (float)i;
            w[i] = (K == K_IB3) ? ib3_f(a) : (K == K_PCUBIC) ? pcubic_f(a) : bspline4_f(a);
        }
    }
}

// Compensated accumulation into shared memory: the FP32 atomic returns the
// previous value, so the exact rounding error of the stored sum follows from
// Knuth's TwoSum and is accumulated into the low word (double-FP32 sum).
__device__ __forceinline__ void
acc2(float* hi, float* lo, float v)
{
    const float old = atomicAdd(hi, v);
    const float s = old + v;
    const float bp = s - old;
    const float err = (old - (s - bp)) + (v - bp);
    if (err != 0.f) atomicAdd(lo, err);
}

// Launchers (ibx_bin.cu, ibx_spread.cu, ibx_interp.cu).
// phase 0: bin (records, home counts); 1: home placement and visit counts;
// 2: visit placement.  The tile shape is D.tile_shape.
int launch_bin(int dim, int kernel, const DevPlan& D, cudaStream_t s, int phase);
// Exclusive scans of `count` arrays of n ints laid out back to back; tmp
// holds count * 2048 ints.
int exclusive_scan(int* data, int n, int count, int* tmp, cudaStream_t s);
int launch_items_fill(const DevPlan& D, cudaStream_t s);
// The visit placement (launch_bin phase 2) of a binning run with
// defer_visits.
int launch_visits(int dim, int kernel, const DevPlan& D, cudaStream_t s);
// The dense-tile spread, then the per-visit spread; visits_done (optional):
// an event the per-visit kernel waits for (the deferred visit placement).
int launch_spread(int dim, int kernel, const DevPlan& D, int max_ncomp, cudaStream_t s,
                  cudaEvent_t visits_done = nullptr);
// Spread and interpolation of the binned markers in one persistent launch
// (ibx_spread.cu: step_fused).
int launch_fused(int dim, int kernel, const DevPlan& D, int max_ncomp, cudaStream_t s);
int launch_interp(int dim, int kernel, const DevPlan& D, cudaStream_t s);

} // namespace ibx
