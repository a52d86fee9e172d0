// ibx_noalloc.cu -- binned mixed-precision spreading without any device
// allocation (ibx_spread_noalloc in include/ibx.h).
//
// Some callers cannot call cudaMalloc at all: code that runs while a CUDA
// graph is being captured with a fixed memory footprint, host code inside a
// real-time or fault-handling path, or an embedding that forbids the CUDA
// allocator (for instance because a separate pool owns all device memory).
// For them the scratch memory of the binned pipeline (stencil records,
// tile counters, counting-sort lists, run units) lives in one file-scope
// __device__ array of fixed size, which every GPU that loads this library
// holds until the process exits.  The inputs and outputs stay the caller's.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it.  Make
// that first call before any stream capture.
//
// All calls share the one array and it keeps the contents of the last call:
// every call re-initialises what must start at zero, and calls whose work
// overlaps on the GPU (different streams, or different host threads on the
// same device without ordering) race on it.  Serialise them.

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

#include <cmath>
#include <cstring>
#include <mutex>

namespace
{
// Limits of the allocation-free path.
constexpr long long NOALLOC_MAX_MARKERS = IBX_NOALLOC_MAX_MARKERS;
constexpr int NOALLOC_MAX_TILES = IBX_NOALLOC_MAX_TILES;
constexpr int NOALLOC_UNITS_PER_ITEM = 256;
constexpr size_t NOALLOC_SCRATCH_BYTES = 6u << 20; // 6 MiB

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device (set-up on
// first use per device).
int
scratch_address(void** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return IBX_E_CUDA;
    if (dev < 0 || dev >= MAX_DEVICES) return IBX_E_TOO_LARGE;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev])
    {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return IBX_E_CUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return IBX_OK;
}

size_t
up256(size_t v)
{
    return (v + 255) & ~size_t(255);
}

int
ceil_log2_ld(long double v)
{
    int e = 0;
    while (std::ldexp(1.0L, e) < v) ++e;
    return e;
}

// Constants of the exact fixed-point index path (the rules of ibx_bin.cu).
bool
fixed_constants(double x_lower, double x_upper, double dx, ibx::FixedDim& fx)
{
    const long double xmax = 2.0L * std::max(std::fabs((long double)x_lower), std::fabs((long double)x_upper)) +
                             8.0L * dx + 1e-30L;
    fx.sx = 62 - ceil_log2_ld(xmax);
    const long double inv = 1.0L / (long double)dx;
    const int si = 62 - (std::ilogb(inv) + 1);
    fx.inv_f = std::llround(std::ldexp(inv, si));
    fx.F = fx.sx + si - 64;
    const int tb = ceil_log2_ld(xmax * inv + 2.0L);
    fx.dshift = fx.F - 48 + tb;
    fx.xlo_c_f = std::llround(std::ldexp((long double)x_lower, fx.sx));
    const double xlo_s = x_lower - 0.5 * dx;
    fx.xlo_s_f = std::llround(std::ldexp((long double)xlo_s, fx.sx));
    return fx.sx > 0 && fx.F >= 24 && fx.F <= 62 && fx.dshift >= 2 && fx.dshift <= fx.F - 4 && tb <= 30;
}
} // namespace

namespace ibx
{
int build_prob(const ibx_problem& in, int kernel, bool spread, Prob& P);
}

extern "C" int
ibx_spread_noalloc(const ibx_problem* problem, int kernel, void* stream)
{
    using namespace ibx;
    if (!problem) return IBX_E_ARG;
    const ibx_problem& in = *problem;
    Prob chk;
    const int rc0 = build_prob(in, kernel, true, chk);
    if (rc0) return rc0;
    if (in.mode != IBX_MODE_PERIODIC || in.indices || in.Xshift) return IBX_E_ARG;
    const int dim = in.dim;
    const int ncomp = in.centering == IBX_SIDE ? dim : in.q_depth;
    if (ncomp > 3) return IBX_E_TOO_LARGE;
    if ((long long)in.n_markers > NOALLOC_MAX_MARKERS) return IBX_E_TOO_LARGE;
    const int E = dim == 3 ? TILE3 : TILE2;

    // Problem descriptor (host side), as ibx_plan_create builds it.
    PlanProb P;
    std::memset(&P, 0, sizeof(P));
    P.dim = dim;
    P.ncomp = ncomp;
    P.side = in.centering == IBX_SIDE;
    P.Q_depth = in.Q_depth;
    long long ntiles = 1, vol = 1;
    bool fixed_ok = true;
    for (int d = 0; d < 3; ++d)
    {
        if (d >= dim)
        {
            P.N[d] = 1;
            P.ntile[d] = 1;
            P.dx[d] = P.inv_dx[d] = 1.0;
            continue;
        }
        P.N[d] = in.iupper[d] - in.ilower[d] + 1;
        if (P.N[d] > 30000) return IBX_E_TOO_LARGE;
        P.ntile[d] = (P.N[d] + E - 1) / E;
        ntiles *= P.ntile[d];
        vol *= P.N[d];
        P.dx[d] = chk.dx[d];
        P.inv_dx[d] = chk.inv_dx[d];
        P.dx_pow2[d] = chk.dx_pow2[d];
        P.xlo_c[d] = in.x_lower[d];
        P.xlo_s[d] = in.x_lower[d] - 0.5 * in.dx[d];
        fixed_ok = fixed_constants(in.x_lower[d], in.x_upper[d], in.dx[d], P.fx[d]) && fixed_ok;
    }
    if (ntiles > NOALLOC_MAX_TILES) return IBX_E_TOO_LARGE;
    P.fixed_ok = fixed_ok ? 1 : 0;
    P.inv_vol = (float)(1.0 / chk.vol);
    P.X = in.X;
    P.Q = in.Q;
    P.Qi = in.Q;
    for (int c = 0; c < ncomp; ++c)
    {
        P.q[c] = P.side ? in.q[c] : static_cast<void*>(static_cast<float*>(in.q[0]) + vol * c);
        P.qi[c] = P.q[c];
    }
    P.tile0 = 0;
    P.marker0 = 0;

    // Carve the scratch array (same buffers as a plan, capacities at the limits).
    const long long nm = in.n_markers;
    const int nt = (int)ntiles;
    const long long visit_cap = nm * (dim == 3 ? 8 : 4);
    const long long item_cap = nt + visit_cap / NOALLOC_UNITS_PER_ITEM + 1;
    const long long hitem_cap = nt + nm / NOALLOC_UNITS_PER_ITEM + 1;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = up256(off + bytes);
        return o;
    };
    const size_t o_probs = take(sizeof(PlanProb));
    const size_t o_moffs = take(sizeof(long long) * 2);
    const size_t o_toffs = take(sizeof(int) * 2);
    const size_t o_rec = take(sizeof(Rec) * nm);
    const size_t o_home_tile = take(sizeof(int) * nm);
    const size_t o_counts = take(sizeof(int) * counter_ints(nt));
    const size_t o_item_tile = take(sizeof(int) * item_cap);
    const size_t o_hitem_tile = take(sizeof(int) * hitem_cap);
    const size_t o_home_list = take(sizeof(int) * nm);
    const size_t o_visit = take(sizeof(int) * visit_cap);
    const size_t o_home_units = take(sizeof(int2) * nm);
    const size_t o_units = take(sizeof(int2) * visit_cap);
    const size_t o_status = take(sizeof(int) * 4);
    const size_t o_scan = take(sizeof(int) * 2048);
    if (off > NOALLOC_SCRATCH_BYTES) return IBX_E_TOO_LARGE;

    void* base = nullptr;
    const int rs = scratch_address(&base);
    if (rs) return rs;
    char* b = static_cast<char*>(base);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long moffs[2] = { 0, nm };
    const int toffs[2] = { 0, nt };
    if (cudaMemcpyAsync(b + o_probs, &P, sizeof(P), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b + o_moffs, moffs, sizeof(moffs), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b + o_toffs, toffs, sizeof(toffs), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(b + o_status, 0, sizeof(int) * 4, s) != cudaSuccess)
        return IBX_E_CUDA;

    DevPlan D;
    std::memset(&D, 0, sizeof(D));
    D.probs = reinterpret_cast<const PlanProb*>(b + o_probs);
    D.marker_offs = reinterpret_cast<const long long*>(b + o_moffs);
    D.tile_offs = reinterpret_cast<const int*>(b + o_toffs);
    D.n_probs = 1;
    D.n_markers = nm;
    D.n_tiles = nt;
    D.rec = reinterpret_cast<Rec*>(b + o_rec);
    D.home_tile = reinterpret_cast<int*>(b + o_home_tile);
    int* counts = reinterpret_cast<int*>(b + o_counts);
    D.hcount = counts;
    D.vcount = counts + (nt + 1);
    D.hucount = counts + 2 * (nt + 1);
    D.ucount = counts + 3 * (nt + 1);
    D.hcursor = counts + 4 * (nt + 1);
    D.vcursor = D.hcursor + nt;
    D.hucursor = D.vcursor + nt;
    D.ucursor = D.hucursor + nt;
    D.items = D.ucursor + nt;
    D.hitems = D.items + (nt + 1);
    D.home_list = reinterpret_cast<int*>(b + o_home_list);
    D.visit_list = reinterpret_cast<int*>(b + o_visit);
    D.n_visit_cap = visit_cap;
    D.home_units = reinterpret_cast<int2*>(b + o_home_units);
    D.units = reinterpret_cast<int2*>(b + o_units);
    D.item_tile = reinterpret_cast<int*>(b + o_item_tile);
    D.n_item_cap = (int)item_cap;
    D.hitem_tile = reinterpret_cast<int*>(b + o_hitem_tile);
    D.n_hitem_cap = (int)hitem_cap;
    D.item_units = NOALLOC_UNITS_PER_ITEM;
    D.status = reinterpret_cast<int*>(b + o_status);
    int* scan_tmp = reinterpret_cast<int*>(b + o_scan);

    // Counters and cursors start at zero on every call.
    if (cudaMemsetAsync(D.hcount, 0, sizeof(int) * counter_ints(nt), s) != cudaSuccess) return IBX_E_CUDA;
    int rc = launch_bin(dim, kernel, D, s, false);
    if (!rc) rc = exclusive_scan(D.hcount, nt + 1, scan_tmp, s);
    if (!rc) rc = exclusive_scan(D.vcount, nt + 1, scan_tmp, s);
    if (!rc) rc = exclusive_scan(D.hucount, nt + 1, scan_tmp, s);
    if (!rc) rc = exclusive_scan(D.ucount, nt + 1, scan_tmp, s);
    if (!rc) rc = launch_bin(dim, kernel, D, s, true);
    if (!rc) rc = launch_items(D, s);
    if (!rc) rc = exclusive_scan(D.items, nt + 1, scan_tmp, s);
    if (!rc) rc = launch_items_fill(D, s);
    if (!rc) rc = launch_spread(dim, kernel, D, ncomp, s);
    return rc;
}
