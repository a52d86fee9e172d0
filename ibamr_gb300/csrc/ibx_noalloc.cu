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
constexpr size_t NOALLOC_SCRATCH_BYTES = 8u << 20; // 8 MiB

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
    int Ed[3];
    tile_edges(dim, 0, Ed);

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
        P.ntile[d] = (P.N[d] + Ed[d] - 1) / Ed[d];
        ntiles *= P.ntile[d];
        vol *= P.N[d];
        P.dx[d] = chk.dx[d];
        P.inv_dx[d] = chk.inv_dx[d];
        P.dx_pow2[d] = chk.dx_pow2[d];
        P.xlo_c[d] = in.x_lower[d];
        P.xlo_s[d] = in.x_lower[d] - 0.5 * in.dx[d];
        fixed_ok = fixed_dim(in.x_lower[d], in.x_upper[d], in.dx[d], P.fx[d]) && fixed_ok;
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
    P.vec4 = P.N[0] % 4 == 0;
    for (int c = 0; c < ncomp; ++c) P.vec4 = P.vec4 && (reinterpret_cast<unsigned long long>(P.q[c]) & 15) == 0;
    P.tile0 = 0;
    P.marker0 = 0;

    // Carve the scratch array (the buffers of a plan, capacities at the limits).
    const long long nm = in.n_markers;
    const int nt = (int)ntiles;
    PlanSizes z;
    z.tile_shape = 0;
    z.n_probs = 1;
    z.n_markers = nm;
    z.n_tiles = nt;
    z.visit_cap = nm * (dim == 3 ? 8 : 4);
    z.item_cap = nt + nm / 10 + 1;
    DevPlan D{};
    if (carve_plan(z, nullptr, D).bytes > NOALLOC_SCRATCH_BYTES) return IBX_E_TOO_LARGE;

    void* base = nullptr;
    const int rs = scratch_address(&base);
    if (rs) return rs;
    char* b = static_cast<char*>(base);
    const PlanCarve c = carve_plan(z, b, D);
    D.zsplit = dense_zsplit(dim, kernel_width(kernel));
    D.item_units = 2 * (256 / (ncomp * D.zsplit)) < 256 ? 2 * (256 / (ncomp * D.zsplit)) : 256;
    if (D.item_units < 32) D.item_units = 32; // at least the units per item the capacity assumes
    D.max_ncomp = ncomp;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long moffs[2] = { 0, nm };
    const int toffs[2] = { 0, nt };
    // The pageable sources are staged by the runtime before these calls return.
    if (cudaMemcpyAsync(b + c.o_probs, &P, sizeof(P), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b + c.o_moffs, moffs, sizeof(moffs), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b + c.o_toffs, toffs, sizeof(toffs), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(b + c.o_status, 0, sizeof(int) * 4, s) != cudaSuccess)
        return IBX_E_CUDA;

    // Counters and cursors are zeroed by the binning sequence on every call.
    int rc = bin_sequence(dim, kernel, D, c.scan_tmp, s);
    if (!rc) rc = launch_spread(dim, kernel, D, ncomp, s);
    return rc;
}
