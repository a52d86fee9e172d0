// ibx_noalloc.cu -- binned mixed-precision spreading without any device
// allocation (ibx_spread_noalloc in include/ibx.h).
//
// Some callers cannot call cudaMalloc at all: host code inside a real-time
// or fault-handling path, where an allocation may block on the driver or
// fail when memory is short, and embeddings whose own pool manager owns all
// of the device memory so that a library may not allocate beside it.  For
// them the scratch memory of the binned pipeline (stencil records, tile
// counters, counting-sort lists, run units, the problem descriptor) lives in
// one file-scope __device__ array of fixed size, which every GPU that loads
// this library holds until the process exits.  The inputs and outputs stay
// the caller's.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it.
//
// The problem descriptor and the offset tables reach the array through the
// arguments of a small kernel (copied by the launch itself), so no host
// buffer has to outlive the call.
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

// Descriptor of the call, written into the scratch array by one thread:
// the problem, the marker offsets {0, n}, the tile offsets {0, n_tiles} and
// a cleared status word.  Everything arrives as launch arguments.
__global__ void
noalloc_setup(ibx::PlanProb P, long long n_markers, int n_tiles, ibx::PlanProb* probs, long long* moffs, int* toffs,
              int* status)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    *probs = P;
    moffs[0] = 0;
    moffs[1] = n_markers;
    toffs[0] = 0;
    toffs[1] = n_tiles;
    status[0] = 0;
}

// The binning's status word as an IBX status code in the caller's int.
__global__ void
noalloc_report(const int* word, int* out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int w = *word;
    *out = (w & 1) ? IBX_E_NONFINITE : (w & 2) ? IBX_E_TOO_LARGE : IBX_OK;
}

} // namespace

namespace ibx
{
int build_prob(const ibx_problem& in, int kernel, bool spread, Prob& P);
}

extern "C" int
ibx_spread_noalloc(const ibx_problem* problem, int kernel, int* status, void* stream)
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
    long long ntiles = 1, vol = 1, per = 1;
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
        // Tiles one footprint can touch along d: two, or three when the last
        // tile is partial (a footprint at the periodic seam straddles the
        // partial tile and both of its neighbours); never more than exist.
        const int bound = 2 + (P.N[d] % Ed[d] != 0);
        per *= P.ntile[d] < bound ? P.ntile[d] : bound;
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

    // Carve the scratch array (the buffers of a plan, with the capacities
    // ibx_plan_create would reserve for this problem).
    const long long nm = in.n_markers;
    const int nt = (int)ntiles;
    PlanSizes z;
    z.tile_shape = 0;
    z.n_probs = 1;
    z.n_markers = nm;
    z.n_tiles = nt;
    z.visit_cap = nm * per;
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
    noalloc_setup<<<1, 1, 0, s>>>(P, nm, nt, reinterpret_cast<PlanProb*>(b + c.o_probs),
                                  reinterpret_cast<long long*>(b + c.o_moffs), reinterpret_cast<int*>(b + c.o_toffs),
                                  reinterpret_cast<int*>(b + c.o_status));
    note_launches(1);
    if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;

    // Counters and cursors are zeroed by the binning sequence on every call.
    int rc = bin_sequence(dim, kernel, D, c.scan_tmp, s);
    if (!rc) rc = launch_spread(dim, kernel, D, ncomp, s);
    if (!rc && status)
    {
        noalloc_report<<<1, 1, 0, s>>>(D.status, status);
        note_launches(1);
        if (cudaGetLastError() != cudaSuccess) rc = IBX_E_CUDA;
    }
    return rc;
}
