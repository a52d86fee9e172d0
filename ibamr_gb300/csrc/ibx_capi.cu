// ibx_capi.cu -- the extern "C" entry points of libibx (include/ibx.h):
// argument validation with the reference's error rules, translation of the
// caller's problem descriptions into device descriptors, dispatch.
//
// LEI = ibtk/src/lagrangian/LEInteractor.cpp (IBAMR tree).

#include "ibx_internal.h"
#include "../../include/ibx.h"

#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

namespace ibx
{
namespace
{
std::atomic<long long> g_launches{ 0 };
} // namespace

void
note_launches(int n)
{
    g_launches.fetch_add(n, std::memory_order_relaxed);
}

namespace
{
bool
valid_kernel(int k)
{
    return k >= IBX_KERNEL_PIECEWISE_LINEAR && k <= IBX_KERNEL_BSPLINE_4;
}

bool
is_pow2(double v)
{
    if (!(v > 0.0) || !std::isfinite(v)) return false;
    int e;
    const double m = std::frexp(v, &e);
    return m == 0.5;
}
} // namespace

// Validate one caller problem and derive the device descriptor.  Error
// precedence follows the reference: kernel name, then depth (LEI:2197-2201,
// 3650-3654), then ghost width (LEI:4488-4498 interpolation always,
// LEI:5250-5268 spreading only at a physical boundary).
int
build_prob(const ibx_problem& in, int kernel, bool spread, Prob& P)
{
    std::memset(&P, 0, sizeof(P));
    if (!valid_kernel(kernel)) return IBX_E_BAD_KERNEL;
    const int dim = in.dim;
    if (dim != 2 && dim != 3) return IBX_E_ARG;
    if (in.centering != IBX_CELL && in.centering != IBX_SIDE) return IBX_E_ARG;
    if (in.mode != IBX_MODE_PATCH && in.mode != IBX_MODE_PERIODIC) return IBX_E_ARG;
    const bool side = in.centering == IBX_SIDE;
    if (side)
    {
        if (in.Q_depth != dim || in.q_depth != 1) return IBX_E_DEPTH;
    }
    else if (in.q_depth < 1 || in.Q_depth != in.q_depth)
        return IBX_E_DEPTH;
    for (int d = 0; d < dim; ++d)
    {
        if (in.iupper[d] < in.ilower[d]) return IBX_E_ARG;
        if (!(in.dx[d] > 0.0) || !std::isfinite(in.dx[d]) || !std::isfinite(in.x_lower[d])) return IBX_E_ARG;
        if (in.mode == IBX_MODE_PATCH && in.gcw[d] < 0) return IBX_E_ARG;
    }
    if (in.mode == IBX_MODE_PATCH)
    {
        int gmin = in.gcw[0];
        bool phys = false;
        for (int d = 0; d < dim; ++d)
        {
            gmin = gmin < in.gcw[d] ? gmin : in.gcw[d];
            phys = phys || in.touches_physical_lower[d] || in.touches_physical_upper[d];
        }
        const int need = ibx_get_minimum_ghost_width(kernel);
        if ((!spread || phys) && gmin < need) return IBX_E_GHOST_WIDTH;
    }
    const int n_items = in.indices ? in.n_indices : in.n_markers;
    if (n_items < 0 || in.n_markers < 0) return IBX_E_ARG;
    if (n_items > 0 && (!in.X || !in.Q)) return IBX_E_ARG;

    P.dim = dim;
    P.side = side ? 1 : 0;
    P.ncomp = side ? dim : 1;
    P.q_depth = in.q_depth;
    P.Q_depth = in.Q_depth;
    P.mode = in.mode;
    P.n_items = n_items;
    for (int d = 0; d < 3; ++d)
    {
        P.dx[d] = d < dim ? in.dx[d] : 1.0;
        P.inv_dx[d] = 1.0 / P.dx[d];
        P.dx_pow2[d] = d < dim ? (int)is_pow2(in.dx[d]) : 1;
    }
    P.vol = dim == 2 ? in.dx[0] * in.dx[1] : in.dx[0] * in.dx[1] * in.dx[2];
    P.X = in.X;
    P.Q = in.Q;
    P.indices = in.indices;
    P.Xshift = in.Xshift;
    for (int c = 0; c < P.ncomp; ++c)
    {
        Comp& C = P.comp[c];
        C.q = in.q[c];
        if (n_items > 0 && !C.q) return IBX_E_ARG;
        long long vol = 1;
        for (int d = 0; d < 3; ++d)
        {
            if (d >= dim)
            {
                C.lo[d] = 0;
                C.n[d] = 1;
                C.box_lo[d] = 0;
                C.clip_lo[d] = C.clip_hi[d] = 0;
                C.wrapN[d] = 0;
                C.xlo[d] = 0.0;
                continue;
            }
            const int box_lo = in.ilower[d];
            const int box_hi = in.iupper[d] + ((side && d == c) ? 1 : 0);
            C.box_lo[d] = box_lo;
            // LEI:2464-2465 / 3689-3690: side axis geometry shifted by -dx/2.
            C.xlo[d] = (side && d == c) ? in.x_lower[d] - 0.5 * in.dx[d] : in.x_lower[d];
            if (in.mode == IBX_MODE_PATCH)
            {
                C.lo[d] = box_lo - in.gcw[d];
                C.n[d] = box_hi - box_lo + 1 + 2 * in.gcw[d];
                C.clip_lo[d] = box_lo - in.gcw[d];
                C.clip_hi[d] = box_hi + in.gcw[d];
                C.wrapN[d] = 0;
            }
            else
            {
                const int N = in.iupper[d] - in.ilower[d] + 1;
                C.lo[d] = box_lo;
                C.n[d] = N;
                C.clip_lo[d] = box_lo;
                C.clip_hi[d] = box_lo + N - 1;
                C.wrapN[d] = N;
            }
            vol *= C.n[d];
        }
        C.depth_stride = vol;
    }
    return IBX_OK;
}

namespace
{
int
run_generic(const ibx_problem* problems, int n_problems, int kernel, int precision, void* stream, bool spread)
{
    if (!problems || n_problems < 0) return IBX_E_ARG;
    if (!valid_kernel(kernel)) return IBX_E_BAD_KERNEL;
    if (precision != IBX_PRECISION_FP64) return IBX_E_ARG;
    if (n_problems == 0) return IBX_OK;
    std::vector<Prob> probs(n_problems);
    std::vector<long long> offs(n_problems + 1, 0);
    const int dim = problems[0].dim;
    for (int p = 0; p < n_problems; ++p)
    {
        const int rc = build_prob(problems[p], kernel, spread, probs[p]);
        if (rc) return rc;
        if (problems[p].dim != dim) return IBX_E_ARG;
        offs[p + 1] = offs[p] + (long long)probs[p].n_items * probs[p].ncomp;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ProbArg A;
    std::memset(&A, 0, sizeof(A));
    A.n = n_problems;
    A.total = offs[n_problems];
    if (A.total == 0) return IBX_OK;
    if (n_problems == 1)
    {
        A.one = probs[0];
        return launch_generic(spread, dim, kernel, A, s);
    }
    // Several problems: descriptor table in stream-ordered device memory.
    const size_t tbytes = sizeof(Prob) * n_problems;
    const size_t obytes = sizeof(long long) * (n_problems + 1);
    void* dbuf = nullptr;
    if (cudaMallocAsync(&dbuf, tbytes + obytes, s) != cudaSuccess) return IBX_E_OOM;
    char* base = static_cast<char*>(dbuf);
    int rc = IBX_OK;
    if (cudaMemcpyAsync(base, probs.data(), tbytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(base + tbytes, offs.data(), obytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
        rc = IBX_E_CUDA;
    if (!rc)
    {
        A.many = reinterpret_cast<const Prob*>(base);
        A.offs = reinterpret_cast<const long long*>(base + tbytes);
        rc = launch_generic(spread, dim, kernel, A, s);
    }
    cudaFreeAsync(dbuf, s);
    // The host tables must outlive the pageable copies: synchronise on them.
    cudaStreamSynchronize(s);
    return rc;
}
} // namespace
} // namespace ibx

namespace ibx
{
namespace
{
constexpr int MAX_DEVICES = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[MAX_DEVICES] = {};

cudaMemPool_t
staging_pool()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return nullptr;
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pools[dev])
    {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
        // keep freed memory in the pool for the next call
        unsigned long long keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}
} // namespace

void*
staging_alloc(size_t bytes)
{
    cudaMemPool_t pool = staging_pool();
    void* p = nullptr;
    if (!pool || cudaMallocFromPoolAsync(&p, bytes, pool, nullptr) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void
staging_free(void* p)
{
    if (p) cudaFreeAsync(p, nullptr);
}
} // namespace ibx

extern "C" {

int
ibx_get_stencil_size(int kernel)
{
    switch (kernel)
    {
    case IBX_KERNEL_PIECEWISE_LINEAR:
        return 2;
    case IBX_KERNEL_PIECEWISE_CUBIC:
    case IBX_KERNEL_IB_3:
    case IBX_KERNEL_IB_4:
    case IBX_KERNEL_BSPLINE_4:
        return 4;
    case IBX_KERNEL_IB_6:
        return 6;
    default:
        return -1;
    }
}

int
ibx_get_minimum_ghost_width(int kernel)
{
    const int w = ibx_get_stencil_size(kernel);
    return w < 0 ? -1 : static_cast<int>(std::floor(0.5 * w)) + 1;
}

int
ibx_kernel_from_name(const char* name)
{
    if (!name) return -1;
    static const char* const names[] = { "PIECEWISE_LINEAR", "PIECEWISE_CUBIC", "IB_3", "IB_4", "IB_6", "BSPLINE_4" };
    for (int k = 0; k < 6; ++k)
        if (std::strcmp(name, names[k]) == 0) return k;
    return -1;
}

const char*
ibx_status_string(int status)
{
    switch (status)
    {
    case IBX_OK:
        return "success";
    case IBX_E_BAD_KERNEL:
        return "unknown kernel function";
    case IBX_E_GHOST_WIDTH:
        return "insufficient ghost cells";
    case IBX_E_DEPTH:
        return "data depth mismatch";
    case IBX_E_ARG:
        return "invalid argument";
    case IBX_E_CUDA:
        return "CUDA runtime error";
    case IBX_E_OOM:
        return "out of device memory";
    case IBX_E_TIMEOUT:
        return "bounded device wait timed out";
    case IBX_E_NONFINITE:
        return "non-finite marker position";
    case IBX_E_TOO_LARGE:
        return "size exceeds a documented limit";
    default:
        return "unknown status";
    }
}

int
ibx_device_alloc(void** ptr, long long bytes)
{
    if (!ptr || bytes < 0) return IBX_E_ARG;
    *ptr = nullptr;
    if (bytes == 0) return IBX_OK;
    *ptr = ibx::staging_alloc((size_t)bytes);
    return *ptr ? IBX_OK : IBX_E_OOM;
}

int
ibx_device_free(void* ptr)
{
    if (!ptr) return IBX_OK;
    ibx::staging_free(ptr);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

int
ibx_memcpy(void* dst, const void* src, long long bytes, int to_device)
{
    if (bytes <= 0) return IBX_OK;
    return cudaMemcpy(dst, src, (size_t)bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost) ==
                   cudaSuccess
               ? IBX_OK
               : IBX_E_CUDA;
}

long long
ibx_kernel_launches(void)
{
    return ibx::g_launches.load(std::memory_order_relaxed);
}

int
ibx_synchronize(void)
{
    return cudaDeviceSynchronize() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

int
ibx_interpolate(const ibx_problem* problems, int n_problems, int kernel, int precision, void* stream)
{
    return ibx::run_generic(problems, n_problems, kernel, precision, stream, false);
}

int
ibx_spread(const ibx_problem* problems, int n_problems, int kernel, int precision, void* stream)
{
    return ibx::run_generic(problems, n_problems, kernel, precision, stream, true);
}

} // extern "C"
