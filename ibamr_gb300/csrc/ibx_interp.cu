// ibx_interp.cu -- interpolation of the plan pipeline (mixed precision).
//
// Markers are split like the spread: dense-homed (home tile with more than
// dense_min markers) and sparse-homed.  Two kernels, combined by the
// interpolation form (ibx_plan_set_interp_kernel):
//  - interp_chunks: each thread handles a short chunk of consecutive
//    home-order markers for one component and keeps the W^d grid values of
//    the current stencil in registers, so markers of a run (same stencil
//    base) reuse them and only evaluate their weights and the FP32
//    multiply-adds.  Every marker in home order (form 0), the sparse-homed
//    ones (form 1), or every marker in the caller's order (form 2: it needs
//    only the stencil records, so the step can start it before the counting
//    sort; fibre markers given in fibre order share runs as in home order).
//    In forms 1 and 4 the sparse-homed markers, which seldom share a
//    stencil, go to interp_chunks_sparse: the same sums without the register
//    cache, in 80 registers instead of 128 (24 resident warps per SM instead
//    of 16).
//  - interp_units (form 1, dense-homed): the work items of the dense spread
//    (item_units home units of one tile); a group of lanes per (unit,
//    component), the footprint's z-planes split over the group, loads the
//    unit's stencil values once and sums every marker of the unit from
//    registers.
// Sum order everywhere: V = sum_z w_z sum_y w_y sum_x w_x u, the separable
// form of the reference's w(i0,i1,i2) * u (F3D:1309-1328), so every form
// gives bit-identical results.

#include "ibx_interp_body.cuh"
#include "../../include/ibx.h"

#include <cudaTypedefs.h> // PFN_cuTensorMapEncodeTiled

namespace ibx
{
namespace
{
// Chunks of consecutive home-order markers, one component per thread
// (chunk_body), the stencil values cached in registers across a run; or,
// for the sparse-homed markers alone (which seldom share a stencil), read
// as they are summed, in fewer registers (more resident warps).
template <int DIM, int K>
__global__ void __launch_bounds__(INTERP_THREADS) interp_chunks(const DevPlan D, int select, int marker_order)
{
    chunk_body<DIM, K, true>(D, blockIdx.x * (long long)blockDim.x + threadIdx.x, select, marker_order);
}

template <int DIM, int K>
__global__ void __launch_bounds__(INTERP_THREADS, 3) interp_chunks_sparse(const DevPlan D)
{
    chunk_body<DIM, K, false, true>(D, blockIdx.x * (long long)blockDim.x + threadIdx.x, SEL_SPARSE, 0);
}

// CTAs per SM the per-unit interpolation's registers are cut for: 3 in 3D
// (80 registers; at 64 its cached planes spill), 4 in 2D (64, no spill).
template <int DIM>
struct UnitsOccupancy
{
    static constexpr int value = DIM == 3 ? 3 : 4;
};

// Dense-homed markers by home unit (units_item); items are taken from a
// counter (no tail from CTAs resident late).
template <int DIM, int K>
__global__ void __launch_bounds__(INTERP_THREADS, UnitsOccupancy<DIM>::value) interp_units(const DevPlan D)
{
    const int n_items = min(D.items[D.n_tiles], D.n_item_cap);
    __shared__ int s_item;
    __shared__ int s_order[256];
    __shared__ int s_start[33];
    for (;;)
    {
        __syncthreads(); // the previous item's readers of s_item and s_order are done
        if (threadIdx.x == 0) s_item = atomicAdd(&D.work[2], 1);
        __syncthreads();
        const int item = s_item;
        if (item >= n_items) break;
        units_item<DIM, K>(D, item, s_order, s_start);
    }
}

// ---- interpolation from TMA-staged tile regions -----------------------------
// One CTA per chunk of TILE_CHUNK consecutive home-order markers.  The CTA
// first cuts its chunk into segments -- its markers of one home tile -- in
// one parallel pass (each thread looks up one marker's tile), then works
// through the segments: for each it stages the tile's region of every
// interpolation source (IBox: the cells of all stencils of markers homed in
// the tile) in shared memory -- one tensor copy (cp.async.bulk.tensor) per
// component when the region lies inside the grid, plain loads with periodic
// wrapping otherwise -- and its threads evaluate the segment's (component,
// marker) pairs from shared memory in the separable order of the other forms
// (bit-identical results).  Two region buffers when every marker is taken
// (a chunk of sparse tiles holds many segments: the copies of the next one
// are in flight while one is evaluated), one when only dense tiles are (a
// chunk is then one segment or two, and the smaller footprint leaves room
// on the SMs for the spread running beside).  Thread 0 issues the copies;
// every wait on a copy is bounded and reported through bit 2 of the plan's
// status word.
constexpr int TILE_THREADS = 256;
constexpr int TILE_CHUNK = 256; // home-order markers per CTA (one per thread when cutting segments)
constexpr int MBAR_SPINS = 1 << 24;

__device__ __forceinline__ unsigned
smem_addr(const void* p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void
mbar_init(unsigned a)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
}

__device__ __forceinline__ void
mbar_expect_tx(unsigned a, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool
mbar_try_wait(unsigned a, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(a), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Waits for phase `parity` of the barrier to complete; false after
// MBAR_SPINS polls (seconds), never hangs.
__device__ __forceinline__ bool
mbar_wait(unsigned a, unsigned parity)
{
    for (int i = 0; i < MBAR_SPINS; ++i)
    {
        if (mbar_try_wait(a, parity)) return true;
        if (i >= 8) __nanosleep(64);
    }
    return false;
}

// One box of a tensor map into shared memory, completion counted on `mbar`.
template <int DIM>
__device__ __forceinline__ void
tma_load(unsigned dst, const CUtensorMap* map, int x, int y, int z, unsigned mbar)
{
    if (DIM == 3)
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4}], [%5];" ::"r"(dst),
                     "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(mbar)
                     : "memory");
    else
        asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                     "%3}], [%4];" ::"r"(dst),
                     "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(mbar)
                     : "memory");
}

// Exclusive scan of one int per thread over a CTA of TILE_THREADS threads;
// returns the thread's offset, *total the sum.  `tmp` holds one int per warp.
__device__ __forceinline__ int
cta_exclusive_scan(int v, int* tmp, int* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) tmp[warp] = x;
    __syncthreads();
    int base = 0, all = 0;
#pragma unroll
    for (int w = 0; w < TILE_THREADS / 32; ++w)
    {
        const int t = tmp[w];
        base += w < warp ? t : 0;
        all += t;
    }
    __syncthreads(); // tmp may be reused
    *total = all;
    return base + x - v;
}

template <int DIM, int K, int SH>
__global__ void __launch_bounds__(TILE_THREADS) interp_tiles(const DevPlan D, int select)
{
    constexpr int W = KT<K>::W;
    using B = IBox<DIM, W, SH>;
    extern __shared__ unsigned char smraw[];
    // segments of the chunk: tile, problem, marker range, tensor-copy flag
    __shared__ int s_t[TILE_CHUNK], s_p[TILE_CHUNK], s_mb[TILE_CHUNK], s_me[TILE_CHUNK], s_tma[TILE_CHUNK];
    __shared__ int s_start[TILE_CHUNK + 1];
    __shared__ int s_tmp[TILE_THREADS / 32];
    const long long total = D.hcount[D.n_tiles];
    const long long m0 = (long long)blockIdx.x * TILE_CHUNK;
    if (m0 >= total) return; // uniform over the CTA
    const int n = (int)min((long long)TILE_CHUNK, total - m0);
    // -- cut the chunk into segments (runs of one home tile)
    const int j = threadIdx.x;
    const int tj = j < n ? D.home_tile[D.home_list[m0 + j]] : -1;
    s_t[j] = tj;
    __syncthreads();
    const bool first = j < n && (j == 0 || s_t[j - 1] != tj);
    int n_runs = 0;
    const int r = cta_exclusive_scan(first ? 1 : 0, s_tmp, &n_runs);
    if (first) s_start[r] = j;
    if (j == 0) s_start[n_runs] = n;
    __syncthreads();
    int t = -1, mb = 0, me = 0, keep = 0;
    if (j < n_runs)
    {
        mb = s_start[j];
        me = s_start[j + 1];
        t = s_t[mb];
        keep = select == SEL_ALL || tile_dense(D, t) == (select == SEL_DENSE);
    }
    int n_seg = 0;
    const int k = cta_exclusive_scan(keep, s_tmp, &n_seg);
    if (n_seg == 0) return; // uniform
    if (keep)
    {
        const int p = D.n_probs == 1 ? 0 : find_in_offsets(D.tile_offs, D.n_probs, t);
        const PlanProb& P = D.probs[p];
        int org[3];
        tile_origin<DIM, SH>(P, t - P.tile0, org);
        const int x0 = org[0] - B::X0, y0 = org[1] - B::H, z0 = DIM == 3 ? org[2] - B::H : 0;
        const bool in = P.tma && x0 >= 0 && x0 + B::BX <= P.N[0] && y0 >= 0 && y0 + B::BY <= P.N[1] &&
                        (DIM == 2 || (z0 >= 0 && z0 + B::BZ <= P.N[2]));
        s_t[k] = t; // entry k <= j: every thread has read s_t[mb] before the scan's barriers
        s_p[k] = p;
        s_mb[k] = (int)m0 + mb;
        s_me[k] = (int)m0 + me;
        s_tma[k] = in ? 1 : 0;
    }
    // -- region buffers (128-byte aligned) and their barriers
    const unsigned raw = smem_addr(smraw);
    unsigned char* base = smraw + ((128u - (raw & 127u)) & 127u);
    const unsigned bar0 = smem_addr(base);
    float* bufs = reinterpret_cast<float*>(base + 128);
    const int nc_max = D.max_ncomp;
    const int nbuf = select == SEL_DENSE ? 1 : 2;
    // thread 0: tensor copies of segment i into buffer i % nbuf
    auto issue = [&](int i) {
        const int b = i % nbuf;
        const PlanProb& P = D.probs[s_p[i]];
        int org[3];
        tile_origin<DIM, SH>(P, s_t[i] - P.tile0, org);
        const unsigned bar = bar0 + 8u * b;
        const unsigned dst = smem_addr(bufs + (size_t)b * nc_max * B::CS);
        // the buffer was last accessed through ordinary loads and stores
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bar, (unsigned)(P.ncomp * B::PTS * sizeof(float)));
        for (int c = 0; c < P.ncomp; ++c)
            tma_load<DIM>(dst + 4u * c * B::CS, D.tmaps + 3 * s_p[i] + c, org[0] - B::X0, org[1] - B::H,
                          DIM == 3 ? org[2] - B::H : 0, bar);
    };
    __syncthreads(); // segment list complete
    if (threadIdx.x == 0)
    {
        mbar_init(bar0);
        mbar_init(bar0 + 8);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (s_tma[0]) issue(0);
        if (nbuf == 2 && n_seg > 1 && s_tma[1]) issue(1);
    }
    __syncthreads();
    unsigned phase[2] = { 0u, 0u };
    int i = 0;
    bool failed = false;
    for (; i < n_seg; ++i)
    {
        const int b = i % nbuf;
        const PlanProb& P = D.probs[s_p[i]];
        int org[3];
        tile_origin<DIM, SH>(P, s_t[i] - P.tile0, org);
        float* buf = bufs + (size_t)b * nc_max * B::CS;
        bool late = false;
        if (s_tma[i])
        {
            late = !mbar_wait(bar0 + 8u * b, phase[b]);
            phase[b] ^= 1u;
        }
        else
        {
            // region across the periodic boundary (or no tensor map): plain
            // loads with wrapped indices
            const long long n0 = P.N[0], n01 = (long long)P.N[0] * P.N[1];
            for (int c = 0; c < P.ncomp; ++c)
            {
                const float* q = static_cast<const float*>(P.qi[c]);
                for (int e = threadIdx.x; e < B::PTS; e += TILE_THREADS)
                {
                    const int x = e % B::BX, y = (e / B::BX) % B::BY, z = e / (B::BX * B::BY);
                    const int gx = wrap_cell(org[0] - B::X0 + x, P.N[0]);
                    const int gy = wrap_cell(org[1] - B::H + y, P.N[1]);
                    const int gz = DIM == 3 ? wrap_cell(org[2] - B::H + z, P.N[2]) : 0;
                    buf[c * B::CS + e] = __ldg(q + gz * n01 + gy * n0 + gx);
                }
            }
        }
        if (__syncthreads_or(late))
        {
            failed = true;
            break;
        }
        // the segment's (component, marker) pairs from the staged region:
        // a warp takes consecutive markers of one component
        const int ncomp = P.ncomp;
        const int nm = s_me[i] - s_mb[i];
        float* Qi = static_cast<float*>(P.Qi);
        for (int e = threadIdx.x; e < nm * ncomp; e += TILE_THREADS)
        {
            const int c = e / nm;
            const int m = s_mb[i] + (e - c * nm);
            const Rec R = D.hrec[m];
            float w[3][W];
            record_weights<DIM, K>(P, R, c, w);
            int l[3] = { 0, 0, 0 };
#pragma unroll
            for (int d = 0; d < DIM; ++d)
            {
                const int st = (P.side && d == c) ? R.stagger(d) : 0;
                l[d] = wrap_from_base(R.bc(d) + B::H, P.N[d]) - org[d] + st;
            }
            l[0] += B::X0 - B::H;
            const float* rp = buf + c * B::CS + l[0] + B::BX * (l[1] + B::BY * l[2]);
            const float V = separable_sum<DIM, W>(w, [&](int i0, int i1, int i2) {
                return rp[i0 + B::BX * (i1 + B::BY * i2)];
            });
            Qi[(long long)P.Q_depth * (D.home_list[m] - P.marker0) + c] = V;
        }
        __syncthreads(); // buffer b is free
        if (threadIdx.x == 0 && i + nbuf < n_seg && s_tma[i + nbuf]) issue(i + nbuf);
    }
    if (failed && threadIdx.x == 0)
    {
        atomicOr(D.status, 4);
        // Before the CTA's shared memory is released, wait (bounded) for the
        // copies still in flight: segment i's (its phase already advanced)
        // and, with two buffers, segment i + 1's.
        if (s_tma[i]) mbar_wait(bar0 + 8u * (i % nbuf), phase[i % nbuf] ^ 1u);
        if (nbuf == 2 && i + 1 < n_seg && s_tma[i + 1])
            mbar_wait(bar0 + 8u * ((i + 1) % nbuf), phase[(i + 1) % nbuf]);
    }
}

template <int DIM, int K, int SH>
int
launch_tiles_sh(const DevPlan& D, int select, cudaStream_t s)
{
    using B = IBox<DIM, KT<K>::W, SH>;
    const size_t smem = 256 + (select == SEL_DENSE ? 1 : 2) * sizeof(float) * (size_t)D.max_ncomp * B::CS;
    // the kernel's static arrays count against the same 48 KB default limit:
    // opt in to the dynamic size whatever it is
    if (cudaFuncSetAttribute(interp_tiles<DIM, K, SH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return IBX_E_CUDA;
    const long long chunks = (D.n_markers + TILE_CHUNK - 1) / TILE_CHUNK;
    if (chunks == 0) return IBX_OK;
    interp_tiles<DIM, K, SH><<<(unsigned)chunks, TILE_THREADS, smem, s>>>(D, select);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

template <int DIM, int K>
int
launch_interp_k(const DevPlan& D, cudaStream_t s)
{
    if (D.interp_form == 3 || D.interp_form == 4)
    {
        const int sel = D.interp_form == 3 ? SEL_ALL : SEL_DENSE;
        const int rc = D.tile_shape == 0 ? launch_tiles_sh<DIM, K, 0>(D, sel, s) : launch_tiles_sh<DIM, K, 1>(D, sel, s);
        if (rc || sel == SEL_ALL) return rc;
        const long long chunks = (D.n_markers + CHUNK - 1) / CHUNK;
        const unsigned bx = (unsigned)((chunks * D.max_ncomp + INTERP_THREADS - 1) / INTERP_THREADS);
        if (bx == 0) return IBX_OK;
        interp_chunks_sparse<DIM, K><<<bx, INTERP_THREADS, 0, s>>>(D);
        note_launches(1);
        return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
    }
    constexpr int W = KT<K>::W;
    const bool units = D.interp_form == 1 && UnitSplit<DIM, W>::NC <= 64;
    if (units)
    {
        if (cudaMemsetAsync(D.work + 2, 0, sizeof(int), s) != cudaSuccess) return IBX_E_CUDA;
        int dev = 0, sms = 152, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, interp_units<DIM, K>, INTERP_THREADS, 0);
        if (per_sm < 1) per_sm = 1;
        const unsigned blocks = (unsigned)(D.n_item_cap < per_sm * sms ? D.n_item_cap : per_sm * sms);
        if (blocks > 0)
        {
            interp_units<DIM, K><<<blocks, INTERP_THREADS, 0, s>>>(D);
            note_launches(1);
            if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;
        }
    }
    const long long chunks = (D.n_markers + CHUNK - 1) / CHUNK;
    const unsigned bx = (unsigned)((chunks * D.max_ncomp + INTERP_THREADS - 1) / INTERP_THREADS);
    if (bx == 0) return IBX_OK;
    if (units)
        interp_chunks_sparse<DIM, K><<<bx, INTERP_THREADS, 0, s>>>(D);
    else
        interp_chunks<DIM, K><<<bx, INTERP_THREADS, 0, s>>>(D, SEL_ALL, D.interp_form == 2);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}
} // namespace

namespace
{
// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null when the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000
encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

template <int DIM, int W, int SH>
void
box_of(int* box)
{
    using B = IBox<DIM, W, SH>;
    box[0] = B::BX;
    box[1] = B::BY;
    box[2] = B::BZ;
}

void
interp_box(int dim, int width, int shape, int* box)
{
#define IBX_BOX(DD, WW)                                                                                              \
    if (dim == DD && width == WW)                                                                                    \
    {                                                                                                                \
        if (shape == 0)                                                                                              \
            box_of<DD, WW, 0>(box);                                                                                  \
        else                                                                                                         \
            box_of<DD, WW, 1>(box);                                                                                  \
        return;                                                                                                      \
    }
    IBX_BOX(2, 2) IBX_BOX(2, 3) IBX_BOX(2, 4) IBX_BOX(2, 6) IBX_BOX(3, 2) IBX_BOX(3, 3) IBX_BOX(3, 4) IBX_BOX(3, 6)
#undef IBX_BOX
    box[0] = box[1] = box[2] = 0;
}
} // namespace

void
encode_interp_maps(int dim, int kernel, int tile_shape, PlanProb* probs, int n_probs, CUtensorMap* maps)
{
    const PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    int box[3];
    interp_box(dim, kernel_width(kernel), tile_shape, box);
    for (int p = 0; p < n_probs; ++p)
    {
        PlanProb& P = probs[p];
        P.tma = 0;
        if (!enc || box[0] == 0) continue;
        // global strides must be multiples of 16 bytes, the box no larger than the grid
        bool ok = P.N[0] % 4 == 0;
        for (int d = 0; d < dim; ++d) ok = ok && P.N[d] >= box[d];
        for (int c = 0; c < P.ncomp && ok; ++c)
        {
            void* g = P.qi[c];
            ok = g && (reinterpret_cast<unsigned long long>(g) & 15) == 0;
            if (!ok) break;
            cuuint64_t gdim[3] = { (cuuint64_t)P.N[0], (cuuint64_t)P.N[1], (cuuint64_t)P.N[2] };
            cuuint64_t gstride[2] = { (cuuint64_t)P.N[0] * sizeof(float),
                                      (cuuint64_t)P.N[0] * P.N[1] * sizeof(float) };
            cuuint32_t bdim[3] = { (cuuint32_t)box[0], (cuuint32_t)box[1], (cuuint32_t)box[2] };
            cuuint32_t estride[3] = { 1, 1, 1 };
            const CUresult r = enc(&maps[3 * p + c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)dim, g, gdim,
                                   gstride, bdim, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            ok = r == CUDA_SUCCESS;
        }
        P.tma = ok ? 1 : 0;
    }
}

int
launch_interp(int dim, int kernel, const DevPlan& D, cudaStream_t s)
{
#define IBX_INTERP_CASE(DD, KK)                                                                                      \
    if (dim == DD && kernel == KK) return launch_interp_k<DD, KK>(D, s);
    IBX_INTERP_CASE(2, K_PL) IBX_INTERP_CASE(2, K_PCUBIC) IBX_INTERP_CASE(2, K_IB3) IBX_INTERP_CASE(2, K_IB4)
    IBX_INTERP_CASE(2, K_IB6) IBX_INTERP_CASE(2, K_BSPL4) IBX_INTERP_CASE(3, K_PL) IBX_INTERP_CASE(3, K_PCUBIC)
    IBX_INTERP_CASE(3, K_IB3) IBX_INTERP_CASE(3, K_IB4) IBX_INTERP_CASE(3, K_IB6) IBX_INTERP_CASE(3, K_BSPL4)
#undef IBX_INTERP_CASE
    return IBX_E_BAD_KERNEL;
}

} // namespace ibx
