// ibx_generic.cu -- marker-parallel FP64 spread and interpolate.
//
// One thread per (selected marker, Eulerian component).  The per-marker
// arithmetic is the reference's: stencil and weights exactly as the Fortran
// routines compute them (ibx_device.cuh), the same clipping to the ghost box
// (F3D:1309-1314 for IB_4/IB_6, clip-then-weigh for the floor kernels), the
// same product association (F3D:24-68 macro kernels, F3D:1436-1468 tensor
// kernels).  Spreading accumulates with FP64 atomics at L2 (RED.ADD.F64), so
// only the summation order differs from the serial Fortran loop.
//
// IBX_MODE_PERIODIC replaces clipping by index wrap-around on a compact
// periodic array (no ghosts, no image markers needed).

#include "ibx_internal.h"
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
__device__ __forceinline__ const Prob*
find_problem(const ProbArg& A, long long gid, long long& local)
{
    if (A.n == 1)
    {
        local = gid;
        return &A.one;
    }
    int lo = 0, hi = A.n - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (A.offs[mid] <= gid)
            lo = mid;
        else
            hi = mid - 1;
    }
    local = gid - A.offs[lo];
    return &A.many[lo];
}

template <int DIM, int K, bool SPREAD>
__global__ void __launch_bounds__(128) generic_fp64_kernel(const ProbArg A)
{
    constexpr int W = KT<K>::W;
    const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (gid >= A.total) return;
    long long local;
    const Prob& P = *find_problem(A, gid, local);
    const int c = (int)(local % P.ncomp);
    const long long l = local / P.ncomp;
    const int s = P.indices ? P.indices[l] : (int)l;
    const Comp& C = P.comp[c];

    double w[3][W];
    int coord[3][W]; // array coordinate of stencil point i along each dim
    int st[3] = { 0, 0, 0 }, sp[3] = { 0, 0, 0 };
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
        const double X = P.X[(long long)DIM * s + d];
        const double Xsh = P.Xshift ? P.Xshift[(long long)DIM * l + d] : 0.0;
        int base;
        stencil_fp64<K>(X, Xsh, C.xlo[d], P.dx[d], C.box_lo[d], base, w[d]);
        if (C.wrapN[d])
        {
            const int N = C.wrapN[d];
            st[d] = 0;
            sp[d] = W - 1;
            int a = (base - C.box_lo[d]) % N;
            if (a < 0) a += N;
#pragma unroll
            for (int i = 0; i < W; ++i)
            {
                coord[d][i] = a;
                a = (a + 1 == N) ? 0 : a + 1;
            }
        }
        else
        {
            st[d] = max(C.clip_lo[d] - base, 0);
            sp[d] = W - 1 - max(base + W - 1 - C.clip_hi[d], 0);
#pragma unroll
            for (int i = 0; i < W; ++i) coord[d][i] = base + i - C.lo[d];
        }
    }
    if (DIM == 2)
    {
        st[2] = 0;
        sp[2] = 0;
        w[2][0] = 1.0;
        coord[2][0] = 0;
    }
    const long long n0 = C.n[0], n01 = (long long)C.n[0] * C.n[1];
    const double vol = P.vol;
    const int depth = P.side ? 1 : P.q_depth;
    for (int dd = 0; dd < depth; ++dd)
    {
        const long long qi = (long long)P.Q_depth * s + (P.side ? c : dd);
        double* q = static_cast<double*>(C.q) + C.depth_stride * dd;
        double V = 0.0;
        const double Vin = SPREAD ? static_cast<const double*>(P.Q)[qi] : 0.0;
#pragma unroll
        for (int i2 = 0; i2 < (DIM == 3 ? W : 1); ++i2)
        {
            if (i2 < st[2] || i2 > sp[2]) continue;
#pragma unroll
            for (int i1 = 0; i1 < W; ++i1)
            {
                if (i1 < st[1] || i1 > sp[1]) continue;
                double wyz;
                if (IsMacro<K>::value)
                    wyz = 0.0; // unused
                else if (DIM == 3)
                    wyz = w[1][i1] * (SPREAD ? w[2][i2] / vol : w[2][i2]);
                else
                    wyz = SPREAD ? w[1][i1] / vol : w[1][i1];
                const long long row = coord[2][i2] * n01 + coord[1][i1] * n0;
#pragma unroll
                for (int i0 = 0; i0 < W; ++i0)
                {
                    if (i0 < st[0] || i0 > sp[0]) continue;
                    const long long o = row + coord[0][i0];
                    if (IsMacro<K>::value)
                    {
                        double wt = w[0][i0] * w[1][i1];
                        if (DIM == 3) wt = wt * w[2][i2];
                        if (SPREAD)
                            atomicAdd(q + o, wt * Vin / vol);
                        else
                            V = V + wt * q[o];
                    }
                    else
                    {
                        const double t = w[0][i0] * wyz;
                        if (SPREAD)
                            atomicAdd(q + o, t * Vin);
                        else
                            V = V + t * q[o];
                    }
                }
            }
        }
        if (!SPREAD) static_cast<double*>(P.Q)[qi] = V;
    }
}

template <int DIM, int K>
int
launch_dk(bool spread, const ProbArg& A, cudaStream_t stream)
{
    const int threads = 128;
    const long long blocks = (A.total + threads - 1) / threads;
    if (blocks == 0) return 0;
    if (blocks > 0x7fffffffLL) return IBX_E_TOO_LARGE;
    if (spread)
        generic_fp64_kernel<DIM, K, true><<<(unsigned)blocks, threads, 0, stream>>>(A);
    else
        generic_fp64_kernel<DIM, K, false><<<(unsigned)blocks, threads, 0, stream>>>(A);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

template <int DIM>
int
launch_d(bool spread, int kernel, const ProbArg& A, cudaStream_t stream)
{
    switch (kernel)
    {
    case K_PL:
        return launch_dk<DIM, K_PL>(spread, A, stream);
    case K_PCUBIC:
        return launch_dk<DIM, K_PCUBIC>(spread, A, stream);
    case K_IB3:
        return launch_dk<DIM, K_IB3>(spread, A, stream);
    case K_IB4:
        return launch_dk<DIM, K_IB4>(spread, A, stream);
    case K_IB6:
        return launch_dk<DIM, K_IB6>(spread, A, stream);
    case K_BSPL4:
        return launch_dk<DIM, K_BSPL4>(spread, A, stream);
    default:
        return IBX_E_BAD_KERNEL;
    }
}
} // namespace

int
launch_generic(bool spread, int dim, int kernel, const ProbArg& arg, cudaStream_t stream)
{
    return dim == 2 ? launch_d<2>(spread, kernel, arg, stream) : launch_d<3>(spread, kernel, arg, stream);
}

} // namespace ibx
