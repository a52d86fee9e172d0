// ibx_forces.cu -- the Lagrangian forces of IBStandardForceGen on the device,
// computed right before spreading on the same stream (ibx_spring_forces,
// ibx_beam_forces, ibx_target_point_forces, ibx_body_forces in
// include/ibx.h).  One thread per spring, beam, target point or marker;
// contributions to shared nodes are summed with atomics.
//
// Springs: IBStandardForceGen::computeLagrangianSpringForce
// (src/IB/IBStandardForceGen.cpp:825-900) with the default force function
// (include/ibamr/IBSpringForceFunctions.h:104-107): for every spring between
// a master and a slave node, D = X_slave - X_master, R = |D|, springs with
// R < DBL_EPSILON are skipped, T = K (R - R0), and T/R * D is added to the
// master node's force and subtracted from the slave node's.
//
// Beams: computeLagrangianBeamForce (IBStandardForceGen.cpp:1037-1147): per
// beam F = K ((X_next + X_prev) - 2 X_master - D2X0), 2F added to the
// master node's force, F subtracted from each neighbour's.
//
// Target points: computeLagrangianTargetPointForce (:1201-1299):
// F += kappa (X_target - X) - eta U at the point's node; with logging on,
// the largest |X_target - X| over the points.
//
// Body forces: computeLagrangianBodyForce (:1301-1327): the structure's
// uniform force added to every node of a structure that has one.

#include "ibx_internal.h"
#include "../../include/ibx.h"

#include <cfloat>

namespace ibx
{
namespace
{
template <int DIM, typename T>
__global__ void
spring_kernel(int n_markers, const double* X, int n_springs, const int* mastr, const int* slave,
              const double* stiffness, const double* rest, T* F, int* status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_springs) return;
    const int m = mastr[k], s = slave[k];
    if (m < 0 || s < 0 || m >= n_markers || s >= n_markers)
    {
        atomicOr(status, 1);
        return;
    }
    double D[DIM], R2 = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
        D[d] = X[DIM * (long long)s + d] - X[DIM * (long long)m + d];
        R2 += D[d] * D[d];
    }
    const double R = sqrt(R2);
    if (R < DBL_EPSILON) return;
    const double T_over_R = stiffness[k] * (R - rest[k]) / R;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
        const double f = T_over_R * D[d];
        atomicAdd(F + DIM * (long long)m + d, (T)f);
        atomicAdd(F + DIM * (long long)s + d, (T)(-f));
    }
}
template <int DIM, typename T>
__global__ void
beam_kernel(int n_markers, const double* X, int n_beams, const int* mastr, const int* next, const int* prev,
            const double* rigidity, const double* curvature, T* F, int* status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_beams) return;
    const int m = mastr[k], a = next[k], b = prev[k];
    if (m < 0 || a < 0 || b < 0 || m >= n_markers || a >= n_markers || b >= n_markers)
    {
        atomicOr(status, 1);
        return;
    }
    const double K = rigidity[k];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
        // every operation rounded on its own, in the reference's order (no
        // contraction into fused multiply-adds)
        const double f =
            __dmul_rn(K, __dsub_rn(__dsub_rn(__dadd_rn(X[DIM * (long long)a + d], X[DIM * (long long)b + d]),
                                             __dmul_rn(2.0, X[DIM * (long long)m + d])),
                                   curvature[DIM * (long long)k + d]));
        atomicAdd(F + DIM * (long long)m + d, (T)__dmul_rn(2.0, f));
        atomicAdd(F + DIM * (long long)a + d, (T)(-f));
        atomicAdd(F + DIM * (long long)b + d, (T)(-f));
    }
}

// The largest displacement as the bits of a non-negative double (ordered
// like the values), so an integer maximum finds it.
template <int DIM, typename T>
__global__ void
target_kernel(int n_markers, const double* X, const double* U, int n_points, const int* node, const double* kappa,
              const double* eta, const double* X_target, T* F, unsigned long long* max_disp, int* status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_points) return;
    const int i = node[k];
    if (i < 0 || i >= n_markers)
    {
        atomicOr(status, 1);
        return;
    }
    const double K = kappa[k], E = eta[k];
    double dX = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
        const double x0 = X_target[DIM * (long long)k + d], x = X[DIM * (long long)i + d];
        const double u = U ? U[DIM * (long long)i + d] : 0.0;
        const double e = __dsub_rn(x0, x);
        atomicAdd(F + DIM * (long long)i + d, (T)__dsub_rn(__dmul_rn(K, e), __dmul_rn(E, u)));
        dX = __dadd_rn(dX, __dmul_rn(e, e));
    }
    if (max_disp) atomicMax(max_disp, (unsigned long long)__double_as_longlong(sqrt(dX)));
}

template <int DIM, typename T>
__global__ void
body_kernel(int n_markers, const int* structure, int n_structures, const double* force, const int* has_force, T* F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_markers) return;
    const int sid = structure[i];
    if (sid < 0 || sid >= n_structures || (has_force && !has_force[sid])) return;
#pragma unroll
    for (int d = 0; d < DIM; ++d) F[DIM * (long long)i + d] += (T)force[DIM * (long long)sid + d];
}

// Common checks of the force entry points; zeroes F unless accumulating.
int
force_prologue(int dim, int n_markers, int n_items, const void* X, void* F, int precision, int accumulate,
               const int* status, cudaStream_t s)
{
    if (dim != 2 && dim != 3) return IBX_E_ARG;
    if (n_markers < 0 || n_items < 0) return IBX_E_ARG;
    if (precision != IBX_PRECISION_FP64 && precision != IBX_PRECISION_MIXED) return IBX_E_ARG;
    if (n_markers > 0 && (!X || !F)) return IBX_E_ARG;
    if (!status) return IBX_E_ARG;
    const size_t esize = precision == IBX_PRECISION_FP64 ? sizeof(double) : sizeof(float);
    if (!accumulate && n_markers > 0 && cudaMemsetAsync(F, 0, esize * dim * (size_t)n_markers, s) != cudaSuccess)
        return IBX_E_CUDA;
    return IBX_OK;
}
} // namespace
} // namespace ibx

extern "C" int
ibx_beam_forces(int dim, int n_markers, const double* X, int n_beams, const int* master, const int* next,
                const int* prev, const double* rigidity, const double* curvature, void* F, int precision,
                int accumulate, int* status, void* stream)
{
    using namespace ibx;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_beams > 0 && (!master || !next || !prev || !rigidity || !curvature)) return IBX_E_ARG;
    const int rc = force_prologue(dim, n_markers, n_beams, X, F, precision, accumulate, status, s);
    if (rc || n_beams == 0) return rc;
    const unsigned blocks = (unsigned)((n_beams + 255) / 256);
    const bool f64 = precision == IBX_PRECISION_FP64;
#define IBX_BEAM(DD, TT)                                                                                             \
    beam_kernel<DD, TT><<<blocks, 256, 0, s>>>(n_markers, X, n_beams, master, next, prev, rigidity, curvature,       \
                                               static_cast<TT*>(F), status)
    if (dim == 2)
    {
        if (f64)
            IBX_BEAM(2, double);
        else
            IBX_BEAM(2, float);
    }
    else if (f64)
        IBX_BEAM(3, double);
    else
        IBX_BEAM(3, float);
#undef IBX_BEAM
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

extern "C" int
ibx_target_point_forces(int dim, int n_markers, const double* X, const double* U, int n_points, const int* node,
                        const double* kappa, const double* eta, const double* X_target, void* F, int precision,
                        int accumulate, double* max_displacement, int* status, void* stream)
{
    using namespace ibx;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_points > 0 && (!node || !kappa || !eta || !X_target)) return IBX_E_ARG;
    const int rc = force_prologue(dim, n_markers, n_points, X, F, precision, accumulate, status, s);
    if (rc) return rc;
    unsigned long long* md = reinterpret_cast<unsigned long long*>(max_displacement);
    if (md && cudaMemsetAsync(md, 0, sizeof(double), s) != cudaSuccess) return IBX_E_CUDA; // bits of +0.0
    if (n_points == 0) return IBX_OK;
    const unsigned blocks = (unsigned)((n_points + 255) / 256);
    const bool f64 = precision == IBX_PRECISION_FP64;
#define IBX_TARGET(DD, TT)                                                                                           \
    target_kernel<DD, TT><<<blocks, 256, 0, s>>>(n_markers, X, U, n_points, node, kappa, eta, X_target,              \
                                                 static_cast<TT*>(F), md, status)
    if (dim == 2)
    {
        if (f64)
            IBX_TARGET(2, double);
        else
            IBX_TARGET(2, float);
    }
    else if (f64)
        IBX_TARGET(3, double);
    else
        IBX_TARGET(3, float);
#undef IBX_TARGET
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

extern "C" int
ibx_body_forces(int dim, int n_markers, const int* structure, int n_structures, const double* force,
                const int* has_force, void* F, int precision, void* stream)
{
    using namespace ibx;
    if (dim != 2 && dim != 3) return IBX_E_ARG;
    if (n_markers < 0 || n_structures < 0) return IBX_E_ARG;
    if (precision != IBX_PRECISION_FP64 && precision != IBX_PRECISION_MIXED) return IBX_E_ARG;
    if (n_markers > 0 && (!structure || !F)) return IBX_E_ARG;
    if (n_structures > 0 && !force) return IBX_E_ARG;
    if (n_markers == 0 || n_structures == 0) return IBX_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((n_markers + 255) / 256);
    const bool f64 = precision == IBX_PRECISION_FP64;
#define IBX_BODY(DD, TT)                                                                                             \
    body_kernel<DD, TT><<<blocks, 256, 0, s>>>(n_markers, structure, n_structures, force, has_force,                \
                                               static_cast<TT*>(F))
    if (dim == 2)
    {
        if (f64)
            IBX_BODY(2, double);
        else
            IBX_BODY(2, float);
    }
    else if (f64)
        IBX_BODY(3, double);
    else
        IBX_BODY(3, float);
#undef IBX_BODY
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

extern "C" int
ibx_spring_forces(int dim, int n_markers, const double* X, int n_springs, const int* master, const int* slave,
                  const double* stiffness, const double* rest_length, void* F, int precision, int accumulate,
                  int* status, void* stream)
{
    using namespace ibx;
    if (dim != 2 && dim != 3) return IBX_E_ARG;
    if (n_markers < 0 || n_springs < 0) return IBX_E_ARG;
    if (precision != IBX_PRECISION_FP64 && precision != IBX_PRECISION_MIXED) return IBX_E_ARG;
    if ((n_markers > 0 && (!X || !F)) || (n_springs > 0 && (!master || !slave || !stiffness || !rest_length)))
        return IBX_E_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t esize = precision == IBX_PRECISION_FP64 ? sizeof(double) : sizeof(float);
    if (!accumulate && n_markers > 0 && cudaMemsetAsync(F, 0, esize * dim * (size_t)n_markers, s) != cudaSuccess)
        return IBX_E_CUDA;
    if (n_springs == 0) return IBX_OK;
    const unsigned blocks = (unsigned)((n_springs + 255) / 256);
    int* st = status;
    if (!st) return IBX_E_ARG; // a device word that records invalid node indices
    if (dim == 2)
    {
        if (precision == IBX_PRECISION_FP64)
            spring_kernel<2, double><<<blocks, 256, 0, s>>>(n_markers, X, n_springs, master, slave, stiffness,
                                                            rest_length, static_cast<double*>(F), st);
        else
            spring_kernel<2, float><<<blocks, 256, 0, s>>>(n_markers, X, n_springs, master, slave, stiffness,
                                                           rest_length, static_cast<float*>(F), st);
    }
    else
    {
        if (precision == IBX_PRECISION_FP64)
            spring_kernel<3, double><<<blocks, 256, 0, s>>>(n_markers, X, n_springs, master, slave, stiffness,
                                                            rest_length, static_cast<double*>(F), st);
        else
            spring_kernel<3, float><<<blocks, 256, 0, s>>>(n_markers, X, n_springs, master, slave, stiffness,
                                                           rest_length, static_cast<float*>(F), st);
    }
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}
