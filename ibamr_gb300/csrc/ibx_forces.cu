// ibx_forces.cu -- Lagrangian spring forces on the device, computed right
// before spreading on the same stream (ibx_spring_forces in include/ibx.h).
//
// IBStandardForceGen::computeLagrangianSpringForce
// (src/IB/IBStandardForceGen.cpp:825-900) with the default force function
// (include/ibamr/IBSpringForceFunctions.h:104-107): for every spring between
// a master and a slave node, D = X_slave - X_master, R = |D|, springs with
// R < DBL_EPSILON are skipped, T = K (R - R0), and T/R * D is added to the
// master node's force and subtracted from the slave node's.

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
} // namespace
} // namespace ibx

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
