// ibx_device.cuh -- device-side building blocks shared by all kernels:
// kernel traits, exact Fortran index arithmetic, the delta functions in FP64
// (reference-faithful) and FP32 (mixed form), and the problem descriptors.
//
// Reference files (paths inside the IBAMR tree):
//   F2D/F3D = ibtk/src/lagrangian/fortran/lagrangian_interaction{2d,3d}.f.m4
//   FDELTA  = ibtk/src/lagrangian/fortran/lagrangian_delta.f.m4
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ibx
{
enum
{
    K_PL = 0,     // PIECEWISE_LINEAR
    K_PCUBIC = 1, // PIECEWISE_CUBIC
    K_IB3 = 2,    // IB_3
    K_IB4 = 3,    // IB_4
    K_IB6 = 4,    // IB_6
    K_BSPL4 = 5   // BSPLINE_4
};

// Stencil width actually touched by the Fortran loops (IB_3 reports 4 to
// getStencilSize but loops over 3 points).
template <int K>
struct KT;
template <>
struct KT<K_PL>
{
    static constexpr int W = 2;
};
template <>
struct KT<K_PCUBIC>
{
    static constexpr int W = 4;
};
template <>
struct KT<K_IB3>
{
    static constexpr int W = 3;
};
template <>
struct KT<K_IB4>
{
    static constexpr int W = 4;
};
template <>
struct KT<K_IB6>
{
    static constexpr int W = 6;
};
template <>
struct KT<K_BSPL4>
{
    static constexpr int W = 4;
};

// Kernels whose Fortran uses the SPREAD_INNER / INTERPOLATE_INNER macros
// (product w0*w1*w2*V/vol evaluated left to right) instead of an explicit
// tensor-product array.
template <int K>
struct IsMacro
{
    static constexpr bool value = (K == K_PL || K == K_PCUBIC || K == K_IB3 || K == K_BSPL4);
};

// ---------------------------------------------------------------------------
// Problem descriptors as the kernels see them.
// ---------------------------------------------------------------------------
struct Comp
{
    void* q;                  // array base
    int lo[3];                // index of element 0 along each dim
    int n[3];                 // array extents
    int box_lo[3];            // Fortran ilower of this component's data box
    int clip_lo[3], clip_hi[3]; // ghost box (IBX_MODE_PATCH)
    int wrapN[3];             // IBX_MODE_PERIODIC: cells (faces) per dim, else 0
    double xlo[3];            // x_lower of this component (side: shifted by -dx/2)
    long long depth_stride;   // elements between depth components
};

struct Prob
{
    int dim, ncomp, q_depth, Q_depth, side, mode;
    int n_items;              // selected markers
    double dx[3];
    double inv_dx[3];         // 1/dx
    int dx_pow2[3];           // dx is a power of two: (X-xlo)*inv_dx == (X-xlo)/dx exactly
    double vol;               // dx0*dx1[*dx2], association as in the Fortran
    const double* X;
    void* Q;
    const int* indices;
    const double* Xshift;
    Comp comp[3];
};

// ---------------------------------------------------------------------------
// Exact Fortran index arithmetic.
// ---------------------------------------------------------------------------

// Fortran NINT (halves away from zero); a - trunc(a) is exact.
__device__ __forceinline__ int
nint_exact(double a)
{
    double t = trunc(a);
    const double r = __dsub_rn(a, t);
    if (r >= 0.5)
        t = __dadd_rn(t, 1.0);
    else if (r <= -0.5)
        t = __dsub_rn(t, 1.0);
    return (int)t;
}

// Keeps index arithmetic in int range for any input (NaN and huge values
// land far outside every box and are clipped or wrapped harmlessly).
__device__ __forceinline__ double
clamp_index_arg(double t)
{
    return fmin(fmax(t, -1.0e8), 1.0e8);
}

// (X + Xshift - xlo)/dx rounded exactly as the Fortran expression.
__device__ __forceinline__ double
cell_coord(double Xs, double xlo, double dx)
{
    return clamp_index_arg(__ddiv_rn(__dsub_rn(Xs, xlo), dx));
}

// x_lower + (dble(ic - ilower) + 0.5)*dx without contraction.
__device__ __forceinline__ double
cell_center(int k, double xlo, double dx)
{
    return __dadd_rn(xlo, __dmul_rn(__dadd_rn((double)k, 0.5), dx));
}

// ---------------------------------------------------------------------------
// Delta functions (FDELTA), FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double
pcubic_delta(double r)
{
    if (r < 0.0) r = -r;
    if (r < 1.0) return 1.0 - 0.5 * r - r * r + 0.5 * r * r * r;
    if (r < 2.0) return 1.0 - (11.0 / 6.0) * r + r * r - (1.0 / 6.0) * r * r * r;
    return 0.0;
}

__device__ __forceinline__ double
ib3_delta(double r)
{
    const double sixth = 0.16666666666667;   // FDELTA:131, rounded as in the reference
    const double third = 0.333333333333333;  // FDELTA:132
    if (r < 0.0) r = -r;
    if (r < 0.5) return third * (1.0 + sqrt(1.0 - 3.0 * r * r));
    if (r < 1.5) return sixth * (5.0 - 3.0 * r - sqrt(1.0 - 3.0 * (1.0 - r) * (1.0 - r)));
    return 0.0;
}

__device__ __forceinline__ double
bspline4_delta(double x)
{
    const double modx = fabs(x);
    const double r = modx + 2.0;
    const double r2 = r * r;
    const double r3 = r2 * r;
    if (modx <= 1.0) return (1.0 / 6.0) * (3.0 * r3 - 24.0 * r2 + 60.0 * r - 44.0);
    if (modx <= 2.0) return (1.0 / 6.0) * (-r3 + 12.0 * r2 - 48.0 * r + 64.0);
    return 0.0;
}

// IB_6 weights from the kernel argument r (F2D:2013-2094).
template <typename T>
__device__ __forceinline__ void
ib6_weights(T r, T* w)
{
    const T K = (T)0.714075092976608; // (59/60)*(1-sqrt(1-3220/3481)), the Fortran PARAMETER
    const T r2 = r * r;
    const T r3 = r2 * r;
    const T r4 = r2 * r2;
    const T r6 = r3 * r3;
    const T alpha = (T)28.0;
    const T beta = (T)(9.0 / 4.0) - (T)(3.0 / 2.0) * (K + r2) + ((T)(22.0 / 3.0) - (T)7.0 * K) * r -
                   (T)(7.0 / 3.0) * r3;
    const T gamma = (T)(1.0 / 4.0) * (((T)(161.0 / 36.0) - (T)(59.0 / 6.0) * K + (T)5.0 * K * K) * (T)(1.0 / 2.0) * r2 +
                                      (-(T)(109.0 / 24.0) + (T)5.0 * K) * (T)(1.0 / 3.0) * r4 + (T)(5.0 / 18.0) * r6);
    const T discr = beta * beta - (T)4.0 * alpha * gamma;
    const T pm3 = (-beta + sqrt(discr)) / ((T)2.0 * alpha); // sign(1, 3/2 - K) = +1
    const T pm2 = -((T)3.0 * pm3) - (T)(1.0 / 16.0) + (T)(1.0 / 8.0) * (K + r2) +
                  (T)(1.0 / 12.0) * ((T)3.0 * K - (T)1.0) * r + (T)(1.0 / 12.0) * r3;
    const T pm1 = (T)2.0 * pm3 + (T)(1.0 / 4.0) + (T)(1.0 / 6.0) * ((T)4.0 - (T)3.0 * K) * r - (T)(1.0 / 6.0) * r3;
    const T p = (T)2.0 * pm3 + (T)(5.0 / 8.0) - (T)(1.0 / 4.0) * (K + r2);
    const T pp1 = -((T)3.0 * pm3) + (T)(1.0 / 4.0) - (T)(1.0 / 6.0) * ((T)4.0 - (T)3.0 * K) * r + (T)(1.0 / 6.0) * r3;
    const T pp2 = pm3 - (T)(1.0 / 16.0) + (T)(1.0 / 8.0) * (K + r2) - (T)(1.0 / 12.0) * ((T)3.0 * K - (T)1.0) * r -
                  (T)(1.0 / 12.0) * r3;
    w[0] = pm3;
    w[1] = pm2;
    w[2] = pm1;
    w[3] = p;
    w[4] = pp1;
    w[5] = pp2;
}

// The IB_6 constant K = (59/60)*(1-sqrt(1-3220/3481)) of the Fortran
// PARAMETER (F2D:2009); the literal is the correctly rounded double.
__device__ __forceinline__ double
ib6_K()
{
    return 0.714075092976608;
}

__device__ __forceinline__ void
ib6_weights_fp64(double r, double* w)
{
    const double K = ib6_K();
    const double r2 = r * r;
    const double r3 = r2 * r;
    const double r4 = r2 * r2;
    const double r6 = r3 * r3;
    const double alpha = 28.0;
    const double beta = (9.0 / 4.0) - (3.0 / 2.0) * (K + r2) + ((22.0 / 3.0) - 7.0 * K) * r - (7.0 / 3.0) * r3;
    const double gamma = (1.0 / 4.0) * (((161.0 / 36.0) - (59.0 / 6.0) * K + 5.0 * K * K) * (1.0 / 2.0) * r2 +
                                        (-(109.0 / 24.0) + 5.0 * K) * (1.0 / 3.0) * r4 + (5.0 / 18.0) * r6);
    const double discr = beta * beta - 4.0 * alpha * gamma;
    const double pm3 = (-beta + sqrt(discr)) / (2.0 * alpha);
    w[0] = pm3;
    w[1] = -(3.0 * pm3) - (1.0 / 16.0) + (1.0 / 8.0) * (K + r2) + (1.0 / 12.0) * (3.0 * K - 1.0) * r +
           (1.0 / 12.0) * r3;
    w[2] = 2.0 * pm3 + (1.0 / 4.0) + (1.0 / 6.0) * (4.0 - 3.0 * K) * r - (1.0 / 6.0) * r3;
    w[3] = 2.0 * pm3 + (5.0 / 8.0) - (1.0 / 4.0) * (K + r2);
    w[4] = -(3.0 * pm3) + (1.0 / 4.0) - (1.0 / 6.0) * (4.0 - 3.0 * K) * r + (1.0 / 6.0) * r3;
    w[5] = pm3 - (1.0 / 16.0) + (1.0 / 8.0) * (K + r2) - (1.0 / 12.0) * (3.0 * K - 1.0) * r - (1.0 / 12.0) * r3;
}

// ---------------------------------------------------------------------------
// Reference-faithful FP64 stencil of one dimension: base index (unclipped
// lower end) and all W weights, computed exactly as the Fortran routine.
// X is the marker position, Xsh its periodic shift, xlo/dx/ilo the geometry
// of the component's data box.
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void
stencil_fp64(double X, double Xsh, double xlo, double dx, int ilo, int& base, double* w)
{
    const double Xs = __dadd_rn(X, Xsh);
    if (K == K_IB4)
    {
        // F3D:1265-1293
        const double t = cell_coord(Xs, xlo, dx);
        const int m = nint_exact(t);
        base = m + ilo - 2;
        const double r = t - ((double)(m - 1) + 0.5);
        const double q = sqrt(1.0 + 4.0 * r * (1.0 - r));
        w[0] = 0.125 * (3.0 - 2.0 * r - q);
        w[1] = 0.125 * (3.0 - 2.0 * r + q);
        w[2] = 0.125 * (1.0 + 2.0 * r + q);
        w[3] = 0.125 * (1.0 + 2.0 * r - q);
    }
    else if (K == K_IB6)
    {
        // F3D:2244-2330
        const double t = cell_coord(Xs, xlo, dx);
        const int m = nint_exact(t);
        base = m + ilo - 3;
        const double r = (1.0 - t) + ((double)(m - 1) + 0.5);
        ib6_weights_fp64(r, w);
    }
    else if (K == K_PL)
    {
        // F3D:305-330
        const double t = clamp_index_arg(__dsub_rn(__ddiv_rn(__dsub_rn(Xs, xlo), dx), 0.5));
        const int icc = ilo + nint_exact(t);
        const double Xc = cell_center(icc - ilo, xlo, dx);
        if (Xs < Xc)
        {
            base = icc - 1;
            w[0] = (Xc - Xs) / dx;
        }
        else
        {
            base = icc;
            w[0] = 1.0 + (Xc - Xs) / dx;
        }
        w[1] = 1.0 - w[0];
    }
    else
    {
        // IB_3 (F3D:1040-1070), PIECEWISE_CUBIC (F3D:808-840), BSPLINE_4
        // (F3D:2879-2907): floor-based cell; the half-cell test of the even
        // kernels uses the UNSHIFTED position.
        const double t = cell_coord(Xs, xlo, dx);
        const int icc = (int)floor(t) + ilo;
        if (K == K_IB3)
            base = icc - 1;
        else
            base = (X < cell_center(icc - ilo, xlo, dx)) ? icc - 2 : icc - 1;
#pragma unroll
        for (int i = 0; i < KT<K>::W; ++i)
        {
            const double Xc = cell_center(base + i - ilo, xlo, dx);
            const double arg = (Xs - Xc) / dx;
            w[i] = (K == K_IB3) ? ib3_delta(arg) : (K == K_PCUBIC) ? pcubic_delta(arg) : bspline4_delta(arg);
        }
    }
}

} // namespace ibx
