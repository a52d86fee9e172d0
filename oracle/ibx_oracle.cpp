// ibx_oracle.cpp -- CPU oracle (test infrastructure only; see ibx_oracle.h).
//
// A line-by-line restatement of IBAMR's Fortran Lagrangian-Eulerian
// interaction routines and of the LEInteractor wrapper layer around them.
// Compiled with -O2 -ffp-contract=off and no fast-math so that every
// floating-point operation rounds as the Fortran source states it.
//
// F2D/F3D/FDELTA/LEI abbreviations as in ibx_oracle.h.

#include "ibx_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <atomic>
#include <thread>
#include <vector>

namespace
{
// ---------------------------------------------------------------------------
// Scalar helpers.
// ---------------------------------------------------------------------------

// Fortran NINT: nearest integer, halves away from zero.  a - trunc(a) is exact
// for every finite double (Sterbenz), so the tie test is exact.
inline int
nint(double a)
{
    double t = std::trunc(a);
    const double r = a - t;
    if (r >= 0.5)
        t += 1.0;
    else if (r <= -0.5)
        t -= 1.0;
    return static_cast<int>(t);
}

// FDELTA:29-45 lagrangian_piecewise_linear_delta.
inline double
piecewise_linear_delta(double r)
{
    if (r < 0.0) r = -r;
    return r < 1.0 ? 1.0 - r : 0.0;
}

// FDELTA:74-101 lagrangian_piecewise_cubic_delta.
inline double
piecewise_cubic_delta(double r)
{
    if (r < 0.0) r = -r;
    if (r < 1.0) return 1.0 - 0.5 * r - r * r + 0.5 * r * r * r;
    if (r < 2.0) return 1.0 - (11.0 / 6.0) * r + r * r - (1.0 / 6.0) * r * r * r;
    return 0.0;
}

// FDELTA:123-153 lagrangian_ib_3_delta, with the reference's rounded
// constants sixth = 0.16666666666667d0 and third = 0.333333333333333d0.
inline double
ib_3_delta(double r)
{
    const double sixth = 0.16666666666667;
    const double third = 0.333333333333333;
    if (r < 0.0) r = -r;
    if (r < 0.5) return third * (1.0 + std::sqrt(1.0 - 3.0 * r * r));
    if (r < 1.5) return sixth * (5.0 - 3.0 * r - std::sqrt(1.0 - 3.0 * (1.0 - r) * (1.0 - r)));
    return 0.0;
}

// FDELTA:268-294 lagrangian_bspline_4_delta (note the .le. bounds).
inline double
bspline_4_delta(double x)
{
    const double modx = std::fabs(x);
    const double r = modx + 2.0;
    const double r2 = r * r;
    const double r3 = r2 * r;
    if (modx <= 1.0) return (1.0 / 6.0) * (3.0 * r3 - 24.0 * r2 + 60.0 * r - 44.0);
    if (modx <= 2.0) return (1.0 / 6.0) * (-r3 + 12.0 * r2 - 48.0 * r + 64.0);
    return 0.0;
}

// IB_6 weights for one dimension (F2D:2013-2094, F3D:2244-2330): the
// quadratic-root construction of the 6-point kernel.
inline void
ib_6_weights(double r, double* w)
{
    const double K = (59.0 / 60.0) * (1.0 - std::sqrt(1.0 - (3220.0 / 3481.0)));
    const double r2 = r * r;
    const double r3 = r2 * r;
    const double r4 = r2 * r2;
    const double r6 = r3 * r3;
    const double alpha = 28.0;
    const double beta = (9.0 / 4.0) - (3.0 / 2.0) * (K + r2) + ((22.0 / 3.0) - 7.0 * K) * r - (7.0 / 3.0) * r3;
    const double gamma = (1.0 / 4.0) * (((161.0 / 36.0) - (59.0 / 6.0) * K + 5.0 * K * K) * (1.0 / 2.0) * r2 +
                                        (-(109.0 / 24.0) + 5.0 * K) * (1.0 / 3.0) * r4 + (5.0 / 18.0) * r6);
    const double discr = beta * beta - 4.0 * alpha * gamma;
    const double sgn = ((3.0 / 2.0) - K) >= 0.0 ? 1.0 : -1.0; // sign(1.d0, 3/2 - K)
    const double pm3 = (-beta + sgn * std::sqrt(discr)) / (2.0 * alpha);
    const double pm2 = -(3.0 * pm3) - (1.0 / 16.0) + (1.0 / 8.0) * (K + r2) + (1.0 / 12.0) * (3.0 * K - 1.0) * r +
                       (1.0 / 12.0) * r3;
    const double pm1 = 2.0 * pm3 + (1.0 / 4.0) + (1.0 / 6.0) * (4.0 - 3.0 * K) * r - (1.0 / 6.0) * r3;
    const double p = 2.0 * pm3 + (5.0 / 8.0) - (1.0 / 4.0) * (K + r2);
    const double pp1 = -(3.0 * pm3) + (1.0 / 4.0) - (1.0 / 6.0) * (4.0 - 3.0 * K) * r + (1.0 / 6.0) * r3;
    const double pp2 = pm3 - (1.0 / 16.0) + (1.0 / 8.0) * (K + r2) - (1.0 / 12.0) * (3.0 * K - 1.0) * r -
                       (1.0 / 12.0) * r3;
    w[0] = pm3;
    w[1] = pm2;
    w[2] = pm1;
    w[3] = p;
    w[4] = pp1;
    w[5] = pp2;
}

// ---------------------------------------------------------------------------
// One-dimensional stencils.  A stencil covers indices base+i for i in
// [start, stop]; w[i] is the weight of index base+i.  Kernels whose Fortran
// computes every weight and clips the loop (IB_4, IB_6, PIECEWISE_LINEAR) set
// base to the unclipped lower index; kernels that clip first and evaluate the
// weights on the clipped range (IB_3, PIECEWISE_CUBIC, BSPLINE_4) set base to
// the clipped lower index and start to 0.
// ---------------------------------------------------------------------------
struct Sten
{
    int base, start, stop;
    double w[6];
};

// Macro-loop kernels (floor-based stencil, SPREAD_INNER/INTERPOLATE_INNER
// product order) versus kernels with an explicit tensor product.
inline bool
is_macro_kernel(int k)
{
    return k == IBXO_PIECEWISE_LINEAR || k == IBXO_PIECEWISE_CUBIC || k == IBXO_IB_3 || k == IBXO_BSPLINE_4;
}

void
stencil_1d(int kernel, double X, double Xsh, double xlo, double dx, int ilo, int iup, int g, Sten& S)
{
    const int glo = ilo - g;
    const int gup = iup + g;
    switch (kernel)
    {
    case IBXO_IB_4:
    {
        // F2D:1209-1218 / F3D:1265-1293.
        const double X_o_dx = (X + Xsh - xlo) / dx;
        const int icl = nint(X_o_dx) + ilo - 2;
        const int icu = icl + 3;
        const double r = X_o_dx - (static_cast<double>(icl + 1 - ilo) + 0.5);
        const double q = std::sqrt(1.0 + 4.0 * r * (1.0 - r));
        S.w[0] = 0.125 * (3.0 - 2.0 * r - q);
        S.w[1] = 0.125 * (3.0 - 2.0 * r + q);
        S.w[2] = 0.125 * (1.0 + 2.0 * r + q);
        S.w[3] = 0.125 * (1.0 + 2.0 * r - q);
        S.base = icl;
        S.start = std::max(glo - icl, 0);
        S.stop = 3 - std::max(icu - gup, 0);
        return;
    }
    case IBXO_IB_6:
    {
        // F2D:2013-2094 / F3D:2244-2330.
        const double X_o_dx = (X + Xsh - xlo) / dx;
        const int icl = nint(X_o_dx) + ilo - 3;
        const int icu = icl + 5;
        const double r = 1.0 - X_o_dx + (static_cast<double>(icl + 2 - ilo) + 0.5);
        ib_6_weights(r, S.w);
        S.base = icl;
        S.start = std::max(glo - icl, 0);
        S.stop = 5 - std::max(icu - gup, 0);
        return;
    }
    case IBXO_PIECEWISE_LINEAR:
    {
        // F2D:525-551 / F3D:305-330: NINT-based centre, shifted position.
        const double Xs = X + Xsh;
        const int icc = ilo + nint((Xs - xlo) / dx - 0.5);
        const double Xcell = xlo + (static_cast<double>(icc - ilo) + 0.5) * dx;
        int lo;
        if (Xs < Xcell)
        {
            lo = icc - 1;
            S.w[0] = (Xcell - Xs) / dx;
            S.w[1] = 1.0 - S.w[0];
        }
        else
        {
            lo = icc;
            S.w[0] = 1.0 + (Xcell - Xs) / dx;
            S.w[1] = 1.0 - S.w[0];
        }
        const int hi = lo + 1;
        S.base = lo;
        S.start = std::max(lo, glo) - lo;
        S.stop = std::min(hi, gup) - lo;
        return;
    }
    case IBXO_IB_3:
    case IBXO_PIECEWISE_CUBIC:
    case IBXO_BSPLINE_4:
    {
        // IB_3: F2D:989-1020; PIECEWISE_CUBIC: F2D:764-793 (F3D:808-840);
        // BSPLINE_4: F2D:2565-2595 (F3D:2879-2907).  Cell from floor() of
        // the shifted position; the even-width half-cell test compares the
        // UNSHIFTED X with the cell centre (F2D:777, F3D:816, F3D:2891).
        const int icc = static_cast<int>(std::floor((X + Xsh - xlo) / dx)) + ilo;
        const double Xcell = xlo + (static_cast<double>(icc - ilo) + 0.5) * dx;
        int lo, hi;
        if (kernel == IBXO_IB_3)
        {
            lo = icc - 1;
            hi = icc + 1;
        }
        else if (X < Xcell)
        {
            lo = icc - 2;
            hi = icc + 1;
        }
        else
        {
            lo = icc - 1;
            hi = icc + 2;
        }
        lo = std::max(lo, glo);
        hi = std::min(hi, gup);
        for (int ic = lo; ic <= hi; ++ic)
        {
            const double Xc = xlo + (static_cast<double>(ic - ilo) + 0.5) * dx;
            const double arg = (X + Xsh - Xc) / dx;
            double wv;
            if (kernel == IBXO_IB_3)
                wv = ib_3_delta(arg);
            else if (kernel == IBXO_PIECEWISE_CUBIC)
                wv = piecewise_cubic_delta(arg);
            else
                wv = bspline_4_delta(arg);
            S.w[ic - lo] = wv;
        }
        S.base = lo;
        S.start = 0;
        S.stop = hi - lo;
        return;
    }
    default:
        S.base = 0;
        S.start = 0;
        S.stop = -1;
        return;
    }
}

// Fortran-order offset into u(CELLnDVECG(ilower,iupper,nugc), 0:depth-1).
struct ArrayGeom
{
    int dim;
    int glo[3], n[3];
    long long vol;
    long long off(const int* ic, int d) const
    {
        long long o = 0;
        for (int k = dim - 1; k >= 0; --k) o = o * n[k] + (ic[k] - glo[k]);
        return o + vol * d;
    }
};

ArrayGeom
make_geom(int dim, const int* ilower, const int* iupper, const int* nugc)
{
    ArrayGeom G;
    G.dim = dim;
    G.vol = 1;
    for (int d = 0; d < 3; ++d)
    {
        G.glo[d] = 0;
        G.n[d] = 1;
    }
    for (int d = 0; d < dim; ++d)
    {
        G.glo[d] = ilower[d] - nugc[d];
        G.n[d] = iupper[d] + nugc[d] - G.glo[d] + 1;
        G.vol *= G.n[d];
    }
    return G;
}

bool
valid_kernel(int k)
{
    return k == IBXO_PIECEWISE_LINEAR || k == IBXO_PIECEWISE_CUBIC || k == IBXO_IB_3 || k == IBXO_IB_4 ||
           k == IBXO_IB_6 || k == IBXO_BSPLINE_4;
}

// The per-marker interpolation / spreading loop shared by all kernels.  The
// weight products follow the reference's association order:
//  - explicit tensor kernels (IB_4, IB_6): w = w0*(w1*(w2[/vol])) then
//    V += w*u or u += w*V (F3D:1296-1328, 1436-1468);
//  - macro kernels: V += w0*w1*w2*u and u += w0*w1*w2*V/vol, evaluated left
//    to right (F3D:24-68).
template <bool SPREAD>
int
interaction(int kernel, int dim, const double* dx, const double* x_lower, int depth, const int* ilower,
            const int* iupper, const int* nugc, double* u, const double* uc, const int* indices, const double* Xshift,
            int nindices, const double* X, double* V, const double* Vc)
{
    if (!valid_kernel(kernel)) return IBXO_E_BAD_KERNEL;
    if (dim != 2 && dim != 3) return IBXO_E_ARG;
    const ArrayGeom G = make_geom(dim, ilower, iupper, nugc);
    const bool macro = is_macro_kernel(kernel);
    const double vol = dim == 2 ? dx[0] * dx[1] : dx[0] * dx[1] * dx[2];
    for (int l = 0; l < nindices; ++l)
    {
        const int s = indices[l];
        Sten S[3];
        for (int d = 0; d < 3; ++d)
        {
            S[d].base = 0;
            S[d].start = 0;
            S[d].stop = 0;
            S[d].w[0] = 1.0;
        }
        for (int d = 0; d < dim; ++d)
            stencil_1d(kernel, X[dim * s + d], Xshift[dim * l + d], x_lower[d], dx[d], ilower[d], iupper[d], nugc[d],
                       S[d]);
        for (int dd = 0; dd < depth; ++dd)
        {
            if (!SPREAD) V[depth * s + dd] = 0.0;
            int ic[3] = { 0, 0, 0 };
            for (int i2 = S[2].start; i2 <= S[2].stop; ++i2)
            {
                ic[2] = S[2].base + i2;
                for (int i1 = S[1].start; i1 <= S[1].stop; ++i1)
                {
                    ic[1] = S[1].base + i1;
                    for (int i0 = S[0].start; i0 <= S[0].stop; ++i0)
                    {
                        ic[0] = S[0].base + i0;
                        const long long o = G.off(ic, dd);
                        if (macro)
                        {
                            double w = S[0].w[i0] * S[1].w[i1];
                            if (dim == 3) w = w * S[2].w[i2];
                            if (SPREAD)
                                u[o] = u[o] + (w * Vc[depth * s + dd] / vol);
                            else
                                V[depth * s + dd] = V[depth * s + dd] + w * uc[o];
                        }
                        else
                        {
                            double t;
                            if (dim == 3)
                            {
                                const double wz = SPREAD ? S[2].w[i2] / vol : S[2].w[i2];
                                t = S[0].w[i0] * (S[1].w[i1] * wz);
                            }
                            else
                            {
                                const double wy = SPREAD ? S[1].w[i1] / vol : S[1].w[i1];
                                t = S[0].w[i0] * wy;
                            }
                            if (SPREAD)
                                u[o] = u[o] + t * Vc[depth * s + dd];
                            else
                                V[depth * s + dd] = V[depth * s + dd] + t * uc[o];
                        }
                    }
                }
            }
        }
    }
    return IBXO_OK;
}

void
side_box(const ibxo_patch* P, int axis, int* lo, int* hi)
{
    for (int d = 0; d < P->dim; ++d)
    {
        lo[d] = P->ilower[d];
        hi[d] = P->iupper[d] + (d == axis ? 1 : 0);
    }
}

int
min_gcw(const ibxo_patch_data* q, int dim)
{
    int m = q->gcw[0];
    for (int d = 1; d < dim; ++d) m = std::min(m, q->gcw[d]);
    return m;
}

bool
touches_physical(const ibxo_patch* P)
{
    for (int d = 0; d < P->dim; ++d)
        if (P->touches_regular_lower[d] || P->touches_regular_upper[d]) return true;
    return false;
}

} // namespace

extern "C" {

int
ibxo_stencil_size(int kernel)
{
    switch (kernel)
    {
    case IBXO_PIECEWISE_LINEAR:
        return 2;
    case IBXO_PIECEWISE_CUBIC:
    case IBXO_IB_3:
    case IBXO_IB_4:
    case IBXO_BSPLINE_4:
        return 4;
    case IBXO_IB_6:
        return 6;
    default:
        return -1;
    }
}

int
ibxo_min_ghost_width(int kernel)
{
    const int w = ibxo_stencil_size(kernel);
    if (w < 0) return -1;
    return static_cast<int>(std::floor(0.5 * w)) + 1;
}

int
ibxo_kernel_from_name(const char* name)
{
    const std::string s(name ? name : "");
    if (s == "PIECEWISE_LINEAR") return IBXO_PIECEWISE_LINEAR;
    if (s == "PIECEWISE_CUBIC") return IBXO_PIECEWISE_CUBIC;
    if (s == "IB_3") return IBXO_IB_3;
    if (s == "IB_4") return IBXO_IB_4;
    if (s == "IB_6") return IBXO_IB_6;
    if (s == "BSPLINE_4") return IBXO_BSPLINE_4;
    return -1;
}

int
ibxo_nint(double a)
{
    return nint(a);
}

int
ibxo_stencil_1d(int kernel, double X, double Xshift, double x_lower, double dx, int ilower, int iupper, int ghost,
                int* base, int* start, int* stop, double* w)
{
    if (!valid_kernel(kernel)) return IBXO_E_BAD_KERNEL;
    Sten S;
    stencil_1d(kernel, X, Xshift, x_lower, dx, ilower, iupper, ghost, S);
    *base = S.base;
    *start = S.start;
    *stop = S.stop;
    for (int i = 0; i < 6; ++i) w[i] = i <= S.stop ? S.w[i] : 0.0;
    return IBXO_OK;
}

int
ibxo_fortran_interp(int kernel, int dim, const double* dx, const double* x_lower, const double* /*x_upper*/,
                    int depth, const int* ilower, const int* iupper, const int* nugc, const double* u,
                    const int* indices, const double* Xshift, int nindices, const double* X, double* V)
{
    return interaction<false>(kernel, dim, dx, x_lower, depth, ilower, iupper, nugc, nullptr, u, indices, Xshift,
                              nindices, X, V, nullptr);
}

int
ibxo_fortran_spread(int kernel, int dim, const double* dx, const double* x_lower, const double* /*x_upper*/,
                    int depth, const int* indices, const double* Xshift, int nindices, const double* X,
                    const double* V, const int* ilower, const int* iupper, const int* nugc, double* u)
{
    return interaction<true>(kernel, dim, dx, x_lower, depth, ilower, iupper, nugc, u, nullptr, indices, Xshift,
                             nindices, X, nullptr, V);
}

void
ibxo_get_cell_index(int dim, const double* X, const double* x_lower, const double* x_upper, const double* dx,
                    const int* ilower, const int* iupper, int* idx)
{
    for (int d = 0; d < dim; ++d)
    {
        const double dX_lower = X[d] - x_lower[d];
        const double dX_upper = X[d] - x_upper[d];
        if (std::fabs(dX_lower) <= std::fabs(dX_upper))
            idx[d] = static_cast<int>(ilower[d] + std::floor(dX_lower / dx[d]));
        else
            idx[d] = static_cast<int>(iupper[d] + std::floor(dX_upper / dx[d]) + 1);
    }
}

int
ibxo_build_local_indices(const ibxo_patch* P, const int* box_lo, const int* box_hi, const double* X, int n_markers,
                         int* local_indices)
{
    int n = 0;
    for (int k = 0; k < n_markers; ++k)
    {
        int i[3];
        ibxo_get_cell_index(P->dim, &X[P->dim * k], P->x_lower, P->x_upper, P->dx, P->ilower, P->iupper, i);
        bool inside = true;
        for (int d = 0; d < P->dim; ++d) inside = inside && i[d] >= box_lo[d] && i[d] <= box_hi[d];
        if (inside) local_indices[n++] = k;
    }
    return n;
}

int
ibxo_cache_local_indices(const ibxo_patch* P, const int* periodic_shift, const int* ghost_width, int want_ghost_box,
                         const double* X, int n_markers, int capacity, int* local_indices, double* periodic_shifts)
{
    const int dim = P->dim;
    int lo[3], hi[3];
    for (int d = 0; d < dim; ++d)
    {
        const int g = want_ghost_box ? ghost_width[d] : 0;
        lo[d] = P->ilower[d] - g;
        hi[d] = P->iupper[d] + g;
    }
    int n = 0;
    for (int s = 0; s < n_markers; ++s)
    {
        int c[3];
        ibxo_get_cell_index(dim, &X[dim * s], P->x_lower, P->x_upper, P->dx, P->ilower, P->iupper, c);
        // Candidate periodic images k in {-1,0,1}^dim (only along periodic sides).
        const int nimg = dim == 2 ? 9 : 27;
        for (int m = 0; m < nimg; ++m)
        {
            const int k[3] = { m % 3 - 1, (m / 3) % 3 - 1, dim == 3 ? (m / 9) % 3 - 1 : 0 };
            bool ok = true;
            int off[3] = { 0, 0, 0 };
            for (int d = 0; d < dim && ok; ++d)
            {
                const int i = c[d] + k[d] * periodic_shift[d];
                if (k[d] != 0 && periodic_shift[d] == 0) ok = false;
                if (i < lo[d] || i > hi[d]) ok = false;
                // LIndexSetData.cpp:83-100: the offset follows from where the
                // image cell sits relative to the patch box.
                if (P->touches_periodic_lower[d] && i < P->ilower[d])
                    off[d] = -periodic_shift[d];
                else if (P->touches_periodic_upper[d] && i > P->iupper[d])
                    off[d] = +periodic_shift[d];
                else
                    off[d] = 0;
                if (off[d] != k[d] * periodic_shift[d]) ok = false;
            }
            if (!ok) continue;
            if (n < capacity)
            {
                local_indices[n] = s;
                for (int d = 0; d < dim; ++d) periodic_shifts[dim * n + d] = static_cast<double>(off[d]) * P->dx[d];
            }
            ++n;
        }
    }
    return n;
}

int
ibxo_lei_interpolate_idx(double* Q, int Q_depth, const double* X, const int* local_indices,
                         const double* periodic_shifts, int n_idx, const ibxo_patch_data* q, const ibxo_patch* P,
                         int kernel)
{
    const int dim = P->dim;
    if (!valid_kernel(kernel)) return IBXO_E_BAD_KERNEL;
    // LEI:4488-4498: interpolation always requires the minimum ghost width.
    if (min_gcw(q, dim) < ibxo_min_ghost_width(kernel)) return IBXO_E_GHOST_WIDTH;
    if (n_idx == 0) return IBXO_OK;
    if (q->centering == 0)
    {
        if (Q_depth != q->depth) return IBXO_E_DEPTH;
        return ibxo_fortran_interp(kernel, dim, P->dx, P->x_lower, P->x_upper, q->depth, P->ilower, P->iupper, q->gcw,
                                   q->ptr[0], local_indices, periodic_shifts, n_idx, X, Q);
    }
    // LEI:2402-2489: one scalar interpolation per side axis.
    if (Q_depth != dim || q->depth != 1) return IBXO_E_DEPTH;
    const int local_sz = *std::max_element(local_indices, local_indices + n_idx) + 1;
    std::vector<double> Q_axis(local_sz);
    for (int axis = 0; axis < dim; ++axis)
    {
        double xlo[3], xup[3];
        for (int d = 0; d < dim; ++d)
        {
            xlo[d] = P->x_lower[d];
            xup[d] = P->x_upper[d];
        }
        xlo[axis] -= 0.5 * P->dx[axis];
        xup[axis] += 0.5 * P->dx[axis];
        int lo[3], hi[3];
        side_box(P, axis, lo, hi);
        const int rc = ibxo_fortran_interp(kernel, dim, P->dx, xlo, xup, 1, lo, hi, q->gcw, q->ptr[axis],
                                           local_indices, periodic_shifts, n_idx, X, Q_axis.data());
        if (rc) return rc;
        for (int l = 0; l < n_idx; ++l) Q[dim * local_indices[l] + axis] = Q_axis[local_indices[l]];
    }
    return IBXO_OK;
}

int
ibxo_lei_spread_idx(const ibxo_patch_data* q, const double* Q, int Q_depth, const double* X,
                    const int* local_indices, const double* periodic_shifts, int n_idx, const ibxo_patch* P,
                    int kernel)
{
    const int dim = P->dim;
    if (!valid_kernel(kernel)) return IBXO_E_BAD_KERNEL;
    // LEI:5250-5268: spreading checks the ghost width only at a physical boundary.
    if (touches_physical(P) && min_gcw(q, dim) < ibxo_min_ghost_width(kernel)) return IBXO_E_GHOST_WIDTH;
    if (n_idx == 0) return IBXO_OK;
    if (q->centering == 0)
    {
        if (Q_depth != q->depth) return IBXO_E_DEPTH;
        return ibxo_fortran_spread(kernel, dim, P->dx, P->x_lower, P->x_upper, q->depth, local_indices,
                                   periodic_shifts, n_idx, X, Q, P->ilower, P->iupper, q->gcw, q->ptr[0]);
    }
    // LEI:3627-3714: one scalar spread per side axis.
    if (Q_depth != dim || q->depth != 1) return IBXO_E_DEPTH;
    const int local_sz = *std::max_element(local_indices, local_indices + n_idx) + 1;
    std::vector<double> Q_axis(local_sz);
    for (int axis = 0; axis < dim; ++axis)
    {
        double xlo[3], xup[3];
        for (int d = 0; d < dim; ++d)
        {
            xlo[d] = P->x_lower[d];
            xup[d] = P->x_upper[d];
        }
        xlo[axis] -= 0.5 * P->dx[axis];
        xup[axis] += 0.5 * P->dx[axis];
        for (int l = 0; l < n_idx; ++l) Q_axis[local_indices[l]] = Q[dim * local_indices[l] + axis];
        int lo[3], hi[3];
        side_box(P, axis, lo, hi);
        const int rc = ibxo_fortran_spread(kernel, dim, P->dx, xlo, xup, 1, local_indices, periodic_shifts, n_idx, X,
                                           Q_axis.data(), lo, hi, q->gcw, q->ptr[axis]);
        if (rc) return rc;
    }
    return IBXO_OK;
}

int
ibxo_lei_interpolate_raw(double* Q, int Q_depth, const double* X, int n_markers, const ibxo_patch_data* q,
                         const ibxo_patch* P, const int* box_lo, const int* box_hi, int kernel)
{
    std::vector<int> idx(std::max(n_markers, 1));
    const int n = ibxo_build_local_indices(P, box_lo, box_hi, X, n_markers, idx.data());
    std::vector<double> shifts(static_cast<size_t>(P->dim) * std::max(n, 1), 0.0);
    // LEI:4488-4498 checks ghosts before looking at the indices.
    if (!valid_kernel(kernel)) return IBXO_E_BAD_KERNEL;
    if (min_gcw(q, P->dim) < ibxo_min_ghost_width(kernel)) return IBXO_E_GHOST_WIDTH;
    return ibxo_lei_interpolate_idx(Q, Q_depth, X, idx.data(), shifts.data(), n, q, P, kernel);
}

int
ibxo_lei_spread_raw(const ibxo_patch_data* q, const double* Q, int Q_depth, const double* X, int n_markers,
                    const ibxo_patch* P, const int* box_lo, const int* box_hi, int kernel)
{
    std::vector<int> idx(std::max(n_markers, 1));
    const int n = ibxo_build_local_indices(P, box_lo, box_hi, X, n_markers, idx.data());
    std::vector<double> shifts(static_cast<size_t>(P->dim) * std::max(n, 1), 0.0);
    return ibxo_lei_spread_idx(q, Q, Q_depth, X, idx.data(), shifts.data(), n, P, kernel);
}

int
ibxo_accumulate_ghosts_single_patch(const ibxo_patch_data* q, const ibxo_patch* P, const int* domain_lo,
                                    const int* domain_hi, const int* periodic)
{
    const int dim = P->dim;
    const int ncomp = q->centering == 0 ? 1 : dim;
    for (int c = 0; c < ncomp; ++c)
    {
        int lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
        if (q->centering == 0)
            for (int d = 0; d < dim; ++d)
            {
                lo[d] = P->ilower[d];
                hi[d] = P->iupper[d];
            }
        else
            side_box(P, c, lo, hi);
        const ArrayGeom G = make_geom(dim, lo, hi, q->gcw);
        // DOF of a position: periodic dims wrap modulo N (so side face N is
        // face 0); non-periodic positions outside the domain have no DOF.
        auto dof = [&](const int* i, int* out) -> bool {
            for (int d = 0; d < dim; ++d)
            {
                const int dlo = domain_lo[d];
                const int dhi = domain_hi[d] + ((q->centering == 1 && d == c) ? 1 : 0);
                const int N = domain_hi[d] - domain_lo[d] + 1;
                if (periodic[d])
                    out[d] = ((i[d] - dlo) % N + N) % N + dlo;
                else
                {
                    if (i[d] < dlo || i[d] > dhi) return false;
                    out[d] = i[d];
                }
            }
            return true;
        };
        for (int dd = 0; dd < q->depth; ++dd)
        {
            double* u = q->ptr[q->centering == 0 ? 0 : c];
            std::vector<double> sum(G.vol, 0.0);
            std::vector<char> has(G.vol, 0);
            int i[3] = { 0, 0, 0 };
            const int n2 = dim == 3 ? G.n[2] : 1;
            for (int k2 = 0; k2 < n2; ++k2)
                for (int k1 = 0; k1 < G.n[1]; ++k1)
                    for (int k0 = 0; k0 < G.n[0]; ++k0)
                    {
                        i[0] = G.glo[0] + k0;
                        i[1] = G.glo[1] + k1;
                        i[2] = G.glo[2] + k2;
                        int j[3] = { 0, 0, 0 };
                        if (!dof(i, j)) continue;
                        const long long oj = G.off(j, 0);
                        sum[oj] += u[G.off(i, dd)];
                        has[oj] = 1;
                    }
            for (int k2 = 0; k2 < n2; ++k2)
                for (int k1 = 0; k1 < G.n[1]; ++k1)
                    for (int k0 = 0; k0 < G.n[0]; ++k0)
                    {
                        i[0] = G.glo[0] + k0;
                        i[1] = G.glo[1] + k1;
                        i[2] = G.glo[2] + k2;
                        int j[3] = { 0, 0, 0 };
                        if (!dof(i, j)) continue;
                        u[G.off(i, dd)] = sum[G.off(j, 0)];
                    }
        }
    }
    return IBXO_OK;
}

int
ibxo_fill_periodic_ghosts(const ibxo_patch_data* q, const ibxo_patch* P)
{
    const int dim = P->dim;
    const int ncomp = q->centering == 0 ? 1 : dim;
    for (int c = 0; c < ncomp; ++c)
    {
        int lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
        if (q->centering == 0)
            for (int d = 0; d < dim; ++d)
            {
                lo[d] = P->ilower[d];
                hi[d] = P->iupper[d];
            }
        else
            side_box(P, c, lo, hi);
        const ArrayGeom G = make_geom(dim, lo, hi, q->gcw);
        double* u = q->ptr[q->centering == 0 ? 0 : c];
        const int n2 = dim == 3 ? G.n[2] : 1;
        for (int dd = 0; dd < q->depth; ++dd)
            for (int k2 = 0; k2 < n2; ++k2)
                for (int k1 = 0; k1 < G.n[1]; ++k1)
                    for (int k0 = 0; k0 < G.n[0]; ++k0)
                    {
                        int i[3] = { G.glo[0] + k0, G.glo[1] + k1, G.glo[2] + k2 };
                        int j[3] = { i[0], i[1], i[2] };
                        bool moved = false;
                        for (int d = 0; d < dim; ++d)
                        {
                            const int N = P->iupper[d] - P->ilower[d] + 1;
                            const int w = ((i[d] - P->ilower[d]) % N + N) % N + P->ilower[d];
                            if (w != i[d]) moved = true;
                            j[d] = w;
                        }
                        if (moved) u[G.off(i, dd)] = u[G.off(j, dd)];
                    }
    }
    return IBXO_OK;
}

void
ibxo_mt19937_uniform(unsigned seed, int n, double a, double b, double* out)
{
    std::mt19937 gen(seed);
    std::uniform_real_distribution<double> dist(a, b);
    for (int k = 0; k < n; ++k) out[k] = dist(gen);
}

} // extern "C"

// ---------------------------------------------------------------------------
// CPU baseline: the reference's per-patch flow (LDataManager::spread /
// interp, src/IB/LDataManager.cpp:552-811, one LEInteractor call per patch
// and field) over box patches of a periodic domain.  The boxes come from a
// recursive bisection of the domain by marker workload, as a load balancer
// with per-marker workload estimates would cut a level (many boxes per
// thread, the densest regions in the smallest boxes); a pool of threads takes
// the boxes largest first, like ranks each working through their patches.
// Every patch spreads its ghost-box markers (with periodic shifts) into
// zeroed patch data and adds its own faces into the global field, then fills
// the ghosts of its copy of u from the global field and interpolates at its
// interior markers.  The copies between global and patch arrays run row by
// row (contiguous along x, with the periodic wrap resolved per row).
// ---------------------------------------------------------------------------
namespace
{
struct CpuPatch
{
    ibxo_patch P;
    std::vector<int> sp_idx, in_idx;
    std::vector<double> sp_shift, in_shift;
    int lo[3][3], hi[3][3]; // side box per axis (cell box with upper(axis) + 1)
    long long work;         // ghost-box markers + cells / 8: the scheduling order
};

struct CpuPlan
{
    int dim, N[3], kernel, n_markers, gcw, n_threads;
    const double* X;
    std::vector<CpuPatch> patches; // largest work first
    long long max_ghosted;         // largest ghosted side array over patches and axes
};

struct Box
{
    int lo[3], hi[3];
};

// Recursive bisection of `box` into n leaves: the longest side is cut where
// the workload (markers + cells / 8) on the lower side reaches its share;
// no side shorter than min_edge.
void
bisect(const CpuPlan& plan, const Box& box, const std::vector<int>& cell, std::vector<int> members, int n,
       int min_edge, std::vector<Box>& out)
{
    const int dim = plan.dim;
    int ax = 0;
    for (int d = 1; d < dim; ++d)
        if (box.hi[d] - box.lo[d] > box.hi[ax] - box.lo[ax]) ax = d;
    const int len = box.hi[ax] - box.lo[ax] + 1;
    if (n <= 1 || len < 2 * min_edge)
    {
        out.push_back(box);
        return;
    }
    long long cross = 1;
    for (int d = 0; d < dim; ++d)
        if (d != ax) cross *= box.hi[d] - box.lo[d] + 1;
    std::vector<double> w(len, cross / 8.0);
    for (int s : members) w[cell[(size_t)dim * s + ax] - box.lo[ax]] += 1.0;
    double total = 0.0;
    for (double v : w) total += v;
    const int n_lo = n / 2;
    const double target = total * n_lo / n;
    double acc = 0.0;
    int cut = box.lo[ax] + min_edge; // first cell of the upper part
    for (int i = 0; i < len; ++i)
    {
        acc += w[i];
        if (acc >= target)
        {
            cut = box.lo[ax] + i + 1;
            break;
        }
    }
    cut = std::max(cut, box.lo[ax] + min_edge);
    cut = std::min(cut, box.hi[ax] + 1 - min_edge);
    Box a = box, b = box;
    a.hi[ax] = cut - 1;
    b.lo[ax] = cut;
    std::vector<int> ma, mb;
    for (int s : members) (cell[(size_t)dim * s + ax] < cut ? ma : mb).push_back(s);
    members.clear();
    members.shrink_to_fit();
    bisect(plan, a, cell, std::move(ma), n_lo, min_edge, out);
    bisect(plan, b, cell, std::move(mb), n - n_lo, min_edge, out);
}

// Markers whose cell lies in the box grown by g (periodic images along every
// dimension), with the periodic shift rule of LIndexSetData.cpp:83-100 as
// ibxo_cache_local_indices states it.
void
select_markers(const CpuPlan& plan, const ibxo_patch& P, const std::vector<int>& cell, int g, std::vector<int>& idx,
               std::vector<double>& shift)
{
    const int dim = plan.dim;
    idx.clear();
    shift.clear();
    for (int s = 0; s < plan.n_markers; ++s)
    {
        int kk[3][3], nk[3] = { 0, 0, 0 };
        bool any = true;
        for (int d = 0; d < dim && any; ++d)
        {
            const int c = cell[(size_t)dim * s + d];
            for (int k = -1; k <= 1; ++k)
            {
                const int i = c + k * plan.N[d];
                if (i < P.ilower[d] - g || i > P.iupper[d] + g) continue;
                const int off = (P.touches_periodic_lower[d] && i < P.ilower[d])   ? -1
                                : (P.touches_periodic_upper[d] && i > P.iupper[d]) ? 1
                                                                                   : 0;
                if (off == k) kk[d][nk[d]++] = k;
            }
            any = nk[d] > 0;
        }
        if (!any) continue;
        const int nimg = nk[0] * nk[1] * (dim == 3 ? nk[2] : 1);
        for (int m = 0; m < nimg; ++m)
        {
            const int j[3] = { m % nk[0], (m / nk[0]) % nk[1], dim == 3 ? m / (nk[0] * nk[1]) : 0 };
            idx.push_back(s);
            for (int d = 0; d < dim; ++d) shift.push_back(kk[d][j[d]] * plan.N[d] * P.dx[d]);
        }
    }
}

struct CpuScratch
{
    std::vector<double> f_loc[3], u_loc[3];
};

void
cpu_patch_step(const CpuPlan& plan, const CpuPatch& cp, CpuScratch& sc, const double* F, double* f, const double* u,
               double* U)
{
    const int dim = plan.dim;
    const long long n0 = plan.N[0], n01 = (long long)plan.N[0] * plan.N[1];
    const long long vol = n01 * (dim == 3 ? plan.N[2] : 1);
    ibxo_patch_data q;
    q.depth = 1;
    q.centering = 1;
    for (int d = 0; d < 3; ++d) q.gcw[d] = d < dim ? plan.gcw : 0;
    ArrayGeom G[3];
    for (int a = 0; a < dim; ++a)
    {
        G[a] = make_geom(dim, cp.lo[a], cp.hi[a], q.gcw);
        std::fill(sc.f_loc[a].begin(), sc.f_loc[a].begin() + G[a].vol, 0.0);
        q.ptr[a] = sc.f_loc[a].data();
    }
    // Spread into zeroed patch data, then add the patch's own faces into f
    // (cells ilower..iupper along every axis: face iupper + 1 of a side axis
    // belongs to the next patch).
    ibxo_lei_spread_idx(&q, F, dim, plan.X, cp.sp_idx.data(), cp.sp_shift.data(), (int)cp.sp_idx.size(), &cp.P,
                        plan.kernel);
    const int z0 = dim == 3 ? cp.P.ilower[2] : 0, z1 = dim == 3 ? cp.P.iupper[2] : 0;
    const int x0 = cp.P.ilower[0], nx = cp.P.iupper[0] - x0 + 1;
    for (int a = 0; a < dim; ++a)
        for (int z = z0; z <= z1; ++z)
            for (int y = cp.P.ilower[1]; y <= cp.P.iupper[1]; ++y)
            {
                const int i[3] = { x0, y, z };
                const double* src = sc.f_loc[a].data() + G[a].off(i, 0);
                double* dst = f + vol * a + z * n01 + y * n0 + x0;
                for (int k = 0; k < nx; ++k) dst[k] += src[k];
            }
    // Ghost fill of u (periodic copy of the global field) row by row, then
    // interpolation at the interior markers.
    for (int a = 0; a < dim; ++a)
    {
        const ArrayGeom& g = G[a];
        const int n2 = dim == 3 ? g.n[2] : 1;
        for (int k2 = 0; k2 < n2; ++k2)
        {
            int jz = dim == 3 ? g.glo[2] + k2 : 0;
            if (dim == 3) jz = ((jz % plan.N[2]) + plan.N[2]) % plan.N[2];
            for (int k1 = 0; k1 < g.n[1]; ++k1)
            {
                const int jy = (((g.glo[1] + k1) % plan.N[1]) + plan.N[1]) % plan.N[1];
                const double* row = u + vol * a + jz * n01 + jy * n0;
                double* dst = sc.u_loc[a].data() + ((long long)k2 * g.n[1] + k1) * g.n[0];
                int jx = ((g.glo[0] % plan.N[0]) + plan.N[0]) % plan.N[0];
                for (int k0 = 0; k0 < g.n[0]; ++k0)
                {
                    dst[k0] = row[jx];
                    if (++jx == plan.N[0]) jx = 0;
                }
            }
        }
        q.ptr[a] = sc.u_loc[a].data();
    }
    ibxo_lei_interpolate_idx(U, dim, plan.X, cp.in_idx.data(), cp.in_shift.data(), (int)cp.in_idx.size(), &q, &cp.P,
                             plan.kernel);
}
} // namespace

extern "C" {

void*
ibxo_cpu_plan_create(int dim, const int* N, int kernel, int n_markers, const double* X, int n_threads, int n_boxes)
{
    if ((dim != 2 && dim != 3) || !valid_kernel(kernel) || n_threads < 1 || n_boxes < 1) return nullptr;
    CpuPlan* plan = new CpuPlan;
    plan->dim = dim;
    plan->kernel = kernel;
    plan->n_markers = n_markers;
    plan->n_threads = n_threads;
    plan->X = X;
    plan->gcw = ibxo_min_ghost_width(kernel);
    for (int d = 0; d < 3; ++d) plan->N[d] = d < dim ? N[d] : 1;
    // Cell of every marker on the domain (getCellIndex, unit domain).
    double xl[3] = { 0, 0, 0 }, xu[3] = { 1, 1, 1 }, dx[3] = { 1, 1, 1 };
    int il[3] = { 0, 0, 0 }, iu[3] = { 0, 0, 0 };
    for (int d = 0; d < dim; ++d)
    {
        dx[d] = 1.0 / plan->N[d];
        iu[d] = plan->N[d] - 1;
    }
    std::vector<int> cell((size_t)dim * n_markers);
    for (int s = 0; s < n_markers; ++s)
    {
        int c[3];
        ibxo_get_cell_index(dim, &X[(size_t)dim * s], xl, xu, dx, il, iu, c);
        for (int d = 0; d < dim; ++d) cell[(size_t)dim * s + d] = ((c[d] % plan->N[d]) + plan->N[d]) % plan->N[d];
    }
    Box dom;
    for (int d = 0; d < 3; ++d)
    {
        dom.lo[d] = 0;
        dom.hi[d] = plan->N[d] - 1;
    }
    std::vector<int> all(n_markers);
    for (int s = 0; s < n_markers; ++s) all[s] = s;
    std::vector<Box> boxes;
    bisect(*plan, dom, cell, std::move(all), n_boxes, std::max(4, plan->gcw), boxes);
    plan->patches.resize(boxes.size());
    auto build_patch = [plan, dim, &boxes, &cell](size_t p) {
        CpuPatch& cp = plan->patches[p];
        ibxo_patch& P = cp.P;
        std::memset(&P, 0, sizeof(P));
        P.dim = dim;
        for (int d = 0; d < dim; ++d)
        {
            P.dx[d] = 1.0 / plan->N[d];
            P.ilower[d] = boxes[p].lo[d];
            P.iupper[d] = boxes[p].hi[d];
            P.x_lower[d] = P.ilower[d] * P.dx[d];
            P.x_upper[d] = (P.iupper[d] + 1) * P.dx[d];
            P.touches_periodic_lower[d] = P.ilower[d] == 0;
            P.touches_periodic_upper[d] = P.iupper[d] == plan->N[d] - 1;
        }
        select_markers(*plan, P, cell, plan->gcw, cp.sp_idx, cp.sp_shift);
        select_markers(*plan, P, cell, 0, cp.in_idx, cp.in_shift);
        long long cells = 1;
        for (int a = 0; a < dim; ++a)
            for (int d = 0; d < dim; ++d)
            {
                cp.lo[a][d] = P.ilower[d];
                cp.hi[a][d] = P.iupper[d] + (d == a ? 1 : 0);
            }
        for (int d = 0; d < dim; ++d) cells *= P.iupper[d] - P.ilower[d] + 1;
        cp.work = (long long)cp.sp_idx.size() + cells / 8;
    };
    // Patches are independent: build their index sets concurrently.
    {
        std::atomic<size_t> next(0);
        auto worker = [&]() {
            for (size_t p = next++; p < boxes.size(); p = next++) build_patch(p);
        };
        std::vector<std::thread> threads;
        for (int t = 1; t < n_threads; ++t) threads.emplace_back(worker);
        worker();
        for (auto& t : threads) t.join();
    }
    std::sort(plan->patches.begin(), plan->patches.end(),
              [](const CpuPatch& a, const CpuPatch& b) { return a.work > b.work; });
    plan->max_ghosted = 0;
    for (const CpuPatch& cp : plan->patches)
        for (int a = 0; a < dim; ++a)
        {
            long long v = 1;
            for (int d = 0; d < dim; ++d) v *= cp.hi[a][d] - cp.lo[a][d] + 1 + 2 * plan->gcw;
            plan->max_ghosted = std::max(plan->max_ghosted, v);
        }
    return plan;
}

int
ibxo_cpu_plan_step(void* handle, const double* F, double* f, const double* u, double* U)
{
    CpuPlan* plan = static_cast<CpuPlan*>(handle);
    if (!plan) return IBXO_E_ARG;
    std::atomic<size_t> next(0);
    auto worker = [&]() {
        CpuScratch sc;
        for (int a = 0; a < plan->dim; ++a)
        {
            sc.f_loc[a].resize(plan->max_ghosted);
            sc.u_loc[a].resize(plan->max_ghosted);
        }
        for (size_t p = next++; p < plan->patches.size(); p = next++)
            cpu_patch_step(*plan, plan->patches[p], sc, F, f, u, U);
    };
    std::vector<std::thread> threads;
    for (int t = 1; t < plan->n_threads; ++t) threads.emplace_back(worker);
    worker();
    for (auto& t : threads) t.join();
    return IBXO_OK;
}

int
ibxo_cpu_plan_patches(void* handle)
{
    CpuPlan* plan = static_cast<CpuPlan*>(handle);
    return plan ? (int)plan->patches.size() : -1;
}

void
ibxo_cpu_plan_destroy(void* handle)
{
    delete static_cast<CpuPlan*>(handle);
}

} // extern "C"
