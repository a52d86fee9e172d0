/*
 * ibx_fortran.h -- the Fortran-ABI entry points of IBAMR's interaction
 * routines, implemented by libibx on the GPU.
 *
 * IBAMR's LEInteractor calls lagrangian_<kernel>_{interp,spread}{2d,3d}
 * through IBTK_FC_FUNC_ (ibtk/src/lagrangian/LEInteractor.cpp:59-235; the
 * argument lists are declared at LEInteractor.cpp:237-1516 and the calls made
 * at LEInteractor.cpp:4470-6006).  libibx exports the same names with the
 * gfortran convention (lower case, trailing underscore) and the same argument
 * order, every argument passed by reference, so that LEInteractor.cpp links
 * against libibx unchanged for the six kernels below.
 *
 *   interp: dx, x_lower, x_upper, depth, ilower0, iupper0, ilower1, iupper1,
 *           [ilower2, iupper2,] nugc0, nugc1, [nugc2,] u, indices, Xshift,
 *           nindices, X, V
 *   spread: dx, x_lower, x_upper, depth, indices, Xshift, nindices, X, V,
 *           ilower0, iupper0, ilower1, iupper1, [ilower2, iupper2,] nugc0,
 *           nugc1, [nugc2,] u
 *
 * u is the ghosted patch array (Fortran order, depth slowest), X the marker
 * positions X(NDIM, *), V the marker values V(depth, *); only the markers
 * listed in indices (shifted by Xshift(NDIM, l)) take part.  Interpolation
 * overwrites V(:, indices(l)); spreading adds into u.  Stencils are clipped to
 * the ghost box as in the Fortran routines; no ghost-width check is made here
 * (LEInteractor makes it before calling).
 *
 * Arrays may be host or device memory (the CUDA pointer attributes decide);
 * host arrays are copied to the device and the results copied back, so the
 * call returns with its results in place (synchronous).  The arithmetic is
 * the plain FP64 form.  A failure of the CUDA runtime aborts the process with
 * a message on stderr, as the reference's TBOX_ERROR would.
 */
#ifndef IBX_FORTRAN_H
#define IBX_FORTRAN_H

#ifdef __cplusplus
extern "C" {
#endif

#define IBX_FORTRAN_INTERP2D(name)                                                                                 \
    void name(const double* dx, const double* x_lower, const double* x_upper, const int* depth,                   \
              const int* ilower0, const int* iupper0, const int* ilower1, const int* iupper1, const int* nugc0,   \
              const int* nugc1, const double* u, const int* indices, const double* Xshift, const int* nindices,   \
              const double* X, double* V)
#define IBX_FORTRAN_INTERP3D(name)                                                                                 \
    void name(const double* dx, const double* x_lower, const double* x_upper, const int* depth,                   \
              const int* ilower0, const int* iupper0, const int* ilower1, const int* iupper1, const int* ilower2, \
              const int* iupper2, const int* nugc0, const int* nugc1, const int* nugc2, const double* u,          \
              const int* indices, const double* Xshift, const int* nindices, const double* X, double* V)
#define IBX_FORTRAN_SPREAD2D(name)                                                                                 \
    void name(const double* dx, const double* x_lower, const double* x_upper, const int* depth,                   \
              const int* indices, const double* Xshift, const int* nindices, const double* X, const double* V,    \
              const int* ilower0, const int* iupper0, const int* ilower1, const int* iupper1, const int* nugc0,   \
              const int* nugc1, double* u)
#define IBX_FORTRAN_SPREAD3D(name)                                                                                 \
    void name(const double* dx, const double* x_lower, const double* x_upper, const int* depth,                   \
              const int* indices, const double* Xshift, const int* nindices, const double* X, const double* V,    \
              const int* ilower0, const int* iupper0, const int* ilower1, const int* iupper1, const int* ilower2, \
              const int* iupper2, const int* nugc0, const int* nugc1, const int* nugc2, double* u)

/* PIECEWISE_LINEAR (lagrangian_interaction2d.f.m4:469-700, 3d:493-738) */
IBX_FORTRAN_INTERP2D(lagrangian_piecewise_linear_interp2d_);
IBX_FORTRAN_SPREAD2D(lagrangian_piecewise_linear_spread2d_);
IBX_FORTRAN_INTERP3D(lagrangian_piecewise_linear_interp3d_);
IBX_FORTRAN_SPREAD3D(lagrangian_piecewise_linear_spread3d_);
/* PIECEWISE_CUBIC (2d:703-931, 3d:739-975) */
IBX_FORTRAN_INTERP2D(lagrangian_piecewise_cubic_interp2d_);
IBX_FORTRAN_SPREAD2D(lagrangian_piecewise_cubic_spread2d_);
IBX_FORTRAN_INTERP3D(lagrangian_piecewise_cubic_interp3d_);
IBX_FORTRAN_SPREAD3D(lagrangian_piecewise_cubic_spread3d_);
/* IB_3 (2d:933-1150, 3d:976-1201) */
IBX_FORTRAN_INTERP2D(lagrangian_ib_3_interp2d_);
IBX_FORTRAN_SPREAD2D(lagrangian_ib_3_spread2d_);
IBX_FORTRAN_INTERP3D(lagrangian_ib_3_interp3d_);
IBX_FORTRAN_SPREAD3D(lagrangian_ib_3_spread3d_);
/* IB_4 (2d:1152-1391, 3d:1203-1484) */
IBX_FORTRAN_INTERP2D(lagrangian_ib_4_interp2d_);
IBX_FORTRAN_SPREAD2D(lagrangian_ib_4_spread2d_);
IBX_FORTRAN_INTERP3D(lagrangian_ib_4_interp3d_);
IBX_FORTRAN_SPREAD3D(lagrangian_ib_4_spread3d_);
/* IB_6 (2d:1971-2299, 3d:2178-2590) */
IBX_FORTRAN_INTERP2D(lagrangian_ib_6_interp2d_);
IBX_FORTRAN_SPREAD2D(lagrangian_ib_6_spread2d_);
IBX_FORTRAN_INTERP3D(lagrangian_ib_6_interp3d_);
IBX_FORTRAN_SPREAD3D(lagrangian_ib_6_spread3d_);
/* BSPLINE_4 (2d:2519-2746, 3d:2814-3049) */
IBX_FORTRAN_INTERP2D(lagrangian_bspline_4_interp2d_);
IBX_FORTRAN_SPREAD2D(lagrangian_bspline_4_spread2d_);
IBX_FORTRAN_INTERP3D(lagrangian_bspline_4_interp3d_);
IBX_FORTRAN_SPREAD3D(lagrangian_bspline_4_spread3d_);

#ifdef __cplusplus
}
#endif

#endif /* IBX_FORTRAN_H */
