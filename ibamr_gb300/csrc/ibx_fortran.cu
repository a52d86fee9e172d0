// ibx_fortran.cu -- the Fortran-ABI entry points of include/ibx_fortran.h:
// IBAMR's lagrangian_<kernel>_{interp,spread}{2d,3d} routines (called from
// ibtk/src/lagrangian/LEInteractor.cpp:4470-6006) run on the GPU through the
// patch-mode FP64 path of ibx_interpolate / ibx_spread.

#include "ibx_internal.h"
#include "../../include/ibx.h"
#include "../../include/ibx_fortran.h"

#include <cstdio>
#include <cstdlib>
#include <vector>

namespace
{
[[noreturn]] void
die(const char* routine, const char* what)
{
    std::fprintf(stderr, "libibx: %s: %s\n", routine, what);
    std::abort();
}

bool
on_device(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError(); // plain host memory on older runtimes
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A caller array made available on the device: used in place when it is
// device memory, else copied into a buffer of the library's staging pool
// (and back on request).
struct Staged
{
    void* host = nullptr;
    void* dev = nullptr;
    size_t bytes = 0;
    bool owned = false;

    void
    stage(const char* routine, const void* p, size_t n, bool copy_in)
    {
        host = const_cast<void*>(p);
        bytes = n;
        if (!p || n == 0) return;
        if (on_device(p))
        {
            dev = host;
            return;
        }
        dev = ibx::staging_alloc(n);
        if (!dev) die(routine, "device allocation failed");
        owned = true;
        if (copy_in && cudaMemcpy(dev, p, n, cudaMemcpyHostToDevice) != cudaSuccess) die(routine, "copy to the device failed");
    }
    void
    copy_out(const char* routine)
    {
        if (owned && cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            die(routine, "copy from the device failed");
    }
    ~Staged()
    {
        if (owned) ibx::staging_free(dev);
    }
};

// One Fortran-routine call: marker values V(depth, *), positions X(dim, *),
// the markers indices[0..nind) shifted by Xshift(dim, l), the ghosted patch
// array u of cell box [ilo, ihi] with ghost width gcw.
void
run(const char* routine, bool spread, int dim, int kernel, const double* dx, const double* x_lower,
    const double* x_upper, int depth, const int* ilo, const int* ihi, const int* gcw, const double* u,
    const int* indices, const double* Xshift, int nind, const double* X, const double* V)
{
    if (nind <= 0) return;
    // The marker arrays hold at least max(indices) + 1 markers.
    std::vector<int> idx(nind);
    if (on_device(indices))
    {
        if (cudaMemcpy(idx.data(), indices, sizeof(int) * nind, cudaMemcpyDeviceToHost) != cudaSuccess)
            die(routine, "copy of the indices failed");
    }
    else
        for (int l = 0; l < nind; ++l) idx[l] = indices[l];
    int nm = 0;
    for (int l = 0; l < nind; ++l)
    {
        if (idx[l] < 0) die(routine, "negative marker index");
        nm = idx[l] + 1 > nm ? idx[l] + 1 : nm;
    }
    size_t vol = 1;
    for (int d = 0; d < dim; ++d) vol *= (size_t)(ihi[d] - ilo[d] + 1 + 2 * gcw[d]);
    Staged su, sx, sv, si, ss;
    su.stage(routine, u, sizeof(double) * vol * depth, true);
    sx.stage(routine, X, sizeof(double) * dim * (size_t)nm, true);
    sv.stage(routine, V, sizeof(double) * depth * (size_t)nm, true);
    si.stage(routine, indices, sizeof(int) * nind, true);
    ss.stage(routine, Xshift, sizeof(double) * dim * (size_t)nind, true);

    ibx_problem p{};
    p.dim = dim;
    p.centering = IBX_CELL;
    p.mode = IBX_MODE_PATCH;
    for (int d = 0; d < dim; ++d)
    {
        p.ilower[d] = ilo[d];
        p.iupper[d] = ihi[d];
        p.gcw[d] = gcw[d];
        p.dx[d] = dx[d];
        p.x_lower[d] = x_lower[d];
        p.x_upper[d] = x_upper[d];
    }
    p.q_depth = depth;
    p.q[0] = su.dev;
    p.X = static_cast<const double*>(sx.dev);
    p.Q = sv.dev;
    p.Q_depth = depth;
    p.n_markers = nm;
    p.indices = static_cast<const int*>(si.dev);
    p.n_indices = nind;
    p.Xshift = static_cast<const double*>(ss.dev);
    const int rc = spread ? ibx_spread(&p, 1, kernel, IBX_PRECISION_FP64, nullptr)
                          : ibx_interpolate(&p, 1, kernel, IBX_PRECISION_FP64, nullptr);
    if (rc != IBX_OK) die(routine, ibx_status_string(rc));
    if (cudaDeviceSynchronize() != cudaSuccess) die(routine, "device execution failed");
    if (spread)
        su.copy_out(routine);
    else
        sv.copy_out(routine);
}
} // namespace

#define IBX_DEFINE_FORTRAN(KNAME, KID)                                                                               \
    IBX_FORTRAN_INTERP2D(lagrangian_##KNAME##_interp2d_)                                                             \
    {                                                                                                                \
        const int lo[2] = { *ilower0, *ilower1 }, hi[2] = { *iupper0, *iupper1 }, g[2] = { *nugc0, *nugc1 };         \
        run("lagrangian_" #KNAME "_interp2d", false, 2, KID, dx, x_lower, x_upper, *depth, lo, hi, g, u, indices,    \
            Xshift, *nindices, X, V);                                                                                \
    }                                                                                                                \
    IBX_FORTRAN_SPREAD2D(lagrangian_##KNAME##_spread2d_)                                                             \
    {                                                                                                                \
        const int lo[2] = { *ilower0, *ilower1 }, hi[2] = { *iupper0, *iupper1 }, g[2] = { *nugc0, *nugc1 };         \
        run("lagrangian_" #KNAME "_spread2d", true, 2, KID, dx, x_lower, x_upper, *depth, lo, hi, g, u, indices,     \
            Xshift, *nindices, X, V);                                                                                \
    }                                                                                                                \
    IBX_FORTRAN_INTERP3D(lagrangian_##KNAME##_interp3d_)                                                             \
    {                                                                                                                \
        const int lo[3] = { *ilower0, *ilower1, *ilower2 }, hi[3] = { *iupper0, *iupper1, *iupper2 },                \
                  g[3] = { *nugc0, *nugc1, *nugc2 };                                                                 \
        run("lagrangian_" #KNAME "_interp3d", false, 3, KID, dx, x_lower, x_upper, *depth, lo, hi, g, u, indices,    \
            Xshift, *nindices, X, V);                                                                                \
    }                                                                                                                \
    IBX_FORTRAN_SPREAD3D(lagrangian_##KNAME##_spread3d_)                                                             \
    {                                                                                                                \
        const int lo[3] = { *ilower0, *ilower1, *ilower2 }, hi[3] = { *iupper0, *iupper1, *iupper2 },                \
                  g[3] = { *nugc0, *nugc1, *nugc2 };                                                                 \
        run("lagrangian_" #KNAME "_spread3d", true, 3, KID, dx, x_lower, x_upper, *depth, lo, hi, g, u, indices,     \
            Xshift, *nindices, X, V);                                                                                \
    }

extern "C" {
IBX_DEFINE_FORTRAN(piecewise_linear, IBX_KERNEL_PIECEWISE_LINEAR)
IBX_DEFINE_FORTRAN(piecewise_cubic, IBX_KERNEL_PIECEWISE_CUBIC)
IBX_DEFINE_FORTRAN(ib_3, IBX_KERNEL_IB_3)
IBX_DEFINE_FORTRAN(ib_4, IBX_KERNEL_IB_4)
IBX_DEFINE_FORTRAN(ib_6, IBX_KERNEL_IB_6)
IBX_DEFINE_FORTRAN(bspline_4, IBX_KERNEL_BSPLINE_4)
}
