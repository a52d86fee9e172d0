/*
 * ibx_leinteractor.h -- C++ host layer of libibx with the call signatures of
 * IBAMR's IBTK::LEInteractor (ibtk/include/ibtk/LEInteractor.h), over
 * minimal stand-ins for the SAMRAI types those signatures use.
 *
 * Header-only, so it compiles with the caller's NDIM (2 or 3) as IBAMR's
 * own 2D and 3D libraries do.  Each call selects the markers the way the
 * reference does (getCellIndex in the given box, LEInteractor.cpp:6088-6126),
 * moves host arrays to the GPU when needed, and calls the C ABI of
 * include/ibx.h (plain FP64 form).  Errors the reference
 * reports with TBOX_ERROR (unknown kernel, depth mismatch, insufficient
 * ghost width) are thrown as std::runtime_error with the reference's text.
 *
 * Patch data may live on the host (copied in and out per call) or on the
 * device (used in place); marker arrays are host arrays as in the reference.
 */
#ifndef IBX_LEINTERACTOR_H
#define IBX_LEINTERACTOR_H

#include "ibx.h"

#include <array>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#ifndef NDIM
#define NDIM 3
#endif

namespace ibx
{
namespace samrai
{
// hier::IntVector<NDIM> / hier::Index<NDIM>
struct IntVector
{
    std::array<int, NDIM> v{};
    IntVector() = default;
    explicit IntVector(int a)
    {
        v.fill(a);
    }
    int& operator()(int d)
    {
        return v[d];
    }
    int operator()(int d) const
    {
        return v[d];
    }
    int min() const
    {
        int m = v[0];
        for (int d = 1; d < NDIM; ++d) m = v[d] < m ? v[d] : m;
        return m;
    }
};
using Index = IntVector;

// hier::Box<NDIM>
struct Box
{
    Index lo, hi;
    Box() = default;
    Box(const Index& l, const Index& h) : lo(l), hi(h)
    {
    }
    const Index& lower() const
    {
        return lo;
    }
    const Index& upper() const
    {
        return hi;
    }
    bool contains(const Index& i) const
    {
        for (int d = 0; d < NDIM; ++d)
            if (i(d) < lo(d) || i(d) > hi(d)) return false;
        return true;
    }
};

// geom::CartesianPatchGeometry<NDIM>
struct CartesianPatchGeometry
{
    std::array<double, NDIM> x_lower{}, x_upper{}, dx{};
    std::array<std::array<int, 2>, NDIM> touches_regular{};
    std::array<std::array<int, 2>, NDIM> touches_periodic{};
    const double* getXLower() const
    {
        return x_lower.data();
    }
    const double* getXUpper() const
    {
        return x_upper.data();
    }
    const double* getDx() const
    {
        return dx.data();
    }
    bool getTouchesRegularBoundary(int axis, int side) const
    {
        return touches_regular[axis][side] != 0;
    }
    bool getTouchesPeriodicBoundary(int axis, int side) const
    {
        return touches_periodic[axis][side] != 0;
    }
};

// hier::Patch<NDIM>
struct Patch
{
    Box box;
    CartesianPatchGeometry geom;
    const Box& getBox() const
    {
        return box;
    }
    const CartesianPatchGeometry& getPatchGeometry() const
    {
        return geom;
    }
};

// pdat::CellData<NDIM,double> / pdat::SideData<NDIM,double>: SAMRAI layout
// (ghosts included, Fortran order, depth slowest); side data holds one array
// per axis on toSideBox(box, axis).
struct CellData
{
    Box box;
    IntVector gcw;
    int depth = 1;
    double* data = nullptr;
    bool on_device = false;
    const Box& getBox() const
    {
        return box;
    }
    const IntVector& getGhostCellWidth() const
    {
        return gcw;
    }
    int getDepth() const
    {
        return depth;
    }
    double* getPointer(int d = 0) const
    {
        long long vol = 1;
        for (int k = 0; k < NDIM; ++k) vol *= box.hi(k) - box.lo(k) + 1 + 2 * gcw(k);
        return data + vol * d;
    }
};

struct SideData
{
    Box box;
    IntVector gcw;
    int depth = 1;
    std::array<double*, NDIM> data{};
    bool on_device = false;
    const Box& getBox() const
    {
        return box;
    }
    const IntVector& getGhostCellWidth() const
    {
        return gcw;
    }
    int getDepth() const
    {
        return depth;
    }
    double* getPointer(int axis) const
    {
        return data[axis];
    }
};
} // namespace samrai
} // namespace ibx

namespace IBTK
{
namespace ibx_detail
{
using namespace ibx::samrai;

inline int
kernel_id(const std::string& fcn)
{
    const int k = ibx_kernel_from_name(fcn.c_str());
    if (k < 0) throw std::runtime_error("Unknown kernel function " + fcn);
    return k;
}

inline void
check(int rc, const std::string& where)
{
    if (rc != IBX_OK) throw std::runtime_error(where + ": " + ibx_status_string(rc));
}

// Owning device buffer.
struct DeviceBuffer
{
    void* p = nullptr;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer()
    {
        if (p) ibx_device_free(p);
    }
    void* upload(const void* host, long long bytes)
    {
        check(ibx_device_alloc(&p, bytes), "libibx device allocation");
        if (host) check(ibx_memcpy(p, host, bytes, 1), "libibx copy to device");
        return p;
    }
};

// IndexUtilities::getCellIndex (IndexUtilities-inl.h:52-75).
inline Index
getCellIndex(const double* X, const CartesianPatchGeometry& g, const Box& patch_box)
{
    Index idx;
    for (int d = 0; d < NDIM; ++d)
    {
        const double dX_lower = X[d] - g.x_lower[d], dX_upper = X[d] - g.x_upper[d];
        if (std::abs(dX_lower) <= std::abs(dX_upper))
            idx(d) = static_cast<int>(patch_box.lo(d) + std::floor(dX_lower / g.dx[d]));
        else
            idx(d) = static_cast<int>(patch_box.hi(d) + std::floor(dX_upper / g.dx[d]) + 1);
    }
    return idx;
}

// Values of one SAMRAI array (axis < 0: cell data, else side axis).
inline long long
array_values(const Box& box, const IntVector& gcw, int axis)
{
    long long n = 1;
    for (int d = 0; d < NDIM; ++d) n *= box.hi(d) - box.lo(d) + 1 + 2 * gcw(d) + (d == axis ? 1 : 0);
    return n;
}

inline ibx_problem
make_problem(const Patch& patch, const Box& data_box, const IntVector& gcw, int centering)
{
    ibx_problem p{};
    p.dim = NDIM;
    p.centering = centering;
    p.mode = IBX_MODE_PATCH;
    const CartesianPatchGeometry& g = patch.getPatchGeometry();
    for (int d = 0; d < NDIM; ++d)
    {
        p.ilower[d] = data_box.lo(d);
        p.iupper[d] = data_box.hi(d);
        p.gcw[d] = gcw(d);
        p.dx[d] = g.dx[d];
        p.x_lower[d] = g.x_lower[d];
        p.x_upper[d] = g.x_upper[d];
        p.touches_physical_lower[d] = g.getTouchesRegularBoundary(d, 0);
        p.touches_physical_upper[d] = g.getTouchesRegularBoundary(d, 1);
    }
    return p;
}

// Marker data and index list on the device, patch data on the device (copied
// for host-resident patch data), one ibx call, results copied back.
template <class Data>
inline void
run(bool spread, Data& q, int centering, int q_depth, const Patch& patch, double* Q, int Q_values, int Q_depth,
    const double* X, int n_markers, const std::vector<int>& idx, const std::vector<double>* shifts, int kernel,
    const std::string& where)
{
    ibx_problem p = make_problem(patch, q.getBox(), q.getGhostCellWidth(), centering);
    p.q_depth = q_depth;
    p.Q_depth = Q_depth;
    p.n_markers = n_markers;
    DeviceBuffer dX, dQ, dIdx, dShift;
    DeviceBuffer dq[NDIM];
    const int ncomp = centering == IBX_SIDE ? NDIM : 1;
    for (int c = 0; c < ncomp; ++c)
    {
        double* ptr = centering == IBX_SIDE ? q.getPointer(c) : q.getPointer(0);
        const long long n = array_values(q.getBox(), q.getGhostCellWidth(), centering == IBX_SIDE ? c : -1) *
                            (centering == IBX_SIDE ? 1 : q_depth);
        p.q[c] = q.on_device ? static_cast<void*>(ptr) : dq[c].upload(ptr, n * (long long)sizeof(double));
    }
    p.X = static_cast<const double*>(dX.upload(X, (long long)sizeof(double) * NDIM * n_markers));
    p.Q = dQ.upload(Q, (long long)sizeof(double) * Q_values);
    p.indices = static_cast<const int*>(dIdx.upload(idx.data(), (long long)sizeof(int) * idx.size()));
    p.n_indices = static_cast<int>(idx.size());
    if (shifts && !shifts->empty())
        p.Xshift = static_cast<const double*>(dShift.upload(shifts->data(), (long long)sizeof(double) * shifts->size()));
    const int rc = spread ? ibx_spread(&p, 1, kernel, IBX_PRECISION_FP64, nullptr)
                          : ibx_interpolate(&p, 1, kernel, IBX_PRECISION_FP64, nullptr);
    if (rc == IBX_E_GHOST_WIDTH)
        throw std::runtime_error(where + (spread ? ": insufficient ghost cells at physical boundary"
                                                 : ": insufficient ghost cells"));
    check(rc, where);
    check(ibx_synchronize(), where);
    if (spread && !q.on_device)
        for (int c = 0; c < ncomp; ++c)
        {
            double* ptr = centering == IBX_SIDE ? q.getPointer(c) : q.getPointer(0);
            const long long n = array_values(q.getBox(), q.getGhostCellWidth(), centering == IBX_SIDE ? c : -1) *
                                (centering == IBX_SIDE ? 1 : q_depth);
            check(ibx_memcpy(ptr, p.q[c], n * (long long)sizeof(double), 0), where);
        }
    if (!spread) check(ibx_memcpy(Q, p.Q, (long long)sizeof(double) * Q_values, 0), where);
}

inline void
ghost_check(const IntVector& gcw, const std::string& fcn, const std::string& where)
{
    const int need = ibx_get_minimum_ghost_width(kernel_id(fcn));
    if (gcw.min() < need) throw std::runtime_error(where + ": insufficient ghost cells");
}
} // namespace ibx_detail

class LEInteractor
{
public:
    using Box = ibx::samrai::Box;
    using Patch = ibx::samrai::Patch;
    using CellData = ibx::samrai::CellData;
    using SideData = ibx::samrai::SideData;

    LEInteractor() = delete;

    static bool isKnownKernel(const std::string& kernel_fcn)
    {
        return ibx_kernel_from_name(kernel_fcn.c_str()) >= 0;
    }
    static int getStencilSize(const std::string& kernel_fcn)
    {
        return ibx_get_stencil_size(ibx_detail::kernel_id(kernel_fcn));
    }
    static int getMinimumGhostWidth(const std::string& kernel_fcn)
    {
        return ibx_get_minimum_ghost_width(ibx_detail::kernel_id(kernel_fcn));
    }

    // LEInteractor::buildLocalIndices, raw-array form (LEInteractor.cpp:6088-6126).
    static std::vector<int> buildLocalIndices(const Box& box, const Patch& patch, const double* X_data, int X_size,
                                              int X_depth)
    {
        std::vector<int> idx;
        const int n = X_size / X_depth;
        for (int k = 0; k < n; ++k)
            if (box.contains(ibx_detail::getCellIndex(&X_data[NDIM * k], patch.getPatchGeometry(), patch.getBox())))
                idx.push_back(k);
        return idx;
    }

    // Raw marker arrays (LEInteractor.h:487-628; LEInteractor.cpp:2804-2862).
    static void interpolate(double* Q_data, int Q_size, int Q_depth, const double* X_data, int X_size, int X_depth,
                            const CellData& q_data, const Patch& patch, const Box& interp_box,
                            const std::string& interp_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::interpolate()";
        const int k = ibx_detail::kernel_id(interp_fcn);
        ibx_detail::ghost_check(q_data.getGhostCellWidth(), interp_fcn, where);
        if (Q_depth != q_data.getDepth()) throw std::runtime_error(where + ": Q_depth != q_data depth");
        const std::vector<int> idx = buildLocalIndices(interp_box, patch, X_data, X_size, X_depth);
        if (idx.empty()) return;
        CellData q = q_data;
        ibx_detail::run(false, q, IBX_CELL, q_data.getDepth(), patch, Q_data, Q_size, Q_depth, X_data,
                        X_size / X_depth, idx, nullptr, k, where);
    }
    // LEInteractor.cpp:3044-3127.
    static void interpolate(double* Q_data, int Q_size, int Q_depth, const double* X_data, int X_size, int X_depth,
                            const SideData& q_data, const Patch& patch, const Box& interp_box,
                            const std::string& interp_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::interpolate()";
        if (Q_depth != NDIM || q_data.getDepth() != 1)
            throw std::runtime_error(where + ":\n  side-centered interpolation requires vector-valued data.\n");
        const int k = ibx_detail::kernel_id(interp_fcn);
        ibx_detail::ghost_check(q_data.getGhostCellWidth(), interp_fcn, where);
        const std::vector<int> idx = buildLocalIndices(interp_box, patch, X_data, X_size, X_depth);
        if (idx.empty()) return;
        SideData q = q_data;
        ibx_detail::run(false, q, IBX_SIDE, 1, patch, Q_data, Q_size, Q_depth, X_data, X_size / X_depth, idx,
                        nullptr, k, where);
    }
    // std::vector forms (LEInteractor.h:342-470).
    static void interpolate(std::vector<double>& Q_data, int Q_depth, const std::vector<double>& X_data, int X_depth,
                            const CellData& q_data, const Patch& patch, const Box& interp_box,
                            const std::string& interp_fcn = "IB_4")
    {
        interpolate(Q_data.data(), static_cast<int>(Q_data.size()), Q_depth, X_data.data(),
                    static_cast<int>(X_data.size()), X_depth, q_data, patch, interp_box, interp_fcn);
    }
    static void interpolate(std::vector<double>& Q_data, int Q_depth, const std::vector<double>& X_data, int X_depth,
                            const SideData& q_data, const Patch& patch, const Box& interp_box,
                            const std::string& interp_fcn = "IB_4")
    {
        interpolate(Q_data.data(), static_cast<int>(Q_data.size()), Q_depth, X_data.data(),
                    static_cast<int>(X_data.size()), X_depth, q_data, patch, interp_box, interp_fcn);
    }

    // Raw marker arrays (LEInteractor.h:880-1200; LEInteractor.cpp:3950-4008).
    static void spread(CellData& q_data, const double* Q_data, int Q_size, int Q_depth, const double* X_data,
                       int X_size, int X_depth, const Patch& patch, const Box& spread_box,
                       const std::string& spread_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::spread()";
        const int k = ibx_detail::kernel_id(spread_fcn);
        if (Q_depth != q_data.getDepth()) throw std::runtime_error(where + ": Q_depth != q_data depth");
        const std::vector<int> idx = buildLocalIndices(spread_box, patch, X_data, X_size, X_depth);
        if (idx.empty()) return;
        ibx_detail::run(true, q_data, IBX_CELL, q_data.getDepth(), patch, const_cast<double*>(Q_data), Q_size,
                        Q_depth, X_data, X_size / X_depth, idx, nullptr, k, where);
    }
    // LEInteractor.cpp:4187-4264.
    static void spread(SideData& q_data, const double* Q_data, int Q_size, int Q_depth, const double* X_data,
                       int X_size, int X_depth, const Patch& patch, const Box& spread_box,
                       const std::string& spread_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::spread()";
        if (Q_depth != NDIM || q_data.getDepth() != 1)
            throw std::runtime_error(where + ":\n  side-centered spreading requires vector-valued data.\n");
        const int k = ibx_detail::kernel_id(spread_fcn);
        const std::vector<int> idx = buildLocalIndices(spread_box, patch, X_data, X_size, X_depth);
        if (idx.empty()) return;
        ibx_detail::run(true, q_data, IBX_SIDE, 1, patch, const_cast<double*>(Q_data), Q_size, Q_depth, X_data,
                        X_size / X_depth, idx, nullptr, k, where);
    }
    static void spread(CellData& q_data, const std::vector<double>& Q_data, int Q_depth,
                       const std::vector<double>& X_data, int X_depth, const Patch& patch, const Box& spread_box,
                       const std::string& spread_fcn = "IB_4")
    {
        spread(q_data, Q_data.data(), static_cast<int>(Q_data.size()), Q_depth, X_data.data(),
               static_cast<int>(X_data.size()), X_depth, patch, spread_box, spread_fcn);
    }
    static void spread(SideData& q_data, const std::vector<double>& Q_data, int Q_depth,
                       const std::vector<double>& X_data, int X_depth, const Patch& patch, const Box& spread_box,
                       const std::string& spread_fcn = "IB_4")
    {
        spread(q_data, Q_data.data(), static_cast<int>(Q_data.size()), Q_depth, X_data.data(),
               static_cast<int>(X_data.size()), X_depth, patch, spread_box, spread_fcn);
    }

    // Index-set forms (the LData overloads after buildLocalIndices,
    // LEInteractor.cpp:2402-2489, 3627-3714): local marker indices and NDIM
    // periodic shifts per index.
    static void interpolate(double* Q_data, int Q_depth, const double* X_data, int n_markers,
                            const std::vector<int>& local_indices, const std::vector<double>& periodic_shifts,
                            const SideData& q_data, const Patch& patch, const std::string& interp_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::interpolate()";
        if (Q_depth != NDIM || q_data.getDepth() != 1)
            throw std::runtime_error(where + ":\n  side-centered interpolation requires vector-valued data.\n");
        const int k = ibx_detail::kernel_id(interp_fcn);
        ibx_detail::ghost_check(q_data.getGhostCellWidth(), interp_fcn, where);
        if (local_indices.empty()) return;
        SideData q = q_data;
        ibx_detail::run(false, q, IBX_SIDE, 1, patch, Q_data, NDIM * n_markers, Q_depth, X_data, n_markers,
                        local_indices, &periodic_shifts, k, where);
    }
    static void spread(SideData& q_data, const double* Q_data, int Q_depth, const double* X_data, int n_markers,
                       const std::vector<int>& local_indices, const std::vector<double>& periodic_shifts,
                       const Patch& patch, const std::string& spread_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::spread()";
        if (Q_depth != NDIM || q_data.getDepth() != 1)
            throw std::runtime_error(where + ":\n  side-centered spreading requires vector-valued data.\n");
        const int k = ibx_detail::kernel_id(spread_fcn);
        if (local_indices.empty()) return;
        ibx_detail::run(true, q_data, IBX_SIDE, 1, patch, const_cast<double*>(Q_data), NDIM * n_markers, Q_depth,
                        X_data, n_markers, local_indices, &periodic_shifts, k, where);
    }
};
} // namespace IBTK

#endif
