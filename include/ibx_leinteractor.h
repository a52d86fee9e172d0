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
 *
 * The reference's own signatures take SAMRAI::tbox::Pointer<> handles and
 * IBTK::LData / IBTK::LIndexSetData<T> objects; this header provides
 * stand-ins with the members those signatures use (namespace SAMRAI: tbox,
 * hier, pdat, geom; IBTK::LData, IBTK::LIndexSetData, IBTK::LNode,
 * IBTK::LNodeIndex), so code written against the reference's LEInteractor
 * compiles against this one.  LIndexSetData's cached lists are built on the
 * device (ibx_cache_local_indices).
 */
#ifndef IBX_LEINTERACTOR_H
#define IBX_LEINTERACTOR_H

#include "ibx.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <memory>
#include <stdexcept>
#include <type_traits>
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

// The SAMRAI names the reference's signatures spell, bound to the stand-ins
// above (the dimension parameter must equal NDIM).
namespace SAMRAI
{
namespace tbox
{
// tbox::Pointer<T>: a shared handle (operator->, getPointer, isNull, bool).
template <class T>
class Pointer
{
public:
    Pointer() = default;
    explicit Pointer(T* raw, bool managed = true)
        : d_p(managed ? std::shared_ptr<T>(raw) : std::shared_ptr<T>(raw, [](T*) {}))
    {
    }
    Pointer(std::shared_ptr<T> p) : d_p(std::move(p))
    {
    }
    T* operator->() const
    {
        return d_p.get();
    }
    T& operator*() const
    {
        return *d_p;
    }
    T* getPointer() const
    {
        return d_p.get();
    }
    bool isNull() const
    {
        return !d_p;
    }
    explicit operator bool() const
    {
        return static_cast<bool>(d_p);
    }

private:
    std::shared_ptr<T> d_p;
};
} // namespace tbox
namespace hier
{
template <int D>
using IntVector = typename std::enable_if<D == NDIM, ibx::samrai::IntVector>::type;
template <int D>
using Index = typename std::enable_if<D == NDIM, ibx::samrai::Index>::type;
template <int D>
using Box = typename std::enable_if<D == NDIM, ibx::samrai::Box>::type;
template <int D>
using Patch = typename std::enable_if<D == NDIM, ibx::samrai::Patch>::type;
} // namespace hier
namespace geom
{
template <int D>
using CartesianPatchGeometry = typename std::enable_if<D == NDIM, ibx::samrai::CartesianPatchGeometry>::type;
} // namespace geom
namespace pdat
{
template <int D, class T>
using CellData = typename std::enable_if<D == NDIM && std::is_same<T, double>::value, ibx::samrai::CellData>::type;
template <int D, class T>
using SideData = typename std::enable_if<D == NDIM && std::is_same<T, double>::value, ibx::samrai::SideData>::type;
} // namespace pdat
} // namespace SAMRAI

namespace IBTK
{
// Node types LIndexSetData is instantiated with in the reference
// (ibtk/src/lagrangian/LIndexSetData.cpp: LNode and LNodeIndex); tags here.
struct LNode
{
};
struct LNodeIndex
{
};

// IBTK::LData (ibtk/include/ibtk/LData.h): depth values per local node in
// one host array; getGhostedLocalFormVecArray()->data() is the array the
// reference's LEInteractor reads (no ghost nodes in a single process).
class LData
{
public:
    struct ArrayRef
    {
        double* p;
        double* data() const
        {
            return p;
        }
    };
    LData(std::string name, unsigned int num_local_nodes, unsigned int depth)
        : d_name(std::move(name)), d_n(num_local_nodes), d_depth(depth), d_values((size_t)num_local_nodes * depth, 0.0)
    {
    }
    const std::string& getName() const
    {
        return d_name;
    }
    unsigned int getDepth() const
    {
        return d_depth;
    }
    unsigned int getLocalNodeCount() const
    {
        return d_n;
    }
    unsigned int getGhostNodeCount() const
    {
        return 0;
    }
    ArrayRef* getGhostedLocalFormVecArray()
    {
        d_ref.p = d_values.data();
        return &d_ref;
    }
    ArrayRef* getLocalFormVecArray()
    {
        d_ref.p = d_values.data();
        return &d_ref;
    }
    void restoreArrays()
    {
    }
    // the values, depth per node (the PETSc vector's local form)
    std::vector<double>& values()
    {
        return d_values;
    }
    const std::vector<double>& values() const
    {
        return d_values;
    }

private:
    std::string d_name;
    unsigned int d_n, d_depth;
    std::vector<double> d_values;
    ArrayRef d_ref{ nullptr };
};

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

inline bool
same_box(const Box& a, const Box& b)
{
    for (int d = 0; d < NDIM; ++d)
        if (a.lo(d) != b.lo(d) || a.hi(d) != b.hi(d)) return false;
    return true;
}
} // namespace ibx_detail

// IBTK::LIndexSetData<T> (ibtk/include/ibtk/LIndexSetData.h): the markers of
// the cells of a patch's ghost box and the cached flattened lists of
// cacheLocalIndices (LIndexSetData.cpp:50-140).  In the reference the cells
// are filled by LDataManager's redistribution; here the markers are given by
// their positions (setMarkerPositions, the local nodes in PETSc order) and
// each one sits in the cell getCellIndex assigns it on the patch, with its
// periodic images in the ghost cells across periodic boundaries.  One
// process: Lagrangian, global and local PETSc indices coincide.
template <class T>
class LIndexSetData
{
public:
    using Box = ibx::samrai::Box;
    using IntVector = ibx::samrai::IntVector;
    using Patch = ibx::samrai::Patch;

    LIndexSetData(Box box, IntVector ghosts) : d_box(box), d_ghosts(ghosts)
    {
    }
    const Box& getBox() const
    {
        return d_box;
    }
    const IntVector& getGhostCellWidth() const
    {
        return d_ghosts;
    }
    Box getGhostBox() const
    {
        Box g = d_box;
        for (int d = 0; d < NDIM; ++d)
        {
            g.lo(d) -= d_ghosts(d);
            g.hi(d) += d_ghosts(d);
        }
        return g;
    }
    // Positions of the local markers (NDIM per marker, host array, kept by pointer).
    void setMarkerPositions(const double* X, int n_markers)
    {
        d_X = X;
        d_n = n_markers;
    }
    // LIndexSetData::cacheLocalIndices: lists of every marker image in the
    // ghost box, split into interior (cell in the patch box) and ghost
    // entries, with the periodic shifts of LIndexSetData.cpp:83-100; built on
    // the device by ibx_cache_local_indices.
    void cacheLocalIndices(SAMRAI::tbox::Pointer<Patch> patch, const IntVector& periodic_shift)
    {
        using namespace ibx_detail;
        clear();
        if (d_n == 0) return;
        ibx_patch_geometry G{};
        G.dim = NDIM;
        const auto& g = patch->getPatchGeometry();
        int ps[3] = { 0, 0, 0 }, gw[3] = { 0, 0, 0 };
        for (int d = 0; d < NDIM; ++d)
        {
            G.ilower[d] = patch->getBox().lo(d);
            G.iupper[d] = patch->getBox().hi(d);
            G.x_lower[d] = g.x_lower[d];
            G.x_upper[d] = g.x_upper[d];
            G.dx[d] = g.dx[d];
            G.touches_periodic_lower[d] = g.getTouchesPeriodicBoundary(d, 0);
            G.touches_periodic_upper[d] = g.getTouchesPeriodicBoundary(d, 1);
            ps[d] = periodic_shift(d);
            gw[d] = d_ghosts(d);
        }
        int cap = 1;
        for (int d = 0; d < NDIM; ++d) cap *= 3;
        cap *= d_n;
        DeviceBuffer dX, dIdx, dShift, dCell;
        const double* X = static_cast<const double*>(dX.upload(d_X, (long long)sizeof(double) * NDIM * d_n));
        int* idx = static_cast<int*>(dIdx.upload(nullptr, (long long)sizeof(int) * cap));
        double* sh = static_cast<double*>(dShift.upload(nullptr, (long long)sizeof(double) * NDIM * cap));
        int* cells = static_cast<int*>(dCell.upload(nullptr, (long long)sizeof(int) * NDIM * cap));
        int count = 0;
        check(ibx_cache_local_indices(&G, ps, gw, 1, X, d_n, cap, idx, sh, cells, &count, nullptr),
              "LIndexSetData::cacheLocalIndices()");
        d_local.resize(count);
        d_shifts.resize((size_t)NDIM * count);
        d_cells.resize((size_t)NDIM * count);
        if (count > 0)
        {
            check(ibx_memcpy(d_local.data(), idx, (long long)sizeof(int) * count, 0), "cacheLocalIndices");
            check(ibx_memcpy(d_shifts.data(), sh, (long long)sizeof(double) * NDIM * count, 0), "cacheLocalIndices");
            check(ibx_memcpy(d_cells.data(), cells, (long long)sizeof(int) * NDIM * count, 0), "cacheLocalIndices");
        }
        for (int e = 0; e < count; ++e)
        {
            Index c;
            for (int d = 0; d < NDIM; ++d) c(d) = d_cells[(size_t)NDIM * e + d];
            const bool interior = patch->getBox().contains(c);
            (interior ? d_interior : d_ghost).push_back(d_local[e]);
            auto& s = interior ? d_interior_shifts : d_ghost_shifts;
            for (int d = 0; d < NDIM; ++d) s.push_back(d_shifts[(size_t)NDIM * e + d]);
        }
    }
    const std::vector<int>& getLagrangianIndices() const
    {
        return d_local;
    }
    const std::vector<int>& getInteriorLagrangianIndices() const
    {
        return d_interior;
    }
    const std::vector<int>& getGhostLagrangianIndices() const
    {
        return d_ghost;
    }
    const std::vector<int>& getGlobalPETScIndices() const
    {
        return d_local;
    }
    const std::vector<int>& getInteriorGlobalPETScIndices() const
    {
        return d_interior;
    }
    const std::vector<int>& getGhostGlobalPETScIndices() const
    {
        return d_ghost;
    }
    const std::vector<int>& getLocalPETScIndices() const
    {
        return d_local;
    }
    const std::vector<int>& getInteriorLocalPETScIndices() const
    {
        return d_interior;
    }
    const std::vector<int>& getGhostLocalPETScIndices() const
    {
        return d_ghost;
    }
    const std::vector<double>& getPeriodicShifts() const
    {
        return d_shifts;
    }
    const std::vector<double>& getInteriorPeriodicShifts() const
    {
        return d_interior_shifts;
    }
    const std::vector<double>& getGhostPeriodicShifts() const
    {
        return d_ghost_shifts;
    }
    // Cell of each entry of the local lists (NDIM per entry): the cell whose
    // marker set holds it, what the reference's SetIterator reports.
    const std::vector<int>& getCells() const
    {
        return d_cells;
    }

private:
    using Index = ibx::samrai::Index;
    void clear()
    {
        d_local.clear();
        d_interior.clear();
        d_ghost.clear();
        d_shifts.clear();
        d_interior_shifts.clear();
        d_ghost_shifts.clear();
        d_cells.clear();
    }
    Box d_box;
    IntVector d_ghosts;
    const double* d_X = nullptr;
    int d_n = 0;
    std::vector<int> d_local, d_interior, d_ghost, d_cells;
    std::vector<double> d_shifts, d_interior_shifts, d_ghost_shifts;
};

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

    // ---- LIndexSetData forms ----------------------------------------------
    // LEInteractor::buildLocalIndices (LEInteractor.cpp:6008-6086): the
    // index-set entries whose cell lies in `box`, with their periodic shifts;
    // the interior lists for the patch box, every entry for the ghost box.
    template <class T>
    static void buildLocalIndices(std::vector<int>& local_indices, std::vector<double>& periodic_shifts,
                                  const Box& box, const SAMRAI::tbox::Pointer<Patch> patch,
                                  const ibx::samrai::IntVector& periodic_shift,
                                  const SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data)
    {
        local_indices.clear();
        periodic_shifts.clear();
        if (idx_data->getLocalPETScIndices().empty()) return;
        if (ibx_detail::same_box(box, patch->getBox()))
        {
            local_indices = idx_data->getInteriorLocalPETScIndices();
            periodic_shifts = idx_data->getInteriorPeriodicShifts();
            return;
        }
        if (ibx_detail::same_box(box, idx_data->getGhostBox()))
        {
            local_indices = idx_data->getLocalPETScIndices();
            periodic_shifts = idx_data->getPeriodicShifts();
            return;
        }
        // other boxes: the entries of the cells in the box, the shift of each
        // by the reference's rule (LEInteractor.cpp:6050-6069)
        const auto& g = patch->getPatchGeometry();
        const auto& cells = idx_data->getCells();
        const auto& all = idx_data->getLocalPETScIndices();
        for (size_t e = 0; e < all.size(); ++e)
        {
            ibx::samrai::Index c;
            for (int d = 0; d < NDIM; ++d) c(d) = cells[NDIM * e + d];
            if (!box.contains(c)) continue;
            local_indices.push_back(all[e]);
            for (int d = 0; d < NDIM; ++d)
            {
                int offset = 0;
                if (g.getTouchesPeriodicBoundary(d, 0) && c(d) < patch->getBox().lo(d))
                    offset = -periodic_shift(d);
                else if (g.getTouchesPeriodicBoundary(d, 1) && c(d) > patch->getBox().hi(d))
                    offset = +periodic_shift(d);
                periodic_shifts.push_back(static_cast<double>(offset) * g.dx[d]);
            }
        }
    }

    // LEInteractor.cpp:2270-2330 (cell) and 2404-2489 (side): interpolate at
    // the index set's markers in interp_box.
    template <class T>
    static void interpolate(double* Q_data, int Q_depth, const double* X_data, int X_depth,
                            SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data, SAMRAI::tbox::Pointer<CellData> q_data,
                            SAMRAI::tbox::Pointer<Patch> patch, const Box& interp_box,
                            const ibx::samrai::IntVector& periodic_shift, const std::string& interp_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::interpolate()";
        if (Q_depth != q_data->getDepth()) throw std::runtime_error(where + ": Q_depth != q_data depth");
        indexed(false, *q_data, IBX_CELL, q_data->getDepth(), Q_data, Q_depth, X_data, X_depth, idx_data, patch,
                interp_box, periodic_shift, interp_fcn, where);
    }
    template <class T>
    static void interpolate(double* Q_data, int Q_depth, const double* X_data, int X_depth,
                            SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data, SAMRAI::tbox::Pointer<SideData> q_data,
                            SAMRAI::tbox::Pointer<Patch> patch, const Box& interp_box,
                            const ibx::samrai::IntVector& periodic_shift, const std::string& interp_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::interpolate()";
        if (Q_depth != NDIM || q_data->getDepth() != 1)
            throw std::runtime_error(where + ":\n  side-centered interpolation requires vector-valued data.\n");
        indexed(false, *q_data, IBX_SIDE, 1, Q_data, Q_depth, X_data, X_depth, idx_data, patch, interp_box,
                periodic_shift, interp_fcn, where);
    }
    // LEInteractor.cpp:2118-2151 (cell) and 2188-2225 (side): the LData forms.
    template <class T>
    static void interpolate(SAMRAI::tbox::Pointer<LData> Q_data, SAMRAI::tbox::Pointer<LData> X_data,
                            SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data, SAMRAI::tbox::Pointer<CellData> q_data,
                            SAMRAI::tbox::Pointer<Patch> patch, const Box& interp_box,
                            const ibx::samrai::IntVector& periodic_shift, const std::string& interp_fcn = "IB_4")
    {
        interpolate(Q_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(Q_data->getDepth()),
                    X_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(X_data->getDepth()), idx_data,
                    q_data, patch, interp_box, periodic_shift, interp_fcn);
        Q_data->restoreArrays();
        X_data->restoreArrays();
    }
    template <class T>
    static void interpolate(SAMRAI::tbox::Pointer<LData> Q_data, SAMRAI::tbox::Pointer<LData> X_data,
                            SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data, SAMRAI::tbox::Pointer<SideData> q_data,
                            SAMRAI::tbox::Pointer<Patch> patch, const Box& interp_box,
                            const ibx::samrai::IntVector& periodic_shift, const std::string& interp_fcn = "IB_4")
    {
        if (Q_data->getDepth() != NDIM || q_data->getDepth() != 1)
            throw std::runtime_error("LEInteractor::interpolate():\n"
                                     "  side-centered interpolation requires vector-valued data.\n");
        interpolate(Q_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(Q_data->getDepth()),
                    X_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(X_data->getDepth()), idx_data,
                    q_data, patch, interp_box, periodic_shift, interp_fcn);
        Q_data->restoreArrays();
        X_data->restoreArrays();
    }

    // LEInteractor.cpp:3495-3555 (cell) and 3629-3714 (side): spread the
    // index set's markers in spread_box.
    template <class T>
    static void spread(SAMRAI::tbox::Pointer<CellData> q_data, const double* Q_data, int Q_depth,
                       const double* X_data, int X_depth, SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data,
                       SAMRAI::tbox::Pointer<Patch> patch, const Box& spread_box,
                       const ibx::samrai::IntVector& periodic_shift, const std::string& spread_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::spread()";
        if (Q_depth != q_data->getDepth()) throw std::runtime_error(where + ": Q_depth != q_data depth");
        indexed(true, *q_data, IBX_CELL, q_data->getDepth(), const_cast<double*>(Q_data), Q_depth, X_data, X_depth,
                idx_data, patch, spread_box, periodic_shift, spread_fcn, where);
    }
    template <class T>
    static void spread(SAMRAI::tbox::Pointer<SideData> q_data, const double* Q_data, int Q_depth,
                       const double* X_data, int X_depth, SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data,
                       SAMRAI::tbox::Pointer<Patch> patch, const Box& spread_box,
                       const ibx::samrai::IntVector& periodic_shift, const std::string& spread_fcn = "IB_4")
    {
        const std::string where = "LEInteractor::spread()";
        if (Q_depth != NDIM || q_data->getDepth() != 1)
            throw std::runtime_error(where + ":\n  side-centered spreading requires vector-valued data.\n");
        indexed(true, *q_data, IBX_SIDE, 1, const_cast<double*>(Q_data), Q_depth, X_data, X_depth, idx_data, patch,
                spread_box, periodic_shift, spread_fcn, where);
    }
    // LEInteractor.cpp:3343-3376 (cell) and 3413-3450 (side): the LData forms.
    template <class T>
    static void spread(SAMRAI::tbox::Pointer<CellData> q_data, SAMRAI::tbox::Pointer<LData> Q_data,
                       SAMRAI::tbox::Pointer<LData> X_data, SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data,
                       SAMRAI::tbox::Pointer<Patch> patch, const Box& spread_box,
                       const ibx::samrai::IntVector& periodic_shift, const std::string& spread_fcn = "IB_4")
    {
        spread(q_data, Q_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(Q_data->getDepth()),
               X_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(X_data->getDepth()), idx_data, patch,
               spread_box, periodic_shift, spread_fcn);
        Q_data->restoreArrays();
        X_data->restoreArrays();
    }
    template <class T>
    static void spread(SAMRAI::tbox::Pointer<SideData> q_data, SAMRAI::tbox::Pointer<LData> Q_data,
                       SAMRAI::tbox::Pointer<LData> X_data, SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data,
                       SAMRAI::tbox::Pointer<Patch> patch, const Box& spread_box,
                       const ibx::samrai::IntVector& periodic_shift, const std::string& spread_fcn = "IB_4")
    {
        if (Q_data->getDepth() != NDIM || q_data->getDepth() != 1)
            throw std::runtime_error("LEInteractor::spread():\n"
                                     "  side-centered spreading requires vector-valued data.\n");
        spread(q_data, Q_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(Q_data->getDepth()),
               X_data->getGhostedLocalFormVecArray()->data(), static_cast<int>(X_data->getDepth()), idx_data, patch,
               spread_box, periodic_shift, spread_fcn);
        Q_data->restoreArrays();
        X_data->restoreArrays();
    }

    // ---- Pointer forms of the raw-array calls (LEInteractor.h:487-628, 880-1200)
    static void interpolate(double* Q_data, int Q_size, int Q_depth, const double* X_data, int X_size, int X_depth,
                            SAMRAI::tbox::Pointer<CellData> q_data, SAMRAI::tbox::Pointer<Patch> patch,
                            const Box& interp_box, const std::string& interp_fcn = "IB_4")
    {
        interpolate(Q_data, Q_size, Q_depth, X_data, X_size, X_depth, *q_data, *patch, interp_box, interp_fcn);
    }
    static void interpolate(double* Q_data, int Q_size, int Q_depth, const double* X_data, int X_size, int X_depth,
                            SAMRAI::tbox::Pointer<SideData> q_data, SAMRAI::tbox::Pointer<Patch> patch,
                            const Box& interp_box, const std::string& interp_fcn = "IB_4")
    {
        interpolate(Q_data, Q_size, Q_depth, X_data, X_size, X_depth, *q_data, *patch, interp_box, interp_fcn);
    }
    static void spread(SAMRAI::tbox::Pointer<CellData> q_data, const double* Q_data, int Q_size, int Q_depth,
                       const double* X_data, int X_size, int X_depth, SAMRAI::tbox::Pointer<Patch> patch,
                       const Box& spread_box, const std::string& spread_fcn = "IB_4")
    {
        spread(*q_data, Q_data, Q_size, Q_depth, X_data, X_size, X_depth, *patch, spread_box, spread_fcn);
    }
    static void spread(SAMRAI::tbox::Pointer<SideData> q_data, const double* Q_data, int Q_size, int Q_depth,
                       const double* X_data, int X_size, int X_depth, SAMRAI::tbox::Pointer<Patch> patch,
                       const Box& spread_box, const std::string& spread_fcn = "IB_4")
    {
        spread(*q_data, Q_data, Q_size, Q_depth, X_data, X_size, X_depth, *patch, spread_box, spread_fcn);
    }

private:
    // The private interpolate / spread after buildLocalIndices: the selected
    // entries, the per-marker arrays sized max(local index) + 1 as the
    // reference's scratch is (LEInteractor.cpp:2455-2456, 3687-3688).
    template <class Data, class T>
    static void indexed(bool do_spread, Data& q, int centering, int q_depth, double* Q_data, int Q_depth,
                        const double* X_data, int X_depth, SAMRAI::tbox::Pointer<LIndexSetData<T>> idx_data,
                        SAMRAI::tbox::Pointer<Patch> patch, const Box& box,
                        const ibx::samrai::IntVector& periodic_shift, const std::string& fcn, const std::string& where)
    {
        const int k = ibx_detail::kernel_id(fcn);
        if (!do_spread) ibx_detail::ghost_check(q.getGhostCellWidth(), fcn, where);
        if (X_depth != NDIM) throw std::runtime_error(where + ": X_depth != NDIM");
        std::vector<int> local_indices;
        std::vector<double> periodic_shifts;
        buildLocalIndices(local_indices, periodic_shifts, box, patch, periodic_shift, idx_data);
        if (local_indices.empty()) return;
        const int n = *std::max_element(local_indices.begin(), local_indices.end()) + 1;
        Data qq = q; // host-resident data is copied in and (spread) out by the call
        ibx_detail::run(do_spread, do_spread ? q : qq, centering, q_depth, *patch, Q_data, Q_depth * n, Q_depth,
                        X_data, n, local_indices, &periodic_shifts, k, where);
    }
};
} // namespace IBTK

#endif
