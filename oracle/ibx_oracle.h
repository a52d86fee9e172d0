/*
 * ibx_oracle.h -- CPU oracle for the Lagrangian-Eulerian interaction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of IBAMR's
 * Fortran interaction routines and of the LEInteractor selection / side-axis
 * layer, used as the checker for the CUDA path.  Only the test suite, the
 * smoke check and the CPU-baseline leg of the benchmark load it; the product
 * library (ibamr_gb300/lib/libibx.so) never links or calls it.
 *
 * Parity is pinned against the reference's own golden outputs:
 *   - tests/IBTK/ghost_accumulation_01_{2d,3d}.{cell,side}.spread.{a,b}.output
 *     (16-digit PIECEWISE_LINEAR spread values, mt19937(42) inputs), and
 *   - tests/interpolate/interpolate_01_{2d,3d}.<kernel>.exact.{input,output}
 *     (polynomial-reproduction known-answer tests, error <= 1e-12 / 1e-10).
 * The reference Fortran cannot be compiled here (no Fortran compiler, no m4,
 * no SAMRAI), so the reference binary itself is not available as a second
 * oracle; the restatement follows the source line by line instead.
 *
 * Reference files (paths inside the IBAMR tree):
 *   F2D    = ibtk/src/lagrangian/fortran/lagrangian_interaction2d.f.m4
 *   F3D    = ibtk/src/lagrangian/fortran/lagrangian_interaction3d.f.m4
 *   FDELTA = ibtk/src/lagrangian/fortran/lagrangian_delta.f.m4
 *   LEI    = ibtk/src/lagrangian/LEInteractor.cpp
 */
#ifndef IBX_ORACLE_H
#define IBX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel ids: identical numbering to include/ibx.h (IBX_KERNEL_*). */
enum
{
    IBXO_PIECEWISE_LINEAR = 0,
    IBXO_PIECEWISE_CUBIC = 1,
    IBXO_IB_3 = 2,
    IBXO_IB_4 = 3,
    IBXO_IB_6 = 4,
    IBXO_BSPLINE_4 = 5
};

/* Status codes: identical numbering to include/ibx.h (IBX_*). */
enum
{
    IBXO_OK = 0,
    IBXO_E_BAD_KERNEL = 1,
    IBXO_E_GHOST_WIDTH = 2,
    IBXO_E_DEPTH = 3,
    IBXO_E_ARG = 4
};

/* Patch geometry (SAMRAI Patch + CartesianPatchGeometry). */
typedef struct ibxo_patch
{
    int dim;
    int ilower[3], iupper[3];            /* patch cell box */
    double dx[3], x_lower[3], x_upper[3];
    int touches_regular_lower[3];        /* getTouchesRegularBoundary(axis, 0) */
    int touches_regular_upper[3];        /* getTouchesRegularBoundary(axis, 1) */
    int touches_periodic_lower[3];       /* getTouchesPeriodicBoundary(axis, 0) */
    int touches_periodic_upper[3];       /* getTouchesPeriodicBoundary(axis, 1) */
} ibxo_patch;

/* Eulerian patch data in SAMRAI layout (Fortran order, ghosts included,
 * depth slowest).  centering 0 = CellData (ptr[0]), 1 = SideData (ptr[axis],
 * each on toSideBox(box, axis)). */
typedef struct ibxo_patch_data
{
    double* ptr[3];
    int gcw[3];
    int depth;
    int centering;
} ibxo_patch_data;

/* LEInteractor::getStencilSize / getMinimumGhostWidth / name lookup
 * (LEI:2052-2114, 1923-2016). Return -1 on an unknown kernel. */
int ibxo_stencil_size(int kernel);
int ibxo_min_ghost_width(int kernel);
int ibxo_kernel_from_name(const char* name);

/* Fortran NINT (round half away from zero), as the reference's routines use. */
int ibxo_nint(double a);

/* One dimension of a kernel's stencil as the Fortran routines compute it:
 * indices base+i for i in [start, stop] (clipped to the ghost box
 * [ilower-ghost, iupper+ghost]), w[i] their weights. */
int ibxo_stencil_1d(int kernel, double X, double Xshift, double x_lower, double dx, int ilower, int iupper, int ghost,
                    int* base, int* start, int* stop, double* w);

/* Literal restatement of lagrangian_<kernel>_interp{2,3}d / _spread{2,3}d.
 * Arguments carry the Fortran meaning (LEI:481-599); arrays are plain
 * pointers, scalars by value.  ilower/iupper/nugc have dim entries. */
int ibxo_fortran_interp(int kernel, int dim, const double* dx, const double* x_lower, const double* x_upper,
                        int depth, const int* ilower, const int* iupper, const int* nugc, const double* u,
                        const int* indices, const double* Xshift, int nindices, const double* X, double* V);
int ibxo_fortran_spread(int kernel, int dim, const double* dx, const double* x_lower, const double* x_upper,
                        int depth, const int* indices, const double* Xshift, int nindices, const double* X,
                        const double* V, const int* ilower, const int* iupper, const int* nugc, double* u);

/* IndexUtilities::getCellIndex (IndexUtilities-inl.h:52-75). */
void ibxo_get_cell_index(int dim, const double* X, const double* x_lower, const double* x_upper, const double* dx,
                         const int* ilower, const int* iupper, int* idx);

/* LEInteractor::buildLocalIndices, raw-array form (LEI:6088-6126): indices of
 * the markers whose cell lies in [box_lo, box_hi]. Returns the count. */
int ibxo_build_local_indices(const ibxo_patch* patch, const int* box_lo, const int* box_hi, const double* X,
                             int n_markers, int* local_indices);

/* LIndexSetData::cacheLocalIndices + buildLocalIndices(box == ghost box or
 * patch box) (LIndexSetData.cpp:50-140, LEI:6008-6086) for one patch of a
 * periodic domain of periodic_shift[d] cells: every marker image whose cell
 * lies in the patch box grown by ghost_width (want_ghost_box != 0) or in the
 * patch box (want_ghost_box == 0) is listed with its periodic shift.
 * Returns the count; at most capacity entries are written. */
int ibxo_cache_local_indices(const ibxo_patch* patch, const int* periodic_shift, const int* ghost_width,
                             int want_ghost_box, const double* X, int n_markers, int capacity, int* local_indices,
                             double* periodic_shifts);

/* LEInteractor::interpolate / spread on Cell or Side data, raw marker arrays
 * (LEI:2804-2862, 3044-3127, 3950-4008, 4187-4264): markers selected by
 * getCellIndex in [box_lo, box_hi], zero periodic shifts. */
int ibxo_lei_interpolate_raw(double* Q, int Q_depth, const double* X, int n_markers, const ibxo_patch_data* q,
                             const ibxo_patch* patch, const int* box_lo, const int* box_hi, int kernel);
int ibxo_lei_spread_raw(const ibxo_patch_data* q, const double* Q, int Q_depth, const double* X, int n_markers,
                        const ibxo_patch* patch, const int* box_lo, const int* box_hi, int kernel);

/* The index-set forms (LEI:2268-2330, 2402-2489, 3493-3555, 3627-3714): the
 * caller supplies local indices and periodic shifts (dim per index). */
int ibxo_lei_interpolate_idx(double* Q, int Q_depth, const double* X, const int* local_indices,
                             const double* periodic_shifts, int n_idx, const ibxo_patch_data* q,
                             const ibxo_patch* patch, int kernel);
int ibxo_lei_spread_idx(const ibxo_patch_data* q, const double* Q, int Q_depth, const double* X,
                        const int* local_indices, const double* periodic_shifts, int n_idx,
                        const ibxo_patch* patch, int kernel);

/* SAMRAIGhostDataAccumulator::accumulateGhostData for a single patch
 * (ibtk/src/math/SAMRAIGhostDataAccumulator.cpp): every value stored at a
 * ghost or interior position is summed into the degree of freedom it maps to
 * (periodic images identified, positions outside a non-periodic domain
 * dropped), and the sum is written back to every position of that DOF. */
int ibxo_accumulate_ghosts_single_patch(const ibxo_patch_data* q, const ibxo_patch* patch,
                                        const int* domain_lo, const int* domain_hi, const int* periodic);

/* Periodic ghost fill of a single patch that covers a periodic domain:
 * ghost(i) = interior(i mod N); side arrays also get face N := face 0. */
int ibxo_fill_periodic_ghosts(const ibxo_patch_data* q, const ibxo_patch* patch);

/* std::mt19937(seed) + std::uniform_real_distribution<double>(a, b): the
 * generator the reference tests use (libstdc++ semantics). */
void ibxo_mt19937_uniform(unsigned seed, int n, double a, double b, double* out);

/* CPU baseline (the reference's per-patch CPU path, multi-threaded the way
 * IBAMR runs ranks that each work through their patches).  One periodic
 * single-level problem on [0,1)^dim with N[d] cells is cut into n_boxes box
 * patches by recursive bisection on marker workload (markers + cells / 8
 * per cell, longest side first, no side below max(4, ghost width)).  The
 * plan caches each patch's LIndexSetData lists (ghost-box markers with
 * periodic shifts for spreading, interior markers for interpolation), as
 * LDataManager does between regrids.  A step then runs the patches on
 * n_threads threads, largest first: per patch it zeroes ghosted side arrays,
 * spreads (LEI:3627-3714), adds the patch interior into f; copies u into
 * ghosted side arrays (the periodic ghost fill) and interpolates
 * (LEI:2402-2489) into U.  f and u are compact periodic side arrays: dim
 * arrays of prod(N) doubles, x fastest, face i of axis a at x_lower + i*dx
 * (face N == face 0).  F and U hold dim values per marker.  The plan keeps
 * pointers to X.  ibxo_cpu_plan_patches: number of patches. */
void* ibxo_cpu_plan_create(int dim, const int* N, int kernel, int n_markers, const double* X, int n_threads,
                           int n_boxes);
int ibxo_cpu_plan_patches(void* plan);
int ibxo_cpu_plan_step(void* plan, const double* F, double* f, const double* u, double* U);
void ibxo_cpu_plan_destroy(void* plan);

#ifdef __cplusplus
}
#endif

#endif
