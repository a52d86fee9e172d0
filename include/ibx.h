/*
 * ibx.h -- C ABI of the GB300 Lagrangian-Eulerian interaction library
 * (libibx.so).  Spreading of marker values onto staggered (side-centred) or
 * cell-centred grids and interpolation of grid values onto markers with the
 * regularized delta kernels of IBAMR's IBTK::LEInteractor.
 *
 * Every entry point is stream-ordered, reentrant and returns a status code
 * instead of aborting.  Pointers inside ibx_problem are DEVICE pointers
 * unless stated otherwise.  Only ibx_plan_create* allocate memory that
 * outlives the call; ibx_spread / ibx_interpolate with several problems and
 * ibx_redistribute use stream-ordered scratch freed before they return.
 *
 * Reference interfaces replaced (paths inside the IBAMR tree):
 *   LEI.h  = ibtk/include/ibtk/LEInteractor.h
 *   LEI    = ibtk/src/lagrangian/LEInteractor.cpp
 */
#ifndef IBX_H
#define IBX_H

#include <stddef.h> /* size_t */

#ifdef __cplusplus
extern "C" {
#endif

/* ---- kernels (LEI:1923-2016 string_to_kernel) ------------------------- */
enum
{
    IBX_KERNEL_PIECEWISE_LINEAR = 0,
    IBX_KERNEL_PIECEWISE_CUBIC = 1,
    IBX_KERNEL_IB_3 = 2,
    IBX_KERNEL_IB_4 = 3,
    IBX_KERNEL_IB_6 = 4,
    IBX_KERNEL_BSPLINE_4 = 5
};

/* ---- precision forms -------------------------------------------------- */
enum
{
    /* FP64 everywhere: grid values, marker values, weights, accumulation. */
    IBX_PRECISION_FP64 = 0,
    /* Grid and marker values stored and multiplied in FP32; positions,
     * stencil indices and kernel arguments in FP64; spread sums accumulated
     * in a double-FP32 (compensated, ~48-bit) accumulator. */
    IBX_PRECISION_MIXED = 1
};

/* ---- data centering --------------------------------------------------- */
enum
{
    IBX_CELL = 0, /* SAMRAI CellData: one array of q_depth components */
    IBX_SIDE = 1  /* SAMRAI SideData: one array per axis, on toSideBox(box, axis) */
};

/* ---- problem modes ---------------------------------------------------- */
enum
{
    /* Reference semantics of one LEInteractor call on one patch: markers
     * selected by indices (+ periodic shifts Xshift), stencils clipped to
     * the ghost box, arrays in SAMRAI layout (ghosts included, Fortran
     * order, depth slowest).  Ghost values are written by spreading. */
    IBX_MODE_PATCH = 0,
    /* One patch that covers a periodic domain, stored compactly: each
     * component is N0 x N1 (x N2) values, x fastest, no ghosts, and side
     * arrays hold N faces along their normal (face N is face 0).  Stencil
     * indices wrap modulo N, so no periodic image markers are needed. */
    IBX_MODE_PERIODIC = 1
};

/* ---- status codes ----------------------------------------------------- */
enum
{
    IBX_OK = 0,
    IBX_E_BAD_KERNEL = 1,  /* unknown kernel id or name (LEI:2014) */
    IBX_E_GHOST_WIDTH = 2, /* ghost width below getMinimumGhostWidth (LEI:4488-4498, 5250-5268) */
    IBX_E_DEPTH = 3,       /* Q_depth / q_depth mismatch (LEI:2197-2201, 3650-3654) */
    IBX_E_ARG = 4,         /* malformed argument (null pointer, bad dim, bad sizes) */
    IBX_E_CUDA = 5,        /* a CUDA runtime call failed */
    IBX_E_OOM = 6,         /* device memory exhausted */
    IBX_E_TIMEOUT = 7,     /* a bounded device-side wait gave up */
    IBX_E_NONFINITE = 8,   /* a marker position is NaN or infinite */
    IBX_E_TOO_LARGE = 9    /* a size exceeds a documented limit */
};

/* One patch-level interaction problem: the arguments of the reference's
 * private LEInteractor::interpolate / spread (LEI.h:1326-1361) with device
 * pointers.  Several problems can be passed in one call; they run in one
 * launch and must not share output memory. */
typedef struct ibx_problem
{
    int dim;       /* 2 or 3 */
    int centering; /* IBX_CELL or IBX_SIDE */
    int mode;      /* IBX_MODE_PATCH or IBX_MODE_PERIODIC */
    int ilower[3]; /* patch cell box (Patch::getBox()) */
    int iupper[3];
    int gcw[3];    /* ghost cell width of the Eulerian data (IBX_MODE_PATCH) */
    double dx[3];  /* CartesianPatchGeometry::getDx/getXLower/getXUpper */
    double x_lower[3];
    double x_upper[3];
    int touches_physical_lower[3]; /* getTouchesRegularBoundary(axis, 0/1) */
    int touches_physical_upper[3];
    int q_depth;        /* CellData depth; SideData requires 1 */
    void* q[3];         /* cell: q[0]; side: q[axis].  double or float */
    const double* X;    /* X[dim*s + d], FP64 */
    void* Q;            /* Q[Q_depth*s + k]; double (FP64) or float (MIXED) */
    int Q_depth;        /* cell: == q_depth; side: == dim */
    int n_markers;      /* marker slots addressed by s */
    const int* indices; /* IBX_MODE_PATCH: local marker indices, or NULL = 0..n_markers-1 */
    int n_indices;      /* entries of indices (ignored when indices is NULL) */
    const double* Xshift; /* IBX_MODE_PATCH: dim shifts per index entry, or NULL = 0 */
} ibx_problem;

/* LEInteractor::getStencilSize (LEI:2052-2108); -1 for an unknown kernel. */
int ibx_get_stencil_size(int kernel);
/* LEInteractor::getMinimumGhostWidth (LEI:2110-2114); -1 for an unknown kernel. */
int ibx_get_minimum_ghost_width(int kernel);
/* LEInteractor::isKnownKernel + string_to_kernel (LEI:1923-2050) restricted
 * to the kernels this library implements; -1 for any other name. */
int ibx_kernel_from_name(const char* name);
/* Human-readable text of a status code. */
const char* ibx_status_string(int status);

/* LEInteractor::interpolate (LEI:2186-2489, 2804-2862, 3044-3127 and the
 * private form LEI:4470-5230): overwrite Q at the selected markers with the
 * kernel-weighted sum of q.  Markers not selected are left untouched.
 * Direct marker-parallel form without scratch memory; with n_problems > 1
 * the descriptor table is staged in stream-ordered device memory
 * (cudaMallocAsync) and the call synchronises the stream. */
int ibx_interpolate(const ibx_problem* problems, int n_problems, int kernel, int precision, void* stream);

/* LEInteractor::spread (LEI:3341-3714, 3950-4264 and the private form
 * LEI:5232-6006): q += kernel-weighted Q / prod(dx) for the selected
 * markers.  Direct marker-parallel form using FP64 device atomics, no
 * scratch memory; n_problems > 1 as for ibx_interpolate. */
int ibx_spread(const ibx_problem* problems, int n_problems, int kernel, int precision, void* stream);

/* ---- ghost data of IBX_MODE_PATCH arrays (FP64) ---------------------- */
/* SAMRAIGhostDataAccumulator::accumulateGhostData
 * (ibtk/src/math/SAMRAIGhostDataAccumulator.cpp:295-353) for one patch that
 * covers the whole domain: every value of the ghosted arrays is added into
 * its degree of freedom (periodic images along dims with periodic[d] != 0;
 * along other dims positions outside the domain have none and are left as
 * they are), then every copy of a DOF receives the total (so face N and face
 * 0 of a periodic side axis hold the same sum).  Sums are taken in array
 * order, as the reference's vector assembly does. */
int ibx_accumulate_ghosts(const ibx_problem* problem, const int* periodic, void* stream);
/* Periodic ghost fill of one patch covering the domain (the periodic copy of
 * a SAMRAI refine schedule): along dims with periodic[d] != 0 every value
 * outside the cell box takes the value of its image inside it. */
int ibx_fill_ghosts(const ibx_problem* problem, const int* periodic, void* stream);

/* ---- marker redistribution over the patches of a level ----------------- */
/* One patch of a level: cell box and geometry (CartesianPatchGeometry). */
typedef struct ibx_patch_box
{
    int ilower[3], iupper[3];
    double x_lower[3], x_upper[3], dx[3];
} ibx_patch_box;

/* Which patch owns each marker (LDataManager::redistribute,
 * src/IB/LDataManager.cpp:1351-1522, with the index rule of
 * IndexUtilities::getCellIndex, ibtk/include/ibtk/private/
 * IndexUtilities-inl.h:52-75, evaluated with every patch's geometry in FP64):
 * owner[s] = the first patch in `patches` (a host array) whose cell box holds
 * the marker's cell index, -1 for none; order = the markers grouped by owner
 * (counting sort; patch p's markers are order[patch_offsets[p] ..
 * patch_offsets[p+1]), the unowned ones follow, patch_offsets has
 * n_patches + 2 entries and patch_offsets[n_patches + 1] = n_markers; the
 * order within a patch is unspecified).  X, owner, order and patch_offsets
 * are device arrays.  Uses stream-ordered scratch memory and synchronises
 * the stream before returning. */
int ibx_redistribute(int dim, const ibx_patch_box* patches, int n_patches, const double* X, int n_markers, int* owner,
                     int* order, int* patch_offsets, void* stream);

/* ---- cached index sets of a patch --------------------------------------- */
/* One patch: cell box, CartesianPatchGeometry (getXLower/getXUpper/getDx)
 * and getTouchesPeriodicBoundary(axis, 0/1). */
typedef struct ibx_patch_geometry
{
    int dim;
    int ilower[3], iupper[3];
    double x_lower[3], x_upper[3], dx[3];
    int touches_periodic_lower[3], touches_periodic_upper[3];
} ibx_patch_geometry;

/* LIndexSetData::cacheLocalIndices (ibtk/src/lagrangian/LIndexSetData.cpp:
 * 50-140) on the device, for markers whose cells are given by their
 * positions: marker s sits in cell c = getCellIndex(X_s) on the patch
 * geometry (IndexUtilities-inl.h:52-75) and its periodic images in cells
 * c + k * periodic_shift (k in {-1,0,1}^dim, k_d != 0 only where
 * periodic_shift_d != 0).  Every image whose cell lies in the patch box grown
 * by ghost_width (want_ghost_box != 0; the getLocalPETScIndices /
 * getPeriodicShifts lists) or in the patch box (want_ghost_box == 0; the
 * getInteriorLocalPETScIndices / getInteriorPeriodicShifts lists) and whose
 * offset by the reference's rule (LIndexSetData.cpp:83-100: -periodic_shift
 * below ilower at a lower periodic boundary, +periodic_shift above iupper at
 * an upper one, else 0) equals k * periodic_shift is listed: local_indices[e]
 * = s, periodic_shifts[dim*e + d] = offset_d * dx_d and, when cells is not
 * NULL, cells[dim*e + d] = the image's cell.  Entries in marker order,
 * images of a marker with k_0 fastest.  X, local_indices, periodic_shifts and
 * cells are device arrays; *count (host) receives the number of entries.
 * More entries than capacity: IBX_E_TOO_LARGE, the first capacity written.
 * Uses stream-ordered scratch and synchronises the stream. */
int ibx_cache_local_indices(const ibx_patch_geometry* patch, const int* periodic_shift, const int* ghost_width,
                            int want_ghost_box, const double* X, int n_markers, int capacity, int* local_indices,
                            double* periodic_shifts, int* cells, int* count, void* stream);

/* ---- finite-element quadrature points (FEDataManager) ------------------- */
/* Element families of ibx_fe_mesh (first-order Lagrange elements). */
enum
{
    IBX_FE_SIMPLEX_P1 = 0, /* TRI3 (2D), TET4 (3D) */
    IBX_FE_TENSOR_Q1 = 1   /* QUAD4 (2D), HEX8 (3D) */
};
/* A mesh of one element family.  Simplices: node k of element e is
 * elem_nodes[(dim+1)*e + k] (libMesh's vertex order: the reference element's
 * vertices 0, e_1, ..., e_dim).  Tensor-product cells: node k of element e is
 * elem_nodes[npe*e + k], npe = 4 (QUAD4) or 8 (HEX8), in libMesh's order on
 * the reference cell [-1, 1]^dim: (-1,-1), (1,-1), (1,1), (-1,1) in each z
 * layer, the z = -1 layer first.  X holds dim coordinates per node.  Both
 * are device arrays.  elem_type: IBX_FE_SIMPLEX_P1 or IBX_FE_TENSOR_Q1. */
typedef struct ibx_fe_mesh
{
    int dim;
    int n_nodes;
    int n_elems;
    const int* elem_nodes;
    const double* X;
    int elem_type;
} ibx_fe_mesh;

/* A quadrature rule on the reference element (host arrays): n_points points
 * (dim reference coordinates each) and their weights, summing to the
 * reference element's measure as libMesh's rules do (simplices: 1/2 in 2D,
 * 1/6 in 3D; tensor-product cells: 4 in 2D, 8 in 3D); at most 64 points. */
typedef struct ibx_quad_rule
{
    int n_points;
    const double* points;
    const double* weights;
} ibx_quad_rule;

/* The quadrature-point side of FEDataManager::spread
 * (ibtk/src/lagrangian/FEDataManager.cpp:1088-1219, sum_weighted_elem_solution
 * :824-858): for point q of element e (entry e*n_points + q),
 * X_qp = sum_k X_k phi_k(q) and, when F_nodes is given (n_vars values per
 * node), F_JxW_qp = (sum_k F_k phi_k(q)) * JxW(q), with the element's basis
 * phi (barycentric on simplices; products of the 1D linear shapes
 * (1 -+ xi)/2 on tensor-product cells) and JxW(q) = |det J(q)| * weight(q),
 * J(q) = sum_k X_k (grad phi_k(q))^T; JxW receives JxW(q) when not NULL.
 * Sums run from zero over the basis in order, every operation rounded as
 * written.  The outputs feed ibx_spread (positions X_qp, values F_JxW_qp) as
 * LEInteractor::spread's raw-array form does in the reference.  An element
 * with a negative node index is skipped and sets bit 0 of the device word
 * *status.  Device pointers; stream-ordered. */
int ibx_fe_quadrature_points(const ibx_fe_mesh* mesh, const ibx_quad_rule* rule, const double* F_nodes, int n_vars,
                             double* X_qp, double* F_JxW_qp, double* JxW, int* status, void* stream);

/* The assembly side of FEDataManager::interp (FEDataManager.cpp:1873-2005,
 * integrate_elem_rhs :1569-1604): with U_qp the values interpolated at the
 * quadrature points (n_vars per point, as ibx_interpolate writes them at
 * X_qp), rhs[n_vars*node + i] += sum_q U_qp[q][i] * (phi_k(q) * JxW(q)) for
 * every element and every node k of it -- the right-hand side of the L2
 * projection (the projection's solve is the caller's).  Element sums in point
 * order; elements are added with FP64 atomics (their order may differ from
 * the reference's vector assembly).  Device pointers; stream-ordered. */
int ibx_fe_assemble_rhs(const ibx_fe_mesh* mesh, const ibx_quad_rule* rule, const double* U_qp, int n_vars,
                        double* rhs, void* stream);

/* ---- Lagrangian forces before spreading -------------------------------- */
/* IBStandardForceGen::computeLagrangianSpringForce
 * (src/IB/IBStandardForceGen.cpp:825-900) with the default linear spring
 * (include/ibamr/IBSpringForceFunctions.h:104-107), on the device: for spring
 * k between master[k] and slave[k], D = X_slave - X_master, R = |D|, springs
 * with R < DBL_EPSILON skipped, T = stiffness[k] * (R - rest_length[k]), and
 * T/R * D added to F(master) and subtracted from F(slave).  F holds dim
 * values per marker, double (IBX_PRECISION_FP64) or float (MIXED);
 * accumulate = 0 zeroes F first.  Node indices outside [0, n_markers) are
 * skipped and set bit 0 of the device word *status.  All pointers are device
 * pointers; stream-ordered, so the spread that reads F can follow on the
 * same stream (or in the same CUDA graph).  Contributions are summed with
 * atomics: the order of additions, not the values, may differ from the
 * reference's sequential loop. */
int ibx_spring_forces(int dim, int n_markers, const double* X, int n_springs, const int* master, const int* slave,
                      const double* stiffness, const double* rest_length, void* F, int precision, int accumulate,
                      int* status, void* stream);
/* IBStandardForceGen::computeLagrangianBeamForce
 * (src/IB/IBStandardForceGen.cpp:1037-1147) on the device: for beam k with
 * master node master[k] and neighbours next[k], prev[k], rigidity K =
 * rigidity[k] and reference curvature D2X0 = curvature[dim*k ..],
 * F = K * ((X_next + X_prev) - 2 X_master - D2X0); 2F is added to the master
 * node's force, F subtracted from each neighbour's.  Arguments, precision,
 * accumulate and status as for ibx_spring_forces. */
int ibx_beam_forces(int dim, int n_markers, const double* X, int n_beams, const int* master, const int* next,
                    const int* prev, const double* rigidity, const double* curvature, void* F, int precision,
                    int accumulate, int* status, void* stream);
/* IBStandardForceGen::computeLagrangianTargetPointForce (:1201-1299) on the
 * device: for target point k at node node[k], F += kappa[k] *
 * (X_target[dim*k ..] - X) - eta[k] * U (U: the nodes' velocities, dim per
 * marker; NULL = 0).  max_displacement (a device double, or NULL) receives
 * the largest |X_target - X| over the points, the value the reference logs.
 * Arguments, precision, accumulate and status as for ibx_spring_forces. */
int ibx_target_point_forces(int dim, int n_markers, const double* X, const double* U, int n_points, const int* node,
                            const double* kappa, const double* eta, const double* X_target, void* F, int precision,
                            int accumulate, double* max_displacement, int* status, void* stream);
/* IBStandardForceGen::computeLagrangianBodyForce (:1301-1327) on the device:
 * marker i of structure structure[i] gets the structure's uniform force
 * force[dim*sid ..] added to F, for sid in [0, n_structures) with
 * has_force[sid] != 0 (has_force NULL: every structure).  Device pointers;
 * F as for ibx_spring_forces (always accumulated). */
int ibx_body_forces(int dim, int n_markers, const int* structure, int n_structures, const double* force,
                    const int* has_force, void* F, int precision, void* stream);

/* ---- host helpers (used by the C++ LEInteractor layer) ----------------- */
/* Device memory and copies for callers without the CUDA runtime headers.
 * ibx_device_alloc / ibx_device_free take buffers from a memory pool of the
 * library that keeps freed memory for the next allocation (no cudaMalloc /
 * cudaFree per call); both are ordered on the legacy default stream, so work
 * on non-blocking streams that uses a buffer must be synchronised before it
 * is freed.  ibx_memcpy is a blocking cudaMemcpy (to_device != 0: host to
 * device); ibx_synchronize is cudaDeviceSynchronize. */
int ibx_device_alloc(void** ptr, long long bytes);
int ibx_device_free(void* ptr);
int ibx_memcpy(void* dst, const void* src, long long bytes, int to_device);
int ibx_synchronize(void);

/* Diagnostic without a reference counterpart: number of CUDA kernels this
 * library has launched in the process so far (host-side count, all threads,
 * all devices). */
long long ibx_kernel_launches(void);

/* ---- binned plans (the fast path) ------------------------------------- */
/* A plan owns the scratch memory of the binned spread/interpolate pipeline
 * for a fixed set of IBX_MODE_PERIODIC problems (grids, marker arrays and
 * capacities fixed at creation; positions and values may change between
 * steps).  ibx_plan_bin sorts the markers of every problem by grid tile
 * (integer counting sort) and derives their stencil indices and kernel
 * arguments in FP64; ibx_plan_spread / ibx_plan_interpolate then run one
 * launch each over all problems.  All three are CUDA-graph capturable once
 * the plan exists.  ibx_plan_create allocates device memory (the only entry
 * point that does). */
typedef struct ibx_plan ibx_plan;

int ibx_plan_create(const ibx_problem* problems, int n_problems, int kernel, int precision, ibx_plan** plan);
/* As ibx_plan_create, with separate data for interpolation: spreading
 * reads Q and adds into q of `problems`, interpolation reads q and writes Q
 * of `interp_problems`.  Both arrays must describe the same geometry and the
 * same marker positions X (one binning serves both). */
int ibx_plan_create2(const ibx_problem* problems, const ibx_problem* interp_problems, int n_problems, int kernel,
                     int precision, ibx_plan** plan);
/* ibx_plan_create2 with a tile shape (no reference counterpart; chosen by
 * the autotuner): 0 = 8x8x8 cells in 3D, 16x16 in 2D (the default);
 * 1 = 16x8x8 in 3D, 32x16 in 2D.  ibx_plan_tile_shape returns the shape id
 * and, when edges is not NULL, the tile edges per dimension. */
int ibx_plan_create3(const ibx_problem* problems, const ibx_problem* interp_problems, int n_problems, int kernel,
                     int precision, int tile_shape, ibx_plan** plan);
int ibx_plan_tile_shape(const ibx_plan* plan, int* edges);
int ibx_plan_bin(ibx_plan* plan, void* stream);
/* One whole step: ibx_plan_bin on `stream`, then ibx_plan_spread and
 * ibx_plan_interpolate on two streams owned by the plan, running
 * concurrently (they read the same bins and write different arrays; the
 * spread's stream has the device's greatest priority, the interpolation's
 * the least, so the longer phase gets the SMs first), both joined back into
 * `stream` before the call's work ends.  The binning's last kernel (the
 * placement of the sparse-homed markers' visits) runs on `stream` beside
 * them: only the per-visit spread waits for it.  Graph-capturable like the
 * others. */
int ibx_plan_step(ibx_plan* plan, void* stream);
/* One copy of ibx_plan_step_io: `bytes` bytes from src to dst, either of
 * them host or device memory (cudaMemcpyDefault).  Host buffers must be
 * page-locked for the copies to run beside the kernels (and for the call to
 * be captured in a CUDA graph). */
typedef struct ibx_transfer
{
    void* dst;
    const void* src;
    size_t bytes;
} ibx_transfer;
/* ibx_plan_step with the step's host transfers ordered around it, for a
 * caller whose marker data live in host memory (no reference counterpart:
 * the reference's LData are host arrays, which this call moves in and out).
 * in_X (positions) are copied first, on `stream` -- or, when in_X is one
 * copy from page-locked host memory onto the plan's whole position array
 * (every problem's X one array in marker order), read by the binning kernel
 * straight from the host buffer and stored into the array on the way;
 * in_Q (the values to spread) on a stream of the plan behind them, beside
 * the binning, and the
 * spread waits for them; out_Q (the interpolated values) are copied as soon
 * as the interpolation ends, beside the rest of the spread (with out_Q the
 * concurrent mode gives the interpolation the greater stream priority, so
 * that it ends first).  Any count may be 0.  Everything is joined back into `stream` (also after a failure);
 * graph-capturable with page-locked host buffers. */
int ibx_plan_step_io(ibx_plan* plan, const ibx_transfer* in_X, int n_in_X, const ibx_transfer* in_Q, int n_in_Q,
                     const ibx_transfer* out_Q, int n_out_Q, void* stream);
/* A step of ibx_plan_step_io (any counts 0: of ibx_plan_step) captured on
 * `stream` into a CUDA graph and instantiated so that its kernels keep the
 * priorities of the plan's streams (cudaGraphInstantiateFlagUseNodePriority:
 * a graph instantiated without it runs every kernel at the priority of the
 * stream it is launched into, and the spread then no longer comes first).
 * No reference counterpart: the graph of a time stepper's step.  `stream`
 * must not be the legacy default stream (it cannot be captured); host
 * buffers must be page-locked.  The graph holds the plan's buffers and the
 * transfers' addresses: launch it while they live, destroy it before the
 * plan.  ibx_graph_launch replays the step on any stream; ibx_graph_kernels
 * is the number of library kernels one launch runs. */
typedef struct ibx_graph ibx_graph;
int ibx_plan_graph(ibx_plan* plan, const ibx_transfer* in_X, int n_in_X, const ibx_transfer* in_Q, int n_in_Q,
                   const ibx_transfer* out_Q, int n_out_Q, void* stream, ibx_graph** graph);
int ibx_graph_launch(ibx_graph* graph, void* stream);
int ibx_graph_kernels(const ibx_graph* graph);
int ibx_graph_destroy(ibx_graph* graph);
int ibx_plan_spread(ibx_plan* plan, void* stream);
int ibx_plan_interpolate(ibx_plan* plan, void* stream);
/* Status of the marker data seen by the last ibx_plan_bin (synchronises
 * the stream, then clears the word): IBX_OK, IBX_E_NONFINITE (a position
 * was NaN or infinite; that marker was skipped), IBX_E_TOO_LARGE (a list
 * capacity overflowed) or IBX_E_TIMEOUT (a bounded wait gave up: for a
 * staged copy, the interpolated values are incomplete; in step mode 2, for
 * the dense spread, the per-visit spread went ahead without it). */
int ibx_plan_status(ibx_plan* plan, void* stream, int* status);
/* Copy the binning of the last ibx_plan_bin to host arrays (any may be
 * NULL; synchronises the device).  Markers are numbered across problems in
 * order.  base_c / base_s: 3 ints per marker, the stencil base index of the
 * cell-centred and of the staggered position per dimension, relative to
 * ilower and shifted by a multiple of N into [0, N) (base_c); home_tile: the
 * tile owning the marker; tile_start: n_tiles+1 offsets of each tile's
 * markers in home_list. */
int ibx_plan_get_bins(const ibx_plan* plan, int* base_c, int* base_s, int* home_tile, int* tile_start,
                      int* home_list);
/* Number of tiles of the plan (all problems). */
int ibx_plan_n_tiles(const ibx_plan* plan);

/* Tuning knobs of a plan's spread (no reference counterpart; set by the
 * autotuner of the Python package, ibamr_gb300/tuning.py):
 *   item_units           home units (runs of markers with equal stencil
 *                        bases) per CTA of the dense-tile kernel, 32..256;
 *   dense_min            a tile homing more markers than this is spread by
 *                        the dense-tile kernel (tile + halo region in shared
 *                        memory), the others by the per-visit kernel;
 *   dense_blocks_per_sm  CTAs per SM of the dense-tile kernel, 1..32.
 * Results do not depend on them beyond FP32 rounding.  Takes effect at the
 * next ibx_plan_bin. */
int ibx_plan_set_tuning(ibx_plan* plan, int item_units, int dense_min, int dense_blocks_per_sm);
int ibx_plan_get_tuning(const ibx_plan* plan, int* item_units, int* dense_min, int* dense_blocks_per_sm);
/* Form of the per-visit spread kernel (no reference counterpart; chosen by
 * the autotuner): 0 = the in-tile points of 32 visits flattened over the
 * lanes, 1 = one lane per (visit, component) with all components of the
 * tile accumulated at once, 2 = the tile gathered: each lane owns values of
 * the tile in registers and adds every visit's separable weights, no
 * atomics (default), 3 = form 2 with each visit's tile-restricted weight
 * vectors assembled in registers and written with 16-byte stores (fewer
 * shared-memory accesses, more arithmetic).  Same results up to FP32
 * rounding. */
int ibx_plan_set_visit_kernel(ibx_plan* plan, int form);
int ibx_plan_get_visit_kernel(const ibx_plan* plan);
/* Form of the interpolation (no reference counterpart; chosen by the
 * autotuner): 0 = every marker in chunks of consecutive home-order markers
 * (default); 1 = markers of dense home tiles interpolated per home unit (the
 * unit's stencil values loaded once, every marker of the unit summed from
 * them), the others in chunks; 2 = every marker in chunks in the caller's
 * marker order, which needs only the stencil records, so that
 * ibx_plan_step (concurrent mode) starts it beside the counting sort;
 * 3 = every marker from its home tile's region of the grid staged in shared
 * memory (tensor-memory-access copies for regions inside the grid, plain
 * loads for regions across the periodic boundary), the next tile's copies in
 * flight while one is evaluated; 4 = markers of dense home tiles as in 3,
 * the others in chunks.  Every form sums in the same order: identical
 * results. */
int ibx_plan_set_interp_kernel(ibx_plan* plan, int form);
int ibx_plan_get_interp_kernel(const ibx_plan* plan);
/* How ibx_plan_step orders spread and interpolation after the binning (no
 * reference counterpart; chosen by the autotuner): 1 = concurrently, the
 * interpolation on a stream of the plan forked from and joined back to the
 * caller's stream, the spread's stream of the device's greatest priority
 * (default); 3 = concurrently with both streams of the same priority; 4 =
 * concurrently with the interpolation's stream of the greatest priority (the
 * shorter phase first, then the spread alone; the fastest order for some
 * marker sets); 0 = one after the other on the caller's
 * stream, the interpolation first; 2 = both in one persistent launch on the caller's stream, whose
 * blocks take the dense spread's work items, the interpolation of the same
 * items, the interpolation of the other markers and then the per-visit
 * spread of the tiles from one work counter (the interpolation form and the
 * per-visit form set by ibx_plan_set_interp_kernel / _visit_kernel do not
 * apply: it runs forms 1 and 2).  Same results: the interpolation bit for
 * bit, the spread to rounding (its atomic additions come in another order).
 * The per-visit spread of mode 2 waits, at most about a second, for the
 * dense spread of every tile to finish; a wait that runs out is reported
 * by ibx_plan_status as IBX_E_TIMEOUT. */
int ibx_plan_set_step_mode(ibx_plan* plan, int mode);
int ibx_plan_get_step_mode(const ibx_plan* plan);
/* Most markers per home unit (1..32; no reference counterpart; chosen by the
 * autotuner).  A home unit is a run of markers of one home tile that share
 * every stencil base, spread by one thread per component of the dense-tile
 * kernel; shorter units balance the threads of a warp at the cost of more
 * merges.  Default 32.  Takes effect at the next ibx_plan_bin. */
int ibx_plan_set_unit_cap(ibx_plan* plan, int cap);
int ibx_plan_get_unit_cap(const ibx_plan* plan);
/* Number of the plan's problems whose interpolation sources the staged
 * forms (3, 4) load by tensor copies: the x extent a multiple of 4 values,
 * every grid dimension at least the staged box, 16-byte aligned arrays, and
 * a driver that encodes tensor maps.  The others are staged with plain
 * loads.  No reference counterpart. */
int ibx_plan_tma_problems(const ibx_plan* plan);
/* Bytes of device scratch the plan holds. */
long long ibx_plan_scratch_bytes(const ibx_plan* plan);
int ibx_plan_destroy(ibx_plan* plan);

/* ---- allocation-free spreading ----------------------------------------- */
/* No counterpart in the reference (IBAMR's LEInteractor runs on the CPU and
 * allocates freely); it exists for callers of this library that cannot
 * allocate device memory: real-time or fault-handling host paths, where a
 * cudaMalloc may block on the driver or fail when memory is short, and
 * embeddings whose own memory pool owns the whole device, so that a library
 * may not allocate beside it.
 *
 * ibx_spread_noalloc: the binned mixed-precision spread of ibx_plan_bin +
 * ibx_plan_spread for one IBX_MODE_PERIODIC problem (float q and Q), with
 * every scratch buffer placed in a fixed 8 MiB array inside the library
 * (held on every GPU that loads it until the process exits).  It calls no
 * allocating routine.  Limits: at most IBX_NOALLOC_MAX_MARKERS markers and
 * IBX_NOALLOC_MAX_TILES grid tiles (8^3 cells in 3D, 16^2 in 2D), and the
 * scratch the problem needs must fit the array (grids whose cell count is
 * not a multiple of the tile edge need more visit slots per marker); larger
 * problems return IBX_E_TOO_LARGE and nothing is launched.  The first call
 * on a device, with that device current, looks up the array's address.  All
 * calls share the array, which keeps the last call's contents: each call
 * clears what must start at zero, and calls whose work overlaps on the GPU
 * race and must be serialised.
 *
 * status: a DEVICE int, or NULL.  When given, it receives, in stream order
 * after the spread, IBX_OK, IBX_E_NONFINITE (a marker position was NaN or
 * infinite; that marker was skipped) or IBX_E_TOO_LARGE (a list capacity
 * overflowed; the result is incomplete). */
#define IBX_NOALLOC_MAX_MARKERS 32768
#define IBX_NOALLOC_MAX_TILES 4096
int ibx_spread_noalloc(const ibx_problem* problem, int kernel, int* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* IBX_H */
