// ibx_indexset.cu -- the cached index sets of one patch on the device
// (ibx_cache_local_indices in include/ibx.h).
//
// LIndexSetData::cacheLocalIndices (ibtk/src/lagrangian/LIndexSetData.cpp:
// 50-140) flattens the marker sets of every cell of a patch's ghost box into
// a list of local marker indices and, per entry, the periodic shift
// offset * dx with offset = -periodic_shift on a cell below ilower of a patch
// touching the lower periodic boundary, +periodic_shift above iupper at the
// upper one, 0 elsewhere (LIndexSetData.cpp:83-100).  The cells hold the
// markers and their periodic images: a marker whose cell index
// (IndexUtilities::getCellIndex, ibtk/include/ibtk/private/
// IndexUtilities-inl.h:52-75, on the patch geometry) is c appears in cell
// c + k * periodic_shift for every k in {-1, 0, 1}^dim (k_d != 0 only where
// periodic_shift_d != 0) that lies in the box and whose shift rule gives
// back k * periodic_shift.
//
// Two passes over the markers: count each marker's images, exclusive scan,
// write each marker's images at its offset.  Entries come in marker order,
// images of one marker in the order k = (-1,-1,-1), (0,-1,-1), (1,-1,-1),
// ..., x fastest -- a fixed order, so the lists are reproducible bit for bit.

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

namespace ibx
{
int exclusive_scan(int* data, int n, int count, int* tmp, cudaStream_t s);

namespace
{
struct IndexSetArgs
{
    int dim;
    int ilower[3], iupper[3];
    double x_lower[3], x_upper[3], dx[3];
    int touches_lower[3], touches_upper[3];
    int shift[3];          // periodic_shift (cells)
    int lo[3], hi[3];      // the box whose cells are selected (patch box grown by the ghost width)
};

// getCellIndex in FP64, the reference's arithmetic: false for a non-finite
// position (no cell).
__device__ __forceinline__ bool
cell_index(const IndexSetArgs& A, const double* X, int* c)
{
    for (int d = 0; d < A.dim; ++d)
    {
        const double x = X[d];
        if (!isfinite(x)) return false;
        const double dl = __dsub_rn(x, A.x_lower[d]);
        const double du = __dsub_rn(x, A.x_upper[d]);
        double v;
        if (fabs(dl) <= fabs(du))
            v = __dadd_rn((double)A.ilower[d], floor(__ddiv_rn(dl, A.dx[d])));
        else
            v = __dadd_rn(__dadd_rn((double)A.iupper[d], floor(__ddiv_rn(du, A.dx[d]))), 1.0);
        if (!(v > -1.0e9 && v < 1.0e9)) return false; // far outside every box
        c[d] = (int)v;
    }
    return true;
}

// Offset of image k along d if the image is selected, or INT_MIN.
__device__ __forceinline__ bool
image_ok(const IndexSetArgs& A, const int* c, int m, int* off)
{
    int t = m;
    for (int d = 0; d < A.dim; ++d)
    {
        const int k = t % 3 - 1;
        t /= 3;
        if (k != 0 && A.shift[d] == 0) return false;
        const int i = c[d] + k * A.shift[d];
        if (i < A.lo[d] || i > A.hi[d]) return false;
        const int o = (A.touches_lower[d] && i < A.ilower[d])   ? -A.shift[d]
                      : (A.touches_upper[d] && i > A.iupper[d]) ? A.shift[d]
                                                                : 0;
        if (o != k * A.shift[d]) return false;
        off[d] = o;
    }
    return true;
}

__global__ void
count_images(const IndexSetArgs A, const double* X, int n, int* counts)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int c[3], off[3];
    int cnt = 0;
    if (cell_index(A, X + (long long)A.dim * s, c))
    {
        const int nimg = A.dim == 2 ? 9 : 27;
        for (int m = 0; m < nimg; ++m) cnt += image_ok(A, c, m, off) ? 1 : 0;
    }
    counts[s] = cnt;
}

__global__ void
write_images(const IndexSetArgs A, const double* X, int n, const int* offsets, int capacity, int* local_indices,
             double* shifts, int* cells)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int c[3], off[3];
    if (!cell_index(A, X + (long long)A.dim * s, c)) return;
    int e = offsets[s];
    const int nimg = A.dim == 2 ? 9 : 27;
    for (int m = 0; m < nimg; ++m)
    {
        if (!image_ok(A, c, m, off)) continue;
        if (e < capacity)
        {
            local_indices[e] = s;
            for (int d = 0; d < A.dim; ++d)
            {
                if (shifts) shifts[(long long)A.dim * e + d] = (double)off[d] * A.dx[d];
                if (cells) cells[(long long)A.dim * e + d] = c[d] + off[d];
            }
        }
        ++e;
    }
}
} // namespace
} // namespace ibx

extern "C" int
ibx_cache_local_indices(const ibx_patch_geometry* patch, const int* periodic_shift, const int* ghost_width,
                        int want_ghost_box, const double* X, int n_markers, int capacity, int* local_indices,
                        double* periodic_shifts, int* cells, int* count, void* stream)
{
    using namespace ibx;
    if (!patch || !periodic_shift || !ghost_width || !count || n_markers < 0 || capacity < 0) return IBX_E_ARG;
    if (patch->dim != 2 && patch->dim != 3) return IBX_E_ARG;
    if (n_markers > 0 && !X) return IBX_E_ARG;
    if (capacity > 0 && !local_indices) return IBX_E_ARG;
    *count = 0;
    IndexSetArgs A{};
    A.dim = patch->dim;
    for (int d = 0; d < A.dim; ++d)
    {
        if (!(patch->dx[d] > 0.0) || patch->iupper[d] < patch->ilower[d] || ghost_width[d] < 0 ||
            periodic_shift[d] < 0)
            return IBX_E_ARG;
        A.ilower[d] = patch->ilower[d];
        A.iupper[d] = patch->iupper[d];
        A.x_lower[d] = patch->x_lower[d];
        A.x_upper[d] = patch->x_upper[d];
        A.dx[d] = patch->dx[d];
        A.touches_lower[d] = patch->touches_periodic_lower[d] != 0;
        A.touches_upper[d] = patch->touches_periodic_upper[d] != 0;
        A.shift[d] = periodic_shift[d];
        const int g = want_ghost_box ? ghost_width[d] : 0;
        A.lo[d] = patch->ilower[d] - g;
        A.hi[d] = patch->iupper[d] + g;
    }
    if (n_markers == 0) return IBX_OK;
    if ((long long)n_markers + 1 > 2048LL * 2048LL) return IBX_E_TOO_LARGE; // two-level scan
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // per-marker counts, scanned in place into offsets ([n + 1]), and the scan's block sums
    int* scratch = nullptr;
    const size_t ints = (size_t)n_markers + 1 + SCAN_TMP_INTS;
    if (cudaMallocAsync(reinterpret_cast<void**>(&scratch), ints * sizeof(int), s) != cudaSuccess) return IBX_E_OOM;
    int rc = IBX_OK;
    const unsigned blocks = (unsigned)((n_markers + 255) / 256);
    if (cudaMemsetAsync(scratch + n_markers, 0, sizeof(int), s) != cudaSuccess) rc = IBX_E_CUDA;
    if (!rc)
    {
        count_images<<<blocks, 256, 0, s>>>(A, X, n_markers, scratch);
        note_launches(1);
        if (cudaGetLastError() != cudaSuccess) rc = IBX_E_CUDA;
    }
    if (!rc) rc = exclusive_scan(scratch, n_markers + 1, 1, scratch + n_markers + 1, s);
    int total = 0;
    if (!rc && (cudaMemcpyAsync(&total, scratch + n_markers, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess))
        rc = IBX_E_CUDA;
    if (!rc && total > 0 && capacity > 0)
    {
        write_images<<<blocks, 256, 0, s>>>(A, X, n_markers, scratch, capacity, local_indices, periodic_shifts,
                                            cells);
        note_launches(1);
        if (cudaGetLastError() != cudaSuccess) rc = IBX_E_CUDA;
    }
    if (cudaFreeAsync(scratch, s) != cudaSuccess && !rc) rc = IBX_E_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = IBX_E_CUDA;
    *count = total;
    if (!rc && total > capacity) rc = IBX_E_TOO_LARGE;
    return rc;
}
