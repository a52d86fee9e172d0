// ibx_redistribute.cu -- markers assigned to the patches of a level and
// grouped by patch on the device (ibx_redistribute in include/ibx.h).
//
// The reference moves Lagrangian markers between patches in
// LDataManager::redistribute (src/IB/LDataManager.cpp:1351-1522); which
// patch owns a marker is decided by IndexUtilities::getCellIndex
// (ibtk/include/ibtk/private/IndexUtilities-inl.h:52-75), evaluated with each
// patch's geometry: the cell index is measured from the nearer of the
// patch's lower and upper faces.  Here every marker takes the first patch (in
// the given order) whose cell box holds that index, with the reference's FP64
// expression, and an integer counting sort groups the markers by owner.

#include "ibx_internal.h"
#include "../../include/ibx.h"


namespace ibx
{
namespace
{
__device__ __forceinline__ int
cell_index_1d(double X, double xlo, double xup, double dx, int ilo, int iup)
{
    const double dl = X - xlo, du = X - xup;
    if (fabs(dl) <= fabs(du)) return (int)(ilo + floor(dl / dx));
    return (int)(iup + floor(du / dx) + 1);
}

__global__ void
locate_kernel(int dim, const ibx_patch_box* boxes, int n_patches, const double* X, int n_markers, int* owner,
              int* counts)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_markers) return;
    int own = -1;
    for (int p = 0; p < n_patches && own < 0; ++p)
    {
        const ibx_patch_box& B = boxes[p];
        bool in = true;
        for (int d = 0; d < dim; ++d)
        {
            const int i = cell_index_1d(X[dim * (long long)s + d], B.x_lower[d], B.x_upper[d], B.dx[d], B.ilower[d],
                                        B.iupper[d]);
            in = in && i >= B.ilower[d] && i <= B.iupper[d];
        }
        if (in) own = p;
    }
    owner[s] = own;
    atomicAdd(&counts[own < 0 ? n_patches : own], 1);
}

// Exclusive scan of counts[0..n] into offsets[0..n] (one block; n small).
__global__ void
offsets_kernel(const int* counts, int n, int* offsets, int* cursors)
{
    __shared__ int partial[1024];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per;
    int sum = 0;
    for (int i = b; i < b + per && i < n; ++i) sum += counts[i];
    partial[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int run = 0;
        for (int t = 0; t < (int)blockDim.x; ++t)
        {
            const int v = partial[t];
            partial[t] = run;
            run += v;
        }
    }
    __syncthreads();
    int run = partial[threadIdx.x];
    for (int i = b; i < b + per && i < n; ++i)
    {
        offsets[i] = run;
        cursors[i] = 0;
        run += counts[i];
    }
    if (threadIdx.x == blockDim.x - 1) offsets[n] = run;
}

__global__ void
place_kernel(const int* owner, int n_markers, int n_patches, const int* offsets, int* cursors, int* order)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_markers) return;
    const int o = owner[s] < 0 ? n_patches : owner[s];
    order[offsets[o] + atomicAdd(&cursors[o], 1)] = s;
}
} // namespace
} // namespace ibx

extern "C" int
ibx_redistribute(int dim, const ibx_patch_box* patches, int n_patches, const double* X, int n_markers, int* owner,
                 int* order, int* patch_offsets, void* stream)
{
    using namespace ibx;
    if ((dim != 2 && dim != 3) || n_patches < 0 || n_markers < 0) return IBX_E_ARG;
    if ((n_patches > 0 && !patches) || !patch_offsets || (n_markers > 0 && (!X || !owner || !order)))
        return IBX_E_ARG;
    for (int p = 0; p < n_patches; ++p)
        for (int d = 0; d < dim; ++d)
            if (!(patches[p].dx[d] > 0.0) || patches[p].iupper[d] < patches[p].ilower[d]) return IBX_E_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Stream-ordered scratch: the patch table, counts and cursors.
    const size_t tb = sizeof(ibx_patch_box) * (size_t)(n_patches > 0 ? n_patches : 1);
    const size_t cb = sizeof(int) * (size_t)(n_patches + 2); // counts of patches + unowned (+ pad)
    void* scratch = nullptr;
    if (cudaMallocAsync(&scratch, tb + 2 * cb, s) != cudaSuccess) return IBX_E_OOM;
    char* base = static_cast<char*>(scratch);
    ibx_patch_box* dboxes = reinterpret_cast<ibx_patch_box*>(base);
    int* counts = reinterpret_cast<int*>(base + tb);
    int* cursors = reinterpret_cast<int*>(base + tb + cb);
    int rc = IBX_OK;
    if ((n_patches > 0 && cudaMemcpyAsync(dboxes, patches, sizeof(ibx_patch_box) * n_patches, cudaMemcpyHostToDevice,
                                          s) != cudaSuccess) ||
        cudaMemsetAsync(counts, 0, cb, s) != cudaSuccess)
        rc = IBX_E_CUDA;
    if (!rc && n_markers > 0)
    {
        locate_kernel<<<(n_markers + 255) / 256, 256, 0, s>>>(dim, dboxes, n_patches, X, n_markers, owner, counts);
        note_launches(1);
    }
    if (!rc)
    {
        offsets_kernel<<<1, 1024, 0, s>>>(counts, n_patches + 1, patch_offsets, cursors);
        note_launches(1);
    }
    if (!rc && n_markers > 0)
    {
        place_kernel<<<(n_markers + 255) / 256, 256, 0, s>>>(owner, n_markers, n_patches, patch_offsets, cursors,
                                                              order);
        note_launches(1);
    }
    if (!rc && cudaGetLastError() != cudaSuccess) rc = IBX_E_CUDA;
    cudaFreeAsync(scratch, s);
    // the pageable patch table must outlive its copy
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = IBX_E_CUDA;
    return rc;
}
