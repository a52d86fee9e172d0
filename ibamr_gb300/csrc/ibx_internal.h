// ibx_internal.h -- declarations shared by the translation units of libibx.
#pragma once

#include "ibx_device.cuh"

#include <cuda_runtime.h>

namespace ibx
{
// Problems handed to a marker-parallel launch: one inline descriptor, or a
// device table plus per-problem item offsets (work items = markers x comps).
struct ProbArg
{
    Prob one;
    const Prob* many;
    const long long* offs;
    int n;
    long long total;
};

// Host-side count of the kernels libibx has launched (ibx_kernel_launches()).
void note_launches(int n);

// Device buffers of the host-array entry points (the Fortran ABI, the C++
// LEInteractor layer through ibx_device_alloc): a memory pool of the library
// per device that keeps freed memory, so that the buffers of one call are
// reused by the next without cudaMalloc / cudaFree (which maps memory and
// synchronises the device).  Allocation and release are ordered on the
// legacy default stream; nullptr when the pool cannot serve the request.
void* staging_alloc(size_t bytes);
void staging_free(void* p);

// Generic (marker-parallel, reference-faithful FP64) spread / interpolate.
int launch_generic(bool spread, int dim, int kernel, const ProbArg& arg, cudaStream_t stream);

} // namespace ibx
