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

// Generic (marker-parallel, reference-faithful FP64) spread / interpolate.
int launch_generic(bool spread, int dim, int kernel, const ProbArg& arg, cudaStream_t stream);

} // namespace ibx
