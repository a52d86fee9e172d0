// ibx_ghost.cu -- ghost accumulation and periodic ghost fill of patch data
// on the device (ibx_accumulate_ghosts / ibx_fill_ghosts in include/ibx.h).
//
// After spreading in IBX_MODE_PATCH the ghost cells of a patch hold
// contributions that belong to periodic images of interior values; the
// reference sums them with SAMRAIGhostDataAccumulator::accumulateGhostData
// (ibtk/src/math/SAMRAIGhostDataAccumulator.cpp:295-353: every ghosted value
// is added into its degree of freedom, then every copy of the DOF receives
// the total).  Before interpolation the ghosts are filled from the interior
// (the periodic part of a SAMRAI refine schedule).  Both are done here for a
// patch that covers the whole domain, in FP64, with the data layout of
// IBX_MODE_PATCH (SAMRAI ghosted arrays, side data on toSideBox).

#include "ibx_internal.h"
#include "../../include/ibx.h"

namespace ibx
{
namespace
{
struct GhostGeom
{
    int dim, ncomp, depth, side;
    int ilo[3], ihi[3], gcw[3], periodic[3];
    double* q[3];
};

// Array box of component c: [lo, hi] (ghosts included) and extents.
__device__ __forceinline__ void
comp_box(const GhostGeom& G, int c, int* glo, int* ghi, int* n)
{
    for (int d = 0; d < 3; ++d)
    {
        if (d >= G.dim)
        {
            glo[d] = ghi[d] = 0;
            n[d] = 1;
            continue;
        }
        const int bhi = G.ihi[d] + ((G.side && d == c) ? 1 : 0);
        glo[d] = G.ilo[d] - G.gcw[d];
        ghi[d] = bhi + G.gcw[d];
        n[d] = ghi[d] - glo[d] + 1;
    }
}

// One thread per (degree of freedom, component, depth): the sum over every
// array position that maps to the DOF (periodic images along periodic dims),
// taken in increasing array order, written back to all of them.
__global__ void
accumulate_kernel(const GhostGeom G, long long total)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= total) return;
    // Decode (component, depth, DOF) with the DOF index fastest.  DOFs per
    // dim: N cells along periodic dims, the (side-extended) box along others.
    long long r = t;
    int c = 0, j[3] = { 0, 0, 0 };
    long long before = 0;
    for (c = 0; c < G.ncomp; ++c)
    {
        long long cnt = G.depth;
        for (int d = 0; d < G.dim; ++d)
        {
            const int N = G.ihi[d] - G.ilo[d] + 1;
            cnt *= G.periodic[d] ? N : N + ((G.side && d == c) ? 1 : 0);
        }
        if (r < before + cnt) break;
        before += cnt;
    }
    if (c >= G.ncomp) return;
    r -= before;
    for (int d = 0; d < G.dim; ++d)
    {
        const int N = G.ihi[d] - G.ilo[d] + 1;
        const int md = G.periodic[d] ? N : N + ((G.side && d == c) ? 1 : 0);
        j[d] = G.ilo[d] + (int)(r % md);
        r /= md;
    }
    const int dd = (int)r;
    int glo[3], ghi[3], n[3];
    comp_box(G, c, glo, ghi, n);
    double* u = G.q[G.side ? c : 0];
    const long long vol = (long long)n[0] * n[1] * n[2];
    u += vol * (G.side ? 0 : dd);
    // images per dim: first image, stride and count (one image along
    // non-periodic dims)
    int first[3], stride[3], cnt[3];
    for (int d = 0; d < 3; ++d)
    {
        if (d >= G.dim)
        {
            first[d] = 0;
            stride[d] = 1;
            cnt[d] = 1;
            continue;
        }
        if (G.periodic[d])
        {
            const int N = G.ihi[d] - G.ilo[d] + 1;
            // smallest i >= glo with i = j (mod N)
            const int k = (j[d] - glo[d]) / N;
            first[d] = j[d] - k * N;
            stride[d] = N;
            cnt[d] = (ghi[d] - first[d]) / N + 1;
        }
        else
        {
            first[d] = j[d];
            stride[d] = 1;
            cnt[d] = 1;
        }
    }
    double sum = 0.0;
    for (int a2 = 0; a2 < cnt[2]; ++a2)
        for (int a1 = 0; a1 < cnt[1]; ++a1)
            for (int a0 = 0; a0 < cnt[0]; ++a0)
            {
                const int i0 = first[0] + a0 * stride[0] - glo[0];
                const int i1 = first[1] + a1 * stride[1] - glo[1];
                const int i2 = first[2] + a2 * stride[2] - glo[2];
                sum += u[i0 + (long long)n[0] * (i1 + (long long)n[1] * i2)];
            }
    for (int a2 = 0; a2 < cnt[2]; ++a2)
        for (int a1 = 0; a1 < cnt[1]; ++a1)
            for (int a0 = 0; a0 < cnt[0]; ++a0)
            {
                const int i0 = first[0] + a0 * stride[0] - glo[0];
                const int i1 = first[1] + a1 * stride[1] - glo[1];
                const int i2 = first[2] + a2 * stride[2] - glo[2];
                u[i0 + (long long)n[0] * (i1 + (long long)n[1] * i2)] = sum;
            }
}

// One thread per array position: a position outside the cell box along a
// periodic dim takes the value of its image inside (side faces on the upper
// box face included, so face N takes face 0).
__global__ void
fill_kernel(const GhostGeom G, int c, long long total)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= total) return;
    int glo[3], ghi[3], n[3];
    comp_box(G, c, glo, ghi, n);
    const long long vol = (long long)n[0] * n[1] * n[2];
    const long long o = t % vol;
    const int dd = (int)(t / vol);
    const int i[3] = { (int)(o % n[0]) + glo[0], (int)((o / n[0]) % n[1]) + glo[1],
                       (int)(o / ((long long)n[0] * n[1])) + glo[2] };
    int jj[3] = { i[0], i[1], i[2] };
    bool moved = false;
    for (int d = 0; d < G.dim; ++d)
    {
        if (!G.periodic[d]) continue;
        const int N = G.ihi[d] - G.ilo[d] + 1;
        const int w = ((i[d] - G.ilo[d]) % N + N) % N + G.ilo[d];
        moved = moved || w != i[d];
        jj[d] = w;
    }
    if (!moved) return;
    double* u = G.q[G.side ? c : 0] + vol * (G.side ? 0 : dd);
    const long long src =
        (jj[0] - glo[0]) + (long long)n[0] * ((jj[1] - glo[1]) + (long long)n[1] * (jj[2] - glo[2]));
    u[o] = u[src];
}

int
make_geom(const ibx_problem* p, const int* periodic, GhostGeom& G)
{
    if (!p || !periodic) return IBX_E_ARG;
    if (p->dim != 2 && p->dim != 3) return IBX_E_ARG;
    if (p->mode != IBX_MODE_PATCH) return IBX_E_ARG;
    if (p->centering != IBX_CELL && p->centering != IBX_SIDE) return IBX_E_ARG;
    G.dim = p->dim;
    G.side = p->centering == IBX_SIDE;
    G.ncomp = G.side ? p->dim : 1;
    G.depth = G.side ? 1 : p->q_depth;
    if (G.depth < 1 || (G.side && p->q_depth != 1)) return IBX_E_DEPTH;
    for (int d = 0; d < 3; ++d)
    {
        G.ilo[d] = d < p->dim ? p->ilower[d] : 0;
        G.ihi[d] = d < p->dim ? p->iupper[d] : 0;
        G.gcw[d] = d < p->dim ? p->gcw[d] : 0;
        G.periodic[d] = d < p->dim ? (periodic[d] != 0) : 0;
        if (d < p->dim && (G.ihi[d] < G.ilo[d] || G.gcw[d] < 0)) return IBX_E_ARG;
        G.q[d] = static_cast<double*>(p->q[d]);
    }
    for (int c = 0; c < G.ncomp; ++c)
        if (!G.q[G.side ? c : 0]) return IBX_E_ARG;
    return IBX_OK;
}
} // namespace
} // namespace ibx

extern "C" {

int
ibx_accumulate_ghosts(const ibx_problem* problem, const int* periodic, void* stream)
{
    using namespace ibx;
    GhostGeom G;
    const int rc = make_geom(problem, periodic, G);
    if (rc) return rc;
    long long total = 0;
    for (int c = 0; c < G.ncomp; ++c)
    {
        long long cnt = G.depth;
        for (int d = 0; d < G.dim; ++d)
        {
            const int N = G.ihi[d] - G.ilo[d] + 1;
            cnt *= G.periodic[d] ? N : N + ((G.side && d == c) ? 1 : 0);
        }
        total += cnt;
    }
    if (total == 0) return IBX_OK;
    const long long blocks = (total + 255) / 256;
    if (blocks > 0x7fffffffLL) return IBX_E_TOO_LARGE;
    accumulate_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(G, total);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

int
ibx_fill_ghosts(const ibx_problem* problem, const int* periodic, void* stream)
{
    using namespace ibx;
    GhostGeom G;
    const int rc = make_geom(problem, periodic, G);
    if (rc) return rc;
    for (int c = 0; c < G.ncomp; ++c)
    {
        long long total = G.depth;
        for (int d = 0; d < G.dim; ++d)
            total *= G.ihi[d] - G.ilo[d] + 1 + ((G.side && d == c) ? 1 : 0) + 2 * G.gcw[d];
        const long long blocks = (total + 255) / 256;
        if (blocks > 0x7fffffffLL) return IBX_E_TOO_LARGE;
        fill_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(G, c, total);
        note_launches(1);
        if (cudaGetLastError() != cudaSuccess) return IBX_E_CUDA;
    }
    return IBX_OK;
}

} // extern "C"
