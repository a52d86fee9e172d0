// Replays of the reference's own LEInteractor tests through the C++ layer of
// libibx (include/ibx_leinteractor.h), compiled with -DNDIM=2 or -DNDIM=3.
//
//   leinteractor_test kat <KERNEL>
//       tests/interpolate/interpolate_01.cpp with use_exact = TRUE: a
//       multilinear field on the level-1 patch [8,15]^d (dx = 1/32) of an
//       8^d domain, 100 std::mt19937(42) points, every component must be
//       reproduced to 1e-12 (1e-10 for stencils wider than 4).  Prints OK.
//   leinteractor_test spread <cell|side>
//       tests/IBTK/ghost_accumulation_01 with fill_test = "spread" on one
//       non-periodic 8^d patch, ghost width 2, PIECEWISE_LINEAR: prints the
//       patch values as array(i,j[,k]) = value, the reference's format.
#include "ibx_leinteractor.h"

#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <vector>

using ibx::samrai::Box;
using ibx::samrai::CellData;
using ibx::samrai::Index;
using ibx::samrai::IntVector;
using ibx::samrai::Patch;
using ibx::samrai::SideData;

namespace
{
double
exact(const double* x)
{
#if NDIM == 2
    return 1 + 2 * x[0] + 3 * x[1] + 4 * x[0] * x[1];
#else
    return 1 + 2 * x[0] + 3 * x[1] - x[2] + 4 * x[0] * x[1] + 2 * x[0] * x[2] + 3 * x[0] * x[1] * x[2];
#endif
}

int
run_kat(const std::string& kernel)
{
    const int g = IBTK::LEInteractor::getMinimumGhostWidth(kernel);
    Patch patch;
    for (int d = 0; d < NDIM; ++d)
    {
        patch.box.lo(d) = 8;
        patch.box.hi(d) = 15;
        patch.geom.dx[d] = 1.0 / 32.0;
        patch.geom.x_lower[d] = 0.25;
        patch.geom.x_upper[d] = 0.5;
    }
    CellData q;
    q.box = patch.box;
    q.gcw = IntVector(g);
    q.depth = NDIM;
    const long long vol = IBTK::ibx_detail::array_values(q.box, q.gcw, -1);
    std::vector<double> host(vol * NDIM);
    // exact field at every cell centre, ghosts included
    long long n[3] = { 1, 1, 1 };
    for (int d = 0; d < NDIM; ++d) n[d] = q.box.hi(d) - q.box.lo(d) + 1 + 2 * g;
    for (long long k2 = 0; k2 < n[2]; ++k2)
        for (long long k1 = 0; k1 < n[1]; ++k1)
            for (long long k0 = 0; k0 < n[0]; ++k0)
            {
                const long long kk[3] = { k0, k1, k2 };
                double x[3] = { 0, 0, 0 };
                for (int d = 0; d < NDIM; ++d)
                    x[d] = patch.geom.x_lower[d] + (kk[d] - g + 0.5) * patch.geom.dx[d];
                const double v = exact(x);
                for (int dd = 0; dd < NDIM; ++dd) host[vol * dd + k0 + n[0] * (k1 + n[1] * k2)] = v;
            }
    q.data = host.data();
    std::mt19937 std_seq(42u);
    std::uniform_real_distribution<double> distribution(0.25, 0.5);
    std::vector<double> X(NDIM * 100), Q(NDIM * 100, std::numeric_limits<double>::max());
    for (double& v : X) v = distribution(std_seq);
    IBTK::LEInteractor::interpolate(Q, NDIM, X, NDIM, q, patch, patch.box, kernel);
    const double tol = IBTK::LEInteractor::getStencilSize(kernel) > 4 ? 1e-10 : 1e-12;
    bool ok = true;
    for (int s = 0; s < 100; ++s)
        for (int d = 0; d < NDIM; ++d)
        {
            const double err = std::abs(Q[NDIM * s + d] - exact(&X[NDIM * s]));
            if (err > tol)
            {
                std::printf("point %d component %d error %g\n", s, d, err);
                ok = false;
            }
        }
    if (ok) std::printf("OK\n");
    return ok ? 0 : 1;
}

template <class Data>
void
print_array(const Data& q, const std::vector<double>& host, int axis, long long off, const Box& patch_box)
{
    const int g = q.gcw(0);
    long long n[3] = { 1, 1, 1 };
    int hi[3] = { 0, 0, 0 };
    for (int d = 0; d < NDIM; ++d)
    {
        n[d] = patch_box.hi(d) - patch_box.lo(d) + 1 + 2 * g + (d == axis ? 1 : 0);
        hi[d] = patch_box.hi(d) + (d == axis ? 1 : 0);
    }
    const int k_lo = NDIM == 3 ? patch_box.lo(NDIM - 1) : 0;
    for (int k = k_lo; k <= (NDIM == 3 ? hi[2] : 0); ++k)
        for (int j = patch_box.lo(1); j <= hi[1]; ++j)
            for (int i = patch_box.lo(0); i <= hi[0]; ++i)
            {
                const long long o = (i - patch_box.lo(0) + g) +
                                    n[0] * ((j - patch_box.lo(1) + g) + n[1] * (NDIM == 3 ? (k - k_lo + g) : 0));
                if (NDIM == 3)
                    std::printf("array(%d,%d,%d) = %.17g\n", i, j, k, host[off + o]);
                else
                    std::printf("array(%d,%d) = %.17g\n", i, j, host[off + o]);
            }
}

int
run_spread(const std::string& centering)
{
    const bool side = centering == "side";
    Patch patch;
    for (int d = 0; d < NDIM; ++d)
    {
        patch.box.lo(d) = 0;
        patch.box.hi(d) = 7;
        patch.geom.dx[d] = 1.0 / 8.0;
        patch.geom.x_lower[d] = 0.0;
        patch.geom.x_upper[d] = 1.0;
        patch.geom.touches_regular[d][0] = patch.geom.touches_regular[d][1] = 1;
    }
    const int Q_depth = side ? NDIM : 1;
    std::mt19937 std_seq(42u);
    std::uniform_real_distribution<double> distribution(0.0, 1.0);
    std::vector<double> Q(Q_depth * 100), X(NDIM * 100);
    for (double& v : Q) v = distribution(std_seq);
    for (double& v : X) v = distribution(std_seq);
    const IntVector gcw(2);
    if (side)
    {
        // device-resident patch data
        SideData q;
        q.box = patch.box;
        q.gcw = gcw;
        q.on_device = true;
        std::vector<long long> nval(NDIM);
        for (int a = 0; a < NDIM; ++a)
        {
            nval[a] = IBTK::ibx_detail::array_values(q.box, gcw, a);
            std::vector<double> zeros(nval[a], 0.0);
            void* p = nullptr;
            if (ibx_device_alloc(&p, nval[a] * 8) || ibx_memcpy(p, zeros.data(), nval[a] * 8, 1)) return 2;
            q.data[a] = static_cast<double*>(p);
        }
        IBTK::LEInteractor::spread(q, Q, Q_depth, X, NDIM, patch, patch.box, "PIECEWISE_LINEAR");
        for (int a = 0; a < NDIM; ++a)
        {
            std::vector<double> host(nval[a]);
            if (ibx_memcpy(host.data(), q.data[a], nval[a] * 8, 0)) return 2;
            std::printf("Array side normal = %d\n", a);
            print_array(q, host, a, 0, patch.box);
            ibx_device_free(q.data[a]);
        }
    }
    else
    {
        // host-resident patch data (copied in and out by the call)
        CellData q;
        q.box = patch.box;
        q.gcw = gcw;
        q.depth = 1;
        std::vector<double> host(IBTK::ibx_detail::array_values(q.box, gcw, -1), 0.0);
        q.data = host.data();
        IBTK::LEInteractor::spread(q, Q, Q_depth, X, NDIM, patch, patch.box, "PIECEWISE_LINEAR");
        std::printf("Array depth = 0\n");
        print_array(q, host, -1, 0, patch.box);
    }
    return 0;
}
} // namespace

int
main(int argc, char** argv)
{
    if (argc < 3) return 2;
    try
    {
        if (std::strcmp(argv[1], "kat") == 0) return run_kat(argv[2]);
        if (std::strcmp(argv[1], "spread") == 0) return run_spread(argv[2]);
    }
    catch (const std::exception& e)
    {
        std::printf("error: %s\n", e.what());
        return 3;
    }
    return 2;
}
