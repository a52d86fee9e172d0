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
//   leinteractor_test ldata <cell|side> <KERNEL> <N> <in.bin> <out.bin>
//       The reference's LData / LIndexSetData signatures on one patch that
//       covers a periodic unit domain of N^NDIM cells (ghost width
//       getMinimumGhostWidth): SAMRAI::tbox::Pointer handles, IBTK::LData
//       markers and forces, IBTK::LIndexSetData<IBTK::LNode> cached with
//       cacheLocalIndices(patch, periodic_shift = N).  Spread over the ghost
//       box into zeroed data (LDataManager::spread's flow), interpolate over
//       the patch box from data with periodically filled ghosts
//       (LDataManager::interp's), and interpolate over the patch box shrunk
//       by 2 cells (buildLocalIndices' general path).  in.bin: int32 n,
//       int32 depth, X (n*NDIM f64), F (n*Q_depth), u (ncomp*N^NDIM,
//       compact periodic, x fastest); out.bin: f interior (compact), U, U of
//       the sub-box (markers outside it keep the value 7).
#include "ibx_leinteractor.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
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
// Compact periodic index of cell / face i (ghosted indices wrap).
long long
compact(const int* i, int N)
{
    long long o = 0;
    for (int d = NDIM - 1; d >= 0; --d) o = o * N + (((i[d] % N) + N) % N);
    return o;
}

template <class Data>
void
fill_or_read(Data& q, const std::vector<long long>& nval, std::vector<std::vector<double>>& arrays, int ncomp,
             int depth, int N, int g, const double* u, double* f_out, bool side)
{
    // u != nullptr: every ghosted value from its periodic image of u;
    // f_out != nullptr: the interior values into the compact array
    const long long vol = (long long)std::pow(N, NDIM);
    for (int c = 0; c < ncomp; ++c)
    {
        const int axis = side ? c : -1;
        const double* base = side ? arrays[c].data() : arrays[0].data() + nval[0] * c;
        long long n[3] = { 1, 1, 1 };
        for (int d = 0; d < NDIM; ++d) n[d] = N + 2 * g + (d == axis ? 1 : 0);
        for (long long k2 = 0; k2 < n[2]; ++k2)
            for (long long k1 = 0; k1 < n[1]; ++k1)
                for (long long k0 = 0; k0 < n[0]; ++k0)
                {
                    const int i[3] = { (int)k0 - g, (int)k1 - g, (int)k2 - g };
                    const long long o = k0 + n[0] * (k1 + n[1] * k2);
                    if (u) const_cast<double*>(base)[o] = u[vol * c + compact(i, N)];
                    bool interior = true;
                    for (int d = 0; d < NDIM; ++d) interior = interior && i[d] >= 0 && i[d] < N;
                    if (f_out && interior) f_out[vol * c + compact(i, N)] = base[o];
                }
    }
    (void)q;
    (void)depth;
}

int
run_ldata(const std::string& centering, const std::string& kernel, int N, const char* in_path, const char* out_path)
{
    using namespace SAMRAI;
    const bool side = centering == "side";
    FILE* in = std::fopen(in_path, "rb");
    if (!in) return 2;
    int n = 0, depth = 1;
    if (std::fread(&n, 4, 1, in) != 1 || std::fread(&depth, 4, 1, in) != 1) return 2;
    const int Q_depth = side ? NDIM : depth;
    const int ncomp = side ? NDIM : depth;
    const long long vol = (long long)std::pow(N, NDIM);
    tbox::Pointer<IBTK::LData> X_data(new IBTK::LData("X", n, NDIM));
    tbox::Pointer<IBTK::LData> F_data(new IBTK::LData("F", n, Q_depth));
    tbox::Pointer<IBTK::LData> U_data(new IBTK::LData("U", n, Q_depth));
    std::vector<double> u(vol * ncomp);
    if (std::fread(X_data->values().data(), 8, (size_t)n * NDIM, in) != (size_t)n * NDIM ||
        std::fread(F_data->values().data(), 8, (size_t)n * Q_depth, in) != (size_t)n * Q_depth ||
        std::fread(u.data(), 8, u.size(), in) != u.size())
        return 2;
    std::fclose(in);

    tbox::Pointer<hier::Patch<NDIM>> patch(new hier::Patch<NDIM>());
    hier::IntVector<NDIM> periodic_shift(N);
    for (int d = 0; d < NDIM; ++d)
    {
        patch->box.lo(d) = 0;
        patch->box.hi(d) = N - 1;
        patch->geom.dx[d] = 1.0 / N;
        patch->geom.x_lower[d] = 0.0;
        patch->geom.x_upper[d] = 1.0;
        patch->geom.touches_periodic[d][0] = patch->geom.touches_periodic[d][1] = 1;
    }
    const int g = IBTK::LEInteractor::getMinimumGhostWidth(kernel);
    const hier::IntVector<NDIM> gcw(g);
    tbox::Pointer<IBTK::LIndexSetData<IBTK::LNode>> idx_data(
        new IBTK::LIndexSetData<IBTK::LNode>(patch->getBox(), gcw));
    idx_data->setMarkerPositions(X_data->values().data(), n);
    idx_data->cacheLocalIndices(patch, periodic_shift);

    // host patch data: one array per side axis, or one array of `depth` components
    std::vector<long long> nval(side ? NDIM : 1);
    std::vector<std::vector<double>> f_arr(nval.size()), u_arr(nval.size());
    for (size_t a = 0; a < nval.size(); ++a)
    {
        nval[a] = IBTK::ibx_detail::array_values(patch->getBox(), gcw, side ? (int)a : -1);
        f_arr[a].assign(nval[a] * (side ? 1 : depth), 0.0);
        u_arr[a].assign(nval[a] * (side ? 1 : depth), 0.0);
    }
    std::vector<double> f_out(vol * ncomp, 0.0);
    if (side)
    {
        tbox::Pointer<pdat::SideData<NDIM, double>> f_data(new pdat::SideData<NDIM, double>());
        tbox::Pointer<pdat::SideData<NDIM, double>> u_data(new pdat::SideData<NDIM, double>());
        for (auto* q : { f_data.getPointer(), u_data.getPointer() })
        {
            q->box = patch->getBox();
            q->gcw = gcw;
        }
        for (int a = 0; a < NDIM; ++a)
        {
            f_data->data[a] = f_arr[a].data();
            u_data->data[a] = u_arr[a].data();
        }
        IBTK::LEInteractor::spread(f_data, F_data, X_data, idx_data, patch, idx_data->getGhostBox(), periodic_shift,
                                   kernel);
        fill_or_read(*f_data, nval, f_arr, ncomp, depth, N, g, nullptr, f_out.data(), true);
        fill_or_read(*u_data, nval, u_arr, ncomp, depth, N, g, u.data(), nullptr, true);
        IBTK::LEInteractor::interpolate(U_data, X_data, idx_data, u_data, patch, patch->getBox(), periodic_shift,
                                        kernel);
    }
    else
    {
        tbox::Pointer<pdat::CellData<NDIM, double>> f_data(new pdat::CellData<NDIM, double>());
        tbox::Pointer<pdat::CellData<NDIM, double>> u_data(new pdat::CellData<NDIM, double>());
        for (auto* q : { f_data.getPointer(), u_data.getPointer() })
        {
            q->box = patch->getBox();
            q->gcw = gcw;
            q->depth = depth;
        }
        f_data->data = f_arr[0].data();
        u_data->data = u_arr[0].data();
        IBTK::LEInteractor::spread(f_data, F_data, X_data, idx_data, patch, idx_data->getGhostBox(), periodic_shift,
                                   kernel);
        fill_or_read(*f_data, nval, f_arr, ncomp, depth, N, g, nullptr, f_out.data(), false);
        fill_or_read(*u_data, nval, u_arr, ncomp, depth, N, g, u.data(), nullptr, false);
        IBTK::LEInteractor::interpolate(U_data, X_data, idx_data, u_data, patch, patch->getBox(), periodic_shift,
                                        kernel);
    }
    // the sub-box: interpolation through the raw-pointer index-set form
    std::vector<double> U_sub((size_t)n * Q_depth, 7.0);
    hier::Box<NDIM> sub = patch->getBox();
    for (int d = 0; d < NDIM; ++d)
    {
        sub.lo(d) += 2;
        sub.hi(d) -= 2;
    }
    if (side)
    {
        tbox::Pointer<pdat::SideData<NDIM, double>> u_data(new pdat::SideData<NDIM, double>());
        u_data->box = patch->getBox();
        u_data->gcw = gcw;
        for (int a = 0; a < NDIM; ++a) u_data->data[a] = u_arr[a].data();
        IBTK::LEInteractor::interpolate(U_sub.data(), Q_depth, X_data->values().data(), NDIM, idx_data, u_data, patch,
                                        sub, periodic_shift, kernel);
    }
    else
    {
        tbox::Pointer<pdat::CellData<NDIM, double>> u_data(new pdat::CellData<NDIM, double>());
        u_data->box = patch->getBox();
        u_data->gcw = gcw;
        u_data->depth = depth;
        u_data->data = u_arr[0].data();
        IBTK::LEInteractor::interpolate(U_sub.data(), Q_depth, X_data->values().data(), NDIM, idx_data, u_data, patch,
                                        sub, periodic_shift, kernel);
    }
    FILE* out = std::fopen(out_path, "wb");
    if (!out) return 2;
    std::fwrite(f_out.data(), 8, f_out.size(), out);
    std::fwrite(U_data->values().data(), 8, U_data->values().size(), out);
    std::fwrite(U_sub.data(), 8, U_sub.size(), out);
    std::fclose(out);
    std::printf("OK %zu\n", idx_data->getLocalPETScIndices().size());
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
        if (std::strcmp(argv[1], "ldata") == 0 && argc >= 7)
            return run_ldata(argv[2], argv[3], std::atoi(argv[4]), argv[5], argv[6]);
    }
    catch (const std::exception& e)
    {
        std::printf("error: %s\n", e.what());
        return 3;
    }
    return 2;
}
