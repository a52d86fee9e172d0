// ibx_plan.cu -- host side of the binned spread / interpolate pipeline
// (ibx_plan_* in include/ibx.h).
//
// Per step:
//   1. bin (ibx_bin.cu): one thread per marker derives the exact stencil
//      bases and kernel arguments (cell-centred and staggered position) and
//      counts the marker into its home tile (warp-aggregated atomics).
//   2. exclusive scans (exact integer).
//   3. counting sort by home tile, which also cuts dense home tiles into
//      work items of home units; markers of sparse home tiles count the
//      tiles their footprints touch; scans; counting sort of those visits.
//   4. spread (ibx_spread.cu): dense tiles spread their home markers into a
//      tile+halo region, sparse-homed markers are spread by the owner of
//      every tile they visit.
//   5. interpolate (ibx_interp.cu): markers in home-tile (or marker) order,
//      concurrently with the spread in ibx_plan_step.
// Geometry: IBX_MODE_PERIODIC problems (compact periodic arrays).

#include "ibx_plan.cuh"
#include "../../include/ibx.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace ibx
{
int build_prob(const ibx_problem& in, int kernel, bool spread, Prob& P);

namespace
{
constexpr int ITEM_UNITS = 256; // home units per dense spread work item (one per thread)
constexpr int MIN_ITEM_UNITS = 32; // smallest setting of ibx_plan_set_tuning
// Items hold ITEM_UNITS / ncomp units by default (one thread per unit and
// component); the capacity below allows MIN_ITEM_UNITS / 3 per item.
constexpr int DENSE_MIN = 32;   // home tiles with more markers are spread by home region

int
ceil_log2(long double v)
{
    int e = 0;
    while (std::ldexp(1.0L, e) < v) ++e;
    return e;
}

size_t
align256(size_t v)
{
    return (v + 255) & ~size_t(255);
}
} // namespace

// Constants of the exact fixed-point index path for one dimension (see
// ibx_bin.cu); returns false when the problem's range does not fit.
bool
fixed_dim(double x_lower, double x_upper, double dx, FixedDim& fx)
{
    const long double xmax = 2.0L * std::max(std::fabs((long double)x_lower), std::fabs((long double)x_upper)) +
                             8.0L * dx + 1e-30L;
    fx.sx = 62 - ceil_log2(xmax);
    const long double inv = 1.0L / (long double)dx;
    const int si = 62 - (std::ilogb(inv) + 1);
    fx.inv_f = std::llround(std::ldexp(inv, si));
    fx.F = fx.sx + si - 64;
    const int tb = ceil_log2(xmax * inv + 2.0L);
    fx.dshift = fx.F - 48 + tb;
    fx.xlo_c_f = std::llround(std::ldexp((long double)x_lower, fx.sx));
    const double xlo_s = x_lower - 0.5 * dx; // the reference's FP64 side-axis origin
    fx.xlo_s_f = std::llround(std::ldexp((long double)xlo_s, fx.sx));
    return fx.sx > 0 && fx.F >= 24 && fx.F <= 62 && fx.dshift >= 2 && fx.dshift <= fx.F - 4 && tb <= 30;
}

PlanCarve
carve_plan(const PlanSizes& z, char* b, DevPlan& D)
{
    PlanCarve c;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    const long long nm = z.n_markers;
    const int nt = z.n_tiles;
    c.o_probs = take(sizeof(PlanProb) * z.n_probs);
    c.o_moffs = take(sizeof(long long) * (z.n_probs + 1));
    c.o_toffs = take(sizeof(int) * (z.n_probs + 1));
    const size_t o_rec = take(sizeof(Rec) * nm);
    const size_t o_hrec = take(sizeof(Rec) * nm);
    const size_t o_home_tile = take(sizeof(int) * nm);
    const size_t o_counts = take(sizeof(int) * counter_ints(nt));
    const size_t o_item_tile = take(sizeof(int) * z.item_cap);
    const size_t o_home_list = take(sizeof(int) * nm);
    const size_t o_visit = take(sizeof(int) * z.visit_cap);
    const size_t o_home_units = take(sizeof(int2) * nm);
    c.o_status = take(sizeof(int) * 4);
    const size_t o_scan = take(sizeof(int) * SCAN_TMP_INTS);
    c.o_tmaps = take(sizeof(CUtensorMap) * 3 * z.n_probs);
    c.bytes = off;
    c.scan_tmp = nullptr;
    if (!b) return c;
    std::memset(&D, 0, sizeof(D));
    D.probs = reinterpret_cast<const PlanProb*>(b + c.o_probs);
    D.marker_offs = reinterpret_cast<const long long*>(b + c.o_moffs);
    D.tile_offs = reinterpret_cast<const int*>(b + c.o_toffs);
    D.n_probs = z.n_probs;
    D.n_markers = nm;
    D.n_tiles = nt;
    D.rec = reinterpret_cast<Rec*>(b + o_rec);
    D.hrec = reinterpret_cast<Rec*>(b + o_hrec);
    D.home_tile = reinterpret_cast<int*>(b + o_home_tile);
    int* counts = reinterpret_cast<int*>(b + o_counts);
    D.hcount = counts;
    D.hucount = counts + (nt + 1);
    D.vcount = counts + 2 * (nt + 1);
    D.items = counts + 3 * (nt + 1);
    D.hcursor = counts + 4 * (nt + 1);
    D.hucursor = D.hcursor + nt;
    D.vcursor = D.hucursor + nt;
    D.home_list = reinterpret_cast<int*>(b + o_home_list);
    D.visit_list = reinterpret_cast<int*>(b + o_visit);
    D.n_visit_cap = z.visit_cap;
    D.home_units = reinterpret_cast<int2*>(b + o_home_units);
    D.item_tile = reinterpret_cast<int*>(b + o_item_tile);
    D.n_item_cap = (int)z.item_cap;
    D.item_units = ITEM_UNITS;
    D.dense_min = DENSE_MIN;
    D.interp_form = 0;
    D.visit_kernel = 2;
    D.unit_cap = 32;
    D.tile_shape = z.tile_shape;
    D.dense_blocks_per_sm = 2;
    D.status = reinterpret_cast<int*>(b + c.o_status);
    D.work = D.status + 1;
    D.tmaps = reinterpret_cast<const CUtensorMap*>(b + c.o_tmaps);
    c.scan_tmp = reinterpret_cast<int*>(b + o_scan);
    return c;
}
} // namespace ibx

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct ibx_plan
{
    int dim, kernel, precision, n_probs, max_ncomp;
    ibx::DevPlan D;
    void* dmem;
    size_t dbytes;
    int* scan_tmp;
    // ibx_plan_step: after the binning, the spread forks onto `spread_s`
    // (greatest stream priority: it is the longer phase) and the
    // interpolation onto `side` (least priority), both joined back into the
    // caller's stream (step_mode 1); or the spread then the interpolation on
    // the caller's stream (0)
    cudaStream_t side, spread_s;
    // step_mode 3: the spread on `level`, of the interpolation's priority
    cudaStream_t level;
    cudaEvent_t ev_fork, ev_join, ev_join2;
    // the visit placement, deferred out of the binning to run beside the
    // dense-tile spread and the interpolation; the per-visit spread waits
    // for it
    cudaEvent_t ev_vis;
    // ibx_plan_step_io: the spread values' upload runs on `up`, behind the
    // positions' upload on the caller's stream (ev_x), and the spread waits
    // for it (ev_q)
    cudaStream_t up;
    cudaEvent_t ev_x, ev_q;
    // The problems' positions as one array in global marker order (problem
    // p's X at base + dim * its first marker), or null: then positions copied
    // into it from page-locked host memory are read by the binning directly.
    double* x_base;
    int step_mode;
    int n_tma; // problems whose interpolation sources have tensor maps
};

extern "C" {

int
ibx_plan_create(const ibx_problem* problems, int n_problems, int kernel, int precision, ibx_plan** out)
{
    return ibx_plan_create2(problems, problems, n_problems, kernel, precision, out);
}

int
ibx_plan_create2(const ibx_problem* problems, const ibx_problem* interp_problems, int n_problems, int kernel,
                 int precision, ibx_plan** out)
{
    return ibx_plan_create3(problems, interp_problems, n_problems, kernel, precision, 0, out);
}

int
ibx_plan_create3(const ibx_problem* problems, const ibx_problem* interp_problems, int n_problems, int kernel,
                 int precision, int tile_shape, ibx_plan** out)
{
    using namespace ibx;
    if (!out) return IBX_E_ARG;
    *out = nullptr;
    if (!problems || !interp_problems || n_problems < 1) return IBX_E_ARG;
    if (tile_shape < 0 || tile_shape >= N_TILE_SHAPES) return IBX_E_ARG;
    if (kernel < IBX_KERNEL_PIECEWISE_LINEAR || kernel > IBX_KERNEL_BSPLINE_4) return IBX_E_BAD_KERNEL;
    if (precision != IBX_PRECISION_MIXED) return IBX_E_ARG;
    const int dim = problems[0].dim;
    std::vector<PlanProb> hp(n_problems);
    std::vector<long long> moffs(n_problems + 1, 0);
    std::vector<int> toffs(n_problems + 1, 0);
    long long visit_cap = 0;
    int max_ncomp = 1;
    if (dim != 2 && dim != 3) return IBX_E_ARG;
    int Ed[3];
    tile_edges(dim, tile_shape, Ed);
    for (int p = 0; p < n_problems; ++p)
    {
        const ibx_problem& in = problems[p];
        Prob chk;
        const int rc = build_prob(in, kernel, true, chk);
        if (rc) return rc;
        if (in.dim != dim || in.mode != IBX_MODE_PERIODIC) return IBX_E_ARG;
        if (in.indices || in.Xshift) return IBX_E_ARG; // periodic plans take every marker
        const int ncomp = in.centering == IBX_SIDE ? dim : in.q_depth;
        if (ncomp > 3) return IBX_E_TOO_LARGE;
        max_ncomp = ncomp > max_ncomp ? ncomp : max_ncomp;
        PlanProb& P = hp[p];
        std::memset(&P, 0, sizeof(P));
        P.dim = dim;
        P.ncomp = ncomp;
        P.side = in.centering == IBX_SIDE;
        P.Q_depth = in.Q_depth;
        long long ntiles = 1, vol = 1, per = 1;
        for (int d = 0; d < 3; ++d)
        {
            if (d >= dim)
            {
                P.N[d] = 1;
                P.ntile[d] = 1;
                P.dx[d] = P.inv_dx[d] = 1.0;
                continue;
            }
            P.N[d] = in.iupper[d] - in.ilower[d] + 1;
            if (P.N[d] > 30000) return IBX_E_TOO_LARGE; // stencil bases are stored as int16
            const int E = Ed[d];
            P.ntile[d] = (P.N[d] + E - 1) / E;
            ntiles *= P.ntile[d];
            vol *= P.N[d];
            P.dx[d] = chk.dx[d];
            P.inv_dx[d] = chk.inv_dx[d];
            P.dx_pow2[d] = chk.dx_pow2[d];
            // Positions are measured from the box origin: index ilower sits at
            // x_lower, so the stencil bases come out relative to ilower.
            P.xlo_c[d] = in.x_lower[d];
            P.xlo_s[d] = in.x_lower[d] - 0.5 * in.dx[d];
            if (!fixed_dim(in.x_lower[d], in.x_upper[d], in.dx[d], P.fx[d])) P.fixed_ok = -1;
            const int bound = P.ntile[d] < 2 + (P.N[d] % E != 0) ? P.ntile[d] : 2 + (P.N[d] % E != 0);
            per *= bound;
        }
        const ibx_problem& ii = interp_problems[p];
        if (&ii != &in)
        {
            // Same geometry and markers; only the data arrays may differ.
            Prob chk2;
            const int rc2 = build_prob(ii, kernel, false, chk2);
            if (rc2) return rc2;
            bool same = ii.dim == in.dim && ii.centering == in.centering && ii.mode == in.mode && ii.X == in.X &&
                        ii.n_markers == in.n_markers && ii.Q_depth == in.Q_depth && ii.q_depth == in.q_depth &&
                        !ii.indices && !ii.Xshift;
            for (int d = 0; d < dim; ++d)
                same = same && ii.ilower[d] == in.ilower[d] && ii.iupper[d] == in.iupper[d] &&
                       ii.dx[d] == in.dx[d] && ii.x_lower[d] == in.x_lower[d];
            if (!same) return IBX_E_ARG;
        }
        P.fixed_ok = P.fixed_ok < 0 ? 0 : 1;
        P.inv_vol = (float)(1.0 / chk.vol);
        P.X = in.X;
        P.Q = in.Q;
        P.Qi = ii.Q;
        for (int c = 0; c < ncomp; ++c)
        {
            P.q[c] = P.side ? in.q[c] : static_cast<void*>(static_cast<float*>(in.q[0]) + vol * c);
            P.qi[c] = P.side ? ii.q[c] : static_cast<void*>(static_cast<float*>(ii.q[0]) + vol * c);
        }
        P.vec4 = P.N[0] % 4 == 0;
        for (int c = 0; c < ncomp; ++c) P.vec4 = P.vec4 && (reinterpret_cast<unsigned long long>(P.q[c]) & 15) == 0;
        P.tile0 = toffs[p];
        P.marker0 = moffs[p];
        if ((long long)toffs[p] + ntiles > 0x3fffffffLL) return IBX_E_TOO_LARGE;
        toffs[p + 1] = toffs[p] + (int)ntiles;
        moffs[p + 1] = moffs[p] + in.n_markers;
        visit_cap += (long long)in.n_markers * per;
    }
    if (moffs[n_problems] > 0x7fffffffLL) return IBX_E_TOO_LARGE;
    // Dense work items: at most one per tile plus one per MIN_ITEM_UNITS units.
    const long long item_cap = toffs[n_problems] + moffs[n_problems] / (MIN_ITEM_UNITS / 3) + 1;
    if (item_cap > 0x7fffffffLL || visit_cap > 0x7fffffffLL) return IBX_E_TOO_LARGE;
    ibx_plan* plan = new (std::nothrow) ibx_plan();
    if (!plan) return IBX_E_OOM;
    std::memset(plan, 0, sizeof(*plan));
    plan->dim = dim;
    plan->kernel = kernel;
    plan->precision = precision;
    plan->n_probs = n_problems;
    plan->max_ncomp = max_ncomp;
    PlanSizes z;
    z.tile_shape = tile_shape;
    z.n_probs = n_problems;
    z.n_markers = moffs[n_problems];
    bool x_contiguous = true;
    for (int p = 0; p < n_problems; ++p)
        x_contiguous = x_contiguous && hp[p].X == hp[0].X + (long long)dim * moffs[p];
    z.n_tiles = toffs[n_problems];
    z.visit_cap = visit_cap;
    z.item_cap = item_cap;
    // One device allocation holds every buffer of the plan.
    DevPlan& D = plan->D;
    const PlanCarve size_only = carve_plan(z, nullptr, D);
    void* dmem = nullptr;
    if (cudaMalloc(&dmem, size_only.bytes) != cudaSuccess)
    {
        delete plan;
        return IBX_E_OOM;
    }
    char* b = static_cast<char*>(dmem);
    const PlanCarve c = carve_plan(z, b, D);
    // Tensor maps of the interpolation sources (TMA-staged tile regions).
    std::vector<CUtensorMap> maps(3 * (size_t)n_problems);
    std::memset(maps.data(), 0, sizeof(CUtensorMap) * maps.size());
    encode_interp_maps(dim, kernel, tile_shape, hp.data(), n_problems, maps.data());
    int n_tma = 0;
    for (int p = 0; p < n_problems; ++p) n_tma += hp[p].tma;
    if (cudaMemcpy(b + c.o_tmaps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(b + c.o_probs, hp.data(), sizeof(PlanProb) * n_problems, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b + c.o_moffs, moffs.data(), sizeof(long long) * (n_problems + 1), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(b + c.o_toffs, toffs.data(), sizeof(int) * (n_problems + 1), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemset(b + c.o_status, 0, sizeof(int) * 4) != cudaSuccess)
    {
        cudaFree(dmem);
        delete plan;
        return IBX_E_CUDA;
    }
    plan->scan_tmp = c.scan_tmp;
    plan->step_mode = 1;
    plan->x_base = x_contiguous ? const_cast<double*>(hp[0].X) : nullptr;
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&plan->side, cudaStreamNonBlocking, least) != cudaSuccess ||
        cudaStreamCreateWithPriority(&plan->level, cudaStreamNonBlocking, least) != cudaSuccess ||
        cudaStreamCreateWithPriority(&plan->spread_s, cudaStreamNonBlocking, greatest) != cudaSuccess ||
        cudaEventCreateWithFlags(&plan->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&plan->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&plan->ev_join2, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&plan->ev_vis, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithPriority(&plan->up, cudaStreamNonBlocking, greatest) != cudaSuccess ||
        cudaEventCreateWithFlags(&plan->ev_x, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&plan->ev_q, cudaEventDisableTiming) != cudaSuccess)
    {
        cudaFree(dmem);
        delete plan;
        return IBX_E_CUDA;
    }
    D.zsplit = dense_zsplit(dim, kernel_width(kernel));
    // two units per thread: the region is zeroed and flushed once per item
    D.item_units = std::max(MIN_ITEM_UNITS, std::min(ITEM_UNITS, 2 * (ITEM_UNITS / (max_ncomp * D.zsplit))));
    D.max_ncomp = max_ncomp;
    plan->dmem = dmem;
    plan->dbytes = c.bytes;
    plan->n_tma = n_tma;
    *out = plan;
    return IBX_OK;
}

int
ibx_plan_bin(ibx_plan* plan, void* stream)
{
    if (!plan) return IBX_E_ARG;
    return ibx::bin_sequence(plan->dim, plan->kernel, plan->D, plan->scan_tmp, static_cast<cudaStream_t>(stream));
}

} // extern "C"

namespace
{
bool
transfers_ok(const ibx_transfer* t, int n)
{
    if (n < 0 || (n > 0 && !t)) return false;
    for (int i = 0; i < n; ++i)
        if (t[i].bytes > 0 && (!t[i].dst || !t[i].src)) return false;
    return true;
}

int
copy_all(const ibx_transfer* t, int n, cudaStream_t s)
{
    for (int i = 0; i < n; ++i)
        if (t[i].bytes > 0 && cudaMemcpyAsync(t[i].dst, t[i].src, t[i].bytes, cudaMemcpyDefault, s) != cudaSuccess)
            return IBX_E_CUDA;
    return IBX_OK;
}

// One step with its transfers: positions in on s; spread values in on `up`
// behind them; binning on s; spread and interpolation by the step mode, the
// spread after the spread values; interpolated values out after the
// interpolation.  Every stream of the plan is joined back into s, also after
// a failure, so that a capture in progress stays valid.
int
plan_step(ibx_plan* plan, cudaStream_t s, const ibx_transfer* in_X, int n_in_X, const ibx_transfer* in_Q, int n_in_Q,
          const ibx_transfer* out_Q, int n_out_Q)
{
    using namespace ibx;
    // Positions that fill the plan's whole position array from page-locked
    // host memory are read by the binning itself over the host link (and
    // stored into the array on the way): no separate copy before it.
    DevPlan D = plan->D;
    bool direct = false;
    if (n_in_X == 1 && plan->x_base && in_X[0].dst == plan->x_base &&
        in_X[0].bytes == sizeof(double) * (size_t)plan->dim * (size_t)plan->D.n_markers)
    {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, in_X[0].src) == cudaSuccess && a.type == cudaMemoryTypeHost &&
            a.devicePointer)
        {
            direct = true;
            D.x_src = static_cast<const double*>(a.devicePointer);
            D.x_dst = plan->x_base;
        }
        cudaGetLastError(); // an unregistered pointer leaves an error behind on some runtimes
    }
    int rc = direct ? IBX_OK : copy_all(in_X, n_in_X, s);
    if (rc) return rc;
    bool up = false;
    for (int i = 0; i < n_in_Q; ++i) up = up || in_Q[i].bytes > 0;
    // the spread values go up behind the positions: after the copy, or after
    // the binning kernel that reads the positions directly
    auto upload = [&]() -> int {
        if (!up) return IBX_OK;
        if (cudaStreamWaitEvent(plan->up, plan->ev_x, 0) != cudaSuccess) return IBX_E_CUDA;
        const int r = copy_all(in_Q, n_in_Q, plan->up);
        if (cudaEventRecord(plan->ev_q, plan->up) != cudaSuccess) return IBX_E_CUDA;
        return r;
    };
    if (up && !direct)
    {
        if (cudaEventRecord(plan->ev_x, s) != cudaSuccess) return IBX_E_CUDA;
        rc = upload();
        if (rc) return cudaStreamWaitEvent(s, plan->ev_q, 0) == cudaSuccess ? rc : IBX_E_CUDA;
    }
    // joins the upload into `st` (the stream the spread runs on)
    auto wait_up = [&](cudaStream_t st) { return !up || cudaStreamWaitEvent(st, plan->ev_q, 0) == cudaSuccess; };
    // Interpolation in marker order needs only the stencil records: in the
    // concurrent mode it forks as soon as they exist, beside the counting
    // sort; the other forms fork after the whole binning.
    const bool concurrent = plan->step_mode == 1 || plan->step_mode == 3 || plan->step_mode == 4;
    const bool early = concurrent && plan->D.interp_form == 2;
    // the visit placement is left out of the binning in the concurrent
    // modes: it runs beside the dense-tile spread and the interpolation,
    // which do not read the visits
    const bool defer = concurrent;
    rc = bin_sequence(plan->dim, plan->kernel, D, plan->scan_tmp, s, early ? plan->ev_fork : nullptr,
                      up && direct ? plan->ev_x : nullptr, defer);
    if (up && direct)
    {
        const int ru = rc ? IBX_OK : upload();
        if (rc || ru)
        {
            // the upload stream waited on an event of this step or nothing: join it
            if (cudaEventRecord(plan->ev_q, plan->up) == cudaSuccess) cudaStreamWaitEvent(s, plan->ev_q, 0);
            return rc ? rc : ru;
        }
    }
    if (rc) return wait_up(s) ? rc : IBX_E_CUDA;
    bool out = false;
    for (int i = 0; i < n_out_Q; ++i) out = out || out_Q[i].bytes > 0;
    if (plan->step_mode == 2)
    {
        if (!wait_up(s)) return IBX_E_CUDA;
        rc = launch_fused(plan->dim, plan->kernel, plan->D, plan->max_ncomp, s);
        return rc ? rc : copy_all(out_Q, n_out_Q, s);
    }
    if (plan->step_mode == 0)
    {
        // the interpolation first, its values copied out on `side` while the
        // spread runs
        rc = launch_interp(plan->dim, plan->kernel, plan->D, s);
        bool forked = false;
        if (!rc && out)
        {
            if (cudaEventRecord(plan->ev_fork, s) != cudaSuccess ||
                cudaStreamWaitEvent(plan->side, plan->ev_fork, 0) != cudaSuccess)
                rc = IBX_E_CUDA;
            else
            {
                forked = true;
                rc = copy_all(out_Q, n_out_Q, plan->side);
            }
        }
        if (!wait_up(s)) rc = rc ? rc : IBX_E_CUDA;
        if (!rc) rc = launch_spread(plan->dim, plan->kernel, plan->D, plan->max_ncomp, s);
        if (forked && (cudaEventRecord(plan->ev_join, plan->side) != cudaSuccess ||
                       cudaStreamWaitEvent(s, plan->ev_join, 0) != cudaSuccess))
            rc = rc ? rc : IBX_E_CUDA;
        return rc;
    }
    // spread and interpolation read the same records and write different
    // arrays: they overlap on the device.  Mode 1: the longer phase, the
    // spread, runs on the stream of greatest priority -- unless the
    // interpolated values are copied out, then the interpolation does, so
    // that the copy runs beside the rest of the spread instead of after it.
    // Mode 3: both on streams of the least priority.  Mode 4: the
    // interpolation's stream first.
    const bool level = plan->step_mode == 3;
    const bool interp_first = out || plan->step_mode == 4;
    cudaStream_t s_int = level ? plan->side : interp_first ? plan->spread_s : plan->side;
    cudaStream_t s_spr = level ? plan->level : interp_first ? plan->side : plan->spread_s;
    if ((!early && cudaEventRecord(plan->ev_fork, s) != cudaSuccess) ||
        cudaStreamWaitEvent(s_int, plan->ev_fork, 0) != cudaSuccess)
        return wait_up(s) ? IBX_E_CUDA : IBX_E_CUDA;
    if ((early && cudaEventRecord(plan->ev_join2, s) != cudaSuccess) || // the whole binning
        cudaStreamWaitEvent(s_spr, early ? plan->ev_join2 : plan->ev_fork, 0) != cudaSuccess || !wait_up(s_spr))
    {
        // join the forked interpolation stream and the upload before failing
        if (cudaEventRecord(plan->ev_join, s_int) == cudaSuccess) cudaStreamWaitEvent(s, plan->ev_join, 0);
        wait_up(s);
        return IBX_E_CUDA;
    }
    // the visits placed on the caller's stream beside both phases; the
    // per-visit spread waits for them
    int rv = launch_visits(plan->dim, plan->kernel, plan->D, s);
    if (!rv && cudaEventRecord(plan->ev_vis, s) != cudaSuccess) rv = IBX_E_CUDA;
    rc = launch_interp(plan->dim, plan->kernel, plan->D, s_int);
    if (!rc) rc = copy_all(out_Q, n_out_Q, s_int);
    const int rs = rv ? rv : launch_spread(plan->dim, plan->kernel, plan->D, plan->max_ncomp, s_spr, plan->ev_vis);
    // join even after a failed launch, so that no stream of the plan is left forked
    if (cudaEventRecord(plan->ev_join, s_int) != cudaSuccess || cudaEventRecord(plan->ev_join2, s_spr) != cudaSuccess ||
        cudaStreamWaitEvent(s, plan->ev_join, 0) != cudaSuccess || cudaStreamWaitEvent(s, plan->ev_join2, 0) != cudaSuccess)
        return IBX_E_CUDA;
    return rc ? rc : rs;
}
} // namespace

extern "C" {

int
ibx_plan_step(ibx_plan* plan, void* stream)
{
    if (!plan) return IBX_E_ARG;
    return plan_step(plan, static_cast<cudaStream_t>(stream), nullptr, 0, nullptr, 0, nullptr, 0);
}

int
ibx_plan_step_io(ibx_plan* plan, const ibx_transfer* in_X, int n_in_X, const ibx_transfer* in_Q, int n_in_Q,
                 const ibx_transfer* out_Q, int n_out_Q, void* stream)
{
    if (!plan || !transfers_ok(in_X, n_in_X) || !transfers_ok(in_Q, n_in_Q) || !transfers_ok(out_Q, n_out_Q))
        return IBX_E_ARG;
    return plan_step(plan, static_cast<cudaStream_t>(stream), in_X, n_in_X, in_Q, n_in_Q, out_Q, n_out_Q);
}

} // extern "C"

// A step captured into an instantiated CUDA graph (ibx_plan_graph).
struct ibx_graph
{
    cudaGraphExec_t exec;
    int kernels;
};

extern "C" {

int
ibx_plan_graph(ibx_plan* plan, const ibx_transfer* in_X, int n_in_X, const ibx_transfer* in_Q, int n_in_Q,
               const ibx_transfer* out_Q, int n_out_Q, void* stream, ibx_graph** graph)
{
    if (graph) *graph = nullptr;
    // the legacy default stream cannot be captured
    if (!plan || !graph || !stream || !transfers_ok(in_X, n_in_X) || !transfers_ok(in_Q, n_in_Q) ||
        !transfers_ok(out_Q, n_out_Q))
        return IBX_E_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return IBX_E_CUDA;
    const long long k0 = ibx_kernel_launches();
    const int rc = plan_step(plan, s, in_X, n_in_X, in_Q, n_in_Q, out_Q, n_out_Q);
    const long long kernels = ibx_kernel_launches() - k0;
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &g); // ends the capture also after a failed step
    if (rc || ec != cudaSuccess || !g)
    {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : IBX_E_CUDA;
    }
    // the kernels keep their streams' priorities (the spread's greatest)
    cudaGraphExec_t x = nullptr;
    const cudaError_t ei = cudaGraphInstantiateWithFlags(&x, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return IBX_E_CUDA;
    *graph = new ibx_graph{ x, (int)kernels };
    return IBX_OK;
}

int
ibx_graph_launch(ibx_graph* graph, void* stream)
{
    if (!graph) return IBX_E_ARG;
    return cudaGraphLaunch(graph->exec, static_cast<cudaStream_t>(stream)) == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

int
ibx_graph_kernels(const ibx_graph* graph)
{
    return graph ? graph->kernels : -1;
}

int
ibx_graph_destroy(ibx_graph* graph)
{
    if (!graph) return IBX_OK;
    const cudaError_t e = cudaGraphExecDestroy(graph->exec);
    delete graph;
    return e == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

int
ibx_plan_spread(ibx_plan* plan, void* stream)
{
    if (!plan) return IBX_E_ARG;
    return ibx::launch_spread(plan->dim, plan->kernel, plan->D, plan->max_ncomp, static_cast<cudaStream_t>(stream));
}

int
ibx_plan_interpolate(ibx_plan* plan, void* stream)
{
    if (!plan) return IBX_E_ARG;
    return ibx::launch_interp(plan->dim, plan->kernel, plan->D, static_cast<cudaStream_t>(stream));
}

int
ibx_plan_get_bins(const ibx_plan* plan, int* base_c, int* base_s, int* home_tile, int* tile_start, int* home_list)
{
    using namespace ibx;
    if (!plan) return IBX_E_ARG;
    if (cudaDeviceSynchronize() != cudaSuccess) return IBX_E_CUDA;
    const DevPlan& D = plan->D;
    const long long nm = D.n_markers;
    if (base_c || base_s)
    {
        std::vector<Rec> rec(nm);
        if (nm && cudaMemcpy(rec.data(), D.rec, sizeof(Rec) * nm, cudaMemcpyDeviceToHost) != cudaSuccess)
            return IBX_E_CUDA;
        for (long long g = 0; g < nm; ++g)
            for (int d = 0; d < 3; ++d)
            {
                if (base_c) base_c[3 * g + d] = rec[g].bc(d);
                if (base_s) base_s[3 * g + d] = rec[g].bs(d);
            }
    }
    if (home_tile && nm && cudaMemcpy(home_tile, D.home_tile, sizeof(int) * nm, cudaMemcpyDeviceToHost) != cudaSuccess)
        return IBX_E_CUDA;
    if (tile_start &&
        cudaMemcpy(tile_start, D.hcount, sizeof(int) * (D.n_tiles + 1), cudaMemcpyDeviceToHost) != cudaSuccess)
        return IBX_E_CUDA;
    if (home_list && nm && cudaMemcpy(home_list, D.home_list, sizeof(int) * nm, cudaMemcpyDeviceToHost) != cudaSuccess)
        return IBX_E_CUDA;
    return IBX_OK;
}

int
ibx_plan_status(ibx_plan* plan, void* stream, int* status)
{
    using namespace ibx;
    if (!plan || !status) return IBX_E_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int word = 0;
    if (cudaMemcpyAsync(&word, plan->D.status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess || cudaMemsetAsync(plan->D.status, 0, sizeof(int), s) != cudaSuccess)
        return IBX_E_CUDA;
    *status = (word & 1) ? IBX_E_NONFINITE : (word & 2) ? IBX_E_TOO_LARGE : (word & 4) ? IBX_E_TIMEOUT : IBX_OK;
    return IBX_OK;
}

int
ibx_plan_set_tuning(ibx_plan* plan, int item_units, int dense_min, int dense_blocks_per_sm)
{
    if (!plan) return IBX_E_ARG;
    if (item_units < ibx::MIN_ITEM_UNITS || item_units > ibx::ITEM_UNITS || dense_min < 0 || dense_blocks_per_sm < 1 ||
        dense_blocks_per_sm > 32)
        return IBX_E_ARG;
    plan->D.item_units = item_units;
    plan->D.dense_min = dense_min;
    plan->D.dense_blocks_per_sm = dense_blocks_per_sm;
    return IBX_OK;
}

int
ibx_plan_set_visit_kernel(ibx_plan* plan, int form)
{
    if (!plan || form < 0 || form > 3) return IBX_E_ARG;
    plan->D.visit_kernel = form;
    return IBX_OK;
}

int
ibx_plan_get_visit_kernel(const ibx_plan* plan)
{
    return plan ? plan->D.visit_kernel : -1;
}

int
ibx_plan_set_unit_cap(ibx_plan* plan, int cap)
{
    if (!plan || cap < 1 || cap > 32) return IBX_E_ARG;
    plan->D.unit_cap = cap;
    return IBX_OK;
}

int
ibx_plan_get_unit_cap(const ibx_plan* plan)
{
    return plan ? plan->D.unit_cap : -1;
}

int
ibx_plan_set_step_mode(ibx_plan* plan, int mode)
{
    if (!plan || mode < 0 || mode > 4) return IBX_E_ARG;
    plan->step_mode = mode;
    return IBX_OK;
}

int
ibx_plan_get_step_mode(const ibx_plan* plan)
{
    return plan ? plan->step_mode : -1;
}

int
ibx_plan_set_interp_kernel(ibx_plan* plan, int form)
{
    if (!plan || form < 0 || form > 4) return IBX_E_ARG;
    plan->D.interp_form = form;
    return IBX_OK;
}

int
ibx_plan_get_interp_kernel(const ibx_plan* plan)
{
    return plan ? plan->D.interp_form : -1;
}

int
ibx_plan_get_tuning(const ibx_plan* plan, int* item_units, int* dense_min, int* dense_blocks_per_sm)
{
    if (!plan) return IBX_E_ARG;
    if (item_units) *item_units = plan->D.item_units;
    if (dense_min) *dense_min = plan->D.dense_min;
    if (dense_blocks_per_sm) *dense_blocks_per_sm = plan->D.dense_blocks_per_sm;
    return IBX_OK;
}

int
ibx_plan_tile_shape(const ibx_plan* plan, int* edges)
{
    if (!plan) return -1;
    if (edges) ibx::tile_edges(plan->dim, plan->D.tile_shape, edges);
    return plan->D.tile_shape;
}

int
ibx_plan_n_tiles(const ibx_plan* plan)
{
    return plan ? plan->D.n_tiles : -1;
}

int
ibx_plan_tma_problems(const ibx_plan* plan)
{
    return plan ? plan->n_tma : -1;
}

long long
ibx_plan_scratch_bytes(const ibx_plan* plan)
{
    return plan ? (long long)plan->dbytes : 0;
}

int
ibx_plan_destroy(ibx_plan* plan)
{
    if (!plan) return IBX_OK;
    cudaStreamSynchronize(plan->side);
    cudaStreamSynchronize(plan->spread_s);
    cudaStreamSynchronize(plan->level);
    cudaStreamSynchronize(plan->up);
    cudaStreamDestroy(plan->side);
    cudaStreamDestroy(plan->spread_s);
    cudaStreamDestroy(plan->level);
    cudaStreamDestroy(plan->up);
    cudaEventDestroy(plan->ev_fork);
    cudaEventDestroy(plan->ev_join);
    cudaEventDestroy(plan->ev_join2);
    cudaEventDestroy(plan->ev_vis);
    cudaEventDestroy(plan->ev_x);
    cudaEventDestroy(plan->ev_q);
    const cudaError_t e = cudaFree(plan->dmem);
    delete plan;
    return e == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

} // extern "C"
