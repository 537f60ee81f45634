// Gridding (absorption-map) mode: C ABI and host set-up.
//
// The reference's approximate accelerator (AnACor/utils/utils_gridding.py:
// 63-473, AnACor/src/ray_tracing.c:427-534, AnACor/src/gridding_interpolation.c)
// replaces the per-reflection march by
//   1. a map: for every direction of a regular (theta, phi) grid and every
//      crystal voxel, the diffracted leg alone, stored as float32
//      sum_m mu_m L_m (method 2, the default) or exp(-sum) (method 1);
//   2. per reflection, each leg's map value looked up at the leg's polar
//      angles (nearest grid point, the default, or bilinear) and
//      A_h = mean_k exp(-(z_incident + z_diffracted)).
// Here the map is built by one persistent sm_103a launch over (direction,
// voxel tile) work items with the absorption kernel's march, and kept on the
// device direction-major ([direction][voxel], the voxel order of the plan);
// the lookups are one CTA per reflection streaming two contiguous map rows.
// Everything that decides which grid point or weight a value gets -- the grid
// directions, the polar angles, the padded axes, the index arithmetic -- runs
// on the host in FP64 with the reference's expressions (this file is compiled
// with -ffp-contract=off).
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "anacor_gb300.h"
#include "anacor_internal.h"
#include "trace_launch.h"

namespace anacor {
int report_status(int st, const char *msg);
}

using namespace anacor;

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kMinGrid = 18;   // below this the reference's wrap padding is empty

int cuda_err(cudaError_t e) { return report_status(kErrCuda, cudaGetErrorString(e)); }

template <class T>
cudaError_t dalloc(T **p, size_t n)
{
    *p = nullptr;
    return cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * std::max<size_t>(n, 1));
}

template <class T>
void dfree(T *&p)
{
    if (p)
        cudaFree(p);
    p = nullptr;
}

// numpy.linspace(start, stop, num, endpoint=False)[i]
double linspace_open(double start, double stop, int num, int i)
{
    const double step = (stop - start) / (double)num;
    return (double)i * step + start;
}

// Direction i of the grid (row i = i_phi * n_theta + i_theta): the grid point
// of mp_create_gridding (utils_gridding.py:270-276, degrees / 180 * pi), its
// DIALS vector (thetaphi_2_myframe, utils_rt.py:321-325, then
// myframe_2_dials, :483-503) and that vector's polar angles as
// worker_function_create_gridding recomputes them (utils_gridding.py:152).
void grid_direction(int n_theta, int n_phi, long long i, double *s1, double *theta, double *phi)
{
    const int it = (int)(i % n_theta), ip = (int)(i / n_theta);
    const double tg = linspace_open(-180.0, 180.0, n_theta, it) / 180.0 * kPi;
    const double pg = linspace_open(-90.0, 90.0, n_phi, ip) / 180.0 * kPi;
    const double z = std::cos(tg) * std::sin(pg);
    const double y = -std::sin(tg);
    const double x = -std::cos(tg) * std::cos(pg);
    // the permutation product adds zeros: -0 becomes +0
    s1[0] = z + 0.0;
    s1[1] = x + 0.0;
    s1[2] = y + 0.0;
    polar_angles(s1, false, theta, phi);
}

// Padded axis of the interpolation (utils_gridding.py:408-440): the map is
// wrapped by round((n // 6) / 2) points at each end and the axis spans
// +-round(half * 7 / 6) degrees.
struct Axis {
    int n = 0, pad = 0, len = 0;
    std::vector<double> v;   // radians, increasing
    double lo = 0.0, hi = 0.0;
    void make(int n_, double half_deg)
    {
        n = n_;
        pad = (int)std::nearbyint((double)(n / 6) / 2.0);
        len = n + 2 * pad;
        const double edge = std::nearbyint(half_deg * 7.0 / 6.0);
        v.resize(len);
        for (int i = 0; i < len; i++)
            v[i] = linspace_open(-edge, edge, len, i) / 180.0 * kPi;
        lo = v.front();
        hi = v.back();
    }
    // padded index -> index of the unpadded map (the wrap)
    int wrap(int i) const { return ((i - pad) % n + n) % n; }
};

// nearest_neighbor_custom (gridding_interpolation.c:16-31): truncating index
// against a step of (max - min) / (n - 1), clamped
int nearest_index(double x, double lo, double hi, int n)
{
    const double step = (hi - lo) / (double)(n - 1);
    const double t = (x - lo) / step;
    int i = (t > -2147483648.0 && t < 2147483647.0) ? (int)t : (t > 0 ? n - 1 : 0);
    if (i < 0)
        i = 0;
    if (i >= n)
        i = n - 1;
    return i;
}

// index search of a bilinear lookup on an increasing axis: xa[i] <= x < xa[i+1]
// (x == xa[n-1] gives n-2); false outside [xa[0], xa[n-1]]
bool bracket(const double *xa, int n, double x, int &i)
{
    if (!(x >= xa[0] && x <= xa[n - 1]))
        return false;
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const int mid = (hi + lo) / 2;
        if (xa[mid] > x)
            hi = mid;
        else
            lo = mid;
    }
    i = lo;
    return true;
}

// row/weight entries of one leg; `row_of(ti, pi)` maps grid indices to a map row
template <class RowOf>
bool leg_lookup(double theta, double phi, const double *ta, int nt, double tlo, double thi, const double *pa, int np,
                double plo, double phi_hi, bool linear, RowOf row_of, long long *row, double *w)
{
    if (!linear) {
        const int ti = nearest_index(theta, tlo, thi, nt);
        const int pi = nearest_index(phi, plo, phi_hi, np);
        row[0] = row[1] = row[2] = row[3] = row_of(ti, pi);
        w[0] = 1.0;
        w[1] = w[2] = w[3] = 0.0;
        return true;
    }
    int xi, yi;
    if (!bracket(ta, nt, theta, xi) || !bracket(pa, np, phi, yi))
        return false;
    const double t = (theta - ta[xi]) / (ta[xi + 1] - ta[xi]);
    const double u = (phi - pa[yi]) / (pa[yi + 1] - pa[yi]);
    row[0] = row_of(xi, yi);
    row[1] = row_of(xi + 1, yi);
    row[2] = row_of(xi, yi + 1);
    row[3] = row_of(xi + 1, yi + 1);
    w[0] = (1.0 - t) * (1.0 - u);
    w[1] = t * (1.0 - u);
    w[2] = (1.0 - t) * u;
    w[3] = t * u;
    return true;
}

// polar angles of both legs of a reflection as nearest_neighbor_interpolate_overall
// computes them (gridding_interpolation.c:121-145)
void reflection_angles(const double *axis, double omega, const double *F, const double *xray, const double *s1,
                       double *th1, double *ph1, double *th2, double *ph2)
{
    double xr[3], sr[3];
    rotate_reflection(axis, omega, F, xray, s1, xr, sr);
    polar_angles(sr, false, th2, ph2);
    polar_angles(xr, true, th1, ph1);
}

}  // namespace

struct anacor_gridding {
    anacor_plan *plan = nullptr;
    PlanView pv{};
    int n_theta = 0, n_phi = 0, method = 2;
    long long G = 0;
    Axis ta, pa;
    float *d_map = nullptr;
    long long ld = 0;
    int *d_col = nullptr;          // packed voxel -> caller column (reordered plans)
    std::vector<int> col;          // host copy
    int *d_status = nullptr;
    unsigned long long *d_counter = nullptr;
    MapDesc *d_desc = nullptr;
    bool built = false;
    InterpRow *d_rows = nullptr;
    double *d_out = nullptr;
    long long rows_cap = 0;
    long long n_prepared = 0;      // rows uploaded by anacor_gridding_prepare
    int prepared_linear = 0;
    int map_grid = 0;
};

namespace {

int interp_rows(anacor_gridding *g, const double *s1, const double *omega, int64_t n, const double *xray,
                const double *axis, const double *F, bool linear, std::vector<InterpRow> &rows)
{
    rows.resize((size_t)n);
    int bad = 0;
    const Axis &ta = g->ta, &pa = g->pa;
    const int nt = g->n_theta;
    auto row_of = [&](int ti, int pi) { return (long long)pa.wrap(pi) * nt + ta.wrap(ti); };
#pragma omp parallel for schedule(static) if (n > 256)
    for (int64_t i = 0; i < n; i++) {
        double th1, ph1, th2, ph2;
        reflection_angles(axis, omega[i], F, xray, s1 + 3 * i, &th1, &ph1, &th2, &ph2);
        InterpRow &r = rows[(size_t)i];
        const bool ok = leg_lookup(th1, ph1, ta.v.data(), ta.len, ta.lo, ta.hi, pa.v.data(), pa.len, pa.lo, pa.hi,
                                   linear, row_of, r.row[0], r.w[0]) &&
                        leg_lookup(th2, ph2, ta.v.data(), ta.len, ta.lo, ta.hi, pa.v.data(), pa.len, pa.lo, pa.hi,
                                   linear, row_of, r.row[1], r.w[1]);
        if (!ok) {
#pragma omp atomic write
            bad = 1;
        }
    }
    return bad ? report_status(kErrArgs, "gridding: a leg's angles fall outside the interpolation grid") : kOk;
}

int ensure_rows(anacor_gridding *g, int64_t n)
{
    if (n <= g->rows_cap)
        return kOk;
    dfree(g->d_rows);
    dfree(g->d_out);
    cudaError_t e;
    if ((e = dalloc(&g->d_rows, (size_t)n)) || (e = dalloc(&g->d_out, (size_t)n)))
        return cuda_err(e);
    g->rows_cap = n;
    return kOk;
}

int check_map_status(int *d_status, cudaStream_t st)
{
    int h = 0;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(&h, d_status, sizeof(int), cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
        return cuda_err(e);
    if (h & (1 << kErrAssert))
        return report_status(kErrAssert, "exit face inconsistent with the ray angles (the reference asserts here)");
    if (h & (1 << kErrNoFace))
        return report_status(kErrNoFace, "a ray found no exit plane");
    if (h)
        return report_status(kErrArgs, "gridding: the map launch reported an error");
    return kOk;
}

// Map values of n_dirs directions (tables on the device) for the voxels of a
// plan view, into out[d * ld + k] (k in the view's packed order, or col[k]).
int run_map(const PlanView &pv, const ReflTable *d_dirs, long long n_dirs, int is_exp, const double *mu, float *out,
            double *out64, long long ld, const int *col, MapDesc *d_desc, unsigned long long *d_counter,
            int *d_status, int grid, cudaStream_t st)
{
    MapDesc d;
    std::memset(&d, 0, sizeof(d));
    d.vol = pv.vol;
    for (int a = 0; a < 3; a++) {
        d.dim[a] = pv.dims[a];
        d.voxel[a] = pv.voxel[a];
    }
    for (int a = 0; a < 4; a++)
        d.mu[a] = mu[a];
    d.n_vox = pv.n_vox;
    d.coords = pv.coords;
    d.dirs = d_dirs;
    d.n_dirs = n_dirs;
    d.tile = kTile;
    d.tiles = (pv.n_vox + kTile - 1) / kTile;
    d.full_iteration = pv.full_iteration;
    d.is_exp = is_exp;
    d.out = out;
    d.out64 = out64;
    d.ld = ld;
    d.col = col;
    d.status = d_status;
    d.sq = pv.sq;
    d.sq_stride = pv.sq_stride;
    d.qtab = pv.qtab;
    d.field = pv.field;
    d.field_stride = pv.field_stride;
    cudaError_t e;
    if ((e = cudaMemsetAsync(d_status, 0, sizeof(int), st)) ||
        (e = cudaMemcpyAsync(d_desc, &d, sizeof(d), cudaMemcpyHostToDevice, st)))
        return cuda_err(e);
    const long long items = n_dirs * d.tiles;
    if ((e = launch_gridding_map(d_desc, items, d_counter, (int)std::max(1ll, std::min<long long>(items, grid)), st,
                                 pv.field != nullptr)))
        return cuda_err(e);
    // the descriptor is on the stack
    return check_map_status(d_status, st);
}

int map_grid_size(int sms)
{
    int b = 0;
    if (gridding_map_occupancy(&b) != kOk || b <= 0)
        b = 1;
    return std::max(1, sms) * b;
}

}  // namespace

extern "C" {

int anacor_gridding_directions(int n_theta, int n_phi, double *rotated_s1, double *theta, double *phi)
{
    if (n_theta < 1 || n_phi < 1 || !rotated_s1 || !theta || !phi)
        return report_status(kErrArgs, "bad arguments");
    const long long G = (long long)n_theta * n_phi;
    for (long long i = 0; i < G; i++)
        grid_direction(n_theta, n_phi, i, rotated_s1 + 3 * i, theta + i, phi + i);
    return report_status(kOk, "");
}

anacor_gridding *anacor_gridding_create(anacor_plan *plan, int n_theta, int n_phi, int method)
{
    if (!plan || n_theta < kMinGrid || n_phi < kMinGrid || (method != 1 && method != 2)) {
        report_status(kErrArgs, "gridding: a plan, n_theta and n_phi >= 18, method 1 or 2");
        return nullptr;
    }
    anacor_gridding *g = new (std::nothrow) anacor_gridding();
    if (!g) {
        report_status(kErrNoMem, "out of host memory");
        return nullptr;
    }
    g->plan = plan;
    // the map marches every voxel in every grid direction: on the octant fields
    if (plan_view_field(plan, &g->pv)) {
        delete g;
        return nullptr;
    }
    g->n_theta = n_theta;
    g->n_phi = n_phi;
    g->method = method;
    g->G = (long long)n_theta * n_phi;
    g->ta.make(n_theta, 180.0);
    g->pa.make(n_phi, 90.0);
    g->ld = ((long long)g->pv.n_vox + 31) / 32 * 32;
    g->map_grid = map_grid_size(g->pv.sms);
    cudaError_t e;
    cudaStream_t st = g->pv.stream;
    if ((e = dalloc(&g->d_map, (size_t)(g->G * std::max(1ll, g->ld)))) || (e = dalloc(&g->d_status, 1)) ||
        (e = dalloc(&g->d_counter, 1)) || (e = dalloc(&g->d_desc, 1))) {
        cuda_err(e);
        anacor_gridding_destroy(g);
        return nullptr;
    }
    if (g->pv.order && g->pv.n_vox > 0) {
        if ((e = dalloc(&g->d_col, (size_t)g->pv.n_vox)) ||
            (e = launch_order_permutation(g->pv.c64, g->pv.n_vox, g->pv.dims, g->pv.order, g->d_col, st)) ||
            (e = cudaStreamSynchronize(st))) {
            cuda_err(e);
            anacor_gridding_destroy(g);
            return nullptr;
        }
        g->col.resize((size_t)g->pv.n_vox);
        if ((e = cudaMemcpy(g->col.data(), g->d_col, g->col.size() * sizeof(int), cudaMemcpyDeviceToHost))) {
            cuda_err(e);
            anacor_gridding_destroy(g);
            return nullptr;
        }
    }
    report_status(kOk, "");
    return g;
}

void anacor_gridding_destroy(anacor_gridding *g)
{
    if (!g)
        return;
    if (g->pv.stream)
        cudaStreamSynchronize(g->pv.stream);
    dfree(g->d_map);
    dfree(g->d_col);
    dfree(g->d_status);
    dfree(g->d_counter);
    dfree(g->d_desc);
    dfree(g->d_rows);
    dfree(g->d_out);
    delete g;
}

int anacor_gridding_build(anacor_gridding *g, const double *rotated_s1, const double *theta, const double *phi)
{
    if (!g || ((rotated_s1 || theta || phi) && !(rotated_s1 && theta && phi)))
        return report_status(kErrArgs, "bad arguments");
    const long long G = g->G;
    std::vector<ReflTable> tabs((size_t)G);
    int bad = kOk;
#pragma omp parallel for schedule(static) if (G > 256)
    for (long long i = 0; i < G; i++) {
        double s[3], th, ph;
        if (rotated_s1) {
            s[0] = rotated_s1[3 * i];
            s[1] = rotated_s1[3 * i + 1];
            s[2] = rotated_s1[3 * i + 2];
            th = theta[i];
            ph = phi[i];
        } else {
            grid_direction(g->n_theta, g->n_phi, i, s, &th, &ph);
        }
        if (const int st = setup_direction(s, th, ph, &tabs[(size_t)i])) {
#pragma omp atomic write
            bad = st;
        }
    }
    if (bad)
        return report_status(bad, "gridding: non-finite or zero grid direction");
    if (g->pv.n_vox == 0) {
        g->built = true;
        return report_status(kOk, "");
    }
    cudaStream_t st = g->pv.stream;
    ReflTable *d_dirs = nullptr;
    cudaError_t e;
    if ((e = dalloc(&d_dirs, (size_t)G)) ||
        (e = cudaMemcpyAsync(d_dirs, tabs.data(), tabs.size() * sizeof(ReflTable), cudaMemcpyHostToDevice, st))) {
        dfree(d_dirs);
        return cuda_err(e);
    }
    const int r = run_map(g->pv, d_dirs, G, g->method == 1, g->pv.mu, g->d_map, nullptr, g->ld, nullptr, g->d_desc,
                          g->d_counter, g->d_status, g->map_grid, st);
    dfree(d_dirs);
    if (r)
        return r;
    g->built = true;
    return report_status(kOk, "");
}

int anacor_gridding_info(const anacor_gridding *g, int64_t *n_dirs, int64_t *n_vox, int *len_theta, int *len_phi)
{
    if (!g)
        return report_status(kErrArgs, "bad arguments");
    if (n_dirs)
        *n_dirs = g->G;
    if (n_vox)
        *n_vox = g->pv.n_vox;
    if (len_theta)
        *len_theta = g->ta.len;
    if (len_phi)
        *len_phi = g->pa.len;
    return report_status(kOk, "");
}

// the padded interpolation axes (len_theta and len_phi values, radians)
int anacor_gridding_axes(const anacor_gridding *g, double *theta_axis, double *phi_axis)
{
    if (!g || !theta_axis || !phi_axis)
        return report_status(kErrArgs, "bad arguments");
    std::memcpy(theta_axis, g->ta.v.data(), g->ta.v.size() * sizeof(double));
    std::memcpy(phi_axis, g->pa.v.data(), g->pa.v.size() * sizeof(double));
    return report_status(kOk, "");
}

const float *anacor_gridding_device_map(const anacor_gridding *g, int64_t *ld)
{
    if (!g)
        return nullptr;
    if (ld)
        *ld = g->ld;
    return g->d_map;
}

// host copy [n_dirs][n_vox] in the caller's voxel order (the reference's
// absorption_map layout, utils_gridding.py:137,233)
int anacor_gridding_map(const anacor_gridding *g, float *host_map)
{
    if (!g || !host_map)
        return report_status(kErrArgs, "bad arguments");
    if (!g->built)
        return report_status(kErrArgs, "gridding: the map has not been built");
    const int N = g->pv.n_vox;
    std::vector<float> row((size_t)std::max(1ll, g->ld));
    for (long long d = 0; d < g->G; d++) {
        float *dst = host_map + d * (long long)N;
        cudaError_t e;
        if (g->col.empty()) {
            e = cudaMemcpy(dst, g->d_map + d * g->ld, (size_t)N * sizeof(float), cudaMemcpyDeviceToHost);
        } else {
            e = cudaMemcpy(row.data(), g->d_map + d * g->ld, (size_t)N * sizeof(float), cudaMemcpyDeviceToHost);
            for (int k = 0; k < N; k++)
                dst[g->col[(size_t)k]] = row[(size_t)k];
        }
        if (e)
            return cuda_err(e);
    }
    return report_status(kOk, "");
}

int anacor_gridding_set_map(anacor_gridding *g, const float *host_map)
{
    if (!g || !host_map)
        return report_status(kErrArgs, "bad arguments");
    const int N = g->pv.n_vox;
    std::vector<float> row((size_t)std::max(1ll, g->ld), 0.0f);
    for (long long d = 0; d < g->G; d++) {
        const float *src = host_map + d * (long long)N;
        for (int k = 0; k < N; k++)
            row[(size_t)k] = g->col.empty() ? src[k] : src[g->col[(size_t)k]];
        if (cudaError_t e = cudaMemcpy(g->d_map + d * g->ld, row.data(), (size_t)g->ld * sizeof(float),
                                       cudaMemcpyHostToDevice))
            return cuda_err(e);
    }
    g->built = true;
    return report_status(kOk, "");
}

// A_h of n reflections from the map: method 1 nearest, 2 bilinear
int anacor_gridding_interpolate(anacor_gridding *g, const double *s1, const double *omega, int64_t n,
                                const double *xray, const double *omega_axis, const double *F, int method,
                                double *out)
{
    if (!g || n < 0 || (n > 0 && (!s1 || !omega || !xray || !omega_axis || !F || !out)) ||
        (method != 1 && method != 2))
        return report_status(kErrArgs, "bad arguments");
    if (!g->built)
        return report_status(kErrArgs, "gridding: the map has not been built");
    if (n == 0)
        return report_status(kOk, "");
    if (g->pv.n_vox == 0) {
        for (int64_t i = 0; i < n; i++)
            out[i] = std::nan("");
        return report_status(kOk, "");
    }
    std::vector<InterpRow> rows;
    if (int st = interp_rows(g, s1, omega, n, xray, omega_axis, F, method == 2, rows))
        return st;
    if (int st = ensure_rows(g, n))
        return st;
    cudaStream_t st = g->pv.stream;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(g->d_rows, rows.data(), rows.size() * sizeof(InterpRow), cudaMemcpyHostToDevice, st)) ||
        (e = launch_gridding_interp_f32(g->d_map, 1, g->ld, g->pv.n_vox, g->d_rows, n, method == 2, g->d_out, st)) ||
        (e = cudaMemcpyAsync(out, g->d_out, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st)))
        return cuda_err(e);
    return report_status(kOk, "");
}

// Lookup rows of n reflections computed on the host and kept on the device,
// so that anacor_gridding_run launches the interpolation alone.
int anacor_gridding_prepare(anacor_gridding *g, const double *s1, const double *omega, int64_t n, const double *xray,
                            const double *omega_axis, const double *F, int method)
{
    if (!g || n < 0 || (n > 0 && (!s1 || !omega || !xray || !omega_axis || !F)) || (method != 1 && method != 2))
        return report_status(kErrArgs, "bad arguments");
    std::vector<InterpRow> rows;
    if (int st = interp_rows(g, s1, omega, n, xray, omega_axis, F, method == 2, rows))
        return st;
    if (int st = ensure_rows(g, n))
        return st;
    cudaError_t e;
    if (n > 0 && ((e = cudaMemcpyAsync(g->d_rows, rows.data(), rows.size() * sizeof(InterpRow), cudaMemcpyHostToDevice,
                                       g->pv.stream)) ||
                  (e = cudaStreamSynchronize(g->pv.stream))))
        return cuda_err(e);
    g->n_prepared = n;
    g->prepared_linear = method == 2;
    return report_status(kOk, "");
}

int anacor_gridding_run(anacor_gridding *g, double *d_out, void *stream)
{
    if (!g || !d_out || !g->built || g->pv.n_vox == 0)
        return report_status(kErrArgs, "bad arguments or no map");
    cudaStream_t st = stream ? (cudaStream_t)stream : g->pv.stream;
    if (cudaError_t e = launch_gridding_interp_f32(g->d_map, 1, g->ld, g->pv.n_vox, g->d_rows, g->n_prepared,
                                                   g->prepared_linear, d_out, st))
        return cuda_err(e);
    return report_status(kOk, "");
}

// The same, leaving the n results on the device (d_out) without waiting for
// the kernel.  Calls on one map object must not overlap (they share the
// lookup-row buffer).
int anacor_gridding_interpolate_async(anacor_gridding *g, const double *s1, const double *omega, int64_t n,
                                      const double *xray, const double *omega_axis, const double *F, int method,
                                      double *d_out, void *stream)
{
    if (!g || n < 0 || (n > 0 && (!s1 || !omega || !xray || !omega_axis || !F || !d_out)) ||
        (method != 1 && method != 2) || !g->built || g->pv.n_vox == 0)
        return report_status(kErrArgs, "bad arguments or no map");
    if (n == 0)
        return report_status(kOk, "");
    std::vector<InterpRow> rows;
    if (int st = interp_rows(g, s1, omega, n, xray, omega_axis, F, method == 2, rows))
        return st;
    if (int st = ensure_rows(g, n))
        return st;
    cudaStream_t st = stream ? (cudaStream_t)stream : g->pv.stream;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(g->d_rows, rows.data(), rows.size() * sizeof(InterpRow), cudaMemcpyHostToDevice, st)) ||
        (e = launch_gridding_interp_f32(g->d_map, 1, g->ld, g->pv.n_vox, g->d_rows, n, method == 2, d_out, st)))
        return cuda_err(e);
    // `rows` is pageable memory: cudaMemcpyAsync returns once it has been staged
    return report_status(kOk, "");
}

}  // extern "C"

// ---------------------------------------------------- reference drop-ins

namespace {

// The volume of the single-voxel drop-ins (ray_tracing_single_gridding,
// ib_single_gridding), kept on the device between calls with the same row
// table (address and shape); a caller that changes the volume's contents in
// place between calls must pass a new table.
struct SingleCache {
    const int8_t *base = nullptr;
    int64_t shape[3] = {0, 0, 0};
    double voxel[3] = {0, 0, 0};
    int full = -1;
    anacor_plan *plan = nullptr;
    short4 *d_coord = nullptr;
    ReflTable *d_dir = nullptr;
    double *d_val = nullptr;
    double *d_vox_mu = nullptr;   // voxel[3], mu[4] (bisection)
    MapDesc *d_desc = nullptr;
    unsigned long long *d_counter = nullptr;
    int *d_status = nullptr;
    int dev = -1;
};
std::mutex g_single_mu;
SingleCache g_single;

// Argument checks of the single-voxel drop-ins, the cached volume, and the
// voxel and direction uploaded on the plan's stream (caller holds
// g_single_mu).  Status as report_status.
int single_setup(int64_t *coord, const double *rotated_s1, double theta, double phi, double *voxel_size,
                 double *coefficients, int8_t ***label_list, int64_t *shape, int full_iteration, int IsExp,
                 PlanView &pv)
{
    if (!coord || !rotated_s1 || !voxel_size || !coefficients || !label_list || !shape)
        return report_status(kErrArgs, "null argument");
    // the reference asserts that the given angles are the vector's (to 1e-6)
    double th, ph;
    polar_angles(rotated_s1, false, &th, &ph);
    if (!(std::fabs(th - theta) < 1e-6) || !(std::fabs(ph - phi) < 1e-6))
        return report_status(kErrAssert, "theta/phi do not belong to rotated_s1 (the reference asserts here)");
    for (int a = 0; a < 3; a++)
        if (shape[a] <= 0 || shape[a] > kMaxDim || coord[a] < 0 || coord[a] >= shape[a])
            return report_status(kErrArgs, "a coordinate lies outside the volume");
    SingleCache &c = g_single;
    const int8_t *base = label_list[0] ? label_list[0][0] : nullptr;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!base)
        return report_status(kErrArgs, "empty label table");
    if (c.plan && (c.base != base || std::memcmp(c.shape, shape, sizeof(c.shape)) ||
                   std::memcmp(c.voxel, voxel_size, sizeof(c.voxel)) || c.full != full_iteration || c.dev != dev)) {
        anacor_plan_destroy(c.plan);
        c.plan = nullptr;
    }
    if (!c.plan) {
        // the row table must be one C-contiguous block (utils_os.py:45-68)
        const int64_t Y = shape[1], X = shape[2];
        for (int64_t z = 0; z < shape[0]; z++)
            for (int64_t y = 0; y < Y; y++)
                if (!label_list[z] || label_list[z][y] != base + (z * Y + y) * X)
                    return report_status(kErrArgs, "label table rows are not one contiguous volume");
        const int64_t none[3] = {0, 0, 0};
        c.plan = anacor_plan_create(base, shape, none, 0, voxel_size, coefficients, full_iteration, IsExp);
        if (!c.plan)
            return anacor_last_status();
        if (!c.d_coord) {
            cudaError_t e;
            if ((e = dalloc(&c.d_coord, 1)) || (e = dalloc(&c.d_dir, 1)) || (e = dalloc(&c.d_val, 1)) ||
                (e = dalloc(&c.d_vox_mu, 7)) || (e = dalloc(&c.d_desc, 1)) || (e = dalloc(&c.d_counter, 1)) ||
                (e = dalloc(&c.d_status, 1)))
                return cuda_err(e);
        }
        c.base = base;
        std::memcpy(c.shape, shape, sizeof(c.shape));
        std::memcpy(c.voxel, voxel_size, sizeof(c.voxel));
        c.full = full_iteration;
        c.dev = dev;
    }
    if (int st = plan_view(c.plan, &pv))
        return st;
    ReflTable tab;
    if (setup_direction(rotated_s1, theta, phi, &tab))
        return report_status(kErrDirection, "non-finite or zero direction vector");
    const short4 cv = make_short4((short)coord[0], (short)coord[1], (short)coord[2], 0);
    double vm[7];
    for (int a = 0; a < 3; a++)
        vm[a] = voxel_size[a];
    for (int a = 0; a < 4; a++)
        vm[3 + a] = coefficients[a];
    cudaError_t e;
    if ((e = cudaMemcpyAsync(c.d_coord, &cv, sizeof(cv), cudaMemcpyHostToDevice, pv.stream)) ||
        (e = cudaMemcpyAsync(c.d_dir, &tab, sizeof(tab), cudaMemcpyHostToDevice, pv.stream)) ||
        (e = cudaMemcpyAsync(c.d_vox_mu, vm, sizeof(vm), cudaMemcpyHostToDevice, pv.stream)) ||
        (e = cudaStreamSynchronize(pv.stream)))
        return cuda_err(e);
    return kOk;
}

}  // namespace

extern "C" {

// ray_tracing_single_gridding (AnACor/src/ray_tracing.c:484-534): the map
// value of one voxel for one direction.  The volume is kept on the device
// between calls with the same row table (address and shape); a caller that
// changes the volume's contents in place between calls must pass a new table.
double ray_tracing_single_gridding(int64_t *coord, const double *rotated_s1, double theta, double phi,
                                   double *voxel_size, double *coefficients, int8_t ***label_list, int64_t *shape,
                                   int full_iteration, int index, int IsExp)
{
    (void)index;
    const double nan = std::nan("");
    std::lock_guard<std::mutex> lk(g_single_mu);
    PlanView pv;
    if (single_setup(coord, rotated_s1, theta, phi, voxel_size, coefficients, label_list, shape, full_iteration,
                     IsExp, pv))
        return nan;
    SingleCache &c = g_single;
    pv.coords = c.d_coord;
    pv.n_vox = 1;
    if (run_map(pv, c.d_dir, 1, IsExp ? 1 : 0, coefficients, nullptr, c.d_val, 1, nullptr, c.d_desc, c.d_counter,
                c.d_status, 1, pv.stream))
        return nan;
    double v = 0.0;
    cudaError_t e;
    if ((e = cudaMemcpy(&v, c.d_val, sizeof(double), cudaMemcpyDeviceToHost))) {
        cuda_err(e);
        return nan;
    }
    report_status(kOk, "");
    return v;
}

// ib_single_gridding (AnACor/src/ray_tracing.c:427-482): the same value with
// the diffracted leg's lengths found by iterative bisection (resolution 1.0,
// num_cls 4 also searches bubble boundaries) instead of the march.  The
// exponent sum_m mu_m (0 + L_m) comes from the GPU in cal_rate's order and
// exp(-a) is taken here, with the host's libm as the reference takes it.
double ib_single_gridding(int64_t *coord, const double *rotated_s1, double theta, double phi, double *voxel_size,
                          double *coefficients, int8_t ***label_list, int64_t *shape, int full_iteration, int index,
                          int num_cls, int IsExp)
{
    (void)index;
    const double nan = std::nan("");
    std::lock_guard<std::mutex> lk(g_single_mu);
    PlanView pv;
    if (single_setup(coord, rotated_s1, theta, phi, voxel_size, coefficients, label_list, shape, full_iteration,
                     IsExp, pv))
        return nan;
    SingleCache &c = g_single;
    cudaError_t e;
    double a = 0.0;
    int status = 0;
    if ((e = launch_ib_direction(c.d_dir, pv.vol, pv.dims, c.d_coord, 1, c.d_vox_mu, num_cls, c.d_val, c.d_status,
                                 pv.stream)) ||
        (e = cudaMemcpyAsync(&a, c.d_val, sizeof(double), cudaMemcpyDeviceToHost, pv.stream)) ||
        (e = cudaMemcpyAsync(&status, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, pv.stream)) ||
        (e = cudaStreamSynchronize(pv.stream))) {
        cuda_err(e);
        return nan;
    }
    if (status) {
        report_status(status, status == kErrArgs ? "a bisection point left the volume (undefined in the reference)"
                              : status == kErrAssert ? "exit face inconsistent with the ray angles (the reference "
                                                       "asserts here)"
                                                     : "the ray found no exit plane");
        return nan;
    }
    report_status(kOk, "");
    return IsExp ? std::exp(-a) : a;
}

// nearest_neighbor_interpolate_overall (AnACor/src/gridding_interpolation.c:
// 100-163) with its arguments: gridding_data is the padded map in the
// reference's voxel-major layout [len_coord_list][ny][nx] (FP64); method 1
// nearest, 2 bilinear.  Returns a malloc()ed array of len_result values
// (NULL on error, anacor_last_error()).
double *nearest_neighbor_interpolate_overall(int64_t low, int64_t up, int64_t *coord_list, int64_t len_coord_list,
                                             const double *scattering_vector_list, const double *omega_list,
                                             const double *raw_xray, const double *omega_axis,
                                             const double *kp_rotation_matrix, int64_t len_result,
                                             double *voxel_size, double *coefficients, int num_workers, int IsExp,
                                             double *theta_list, double *phi_list, double *gridding_data, size_t nx,
                                             size_t ny, double theta_min, double theta_max, double phi_min,
                                             double phi_max, int interpolation_method)
{
    (void)low; (void)up; (void)coord_list; (void)voxel_size; (void)coefficients; (void)IsExp;
    if (len_result < 0 || len_coord_list <= 0 || !scattering_vector_list || !omega_list || !raw_xray ||
        !omega_axis || !kp_rotation_matrix || !theta_list || !phi_list || !gridding_data || nx < 2 || ny < 2 ||
        nx > (1u << 30) || ny > (1u << 30) || (interpolation_method != 1 && interpolation_method != 2)) {
        report_status(kErrArgs, "bad arguments");
        return nullptr;
    }
    double *res = (double *)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(len_result, 1));
    if (!res) {
        report_status(kErrNoMem, "out of host memory");
        return nullptr;
    }
    const bool linear = interpolation_method == 2;
    std::vector<InterpRow> rows((size_t)len_result);
    const int nxi = (int)nx, nyi = (int)ny;
    auto row_of = [&](int ti, int pi) { return (long long)pi * nxi + ti; };
    int bad = 0;
    const int threads = num_workers > 0 ? num_workers : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(threads) if (len_result > 256)
    for (int64_t i = 0; i < len_result; i++) {
        double th1, ph1, th2, ph2;
        reflection_angles(omega_axis, omega_list[i], kp_rotation_matrix, raw_xray, scattering_vector_list + 3 * i,
                          &th1, &ph1, &th2, &ph2);
        InterpRow &r = rows[(size_t)i];
        const bool ok = leg_lookup(th1, ph1, theta_list, nxi, theta_min, theta_max, phi_list, nyi, phi_min, phi_max,
                                   linear, row_of, r.row[0], r.w[0]) &&
                        leg_lookup(th2, ph2, theta_list, nxi, theta_min, theta_max, phi_list, nyi, phi_min, phi_max,
                                   linear, row_of, r.row[1], r.w[1]);
        if (!ok) {
#pragma omp atomic write
            bad = 1;
        }
    }
    if (bad) {
        std::free(res);
        report_status(kErrArgs, "gridding: a leg's angles fall outside the interpolation grid");
        return nullptr;
    }
    const size_t cells = (size_t)nx * ny;
    double *d_map = nullptr, *d_out = nullptr;
    InterpRow *d_rows = nullptr;
    cudaError_t e;
    if (!(e = dalloc(&d_map, cells * (size_t)len_coord_list)) && !(e = dalloc(&d_out, (size_t)len_result)) &&
        !(e = dalloc(&d_rows, rows.size())) &&
        !(e = cudaMemcpy(d_map, gridding_data, cells * (size_t)len_coord_list * sizeof(double),
                         cudaMemcpyHostToDevice)) &&
        !(e = cudaMemcpy(d_rows, rows.data(), rows.size() * sizeof(InterpRow), cudaMemcpyHostToDevice)) &&
        !(e = launch_gridding_interp_f64(d_map, (long long)cells, 1, (int)len_coord_list, d_rows, len_result, linear,
                                         d_out, 0)) &&
        !(e = cudaDeviceSynchronize()))
        e = cudaMemcpy(res, d_out, (size_t)len_result * sizeof(double), cudaMemcpyDeviceToHost);
    dfree(d_map);
    dfree(d_out);
    dfree(d_rows);
    if (e) {
        std::free(res);
        cuda_err(e);
        return nullptr;
    }
    report_status(kOk, "");
    return res;
}

}  // extern "C"
