// sm_103a kernels of the absorption-factor path.
//
// One CTA processes one work item = (sample, reflection, tile of kTile
// consecutive coordinate-list voxels).  Thread k of the CTA takes voxels
// tile*kTile + k + j*kBlock, so the 32 lanes of a warp march 32 adjacent
// crystal voxels (np.where order: adjacent x) along the same two directions.
// Their positions differ by the same integer offset at every increment, so the
// label reads of a warp stay within one or a few 32-byte sectors.
//
// Per voxel (the body of AnACor/src/ray_tracing.c:199-278):
//   exit face  (cube_face, ray_tracing_basic.c:69-186): FP32 estimate of the
//              three candidate distances, exact FP64 division only when the
//              two smallest are within 2^-20 relative.
//   march      (cal_coord, :396-1460): 32.32 fixed-point positions with one
//              64-bit add per axis and step; a step whose fraction lies within
//              kAmbiguityMargin of a rounding boundary is recomputed with the
//              reference's two-rounding FP64 expression.  Faces whose ratios
//              are too large for fixed point march in FP64 throughout.
//   lengths    (cal_path2_plus, :1462-1552): FP64, same operation order; the
//              per-segment quotient fl(span / (len-1)) comes from a correctly
//              rounded reciprocal table and one FMA correction (exhaustively
//              checked for every span <= len <= kMaxDim+1 by the test suite).
//   rate       (cal_rate, :1554-1583): FP64 sum, exp in FP32 after an FP64
//              range reduction; per-thread Neumaier sums, warp-shuffle TwoSum
//              reduction, FP64 combination of the tile partials in a fixed
//              order (deterministic for any schedule).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "anacor_internal.h"
#include "trace_launch.h"

namespace anacor {

__device__ double g_rcp[kMaxDim + 2];   // g_rcp[d] = fl(1 / d)

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

struct Vol {
    const int8_t *p;
    int dz, dy, dx;
};

__device__ __forceinline__ int clampi(int v, int hi)
{
    return min(max(v, 0), hi - 1);
}

// C's `int64_t n = floor(v)` / `round(v)`, then the reference's clamp.
// Out-of-range and NaN conversions give INT64_MIN (x86-64 behaviour).
__device__ __forceinline__ int exact_axis(int c, int i, double q, bool use_round, int dim)
{
    const double v = __dadd_rn((double)c, __dmul_rn((double)i, q));
    const double r = use_round ? round(v) : floor(v);
    long long n;
    if (!(r >= -9223372036854775808.0 && r < 9223372036854775808.0))
        n = LLONG_MIN;
    else
        n = (long long)r;
    if (n >= dim)
        n = dim - 1;
    else if (n < 0)
        n = 0;
    return (int)n;
}

// Exit face of the ray from (cz, cy, cx).  Returns the face code 1..6 or 0.
__device__ __forceinline__ int exit_face(const LegHead &h, int cz, int cy, int cx, const Vol &v)
{
    // A zero distance (origin on a min plane, non-zero component) wins; ties
    // follow the reference's test order x_min, y_min, z_min.
    if (cx == 0 && h.e[2] != 0.0) return 6;
    if (cy == 0 && h.e[1] != 0.0) return 4;
    if (cz == 0 && h.e[0] != 0.0) return 2;
    const uint32_t sb = h.sign_bits;
    // one candidate per axis: numerator n_a, face f_a
    int nx = (sb & 4u) ? v.dx - cx : cx;
    int ny = (sb & 2u) ? v.dy - cy : cy;
    int nz = (sb & 1u) ? v.dz - cz : cz;
    const bool hx = (sb & (4u | 32u)) != 0, hy = (sb & (2u | 16u)) != 0, hz = (sb & (1u | 8u)) != 0;
    const float inf = __int_as_float(0x7f800000);
    float tx = hx ? (float)nx * h.inv[2] : inf;
    float ty = hy ? (float)ny * h.inv[1] : inf;
    float tz = hz ? (float)nz * h.inv[0] : inf;
    // argmin with ties to the earlier axis (x, y, z)
    int best = 2;
    float t1 = tx, t2;
    if (ty < t1) { t2 = t1; t1 = ty; best = 1; } else { t2 = ty; }
    if (tz < t1) { t2 = t1; t1 = tz; best = 0; } else { t2 = fminf(t2, tz); }
    if ((sb & 64u) || !(t1 < inf && t2 > t1 * (1.0f + 0x1p-20f))) {
        // close call: the reference's FP64 quotients decide
        const double dinf = __longlong_as_double(0x7ff0000000000000ll);
        double ex = hx ? __ddiv_rn((double)nx, fabs(h.e[2])) : dinf;
        double ey = hy ? __ddiv_rn((double)ny, fabs(h.e[1])) : dinf;
        double ez = hz ? __ddiv_rn((double)nz, fabs(h.e[0])) : dinf;
        best = 2;
        double b = ex;
        if (ey < b) { b = ey; best = 1; }
        if (ez < b) { b = ez; best = 0; }
        if (!(b < dinf))
            return 0;
    }
    const bool pos = (sb >> best) & 1u;
    // faces: x: 1 max / 6 min, y: 5 max / 4 min, z: 3 max / 2 min
    if (best == 2) return pos ? 1 : 6;
    if (best == 1) return pos ? 5 : 4;
    return pos ? 3 : 2;
}

struct March {
    int len, nseg, prev, vac;
    int fz, fy, fx;     // first path point
    int lz, ly, lx;     // last path point
};

// Segment sink: mode 0 records (class, start) in shared memory; mode 1
// accumulates lengths directly (second pass, when a leg has more class
// changes than the shared buffer holds).
struct Sink {
    uint16_t *seg;      // stride kBlock
    // second-pass state
    double tot, den, rcp;
    double L0, L1, L2, L3;
    int open_cls, open_pos;
};

__device__ __forceinline__ double span_quotient(int span, double den, double rcp)
{
    // fl(span / den) from rcp = fl(1/den): q0 = fl(span*rcp), one FMA-exact
    // remainder and one correction step.
    const double s = (double)span;
    const double q0 = __dmul_rn(s, rcp);
    const double r = __fma_rn(-q0, den, s);
    return __fma_rn(r, rcp, q0);
}

__device__ __forceinline__ void add_class(int cls, double term, double &L0, double &L1, double &L2, double &L3)
{
    if (cls < 1 || cls > 4)
        return;
    double cur = cls == 1 ? L0 : (cls == 2 ? L1 : (cls == 3 ? L2 : L3));
    double nv = __dadd_rn(cur, term);
    L0 = cls == 1 ? nv : L0;
    L1 = cls == 2 ? nv : L1;
    L2 = cls == 3 ? nv : L2;
    L3 = cls == 4 ? nv : L3;
}

template <int kMode>
__device__ __forceinline__ bool visit(March &m, Sink &sk, int i, int lab, int pz, int py, int px,
                                      int full, int vac_limit)
{
    if (!full) {
        if (lab == 0)
            return false;
    } else {
        m.vac = lab == 0 ? m.vac + 1 : 0;
        if (m.vac > vac_limit)
            return false;
    }
    if (lab != m.prev && (unsigned)lab <= 4u) {
        if (kMode == 0) {
            if (m.nseg < kMaxSegments)
                sk.seg[m.nseg * kBlock] = (uint16_t)((lab << 13) | i);
        } else {
            const double q = span_quotient(i - sk.open_pos, sk.den, sk.rcp);
            add_class(sk.open_cls, __dmul_rn(sk.tot, q), sk.L0, sk.L1, sk.L2, sk.L3);
            sk.open_cls = lab;
            sk.open_pos = i;
        }
        m.nseg++;
    }
    m.len++;
    m.prev = lab;
    m.lz = pz; m.ly = py; m.lx = px;
    return true;
}

// March one leg (cal_coord).  Returns false if the start voxel stops it.
template <int kMode>
__device__ __forceinline__ void march(const FaceRule &R, int cz, int cy, int cx, int steps, const Vol &v,
                                      int full, March &m, Sink &sk)
{
    const int8_t *__restrict__ vol = v.p;
    const int sy = v.dx, sz = v.dy * v.dx;
    const bool rnd = R.use_round;
    int pz, py, px;
    if (R.fast) {
        pz = cz; py = cy; px = cx;
    } else {
        pz = exact_axis(cz, 0, R.q[0], rnd, v.dz);
        py = exact_axis(cy, 0, R.q[1], rnd, v.dy);
        px = exact_axis(cx, 0, R.q[2], rnd, v.dx);
    }
    m.len = 1; m.nseg = 1; m.vac = 0;
    m.fz = pz; m.fy = py; m.fx = px;
    m.lz = pz; m.ly = py; m.lx = px;
    if (kMode == 0)
        sk.seg[0] = (uint16_t)(3 << 13);
    if (steps <= 0)
        return;
    int lab = __ldg(vol + (pz * sz + py * sy + px));
    if (!full) {
        if (lab == 0)
            return;
    } else {
        m.vac = lab == 0;
        if (m.vac > R.vac_limit)
            return;
    }
    m.prev = lab;
    if (R.fast) {
        const long long off = rnd ? 0x80000000ll : 0ll;
        long long E0 = ((long long)cz << 32) + off;
        long long E1 = ((long long)cy << 32) + off;
        long long E2 = ((long long)cx << 32) + off;
        const long long Q0 = R.Q[0], Q1 = R.Q[1], Q2 = R.Q[2];
        const uint32_t M0 = (R.exact_mask & 1) ? 0u : kAmbiguityMargin;
        const uint32_t M1 = (R.exact_mask & 2) ? 0u : kAmbiguityMargin;
        const uint32_t M2 = (R.exact_mask & 4) ? 0u : kAmbiguityMargin;
        for (int i = 1; i < steps; i += 4) {
            int qz[4], qy[4], qx[4], lb[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                E0 += Q0; E1 += Q1; E2 += Q2;
                int z = (int)(E0 >> 32), y = (int)(E1 >> 32), x = (int)(E2 >> 32);
                const bool amb = ((uint32_t)E0 + M0 < 2u * M0) | ((uint32_t)E1 + M1 < 2u * M1) |
                                 ((uint32_t)E2 + M2 < 2u * M2);
                if (amb) {
                    z = exact_axis(cz, i + k, R.q[0], rnd, v.dz);
                    y = exact_axis(cy, i + k, R.q[1], rnd, v.dy);
                    x = exact_axis(cx, i + k, R.q[2], rnd, v.dx);
                } else {
                    z = clampi(z, v.dz); y = clampi(y, v.dy); x = clampi(x, v.dx);
                }
                qz[k] = z; qy[k] = y; qx[k] = x;
            }
            // every position is clamped inside the volume, so reading ahead of
            // a vacuum stop or of `steps` is always in bounds
#pragma unroll
            for (int k = 0; k < 4; k++)
                lb[k] = __ldg(vol + (qz[k] * sz + qy[k] * sy + qx[k]));
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (i + k >= steps)
                    return;
                if (!visit<kMode>(m, sk, i + k, lb[k], qz[k], qy[k], qx[k], full, R.vac_limit))
                    return;
            }
        }
    } else {
        for (int i = 1; i < steps; i++) {
            const int z = exact_axis(cz, i, R.q[0], rnd, v.dz);
            const int y = exact_axis(cy, i, R.q[1], rnd, v.dy);
            const int x = exact_axis(cx, i, R.q[2], rnd, v.dx);
            const int l = __ldg(vol + (z * sz + y * sy + x));
            if (!visit<kMode>(m, sk, i, l, z, y, x, full, R.vac_limit))
                return;
        }
    }
}

struct LegResult {
    double L[4];
    int face, len, nseg, status;
    int first[3], last[3];
};

// cube_face + cal_coord + cal_path2_plus for one leg.
__device__ __forceinline__ void trace_leg(const LegHead &h, const FaceRule *rules, int cz, int cy, int cx,
                                          const Vol &v, int full, const double *voxel, uint16_t *seg,
                                          LegResult &out)
{
    out.L[0] = out.L[1] = out.L[2] = out.L[3] = 0.0;
    out.len = 1; out.nseg = 1; out.status = kOk;
    out.first[0] = cz; out.first[1] = cy; out.first[2] = cx;
    out.last[0] = cz; out.last[1] = cy; out.last[2] = cx;
    const int face = exit_face(h, cz, cy, cx, v);
    out.face = face;
    if (face == 0) {
        out.status = kErrNoFace;
        return;
    }
    const FaceRule &R = rules[face - 1];
    if (R.status) {
        out.status = R.status;
        return;
    }
    const int cc = R.count_axis == 0 ? cz : (R.count_axis == 1 ? cy : cx);
    const int dd = R.count_axis == 0 ? v.dz : (R.count_axis == 1 ? v.dy : v.dx);
    const int steps = R.count_kind == 0 ? cc + 1 : (R.count_kind == 1 ? dd - cc : dd - cc + 1);
    March m;
    Sink sk;
    sk.seg = seg;
    march<0>(R, cz, cy, cx, steps, v, full, m, sk);
    out.len = m.len; out.nseg = m.nseg;
    out.first[0] = m.fz; out.first[1] = m.fy; out.first[2] = m.fx;
    out.last[0] = m.lz; out.last[1] = m.ly; out.last[2] = m.lx;
    if (m.len == 1)
        return;
    // total from the first and last path points, y then z then x
    const double dy = __dmul_rn((double)(m.ly - m.fy), voxel[1]);
    const double dz = __dmul_rn((double)(m.lz - m.fz), voxel[0]);
    const double dx = __dmul_rn((double)(m.lx - m.fx), voxel[2]);
    const double tot = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dz, dz)), __dmul_rn(dx, dx)));
    const int den_i = m.len - 1;
    const double den = (double)den_i;
    const double rcp = g_rcp[den_i];
    double L0 = 0.0, L1 = 0.0, L2 = 0.0, L3 = 0.0;
    if (m.nseg <= kMaxSegments) {
        int cur = seg[0];
        for (int j = 0; j < m.nseg; j++) {
            const int nxt = (j + 1 < m.nseg) ? (int)seg[(j + 1) * kBlock] : -1;
            const int start = cur & 0x1fff;
            const int end = (j + 1 < m.nseg) ? (nxt & 0x1fff) : m.len;
            const double q = span_quotient(end - start, den, rcp);
            add_class(cur >> 13, __dmul_rn(tot, q), L0, L1, L2, L3);
            cur = nxt;
        }
    } else {
        // more class changes than the shared buffer holds: march again and
        // accumulate as segments close (same terms, same order)
        March m2;
        Sink s2;
        s2.seg = seg;
        s2.tot = tot; s2.den = den; s2.rcp = rcp;
        s2.L0 = s2.L1 = s2.L2 = s2.L3 = 0.0;
        s2.open_cls = 3; s2.open_pos = 0;
        march<1>(R, cz, cy, cx, steps, v, full, m2, s2);
        const double q = span_quotient(m.len - s2.open_pos, den, rcp);
        add_class(s2.open_cls, __dmul_rn(tot, q), s2.L0, s2.L1, s2.L2, s2.L3);
        L0 = s2.L0; L1 = s2.L1; L2 = s2.L2; L3 = s2.L3;
    }
    out.L[0] = L0; out.L[1] = L1; out.L[2] = L2; out.L[3] = L3;
}

// cal_rate's exponent, operand order of AnACor/src/ray_tracing_basic.c:1573-1576
__device__ __forceinline__ double rate_exponent(const double *mu, const double *a, const double *b)
{
    const double t0 = __dmul_rn(mu[0], __dadd_rn(a[0], b[0]));
    const double t1 = __dmul_rn(mu[1], __dadd_rn(a[1], b[1]));
    const double t2 = __dmul_rn(mu[2], __dadd_rn(a[2], b[2]));
    const double t3 = __dmul_rn(mu[3], __dadd_rn(a[3], b[3]));
    return __dadd_rn(__dadd_rn(__dadd_rn(t0, t1), t2), t3);
}

// exp(-x) in FP32 after an FP64 reduction x = k ln2 + r, |r| <= ln2/2.
__device__ __forceinline__ float exp_neg(double x)
{
    const double kd = rint(__dmul_rn(x, 1.4426950408889634));
    const double r = __fma_rn(-kd, 0.6931471805599453, x);
    const float e = expf(-(float)r);
    const int k = (int)fmaxf(fminf((float)kd, 400.0f), -400.0f);
    return ldexpf(e, -k);
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

__device__ __forceinline__ int find_sample(const SampleDesc *d, int n, long long item)
{
    int s = 0;
    while (s + 1 < n && item >= d[s + 1].work_begin)
        s++;
    return s;
}

__global__ void __launch_bounds__(kBlock) absorption_kernel(const SampleDesc *__restrict__ descs, int n_desc,
                                                            long long total_items,
                                                            unsigned long long *__restrict__ work_counter)
{
    __shared__ ReflTable tab;
    __shared__ uint16_t seg[kMaxSegments * kBlock];
    __shared__ float red_s[kWarps], red_c[kWarps];
    __shared__ long long item_s;
    __shared__ int last_s;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (;;) {
        if (tid == 0)
            item_s = (long long)atomicAdd(work_counter, 1ull);
        __syncthreads();
        const long long item = item_s;
        if (item >= total_items)
            break;
        const int si = find_sample(descs, n_desc, item);
        const SampleDesc &D = descs[si];
        const long long local = item - D.work_begin;
        const long long r = local / D.tiles;
        const int t = (int)(local - r * D.tiles);
        {
            const int4 *src = reinterpret_cast<const int4 *>(D.refl + r);
            int4 *dst = reinterpret_cast<int4 *>(&tab);
            for (int k = tid; k < (int)(sizeof(ReflTable) / 16); k += kBlock)
                dst[k] = __ldg(src + k);
        }
        __syncthreads();

        const Vol v{D.vol, D.dim[0], D.dim[1], D.dim[2]};
        float s = 0.0f, c = 0.0f;
        int bad = kOk;
        unsigned nsteps = 0;
        const int v0 = t * kTile;
        const int v1 = min(D.n_vox, v0 + kTile);
        for (int vi = v0 + tid; vi < v1; vi += kBlock) {
            const short4 cv = __ldg(D.coords + vi);
            LegResult a, b;
            trace_leg(tab.head[0], tab.rule[0], cv.x, cv.y, cv.z, v, D.full_iteration, D.voxel, seg + tid, a);
            trace_leg(tab.head[1], tab.rule[1], cv.x, cv.y, cv.z, v, D.full_iteration, D.voxel, seg + tid, b);
            bad |= a.status | b.status;
            nsteps += (unsigned)(a.len + b.len);
            const double ex = rate_exponent(D.mu, a.L, b.L);
            const float term = D.is_exp ? exp_neg(ex) : (float)ex;
            float ns, e;
            two_sum(s, term, ns, e);
            s = ns;
            c += e;
        }
        if (bad)
            atomicOr(D.status, 1 << bad);
        if (D.steps) {
            unsigned long long w = nsteps;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                w += __shfl_down_sync(0xffffffffu, w, o);
            if (lane == 0)
                atomicAdd(D.steps, w);
        }
        // warp-shuffle TwoSum reduction of (s, c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float so = __shfl_down_sync(0xffffffffu, s, o);
            const float co = __shfl_down_sync(0xffffffffu, c, o);
            float ns, e;
            two_sum(s, so, ns, e);
            s = ns;
            c = c + co + e;
        }
        if (lane == 0) {
            red_s[warp] = s;
            red_c[warp] = c;
        }
        __syncthreads();
        if (tid == 0) {
            float bs = red_s[0], bc = red_c[0];
            for (int w = 1; w < kWarps; w++) {
                float ns, e;
                two_sum(bs, red_s[w], ns, e);
                bs = ns;
                bc = bc + red_c[w] + e;
            }
            D.partial[r * D.tiles + t] = (double)bs + (double)bc;
            __threadfence();
            const unsigned prev = atomicAdd(D.arrive + r, 1u);
            last_s = prev == (unsigned)(D.tiles - 1);
        }
        __syncthreads();
        if (last_s && warp == 0) {
            // the last tile of this reflection combines all partials in a fixed order
            __threadfence();
            const volatile double *p = D.partial + r * D.tiles;
            double acc = 0.0;
            for (int k = lane; k < D.tiles; k += 32)
                acc += p[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) {
                D.out[r] = acc / (double)D.n_vox;
                D.arrive[r] = 0u;   // ready for the next launch
            }
        }
    }
}

// Per-voxel, per-leg detail for one reflection (path-level parity checks).
__global__ void __launch_bounds__(kBlock) leg_detail_kernel(const ReflTable *__restrict__ tabp, const int8_t *vol,
                                                            int dz, int dy, int dx, const short4 *coords, int n,
                                                            const double *voxel3, int full, int *face, int *len,
                                                            int *nseg, int *first, int *last, double *L, int *status)
{
    __shared__ ReflTable tab;
    __shared__ uint16_t seg[kMaxSegments * kBlock];
    __shared__ double vox[3];
    {
        const int4 *src = reinterpret_cast<const int4 *>(tabp);
        int4 *dst = reinterpret_cast<int4 *>(&tab);
        for (int k = threadIdx.x; k < (int)(sizeof(ReflTable) / 16); k += kBlock)
            dst[k] = src[k];
        if (threadIdx.x < 3)
            vox[threadIdx.x] = voxel3[threadIdx.x];
    }
    __syncthreads();
    const int vi = blockIdx.x * kBlock + threadIdx.x;
    if (vi >= n)
        return;
    const Vol v{vol, dz, dy, dx};
    const short4 cv = coords[vi];
    for (int leg = 0; leg < 2; leg++) {
        LegResult a;
        trace_leg(tab.head[leg], tab.rule[leg], cv.x, cv.y, cv.z, v, full, vox, seg + threadIdx.x, a);
        const int o = 2 * vi + leg;
        face[o] = a.face;
        len[o] = a.len;
        nseg[o] = a.nseg;
        status[o] = a.status;
        for (int k = 0; k < 3; k++) {
            first[3 * o + k] = a.first[k];
            last[3 * o + k] = a.last[k];
        }
        for (int k = 0; k < 4; k++)
            L[4 * o + k] = a.L[k];
    }
}

// int64 (z, y, x) coordinates -> short4; flags out-of-range voxels.
__global__ void pack_coords_kernel(const long long *__restrict__ c, int n, int dz, int dy, int dx,
                                   short4 *__restrict__ out, int *__restrict__ status_word)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const long long z = c[3 * i], y = c[3 * i + 1], x = c[3 * i + 2];
    if (z < 0 || z >= dz || y < 0 || y >= dy || x < 0 || x >= dx) {
        atomicOr(status_word, 1 << kErrArgs);
        out[i] = make_short4(0, 0, 0, 0);
        return;
    }
    out[i] = make_short4((short)z, (short)y, (short)x, 0);
}

}  // namespace

int rcp_table_init()
{
    static double host[kMaxDim + 2];
    host[0] = 0.0;
    for (int d = 1; d < kMaxDim + 2; d++)
        host[d] = 1.0 / (double)d;
    return cudaMemcpyToSymbol(g_rcp, host, sizeof(host)) == cudaSuccess ? kOk : kErrCuda;
}

cudaError_t launch_pack_coords(const long long *d_c, int n, const int *dims, short4 *d_out, int *d_status,
                               cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    pack_coords_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_c, n, dims[0], dims[1], dims[2], d_out, d_status);
    return cudaGetLastError();
}

cudaError_t launch_absorption(const SampleDesc *d_descs, int n_desc, long long total_items,
                              unsigned long long *d_counter, int grid, cudaStream_t st)
{
    if (total_items <= 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess)
        return e;
    absorption_kernel<<<grid, kBlock, 0, st>>>(d_descs, n_desc, total_items, d_counter);
    return cudaGetLastError();
}

cudaError_t launch_leg_detail(const ReflTable *d_tab, const int8_t *d_vol, const int *dims, const short4 *d_coords,
                              int n, const double *d_voxel, int full, int *face, int *len, int *nseg, int *first,
                              int *last, double *L, int *status, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    leg_detail_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(d_tab, d_vol, dims[0], dims[1], dims[2],
                                                                    d_coords, n, d_voxel, full, face, len, nseg,
                                                                    first, last, L, status);
    return cudaGetLastError();
}

int absorption_block_threads() { return kBlock; }

int absorption_occupancy(int *blocks_per_sm)
{
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, absorption_kernel, kBlock, 0) ==
                   cudaSuccess
               ? kOk
               : kErrCuda;
}

}  // namespace anacor
