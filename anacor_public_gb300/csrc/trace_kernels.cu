// sm_103a kernels of the absorption-factor path.
//
// One warp processes one work item = (sample, reflection, tile of consecutive
// voxels of the packed list) taken from an atomic counter, so a warp that
// finishes early takes the next item instead of waiting for its CTA.  Lane k
// takes voxels tile*t + k + 32*j: the 32 lanes hold 32 consecutive entries of
// the Morton-ordered list (a compact 3-D block) and march them along the same
// two directions.
//
// Per voxel (the body of AnACor/src/ray_tracing.c:199-278), per leg:
//   exit face  (cube_face, ray_tracing_basic.c:69-186): FP32 estimate of the
//              three candidate distances, exact FP64 division only when the
//              two smallest are within 2^-20 relative.
//   march      (cal_coord, :396-1460), warp-cooperative: lanes leaving through
//              the same face share its step rule and differ only by an integer
//              start offset, so one lane per increment computes the 32.32
//              fixed-point displacement and the warp broadcasts it; each lane
//              loads its label at base + displacement, eight increments in
//              flight, and checks four labels per packed word.  Increments
//              whose fraction lies within kAmbiguityMargin of a rounding
//              boundary are recomputed with the reference's FP64 expression.
//              Lanes that may touch a volume wall, faces with ratios beyond
//              fixed-point range and full_iteration march per lane in FP64.
//              Field variants: each lane marches alone on a packed label +
//              chessboard-distance field (centred, or one per direction
//              octant) and steps over the increments the field proves to keep
//              their label; stops, class changes and len_path_2 are those of
//              the per-increment march.
//   lengths    (cal_path2_plus, :1462-1552): for A_h in FP32 (the segments and
//              len_path_2 come from the exact march; A_h needs 1e-6); for the
//              per-voxel detail and the gridding map in FP64 with the
//              reference's operation order, the per-segment quotient
//              fl(span / (len-1)) from a table of correctly rounded quotients,
//              or a correctly rounded reciprocal and one FMA correction.  A
//              leg that stopped at vacuum takes its last point from the march.
//   rate       (cal_rate, :1554-1583): FP32 exponent and exp; per-thread
//              Neumaier sums, warp-shuffle TwoSum reduction, tile partials
//              combined in FP64 in a fixed order (deterministic for any
//              schedule).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cstdlib>

#include "anacor_internal.h"
#include "device_math.cuh"
#include "trace_launch.h"

namespace anacor {

// g_num_rcp[d] = {(double)d, fl(1 / d)}: the quotient's operands without an
// integer-to-double conversion on the FP64 pipe
__device__ double2 g_num_rcp[kMaxDim + 2];

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
// CTAs per SM the absorption kernel's register budget is sized for: the
// kernel is instantiated for 1..4 (times the two marches); the plan's
// variant, or the process default (ANACOR_CTAS_PER_SM, default
// kDefaultMinBlocks), picks one.
constexpr int kDefaultMinBlocks = 4;
// Label loads a lane has in flight before checking them (divides 32).
constexpr int kMarchBatch = 8;
constexpr unsigned kAll = 0xffffffffu;

// The kernels' shared arrays (per-warp tables, segment lists, lane sums) are
// sized for kBlock threads.  A launch with any other block shape sets the
// ANACOR_ERR_ARGS bit in `status` (from one thread) and returns before any
// shared or global access; the test is uniform over the block, so no thread
// is left waiting at a barrier.
__device__ __forceinline__ bool block_shape_ok(int *status)
{
    if (blockDim.x == kBlock && blockDim.y == 1 && blockDim.z == 1)
        return true;
    if (status && threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0)
        atomicOr(status, 1 << kErrArgs);
    return false;
}

struct Vol {
    const int8_t *p;
    int dz, dy, dx;
    const uint8_t *field = nullptr;   // label | distance << 3, for the distance-field march
    long long field_stride = 0;       // 0: one centred field; else 8 octant fields this far apart
    int bsy = 0, bsz = 0;             // bricked fields: byte strides of a brick step in y and z
};

// Offset of voxel (z, y, x) in a field stored in 4x4x4 bricks of 64 bytes:
// bricks in (z, y, x) order, bytes inside a brick (z, y, x) with x fastest, so
// a 32-byte sector holds a 2x4x4 (z, y, x) box.  A ray that steps by one voxel
// along any axis mostly stays in the sector its previous load brought into L1
// (in the linear layout only steps along x do).
//
// Axis coordinate u = 4 U + w contributes U * BS + w * IS (BS the axis's
// brick stride, IS its stride inside a brick), which equals
// (u & ~3) * K + u * IS with K = BS / 4 - IS: a mask and two multiply-adds.
__device__ __forceinline__ int brick_term(int u, int k, int is)
{
    return (u & ~3) * k + u * is;
}

// K and IS of axis a (0 z, 1 y, 2 x)
__device__ __forceinline__ int brick_k(int a, const Vol &v)
{
    return a == 0 ? v.bsz / 4 - 16 : (a == 1 ? v.bsy / 4 - 4 : 64 / 4 - 1);
}

__device__ __forceinline__ int brick_is(int a)
{
    return 16 >> (2 * a);
}

__device__ __forceinline__ int brick_offset(int z, int y, int x, const Vol &v)
{
    return brick_term(z, brick_k(0, v), 16) + brick_term(y, brick_k(1, v), 4) + brick_term(x, brick_k(2, v), 1);
}

__device__ __forceinline__ int pick3(int k, int z, int y, int x)
{
    return k == 0 ? z : (k == 1 ? y : x);
}

// C's `int64_t n = floor(v)` / `round(v)`, then the reference's clamp.
// Out-of-range and NaN conversions give INT64_MIN (x86-64 behaviour).
__device__ __noinline__ int exact_axis(int c, int i, double q, bool use_round, int dim)
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
    const uint32_t sb = h.sign_bits;
    const bool hx = (sb & (4u | 32u)) != 0, hy = (sb & (2u | 16u)) != 0, hz = (sb & (1u | 8u)) != 0;
    if (cx == 0 && hx) return 6;
    if (cy == 0 && hy) return 4;
    if (cz == 0 && hz) return 2;
    // one candidate per axis: numerator n_a
    const int nx = (sb & 4u) ? v.dx - cx : cx;
    const int ny = (sb & 2u) ? v.dy - cy : cy;
    const int nz = (sb & 1u) ? v.dz - cz : cz;
    const float inf = __int_as_float(0x7f800000);
    const float tx = hx ? (float)nx * h.inv[2] : inf;
    const float ty = hy ? (float)ny * h.inv[1] : inf;
    const float tz = hz ? (float)nz * h.inv[0] : inf;
    // argmin with ties to the earlier axis (x, y, z)
    int best = 2;
    float t1 = tx, t2;
    if (ty < t1) { t2 = t1; t1 = ty; best = 1; } else { t2 = ty; }
    if (tz < t1) { t2 = t1; t1 = tz; best = 0; } else { t2 = fminf(t2, tz); }
    if ((sb & 64u) || !(t1 < inf && t2 > t1 * (1.0f + 0x1p-20f))) {
        // close call: the reference's FP64 quotients decide
        const double dinf = __longlong_as_double(0x7ff0000000000000ll);
        const double ex = hx ? __ddiv_rn((double)nx, fabs(h.e[2])) : dinf;
        const double ey = hy ? __ddiv_rn((double)ny, fabs(h.e[1])) : dinf;
        const double ez = hz ? __ddiv_rn((double)nz, fabs(h.e[0])) : dinf;
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

// fl(span / den): from the quotient table (row den holds span = 1 .. den+1)
// or from rcp = fl(1/den) with one FMA-exact remainder and one correction.
__device__ __forceinline__ double seg_quotient(const double *qtab, int den_i, int span, double den, double rcp)
{
    if (qtab)
        return __ldg(qtab + ((den_i - 1) * (den_i + 2)) / 2 + (span - 1));
    const double s = g_num_rcp[span].x;
    const double q0 = __dmul_rn(s, rcp);
    const double r = __fma_rn(-q0, den, s);
    return __fma_rn(r, rcp, q0);
}

// L[cls-1] += term in segment order.  The first term of a class is stored
// as is (0.0 + term == term for the non-negative terms of cal_path2_plus).
__device__ __forceinline__ void add_class(int cls, double term, int &seen, double *L)
{
    if (cls < 1 || cls > 4)
        return;
    const int bit = 1 << cls;
    double nv = term;
    if (seen & bit) {
        const double cur = cls == 1 ? L[0] : (cls == 2 ? L[1] : (cls == 3 ? L[2] : L[3]));
        nv = __dadd_rn(cur, term);
    }
    seen |= bit;
    L[0] = cls == 1 ? nv : L[0];
    L[1] = cls == 2 ? nv : L[1];
    L[2] = cls == 3 ? nv : L[2];
    L[3] = cls == 4 ? nv : L[3];
}

// Per-leg march state.  Accepted path points are the increments 0..last_i
// (the march never skips one), so len_path_2 = last_i + 1.
struct March {
    int last_i, nseg, prev, vac;
};

// Where class changes go: mode 0 records (class, start) in shared memory;
// mode 1 (second pass, when a leg has more class changes than the shared
// buffer holds) accumulates the lengths directly.
struct Sink {
    uint16_t *seg;      // stride kBlock
    const double *qtab;
    double tot, den, rcp;
    int den_i;
    double L[4];
    int open_cls, open_pos, seen;
};

template <int kMode>
__device__ __forceinline__ bool visit(March &m, Sink &sk, int i, int lab, int full, int vac_limit)
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
            const double q = seg_quotient(sk.qtab, sk.den_i, i - sk.open_pos, sk.den, sk.rcp);
            add_class(sk.open_cls, __dmul_rn(sk.tot, q), sk.seen, sk.L);
            sk.open_cls = lab;
            sk.open_pos = i;
        }
        m.nseg++;
    }
    m.last_i = i;
    m.prev = lab;
    return true;
}

// Geometry of one leg through one exit face in the face's own axis order:
// s = the step axis (the reference's loop axis, ratio exactly +-1), a and b
// the two other axes (32.32 fixed point).
struct LegGeom {
    int cs, ca, cb;          // start coordinates
    int hs, ha, hb;          // dim - 1
    int Ss, Sa, Sb;          // element strides
    int ds;                  // step direction (+1 / -1)
    int ia, ib;              // axis index (0 z, 1 y, 2 x) of a and b
    long long Qa, Qb;
    uint32_t Ma, Mb;         // ambiguity margins (0 for exact axes)
    long long off;           // 2^31 for round mode
};

__device__ __forceinline__ void leg_geom(const FaceRule &R, int cz, int cy, int cx, const Vol &v, LegGeom &g)
{
    const int s = R.count_axis;
    const int a = s == 0 ? 1 : 0;
    const int b = s == 2 ? 1 : 2;
    g.ia = a; g.ib = b;
    g.cs = pick3(s, cz, cy, cx); g.ca = pick3(a, cz, cy, cx); g.cb = pick3(b, cz, cy, cx);
    g.hs = pick3(s, v.dz, v.dy, v.dx) - 1; g.ha = pick3(a, v.dz, v.dy, v.dx) - 1;
    g.hb = pick3(b, v.dz, v.dy, v.dx) - 1;
    const int sz = v.dy * v.dx, sy = v.dx;
    g.Ss = pick3(s, sz, sy, 1); g.Sa = pick3(a, sz, sy, 1); g.Sb = pick3(b, sz, sy, 1);
    g.ds = R.Q[s] > 0 ? 1 : -1;   // the step axis's ratio is exactly +-1, so Q[s] = +-2^32
    g.Qa = R.Q[a]; g.Qb = R.Q[b];
    g.Ma = ((R.exact_mask >> a) & 1) ? 0u : kAmbiguityMargin;
    g.Mb = ((R.exact_mask >> b) & 1) ? 0u : kAmbiguityMargin;
    g.off = R.use_round ? 0x80000000ll : 0ll;
}

// Path point at increment i, (z, y, x).
__device__ __forceinline__ void point_at(const FaceRule &R, const LegGeom &g, int i, int cz, int cy, int cx,
                                         const Vol &v, int &pz, int &py, int &px)
{
    if (R.fast) {
        const int ps = min(max(g.cs + i * g.ds, 0), g.hs);
        const long long Ea = ((long long)g.ca << 32) + g.off + (long long)i * g.Qa;
        const long long Eb = ((long long)g.cb << 32) + g.off + (long long)i * g.Qb;
        int pa, pb;
        if (((uint32_t)Ea + g.Ma < 2u * g.Ma) | ((uint32_t)Eb + g.Mb < 2u * g.Mb)) {
            pa = exact_axis(g.ca, i, R.q[g.ia], R.use_round, g.ha + 1);
            pb = exact_axis(g.cb, i, R.q[g.ib], R.use_round, g.hb + 1);
        } else {
            pa = min(max((int)(Ea >> 32), 0), g.ha);
            pb = min(max((int)(Eb >> 32), 0), g.hb);
        }
        const int s = R.count_axis;
        pz = s == 0 ? ps : pa;
        py = s == 1 ? ps : (s == 0 ? pa : pb);
        px = s == 2 ? ps : pb;
    } else {
        pz = exact_axis(cz, i, R.q[0], R.use_round, v.dz);
        py = exact_axis(cy, i, R.q[1], R.use_round, v.dy);
        px = exact_axis(cx, i, R.q[2], R.use_round, v.dx);
    }
}

// Per-lane march (cal_coord) for the lanes the cooperative march does not
// take: walls within reach, huge ratios, full_iteration; the second pass; and
// (i_begin > 0) the increments after the cooperative part of a leg that did
// not stop before the cooperative march's wall limit, continuing `m`.
//
// Out of line, with everything it needs passed by value or recomputed: a
// by-reference argument whose object lives in the caller's registers would
// move that object to the stack for the whole of the caller.
template <int kMode>
__device__ __noinline__ void march_lane(const FaceRule &R, int cz, int cy, int cx, int steps, const Vol v, int full,
                                        March &m, Sink &sk, int i_begin = 0)
{
    LegGeom g;
    leg_geom(R, cz, cy, cx, v, g);
    const int sz = v.dy * v.dx, sy = v.dx;
    int z, y, x;
    if (i_begin > 0) {
        for (int i = i_begin; i < steps; i++) {
            point_at(R, g, i, cz, cy, cx, v, z, y, x);
            if (!visit<kMode>(m, sk, i, __ldg(v.p + (z * sz + y * sy + x)), full, R.vac_limit))
                return;
        }
        return;
    }
    m.last_i = 0; m.nseg = 1; m.vac = 0;
    if (kMode == 0)
        sk.seg[0] = (uint16_t)(3 << 13);
    if (steps <= 0)
        return;
    point_at(R, g, 0, cz, cy, cx, v, z, y, x);
    const int lab = __ldg(v.p + (z * sz + y * sy + x));
    if (!full) {
        if (lab == 0)
            return;
    } else {
        m.vac = lab == 0;
        if (m.vac > R.vac_limit)
            return;
    }
    m.prev = lab;
    for (int i = 1; i < steps; i++) {
        point_at(R, g, i, cz, cy, cx, v, z, y, x);
        if (!visit<kMode>(m, sk, i, __ldg(v.p + (z * sz + y * sy + x)), full, R.vac_limit))
            return;
    }
}

// Byte of `bytes` (the label volume or its packed distance field) at
// increment `inc`, from the reference's FP64 expression (an increment whose
// fixed-point fraction lies near a rounding boundary).
__device__ __noinline__ uint32_t exact_byte(const FaceRule &G, int cz, int cy, int cx, int inc, const Vol v,
                                            const uint8_t *bytes, bool brick)
{
    int pz, py, px;
    const int s = G.count_axis;
    const int ds = G.q[s] > 0.0 ? 1 : -1;
    pz = s == 0 ? cz + inc * ds : exact_axis(cz, inc, G.q[0], G.use_round, v.dz);
    py = s == 1 ? cy + inc * ds : exact_axis(cy, inc, G.q[1], G.use_round, v.dy);
    px = s == 2 ? cx + inc * ds : exact_axis(cx, inc, G.q[2], G.use_round, v.dx);
    return (uint32_t)__ldg(bytes + (brick ? brick_offset(pz, py, px, v) : (pz * v.dy + py) * v.dx + px));
}

__device__ __forceinline__ uint32_t exact_label(const FaceRule &G, int cz, int cy, int cx, int inc, const Vol &v)
{
    return exact_byte(G, cz, cy, cx, inc, v, reinterpret_cast<const uint8_t *>(v.p), false);
}

// Increments i >= 0 for which c + i*q stays at least 2 voxels inside [0, h]
// (an estimate in FP32 with a margin; -1 when increment 0 is already too
// close).  The cooperative march's end-point test decides; this only picks
// the end point.
__device__ __forceinline__ int wall_increments(double q, int c, int h)
{
    const float qf = (float)q;
    float k;
    if (qf > 0.0f)
        k = __fdiv_rn((float)(h - 2 - c), qf);
    else if (qf < 0.0f)
        k = __fdiv_rn((float)(c - 2), -qf);
    else
        return (c >= 1 && c <= h - 1) ? 0x3fffffff : -1;
    if (!(k >= 0.0f))
        return -1;
    return (int)fminf(floorf(k * 0.9999f), 1.0e9f);
}

// Distance-field march of one lane over increments 1 .. lim-1 (all clear of
// the volume's walls, as for the cooperative march).  The field byte of the
// current increment i gives the label and D, the chessboard distance to the
// nearest voxel with another label.  Increment i + n lies n voxels away on
// the step axis and at most ceil(n qmax) + 1 on the other two (two roundings
// of c + n q), so every increment up to i + nmax(D) with
//     nmax(D) = min(D - 1, floor((D - 2) / qmax))
// carries increment i's label: it is accepted without a load, and the march
// goes on at i + nmax + 1.  Labels, stops, class changes and len_path_2 are
// therefore exactly those of the per-increment march.
// One lane's field march over one leg, as a chain of dependent loads.  With
// a bricked field (kBrick) the chain holds absolute coordinates instead of
// linear strides (the members of the other layout are never set).
struct FieldChain {
    const FaceRule *R;
    const uint8_t *fld;       // the field this leg marches on (its octant's)
    const uint8_t *pk;        // linear: fld + the leg's start voxel
    long long off, Qa, Qb;    // bricked: off of axis a, offb of axis b, with the start coordinates
    long long offb;
    uint32_t Ma, Mb, rq;
    int dS, Sa, Sb;           // linear: strides of the step axis (signed) and the two others
    int cs, ds;               // bricked: start coordinate and direction on the step axis
    int k_s, k_a, k_b;        // bricked: brick_term's K of the step axis and the two others
    int is_s, is_a, is_b;     // bricked: their in-brick strides
    int i, lim, last, prev, nseg;
    bool on;
};

__device__ __forceinline__ int field_nmax(uint32_t d, uint32_t rq)
{
    return d < 2u ? 0 : min((int)d - 1, (int)(((d - 2u) * rq) >> 16));
}

template <bool kBrick>
__device__ __forceinline__ void chain_init(FieldChain &c, const FaceRule &R, const LegGeom &g, const uint8_t *fld,
                                           int base, int lim, uint32_t b0, const March &m, const Vol &v)
{
    c.R = &R;
    c.fld = fld;
    c.Qa = g.Qa;
    c.Qb = g.Qb;
    c.Ma = g.Ma;
    c.Mb = g.Mb;
    c.rq = R.skip_rq;   // below 2^16 / qmax: the skip never exceeds nmax
    if (kBrick) {
        // adding c * 2^32 changes neither the fraction nor the ambiguity test
        c.off = ((long long)g.ca << 32) + g.off;
        c.offb = ((long long)g.cb << 32) + g.off;
        c.cs = g.cs;
        c.ds = g.ds;
        const int s = R.count_axis;
        c.k_s = brick_k(s, v);
        c.k_a = brick_k(g.ia, v);
        c.k_b = brick_k(g.ib, v);
        c.is_s = brick_is(s);
        c.is_a = brick_is(g.ia);
        c.is_b = brick_is(g.ib);
    } else {
        c.pk = fld + base;
        c.off = g.off;
        c.dS = g.ds * g.Ss;
        c.Sa = g.Sa;
        c.Sb = g.Sb;
    }
    c.lim = lim;
    c.prev = m.prev;
    c.nseg = m.nseg;
    c.i = 1 + field_nmax(b0 >> 3, c.rq);
    c.last = min(c.i - 1, lim - 1);
    c.on = c.i < lim;
}

// field byte of the chain's current increment
template <bool kBrick>
__device__ __forceinline__ uint32_t chain_load(const FieldChain &c, int cz, int cy, int cx, const Vol &v)
{
    const long long ea = c.off + (long long)c.i * c.Qa;
    const long long eb = (kBrick ? c.offb : c.off) + (long long)c.i * c.Qb;
    if (((uint32_t)ea + c.Ma < 2u * c.Ma) | ((uint32_t)eb + c.Mb < 2u * c.Mb))
        return exact_byte(*c.R, cz, cy, cx, c.i, v, c.fld, kBrick);
    if (kBrick)
        return __ldg(c.fld + (brick_term(c.cs + c.i * c.ds, c.k_s, c.is_s) + brick_term((int)(ea >> 32), c.k_a, c.is_a) +
                              brick_term((int)(eb >> 32), c.k_b, c.is_b)));
    return __ldg(c.pk + (c.i * c.dS + (int)(ea >> 32) * c.Sa + (int)(eb >> 32) * c.Sb));
}

// the stop / class-change test of the current increment, then the skip
__device__ __forceinline__ void chain_step(FieldChain &c, uint32_t b, uint16_t *seg, bool &stopped)
{
    const int lab = (int)(b & 7u);
    if (lab == 0) {
        stopped = true;
        c.last = c.i - 1;
        c.on = false;
        return;
    }
    if (lab != c.prev) {
        if (lab <= 4) {
            if (c.nseg < kMaxSegments)
                seg[c.nseg * kBlock] = (uint16_t)((lab << 13) | c.i);
            c.nseg++;
        }
        c.prev = lab;
    }
    const int n = field_nmax(b >> 3, c.rq);
    c.last = min(c.i + n, c.lim - 1);
    c.i += n + 1;
    c.on = c.i < c.lim;
}

__device__ __forceinline__ void chain_done(const FieldChain &c, March &m)
{
    m.last_i = c.last;
    m.prev = c.prev;
    m.nseg = c.nseg;
}

// The march of one lane on its field.  dlast: |displacement| of the last
// accepted increment on the two non-step axes (a | b << 16), when its
// fixed-point position is not near a rounding boundary; else -1.
template <bool kBrick>
__device__ __forceinline__ void field_march(const FaceRule &R, const LegGeom &g, int cz, int cy, int cx,
                                            const Vol &v, const uint8_t *fld, int base, int lim, uint32_t b0,
                                            March &m, bool &stopped, uint16_t *seg, int &dlast)
{
    FieldChain c;
    chain_init<kBrick>(c, R, g, fld, base, lim, b0, m, v);
    while (c.on)
        chain_step(c, chain_load<kBrick>(c, cz, cy, cx, v), seg, stopped);
    chain_done(c, m);
    const long long ea = g.off + (long long)c.last * g.Qa, eb = g.off + (long long)c.last * g.Qb;
    const bool amb = ((uint32_t)ea + c.Ma < 2u * c.Ma) | ((uint32_t)eb + c.Mb < 2u * c.Mb);
    dlast = amb ? -1 : (abs((int)(ea >> 32)) | abs((int)(eb >> 32)) << 16);
}

// fl(fl(d * v_axis)^2), from the sample's table when it has one
__device__ __forceinline__ double sq_len(const double *sq, int stride, int axis, int d, double vox)
{
    if (sq)
        return __ldg(sq + axis * stride + d);
    const double t = __dmul_rn((double)d, vox);
    return __dmul_rn(t, t);
}

struct L4 {
    double v[4];
};

// cal_path2_plus by a second march, accumulating segments as they close (a
// leg with more class changes than the shared buffer holds), out of line.
__device__ __noinline__ L4 lengths_second_pass(const FaceRule &R, int cz, int cy, int cx, int steps, const Vol v,
                                               int full, int len, int fz, int fy, int fx, int lz, int ly, int lx,
                                               const double *voxel, const double *sq, int sq_stride,
                                               const double *qtab, uint16_t *seg)
{
    const double yy = sq_len(sq, sq_stride, 1, abs(ly - fy), voxel[1]);
    const double zz = sq_len(sq, sq_stride, 0, abs(lz - fz), voxel[0]);
    const double xx = sq_len(sq, sq_stride, 2, abs(lx - fx), voxel[2]);
    const double tot = __dsqrt_rn(__dadd_rn(__dadd_rn(yy, zz), xx));
    const int den_i = len - 1;
    const double2 dr = g_num_rcp[den_i];
    March m2;
    Sink s2;
    s2.seg = seg;
    s2.qtab = qtab;
    s2.tot = tot; s2.den = dr.x; s2.rcp = dr.y; s2.den_i = den_i;
    s2.L[0] = s2.L[1] = s2.L[2] = s2.L[3] = 0.0;
    s2.open_cls = 3; s2.open_pos = 0; s2.seen = 0;
    march_lane<1>(R, cz, cy, cx, steps, v, full, m2, s2);
    const double q = seg_quotient(qtab, den_i, len - s2.open_pos, dr.x, dr.y);
    add_class(s2.open_cls, __dmul_rn(tot, q), s2.seen, s2.L);
    L4 r;
    for (int k = 0; k < 4; k++)
        r.v[k] = s2.L[k];
    return r;
}

struct LegResult {
    double L[4];       // FP64 lengths (kF32 == false)
    float Lf[4];       // FP32 lengths (kF32 == true)
    int face, len, nseg, status;
    int first[3], last[3];
};


// cal_path2_plus in FP32 for A_h: total = |(dz, dy, dx) * voxel| (y, z, x
// order) and tot * (span / (len - 1)) per class segment of the shared buffer.
__device__ __forceinline__ void lengths_f32(int dz, int dy, int dx, int len, int nseg, const uint16_t *seg,
                                            const double *voxel, const float *voxelf, LegResult &out)
{
    const float vy = voxelf ? voxelf[1] : (float)voxel[1];
    const float vz = voxelf ? voxelf[0] : (float)voxel[0];
    const float vx = voxelf ? voxelf[2] : (float)voxel[2];
    const float ty = __fmul_rn((float)dy, vy);
    const float tz = __fmul_rn((float)dz, vz);
    const float tx = __fmul_rn((float)dx, vx);
    const float totf = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ty, ty), __fmul_rn(tz, tz)), __fmul_rn(tx, tx)));
    const float scale = __fdiv_rn(totf, (float)(len - 1));
    int cur = seg[0];
    for (int j = 0; j < nseg; j++) {
        const int nxt = (j + 1 < nseg) ? (int)seg[(j + 1) * kBlock] : -1;
        const int start = cur & 0x1fff;
        const int end = (j + 1 < nseg) ? (nxt & 0x1fff) : len;
        const int cls = cur >> 13;
        const float term = scale * (float)(end - start);
        out.Lf[0] += cls == 1 ? term : 0.0f;
        out.Lf[1] += cls == 2 ? term : 0.0f;
        out.Lf[2] += cls == 3 ? term : 0.0f;
        out.Lf[3] += cls == 4 ? term : 0.0f;
        cur = nxt;
    }
}

// cal_path2_plus in FP64, bit for bit as the reference: total from the
// squares fl(fl(d * voxel)^2) summed y, z, x, then tot * fl(span / (len - 1))
// per class segment of the shared buffer, added in segment order.
__device__ __forceinline__ void lengths_f64(int dz, int dy, int dx, int len, int nseg, const uint16_t *seg,
                                            const double *voxel, const double *sq, int sq_stride, const double *qtab,
                                            LegResult &out)
{
    const double yy = sq_len(sq, sq_stride, 1, dy, voxel[1]);
    const double zz = sq_len(sq, sq_stride, 0, dz, voxel[0]);
    const double xx = sq_len(sq, sq_stride, 2, dx, voxel[2]);
    const double tot = __dsqrt_rn(__dadd_rn(__dadd_rn(yy, zz), xx));
    const int den_i = len - 1;
    const double2 dr = g_num_rcp[den_i];
    int seen = 0;
    int cur = seg[0];
    for (int j = 0; j < nseg; j++) {
        const int nxt = (j + 1 < nseg) ? (int)seg[(j + 1) * kBlock] : -1;
        const int start = cur & 0x1fff;
        const int end = (j + 1 < nseg) ? (nxt & 0x1fff) : len;
        const double q = seg_quotient(qtab, den_i, end - start, dr.x, dr.y);
        add_class(cur >> 13, __dmul_rn(tot, q), seen, out.L);
        cur = nxt;
    }
}

// State of one leg between its set-up, its march and its lengths.
struct LegState {
    March m;
    int face, lim, base;
    bool need, coop, stopped, live;
    uint32_t b0;   // field byte of increment 0 (field march)
    int dlast;     // field march: the last point's displacement (see field_march), else -1
};

// cube_face and the march set-up of one leg (warp-synchronous).  With kField
// the lane's field march runs here too.
template <bool kDetail, bool kField, bool kBrick>
__device__ __forceinline__ void leg_setup(const LegHead &h, const FaceRule *rules, int cz, int cy, int cx, bool valid,
                                          const Vol &v, int full, uint16_t *seg, LegResult &out, LegState &S)
{
    out.L[0] = out.L[1] = out.L[2] = out.L[3] = 0.0;
    out.Lf[0] = out.Lf[1] = out.Lf[2] = out.Lf[3] = 0.0f;
    out.len = 1; out.nseg = 1; out.status = kOk;
    if (kDetail) {
        out.first[0] = cz; out.first[1] = cy; out.first[2] = cx;
        out.last[0] = cz; out.last[1] = cy; out.last[2] = cx;
    }
    const int face = valid ? exit_face(h, cz, cy, cx, v) : 0;
    out.face = face;
    bool need = valid;
    if (valid && face == 0) {
        out.status = kErrNoFace;
        need = false;
    }
    if (need && rules[face - 1].status) {
        out.status = rules[face - 1].status;
        need = false;
    }
    March m;
    m.last_i = 0; m.nseg = 1; m.vac = 0; m.prev = 0;

    // ---- set-up: step count, cooperative eligibility, increment 0.  Only a
    // few values cross the cooperative loop; the geometry is recomputed after.
    bool coop = false, stopped = false, live = false;
    int lim = 0, base = 0;
    uint32_t b0 = 0;
    int dlast = -1;
    if (need) {
        const FaceRule &R = rules[face - 1];
        LegGeom g;
        leg_geom(R, cz, cy, cx, v, g);
        const int cc = pick3(R.count_axis, cz, cy, cx);
        const int dd = pick3(R.count_axis, v.dz, v.dy, v.dx);
        const int steps = R.count_kind == 0 ? cc + 1 : (R.count_kind == 1 ? dd - cc : dd - cc + 1);
        // the last increment of a count_kind 2 face clamps the step axis; it is
        // taken separately after the cooperative part
        const int steps_eff = R.count_kind == 2 ? steps - 1 : steps;
        coop = R.fast && !full && steps >= 1;
        lim = steps_eff;
        if (coop && steps_eff > 1) {
            // No increment of the cooperative part may clamp: its first and last
            // points (the path is monotone on every axis) lie at least one voxel
            // inside the volume.  When the volume's far wall is within reach of
            // the full leg, the cooperative part ends at the last increment that
            // stays clear of it; a leg still running there continues per lane.
            int kend = steps_eff - 1;
            for (int pass = 0; pass < 2; pass++) {
                const long long ena = g.off + (long long)kend * g.Qa;
                const long long enb = g.off + (long long)kend * g.Qb;
                const int a1 = g.ca + (int)((g.off + g.Qa) >> 32), an = g.ca + (int)(ena >> 32);
                const int b1 = g.cb + (int)((g.off + g.Qb) >> 32), bn = g.cb + (int)(enb >> 32);
                coop = min(a1, an) >= 1 && max(a1, an) <= g.ha - 1 && min(b1, bn) >= 1 && max(b1, bn) <= g.hb - 1;
                if (coop || pass == 1)
                    break;
                kend = min(kend, min(wall_increments(R.q[g.ia], g.ca, g.ha), wall_increments(R.q[g.ib], g.cb, g.hb)));
                if (kend < 1)
                    break;
            }
            lim = kend + 1;
        }
        if (coop) {
            base = g.cs * g.Ss + g.ca * g.Sa + g.cb * g.Sb;
            seg[0] = (uint16_t)(3 << 13);
            if (kField) {
                // per lane, no warp synchronisation: the field march
                const uint8_t *fld = v.field + R.octant * v.field_stride;
                b0 = __ldg(fld + (kBrick ? brick_offset(cz, cy, cx, v) : base));
                if ((b0 & 7u) == 0) {
                    stopped = true;
                } else {
                    m.prev = (int)(b0 & 7u);
                    live = lim > 1;
                    if (live)
                        field_march<kBrick>(R, g, cz, cy, cx, v, fld, base, lim, b0, m, stopped, seg, dlast);
                }
            } else {
                const int lab0 = __ldg(v.p + base);
                if (lab0 == 0) {
                    stopped = true;
                } else {
                    m.prev = lab0;
                    live = lim > 1;
                }
            }
        }
    }

    S.m = m;
    S.face = face;
    S.lim = lim;
    S.base = base;
    S.need = need;
    S.coop = coop;
    S.stopped = stopped;
    S.live = live;
    S.b0 = b0;
    S.dlast = dlast;
}

// The warp-cooperative march of the legs set up by leg_setup<.., false>.
__device__ __forceinline__ void leg_coop(const FaceRule *rules, int cz, int cy, int cx, const Vol &v, uint16_t *seg,
                                         LegState &S)
{
    const int lane = threadIdx.x & 31;
    const int face = S.face, lim = S.lim, base = S.base;
    const bool coop = S.coop, live = S.live;
    bool stopped = S.stopped;
    March m = S.m;
    // ---- cooperative march, one exit-face group at a time
    unsigned pend = __ballot_sync(kAll, coop);
    while (pend) {
        const int f = __shfl_sync(kAll, face, __ffs(pend) - 1);
        const unsigned grp = __ballot_sync(kAll, coop && face == f);
        pend &= ~grp;
        const bool mine = (grp >> lane) & 1u;
        const FaceRule &G = rules[f - 1];
        const int glim = mine ? lim : 0;
        const int gmax = __reduce_max_sync(kAll, glim);
        const uint8_t *p = reinterpret_cast<const uint8_t *>(v.p) + base;
        bool on = mine && live;
        uint32_t prev4 = (uint32_t)(uint8_t)m.prev * 0x01010101u;
        for (int i0 = 1; i0 < gmax; i0 += 32) {
            if (!__any_sync(kAll, on))
                break;
            int delta;
            unsigned ambm;
            {
                // group constants, re-read from shared memory per chunk
                const int gs = G.count_axis, ga = gs == 0 ? 1 : 0, gb = gs == 2 ? 1 : 2;
                const int sz = v.dy * v.dx, sy = v.dx;
                const int ds = G.Q[gs] > 0 ? 1 : -1;
                const long long off = G.use_round ? 0x80000000ll : 0ll;
                const uint32_t Ma = ((G.exact_mask >> ga) & 1) ? 0u : kAmbiguityMargin;
                const uint32_t Mb = ((G.exact_mask >> gb) & 1) ? 0u : kAmbiguityMargin;
                const int i = i0 + lane;
                const long long ea = off + (long long)i * G.Q[ga], eb = off + (long long)i * G.Q[gb];
                const bool amb = ((uint32_t)ea + Ma < 2u * Ma) | ((uint32_t)eb + Mb < 2u * Mb);
                delta = i * ds * pick3(gs, sz, sy, 1) + (int)(ea >> 32) * pick3(ga, sz, sy, 1) +
                        (int)(eb >> 32) * pick3(gb, sz, sy, 1);
                ambm = __ballot_sync(kAll, amb);
            }
#pragma unroll 1
            for (int t = 0; t < 32; t += kMarchBatch) {
                if (!__any_sync(kAll, on))
                    break;
                const int ib = i0 + t;
                const int n = on ? glim - ib : 0;   // increments this lane still takes
                // kMarchBatch label loads in flight per lane before any is checked
                uint32_t lb[kMarchBatch];
#pragma unroll
                for (int k = 0; k < kMarchBatch; k++) {
                    const int dk = __shfl_sync(kAll, delta, t + k);
                    lb[k] = k < n ? (uint32_t)__ldg(p + dk) : 0u;
                }
                const unsigned amb_here = (ambm >> t) & ((1u << kMarchBatch) - 1u);
                if (amb_here) {
                    // the reference's FP64 expression decides, per lane (c enters its rounding)
#pragma unroll
                    for (int k = 0; k < kMarchBatch; k++)
                        if (((amb_here >> k) & 1u) && k < n)
                            lb[k] = exact_label(G, cz, cy, cx, ib + k, v);
                }
                if (n > 0) {
                    // Four increments per packed word.  prev is never 0 here, so
                    // a word equal to prev4 holds neither a stop nor a class
                    // change: the common case costs one compare per word.
                    const uint32_t w0 = lb[0] | (lb[1] << 8) | (lb[2] << 16) | (lb[3] << 24);
                    const uint32_t w1 = lb[4] | (lb[5] << 8) | (lb[6] << 16) | (lb[7] << 24);
                    if (n >= kMarchBatch && w0 == prev4 && w1 == prev4) {
                        m.last_i = ib + kMarchBatch - 1;
                    } else {
#pragma unroll
                        for (int q = 0; q < 2; q++) {
                            const int nq = n - 4 * q;
                            if (stopped || nq <= 0)
                                break;
                            const uint32_t w = q == 0 ? w0 : w1;
                            const int b4 = ib + 4 * q;
                            const uint32_t valid_bytes = nq >= 4 ? 0xffffffffu : (1u << (8 * nq)) - 1u;
                            // the lowest set bit of w ^ prev4 lies in the first byte
                            // that differs: a stop (0) or a class change
                            uint32_t x = (w ^ prev4) & valid_bytes;
                            while (x) {
                                const int byte = (__ffs(x) - 1) >> 3;
                                const int lab = (int)(signed char)(w >> (8 * byte));
                                const int inc = b4 + byte;
                                if (lab == 0) {
                                    stopped = true;
                                    m.last_i = inc - 1;
                                    break;
                                }
                                if ((unsigned)lab <= 4u) {
                                    if (m.nseg < kMaxSegments)
                                        seg[m.nseg * kBlock] = (uint16_t)((lab << 13) | inc);
                                    m.nseg++;
                                }
                                m.prev = lab;
                                prev4 = (uint32_t)(uint8_t)lab * 0x01010101u;
                                const uint32_t above = byte == 3 ? 0u : (0xffffffffu << (8 * (byte + 1)));
                                x = (w ^ prev4) & valid_bytes & above;
                            }
                            if (!stopped)
                                m.last_i = b4 + min(nq, 4) - 1;
                        }
                    }
                    if (stopped || n <= kMarchBatch)
                        on = false;
                }
            }
        }
    }
    S.m = m;
    S.stopped = stopped;
    if (coop && stopped) {
        // the last point of a leg that stopped at vacuum, as the field march
        // gives it (see field_march's dlast)
        const FaceRule &R = rules[face - 1];
        const int s = R.count_axis, a = s == 0 ? 1 : 0, b = s == 2 ? 1 : 2;
        const long long off = R.use_round ? 0x80000000ll : 0ll;
        const uint32_t Ma = ((R.exact_mask >> a) & 1) ? 0u : kAmbiguityMargin;
        const uint32_t Mb = ((R.exact_mask >> b) & 1) ? 0u : kAmbiguityMargin;
        const long long ea = off + (long long)m.last_i * R.Q[a], eb = off + (long long)m.last_i * R.Q[b];
        const bool amb = ((uint32_t)ea + Ma < 2u * Ma) | ((uint32_t)eb + Mb < 2u * Mb);
        S.dlast = amb ? -1 : (abs((int)(ea >> 32)) | abs((int)(eb >> 32)) << 16);
    }
}

// After the march: the per-lane remainder of the path and cal_path2_plus.
template <bool kDetail, bool kF32>
__device__ __forceinline__ void leg_finish(const FaceRule *rules, int cz, int cy, int cx, const Vol &v, int full,
                                           const double *voxel, const double *sq, int sq_stride, const double *qtab,
                                           uint16_t *seg, LegState &S, LegResult &out, const float *voxelf)
{
    const int face = S.face, lim = S.lim;
    const bool need = S.need, coop = S.coop, stopped = S.stopped;
    March m = S.m;
    Sink sk;
    sk.seg = seg;
    if (!need)
        return;

    if (!kDetail && coop && stopped && S.dlast >= 0 && m.nseg <= kMaxSegments) {
        // a field march that stopped at vacuum: the last point is known
        // (step axis: last_i increments; the others: dlast), so the lengths
        // need neither the geometry nor the point
        const int len = m.last_i + 1;
        out.len = len;
        out.nseg = m.nseg;
        if (len == 1)
            return;
        const int s = rules[face - 1].count_axis;
        const int da = S.dlast & 0xffff, db = S.dlast >> 16;
        const int d0 = s == 0 ? m.last_i : da;
        const int d1 = s == 1 ? m.last_i : (s == 0 ? da : db);
        const int d2 = s == 2 ? m.last_i : db;
        if (kF32)
            lengths_f32(d0, d1, d2, len, m.nseg, seg, voxel, voxelf, out);
        else
            lengths_f64(d0, d1, d2, len, m.nseg, seg, voxel, sq, sq_stride, qtab, out);
        return;
    }

    // ---- after the march: geometry again, the per-lane paths, lengths
    const FaceRule &R = rules[face - 1];
    LegGeom g;
    leg_geom(R, cz, cy, cx, v, g);
    const int cc = pick3(R.count_axis, cz, cy, cx);
    const int dd = pick3(R.count_axis, v.dz, v.dy, v.dx);
    const int steps = R.count_kind == 0 ? cc + 1 : (R.count_kind == 1 ? dd - cc : dd - cc + 1);
    if (coop && !stopped && lim < (R.count_kind == 2 ? steps - 1 : steps)) {
        // the cooperative part ended at the wall limit: the rest per lane
        March mc = m;
        Sink sc;
        sc.seg = seg;
        march_lane<0>(R, cz, cy, cx, steps, v, full, mc, sc, lim);
        m = mc;
    } else if (coop && !stopped && R.count_kind == 2) {
        // the clamped last increment of a count_kind 2 face
        int pz, py, px;
        const int inc = steps - 1;
        point_at(R, g, inc, cz, cy, cx, v, pz, py, px);
        const int lab = __ldg(v.p + (pz * v.dy * v.dx + py * v.dx + px));
        if (inc >= 1)
            visit<0>(m, sk, inc, lab, 0, R.vac_limit);
    }
    if (!coop) {
        // separate objects for the out-of-line call (see march_lane)
        March mc = m;
        Sink sc;
        sc.seg = seg;
        march_lane<0>(R, cz, cy, cx, steps, v, full, mc, sc);
        m = mc;
    }

    // ---- cal_path2_plus
    const int len = m.last_i + 1;
    out.len = len;
    out.nseg = m.nseg;
    if (len == 1 && !kDetail)
        return;
    int fz = cz, fy = cy, fx = cx;
    if (!R.fast)
        point_at(R, g, 0, cz, cy, cx, v, fz, fy, fx);
    int lz, ly, lx;
    point_at(R, g, m.last_i, cz, cy, cx, v, lz, ly, lx);
    if (kDetail) {
        out.first[0] = fz; out.first[1] = fy; out.first[2] = fx;
        out.last[0] = lz; out.last[1] = ly; out.last[2] = lx;
        if (len == 1)
            return;
    }
    if (kF32 && m.nseg <= kMaxSegments) {
        lengths_f32(abs(lz - fz), abs(ly - fy), abs(lx - fx), len, m.nseg, seg, voxel, voxelf, out);
        return;
    }
    if (kF32) {
        const L4 r = lengths_second_pass(R, cz, cy, cx, steps, v, full, len, fz, fy, fx, lz, ly, lx, voxel, sq,
                                         sq_stride, qtab, seg);
        for (int k = 0; k < 4; k++)
            out.Lf[k] = (float)r.v[k];
        return;
    }
    if (m.nseg <= kMaxSegments) {
        lengths_f64(abs(lz - fz), abs(ly - fy), abs(lx - fx), len, m.nseg, seg, voxel, sq, sq_stride, qtab, out);
    } else {
        // total from the first and last path points, y then z then x
        const double yy = sq_len(sq, sq_stride, 1, abs(ly - fy), voxel[1]);
        const double zz = sq_len(sq, sq_stride, 0, abs(lz - fz), voxel[0]);
        const double xx = sq_len(sq, sq_stride, 2, abs(lx - fx), voxel[2]);
        const double tot = __dsqrt_rn(__dadd_rn(__dadd_rn(yy, zz), xx));
        const int den_i = len - 1;
        const double2 dr = g_num_rcp[den_i];
        // more class changes than the shared buffer holds: march again and
        // accumulate as segments close (same terms, same order)
        March m2;
        Sink s2;
        s2.seg = seg;
        s2.qtab = qtab;
        s2.tot = tot; s2.den = dr.x; s2.rcp = dr.y; s2.den_i = den_i;
        s2.L[0] = s2.L[1] = s2.L[2] = s2.L[3] = 0.0;
        s2.open_cls = 3; s2.open_pos = 0; s2.seen = 0;
        march_lane<1>(R, cz, cy, cx, steps, v, full, m2, s2);
        const double q = seg_quotient(qtab, den_i, len - s2.open_pos, dr.x, dr.y);
        add_class(s2.open_cls, __dmul_rn(tot, q), s2.seen, s2.L);
        for (int k = 0; k < 4; k++) {
            out.L[k] = s2.L[k];
            out.Lf[k] = (float)s2.L[k];
        }
    }
}

// cube_face + cal_coord + cal_path2_plus for one leg.  Called by all 32 lanes
// of a warp together (warp-synchronous); `valid` marks lanes that hold a voxel.
//
// Warp-cooperative march: lanes whose rays leave through the same face share
// that face's step rule, and their 32.32 positions differ only in the integer
// part (c * 2^32).  So the displacement of increment i -- and whether its
// fraction is near a rounding boundary -- is the same for every lane of the
// group: lane j computes it for increment i0 + j, the warp broadcasts it with
// shuffles, and each lane only adds it to its own start address, loads the
// label and checks it.  A lane joins the group only if no clamp can occur on
// its increments (both end points at least one voxel inside the volume) and
// the face has fixed-point ratios; other lanes, and full_iteration, use the
// per-lane march.
// kF32: the per-class lengths in FP32 (for A_h, which needs 1e-6; the march
// itself, and hence the visited voxels, segments and len_path_2, is the same);
// otherwise FP64 in the reference's order (bit-exact lengths).
template <bool kDetail, bool kF32 = false, bool kField = false, bool kBrick = false>
__device__ __forceinline__ void trace_leg(const LegHead &h, const FaceRule *rules, int cz, int cy, int cx,
                                          bool valid, const Vol &v, int full, const double *voxel,
                                          const double *sq, int sq_stride, const double *qtab, uint16_t *seg,
                                          LegResult &out, const float *voxelf = nullptr)
{
    LegState S;
    leg_setup<kDetail, kField, kBrick>(h, rules, cz, cy, cx, valid, v, full, seg, out, S);
    if (!kField)
        leg_coop(rules, cz, cy, cx, v, seg, S);
    leg_finish<kDetail, kF32>(rules, cz, cy, cx, v, full, voxel, sq, sq_stride, qtab, seg, S, out, voxelf);
}

__device__ __forceinline__ int find_sample(const SampleDesc *d, int n, long long item)
{
    int s = 0;
    while (s + 1 < n && item >= d[s + 1].work_begin)
        s++;
    return s;
}

// End of a work item: block reduction of the per-thread compensated sums
// (warp-shuffle TwoSum, then across warps), the item's FP64 partial, and --
// for the last tile of the reflection to arrive -- the fixed-order
// combination of the partials into A_h.
__device__ __forceinline__ void finish_item(float s, float c, const SampleDesc &D, long long r, int t, float *red_s,
                                            float *red_c, int &last_s)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float so = __shfl_down_sync(kAll, s, o);
        const float co = __shfl_down_sync(kAll, c, o);
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
        const volatile double *pp = D.partial + r * D.tiles;
        double acc = 0.0;
        for (int k = lane; k < D.tiles; k += 32)
            acc += pp[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            acc += __shfl_down_sync(kAll, acc, o);
        if (lane == 0) {
            D.out[r] = acc / (double)D.n_vox;
            D.arrive[r] = 0u;   // ready for the next launch
        }
    }
}

template <int kMinBlocks, bool kField, bool kBrick = false>
__global__ void __launch_bounds__(kBlock, kMinBlocks) absorption_kernel(const SampleDesc *__restrict__ descs,
                                                                        int n_desc, long long total_items,
                                                                        unsigned long long *__restrict__ work_counter)
{
    __shared__ ReflTable tabs[kWarps];   // one per warp: items are taken per warp
    __shared__ uint16_t seg[kMaxSegments * kBlock];
    __shared__ float lsum[4][kBlock];

    if (!block_shape_ok(n_desc > 0 ? descs[0].status : nullptr))
        return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    ReflTable &tab = tabs[warp];
    for (;;) {
        unsigned long long it = 0;
        if (lane == 0)
            it = atomicAdd(work_counter, 1ull);
        const long long item = (long long)__shfl_sync(kAll, it, 0);
        if (item >= total_items)
            break;
        const int si = find_sample(descs, n_desc, item);
        const SampleDesc &D = descs[si];
        if (kField && (!D.field || (D.brick_sz != 0) != kBrick)) {
            // a field variant launched over a sample without its field (or
            // with the other layout): an error status, no reads
            if (lane == 0)
                atomicOr(D.status, 1 << kErrArgs);
            continue;
        }
        const long long local = item - D.work_begin;
        const long long k = local / D.tiles;
        const long long r = D.order ? (long long)__ldg(D.order + k) : k;
        const int t = (int)(local - k * D.tiles);
        __syncwarp();   // the previous item's reads of the table are done
        {
            const int4 *src = reinterpret_cast<const int4 *>(D.refl + r);
            int4 *dst = reinterpret_cast<int4 *>(&tab);
            for (int k = lane; k < (int)(sizeof(ReflTable) / 16); k += 32)
                dst[k] = __ldg(src + k);
        }
        __syncwarp();

        const Vol v{D.vol, D.dim[0], D.dim[1], D.dim[2], D.field, D.field_stride, D.brick_sy, D.brick_sz};
        float s = 0.0f, c = 0.0f;
        int bad = kOk;
        unsigned nsteps = 0;
        const int v0 = t * D.tile;
        const int v1 = min(D.n_vox, v0 + D.tile);
        // every lane runs the same number of iterations (the march is warp-synchronous)
        for (int vb = v0; vb < v1; vb += 32) {
            const int vi = vb + lane;
            const bool valid = vi < v1;
            const short4 cv = valid ? __ldg(D.coords + vi) : make_short4(0, 0, 0, 0);
#pragma unroll 1
            for (int leg = 0; leg < 2; leg++) {
                LegResult a;
                trace_leg<false, true, kField, kBrick>(tab.head[leg], tab.rule[leg], cv.x, cv.y, cv.z, valid, v,
                                       D.full_iteration, D.voxel, D.sq, D.sq_stride, D.qtab, seg + tid, a,
                                       D.voxelf);
                bad |= a.status;
                nsteps += valid ? (unsigned)a.len : 0u;
                // the incident leg's lengths wait in shared memory while the
                // diffracted leg marches; then (L_incident + L_diffracted) per
                // class, as cal_rate adds them
#pragma unroll
                for (int k = 0; k < 4; k++)
                    lsum[k][tid] = leg == 0 ? a.Lf[k] : lsum[k][tid] + a.Lf[k];
            }
            if (valid) {
                // cal_rate's exponent (AnACor/src/ray_tracing_basic.c:1573-1576), in FP32
                const float ex = D.muf[0] * lsum[0][tid] + D.muf[1] * lsum[1][tid] + D.muf[2] * lsum[2][tid] +
                                 D.muf[3] * lsum[3][tid];
                const float term = D.is_exp ? expf(-ex) : ex;
                float ns, e;
                two_sum(s, term, ns, e);
                s = ns;
                c += e;
            }
        }
        if (bad)
            atomicOr(D.status, 1 << bad);
        if (D.steps) {
            unsigned long long w = nsteps;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                w += __shfl_down_sync(kAll, w, o);
            if (lane == 0)
                atomicAdd(D.steps, w);
        }
        // warp TwoSum reduction, the item's partial, and the fixed-order
        // combination of the reflection's partials by the last item to arrive
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float so = __shfl_down_sync(kAll, s, o);
            const float co = __shfl_down_sync(kAll, c, o);
            float ns, e;
            two_sum(s, so, ns, e);
            s = ns;
            c = c + co + e;
        }
        int last = 0;
        if (lane == 0) {
            D.partial[r * D.tiles + t] = (double)s + (double)c;
            __threadfence();
            last = atomicAdd(D.arrive + r, 1u) == (unsigned)(D.tiles - 1);
        }
        if (__shfl_sync(kAll, last, 0)) {
            __threadfence();
            const volatile double *pp = D.partial + r * D.tiles;
            double acc = 0.0;
            for (int k = lane; k < D.tiles; k += 32)
                acc += pp[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_down_sync(kAll, acc, o);
            if (lane == 0) {
                D.out[r] = acc / (double)D.n_vox;
                D.arrive[r] = 0u;   // ready for the next launch
            }
        }
    }
}

// ---- iterative bisection (the reference's ib_test) ------------------------

// One boundary search of AnACor/src/bisection.c:150-238 on the ray
// c + m * q (q = the face rule's signed ratios, which are the ratios of the
// reference's increments(), bisection.c:21-148): halve [shortest, longest]
// down to the resolution 1.0; boundary 0: a label equal to cls moves longest
// in, boundary 1: it moves shortest out.  The point is floor(c + floor(mid) q).
// A position outside the volume (undefined in the reference) fails the ray.
//
// The probe points floor(c + fl(mid * q)) come from fixed point where that is
// exact: mid in 24.40 (truncated) times the rule's Q = llrint(q * 2^32) is a
// 128-bit product read as 56.72; its error is below 1.1e-6 for |q| < 2^16 and
// |mid q| < 2^14 (every point inside the volume), and the FP64 expression's
// own rounding below 1e-11, so a fraction more than 2^-18 from an integer has
// the reference's floor.  Nearer than that (or a rule without Q) the FP64
// expression is evaluated; the range tests sit on integers and are covered by
// the same margin.  The FP64 pipe, which binds this kernel, keeps only the
// bisection of [shortest, longest] itself.
__device__ __forceinline__ bool bisect_dev(double longest, double shortest, int cz, int cy, int cx,
                                           const FaceRule &R, const Vol &v, int boundary, int cls, int *p,
                                           double &mid)
{
    const double *q = R.q;
    const double c[3] = {(double)cz, (double)cy, (double)cx};
    const int ci[3] = {cz, cy, cx};
    const int dim[3] = {v.dz, v.dy, v.dx};
    constexpr unsigned long long kMargin = 1ull << 46;   // 2^-18 of the 64-bit fraction
    double diff = __dadd_rn(longest, -shortest);
    mid = __dmul_rn(__dadd_rn(longest, shortest), 0.5);
    while (diff > 1.0) {
        mid = __dmul_rn(__dadd_rn(longest, shortest), 0.5);
        const long long mfx = R.fast ? __double2ll_rz(__dmul_rn(mid, 1099511627776.0)) : 0ll;   // mid * 2^40
        int pp[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            bool exact = !R.fast;
            long long x = 0;
            if (!exact) {
                const long long hi = __mul64hi(mfx, R.Q[a]);
                const unsigned long long lo = (unsigned long long)mfx * (unsigned long long)R.Q[a];
                const unsigned long long frac = ((unsigned long long)(hi & 0xff) << 56) | (lo >> 8);
                exact = frac < kMargin || frac > ~kMargin;
                x = (long long)ci[a] + (hi >> 8);
            }
            if (exact) {
                const double xd = floor(__dadd_rn(c[a], __dmul_rn(mid, q[a])));
                if (!(xd >= 0.0 && xd < (double)dim[a]))
                    return false;
                x = (long long)xd;
            } else if (x < 0 || x >= dim[a]) {
                return false;
            }
            pp[a] = (int)x;
        }
        const int lab = __ldg(v.p + ((long long)pp[0] * v.dy + pp[1]) * v.dx + pp[2]);
        const bool hit = lab == cls;
        if (boundary == 0) {
            if (hit) longest = mid; else shortest = mid;
        } else {
            if (hit) shortest = mid; else longest = mid;
        }
        diff = __dadd_rn(longest, -shortest);
    }
    const double fm = floor(mid);
#pragma unroll
    for (int a = 0; a < 3; a++)
        p[a] = (int)floor(__dadd_rn(c[a], __dmul_rn(fm, q[a])));
    return true;
}

__device__ __forceinline__ double abs_sum3(const int *a, const int *b)
{
    return __dadd_rn(__dadd_rn(fabs((double)(a[0] - b[0])), fabs((double)(a[1] - b[1]))), fabs((double)(a[2] - b[2])));
}

// difference_length (bisection.c:260-270): z, then y, then x
__device__ __forceinline__ double seg_len(const int *s, const int *e, const double *vox)
{
    const double dz = __dmul_rn((double)(s[0] - e[0]), vox[0]);
    const double dy = __dmul_rn((double)(s[1] - e[1]), vox[1]);
    const double dx = __dmul_rn((double)(s[2] - e[2]), vox[2]);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dz, dz), __dmul_rn(dy, dy)), __dmul_rn(dx, dx)));
}

// iterative_bisection + cal_path_bisection (bisection.c:272-463) for one leg;
// returns a status.  L = [liquor, loop, crystal, bubble].
__device__ __noinline__ int ib_leg(const LegHead &h, const FaceRule *rules, int cz, int cy, int cx, const Vol &v,
                                   int num_cls, const double *vox, double *L)
{
    L[0] = L[1] = L[2] = L[3] = 0.0;
    const int face = exit_face(h, cz, cy, cx, v);
    if (face == 0)
        return kErrNoFace;
    const FaceRule &R = rules[face - 1];
    if (R.status)
        return R.status;
    double air_longest;
    switch (face) {
    case 4: air_longest = (double)cy; break;
    case 5: air_longest = (double)(v.dy - 1 - cy); break;
    case 6: air_longest = (double)cx; break;
    case 1: air_longest = (double)(v.dx - 1 - cx); break;
    case 2: air_longest = (double)cz; break;
    default: air_longest = (double)(v.dz - 1 - cz); break;
    }
    const int p0[3] = {cz, cy, cx};
    int air[3], cr[3], li[3], lo[3], bi[3], bo[3];
    double m_air, m_cr, m_li, m_lo, m_bi, m_bo;
    if (!bisect_dev(air_longest, 0.0, cz, cy, cx, R, v, 0, 0, air, m_air) ||
        !bisect_dev(m_air, 0.0, cz, cy, cx, R, v, 1, 3, cr, m_cr))
        return kErrArgs;
    int npts = 3;
    const int *pa = nullptr, *pb = nullptr, *pc = nullptr, *pd = nullptr;   // points 3..6
    do {
        if (!bisect_dev(m_air, m_cr, cz, cy, cx, R, v, 0, 2, li, m_li))
            return kErrArgs;
        if (__ddiv_rn(abs_sum3(li, air), 3.0) > 1.0) {
            if (!bisect_dev(m_air, m_li, cz, cy, cx, R, v, 1, 2, lo, m_lo))
                return kErrArgs;
            if (__ddiv_rn(abs_sum3(li, lo), 3.0) <= 2.0)
                break;
            pa = li;
            pb = lo;
            npts = 5;
        }
        if (num_cls > 3) {
            if (!bisect_dev(m_air, m_cr, cz, cy, cx, R, v, 0, 4, bi, m_bi))
                return kErrArgs;
            if (abs_sum3(bi, air) > 1.0) {
                if (!bisect_dev(m_air, m_bi, cz, cy, cx, R, v, 1, 4, bo, m_bo))
                    return kErrArgs;
                if (__ddiv_rn(abs_sum3(bi, bo), 3.0) <= 2.0)
                    break;
                if (npts == 3) {
                    pa = bi;
                    pb = bo;
                } else {
                    pc = bi;
                    pd = bo;
                }
                npts += 2;
            }
        }
    } while (false);
    const double total = seg_len(p0, air, vox);
    const double cr_l = seg_len(p0, cr, vox);
    double lo_l = 0.0, bu_l = 0.0;
    // the lengths are read from the path by its length (5 points: loop, 7: bubble)
    if (npts == 5)
        lo_l = seg_len(pa, pb, vox);
    else if (npts == 7)
        bu_l = seg_len(pc, pd, vox);
    L[0] = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(total, -lo_l), -bu_l), -cr_l), -0.0);
    L[1] = lo_l;
    L[2] = cr_l;
    L[3] = bu_l;
    return kOk;
}

// ib_single_gridding's value (AnACor/src/ray_tracing.c:427-481) for n voxels
// and one direction (leg 1 of `dir`): the diffracted leg's lengths by
// iterative bisection, then cal_rate's exponent with a zero incident leg,
// sum_m mu_m (0 + L_m) left to right.  vox_mu = voxel[3], mu[4].
__global__ void __launch_bounds__(kBlock) ib_direction_kernel(const ReflTable *__restrict__ dir, const int8_t *vol,
                                                              int dz, int dy, int dx, const short4 *coords, int n,
                                                              const double *vox_mu, int num_cls, double *out,
                                                              int *status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    const short4 cv = coords[k];
    const Vol v{vol, dz, dy, dx};
    double L[4];
    const int st = ib_leg(dir->head[1], dir->rule[1], cv.x, cv.y, cv.z, v, num_cls, vox_mu, L);
    status[k] = st;
    if (st) {
        out[k] = 0.0;
        return;
    }
    const double *mu = vox_mu + 3;
    double a = __dmul_rn(mu[0], __dadd_rn(0.0, L[0]));
    a = __dadd_rn(a, __dmul_rn(mu[1], __dadd_rn(0.0, L[1])));
    a = __dadd_rn(a, __dmul_rn(mu[2], __dadd_rn(0.0, L[2])));
    a = __dadd_rn(a, __dmul_rn(mu[3], __dadd_rn(0.0, L[3])));
    out[k] = a;
}

// ib_test over every work item: as absorption_kernel, with bisection paths.
__global__ void __launch_bounds__(kBlock, 2) bisection_kernel(const SampleDesc *__restrict__ descs, int n_desc,
                                                              long long total_items,
                                                              unsigned long long *__restrict__ work_counter,
                                                              int num_cls)
{
    __shared__ ReflTable tab;
    __shared__ float red_s[kWarps], red_c[kWarps];
    __shared__ long long item_s;
    __shared__ int last_s;
    if (!block_shape_ok(n_desc > 0 ? descs[0].status : nullptr))
        return;
    const int tid = threadIdx.x;
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
        const long long k = local / D.tiles;
        const long long r = D.order ? (long long)__ldg(D.order + k) : k;
        const int t = (int)(local - k * D.tiles);
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
        const int v1 = min(D.n_vox, (t + 1) * D.tile);
        for (int vi = t * D.tile + tid; vi < v1; vi += kBlock) {
            const short4 cv = __ldg(D.coords + vi);
            double a[4], b[4];
            int st = ib_leg(tab.head[0], tab.rule[0], cv.x, cv.y, cv.z, v, num_cls, D.voxel, a);
            if (!st)
                st = ib_leg(tab.head[1], tab.rule[1], cv.x, cv.y, cv.z, v, num_cls, D.voxel, b);
            if (st) {
                bad |= st;
                continue;
            }
            // cal_rate, operand order of AnACor/src/ray_tracing_basic.c:1573-1576
            const double t0 = __dmul_rn(D.mu[0], __dadd_rn(a[0], b[0]));
            const double t1 = __dmul_rn(D.mu[1], __dadd_rn(a[1], b[1]));
            const double t2 = __dmul_rn(D.mu[2], __dadd_rn(a[2], b[2]));
            const double t3 = __dmul_rn(D.mu[3], __dadd_rn(a[3], b[3]));
            const double ex = __dadd_rn(__dadd_rn(__dadd_rn(t0, t1), t2), t3);
            float ns, e;
            two_sum(s, exp_neg(ex), ns, e);
            s = ns;
            c += e;
        }
        if (bad)
            atomicOr(D.status, 1 << bad);
        finish_item(s, c, D, r, t, red_s, red_c, last_s);
    }
}

// Absorption map: work item = (grid direction, tile of voxels); the
// diffracted leg of every voxel, one output per (direction, voxel).
template <bool kField>
__global__ void __launch_bounds__(kBlock, 2) gridding_map_kernel(const MapDesc *__restrict__ dp, long long total_items,
                                                                 unsigned long long *__restrict__ work_counter)
{
    __shared__ ReflTable tab;
    __shared__ uint16_t seg[kMaxSegments * kBlock];
    __shared__ long long item_s;
    const MapDesc &D = *dp;
    if (!block_shape_ok(D.status))
        return;
    const int tid = threadIdx.x;
    const Vol v{D.vol, D.dim[0], D.dim[1], D.dim[2], D.field, D.field_stride};
    for (;;) {
        if (tid == 0)
            item_s = (long long)atomicAdd(work_counter, 1ull);
        __syncthreads();
        const long long item = item_s;
        if (item >= total_items)
            break;
        const long long d = item / D.tiles;
        const int t = (int)(item - d * D.tiles);
        {
            const int4 *src = reinterpret_cast<const int4 *>(D.dirs + d);
            int4 *dst = reinterpret_cast<int4 *>(&tab);
            for (int k = tid; k < (int)(sizeof(ReflTable) / 16); k += kBlock)
                dst[k] = __ldg(src + k);
        }
        __syncthreads();
        int bad = kOk;
        const int v0 = t * D.tile;
        const int v1 = min(D.n_vox, v0 + D.tile);
        float *row = D.out + d * D.ld;
        for (int vb = v0; vb < v1; vb += kBlock) {
            const int vi = vb + tid;
            const bool valid = vi < v1;
            const short4 cv = valid ? __ldg(D.coords + vi) : make_short4(0, 0, 0, 0);
            LegResult a;
            trace_leg<false, false, kField>(tab.head[1], tab.rule[1], cv.x, cv.y, cv.z, valid, v, D.full_iteration,
                                            D.voxel, D.sq, D.sq_stride, D.qtab, seg + tid, a);
            if (!valid)
                continue;
            double val;
            if (a.status) {
                bad |= a.status;
                val = __longlong_as_double(0x7ff8000000000000ll);
            } else {
                // cal_rate with a zero incident leg: (0 + L) == L per class
                const double t0 = __dmul_rn(D.mu[0], a.L[0]);
                const double t1 = __dmul_rn(D.mu[1], a.L[1]);
                const double t2 = __dmul_rn(D.mu[2], a.L[2]);
                const double t3 = __dmul_rn(D.mu[3], a.L[3]);
                const double ex = __dadd_rn(__dadd_rn(__dadd_rn(t0, t1), t2), t3);
                val = D.is_exp ? exp(-ex) : ex;
            }
            const long long o = D.col ? __ldg(D.col + vi) : vi;
            if (D.out64)
                D.out64[d * D.ld + o] = val;
            else
                row[o] = (float)val;
        }
        if (bad)
            atomicOr(D.status, 1 << bad);
        __syncthreads();   // the table and item_s are rewritten next
    }
}

// Per-voxel, per-leg detail for one reflection (path-level parity checks);
// same march code as the absorption kernel.
__global__ void __launch_bounds__(kBlock) leg_detail_kernel(const ReflTable *__restrict__ tabp, const int8_t *vol,
                                                            int dz, int dy, int dx, const short4 *coords, int n,
                                                            const double *voxel3, int full, const double *sq,
                                                            int sq_stride, const double *qtab, int *face, int *len,
                                                            int *nseg, int *first, int *last, double *L,
                                                            int *status)
{
    __shared__ ReflTable tab;
    __shared__ uint16_t seg[kMaxSegments * kBlock];
    __shared__ double vox[3];
    if (!block_shape_ok(status))
        return;
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
    const bool valid = vi < n;
    const Vol v{vol, dz, dy, dx};
    const short4 cv = valid ? coords[vi] : make_short4(0, 0, 0, 0);
#pragma unroll 1
    for (int leg = 0; leg < 2; leg++) {
        LegResult a;
        trace_leg<true>(tab.head[leg], tab.rule[leg], cv.x, cv.y, cv.z, valid, v, full, vox, sq, sq_stride, qtab,
                        seg + threadIdx.x, a);
        if (!valid)
            continue;
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

// Quotient table: row d (1 <= d <= max_den) holds fl(s / d) for s = 1 .. d+1,
// rows packed one after another (row d starts at (d-1)(d+2)/2).
__global__ void quotient_table_kernel(double *__restrict__ q, int max_den)
{
    const long long total = (long long)max_den * (max_den + 3) / 2;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        // row d: the largest d with (d-1)(d+2)/2 <= k
        int d = (int)floor((sqrt(8.0 * (double)k + 9.0) - 1.0) / 2.0);
        if (d < 1)
            d = 1;
        while (d > 1 && (long long)(d - 1) * (d + 2) / 2 > k)
            d--;
        while ((long long)d * (d + 3) / 2 <= k)
            d++;
        const int s = (int)(k - (long long)(d - 1) * (d + 2) / 2) + 1;
        q[k] = __ddiv_rn((double)s, (double)d);
    }
}

}  // namespace

int rcp_table_init()
{
    static double2 host[kMaxDim + 2];
    host[0] = make_double2(0.0, 0.0);
    for (int d = 1; d < kMaxDim + 2; d++)
        host[d] = make_double2((double)d, 1.0 / (double)d);
    return cudaMemcpyToSymbol(g_num_rcp, host, sizeof(host)) == cudaSuccess ? kOk : kErrCuda;
}

size_t quotient_table_entries(int max_den)
{
    return max_den > 0 ? (size_t)max_den * (size_t)(max_den + 3) / 2 : 0;
}

cudaError_t launch_quotient_table(double *d_q, int max_den, cudaStream_t st)
{
    if (max_den <= 0)
        return cudaSuccess;
    quotient_table_kernel<<<1024, 256, 0, st>>>(d_q, max_den);
    return cudaGetLastError();
}

cudaError_t launch_pack_coords(const long long *d_c, int n, const int *dims, short4 *d_out, int *d_status,
                               cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    pack_coords_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_c, n, dims[0], dims[1], dims[2], d_out, d_status);
    return cudaGetLastError();
}

int absorption_variant()
{
    static const int v = [] {
        const char *e = std::getenv("ANACOR_CTAS_PER_SM");
        const int x = e ? std::atoi(e) : kDefaultMinBlocks;
        return (x >= 1 && x <= 4) ? x : kDefaultMinBlocks;
    }();
    return v;
}

cudaError_t launch_absorption(const SampleDesc *d_descs, int n_desc, long long total_items,
                              unsigned long long *d_counter, int grid, cudaStream_t st, int variant)
{
    if (total_items <= 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess)
        return e;
#define ANACOR_LAUNCH(B, F, K) \
    absorption_kernel<B, F, K><<<grid, kBlock, 0, st>>>(d_descs, n_desc, total_items, d_counter)
    switch (variant > 0 ? variant : absorption_variant()) {
    case 1: ANACOR_LAUNCH(1, false, false); break;
    case 3: ANACOR_LAUNCH(3, false, false); break;
    case 4: ANACOR_LAUNCH(4, false, false); break;
    case 5: ANACOR_LAUNCH(1, true, false); break;
    case 6: ANACOR_LAUNCH(2, true, false); break;
    case 7: ANACOR_LAUNCH(3, true, false); break;
    case 8: ANACOR_LAUNCH(4, true, false); break;
    case 9: ANACOR_LAUNCH(1, true, true); break;
    case 10: ANACOR_LAUNCH(2, true, true); break;
    case 11: ANACOR_LAUNCH(3, true, true); break;
    case 12: ANACOR_LAUNCH(4, true, true); break;
    default: ANACOR_LAUNCH(2, false, false); break;
    }
#undef ANACOR_LAUNCH
    return cudaGetLastError();
}

cudaError_t launch_leg_detail(const ReflTable *d_tab, const int8_t *d_vol, const int *dims, const short4 *d_coords,
                              int n, const double *d_voxel, int full, const double *d_sq, int sq_stride,
                              const double *d_qtab, int *face, int *len, int *nseg, int *first, int *last, double *L,
                              int *status, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    leg_detail_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(d_tab, d_vol, dims[0], dims[1], dims[2],
                                                                    d_coords, n, d_voxel, full, d_sq, sq_stride,
                                                                    d_qtab, face, len, nseg, first, last, L, status);
    return cudaGetLastError();
}

cudaError_t launch_bisection(const SampleDesc *d_descs, int n_desc, long long total_items,
                             unsigned long long *d_counter, int grid, int num_cls, cudaStream_t st)
{
    if (total_items <= 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess)
        return e;
    bisection_kernel<<<grid, kBlock, 0, st>>>(d_descs, n_desc, total_items, d_counter, num_cls);
    return cudaGetLastError();
}

cudaError_t launch_ib_direction(const ReflTable *d_dir, const int8_t *d_vol, const int *dims, const short4 *d_coords,
                                int n, const double *d_vox_mu, int num_cls, double *d_out, int *d_status,
                                cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    ib_direction_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(d_dir, d_vol, dims[0], dims[1], dims[2],
                                                                      d_coords, n, d_vox_mu, num_cls, d_out,
                                                                      d_status);
    return cudaGetLastError();
}

int bisection_occupancy(int *blocks_per_sm)
{
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, bisection_kernel, kBlock, 0) == cudaSuccess
               ? kOk
               : kErrCuda;
}

cudaError_t launch_gridding_map(const MapDesc *d_desc, long long total_items, unsigned long long *d_counter, int grid,
                                cudaStream_t st, bool field)
{
    if (total_items <= 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess)
        return e;
    if (field)
        gridding_map_kernel<true><<<grid, kBlock, 0, st>>>(d_desc, total_items, d_counter);
    else
        gridding_map_kernel<false><<<grid, kBlock, 0, st>>>(d_desc, total_items, d_counter);
    return cudaGetLastError();
}

int gridding_map_occupancy(int *blocks_per_sm, bool field)
{
    const cudaError_t e = field ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gridding_map_kernel<true>,
                                                                                kBlock, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gridding_map_kernel<false>,
                                                                                kBlock, 0);
    return e == cudaSuccess ? kOk : kErrCuda;
}

int absorption_block_threads() { return kBlock; }

int block_guard_selftest(int threads, int *status_out)
{
    // Launch the absorption kernel over no work with `threads` threads per
    // block, fewer than kBlock (a whole number of warps), and report the
    // status word it leaves.  The guard must refuse the launch before any
    // access; threads == kBlock must pass it and find no work.
    if (threads <= 0 || threads > kBlock || threads % 32 != 0 || !status_out)
        return kErrArgs;
    SampleDesc h{};
    SampleDesc *d = nullptr;
    unsigned long long *counter = nullptr;
    int *status = nullptr;
    if (cudaMalloc(&d, sizeof(SampleDesc)) != cudaSuccess)
        return kErrCuda;
    int rc = kErrCuda;
    if (cudaMalloc(&counter, sizeof(unsigned long long)) == cudaSuccess &&
        cudaMalloc(&status, sizeof(int)) == cudaSuccess && cudaMemset(status, 0, sizeof(int)) == cudaSuccess &&
        cudaMemset(counter, 0, sizeof(unsigned long long)) == cudaSuccess) {
        h.status = status;
        if (cudaMemcpy(d, &h, sizeof(h), cudaMemcpyHostToDevice) == cudaSuccess) {
            absorption_kernel<2, false><<<2, threads>>>(d, 1, 0, counter);
            if (cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
                cudaMemcpy(status_out, status, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess)
                rc = kOk;
        }
    }
    cudaFree(status);
    cudaFree(counter);
    cudaFree(d);
    return rc;
}

// Preferred shared-memory carveout (percent of the unified L1/shared storage)
// of every absorption kernel; a hint to the driver.
int absorption_set_carveout(int pct)
{
    cudaError_t e = cudaSuccess;
#define ANACOR_CARVE(B, F) \
    if (e == cudaSuccess) \
        e = cudaFuncSetAttribute(absorption_kernel<B, F>, cudaFuncAttributePreferredSharedMemoryCarveout, pct)
    ANACOR_CARVE(1, false); ANACOR_CARVE(2, false); ANACOR_CARVE(3, false); ANACOR_CARVE(4, false);
    ANACOR_CARVE(1, true); ANACOR_CARVE(2, true); ANACOR_CARVE(3, true); ANACOR_CARVE(4, true);
#undef ANACOR_CARVE
    return e == cudaSuccess ? kOk : kErrCuda;
}

int absorption_occupancy(int *blocks_per_sm, int variant)
{
    cudaError_t e;
#define ANACOR_OCC(B, F, K) \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, absorption_kernel<B, F, K>, kBlock, 0)
    switch (variant > 0 ? variant : absorption_variant()) {
    case 1: e = ANACOR_OCC(1, false, false); break;
    case 3: e = ANACOR_OCC(3, false, false); break;
    case 4: e = ANACOR_OCC(4, false, false); break;
    case 5: e = ANACOR_OCC(1, true, false); break;
    case 6: e = ANACOR_OCC(2, true, false); break;
    case 7: e = ANACOR_OCC(3, true, false); break;
    case 8: e = ANACOR_OCC(4, true, false); break;
    case 9: e = ANACOR_OCC(1, true, true); break;
    case 10: e = ANACOR_OCC(2, true, true); break;
    case 11: e = ANACOR_OCC(3, true, true); break;
    case 12: e = ANACOR_OCC(4, true, true); break;
    default: e = ANACOR_OCC(2, false, false); break;
    }
#undef ANACOR_OCC
    return e == cudaSuccess ? kOk : kErrCuda;
}

}  // namespace anacor
