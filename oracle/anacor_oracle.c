/*
 * anacor_oracle.c -- CPU restatement of AnACor's analytical absorption path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to obtain the
 * answers the GPU library must reproduce.  The product library never links,
 * loads or calls it.
 *
 * It restates, in plain C99, the per-reflection algorithm of the reference's
 * C/OpenMP library (paths relative to the AnACor project):
 *
 *   ray_tracing_overall   AnACor/src/ray_tracing.c:365-425
 *   ray_tracing_single    AnACor/src/ray_tracing.c:166-292
 *   kp_rotation / dot_product / transpose   AnACor/src/matrices.h:49-68,14-29,6-12
 *   dials_2_thetaphi_22   AnACor/src/ray_tracing_basic.c:13-50
 *   dials_2_myframe       AnACor/src/ray_tracing_basic.c:52-67
 *   cube_face             AnACor/src/ray_tracing_basic.c:69-186
 *   cal_coord + appending AnACor/src/ray_tracing_basic.c:396-1460, 343-394
 *   cal_path2_plus        AnACor/src/ray_tracing_basic.c:1462-1552
 *   cal_rate              AnACor/src/ray_tracing_basic.c:1554-1583
 *
 * Every floating-point expression keeps the reference's operand order and
 * rounding points.  Build with -ffp-contract=off (the reference's x86-64
 * build, which has no -march, never contracts into FMA; on aarch64 GCC would
 * contract by default, so the flag keeps both machines on the same
 * arithmetic).  Parity is pinned against the reference library compiled from
 * its own sources (see oracle/Makefile, target `ref`).
 *
 * Differences from the reference that do not change any result:
 *  - the six face-specific march loops of cal_coord are written once, driven
 *    by a per-face table of signed step ratios, a rounding mode and a step
 *    count (the table is derived line by line in face_rule());
 *  - the visited-voxel path is not stored: only its first and last points
 *    (the two cal_path2_plus reads) and the class-change list are kept, in
 *    per-thread buffers allocated once instead of malloc/realloc per ray;
 *  - where the reference aborts (assert in cal_coord, exit in cube_face) the
 *    oracle returns an error status instead.
 * Double-to-int64 conversion of out-of-range or NaN values follows x86-64
 * (cvttsd2si yields INT64_MIN); the reference leaves it undefined.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

enum {
    ORC_OK = 0,
    ORC_ERR_FACE = 1,     /* cube_face found no exit plane (reference: exit()) */
    ORC_ERR_ASSERT = 2,   /* face / angle combination rejected by an assert   */
    ORC_ERR_ARGS = 3,
    ORC_ERR_NOMEM = 4,
};

/* ---------------------------------------------------------------- helpers */

static int64_t to_i64(double v)
{
    /* x86-64 cvttsd2si semantics for the conversions `int64_t new_x = floor(..)` */
    if (!(v >= -9223372036854775808.0 && v < 9223372036854775808.0))
        return INT64_MIN;
    return (int64_t)v;
}

/* Rodrigues matrix, AnACor/src/matrices.h:49-68 (same products, same order) */
static void rodrigues(const double *axis, double ang, double *m)
{
    double x = axis[0], y = axis[1], z = axis[2];
    double c = cos(ang), s = sin(ang);
    double k = 1 - c;
    m[0] = c + (x * x) * k;
    m[1] = x * y * k - z * s;
    m[2] = y * s + x * z * k;
    m[3] = z * s + x * y * k;
    m[4] = c + (y * y) * k;
    m[5] = -x * s + y * z * k;
    m[6] = -y * s + x * z * k;
    m[7] = x * s + y * z * k;
    m[8] = c + (z * z) * k;
}

/* C[m x p] = A[m x n] B[n x p], sum started at 0.0 (AnACor/src/matrices.h:14-29) */
static void matmul(const double *A, const double *B, double *C, int m, int n, int p)
{
    for (int i = 0; i < m; i++)
        for (int j = 0; j < p; j++) {
            double acc = 0.0;
            for (int k = 0; k < n; k++)
                acc += A[i * n + k] * B[k * p + j];
            C[i * p + j] = acc;
        }
}

/* rotated incident / diffracted vectors of one reflection
 * (AnACor/src/ray_tracing.c:397-407): T = (R(omega) F)^T; xray' = T xray, s1' = T s1 */
void oracle_rotate(const double *omega_axis, double omega, const double *F,
                   const double *xray, const double *s1, double *xray_out, double *s1_out)
{
    double r[9], rf[9], t[9];
    rodrigues(omega_axis, omega, r);
    matmul(r, F, rf, 3, 3, 3);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            t[j * 3 + i] = rf[i * 3 + j];
    matmul(t, xray, xray_out, 3, 3, 1);
    matmul(t, s1, s1_out, 3, 3, 1);
}

/* polar angles of a DIALS-frame vector (AnACor/src/ray_tracing_basic.c:13-50).
 * The incident leg negates the vector first. */
void oracle_theta_phi(const double *vin, int incident, double *theta, double *phi)
{
    double v0 = vin[0], v1 = vin[1], v2 = vin[2];
    if (incident) {
        v0 = -v0; v1 = -v1; v2 = -v2;
    }
    double rxy = sqrt(v0 * v0 + v1 * v1);
    if (v1 == 0) {
        *theta = atan(-v2 / (-rxy + 0.001));
        *phi = atan(-v0 / (v1 + 0.001));
    } else if (v1 < 0) {
        *theta = atan(-v2 / rxy);
        *phi = atan(-v0 / v1);
    } else {
        if (v2 < 0)
            *theta = ORC_PI - atan(-v2 / rxy);
        else
            *theta = -ORC_PI - atan(-v2 / rxy);
        *phi = -atan(-v0 / (-v1));
    }
}

/* (x, y, z) -> (x, z, y) accumulated from 0.0 like the reference's 3x3
 * permutation product (AnACor/src/ray_tracing_basic.c:52-67); this turns
 * -0.0 components into +0.0 exactly as the reference does. */
void oracle_myframe(const double *v, double *out)
{
    static const double P[3][3] = {{1, 0, 0}, {0, 0, 1}, {0, 1, 0}};
    for (int i = 0; i < 3; i++) {
        double acc = 0.0;
        for (int j = 0; j < 3; j++)
            acc += P[i][j] * v[j];
        out[i] = acc;
    }
}

/* exit face of the ray from voxel `o` (z,y,x) along `d` (my-frame z,y,x
 * components), AnACor/src/ray_tracing_basic.c:69-186.  Face codes:
 * 1 x_max, 2 z_min, 3 z_max, 4 y_min, 5 y_max, 6 x_min.  Returns 0 when no
 * plane has t >= 0 (the reference exits the process there). */
int64_t oracle_cube_face(const int64_t *o, const double *d, const int64_t *shape, int incident)
{
    double t[6];
    t[0] = (double)(0 - o[2]) / d[2];          /* x_min */
    t[3] = (double)(shape[2] - o[2]) / d[2];   /* x_max */
    t[1] = (double)(0 - o[1]) / d[1];          /* y_min */
    t[4] = (double)(shape[1] - o[1]) / d[1];   /* y_max */
    t[2] = (double)(0 - o[0]) / d[0];          /* z_min */
    t[5] = (double)(shape[0] - o[0]) / d[0];   /* z_max */
    if (incident)
        for (int k = 0; k < 6; k++)
            t[k] = -t[k];
    int have = 0;
    double best = 0;
    for (int k = 0; k < 6; k++) {
        if (t[k] >= 0) {
            if (!have || t[k] < best)
                best = t[k];
            have = 1;
        }
    }
    if (!have)
        return 0;
    /* first match in the reference's test order */
    static const int order[6] = {0, 3, 1, 4, 2, 5};
    static const int64_t face_code[6] = {6, 4, 2, 1, 5, 3};
    for (int k = 0; k < 6; k++)
        if (best == t[order[k]])
            return face_code[order[k]];
    return 0;
}

/* ------------------------------------------------------ march description */

/* One face's march: position on axis a at increment i is
 *   R(c_a + fl(i * q[a]))     R = floor or C round (half away from zero),
 * clamped to [0, dim_a - 1], for i = 0 .. count-1.  q is (z, y, x). */
typedef struct {
    double q[3];
    int use_round;
    int vac_limit;   /* consecutive-vacuum limit under full_iteration */
} orc_rule;

/* Derivation of the per-face table from cal_coord
 * (AnACor/src/ray_tracing_basic.c line numbers):
 *  face 6 (:418-509)  |th|<=pi/2; x += -1, y -= tan th/cos ph, z += tan ph;
 *                     floor if th>0 else round; i = 0..x
 *  face 2 (:512-709)  |th|<pi/2 (ph<0): x -= 1/tan|ph|, y -= tan th/sin|ph|
 *                     else (ph>0):      x += 1/tan|ph|, y -= tan(pi-th)/sin|ph|
 *                     z -= 1; floor if th>0 else round; i = 0..z
 *  face 3 (:712-896)  |th|<pi/2 (ph>0): x -= 1/tan|ph|, y -= tan th/sin|ph|, i < zmax-z
 *                     else (ph<0):      x += 1/tan|ph|, y -= tan(pi-th)/sin|ph|, i <= zmax-z
 *                     z += 1; floor if th>0 else round
 *  face 4 (:899-1101) th>0; |th|<pi/2: x -= cos|ph|/tan|th|, z += sin ph/tan|th|
 *                     else: x += cos|ph|/tan(pi-|th|), z += sin(-ph)/tan(pi-|th|)
 *                     y -= 1; always floor; i = 0..y
 *  face 5 (:1104-1277) th<0; |th|<pi/2: x -= cos|ph|/tan|th|, z += sin ph/tan|th|, i < ymax-y
 *                     else: x += cos|ph|/tan(pi-|th|), z -= sin ph/tan(pi-|th|), i <= ymax-y
 *                     y += 1; always round
 *  face 1 (:1280-1372) |th|>=pi/2; x += 1, y -= tan(pi-th)/cos|ph|, z -= tan ph;
 *                     floor if th>0 else round; i < xmax-x; vacuum limit 10 (else 50)
 * "c - fl(i*r)" is the same IEEE operation as "c + fl(i*(-r))", so every
 * sign is folded into q.  Returns ORC_ERR_ASSERT where the reference's
 * assert would fire. */
static int face_rule(int64_t face, double th, double ph, orc_rule *r)
{
    const double half = ORC_PI / 2;
    int flr = th > 0;
    r->vac_limit = 50;
    switch (face) {
    case 6:
        if (!(fabs(th) <= half)) return ORC_ERR_ASSERT;
        r->q[2] = -1;
        r->q[1] = -(tan(th) / cos(ph));
        r->q[0] = tan(ph);
        r->use_round = !flr;
        return ORC_OK;
    case 2:
        if (fabs(th) < half) {
            if (!(ph < 0)) return ORC_ERR_ASSERT;
            r->q[2] = -(1 / tan(fabs(ph)));
            r->q[1] = -(tan(th) / sin(fabs(ph)));
        } else {
            if (!(ph > 0)) return ORC_ERR_ASSERT;
            r->q[2] = 1 / tan(fabs(ph));
            r->q[1] = -(tan(ORC_PI - th) / sin(fabs(ph)));
        }
        r->q[0] = -1;
        r->use_round = !flr;
        return ORC_OK;
    case 3:
        if (fabs(th) < half) {
            if (!(ph > 0)) return ORC_ERR_ASSERT;
            r->q[2] = -(1 / tan(fabs(ph)));
            r->q[1] = -(tan(th) / sin(fabs(ph)));
        } else {
            if (!(ph < 0)) return ORC_ERR_ASSERT;
            r->q[2] = 1 / (tan(fabs(ph)));
            r->q[1] = -(tan(ORC_PI - th) / sin(fabs(ph)));
        }
        r->q[0] = 1;
        r->use_round = !flr;
        return ORC_OK;
    case 4:
        if (!(th > 0)) return ORC_ERR_ASSERT;
        if (fabs(th) < half) {
            r->q[2] = -(cos(fabs(ph)) / tan(fabs(th)));
            r->q[0] = sin(ph) / tan(fabs(th));
        } else {
            r->q[2] = cos(fabs(ph)) / (tan((ORC_PI - fabs(th))));
            r->q[0] = sin(-ph) / (tan((ORC_PI - fabs(th))));
        }
        r->q[1] = -1;
        r->use_round = 0;
        return ORC_OK;
    case 5:
        if (!(th < 0)) return ORC_ERR_ASSERT;
        if (fabs(th) < half) {
            r->q[2] = -(cos(fabs(ph)) / (tan(fabs(th))));
            r->q[0] = sin(ph) / (tan(fabs(th)));
        } else {
            r->q[2] = cos(fabs(ph)) / (tan(ORC_PI - fabs(th)));
            r->q[0] = -(sin(ph) / (tan(ORC_PI - fabs(th))));
        }
        r->q[1] = 1;
        r->use_round = 1;
        return ORC_OK;
    case 1:
        if (!(fabs(th) >= half)) return ORC_ERR_ASSERT;
        r->q[2] = 1;
        r->q[1] = -(tan(ORC_PI - th) / cos(fabs(ph)));
        r->q[0] = -(tan(ph));
        r->use_round = !flr;
        r->vac_limit = 10;
        return ORC_OK;
    default:
        return ORC_ERR_FACE;
    }
}

/* number of increments the face's loop runs (see face_rule) */
static int64_t face_steps(int64_t face, double th, const int64_t *c, const int64_t *shape)
{
    const double half = ORC_PI / 2;
    switch (face) {
    case 6: return c[2] + 1;
    case 2: return c[0] + 1;
    case 3: return fabs(th) < half ? shape[0] - c[0] : shape[0] - c[0] + 1;
    case 4: return c[1] + 1;
    case 5: return fabs(th) < half ? shape[1] - c[1] : shape[1] - c[1] + 1;
    case 1: return shape[2] - c[2];
    default: return 0;
    }
}

static inline int64_t step_axis(int64_t c, int64_t i, double q, int use_round, int64_t dim)
{
    double v = (double)c + (double)i * q;
    int64_t n = to_i64(use_round ? round(v) : floor(v));
    if (n >= dim)
        n = dim - 1;
    else if (n < 0)
        n = 0;
    return n;
}

/* result of one leg (one cal_coord + cal_path2_plus) */
typedef struct {
    int64_t face;
    int64_t len;       /* len_path_2 */
    int64_t nseg;      /* len_classes_posi */
    int64_t first[3];
    int64_t last[3];
    double L[4];       /* [liquor, loop, crystal, bubble] */
} orc_leg;

/* march one leg: cal_coord (AnACor/src/ray_tracing_basic.c:396-1460) followed
 * by cal_path2_plus (:1462-1552).  `seg_cls` / `seg_pos` need room for
 * max(shape)+2 entries. */
static int march_leg(const int64_t *c, const double *dir, double th, double ph, int incident,
                     const int8_t *vol, const int64_t *shape, int full_iteration,
                     const double *voxel, int64_t *seg_cls, int64_t *seg_pos, orc_leg *out)
{
    int64_t face = oracle_cube_face(c, dir, shape, incident);
    out->face = face;
    if (face == 0)
        return ORC_ERR_FACE;
    orc_rule r;
    int st = face_rule(face, th, ph, &r);
    if (st)
        return st;
    int64_t count = face_steps(face, th, c, shape);
    const int64_t sy = shape[2], sz = shape[1] * shape[2];

    int64_t len = 1, nseg = 1, vac = 0;
    int64_t prev_label = 0;
    int64_t pz = 0, py = 0, px = 0;
    seg_cls[0] = 3;   /* the start voxel always opens a crystal segment */
    seg_pos[0] = 0;
    out->first[0] = out->first[1] = out->first[2] = 0;
    for (int64_t i = 0; i < count; i++) {
        int64_t nz = step_axis(c[0], i, r.q[0], r.use_round, shape[0]);
        int64_t ny = step_axis(c[1], i, r.q[1], r.use_round, shape[1]);
        int64_t nx = step_axis(c[2], i, r.q[2], r.use_round, shape[2]);
        int64_t label = vol[nz * sz + ny * sy + nx];
        if (!full_iteration) {
            if (label == 0)
                break;
        } else {
            vac = label == 0 ? vac + 1 : 0;
            if (vac > r.vac_limit)
                break;
        }
        if (i == 0) {
            out->first[0] = nz; out->first[1] = ny; out->first[2] = nx;
        } else {
            if (label != prev_label && label >= 0 && label <= 4) {
                seg_cls[nseg] = label;
                seg_pos[nseg] = i;
                nseg++;
            }
            len++;
        }
        pz = nz; py = ny; px = nx;
        prev_label = label;
    }
    out->len = len;
    out->nseg = nseg;
    if (len == 1) {
        /* the reference reads an unwritten first point here but returns zeros */
        out->last[0] = out->first[0]; out->last[1] = out->first[1]; out->last[2] = out->first[2];
        out->L[0] = out->L[1] = out->L[2] = out->L[3] = 0.0;
        return ORC_OK;
    }
    out->last[0] = pz; out->last[1] = py; out->last[2] = px;
    /* cal_path2_plus: total from first/last point, y then z then x */
    double dy = (double)(py - out->first[1]) * voxel[1];
    double dz = (double)(pz - out->first[0]) * voxel[0];
    double dx = (double)(px - out->first[2]) * voxel[2];
    double total = sqrt(dy * dy + dz * dz + dx * dx);
    double acc[5] = {0, 0, 0, 0, 0};   /* indexed by class code 0..4 */
    double den = (double)(len - 1);
    for (int64_t j = 0; j < nseg; j++) {
        int64_t span = (j < nseg - 1) ? seg_pos[j + 1] - seg_pos[j] : len - seg_pos[j];
        int64_t k = seg_cls[j];
        if (k >= 1 && k <= 4)
            acc[k] += total * ((double)span / den);
    }
    out->L[0] = acc[1];
    out->L[1] = acc[2];
    out->L[2] = acc[3];
    out->L[3] = acc[4];
    return ORC_OK;
}

/* cal_rate (AnACor/src/ray_tracing_basic.c:1554-1583) */
static double rate(const double *a, const double *b, const double *mu, int is_exp)
{
    double s = (mu[0] * (a[0] + b[0]) +
                mu[1] * (a[1] + b[1]) +
                mu[2] * (a[2] + b[2]) +
                mu[3] * (a[3] + b[3]));
    if (is_exp == 1)
        s = exp(-s);
    return s;
}

/* per-reflection angle set */
typedef struct {
    double th_in, ph_in, th_out, ph_out;
    double d_in[3], d_out[3];
} orc_dirs;

static void reflection_dirs(const double *s1_rot, const double *xray_rot, orc_dirs *d)
{
    oracle_theta_phi(s1_rot, 0, &d->th_out, &d->ph_out);
    oracle_theta_phi(xray_rot, 1, &d->th_in, &d->ph_in);
    oracle_myframe(xray_rot, d->d_in);
    oracle_myframe(s1_rot, d->d_out);
}

static int64_t max_dim(const int64_t *shape)
{
    int64_t m = shape[0];
    if (shape[1] > m) m = shape[1];
    if (shape[2] > m) m = shape[2];
    return m;
}

/* ray_tracing_single (AnACor/src/ray_tracing.c:166-292) with caller scratch */
static int single(const int64_t *coords, int64_t n, const double *s1_rot, const double *xray_rot,
                  const double *voxel, const double *mu, const int8_t *vol, const int64_t *shape,
                  int full_iteration, int is_exp, int64_t *scratch, double *out)
{
    orc_dirs d;
    reflection_dirs(s1_rot, xray_rot, &d);
    int64_t cap = max_dim(shape) + 2;
    int64_t *cls = scratch, *pos = scratch + cap;
    double sum = 0;
    for (int64_t k = 0; k < n; k++) {
        const int64_t *c = coords + 3 * k;
        orc_leg l1, l2;
        int st = march_leg(c, d.d_in, d.th_in, d.ph_in, 1, vol, shape, full_iteration, voxel, cls, pos, &l1);
        if (st) return st;
        st = march_leg(c, d.d_out, d.th_out, d.ph_out, 0, vol, shape, full_iteration, voxel, cls, pos, &l2);
        if (st) return st;
        sum += rate(l1.L, l2.L, mu, is_exp);
    }
    *out = sum / n;
    return ORC_OK;
}

static int check_coords(const int64_t *coords, int64_t n, const int64_t *shape)
{
    for (int64_t k = 0; k < n; k++)
        for (int a = 0; a < 3; a++)
            if (coords[3 * k + a] < 0 || coords[3 * k + a] >= shape[a])
                return ORC_ERR_ARGS;
    return ORC_OK;
}

/* --------------------------------------------------------------- exports */

int oracle_single(const int64_t *coords, int64_t n, const double *s1_rot, const double *xray_rot,
                  const double *voxel, const double *mu, const int8_t *vol, const int64_t *shape,
                  int full_iteration, int is_exp, double *out)
{
    if (n <= 0 || check_coords(coords, n, shape))
        return ORC_ERR_ARGS;
    int64_t *scratch = malloc(sizeof(int64_t) * 2 * (max_dim(shape) + 2));
    if (!scratch)
        return ORC_ERR_NOMEM;
    int st = single(coords, n, s1_rot, xray_rot, voxel, mu, vol, shape, full_iteration, is_exp, scratch, out);
    free(scratch);
    return st;
}

/* ray_tracing_overall (AnACor/src/ray_tracing.c:365-425): one OpenMP
 * iteration per reflection, `threads` workers (<=0: runtime default). */
int oracle_overall(const int64_t *coords, int64_t n, const double *s1, const double *omega,
                   const double *xray, const double *omega_axis, const double *F, int64_t n_refl,
                   const double *voxel, const double *mu, const int8_t *vol, const int64_t *shape,
                   int full_iteration, int is_exp, int threads, double *out)
{
    if (n <= 0 || n_refl < 0 || check_coords(coords, n, shape))
        return ORC_ERR_ARGS;
    int status = ORC_OK;
    int64_t cap = max_dim(shape) + 2;
#ifdef _OPENMP
    if (threads > 0)
        omp_set_num_threads(threads);
#else
    (void)threads;
#endif
#pragma omp parallel
    {
        int64_t *scratch = malloc(sizeof(int64_t) * 2 * cap);
        if (!scratch) {
#pragma omp atomic write
            status = ORC_ERR_NOMEM;
        }
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n_refl; i++) {
            if (!scratch)
                continue;
            double x_rot[3], s_rot[3];
            oracle_rotate(omega_axis, omega[i], F, xray, s1 + 3 * i, x_rot, s_rot);
            int st = single(coords, n, s_rot, x_rot, voxel, mu, vol, shape, full_iteration, is_exp,
                            scratch, out + i);
            if (st) {
#pragma omp atomic write
                status = st;
            }
        }
        free(scratch);
    }
    return status;
}

/* Per-voxel, per-leg detail of one reflection (given rotated vectors), for
 * path-level parity: face, len_path_2, number of class segments, first and
 * last path point and the four lengths.  Arrays are [n][2] (leg 0 incident,
 * leg 1 diffracted), points [n][2][3], lengths [n][2][4]. */
int oracle_leg_detail(const int64_t *coords, int64_t n, const double *s1_rot, const double *xray_rot,
                      const double *voxel, const int8_t *vol, const int64_t *shape, int full_iteration,
                      int64_t *face, int64_t *len, int64_t *nseg, int64_t *first, int64_t *last,
                      double *L, int32_t *status)
{
    if (n < 0 || check_coords(coords, n, shape))
        return ORC_ERR_ARGS;
    orc_dirs d;
    reflection_dirs(s1_rot, xray_rot, &d);
    int64_t cap = max_dim(shape) + 2;
    int64_t *scratch = malloc(sizeof(int64_t) * 2 * cap);
    if (!scratch)
        return ORC_ERR_NOMEM;
    for (int64_t k = 0; k < n; k++) {
        for (int leg = 0; leg < 2; leg++) {
            orc_leg r;
            memset(&r, 0, sizeof(r));
            int st = leg == 0
                ? march_leg(coords + 3 * k, d.d_in, d.th_in, d.ph_in, 1, vol, shape, full_iteration, voxel,
                            scratch, scratch + cap, &r)
                : march_leg(coords + 3 * k, d.d_out, d.th_out, d.ph_out, 0, vol, shape, full_iteration, voxel,
                            scratch, scratch + cap, &r);
            int64_t o = 2 * k + leg;
            status[o] = st;
            face[o] = r.face;
            len[o] = r.len;
            nseg[o] = r.nseg;
            for (int a = 0; a < 3; a++) {
                first[3 * o + a] = r.first[a];
                last[3 * o + a] = r.last[a];
            }
            for (int a = 0; a < 4; a++)
                L[4 * o + a] = r.L[a];
        }
    }
    free(scratch);
    return ORC_OK;
}

/* angles and my-frame directions of one reflection (for host-side parity) */
void oracle_reflection_dirs(const double *s1_rot, const double *xray_rot, double *out10)
{
    orc_dirs d;
    reflection_dirs(s1_rot, xray_rot, &d);
    out10[0] = d.th_in; out10[1] = d.ph_in; out10[2] = d.th_out; out10[3] = d.ph_out;
    for (int a = 0; a < 3; a++) {
        out10[4 + a] = d.d_in[a];
        out10[7 + a] = d.d_out[a];
    }
}

/* ------------------------------------------------- iterative bisection */

/* The reference's boundary search (AnACor/src/bisection.c:150-238): on the
 * ray c + m * q (q as in face_rule, which equals the ratios of increments(),
 * bisection.c:21-148, with the y sign folded), halve [shortest, longest] until
 * it is at most `resolution` long.  boundary 0: a label equal to cls moves
 * longest in; boundary 1: it moves shortest out.  The point returned is
 * floor(c + floor(mid) * q).  Positions outside the volume are undefined in
 * the reference; here they end the search with ORC_ERR_ARGS. */
typedef struct {
    int64_t p[3];
    double mid;
} orc_bis;

static int bisect(double longest, double shortest, double resolution, const int64_t *c, const double *q,
                  const int8_t *vol, const int64_t *shape, int boundary, int cls, orc_bis *out)
{
    double diff = longest - shortest;
    double mid = (longest + shortest) / 2.0;
    while (diff > resolution) {
        mid = (longest + shortest) / 2.0;
        int64_t p[3];
        for (int a = 0; a < 3; a++) {
            p[a] = (int64_t)floor((double)c[a] + mid * q[a]);
            if (p[a] < 0 || p[a] >= shape[a])
                return ORC_ERR_ARGS;
        }
        const int lab = vol[(p[0] * shape[1] + p[1]) * shape[2] + p[2]];
        if (boundary == 0) {
            if (lab == cls)
                longest = mid;
            else
                shortest = mid;
        } else {
            if (lab == cls)
                shortest = mid;
            else
                longest = mid;
        }
        diff = longest - shortest;
    }
    for (int a = 0; a < 3; a++)
        out->p[a] = (int64_t)floor((double)c[a] + floor(mid) * q[a]);
    out->mid = mid;
    return ORC_OK;
}

/* difference_length (bisection.c:260-270): z, then y, then x */
static double seg_len(const int64_t *s, const int64_t *e, const double *voxel)
{
    const double dz = (double)(s[0] - e[0]) * voxel[0];
    const double dy = (double)(s[1] - e[1]) * voxel[1];
    const double dx = (double)(s[2] - e[2]) * voxel[2];
    return sqrt(dz * dz + dy * dy + dx * dx);
}

static double abs_sum3(const int64_t *a, const int64_t *b)
{
    return fabs((double)(a[0] - b[0])) + fabs((double)(a[1] - b[1])) + fabs((double)(a[2] - b[2]));
}

/* iterative_bisection (bisection.c:312-463) + cal_path_bisection (:272-310)
 * for one leg: L = [liquor, loop, crystal, bubble].  The path holds the start
 * voxel, the sample's outer boundary, the crystal's outer boundary, then a
 * loop pair and a bubble pair when found; the lengths are read from the path
 * by its length only (5 points: the pair is counted as loop, 7: only the
 * second pair, as bubble), as the reference does. */
static int ib_leg(const int64_t *c, int64_t face, double th, double ph, const int8_t *vol, const int64_t *shape,
                  int num_cls, const double *voxel, double *L)
{
    orc_rule r;
    int st = face_rule(face, th, ph, &r);
    if (st)
        return st;
    const double res = 1.0;
    double air_longest;
    switch (face) {
    case 4: air_longest = (double)c[1]; break;
    case 5: air_longest = (double)(shape[1] - 1 - c[1]); break;
    case 6: air_longest = (double)c[2]; break;
    case 1: air_longest = (double)(shape[2] - 1 - c[2]); break;
    case 2: air_longest = (double)c[0]; break;
    default: air_longest = (double)(shape[0] - 1 - c[0]); break;
    }
    int64_t pts[7][3];
    int n = 0;
    for (int a = 0; a < 3; a++)
        pts[0][a] = c[a];
    n = 1;
    orc_bis air, cr, li, lo, bi, bo;
    if ((st = bisect(air_longest, 0.0, res, c, r.q, vol, shape, 0, 0, &air)))
        return st;
    memcpy(pts[n++], air.p, sizeof(air.p));
    if ((st = bisect(air.mid, 0.0, res, c, r.q, vol, shape, 1, 3, &cr)))
        return st;
    memcpy(pts[n++], cr.p, sizeof(cr.p));
    for (;;) {
        if ((st = bisect(air.mid, cr.mid, res, c, r.q, vol, shape, 0, 2, &li)))
            return st;
        if (abs_sum3(li.p, air.p) / 3 > 1) {
            if ((st = bisect(air.mid, li.mid, res, c, r.q, vol, shape, 1, 2, &lo)))
                return st;
            if (abs_sum3(li.p, lo.p) / 3 <= 2)
                break;
            memcpy(pts[n++], li.p, sizeof(li.p));
            memcpy(pts[n++], lo.p, sizeof(lo.p));
        }
        if (num_cls > 3) {
            if ((st = bisect(air.mid, cr.mid, res, c, r.q, vol, shape, 0, 4, &bi)))
                return st;
            if (abs_sum3(bi.p, air.p) > 1) {
                if ((st = bisect(air.mid, bi.mid, res, c, r.q, vol, shape, 1, 4, &bo)))
                    return st;
                if (abs_sum3(bi.p, bo.p) / 3 <= 2)
                    break;
                memcpy(pts[n++], bi.p, sizeof(bi.p));
                memcpy(pts[n++], bo.p, sizeof(bo.p));
            }
        }
        break;
    }
    const double total = seg_len(pts[0], pts[1], voxel);
    const double cr_l = seg_len(pts[0], pts[2], voxel);
    double lo_l = 0, bu_l = 0;
    if (n == 5)
        lo_l = seg_len(pts[3], pts[4], voxel);
    else if (n == 7)
        bu_l = seg_len(pts[5], pts[6], voxel);
    L[0] = total - lo_l - bu_l - cr_l - 0.0;
    L[1] = lo_l;
    L[2] = cr_l;
    L[3] = bu_l;
    return ORC_OK;
}

/* ib_test (AnACor/src/ray_tracing.c:25-163): mean over voxels of
 * exp(-sum mu (L_incident + L_diffracted)) with bisection paths
 * (resolution 1.0).  L_out (optional) receives [n][2][4] lengths. */
int oracle_ib(const int64_t *coords, int64_t n, const double *s1_rot, const double *xray_rot, const double *voxel,
              const double *mu, const int8_t *vol, const int64_t *shape, int num_cls, double *out, double *L_out)
{
    if (n <= 0 || check_coords(coords, n, shape))
        return ORC_ERR_ARGS;
    orc_dirs d;
    reflection_dirs(s1_rot, xray_rot, &d);
    double sum = 0;
    for (int64_t k = 0; k < n; k++) {
        const int64_t *c = coords + 3 * k;
        const int64_t f1 = oracle_cube_face(c, d.d_in, shape, 1);
        const int64_t f2 = oracle_cube_face(c, d.d_out, shape, 0);
        if (!f1 || !f2)
            return ORC_ERR_FACE;
        double l1[4], l2[4];
        int st = ib_leg(c, f1, d.th_in, d.ph_in, vol, shape, num_cls, voxel, l1);
        if (!st)
            st = ib_leg(c, f2, d.th_out, d.ph_out, vol, shape, num_cls, voxel, l2);
        if (st)
            return st;
        if (L_out)
            for (int m = 0; m < 4; m++) {
                L_out[8 * k + m] = l1[m];
                L_out[8 * k + 4 + m] = l2[m];
            }
        sum += rate(l1, l2, mu, 1);
    }
    *out = sum / n;
    return ORC_OK;
}

/* ib_single_gridding (AnACor/src/ray_tracing.c:427-482) for n voxels and one
 * direction: the given theta/phi must be the vector's to 1e-6 (the reference
 * asserts), the diffracted leg's exit face from cube_face, its lengths by
 * iterative bisection with those angles, then cal_rate with a zero incident
 * leg.  out[k] per voxel. */
int oracle_ib_gridding(const int64_t *coords, int64_t n, const double *s1_rot, double theta, double phi,
                       const double *voxel, const double *mu, const int8_t *vol, const int64_t *shape, int num_cls,
                       int is_exp, double *out)
{
    if (n <= 0 || check_coords(coords, n, shape))
        return ORC_ERR_ARGS;
    double th, ph, d_out[3];
    oracle_theta_phi(s1_rot, 0, &th, &ph);
    if (!(fabs(th - theta) < 1e-6) || !(fabs(ph - phi) < 1e-6))
        return ORC_ERR_ASSERT;
    oracle_myframe(s1_rot, d_out);
    const double zero[4] = {0, 0, 0, 0};
    for (int64_t k = 0; k < n; k++) {
        const int64_t *c = coords + 3 * k;
        const int64_t f = oracle_cube_face(c, d_out, shape, 0);
        if (!f)
            return ORC_ERR_FACE;
        double l2[4];
        const int st = ib_leg(c, f, theta, phi, vol, shape, num_cls, voxel, l2);
        if (st)
            return st;
        out[k] = rate(zero, l2, mu, is_exp);
    }
    return ORC_OK;
}
