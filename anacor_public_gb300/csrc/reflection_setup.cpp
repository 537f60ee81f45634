// Host-side per-reflection set-up (FP64, C library libm).
//
// Compiled with -ffp-contract=off: every expression below must round exactly
// where the reference's C does (AnACor/src/ray_tracing.c:397-407,
// AnACor/src/matrices.h, AnACor/src/ray_tracing_basic.c:13-67 and the ratio
// definitions inside cal_coord, :396-1460), so the tables handed to the GPU
// are bit-identical to the quantities the reference computes per ray.
#include <cmath>
#include <cstring>
#include <limits>

#include <omp.h>

#include "anacor_internal.h"

namespace anacor {
namespace {

constexpr double kPi = 3.14159265358979323846;

// Rodrigues rotation about `a` by `w` (AnACor/src/matrices.h:49-68).
void rotation_about(const double *a, double w, double *m)
{
    const double x = a[0], y = a[1], z = a[2];
    const double c = std::cos(w), s = std::sin(w);
    const double k = 1 - c;
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

// Row-major product with the accumulator started at 0.0 (AnACor/src/matrices.h:14-29).
void product(const double *A, const double *B, double *C, int m, int n, int p)
{
    for (int i = 0; i < m; i++)
        for (int j = 0; j < p; j++) {
            double acc = 0.0;
            for (int k = 0; k < n; k++)
                acc += A[i * n + k] * B[k * p + j];
            C[i * p + j] = acc;
        }
}

// Polar angles (AnACor/src/ray_tracing_basic.c:13-50); the incident leg uses -v.
void polar(const double *v, bool incident, double &th, double &ph)
{
    double a = v[0], b = v[1], c = v[2];
    if (incident) {
        a = -a; b = -b; c = -c;
    }
    const double r = std::sqrt(a * a + b * b);
    if (b == 0) {
        th = std::atan(-c / (-r + 0.001));
        ph = std::atan(-a / (b + 0.001));
    } else if (b < 0) {
        th = std::atan(-c / r);
        ph = std::atan(-a / b);
    } else {
        th = (c < 0) ? kPi - std::atan(-c / r) : -kPi - std::atan(-c / r);
        ph = -std::atan(-a / (-b));
    }
}

// DIALS (x, y, z) -> my frame (x, z, y), accumulated from 0.0 as the
// reference's permutation product does (-0.0 becomes +0.0).
void my_frame(const double *v, double *out)
{
    static const double P[3][3] = {{1, 0, 0}, {0, 0, 1}, {0, 1, 0}};
    for (int i = 0; i < 3; i++) {
        double acc = 0.0;
        for (int j = 0; j < 3; j++)
            acc += P[i][j] * v[j];
        out[i] = acc;
    }
}

// Signed step ratios per exit face.  The reference writes each face as
// "new = R(c +/- i * ratio)"; "c - fl(i*r)" is the IEEE operation
// "c + fl(i*(-r))", so the sign is folded into q.  Axis order (z, y, x).
// The libm values the six face rules of one leg use, each evaluated once
// (several rules share them; every rule reads the same expressions as its
// reference formula, so the ratios are bit for bit those of separate calls).
struct LegTrig {
    double tan_th, tan_pi_th, tan_ph, cos_ph, tan_aph, sin_aph, cos_aph, sin_ph;
    double tan_ath, tan_pi_ath, sin_mph;   // by the |theta| < pi/2 branch
};

void leg_trig(double th, double ph, LegTrig &t)
{
    const double half = kPi / 2;
    t.tan_th = std::tan(th);
    t.tan_pi_th = std::tan(kPi - th);
    t.tan_ph = std::tan(ph);
    t.cos_ph = std::cos(ph);
    t.tan_aph = std::tan(std::fabs(ph));
    t.sin_aph = std::sin(std::fabs(ph));
    t.cos_aph = std::cos(std::fabs(ph));
    t.sin_ph = std::sin(ph);
    if (std::fabs(th) < half) {
        t.tan_ath = std::tan(std::fabs(th));
        t.tan_pi_ath = t.sin_mph = 0.0;
    } else {
        t.tan_ath = 0.0;
        t.tan_pi_ath = std::tan(kPi - std::fabs(th));
        t.sin_mph = std::sin(-ph);
    }
}

void face_rule(int face, double th, double ph, const LegTrig &t, FaceRule &r)
{
    const double half = kPi / 2;
    const bool lower = th > 0;   // floor when theta > 0, else round (faces 6, 2, 3, 1)
    r.status = kOk;
    r.vac_limit = 50;
    r.use_round = !lower;
    switch (face) {
    case 6:   // x_min, ray_tracing_basic.c:418-509
        r.status = std::fabs(th) <= half ? kOk : kErrAssert;
        r.q[2] = -1;
        r.q[1] = -(t.tan_th / t.cos_ph);
        r.q[0] = t.tan_ph;
        r.count_axis = 2; r.count_kind = 0;
        break;
    case 2:   // z_min, :512-709
        if (std::fabs(th) < half) {
            r.status = ph < 0 ? kOk : kErrAssert;
            r.q[2] = -(1 / t.tan_aph);
            r.q[1] = -(t.tan_th / t.sin_aph);
        } else {
            r.status = ph > 0 ? kOk : kErrAssert;
            r.q[2] = 1 / t.tan_aph;
            r.q[1] = -(t.tan_pi_th / t.sin_aph);
        }
        r.q[0] = -1;
        r.count_axis = 0; r.count_kind = 0;
        break;
    case 3:   // z_max, :712-896
        if (std::fabs(th) < half) {
            r.status = ph > 0 ? kOk : kErrAssert;
            r.q[2] = -(1 / t.tan_aph);
            r.q[1] = -(t.tan_th / t.sin_aph);
            r.count_kind = 1;
        } else {
            r.status = ph < 0 ? kOk : kErrAssert;
            r.q[2] = 1 / t.tan_aph;
            r.q[1] = -(t.tan_pi_th / t.sin_aph);
            r.count_kind = 2;
        }
        r.q[0] = 1;
        r.count_axis = 0;
        break;
    case 4:   // y_min, :899-1101; always floor
        r.status = th > 0 ? kOk : kErrAssert;
        if (std::fabs(th) < half) {
            r.q[2] = -(t.cos_aph / t.tan_ath);
            r.q[0] = t.sin_ph / t.tan_ath;
        } else {
            r.q[2] = t.cos_aph / t.tan_pi_ath;
            r.q[0] = t.sin_mph / t.tan_pi_ath;
        }
        r.q[1] = -1;
        r.use_round = 0;
        r.count_axis = 1; r.count_kind = 0;
        break;
    case 5:   // y_max, :1104-1277; always round
        r.status = th < 0 ? kOk : kErrAssert;
        if (std::fabs(th) < half) {
            r.q[2] = -(t.cos_aph / t.tan_ath);
            r.q[0] = t.sin_ph / t.tan_ath;
            r.count_kind = 1;
        } else {
            r.q[2] = t.cos_aph / t.tan_pi_ath;
            r.q[0] = -(t.sin_ph / t.tan_pi_ath);
            r.count_kind = 2;
        }
        r.q[1] = 1;
        r.use_round = 1;
        r.count_axis = 1;
        break;
    default:  // 1, x_max, :1280-1372
        r.status = std::fabs(th) >= half ? kOk : kErrAssert;
        r.q[2] = 1;
        r.q[1] = -(t.tan_pi_th / t.cos_aph);
        r.q[0] = -(t.tan_ph);
        r.count_axis = 2; r.count_kind = 1;
        r.vac_limit = 10;
        break;
    }
    bool fast = true;
    r.exact_mask = 0;
    for (int a = 0; a < 3; a++) {
        const double q = r.q[a];
        if (!(std::fabs(q) < kFastRatioLimit)) {   // also rejects NaN / inf
            fast = false;
            r.Q[a] = 0;
            continue;
        }
        r.Q[a] = std::llrint(std::ldexp(q, 32));
        if (q == std::trunc(q) && std::fabs(q) <= 128.0)
            r.exact_mask |= uint8_t(1u << a);
    }
    r.fast = fast;
    // signs of the march direction: the count axis steps by q = +-1, the
    // others by their ratios (a zero ratio counts as positive)
    r.octant = uint8_t((r.q[2] < 0) | (r.q[1] < 0) << 1 | (r.q[0] < 0) << 2);
    // never above 2^16 / qmax: the device's skip (D - 2) * skip_rq >> 16 stays
    // within floor((D - 2) / qmax)
    const double qmax = std::max(std::fabs(r.q[r.count_axis == 0 ? 1 : 0]), std::fabs(r.q[r.count_axis == 2 ? 1 : 2]));
    if (!(qmax < kFastRatioLimit))
        r.skip_rq = 0;
    else if (qmax < 1.0 / 64.0)
        r.skip_rq = 1u << 22;
    else
        r.skip_rq = (uint32_t)std::max(0.0, std::floor(65536.0 / qmax) - 1.0);
}

int fill_leg(const double *dir_my, bool incident, double th, double ph, LegHead &h, FaceRule *rules)
{
    bool nonzero = false;
    h.sign_bits = 0;
    for (int a = 0; a < 3; a++) {
        const double e = incident ? -dir_my[a] : dir_my[a];
        if (!std::isfinite(e))
            return kErrDirection;
        h.e[a] = e;
        if (e != 0) {
            nonzero = true;
            h.inv[a] = float(1.0 / std::fabs(e));
            h.sign_bits |= e > 0 ? (1u << a) : (1u << (3 + a));
            // outside this range the FP32 distance estimate may lose range
            if (!(std::fabs(e) >= 0x1p-60 && std::fabs(e) <= 0x1p60))
                h.sign_bits |= 64u;
        } else {
            h.inv[a] = std::numeric_limits<float>::infinity();
        }
    }
    if (!nonzero)
        return kErrDirection;
    LegTrig t;
    leg_trig(th, ph, t);
    for (int f = 1; f <= 6; f++) {
        std::memset(&rules[f - 1], 0, sizeof(FaceRule));
        face_rule(f, th, ph, t, rules[f - 1]);
    }
    return kOk;
}

}  // namespace

int setup_rotated(const double *xr, const double *sr, ReflTable *out)
{
    std::memset(out, 0, sizeof(*out));
    double th_out, ph_out, th_in, ph_in, d_in[3], d_out[3];
    polar(sr, false, th_out, ph_out);
    polar(xr, true, th_in, ph_in);
    my_frame(xr, d_in);
    my_frame(sr, d_out);
    int st = fill_leg(d_in, true, th_in, ph_in, out->head[0], out->rule[0]);
    if (st)
        return st;
    return fill_leg(d_out, false, th_out, ph_out, out->head[1], out->rule[1]);
}

int setup_direction(const double *sr, double theta, double phi, ReflTable *out)
{
    std::memset(out, 0, sizeof(*out));
    double d_out[3];
    my_frame(sr, d_out);
    return fill_leg(d_out, false, theta, phi, out->head[1], out->rule[1]);
}

void polar_angles(const double *v, bool incident, double *theta, double *phi)
{
    polar(v, incident, *theta, *phi);
}

void rotate_reflection(const double *axis, double omega, const double *F, const double *xray, const double *s1,
                       double *xr, double *sr)
{
    double r[9], rf[9], t[9];
    rotation_about(axis, omega, r);
    product(r, F, rf, 3, 3, 3);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            t[j * 3 + i] = rf[i * 3 + j];
    product(t, xray, xr, 3, 3, 1);
    product(t, s1, sr, 3, 3, 1);
}

int setup_reflection(const double *axis, double omega, const double *F, const double *xray,
                     const double *s1, ReflTable *out, double *rx, double *rs)
{
    double xr[3], sr[3];
    rotate_reflection(axis, omega, F, xray, s1, xr, sr);
    if (rx)
        std::memcpy(rx, xr, sizeof(xr));
    if (rs)
        std::memcpy(rs, sr, sizeof(sr));
    return setup_rotated(xr, sr, out);
}

int setup_reflections(const double *axis, const double *omega, const double *F, const double *xray,
                      const double *s1, int64_t n, ReflTable *out, int threads)
{
    int status = kOk;
    const int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt) if (n > 64)
    for (int64_t i = 0; i < n; i++) {
        int st = setup_reflection(axis, omega[i], F, xray, s1 + 3 * i, out + i, nullptr, nullptr);
        if (st) {
#pragma omp atomic write
            status = st;
        }
    }
    return status;
}

}  // namespace anacor
