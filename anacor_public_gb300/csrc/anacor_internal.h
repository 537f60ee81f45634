// Internal layout shared by the host set-up code and the sm_103a kernels.
//
// The path computed here is AnACor's analytical absorption factor (the
// reference's C/OpenMP ray_tracing_overall, AnACor/src/ray_tracing.c:365-425):
// for every reflection, march a ray from every sampled crystal voxel along the
// incident and the diffracted direction through the label volume, sum the
// path length per material and average exp(-sum mu_m L_m) over the voxels.
//
// Split of the work:
//  * host (FP64, the C library's libm, -ffp-contract=off): per reflection the
//    goniometer rotation, the polar angles and, for each leg and each of the
//    six exit faces, the signed step ratios of the reference's cal_coord.
//    These are the only transcendental evaluations of the path; doing them on
//    the host with the same libm keeps them bit-identical to the reference.
//  * device: exit-face selection, the voxel march (exact 32.32 fixed point with
//    an FP64 fallback near rounding boundaries), per-material lengths (FP64,
//    the reference's operation order), Beer-Lambert factor and the mean.
#pragma once
#include <stdint.h>

namespace anacor {

// Volume axes are limited so that path positions fit 13 bits and the
// fixed-point accumulators cannot overflow (see FaceRule).
constexpr int kMaxDim = 8191;
// Fixed-point increments are used when every |ratio| of a face is below this.
constexpr double kFastRatioLimit = 65536.0;
// A 32.32 fixed-point position whose fraction lies within this many 2^-32
// units of a rounding boundary is recomputed with the reference's FP64
// expression.  Worst-case disagreement between the fixed-point value and the
// reference's two-rounding FP64 value is below 4096 + 1024 units (Q rounding
// times i <= 8192, plus two FP64 roundings of magnitudes < 2^30).
constexpr uint32_t kAmbiguityMargin = 1u << 14;
// Class-change entries kept per leg in shared memory before the slow path.
constexpr int kMaxSegments = 16;

enum Status : int {
    kOk = 0,
    kErrNoFace = 1,      // no exit plane (reference: exit(EXIT_FAILURE))
    kErrAssert = 2,      // face / angle combination the reference asserts on
    kErrArgs = 3,
    kErrCuda = 4,
    kErrNoMem = 5,
    kErrUnsupported = 6,
    kErrDirection = 7,   // non-finite or zero direction vector
};

// March of one leg through one exit face (AnACor/src/ray_tracing_basic.c:396-1460).
// Position on axis a (0 = z, 1 = y, 2 = x) at increment i:
//     R(c_a + fl(i * q[a]))     R = floor, or C round() when use_round
// clamped to [0, dim_a - 1], for i = 0 .. steps-1.
struct alignas(16) FaceRule {
    double q[3];          // signed FP64 step ratios
    long long Q[3];       // llrint(q * 2^32) when `fast`
    uint8_t status;       // kOk or kErrAssert
    uint8_t use_round;
    uint8_t fast;         // all |q| < kFastRatioLimit and finite
    uint8_t exact_mask;   // bit a: q[a] is a small integer, fixed point exact
    uint8_t count_axis;   // axis whose coordinate sets the step count
    uint8_t count_kind;   // 0: c+1, 1: dim-c, 2: dim-c+1
    uint8_t vac_limit;    // consecutive-vacuum limit under full_iteration
    uint8_t octant;       // (dx < 0) | (dy < 0) << 1 | (dz < 0) << 2 of the march direction
    // floor(2^16 / qmax) - 1 (at most 2^22), qmax the larger |q| of the two
    // axes besides count_axis: the distance-field march's skip multiplier
    uint32_t skip_rq;
};
static_assert(sizeof(FaceRule) == 64, "FaceRule layout");

// Direction data for the exit-face test of one leg (AnACor/src/ray_tracing_basic.c:69-186).
// e is the my-frame direction (z, y, x components), negated for the incident leg
// so that every candidate distance is fl(n / |e_a|).
struct alignas(16) LegHead {
    double e[3];
    float inv[3];         // (float)(1 / |e_a|), +inf for a zero component
    uint32_t sign_bits;   // bit a: e_a > 0; bit 3+a: e_a < 0; bit 6: exact face test only
};
static_assert(sizeof(LegHead) == 48, "LegHead layout");

// Everything the kernels need about one reflection: leg 0 incident, leg 1 diffracted.
struct alignas(16) ReflTable {
    LegHead head[2];
    FaceRule rule[2][6];  // indexed by face code - 1
};
static_assert(sizeof(ReflTable) == 96 + 768, "ReflTable layout");

// Host-side set-up of one reflection.  Returns kOk, kErrDirection.
int setup_reflection(const double *omega_axis, double omega, const double *F, const double *xray,
                     const double *s1, ReflTable *out, double *rotated_xray, double *rotated_s1);
// Set-up from already rotated vectors (ray_tracing_single's inputs).
int setup_rotated(const double *rotated_xray, const double *rotated_s1, ReflTable *out);
// Diffracted leg only (leg 0 zeroed) of a direction whose polar angles are
// given, as ray_tracing_single_gridding takes them
// (AnACor/src/ray_tracing.c:484-534).
int setup_direction(const double *rotated_s1, double theta, double phi, ReflTable *out);
// dials_2_thetaphi_22 (AnACor/src/ray_tracing_basic.c:13-50); incident legs use -v.
void polar_angles(const double *v, bool incident, double *theta, double *phi);
// Rotated incident and diffracted vectors of one reflection (matrices.h:49-68 order).
void rotate_reflection(const double *omega_axis, double omega, const double *F, const double *xray,
                       const double *s1, double *rotated_xray, double *rotated_s1);
// OpenMP-parallel set-up of many reflections; returns the first error status.
int setup_reflections(const double *omega_axis, const double *omega, const double *F, const double *xray,
                      const double *s1, int64_t n, ReflTable *out, int threads);

}  // namespace anacor
