// Launch interface of the absorption kernels (host C++ <-> trace_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "anacor_internal.h"

struct anacor_plan;

namespace anacor {

// Voxels per work item unless a sample sets its own: a sample with N voxels
// and R reflections is R * ceil(N / tile) work items (taken per warp by the
// absorption kernel, per CTA by the map and bisection kernels).
constexpr int kTile = 2048;
constexpr int kMinTile = 128;
// A plan's tile is raised where needed so that a reflection has at most this
// many tiles (bounds the per-(reflection, tile) partial sums).
constexpr int kMaxTilesPerRefl = 4096;

// One sample (volume + voxel list + reflections) of a launch.  All pointers
// are device pointers.
struct SampleDesc {
    const int8_t *vol;
    int dim[3];             // z, y, x
    int n_vox;
    const short4 *coords;   // (z, y, x, 0)
    const ReflTable *refl;  // [n_refl]
    long long n_refl;
    int tiles;              // ceil(n_vox / tile)
    int tile;               // voxels per work item
    int full_iteration;
    int is_exp;
    double mu[4];           // [liquor, loop, crystal, bubble]
    double voxel[3];        // z, y, x
    float voxelf[3];        // (float) voxel, for the FP32 lengths of A_h
    float muf[4];           // (float) mu, for the FP32 exponent of A_h
    double *out;            // [n_refl]
    double *partial;        // [n_refl * tiles] scratch
    unsigned int *arrive;   // [n_refl] scratch, zero before the first launch
    int *status;            // bit (1 << code) set for every failing voxel's status
    unsigned long long *steps;  // optional: += sum of len_path_2 over all rays
    const double *sq;       // optional [3][sq_stride]: fl(fl(d * voxel_a)^2) for d < dim_a
    int sq_stride;
    const double *qtab;     // optional quotient table covering den <= max(dim)
    long long work_begin;   // first global work item of this sample
    const uint8_t *field;   // label | distance << 3 (launch_distance_field); required by variants 5..12
    long long field_stride; // 0: one centred field; else 8 octant fields this far apart (launch_octant_fields)
    int brick_sy, brick_sz; // 0: linear fields; else 4^3-bricked (launch_brick_fields), byte strides of a
                            // brick step in y and z; required by variants 9..12
    const int *order;       // optional [n_refl]: the k-th reflection processed (octant-sorted), else k
};

// Absorption map of one sample (gridding mode): for every grid direction d and
// voxel k the diffracted leg alone, out[d * ld + k] = (float) sum_m mu_m L_m
// (or (float) exp(-sum) when is_exp), as ray_tracing_single_gridding computes
// it (AnACor/src/ray_tracing.c:484-534) with cal_rate's zero incident leg.
struct MapDesc {
    const int8_t *vol;
    int dim[3];
    int n_vox;
    const short4 *coords;
    const ReflTable *dirs;  // [n_dirs], leg 1 set
    long long n_dirs;
    int tiles, tile;
    int full_iteration;
    int is_exp;
    double mu[4];
    double voxel[3];
    float *out;
    double *out64;          // optional: the FP64 values instead (out unused)
    long long ld;
    const int *col;         // optional: output column of packed voxel k
    int *status;
    const double *sq;
    int sq_stride;
    const double *qtab;
    const uint8_t *field;   // optional: octant fields (launch_octant_fields) for the field march
    long long field_stride;
};

// Device-resident sample of a plan, for the other entry points that march it.
struct PlanView {
    const int8_t *vol;
    int dims[3];
    int n_vox;
    const short4 *coords;     // packed list (Morton order when morton)
    const long long *c64;     // the caller's (z, y, x) list, device
    int order;                // voxel order of `coords` (0: the caller's)
    int full_iteration, is_exp;
    double mu[4], voxel[3];
    const double *sq;
    int sq_stride;
    const double *qtab;
    cudaStream_t stream;
    int sms;
    const uint8_t *field;     // the plan's octant fields, when built (plan_view_field)
    long long field_stride;
};
int plan_view(const anacor_plan *p, PlanView *out);
// plan_view with the plan's octant fields, built if needed (left out, with
// no error, when the labels do not fit 3 bits)
int plan_view_field(anacor_plan *p, PlanView *out);

int rcp_table_init();
// Stream-ordered allocation from the library's pool of the current device
// (the device's default pool when it has none); freed with cudaFreeAsync.
cudaError_t lib_malloc_async(void **p, size_t bytes, cudaStream_t st);
int absorption_block_threads();
// Launch the absorption kernel over no work with `threads` (a multiple of 32,
// at most the kernel's block size) threads per block; *status_out is the
// status word it leaves (ANACOR_ERR_ARGS bit set when the block-shape guard
// refused the launch).
int block_guard_selftest(int threads, int *status_out);
int absorption_set_carveout(int pct);
// Kernel variants: 1..4 the cooperative march with a register budget for
// 1..4 CTAs per SM; 5..8 the same budgets with the distance-field march on
// linear fields; 9..12 on 4^3-bricked fields (every sample needs its `field`
// in the variant's layout).
constexpr int kVariants = 12;
// CTAs per SM of a variant (0 = the process default)
int absorption_occupancy(int *blocks_per_sm, int variant = 0);
// the process-default register-budget variant (CTAs per SM it targets)
int absorption_variant();

cudaError_t launch_pack_coords(const long long *d_c, int n, const int *dims, short4 *d_out, int *d_status,
                               cudaStream_t st);
// Voxel orders of the packed list: 0 the caller's, 1 Morton (Z-order) of
// (z, y, x), 2 .. kVoxelOrders-1 blocked (Morton order of blocks, row order
// inside a block; block shapes in voxel_order.cu).
constexpr int kVoxelOrders = 8;
cudaError_t launch_pack_coords_order(const long long *d_c, int n, const int *dims, int order, short4 *d_out,
                                     int *d_status, cudaStream_t st);
// Crystal-voxel sampling (sampling.cu): voxels with label == code (and, for
// stride > 1, z, y, x multiples of stride) in C order as linear indices;
// unravel_voxels writes (z, y, x) int64 of entry floor(j * step) (step > 0,
// the reference's 'even' picks) or of every entry (step == 0).
cudaError_t count_sampled_voxels(const int8_t *d_vol, const int *dims, int code, int stride, long long *d_count,
                                 cudaStream_t st);
cudaError_t select_sampled_voxels(const int8_t *d_vol, const int *dims, int code, int stride, long long *d_lin,
                                  long long *d_count, cudaStream_t st);
cudaError_t unravel_voxels(const long long *d_lin, long long n_out, double step, const int *dims, long long *d_coords,
                           cudaStream_t st);
// perm[k] = index in the caller's list of the k-th voxel of the packed list
cudaError_t launch_order_permutation(const long long *d_c, int n, const int *dims, int order, int *d_perm,
                                     cudaStream_t st);
// Chessboard distance field of a volume packed with its labels (see
// distance_field.cu): d_out and d_tmp hold dims[0]*dims[1]*dims[2] bytes each;
// *d_bad becomes nonzero when a label lies outside 0..7 (no field then).
cudaError_t launch_distance_field(const int8_t *d_vol, const int *dims, uint8_t *d_out, uint8_t *d_tmp, int *d_bad,
                                  cudaStream_t st);
// The 8 octant fields ([octant][Z][Y][X], octant = (sx<0) | (sy<0)<<1 | (sz<0)<<2):
// d_out holds 8 volumes, d_tmp 6.
cudaError_t launch_octant_fields(const int8_t *d_vol, const int *dims, uint8_t *d_out, uint8_t *d_tmp, int *d_bad,
                                 cudaStream_t st);
// Bricked copies of `n_fields` linear fields (each dims[0]*dims[1]*dims[2]
// bytes, consecutive): 4x4x4 bricks of 64 bytes in (z, y, x) brick order,
// bytes (z, y, x) inside a brick, padding bytes 0.  Each copy holds
// brick_field_bytes(dims) bytes; brick_strides gives the y and z brick steps.
size_t brick_field_bytes(const int *dims);
void brick_strides(const int *dims, int *sy, int *sz);
cudaError_t launch_brick_fields(const uint8_t *d_lin, const int *dims, int n_fields, uint8_t *d_out,
                                cudaStream_t st);
// Persistent launch over every work item of `n_desc` samples; `grid` CTAs
// take items from `d_counter` (reset inside the launch sequence).
cudaError_t launch_absorption(const SampleDesc *d_descs, int n_desc, long long total_items,
                              unsigned long long *d_counter, int grid, cudaStream_t st, int variant = 0);
cudaError_t launch_leg_detail(const ReflTable *d_tab, const int8_t *d_vol, const int *dims, const short4 *d_coords,
                              int n, const double *d_voxel, int full, const double *d_sq, int sq_stride,
                              const double *d_qtab, int *face, int *len, int *nseg, int *first, int *last, double *L,
                              int *status, cudaStream_t st);
// The reference's iterative-bisection variant (ib_test) over the same work
// items as launch_absorption; num_cls > 3 also searches bubble boundaries.
cudaError_t launch_bisection(const SampleDesc *d_descs, int n_desc, long long total_items,
                             unsigned long long *d_counter, int grid, int num_cls, cudaStream_t st);
int bisection_occupancy(int *blocks_per_sm);
// ib_single_gridding for n voxels of one direction (leg 1 of d_dir):
// d_out[k] = sum_m mu_m (0 + L_m) with the bisection lengths (exp is left to
// the caller), d_status[k] its status; d_vox_mu = voxel[3], mu[4].
cudaError_t launch_ib_direction(const ReflTable *d_dir, const int8_t *d_vol, const int *dims, const short4 *d_coords,
                                int n, const double *d_vox_mu, int num_cls, double *d_out, int *d_status,
                                cudaStream_t st);
// Persistent launch over n_dirs * tiles work items of the map.
cudaError_t launch_gridding_map(const MapDesc *d_desc, long long total_items, unsigned long long *d_counter, int grid,
                                cudaStream_t st, bool field = false);
int gridding_map_occupancy(int *blocks_per_sm, bool field = false);
// Lookup of one reflection in an absorption map: for each leg (0 incident,
// 1 diffracted) the map rows (grid directions) and weights of the value, as
// the reference's interpolation reads it
// (AnACor/src/gridding_interpolation.c:16-45, 48-76): nearest uses row[l][0];
// bilinear sums w[l][j] * z(row[l][j]) for j = 0..3 in that order.
struct InterpRow {
    long long row[2][4];
    double w[2][4];
};
// out[r] = mean over voxels k of exp(-(z_0 + z_1)), z_l the leg's map value;
// value (k, row) is map[k * sK + row * sR]
cudaError_t launch_gridding_interp_f32(const float *map, long long sK, long long sR, int n_vox, const InterpRow *rows,
                                       long long n_refl, int linear, double *out, cudaStream_t st);
cudaError_t launch_gridding_interp_f64(const double *map, long long sK, long long sR, int n_vox,
                                       const InterpRow *rows, long long n_refl, int linear, double *out,
                                       cudaStream_t st);
// Table of correctly rounded quotients fl(s / d), 1 <= d <= max_den,
// 1 <= s <= d + 1 (row d starts at (d-1)(d+2)/2).
size_t quotient_table_entries(int max_den);
cudaError_t launch_quotient_table(double *d_q, int max_den, cudaStream_t st);
// Largest denominator a quotient table is built for (67 MB); larger volumes
// use the reciprocal-and-correction quotient.
constexpr int kQuotientTableMaxDen = 4097;

}  // namespace anacor
