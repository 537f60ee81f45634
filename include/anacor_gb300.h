/*
 * anacor_gb300.h -- C ABI of libanacor_gb300.so, the GB300 (sm_103a)
 * implementation of AnACor's analytical absorption-correction path.
 *
 * The first four entry points have exactly the signatures of the reference
 * library that AnACor's worker loads with ctypes (AnACor/utils/utils_mp.py:51-148),
 * so the library is a drop-in for AnACor/src/ray_tracing_cpu.so on that path.
 * Everything runs on the current CUDA device; there is no CPU fallback: when
 * no usable GPU is present every entry point fails with a status and a
 * message (anacor_last_error) instead of computing on the host.
 *
 * Conventions (same as the reference): coordinates are int64 (z, y, x) rows,
 * C-contiguous; shape is (z, y, x); voxel_size is (z, y, x); coefficients are
 * [liquor, loop, crystal, bubble]; label codes 0 vacuum, 1 liquor, 2 loop,
 * 3 crystal, 4 bubble; vectors are in the DIALS laboratory frame.
 */
#ifndef ANACOR_GB300_H
#define ANACOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ drop-ins -- */

/* Replaces AnACor/src/ray_tracing.c:365-374 (ray_tracing_overall).
 * Absorption factor A_h of reflections [0, len_result) (low/up are labels
 * only, as in the reference).  For reflection i the incident and diffracted
 * vectors are rotated by (R(omega_axis, omega_list[i]) * kp_rotation_matrix)^T
 * and A_i is the mean over the len_coord_list voxels of exp(-sum mu_m L_m).
 * label_list is the int8*** row table of a C-contiguous volume
 * (AnACor/utils/utils_os.py:45-68).  num_workers and store_paths are
 * accepted and ignored.  IsExp == 1 gives exp(-mu L), otherwise mu L.
 * Returns a malloc()ed double[len_result] that the caller releases with the C
 * library's free(), or NULL on error (see anacor_last_error). */
double *ray_tracing_overall(int64_t low, int64_t up, int64_t *coord_list, int64_t len_coord_list,
                            const double *scattering_vector_list, const double *omega_list,
                            const double *raw_xray, const double *omega_axis, const double *kp_rotation_matrix,
                            int64_t len_result, double *voxel_size, double *coefficients,
                            int8_t ***label_list, int64_t *shape, int full_iteration, int store_paths,
                            int num_workers, int IsExp);

/* Replaces AnACor/src/ray_tracing.c:166-171 (ray_tracing_single): A_h of one
 * reflection from already rotated vectors.  Returns NaN on error. */
double ray_tracing_single(int64_t *coord_list, int64_t len_coord_list, const double *rotated_s1,
                          const double *xray, double *voxel_size, double *coefficients, int8_t ***label_list,
                          int64_t *shape, int full_iteration, int64_t store_paths, int IsExp);

/* Replaces AnACor/src/ray_tracing.c:25-163 (ib_test, the iterative-bisection
 * variant, bound at utils_mp.py:95-109): A_h of one reflection from rotated
 * vectors with each leg's class boundaries found by bisection
 * (AnACor/src/bisection.c) instead of a march; num_cls > 3 also searches
 * bubbles.  An approximation of ray_tracing_single.  NaN on error (the
 * reference reads outside the volume where a search leaves it; here that is
 * ANACOR_ERR_ARGS). */
double ib_test(int64_t *coord_list, int64_t len_coord_list, double *rotated_s1, double *xray,
               double *voxel_size, double *coefficients, int8_t ***label_list, int64_t *shape,
               int full_iteration, int64_t store_paths, int num_cls);

/* Replaces AnACor/src/ray_tracing_gpu.c:33-42 (ray_tracing_gpu_overall, the
 * FP32 ABI of the reference's CUDA library).  Inputs are widened to double
 * and the same path runs; label_list_1d (the flat volume) is used when
 * non-NULL, else label_list.  gpumethod is ignored.  Returns a malloc()ed
 * float[len_result], or NULL on error. */
float *ray_tracing_gpu_overall(size_t low, size_t up, int *coord_list, size_t len_coord_list,
                               const float *scattering_vector_list, const float *omega_list,
                               const float *raw_xray, const float *omega_axis, const float *kp_rotation_matrix,
                               size_t len_result, float *voxel_size, float *coefficients, int8_t ***label_list,
                               int8_t *label_list_1d, int *shape, int full_iteration, int store_paths,
                               int gpumethod);

/* --------------------------------------------------------------- status -- */

enum {
    ANACOR_OK = 0,
    ANACOR_ERR_NO_FACE = 1,     /* a ray found no exit plane (reference: exit()) */
    ANACOR_ERR_ASSERT = 2,      /* face/angle combination the reference asserts on */
    ANACOR_ERR_ARGS = 3,
    ANACOR_ERR_CUDA = 4,
    ANACOR_ERR_NOMEM = 5,
    ANACOR_ERR_UNSUPPORTED = 6,
    ANACOR_ERR_DIRECTION = 7    /* non-finite or zero direction */
};

/* Status and message of the calling thread's last call (no counterpart in
 * the reference, which aborts the process instead). */
int anacor_last_status(void);
const char *anacor_last_error(void);
const char *anacor_version(void);

/* ------------------------------------------------------ flat-buffer API -- */

/* ray_tracing_overall over flat buffers: label is the C-contiguous int8
 * volume itself instead of a row table.  Writes A_h to out[n_refl].
 * Returns a status.  (No reference counterpart: the reference only takes the
 * int8*** table.) */
int anacor_absorption(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n_coords,
                      const double *s1, const double *omega, int64_t n_refl, const double *xray,
                      const double *omega_axis, const double *F, const double *voxel, const double *mu,
                      int full_iteration, int is_exp, double *out);

/* ------------------------------------------------------- resident plans -- */

/* A plan keeps one sample's volume, voxel list and reflection tables in
 * device memory so that the march can be re-run without host traffic.
 * (No reference counterpart.) */
typedef struct anacor_plan anacor_plan;

anacor_plan *anacor_plan_create(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n_coords,
                                const double *voxel, const double *mu, int full_iteration, int is_exp);
/* Host FP64 set-up of n_refl reflections and upload of their tables. */
int anacor_plan_set_reflections(anacor_plan *p, const double *s1, const double *omega, int64_t n_refl,
                                const double *xray, const double *omega_axis, const double *F);
/* Enqueue the march on `stream` (a cudaStream_t, NULL for the plan's own
 * stream).  Results stay on the device. */
int anacor_plan_run(anacor_plan *p, void *stream);
/* Copy the last results to out[n_refl], synchronise and check the device
 * status word. */
int anacor_plan_result(anacor_plan *p, double *out, void *stream);
/* Device pointer of the result array (valid until the plan is destroyed or
 * its reflections change). */
const double *anacor_plan_device_result(anacor_plan *p);
int64_t anacor_plan_n_refl(const anacor_plan *p);
/* Run once with step counting: *total = sum of len_path_2 over every ray of
 * every reflection (the label bytes the reference's march reads). */
int anacor_plan_count_steps(anacor_plan *p, uint64_t *total);
/* Number of CTAs one run launches and the number of kernels it enqueues. */
int anacor_plan_launch_info(const anacor_plan *p, int *grid, int *kernels);
void anacor_plan_destroy(anacor_plan *p);
/* The bisection variant (ib_test per reflection) over the plan's reflections;
 * results as for anacor_plan_run. */
int anacor_plan_run_bisection(anacor_plan *p, int num_cls, void *stream);
/* ib_test for every reflection (omega, s1 as for anacor_absorption). */
int anacor_bisection(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n_coords,
                     const double *s1, const double *omega, int64_t n_refl, const double *xray,
                     const double *omega_axis, const double *F, const double *voxel, const double *mu, int num_cls,
                     double *out);

/* Execution parameters of a plan (no counterpart in the reference; they do
 * not change the per-ray results, only the FP32 summation order of A_h):
 * variant = kernel variant: 1..4 the warp-cooperative march compiled for
 * 1..4 CTAs per SM, 5..8 the same register budgets with the distance-field
 * march (steps over increments that a chessboard distance field proves to
 * keep the label; needs labels in 0..7, else kErrUnsupported), 9..12 the
 * same on the 8 octant fields (each leg reads the field of its direction's
 * octant), 13..16 the same on a copy of the octant fields stored in 4x4x4
 * bricks of 64 bytes (a ray's next step along any axis mostly stays in the
 * 32-byte sector of its last load), 0 = process default; tile = voxels per
 * work item
 * (>= 128, 0 = unchanged); order = voxel order of the packed list: 0 the
 * caller's, 1 Morton (Z-order) of (z, y, x), 2..7 blocked (Morton order of
 * blocks of 1x2x16, 1x4x8, 2x4x32, 4x8x64, 4x16x32 or 8x16x128 voxels, row
 * order inside a block), -1 unchanged. */
int anacor_plan_configure(anacor_plan *p, int variant, int tile, int order);
/* The packed distance field the variants 5..8 march on, for a host volume:
 * out[v] = (label & 7) | (min(D, 31) << 3), D the chessboard distance from v
 * to the nearest voxel of the volume with another label (0 for label-0
 * voxels).  kErrUnsupported when a label lies outside 0..7.  No counterpart
 * in the reference. */
int anacor_distance_field(const int8_t *label, const int64_t *shape, uint8_t *out);
/* The 8 octant fields variants 9..12 march on: out[o][v] (8 volumes,
 * o = (sx < 0) | (sy < 0) << 1 | (sz < 0) << 2) = (label & 7) | (min(r + 1, 31) << 3),
 * r the largest box v + [0..r]^3 * (sz, sy, sx) (clipped to the volume) that
 * holds one label; 0 for label-0 voxels.  No counterpart in the reference. */
int anacor_octant_fields(const int8_t *label, const int64_t *shape, uint8_t *out);
int anacor_plan_config(const anacor_plan *p, int *variant, int *tile, int *order);
/* Autotuner: times every (variant, tile, order) candidate on the first
 * reflections of the plan (at least sample_refl of them) and keeps the
 * fastest; results are cached per volume shape and voxel-count class.
 * *best_ms = the chosen configuration's time scaled to all reflections. */
int anacor_plan_autotune(anacor_plan *p, int64_t sample_refl, float *best_ms);

/* One persistent launch over several plans (independent samples with their
 * own volumes, voxel lists and reflections).  Results land in each plan. */
int anacor_batch_run(anacor_plan *const *plans, int n_plans, void *stream);

/* A batch object: the same launch kept ready for repeated runs, optionally
 * captured once into a CUDA graph and replayed.  The plans must outlive it;
 * after a plan's reflections or configuration change, call
 * anacor_batch_configure to refresh it. */
typedef struct anacor_batch anacor_batch;
anacor_batch *anacor_batch_create(anacor_plan *const *plans, int n_plans);
/* variant (as for anacor_plan_configure) of the whole launch: 1..4 every
 * sample on the cooperative march; 5..16 every sample on its field of that
 * kind (built here when missing), one launch; each sample keeps its own tile
 * and voxel order. */
int anacor_batch_configure(anacor_batch *b, int variant);
/* Each plan's tile and voxel order by anacor_plan_autotune, then the
 * launch variant: the fastest of every register budget of the cooperative
 * march and of each field kind the samples allow, timed as whole launches. */
int anacor_batch_autotune(anacor_batch *b, int64_t sample_refl);
int anacor_batch_launch(anacor_batch *b, void *stream);
int anacor_batch_capture(anacor_batch *b, void *stream);
int anacor_batch_replay(anacor_batch *b, void *stream);
/* synchronise `stream` and check every plan's device status word */
int anacor_batch_wait(anacor_batch *b, void *stream);
int anacor_batch_info(const anacor_batch *b, int *grid, long long *items, int *variant);
/* Kernel launches per batch run: 1, or 2 under a field variant when some
 * sample's labels allow no field (labels outside 0..7): those samples run
 * first in the cooperative kernel of the same register budget. */
int anacor_batch_kernels(const anacor_batch *b);
void anacor_batch_destroy(anacor_batch *b);

/* ------------------------------------------------- no-allocation entry -- */

/* Size of the fixed device array behind anacor_absorption_noalloc.  Every GPU
 * that loads the library holds it until the process exits. */
#define ANACOR_NOALLOC_SCRATCH_BYTES (32u << 20)

/* No counterpart in the reference.  The absorption path for callers that must
 * not allocate device memory: hosts whose device memory belongs to a pool
 * they do not control (a framework allocator that has reserved the device),
 * and pipelines that forbid allocation after start-up because cudaMalloc and
 * cudaFree may synchronise the whole device.  The caller
 * passes device pointers for the C-contiguous int8 volume (d_label), the
 * int64 (z, y, x) voxel list (d_coords) and the result array (d_out,
 * n_refl doubles); s1, omega, xray, omega_axis, F, voxel, mu and shape are
 * host arrays as for anacor_absorption.  Everything else -- packed voxels,
 * reflection tables, tile partial sums, counters, the status word -- lives in
 * one file-scope device array of ANACOR_NOALLOC_SCRATCH_BYTES bytes, so the
 * call uses no cudaMalloc, cudaFree or other device allocator.  It needs
 *   8*n_coords + n_refl*(868 + 8*ceil(n_coords/2048)) bytes + ~1 KiB;
 * larger requests are rejected with ANACOR_ERR_ARGS (split the reflections
 * over several calls).  The first call on a device looks up the array's
 * address and uploads a constant table, so make that first call before any
 * stream capture.  All calls share the one array and it keeps the previous
 * call's contents: the call clears what must start at zero itself.  Calls
 * from several host threads of one process take a lock and run one after
 * another; work on the array that the library cannot see (another process's
 * calls, a replayed graph) races with a call.  Work is enqueued on `stream`
 * (a cudaStream_t), from pageable host memory, and the call waits for that
 * stream to drain before it returns, with a status, on success and on every
 * error after the first enqueue. */
int anacor_absorption_noalloc(const int8_t *d_label, const int64_t *shape, const int64_t *d_coords,
                              int64_t n_coords, const double *s1, const double *omega, int64_t n_refl,
                              const double *xray, const double *omega_axis, const double *F,
                              const double *voxel, const double *mu, int full_iteration, int is_exp,
                              double *d_out, void *stream);

/* ---------------------------------------------------- GPU voxel sampling -- */

/* The crystal-voxel list chosen on the GPU from a volume uploaded once
 * (AnACor/utils/utils_rt.py:27-253 samples on the host with np.where):
 * method 0 every voxel with label == crystal_code, in C order; 1 the
 * reference's 'even' method, entries np.linspace(0, M, n, endpoint=False,
 * dtype=int) of that list with n = int(M * sampling_ratio / 100) when
 * sampling_ratio > 0, else M // sampling_size (M when M < sampling_size); 2
 * the stride lattice (z, y, x multiples of stride).  Rows are int64 (z, y, x). */
anacor_plan *anacor_plan_create_sampled(const int8_t *label, const int64_t *shape, int crystal_code, int method,
                                        int64_t sampling_size, double sampling_ratio, int stride, const double *voxel,
                                        const double *mu, int full_iteration, int is_exp);
int64_t anacor_plan_n_voxels(const anacor_plan *p);
/* the plan's voxel list [n][3] in the order it was given or selected */
int anacor_plan_voxels(const anacor_plan *p, int64_t *coords_out);
/* the same selection returned to the host (capacity rows; *n_out = count,
 * ANACOR_ERR_ARGS when capacity is too small) */
int anacor_sample_voxels(const int8_t *label, const int64_t *shape, int crystal_code, int method,
                         int64_t sampling_size, double sampling_ratio, int stride, int64_t *coords_out,
                         int64_t capacity, int64_t *n_out);

/* ------------------------------------------------ gridding (absorption map) -- */

/* The reference's approximate mode (AnACor/utils/utils_gridding.py:63-473):
 * a map of the diffracted leg alone for every direction of a regular
 * (theta, phi) grid and every crystal voxel, then per reflection a lookup of
 * both legs' map values and A_h = mean_k exp(-(z_incident + z_diffracted)).
 * The map stays on the GPU ([direction][voxel], the plan's voxel order);
 * the object borrows the plan, which must outlive it. */
typedef struct anacor_gridding anacor_gridding;

/* Grid direction i = i_phi * n_theta + i_theta (utils_gridding.py:270-276 and
 * :140-152): its DIALS-frame unit vector [3] and polar angles. */
int anacor_gridding_directions(int n_theta, int n_phi, double *rotated_s1, double *theta, double *phi);
/* method 2 (the reference's default): map = float32 sum_m mu_m L_m; method 1:
 * float32 exp(-sum).  n_theta, n_phi >= 18 (the reference uses 360 x 180). */
anacor_gridding *anacor_gridding_create(anacor_plan *plan, int n_theta, int n_phi, int method);
/* Build the map.  With NULL arrays the directions are those of
 * anacor_gridding_directions; otherwise the caller's per-direction vector and
 * angles, as ray_tracing_single_gridding takes them. */
int anacor_gridding_build(anacor_gridding *g, const double *rotated_s1, const double *theta, const double *phi);
int anacor_gridding_info(const anacor_gridding *g, int64_t *n_dirs, int64_t *n_vox, int *len_theta, int *len_phi);
/* the padded interpolation axes (utils_gridding.py:408-440), radians */
int anacor_gridding_axes(const anacor_gridding *g, double *theta_axis, double *phi_axis);
const float *anacor_gridding_device_map(const anacor_gridding *g, int64_t *ld);
/* host copy / replacement of the map, [n_dirs][n_vox] in the caller's voxel
 * order (the reference's saved absorption_map layout) */
int anacor_gridding_map(const anacor_gridding *g, float *host_map);
int anacor_gridding_set_map(anacor_gridding *g, const float *host_map);
/* A_h of n reflections (omega, s1 as for anacor_absorption): method 1
 * nearest grid point (the reference's default), 2 bilinear */
int anacor_gridding_interpolate(anacor_gridding *g, const double *s1, const double *omega, int64_t n,
                                const double *xray, const double *omega_axis, const double *F, int method,
                                double *out);
int anacor_gridding_interpolate_async(anacor_gridding *g, const double *s1, const double *omega, int64_t n,
                                      const double *xray, const double *omega_axis, const double *F, int method,
                                      double *d_out, void *stream);
/* The lookups of n reflections prepared once (host set-up, rows kept on the
 * device), then the interpolation kernel alone into d_out[n] on `stream`. */
int anacor_gridding_prepare(anacor_gridding *g, const double *s1, const double *omega, int64_t n, const double *xray,
                            const double *omega_axis, const double *F, int method);
int anacor_gridding_run(anacor_gridding *g, double *d_out, void *stream);
void anacor_gridding_destroy(anacor_gridding *g);

/* Drop-in for AnACor/src/ray_tracing.c:484-534 (bound at
 * utils_gridding.py:104-118): one voxel's map value for one direction
 * (IsExp = 0: sum_m mu_m L_m; 1: exp(-sum)).  NaN with
 * ANACOR_ERR_ASSERT where the reference asserts (angles not those of
 * rotated_s1).  The volume is cached on the GPU by row-table address and shape
 * between calls. */
double ray_tracing_single_gridding(int64_t *coord, const double *rotated_s1, double theta, double phi,
                                   double *voxel_size, double *coefficients, int8_t ***label_list, int64_t *shape,
                                   int full_iteration, int index, int IsExp);
/* Drop-in for AnACor/src/ray_tracing.c:427-482 (bound at
 * utils_gridding.py:120-134): the same value with the diffracted leg's
 * lengths found by iterative bisection (resolution 1.0; num_cls > 3 also
 * searches bubble boundaries) on the GPU; exp(-sum) taken on the host when
 * IsExp.  NaN with ANACOR_ERR_ASSERT where the reference asserts, and
 * ANACOR_ERR_ARGS where a search leaves the volume (undefined in the
 * reference).  Shares the cached volume of ray_tracing_single_gridding. */
double ib_single_gridding(int64_t *coord, const double *rotated_s1, double theta, double phi, double *voxel_size,
                          double *coefficients, int8_t ***label_list, int64_t *shape, int full_iteration, int index,
                          int num_cls, int IsExp);
/* Drop-in for AnACor/src/gridding_interpolation.c:100-163 (bound at
 * utils_gridding.py:547-573): the padded map in the reference's layout
 * [len_coord_list][ny][nx] (FP64), interpolation_method 1 nearest / 2
 * bilinear.  Returns a malloc()ed array (free() it) or NULL with
 * anacor_last_error(). */
double *nearest_neighbor_interpolate_overall(int64_t low, int64_t up, int64_t *coord_list, int64_t len_coord_list,
                                             const double *scattering_vector_list, const double *omega_list,
                                             const double *raw_xray, const double *omega_axis,
                                             const double *kp_rotation_matrix, int64_t len_result,
                                             double *voxel_size, double *coefficients, int num_workers, int IsExp,
                                             double *theta_list, double *phi_list, double *gridding_data, size_t nx,
                                             size_t ny, double theta_min, double theta_max, double phi_min,
                                             double phi_max, int interpolation_method);

/* ------------------------------------------------------ learned surrogate -- */

/* No counterpart in the reference (its absorption factors always come from
 * the ray tracer).  An ensemble of MLPs per sample: x7 = (omega / 2pi wrapped
 * to [0, 1), incident and diffracted unit vectors in the crystal frame) ->
 * 64 Fourier features [sin 2pi(Bx), cos 2pi(Bx)] -> 4 x 256 GELU -> the
 * standardised log A_h.  BF16 weights and activations, FP32 accumulation on
 * the tcgen05 tensor cores, FP32 Adam masters.  Training targets are absorption
 * factors computed by the tracer; at inference the ensemble spread flags the
 * reflections to re-trace.  Calls run on the object's own stream unless a
 * stream is passed, and are not thread-safe on one object. */
typedef struct anacor_surrogate anacor_surrogate;

anacor_surrogate *anacor_surrogate_create(int n_members, uint32_t seed, float fourier_scale);
void anacor_surrogate_destroy(anacor_surrogate *s);
/* FP32 parameters per member (layers 1-4 weights [out][in] and biases, then
 * the output weights and bias, padded to a multiple of 8) */
int64_t anacor_surrogate_param_count(void);
int anacor_surrogate_members(const anacor_surrogate *s);
/* copy all members' parameters [members][param_count] to (to_device = 0) or
 * from (1) host memory */
int anacor_surrogate_params(anacor_surrogate *s, float *host, int to_device);
/* the 32 x 7 Fourier matrix B, read (0) or written (1) */
int anacor_surrogate_fourier(anacor_surrogate *s, float *host32x7, int to_device);
/* output scale: log A_h = mean + std_dev * y; read (set = 0) or written */
int anacor_surrogate_scale(anacor_surrogate *s, double *mean, double *std_dev, int set);
/* x7 rows [n][7] of reflections (omega, s1 as for anacor_absorption) */
int anacor_surrogate_inputs(const double *omega, const double *s1, int64_t n, const double *xray,
                            const double *omega_axis, const double *F, float *x7_out);
int anacor_surrogate_inputs_device(const double *d_omega, const double *d_s1, int64_t n, const double *xray,
                                   const double *omega_axis, const double *F, float *d_x7, void *stream);
/* training set: n rows of x7 and their log A_h; sets the output scale to the
 * targets' mean and standard deviation */
int anacor_surrogate_set_data(anacor_surrogate *s, const float *x7, const double *log_ah, int64_t n);
/* `steps` Adam steps; each member draws its own batch of `batch` rows (a
 * multiple of 1024) with replacement.  The learning rate follows a cosine
 * from lr_max to lr_min over total_steps (counted from the first step ever
 * taken).  loss_out (optional, `steps` floats): mean member loss per step. */
int anacor_surrogate_train(anacor_surrogate *s, int steps, int batch, float lr_max, float lr_min, int total_steps,
                           float *loss_out);
/* gradients of every member's loss on one batch (rows a multiple of 1024;
 * targets in output units y), without an update: grads_out [members][param
 * count] (optional), y_out [members][rows] (optional) */
int anacor_surrogate_gradients(anacor_surrogate *s, const float *x7, const float *target, int rows,
                               float *grads_out, float *y_out);
/* ensemble mean of A_h and relative spread (std / mean over members) for n
 * rows of x7; members_out (optional) [members][n] log A_h per member */
int anacor_surrogate_predict(anacor_surrogate *s, const float *x7, int64_t n, float *mean_out, float *spread_out,
                             float *members_out);
int anacor_surrogate_predict_device(anacor_surrogate *s, const float *d_x7, int64_t n, float *d_mean,
                                    float *d_spread, float *d_members, void *stream);
/* How inference runs: fused = 1 (the default) one persistent kernel per call
 * that keeps a 128-row tile's features and activations in shared memory and
 * its accumulator in tensor memory through all four layers and the head of
 * every member (weights streamed by bulk copies); 0 layer by layer, each
 * layer a tensor-core GEMM whose activations go through device memory.  Both
 * give the same numbers. */
int anacor_surrogate_set_inference(anacor_surrogate *s, int fused);
/* flags[i] bit 0: row i is in the seeded random audit sample (probability
 * audit_fraction); bit 1: spread[i] > spread_threshold or not finite */
int anacor_surrogate_audit_flags(const float *d_spread, int64_t n, uint32_t seed, double audit_fraction,
                                 float spread_threshold, uint8_t *d_flags, void *stream);
int anacor_surrogate_save(anacor_surrogate *s, const char *path);
int anacor_surrogate_load(anacor_surrogate *s, const char *path);

/* the surrogate's tensor-core GEMM alone, for checks: C[z] = A[z] B[z]^T with
 * A [batch][M][K], B [batch][N][K] rounded to BF16, FP32 accumulation, the K
 * range split into ksplit slices whose partial products are summed in order */
int anacor_tc_gemm_check(const float *A, const float *B, int M, int N, int K, int batch, int ksplit, float *C);
/* The error path of the tensor-core kernels' bounded mbarrier waits: one CTA
 * allocates tensor memory, waits at most `iterations` polls for a phase that
 * nothing completes, records the error, releases the tensor memory and
 * returns; *status = 1 when the wait gave up (the device stays usable). */
int anacor_wait_guard_check(unsigned iterations, int32_t *status);

/* ---------------------------------------------------------- diagnostics -- */

/* Rotated incident and diffracted vectors of n reflections, computed by the
 * host set-up code (AnACor/src/ray_tracing.c:397-407). */
int anacor_rotated_vectors(const double *omega_axis, const double *omega, const double *F, const double *xray,
                           const double *s1, int64_t n, double *rotated_xray, double *rotated_s1);

/* Per-voxel, per-leg march detail of one reflection (rotated vectors as for
 * ray_tracing_single), computed on the GPU: exit face, path length in steps
 * (len_path_2), number of class segments, first and last path point and the
 * four material lengths.  Arrays are [n][2] (leg 0 incident, leg 1
 * diffracted), points [n][2][3], lengths [n][2][4]. */
int anacor_leg_detail(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n,
                      const double *rotated_s1, const double *rotated_xray, const double *voxel,
                      int full_iteration, int32_t *face, int32_t *len, int32_t *nseg, int32_t *first,
                      int32_t *last, double *L, int32_t *status);

/* The absorption kernel's shared arrays are sized for its fixed block of 256
 * threads, and the kernels refuse any other block shape on the device (status
 * bit 1 << ANACOR_ERR_ARGS, no access).  This launches the absorption kernel
 * over no work with `threads` threads per block (a multiple of 32, at most
 * 256) and returns the status word it left in *status: the guard bit for
 * fewer than 256 threads, 0 for 256. */
int anacor_block_guard_check(int threads, int32_t *status);

#ifdef __cplusplus
}
#endif

#endif /* ANACOR_GB300_H */
