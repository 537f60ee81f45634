// Launch interface of the absorption kernels (host C++ <-> trace_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "anacor_internal.h"

namespace anacor {

// Voxels per work item (one CTA pass) unless a sample sets its own: a sample
// with N voxels and R reflections is R * ceil(N / tile) work items.
constexpr int kTile = 2048;
constexpr int kMinTile = 512;

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
    double *out;            // [n_refl]
    double *partial;        // [n_refl * tiles] scratch
    unsigned int *arrive;   // [n_refl] scratch, zero before the first launch
    int *status;            // bit (1 << code) set for every failing voxel's status
    unsigned long long *steps;  // optional: += sum of len_path_2 over all rays
    const double *sq;       // optional [3][sq_stride]: fl(fl(d * voxel_a)^2) for d < dim_a
    int sq_stride;
    const double *qtab;     // optional quotient table covering den <= max(dim)
    long long work_begin;   // first global work item of this sample
};

int rcp_table_init();
int absorption_block_threads();
// CTAs per SM of a register-budget variant (1..4; 0 = the process default)
int absorption_occupancy(int *blocks_per_sm, int variant = 0);
// the process-default register-budget variant (CTAs per SM it targets)
int absorption_variant();

cudaError_t launch_pack_coords(const long long *d_c, int n, const int *dims, short4 *d_out, int *d_status,
                               cudaStream_t st);
// Same, with the packed list sorted by the Morton code of (z, y, x).
cudaError_t launch_pack_coords_morton(const long long *d_c, int n, const int *dims, short4 *d_out, int *d_status,
                                      cudaStream_t st);
// Persistent launch over every work item of `n_desc` samples; `grid` CTAs
// take items from `d_counter` (reset inside the launch sequence).
cudaError_t launch_absorption(const SampleDesc *d_descs, int n_desc, long long total_items,
                              unsigned long long *d_counter, int grid, cudaStream_t st, int variant = 0);
cudaError_t launch_leg_detail(const ReflTable *d_tab, const int8_t *d_vol, const int *dims, const short4 *d_coords,
                              int n, const double *d_voxel, int full, const double *d_sq, int sq_stride,
                              const double *d_qtab, int *face, int *len, int *nseg, int *first, int *last, double *L,
                              int *status, cudaStream_t st);
// Table of correctly rounded quotients fl(s / d), 1 <= d <= max_den,
// 1 <= s <= d + 1 (row d starts at (d-1)(d+2)/2).
size_t quotient_table_entries(int max_den);
cudaError_t launch_quotient_table(double *d_q, int max_den, cudaStream_t st);
// Largest denominator a quotient table is built for (67 MB); larger volumes
// use the reciprocal-and-correction quotient.
constexpr int kQuotientTableMaxDen = 4097;

}  // namespace anacor
