// anacor_absorption_noalloc: the absorption path for callers that must not
// allocate device memory.
//
// Some callers cannot call cudaMalloc (or any allocator) at the moment they
// need absorption factors: hosts whose device memory is owned by a pool they
// do not control (a framework allocator that has reserved the device), or
// real-time pipelines that forbid allocation after start-up because
// cudaMalloc and cudaFree may synchronise the whole device.
// This entry point takes device-resident inputs and output from the caller and
// keeps everything else the kernel needs -- packed voxel coordinates,
// per-reflection tables, per-tile partial sums, arrival counters, the work
// counter, the status word and the launch descriptor -- in one file-scope
// device array of fixed size, ANACOR_NOALLOC_SCRATCH_BYTES.  Every GPU that
// loads the library holds that array until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "anacor_gb300.h"
#include "anacor_internal.h"
#include "trace_launch.h"

namespace anacor {
int report_status(int st, const char *msg);
}

using namespace anacor;

namespace {

constexpr size_t kScratchBytes = ANACOR_NOALLOC_SCRATCH_BYTES;

// The scratch array.  In host code `g_noalloc_scratch` is only a stand-in
// for the symbol, not a device address: its address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceSetup {
    bool ready = false;
    unsigned char *scratch = nullptr;   // device address of g_noalloc_scratch
    int sms = 0;
    int blocks_per_sm = 0;
};

std::mutex g_mu;
DeviceSetup g_setup[64];

// host staging for reflection tables, filled and copied in chunks
constexpr int kStageTables = 256;
ReflTable g_stage[kStageTables];

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int device_setup(DeviceSetup **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return report_status(kErrCuda, "anacor_absorption_noalloc: no usable CUDA device");
    if (dev < 0 || dev >= 64)
        return report_status(kErrCuda, "anacor_absorption_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceSetup &d = g_setup[dev];
    if (!d.ready) {
        void *p = nullptr;
        if ((e = cudaGetSymbolAddress(&p, g_noalloc_scratch)) != cudaSuccess || !p)
            return report_status(kErrCuda, "anacor_absorption_noalloc: cudaGetSymbolAddress failed");
        cudaDeviceProp prop;
        if ((e = cudaGetDeviceProperties(&prop, dev)) != cudaSuccess)
            return report_status(kErrCuda, "anacor_absorption_noalloc: cudaGetDeviceProperties failed");
        if (rcp_table_init() != kOk)
            return report_status(kErrCuda, "anacor_absorption_noalloc: reciprocal table upload failed");
        if (absorption_occupancy(&d.blocks_per_sm) != kOk || d.blocks_per_sm <= 0)
            return report_status(kErrCuda, "anacor_absorption_noalloc: kernel not loadable on this device");
        d.scratch = static_cast<unsigned char *>(p);
        d.sms = prop.multiProcessorCount;
        d.ready = true;
    }
    *out = &d;
    return kOk;
}

int cuda_error(cudaError_t e, const char *what)
{
    char msg[256];
    std::snprintf(msg, sizeof(msg), "anacor_absorption_noalloc: %s: %s", what, cudaGetErrorString(e));
    return report_status(kErrCuda, msg);
}

// Error return once work is enqueued: drain the stream first, so that no
// kernel of this call still reads the caller's buffers or writes the scratch
// array when the caller gets control back.
int drained(cudaStream_t st, int status)
{
    cudaStreamSynchronize(st);
    return status;
}

// Held from the first write to the scratch array until the call returns: calls
// from several host threads run one after another.
std::mutex g_call_mu;

}  // namespace

extern "C" int anacor_absorption_noalloc(const int8_t *d_label, const int64_t *shape, const int64_t *d_coords,
                                         int64_t n_coords, const double *s1, const double *omega, int64_t n_refl,
                                         const double *xray, const double *omega_axis, const double *F,
                                         const double *voxel, const double *mu, int full_iteration, int is_exp,
                                         double *d_out, void *stream)
{
    if (!d_label || !shape || !voxel || !mu || n_coords < 0 || n_refl < 0 ||
        (n_coords > 0 && !d_coords) ||
        (n_refl > 0 && (!s1 || !omega || !xray || !omega_axis || !F || !d_out)))
        return report_status(kErrArgs, "anacor_absorption_noalloc: bad arguments");
    for (int a = 0; a < 3; a++)
        if (shape[a] <= 0 || shape[a] > kMaxDim)
            return report_status(kErrArgs, "anacor_absorption_noalloc: volume axes must lie in [1, 8191]");
    if ((uint64_t)shape[0] * shape[1] * shape[2] >= (1ull << 31))
        return report_status(kErrArgs, "anacor_absorption_noalloc: volume must hold fewer than 2^31 voxels");
    if (n_coords == 0)
        return report_status(kErrArgs, "anacor_absorption_noalloc: the voxel list is empty");

    // scratch layout, each part 256-byte aligned
    const long long tiles = (n_coords + kTile - 1) / kTile;
    const size_t off_desc = 0;
    const size_t off_counter = align256(off_desc + sizeof(SampleDesc));
    const size_t off_status = off_counter + sizeof(unsigned long long);
    const size_t off_coords = align256(off_status + sizeof(int));
    const size_t off_tables = align256(off_coords + (size_t)n_coords * sizeof(short4));
    const size_t off_partial = align256(off_tables + (size_t)n_refl * sizeof(ReflTable));
    const size_t off_arrive = align256(off_partial + (size_t)n_refl * (size_t)tiles * sizeof(double));
    const size_t need = align256(off_arrive + (size_t)n_refl * sizeof(unsigned));
    if (need > kScratchBytes) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "anacor_absorption_noalloc: %lld voxels x %lld reflections need %zu scratch bytes, "
                      "more than the fixed %zu; split the reflections over several calls",
                      (long long)n_coords, (long long)n_refl, need, kScratchBytes);
        return report_status(kErrArgs, msg);
    }

    std::lock_guard<std::mutex> call_lock(g_call_mu);
    DeviceSetup *dev = nullptr;
    if (int st = device_setup(&dev))
        return st;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *base = dev->scratch;
    int *d_status = reinterpret_cast<int *>(base + off_status);
    short4 *d_pack = reinterpret_cast<short4 *>(base + off_coords);
    ReflTable *d_tables = reinterpret_cast<ReflTable *>(base + off_tables);
    double *d_partial = reinterpret_cast<double *>(base + off_partial);
    unsigned *d_arrive = reinterpret_cast<unsigned *>(base + off_arrive);
    SampleDesc *d_desc = reinterpret_cast<SampleDesc *>(base + off_desc);
    unsigned long long *d_counter = reinterpret_cast<unsigned long long *>(base + off_counter);
    const int dims[3] = {(int)shape[0], (int)shape[1], (int)shape[2]};

    cudaError_t e;
    // the array keeps the previous call's contents: zero what must start at zero
    if ((e = cudaMemsetAsync(d_status, 0, sizeof(int), st)) ||
        (n_refl > 0 && (e = cudaMemsetAsync(d_arrive, 0, (size_t)n_refl * sizeof(unsigned), st))))
        return drained(st, cuda_error(e, "cudaMemsetAsync"));
    if ((e = launch_pack_coords(reinterpret_cast<const long long *>(d_coords), (int)n_coords, dims, d_pack,
                                d_status, st)))
        return drained(st, cuda_error(e, "coordinate packing"));

    // reflection tables: host FP64 set-up, one thread, in chunks through a
    // static staging area (no heap, no thread pool)
    for (int64_t r0 = 0; r0 < n_refl; r0 += kStageTables) {
        const int64_t m = std::min<int64_t>(kStageTables, n_refl - r0);
        for (int64_t k = 0; k < m; k++)
            if (setup_reflection(omega_axis, omega[r0 + k], F, xray, s1 + 3 * (r0 + k), &g_stage[k], nullptr,
                                 nullptr))
                return drained(st, report_status(kErrDirection,
                                                 "anacor_absorption_noalloc: non-finite or zero direction"));
        if ((e = cudaMemcpyAsync(d_tables + r0, g_stage, (size_t)m * sizeof(ReflTable), cudaMemcpyHostToDevice,
                                 st)) ||
            (e = cudaStreamSynchronize(st)))
            return drained(st, cuda_error(e, "table upload"));
    }

    static SampleDesc desc;
    std::memset(&desc, 0, sizeof(desc));
    desc.vol = d_label;
    for (int a = 0; a < 3; a++) {
        desc.dim[a] = dims[a];
        desc.voxel[a] = voxel[a];
        desc.voxelf[a] = (float)voxel[a];
    }
    for (int a = 0; a < 4; a++) {
        desc.mu[a] = mu[a];
        desc.muf[a] = (float)mu[a];
    }
    desc.n_vox = (int)n_coords;
    desc.coords = d_pack;
    desc.refl = d_tables;
    desc.n_refl = n_refl;
    desc.tiles = (int)tiles;
    desc.tile = kTile;
    desc.full_iteration = full_iteration;
    desc.is_exp = is_exp;
    desc.out = d_out;
    desc.partial = d_partial;
    desc.arrive = d_arrive;
    desc.status = d_status;
    desc.steps = nullptr;
    desc.work_begin = 0;
    if ((e = cudaMemcpyAsync(d_desc, &desc, sizeof(desc), cudaMemcpyHostToDevice, st)))
        return drained(st, cuda_error(e, "descriptor upload"));

    const long long items = (long long)n_refl * tiles;
    if (items > 0) {
        const long long cap = (long long)dev->sms * dev->blocks_per_sm;
        const int grid = (int)std::max(1ll, std::min(items, cap));
        if ((e = launch_absorption(d_desc, 1, items, d_counter, grid, st)))
            return drained(st, cuda_error(e, "kernel launch"));
    }
    int status = 0;
    if ((e = cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st)))
        return drained(st, cuda_error(e, "status download"));
    for (int b = 1; b < 16; b++)
        if (status & (1 << b))
            return report_status(b, b == kErrArgs ? "anacor_absorption_noalloc: a coordinate lies outside the volume"
                                 : b == kErrAssert ? "anacor_absorption_noalloc: exit face inconsistent with the "
                                                     "ray angles (the reference asserts here)"
                                                   : "anacor_absorption_noalloc: a ray found no exit plane");
    return report_status(kOk, "");
}
