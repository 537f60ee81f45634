// C ABI of libanacor_gb300.so (declared in include/anacor_gb300.h).
//
// Host side of the path: argument checks, the FP64 per-reflection set-up
// (reflection_setup.cpp), device buffers, launches and the reference's
// ownership rules (malloc()ed result freed by the caller's free()).
#include <cuda_runtime.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <thread>
#include <vector>

#include "anacor_gb300.h"
#include "anacor_internal.h"
#include "trace_launch.h"

using namespace anacor;

namespace {

thread_local int t_status = 0;
thread_local std::string t_msg;

int fail(int st, const std::string &msg)
{
    t_status = st;
    t_msg = msg;
    return st;
}

int cuda_fail(cudaError_t e, const char *what)
{
    return fail(kErrCuda, std::string(what) + ": " + cudaGetErrorString(e));
}

int succeed()
{
    t_status = kOk;
    t_msg.clear();
    return kOk;
}

const char *status_text(int st)
{
    switch (st) {
    case kErrNoFace: return "a ray found no exit plane";
    case kErrAssert: return "exit face inconsistent with the ray angles (the reference asserts here)";
    case kErrArgs: return "a coordinate lies outside the volume";
    case kErrDirection: return "non-finite or zero direction vector";
    default: return "error";
    }
}

// ---------------------------------------------------------------- devices

struct DeviceState {
    bool ready = false;
    int sms = 0;
    int blocks_per_sm = 0;
    cudaStream_t stream = nullptr;
    double *qtab = nullptr;   // quotient table for den <= qtab_den (never freed: plans keep pointers)
    int qtab_den = 0;
    int bps[kVariants + 1] = {};    // CTAs per SM of each kernel variant (index 1..kVariants)
};


std::mutex g_mu;
DeviceState g_dev[64];
// The library's stream-ordered memory pool per device.  It keeps up to
// ANACOR_POOL_KEEP_MB (default 16 GiB) of freed memory between calls, so that
// a drop-in call does not unmap and map again the gigabyte or so of volume,
// fields and partial sums it allocates (the default pool returns freed memory
// at every synchronisation).
cudaMemPool_t g_pool[64] = {};

// Plan-level variants: 1..4 cooperative march, 5..8 the centred distance
// field, 9..12 the octant fields, 13..16 the octant fields in 4^3 bricks;
// 9..12 run the kernels of 5..8 (linear fields), 13..16 those of 9..12.
constexpr int kPlanVariants = 16;
int kernel_variant(int v) { return v > 8 ? v - 4 : v; }
int budget_of(int v) { return v > 0 ? (v - 1) % 4 + 1 : absorption_variant(); }
// field a plan variant marches on: 0 none, 1 centred, 2 octant, 3 bricked octant
int field_kind(int v) { return v <= 4 ? 0 : (v <= 8 ? 1 : (v <= 12 ? 2 : 3)); }

// CTAs per SM of `variant` (0: the process default) on this device
int variant_occupancy(DeviceState *d, int variant)
{
    const int v = variant > 0 ? kernel_variant(variant) : absorption_variant();
    std::lock_guard<std::mutex> lk(g_mu);
    if (!d->bps[v]) {
        int b = 0;
        if (absorption_occupancy(&b, v) != kOk || b <= 0)
            b = 1;
        d->bps[v] = b;
    }
    return d->bps[v];
}


int current_device(DeviceState **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "no usable CUDA device");
    if (dev < 0 || dev >= 64)
        return fail(kErrCuda, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceState &d = g_dev[dev];
    if (!d.ready) {
        cudaDeviceProp prop;
        if ((e = cudaGetDeviceProperties(&prop, dev)) != cudaSuccess)
            return cuda_fail(e, "cudaGetDeviceProperties");
        if (prop.major < 10)
            return fail(kErrCuda, "this library is built for sm_103a (Blackwell Ultra) only");
        if (rcp_table_init() != kOk)
            return fail(kErrCuda, "reciprocal table upload failed");
        // 40 % of the unified storage as shared memory: room for 4 CTAs' 19 KB and
        // the rest L1 for the label gathers (measured best of 0/25/40/60/100 %,
        // by about 1 %); ANACOR_SMEM_CARVEOUT overrides
        const char *cv = std::getenv("ANACOR_SMEM_CARVEOUT");
        absorption_set_carveout(cv ? std::atoi(cv) : 40);
        if (absorption_occupancy(&d.blocks_per_sm) != kOk || d.blocks_per_sm <= 0)
            return fail(kErrCuda, "kernel not loadable on this device");
        if ((e = cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_fail(e, "cudaStreamCreate");
        {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t pool = nullptr;
            if (cudaMemPoolCreate(&pool, &props) == cudaSuccess) {
                const char *mb = std::getenv("ANACOR_POOL_KEEP_MB");
                uint64_t keep = (uint64_t)(mb ? std::atoll(mb) : 16384) << 20;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
                g_pool[dev] = pool;
            } else {
                cudaGetLastError();   // no pool of our own: the device's default pool serves
            }
        }
        d.sms = prop.multiProcessorCount;
        d.ready = true;
    }
    *out = &d;
    return kOk;
}

}  // namespace

cudaError_t anacor::lib_malloc_async(void **p, size_t bytes, cudaStream_t st)
{
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && g_pool[dev])
        return cudaMallocFromPoolAsync(p, bytes, g_pool[dev], st);
    return cudaMallocAsync(p, bytes, st);
}

namespace {

template <class T>
cudaError_t dev_alloc(T **p, size_t count, cudaStream_t st)
{
    *p = nullptr;
    if (count == 0)
        return cudaSuccess;
    return lib_malloc_async(reinterpret_cast<void **>(p), count * sizeof(T), st);
}

template <class T>
void dev_free(T *&p, cudaStream_t st)
{
    if (p)
        cudaFreeAsync(p, st);
    p = nullptr;
}

// Quotient table covering den <= max_den on this device (nullptr when the
// volume is larger than the table limit).
const double *quotient_table(DeviceState *d, int max_den)
{
    if (max_den > kQuotientTableMaxDen)
        return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (d->qtab_den < max_den) {
        // grow in steps so that a series of plans does not rebuild it each time
        const int den = std::min(kQuotientTableMaxDen, std::max(max_den, std::max(1025, 2 * d->qtab_den)));
        double *q = nullptr;
        if (cudaMalloc(&q, quotient_table_entries(den) * sizeof(double)) != cudaSuccess)
            return nullptr;
        if (launch_quotient_table(q, den, d->stream) != cudaSuccess || cudaStreamSynchronize(d->stream) != cudaSuccess) {
            cudaFree(q);
            return nullptr;
        }
        d->qtab = q;
        d->qtab_den = den;
    }
    return d->qtab;
}

bool valid_shape(const int64_t *shape)
{
    for (int a = 0; a < 3; a++)
        if (shape[a] <= 0 || shape[a] > kMaxDim)
            return false;
    return (uint64_t)shape[0] * shape[1] * shape[2] < (1ull << 31);
}

// Flat base of an int8*** row table built over a C-contiguous volume
// (AnACor/utils/utils_os.py:45-68).  Returns nullptr if the rows are not one
// uniformly strided block.
const int8_t *flat_base(int8_t ***table, const int64_t *shape)
{
    if (!table || !table[0] || !table[0][0])
        return nullptr;
    const int8_t *base = table[0][0];
    const int64_t Y = shape[1], X = shape[2];
    for (int64_t z = 0; z < shape[0]; z++) {
        if (!table[z])
            return nullptr;
        for (int64_t y = 0; y < Y; y++)
            if (table[z][y] != base + (z * Y + y) * X)
                return nullptr;
    }
    return base;
}

}  // namespace

// Error reporting for entry points defined in other translation units.
namespace anacor {
int report_status(int st, const char *msg)
{
    return st ? fail(st, msg) : succeed();
}
}  // namespace anacor

// ------------------------------------------------------------------ plans

struct anacor_plan {
    int dims[3] = {0, 0, 0};
    int n_vox = 0;
    int full = 0, is_exp = 1;
    double mu[4] = {0, 0, 0, 0};
    double voxel[3] = {0, 0, 0};
    cudaStream_t stream = nullptr;
    DeviceState *dev = nullptr;
    int8_t *d_vol = nullptr;
    short4 *d_coords = nullptr;
    ReflTable *d_refl = nullptr;
    double *d_out = nullptr;
    double *d_partial = nullptr;
    unsigned *d_arrive = nullptr;
    int *d_status = nullptr;
    unsigned long long *d_counter = nullptr;
    SampleDesc *d_desc = nullptr;
    unsigned long long *d_steps = nullptr;
    double *d_sq = nullptr;        // [3][sq_stride] fl(fl(d * voxel_a)^2)
    int sq_stride = 0;
    const double *d_qtab = nullptr;  // device quotient table (owned by the device state)
    ReflTable *h_refl = nullptr;   // pinned staging
    bool h_refl_borrowed = false;  // h_refl is the calling thread's staging buffer (one-call plans)
    int *d_order = nullptr;        // processing order of the reflections (grouped by direction octants)
    std::vector<int> h_order;
    int64_t n_refl = 0, refl_cap = 0;
    size_t partial_cap = 0;        // entries of d_partial (refl_cap * tiles)
    int tiles = 0;
    int tile = kTile;              // voxels per work item
    int variant = 0;               // register-budget variant (0: process default)
    int order = 1;                 // voxel order of the packed list (0 the caller's, 1 Morton, 2.. blocked)
    long long *d_c64 = nullptr;    // the caller's int64 voxel list (for re-packing)
    uint8_t *d_field = nullptr;    // label | distance << 3, built on first use by variants 5..8
    int field_state = 0;           // 0 not built, 1 built, -1 labels outside 0..7 (no field)
    uint8_t *d_field8 = nullptr;   // the 8 octant fields, built on first use by variants 9..12
    int field8_state = 0;
    uint8_t *d_field8b = nullptr;  // the same in 4^3 bricks, built on first use by variants 13..16
    int field8b_state = 0;
};

namespace {

void plan_release(anacor_plan *p)
{
    cudaStream_t st = p->stream;
    dev_free(p->d_vol, st);
    dev_free(p->d_coords, st);
    dev_free(p->d_refl, st);
    dev_free(p->d_out, st);
    dev_free(p->d_partial, st);
    dev_free(p->d_arrive, st);
    dev_free(p->d_status, st);
    dev_free(p->d_counter, st);
    dev_free(p->d_desc, st);
    dev_free(p->d_steps, st);
    dev_free(p->d_sq, st);
    dev_free(p->d_c64, st);
    dev_free(p->d_field, st);
    dev_free(p->d_field8, st);
    dev_free(p->d_field8b, st);
    dev_free(p->d_order, st);
    if (p->h_refl && !p->h_refl_borrowed)
        cudaFreeHost(p->h_refl);
    p->h_refl = nullptr;
    cudaStreamSynchronize(st);
}

// True when p lies in page-locked host memory (cudaHostAlloc'd or registered).
bool host_pinned(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Pinned staging for the reflection tables of one-call plans (the drop-in
// entry points), kept per thread and grown on demand: a pinned allocation and
// release per call cost more than the set-up of a few hundred reflections.
ReflTable *thread_staging(int64_t n_refl)
{
    struct Staging {
        ReflTable *p = nullptr;
        int64_t cap = 0;
        ~Staging()
        {
            if (p)
                cudaFreeHost(p);
        }
    };
    static thread_local Staging s;
    if (n_refl > s.cap) {
        if (s.p)
            cudaFreeHost(s.p);
        s.p = nullptr;
        s.cap = 0;
        const int64_t cap = std::max<int64_t>(n_refl, 1024);
        if (cudaMallocHost(reinterpret_cast<void **>(&s.p), (size_t)cap * sizeof(ReflTable)) != cudaSuccess) {
            s.p = nullptr;
            return nullptr;
        }
        s.cap = cap;
    }
    return s.p;
}

// A helper thread per calling thread, kept between calls, for the
// reflections' host set-up while the caller drives the device.  The OpenMP
// team the set-up opens belongs to the helper and is reused by the next call
// (a new thread per call opened a new team each time: about a millisecond,
// as long as the whole device work of a few hundred reflections).
class SetupHelper {
public:
    ~SetupHelper()
    {
        if (!owned())
            return;
        {
            std::lock_guard<std::mutex> lk(mu_);
            quit_ = true;
        }
        cv_.notify_all();
        if (th_.joinable())
            th_.join();
    }
    // false when no helper thread can be started (the caller runs f itself)
    bool submit(std::function<int()> f)
    {
        std::lock_guard<std::mutex> lk(mu_);
        owned();
        if (!th_.joinable()) {
            try {
                th_ = std::thread([this] { loop(); });
                pid_ = getpid();
            } catch (...) {
                return false;
            }
        }
        job_ = std::move(f);
        pending_ = true;
        finished_ = false;
        cv_.notify_all();
        return true;
    }
    int wait()
    {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [this] { return finished_; });
        finished_ = false;
        return result_;
    }

private:
    // After fork() a child inherits the handle of a helper that runs only in
    // the parent: the handle is given up (never joined) and a new helper is
    // started on the child's first call.
    bool owned()
    {
        if (th_.joinable() && pid_ != getpid()) {
            new std::thread(std::move(th_));   // left to the parent's process
            return false;
        }
        return true;
    }
    void loop()
    {
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [this] { return pending_ || quit_; });
            if (!pending_)
                return;
            std::function<int()> f = std::move(job_);
            pending_ = false;
            lk.unlock();
            int r;
            try {
                r = f();
            } catch (...) {
                r = kErrNoMem;
            }
            lk.lock();
            result_ = r;
            finished_ = true;
            cv_.notify_all();
        }
    }
    std::thread th_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::function<int()> job_;
    bool pending_ = false, finished_ = false, quit_ = false;
    int result_ = kOk;
    pid_t pid_ = 0;
};

// the tile actually used: at least `tile`, and large enough that a reflection
// has at most kMaxTilesPerRefl tiles (a multiple of 32 voxels)
int effective_tile(int n_vox, int tile)
{
    const long long need = ((long long)n_vox + kMaxTilesPerRefl - 1) / kMaxTilesPerRefl;
    if (need > tile)
        tile = (int)((need + 31) / 32 * 32);
    return tile;
}

// Volume, tables and sizes of a plan (the voxel list comes next).
int plan_init_volume(anacor_plan *p, const int8_t *label, const int64_t *shape, const double *voxel, const double *mu,
                     int full, int is_exp, int order)
{
    if (!label || !shape || !voxel || !mu)
        return fail(kErrArgs, "null argument");
    if (!valid_shape(shape))
        return fail(kErrArgs, "volume axes must lie in [1, 8191] and the volume below 2^31 voxels");
    DeviceState *dev = nullptr;
    if (int st = current_device(&dev))
        return st;
    p->dev = dev;
    p->stream = dev->stream;
    for (int a = 0; a < 3; a++) {
        p->dims[a] = (int)shape[a];
        p->voxel[a] = voxel[a];
    }
    for (int a = 0; a < 4; a++)
        p->mu[a] = mu[a];
    p->full = full;
    p->is_exp = is_exp;
    p->order = order;
    p->tile = kTile;
    cudaStream_t st = p->stream;
    const size_t nvol = (size_t)shape[0] * shape[1] * shape[2];
    cudaError_t e;
    if ((e = dev_alloc(&p->d_vol, nvol, st)) != cudaSuccess || (e = dev_alloc(&p->d_status, 1, st)) ||
        (e = dev_alloc(&p->d_counter, 1, st)) || (e = dev_alloc(&p->d_desc, 1, st)))
        return cuda_fail(e, "device allocation");
    if ((e = cudaMemcpyAsync(p->d_vol, label, nvol, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemsetAsync(p->d_status, 0, sizeof(int), st)))
        return cuda_fail(e, "volume upload");
    // squared axis lengths for cal_path2_plus's total, as the reference
    // computes them: pow((last - first) * voxel, 2) == t * t, t = d * voxel
    p->sq_stride = std::max(p->dims[0], std::max(p->dims[1], p->dims[2]));
    std::vector<double> sq((size_t)3 * p->sq_stride, 0.0);
    for (int a = 0; a < 3; a++)
        for (int d = 0; d < p->dims[a]; d++) {
            const double t = (double)d * voxel[a];
            sq[(size_t)a * p->sq_stride + d] = t * t;
        }
    if ((e = dev_alloc(&p->d_sq, sq.size(), st)) ||
        (e = cudaMemcpyAsync(p->d_sq, sq.data(), sq.size() * sizeof(double), cudaMemcpyHostToDevice, st)) ||
        (e = cudaStreamSynchronize(st)))
        return cuda_fail(e, "table upload");
    p->d_qtab = quotient_table(dev, p->sq_stride);
    return kOk;
}

// The voxel list: the caller's int64 (z, y, x) rows, from host or device
// memory, kept as given (d_c64) and packed for the kernels.
int plan_set_voxels(anacor_plan *p, const int64_t *coords, int64_t n, bool on_device)
{
    if (n < 0 || n >= (1ll << 31))
        return fail(kErrArgs, "coordinate count out of range");
    if (n > 0 && !coords)
        return fail(kErrArgs, "null argument");
    cudaStream_t st = p->stream;
    dev_free(p->d_coords, st);
    dev_free(p->d_c64, st);
    p->n_vox = (int)n;
    p->tile = effective_tile(p->n_vox, p->tile);
    p->tiles = (int)((n + p->tile - 1) / p->tile);
    cudaError_t e;
    if ((e = dev_alloc(&p->d_coords, (size_t)n, st)) || (e = dev_alloc(&p->d_c64, (size_t)n * 3, st)))
        return cuda_fail(e, "device allocation");
    if (n > 0) {
        if ((e = cudaMemcpyAsync(p->d_c64, coords, (size_t)n * 3 * sizeof(long long),
                                 on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st)) ||
            (e = launch_pack_coords_order(p->d_c64, (int)n, p->dims, p->order, p->d_coords, p->d_status, st)) ||
            (e = cudaStreamSynchronize(st)))
            return cuda_fail(e, "coordinate upload");
    }
    return kOk;
}

// `order`: voxel order of the packed list (A_h does not depend on it; Morton
// by default); per-voxel outputs keep the caller's order (0) instead.
int plan_init(anacor_plan *p, const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n,
              const double *voxel, const double *mu, int full, int is_exp, int order = 1)
{
    if (!coords)
        return fail(kErrArgs, "null argument");
    if (n < 0 || n >= (1ll << 31))
        return fail(kErrArgs, "coordinate count out of range");
    if (int st = plan_init_volume(p, label, shape, voxel, mu, full, is_exp, order))
        return st;
    return plan_set_voxels(p, coords, n, false);
}

// Crystal voxels of the plan's volume chosen on the device (method 0: all,
// 1: the reference's 'even' picks, 2: stride lattice) into a fresh device
// int64 [n][3] list (freed by the caller with cudaFreeAsync on the plan stream).
int sample_voxels_device(anacor_plan *p, int code, int method, int64_t sampling_size, double sampling_ratio,
                         int stride, long long **d_out, int64_t *n_out)
{
    cudaStream_t st = p->stream;
    const int lattice = method == 2 ? stride : 1;
    long long *d_count = nullptr, *d_lin = nullptr;
    long long M = 0;
    cudaError_t e;
    if ((e = dev_alloc(&d_count, 1, st)) || (e = count_sampled_voxels(p->d_vol, p->dims, code, lattice, d_count, st)) ||
        (e = cudaMemcpyAsync(&M, d_count, sizeof(long long), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st))) {
        dev_free(d_count, st);
        return cuda_fail(e, "voxel count");
    }
    // the number kept (AnACor/utils/utils_rt.py:55-67)
    long long n = M;
    double step = 0.0;
    if (method == 1) {
        if (sampling_ratio > 0.0)
            n = (long long)((double)M * sampling_ratio / 100.0);
        else
            n = M < sampling_size ? M : M / sampling_size;
        step = n > 0 ? (double)M / (double)n : 0.0;
        if (step == 0.0)
            n = 0;
    }
    long long *d_c = nullptr;
    if ((e = dev_alloc(&d_lin, (size_t)std::max(1ll, M), st)) ||
        (e = select_sampled_voxels(p->d_vol, p->dims, code, lattice, d_lin, d_count, st)) ||
        (e = dev_alloc(&d_c, (size_t)std::max(1ll, n) * 3, st)) ||
        (e = unravel_voxels(d_lin, n, step, p->dims, d_c, st)) || (e = cudaStreamSynchronize(st))) {
        dev_free(d_count, st);
        dev_free(d_lin, st);
        dev_free(d_c, st);
        return cuda_fail(e, "voxel selection");
    }
    dev_free(d_count, st);
    dev_free(d_lin, st);
    *d_out = d_c;
    *n_out = n;
    return kOk;
}

// tile partial sums: one per (reflection, tile) for the reserved reflections
int plan_ensure_partial(anacor_plan *p)
{
    const size_t need = (size_t)p->refl_cap * (size_t)std::max(1, p->tiles);
    if (need <= p->partial_cap)
        return kOk;
    cudaStream_t st = p->stream;
    dev_free(p->d_partial, st);
    p->partial_cap = 0;
    if (cudaError_t e = dev_alloc(&p->d_partial, need, st))
        return cuda_fail(e, "device allocation");
    p->partial_cap = need;
    return kOk;
}

int plan_reserve_refl(anacor_plan *p, int64_t n_refl)
{
    cudaStream_t st = p->stream;
    cudaError_t e;
    if (n_refl > p->refl_cap) {
        dev_free(p->d_refl, st);
        dev_free(p->d_out, st);
        dev_free(p->d_partial, st);
        dev_free(p->d_arrive, st);
        dev_free(p->d_order, st);
        if (p->h_refl && !p->h_refl_borrowed) {
            cudaStreamSynchronize(st);
            cudaFreeHost(p->h_refl);
            p->h_refl = nullptr;
        }
        p->partial_cap = 0;
        if ((e = dev_alloc(&p->d_refl, (size_t)n_refl, st)) || (e = dev_alloc(&p->d_out, (size_t)n_refl, st)) ||
            (e = dev_alloc(&p->d_arrive, (size_t)n_refl, st)) || (e = dev_alloc(&p->d_order, (size_t)n_refl, st)))
            return cuda_fail(e, "device allocation");
        if ((e = cudaMemsetAsync(p->d_arrive, 0, (size_t)n_refl * sizeof(unsigned), st)))
            return cuda_fail(e, "cudaMemset");
        if (!p->h_refl_borrowed &&
            (e = cudaMallocHost(reinterpret_cast<void **>(&p->h_refl), (size_t)n_refl * sizeof(ReflTable))))
            return cuda_fail(e, "pinned allocation");
        p->refl_cap = n_refl;
    }
    p->n_refl = n_refl;
    return plan_ensure_partial(p);
}

// The packed distance field of the plan's volume (variants 5..8), built once.
// The packed distance field(s) of the plan's volume, built once: kind 1 the
// centred field (variants 5..8), kind 2 the 8 octant fields (9..12).
int plan_ensure_field(anacor_plan *p, int kind = 1)
{
    if (kind == 3) {
        // the bricked copy of the octant fields
        if (p->field8b_state == 1)
            return kOk;
        if (p->field8b_state < 0)
            return fail(kErrUnsupported, "bricked fields need fewer than 2^31 bytes per field");
        const size_t per = brick_field_bytes(p->dims);
        if (per >= (size_t)INT32_MAX) {
            p->field8b_state = -1;
            return fail(kErrUnsupported, "bricked fields need fewer than 2^31 bytes per field");
        }
        if (int st = plan_ensure_field(p, 2))
            return st;
        cudaError_t e;
        if ((e = dev_alloc(&p->d_field8b, per * 8, p->stream)) ||
            (e = launch_brick_fields(p->d_field8, p->dims, 8, p->d_field8b, p->stream)) ||
            (e = cudaStreamSynchronize(p->stream))) {
            dev_free(p->d_field8b, p->stream);
            return cuda_fail(e, "bricked fields");
        }
        p->field8b_state = 1;
        return kOk;
    }
    uint8_t *&field = kind == 2 ? p->d_field8 : p->d_field;
    int &state = kind == 2 ? p->field8_state : p->field_state;
    if (state == 1)
        return kOk;
    if (state < 0 || p->field_state < 0 || p->field8_state < 0)
        return fail(kErrUnsupported, "the distance-field march needs labels in 0..7");
    cudaStream_t st = p->stream;
    const size_t nvol = (size_t)p->dims[0] * p->dims[1] * p->dims[2];
    const size_t copies = kind == 2 ? 8 : 1, tmp_copies = kind == 2 ? 6 : 1;
    uint8_t *tmp = nullptr;
    int *d_bad = nullptr;
    int bad = 0;
    cudaError_t e;
    if ((e = dev_alloc(&field, nvol * copies, st)) || (e = dev_alloc(&tmp, nvol * tmp_copies, st)) ||
        (e = dev_alloc(&d_bad, 1, st)) ||
        (e = kind == 2 ? launch_octant_fields(p->d_vol, p->dims, field, tmp, d_bad, st)
                       : launch_distance_field(p->d_vol, p->dims, field, tmp, d_bad, st)) ||
        (e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st))) {
        dev_free(tmp, st);
        dev_free(d_bad, st);
        dev_free(field, st);
        return cuda_fail(e, "distance field");
    }
    dev_free(tmp, st);
    dev_free(d_bad, st);
    if (bad) {
        dev_free(field, st);
        state = -1;
        return fail(kErrUnsupported, "the distance-field march needs labels in 0..7");
    }
    state = 1;
    return kOk;
}

// whether the plan's configured variant marches on a field it has
bool plan_marches_field(const anacor_plan *p)
{
    switch (field_kind(p->variant)) {
    case 1: return p->field_state == 1;
    case 2: return p->field8_state == 1;
    case 3: return p->field8b_state == 1;
    default: return false;
    }
}

// whether that field is the bricked one
bool plan_field_bricked(const anacor_plan *p)
{
    return field_kind(p->variant) == 3 && p->field8b_state == 1;
}

// The plan's sample as a launch descriptor; fk >= 0 names the field it
// marches on (0 none, 1 centred, 2 octant, 3 bricked octant; the field must be
// built), else the field of the plan's own variant.
SampleDesc plan_desc(const anacor_plan *p, long long work_begin, int fk = -1)
{
    SampleDesc d;
    std::memset(&d, 0, sizeof(d));
    d.vol = p->d_vol;
    for (int a = 0; a < 3; a++) {
        d.dim[a] = p->dims[a];
        d.voxel[a] = p->voxel[a];
        d.voxelf[a] = (float)p->voxel[a];
    }
    for (int a = 0; a < 4; a++) {
        d.mu[a] = p->mu[a];
        d.muf[a] = (float)p->mu[a];
    }
    d.n_vox = p->n_vox;
    d.coords = p->d_coords;
    d.refl = p->d_refl;
    d.n_refl = p->n_refl;
    d.tiles = p->tiles;
    d.tile = p->tile;
    d.full_iteration = p->full;
    d.is_exp = p->is_exp;
    d.out = p->d_out;
    d.partial = p->d_partial;
    d.arrive = p->d_arrive;
    d.status = p->d_status;
    d.sq = p->d_sq;
    d.sq_stride = p->sq_stride;
    d.qtab = p->d_qtab;
    d.work_begin = work_begin;
    d.order = p->n_refl > 0 ? p->d_order : nullptr;
    if (fk < 0)
        fk = field_kind(p->variant);
    if (fk == 0) {
        d.field = nullptr;
        d.field_stride = 0;
    } else if (fk == 3) {
        d.field = p->field8b_state == 1 ? p->d_field8b : nullptr;
        d.field_stride = (long long)brick_field_bytes(p->dims);
        brick_strides(p->dims, &d.brick_sy, &d.brick_sz);
    } else if (fk == 2) {
        d.field = p->field8_state == 1 ? p->d_field8 : nullptr;
        d.field_stride = (long long)p->dims[0] * p->dims[1] * p->dims[2];
    } else {
        d.field = p->field_state == 1 ? p->d_field : nullptr;
        d.field_stride = 0;
    }
    return d;
}

int plan_upload_desc(anacor_plan *p, unsigned long long *steps)
{
    cudaError_t e;
    SampleDesc d = plan_desc(p, 0);
    d.steps = steps;
    if ((e = cudaMemcpyAsync(p->d_desc, &d, sizeof(d), cudaMemcpyHostToDevice, p->stream)))
        return cuda_fail(e, "descriptor upload");
    // the descriptor lives on the stack: make sure it has been read
    if ((e = cudaStreamSynchronize(p->stream)))
        return cuda_fail(e, "upload");
    return kOk;
}

// Upload the staged tables, the processing order and the plan's own
// one-sample descriptor.  Reflections are processed grouped by the direction
// octants of their two legs (a stable counting sort on 6 bits), so that the
// work items in flight at one time read the same two of the 8 octant fields
// (and nearby parts of the volume); results stay in the caller's order.
int plan_upload_tables(anacor_plan *p)
{
    cudaError_t e;
    const int64_t n = p->n_refl;
    if (n > 0) {
        int count[65] = {0};
        auto key = [&](int64_t r) { return p->h_refl[r].rule[0][0].octant | p->h_refl[r].rule[1][0].octant << 3; };
        for (int64_t r = 0; r < n; r++)
            count[key(r) + 1]++;
        for (int k = 0; k < 64; k++)
            count[k + 1] += count[k];
        p->h_order.resize((size_t)n);
        for (int64_t r = 0; r < n; r++)
            p->h_order[(size_t)count[key(r)]++] = (int)r;
        if ((e = cudaMemcpyAsync(p->d_refl, p->h_refl, (size_t)n * sizeof(ReflTable), cudaMemcpyHostToDevice,
                                 p->stream)) ||
            (e = cudaMemcpyAsync(p->d_order, p->h_order.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice,
                                 p->stream)))
            return cuda_fail(e, "table upload");
    }
    return plan_upload_desc(p, nullptr);
}

int grid_for(DeviceState *d, int variant, long long items)
{
    const long long cap = (long long)d->sms * variant_occupancy(d, variant);
    return (int)std::max(1ll, std::min(items, cap));
}

int plan_grid(const anacor_plan *p, long long items)
{
    return grid_for(p->dev, p->variant, items);
}

int plan_launch(anacor_plan *p, cudaStream_t st)
{
    const long long items = (long long)p->n_refl * p->tiles;
    if (items == 0)
        return kOk;
    cudaError_t e = launch_absorption(p->d_desc, 1, items, p->d_counter, plan_grid(p, items), st,
                                      kernel_variant(p->variant));
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    return kOk;
}

int plan_fetch(anacor_plan *p, double *out, cudaStream_t st)
{
    int status = 0;
    cudaError_t e;
    if (p->n_refl > 0 && p->n_vox > 0 &&
        (e = cudaMemcpyAsync(out, p->d_out, (size_t)p->n_refl * sizeof(double), cudaMemcpyDeviceToHost, st)))
        return cuda_fail(e, "result download");
    if ((e = cudaMemcpyAsync(&status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st)))
        return cuda_fail(e, "result download");
    if (p->n_vox == 0)
        for (int64_t i = 0; i < p->n_refl; i++)
            out[i] = std::nan("");   // the reference's 0/0 mean
    if (status) {
        for (int b = 1; b < 16; b++)
            if (status & (1 << b))
                return fail(b, status_text(b));
    }
    return succeed();
}

// transient plan: upload, set up, run, fetch (the drop-in entry points)
// the bisection variant (ib_test) over a plan's reflections
int plan_launch_bisection(anacor_plan *p, cudaStream_t st, int num_cls)
{
    const long long items = (long long)p->n_refl * p->tiles;
    if (items == 0)
        return kOk;
    static int bps = 0;
    if (!bps && (bisection_occupancy(&bps) != kOk || bps <= 0))
        bps = 1;
    const int grid = (int)std::max(1ll, std::min(items, (long long)p->dev->sms * bps));
    cudaError_t e = launch_bisection(p->d_desc, 1, items, p->d_counter, grid, num_cls, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "kernel launch");
    return kOk;
}

int plan_default_config(anacor_plan *p);

int run_once(const int8_t *flat, const int64_t *shape, const int64_t *coords, int64_t n, const double *voxel,
             const double *mu, int full, int is_exp, const double *s1, const double *omega, int64_t n_refl,
             const double *xray, const double *axis, const double *F, const ReflTable *tables, int threads,
             double *out, int ib_cls = 0)
{
    // the tables go through this thread's pinned staging (no pinned
    // allocation per call); the plan lives for this call only
    ReflTable *staged = n_refl > 0 ? thread_staging(n_refl) : nullptr;
    // The reflections' host set-up (FP64 rotation, angles, face rules) does
    // not depend on the device: it runs on this thread's helper while this
    // one uploads the volume and voxels and builds the march's fields.
    static thread_local SetupHelper helper;
    const bool on_helper = staged && !tables && helper.submit([=] {
        return setup_reflections(axis, omega, F, xray, s1, n_refl, staged, threads);
    });
    // A volume in pageable memory is page-locked for the upload (about 0.2 ms
    // per 100 MB; the copy then runs at the DMA rate, 0.5 ms, where a copy
    // from pageable memory took 1.5-3.8 ms) and released once it has landed.
    // One call at a time does this, so that no concurrent call sees a buffer
    // pinned only for the moment.
    static std::mutex register_mu;
    std::unique_lock<std::mutex> reg_lock(register_mu, std::defer_lock);
    bool registered = false;
    if (flat && shape && valid_shape(shape)) {
        const size_t nvol = (size_t)shape[0] * shape[1] * shape[2];
        if (nvol >= (4u << 20)) {
            reg_lock.lock();
            if (!host_pinned(flat)) {
                registered =
                    cudaHostRegister(const_cast<int8_t *>(flat), nvol, cudaHostRegisterDefault) == cudaSuccess;
                if (!registered)
                    cudaGetLastError();   // the plain copy serves
            }
        }
    }
    anacor_plan p;
    int st = plan_init(&p, flat, shape, coords, n, voxel, mu, full, is_exp);
    if (registered) {
        // plan_init synchronised its stream: the volume is on the device
        cudaStreamSynchronize(p.stream);
        cudaHostUnregister(const_cast<int8_t *>(flat));
        cudaGetLastError();
    }
    if (reg_lock.owns_lock())
        reg_lock.unlock();
    if (!st) {
        p.h_refl = staged;
        p.h_refl_borrowed = staged != nullptr;
        st = plan_reserve_refl(&p, n_refl);
    }
    if (!st && !ib_cls)
        st = plan_default_config(&p);
    // joined on every path (or run here when no second thread was started)
    const int setup_st = on_helper ? helper.wait()
                         : (staged && !tables) ? setup_reflections(axis, omega, F, xray, s1, n_refl, staged, threads)
                                               : kOk;
    if (!st) {
        if (tables)
            std::memcpy(p.h_refl, tables, (size_t)n_refl * sizeof(ReflTable));
        else if (n_refl > 0 &&
                 (st = staged ? setup_st : setup_reflections(axis, omega, F, xray, s1, n_refl, p.h_refl, threads)))
            fail(st, status_text(st));
    }
    if (!st)
        st = plan_upload_tables(&p);
    if (!st)
        st = ib_cls ? plan_launch_bisection(&p, p.stream, ib_cls) : plan_launch(&p, p.stream);
    if (!st)
        st = plan_fetch(&p, out, p.stream);
    const int keep = t_status;
    const std::string msg = t_msg;
    plan_release(&p);
    t_status = keep;
    t_msg = msg;
    return st;
}


int plan_configure(anacor_plan *p, int variant, int tile, int order)
{
    if (variant < 0 || variant > kPlanVariants || (tile != 0 && (tile < kMinTile || tile > (1 << 22))) ||
        order < -1 || order >= kVoxelOrders)
        return fail(kErrArgs, "bad plan configuration");
    if (variant > 4)
        if (int st = plan_ensure_field(p, field_kind(variant)))
            return st;
    cudaError_t e;
    if (order >= 0 && order != p->order && p->n_vox > 0) {
        e = launch_pack_coords_order(p->d_c64, p->n_vox, p->dims, order, p->d_coords, p->d_status, p->stream);
        if (e)
            return cuda_fail(e, "voxel list packing");
    }
    if (order >= 0)
        p->order = order;
    if (tile) {
        p->tile = effective_tile(p->n_vox, tile);
        p->tiles = (int)(((long long)p->n_vox + p->tile - 1) / p->tile);
        if (int st = plan_ensure_partial(p))
            return st;
    }
    p->variant = variant;
    return plan_upload_desc(p, nullptr);
}

// Time `reps` launches over the first k reflections of the plan (ms each).
int plan_time(anacor_plan *p, int64_t k, int reps, float *ms)
{
    const int64_t keep = p->n_refl;
    cudaError_t e = cudaSuccess;
    // the sample: k reflections spread evenly over the processing order (so
    // every octant pair and the whole range of directions is in it), not the
    // first k, which all share one pair of direction octants
    const bool spread = k < keep && p->h_order.size() >= (size_t)keep;
    if (spread) {
        std::vector<int> sub((size_t)k);
        for (int64_t j = 0; j < k; j++)
            sub[(size_t)j] = p->h_order[(size_t)((j * keep) / k)];
        if ((e = cudaMemcpyAsync(p->d_order, sub.data(), (size_t)k * sizeof(int), cudaMemcpyHostToDevice,
                                 p->stream)) ||
            (e = cudaStreamSynchronize(p->stream)))
            return cuda_fail(e, "tuning sample");
    }
    p->n_refl = k;
    int st = plan_upload_desc(p, nullptr);
    cudaEvent_t a = nullptr, b = nullptr;
    if (!st && ((e = cudaEventCreate(&a)) || (e = cudaEventCreate(&b))))
        st = cuda_fail(e, "event");
    if (!st)
        st = plan_launch(p, p->stream);   // warm-up
    if (!st && (e = cudaEventRecord(a, p->stream)))
        st = cuda_fail(e, "event");
    for (int r = 0; !st && r < reps; r++)
        st = plan_launch(p, p->stream);
    if (!st && ((e = cudaEventRecord(b, p->stream)) || (e = cudaEventSynchronize(b)) ||
                (e = cudaEventElapsedTime(ms, a, b))))
        st = cuda_fail(e, "timing");
    if (ms && !st)
        *ms /= (float)reps;
    if (a)
        cudaEventDestroy(a);
    if (b)
        cudaEventDestroy(b);
    p->n_refl = keep;
    if (spread && ((e = cudaMemcpyAsync(p->d_order, p->h_order.data(), (size_t)k * sizeof(int),
                                        cudaMemcpyHostToDevice, p->stream)) ||
                   (e = cudaStreamSynchronize(p->stream))))
        return st ? st : cuda_fail(e, "processing order");
    const int st2 = plan_upload_desc(p, nullptr);
    return st ? st : st2;
}

struct TuneKey {
    int d0, d1, d2, nbucket;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(d0, d1, d2, nbucket) < std::tie(o.d0, o.d1, o.d2, o.nbucket);
    }
};
struct TuneVal {
    int variant, tile, order;
    float ms;
};
std::map<TuneKey, TuneVal> g_tune_cache;

TuneKey tune_key(const anacor_plan *p)
{
    int nb = 0;
    while ((1 << nb) < p->n_vox)
        nb++;
    return TuneKey{p->dims[0], p->dims[1], p->dims[2], nb};
}

bool tune_lookup(const anacor_plan *p, TuneVal &v)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_tune_cache.find(tune_key(p));
    if (it == g_tune_cache.end())
        return false;
    v = it->second;
    return true;
}

// Configuration of a plan run without autotuning (the drop-in entry points):
// the process's tuned choice for this volume class when there is one; else
// the distance-field march for volumes with an axis of 256 voxels or more
// (long legs: it steps over most increments; 25-50 % faster there, while the
// cooperative march is as fast on a 96^3 volume) and the cooperative march
// below that, with the largest tile up to 1024 voxels that still gives every
// warp four work items.
int plan_default_config(anacor_plan *p)
{
    TuneVal v{0, 0, 1, 0.0f};
    if (tune_lookup(p, v) && (v.variant <= 4 || plan_ensure_field(p, field_kind(v.variant)) == kOk))
        return plan_configure(p, v.variant, v.tile, v.order);
    int variant = 0;
    const int big = std::max(p->dims[0], std::max(p->dims[1], p->dims[2]));
    if (!std::getenv("ANACOR_CTAS_PER_SM") && big >= 256) {
        // the octant fields march 15-25 % faster than the centred field and
        // take no longer to build (1.3 vs 1.5 ms on 512x512x400)
        if (plan_ensure_field(p, 2) == kOk)
            variant = 12;
        succeed();   // labels outside 0..7: the cooperative march, no error
    }
    // the largest tile that still gives every warp slot four items
    const long long warps = (long long)p->dev->sms * 32;
    int tile = kMinTile;
    for (int t : {2048, 1024, 512, 256})
        if (p->n_refl * (((long long)p->n_vox + t - 1) / t) >= 4 * warps) {
            tile = t;
            break;
        }
    return plan_configure(p, variant, tile, -1);
}

}  // namespace

// A batch: several plans run by one persistent launch, optionally replayed
// from a captured CUDA graph.
struct anacor_batch {
    std::vector<anacor_plan *> plans;
    SampleDesc *d_descs = nullptr;        // every sample; the cooperative group first
    unsigned long long *d_counter = nullptr;
    long long items = 0;
    int variant = 0;
    int grid = 0;
    // With a distance-field variant (5..8) the samples whose own plan marches
    // on its field run in a second launch (d_descs_field, numbered from 0)
    // and the others in a first, cooperative one with the same register budget.
    SampleDesc *d_descs_field = nullptr;
    unsigned long long *d_counter_field = nullptr;
    int n_coop = 0, n_field = 0;
    long long items_coop = 0, items_field = 0;
    int grid_coop = 0, grid_field = 0;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// The batch's samples as descriptors.  Under a field variant every sample
// marches on its field of that kind (built here if needed), so the batch is
// one launch; a sample whose labels allow no field (outside 0..7) runs in a
// first, cooperative launch of the same register budget.
int batch_upload(anacor_batch *b)
{
    std::vector<anacor_plan *> coop, field;
    const int fk = field_kind(b->variant);
    for (anacor_plan *p : b->plans) {
        if (fk > 0) {
            const int st = plan_ensure_field(p, fk);
            if (st == kOk) {
                field.push_back(p);
                continue;
            }
            if (st != kErrUnsupported)
                return st;
            succeed();   // no field for these labels: the cooperative group
        }
        coop.push_back(p);
    }
    std::vector<SampleDesc> descs, descs_field;
    long long total = 0, items_coop = 0;
    for (anacor_plan *p : coop) {
        descs.push_back(plan_desc(p, total, 0));
        total += (long long)p->n_refl * p->tiles;
    }
    items_coop = total;
    long long rebased = 0;
    for (anacor_plan *p : field) {
        descs.push_back(plan_desc(p, total, fk));
        descs_field.push_back(plan_desc(p, rebased, fk));
        const long long n = (long long)p->n_refl * p->tiles;
        total += n;
        rebased += n;
    }
    DeviceState *dev = b->plans[0]->dev;
    b->items = total;
    const int cv = b->variant > 4 ? budget_of(b->variant) : b->variant;   // cooperative kernel
    b->grid = total ? grid_for(dev, cv, total) : 0;
    b->n_coop = (int)coop.size();
    b->n_field = (int)field.size();
    b->items_coop = items_coop;
    b->items_field = rebased;
    b->grid_coop = items_coop ? grid_for(dev, cv, items_coop) : 0;
    b->grid_field = rebased ? grid_for(dev, b->variant, rebased) : 0;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b->d_descs, descs.data(), sizeof(SampleDesc) * descs.size(), cudaMemcpyHostToDevice,
                             b->stream)) ||
        (!descs_field.empty() &&
         (e = cudaMemcpyAsync(b->d_descs_field, descs_field.data(), sizeof(SampleDesc) * descs_field.size(),
                              cudaMemcpyHostToDevice, b->stream))) ||
        (e = cudaStreamSynchronize(b->stream)))
        return cuda_fail(e, "descriptor upload");
    // a captured graph holds the old grid: drop it
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    return kOk;
}

// The batch's kernel launches on `st`: one over every sample, or (a
// distance-field variant) the cooperative group then the field group.
cudaError_t batch_enqueue(anacor_batch *b, cudaStream_t st)
{
    if (b->items <= 0)
        return cudaSuccess;
    const int cv = b->variant > 4 ? budget_of(b->variant) : b->variant;
    if (b->variant <= 4 || b->n_field == 0)
        return launch_absorption(b->d_descs, (int)b->plans.size(), b->items, b->d_counter, b->grid, st, cv);
    cudaError_t e = cudaSuccess;
    if (b->items_coop > 0)
        e = launch_absorption(b->d_descs, b->n_coop, b->items_coop, b->d_counter, b->grid_coop, st, cv);
    if (e == cudaSuccess && b->items_field > 0)
        e = launch_absorption(b->d_descs_field, b->n_field, b->items_field, b->d_counter_field, b->grid_field, st,
                              kernel_variant(b->variant));
    return e;
}

int batch_kernels(const anacor_batch *b)
{
    if (b->items <= 0)
        return 0;
    if (b->variant <= 4 || b->n_field == 0)
        return 1;
    return (b->items_coop > 0) + (b->items_field > 0);
}

int batch_check(anacor_batch *b, cudaStream_t st)
{
    cudaError_t e;
    for (anacor_plan *p : b->plans) {
        int status = 0;
        if ((e = cudaMemcpyAsync(&status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaStreamSynchronize(st)))
            return cuda_fail(e, "status");
        for (int bit = 1; bit < 16; bit++)
            if (status & (1 << bit))
                return fail(bit, status_text(bit));
    }
    return succeed();
}

}  // namespace

namespace anacor {
int plan_view_field(anacor_plan *p, PlanView *v)
{
    if (int st = plan_view(p, v))
        return st;
    if (plan_ensure_field(p, 2) == kOk) {
        v->field = p->d_field8;
        v->field_stride = (long long)p->dims[0] * p->dims[1] * p->dims[2];
    } else {
        succeed();   // labels outside 0..7: the cooperative march
    }
    return kOk;
}

int plan_view(const anacor_plan *p, PlanView *v)
{
    if (!p || !v)
        return fail(kErrArgs, "null plan");
    std::memset(v, 0, sizeof(*v));
    v->vol = p->d_vol;
    for (int a = 0; a < 3; a++) {
        v->dims[a] = p->dims[a];
        v->voxel[a] = p->voxel[a];
    }
    for (int a = 0; a < 4; a++)
        v->mu[a] = p->mu[a];
    v->n_vox = p->n_vox;
    v->coords = p->d_coords;
    v->c64 = p->d_c64;
    v->order = p->order;
    v->full_iteration = p->full;
    v->is_exp = p->is_exp;
    v->sq = p->d_sq;
    v->sq_stride = p->sq_stride;
    v->qtab = p->d_qtab;
    v->stream = p->stream;
    v->sms = p->dev ? p->dev->sms : 0;
    return kOk;
}
}  // namespace anacor

extern "C" {

int anacor_last_status(void) { return t_status; }
const char *anacor_last_error(void) { return t_msg.c_str(); }
const char *anacor_version(void) { return "anacor_gb300 1.0 (sm_103a)"; }

anacor_plan *anacor_plan_create(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n,
                                const double *voxel, const double *mu, int full_iteration, int is_exp)
{
    anacor_plan *p = new (std::nothrow) anacor_plan();
    if (!p) {
        fail(kErrNoMem, "out of host memory");
        return nullptr;
    }
    if (plan_init(p, label, shape, coords, n, voxel, mu, full_iteration, is_exp)) {
        const int keep = t_status;
        const std::string msg = t_msg;
        if (p->stream)
            plan_release(p);
        delete p;
        t_status = keep;
        t_msg = msg;
        return nullptr;
    }
    cudaError_t e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        cuda_fail(e, "plan upload");
        plan_release(p);
        delete p;
        return nullptr;
    }
    succeed();
    return p;
}

anacor_plan *anacor_plan_create_sampled(const int8_t *label, const int64_t *shape, int crystal_code, int method,
                                        int64_t sampling_size, double sampling_ratio, int stride, const double *voxel,
                                        const double *mu, int full_iteration, int is_exp)
{
    if (method < 0 || method > 2 || (method == 1 && sampling_size <= 0 && !(sampling_ratio > 0.0)) ||
        (method == 2 && stride < 1)) {
        fail(kErrArgs, "sampling: method 0 (all), 1 (even: sampling_size > 0 or ratio > 0) or 2 (stride >= 1)");
        return nullptr;
    }
    anacor_plan *p = new (std::nothrow) anacor_plan();
    if (!p) {
        fail(kErrNoMem, "out of host memory");
        return nullptr;
    }
    long long *d_c = nullptr;
    int64_t n = 0;
    int st = plan_init_volume(p, label, shape, voxel, mu, full_iteration, is_exp, 1);
    if (!st)
        st = sample_voxels_device(p, crystal_code, method, sampling_size, sampling_ratio, stride, &d_c, &n);
    if (!st)
        st = plan_set_voxels(p, reinterpret_cast<const int64_t *>(d_c), n, true);
    if (d_c)
        dev_free(d_c, p->stream);
    if (st) {
        const int keep = t_status;
        const std::string msg = t_msg;
        if (p->stream)
            plan_release(p);
        delete p;
        t_status = keep;
        t_msg = msg;
        return nullptr;
    }
    succeed();
    return p;
}

int64_t anacor_plan_n_voxels(const anacor_plan *p) { return p ? p->n_vox : 0; }

int anacor_plan_voxels(const anacor_plan *p, int64_t *coords_out)
{
    if (!p || !coords_out)
        return fail(kErrArgs, "bad arguments");
    cudaError_t e;
    if (p->n_vox > 0 && ((e = cudaMemcpyAsync(coords_out, p->d_c64, (size_t)p->n_vox * 3 * sizeof(long long),
                                              cudaMemcpyDeviceToHost, p->stream)) ||
                         (e = cudaStreamSynchronize(p->stream))))
        return cuda_fail(e, "voxel download");
    return succeed();
}

int anacor_sample_voxels(const int8_t *label, const int64_t *shape, int crystal_code, int method,
                         int64_t sampling_size, double sampling_ratio, int stride, int64_t *coords_out,
                         int64_t capacity, int64_t *n_out)
{
    if (!n_out)
        return fail(kErrArgs, "null argument");
    const double vox[3] = {1.0, 1.0, 1.0}, mu[4] = {0.0, 0.0, 0.0, 0.0};
    anacor_plan *p = anacor_plan_create_sampled(label, shape, crystal_code, method, sampling_size, sampling_ratio,
                                                stride, vox, mu, 0, 1);
    if (!p)
        return t_status;
    *n_out = p->n_vox;
    int st = kOk;
    if (p->n_vox > capacity || (p->n_vox > 0 && !coords_out))
        st = fail(kErrArgs, "sampling: the output holds fewer rows than were selected (n_out has the count)");
    else
        st = anacor_plan_voxels(p, coords_out);
    const int keep = t_status;
    const std::string msg = t_msg;
    plan_release(p);
    delete p;
    t_status = keep;
    t_msg = msg;
    return st;
}

int anacor_plan_set_reflections(anacor_plan *p, const double *s1, const double *omega, int64_t n_refl,
                                const double *xray, const double *omega_axis, const double *F)
{
    if (!p || n_refl < 0 || (n_refl > 0 && (!s1 || !omega || !xray || !omega_axis || !F)))
        return fail(kErrArgs, "bad arguments");
    if (int st = plan_reserve_refl(p, n_refl))
        return st;
    if (n_refl > 0) {
        if (int st = setup_reflections(omega_axis, omega, F, xray, s1, n_refl, p->h_refl, 0))
            return fail(st, status_text(st));
    }
    if (int st = plan_upload_tables(p))
        return st;
    return succeed();
}

int anacor_plan_run(anacor_plan *p, void *stream)
{
    if (!p)
        return fail(kErrArgs, "null plan");
    cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
    if (int s = plan_launch(p, st))
        return s;
    return succeed();
}

int anacor_plan_run_bisection(anacor_plan *p, int num_cls, void *stream)
{
    if (!p || num_cls < 1)
        return fail(kErrArgs, "bad arguments");
    cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
    if (int s = plan_launch_bisection(p, st, num_cls))
        return s;
    return succeed();
}

int anacor_bisection(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n_coords,
                     const double *s1, const double *omega, int64_t n_refl, const double *xray,
                     const double *omega_axis, const double *F, const double *voxel, const double *mu, int num_cls,
                     double *out)
{
    if (n_refl < 0 || (n_refl > 0 && (!s1 || !omega || !xray || !omega_axis || !F || !out)) || num_cls < 1)
        return fail(kErrArgs, "bad arguments");
    return run_once(label, shape, coords, n_coords, voxel, mu, 0, 1, s1, omega, n_refl, xray, omega_axis, F,
                    nullptr, 0, out, num_cls);
}

int anacor_plan_result(anacor_plan *p, double *out, void *stream)
{
    if (!p || (!out && p->n_refl > 0))
        return fail(kErrArgs, "bad arguments");
    return plan_fetch(p, out, stream ? (cudaStream_t)stream : p->stream);
}

int anacor_plan_count_steps(anacor_plan *p, uint64_t *total)
{
    if (!p || !total)
        return fail(kErrArgs, "bad arguments");
    cudaError_t e;
    if (!p->d_steps && (e = dev_alloc(&p->d_steps, 1, p->stream)))
        return cuda_fail(e, "device allocation");
    if ((e = cudaMemsetAsync(p->d_steps, 0, sizeof(unsigned long long), p->stream)))
        return cuda_fail(e, "cudaMemset");
    if (int st = plan_upload_desc(p, p->d_steps))
        return st;
    int st = plan_launch(p, p->stream);
    unsigned long long h = 0;
    if (!st && (e = cudaMemcpyAsync(&h, p->d_steps, sizeof(h), cudaMemcpyDeviceToHost, p->stream)))
        st = cuda_fail(e, "download");
    if (!st && (e = cudaStreamSynchronize(p->stream)))
        st = cuda_fail(e, "count");
    if (int s2 = plan_upload_desc(p, nullptr))
        return s2;
    if (st)
        return st;
    *total = h;
    return succeed();
}

namespace {
int distance_fields(const int8_t *label, const int64_t *shape, uint8_t *out, bool octants)
{
    if (!label || !shape || !out)
        return fail(kErrArgs, "null argument");
    if (!valid_shape(shape))
        return fail(kErrArgs, "volume axes must lie in [1, 8191] and the volume below 2^31 voxels");
    DeviceState *dev = nullptr;
    if (int st = current_device(&dev))
        return st;
    cudaStream_t st = dev->stream;
    const int dims[3] = {(int)shape[0], (int)shape[1], (int)shape[2]};
    const size_t nvol = (size_t)shape[0] * shape[1] * shape[2];
    int8_t *d_vol = nullptr;
    uint8_t *d_out = nullptr, *d_tmp = nullptr;
    int *d_bad = nullptr;
    int bad = 0;
    cudaError_t e;
    if (!(e = dev_alloc(&d_vol, nvol, st)) && !(e = dev_alloc(&d_out, nvol * (octants ? 8 : 1), st)) &&
        !(e = dev_alloc(&d_tmp, nvol * (octants ? 6 : 1), st)) &&
        !(e = dev_alloc(&d_bad, 1, st)) &&
        !(e = cudaMemcpyAsync(d_vol, label, nvol, cudaMemcpyHostToDevice, st)) &&
        !(e = octants ? launch_octant_fields(d_vol, dims, d_out, d_tmp, d_bad, st)
                   : launch_distance_field(d_vol, dims, d_out, d_tmp, d_bad, st)) &&
        !(e = cudaMemcpyAsync(out, d_out, nvol * (octants ? 8 : 1), cudaMemcpyDeviceToHost, st)) &&
        !(e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st)))
        e = cudaStreamSynchronize(st);
    dev_free(d_vol, st);
    dev_free(d_out, st);
    dev_free(d_tmp, st);
    dev_free(d_bad, st);
    if (e)
        return cuda_fail(e, "distance field");
    if (bad)
        return fail(kErrUnsupported, "the distance field needs labels in 0..7");
    return succeed();
}
}  // namespace

int anacor_distance_field(const int8_t *label, const int64_t *shape, uint8_t *out)
{
    return distance_fields(label, shape, out, false);
}

int anacor_octant_fields(const int8_t *label, const int64_t *shape, uint8_t *out)
{
    return distance_fields(label, shape, out, true);
}

const double *anacor_plan_device_result(anacor_plan *p) { return p ? p->d_out : nullptr; }
int64_t anacor_plan_n_refl(const anacor_plan *p) { return p ? p->n_refl : 0; }

int anacor_plan_launch_info(const anacor_plan *p, int *grid, int *kernels)
{
    if (!p)
        return fail(kErrArgs, "null plan");
    const long long items = (long long)p->n_refl * p->tiles;
    if (grid)
        *grid = items ? plan_grid(p, items) : 0;
    if (kernels)
        *kernels = items ? 1 : 0;
    return succeed();
}

void anacor_plan_destroy(anacor_plan *p)
{
    if (!p)
        return;
    plan_release(p);
    delete p;
}

int anacor_batch_run(anacor_plan *const *plans, int n_plans, void *stream)
{
    if (!plans || n_plans <= 0)
        return fail(kErrArgs, "empty batch");
    anacor_plan *p0 = plans[0];
    cudaStream_t st = stream ? (cudaStream_t)stream : p0->stream;
    std::vector<SampleDesc> descs;
    long long total = 0;
    for (int i = 0; i < n_plans; i++) {
        if (!plans[i])
            return fail(kErrArgs, "null plan in batch");
        descs.push_back(plan_desc(plans[i], total));
        total += (long long)plans[i]->n_refl * plans[i]->tiles;
    }
    // batch descriptors live in a device buffer owned by the first plan's device state
    static thread_local SampleDesc *d_descs = nullptr;
    static thread_local int d_cap = 0;
    cudaError_t e;
    if (n_plans > d_cap) {
        if (d_descs)
            cudaFree(d_descs);
        if ((e = cudaMalloc(&d_descs, sizeof(SampleDesc) * (size_t)n_plans)))
            return cuda_fail(e, "device allocation");
        d_cap = n_plans;
    }
    if ((e = cudaMemcpyAsync(d_descs, descs.data(), sizeof(SampleDesc) * descs.size(), cudaMemcpyHostToDevice, st)))
        return cuda_fail(e, "descriptor upload");
    if (total > 0) {
        // one launch: the field march only when every sample marches on a field
        int variant = kernel_variant(p0->variant);
        for (int i = 0; i < n_plans && variant > 4; i++)
            if (!plan_marches_field(plans[i]) || plan_field_bricked(plans[i]) != plan_field_bricked(p0))
                variant = budget_of(p0->variant);
        const int grid = grid_for(p0->dev, variant, total);
        if ((e = launch_absorption(d_descs, n_plans, total, p0->d_counter, grid, st, variant)))
            return cuda_fail(e, "kernel launch");
    }
    if ((e = cudaStreamSynchronize(st)))
        return cuda_fail(e, "batch");
    return succeed();
}

int anacor_absorption(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n_coords,
                      const double *s1, const double *omega, int64_t n_refl, const double *xray,
                      const double *omega_axis, const double *F, const double *voxel, const double *mu,
                      int full_iteration, int is_exp, double *out)
{
    if (n_refl < 0 || (n_refl > 0 && (!s1 || !omega || !xray || !omega_axis || !F || !out)))
        return fail(kErrArgs, "bad arguments");
    return run_once(label, shape, coords, n_coords, voxel, mu, full_iteration, is_exp, s1, omega, n_refl, xray,
                    omega_axis, F, nullptr, 0, out);
}

double *ray_tracing_overall(int64_t low, int64_t up, int64_t *coord_list, int64_t len_coord_list,
                            const double *scattering_vector_list, const double *omega_list,
                            const double *raw_xray, const double *omega_axis, const double *kp_rotation_matrix,
                            int64_t len_result, double *voxel_size, double *coefficients, int8_t ***label_list,
                            int64_t *shape, int full_iteration, int store_paths, int num_workers, int IsExp)
{
    (void)low; (void)up; (void)store_paths;
    if (!shape || !valid_shape(shape)) {
        fail(kErrArgs, "volume axes must lie in [1, 8191] and the volume below 2^31 voxels");
        return nullptr;
    }
    if (len_result < 0 || !scattering_vector_list || !omega_list || !raw_xray || !omega_axis ||
        !kp_rotation_matrix || !voxel_size || !coefficients || !coord_list) {
        fail(kErrArgs, "bad arguments");
        return nullptr;
    }
    std::vector<int8_t> gathered;
    const int8_t *flat = flat_base(label_list, shape);
    if (!flat) {
        if (!label_list) {
            fail(kErrArgs, "null label table");
            return nullptr;
        }
        // rows are not one strided block: gather them
        gathered.resize((size_t)shape[0] * shape[1] * shape[2]);
        for (int64_t z = 0; z < shape[0]; z++)
            for (int64_t y = 0; y < shape[1]; y++)
                std::memcpy(&gathered[(z * shape[1] + y) * shape[2]], label_list[z][y], (size_t)shape[2]);
        flat = gathered.data();
    }
    double *result = static_cast<double *>(std::malloc((size_t)std::max<int64_t>(len_result, 1) * sizeof(double)));
    if (!result) {
        fail(kErrNoMem, "out of host memory");
        return nullptr;
    }
    const int is_exp = (signed char)IsExp == 1;   // the reference passes it on as char
    if (run_once(flat, shape, coord_list, len_coord_list, voxel_size, coefficients, full_iteration, is_exp,
                 scattering_vector_list, omega_list, len_result, raw_xray, omega_axis, kp_rotation_matrix, nullptr,
                 num_workers, result)) {
        std::free(result);
        return nullptr;
    }
    return result;
}

double ray_tracing_single(int64_t *coord_list, int64_t len_coord_list, const double *rotated_s1,
                          const double *xray, double *voxel_size, double *coefficients, int8_t ***label_list,
                          int64_t *shape, int full_iteration, int64_t store_paths, int IsExp)
{
    (void)store_paths;
    const double nan = std::nan("");
    if (!shape || !valid_shape(shape) || !rotated_s1 || !xray || !voxel_size || !coefficients || !coord_list) {
        fail(kErrArgs, "bad arguments");
        return nan;
    }
    std::vector<int8_t> gathered;
    const int8_t *flat = flat_base(label_list, shape);
    if (!flat) {
        if (!label_list) {
            fail(kErrArgs, "null label table");
            return nan;
        }
        gathered.resize((size_t)shape[0] * shape[1] * shape[2]);
        for (int64_t z = 0; z < shape[0]; z++)
            for (int64_t y = 0; y < shape[1]; y++)
                std::memcpy(&gathered[(z * shape[1] + y) * shape[2]], label_list[z][y], (size_t)shape[2]);
        flat = gathered.data();
    }
    ReflTable tab;
    if (int st = setup_rotated(xray, rotated_s1, &tab)) {
        fail(st, status_text(st));
        return nan;
    }
    double out = nan;
    const int is_exp = (signed char)IsExp == 1;
    if (run_once(flat, shape, coord_list, len_coord_list, voxel_size, coefficients, full_iteration, is_exp, nullptr,
                 nullptr, 1, nullptr, nullptr, nullptr, &tab, 0, &out))
        return nan;
    return out;
}

double ib_test(int64_t *coord_list, int64_t len_coord_list, double *rotated_s1, double *xray, double *voxel_size,
               double *coefficients, int8_t ***label_list, int64_t *shape, int full_iteration, int64_t store_paths,
               int num_cls)
{
    (void)full_iteration;
    (void)store_paths;
    const double nan = std::nan("");
    if (!shape || !valid_shape(shape) || !rotated_s1 || !xray || !voxel_size || !coefficients || !coord_list ||
        len_coord_list <= 0) {
        fail(kErrArgs, "bad arguments");
        return nan;
    }
    std::vector<int8_t> gathered;
    const int8_t *flat = flat_base(label_list, shape);
    if (!flat) {
        if (!label_list) {
            fail(kErrArgs, "null label table");
            return nan;
        }
        gathered.resize((size_t)shape[0] * shape[1] * shape[2]);
        for (int64_t z = 0; z < shape[0]; z++)
            for (int64_t y = 0; y < shape[1]; y++)
                std::memcpy(&gathered[(z * shape[1] + y) * shape[2]], label_list[z][y], (size_t)shape[2]);
        flat = gathered.data();
    }
    ReflTable tab;
    if (int st = setup_rotated(xray, rotated_s1, &tab)) {
        fail(st, status_text(st));
        return nan;
    }
    double out = nan;
    if (run_once(flat, shape, coord_list, len_coord_list, voxel_size, coefficients, 0, 1, nullptr, nullptr, 1,
                 nullptr, nullptr, nullptr, &tab, 0, &out, std::max(1, num_cls)))
        return nan;
    return out;
}

float *ray_tracing_gpu_overall(size_t low, size_t up, int *coord_list, size_t len_coord_list,
                               const float *scattering_vector_list, const float *omega_list, const float *raw_xray,
                               const float *omega_axis, const float *kp_rotation_matrix, size_t len_result,
                               float *voxel_size, float *coefficients, int8_t ***label_list, int8_t *label_list_1d,
                               int *shape, int full_iteration, int store_paths, int gpumethod)
{
    (void)gpumethod;
    if (!shape || !coord_list || !scattering_vector_list || !omega_list || !raw_xray || !omega_axis ||
        !kp_rotation_matrix || !voxel_size || !coefficients) {
        fail(kErrArgs, "bad arguments");
        return nullptr;
    }
    int64_t shp[3] = {shape[0], shape[1], shape[2]};
    if (!valid_shape(shp)) {
        fail(kErrArgs, "volume axes must lie in [1, 8191] and the volume below 2^31 voxels");
        return nullptr;
    }
    std::vector<int64_t> c((size_t)len_coord_list * 3);
    for (size_t i = 0; i < c.size(); i++)
        c[i] = coord_list[i];
    std::vector<double> s1(len_result * 3), om(len_result);
    for (size_t i = 0; i < len_result * 3; i++)
        s1[i] = scattering_vector_list[i];
    for (size_t i = 0; i < len_result; i++)
        om[i] = omega_list[i];
    double xr[3], ax[3], F[9], vox[3], mu[4];
    for (int a = 0; a < 3; a++) {
        xr[a] = raw_xray[a];
        ax[a] = omega_axis[a];
        vox[a] = voxel_size[a];
    }
    for (int a = 0; a < 9; a++)
        F[a] = kp_rotation_matrix[a];
    for (int a = 0; a < 4; a++)
        mu[a] = coefficients[a];
    std::vector<int8_t> gathered;
    const int8_t *flat = label_list_1d ? label_list_1d : flat_base(label_list, shp);
    if (!flat) {
        if (!label_list) {
            fail(kErrArgs, "null label table");
            return nullptr;
        }
        gathered.resize((size_t)shp[0] * shp[1] * shp[2]);
        for (int64_t z = 0; z < shp[0]; z++)
            for (int64_t y = 0; y < shp[1]; y++)
                std::memcpy(&gathered[(z * shp[1] + y) * shp[2]], label_list[z][y], (size_t)shp[2]);
        flat = gathered.data();
    }
    std::vector<double> res(std::max<size_t>(len_result, 1));
    (void)low; (void)up; (void)store_paths;
    if (run_once(flat, shp, c.data(), (int64_t)len_coord_list, vox, mu, full_iteration, 1, s1.data(), om.data(),
                 (int64_t)len_result, xr, ax, F, nullptr, 0, res.data()))
        return nullptr;
    float *out = static_cast<float *>(std::malloc(std::max<size_t>(len_result, 1) * sizeof(float)));
    if (!out) {
        fail(kErrNoMem, "out of host memory");
        return nullptr;
    }
    for (size_t i = 0; i < len_result; i++)
        out[i] = (float)res[i];
    return out;
}

int anacor_rotated_vectors(const double *omega_axis, const double *omega, const double *F, const double *xray,
                           const double *s1, int64_t n, double *rx, double *rs)
{
    if (!omega_axis || !omega || !F || !xray || !s1 || !rx || !rs || n < 0)
        return fail(kErrArgs, "bad arguments");
    ReflTable tab;
    for (int64_t i = 0; i < n; i++)
        setup_reflection(omega_axis, omega[i], F, xray, s1 + 3 * i, &tab, rx + 3 * i, rs + 3 * i);
    return succeed();
}

int anacor_block_guard_check(int threads, int32_t *status)
{
    DeviceState *d = nullptr;
    if (int st = current_device(&d))
        return st;
    int word = 0;
    const int st = block_guard_selftest(threads, &word);
    if (st)
        return fail(st, st == kErrArgs ? "threads must be a positive multiple of 32, at most the block size"
                                       : "block-guard launch failed");
    if (status)
        *status = word;
    return succeed();
}

int anacor_leg_detail(const int8_t *label, const int64_t *shape, const int64_t *coords, int64_t n,
                      const double *rotated_s1, const double *rotated_xray, const double *voxel,
                      int full_iteration, int32_t *face, int32_t *len, int32_t *nseg, int32_t *first,
                      int32_t *last, double *L, int32_t *status)
{
    if (!face || !len || !nseg || !first || !last || !L || !status || !rotated_s1 || !rotated_xray)
        return fail(kErrArgs, "bad arguments");
    ReflTable tab;
    if (int st = setup_rotated(rotated_xray, rotated_s1, &tab))
        return fail(st, status_text(st));
    static const double mu0[4] = {0, 0, 0, 0};
    anacor_plan p;
    int st = plan_init(&p, label, shape, coords, n, voxel, mu0, full_iteration, 1, 0);
    ReflTable *d_tab = nullptr;
    double *d_vox = nullptr;
    int *d_i = nullptr;
    double *d_L = nullptr;
    cudaError_t e = cudaSuccess;
    const size_t m = (size_t)std::max<int64_t>(n, 1) * 2;
    if (!st) {
        if ((e = dev_alloc(&d_tab, 1, p.stream)) || (e = dev_alloc(&d_vox, 3, p.stream)) ||
            (e = dev_alloc(&d_i, m * 10, p.stream)) || (e = dev_alloc(&d_L, m * 4, p.stream)) ||
            (e = cudaMemcpyAsync(d_tab, &tab, sizeof(tab), cudaMemcpyHostToDevice, p.stream)) ||
            (e = cudaMemcpyAsync(d_vox, voxel, 3 * sizeof(double), cudaMemcpyHostToDevice, p.stream)) ||
            (e = launch_leg_detail(d_tab, p.d_vol, p.dims, p.d_coords, (int)n, d_vox, full_iteration, p.d_sq,
                                   p.sq_stride, p.d_qtab, d_i, d_i + m, d_i + 2 * m, d_i + 3 * m, d_i + 6 * m, d_L,
                                   d_i + 9 * m, p.stream)))
            st = cuda_fail(e, "leg detail");
    }
    if (!st && n > 0) {
        std::vector<int32_t> h(m * 10);
        if ((e = cudaMemcpyAsync(h.data(), d_i, m * 10 * sizeof(int), cudaMemcpyDeviceToHost, p.stream)) ||
            (e = cudaMemcpyAsync(L, d_L, (size_t)n * 2 * 4 * sizeof(double), cudaMemcpyDeviceToHost, p.stream)) ||
            (e = cudaStreamSynchronize(p.stream)))
            st = cuda_fail(e, "leg detail download");
        else {
            const size_t k = (size_t)n * 2;
            std::memcpy(face, h.data(), k * sizeof(int32_t));
            std::memcpy(len, h.data() + m, k * sizeof(int32_t));
            std::memcpy(nseg, h.data() + 2 * m, k * sizeof(int32_t));
            std::memcpy(first, h.data() + 3 * m, 3 * k * sizeof(int32_t));
            std::memcpy(last, h.data() + 6 * m, 3 * k * sizeof(int32_t));
            std::memcpy(status, h.data() + 9 * m, k * sizeof(int32_t));
        }
    }
    if (!st) {
        int dst = 0;
        if ((e = cudaMemcpy(&dst, p.d_status, sizeof(int), cudaMemcpyDeviceToHost)))
            st = cuda_fail(e, "status");
        else if (dst & (1 << kErrArgs))
            st = fail(kErrArgs, status_text(kErrArgs));
    }
    const int keep = t_status;
    const std::string msg = t_msg;
    if (p.stream) {
        dev_free(d_tab, p.stream);
        dev_free(d_vox, p.stream);
        dev_free(d_i, p.stream);
        dev_free(d_L, p.stream);
        plan_release(&p);
    }
    if (st) {
        t_status = keep;
        t_msg = msg;
        return st;
    }
    return succeed();
}


int anacor_plan_configure(anacor_plan *p, int variant, int tile, int order)
{
    if (!p)
        return fail(kErrArgs, "null plan");
    if (int st = plan_configure(p, variant, tile, order))
        return st;
    return succeed();
}

int anacor_plan_config(const anacor_plan *p, int *variant, int *tile, int *order)
{
    if (!p)
        return fail(kErrArgs, "null plan");
    if (variant)
        *variant = p->variant ? p->variant : absorption_variant();
    if (tile)
        *tile = p->tile;
    if (order)
        *order = p->order;
    return succeed();
}

int anacor_plan_autotune(anacor_plan *p, int64_t sample_refl, float *best_ms)
{
    if (!p || p->n_refl <= 0 || p->n_vox <= 0)
        return fail(kErrArgs, "autotune needs a plan with voxels and reflections");
    const TuneKey key = tune_key(p);
    TuneVal cv{0, 0, 1, 0.0f};
    const bool cached = tune_lookup(p, cv);
    // a cached distance-field choice does not apply to a volume without a field
    if (cached && (cv.variant <= 4 || plan_ensure_field(p, field_kind(cv.variant)) == kOk)) {
        if (best_ms)
            *best_ms = cv.ms;
        return plan_configure(p, cv.variant, cv.tile, cv.order) ? t_status : succeed();
    }
    // first the voxel order at the default variant and tile, then variant x tile with that order
    TuneVal best{0, 0, 1, 1e30f};
    // time of one candidate (ms for all reflections): best of five runs over
    // enough reflections for about eight waves of work items
    auto timed = [&](int variant, int tile, int order, float &out) -> int {
        if (int st = plan_configure(p, variant, tile, order))
            return st;
        // about eight waves of warp work items, and at least 32 reflections
        // (spread over all of them) so that the sample's directions are the
        // workload's
        const long long warps = (long long)p->dev->sms * variant_occupancy(p->dev, variant) * 8;
        int64_t k = (int64_t)((8 * warps + p->tiles - 1) / p->tiles);
        k = std::max<int64_t>(k, std::max<int64_t>(32, sample_refl));
        k = std::min<int64_t>(k, p->n_refl);
        out = 1e30f;
        for (int rep = 0; rep < 5; rep++) {
            float ms = 0.0f;
            if (int st = plan_time(p, k, 1, &ms))
                return st;
            out = std::min(out, ms * (float)p->n_refl / (float)k);
            if (ms > 20.0f && rep >= 1)   // long runs: best of two is steady enough
                break;
        }
        return kOk;
    };
    // voxel order first: Morton unless another order is clearly faster (the
    // differences between orders are small and the sample is short)
    float t_ref = 0.0f;
    if (int st = timed(0, kTile, 1, t_ref))
        return st;
    int order = 1;
    float t_order = t_ref;
    for (int o = 0; o < kVoxelOrders; o++) {
        if (o == 1)
            continue;
        float t = 0.0f;
        if (int st = timed(0, kTile, o, t))
            return st;
        if (t < 0.97f * t_ref && t < t_order) {
            order = o;
            t_order = t;
        }
    }
    // the distance-field variants where the labels allow a field
    std::vector<int> variants{2, 3, 4};
    if (plan_ensure_field(p, 1) == kOk)
        variants.insert(variants.end(), {6, 7, 8});
    if (plan_ensure_field(p, 2) == kOk)
        variants.insert(variants.end(), {10, 11, 12});
    if (plan_ensure_field(p, 3) == kOk)
        variants.insert(variants.end(), {14, 15, 16});
    for (int tile : {128, 256, 512, 1024, 2048})
        for (int variant : variants) {
            float t = 0.0f;
            if (int st = timed(variant, tile, order, t))
                return st;
            if (t < best.ms)
                best = TuneVal{variant, tile, order, t};
        }
    if (int st = plan_configure(p, best.variant, best.tile, best.order))
        return st;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_tune_cache[key] = best;
    }
    if (best_ms)
        *best_ms = best.ms;
    return succeed();
}

anacor_batch *anacor_batch_create(anacor_plan *const *plans, int n_plans)
{
    if (!plans || n_plans <= 0) {
        fail(kErrArgs, "empty batch");
        return nullptr;
    }
    anacor_batch *b = new (std::nothrow) anacor_batch();
    if (!b) {
        fail(kErrNoMem, "out of host memory");
        return nullptr;
    }
    for (int i = 0; i < n_plans; i++) {
        if (!plans[i]) {
            delete b;
            fail(kErrArgs, "null plan in batch");
            return nullptr;
        }
        b->plans.push_back(plans[i]);
    }
    b->stream = plans[0]->stream;
    cudaError_t e;
    if ((e = cudaMalloc(&b->d_descs, sizeof(SampleDesc) * (size_t)n_plans)) ||
        (e = cudaMalloc(&b->d_counter, sizeof(unsigned long long))) ||
        (e = cudaMalloc(&b->d_descs_field, sizeof(SampleDesc) * (size_t)n_plans)) ||
        (e = cudaMalloc(&b->d_counter_field, sizeof(unsigned long long)))) {
        cuda_fail(e, "device allocation");
        anacor_batch_destroy(b);
        return nullptr;
    }
    if (batch_upload(b)) {
        const int keep = t_status;
        const std::string msg = t_msg;
        anacor_batch_destroy(b);
        t_status = keep;
        t_msg = msg;
        return nullptr;
    }
    succeed();
    return b;
}

int anacor_batch_configure(anacor_batch *b, int variant)
{
    if (!b || variant < 0 || variant > kPlanVariants)
        return fail(kErrArgs, "bad arguments");
    b->variant = variant;
    if (int st = batch_upload(b))
        return st;
    return succeed();
}

int anacor_batch_launch(anacor_batch *b, void *stream)
{
    if (!b)
        return fail(kErrArgs, "null batch");
    cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
    if (cudaError_t e = batch_enqueue(b, st))
        return cuda_fail(e, "kernel launch");
    return succeed();
}

int anacor_batch_capture(anacor_batch *b, void *stream)
{
    if (!b)
        return fail(kErrArgs, "null batch");
    cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    cudaError_t e;
    if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)))
        return cuda_fail(e, "cudaStreamBeginCapture");
    const cudaError_t le = batch_enqueue(b, st);
    e = cudaStreamEndCapture(st, &b->graph);
    if (le)
        return cuda_fail(le, "kernel launch during capture");
    if (e)
        return cuda_fail(e, "cudaStreamEndCapture");
    if ((e = cudaGraphInstantiate(&b->exec, b->graph, 0)))
        return cuda_fail(e, "cudaGraphInstantiate");
    return succeed();
}

int anacor_batch_replay(anacor_batch *b, void *stream)
{
    if (!b || !b->exec)
        return fail(kErrArgs, "batch has no captured graph");
    cudaError_t e = cudaGraphLaunch(b->exec, stream ? (cudaStream_t)stream : b->stream);
    if (e)
        return cuda_fail(e, "cudaGraphLaunch");
    return succeed();
}

int anacor_batch_wait(anacor_batch *b, void *stream)
{
    if (!b)
        return fail(kErrArgs, "null batch");
    return batch_check(b, stream ? (cudaStream_t)stream : b->stream);
}

int anacor_batch_autotune(anacor_batch *b, int64_t sample_refl)
{
    if (!b)
        return fail(kErrArgs, "null batch");
    // per-sample tile and voxel order, then one register-budget variant for the launch
    for (anacor_plan *p : b->plans)
        if (p->n_refl > 0 && p->n_vox > 0)
            if (int st = anacor_plan_autotune(p, sample_refl, nullptr))
                return st;
    // then one variant for the whole launch: the cooperative march, or every
    // sample on its centred, octant or bricked octant fields
    float best = 1e30f;
    int best_v = 0;
    std::vector<int> variants{2, 3, 4};
    for (int fk = 1; fk <= 3; fk++) {
        bool any = false;
        for (anacor_plan *p : b->plans) {
            const int st = plan_ensure_field(p, fk);
            if (st && st != kErrUnsupported)
                return st;
            any = any || st == kOk;
        }
        succeed();
        if (any)
            for (int budget = 2; budget <= 4; budget++)
                variants.push_back(4 * fk + budget);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int v : variants) {
        b->variant = v;
        if (int st = batch_upload(b))
            return st;
        anacor_batch_launch(b, nullptr);   // warm-up
        cudaEventRecord(e0, b->stream);
        anacor_batch_launch(b, nullptr);
        cudaEventRecord(e1, b->stream);
        cudaError_t e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e || (e = cudaEventElapsedTime(&ms, e0, e1))) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_fail(e, "timing");
        }
        if (ms < best) {
            best = ms;
            best_v = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->variant = best_v;
    if (int st = batch_upload(b))
        return st;
    return succeed();
}

int anacor_batch_kernels(const anacor_batch *b)
{
    return b ? batch_kernels(b) : 0;
}

int anacor_batch_info(const anacor_batch *b, int *grid, long long *items, int *variant)
{
    if (!b)
        return fail(kErrArgs, "null batch");
    if (grid)
        *grid = b->grid;
    if (items)
        *items = b->items;
    if (variant)
        *variant = b->variant ? b->variant : absorption_variant();
    return succeed();
}

void anacor_batch_destroy(anacor_batch *b)
{
    if (!b)
        return;
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    if (b->d_descs)
        cudaFree(b->d_descs);
    if (b->d_counter)
        cudaFree(b->d_counter);
    if (b->d_descs_field)
        cudaFree(b->d_descs_field);
    if (b->d_counter_field)
        cudaFree(b->d_counter_field);
    delete b;
}

}  // extern "C"
