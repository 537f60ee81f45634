// Chessboard distance field of a label volume, packed with the label.
//
// out[v] = (label & 7) | (min(D(v), 31) << 3), where D(v) is the chessboard
// (L-infinity) distance from voxel v to the nearest voxel of the volume whose
// label differs from v's, and 0 for vacuum voxels (label 0: a ray stops there,
// so their distance is never read).  Every voxel within chessboard distance
// D(v) - 1 of v carries v's label: a march that stands on v may step over the
// increments that provably stay inside that cube.
//
// D is found as the largest uniform cube around v, built from one axis at a
// time (the cube of radius r is uniform iff every row segment of half-width r
// inside it is):
//   rows    d_x(v)   = min(31, distance to the nearest other label along x)
//   planes  d_xy(v)  = 1 + max{ r : all |dy| <= r have v's label and d_x >= r + 1 }
//   volume  D(v)     = 1 + max{ r : all |dz| <= r have v's label and d_xy >= r + 1 }
// Voxels outside the volume do not count (marches never leave it).  The
// labels must fit 3 bits (0..7); the first pass flags any that do not.
//
// Octant fields: the same construction with one-sided scans gives, for each
// of the 8 sign combinations (sz, sy, sx), 1 + the largest r for which the
// corner box v + [0..r]^3 * (sz, sy, sx) holds one label.  A ray whose
// direction has those signs only moves into that box, so behind-the-ray
// boundaries (the one just crossed) do not shorten its skips.  Layout:
// [octant][Z][Y][X] with octant = (sx < 0) | (sy < 0) << 1 | (sz < 0) << 2.
// The octant passes find each one-sided r without scanning: the row pass
// from bit masks of label changes, the plane and volume passes by binary
// lifting over tables of window minima in shared memory (octant_lift).
#include "anacor_internal.h"
#include "trace_launch.h"

namespace anacor {
namespace {

constexpr int kFieldCap = 31;
constexpr int kFieldThreads = 256;

// d_x along each row (dir 0: both sides, +1 / -1: ahead / behind only); one
// CTA per (z, y) row
__global__ void __launch_bounds__(kFieldThreads) field_rows(const int8_t *__restrict__ vol, int dx, int dir,
                                                            uint8_t *__restrict__ out, int *__restrict__ bad)
{
    const long long row = (long long)blockIdx.x * dx;
    const int8_t *r = vol + row;
    bool any_bad = false;
    for (int x0 = 0; x0 < dx; x0 += kFieldThreads) {
        const int x = x0 + (int)threadIdx.x;
        if (x < dx) {
            const int lab = r[x];
            uint8_t o = 0;
            if ((unsigned)lab > 7u) {
                any_bad = true;
            } else if (lab != 0) {
                int d = kFieldCap;
                for (int k = 1; k < kFieldCap; k++) {
                    if ((dir >= 0 && x + k < dx && r[x + k] != lab) || (dir <= 0 && x - k >= 0 && r[x - k] != lab)) {
                        d = k;
                        break;
                    }
                }
                o = (uint8_t)(lab | (d << 3));
            }
            out[row + x] = o;
        }
    }
    if (__syncthreads_or(any_bad) && threadIdx.x == 0)
        atomicOr(bad, 1);
}

// One cube-growing pass along an axis of stride `stride` and extent `n`
// (coordinate `c` of the row's voxels on that axis): in holds label | d << 3
// of the previous pass, out receives label | d' << 3.
__global__ void __launch_bounds__(kFieldThreads) field_grow(const uint8_t *__restrict__ in, int dy, int dx,
                                                            int axis, int n, long long stride, int dir,
                                                            uint8_t *__restrict__ out)
{
    const long long row = (long long)blockIdx.x * dx;
    const int c = axis == 1 ? (int)(blockIdx.x % (unsigned)dy) : (int)(blockIdx.x / (unsigned)dy);
    for (int x0 = 0; x0 < dx; x0 += kFieldThreads) {
        const int x = x0 + (int)threadIdx.x;
        if (x >= dx)
            continue;
        const long long v = row + x;
        const uint32_t b = in[v];
        const uint32_t lab = b & 7u;
        if (lab == 0) {
            out[v] = 0;
            continue;
        }
        uint32_t m = b >> 3;
        int d = 1;
        for (int r = 1; r < kFieldCap; r++) {
            if (dir >= 0 && c + r < n) {
                const uint32_t u = in[v + r * stride];
                m = min(m, (u & 7u) == lab ? (u >> 3) : 0u);
            }
            if (dir <= 0 && c - r >= 0) {
                const uint32_t u = in[v - r * stride];
                m = min(m, (u & 7u) == lab ? (u >> 3) : 0u);
            }
            if (m < (uint32_t)(r + 1))
                break;
            d = r + 1;
        }
        out[v] = (uint8_t)(lab | (uint32_t)d << 3);
    }
}

// Octant rows: out[0] = min(31, length of the run of v's label from v toward
// +x), out[1] toward -x (a run that reaches the end of its row counts as 31).
// The volume is taken as one sequence in chunks of kRowChunk voxels; the label
// changes of a chunk and one word either side are a bit mask in shared memory
// (bit p: the labels of p and p + 1 differ within one row), and a run's end
// is the first set bit after (or the last before) v, found with ffs / clz over
// at most two words; a bit in another row means no change in v's row.
constexpr int kRowThreads = 256;
constexpr int kRowChunk = 4 * kRowThreads;   // 4 voxels per thread
constexpr int kRowWords = kRowChunk / 32 + 2;

// (volumes hold fewer than 2^31 voxels: 32-bit positions)
__global__ void __launch_bounds__(kRowThreads) octant_rows(const int8_t *__restrict__ vol, int dx, int nvol, bool vec,
                                                           uint8_t *__restrict__ out, int *__restrict__ bad)
{
    __shared__ uint32_t change[kRowWords];          // word k covers p0 + 32 (k - 1) ...
    __shared__ uint32_t labw[kRowChunk / 4 + 17];   // bytes p0 - 32 ... p0 + kRowChunk + 35
    const int p0 = blockIdx.x * kRowChunk;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint8_t *lb = reinterpret_cast<uint8_t *>(labw);
    // the chunk's labels (a word per thread) and 32 / 36 bytes either side
    {
        const int v = p0 + 4 * (int)threadIdx.x;
        uint32_t w = 0;
        if (vec && v + 3 < nvol)
            w = __ldg(reinterpret_cast<const uint32_t *>(vol + v));
        else
            for (int k = 0; k < 4; k++)
                if (v + k < nvol)
                    w |= (uint32_t)(uint8_t)vol[v + k] << (8 * k);
        labw[8 + threadIdx.x] = w;
        if (threadIdx.x < 68) {
            const int h = threadIdx.x < 32 ? (int)threadIdx.x : kRowChunk + 32 + (int)threadIdx.x - 32;
            const int q = p0 - 32 + h;
            lb[h] = (q >= 0 && q < nvol) ? (uint8_t)vol[q] : 0u;
        }
    }
    __syncthreads();
    const int x0 = p0 % dx;   // x of p0; x of p0 + o is (x0 + o) mod dx
    for (int k = warp; k < kRowWords; k += kRowThreads / 32) {
        const int o = 32 * (k - 1) + lane;   // offset from p0, -32 ... kRowChunk + 31
        const int p = p0 + o;
        bool b = false;
        if (p >= 0 && p + 1 < nvol && (x0 + o + 1 + dx) % dx != 0)
            b = lb[o + 32] != lb[o + 33];
        const uint32_t m = __ballot_sync(0xffffffffu, b);
        if (lane == 0)
            change[k] = m;
    }
    __syncthreads();
    const int v0 = p0 + 4 * (int)threadIdx.x;
    if (v0 >= nvol)
        return;
    const uint32_t labs = labw[8 + threadIdx.x];
    bool any_bad = false;
    uint32_t o0 = 0, o1 = 0;
    const int xb = (x0 + 4 * (int)threadIdx.x) % dx;   // x of v0
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int lab = (int)(int8_t)(labs >> (8 * k));
        if ((unsigned)lab > 7u) {
            any_bad |= v0 + k < nvol;
            continue;
        }
        if (lab == 0)
            continue;
        const int q = 4 * (int)threadIdx.x + k + 32;   // bit index in change[]
        const int w = q >> 5, bit = q & 31;
        const int v = v0 + k;
        int x = xb + k;
        while (x >= dx)   // at most 3 times
            x -= dx;
        const int rs = v - x, re = rs + dx;   // v's row [rs, re)
        int d0 = kFieldCap, d1 = kFieldCap;
        // toward +x: the first change at or after v ends the run at it
        uint32_t m = change[w] >> bit;
        int b = -1;
        if (m)
            b = v + __ffs(m) - 1;
        else if ((m = change[w + 1]) != 0)
            b = v + 32 - bit + __ffs(m) - 1;
        if (b >= 0 && b < re)
            d0 = min(b + 1 - v, kFieldCap);
        // toward -x: the last change before v, at b, leaves v - b voxels
        m = bit ? change[w] & ((1u << bit) - 1u) : 0u;
        b = -1;
        if (m)
            b = v - bit + (31 - __clz(m));
        else if ((m = change[w - 1]) != 0)
            b = v - bit - 32 + (31 - __clz(m));
        if (b >= rs)
            d1 = min(v - b, kFieldCap);
        o0 |= (uint32_t)(lab | (d0 << 3)) << (8 * k);
        o1 |= (uint32_t)(lab | (d1 << 3)) << (8 * k);
    }
    if (vec && v0 + 3 < nvol) {
        *reinterpret_cast<uint32_t *>(out + v0) = o0;
        *reinterpret_cast<uint32_t *>(out + (long long)nvol + v0) = o1;
    } else {
        for (int k = 0; k < 4 && v0 + k < nvol; k++) {
            out[v0 + k] = (uint8_t)(o0 >> (8 * k));
            out[(long long)nvol + v0 + k] = (uint8_t)(o1 >> (8 * k));
        }
    }
    if (any_bad)
        atomicOr(bad, 1);
}

// Growth along one axis by binary lifting.  For an input m (label | d << 3,
// one-sided) and a direction s, the output at v is label | t << 3 with t the
// largest value <= 31 for which the voxels v, v + s, ..., v + (t - 1) s that
// lie inside the volume all carry v's label and m >= t.  Those t form an
// interval [1, t_max], so t_max is reached by trying steps of 16, 8, 4, 2
// and 1 from t = 1, each accepted when the window of the step's voxels passes;
// a window's test is one lookup in a table of window minima, built per tile in
// shared memory: U_w(p) = label | min m << 3 over the w voxels from p when one
// label fills them, else 0 (U_2w(p) from U_w(p) and U_w(p + w)).  The windows
// toward -s are the same tables read from the window's far end.  Positions
// outside the volume hold a copy of the nearest voxel inside, which leaves
// the minimum of any window holding a voxel inside unchanged; a step whose
// first voxel is outside imposes nothing.
//
// Tile: 128 voxels along x (a lane's 4 bytes in one word) by kLiftRows output
// positions along the axis, plus kFieldCap - 1 positions on either side.
constexpr int kLiftWords = 32;
constexpr int kLiftRows = 64;
constexpr int kLiftHalo = kFieldCap - 1;
constexpr int kLiftSpan = kLiftRows + 2 * kLiftHalo;
constexpr int kLiftThreads = 512;
constexpr int kLiftWarps = kLiftThreads / 32;
constexpr int kLiftLevels = 5;   // windows of 1, 2, 4, 8, 16 voxels
constexpr size_t kLiftSmem = (size_t)kLiftLevels * kLiftSpan * kLiftWords * sizeof(uint32_t);

// per byte: the smaller of a and b when their labels (low 3 bits) agree, else 0
__device__ __forceinline__ uint32_t window_merge(uint32_t a, uint32_t b)
{
    const uint32_t d = (a ^ b) & 0x07070707u;
    const uint32_t differ = (d | (d >> 1) | (d >> 2)) & 0x01010101u;
    return __vminu4(a, b) & ~(differ * 0xffu);
}

__device__ __forceinline__ uint32_t load_word(const uint8_t *p, int x, int dx, bool vec)
{
    if (vec && x + 3 < dx)
        return __ldg(reinterpret_cast<const uint32_t *>(p + x));
    uint32_t w = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (x + k < dx)
            w |= (uint32_t)__ldg(p + x + k) << (8 * k);
    return w;
}

__device__ __forceinline__ void store_word(uint8_t *p, int x, int dx, bool vec, uint32_t w)
{
    if (vec && x + 3 < dx) {
        *reinterpret_cast<uint32_t *>(p + x) = w;
        return;
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (x + k < dx)
            p[x + k] = (uint8_t)(w >> (8 * k));
}

// kIn inputs, each grown toward both signs of the axis (n positions, stride
// sa; so the stride of the tile's other coordinate, blockIdx.y): result
// j = 2 * i + s (s = 1 toward -) from in[i], stored as out[j], or (kOctants,
// i = 2 * bx + by, s = bz) as out[bx | by << 1 | bz << 2].
template <int kIn, bool kOctants>
__global__ void __launch_bounds__(kLiftThreads, 2) octant_lift(const uint8_t *__restrict__ in, int n, long long sa,
                                                            long long so, int dx, long long nvol, bool vec,
                                                            uint8_t *__restrict__ out)
{
    extern __shared__ uint32_t lift_tab[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x = blockIdx.x * (kLiftWords * 4) + 4 * lane;
    const long long ob = (long long)blockIdx.y * so;
    const int a0 = blockIdx.z * kLiftRows;
    // a thread's rows of the tile, loaded together (the next input's while
    // the current one is processed)
    constexpr int kPer = (kLiftSpan + kLiftWarps - 1) / kLiftWarps;
    uint32_t wv[kPer];
    auto load_tile = [&](int i) {
        const uint8_t *src = in + i * nvol + ob;
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int j = warp + q * kLiftWarps;
            const int a = min(max(a0 - kLiftHalo + j, 0), n - 1);
            wv[q] = j < kLiftSpan ? load_word(src + a * sa, x, dx, vec) : 0u;
        }
    };
    load_tile(0);
    for (int i = 0; i < kIn; i++) {
        uint32_t live = 0;
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int j = warp + q * kLiftWarps;
            if (j < kLiftSpan)
                lift_tab[j * kLiftWords + lane] = wv[q];
            if (j >= kLiftHalo && j < kLiftHalo + kLiftRows)
                live |= wv[q] & 0x07070707u;
        }
        // a tile whose output rows are all vacuum (the labels are the same in
        // every input) writes zeros
        if (i == 0 && !__syncthreads_or(live != 0u)) {
            for (int jo = warp; jo < kLiftRows && a0 + jo < n; jo += kLiftWarps)
#pragma unroll
                for (int jj = 0; jj < 2 * kIn; jj++)
                    store_word(out + jj * nvol + ob + (a0 + jo) * sa, x, dx, vec, 0u);
            return;
        }
        __syncthreads();
        if (i + 1 < kIn)
            load_tile(i + 1);
#pragma unroll
        for (int lv = 1; lv < kLiftLevels; lv++) {
            const int w = 1 << (lv - 1);
            const uint32_t *A = lift_tab + (lv - 1) * kLiftSpan * kLiftWords;
            uint32_t *B = lift_tab + lv * kLiftSpan * kLiftWords;
            for (int j = warp; j + 2 * w <= kLiftSpan; j += kLiftWarps)
                B[j * kLiftWords + lane] = window_merge(A[j * kLiftWords + lane], A[(j + w) * kLiftWords + lane]);
            __syncthreads();
        }
        for (int jo = warp; jo < kLiftRows; jo += kLiftWarps) {
            const int a = a0 + jo;
            if (a >= n)
                break;
            const int j0 = jo + kLiftHalo;
            const uint32_t cur = lift_tab[j0 * kLiftWords + lane];
            uint32_t res[2] = {0u, 0u};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint32_t c = (cur >> (8 * k)) & 0xffu;
                if ((c & 7u) == 0u)
                    continue;
#pragma unroll
                for (int s = 0; s < 2; s++) {
                    int t = 1;
                    uint32_t P = c >> 3;
#pragma unroll
                    for (int lv = kLiftLevels - 1; lv >= 0; lv--) {
                        const int w = 1 << lv;
                        const int tn = t + w;
                        if ((int)P >= tn) {
                            uint32_t P2 = P;
                            if (s == 0 ? a + t < n : a - t >= 0) {
                                const int jw = s == 0 ? j0 + t : j0 - t - w + 1;
                                const uint32_t u =
                                    (lift_tab[(lv * kLiftSpan + jw) * kLiftWords + lane] >> (8 * k)) & 0xffu;
                                P2 = ((u ^ c) & 7u) ? 0u : min(P, u >> 3);
                            }
                            if ((int)P2 >= tn) {
                                t = tn;
                                P = P2;
                            }
                        }
                    }
                    res[s] |= ((c & 7u) | (uint32_t)t << 3) << (8 * k);
                }
            }
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const int j = 2 * i + s;
                const int o = kOctants ? ((j >> 2) | (((j >> 1) & 1) << 1) | ((j & 1) << 2)) : j;
                store_word(out + o * nvol + ob + a * sa, x, dx, vec, res[s]);
            }
        }
        __syncthreads();   // the tables are refilled for the next input
    }
}

}  // namespace

cudaError_t launch_distance_field(const int8_t *d_vol, const int *dims, uint8_t *d_out, uint8_t *d_tmp, int *d_bad,
                                  cudaStream_t st)
{
    const unsigned rows = (unsigned)dims[0] * (unsigned)dims[1];
    if (rows == 0 || dims[2] == 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
    if (e != cudaSuccess)
        return e;
    const long long plane = (long long)dims[1] * dims[2];
    field_rows<<<rows, kFieldThreads, 0, st>>>(d_vol, dims[2], 0, d_out, d_bad);
    field_grow<<<rows, kFieldThreads, 0, st>>>(d_out, dims[1], dims[2], 1, dims[1], dims[2], 0, d_tmp);
    field_grow<<<rows, kFieldThreads, 0, st>>>(d_tmp, dims[1], dims[2], 0, dims[0], plane, 0, d_out);
    return cudaGetLastError();
}

cudaError_t launch_octant_fields(const int8_t *d_vol, const int *dims, uint8_t *d_out, uint8_t *d_tmp, int *d_bad,
                                 cudaStream_t st)
{
    const unsigned rows = (unsigned)dims[0] * (unsigned)dims[1];
    if (rows == 0 || dims[2] == 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
    if (e != cudaSuccess)
        return e;
    const long long plane = (long long)dims[1] * dims[2];
    const long long nvol = plane * dims[0];
    // tmp[bx]: rows (bx = 1: -x); tmp[2 + 2*bx + by]: squares; out[bx | by << 1 | bz << 2]
    if ((e = cudaFuncSetAttribute(octant_lift<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kLiftSmem)) ||
        (e = cudaFuncSetAttribute(octant_lift<4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kLiftSmem)))
        return e;
    // word loads and stores where every row starts on a 4-byte boundary
    const bool vec = dims[2] % 4 == 0 && ((uintptr_t)d_tmp & 3u) == 0 && ((uintptr_t)d_out & 3u) == 0;
    const unsigned xt = (unsigned)(dims[2] + kLiftWords * 4 - 1) / (kLiftWords * 4);
    const bool vrow = nvol % 4 == 0 && ((uintptr_t)d_vol & 3u) == 0 && ((uintptr_t)d_tmp & 3u) == 0;
    octant_rows<<<(unsigned)((nvol + kRowChunk - 1) / kRowChunk), kRowThreads, 0, st>>>(d_vol, dims[2], (int)nvol,
                                                                                       vrow, d_tmp, d_bad);
    const dim3 gy(xt, (unsigned)dims[0], (unsigned)(dims[1] + kLiftRows - 1) / kLiftRows);
    octant_lift<2, false><<<gy, kLiftThreads, kLiftSmem, st>>>(d_tmp, dims[1], dims[2], plane, dims[2], nvol, vec,
                                                               d_tmp + 2 * nvol);
    const dim3 gz(xt, (unsigned)dims[1], (unsigned)(dims[0] + kLiftRows - 1) / kLiftRows);
    octant_lift<4, true><<<gz, kLiftThreads, kLiftSmem, st>>>(d_tmp + 2 * nvol, dims[0], plane, dims[2], dims[2],
                                                              nvol, vec, d_out);
    return cudaGetLastError();
}

namespace {

// One thread per 16 output bytes (a 4x4 (y, x) slab of one brick row z).
__global__ void brick_fields_kernel(const uint8_t *__restrict__ lin, int dz, int dy, int dx, int nbz, int nby,
                                    int nbx, long long n_fields, uint8_t *__restrict__ out)
{
    const long long nvol = (long long)dz * dy * dx;
    const long long per = (long long)nbz * nby * nbx * 64;
    const long long total = n_fields * (per >> 4);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long f = q / (per >> 4);
        const long long r = q - f * (per >> 4);       // 16-byte slab within the field
        const long long brick = r >> 2;
        const int zl = (int)(r & 3);
        const int bx = (int)(brick % nbx);
        const int by = (int)((brick / nbx) % nby);
        const int bz = (int)(brick / ((long long)nbx * nby));
        const int z = bz * 4 + zl;
        uint32_t w[4];
#pragma unroll
        for (int yl = 0; yl < 4; yl++) {
            const int y = by * 4 + yl;
            uint32_t word = 0;
#pragma unroll
            for (int xl = 0; xl < 4; xl++) {
                const int x = bx * 4 + xl;
                const uint32_t b = (z < dz && y < dy && x < dx) ? lin[f * nvol + ((long long)z * dy + y) * dx + x] : 0u;
                word |= b << (8 * xl);
            }
            w[yl] = word;
        }
        reinterpret_cast<uint4 *>(out + f * per)[r] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

}  // namespace

size_t brick_field_bytes(const int *dims)
{
    return (size_t)((dims[0] + 3) / 4) * ((dims[1] + 3) / 4) * ((dims[2] + 3) / 4) * 64;
}

void brick_strides(const int *dims, int *sy, int *sz)
{
    const int nbx = (dims[2] + 3) / 4, nby = (dims[1] + 3) / 4;
    *sy = 64 * nbx;
    *sz = 64 * nbx * nby;
}

cudaError_t launch_brick_fields(const uint8_t *d_lin, const int *dims, int n_fields, uint8_t *d_out,
                                cudaStream_t st)
{
    const int nbz = (dims[0] + 3) / 4, nby = (dims[1] + 3) / 4, nbx = (dims[2] + 3) / 4;
    const long long total = (long long)n_fields * nbz * nby * nbx * 4;
    if (total <= 0)
        return cudaSuccess;
    const int threads = 256;
    const int blocks = (int)std::min<long long>((total + threads - 1) / threads, 152ll * 64);
    brick_fields_kernel<<<blocks, threads, 0, st>>>(d_lin, dims[0], dims[1], dims[2], nbz, nby, nbx, n_fields, d_out);
    return cudaGetLastError();
}

}  // namespace anacor
