// Slice fold and narrowing kernels of librtmc (sm_103a), and the precision dispatch of
// the transport's attribute helpers.
#include "rtmc_internal.h"

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

namespace rtmc {
namespace {

// Fold the dense index array into the histogram, one time slice at a time: blockIdx.y
// is the slice (so the L2 holds the slice being written), blockIdx.x a contiguous chunk
// of the slice's entries.  While particles crowd a few bins (early times) many entries
// of a chunk share a bin, and 64-bit reductions on the same L2 lines serialise; entries
// therefore go into a shared-memory hash table (bin -> count) of the block, which sends
// one atomic per distinct bin to the L2 at the end.  A probe window decides: unless its
// entries crowd into few bins (at most a quarter of the table, each hit twice on
// average) the rest of the chunk goes straight to the L2; a crowded chunk keeps using
// the table until it is three quarters full.
constexpr int kFoldThreads = 512;
constexpr int kHashSlots = 4096;

__device__ __forceinline__ bool hash_insert(int *keys, unsigned *cnts, int *used, int v)
{
    unsigned h = ((unsigned)v * 2654435761u) >> (32 - 12); // 12 = log2(kHashSlots)
#pragma unroll 1
    for (int probe = 0; probe < 8; ++probe) {
        int k = *((volatile int *)keys + h);
        if (k == -1) {
            k = atomicCAS(keys + h, -1, v);
            if (k == -1) atomicAdd(used, 1);
        }
        if (k == -1 || k == v) {
            atomicAdd(cnts + h, 1u);
            return true;
        }
        h = (h + 1) & (kHashSlots - 1);
    }
    return false;
}

__global__ void __launch_bounds__(kFoldThreads) rt_bin_slices(const BinParams b)
{
    __shared__ int keys[kHashSlots];
    __shared__ unsigned cnts[kHashSlots];
    __shared__ int used, valid, dense;
    const int j = b.j_first + blockIdx.y;
    const int32_t *row = b.idx + (int64_t)(j - 1) * b.rows; // rows is a multiple of 32: 16-byte aligned
    unsigned long long *slice = b.hist + (int64_t)j * b.time_stride;
    const unsigned long long inc = 1ull << b.hist_shift;
    for (int k = threadIdx.x; k < kHashSlots; k += blockDim.x) { keys[k] = -1; cnts[k] = 0u; }
    if (threadIdx.x == 0) { used = 0; valid = 0; }
    // this block's chunk of the slice, in 16-byte vectors
    const int64_t n4 = (b.n + 3) >> 2;
    const int64_t per = (n4 + gridDim.x - 1) / gridDim.x;
    const int64_t q0 = (int64_t)blockIdx.x * per, q1 = min(n4, q0 + per);
    const int4 *row4 = reinterpret_cast<const int4 *>(row);
    __syncthreads();
    // probe window: one vector per thread through the table
    int64_t q = q0 + threadIdx.x;
    if (q < q1) {
        const int4 a = __ldcs(row4 + q);
        const int va[4] = {a.x, a.y, a.z, a.w};
        int nv = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int v = va[u];
            if (v < 0 || q * 4 + u >= b.n) continue;
            ++nv;
            if (!hash_insert(keys, cnts, &used, v))
                atomicAdd(slice + ((v >> 30) ? b.mode_stride : 0) + (v & 0x3fffffff), inc);
        }
        if (nv) atomicAdd(&valid, nv);
    }
    __syncthreads();
    // crowded: the window's entries fell in at most a quarter of the table, with every
    // bin hit twice on average
    if (threadIdx.x == 0) dense = valid >= 64 && used * 4 <= kHashSlots && used * 2 <= valid;
    __syncthreads();
    if (dense) {
        for (q += blockDim.x; q < q1; q += blockDim.x) {
            const int4 a = __ldcs(row4 + q);
            const int va[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int v = va[u];
                if (v < 0 || q * 4 + u >= b.n) continue;
                // a table three-quarters full takes no new bins
                if (*((volatile int *)&used) >= 3 * kHashSlots / 4 || !hash_insert(keys, cnts, &used, v))
                    atomicAdd(slice + ((v >> 30) ? b.mode_stride : 0) + (v & 0x3fffffff), inc);
            }
        }
    } else {
        // two 16-byte loads in flight per thread before their atomics
        for (q += blockDim.x; q < q1; q += 2 * blockDim.x) {
            const int64_t q2 = q + blockDim.x;
            const int4 a = __ldcs(row4 + q);
            const int4 c = q2 < q1 ? __ldcs(row4 + q2) : make_int4(-1, -1, -1, -1);
            const int va[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int v = va[u];
                const int64_t e = (u < 4 ? q : q2) * 4 + (u & 3);
                if (v >= 0 && e < b.n) atomicAdd(slice + ((v >> 30) ? b.mode_stride : 0) + (v & 0x3fffffff), inc);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kHashSlots; k += blockDim.x) {
        const int v = keys[k];
        if (v >= 0) atomicAdd(slice + ((v >> 30) ? b.mode_stride : 0) + (v & 0x3fffffff), (unsigned long long)cnts[k] << b.hist_shift);
    }
}

// Same fold with a group of slices privatised in shared memory (u32 counts), flushed
// with one 64-bit atomic per touched bin: blockIdx.y is the slice group, blockIdx.x a
// contiguous particle range.
__global__ void __launch_bounds__(512) rt_bin_slices_smem(const BinParams b)
{
    extern __shared__ __align__(16) unsigned sh[];
    const int j0 = 1 + blockIdx.y * b.group;
    const int j1 = min(b.n_obs, j0 + b.group - 1);
    const int per = b.slice_bins * b.n_modes; // bins of one slice, all modes
    const int nb = (j1 - j0 + 1) * per;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) sh[k] = 0u;
    __syncthreads();
    const int64_t p0 = (int64_t)blockIdx.x * b.part_per_block;
    const int64_t p1 = min(b.n, p0 + b.part_per_block);
    // 16-byte loads over the vectors covering [p0, p1) (rows are 128-byte aligned and
    // padded to a multiple of 32 entries), two in flight per thread; entries outside the
    // range are skipped
    const int64_t q0 = p0 >> 2, q1 = (p1 + 3) >> 2;
    for (int j = j0; j <= j1; ++j) {
        const int4 *row4 = reinterpret_cast<const int4 *>(b.idx + (int64_t)(j - 1) * b.rows);
        unsigned *sj = sh + (j - j0) * per;
        for (int64_t q = q0 + threadIdx.x; q < q1; q += 2 * (int64_t)blockDim.x) {
            const int64_t q2 = q + blockDim.x;
            const int4 a = __ldcs(row4 + q);
            const int4 c = q2 < q1 ? __ldcs(row4 + q2) : make_int4(-1, -1, -1, -1);
            const int va[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int v = va[u];
                const int64_t k = (u < 4 ? q : q2) * 4 + (u & 3);
                if (v >= 0 && k >= p0 && k < p1) atomicAdd(sj + ((v >> 30) ? b.slice_bins : 0) + (v & 0x3fffffff), 1u);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        const unsigned c = sh[k];
        if (!c) continue;
        const int jj = j0 + k / per, r = k % per;
        const int m = r / b.slice_bins, o = r % b.slice_bins;
        atomicAdd(b.hist + (int64_t)jj * b.time_stride + (m ? b.mode_stride : 0) + o, (unsigned long long)c << b.hist_shift);
    }
}

// The reference's histogram type: counts (value >> shift) of n bins as uint32, saturating
// at 2^32 - 1 as MATLAB's uint32 additions do (initializeObservation.m:133,
// radiativeTransfer.m:88).  HBM-bound: 8 B read and 4 B written per bin; each thread keeps
// four independent loads in flight.
constexpr int kNarrowThreads = 256, kNarrowUnroll = 4;
__global__ void __launch_bounds__(kNarrowThreads) rt_narrow_u32(const unsigned long long *__restrict__ src,
                                                                 uint32_t *__restrict__ dst, int64_t n, int shift)
{
    const int64_t stride = (int64_t)gridDim.x * kNarrowThreads;
    for (int64_t k0 = (int64_t)blockIdx.x * kNarrowThreads * kNarrowUnroll + threadIdx.x; k0 < n;
         k0 += stride * kNarrowUnroll) {
        unsigned long long v[kNarrowUnroll];
#pragma unroll
        for (int u = 0; u < kNarrowUnroll; ++u) {
            const int64_t k = k0 + (int64_t)u * kNarrowThreads;
            v[u] = k < n ? __ldcs(src + k) : 0ull;
        }
#pragma unroll
        for (int u = 0; u < kNarrowUnroll; ++u) {
            const int64_t k = k0 + (int64_t)u * kNarrowThreads;
            const unsigned long long c = v[u] >> shift;
            if (k < n) __stcs(dst + k, c > 0xffffffffull ? 0xffffffffu : (uint32_t)c);
        }
    }
}

// Sets bit 1 of *status when a bin of the unsigned 64-bit fixed-point histogram holds 2^63
// or more, i.e. does not fit the int64 that rtmc_forward returns.  Reads every bin once
// (16-byte streaming loads), one flag per warp.
constexpr int kCheckThreads = 256;
__global__ void __launch_bounds__(kCheckThreads) rt_check_int64(const unsigned long long *__restrict__ h, int64_t n,
                                                                int32_t *status)
{
    unsigned long long acc = 0;
    const int64_t n2 = n >> 1;
    const ulonglong2 *h2 = reinterpret_cast<const ulonglong2 *>(h);
    for (int64_t k = (int64_t)blockIdx.x * kCheckThreads + threadIdx.x; k < n2; k += (int64_t)gridDim.x * kCheckThreads) {
        const ulonglong2 v = __ldcs(h2 + k);
        acc |= v.x | v.y;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) acc |= h[n - 1];
    if (__any_sync(0xffffffffu, (acc >> 63) != 0ull) && (threadIdx.x & 31) == 0) atomicOr(status, 2);
}

// ---- time-blocked FP32 fold ------------------------------------------------------
// A particle moves a fraction of a bin per observation instant (0.24 bin widths for the P
// waves of the 3D elastic workload), so its entries of 4 consecutive instants often share
// a bin.  Laid out with the 4 instants of a bin adjacent (16 bytes), such a run is one
// vector reduction (red.global.add.v4.f32) where the 64-bit histogram takes one per
// instant; the fold's cost is the L2's reduction rate, so fewer reductions is faster.
// Counts are exact in FP32 below 2^24 per bin and instant.  Crowded chunks (early
// instants) aggregate in a shared-memory hash first, as rt_bin_slices does.
constexpr int kTbThreads = 384;
constexpr int kTbAhead = 1; // index vectors a thread loads before folding them
constexpr int kTbSlots = 2048;

__device__ __forceinline__ void red_v4(float *a, float x, float y, float z, float w)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(x), "f"(y), "f"(z), "f"(w) : "memory");
}

// The L2's vector-reduction rate, the bound of rt_fold_tb: every thread issues `iters`
// reductions of 16 bytes (none awaited, as the fold issues them) to slots spread over an
// L2-resident buffer of n_vec 16-byte slots by a linear congruential sequence.
__global__ void __launch_bounds__(256) rt_probe_red_v4(float *buf, uint32_t n_vec, int iters)
{
    uint32_t h = (blockIdx.x * 256u + threadIdx.x) * 2654435761u + 12345u;
#pragma unroll 4
    for (int k = 0; k < iters; ++k) {
        h = h * 1664525u + 1013904223u;
        const uint32_t slot = (uint32_t)(((uint64_t)h * n_vec) >> 32); // below n_vec
        red_v4(buf + (size_t)slot * 4, 1.f, 1.f, 1.f, 1.f);
    }
}

__device__ __forceinline__ bool tb_hash_insert(int *keys, unsigned (*cnt)[4], int *used, int key, const int m[4])
{
    unsigned h = ((unsigned)key * 2654435761u) >> (32 - 11); // 11 = log2(kTbSlots)
#pragma unroll 1
    for (int probe = 0; probe < 8; ++probe) {
        int k = *((volatile int *)keys + h);
        if (k == -1) {
            k = atomicCAS(keys + h, -1, key);
            if (k == -1) atomicAdd(used, 1);
        }
        if (k == -1 || k == key) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (m[r]) atomicAdd(&cnt[h][r], 1u);
            return true;
        }
        h = (h + 1) & (kTbSlots - 1);
    }
    return false;
}

__global__ void __launch_bounds__(kTbThreads) rt_fold_tb(const TbParams t)
{
    __shared__ int keys[kTbSlots];
    __shared__ unsigned cnt[kTbSlots][4];
    __shared__ int used, valid, dense;
    const int tb = t.tb_first + blockIdx.y;
    const int j0 = 4 * tb + 1; // first instant of the t-block
    const int nr = min(4, t.n_obs - j0 + 1);
    const int4 *row[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        row[r] = reinterpret_cast<const int4 *>(t.idx + (int64_t)(j0 - 1 + (r < nr ? r : 0)) * t.rows);
    float *acc = t.acc + (size_t)(tb - t.acc_tb0) * t.S * 4;
    for (int k = threadIdx.x; k < kTbSlots; k += blockDim.x) {
        keys[k] = -1;
        cnt[k][0] = cnt[k][1] = cnt[k][2] = cnt[k][3] = 0u;
    }
    if (threadIdx.x == 0) { used = 0; valid = 0; }
    const int64_t p0 = (int64_t)blockIdx.x * t.part_per_block; // a multiple of 4
    const int64_t p1 = min(t.n, p0 + t.part_per_block);
    const int64_t q0 = p0 >> 2, q1 = (p1 + 3) >> 2;
    __syncthreads();
    // the entries of 4 particles x the t-block's instants: each run of consecutive instants
    // a particle spends in one bin goes out as one vector (to the hash when crowded)
    auto load = [&](int64_t q, int4 (&x)[4]) {
#pragma unroll
        for (int r = 0; r < 4; ++r) x[r] = r < nr && q < q1 ? __ldcs(row[r] + q) : make_int4(-1, -1, -1, -1);
    };
    // masks are kept as floats (compare-selects and products, no int-to-float conversions);
    // the mode bit of an entry becomes the second half of the slice: v + (v >> 30) *
    // (slice_bins - 2^30)
    const int mode_shift = t.slice_bins - (1 << 30);
    auto vector = [&](const int4 (&x)[4], int64_t q, bool use_hash, bool count, int *nvalid) {
        int e[4][4]; // [instant][particle]
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            e[r][0] = x[r].x; e[r][1] = x[r].y; e[r][2] = x[r].z; e[r][3] = x[r].w;
        }
        auto emit = [&](int v, float f0, float f1, float f2, float f3) {
            const int key = v + (v >> 30) * mode_shift;
            if (count) ++*nvalid;
            if (use_hash && *((volatile int *)&used) < 3 * kTbSlots / 4) {
                const int m[4] = {f0 != 0.f, f1 != 0.f, f2 != 0.f, f3 != 0.f};
                if (tb_hash_insert(keys, cnt, &used, key, m)) return;
            }
            red_v4(acc + (size_t)key * 4, f0, f1, f2, f3);
        };
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (q * 4 + u >= p1) continue;
            const int a = e[0][u], b = e[1][u], c = e[2][u], d = e[3][u];
            const float f01 = a == b ? 1.f : 0.f, f12 = b == c ? 1.f : 0.f, f23 = c == d ? 1.f : 0.f;
            // a run starts at every instant whose bin differs from the one before; -1
            // (not observed) is never emitted
            if (a >= 0) emit(a, 1.f, f01, f01 * f12, f01 * f12 * f23);
            if (b >= 0 && a != b) emit(b, 0.f, 1.f, f12, f12 * f23);
            if (c >= 0 && b != c) emit(c, 0.f, 0.f, 1.f, f23);
            if (d >= 0 && c != d) emit(d, 0.f, 0.f, 0.f, 1.f);
        }
    };
    // probe window: one vector per thread through the hash
    int nv = 0;
    int64_t q = q0 + threadIdx.x;
    int4 x[kTbAhead][4];
    if (q < q1) {
        load(q, x[0]);
        vector(x[0], q, true, true, &nv);
    }
    if (nv) atomicAdd(&valid, nv);
    __syncthreads();
    // crowded: the window's runs fell in at most a quarter of the table, each bin hit twice
    if (threadIdx.x == 0) dense = valid >= 64 && used * 4 <= kTbSlots && used * 2 <= valid;
    __syncthreads();
    const bool h = dense;
    // kTbAhead vectors per thread loaded together, then folded
    const int64_t T = blockDim.x;
    for (q += T; q < q1; q += kTbAhead * T) {
#pragma unroll
        for (int w = 0; w < kTbAhead; ++w) load(q + w * T, x[w]);
#pragma unroll
        for (int w = 0; w < kTbAhead; ++w)
            if (q + w * T < q1) vector(x[w], q + w * T, h, false, &nv);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kTbSlots; k += blockDim.x) {
        const int key = keys[k];
        if (key >= 0) red_v4(acc + (size_t)key * 4, (float)cnt[k][0], (float)cnt[k][1], (float)cnt[k][2], (float)cnt[k][3]);
    }
}

// acc -> the int64 histogram (and the uint32 counts): blockIdx.y is the t-block, threads
// run over its bins; each reads 16 bytes and writes the bin at 4 instants (coalesced
// across the threads of a warp)
constexpr int kConvThreads = 256;
__global__ void __launch_bounds__(kConvThreads) rt_tb_convert(const TbParams t, int64_t time_stride, int64_t mode_stride,
                                                              int shift, unsigned long long *__restrict__ hist,
                                                              uint32_t *__restrict__ u32)
{
    const int tb = t.tb_first + blockIdx.y;
    float4 *a4 = reinterpret_cast<float4 *>(t.acc) + (size_t)(tb - t.acc_tb0) * t.S;
    for (int64_t s = (int64_t)blockIdx.x * kConvThreads + threadIdx.x; s < t.S; s += (int64_t)gridDim.x * kConvThreads) {
        float4 c;
        if (t.rezero) { // a rolling accumulator: its lines stay in the L2 for the next turn
            c = __ldcg(a4 + s);
            a4[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            c = __ldcs(a4 + s);
        }
        const int64_t off = s >= t.slice_bins ? mode_stride + (s - t.slice_bins) : s;
        const float cv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int j = 4 * tb + r + 1;
            if (j > t.n_obs) break;
            // counts are exact integers below 2^24: a 32-bit conversion (the 64-bit one runs
            // on the FP64 pipe, which then bounds the kernel next to DRAM)
            const unsigned long long v = (unsigned long long)__float2uint_rz(cv[r]);
            __stcs(hist + (int64_t)j * time_stride + off, v << shift);
            if (u32) __stcs(u32 + (int64_t)j * time_stride + off, (uint32_t)v);
        }
        if (tb == 0) { // instant 0 is never observed
            __stcs(hist + off, 0ull);
            if (u32) __stcs(u32 + off, 0u);
        }
    }
}

} // namespace

namespace {
// ---------------------------------------------------------------------------------
// Particle order for the index path: a counting sort of the chunk's particles by the
// direction cell rt_events recorded (see OrderParams).  Each block takes a contiguous
// range of particles; block-level counts go to the cell totals with one atomic per
// (block, cell), the totals become cell offsets, and each block then reserves a column
// range per cell and places its particles there.
// ---------------------------------------------------------------------------------
constexpr int kOrderThreads = 512;

__global__ void __launch_bounds__(kOrderThreads) rt_order_count(const OrderParams o)
{
    __shared__ int h[kOrderCells];
    for (int c = threadIdx.x; c < kOrderCells; c += blockDim.x) h[c] = 0;
    __syncthreads();
    const int64_t per = (o.n + gridDim.x - 1) / gridDim.x;
    const int64_t a = (int64_t)blockIdx.x * per, b = min(o.n, a + per);
    for (int64_t i = a + threadIdx.x; i < b; i += blockDim.x) atomicAdd(&h[o.key[i]], 1);
    __syncthreads();
    for (int c = threadIdx.x; c < kOrderCells; c += blockDim.x)
        if (h[c]) atomicAdd(&o.cursor[c], h[c]);
}

// cell totals -> first column of each cell (one block; each thread scans a run of cells)
constexpr int kScanThreads = 512;
__global__ void __launch_bounds__(kScanThreads) rt_order_scan(const OrderParams o)
{
    constexpr int per = (kOrderCells + kScanThreads - 1) / kScanThreads;
    __shared__ int v[kScanThreads];
    const int t = threadIdx.x, c0 = t * per;
    int sum = 0;
    for (int c = c0; c < c0 + per && c < kOrderCells; ++c) sum += o.cursor[c];
    v[t] = sum;
    __syncthreads();
    for (int d = 1; d < kScanThreads; d <<= 1) { // inclusive scan of the runs' sums
        const int x = t >= d ? v[t - d] : 0;
        __syncthreads();
        v[t] += x;
        __syncthreads();
    }
    int run = v[t] - sum; // the cells before this thread's run
    for (int c = c0; c < c0 + per && c < kOrderCells; ++c) {
        const int total = o.cursor[c];
        o.cursor[c] = run;
        run += total;
    }
}

__global__ void __launch_bounds__(kOrderThreads) rt_order_place(const OrderParams o)
{
    __shared__ int h[kOrderCells]; // the block's count per cell, then its next column there
    for (int c = threadIdx.x; c < kOrderCells; c += blockDim.x) h[c] = 0;
    __syncthreads();
    const int64_t per = (o.n + gridDim.x - 1) / gridDim.x;
    const int64_t a = (int64_t)blockIdx.x * per, b = min(o.n, a + per);
    for (int64_t i = a + threadIdx.x; i < b; i += blockDim.x) atomicAdd(&h[o.key[i]], 1);
    __syncthreads();
    for (int c = threadIdx.x; c < kOrderCells; c += blockDim.x)
        if (h[c]) h[c] = atomicAdd(&o.cursor[c], h[c]);
    __syncthreads();
    for (int64_t i = a + threadIdx.x; i < b; i += blockDim.x) {
        const int pos = atomicAdd(&h[o.key[i]], 1);
        o.perm[pos] = (int32_t)i;
        o.iperm[i] = pos;
    }
}

} // namespace

int launch_order(const OrderParams &o, int grid, void *stream)
{
    if (o.n <= 0) return 0;
    cudaError_t e = cudaMemsetAsync(o.cursor, 0, kOrderCells * sizeof(int32_t), (cudaStream_t)stream);
    if (e != cudaSuccess) return (int)e;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>(grid, (o.n + kOrderThreads - 1) / kOrderThreads));
    rt_order_count<<<g, kOrderThreads, 0, (cudaStream_t)stream>>>(o);
    rt_order_scan<<<1, kScanThreads, 0, (cudaStream_t)stream>>>(o);
    rt_order_place<<<g, kOrderThreads, 0, (cudaStream_t)stream>>>(o);
    return (int)cudaGetLastError();
}

int launch_probe_red(float *buf, uint32_t n_vec, int grid, int iters, void *stream)
{
    if (!buf || n_vec == 0 || grid < 1 || iters < 1) return (int)cudaErrorInvalidValue;
    rt_probe_red_v4<<<grid, 256, 0, (cudaStream_t)stream>>>(buf, n_vec, iters);
    return (int)cudaGetLastError();
}

int launch_fold_tb(const TbParams &t, int grid_x, void *stream)
{
    if (t.tb_count < 1 || (t.part_per_block & 3)) return (int)cudaErrorInvalidValue;
    constexpr int kMaxGridY = 65535;
    for (int done = 0; done < t.tb_count; done += kMaxGridY) {
        TbParams c = t;
        c.tb_first = t.tb_first + done;
        c.tb_count = t.tb_count - done < kMaxGridY ? t.tb_count - done : kMaxGridY;
        rt_fold_tb<<<dim3(grid_x, c.tb_count), kTbThreads, 0, (cudaStream_t)stream>>>(c);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

int launch_tb_convert(const TbParams &t, int64_t time_stride, int64_t mode_stride, int shift,
                      unsigned long long *hist, uint32_t *u32, int max_grid, void *stream)
{
    if (t.tb_count < 1) return 0;
    constexpr int kMaxGridY = 65535;
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(max_grid, (t.S + kConvThreads - 1) / kConvThreads));
    for (int done = 0; done < t.tb_count; done += kMaxGridY) {
        TbParams c = t;
        c.tb_first = t.tb_first + done;
        c.tb_count = t.tb_count - done < kMaxGridY ? t.tb_count - done : kMaxGridY;
        rt_tb_convert<<<dim3(gx, c.tb_count), kConvThreads, 0, (cudaStream_t)stream>>>(c, time_stride, mode_stride, shift,
                                                                                      hist, u32);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

int launch_check_int64(const unsigned long long *hist, int64_t n, int32_t *status, int max_grid, void *stream)
{
    if (n <= 0) return 0;
    const int64_t need = ((n >> 1) + kCheckThreads - 1) / kCheckThreads;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, max_grid));
    rt_check_int64<<<grid, kCheckThreads, 0, (cudaStream_t)stream>>>(hist, n, status);
    return (int)cudaGetLastError();
}

int launch_bin_slices(const BinParams &b, int grid_x, size_t smem, void *stream)
{
    if (b.group > 0) {
        dim3 g(grid_x, (b.n_obs + b.group - 1) / b.group);
        rt_bin_slices_smem<<<g, 512, smem, (cudaStream_t)stream>>>(b);
    } else {
        if (b.j_first < 1 || b.j_count < 1 || b.j_first + b.j_count - 1 > b.n_obs) return (int)cudaErrorInvalidValue;
        // one slice per blockIdx.y, at most 65535 of them per launch
        constexpr int kMaxGridY = 65535;
        for (int done = 0; done < b.j_count; done += kMaxGridY) {
            BinParams c = b;
            c.j_first = b.j_first + done;
            c.j_count = b.j_count - done < kMaxGridY ? b.j_count - done : kMaxGridY;
            dim3 g(grid_x, c.j_count);
            rt_bin_slices<<<g, kFoldThreads, 0, (cudaStream_t)stream>>>(c);
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return (int)e;
        }
        return 0;
    }
    return (int)cudaGetLastError();
}

int launch_narrow_u32(const unsigned long long *src, uint32_t *dst, int64_t n, int shift, int max_grid, void *stream)
{
    if (n <= 0) return 0;
    if (shift < 0 || shift > 62 || max_grid < 1) return (int)cudaErrorInvalidValue;
    const int64_t per = (int64_t)kNarrowThreads * kNarrowUnroll;
    const int64_t need = (n + per - 1) / per;
    const int grid = (int)(need < max_grid ? need : max_grid);
    rt_narrow_u32<<<grid, kNarrowThreads, 0, (cudaStream_t)stream>>>(src, dst, n, shift);
    return (int)cudaGetLastError();
}

int bin_slices_set_smem(size_t smem)
{
    return (int)cudaFuncSetAttribute((const void *)rt_bin_slices_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int transport_set_smem(int precision, int sink, int obs, size_t smem)
{
    return kernel_set_smem(precision, 0, sink, obs, smem);
}

int transport_max_threads(int precision, int sink, int obs)
{
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, kernel_of(precision, 0, sink, obs)) != cudaSuccess) return 0;
    return a.maxThreadsPerBlock;
}

int transport_occupancy(int precision, int sink, int obs, int block, size_t smem, int *blocks_per_sm)
{
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel_of(precision, 0, sink, obs), block, smem);
}

static int set_and_occupancy(int precision, int kind, int obs, int block, size_t smem, int *blocks_per_sm)
{
    void *fn = kernel_of(precision, kind, 0, obs);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, block, smem);
    return (int)e;
}

int transport_batch_setup(int precision, int obs, int block, size_t smem, int *blocks_per_sm, int split)
{
    return set_and_occupancy(precision, split ? 10 : 1, obs, block, smem, blocks_per_sm);
}

int transport_batch_em_setup(int precision, int obs, int block, size_t smem, int *blocks_per_sm, int shist)
{
    return set_and_occupancy(precision, shist ? 11 : 2, obs, block, smem, blocks_per_sm);
}

int adjoint_occupancy(int precision, int obs, int block, size_t smem, int *blocks_per_sm)
{
    return set_and_occupancy(precision, 3, obs, block, smem, blocks_per_sm);
}

int adjoint_ring_occupancy(int precision, int obs, int block, size_t smem, int *blocks_per_sm)
{
    return set_and_occupancy(precision, 4, obs, block, smem, blocks_per_sm);
}

int adjoint_split_occupancy(int precision, int kind, int obs, int block, size_t smem, int *blocks_per_sm)
{
    return set_and_occupancy(precision, kind, obs, block, smem, blocks_per_sm);
}

int kernel_set_smem(int precision, int kind, int sink, int obs, size_t smem)
{
    return (int)cudaFuncSetAttribute(kernel_of(precision, kind, sink, obs), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

void *kernel_of(int precision, int kind, int sink, int obs)
{
    const bool d = precision == RTMC_FP64;
    switch (kind) {
    case 0: return d ? kernel_of_transport_f64(sink, obs) : kernel_of_transport_f32(sink, obs);
    case 1: case 2: return d ? kernel_of_batch_f64(kind == 2, obs) : kernel_of_batch_f32(kind == 2, obs);
    case 10: return d ? kernel_of_batch_f64(2, obs) : kernel_of_batch_f32(2, obs);
    case 11: return d ? kernel_of_batch_f64(3, obs) : kernel_of_batch_f32(3, obs);
    case 3: case 4: return d ? kernel_of_adjoint_f64(kind - 3, obs) : kernel_of_adjoint_f32(kind - 3, obs);
    case 8: case 9: return d ? kernel_of_adjoint_f64(kind - 6, obs) : kernel_of_adjoint_f32(kind - 6, obs);
    default: return d ? kernel_of_split_f64(kind, sink, obs) : kernel_of_split_f32(kind, sink, obs);
    }
}

} // namespace rtmc
