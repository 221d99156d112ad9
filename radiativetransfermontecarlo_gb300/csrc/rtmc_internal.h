// Internal declarations shared by the host (tables.cpp, context.cpp) and device
// (kernels.cu, fold.cu, noalloc.cu) translation units of librtmc.
#pragma once

#include "../../include/rtmc.h"

#include <atomic>
#include <mutex>
#include <cstdint>
#include <string>
#include <vector>

struct rtmc_tables {
    int32_t n_tables = 0;
    std::vector<double> cdf[4];
    std::vector<double> theta[4];
    rtmc_tables_info info{};
    uint64_t gen = 0; // identity of the knot set, used to cache device uploads
    // host images of the device layout per precision (0 FP32, 1 FP64), built on the first
    // upload and reused: an upload is then one host-to-device copy
    mutable std::mutex image_mu;
    mutable std::vector<unsigned char> image[2];
    mutable bool image_pinned[2] = {false, false}; // page-locked (cudaHostRegister) for async uploads
};

namespace rtmc {

extern thread_local std::string g_thread_error;
int fail(std::string *slot, int code, const std::string &msg);
int validate_tables(const rtmc_tables *t, std::string *err);

inline uint64_t next_generation()
{
    static std::atomic<uint64_t> g{1};
    return g.fetch_add(1);
}

constexpr int kMaxEdges = 4096;  // all axes together, staged in shared memory
// Chen-Asau guide table of 2^b + 1 entries per table, b = ceil(log2(knots)) in [16, 20]:
// about one knot per guide cell, so the search is a guide load and at most a step or two
constexpr int kGuideMinBits = 16, kGuideMaxBits = 20;
inline int guide_bits(size_t n_knots)
{
    int b = kGuideMinBits;
    while (b < kGuideMaxBits && ((size_t)1 << b) < n_knots) ++b;
    return b;
}

// One knot of an inverse-CDF table: u, theta / pi and (theta[i+1] - theta[i]) /
// (pi (u[i+1] - u[i])), built in FP64.  FP64 tables keep u as a double; FP32 tables keep
// it as an unevaluated float sum ch + cl, which compares with a float u and gives the
// interpolation offset (u - ch) - cl without FP64 arithmetic.  16 bytes for FP32, so the
// interpolation reads one vector.
template <typename R> struct Knot {
    double c;
    R th, sl;
};
template <> struct alignas(16) Knot<float> {
    float ch, cl;
    float th, sl;
};

// Device-side view of one precision's tables; R = float or double.
template <typename R> struct DevTables {
    const Knot<R> *knot[4];
    const int32_t *guide[4];
    int32_t n[4];
    int32_t gbits[4];
};

template <typename R> struct DevParams {
    int32_t d, frame, acoustics, src_dir;
    int32_t polarization, n_sub, n_obs, n_bnd;
    int32_t hist_shift, sink, s_end, max_events;
    int32_t ring_cap;  // trajectory segments per lane in the shared-memory ring
    int32_t event_major; // 1: one particle per thread, events and their observations in turn
    int32_t obs_kind;  // 0 general, 1 cartesian linear, 2 radius only
    int32_t bin32;     // FP64 radius-only observation kernel: FP32 estimate first, FP64 near an edge
    float r32_iw, r32_a0; // 1 / width and -lo / width of axis 0 in FP32 (the estimate)
    int32_t radial_3d; // radius-only path: 1 = |x|, 0 = |(x, y)|
    int32_t ax_nbe[4]; // bins of a binned axis, 1 for a range-checked or ignored axis
    R ax_a0;           // -lo / width of axis 0 (radius-only path)
    int64_t n_particles, pid0;
    uint32_t key0, key1;
    R src_pos[3];
    R src_lambda;
    R step[2];      // v * h per mode
    R inv_lam[2];   // mft / h (reciprocal of the per-sub-step scattering rate)
    R inv_q[2];     // Q / (omega h)
    double inv_lam64[2], inv_q64[2]; // the same in FP64 (settles FP32 counts near an integer)
    int32_t scat_on[2], kill_on[2];
    R p2p, s2s;     // FP32: rounded down, so u > p2p in float equals u > p2p in FP64 for float u
    R vs_over_vp, vp_over_vs;
    R cos_half_pi;  // cos(pi/2) in working precision: the 2D source's z direction
    // observation axes (0 X, 1 Y, 2 Z, 3 PSI)
    int32_t ax_mode[4], ax_n[4], ax_off[4], ax_uniform[4];
    R ax_lo[4], ax_hi[4], ax_inv_w[4];
    int64_t ax_stride[4];
    int32_t ax_stride32[4];  // in-slice strides (a time slice holds < 2^31 bins)
    // FP32 cartesian observation kernel: the float bit patterns of the bin counts
    // (unsigned compares against a coordinate's bits), and 0x4B000000 times the sum of the
    // three in-slice strides, mod 2^32 (taken off the direction offset once per segment)
    int32_t ax_nbits[4];
    int32_t cart_bias;
    int64_t time_stride, mode_stride, hist_len;
    int32_t n_edges;
    int32_t bnd_dir[RTMC_MAX_BND], bnd_absorb[RTMC_MAX_BND];
    R bnd_val[RTMC_MAX_BND];
    // source shape (initializeParticle.m:14-148)
    int32_t src_type, src_aperture, src_radial_n, pad_src;
    R src_n[3], src_u[3], src_v[3], src_ext[2];
    const R *edges;  // all binned/range edges, concatenated
    const R *zoe;    // [2][RTMC_ZOE_N]: E_Rpp then E_Rsvsv, then the radial source table
    const R *src_radial;  // [2][src_radial_n]: CDF knots then radii (inside the zoe block)
    DevTables<R> tab;
    unsigned long long *hist;
    unsigned long long *stats;  // [8]
    int32_t *status;
    double *trace;  // optional [n_particles][16] final particle states
    int32_t *obs_idx;  // index sink: [n_obs][obs_rows] in-slice bin | mode << 30, or -1
    // split schedule on the index path: the columns of the index array hold the particles in
    // the order of their starting directions (okey: a direction cell per particle, written
    // by rt_events; perm: column -> particle; iperm: particle -> column), so that a fold
    // block's particles stay close together while they fly out; null: column = particle
    int32_t *okey;
    int32_t *perm, *iperm;
    int64_t obs_rows;
    // split schedule (rt_events, then rt_observe): seg_cap records per particle in segs, its
    // trajectory segments followed by end records (a particle with more than seg_cap - 2
    // segments gets end records only, is listed in ovf_list and rerun by rt_transport_list)
    void *segs;
    void *seg_th;  // split adjoint: [n][seg_cap] theta / pi of the scattering that starts each segment, or -1
    int32_t *ovf_list;
    uint32_t *ovf_count;
    int32_t seg_cap, split;
    // instants obs_j0..obs_j1 (inclusive) that rt_observe and rt_transport_list bin into
    // the index array (0, 0: all); the rerun counts its events only in the range from 1
    int32_t obs_j0, obs_j1;
    // rt_events zeroes clear_words 64-bit words at `clear` as it goes (the histogram, on
    // the first chunk of a split run), so no separate memset pass precedes the transport
    unsigned long long *clear;
    int64_t clear_words;
};

// Parameters of the slice fold (rt_bin_slices*).
struct BinParams {
    const int32_t *idx;
    int64_t rows;          // row length of the index array
    int64_t n;             // particles in this chunk
    int32_t n_obs, n_modes, slice_bins, group;
    int64_t time_stride, mode_stride, part_per_block;
    int32_t hist_shift;
    unsigned long long *hist;
    int32_t j_first, j_count; // rt_bin_slices: slices j_first .. j_first + j_count - 1 (1-based)
};

// Parameters of the time-blocked fold (rt_fold_tb) and its conversion (rt_tb_convert).
// The accumulator holds FP32 counts in blocks of 4 consecutive observation instants:
// acc[(tb * S + s) * 4 + r] counts in-slice bin s (s = in-mode bin + mode * slice_bins) at
// instant j = 4 tb + r + 1.  A bin of one instant receives at most one count per particle,
// so FP32 counts are exact while the particles number fewer than 2^24.
struct TbParams {
    const int32_t *idx;       // index array: instant j in row j - 1
    int64_t rows;             // row stride
    int64_t n;                // particles in this chunk
    int64_t part_per_block;   // multiple of 4
    int64_t S;                // slice_bins * n_modes
    int32_t n_obs, slice_bins;
    int32_t tb_first, tb_count; // t-blocks [tb_first, tb_first + tb_count)
    float *acc;               // [t-block - acc_tb0][S][4] FP32 counts
    int32_t acc_tb0;          // the t-block at the start of acc (0, or a rolling accumulator's turn)
    int32_t rezero;           // the conversion writes zeros back (a rolling accumulator)
};

// One work item of a batched run: particles [first, first + count) of instance inst.
struct BatchItem {
    int32_t inst, pad;
    int64_t first, count;
};

// Early copy of host-output calls: the first observation pass covers the instants of the
// copy groups that hold at least this percent of them (rtmc_set_early_copy).  On the 3D
// elastic workload's uint32 output (1e7 particles, 250 instants, 3.47 GB to the host), the
// median call took 26.7 ms with one observation pass and 26.9 / 26.5 / 26.1 / 25.0 / 25.0 /
// 25.5 ms with 5 / 10 / 20 / 35 / 50 / 70 %: the copies slow down while the fold runs
// (its L2 reductions), so they gain most when they overlap the second observation pass.
constexpr int kEarlyCopyPercent = 40;

// Threads per block of rt_transport_batch_split (one block per SM).
#ifndef RTMC_BATCH_SPLIT_THREADS
#define RTMC_BATCH_SPLIT_THREADS 512
#endif
constexpr int kBatchSplitThreads = RTMC_BATCH_SPLIT_THREADS;

template <typename R> struct BatchArgs {
    const DevParams<R> *params; // per instance (device)
    const BatchItem *items;     // sorted by expected cost, largest first
    int32_t n_items, ring_cap;
    int32_t *counter;           // next work item
    unsigned long long *hists;  // n x hist_len int64, instance-major
    int64_t hist_len;
    const R *edges;             // the grid the instances share
    int32_t n_edges, obs_kind;
    unsigned long long *stats;  // [8]
    int32_t *status;
    // rt_transport_batch_split: each block's segment records for one work item
    void *scratch;              // [gridDim.x][scratch_stride] in R
    int64_t scratch_stride;     // R values per block: work-item size x the largest seg_cap x 8
};

// Score-function adjoint replay (rt_adjoint): the per-particle score of parameter q up to
// observation j is A_q(j) + b_obs[q] * j, where A_q gains dlogsigma_q(theta_i) + a_inc[q]
// at each scattering; grad_q = sum over particles and j of adjoint[bin] * score_q(j).
// The weights, the per-particle score and the per-segment sums use the transport's
// precision; grad accumulates in FP64.
struct AdjointArgs {
    const void *adjoint;      // [hist_len] d L / d count, in the transport's precision
    const double *dlogsigma;  // [n_params][n_theta] on a uniform grid of theta / pi in [0, 1]
    const float *dlogsigma_f; // the same in FP32 (FP32 replay)
    int32_t n_params, n_theta;
    double a_inc[RTMC_MAX_PARAMS];
    double b_obs[RTMC_MAX_PARAMS];
    float a_inc_f[RTMC_MAX_PARAMS];
    double *partial;          // [gridDim.x][n_params] block sums
    double *partial_list;     // split replay: block sums of the overflow reruns (rt_adjoint_list)
};

// Launch shape of the split schedule (rt_events, rt_observe, rt_transport_list).
// A counting sort of particles by direction cell (kOrderCells cells), between rt_events
// and rt_observe: per-block cell counts, the cells' offsets, then each block places its
// particles.  Order within a cell is not fixed; the folds' integer sums do not depend on it.
constexpr int kOrderCells = 512;
struct OrderParams {
    const int32_t *key; // [n] cells
    int32_t *perm, *iperm;
    int32_t *cursor;    // [kOrderCells] cell totals, then the next free column of each cell
    int64_t n;
};

struct SplitLaunch {
    int part; // 0: all kernels; 1: rt_events and the order sort; 2: rt_observe and rt_transport_list
    int grid_events, grid_observe, block_observe, grid_list;
    size_t smem_events, smem_observe;
    void *mid_event; // optional cudaEvent_t recorded after rt_events
    OrderParams order; // order.n > 0: sort the chunk's particles before rt_observe
    int grid_order;
};

// Launch wrappers (kernels.cu, fold.cu).  Return a cudaError_t value.
int launch_split_f32(const DevParams<float> &p, const SplitLaunch &l, void *stream);
int launch_split_f64(const DevParams<double> &p, const SplitLaunch &l, void *stream);
// kind 5: rt_events, 6: rt_observe (sink, obs), 7: rt_transport_list
void *kernel_of_split_f32(int kind, int sink, int obs);
void *kernel_of_split_f64(int kind, int sink, int obs);
// kernel_of(precision, kind, sink, obs): the kernel function of a transport (kind 0, with
// its sink and observation path), batch (1), event-major batch (2), adjoint (3), ring
// adjoint (4), split-schedule events (5), observations (6, with its sink), overflow
// rerun (7), split replay (8, 9), split batch (10) or shared-histogram event-major batch
// (11) variant; kernel_set_smem sets its dynamic shared-memory limit.
void *kernel_of_transport_f32(int sink, int obs);
void *kernel_of_transport_f64(int sink, int obs);
// which: 0 rt_transport_batch, 1 rt_transport_batch_em (device histogram),
// 2 rt_transport_batch_split, 3 rt_transport_batch_em (shared-memory histogram)
void *kernel_of_batch_f32(int which, int obs);
void *kernel_of_batch_f64(int which, int obs);
// which: 0 rt_adjoint, 1 rt_adjoint_ring, 2 rt_observe_adj, 3 rt_adjoint_list
void *kernel_of_adjoint_f32(int which, int obs);
void *kernel_of_adjoint_f64(int which, int obs);
void *kernel_of(int precision, int kind, int sink, int obs);
int kernel_set_smem(int precision, int kind, int sink, int obs, size_t smem);
int launch_transport_f32(const DevParams<float> &p, int grid, int block, size_t smem, void *stream);
int launch_transport_f64(const DevParams<double> &p, int grid, int block, size_t smem, void *stream);
int transport_occupancy(int precision, int sink, int obs, int block, size_t smem, int *blocks_per_sm);
int launch_adjoint_f32(const DevParams<float> &p, const AdjointArgs &a, int grid, int block, size_t smem, void *stream);
int launch_adjoint_f64(const DevParams<double> &p, const AdjointArgs &a, int grid, int block, size_t smem, void *stream);
int adjoint_occupancy(int precision, int obs, int block, size_t smem, int *blocks_per_sm);
int launch_adjoint_ring_f32(const DevParams<float> &p, const AdjointArgs &a, int grid, int block, size_t smem, void *stream);
int launch_adjoint_ring_f64(const DevParams<double> &p, const AdjointArgs &a, int grid, int block, size_t smem, void *stream);
int adjoint_ring_occupancy(int precision, int obs, int block, size_t smem, int *blocks_per_sm);
// the split replay's kernels: kind 8 rt_observe_adj, 9 rt_adjoint_list (sets the dynamic shared memory)
int adjoint_split_occupancy(int precision, int kind, int obs, int block, size_t smem, int *blocks_per_sm);
constexpr int kAdjointRingParams = 4; // parameters the ring-based adjoint carries
constexpr int kAdjointThreads = 256;
int transport_set_smem(int precision, int sink, int obs, size_t smem);
int transport_max_threads(int precision, int sink, int obs);
int launch_bin_slices(const BinParams &b, int grid_x, size_t smem, void *stream);
// n histogram bins as uint32 counts (value >> shift, saturating), at most max_grid blocks
int launch_narrow_u32(const unsigned long long *src, uint32_t *dst, int64_t n, int shift, int max_grid, void *stream);
// time-blocked fold of one chunk over t-blocks [tb_first, tb_first + tb_count)
// the L2 vector-reduction probe (rt_probe_red_v4): grid blocks of 256 threads, iters each
int launch_probe_red(float *buf, uint32_t n_vec, int grid, int iters, void *stream);
int launch_fold_tb(const TbParams &t, int grid_x, void *stream);
// the particle order of OrderParams (three kernels)
int launch_order(const OrderParams &o, int grid, void *stream);
// acc t-blocks [tb_first, tb_first + tb_count) -> the int64 histogram (count << shift) and,
// when u32 is non-null, the uint32 counts; slice 0 (t = 0, never observed) is zeroed with
// t-block 0
int launch_tb_convert(const TbParams &t, int64_t time_stride, int64_t mode_stride, int shift,
                      unsigned long long *hist, uint32_t *u32, int max_grid, void *stream);
// sets bit 1 of *status when a bin of the n-bin histogram is >= 2^63 (out of int64 range)
int launch_check_int64(const unsigned long long *hist, int64_t n, int32_t *status, int max_grid, void *stream);
// a histogram of this problem may hold bins of 2^63 or more (n_particles << hist_shift >= 2^63)
inline bool may_exceed_int64(const rtmc_problem *P)
{
    return P->hist_shift >= 1 && P->n_particles >= ((int64_t)1 << (63 - P->hist_shift));
}
// split: the split kernel (rt_transport_batch_split) instead of the lockstep ring kernel
int launch_transport_batch_f32(const BatchArgs<float> &a, int grid, int block, size_t smem, void *stream, int split);
int launch_transport_batch_f64(const BatchArgs<double> &a, int grid, int block, size_t smem, void *stream, int split);
int transport_batch_setup(int precision, int obs, int block, size_t smem, int *blocks_per_sm, int split);
// shist: the event-major kernel with the shared-memory histogram (else 64-bit device atomics)
int launch_transport_batch_em_f32(const BatchArgs<float> &a, int grid, int block, size_t smem, void *stream, int shist);
int launch_transport_batch_em_f64(const BatchArgs<double> &a, int grid, int block, size_t smem, void *stream, int shist);
int transport_batch_em_setup(int precision, int obs, int block, size_t smem, int *blocks_per_sm, int shist);
int bin_slices_set_smem(size_t smem);
// device address of the static scratch of rtmc_forward_noalloc (noalloc.cu); device current
int static_scratch(int device, unsigned char **ptr, size_t *bytes);
enum { kSinkSmem = 0, kSinkGlobal = 1, kSinkIndex = 2 };

} // namespace rtmc
