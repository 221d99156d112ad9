// Internal declarations shared by the host (tables.cpp, context.cpp) and device
// (transport.cu) translation units of librtmc.
#pragma once

#include "../../include/rtmc.h"

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

struct rtmc_tables {
    int32_t n_tables = 0;
    std::vector<double> cdf[4];
    std::vector<double> theta[4];
    rtmc_tables_info info{};
    uint64_t gen = 0; // identity of the knot set, used to cache device uploads
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
constexpr int kGuideBits = 16;   // Chen-Asau guide table of 2^16 + 1 entries per table
constexpr int kGuideN = 1 << kGuideBits;

// Device-side view of one precision's tables; R = float or double.
template <typename R> struct DevTables {
    const double *cdf[4];   // knots of u, FP64 in both precisions (search + interpolation offset)
    const R *theta[4];      // knot angles
    const R *slope[4];      // (theta[i+1]-theta[i]) / (cdf[i+1]-cdf[i]), built in FP64
    const int32_t *guide[4];
    int32_t n[4];
};

template <typename R> struct DevParams {
    int32_t d, frame, acoustics, src_dir;
    int32_t polarization, n_sub, n_obs, n_bnd;
    int32_t hist_shift, hist_smem, s_end, max_events;
    int64_t n_particles, pid0;
    uint32_t key0, key1;
    R src_pos[3];
    R src_lambda;
    R step[2];      // v * h per mode
    R inv_lam[2];   // mft / h (reciprocal of the per-sub-step scattering rate)
    R inv_q[2];     // Q / (omega h)
    int32_t scat_on[2], kill_on[2];
    R p2p, s2s;
    R vs_over_vp, vp_over_vs;
    R cos_half_pi;  // cos(pi/2) in working precision: the 2D source's z direction
    // observation axes (0 X, 1 Y, 2 Z, 3 PSI)
    int32_t ax_mode[4], ax_n[4], ax_off[4], ax_uniform[4];
    R ax_lo[4], ax_hi[4], ax_inv_w[4];
    int64_t ax_stride[4];
    int64_t time_stride, mode_stride, hist_len;
    int32_t n_edges;
    int32_t bnd_dir[RTMC_MAX_BND], bnd_absorb[RTMC_MAX_BND];
    R bnd_val[RTMC_MAX_BND];
    const R *edges;  // all binned/range edges, concatenated
    const R *zoe;    // [2][RTMC_ZOE_N]: E_Rpp then E_Rsvsv
    DevTables<R> tab;
    unsigned long long *hist;
    unsigned long long *stats;  // [8]
    int32_t *status;
    double *trace;  // optional [n_particles][16] final particle states
};

// Launch wrappers (transport.cu).  Return a cudaError_t value.
int launch_transport_f32(const DevParams<float> &p, int grid, int block, size_t smem, void *stream);
int launch_transport_f64(const DevParams<double> &p, int grid, int block, size_t smem, void *stream);
int transport_occupancy(int precision, int smem_hist, int block, size_t smem, int *blocks_per_sm);
int transport_set_smem(int precision, int smem_hist, size_t smem);

} // namespace rtmc
