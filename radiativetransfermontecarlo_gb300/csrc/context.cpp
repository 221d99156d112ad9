// Context, device memory and the rtmc_forward entry points of librtmc.
//
// rtmc_forward replaces the packet x time loop of radiativeTransfer.m:40-158: it stages
// the inverse-CDF tables (host FP64 knots -> device knots + slopes + Chen-Asau guide
// table), the observation edges and the Zoeppritz tables, zeroes the int64 histogram,
// launches the fused transport kernel and copies the histogram back.
#include "rtmc_internal.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <numeric>
#include <cmath>
#include <limits>
#include <cstring>
#include <string>
#include <vector>

using namespace rtmc;

// NVTX range over a scope: the phases of a call show by name in a timeline profiler (the
// header-only NVTX v3 does nothing unless a tool is attached)
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int grow(size_t bytes)
    {
        if (bytes <= cap) return 0;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) return (int)e;
        cap = bytes;
        return 0;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct rtmc_context {
    int device = 0;
    int num_sms = 0;
    int max_smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_k0 = nullptr, ev_k1 = nullptr, ev_k2 = nullptr, ev_end = nullptr, ev_km = nullptr;
    cudaEvent_t ev_kc = nullptr; // before the time-blocked conversion
    std::string err;
    DevBuf hist, tabs, aux, stats, flush, trace, idx, adj, partial;
    DevBuf narrow; // uint32 copy of the histogram (rtmc_forward_u32)
    DevBuf segs, ovf; // split schedule: trajectory segment records, overflow list
    DevBuf order;     // the particle order of the index path: keys, perm, iperm, cell cursors
    DevBuf segth;     // split replay of the gradient: the scattering angle of each segment
    DevBuf tbacc;               // time-blocked FP32 fold accumulator
    uint64_t tabs_gen = 0;
    int tabs_prec = -1;
    DevTables<float> tf{};
    DevTables<double> td{};
    int64_t hist_len = 0;
    bool hist_may_exceed_int64 = false; // the last histogram may hold bins >= 2^63
    double last_kernel_ms = 0;
    int last_launches = 0;
    int cache_tables = 1;
    int opt_block = 0, opt_ring = 0, opt_index_mb = 0;
    // transport / fold pipeline over particle chunks (index sink): a second stream and
    // per-chunk events, created on first use
    int opt_chunks = 0, opt_k1_bps = 0;
    int opt_event_major = -1; // -1 automatic, 0 two-cursor batches, 1 one particle per thread, 2 split
    int opt_fold = 0;         // 0 automatic, 1 64-bit slice fold, 2 time-blocked FP32 fold, 3 the same, rolling
    int opt_bin32 = 1;        // FP64 radius-only observations through an exact FP32 estimate
    int opt_early_copy = kEarlyCopyPercent; // host-output calls: copies start after the first instants (percent)
    int opt_order = 1;        // index path: particles binned in the order of their starting directions
    static constexpr int kPipe = 32;
    cudaStream_t fold_stream = nullptr;
    cudaEvent_t ev_a0[kPipe] = {}, ev_a1[kPipe] = {}, ev_b0[kPipe] = {}, ev_b1[kPipe] = {};
};

namespace {

int cuda_fail(rtmc_context *c, cudaError_t e, const char *what)
{
    return fail(c ? &c->err : nullptr, RTMC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                                                                                               \
    do {                                                                                                             \
        cudaError_t _e = (call);                                                                                     \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, what);                                                      \
    } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ---- device layout of one inverse-CDF table: interleaved knots, then the guide ----------

// bytes of one staged table: n knots (256-aligned), then 2^b + 1 guide entries
template <typename R> size_t table_bytes(size_t n)
{
    return align_up(n * sizeof(Knot<R>), 256) + align_up((((size_t)1 << guide_bits(n)) + 1) * sizeof(int32_t), 256);
}

// knots [k0, k0 + m) of table (c, th): u, theta / pi and the slope, built in FP64
template <typename R> void fill_knots(const std::vector<double> &c, const std::vector<double> &th, size_t k0, size_t m,
                                      Knot<R> *out)
{
    const double ip = 1.0 / M_PI;
    const size_t n = c.size();
    for (size_t k = 0; k < m; ++k) {
        const size_t q = k0 + k;
        if constexpr (sizeof(R) == 4) {
            out[k].ch = (float)c[q];
            out[k].cl = (float)(c[q] - (double)out[k].ch);
        } else {
            out[k].c = c[q];
        }
        out[k].th = (R)(th[q] * ip);
        out[k].sl = (q + 1 < n) ? (R)((th[q + 1] - th[q]) * ip / (c[q + 1] - c[q])) : (R)0;
    }
}

// guide entries [j0, j0 + m): the last knot index with c <= j / 2^b (a walk that resumes at *k)
inline void fill_guide(const std::vector<double> &c, int bits, int64_t j0, int64_t m, size_t *k, int32_t *out)
{
    const size_t n = c.size();
    const double G = (double)((int64_t)1 << bits);
    for (int64_t jj = 0; jj < m; ++jj) {
        const double target = (double)(j0 + jj) / G;
        while (*k + 1 <= n - 2 && c[*k + 1] <= target) ++*k;
        out[jj] = (int32_t)*k;
    }
}

// table i into a host image at `host` whose device copy starts at `dev`
template <typename R> void stage_table(const std::vector<double> &c, const std::vector<double> &th, unsigned char *host,
                                       unsigned char *dev, DevTables<R> *dt, int i)
{
    const size_t n = c.size();
    const int bits = guide_bits(n);
    fill_knots<R>(c, th, 0, n, reinterpret_cast<Knot<R> *>(host));
    const size_t go = align_up(n * sizeof(Knot<R>), 256);
    size_t k = 0;
    fill_guide(c, bits, 0, ((int64_t)1 << bits) + 1, &k, reinterpret_cast<int32_t *>(host + go));
    dt->knot[i] = reinterpret_cast<const Knot<R> *>(dev);
    dt->guide[i] = reinterpret_cast<const int32_t *>(dev + go);
    dt->n[i] = (int32_t)n;
    dt->gbits[i] = bits;
}

// Stage the tables in precision R (knots, guide) in the context's table buffer.
template <typename R> int upload_tables(rtmc_context *ctx, const rtmc_tables *t, DevTables<R> *dt)
{
    size_t off[4], total = 0;
    for (int i = 0; i < t->n_tables; ++i) {
        off[i] = total;
        total += table_bytes<R>(t->cdf[i].size());
    }
    if (ctx->tabs.grow(total)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for tables failed");
    unsigned char *base = static_cast<unsigned char *>(ctx->tabs.p);
    std::lock_guard<std::mutex> lock(t->image_mu);
    const int k = sizeof(R) == 4 ? 0 : 1;
    std::vector<unsigned char> &host = t->image[k];
    const bool have = host.size() == total;
    if (!have) {
        if (t->image_pinned[k]) cudaHostUnregister(host.data());
        t->image_pinned[k] = false;
        host.assign(total, 0);
    }
    for (int i = 0; i < t->n_tables; ++i) {
        if (!have) {
            stage_table<R>(t->cdf[i], t->theta[i], host.data() + off[i], base + off[i], dt, i);
        } else {
            const size_t n = t->cdf[i].size();
            dt->knot[i] = reinterpret_cast<const Knot<R> *>(base + off[i]);
            dt->guide[i] = reinterpret_cast<const int32_t *>(base + off[i] + align_up(n * sizeof(Knot<R>), 256));
            dt->n[i] = (int32_t)n;
            dt->gbits[i] = guide_bits(n);
        }
    }
    for (int i = t->n_tables; i < 4; ++i) {
        dt->knot[i] = nullptr;
        dt->guide[i] = nullptr;
    }
    // page-lock the image once, so that every later upload is one copy at the link's rate
    // (a pageable copy is staged through a bounce buffer); unpinned it still works
    if (!t->image_pinned[k]) {
        t->image_pinned[k] = cudaHostRegister(host.data(), total, cudaHostRegisterPortable) == cudaSuccess;
        if (!t->image_pinned[k]) cudaGetLastError();
    }
    CK(cudaMemcpyAsync(ctx->tabs.p, host.data(), total, cudaMemcpyHostToDevice, ctx->stream), "table upload");
    CK(cudaStreamSynchronize(ctx->stream), "table upload");
    return RTMC_OK;
}

int check_problem(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t)
{
    std::string *e = &ctx->err;
    if (P->d != 2 && P->d != 3) return fail(e, RTMC_ERR_ARG, "dimension must be 2 or 3");
    if (P->frame < 0 || P->frame > 2) return fail(e, RTMC_ERR_ARG, "frame must be cartesian, cylindrical or spherical");
    if (P->precision != RTMC_FP32 && P->precision != RTMC_FP64) return fail(e, RTMC_ERR_ARG, "unknown precision");
    if (P->src_dir < 0 || P->src_dir > 2) return fail(e, RTMC_ERR_ARG, "source direction must be uniform, outgoing or upper");
    if (P->n_sub < 1 || P->n_obs < 1) return fail(e, RTMC_ERR_ARG, "n_sub and n_obs must be >= 1");
    if ((int64_t)P->n_sub * P->n_obs >= (int64_t)1 << 30)
        return fail(e, RTMC_ERR_ARG, "n_sub * n_obs must stay below 2^30 sub-steps");
    if (P->n_particles < 0 || P->pid0 < 0) return fail(e, RTMC_ERR_ARG, "particle count and first id must be >= 0");
    if (P->hist_shift < 0 || P->hist_shift > 62) return fail(e, RTMC_ERR_ARG, "hist_shift must be in [0, 62]");
    // one bin of one time slice receives at most one count per particle: its unsigned
    // 64-bit fixed-point sum cannot wrap while n_particles < 2^(64 - hist_shift)
    if (P->hist_shift >= 2 && P->n_particles >= ((int64_t)1 << (64 - P->hist_shift)))
        return fail(e, RTMC_ERR_ARG,
                    "n_particles << hist_shift could wrap a 64-bit histogram bin: keep n_particles below 2^(64 - hist_shift)");
    if (P->max_events < 0) return fail(e, RTMC_ERR_ARG, "max_events must be >= 0 (0: automatic)");
    if (P->n_bnd < 0 || P->n_bnd > RTMC_MAX_BND) return fail(e, RTMC_ERR_ARG, "at most 4 boundaries");
    for (int b = 0; b < P->n_bnd; ++b) {
        if (P->bnd_dir[b] < 1 || P->bnd_dir[b] > 4)
            return fail(e, RTMC_ERR_ARG, "boundary dir must be 1, 2, 3 (planes) or 4 (cylinder)");
        if (!std::isfinite(P->bnd_val[b])) return fail(e, RTMC_ERR_ARG, "boundary position must be finite");
        if (P->bnd_dir[b] == 4 && !(P->bnd_val[b] > 0)) return fail(e, RTMC_ERR_ARG, "cylinder radius must be positive");
    }
    if (P->src_type != RTMC_SOURCE_POINT && P->src_type != RTMC_SOURCE_PLANE)
        return fail(e, RTMC_ERR_ARG, "source type must be point or plane");
    if (P->src_type == RTMC_SOURCE_PLANE) {
        if (P->d != 3) return fail(e, RTMC_ERR_ARG, "plane sources are 3D only");
        if (P->src_aperture != RTMC_APERTURE_RECTANGLE && P->src_aperture != RTMC_APERTURE_CIRCLE)
            return fail(e, RTMC_ERR_ARG, "plane-source aperture must be rectangle or circle");
        const double *vs[3] = {P->src_normal, P->src_u, P->src_v};
        for (int i = 0; i < 3; ++i) {
            const double nn = vs[i][0] * vs[i][0] + vs[i][1] * vs[i][1] + vs[i][2] * vs[i][2];
            if (!(std::fabs(nn - 1.0) < 1e-9)) return fail(e, RTMC_ERR_ARG, "plane-source n, u, v must be unit vectors");
        }
        for (int i = 0; i < 2; ++i)
            if (!std::isfinite(P->src_extent[i]) || P->src_extent[i] < 0)
                return fail(e, RTMC_ERR_ARG, "plane-source extent must be finite and >= 0");
    }
    if (P->src_radial_n != 0) {
        if (P->src_type != RTMC_SOURCE_POINT) return fail(e, RTMC_ERR_ARG, "a radial profile applies to point sources");
        if (P->src_radial_n < 2 || P->src_radial_n > RTMC_MAX_RADIAL || !P->src_radial_cdf || !P->src_radial_r)
            return fail(e, RTMC_ERR_ARG, "a radial source profile needs 2 to 65536 knots");
        for (int k = 0; k < P->src_radial_n; ++k) {
            if (!std::isfinite(P->src_radial_cdf[k]) || !std::isfinite(P->src_radial_r[k]) || P->src_radial_r[k] < 0)
                return fail(e, RTMC_ERR_ARG, "radial source knots must be finite, radii >= 0");
            if (k && !(P->src_radial_cdf[k] > P->src_radial_cdf[k - 1]))
                return fail(e, RTMC_ERR_ARG, "radial source CDF knots must be strictly increasing");
        }
    }
    const int nm = P->acoustics ? 1 : 2;
    for (int m = 0; m < nm; ++m) {
        if (!(P->v[m] > 0) || !std::isfinite(P->v[m])) return fail(e, RTMC_ERR_ARG, "propagation speeds must be positive");
        if (!(P->mft[m] > 0)) return fail(e, RTMC_ERR_ARG, "mean free times must be positive (Inf disables scattering)");
        if (!(P->qrate[m] >= 0) || !std::isfinite(P->qrate[m])) return fail(e, RTMC_ERR_ARG, "qrate must be finite and >= 0");
    }
    if (!(P->h > 0) || !std::isfinite(P->h)) return fail(e, RTMC_ERR_ARG, "sub-step h must be positive");
    if (!std::isfinite(P->src_lambda) || P->src_lambda < 0) return fail(e, RTMC_ERR_ARG, "source lambda must be >= 0");
    // the knots were validated when the handle was made (rtmc_tables_build and
    // rtmc_tables_from_knots; a handle never changes): no per-call scan of the ~40 MB
    if (!t) return fail(e, RTMC_ERR_NOTABLES, "tables handle is NULL");
    if (t->n_tables != (P->acoustics ? 1 : 4))
        return fail(e, RTMC_ERR_NOTABLES, "acoustic problems need 1 table, elastic problems 4");
    if (P->hist_len <= 0) return fail(e, RTMC_ERR_ARG, "hist_len must be positive");
    int64_t maxidx = (int64_t)P->n_obs * P->time_stride + (nm - 1) * P->mode_stride;
    int tot_edges = 0;
    for (int a = 0; a < 4; ++a) {
        const int am = P->axis_mode[a];
        if (am < 0 || am > 2) return fail(e, RTMC_ERR_ARG, "axis mode must be ignored, range or binned");
        if (am == RTMC_AXIS_IGNORED) continue;
        const int ne = P->axis_nedges[a];
        if (ne < 2 || !P->axis_edges[a]) return fail(e, RTMC_ERR_ARG, "an observed axis needs at least 2 edges");
        if (am == RTMC_AXIS_RANGE && ne != 2) return fail(e, RTMC_ERR_ARG, "a range-checked axis has exactly 2 edges");
        for (int k = 0; k < ne; ++k)
            if (std::isnan(P->axis_edges[a][k])) return fail(e, RTMC_ERR_ARG, "bin edges must not be NaN");
        for (int k = 1; k < ne; ++k)
            if (!(P->axis_edges[a][k] > P->axis_edges[a][k - 1]))
                return fail(e, RTMC_ERR_ARG, "bin edges must be strictly increasing");
        tot_edges += ne;
        if (am == RTMC_AXIS_BINNED) {
            if (P->axis_stride[a] < 0) return fail(e, RTMC_ERR_ARG, "negative stride");
            maxidx += (int64_t)(ne - 2) * P->axis_stride[a];
        }
    }
    if (tot_edges > kMaxEdges) return fail(e, RTMC_ERR_ARG, "too many bin edges (4096 at most over all axes)");
    if (P->time_stride < 0 || P->mode_stride < 0 || maxidx >= P->hist_len)
        return fail(e, RTMC_ERR_ARG, "histogram strides exceed hist_len");
    int64_t in_slice = 0;
    for (int a = 0; a < 4; ++a)
        if (P->axis_mode[a] == RTMC_AXIS_BINNED) in_slice += (int64_t)(P->axis_nedges[a] - 2) * P->axis_stride[a];
    if (in_slice >= ((int64_t)1 << 31) - 1) return fail(e, RTMC_ERR_ARG, "one time slice must hold fewer than 2^31 bins");
    return RTMC_OK;
}

// True when [lo, hi] holds every value coordinate `axis` of the frame can take (an
// integrated axis whose check always passes): +-Inf, the azimuth atan2 in [-pi, pi], sin of
// the 3D elevation in [-1, 1], and the direction variable (observeTime.m:21-24): dir_z in
// [-1, 1] in 3D, acos(dir_z) in [0, pi] in 2D.
bool range_covers_axis(int frame, int d, int axis, double lo, double hi)
{
    if (lo == -INFINITY && hi == INFINITY) return true;
    if (axis == 1 && frame != RTMC_FRAME_CARTESIAN) return lo <= -M_PI && hi >= M_PI;
    if (axis == 2 && frame == RTMC_FRAME_SPHERICAL && d == 3) return lo <= -1.0 && hi >= 1.0;
    if (axis == 3) return d == 3 ? (lo <= -1.0 && hi >= 1.0) : (lo <= 0.0 && hi >= M_PI);
    return false;
}

// largest R <= x: for every R-valued u, u > round_down(x) exactly when u > x
template <typename R> R round_down(double x)
{
    R r = (R)x;
    if ((double)r > x) r = std::nextafter(r, -std::numeric_limits<R>::infinity());
    return r;
}

template <typename R, typename Vec>
void fill_params(rtmc_context *ctx, const rtmc_problem *P, const DevTables<R> &tab, DevParams<R> *p, int *n_edges_out,
                 Vec *edges, Vec *zoe)
{
    std::memset(p, 0, sizeof *p);
    p->d = P->d; p->frame = P->frame; p->acoustics = P->acoustics; p->src_dir = P->src_dir;
    p->polarization = P->acoustics ? 0 : P->polarization;
    p->n_sub = P->n_sub; p->n_obs = P->n_obs; p->n_bnd = P->n_bnd;
    p->hist_shift = P->hist_shift;
    p->s_end = P->n_sub * P->n_obs;
    p->max_events = P->max_events > 0 ? P->max_events : 4 * p->s_end + 64;
    p->n_particles = P->n_particles; p->pid0 = P->pid0;
    p->key0 = (uint32_t)P->seed; p->key1 = (uint32_t)(P->seed >> 32);
    for (int i = 0; i < 3; ++i) p->src_pos[i] = (R)P->src_pos[i];
    p->src_lambda = (R)P->src_lambda;
    for (int m = 0; m < 2; ++m) {
        const int mm = P->acoustics ? 0 : m;
        p->step[m] = (R)(P->v[mm] * P->h);
        const double mft = P->mft[mm];
        p->scat_on[m] = std::isfinite(mft) ? 1 : 0;
        p->inv_lam64[m] = p->scat_on[m] ? 1.0 / (P->h / mft) : 0.0;
        p->inv_lam[m] = (R)p->inv_lam64[m];
        p->kill_on[m] = P->qrate[mm] > 0 ? 1 : 0;
        p->inv_q64[m] = p->kill_on[m] ? 1.0 / P->qrate[mm] : 0.0;
        p->inv_q[m] = (R)p->inv_q64[m];
    }
    p->p2p = round_down<R>(P->p2p); p->s2s = round_down<R>(P->s2s);
    if (!P->acoustics) {
        p->vs_over_vp = (R)(P->v[1] / P->v[0]);
        p->vp_over_vs = (R)(P->v[0] / P->v[1]);
    }
    p->cos_half_pi = (R)std::cos(M_PI / 2);
    edges->clear();
    bool finite_uniform[4] = {true, true, true, true};
    int am[4]; // effective axis modes: checks that every coordinate passes are dropped
    for (int a = 0; a < 4; ++a) {
        am[a] = P->axis_mode[a];
        const int ne = P->axis_nedges[a];
        const bool one_bin = am[a] == RTMC_AXIS_BINNED && ne == 2;
        if ((am[a] == RTMC_AXIS_RANGE || one_bin) && range_covers_axis(P->frame, P->d, a, P->axis_edges[a][0],
                                                                         P->axis_edges[a][ne - 1]))
            am[a] = RTMC_AXIS_IGNORED;
    }
    for (int a = 0; a < 4; ++a) {
        p->ax_mode[a] = am[a];
        p->ax_nbe[a] = 1;
        if (am[a] == RTMC_AXIS_IGNORED) continue;
        const int ne = P->axis_nedges[a];
        const double *E = P->axis_edges[a];
        p->ax_n[a] = ne;
        p->ax_off[a] = (int)edges->size();
        for (int k = 0; k < ne; ++k) edges->push_back((R)E[k]);
        p->ax_lo[a] = (R)E[0];
        p->ax_hi[a] = (R)E[ne - 1];
        p->ax_stride[a] = P->axis_stride[a];
        p->ax_stride32[a] = (int32_t)P->axis_stride[a];
        const double w = (E[ne - 1] - E[0]) / (ne - 1);
        bool uni = true;
        for (int k = 1; k < ne; ++k)
            if (std::fabs((E[k] - E[k - 1]) - w) > 1e-6 * std::fabs(w)) uni = false;
        p->ax_uniform[a] = uni ? 1 : 0;
        p->ax_inv_w[a] = (R)(1.0 / w);
        if (am[a] == RTMC_AXIS_BINNED) p->ax_nbe[a] = ne - 1;
        else p->ax_stride32[a] = 0;
        finite_uniform[a] = uni && std::isfinite(E[0]) && std::isfinite(E[ne - 1]);
    }
    {
        uint32_t bias = 0;
        for (int a = 0; a < 4; ++a) {
            const float nb = (float)p->ax_nbe[a];
            std::memcpy(&p->ax_nbits[a], &nb, sizeof(nb));
            if (a < 3) bias += 0x4B000000u * (uint32_t)p->ax_stride32[a];
        }
        std::memcpy(&p->cart_bias, &bias, sizeof(bias));
    }
    p->r32_iw = (float)p->ax_inv_w[0];
    p->r32_a0 = 0.f;
    // observation path (see obs_offset in transport.cuh)
    p->obs_kind = 0;
    if (P->frame == RTMC_FRAME_CARTESIAN) {
        bool ok = true;
        for (int a = 0; a < 3; ++a) ok = ok && (am[a] == RTMC_AXIS_IGNORED || finite_uniform[a]);
        if (ok) {
            p->obs_kind = 1;
            p->bin32 = sizeof(R) == 8 && p->s_end < (1 << 24) && (!ctx || ctx->opt_bin32) ? 1 : 0; // FP32 estimates
        }
    } else if (am[1] == RTMC_AXIS_IGNORED && am[2] == RTMC_AXIS_IGNORED && am[0] != RTMC_AXIS_IGNORED &&
               finite_uniform[0]) {
        p->obs_kind = 2;
        p->radial_3d = (P->frame == RTMC_FRAME_SPHERICAL && P->d == 3) ? 1 : 0;
        p->ax_a0 = (R)(-P->axis_edges[0][0] * (double)(P->axis_nedges[0] - 1) /
                       (P->axis_edges[0][P->axis_nedges[0] - 1] - P->axis_edges[0][0]));
        p->r32_a0 = (float)p->ax_a0;
        // FP64: the observation kernel bins through an FP32 estimate (exact, see
        // obs_offset_radial64 and obs_offset_cart64) while sub-step offsets stay exact in FP32
        p->bin32 = sizeof(R) == 8 && p->s_end < (1 << 24) && (!ctx || ctx->opt_bin32) ? 1 : 0;
    }
    p->time_stride = P->time_stride; p->mode_stride = P->mode_stride; p->hist_len = P->hist_len;
    // schedule: events per particle against observations (event-heavy problems run one
    // particle per thread; C3: ~76 events and 400 instants, C2: ~4 events and 250)
    {
        double rate = 0;
        for (int m = 0; m < (P->acoustics ? 1 : 2); ++m)
            if (std::isfinite(P->mft[m])) rate = std::max(rate, 1.0 / P->mft[m]);
        const double events = rate * P->h * (double)P->n_sub * (double)P->n_obs;
        const int o = ctx ? ctx->opt_event_major : -1;
        p->event_major = o == 1 ? 1 : ((o == 0 || o == 2) ? 0 : (events * 8.0 >= (double)P->n_obs ? 1 : 0));
    }
    *n_edges_out = (int)edges->size();
    p->n_edges = *n_edges_out;
    for (int b = 0; b < P->n_bnd; ++b) {
        p->bnd_dir[b] = P->bnd_dir[b];
        p->bnd_absorb[b] = P->bnd_absorb[b];
        p->bnd_val[b] = (R)P->bnd_val[b];
    }
    zoe->resize(2 * RTMC_ZOE_N);
    for (int k = 0; k < RTMC_ZOE_N; ++k) {
        (*zoe)[k] = (R)P->zoe_rpp[k];
        (*zoe)[RTMC_ZOE_N + k] = (R)P->zoe_rsvsv[k];
    }
    p->src_type = P->src_type;
    p->src_aperture = P->src_aperture;
    for (int i = 0; i < 3; ++i) {
        p->src_n[i] = (R)P->src_normal[i];
        p->src_u[i] = (R)P->src_u[i];
        p->src_v[i] = (R)P->src_v[i];
    }
    p->src_ext[0] = (R)P->src_extent[0];
    p->src_ext[1] = (R)P->src_extent[1];
    // the radial source table follows the Zoeppritz tables (p->src_radial is set with p->zoe)
    p->src_radial_n = P->src_radial_n;
    for (int k = 0; k < P->src_radial_n; ++k) zoe->push_back((R)P->src_radial_cdf[k]);
    for (int k = 0; k < P->src_radial_n; ++k) zoe->push_back((R)P->src_radial_r[k]);
    p->tab = tab;
    (void)ctx;
}

constexpr int kCopyGroups = 5; // slice groups of the last fold, each copied as soon as it is final

// Row stride of the index array for a chunk of particles: a multiple of 32 entries, so
// every row starts on a 128-byte boundary (the fold reads rows as 16-byte vectors, up to
// the vector holding the chunk's last particle) and a warp's 32 lanes write whole lines.
inline int64_t index_row_stride(int64_t particles) { return (particles + 31) / 32 * 32; }

// First slice (1-based) of copy group g in [0, kCopyGroups]; g = kCopyGroups gives n_obs + 1.
// The first group is small (1/25 of the slices), so the first copy starts soon after the
// transport; the fold outruns the host link, so later copies follow back to back.
// Copy groups of the time-blocked fold: t-blocks [b[g], b[g + 1]), growing 1, 2, 3, ... up
// to max(9, ntb / 16) t-blocks (at most 23 groups).  The early t-blocks fold slowest (most particles are in
// the grid) and the host link is the bottleneck from the second group on, so small first
// groups start the copies early and keep the link busy: modelled on the 3D elastic
// workload's measured per-t-block fold times, 19.0 ms from the end of the transport to the
// last copy, against 21.1 with 5 groups of which the first held 1/25 of the slices.
int tb_groups(int ntb, int *b)
{
    const int cap = std::max(9, (ntb + 15) / 16);
    int n = 0, t = 0, size = 1;
    b[0] = 0;
    while (t < ntb && n < 23) {
        t = std::min(ntb, t + size);
        b[++n] = t;
        size = std::min(size + 1, cap);
    }
    if (t < ntb) b[n] = ntb; // the last group takes the rest
    return n;
}

int copy_group_start(int n_obs, int g)
{
    if (g <= 0) return 1;
    const int first = std::max(1, n_obs / 25);
    return 1 + first + (int)((int64_t)(n_obs - first) * (g - 1) / (kCopyGroups - 1));
}

// True for host memory that the CUDA runtime has not page-locked or registered
bool host_is_pageable(const void *ptr)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

int ensure_pipeline(rtmc_context *ctx)
{
    cudaError_t e = cudaSuccess;
    if (!ctx->fold_stream) e = cudaStreamCreateWithFlags(&ctx->fold_stream, cudaStreamNonBlocking);
    for (int i = 0; i < rtmc_context::kPipe && e == cudaSuccess; ++i) {
        if (!ctx->ev_a0[i]) e = cudaEventCreate(&ctx->ev_a0[i]);
        if (e == cudaSuccess && !ctx->ev_a1[i]) e = cudaEventCreate(&ctx->ev_a1[i]);
        if (e == cudaSuccess && !ctx->ev_b0[i]) e = cudaEventCreate(&ctx->ev_b0[i]);
        if (e == cudaSuccess && !ctx->ev_b1[i]) e = cudaEventCreate(&ctx->ev_b1[i]);
    }
    return (int)e;
}

// host_out receives the int64 histogram, or host_u32 the uint32 counts (at most one)
template <typename R>
int run(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, int64_t *host_out, rtmc_stats *st,
        double *trace_out, uint32_t *host_u32)
{
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaEventRecord(ctx->ev_start, ctx->stream), "event");
    double h2d = 0, d2h = 0;
    DevTables<R> *dt;
    if constexpr (sizeof(R) == 4) dt = &ctx->tf; else dt = &ctx->td;
    const int prec = sizeof(R) == 4 ? RTMC_FP32 : RTMC_FP64;
    if (!ctx->cache_tables || ctx->tabs_gen != t->gen || ctx->tabs_prec != prec) {
        Range r("tables upload");
        int s = upload_tables<R>(ctx, t, dt);
        if (s) { ctx->tabs_gen = 0; return s; }
        ctx->tabs_gen = t->gen;
        ctx->tabs_prec = prec;
        for (int i = 0; i < t->n_tables; ++i) h2d += (double)table_bytes<R>(t->cdf[i].size());
    }
    DevParams<R> p;
    std::vector<R> edges, zoe;
    int n_edges = 0;
    fill_params<R>(ctx, P, *dt, &p, &n_edges, &edges, &zoe);
    // aux buffer: edges | zoe | stats
    const size_t eb = align_up(std::max<size_t>(1, edges.size()) * sizeof(R), 256);
    const size_t zb = align_up(zoe.size() * sizeof(R), 256);
    if (ctx->aux.grow(eb + zb)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for edges failed");
    if (ctx->stats.grow(256)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for counters failed");
    unsigned char *aux = static_cast<unsigned char *>(ctx->aux.p);
    if (!edges.empty())
        CK(cudaMemcpyAsync(aux, edges.data(), edges.size() * sizeof(R), cudaMemcpyHostToDevice, ctx->stream), "edges");
    CK(cudaMemcpyAsync(aux + eb, zoe.data(), zoe.size() * sizeof(R), cudaMemcpyHostToDevice, ctx->stream), "zoeppritz");
    h2d += (double)(edges.size() + zoe.size()) * sizeof(R);
    p.edges = reinterpret_cast<const R *>(aux);
    p.zoe = reinterpret_cast<const R *>(aux + eb);
    p.src_radial = p.zoe + 2 * RTMC_ZOE_N;
    const size_t hist_bytes = (size_t)P->hist_len * sizeof(int64_t);
    if (ctx->hist.grow(hist_bytes)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the histogram failed");
    CK(cudaMemsetAsync(ctx->stats.p, 0, 256, ctx->stream), "counter clear");
    ctx->hist_len = P->hist_len;
    uint32_t *narrow = nullptr;
    if (host_u32) {
        if (ctx->narrow.grow((size_t)P->hist_len * sizeof(uint32_t)))
            return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the uint32 histogram failed");
        narrow = static_cast<uint32_t *>(ctx->narrow.p);
    }
    const int narrow_grid = 8 * ctx->num_sms;
    p.hist = static_cast<unsigned long long *>(ctx->hist.p);
    p.stats = static_cast<unsigned long long *>(ctx->stats.p);
    p.status = reinterpret_cast<int32_t *>(static_cast<unsigned char *>(ctx->stats.p) + 128);
    const size_t trace_bytes = (size_t)P->n_particles * 16 * sizeof(double);
    p.trace = nullptr;
    if (trace_out && trace_bytes) {
        if (ctx->trace.grow(trace_bytes)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for traces failed");
        p.trace = static_cast<double *>(ctx->trace.p);
    }

    // Sink: the whole histogram in shared memory when it fits beside a segment ring of at
    // least 2 slots per lane at 512 threads; otherwise, for histograms larger than the L2,
    // a dense index array folded afterwards (time-blocked FP32, or slice by slice with
    // rt_bin_slices), or plain global 64-bit atomics when the histogram stays in the L2 or
    // the index array is switched off or does not fit.
    const size_t edge_smem = align_up((size_t)n_edges * sizeof(R), 16);
    const size_t hist_smem = align_up((size_t)P->hist_len * sizeof(uint32_t), 16);
    const size_t seg_bytes = 6 * sizeof(R) + 2 * sizeof(int32_t);
    const size_t budget = (size_t)ctx->max_smem_optin - 1024;
    const int nm = P->acoustics ? 1 : 2;
    int sink = kSinkGlobal, block = ctx->opt_block ? ctx->opt_block : 256;
    int cap = ctx->opt_ring ? ctx->opt_ring : (sizeof(R) == 4 ? 8 : 6);
    {
        const int sb = ctx->opt_block ? ctx->opt_block : 512;
        if (edge_smem + hist_smem + (size_t)sb * 2 * seg_bytes <= budget) {
            sink = kSinkSmem;
            block = sb;
            const int fit = (int)((budget - edge_smem - hist_smem) / ((size_t)sb * seg_bytes));
            cap = std::min(ctx->opt_ring ? ctx->opt_ring : 8, fit);
        }
    }
    int64_t chunk = P->n_particles; // particles per transport launch
    int n_pipe = 0;                 // > 0: chunks pipelined over two index slots
    // A histogram that stays resident in the L2 takes the 64-bit atomics directly (C3,
    // 1.3 MB: 1142 ms against 1369 ms through the index array); larger ones go through the
    // index array unless it is switched off.  An explicit index budget or pipeline asks
    // for the index path.
    const bool l2_resident = hist_bytes <= ((size_t)64 << 20);
    const bool want_index = ctx->opt_index_mb > 0 || ctx->opt_chunks >= 2 || (ctx->opt_index_mb == 0 && !l2_resident);
    if (sink != kSinkSmem && want_index && P->time_stride < ((int64_t)1 << 30)) {
        const int64_t mb = ctx->opt_index_mb ? ctx->opt_index_mb : 12288; // default index budget: 12 GB
        const int64_t rows = std::max<int64_t>(32, ((mb << 20) / (4 * (int64_t)P->n_obs)) / 32 * 32);
        // pipeline: the fold of chunk c overlaps the transport of chunk c + 1 (the fold is
        // bound by L2 atomics, the transport by instruction issue), two index slots
        // off unless asked for: on C2 it measured 25.5 ms against 25.9 ms sequential (the
        // transport at 2 blocks per SM loses what the overlap gains)
        const int want = ctx->opt_chunks ? ctx->opt_chunks : 1;
        if (want >= 2) {
            int nc = want;
            int64_t per = ((P->n_particles + nc - 1) / nc + 31) / 32 * 32;
            while (2 * per > rows && nc < rtmc_context::kPipe) {
                ++nc;
                per = ((P->n_particles + nc - 1) / nc + 31) / 32 * 32;
            }
            if (2 * per <= rows && nc >= 2 && ensure_pipeline(ctx) == 0 &&
                ctx->idx.grow((size_t)2 * per * P->n_obs * sizeof(int32_t)) == 0) {
                sink = kSinkIndex;
                chunk = per;
                n_pipe = nc;
            }
        }
        if (!n_pipe) {
            chunk = std::min<int64_t>(P->n_particles, rows);
            if (chunk > 0 && ctx->idx.grow((size_t)index_row_stride(chunk) * P->n_obs * sizeof(int32_t)) == 0)
                sink = kSinkIndex;
            else
                chunk = P->n_particles;
        }
    }
    {
        // the variant's launch bound caps the block (fill_params chose the observation path)
        const int mt = transport_max_threads(prec, sink, p.obs_kind);
        if (mt > 0 && block > mt) block = mt - mt % 32;
    }
    size_t smem = edge_smem + (sink == kSinkSmem ? hist_smem : 0) + (size_t)block * cap * seg_bytes;
    int bps = 0;
    if (transport_set_smem(prec, sink, p.obs_kind, smem) != 0) return fail(&ctx->err, RTMC_ERR_CUDA, "cudaFuncSetAttribute failed");
    if (transport_occupancy(prec, sink, p.obs_kind, block, smem, &bps) != 0 || bps < 1)
        return fail(&ctx->err, RTMC_ERR_CUDA, "transport kernel does not fit on the device");
    p.sink = sink;
    p.ring_cap = cap;
    // the index array wants each warp's 32 rows written together: keep the batches
    if (sink == kSinkIndex && ctx->opt_event_major < 0) p.event_major = 0;
    // pipelined transport keeps room on every SM for the fold's blocks
    if (n_pipe) bps = std::min(bps, ctx->opt_k1_bps ? ctx->opt_k1_bps : 2);
    int64_t grid = (int64_t)ctx->num_sms * bps;
    const int64_t need = (std::max<int64_t>(chunk, 1) + block - 1) / block;
    grid = std::max<int64_t>(1, std::min<int64_t>(grid, need));
    int le = 0, launches = 0;
    // split schedule (rt_events, rt_observe): the lockstep problems, unless switched off
    const bool split = !p.event_major && ctx->opt_event_major != 0;
    SplitLaunch sl{};
    if (split) {
        // segments per particle: 1 + the expected events + 4 standard deviations + 4
        double rate = 0;
        for (int m = 0; m < nm; ++m)
            if (std::isfinite(P->mft[m])) rate = std::max(rate, 1.0 / P->mft[m]);
        const double mean = rate * P->h * (double)P->n_sub * (double)P->n_obs;
        int K = (int)std::ceil(1.0 + mean + 4.0 * std::sqrt(mean) + 4.0);
        K = std::min(64, std::max(8, (K + 3) / 4 * 4));
        if (ctx->opt_ring) K = ctx->opt_ring; // an explicit ring capacity sets the segments per particle
        K = std::max(1, K) + 2;               // and two end records (rec_put_end)
        const size_t rec = 8 * sizeof(R);
        // particles per launch: the segments of one chunk stay within 8 GB
        constexpr int64_t kSegBudget = (int64_t)8 << 30;
        const int64_t seg_rows = std::max<int64_t>(32, kSegBudget / ((int64_t)K * (int64_t)rec) / 32 * 32);
        chunk = std::min(chunk, seg_rows);
        const int64_t rows_max = std::max<int64_t>(chunk, 1);
        if (ctx->segs.grow((size_t)rows_max * K * rec) || ctx->ovf.grow((size_t)rows_max * 4))
            return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for trajectory segments failed");
        // the index path bins the particles in the order of their starting directions
        if (sink == kSinkIndex && ctx->opt_order) {
            if (ctx->order.grow((size_t)rows_max * 3 * sizeof(int32_t) + kOrderCells * sizeof(int32_t)))
                return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the particle order failed");
            int32_t *o = static_cast<int32_t *>(ctx->order.p);
            p.okey = o;
            p.perm = o + rows_max;
            p.iperm = o + 2 * rows_max;
            sl.order.cursor = o + 3 * rows_max;
            sl.grid_order = 2 * ctx->num_sms;
        }
        p.split = 1;
        p.seg_cap = K;
        p.segs = ctx->segs.p;
        p.ovf_list = static_cast<int32_t *>(ctx->ovf.p);
        p.ovf_count = reinterpret_cast<uint32_t *>(static_cast<unsigned char *>(ctx->stats.p) + 192);
        sl.smem_events = edge_smem;
        int be = 0, bo = 0;
        if (kernel_set_smem(prec, 5, sink, p.obs_kind, sl.smem_events) != 0 ||
            kernel_set_smem(prec, 7, sink, p.obs_kind, sl.smem_events) != 0 ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&be, kernel_of(prec, 5, sink, p.obs_kind), 256, sl.smem_events) !=
                cudaSuccess || be < 1)
            return fail(&ctx->err, RTMC_ERR_CUDA, "event kernel does not fit on the device");
        {
            // the kernel's launch bound is its block size
            cudaFuncAttributes fa{};
            if (cudaFuncGetAttributes(&fa, kernel_of(prec, 6, sink, p.obs_kind)) != cudaSuccess || fa.maxThreadsPerBlock < 32)
                return fail(&ctx->err, RTMC_ERR_CUDA, "observation kernel attributes");
            sl.block_observe = fa.maxThreadsPerBlock - fa.maxThreadsPerBlock % 32;
        }
        sl.smem_observe = edge_smem + (sink == kSinkSmem ? hist_smem : 0);
        if (kernel_set_smem(prec, 6, sink, p.obs_kind, sl.smem_observe) != 0 ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bo, kernel_of(prec, 6, sink, p.obs_kind), sl.block_observe,
                                                          sl.smem_observe) != cudaSuccess || bo < 1)
            return fail(&ctx->err, RTMC_ERR_CUDA, "observation kernel does not fit on the device");
        if (n_pipe) {
            be = std::min(be, ctx->opt_k1_bps ? ctx->opt_k1_bps : 2);
            bo = std::min(bo, ctx->opt_k1_bps ? ctx->opt_k1_bps : 2);
        }
        const int64_t cmax = std::max<int64_t>(chunk, 1);
        sl.grid_events = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->num_sms * be, (cmax + 255) / 256));
        sl.grid_observe = (int)std::max<int64_t>(
            1, std::min<int64_t>((int64_t)ctx->num_sms * bo, (cmax + sl.block_observe - 1) / sl.block_observe));
        sl.grid_list = ctx->num_sms;
        sl.mid_event = n_pipe ? nullptr : (void *)ctx->ev_km; // times rt_events apart
        if (sink == kSinkSmem && chunk / sl.grid_observe >= ((int64_t)1 << 32) - 1)
            return fail(&ctx->err, RTMC_ERR_ARG, "too many particles per block for 32-bit shared-memory counts");
    }
    // time-blocked FP32 fold (index path, one pass over the chunks, exact counts below 2^24
    // particles): it writes every bin of the histogram, so only its accumulator needs a clear
    const bool use_tb = sink == kSinkIndex && !n_pipe && P->n_particles < ((int64_t)1 << 24) && ctx->opt_fold != 1;
    const int ntb = (P->n_obs + 3) / 4;
    int roll = 0; // t-blocks per turn of a rolling accumulator (0: the full accumulator)
    bool timed_convert = false; // ev_kc marks the start of the conversion
    bool narrowed = false; // the conversion also wrote the uint32 counts
    TbParams tpl{};
    int tb_grid = 1;
    if (use_tb) {
        tpl.S = P->time_stride * nm;
        // mode 3 with one particle chunk: the accumulator rolls over the t-blocks, as many at
        // a time as fit in kRollBytes (at least one), so that it stays in the L2 between its
        // reductions and its conversion.  Measured on the 3D elastic workload (1e7
        // particles, 63 t-blocks of 55 MB): 17.3 ms for the fold and conversions against
        // 8.2 ms with the full accumulator (one launch of each over every t-block), whose
        // reductions spread over all t-blocks at once; so the full one is the default.
        constexpr int64_t kRollBytes = (int64_t)64 << 20;
        if (chunk >= P->n_particles && ctx->opt_fold == 3) {
            roll = (int)std::max<int64_t>(1, std::min<int64_t>(ntb, kRollBytes / (tpl.S * 16)));
            if (roll >= ntb) roll = 0;
        }
        const size_t acc_bytes = (size_t)(roll ? roll : ntb) * tpl.S * 4 * sizeof(float);
        if (ctx->tbacc.grow(acc_bytes)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the fold accumulator failed");
        tpl.acc = static_cast<float *>(ctx->tbacc.p);
        tpl.idx = static_cast<const int32_t *>(ctx->idx.p);
        tpl.rows = index_row_stride(chunk);
        tpl.n_obs = P->n_obs;
        tpl.slice_bins = (int32_t)P->time_stride;
        tb_grid = (int)std::max<int64_t>(1, std::min<int64_t>((chunk + 8191) / 8192, 2 * ctx->num_sms));
    }
    // the clear: fused into the first rt_events launch of a split run (the FP32 accumulator
    // of the time-blocked fold, else the histogram), else one memset ahead of the transport.
    // Measured on the 3D elastic workload (rt_events 2.37 ms with the fused clear of the
    // 3.47 GB accumulator): a memset on the second stream during the transport cost
    // rt_events 0.22 ms and the fold 0.4 ms (its blocks take SM slots from both kernels);
    // device-to-device copies from a zero buffer on the copy engines saved rt_events 0.02 ms
    // and cost rt_observe 0.15 ms.
    unsigned long long *to_clear = use_tb ? static_cast<unsigned long long *>(ctx->tbacc.p)
                                          : static_cast<unsigned long long *>(ctx->hist.p);
    const int64_t clear_words = use_tb ? (int64_t)(roll ? roll : ntb) * tpl.S * 2 : P->hist_len;
    if (split) {
        p.clear = to_clear;
        p.clear_words = clear_words;
    } else {
        CK(cudaMemsetAsync(to_clear, 0, (size_t)clear_words * 8, ctx->stream), "histogram clear");
    }
    // one transport launch over q: the fused kernel, or the split schedule's three kernels
    auto launch_one = [&](const DevParams<R> &q) -> int {
        if (split) {
            const cudaError_t e = cudaMemsetAsync(q.ovf_count, 0, sizeof(uint32_t), ctx->stream);
            if (e != cudaSuccess) return (int)e;
            launches += 3;
            p.clear = nullptr; // the first chunk clears the histogram
            p.clear_words = 0;
            if constexpr (sizeof(R) == 4) return launch_split_f32(q, sl, ctx->stream);
            else return launch_split_f64(q, sl, ctx->stream);
        }
        ++launches;
        if constexpr (sizeof(R) == 4) return launch_transport_f32(q, (int)grid, block, smem, ctx->stream);
        else return launch_transport_f64(q, (int)grid, block, smem, ctx->stream);
    };
    if (sink == kSinkSmem && P->n_particles / grid >= ((int64_t)1 << 32) - 1)
        return fail(&ctx->err, RTMC_ERR_ARG, "too many particles per block for 32-bit shared-memory counts");
    // slice fold: privatise groups of slices in shared memory when 8 or more fit
    BinParams bp{};
    size_t fold_smem = 0;
    int fold_grid = 1;
    const int64_t idx_rows = index_row_stride(chunk); // == chunk when pipelined
    if (sink == kSinkIndex) {
        bp.idx = static_cast<const int32_t *>(ctx->idx.p);
        bp.rows = idx_rows;
        bp.n_obs = P->n_obs;
        bp.n_modes = nm;
        bp.slice_bins = (int32_t)P->time_stride;
        bp.time_stride = P->time_stride;
        bp.mode_stride = P->mode_stride;
        bp.hist_shift = P->hist_shift;
        bp.hist = static_cast<unsigned long long *>(ctx->hist.p);
        bp.j_first = 1;
        bp.j_count = P->n_obs;
        const size_t slice_bytes = (size_t)P->time_stride * nm * sizeof(uint32_t);
        const int group = (int)std::min<size_t>((size_t)P->n_obs, (size_t)(200 << 10) / std::max<size_t>(slice_bytes, 1));
        if (group >= 8) {
            bp.group = group;
            fold_smem = (size_t)group * slice_bytes;
            if (bin_slices_set_smem(fold_smem) != 0) return fail(&ctx->err, RTMC_ERR_CUDA, "cudaFuncSetAttribute failed");
            const int ngroups = (P->n_obs + group - 1) / group;
            // enough particle ranges to fill the GPU twice over
            const int64_t ranges = std::max<int64_t>(1, (2 * ctx->num_sms + ngroups - 1) / ngroups);
            bp.part_per_block = (chunk + ranges - 1) / ranges;
            fold_grid = (int)ranges;
        } else {
            bp.group = 0;
            // chunks of at least 8 vectors per thread of a 512-thread block, up to one block per SM per slice
            fold_grid = (int)std::max<int64_t>(1, std::min<int64_t>((chunk + 16383) / 16384, ctx->num_sms));
        }
        p.obs_idx = static_cast<int32_t *>(ctx->idx.p);
        p.obs_rows = idx_rows;
    }
    double kms = 0, fms = 0, ems = 0, cms = 0;
    if (n_pipe) {
        const size_t slot_elems = (size_t)idx_rows * P->n_obs;
        int32_t *idx0 = static_cast<int32_t *>(ctx->idx.p);
        int c = 0;
        for (int64_t base = 0; base < P->n_particles && !le; base += chunk, ++c) {
            DevParams<R> q = p;
            q.pid0 = P->pid0 + base;
            q.n_particles = std::min<int64_t>(chunk, P->n_particles - base);
            q.obs_idx = idx0 + (c & 1) * slot_elems;
            q.obs_rows = idx_rows;
            if (p.trace) q.trace = p.trace + 16 * base;
            if (c >= 2) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_b1[c - 2], 0), "pipeline wait");
            CK(cudaEventRecord(ctx->ev_a0[c], ctx->stream), "event");
            le = launch_one(q);
            if (le) break;
            CK(cudaEventRecord(ctx->ev_a1[c], ctx->stream), "event");
            CK(cudaStreamWaitEvent(ctx->fold_stream, ctx->ev_a1[c], 0), "pipeline wait");
            BinParams b = bp;
            b.idx = q.obs_idx;
            b.rows = idx_rows;
            b.n = q.n_particles;
            if (b.group) b.part_per_block = (b.n + fold_grid - 1) / fold_grid;
            CK(cudaEventRecord(ctx->ev_b0[c], ctx->fold_stream), "event");
            le = launch_bin_slices(b, fold_grid, fold_smem, ctx->fold_stream);
            if (le) break;
            CK(cudaEventRecord(ctx->ev_b1[c], ctx->fold_stream), "event");
            ++launches;
        }
        if (!le) {
            CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_b1[c - 1], 0), "pipeline join");
            CK(cudaStreamSynchronize(ctx->stream), "transport");
            for (int k = 0; k < c; ++k) {
                float a = 0, b = 0;
                cudaEventElapsedTime(&a, ctx->ev_a0[k], ctx->ev_a1[k]);
                cudaEventElapsedTime(&b, ctx->ev_b0[k], ctx->ev_b1[k]);
                kms += a;
                fms += b;
            }
        } else {
            cudaStreamSynchronize(ctx->fold_stream);
        }
    }
    bool copied = false; // the histogram reached host_out during the last fold
    for (int64_t base = 0; !n_pipe && base < P->n_particles && !le; base += chunk) {
        DevParams<R> q = p;
        q.pid0 = P->pid0 + base;
        q.n_particles = std::min<int64_t>(chunk, P->n_particles - base);
        if (p.trace) q.trace = p.trace + 16 * base;
        const bool last = base + chunk >= P->n_particles;
        // the last fold in groups of t-blocks when the histogram goes to the host: each
        // group's slices are final, so their copy runs on the second stream while the next
        // group folds
        const bool groups =
            use_tb && last && (host_out || host_u32) && ntb >= 2 * kCopyGroups && ensure_pipeline(ctx) == 0;
        int gb_[25];
        const int ng = groups ? tb_groups(ntb, gb_) : 1;
        // early copy (split schedule, one chunk): rt_observe bins the instants of the first
        // groups (at least a fifth of them), those groups fold and start their copies, and
        // only then does rt_observe bin the rest, so the host link starts working after a
        // fraction of the observation pass instead of all of it
        int g_split = 0;
        if (groups && split && !roll && base == 0 && last && ctx->opt_early_copy > 0) {
            for (int g = 1; g < ng; ++g)
                if (100 * 4 * (int64_t)gb_[g] >= (int64_t)ctx->opt_early_copy * P->n_obs) { g_split = g; break; }
        }
        CK(cudaEventRecord(ctx->ev_k0, ctx->stream), "event");
        if (g_split) {
            q.obs_j0 = 1;
            q.obs_j1 = 4 * gb_[g_split];
        }
        {
            Range r("transport launches");
            le = launch_one(q);
        }
        CK(cudaEventRecord(ctx->ev_k1, ctx->stream), "event");
        if (!le && use_tb) {
            TbParams tp = tpl;
            tp.n = q.n_particles;
            tp.part_per_block = ((tp.n + tb_grid - 1) / tb_grid + 3) / 4 * 4;
            unsigned long long *hist = p.hist;
            const int64_t ts = P->time_stride;
            // one fold launch and one conversion: the conversion is timed apart
            timed_convert = last && !groups && !roll && ntb <= 65535;
            // a pageable destination (a MEX array, a NumPy array) makes each copy call block
            // the host until it is done: those copies are issued after every launch is queued
            const bool deferred = groups && host_is_pageable(host_u32 ? (const void *)host_u32 : (const void *)host_out);
            int deferred_g[25], n_deferred = 0;
            auto issue_copies = [&](int g) -> int {
                const int ga = gb_[g], gb = gb_[g + 1];
                const int64_t ja = g == 0 ? 0 : 4 * (int64_t)ga + 1; // slice 0 with the first group
                const int64_t jb = std::min<int64_t>(4 * (int64_t)gb, P->n_obs) + 1;
                CK(cudaStreamWaitEvent(ctx->fold_stream, ctx->ev_a1[g], 0), "copy wait");
                for (int m = 0; m < nm; ++m) {
                    const int64_t o = m * P->mode_stride + ja * ts;
                    const size_t cnt = (size_t)((jb - ja) * ts);
                    if (host_u32)
                        CK(cudaMemcpyAsync(host_u32 + o, narrow + o, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                           ctx->fold_stream),
                           "histogram copy");
                    else
                        CK(cudaMemcpyAsync(host_out + o, static_cast<int64_t *>(ctx->hist.p) + o, cnt * sizeof(int64_t),
                                           cudaMemcpyDeviceToHost, ctx->fold_stream),
                           "histogram copy");
                }
                return RTMC_OK;
            };
            for (int g = 0; g < ng && !le; ++g) {
                const int ga = groups ? gb_[g] : 0, gb = groups ? gb_[g + 1] : ntb;
                if (g_split && g == g_split) { // the remaining instants, then their groups
                    DevParams<R> qb = q;
                    qb.obs_j0 = q.obs_j1 + 1;
                    qb.obs_j1 = P->n_obs;
                    SplitLaunch s2 = sl;
                    s2.part = 2;
                    if constexpr (sizeof(R) == 4) le = launch_split_f32(qb, s2, ctx->stream);
                    else le = launch_split_f64(qb, s2, ctx->stream);
                    launches += 2;
                    if (le) break;
                }
                if (gb <= ga) continue;
                // a rolling accumulator takes `roll` t-blocks at a time and is zeroed again by
                // their conversion; the full one takes the group at once
                const int step = roll ? roll : gb - ga;
                for (int t0 = ga; t0 < gb && !le; t0 += step) {
                    tp.tb_first = t0;
                    tp.tb_count = std::min(step, gb - t0);
                    tp.acc_tb0 = roll ? t0 : 0;
                    tp.rezero = roll ? 1 : 0;
                    le = launch_fold_tb(tp, tb_grid, ctx->stream);
                    ++launches;
                    if (!le && last) {
                        if (timed_convert) CK(cudaEventRecord(ctx->ev_kc, ctx->stream), "event");
                        le = launch_tb_convert(tp, ts, P->mode_stride, P->hist_shift, hist, host_u32 ? narrow : nullptr,
                                               narrow_grid, ctx->stream);
                        ++launches;
                        narrowed = host_u32 != nullptr;
                    }
                }
                if (le || !groups) break;
                CK(cudaEventRecord(ctx->ev_a1[g], ctx->stream), "event");
                if (deferred) {
                    deferred_g[n_deferred++] = g;
                } else {
                    const int c = issue_copies(g);
                    if (c) return c;
                }
            }
            if (groups && !le) {
                CK(cudaEventRecord(ctx->ev_k2, ctx->stream), "event");
                Range r("deferred histogram copies"); // pageable destinations (empty otherwise)
                for (int k = 0; k < n_deferred; ++k) {
                    const int c = issue_copies(deferred_g[k]);
                    if (c) return c;
                }
                CK(cudaEventRecord(ctx->ev_b1[0], ctx->fold_stream), "event");
                CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_b1[0], 0), "copy join");
                copied = true;
            } else {
                CK(cudaEventRecord(ctx->ev_k2, ctx->stream), "event");
            }
        } else if (!le && sink == kSinkIndex) {
            BinParams b = bp;
            b.n = q.n_particles;
            if (b.group) b.part_per_block = (b.n + fold_grid - 1) / fold_grid;
            if (last && (host_out || host_u32) && !b.group && P->n_obs >= 2 * kCopyGroups && ensure_pipeline(ctx) == 0) {
                // the last fold in slice groups: each group's slices are final, so their
                // copy to the host runs on the second stream while the next group folds
                const int64_t ts = P->time_stride;
                for (int g = 0; g < kCopyGroups && !le; ++g) {
                    const int ja = copy_group_start(P->n_obs, g);
                    const int jb = copy_group_start(P->n_obs, g + 1); // exclusive
                    b.j_first = ja;
                    b.j_count = jb - ja;
                    le = launch_bin_slices(b, fold_grid, fold_smem, ctx->stream);
                    if (le) break;
                    ++launches;
                    const int64_t s0 = g == 0 ? 0 : (int64_t)ja * ts; // slice 0 (t = 0) goes with the first group
                    const int64_t s1 = (int64_t)jb * ts;
                    for (int m = 0; m < nm && narrow && !le; ++m) {
                        const int64_t o = m * P->mode_stride + s0;
                        le = launch_narrow_u32(p.hist + o, narrow + o, s1 - s0, P->hist_shift, narrow_grid, ctx->stream);
                        ++launches;
                    }
                    if (le) break;
                    CK(cudaEventRecord(ctx->ev_a1[g], ctx->stream), "event");
                    CK(cudaStreamWaitEvent(ctx->fold_stream, ctx->ev_a1[g], 0), "copy wait");
                    for (int m = 0; m < nm; ++m) {
                        const int64_t o = m * P->mode_stride + s0;
                        if (narrow)
                            CK(cudaMemcpyAsync(host_u32 + o, narrow + o, (size_t)(s1 - s0) * sizeof(uint32_t),
                                               cudaMemcpyDeviceToHost, ctx->fold_stream),
                               "histogram copy");
                        else
                            CK(cudaMemcpyAsync(host_out + o, static_cast<int64_t *>(ctx->hist.p) + o,
                                               (size_t)(s1 - s0) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                               ctx->fold_stream),
                               "histogram copy");
                    }
                }
                CK(cudaEventRecord(ctx->ev_b1[0], ctx->fold_stream), "event");
                CK(cudaEventRecord(ctx->ev_k2, ctx->stream), "event");
                CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_b1[0], 0), "copy join");
                copied = true;
            } else {
                le = launch_bin_slices(b, fold_grid, fold_smem, ctx->stream);
                CK(cudaEventRecord(ctx->ev_k2, ctx->stream), "event");
                ++launches;
            }
        }
        {
            Range r("wait for the transport");
            CK(cudaEventSynchronize(sink == kSinkIndex ? ctx->ev_k2 : ctx->ev_k1), "transport");
        }
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, ctx->ev_k0, ctx->ev_k1);
        kms += a;
        if (split && !le) {
            float m = 0;
            cudaEventElapsedTime(&m, ctx->ev_k0, ctx->ev_km);
            ems += m;
        }
        if (sink == kSinkIndex) {
            cudaEventElapsedTime(&b, ctx->ev_k1, ctx->ev_k2);
            fms += b;
            if (timed_convert) {
                float c = 0;
                cudaEventElapsedTime(&c, ctx->ev_kc, ctx->ev_k2);
                cms += c;
                timed_convert = false;
            }
        }
    }
    if (le) return cuda_fail(ctx, (cudaError_t)le, "transport launch");
    if (p.clear) CK(cudaMemsetAsync(ctx->hist.p, 0, hist_bytes, ctx->stream), "histogram clear"); // no launch ran
    ctx->hist_may_exceed_int64 = may_exceed_int64(P);
    if (host_out && ctx->hist_may_exceed_int64) {
        le = launch_check_int64(p.hist, P->hist_len, p.status, narrow_grid, ctx->stream);
        if (le) return cuda_fail(ctx, (cudaError_t)le, "histogram range check");
        ++launches;
    }
    int64_t dstats[32];
    CK(cudaMemcpyAsync(dstats, ctx->stats.p, 256, cudaMemcpyDeviceToHost, ctx->stream), "counters");
    if (host_out) {
        if (!copied)
            CK(cudaMemcpyAsync(host_out, ctx->hist.p, hist_bytes, cudaMemcpyDeviceToHost, ctx->stream), "histogram copy");
        d2h += (double)hist_bytes;
    } else if (host_u32) {
        const size_t u32_bytes = (size_t)P->hist_len * sizeof(uint32_t);
        if (!copied) {
            if (!narrowed) {
                le = launch_narrow_u32(p.hist, narrow, P->hist_len, P->hist_shift, narrow_grid, ctx->stream);
                if (le) return cuda_fail(ctx, (cudaError_t)le, "histogram narrowing");
                ++launches;
            }
            CK(cudaMemcpyAsync(host_u32, narrow, u32_bytes, cudaMemcpyDeviceToHost, ctx->stream), "histogram copy");
        }
        d2h += (double)u32_bytes;
    }
    if (p.trace) {
        CK(cudaMemcpyAsync(trace_out, p.trace, trace_bytes, cudaMemcpyDeviceToHost, ctx->stream), "trace copy");
        d2h += (double)trace_bytes;
    }
    CK(cudaEventRecord(ctx->ev_end, ctx->stream), "event");
    CK(cudaStreamSynchronize(ctx->stream), "transport");
    float tms = 0;
    cudaEventElapsedTime(&tms, ctx->ev_start, ctx->ev_end);
    ctx->last_kernel_ms = kms + fms;
    ctx->last_launches = launches;
    const int32_t status = (int32_t)(dstats[16] & 0xffffffff);
    if (st) {
        std::memset(st, 0, sizeof *st);
        st->scatter_events = dstats[0];
        st->boundary_hits = dstats[1];
        st->kills = dstats[2];
        st->absorbed = dstats[3];
        st->observations = dstats[4];
        st->conversions = dstats[5];
        st->device_status = status;
        st->kernel_ms = kms;
        st->fold_ms = fms;
        st->events_ms = ems;
        st->convert_ms = cms;
        st->launches = launches;
        st->sink = sink;
        st->total_ms = tms;
        st->h2d_bytes = h2d;
        st->d2h_bytes = d2h + 256;
    }
    if (status & 2)
        return fail(&ctx->err, RTMC_ERR_DEVICE,
                    "a histogram bin reached 2^63 and does not fit int64 at this hist_shift: use rtmc_forward_u32 "
                    "or a smaller hist_shift");
    if (status) return fail(&ctx->err, RTMC_ERR_DEVICE, "a transport guard tripped (event cap or histogram index)");
    return RTMC_OK;
}

int forward(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, int64_t *host_out, rtmc_stats *st,
            double *trace_out = nullptr, uint32_t *host_u32 = nullptr)
{
    Range range(host_u32 ? "rtmc_forward_u32" : (host_out ? "rtmc_forward" : "rtmc_forward_device"));
    if (!ctx || !P) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_forward: NULL argument");
    int s = check_problem(ctx, P, t);
    if (s) return s;
    return P->precision == RTMC_FP64 ? run<double>(ctx, P, t, host_out, st, trace_out, host_u32)
                                     : run<float>(ctx, P, t, host_out, st, trace_out, host_u32);
}

// ---- rtmc_gradient: score-function adjoint replay ----------------------------------

int check_score(rtmc_context *ctx, const rtmc_problem *P, const rtmc_score *sc, const double *adjoint, double *grad)
{
    std::string *e = &ctx->err;
    if (!sc || !adjoint || !grad) return fail(e, RTMC_ERR_ARG, "rtmc_gradient: NULL argument");
    if (!P->acoustics) return fail(e, RTMC_ERR_ARG, "rtmc_gradient: acoustic problems only");
    if (P->qrate[0] != 0)
        return fail(e, RTMC_ERR_ARG, "rtmc_gradient: set qrate = 0 and weight the histogram by exp(-omega t / Q)");
    if (sc->n_params < 1 || sc->n_params > RTMC_MAX_PARAMS)
        return fail(e, RTMC_ERR_ARG, "rtmc_gradient: n_params must be in [1, 8]");
    if (sc->n_theta < 2 || sc->n_theta > (1 << 24) || !sc->dlogsigma)
        return fail(e, RTMC_ERR_ARG, "rtmc_gradient: the d log sigma table needs 2 to 2^24 angles");
    for (int64_t k = 0; k < (int64_t)sc->n_params * sc->n_theta; ++k)
        if (!std::isfinite(sc->dlogsigma[k])) return fail(e, RTMC_ERR_ARG, "rtmc_gradient: d log sigma must be finite");
    for (int q = 0; q < sc->n_params; ++q)
        if (!std::isfinite(sc->dlogSigma[q])) return fail(e, RTMC_ERR_ARG, "rtmc_gradient: d log Sigma must be finite");
    return RTMC_OK;
}

// The split replay of rtmc_gradient: per particle chunk, rt_events writes the segment
// records and each segment's scattering angle, rt_observe_adj sums the adjoint weights per
// segment in lockstep, rt_adjoint_list replays the particles that overflowed; block sums
// are added on the host in a fixed order (chunks, then the observation blocks, then the
// list blocks), so a call is reproducible.
template <typename R>
int gradient_split(rtmc_context *ctx, const rtmc_problem *P, const rtmc_score *sc, DevParams<R> p, AdjointArgs a,
                   int n_edges, size_t hb, size_t sb, size_t n_aux, double *grad, rtmc_stats *st)
{
    const int prec = sizeof(R) == 4 ? RTMC_FP32 : RTMC_FP64;
    const int nm = P->acoustics ? 1 : 2;
    double rate = 0;
    for (int m = 0; m < nm; ++m)
        if (std::isfinite(P->mft[m])) rate = std::max(rate, 1.0 / P->mft[m]);
    const double mean = rate * P->h * (double)P->n_sub * (double)P->n_obs;
    int K = (int)std::ceil(1.0 + mean + 4.0 * std::sqrt(mean) + 4.0);
    K = std::min(64, std::max(8, (K + 3) / 4 * 4));
    if (ctx->opt_ring) K = ctx->opt_ring; // an explicit ring capacity sets the segments per particle
    K = std::max(1, K) + 2;               // and two end records
    const size_t rec = 8 * sizeof(R);
    constexpr int64_t kSegBudget = (int64_t)8 << 30;
    const int64_t chunk = std::min<int64_t>(
        P->n_particles, std::max<int64_t>(32, kSegBudget / ((int64_t)K * (int64_t)(rec + sizeof(R))) / 32 * 32));
    if (ctx->segs.grow((size_t)chunk * K * rec) || ctx->segth.grow((size_t)chunk * K * sizeof(R)) ||
        ctx->ovf.grow((size_t)chunk * 4))
        return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for trajectory segments failed");
    p.sink = 3; // no histogram: the records keep the mode apart from the direction offset
    p.split = 1;
    p.seg_cap = K;
    p.segs = ctx->segs.p;
    p.seg_th = ctx->segth.p;
    p.ovf_list = static_cast<int32_t *>(ctx->ovf.p);
    p.ovf_count = reinterpret_cast<uint32_t *>(static_cast<unsigned char *>(ctx->stats.p) + 192);
    p.clear = nullptr;
    p.clear_words = 0;
    const size_t smem = align_up((size_t)n_edges * sizeof(R), 16);
    int be = 0, bo = 0, bl = 0;
    void *fe = kernel_of(prec, 5, 0, p.obs_kind);
    if (kernel_set_smem(prec, 5, 0, p.obs_kind, smem) != 0 ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&be, fe, 256, smem) != cudaSuccess || be < 1 ||
        adjoint_split_occupancy(prec, 8, p.obs_kind, kAdjointThreads, smem, &bo) != 0 || bo < 1 ||
        adjoint_split_occupancy(prec, 9, p.obs_kind, kAdjointThreads, smem, &bl) != 0 || bl < 1)
        return fail(&ctx->err, RTMC_ERR_CUDA, "split adjoint kernels do not fit on the device");
    const int ge = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->num_sms * be, (chunk + 255) / 256));
    const int go = (int)std::max<int64_t>(
        1, std::min<int64_t>((int64_t)ctx->num_sms * bo, (chunk + kAdjointThreads - 1) / kAdjointThreads));
    const int gl = ctx->num_sms;
    const int np = sc->n_params;
    if (ctx->partial.grow((size_t)(go + gl) * np * sizeof(double)))
        return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the gradient failed");
    a.partial = static_cast<double *>(ctx->partial.p);
    a.partial_list = a.partial + (size_t)go * np;
    std::vector<double> part((size_t)(go + gl) * np);
    std::vector<double> acc(np, 0.0);
    double kms = 0;
    int launches = 0;
    for (int64_t base = 0; base < P->n_particles; base += chunk) {
        DevParams<R> q = p;
        q.pid0 = P->pid0 + base;
        q.n_particles = std::min<int64_t>(chunk, P->n_particles - base);
        CK(cudaMemsetAsync(q.ovf_count, 0, sizeof(uint32_t), ctx->stream), "overflow count");
        CK(cudaEventRecord(ctx->ev_k0, ctx->stream), "event");
        void *ea[] = {(void *)&q};
        void *oa[] = {(void *)&q, (void *)&a};
        cudaError_t e = cudaLaunchKernel(fe, dim3(ge), dim3(256), ea, smem, ctx->stream);
        if (e == cudaSuccess)
            e = cudaLaunchKernel(kernel_of(prec, 8, 0, p.obs_kind), dim3(go), dim3(kAdjointThreads), oa, smem, ctx->stream);
        if (e == cudaSuccess)
            e = cudaLaunchKernel(kernel_of(prec, 9, 0, p.obs_kind), dim3(gl), dim3(kAdjointThreads), oa, smem, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "split adjoint launch");
        launches += 3;
        CK(cudaEventRecord(ctx->ev_k1, ctx->stream), "event");
        CK(cudaMemcpyAsync(part.data(), a.partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
           "partial sums");
        CK(cudaStreamSynchronize(ctx->stream), "adjoint");
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev_k0, ctx->ev_k1);
        kms += ms;
        for (int qq = 0; qq < np; ++qq) {
            double v = 0.0;
            for (int b = 0; b < go + gl; ++b) v += part[(size_t)b * np + qq];
            acc[qq] += v;
        }
    }
    int64_t dstats[32];
    CK(cudaMemcpyAsync(dstats, ctx->stats.p, 256, cudaMemcpyDeviceToHost, ctx->stream), "counters");
    CK(cudaEventRecord(ctx->ev_end, ctx->stream), "event");
    CK(cudaStreamSynchronize(ctx->stream), "adjoint");
    for (int qq = 0; qq < np; ++qq) grad[qq] = acc[qq];
    float tms = 0;
    cudaEventElapsedTime(&tms, ctx->ev_start, ctx->ev_end);
    ctx->last_kernel_ms = kms;
    ctx->last_launches = launches;
    const int32_t status = (int32_t)(dstats[16] & 0xffffffff);
    if (st) {
        std::memset(st, 0, sizeof *st);
        st->scatter_events = dstats[0];
        st->boundary_hits = dstats[1];
        st->kills = dstats[2];
        st->absorbed = dstats[3];
        st->observations = dstats[4];
        st->conversions = dstats[5];
        st->device_status = status;
        st->kernel_ms = kms;
        st->launches = launches;
        st->total_ms = tms;
        st->h2d_bytes = (double)(hb + sb + n_aux * sizeof(R));
        st->d2h_bytes = (double)(part.size() * sizeof(double) + 256);
    }
    if (status) return fail(&ctx->err, RTMC_ERR_DEVICE, "an adjoint guard tripped (event cap or histogram index)");
    return RTMC_OK;
}

template <typename R>
int gradient_run(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, const rtmc_score *sc,
                 const double *adjoint, double *grad, rtmc_stats *st)
{
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaEventRecord(ctx->ev_start, ctx->stream), "event");
    DevTables<R> *dt;
    if constexpr (sizeof(R) == 4) dt = &ctx->tf; else dt = &ctx->td;
    const int prec = sizeof(R) == 4 ? RTMC_FP32 : RTMC_FP64;
    if (!ctx->cache_tables || ctx->tabs_gen != t->gen || ctx->tabs_prec != prec) {
        int s = upload_tables<R>(ctx, t, dt);
        if (s) { ctx->tabs_gen = 0; return s; }
        ctx->tabs_gen = t->gen;
        ctx->tabs_prec = prec;
    }
    DevParams<R> p;
    std::vector<R> edges, zoe;
    int n_edges = 0;
    fill_params<R>(ctx, P, *dt, &p, &n_edges, &edges, &zoe);
    const size_t eb = align_up(std::max<size_t>(1, edges.size()) * sizeof(R), 256);
    const size_t zb = align_up(zoe.size() * sizeof(R), 256);
    const size_t hb = (size_t)P->hist_len * sizeof(R);
    const size_t sb = (size_t)sc->n_params * sc->n_theta * sizeof(double);
    const size_t sbf = (size_t)sc->n_params * sc->n_theta * sizeof(float);
    if (ctx->aux.grow(eb + zb) || ctx->stats.grow(256) || ctx->adj.grow(align_up(hb, 256) + align_up(sb, 256) + sbf))
        return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the gradient failed");
    unsigned char *aux = static_cast<unsigned char *>(ctx->aux.p);
    if (!edges.empty())
        CK(cudaMemcpyAsync(aux, edges.data(), edges.size() * sizeof(R), cudaMemcpyHostToDevice, ctx->stream), "edges");
    CK(cudaMemcpyAsync(aux + eb, zoe.data(), zoe.size() * sizeof(R), cudaMemcpyHostToDevice, ctx->stream), "zoeppritz");
    unsigned char *ab = static_cast<unsigned char *>(ctx->adj.p);
    if constexpr (sizeof(R) == 8) {
        CK(cudaMemcpyAsync(ab, adjoint, hb, cudaMemcpyHostToDevice, ctx->stream), "adjoint weights");
    } else {
        std::vector<R> wr((size_t)P->hist_len);
        for (size_t k = 0; k < wr.size(); ++k) wr[k] = (R)adjoint[k];
        CK(cudaMemcpyAsync(ab, wr.data(), hb, cudaMemcpyHostToDevice, ctx->stream), "adjoint weights");
        CK(cudaStreamSynchronize(ctx->stream), "adjoint weights"); // wr is released on return
    }
    CK(cudaMemcpyAsync(ab + align_up(hb, 256), sc->dlogsigma, sb, cudaMemcpyHostToDevice, ctx->stream), "score table");
    std::vector<float> dls_f((size_t)sc->n_params * sc->n_theta);
    for (size_t k = 0; k < dls_f.size(); ++k) dls_f[k] = (float)sc->dlogsigma[k];
    CK(cudaMemcpyAsync(ab + align_up(hb, 256) + align_up(sb, 256), dls_f.data(), sbf, cudaMemcpyHostToDevice,
                       ctx->stream), "score table");
    CK(cudaStreamSynchronize(ctx->stream), "score table"); // dls_f is released on return
    CK(cudaMemsetAsync(ctx->stats.p, 0, 256, ctx->stream), "counter clear");
    p.edges = reinterpret_cast<const R *>(aux);
    p.zoe = reinterpret_cast<const R *>(aux + eb);
    p.src_radial = p.zoe + 2 * RTMC_ZOE_N;
    p.hist = nullptr;
    p.stats = static_cast<unsigned long long *>(ctx->stats.p);
    p.status = reinterpret_cast<int32_t *>(static_cast<unsigned char *>(ctx->stats.p) + 128);
    p.trace = nullptr;
    AdjointArgs a{};
    a.adjoint = ab;
    a.dlogsigma = reinterpret_cast<const double *>(ab + align_up(hb, 256));
    a.dlogsigma_f = reinterpret_cast<const float *>(ab + align_up(hb, 256) + align_up(sb, 256));
    a.n_params = sc->n_params;
    a.n_theta = sc->n_theta;
    // per-sub-step scattering probability 1 - exp(-h Sigma), Sigma = 1 / mean free time
    const double hS = std::isfinite(P->mft[0]) ? P->h / P->mft[0] : 0.0;
    const double kappa = hS > 0 ? hS / std::expm1(hS) : 1.0;
    for (int q = 0; q < sc->n_params; ++q) {
        a.a_inc[q] = sc->dlogSigma[q] * (kappa - 1.0 + hS);
        a.a_inc_f[q] = (float)a.a_inc[q];
        a.b_obs[q] = -sc->dlogSigma[q] * hS * (double)P->n_sub;
    }
    const int block = kAdjointThreads;
    // up to 4 parameters: the split replay (rt_events, then rt_observe_adj and the overflow
    // reruns), or the converged two-phase replay with a segment ring; more: one particle
    // per thread
    const bool ring = sc->n_params <= kAdjointRingParams;
    // (schedules 0 and 1 of rtmc_set_schedule keep the ring replay)
    if (ring && ctx->opt_event_major != 0 && ctx->opt_event_major != 1 && P->n_particles > 0 &&
        P->hist_len < ((int64_t)1 << 31) && P->n_obs < (1 << 24))
        return gradient_split<R>(ctx, P, sc, p, a, n_edges, hb, sb, edges.size() + zoe.size(), grad, st);
    // FP32: 4 ring slots let 3 blocks share an SM (C5: 12.5 ms against 14.4 with 8 slots
    // and 2 blocks)
    const int cap = ctx->opt_ring ? ctx->opt_ring : (sizeof(R) == 4 ? 4 : 6);
    size_t smem = align_up((size_t)n_edges * sizeof(R), 16);
    if (ring) smem += (size_t)block * cap * (7 * sizeof(R) + 2 * sizeof(int32_t));
    p.ring_cap = cap;
    int bps = 0;
    if ((ring ? adjoint_ring_occupancy(prec, p.obs_kind, block, smem, &bps)
              : adjoint_occupancy(prec, p.obs_kind, block, smem, &bps)) != 0 || bps < 1)
        return fail(&ctx->err, RTMC_ERR_CUDA, "adjoint kernel does not fit on the device");
    const int64_t need = (std::max<int64_t>(P->n_particles, 1) + block - 1) / block;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->num_sms * bps, need));
    if (ctx->partial.grow((size_t)grid * sc->n_params * sizeof(double)))
        return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the gradient failed");
    a.partial = static_cast<double *>(ctx->partial.p);
    CK(cudaEventRecord(ctx->ev_k0, ctx->stream), "event");
    int le;
    if constexpr (sizeof(R) == 4)
        le = ring ? launch_adjoint_ring_f32(p, a, grid, block, smem, ctx->stream)
                  : launch_adjoint_f32(p, a, grid, block, smem, ctx->stream);
    else
        le = ring ? launch_adjoint_ring_f64(p, a, grid, block, smem, ctx->stream)
                  : launch_adjoint_f64(p, a, grid, block, smem, ctx->stream);
    if (le) return cuda_fail(ctx, (cudaError_t)le, "adjoint launch");
    CK(cudaEventRecord(ctx->ev_k1, ctx->stream), "event");
    std::vector<double> part((size_t)grid * sc->n_params);
    int64_t dstats[32];
    CK(cudaMemcpyAsync(part.data(), a.partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
       "partial sums");
    CK(cudaMemcpyAsync(dstats, ctx->stats.p, 256, cudaMemcpyDeviceToHost, ctx->stream), "counters");
    CK(cudaEventRecord(ctx->ev_end, ctx->stream), "event");
    CK(cudaStreamSynchronize(ctx->stream), "adjoint");
    for (int q = 0; q < sc->n_params; ++q) {
        double acc = 0.0;
        for (int b = 0; b < grid; ++b) acc += part[(size_t)b * sc->n_params + q];
        grad[q] = acc;
    }
    float kms = 0, tms = 0;
    cudaEventElapsedTime(&kms, ctx->ev_k0, ctx->ev_k1);
    cudaEventElapsedTime(&tms, ctx->ev_start, ctx->ev_end);
    ctx->last_kernel_ms = kms;
    ctx->last_launches = 1;
    const int32_t status = (int32_t)(dstats[16] & 0xffffffff);
    if (st) {
        std::memset(st, 0, sizeof *st);
        st->scatter_events = dstats[0];
        st->boundary_hits = dstats[1];
        st->kills = dstats[2];
        st->absorbed = dstats[3];
        st->observations = dstats[4];
        st->conversions = dstats[5];
        st->device_status = status;
        st->kernel_ms = kms;
        st->launches = 1;
        st->total_ms = tms;
        st->h2d_bytes = (double)(hb + sb + (edges.size() + zoe.size()) * sizeof(R));
        st->d2h_bytes = (double)(part.size() * sizeof(double) + 256);
    }
    if (status) return fail(&ctx->err, RTMC_ERR_DEVICE, "an adjoint guard tripped (event cap or histogram index)");
    return RTMC_OK;
}

// ---- rtmc_forward_noalloc: everything staged in the static device scratch ----------

// fixed-capacity vector on the stack (fill_params' edge and Zoeppritz lists)
// Host staging area of rtmc_forward_noalloc.  It is file-scope, so a call allocates
// nothing and keeps no large stack frame (callers may run on small worker-thread stacks).
// Two halves alternate: a half is filled while the other's copy runs, and the stream is
// synchronised only before a half is refilled, about once per megabyte of tables.  The
// fixed-size edge and Zoeppritz lists live here too.  g_stage_mu serialises the calls of
// the threads of one process.
constexpr size_t kStageHalf = (size_t)1 << 20;
constexpr size_t kListBytes = (2 * RTMC_ZOE_N + 2 * (size_t)RTMC_MAX_RADIAL) * sizeof(double);
alignas(256) unsigned char g_stage[2 * kStageHalf];
alignas(256) unsigned char g_lists[2][kListBytes];
std::mutex g_stage_mu;

// push_back list over a fixed area (fill_params' edge and Zoeppritz lists); values past
// the capacity are counted in `over` rather than stored
template <typename R> struct FixedVec {
    R *v;
    size_t cap, n = 0, over = 0;
    FixedVec(void *area, size_t bytes) : v(static_cast<R *>(area)), cap(bytes / sizeof(R)) {}
    void clear() { n = over = 0; }
    void push_back(R x) { if (n < cap) v[n++] = x; else ++over; }
    void resize(size_t k) { if (k <= cap) n = k; else { n = cap; over += k - cap; } }
    size_t size() const { return n; }
    R &operator[](size_t i) { return v[i]; }
    R *data() { return v; }
};

struct Stager {
    cudaStream_t st;
    int half = 0;
    bool busy[2] = {false, false};
    // a half of the staging area that is free to fill
    int take(unsigned char **out)
    {
        if (busy[half]) {
            const cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return (int)e;
            busy[0] = busy[1] = false;
        }
        *out = g_stage + (size_t)half * kStageHalf;
        return 0;
    }
    // copy the first `bytes` of the half just filled to dst; the next take() uses the other half
    int send(unsigned char *dst, size_t bytes)
    {
        const cudaError_t e = cudaMemcpyAsync(dst, g_stage + (size_t)half * kStageHalf, bytes, cudaMemcpyHostToDevice, st);
        busy[half] = true;
        half ^= 1;
        return (int)e;
    }
};

// host -> device copy of a list that stays untouched until the call has synchronised
template <typename T> int copy_list(unsigned char *dst, const T *src, size_t count, cudaStream_t st)
{
    return (int)cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, st);
}

// same layout as upload_tables, written through the staging area in chunks
template <typename R>
int stage_tables_static(const rtmc_tables *t, unsigned char *base, size_t cap, size_t *used, DevTables<R> *dt,
                        Stager &sg, std::string *err)
{
    size_t off[4], total = 0;
    for (int i = 0; i < t->n_tables; ++i) {
        off[i] = total;
        total += table_bytes<R>(t->cdf[i].size());
    }
    if (total > cap)
        return fail(err, RTMC_ERR_ARG, "rtmc_forward_noalloc: the tables need " + std::to_string(total) +
                                            " bytes, more than the static scratch of " + std::to_string(cap) + " bytes");
    constexpr size_t KB = kStageHalf / sizeof(Knot<R>), GB = kStageHalf / sizeof(int32_t);
    for (int i = 0; i < t->n_tables; ++i) {
        const std::vector<double> &c = t->cdf[i], &th = t->theta[i];
        const size_t n = c.size();
        const int bits = guide_bits(n);
        unsigned char *kd = base + off[i];
        unsigned char *gd = kd + align_up(n * sizeof(Knot<R>), 256);
        unsigned char *h = nullptr;
        int e;
        for (size_t k0 = 0; k0 < n; k0 += KB) {
            const size_t m = std::min(KB, n - k0);
            if ((e = sg.take(&h))) return e;
            fill_knots<R>(c, th, k0, m, reinterpret_cast<Knot<R> *>(h));
            if ((e = sg.send(kd + k0 * sizeof(Knot<R>), m * sizeof(Knot<R>)))) return e;
        }
        const int64_t ng = ((int64_t)1 << bits) + 1;
        size_t k = 0;
        for (int64_t j0 = 0; j0 < ng; j0 += (int64_t)GB) {
            const int64_t m = std::min<int64_t>((int64_t)GB, ng - j0);
            if ((e = sg.take(&h))) return e;
            fill_guide(c, bits, j0, m, &k, reinterpret_cast<int32_t *>(h));
            if ((e = sg.send(gd + (size_t)j0 * sizeof(int32_t), (size_t)m * sizeof(int32_t)))) return e;
        }
        dt->knot[i] = reinterpret_cast<const Knot<R> *>(kd);
        dt->guide[i] = reinterpret_cast<const int32_t *>(gd);
        dt->n[i] = (int32_t)n;
        dt->gbits[i] = bits;
    }
    *used = total;
    return RTMC_OK;
}

template <typename R>
int forward_noalloc(const rtmc_problem *P, const rtmc_tables *t, int64_t *d_hist, cudaStream_t st, rtmc_stats *stats)
{
    rtmc_context slot; // error slot for check_problem; owns no device resources
    int s = check_problem(&slot, P, t);
    if (s) return fail(nullptr, s, slot.err);
    std::lock_guard<std::mutex> lock(g_stage_mu);
    std::string err;
    int dev = 0, sms = 0, smem_optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return fail(nullptr, RTMC_ERR_CUDA, std::string("rtmc_forward_noalloc: ") + cudaGetErrorString(e));
    unsigned char *base = nullptr;
    size_t cap = 0;
    if ((s = static_scratch(dev, &base, &cap)) != 0)
        return fail(nullptr, RTMC_ERR_CUDA, std::string("rtmc_forward_noalloc: static scratch lookup: ") +
                                                cudaGetErrorString((cudaError_t)s));
    const int prec = sizeof(R) == 4 ? RTMC_FP32 : RTMC_FP64;
    DevTables<R> dt{};
    size_t used = 0;
    Stager sg{st};
    if ((s = stage_tables_static<R>(t, base, cap, &used, &dt, sg, &err)) != 0)
        return s == RTMC_ERR_ARG ? fail(nullptr, s, err) : fail(nullptr, RTMC_ERR_CUDA, "rtmc_forward_noalloc: table staging");
    DevParams<R> p;
    FixedVec<R> edges(g_lists[0], sizeof g_lists[0]);
    FixedVec<R> zoe(g_lists[1], sizeof g_lists[1]); // 2 x 181 Zoeppritz values and the radial table
    int n_edges = 0;
    fill_params<R>(&slot, P, dt, &p, &n_edges, &edges, &zoe);
    if (edges.over || zoe.over) return fail(nullptr, RTMC_ERR_ARG, "rtmc_forward_noalloc: edge or source tables too long");
    p.event_major = 0; // index path: each warp writes its 32 rows together
    const size_t e_off = align_up(used, 256);
    const size_t z_off = align_up(e_off + std::max<size_t>(1, edges.size()) * sizeof(R), 256);
    const size_t c_off = align_up(z_off + zoe.size() * sizeof(R), 256);
    const size_t i_off = align_up(c_off + 256, 256);
    const int64_t rows = i_off < cap ? (int64_t)((cap - i_off) / (4 * (size_t)P->n_obs)) / 32 * 32 : 0;
    if (rows < 32)
        return fail(nullptr, RTMC_ERR_ARG, "rtmc_forward_noalloc: tables, edges and 32 particles x " +
                                               std::to_string(P->n_obs) + " observations need more than the static scratch of " +
                                               std::to_string(cap) + " bytes");
    if (P->time_stride >= ((int64_t)1 << 30))
        return fail(nullptr, RTMC_ERR_ARG, "rtmc_forward_noalloc: a time slice must hold fewer than 2^30 bins");
    if (edges.size() && (s = copy_list(base + e_off, edges.data(), edges.size(), st)) != 0)
        return fail(nullptr, RTMC_ERR_CUDA, "rtmc_forward_noalloc: edge staging");
    if ((s = copy_list(base + z_off, zoe.data(), zoe.size(), st)) != 0)
        return fail(nullptr, RTMC_ERR_CUDA, "rtmc_forward_noalloc: Zoeppritz staging");
    e = cudaMemsetAsync(d_hist, 0, (size_t)P->hist_len * sizeof(int64_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + c_off, 0, 256, st);
    if (e != cudaSuccess) return fail(nullptr, RTMC_ERR_CUDA, std::string("rtmc_forward_noalloc: ") + cudaGetErrorString(e));
    p.edges = reinterpret_cast<const R *>(base + e_off);
    p.zoe = reinterpret_cast<const R *>(base + z_off);
    p.src_radial = p.zoe + 2 * RTMC_ZOE_N;
    p.hist = reinterpret_cast<unsigned long long *>(d_hist);
    p.stats = reinterpret_cast<unsigned long long *>(base + c_off);
    p.status = reinterpret_cast<int32_t *>(base + c_off + 128);
    p.trace = nullptr;
    p.sink = kSinkIndex;
    p.ring_cap = sizeof(R) == 4 ? 8 : 6;
    p.obs_idx = reinterpret_cast<int32_t *>(base + i_off);
    const int64_t chunk = std::min<int64_t>(std::max<int64_t>(P->n_particles, 1), rows);
    p.obs_rows = index_row_stride(chunk); // <= rows, a multiple of 32
    int block = 256;
    const int mt = transport_max_threads(prec, kSinkIndex, p.obs_kind);
    if (mt > 0 && block > mt) block = mt - mt % 32;
    const size_t seg_bytes = 6 * sizeof(R) + 2 * sizeof(int32_t);
    const size_t smem = align_up((size_t)n_edges * sizeof(R), 16) + (size_t)block * p.ring_cap * seg_bytes;
    int bps = 0;
    if (transport_set_smem(prec, kSinkIndex, p.obs_kind, smem) != 0 ||
        transport_occupancy(prec, kSinkIndex, p.obs_kind, block, smem, &bps) != 0 || bps < 1)
        return fail(nullptr, RTMC_ERR_CUDA, "rtmc_forward_noalloc: transport kernel does not fit on the device");
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * bps, (chunk + block - 1) / block));
    BinParams bp{};
    bp.idx = p.obs_idx;
    bp.rows = p.obs_rows;
    bp.n_obs = P->n_obs;
    bp.j_first = 1; // every slice (large slices take rt_bin_slices, which reads the range)
    bp.j_count = P->n_obs;
    bp.n_modes = P->acoustics ? 1 : 2;
    bp.slice_bins = (int32_t)P->time_stride;
    bp.time_stride = P->time_stride;
    bp.mode_stride = P->mode_stride;
    bp.hist_shift = P->hist_shift;
    bp.hist = p.hist;
    const size_t slice_bytes = (size_t)P->time_stride * bp.n_modes * sizeof(uint32_t);
    const int group = (int)std::min<size_t>((size_t)P->n_obs, (size_t)(200 << 10) / std::max<size_t>(slice_bytes, 1));
    size_t fold_smem = 0;
    int fold_grid = 1;
    if (group >= 8) {
        bp.group = group;
        fold_smem = (size_t)group * slice_bytes;
        if (bin_slices_set_smem(fold_smem) != 0) return fail(nullptr, RTMC_ERR_CUDA, "rtmc_forward_noalloc: fold attributes");
        const int ngroups = (P->n_obs + group - 1) / group;
        fold_grid = (int)std::max<int64_t>(1, (2 * sms + ngroups - 1) / ngroups);
    } else {
        fold_grid = (int)std::max<int64_t>(1, std::min<int64_t>((chunk + 16383) / 16384, sms));
    }
    int launches = 0;
    for (int64_t b0 = 0; b0 < P->n_particles; b0 += chunk) {
        DevParams<R> q = p;
        q.pid0 = P->pid0 + b0;
        q.n_particles = std::min<int64_t>(chunk, P->n_particles - b0);
        int le;
        if constexpr (sizeof(R) == 4) le = launch_transport_f32(q, (int)grid, block, smem, st);
        else le = launch_transport_f64(q, (int)grid, block, smem, st);
        if (le) return fail(nullptr, RTMC_ERR_CUDA, std::string("rtmc_forward_noalloc: ") + cudaGetErrorString((cudaError_t)le));
        BinParams b = bp;
        b.n = q.n_particles;
        if (b.group) b.part_per_block = (b.n + fold_grid - 1) / fold_grid;
        if ((le = launch_bin_slices(b, fold_grid, fold_smem, st)) != 0)
            return fail(nullptr, RTMC_ERR_CUDA, std::string("rtmc_forward_noalloc: ") + cudaGetErrorString((cudaError_t)le));
        launches += 2;
    }
    int64_t dstats[32];
    e = cudaMemcpyAsync(dstats, base + c_off, 256, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(nullptr, RTMC_ERR_CUDA, std::string("rtmc_forward_noalloc: ") + cudaGetErrorString(e));
    const int32_t status = (int32_t)(dstats[16] & 0xffffffff);
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        stats->scatter_events = dstats[0];
        stats->boundary_hits = dstats[1];
        stats->kills = dstats[2];
        stats->absorbed = dstats[3];
        stats->observations = dstats[4];
        stats->conversions = dstats[5];
        stats->device_status = status;
        stats->launches = launches;
        stats->sink = kSinkIndex;
        stats->h2d_bytes = (double)used + (double)(edges.size() + zoe.size()) * sizeof(R);
        stats->d2h_bytes = 256;
    }
    if (status) return fail(nullptr, RTMC_ERR_DEVICE, "rtmc_forward_noalloc: a transport guard tripped");
    return RTMC_OK;
}

} // namespace

extern "C" int32_t rtmc_abi_version(void) { return RTMC_ABI_VERSION; }

extern "C" int rtmc_abi_sizes(int64_t out[4])
{
    if (!out) return fail(nullptr, RTMC_ERR_ARG, "rtmc_abi_sizes: NULL argument");
    out[0] = (int64_t)sizeof(rtmc_material);
    out[1] = (int64_t)sizeof(rtmc_tables_info);
    out[2] = (int64_t)sizeof(rtmc_problem);
    out[3] = (int64_t)sizeof(rtmc_stats);
    return RTMC_OK;
}

extern "C" int rtmc_create(int32_t device, rtmc_context **out)
{
    if (!out) return fail(nullptr, RTMC_ERR_ARG, "rtmc_create: NULL argument");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(nullptr, RTMC_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= n) return fail(nullptr, RTMC_ERR_ARG, "device index out of range");
    auto *ctx = new (std::nothrow) rtmc_context();
    if (!ctx) return fail(nullptr, RTMC_ERR_ALLOC, "out of host memory");
    ctx->device = device;
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_start);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_k0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_k1);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_k2);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_end);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_km);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_kc);
    if (e != cudaSuccess) {
        rtmc_destroy(ctx);
        return fail(nullptr, RTMC_ERR_CUDA, std::string("rtmc_create: ") + cudaGetErrorString(e));
    }
    *out = ctx;
    return RTMC_OK;
}

extern "C" void rtmc_destroy(rtmc_context *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->fold_stream) cudaStreamSynchronize(ctx->fold_stream);
    ctx->hist.release();
    ctx->narrow.release();
    ctx->tabs.release();
    ctx->aux.release();
    ctx->stats.release();
    ctx->flush.release();
    ctx->trace.release();
    ctx->idx.release();
    ctx->adj.release();
    ctx->partial.release();
    ctx->segs.release();
    ctx->ovf.release();
    ctx->order.release();
    ctx->segth.release();
    ctx->tbacc.release();
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_k0) cudaEventDestroy(ctx->ev_k0);
    if (ctx->ev_km) cudaEventDestroy(ctx->ev_km);
    if (ctx->ev_kc) cudaEventDestroy(ctx->ev_kc);
    if (ctx->ev_k1) cudaEventDestroy(ctx->ev_k1);
    if (ctx->ev_k2) cudaEventDestroy(ctx->ev_k2);
    if (ctx->ev_end) cudaEventDestroy(ctx->ev_end);
    for (int i = 0; i < rtmc_context::kPipe; ++i) {
        if (ctx->ev_a0[i]) cudaEventDestroy(ctx->ev_a0[i]);
        if (ctx->ev_a1[i]) cudaEventDestroy(ctx->ev_a1[i]);
        if (ctx->ev_b0[i]) cudaEventDestroy(ctx->ev_b0[i]);
        if (ctx->ev_b1[i]) cudaEventDestroy(ctx->ev_b1[i]);
    }
    if (ctx->fold_stream) cudaStreamDestroy(ctx->fold_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" const char *rtmc_last_error(const rtmc_context *ctx)
{
    if (ctx) return ctx->err.c_str();
    return g_thread_error.c_str();
}

extern "C" int rtmc_forward(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, int64_t *hist_out,
                            rtmc_stats *st)
{
    if (!hist_out) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_forward: hist_out is NULL");
    return forward(ctx, P, t, hist_out, st);
}

extern "C" int rtmc_forward_u32(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, uint32_t *hist_out,
                                rtmc_stats *st)
{
    if (!hist_out) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_forward_u32: hist_out is NULL");
    return forward(ctx, P, t, nullptr, st, nullptr, hist_out);
}

extern "C" int rtmc_forward_device(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, rtmc_stats *st)
{
    return forward(ctx, P, t, nullptr, st);
}

extern "C" int rtmc_forward_trace(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, int64_t *hist_out,
                                  double *state_out, rtmc_stats *st)
{
    if (!hist_out || !state_out)
        return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_forward_trace: NULL output buffer");
    return forward(ctx, P, t, hist_out, st, state_out);
}

extern "C" int rtmc_gradient(rtmc_context *ctx, const rtmc_problem *P, const rtmc_tables *t, const rtmc_score *score,
                             const double *adjoint, double *grad, rtmc_stats *st)
{
    Range range("rtmc_gradient");
    if (!ctx || !P) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_gradient: NULL argument");
    int s = check_problem(ctx, P, t);
    if (s) return s;
    if ((s = check_score(ctx, P, score, adjoint, grad)) != 0) return s;
    return P->precision == RTMC_FP64 ? gradient_run<double>(ctx, P, t, score, adjoint, grad, st)
                                     : gradient_run<float>(ctx, P, t, score, adjoint, grad, st);
}

extern "C" int rtmc_copy_histogram(rtmc_context *ctx, int64_t *hist_out, int64_t n)
{
    if (!ctx || !hist_out) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_copy_histogram: NULL argument");
    if (n < 0 || n > ctx->hist_len) return fail(&ctx->err, RTMC_ERR_ARG, "rtmc_copy_histogram: n exceeds the histogram");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    int32_t flag = 0;
    int32_t *status = reinterpret_cast<int32_t *>(static_cast<unsigned char *>(ctx->stats.p) + 128);
    if (ctx->hist_may_exceed_int64) {
        CK(cudaMemsetAsync(status, 0, sizeof(int32_t), ctx->stream), "status clear");
        const int le = launch_check_int64(static_cast<const unsigned long long *>(ctx->hist.p), n, status,
                                          8 * ctx->num_sms, ctx->stream);
        if (le) return cuda_fail(ctx, (cudaError_t)le, "histogram range check");
        CK(cudaMemcpyAsync(&flag, status, sizeof flag, cudaMemcpyDeviceToHost, ctx->stream), "status");
    }
    CK(cudaMemcpyAsync(hist_out, ctx->hist.p, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream), "histogram copy");
    CK(cudaStreamSynchronize(ctx->stream), "histogram copy");
    if (flag & 2)
        return fail(&ctx->err, RTMC_ERR_DEVICE, "a histogram bin reached 2^63 and does not fit int64 at this hist_shift");
    return RTMC_OK;
}

extern "C" int rtmc_histogram_device(rtmc_context *ctx, void **ptr, int64_t *n)
{
    if (!ctx || !ptr || !n) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_histogram_device: NULL argument");
    if (!ctx->hist.p || ctx->hist_len <= 0) return fail(&ctx->err, RTMC_ERR_ARG, "rtmc_histogram_device: no histogram yet");
    *ptr = ctx->hist.p;
    *n = ctx->hist_len;
    return RTMC_OK;
}

extern "C" int rtmc_forward_noalloc(const rtmc_problem *P, const rtmc_tables *t, int64_t *hist_device, void *stream,
                                    rtmc_stats *stats)
{
    if (!P || !t || !hist_device) return fail(nullptr, RTMC_ERR_ARG, "rtmc_forward_noalloc: NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return P->precision == RTMC_FP64 ? forward_noalloc<double>(P, t, hist_device, st, stats)
                                     : forward_noalloc<float>(P, t, hist_device, st, stats);
}

extern "C" int rtmc_host_alloc(int64_t bytes, void **out)
{
    if (!out || bytes <= 0) return fail(nullptr, RTMC_ERR_ARG, "rtmc_host_alloc: bad argument");
    cudaError_t e = cudaMallocHost(out, (size_t)bytes);
    if (e != cudaSuccess) { *out = nullptr; return fail(nullptr, RTMC_ERR_ALLOC, "cudaMallocHost failed"); }
    return RTMC_OK;
}

extern "C" int rtmc_host_free(void *p)
{
    if (p && cudaFreeHost(p) != cudaSuccess) return fail(nullptr, RTMC_ERR_CUDA, "cudaFreeHost failed");
    return RTMC_OK;
}

extern "C" int rtmc_set_launch(rtmc_context *ctx, int32_t block, int32_t ring_cap, int32_t index_mb)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_launch: NULL context");
    if (block < 0 || block > 1024 || block % 32) return fail(&ctx->err, RTMC_ERR_ARG, "block must be 0 or a multiple of 32 up to 1024");
    if (ring_cap < 0 || ring_cap == 1 || ring_cap > 64) return fail(&ctx->err, RTMC_ERR_ARG, "ring_cap must be 0 or in [2, 64]");
    if (index_mb < -1) return fail(&ctx->err, RTMC_ERR_ARG, "index_mb must be -1, 0 or a size in MB");
    ctx->opt_block = block;
    ctx->opt_ring = ring_cap;
    ctx->opt_index_mb = index_mb;
    return RTMC_OK;
}

extern "C" int rtmc_set_pipeline(rtmc_context *ctx, int32_t chunks, int32_t transport_blocks_per_sm)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_pipeline: NULL context");
    if (chunks < 0 || chunks > rtmc_context::kPipe) return fail(&ctx->err, RTMC_ERR_ARG, "chunks must be in [0, 32]");
    if (transport_blocks_per_sm < 0 || transport_blocks_per_sm > 16)
        return fail(&ctx->err, RTMC_ERR_ARG, "transport_blocks_per_sm must be in [0, 16]");
    ctx->opt_chunks = chunks;
    ctx->opt_k1_bps = transport_blocks_per_sm;
    return RTMC_OK;
}

extern "C" int rtmc_set_schedule(rtmc_context *ctx, int32_t event_major)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_schedule: NULL context");
    if (event_major < -1 || event_major > 2) return fail(&ctx->err, RTMC_ERR_ARG, "schedule must be -1, 0, 1 or 2");
    ctx->opt_event_major = event_major;
    return RTMC_OK;
}

extern "C" int rtmc_set_fold(rtmc_context *ctx, int32_t mode)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_fold: NULL context");
    if (mode < 0 || mode > 3) return fail(&ctx->err, RTMC_ERR_ARG, "fold mode must be 0, 1, 2 or 3");
    ctx->opt_fold = mode;
    return RTMC_OK;
}

extern "C" int rtmc_set_particle_order(rtmc_context *ctx, int32_t enable)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_particle_order: NULL context");
    ctx->opt_order = enable ? 1 : 0;
    return RTMC_OK;
}

extern "C" int rtmc_set_fp64_estimate(rtmc_context *ctx, int32_t enable)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_fp64_estimate: NULL context");
    ctx->opt_bin32 = enable ? 1 : 0;
    return RTMC_OK;
}

extern "C" int rtmc_set_early_copy(rtmc_context *ctx, int32_t first_percent)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_early_copy: NULL context");
    if (first_percent < -1 || first_percent > 99)
        return fail(&ctx->err, RTMC_ERR_ARG, "rtmc_set_early_copy: first_percent in [0, 99], or -1 for the default");
    ctx->opt_early_copy = first_percent < 0 ? kEarlyCopyPercent : first_percent;
    return RTMC_OK;
}

extern "C" int rtmc_set_table_cache(rtmc_context *ctx, int32_t enable)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_set_table_cache: NULL context");
    ctx->cache_tables = enable ? 1 : 0;
    return RTMC_OK;
}

extern "C" int rtmc_flush_l2(rtmc_context *ctx)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_flush_l2: NULL context");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t bytes = (size_t)512 << 20;
    if (ctx->flush.grow(bytes)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the L2 flush failed");
    CK(cudaMemsetAsync(ctx->flush.p, 0x5a, bytes, ctx->stream), "L2 flush");
    CK(cudaStreamSynchronize(ctx->stream), "L2 flush");
    return RTMC_OK;
}

extern "C" int rtmc_probe_l2_reductions(rtmc_context *ctx, double *reductions_per_s)
{
    if (!ctx || !reductions_per_s) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_probe_l2_reductions: NULL argument");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    // 4M slots of 16 bytes (64 MB, L2-resident, the size of one t-block of the fold's
    // accumulator on the 3D elastic workload) in the flush buffer; 8 blocks of 256 per SM
    constexpr uint32_t kSlots = 1u << 22;
    constexpr int kIters = 512;
    if (ctx->flush.grow((size_t)512 << 20)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the probe failed");
    float *buf = static_cast<float *>(ctx->flush.p);
    const int grid = ctx->num_sms * 8;
    double best = 0;
    for (int rep = 0; rep < 4; ++rep) { // the first is a warm-up
        CK(cudaEventRecord(ctx->ev_k0, ctx->stream), "event");
        const int le = launch_probe_red(buf, kSlots, grid, kIters, ctx->stream);
        if (le) return cuda_fail(ctx, (cudaError_t)le, "probe launch");
        CK(cudaEventRecord(ctx->ev_k1, ctx->stream), "event");
        CK(cudaEventSynchronize(ctx->ev_k1), "probe");
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev_k0, ctx->ev_k1);
        const double rate = (double)grid * 256.0 * kIters / (ms * 1e-3);
        if (rep > 0 && rate > best) best = rate;
    }
    *reductions_per_s = best;
    return RTMC_OK;
}

extern "C" int rtmc_last_timing(const rtmc_context *ctx, double *kernel_ms, int32_t *launches)
{
    if (!ctx) return fail(nullptr, RTMC_ERR_ARG, "rtmc_last_timing: NULL context");
    if (kernel_ms) *kernel_ms = ctx->last_kernel_ms;
    if (launches) *launches = ctx->last_launches;
    return RTMC_OK;
}

// ---- batched runs ----------------------------------------------------------------

struct rtmc_batch {
    rtmc_context *ctx = nullptr;
    int n = 0, prec = RTMC_FP32, obs_kind = 0, n_obs = 0;
    int block = 0, ring = 0, grid = 0, n_items = 0;
    int grid_em = 0, n_items_em = 0; // event-heavy instances, one particle per thread
    int split = 0;                   // lockstep instances on the split kernel (0: the ring kernel)
    int em_shist = 0;                // event-major instances bin into shared memory (0: device memory)
    int em_block = 256;
    int kmax = 0;                    // the largest seg_cap of the lockstep instances
    DevBuf scratch;                  // the split kernel's per-block segment records
    int64_t chunk = 0, hist_len = 0;
    size_t smem = 0, smem_em = 0;
    DevBuf params, items, items_em, tabs, edges, hists, ctl;
    std::vector<int64_t> n_part;
    std::vector<double> cost_per_particle;
    std::vector<int> event_major;    // the kernel of each instance (1: event-major)
    std::vector<int> event_major_auto; // the automatic choice
    std::vector<int> seg_cap;        // the split kernel's segment records per particle
    std::vector<unsigned char> params_host; // the instances' DevParams as uploaded
    int n_edges = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *args_host = nullptr;    // BatchArgs<R>, kept alive for the graph's kernel nodes
    void *args_em_host = nullptr; // the same for the event-major kernel
};

namespace {

bool same_grid(const rtmc_problem &a, const rtmc_problem &b)
{
    if (a.d != b.d || a.frame != b.frame || a.acoustics != b.acoustics || a.precision != b.precision ||
        a.n_obs != b.n_obs || a.time_stride != b.time_stride || a.mode_stride != b.mode_stride ||
        a.hist_len != b.hist_len || a.hist_shift != b.hist_shift)
        return false;
    for (int x = 0; x < 4; ++x) {
        if (a.axis_mode[x] != b.axis_mode[x] || a.axis_stride[x] != b.axis_stride[x]) return false;
        if (a.axis_mode[x] == RTMC_AXIS_IGNORED) continue;
        if (a.axis_nedges[x] != b.axis_nedges[x]) return false;
        for (int k = 0; k < a.axis_nedges[x]; ++k)
            if (a.axis_edges[x][k] != b.axis_edges[x][k]) return false;
    }
    return true;
}

template <typename R> int batch_build_graph(rtmc_batch *b)
{
    rtmc_context *ctx = b->ctx;
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    // launch shape
    const size_t seg_bytes = 6 * sizeof(R) + 2 * sizeof(int32_t);
    const size_t fixed = align_up((size_t)b->n_edges * sizeof(R), 16) + align_up((size_t)b->hist_len * 4, 16);
    const size_t budget = (size_t)ctx->max_smem_optin - 1024 - sizeof(DevParams<R>) - 64;
    int block, ring = 0;
    int64_t chunk;
    int bps = 0;
    {
        // each instance's event_major flag follows the kernel that runs it
        auto *hp = reinterpret_cast<DevParams<R> *>(b->params_host.data());
        bool changed = false;
        for (int i = 0; i < b->n; ++i)
            if (hp[i].event_major != b->event_major[i]) { hp[i].event_major = b->event_major[i]; changed = true; }
        if (changed)
            CK(cudaMemcpy(b->params.p, hp, (size_t)b->n * sizeof(DevParams<R>), cudaMemcpyHostToDevice), "params");
    }
    b->kmax = 0;
    for (int i = 0; i < b->n; ++i)
        if (!b->event_major[i]) b->kmax = std::max(b->kmax, b->seg_cap[i]);
    if (b->split) {
        // the split kernel: 1024 threads, the histogram alone in shared memory, segment
        // records of one work item per block in device memory
        block = kBatchSplitThreads;
        if (fixed > budget) return fail(&ctx->err, RTMC_ERR_ARG, "batched runs need a histogram that fits in shared memory");
        b->smem = fixed;
        chunk = b->chunk ? b->chunk : 4096;
        if (transport_batch_setup(b->prec, b->obs_kind, block, b->smem, &bps, 1) != 0 || bps < 1)
            return fail(&ctx->err, RTMC_ERR_CUDA, "batched transport kernel does not fit on the device");
        b->grid = ctx->num_sms * bps;
        const int64_t stride = chunk * std::max(1, b->kmax) * 8;
        if (b->scratch.grow((size_t)b->grid * stride * sizeof(R)))
            return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for batched segment records failed");
    } else {
        block = b->block ? b->block : 512;
        if (block > 512) block = 512;
        if (fixed + (size_t)block * 2 * seg_bytes > budget) block = 256;
        if (fixed + (size_t)block * 2 * seg_bytes > budget)
            return fail(&ctx->err, RTMC_ERR_ARG, "batched runs need a histogram that fits in shared memory");
        ring = b->ring > 0 ? b->ring : 8;
        ring = std::min<int>(ring, (int)((budget - fixed) / ((size_t)block * seg_bytes)));
        b->smem = fixed + (size_t)block * ring * seg_bytes;
        if (transport_batch_setup(b->prec, b->obs_kind, block, b->smem, &bps, 0) != 0 || bps < 1)
            return fail(&ctx->err, RTMC_ERR_CUDA, "batched transport kernel does not fit on the device");
        b->grid = ctx->num_sms * bps;
        chunk = b->chunk ? b->chunk : 8192;
    }
    // work items: chunks of each instance, largest expected cost first
    // two work lists: lockstep-batch instances (shared-memory histogram kernel) and
    // event-heavy instances (event-major kernel), each sorted by expected cost
    std::vector<BatchItem> sorted, sorted_em;
    for (int em = 0; em < 2; ++em) {
        std::vector<BatchItem> items;
        std::vector<double> cost;
        for (int i = 0; i < b->n; ++i) {
            if (b->event_major[i] != em) continue;
            for (int64_t f = 0; f < b->n_part[i]; f += chunk) {
                BatchItem it{};
                it.inst = i;
                it.first = f;
                it.count = std::min<int64_t>(chunk, b->n_part[i] - f);
                items.push_back(it);
                cost.push_back(b->cost_per_particle[i] * (double)it.count);
            }
        }
        std::vector<size_t> order(items.size());
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
        std::vector<BatchItem> &dst = em ? sorted_em : sorted;
        dst.resize(items.size());
        for (size_t k = 0; k < order.size(); ++k) dst[k] = items[order[k]];
    }
    b->n_items = (int)sorted.size();
    b->n_items_em = (int)sorted_em.size();
    if (b->items.grow(std::max<size_t>(1, sorted.size()) * sizeof(BatchItem)) ||
        b->items_em.grow(std::max<size_t>(1, sorted_em.size()) * sizeof(BatchItem)))
        return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for the work list failed");
    if (!sorted.empty())
        CK(cudaMemcpy(b->items.p, sorted.data(), sorted.size() * sizeof(BatchItem), cudaMemcpyHostToDevice), "work list");
    if (!sorted_em.empty())
        CK(cudaMemcpy(b->items_em.p, sorted_em.data(), sorted_em.size() * sizeof(BatchItem), cudaMemcpyHostToDevice),
           "work list");
    // the event-major kernel bins into device memory unless the shared-memory histogram is
    // asked for (on the 256-instance sweep: 646 ms per launch against 591, as one 512-thread
    // block per SM hides less latency than three of 256)
    const int em_shist = b->em_shist < 0 ? 0 : b->em_shist;
    if (em_shist && fixed > budget)
        return fail(&ctx->err, RTMC_ERR_ARG, "the histogram does not fit in shared memory");
    b->smem_em = em_shist ? fixed : align_up((size_t)b->n_edges * sizeof(R), 16);
    b->em_block = em_shist ? 512 : 256;
    int bps_em = 0;
    if (transport_batch_em_setup(b->prec, b->obs_kind, b->em_block, b->smem_em, &bps_em, em_shist) != 0 || bps_em < 1)
        return fail(&ctx->err, RTMC_ERR_CUDA, "batched event-major kernel does not fit on the device");
    b->grid_em = ctx->num_sms * bps_em;
    // capture: clear histograms and counters, persistent launch
    auto *a = static_cast<BatchArgs<R> *>(b->args_host);
    a->params = static_cast<const DevParams<R> *>(b->params.p);
    a->items = static_cast<const BatchItem *>(b->items.p);
    a->n_items = b->n_items;
    a->ring_cap = ring;
    a->counter = static_cast<int32_t *>(b->ctl.p);
    a->stats = reinterpret_cast<unsigned long long *>(static_cast<unsigned char *>(b->ctl.p) + 64);
    a->status = reinterpret_cast<int32_t *>(static_cast<unsigned char *>(b->ctl.p) + 192);
    a->hists = static_cast<unsigned long long *>(b->hists.p);
    a->hist_len = b->hist_len;
    a->edges = static_cast<const R *>(b->edges.p);
    a->n_edges = b->n_edges;
    a->obs_kind = b->obs_kind;
    a->scratch = b->split ? b->scratch.p : nullptr;
    a->scratch_stride = b->split ? chunk * std::max(1, b->kmax) * 8 : 0;
    auto *ae = static_cast<BatchArgs<R> *>(b->args_em_host);
    *ae = *a;
    ae->items = static_cast<const BatchItem *>(b->items_em.p);
    ae->n_items = b->n_items_em;
    ae->counter = static_cast<int32_t *>(b->ctl.p) + 2;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
    cudaMemsetAsync(b->hists.p, 0, (size_t)b->n * b->hist_len * sizeof(int64_t), ctx->stream);
    cudaMemsetAsync(b->ctl.p, 0, 256, ctx->stream);
    int le = 0;
    if (b->n_items) {
        if constexpr (sizeof(R) == 4) le = launch_transport_batch_f32(*a, b->grid, block, b->smem, ctx->stream, b->split);
        else le = launch_transport_batch_f64(*a, b->grid, block, b->smem, ctx->stream, b->split);
    }
    if (!le && b->n_items_em) {
        const int sh = b->em_block == 512 ? 1 : 0;
        if constexpr (sizeof(R) == 4) le = launch_transport_batch_em_f32(*ae, b->grid_em, b->em_block, b->smem_em, ctx->stream, sh);
        else le = launch_transport_batch_em_f64(*ae, b->grid_em, b->em_block, b->smem_em, ctx->stream, sh);
    }
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &b->graph);
    if (le) return cuda_fail(ctx, (cudaError_t)le, "batched launch capture");
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
    CK(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    b->block = b->split ? 0 : block;
    b->ring = ring;
    b->chunk = chunk;
    return RTMC_OK;
}

template <typename R>
int batch_create(rtmc_context *ctx, int n, const rtmc_problem *P, const rtmc_tables *const *T, rtmc_batch *b)
{
    b->prec = sizeof(R) == 4 ? RTMC_FP32 : RTMC_FP64;
    b->n_obs = P[0].n_obs;
    b->hist_len = P[0].hist_len;
    // tables and Zoeppritz tables of every instance in one device buffer
    std::vector<size_t> toff(n);
    size_t total = 0;
    for (int i = 0; i < n; ++i) {
        toff[i] = total;
        for (int t = 0; t < T[i]->n_tables; ++t) total += table_bytes<R>(T[i]->cdf[t].size());
        total += align_up((2 * RTMC_ZOE_N + 2 * (size_t)P[i].src_radial_n) * sizeof(R), 256);
    }
    if (b->tabs.grow(total)) return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for batched tables failed");
    std::vector<unsigned char> host(total, 0);
    std::vector<DevParams<R>> params(n);
    std::vector<R> edges, zoe;
    int n_edges = 0;
    unsigned char *dev = static_cast<unsigned char *>(b->tabs.p);
    b->n_part.resize(n);
    b->cost_per_particle.resize(n);
    b->event_major.assign(n, 0);
    b->event_major_auto.assign(n, 0);
    b->seg_cap.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        DevTables<R> dt{};
        size_t o = toff[i];
        for (int t = 0; t < T[i]->n_tables; ++t) {
            stage_table<R>(T[i]->cdf[t], T[i]->theta[t], host.data() + o, dev + o, &dt, t);
            o += table_bytes<R>(T[i]->cdf[t].size());
        }
        fill_params<R>(ctx, &P[i], dt, &params[i], &n_edges, &edges, &zoe);
        std::memcpy(host.data() + o, zoe.data(), zoe.size() * sizeof(R));
        params[i].zoe = reinterpret_cast<const R *>(dev + o);
        params[i].src_radial = params[i].zoe + 2 * RTMC_ZOE_N;
        params[i].sink = kSinkSmem;
        params[i].trace = nullptr;
        b->n_part[i] = P[i].n_particles;
        // expected work per particle: its observations plus ~4 observation-equivalents per event
        double rate = 0;
        for (int m = 0; m < (P[i].acoustics ? 1 : 2); ++m)
            if (std::isfinite(P[i].mft[m])) rate = std::max(rate, 1.0 / P[i].mft[m]);
        b->cost_per_particle[i] = P[i].n_obs + 4.0 * rate * P[i].h * P[i].n_sub * P[i].n_obs;
        if (i == 0) b->obs_kind = params[0].obs_kind;
        // the kernel of an instance: event-major when 4 x its expected events per particle
        // reach its observation instants (on the 256-instance sweep: 578 ms per launch,
        // against 589 / 592 / 628 / 691 ms with 2 / 8 / 16 / 32; tune_schedule times it on a
        // batch), unless the context's schedule fixes it
        const double mean = rate * P[i].h * (double)P[i].n_sub * (double)P[i].n_obs;
        const int sched = ctx->opt_event_major;
        params[i].event_major =
            sched == 1 ? 1 : ((sched == 0 || sched == 2) ? 0 : (4.0 * mean >= (double)P[i].n_obs ? 1 : 0));
        b->event_major[i] = b->event_major_auto[i] = params[i].event_major;
        // the split kernel's segment records per particle: as for rtmc_forward's split schedule
        int K = (int)std::ceil(1.0 + mean + 4.0 * std::sqrt(mean) + 4.0);
        K = std::min(64, std::max(8, (K + 3) / 4 * 4));
        if (ctx->opt_ring) K = ctx->opt_ring; // the context's ring capacity, when one is set
        K = std::max(1, K) + 2;
        params[i].seg_cap = b->seg_cap[i] = K;
        params[i].split = 1;
    }
    CK(cudaMemcpy(b->tabs.p, host.data(), total, cudaMemcpyHostToDevice), "batched tables");
    if (b->edges.grow(std::max<size_t>(1, edges.size()) * sizeof(R)) || b->params.grow((size_t)n * sizeof(DevParams<R>)) ||
        b->hists.grow((size_t)n * b->hist_len * sizeof(int64_t)) || b->ctl.grow(256))
        return fail(&ctx->err, RTMC_ERR_ALLOC, "device allocation for a batch failed");
    for (int i = 0; i < n; ++i) params[i].edges = static_cast<const R *>(b->edges.p);
    if (!edges.empty())
        CK(cudaMemcpy(b->edges.p, edges.data(), edges.size() * sizeof(R), cudaMemcpyHostToDevice), "edges");
    b->params_host.assign(reinterpret_cast<const unsigned char *>(params.data()),
                          reinterpret_cast<const unsigned char *>(params.data() + n));
    CK(cudaMemcpy(b->params.p, params.data(), (size_t)n * sizeof(DevParams<R>), cudaMemcpyHostToDevice), "params");
    b->n_edges = n_edges;
    b->args_host = new BatchArgs<R>();
    b->args_em_host = new BatchArgs<R>();
    return batch_build_graph<R>(b);
}

} // namespace

extern "C" int rtmc_batch_create(rtmc_context *ctx, int32_t n, const rtmc_problem *P, const rtmc_tables *const *T,
                                 rtmc_batch **out)
{
    if (!ctx || !P || !T || !out || n < 1) return fail(ctx ? &ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_batch_create: bad argument");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    for (int i = 0; i < n; ++i) {
        int s = check_problem(ctx, &P[i], T[i]);
        if (s) return s;
        if (i && !same_grid(P[0], P[i]))
            return fail(&ctx->err, RTMC_ERR_ARG, "rtmc_batch_create: problem " + std::to_string(i) +
                                                      " does not share the observation grid of problem 0");
    }
    auto *b = new (std::nothrow) rtmc_batch();
    if (!b) return fail(&ctx->err, RTMC_ERR_ALLOC, "out of host memory");
    b->ctx = ctx;
    b->n = n;
    int s = P[0].precision == RTMC_FP64 ? batch_create<double>(ctx, n, P, T, b) : batch_create<float>(ctx, n, P, T, b);
    if (s) {
        rtmc_batch_destroy(b);
        return s;
    }
    *out = b;
    return RTMC_OK;
}

extern "C" int rtmc_batch_set_launch(rtmc_batch *b, int32_t block, int32_t ring_cap, int64_t chunk)
{
    if (!b) return fail(nullptr, RTMC_ERR_ARG, "rtmc_batch_set_launch: NULL batch");
    const bool split = ring_cap == -1;
    if (block < 0 || block > 512 || block % 32 || ring_cap < -1 || ring_cap == 1 || ring_cap > 64 || chunk < 0 ||
        (split && block != 0))
        return fail(&b->ctx->err, RTMC_ERR_ARG,
                    "rtmc_batch_set_launch: block <= 512 (multiple of 32) with ring 0 or 2..64, or block 0 with ring -1; chunk >= 0");
    rtmc_context *ctx = b->ctx;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    b->split = split ? 1 : 0;
    b->block = block;
    b->ring = ring_cap;
    b->chunk = chunk;
    return b->prec == RTMC_FP64 ? batch_build_graph<double>(b) : batch_build_graph<float>(b);
}

extern "C" int rtmc_batch_set_em_histogram(rtmc_batch *b, int32_t shared)
{
    if (!b) return fail(nullptr, RTMC_ERR_ARG, "rtmc_batch_set_em_histogram: NULL batch");
    if (shared < -1 || shared > 1) return fail(&b->ctx->err, RTMC_ERR_ARG, "rtmc_batch_set_em_histogram: -1, 0 or 1");
    rtmc_context *ctx = b->ctx;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    b->em_shist = shared;
    return b->prec == RTMC_FP64 ? batch_build_graph<double>(b) : batch_build_graph<float>(b);
}

extern "C" int rtmc_batch_run(rtmc_batch *b, rtmc_stats *st)
{
    Range range("rtmc_batch_run");
    if (!b) return fail(nullptr, RTMC_ERR_ARG, "rtmc_batch_run: NULL batch");
    rtmc_context *ctx = b->ctx;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaEventRecord(ctx->ev_k0, ctx->stream), "event");
    CK(cudaGraphLaunch(b->exec, ctx->stream), "graph launch");
    CK(cudaEventRecord(ctx->ev_k1, ctx->stream), "event");
    int64_t d[32];
    CK(cudaMemcpyAsync(d, static_cast<unsigned char *>(b->ctl.p) + 64, 192, cudaMemcpyDeviceToHost, ctx->stream), "counters");
    CK(cudaStreamSynchronize(ctx->stream), "batched run");
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev_k0, ctx->ev_k1);
    ctx->last_kernel_ms = ms;
    const int kernels = (b->n_items ? 1 : 0) + (b->n_items_em ? 1 : 0); // kernel nodes of the graph
    ctx->last_launches = kernels;
    const int32_t status = (int32_t)(d[16] & 0xffffffff);
    if (st) {
        std::memset(st, 0, sizeof *st);
        st->scatter_events = d[0];
        st->boundary_hits = d[1];
        st->kills = d[2];
        st->absorbed = d[3];
        st->observations = d[4];
        st->conversions = d[5];
        st->device_status = status;
        st->launches = kernels;
        st->sink = kSinkSmem;
        st->kernel_ms = ms;
        st->total_ms = ms;
        st->d2h_bytes = 192;
    }
    if (status) return fail(&ctx->err, RTMC_ERR_DEVICE, "a transport guard tripped in a batched run");
    return RTMC_OK;
}

extern "C" int rtmc_batch_set_schedule(rtmc_batch *b, const int32_t *event_major)
{
    if (!b) return fail(nullptr, RTMC_ERR_ARG, "rtmc_batch_set_schedule: NULL batch");
    if (event_major)
        for (int i = 0; i < b->n; ++i)
            if (event_major[i] != 0 && event_major[i] != 1)
                return fail(&b->ctx->err, RTMC_ERR_ARG, "rtmc_batch_set_schedule: event_major[i] must be 0 or 1");
    rtmc_context *ctx = b->ctx;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    for (int i = 0; i < b->n; ++i) b->event_major[i] = event_major ? event_major[i] : b->event_major_auto[i];
    return b->prec == RTMC_FP64 ? batch_build_graph<double>(b) : batch_build_graph<float>(b);
}

extern "C" int rtmc_batch_schedule(const rtmc_batch *b, int32_t *event_major)
{
    if (!b || !event_major) return fail(nullptr, RTMC_ERR_ARG, "rtmc_batch_schedule: NULL argument");
    for (int i = 0; i < b->n; ++i) event_major[i] = b->event_major[i];
    return RTMC_OK;
}

extern "C" int rtmc_batch_histograms(rtmc_batch *b, int32_t first, int32_t count, int64_t *out)
{
    if (!b || !out || first < 0 || count < 0 || (int64_t)first + count > b->n)
        return fail(b ? &b->ctx->err : nullptr, RTMC_ERR_ARG, "rtmc_batch_histograms: bad range");
    rtmc_context *ctx = b->ctx;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaMemcpy(out, static_cast<int64_t *>(b->hists.p) + (int64_t)first * b->hist_len,
                  (size_t)count * b->hist_len * sizeof(int64_t), cudaMemcpyDeviceToHost), "histogram copy");
    return RTMC_OK;
}

extern "C" void rtmc_batch_destroy(rtmc_batch *b)
{
    if (!b) return;
    if (b->ctx) cudaSetDevice(b->ctx->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->params.release();
    b->items.release();
    b->items_em.release();
    b->tabs.release();
    b->edges.release();
    b->hists.release();
    b->ctl.release();
    b->scratch.release();
    for (void *h : {b->args_host, b->args_em_host}) {
        if (!h) continue;
        if (b->prec == RTMC_FP64) delete static_cast<BatchArgs<double> *>(h);
        else delete static_cast<BatchArgs<float> *>(h);
    }
    delete b;
}
