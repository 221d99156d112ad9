// Transport kernels of librtmc (sm_103a).
//
// One particle per thread, state in registers for the particle's whole life.  The
// kernel restates, event by event, the small-dt process of propagateParticleSmallDt.m
// (Q-kill :100-138, move :141-143, plane boundary :168-322 with
// MaterialClass.MaterialInterface :1572-1756, scattering decision :591-601, azimuth
// :604-611, mode conversion :619-623, inverse-CDF angle :614-632, rotation :635-639),
// driven by the packet x time loop of radiativeTransfer.m:105-131 and binned as
// observeTime.m:14-144 does:
//
//  * sub-step grid h = dt_obs / n_sub; observation j sits at sub-step j * n_sub;
//  * the sub-steps to the next scattering (or Q-kill) are geometric:
//    ceil(-log(u) * mft/h) (or ceil(-log(u) * Q/(omega h)));
//  * a plane crossing is solved in closed form on that grid;
//  * ties inside one sub-step resolve as the reference orders them: kill (before the
//    move) < boundary (after the move) < scattering (end of the sub-step);
//  * observations between events are straight-line positions on the grid.
//
// Warps walk the observation instants in lockstep, so every lane of a warp bins into
// the same time slice.  Histogram: a block-private u32 copy in shared memory when the
// whole histogram fits (flushed once with 64-bit global atomics), else direct 64-bit
// global atomics.  Random numbers: Philox4x32-10 keyed by (seed), counter
// (particle id, event index, block).
#include "rtmc_internal.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace rtmc {
namespace {

// ----------------------------------------------------------------------------------
// precision-overloaded math (CUDA math library calls)
// ----------------------------------------------------------------------------------
__device__ __forceinline__ float m_log(float x) { return logf(x); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_floor(float x) { return floorf(x); }
__device__ __forceinline__ double m_floor(double x) { return floor(x); }
__device__ __forceinline__ float m_ceil(float x) { return ceilf(x); }
__device__ __forceinline__ double m_ceil(double x) { return ceil(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ float m_acos(float x) { return acosf(x); }
__device__ __forceinline__ double m_acos(double x) { return acos(x); }
__device__ __forceinline__ float m_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double m_atan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float m_hypot(float x, float y) { return hypotf(x, y); }
__device__ __forceinline__ double m_hypot(double x, double y) { return hypot(x, y); }
__device__ __forceinline__ float m_sin(float x) { return sinf(x); }
__device__ __forceinline__ double m_sin(double x) { return sin(x); }
__device__ __forceinline__ void m_sincos(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ void m_sincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void m_sincospi(float x, float *s, float *c) { sincospif(x, s, c); }
__device__ __forceinline__ void m_sincospi(double x, double *s, double *c) { sincospi(x, s, c); }
__device__ __forceinline__ float m_cospi(float x) { return cospif(x); }
__device__ __forceinline__ float m_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double m_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ double m_cospi(double x) { return cospi(x); }

// 32-bit Philox output -> uniform in (0,1): 24 bits for FP32, 32 bits for FP64
__device__ __forceinline__ float to_uniform(uint32_t x, float) { return ((float)(x >> 8) + 0.5f) * 5.9604644775390625e-08f; }
__device__ __forceinline__ double to_uniform(uint32_t x, double) { return ((double)x + 0.5) * 2.3283064365386962890625e-10; }

// ----------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11)
// ----------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

template <typename R> struct U4 {
    R a, b, c, d;
};

template <typename R>
__device__ __forceinline__ U4<R> draw(const DevParams<R> &p, uint64_t pid, uint32_t step, uint32_t block)
{
    uint4 o = philox4x32_10(make_uint4((uint32_t)pid, (uint32_t)(pid >> 32), step, block), p.key0, p.key1);
    return U4<R>{to_uniform(o.x, R()), to_uniform(o.y, R()), to_uniform(o.z, R()), to_uniform(o.w, R())};
}

// sub-steps to the first success of Bernoulli(1 - exp(-rate)) trials; cap = never
template <typename R> __device__ __forceinline__ int geom_steps(R u, R inv_rate, int on, int cap)
{
    if (!on) return cap;
    R k = m_ceil(-m_log(u) * inv_rate);
    if (!(k < (R)cap)) return cap;
    return k < (R)1 ? 1 : (int)k;
}

// ----------------------------------------------------------------------------------
// inverse CDF: guide-table start, binary search, linear (extrapolating) interpolation
// ----------------------------------------------------------------------------------
template <typename R> __device__ __forceinline__ R invcdf(const DevTables<R> &t, int ti, R u)
{
    const double ud = (double)u;
    int g = (int)(ud * (double)kGuideN);
    g = g < 0 ? 0 : (g > kGuideN - 1 ? kGuideN - 1 : g);
    const int32_t *guide = t.guide[ti];
    const double *c = t.cdf[ti];
    int lo = __ldg(guide + g), hi = __ldg(guide + g + 1);
    while (hi > lo) { // largest i in [lo, hi] with c[i] <= u (lo itself when none)
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(c + mid) <= ud) lo = mid; else hi = mid - 1;
    }
    const R off = (R)(ud - __ldg(c + lo));
    return __ldg(t.theta[ti] + lo) + off * __ldg(t.slope[ti] + lo);
}

// ----------------------------------------------------------------------------------
// particle state
// ----------------------------------------------------------------------------------
template <typename R> struct Part {
    R x[3], d[3], q[3];
    int mode, alive;
    int s0, sS, sK, sB;
    int s_death;
    uint32_t k;
};

template <typename R> __device__ __forceinline__ void cross3(const R a[3], const R b[3], R o[3])
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

template <typename R> __device__ __forceinline__ R dot3(const R a[3], const R b[3])
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

template <typename R> __device__ __forceinline__ void normalize3(R a[3])
{
    const R s = (R)1 / m_sqrt(dot3(a, a));
    a[0] *= s; a[1] *= s; a[2] *= s;
}

// next plane crossing of the current segment (sub-step index, or cap)
template <typename R> __device__ __forceinline__ void next_boundary(const DevParams<R> &p, Part<R> &s)
{
    const int cap = p.s_end + 1;
    s.sB = cap;
    const R step = p.step[s.mode];
    for (int b = 0; b < p.n_bnd; ++b) {
        const int k = p.bnd_dir[b] - 1;
        const R a = s.x[k] - p.bnd_val[b];
        const R bs = step * s.d[k];
        if (a == (R)0 || bs == (R)0 || ((a > (R)0) == (bs > (R)0))) continue;
        const R j = m_floor(m_abs(a) / m_abs(bs)) + (R)1;
        if (j < (R)(cap - s.s0)) {
            const int sb = s.s0 + (int)j;
            s.sB = sb < s.sB ? sb : s.sB;
        }
    }
}

// initializeParticle.m:14-58,151-170 (point source); step 0 of the particle's counter
template <typename R> __device__ void init_particle(const DevParams<R> &p, uint64_t pid, Part<R> &s)
{
    const U4<R> a = draw(p, pid, 0u, 0u);  // r1, r2, phi0, theta0
    const U4<R> b = draw(p, pid, 0u, 1u);  // phi, theta, alpha, first scattering
    const U4<R> c = draw(p, pid, 0u, 2u);  // Q-kill
    const R r = m_abs(m_sqrt((R)-2 * m_log(a.a)) * m_cospi((R)2 * a.b)) * p.src_lambda;
    R cphi0, sphi0, cphi, sphi;
    if (p.d == 2) {
        cphi0 = p.cos_half_pi; sphi0 = (R)1;
        cphi = cphi0; sphi = sphi0;
    } else {
        cphi0 = (R)-1 + (R)2 * a.c;
        sphi0 = m_sqrt(m_max((R)0, ((R)1 - cphi0) * ((R)1 + cphi0)));
        cphi = (p.src_dir == 2) ? b.a : (R)-1 + (R)2 * b.a;
        sphi = m_sqrt(m_max((R)0, ((R)1 - cphi) * ((R)1 + cphi)));
    }
    R st0, ct0, st, ct;
    m_sincospi((R)2 * a.d, &st0, &ct0);
    m_sincospi((R)2 * b.b, &st, &ct);
    if (p.src_dir == 1) { st = st0; ct = ct0; cphi = cphi0; sphi = sphi0; }
    s.d[0] = ct * sphi; s.d[1] = st * sphi; s.d[2] = cphi;
    s.q[0] = -st; s.q[1] = ct; s.q[2] = (R)0;
    if (p.d == 3) {
        R sa, ca, cr[3];
        m_sincospi((R)2 * b.c, &sa, &ca);
        cross3(s.d, s.q, cr);
#pragma unroll
        for (int i = 0; i < 3; ++i) s.q[i] = s.q[i] * ca + cr[i] * sa;
    }
    s.x[0] = p.src_pos[0] + r * ct0 * sphi0;
    s.x[1] = p.src_pos[1] + r * st0 * sphi0;
    s.x[2] = p.src_pos[2] + r * cphi0;
    s.mode = (!p.acoustics && p.polarization == 1) ? 1 : 0;
    s.alive = 1;
    s.k = 0;
    s.s0 = 0;
    s.s_death = -1;
    const int cap = p.s_end + 1;
    s.sS = geom_steps(b.d, p.inv_lam[s.mode], p.scat_on[s.mode], cap);
    s.sK = geom_steps(c.a, p.inv_q[s.mode], p.kill_on[s.mode], cap);
    next_boundary(p, s);
}

// interp1(0:0.5:90, tab, ang) (MaterialClass.m:1674)
template <typename R> __device__ __forceinline__ R zoe_lookup(const R *tab, R ang_deg)
{
    const R f = ang_deg * (R)2;
    int i = (int)m_floor(f);
    i = i < 0 ? 0 : (i > RTMC_ZOE_N - 2 ? RTMC_ZOE_N - 2 : i);
    const R w = f - (R)i;
    const R t0 = __ldg(tab + i), t1 = __ldg(tab + i + 1);
    return t0 + w * (t1 - t0);
}

// elastic reflection at the plane normal to e_k: MaterialInterface decisions
// (MaterialClass.m:1587-1756) and the updates of propagateParticleSmallDt.m:197-321.
// Returns 1 if the mode changed.
template <typename R>
__device__ int elastic_reflect(const DevParams<R> &p, Part<R> &s, int k, R u_split, R u_coin)
{
    const R eps = (R)2.220446049250313e-16;
    R n[3] = {(R)0, (R)0, (R)0};
    n[k] = (R)1;
    const int m0 = s.mode;
    R adn = m_abs(s.d[k]);
    adn = adn > (R)1 ? (R)1 : adn;
    const R ang = m_acos(adn) * (R)57.295779513082320876798154814105;
    if (s.mode == 0) {
        const R rpp = zoe_lookup(p.zoe, ang);
        if (u_coin <= rpp) {
            s.d[k] = -s.d[k];
            s.q[k] = -s.q[k];
        } else { // P -> SV, propagateParticleSmallDt.m:212-248
            s.mode = 1;
            const R ratio = p.vs_over_vp;
            const R dn = s.d[k];
            R nd[3] = {s.d[0] * ratio, s.d[1] * ratio, s.d[2] * ratio};
            nd[k] = (R)0;
            const R sin2 = dot3(nd, nd);
            const R cv = m_sqrt(m_max((R)0, (R)1 - sin2));
            const R sg = (R)((dn > (R)0) - (dn < (R)0));
            nd[k] = -sg * cv;
            normalize3(nd);
            s.d[0] = nd[0]; s.d[1] = nd[1]; s.d[2] = nd[2];
            R ax[3];
            cross3(s.d, n, ax);
            normalize3(ax);
            cross3(ax, s.d, s.q);
        }
    } else {
        R eSH[3];
        cross3(s.d, n, eSH);
        R nsh = m_sqrt(dot3(eSH, eSH));
        if (nsh < eps) {
            R t[3] = {(R)1, (R)0, (R)0};
            const R tn = t[k];
            t[k] -= tn;
            eSH[0] = t[0]; eSH[1] = t[1]; eSH[2] = t[2];
            nsh = m_sqrt(dot3(t, t));
        }
        const R inv = (R)1 / nsh;
        eSH[0] *= inv; eSH[1] *= inv; eSH[2] *= inv;
        R eSV[3];
        cross3(eSH, s.d, eSV);
        normalize3(eSV);
        const R aSV = dot3(s.q, eSV), aSH = dot3(s.q, eSH);
        const R Esv = aSV * aSV, Esh = aSH * aSH;
        const R probSV = Esv / (Esv + Esh + eps);
        if (!(u_split < probSV)) { // SH -> SH
            s.d[k] = -s.d[k];
            s.q[k] = -s.q[k];
        } else {
            const R rsv = zoe_lookup(p.zoe + RTMC_ZOE_N, ang);
            if (u_coin <= rsv) { // SV -> SV
                s.d[k] = -s.d[k];
                s.q[k] = -s.q[k];
            } else { // SV -> P, :274-321
                const R ratio = p.vp_over_vs;
                const R dn = s.d[k];
                R nd[3] = {s.d[0] * ratio, s.d[1] * ratio, s.d[2] * ratio};
                nd[k] = (R)0;
                const R sin2 = dot3(nd, nd);
                if (sin2 <= (R)1) {
                    s.mode = 0;
                    const R sg = (R)((dn > (R)0) - (dn < (R)0));
                    nd[k] = -sg * m_sqrt((R)1 - sin2);
                    normalize3(nd);
                    s.d[0] = nd[0]; s.d[1] = nd[1]; s.d[2] = nd[2];
                } else {
                    s.d[k] = -s.d[k]; // total internal reflection: SV, dir mirrored only
                }
            }
        }
    }
    return s.mode != m0;
}

// azimuth, mode conversion, polar angle, rotation (propagateParticleSmallDt.m:603-639)
template <typename R>
__device__ __forceinline__ void scatter(const DevParams<R> &p, Part<R> &s, R u_phi, R u_mode, R u_theta)
{
    if (p.d == 2) {
        if (u_phi >= (R)0.5) { s.q[0] = -s.q[0]; s.q[1] = -s.q[1]; s.q[2] = -s.q[2]; }
    } else {
        R sp, cp, cr[3];
        m_sincospi((R)2 * u_phi, &sp, &cp);
        cross3(s.d, s.q, cr);
#pragma unroll
        for (int i = 0; i < 3; ++i) s.q[i] = cp * s.q[i] + sp * cr[i];
    }
    const int m = s.mode;
    int m2 = m;
    if (!p.acoustics) {
        if (m == 0 && u_mode > p.p2p) m2 = 1;
        else if (m == 1 && u_mode > p.s2s) m2 = 0;
    }
    const int ti = p.acoustics ? 0 : m * 2 + m2;
    const R th = invcdf(p.tab, ti, u_theta);
    R st, ct;
    m_sincos(th, &st, &ct);
    R nd[3], nq[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        nd[i] = ct * s.d[i] + st * s.q[i];
        nq[i] = -st * s.d[i] + ct * s.q[i];
    }
    normalize3(nd);
    normalize3(nq);
#pragma unroll
    for (int i = 0; i < 3; ++i) { s.d[i] = nd[i]; s.q[i] = nq[i]; }
    s.mode = m2;
}

struct Counters {
    unsigned scat, bnd, kill, absorb, obs, conv;
};

// one event: the earliest of kill / boundary / scattering (ties in that order)
template <typename R>
__device__ void process_event(const DevParams<R> &p, uint64_t pid, Part<R> &s, Counters &cnt)
{
    const int cap = p.s_end + 1;
    int e = s.sK, kind = 2;
    if (s.sB < e) { e = s.sB; kind = 1; }
    if (s.sS < e) { e = s.sS; kind = 0; }
    if (kind == 2) {
        s.alive = 0;
        s.s_death = e;
        cnt.kill++;
        return;
    }
    s.k++;
    const R step = p.step[s.mode];
    const R dt = step * (R)(e - s.s0);
    R xe[3] = {s.x[0] + dt * s.d[0], s.x[1] + dt * s.d[1], s.x[2] + dt * s.d[2]};
    if (kind == 1) {
        const R dt1 = step * (R)(e - 1 - s.s0);
        const R x1[3] = {s.x[0] + dt1 * s.d[0], s.x[1] + dt1 * s.d[1], s.x[2] + dt1 * s.d[2]};
        s.x[0] = xe[0]; s.x[1] = xe[1]; s.x[2] = xe[2];
        int changed = 0;
        for (int b = 0; b < p.n_bnd; ++b) {
            const int k = p.bnd_dir[b] - 1;
            const R val = p.bnd_val[b];
            if (!((s.x[k] - val) * (x1[k] - val) < (R)0)) continue;
            cnt.bnd++;
            if (p.bnd_absorb[b]) {
                s.alive = 0;
                s.s0 = e;
                s.s_death = e;
                cnt.absorb++;
                return;
            }
            s.x[k] = (R)2 * val - s.x[k];
            if (p.acoustics) {
                s.d[k] = -s.d[k];
            } else {
                const U4<R> bb = draw(p, pid, s.k, 1u + (uint32_t)b);
                const int ch = elastic_reflect(p, s, k, bb.a, bb.b);
                cnt.conv += ch;
                changed |= ch;
            }
        }
        s.s0 = e;
        if (changed) {
            const U4<R> r0 = draw(p, pid, s.k, 0u);
            const int js = geom_steps(r0.a, p.inv_lam[s.mode], p.scat_on[s.mode], cap);
            s.sS = js >= cap ? cap : e - 1 + js;
            const int jk = geom_steps(r0.b, p.inv_q[s.mode], p.kill_on[s.mode], cap);
            s.sK = jk >= cap ? cap : e + jk;
        }
    } else {
        const U4<R> r0 = draw(p, pid, s.k, 0u); // next, azimuth, mode, theta
        s.x[0] = xe[0]; s.x[1] = xe[1]; s.x[2] = xe[2];
        const int m0 = s.mode;
        scatter(p, s, r0.b, r0.c, r0.d);
        cnt.scat++;
        s.s0 = e;
        const int js = geom_steps(r0.a, p.inv_lam[s.mode], p.scat_on[s.mode], cap);
        s.sS = js >= cap ? cap : e + js;
        if (s.mode != m0) {
            const U4<R> r1 = draw(p, pid, s.k, 1u);
            const int jk = geom_steps(r1.a, p.inv_q[s.mode], p.kill_on[s.mode], cap);
            s.sK = jk >= cap ? cap : e + jk;
        }
    }
    if (s.sS > cap) s.sS = cap;
    if (s.sK > cap) s.sK = cap;
    next_boundary(p, s);
}

// histcounts bin of c on a binned axis (edges staged in shared memory), -1 outside
template <typename R>
__device__ __forceinline__ int bin_of(const DevParams<R> &p, const R *sedges, int a, R c)
{
    if (!(c >= p.ax_lo[a] && c <= p.ax_hi[a])) return -1;
    const R *e = sedges + p.ax_off[a];
    const int nb = p.ax_n[a] - 1;
    int b;
    if (p.ax_uniform[a]) {
        b = (int)((c - p.ax_lo[a]) * p.ax_inv_w[a]);
        b = b < 0 ? 0 : (b > nb - 1 ? nb - 1 : b);
        while (b > 0 && c < e[b]) --b;
        while (b < nb - 1 && c >= e[b + 1]) ++b;
    } else {
        int lo = 0, hi = nb - 1;
        while (hi > lo) {
            int mid = (lo + hi + 1) >> 1;
            if (e[mid] <= c) lo = mid; else hi = mid - 1;
        }
        b = lo;
    }
    return b;
}

// observeTime.m:14-144 for one particle at observation j; returns the histogram index or -1
template <typename R>
__device__ __forceinline__ int64_t obs_index(const DevParams<R> &p, const R *sedges, const R x[3], R dz, int mode, int j)
{
    R c[4];
    if (p.frame == RTMC_FRAME_CARTESIAN) {
        c[0] = x[0]; c[1] = x[1]; c[2] = x[2];
    } else {
        const R rxy = m_hypot(x[0], x[1]);
        c[1] = (p.ax_mode[1] != RTMC_AXIS_IGNORED) ? m_atan2(x[1], x[0]) : (R)0;
        if (p.frame == RTMC_FRAME_CYLINDRICAL || p.d == 2) {
            c[0] = rxy; c[2] = x[2];
        } else {
            const R r = m_hypot(rxy, x[2]);
            c[0] = r;
            c[2] = (p.ax_mode[2] != RTMC_AXIS_IGNORED) ? m_sin(m_atan2(x[2], rxy)) : (R)0;
        }
    }
    if (p.ax_mode[3] != RTMC_AXIS_IGNORED) {
        R cz = dz > (R)1 ? (R)1 : (dz < (R)-1 ? (R)-1 : dz);
        c[3] = (p.d == 3) ? cz : m_acos(cz);
    } else {
        c[3] = (R)0;
    }
    int64_t idx = (int64_t)j * p.time_stride + (int64_t)mode * p.mode_stride;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int am = p.ax_mode[a];
        if (am == RTMC_AXIS_RANGE) {
            if (!(c[a] >= p.ax_lo[a] && c[a] <= p.ax_hi[a])) return -1;
        } else if (am == RTMC_AXIS_BINNED) {
            const int b = bin_of(p, sedges, a, c[a]);
            if (b < 0) return -1;
            idx += (int64_t)b * p.ax_stride[a];
        }
    }
    return idx;
}

template <typename R, bool SMEM>
__global__ void __launch_bounds__(SMEM ? 1024 : 256) rt_transport(const DevParams<R> p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    const int edge_bytes = ((p.n_edges * (int)sizeof(R) + 15) / 16) * 16;
    unsigned *shist = reinterpret_cast<unsigned *>(smem_raw + edge_bytes);

    for (int i = threadIdx.x; i < p.n_edges; i += blockDim.x) sedges[i] = p.edges[i];
    if (SMEM)
        for (int64_t i = threadIdx.x; i < p.hist_len; i += blockDim.x) shist[i] = 0u;
    __syncthreads();

    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const unsigned long long inc = 1ull << p.hist_shift;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_particles; i += stride) {
        const uint64_t pid = (uint64_t)(p.pid0 + i);
        Part<R> s;
        init_particle(p, pid, s);
        const unsigned scat0 = cnt.scat, bnd0 = cnt.bnd;
        int guard = 0;
        for (int j = 1; j <= p.n_obs; ++j) {
            const int so = j * p.n_sub;
            while (s.alive && min(min(s.sK, s.sB), s.sS) <= so) {
                process_event(p, pid, s, cnt);
                if (++guard > p.max_events) { s.alive = 0; bad = true; }
            }
            if (!s.alive) break;
            const R dt = p.step[s.mode] * (R)(so - s.s0);
            const R xo[3] = {s.x[0] + dt * s.d[0], s.x[1] + dt * s.d[1], s.x[2] + dt * s.d[2]};
            const int64_t idx = obs_index(p, sedges, xo, s.d[2], s.mode, j);
            if (idx >= 0) {
                if (idx >= p.hist_len) { bad = true; continue; }
                cnt.obs++;
                if (SMEM) atomicAdd(shist + idx, 1u);
                else atomicAdd(p.hist + idx, inc);
            }
        }
        if (p.trace) { // final state of the particle, the oracle's layout
            double *f = p.trace + 16 * i;
#pragma unroll
            for (int c = 0; c < 3; ++c) { f[c] = s.x[c]; f[3 + c] = s.d[c]; f[6 + c] = s.q[c]; }
            f[9] = s.mode; f[10] = s.alive; f[11] = cnt.scat - scat0; f[12] = cnt.bnd - bnd0;
            f[13] = s.s0; f[14] = s.s_death; f[15] = s.k;
        }
    }

    // counters: warp reduction, one global atomic per warp
    const unsigned full = 0xffffffffu;
    unsigned v[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, v[c]);
        if ((threadIdx.x & 31) == 0 && t) atomicAdd(p.stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(p.status, 1);
    if (SMEM) {
        __syncthreads();
        for (int64_t i = threadIdx.x; i < p.hist_len; i += blockDim.x) {
            const unsigned c = shist[i];
            if (c) atomicAdd(p.hist + i, (unsigned long long)c << p.hist_shift);
        }
    }
}

template <typename R, bool SMEM> void *kernel_ptr() { return (void *)rt_transport<R, SMEM>; }

} // namespace

template <typename R> static int launch(const DevParams<R> &p, int grid, int block, size_t smem, void *stream)
{
    if (p.hist_smem)
        rt_transport<R, true><<<grid, block, smem, (cudaStream_t)stream>>>(p);
    else
        rt_transport<R, false><<<grid, block, smem, (cudaStream_t)stream>>>(p);
    return (int)cudaGetLastError();
}

int launch_transport_f32(const DevParams<float> &p, int grid, int block, size_t smem, void *stream)
{
    return launch(p, grid, block, smem, stream);
}

int launch_transport_f64(const DevParams<double> &p, int grid, int block, size_t smem, void *stream)
{
    return launch(p, grid, block, smem, stream);
}

static void *pick(int precision, int smem_hist)
{
    if (precision == RTMC_FP64) return smem_hist ? kernel_ptr<double, true>() : kernel_ptr<double, false>();
    return smem_hist ? kernel_ptr<float, true>() : kernel_ptr<float, false>();
}

int transport_set_smem(int precision, int smem_hist, size_t smem)
{
    return (int)cudaFuncSetAttribute(pick(precision, smem_hist), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int transport_occupancy(int precision, int smem_hist, int block, size_t smem, int *blocks_per_sm)
{
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pick(precision, smem_hist), block, smem);
}

} // namespace rtmc
