// Transport kernels of librtmc (sm_103a), as templates over the working precision R.
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
//
// kernels.cu instantiates this header once per precision and kernel group, so the
// variants build in parallel.
#pragma once
#include "rtmc_internal.h"

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

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
__device__ __forceinline__ void m_sincospi(float x, float *s, float *c) { sincospif(x, s, c); }
__device__ __forceinline__ void m_sincospi(double x, double *s, double *c) { sincospi(x, s, c); }
__device__ __forceinline__ float m_cospi(float x) { return cospif(x); }
__device__ __forceinline__ float m_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double m_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ double m_cospi(double x) { return cospi(x); }

// 32-bit Philox output -> uniform in (0,1): 23 bits for FP32, 32 bits for FP64.  The
// FP32 value (k + 1/2) 2^-23, k < 2^23, has 24 significant bits, so it is exact in float
// and equal to the double the oracle computes from the same output.
__device__ __forceinline__ float to_uniform(uint32_t x, float) { return ((float)(x >> 9) + 0.5f) * 1.1920928955078125e-07f; }
__device__ __forceinline__ double to_uniform(uint32_t x, double) { return ((double)x + 0.5) * 2.3283064365386962890625e-10; }

// ----------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11)
// ----------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        // one 32 x 32 -> 64-bit product per multiplier gives both halves
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
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

template <typename T> __device__ __forceinline__ T by_mode(const T v[2], int m) { return m ? v[1] : v[0]; }

// sub-steps to the first success of Bernoulli(1 - exp(-rate)) trials, ceil(-log(u) /
// rate) clamped to [1, cap]; cap = never.  inv64 is 1 / rate in FP64.
__device__ __forceinline__ int geom_steps(double u, double inv_rate, double, int on, int cap)
{
    if (!on) return cap;
    const double k = ceil(-log(u) * inv_rate);
    if (!(k < (double)cap)) return cap;
    return k < 1.0 ? 1 : (int)k;
}

// FP32: the float product -logf(u) * inv_rate carries a few ulps of rounding (logf, the
// product, the rounded reciprocal), so when it lies within 8 ulps of an integer its ceil
// may differ from the FP64 one; those rare draws (about 1e-5 of them at C3's rates) are
// settled in FP64 from the same exact uniform, so every sub-step count equals the FP64
// count.  Beyond 2^23 the float has no fraction left and the FP64 branch decides too.
__device__ __forceinline__ int geom_steps(float u, float inv_rate, double inv64, int on, int cap)
{
    if (!on) return cap;
    const float y = -logf(u) * inv_rate;
    if (y > (float)cap * 1.0001f + 1.f) return cap;
    if (fabsf(y - rintf(y)) <= 4.8e-7f * y) return geom_steps((double)u, inv64, inv64, 1, cap);
    const float k = ceilf(y);
    if (!(k < (float)cap)) return cap;
    return k < 1.f ? 1 : (int)k;
}

// sub-steps to the next scattering / Q-kill of a particle in mode m
template <typename R> __device__ __forceinline__ int scat_steps(const DevParams<R> &p, R u, int m, int cap)
{
    return geom_steps(u, by_mode(p.inv_lam, m), by_mode(p.inv_lam64, m), by_mode(p.scat_on, m), cap);
}
template <typename R> __device__ __forceinline__ int kill_steps(const DevParams<R> &p, R u, int m, int cap)
{
    return geom_steps(u, by_mode(p.inv_q, m), by_mode(p.inv_q64, m), by_mode(p.kill_on, m), cap);
}

// ----------------------------------------------------------------------------------
// inverse CDF: guide-table start, binary search, linear (extrapolating) interpolation
// ----------------------------------------------------------------------------------
__device__ __forceinline__ double invcdf_search(const Knot<double> *kn, int lo, int hi, double u)
{
    while (hi > lo) { // largest i in [lo, hi] with c[i] <= u (lo itself when none)
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&kn[mid].c) <= u) lo = mid; else hi = mid - 1;
    }
    return __ldg(&kn[lo].th) + (u - __ldg(&kn[lo].c)) * __ldg(&kn[lo].sl);
}

// FP32: c <= u for c = ch + cl and a float u is ch < u, or ch == u with cl <= 0; the offset
// (u - ch) - cl is exact up to the rounding of cl.  No FP64 instruction on this path.
__device__ __forceinline__ float invcdf_search(const Knot<float> *kn, int lo, int hi, float u)
{
    while (hi > lo) {
        const int mid = (lo + hi + 1) >> 1;
        const float2 c = __ldg(reinterpret_cast<const float2 *>(kn + mid));
        if (c.x < u || (c.x == u && c.y <= 0.f)) lo = mid; else hi = mid - 1;
    }
    const float4 k = __ldg(reinterpret_cast<const float4 *>(kn + lo));
    return k.z + ((u - k.x) - k.y) * k.w;
}

template <typename R> __device__ __forceinline__ R invcdf(const DevTables<R> &t, int ti, R u)
{
    const int G = 1 << t.gbits[ti];
    int g = (int)(u * (R)G); // exact: G is a power of two
    g = g < 0 ? 0 : (g > G - 1 ? G - 1 : g);
    const int32_t *guide = t.guide[ti];
    return invcdf_search(t.knot[ti], __ldg(guide + g), __ldg(guide + g + 1), u);
}

// ----------------------------------------------------------------------------------
// particle state (registers only: every component access below uses a static index or a
// select, so nothing is spilled to local memory)
// ----------------------------------------------------------------------------------
template <typename R> struct Part {
    R x[3], d[3], q[3];
    R th; // polar angle / pi of the last scattering (read by the adjoint replay only)
    int mode, alive;
    int s0, sS, sK, sB;
    int s_death;
    uint32_t k;
};

template <typename R> __device__ __forceinline__ R sel3(const R a[3], int k)
{
    return k == 0 ? a[0] : (k == 1 ? a[1] : a[2]);
}

template <typename R> __device__ __forceinline__ void put3(R a[3], int k, R v)
{
    a[0] = k == 0 ? v : a[0];
    a[1] = k == 1 ? v : a[1];
    a[2] = k == 2 ? v : a[2];
}


__device__ __forceinline__ float m_rnorm(float x) { return rsqrtf(x); }
__device__ __forceinline__ double m_rnorm(double x) { return 1.0 / sqrt(x); }

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
    const R s = m_rnorm(dot3(a, a));
    a[0] *= s; a[1] *= s; a[2] *= s;
}

// outside the cylinder sqrt(x^2 + y^2) = rad after j sub-steps of the segment, evaluated
// as process_event places the particle (propagateParticleSmallDt.m:327-334)
template <typename R> __device__ __forceinline__ bool cyl_outside(const Part<R> &s, R step, int j, R rad)
{
    const R t = step * (R)j;
    const R x = s.x[0] + t * s.d[0], y = s.x[1] + t * s.d[1];
    return m_sqrt(x * x + y * y) > rad;
}

// first sub-step j in [1, lim) of the segment that ends outside the cylinder, or lim:
// larger root of |P + j V|^2 = rad^2 (P, V the x-y position and per-sub-step move), then
// settled on the exact test
template <typename R> __device__ __forceinline__ int cyl_steps(const Part<R> &s, R step, R rad, int lim)
{
    if (cyl_outside(s, step, 1, rad)) return 1;
    const R vx = step * s.d[0], vy = step * s.d[1];
    const R A = vx * vx + vy * vy;
    if (!(A > (R)0)) return lim;
    const R B = s.x[0] * vx + s.x[1] * vy;
    const R C = s.x[0] * s.x[0] + s.x[1] * s.x[1] - rad * rad;
    const R sq = m_sqrt(m_max((R)0, B * B - A * C));
    const R jr = B > (R)0 ? -C / (B + sq) : (sq - B) / A;
    if (!(jr < (R)lim)) return lim;
    int j = jr < (R)1 ? 1 : (int)m_floor(jr);
    for (int it = 0; it < 4 && j < lim && !cyl_outside(s, step, j, rad); ++it) ++j;
    for (int it = 0; it < 4 && j > 1 && cyl_outside(s, step, j - 1, rad); ++it) --j;
    return j < lim ? j : lim;
}

// next boundary event of the current segment (sub-step index, or cap)
template <typename R> __device__ __forceinline__ void next_boundary(const DevParams<R> &p, Part<R> &s)
{
    const int cap = p.s_end + 1;
    s.sB = cap;
    const R step = by_mode(p.step, s.mode);
#pragma unroll
    for (int b = 0; b < RTMC_MAX_BND; ++b) {
        if (b >= p.n_bnd) break;
        if (p.bnd_dir[b] == 4) {
            const int j = cyl_steps(s, step, p.bnd_val[b], cap - s.s0);
            if (j < cap - s.s0) s.sB = s.s0 + j < s.sB ? s.s0 + j : s.sB;
            continue;
        }
        const int k = p.bnd_dir[b] - 1;
        const R a = sel3(s.x, k) - p.bnd_val[b];
        const R bs = step * sel3(s.d, k);
        if (a == (R)0 || bs == (R)0 || ((a > (R)0) == (bs > (R)0))) continue;
        const R j = m_floor(m_abs(a) / m_abs(bs)) + (R)1;
        if (j < (R)(cap - s.s0)) {
            const int sb = s.s0 + (int)j;
            s.sB = sb < s.sB ? sb : s.sB;
        }
    }
}

// griddedInterpolant(cdf, r, 'linear', 'nearest') of initializeParticle.m:201
template <typename R> __device__ __forceinline__ R radial_invcdf(const R *cdf, const R *rad, int n, R u)
{
    if (!(u > cdf[0])) return rad[0];
    if (!(u < cdf[n - 1])) return rad[n - 1];
    int lo = 0, hi = n - 1; // cdf[lo] <= u < cdf[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid; else hi = mid;
    }
    const R w = (u - cdf[lo]) / (cdf[hi] - cdf[lo]);
    return rad[lo] + w * (rad[hi] - rad[lo]);
}

// initializeParticle.m:14-148,151-170; step 0 of the particle's counter
template <typename R> __device__ void init_particle(const DevParams<R> &p, uint64_t pid, Part<R> &s)
{
    const U4<R> a = draw(p, pid, 0u, 0u);  // r1, r2, phi0, theta0 (plane: r1, r2, aperture 1, 2)
    const U4<R> b = draw(p, pid, 0u, 1u);  // phi, theta, alpha, first scattering
    if (p.src_type == RTMC_SOURCE_PLANE) {
        // plane wave (:61-148): Gaussian offset along n, aperture offsets along u and v
        const R c_long = m_sqrt((R)-2 * m_log(a.a)) * m_cospi((R)2 * a.b) * p.src_lambda * (R)0.5;
        R c1, c2;
        if (p.src_aperture == RTMC_APERTURE_CIRCLE) {
            const R rho = p.src_ext[0] * m_sqrt(a.c);
            R sa, ca;
            m_sincospi((R)2 * a.d, &sa, &ca);
            c1 = rho * ca; c2 = rho * sa;
        } else {
            c1 = (a.c - (R)0.5) * p.src_ext[0];
            c2 = (a.d - (R)0.5) * p.src_ext[1];
        }
        R st, ct;
        m_sincospi((R)2 * b.b, &st, &ct);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s.x[i] = p.src_pos[i] + c_long * p.src_n[i] + c1 * p.src_u[i] + c2 * p.src_v[i];
            s.d[i] = p.src_n[i];
            s.q[i] = ct * p.src_u[i] + st * p.src_v[i];
        }
    } else {
        // point source (:18-58): Gaussian radius, or the radial profile's inverse CDF
        const R r = p.src_radial_n > 0
                        ? radial_invcdf(p.src_radial, p.src_radial + p.src_radial_n, p.src_radial_n, a.a)
                        : m_abs(m_sqrt((R)-2 * m_log(a.a)) * m_cospi((R)2 * a.b)) * p.src_lambda;
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
    }
    s.mode = (!p.acoustics && p.polarization == 1) ? 1 : 0;
    s.alive = 1;
    s.k = 0;
    s.s0 = 0;
    s.s_death = -1;
    const int cap = p.s_end + 1;
    s.sS = scat_steps(p, b.d, s.mode, cap);
    s.sK = cap;
    if (by_mode(p.kill_on, s.mode)) {
        const U4<R> c = draw(p, pid, 0u, 2u);  // Q-kill
        s.sK = kill_steps(p, c.a, s.mode, cap);
    }
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
    const R n[3] = {k == 0 ? (R)1 : (R)0, k == 1 ? (R)1 : (R)0, k == 2 ? (R)1 : (R)0};
    const int m0 = s.mode;
    const R dk = sel3(s.d, k);
    R adn = m_abs(dk);
    adn = adn > (R)1 ? (R)1 : adn;
    const R ang = m_acos(adn) * (R)57.295779513082320876798154814105;
    if (s.mode == 0) {
        const R rpp = zoe_lookup(p.zoe, ang);
        if (u_coin <= rpp) {
            put3(s.d, k, -dk);
            put3(s.q, k, -sel3(s.q, k));
        } else { // P -> SV, propagateParticleSmallDt.m:212-248
            s.mode = 1;
            const R ratio = p.vs_over_vp;
            R nd[3] = {s.d[0] * ratio, s.d[1] * ratio, s.d[2] * ratio};
            put3(nd, k, (R)0);
            const R sin2 = dot3(nd, nd);
            const R cv = m_sqrt(m_max((R)0, (R)1 - sin2));
            const R sg = (R)((dk > (R)0) - (dk < (R)0));
            put3(nd, k, -sg * cv);
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
            // arbitrary tangent [1 0 0] projected on the plane (MaterialClass.m:1618-1625)
            eSH[0] = k == 0 ? (R)0 : (R)1; eSH[1] = (R)0; eSH[2] = (R)0;
            nsh = m_sqrt(dot3(eSH, eSH));
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
            put3(s.d, k, -dk);
            put3(s.q, k, -sel3(s.q, k));
        } else {
            const R rsv = zoe_lookup(p.zoe + RTMC_ZOE_N, ang);
            if (u_coin <= rsv) { // SV -> SV
                put3(s.d, k, -dk);
                put3(s.q, k, -sel3(s.q, k));
            } else { // SV -> P, :274-321
                const R ratio = p.vp_over_vs;
                R nd[3] = {s.d[0] * ratio, s.d[1] * ratio, s.d[2] * ratio};
                put3(nd, k, (R)0);
                const R sin2 = dot3(nd, nd);
                if (sin2 <= (R)1) {
                    s.mode = 0;
                    const R sg = (R)((dk > (R)0) - (dk < (R)0));
                    put3(nd, k, -sg * m_sqrt((R)1 - sin2));
                    normalize3(nd);
                    s.d[0] = nd[0]; s.d[1] = nd[1]; s.d[2] = nd[2];
                } else {
                    put3(s.d, k, -dk); // total internal reflection: SV, dir mirrored only
                }
            }
        }
    }
    return s.mode != m0;
}

// mirror of v in the plane normal to the unit vector n: v - 2 (v.n) n
template <typename R> __device__ __forceinline__ void mirror3(R v[3], const R n[3])
{
    const R vn = (R)2 * dot3(v, n);
#pragma unroll
    for (int i = 0; i < 3; ++i) v[i] -= vn * n[i];
}

// elastic reflection at the cylinder wall with outward unit normal n
// (propagateParticleSmallDt.m:356-571): P -> P or P -> SV by E_Rpp; S split into SH / SV by
// the polarisation's component along d x n; SV -> SV or SV -> P by E_Rsvsv, with total
// internal reflection falling back to an SV mirror.  Angles past 90 degrees take the
// 90-degree coefficient ('nearest' extrapolation).  Returns 1 if the mode changed.
template <typename R>
__device__ int cylinder_reflect(const DevParams<R> &p, Part<R> &s, const R n[3], R u_split, R u_coin)
{
    const int m0 = s.mode;
    const R dn = dot3(s.d, n);
    R ang = m_acos(dn < (R)-1 ? (R)-1 : (dn > (R)1 ? (R)1 : dn)) * (R)57.295779513082320876798154814105;
    ang = ang > (R)90 ? (R)90 : ang;
    if (s.mode == 0) {
        if (u_coin <= zoe_lookup(p.zoe, ang)) { // P -> P
            mirror3(s.d, n);
            mirror3(s.q, n);
        } else { // P -> SV (:409-451)
            s.mode = 1;
            const R eta = p.vs_over_vp;
            R nd[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) nd[i] = eta * (s.d[i] - dn * n[i]);
            const R cv = m_sqrt(m_max((R)0, (R)1 - dot3(nd, nd)));
#pragma unroll
            for (int i = 0; i < 3; ++i) nd[i] -= cv * n[i];
            normalize3(nd);
            s.d[0] = nd[0]; s.d[1] = nd[1]; s.d[2] = nd[2];
            R ax[3];
            cross3(s.d, n, ax);
            if (m_sqrt(dot3(ax, ax)) < (R)1e-6) { // normal incidence: axis d x e_x
                const R ex[3] = {(R)1, (R)0, (R)0};
                cross3(s.d, ex, ax);
            }
            normalize3(ax);
            cross3(ax, s.d, s.q);
        }
    } else {
        R ax[3];
        cross3(s.d, n, ax);
        const R a2 = dot3(ax, ax);
        const R sh = dot3(s.q, ax);
        // (q . (d x n) / |d x n|)^2; d parallel to n leaves it undefined and the particle SV
        const R prob_sh = a2 > (R)0 ? sh * sh / a2 : (R)-1;
        if (u_split < prob_sh) { // SH -> SH
            mirror3(s.d, n);
            mirror3(s.q, n);
        } else if (u_coin <= zoe_lookup(p.zoe + RTMC_ZOE_N, ang)) { // SV -> SV
            mirror3(s.d, n);
            mirror3(s.q, n);
        } else { // SV -> P (:523-566)
            const R eta = p.vp_over_vs;
            R nd[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) nd[i] = eta * (s.d[i] - dn * n[i]);
            const R sin2 = dot3(nd, nd);
            if (sin2 <= (R)1) {
                s.mode = 0;
                const R cv = m_sqrt((R)1 - sin2);
#pragma unroll
                for (int i = 0; i < 3; ++i) nd[i] -= cv * n[i];
                normalize3(nd);
                s.d[0] = nd[0]; s.d[1] = nd[1]; s.d[2] = nd[2]; // polarisation kept
            } else { // total internal reflection: SV mirror
                mirror3(s.d, n);
                mirror3(s.q, n);
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
    const R th_pi = invcdf(p.tab, ti, u_theta); // tables hold theta / pi
    s.th = th_pi;
    R st, ct;
    m_sincospi(th_pi, &st, &ct);
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

// one event: the earliest of kill / boundary / scattering (ties in that order); returns
// its kind (2 kill, 1 boundary, 0 scattering)
template <typename R>
__device__ int process_event(const DevParams<R> &p, uint64_t pid, Part<R> &s, Counters &cnt)
{
    const int cap = p.s_end + 1;
    int e = s.sK, kind = 2;
    if (s.sB < e) { e = s.sB; kind = 1; }
    if (s.sS < e) { e = s.sS; kind = 0; }
    if (kind == 2) {
        s.alive = 0;
        s.s_death = e;
        cnt.kill++;
        return kind;
    }
    s.k++;
    const R step = by_mode(p.step, s.mode);
    const R dt = step * (R)(e - s.s0);
    R xe[3] = {s.x[0] + dt * s.d[0], s.x[1] + dt * s.d[1], s.x[2] + dt * s.d[2]};
    if (kind == 1) {
        const R dt1 = step * (R)(e - 1 - s.s0);
        const R x1[3] = {s.x[0] + dt1 * s.d[0], s.x[1] + dt1 * s.d[1], s.x[2] + dt1 * s.d[2]};
        s.x[0] = xe[0]; s.x[1] = xe[1]; s.x[2] = xe[2];
        int changed = 0;
#pragma unroll
        for (int b = 0; b < RTMC_MAX_BND; ++b) {
            if (b >= p.n_bnd) break;
            const R val = p.bnd_val[b];
            if (p.bnd_dir[b] == 4) { // cylinder (propagateParticleSmallDt.m:325-348)
                const R r = m_sqrt(s.x[0] * s.x[0] + s.x[1] * s.x[1]);
                const R over = r - val;
                if (!(over > (R)0)) continue;
                cnt.bnd++;
                if (p.bnd_absorb[b]) {
                    s.alive = 0;
                    s.s0 = e;
                    s.s_death = e;
                    cnt.absorb++;
                    return kind;
                }
                const R n[3] = {s.x[0] / r, s.x[1] / r, (R)0};
                s.x[0] -= (R)2 * over * n[0];
                s.x[1] -= (R)2 * over * n[1];
                if (p.acoustics) {
                    mirror3(s.d, n);
                } else {
                    const U4<R> bb = draw(p, pid, s.k, 1u + (uint32_t)b);
                    const int ch = cylinder_reflect(p, s, n, bb.a, bb.b);
                    cnt.conv += ch;
                    changed |= ch;
                }
                continue;
            }
            const int k = p.bnd_dir[b] - 1;
            const R xk = sel3(s.x, k);
            if (!((xk - val) * (sel3(x1, k) - val) < (R)0)) continue;
            cnt.bnd++;
            if (p.bnd_absorb[b]) {
                s.alive = 0;
                s.s0 = e;
                s.s_death = e;
                cnt.absorb++;
                return kind;
            }
            put3(s.x, k, (R)2 * val - xk);
            if (p.acoustics) {
                put3(s.d, k, -sel3(s.d, k));
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
            const int js = scat_steps(p, r0.a, s.mode, cap);
            s.sS = js >= cap ? cap : e - 1 + js;
            const int jk = kill_steps(p, r0.b, s.mode, cap);
            s.sK = jk >= cap ? cap : e + jk;
        }
    } else {
        const U4<R> r0 = draw(p, pid, s.k, 0u); // next, azimuth, mode, theta
        s.x[0] = xe[0]; s.x[1] = xe[1]; s.x[2] = xe[2];
        const int m0 = s.mode;
        scatter(p, s, r0.b, r0.c, r0.d);
        cnt.scat++;
        s.s0 = e;
        const int js = scat_steps(p, r0.a, s.mode, cap);
        s.sS = js >= cap ? cap : e + js;
        if (s.mode != m0 && by_mode(p.kill_on, s.mode)) {
            const U4<R> r1 = draw(p, pid, s.k, 1u);
            const int jk = kill_steps(p, r1.a, s.mode, cap);
            s.sK = jk >= cap ? cap : e + jk;
        } else if (s.mode != m0) {
            s.sK = cap;
        }
    }
    if (s.sS > cap) s.sS = cap;
    if (s.sK > cap) s.sK = cap;
    next_boundary(p, s);
    return kind;
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
        // the arithmetic guess is off by at most one near an edge: settle it on the edges
        b = b - (c < e[b] ? 1 : 0) + ((b < nb - 1 && c >= e[b + 1]) ? 1 : 0);
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

// observeTime.m:24-32: the direction axis depends on the direction only, so its bin
// offset is computed once per trajectory segment (-1: outside its range)
template <typename R>
__device__ __forceinline__ int dir_offset(const DevParams<R> &p, const R *sedges, R dz)
{
    const int am = p.ax_mode[3];
    if (am == RTMC_AXIS_IGNORED) return 0;
    const R cz = dz > (R)1 ? (R)1 : (dz < (R)-1 ? (R)-1 : dz);
    const R c = (p.d == 3) ? cz : m_acos(cz);
    if (am == RTMC_AXIS_RANGE) return (c >= p.ax_lo[3] && c <= p.ax_hi[3]) ? 0 : -1;
    const int b = bin_of(p, sedges, 3, c);
    return b < 0 ? -1 : b * p.ax_stride32[3];
}

__device__ __forceinline__ float m_fast_sqrt(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }
__device__ __forceinline__ double m_fast_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ int m_floor_int(float x) { return __float2int_rd(x); }
__device__ __forceinline__ int m_floor_int(double x) { return __double2int_rd(x); }

// Bin of a coordinate t measured in bin widths: floor(t) for t in [0, 2^23), and a value
// outside [0, 2^23) (negative, or at least 2^23) for every other t, infinities and NaN
// included, so one unsigned compare against the bin count rejects all of those.  FP32:
// adding 2^23 with rounding toward zero leaves floor(t) in the low mantissa bits (one
// FADD and one integer add on the FMA/ALU pipes instead of a float-to-int conversion).
__device__ __forceinline__ int bin_floor(float t) { return __float_as_int(__fadd_rz(t, 8388608.0f)) - 0x4B000000; }
__device__ __forceinline__ int bin_floor(double t)
{
    return t >= 0.0 && t < 8388608.0 ? __double2int_rd(t) : -1;
}

// Multiply-adds and products of the binning written out, so that every kernel that bins
// (the fused transports, the batch, the split schedule's observation kernel) rounds them
// the same way and puts an observation on a bin edge into the same bin.
__device__ __forceinline__ float m_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double m_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float m_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double m_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float m_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double m_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float m_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double m_sub(double a, double b) { return __dsub_rn(a, b); }

// observeTime.m:14-144 for the position axes X, Y, Z of one observation in any frame:
// offset of the bin inside the time slice (direction part excluded), or -1
template <typename R>
__device__ __forceinline__ int pos_offset(const DevParams<R> &p, const R *sedges, const R x[3])
{
    R c[3];
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
            c[2] = (p.ax_mode[2] != RTMC_AXIS_IGNORED && r > (R)0) ? x[2] / r : (R)0; // sin(elevation)
        }
    }
    int idx = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int am = p.ax_mode[a];
        if (am == RTMC_AXIS_RANGE) {
            if (!(c[a] >= p.ax_lo[a] && c[a] <= p.ax_hi[a])) return -1;
        } else if (am == RTMC_AXIS_BINNED) {
            const int b = bin_of(p, sedges, a, c[a]);
            if (b < 0) return -1;
            idx += b * p.ax_stride32[a];
        }
    }
    return idx;
}

// Observation paths, fixed at compile time from the observation grid:
//   OBS_CART    cartesian frame, uniform finite axes: a coordinate is linear in the
//               sub-step along a segment, so its bin position is t = A + B * (so - s0)
//               with A, B set once per segment (one FMA and a floor per axis);
//   OBS_RADIAL  radius-only frames (the other position axes integrate over their whole
//               range): r = |x0 + D (so - s0)|;
//   OBS_GENERAL anything else (angles, non-uniform edges).
// The fast paths place a coordinate sitting on a bin edge to within rounding by
// arithmetic rather than by comparing with the edge table.
enum { OBS_GENERAL = 0, OBS_CART = 1, OBS_RADIAL = 2 };

// A straight piece of trajectory: position x at sub-step s0, direction d, mode, plus the
// per-segment binning terms of the observation path.  On the cartesian and radius-only
// paths the ring holds the prepared terms (A, B or x, B, and the direction offset), so a
// segment coming into force in the observation phase needs no arithmetic.
template <typename R> struct Seg {
    R x[3], d[3];
    R A[3], B[3];
    int s0, mode, doff;
    R th; // adjoint only: theta / pi of the scattering that starts the segment, or -1
};

template <typename R, int OBS>
__device__ __forceinline__ void seg_prepare(const DevParams<R> &p, const R *sedges, Seg<R> &g)
{
    g.doff = dir_offset(p, sedges, g.d[2]);
    const R step = by_mode(p.step, g.mode);
    if (OBS == OBS_CART) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            g.A[a] = m_mul(m_sub(g.x[a], p.ax_lo[a]), p.ax_inv_w[a]);
            g.B[a] = m_mul(m_mul(step, g.d[a]), p.ax_inv_w[a]);
        }
    } else if (OBS == OBS_RADIAL) {
#pragma unroll
        for (int a = 0; a < 3; ++a) g.B[a] = m_mul(step, g.d[a]);
        // |(x, y)| (2D, or the cylindrical frame): the third coordinate of the observation
        // copy is zero, so every radius is |x| over three coordinates without a branch
        if (!p.radial_3d) g.x[2] = g.B[2] = (R)0;
    }
}

// bin offset inside the time slice of an observation dl sub-steps after the start of
// segment g, or -1
template <typename R, int OBS>
__device__ __forceinline__ int obs_offset_dl(const DevParams<R> &p, const R *sedges, const Seg<R> &g, R dl)
{
    if (OBS == OBS_CART) {
        // branch-free: the three bins, one combined range test
        int idx = g.doff;
        bool ok = g.doff >= 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int b = bin_floor(m_fma(g.B[a], dl, g.A[a]));
            ok = ok && (unsigned)b < (unsigned)p.ax_nbe[a];
            idx += b * p.ax_stride32[a];
        }
        return ok ? idx : -1;
    } else if (OBS == OBS_RADIAL) {
        // the segment's third coordinate is zero where the radius is |(x, y)| (seg_prepare)
        const R x0 = m_fma(g.B[0], dl, g.x[0]), x1 = m_fma(g.B[1], dl, g.x[1]), x2 = m_fma(g.B[2], dl, g.x[2]);
        const R r2 = m_fma(x2, x2, m_fma(x1, x1, m_mul(x0, x0)));
        const int b = bin_floor(m_fma(m_fast_sqrt(r2), p.ax_inv_w[0], p.ax_a0));
        return (g.doff >= 0 && (unsigned)b < (unsigned)p.ax_nbe[0]) ? g.doff + b * p.ax_stride32[0] : -1;
    } else {
        if (g.doff < 0) return -1;
        const R dt = m_mul(by_mode(p.step, g.mode), dl);
        const R xo[3] = {m_fma(dt, g.d[0], g.x[0]), m_fma(dt, g.d[1], g.x[1]), m_fma(dt, g.d[2], g.x[2])};
        const int po = pos_offset(p, sedges, xo);
        return po < 0 ? -1 : po + g.doff;
    }
}

// The FP32 cartesian path of the observation kernel, the same bins as obs_offset_dl with
// one integer add per axis fewer: t's bit pattern, compared unsigned with that of the bin
// count, is below it exactly for 0 <= t < count (negative t, NaN and infinities have
// larger patterns; t is never -0 because the segment's offsets are normalised), and the
// bin's pattern after adding 2^23 toward zero is 0x4B000000 + floor(t), whose bias the
// segment's `base` already carries.  A segment whose direction lies outside the grid has A[0] = inf.
__device__ __forceinline__ int obs_offset_cart32(const DevParams<float> &p, const Seg<float> &g, float dl, int base)
{
    bool ok = true;
    unsigned idx = (unsigned)base;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float t = m_fma(g.B[a], dl, g.A[a]);
        ok = ok && (unsigned)__float_as_int(t) < (unsigned)p.ax_nbits[a];
        idx += (unsigned)__float_as_int(__fadd_rz(t, 8388608.0f)) * (unsigned)p.ax_stride32[a];
    }
    return ok ? (int)idx : -1;
}
__device__ __forceinline__ int obs_offset_cart32(const DevParams<double> &, const Seg<double> &, double, int) { return -1; }

// FP64 radius-only binning through an FP32 estimate.  Per segment: the start position and
// the step in FP32 (xf, Bf) and the sums of their magnitudes (sx, sb).  The FP32 bin
// coordinate t' = |xf + Bf dl| / w - lo / w differs from the FP64 one by at most
//   2^-23 (sb dl + sx) / w        (the positions: two roundings to FP32, one multiply-add)
// + 2^-21 r' / w                  (|x|^2 in FP32 and x * rsqrt(x) for the root)
// + 2^-24 (r' / w + |lo / w| + |t'|)   (the rounded 1/w and -lo/w, the final multiply-add)
// + the FP64 roundings (far below 2^-30 for coordinates below 2^23); M = 2^-19 (...)
// bounds all of it.  When t' - M and t' + M floor to the same integer, so does the FP64
// coordinate, and that is the bin; otherwise (an observation within M of a bin edge) the
// FP64 formula decides.  The bins are those of the FP64 path exactly.
struct SegF {
    float xf[3], Bf[3], sx, sb;
};
// the segment in FP32: start position (radius-only) or start coordinates A (cartesian),
// and the step
template <int OBS> __device__ __forceinline__ void segf_from(const Seg<double> &g, SegF &f)
{
    const double *u = OBS == OBS_CART ? g.A : g.x;
#pragma unroll
    for (int a = 0; a < 3; ++a) { f.xf[a] = (float)u[a]; f.Bf[a] = (float)g.B[a]; }
    f.sx = fabsf(f.xf[0]) + fabsf(f.xf[1]) + fabsf(f.xf[2]);
    f.sb = fabsf(f.Bf[0]) + fabsf(f.Bf[1]) + fabsf(f.Bf[2]);
}
template <int OBS> __device__ __forceinline__ void segf_from(const Seg<float> &, SegF &) {}

// FP64 cartesian binning through FP32 estimates, axis by axis: t' = A' + B' dl from the
// segment's coordinates rounded to FP32 differs from the FP64 coordinate by at most
// 2^-23 (|B| dl + |A| + |t'|) (two roundings to FP32, one multiply-add; the FP64 roundings
// are far smaller), so M = 2^-21 (|B'| dl + |A'| + |t'|) bounds it.  An axis whose
// interval t' -/+ M floors to one integer has that bin; if any axis is within M of an edge
// the FP64 formula decides for the observation.  Axes a problem ignores have A = B = 0
// and so M = 0.
template <typename R>
__device__ __forceinline__ int obs_offset_cart64(const DevParams<R> &p, const R *sedges, const Seg<R> &g, const SegF &f,
                                                 float d)
{
    // d, the sub-steps since the segment start, is an exact integer (below 2^24 here)
    if (g.doff < 0) return -1;
    int idx = g.doff;
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float t = fmaf(f.Bf[a], d, f.xf[a]);
        const float m = 0x1p-21f * (fmaf(fabsf(f.Bf[a]), d, fabsf(f.xf[a])) + fabsf(t));
        const int bl = bin_floor(__fsub_rd(t, m)), bh = bin_floor(__fadd_ru(t, m));
        if (bl != bh) return obs_offset_dl<R, OBS_CART>(p, sedges, g, (R)d); // near an edge: FP64 decides
        ok = ok && (unsigned)bl < (unsigned)p.ax_nbe[a];
        idx += bl * p.ax_stride32[a];
    }
    return ok ? idx : -1;
}

template <typename R>
__device__ __forceinline__ int obs_offset_radial64(const DevParams<R> &p, const R *sedges, const Seg<R> &g, const SegF &f,
                                                   float d)
{
    // d, the sub-steps since the segment start, is an exact integer (below 2^24 here)
    if (g.doff < 0) return -1;
    const float x0 = fmaf(f.Bf[0], d, f.xf[0]), x1 = fmaf(f.Bf[1], d, f.xf[1]), x2 = fmaf(f.Bf[2], d, f.xf[2]);
    const float r2 = fmaf(x2, x2, fmaf(x1, x1, x0 * x0)); // x2 = 0 for |(x, y)| (seg_prepare)
    const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
    const float t = fmaf(r, p.r32_iw, p.r32_a0);
    const float m = 0x1p-19f * (fmaf(fmaf(f.sb, d, f.sx) + r, p.r32_iw, fabsf(p.r32_a0) + fabsf(t)) + 1.f);
    const int bl = bin_floor(__fsub_rd(t, m)), bh = bin_floor(__fadd_ru(t, m));
    if (bl != bh) return obs_offset_dl<R, OBS_RADIAL>(p, sedges, g, (R)d); // near an edge: FP64 decides
    return (unsigned)bl < (unsigned)p.ax_nbe[0] ? g.doff + bl * p.ax_stride32[0] : -1;
}


// the same at sub-step so
template <typename R, int OBS>
__device__ __forceinline__ int obs_offset(const DevParams<R> &p, const R *sedges, const Seg<R> &g, int so)
{
    return obs_offset_dl<R, OBS>(p, sedges, g, (R)(so - g.s0));
}

// The radius-only path for a radius |(x, y)| (2D, the cylindrical frame): the bin of
// obs_offset_dl<R, OBS_RADIAL> without its third coordinate, which seg_prepare zeroed there
// (the same operations and value: the skipped multiply-add adds 0 * 0)
template <typename R>
__device__ __forceinline__ int obs_offset_radius2(const DevParams<R> &p, const Seg<R> &g, R dl)
{
    const R x0 = m_fma(g.B[0], dl, g.x[0]), x1 = m_fma(g.B[1], dl, g.x[1]);
    const R r2 = m_fma(x1, x1, m_mul(x0, x0));
    const int b = bin_floor(m_fma(m_fast_sqrt(r2), p.ax_inv_w[0], p.ax_a0));
    return (g.doff >= 0 && (unsigned)b < (unsigned)p.ax_nbe[0]) ? g.doff + b * p.ax_stride32[0] : -1;
}

// Per-lane ring of segments in shared memory, field-major so that lane t of every
// slot sits in bank t % 32.
template <typename R> struct Ring {
    R *x0, *x1, *x2, *d0, *d1, *d2;
    int *s0, *mode;
    R *th; // adjoint only
    int cap, stride;
    template <bool TH = false> __device__ __forceinline__ void put(int slot, const Part<R> &s, R t = (R)-1) const
    {
        const int k = slot * stride + threadIdx.x;
        x0[k] = s.x[0]; x1[k] = s.x[1]; x2[k] = s.x[2];
        d0[k] = s.d[0]; d1[k] = s.d[1]; d2[k] = s.d[2];
        s0[k] = s.s0; mode[k] = s.mode;
        if (TH) th[k] = t;
    }
    template <bool TH = false> __device__ __forceinline__ void get(int slot, Seg<R> &g) const
    {
        const int k = slot * stride + threadIdx.x;
        g.x[0] = x0[k]; g.x[1] = x1[k]; g.x[2] = x2[k];
        g.d[0] = d0[k]; g.d[1] = d1[k]; g.d[2] = d2[k];
        g.s0 = s0[k]; g.mode = mode[k];
        if (TH) g.th = th[k];
    }
    // prepared segments of the cartesian (A, B) and radius-only (x, B) paths: the start
    // sub-step (below 2^30) carries the mode in bit 30, and the mode slot holds the
    // direction offset (negative: outside the direction range)
    template <int OBS, bool TH = false> __device__ __forceinline__ void put_prepared(int slot, const Seg<R> &g, R t) const
    {
        const int k = slot * stride + threadIdx.x;
        const R *u = OBS == OBS_CART ? g.A : g.x;
        x0[k] = u[0]; x1[k] = u[1]; x2[k] = u[2];
        d0[k] = g.B[0]; d1[k] = g.B[1]; d2[k] = g.B[2];
        s0[k] = g.s0 | (g.mode << 30); mode[k] = g.doff;
        if (TH) th[k] = t;
    }
    template <int OBS, bool TH = false> __device__ __forceinline__ void get_prepared(int slot, Seg<R> &g) const
    {
        const int k = slot * stride + threadIdx.x;
        R *u = OBS == OBS_CART ? g.A : g.x;
        u[0] = x0[k]; u[1] = x1[k]; u[2] = x2[k];
        g.B[0] = d0[k]; g.B[1] = d1[k]; g.B[2] = d2[k];
        const int sm = s0[k];
        g.s0 = sm & 0x3fffffff;
        g.mode = sm >> 30;
        g.doff = mode[k];
        if (TH) g.th = th[k];
    }
    __device__ __forceinline__ int start(int slot) const { return s0[slot * stride + threadIdx.x] & 0x3fffffff; }
};

template <typename R> __device__ __forceinline__ void seg_from(const Part<R> &s, Seg<R> &g)
{
#pragma unroll
    for (int c = 0; c < 3; ++c) { g.x[c] = s.x[c]; g.d[c] = s.d[c]; }
    g.s0 = s.s0;
    g.mode = s.mode;
}

template <typename R> __device__ __forceinline__ int next_event(const Part<R> &s) { return min(min(s.sK, s.sB), s.sS); }

// Where observations go: a block-private u32 histogram in shared memory (the whole
// histogram fits), 64-bit global atomics, or a dense time-major array of 32-bit bin
// indices that rt_bin_slices folds into the histogram one time slice at a time.
enum { SINK_SMEM = 0, SINK_GLOBAL = 1, SINK_INDEX = 2, SINK_ADJOINT = 3 };

// Per-lane score state of the adjoint sink (at most kAdjRingParams parameters).  The
// score of the segment in force is A + b_obs * j: sa sums the adjoint weights of the
// segment's observations, saj the weights times j over the whole particle, and G the
// products A * sa of the particle's finished segments, all in the transport's precision;
// at the particle's end g += G + b_obs * saj in FP64.  FP64 instructions are slow on this
// part, so none runs per observation or per scattering in the FP32 replay.
constexpr int kAdjRingParams = 4;
template <typename R> struct AdjLane {
    const AdjointArgs *a; // read in the rare paths (a new scattering, the particle's end)
    const R *wts;         // adjoint weights, read per observation
    const R *dls;         // d log sigma tables in the transport's precision
    R A[kAdjRingParams], G[kAdjRingParams];
    R sa, saj;
    double g[kAdjRingParams];
    __device__ __forceinline__ void start()
    {
#pragma unroll
        for (int q = 0; q < kAdjRingParams; ++q) { A[q] = (R)0; G[q] = (R)0; }
        sa = saj = (R)0;
    }
    // a new segment is in force; a scattering at theta / pi = th >= 0 started it
    __device__ __forceinline__ void enter(R th)
    {
        if (!(th >= (R)0)) return;
        const int np = a->n_params, nt = a->n_theta;
        R f = th > (R)1 ? (R)1 : th;
        f *= (R)(nt - 1);
        int k = (int)f;
        k = k > nt - 2 ? nt - 2 : k;
        const R w = f - (R)k;
#pragma unroll
        for (int q = 0; q < kAdjRingParams; ++q) {
            if (q < np) {
                G[q] += A[q] * sa;
                const R *t = dls + (size_t)q * nt + k;
                const R t0 = __ldg(t), t1 = __ldg(t + 1);
                A[q] += t0 + w * (t1 - t0) + (sizeof(R) == 4 ? (R)a->a_inc_f[q] : (R)a->a_inc[q]);
            }
        }
        sa = (R)0;
    }
    __device__ __forceinline__ void observe(int64_t idx, int j)
    {
        const R w = __ldg(wts + idx);
        sa += w;
        saj += w * (R)j;
    }
    // an observation of weight w at instant fj, carried as a float (w = 0: none; adding
    // zeros leaves both sums bit for bit as they were)
    __device__ __forceinline__ void observe_w(R w, R fj)
    {
        sa += w;
        saj = m_fma(w, fj, saj);
    }
    // the particle's end
    __device__ __forceinline__ void finish()
    {
#pragma unroll
        for (int q = 0; q < kAdjRingParams; ++q)
            if (q < a->n_params) g[q] += (double)(G[q] + A[q] * sa) + a->b_obs[q] * (double)saj;
    }
};

// launch bounds of the transport variants (build-time knobs for the index/global sinks)
#ifndef RTMC_TRANSPORT_THREADS
#define RTMC_TRANSPORT_THREADS 256
#endif
#ifndef RTMC_TRANSPORT_MIN_BLOCKS
#define RTMC_TRANSPORT_MIN_BLOCKS 3 // FP32: 3 x 256 threads per SM measured fastest
#endif
template <typename R, int SINK> struct Bounds {
    static constexpr int threads = SINK == SINK_SMEM ? 512 : RTMC_TRANSPORT_THREADS;
    static constexpr int min_blocks = SINK == SINK_SMEM ? 1 : (sizeof(R) == 4 ? RTMC_TRANSPORT_MIN_BLOCKS : 2);
};

// One warp's batch of 32 consecutive particles [base, base + 32) of the problem p,
// clipped at n_end: the two-cursor transport described at rt_transport.  The adjoint
// sink (adj non-null) accumulates adjoint weights instead of binning, and carries each
// segment's scattering angle through the ring to update the score when the segment
// comes into force.
template <typename R, int SINK, int OBS>
__device__ __forceinline__ void run_batch(const DevParams<R> &p, const R *sedges, unsigned *shist, const Ring<R> &ring,
                                          int64_t base, int64_t n_end, Counters &cnt, bool &bad,
                                          AdjLane<R> *adj = nullptr)
{
    constexpr bool SMEM = SINK == SINK_SMEM;
    constexpr bool ADJ = SINK == SINK_ADJOINT;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned long long inc = 1ull << p.hist_shift;
    const int s_end = p.s_end;
    const int C = ring.cap;
    const int64_t i = base + lane;
    const bool have = i < n_end;
    const uint64_t pid = (uint64_t)(p.pid0 + i);
    Part<R> s;
    Seg<R> cur;
    int head = 0, count = 0;
    const unsigned scat0 = cnt.scat, bnd0 = cnt.bnd;
    if (have) {
        init_particle(p, pid, s);
    } else {
        s.alive = 0; s.s_death = 0; s.s0 = 0; s.sS = s.sK = s.sB = s_end + 1; s.k = 0; s.mode = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) { s.x[c] = (R)0; s.d[c] = (R)0; s.q[c] = (R)0; }
    }
    seg_from(s, cur);
    seg_prepare<R, OBS>(p, sedges, cur);
    if (ADJ) adj->start();
    // the cartesian and radius-only paths keep prepared segments in the ring: their binning
    // terms are computed in phase 1, where events run converged, not when a lane's segment
    // comes into force in phase 2
    constexpr bool PREP = OBS == OBS_CART || OBS == OBS_RADIAL;
    auto take = [&](int slot) { // cur = the ring's segment in `slot`, ready for binning
        if constexpr (PREP) {
            ring.template get_prepared<OBS, ADJ>(slot, cur);
        } else {
            ring.template get<ADJ>(slot, cur);
            seg_prepare<R, OBS>(p, sedges, cur);
        }
    };
    int32_t *optr = (SINK == SINK_INDEX && have) ? p.obs_idx + i : nullptr;
    int jn = 1; // warp-uniform
    while (jn <= p.n_obs) {
        // ---- phase 1: refill the rings (events of all lanes with room run together)
        const int so_next = jn * p.n_sub;
        for (;;) {
            // segments starting at or before the next observation supersede the
            // current one: consume them, so the ring only holds later segments
            while (count > 0 && ring.start(head) <= so_next) {
                take(head);
                if (ADJ) adj->enter(cur.th);
                head = (head + 1) % C;
                --count;
            }
            const bool need = s.alive && count < C && next_event(s) <= s_end;
            if (!__any_sync(full, need)) break;
            if (need) {
                const int kind = process_event(p, pid, s, cnt);
                if ((int)s.k > p.max_events) { s.alive = 0; s.s_death = s.s0; bad = true; }
                if (s.alive) {
                    const R th = (ADJ && kind == 0) ? s.th : (R)-1;
                    if (count == 0 && s.s0 <= so_next) {
                        seg_from(s, cur);
                        if (ADJ) adj->enter(th);
                        seg_prepare<R, OBS>(p, sedges, cur);
                    } else {
                        if constexpr (PREP) {
                            Seg<R> g;
                            seg_from(s, g);
                            seg_prepare<R, OBS>(p, sedges, g);
                            ring.template put_prepared<OBS, ADJ>((head + count) % C, g, th);
                        } else {
                            ring.template put<ADJ>((head + count) % C, s, th);
                        }
                        ++count;
                    }
                }
            }
        }
        // ---- window: observations every live lane has covered (dead lanes never limit)
        unsigned avail = 0x7fffffffu;
        if (s.alive) {
            const int limit = next_event(s) <= s_end ? next_event(s) : s_end + 1;
            int last = (limit - 1) / p.n_sub;
            last = last < p.n_obs ? last : p.n_obs;
            avail = (unsigned)(last - jn + 1);
        }
        unsigned nw = __reduce_min_sync(full, avail);
        if (nw > (unsigned)(p.n_obs - jn + 1)) {
            if (SINK == SINK_INDEX) {
                nw = (unsigned)(p.n_obs - jn + 1); // no live lane left: write the rest
            } else {
                // no live lane left: bin what the dead lanes observed before dying
                int rem = 0;
                if (have && s.s_death > jn * p.n_sub) rem = min(p.n_obs, (s.s_death - 1) / p.n_sub) - jn + 1;
                nw = __reduce_max_sync(full, (unsigned)(rem > 0 ? rem : 0));
                if (nw == 0) break;
            }
        }
        // ---- phase 2: nw observations per lane, two at a time (independent chains)
        const int obs_limit = s.alive ? 0x7fffffff : s.s_death;
        int next_start = count > 0 ? ring.start(head) : 0x7fffffff;
        int so = jn * p.n_sub;
        // make cur the segment in force at sub-step at
        auto advance = [&](int at) {
            do {
                take(head);
                if (ADJ) adj->enter(cur.th);
                head = (head + 1) % C;
                --count;
            } while (count > 0 && ring.start(head) <= at);
            next_start = count > 0 ? ring.start(head) : 0x7fffffff;
        };
        auto emit = [&](int v, int mode, int j) {
            if (SINK == SINK_INDEX) {
                if (have) {
                    *optr = v < 0 ? -1 : (v | (mode << 30));
                    optr += p.obs_rows;
                }
                if (v >= 0) cnt.obs++;
            } else if (v >= 0) {
                const int64_t idx = (int64_t)j * p.time_stride + (mode ? p.mode_stride : 0) + v;
                if (idx < p.hist_len) {
                    cnt.obs++;
                    if (ADJ) adj->observe(idx, j);
                    else if (SMEM) atomicAdd(shist + idx, 1u);
                    else atomicAdd(p.hist + idx, inc);
                } else {
                    bad = true;
                }
            }
        };
        unsigned w = 0;
        // pairs (the adjoint goes one at a time: the score may change between the two)
        for (; !ADJ && w + 1 < nw; w += 2, jn += 2, so += 2 * p.n_sub) {
            const int so1 = so + p.n_sub;
            int v0 = -1, v1 = -1, m0 = cur.mode, m1 = cur.mode;
            if (so < obs_limit) {
                if (so >= next_start) advance(so);
                m0 = m1 = cur.mode;
                v0 = obs_offset<R, OBS>(p, sedges, cur, so);
                if (so1 < obs_limit) {
                    if (so1 >= next_start) {
                        advance(so1);
                        m1 = cur.mode;
                    }
                    v1 = obs_offset<R, OBS>(p, sedges, cur, so1);
                }
            }
            emit(v0, m0, jn);
            emit(v1, m1, jn + 1);
        }
        for (; w < nw; ++w, ++jn, so += p.n_sub) {
            int v = -1;
            if (so < obs_limit) {
                if (so >= next_start) advance(so);
                v = obs_offset<R, OBS>(p, sedges, cur, so);
            }
            emit(v, cur.mode, jn);
        }
    }
    if (ADJ) adj->finish();
    if (have && p.trace) { // final state of the particle, the oracle's layout
        double *f = p.trace + 16 * i;
#pragma unroll
        for (int c = 0; c < 3; ++c) { f[c] = s.x[c]; f[3 + c] = s.d[c]; f[6 + c] = s.q[c]; }
        f[9] = s.mode; f[10] = s.alive; f[11] = cnt.scat - scat0; f[12] = cnt.bnd - bnd0;
        f[13] = s.s0; f[14] = s.s_death; f[15] = s.k;
    }
}

// Event-major schedule for event-heavy problems: one particle per thread, each event
// followed by the observations of the segment it ends.  A warp then runs as many
// iterations as its busiest lane has events (tens to hundreds, close to the mean), where
// the two-cursor batch would refill its rings a few lanes at a time.  Same events, same
// bins, same order of kill / boundary / scattering as run_batch.
template <typename R, int SINK, int OBS>
__device__ __forceinline__ void run_particle(const DevParams<R> &p, const R *sedges, unsigned *shist, int64_t i,
                                             Counters &cnt, bool &bad)
{
    const unsigned long long inc = 1ull << p.hist_shift;
    const uint64_t pid = (uint64_t)(p.pid0 + i);
    Part<R> s;
    init_particle(p, pid, s);
    // row j - 1 holds instant j; the particle's column (its place in the particle order)
    int32_t *optr = SINK == SINK_INDEX ? p.obs_idx + (p.iperm ? p.iperm[i] : i) : nullptr;
    // the index sink writes the rows of instants jr0..jr1 only (all by default)
    const int jr0 = p.obs_j0 > 1 ? p.obs_j0 : 1, jr1 = p.obs_j1 > 0 ? p.obs_j1 : p.n_obs;
    const unsigned scat0 = cnt.scat, bnd0 = cnt.bnd;
    int j = 1;
    for (;;) {
        const int e = next_event(s);
        const int lim = s.alive ? (e <= p.s_end ? e : p.s_end + 1) : s.s_death;
        Seg<R> g;
        seg_from(s, g);
        seg_prepare<R, OBS>(p, sedges, g);
        // observations strictly before the event; R2D: a radius |(x, y)| (2D, cylindrical),
        // whose zero third coordinate is left out (the same value: x2 = 0 adds nothing)
        auto observe = [&](auto r2d_tag) {
            constexpr bool R2D = decltype(r2d_tag)::value;
            for (; j <= p.n_obs && j * p.n_sub < lim; ++j) {
                const int v = R2D ? obs_offset_radius2(p, g, (R)(j * p.n_sub - g.s0))
                                  : obs_offset<R, OBS>(p, sedges, g, j * p.n_sub);
                if (SINK == SINK_INDEX) {
                    if (j >= jr0 && j <= jr1) {
                        *optr = v < 0 ? -1 : (v | (g.mode << 30));
                        if (v >= 0) cnt.obs++;
                    }
                    optr += p.obs_rows;
                } else if (v >= 0) {
                    const int64_t idx = (int64_t)j * p.time_stride + (g.mode ? p.mode_stride : 0) + v;
                    if (idx < p.hist_len) {
                        cnt.obs++;
                        if (SINK == SINK_SMEM) atomicAdd(shist + idx, 1u);
                        else atomicAdd(p.hist + idx, inc);
                    } else {
                        bad = true;
                    }
                }
            }
        };
        if (OBS == OBS_RADIAL && !p.radial_3d) observe(std::true_type{});
        else observe(std::false_type{});
        if (j > p.n_obs || !s.alive || e > p.s_end) break;
        process_event(p, pid, s, cnt);
        if ((int)s.k > p.max_events) { s.alive = 0; s.s_death = s.s0; bad = true; }
    }
    if (SINK == SINK_INDEX)
        for (; j <= p.n_obs; ++j, optr += p.obs_rows)
            if (j >= jr0 && j <= jr1) *optr = -1; // after death
    if (p.trace) { // final state of the particle, the oracle's layout
        double *f = p.trace + 16 * i;
#pragma unroll
        for (int c = 0; c < 3; ++c) { f[c] = s.x[c]; f[3 + c] = s.d[c]; f[6 + c] = s.q[c]; }
        f[9] = s.mode; f[10] = s.alive; f[11] = cnt.scat - scat0; f[12] = cnt.bnd - bnd0;
        f[13] = s.s0; f[14] = s.s_death; f[15] = s.k;
    }
}

// The transport kernel.  A warp takes 32 consecutive particles at a time and walks the
// observation instants in lockstep.  Each lane keeps two cursors on its particle's
// trajectory: the event state s (phase 1, runs ahead and pushes one segment per event
// into the lane's ring) and the observation cursor (phase 2, bins observation instants
// with the segment in force).  Phase 1 runs with every lane that has room in its ring
// taking part, so events execute converged; phase 2 then bins the number of
// observations that every live lane has covered, fully converged.
template <typename R, int SINK, int OBS>
__global__ void __launch_bounds__(Bounds<R, SINK>::threads, Bounds<R, SINK>::min_blocks) rt_transport(const DevParams<R> p)
{
    constexpr bool SMEM = SINK == SINK_SMEM;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    size_t off = (((size_t)p.n_edges * sizeof(R) + 15) / 16) * 16;
    unsigned *shist = reinterpret_cast<unsigned *>(smem_raw + off);
    if (SMEM) off += (((size_t)p.hist_len * 4 + 15) / 16) * 16;
    const int T = blockDim.x, C = p.ring_cap;
    Ring<R> ring;
    ring.cap = C;
    ring.stride = T;
    {
        R *r = reinterpret_cast<R *>(smem_raw + off);
        ring.x0 = r; ring.x1 = r + C * T; ring.x2 = r + 2 * C * T;
        ring.d0 = r + 3 * C * T; ring.d1 = r + 4 * C * T; ring.d2 = r + 5 * C * T;
        int *ri = reinterpret_cast<int *>(r + 6 * C * T);
        ring.s0 = ri; ring.mode = ri + C * T;
    }

    for (int k = threadIdx.x; k < p.n_edges; k += T) sedges[k] = p.edges[k];
    if (SMEM)
        for (int64_t k = threadIdx.x; k < p.hist_len; k += T) shist[k] = 0u;
    __syncthreads();

    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    const int64_t warps = ((int64_t)gridDim.x * T) >> 5;

    if (p.event_major) {
        for (int64_t i = (int64_t)blockIdx.x * T + threadIdx.x; i < p.n_particles; i += (int64_t)gridDim.x * T)
            run_particle<R, SINK, OBS>(p, sedges, shist, i, cnt, bad);
    } else {
        for (int64_t base = (((int64_t)blockIdx.x * T + threadIdx.x) >> 5) << 5; base < p.n_particles; base += warps * 32)
            run_batch<R, SINK, OBS>(p, sedges, shist, ring, base, p.n_particles, cnt, bad);
    }

    // counters: warp reduction, one global atomic per warp
    unsigned v[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, v[c]);
        if (lane == 0 && t) atomicAdd(p.stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(p.status, 1);
    if (SMEM) {
        __syncthreads();
        for (int64_t k = threadIdx.x; k < p.hist_len; k += T) {
            const unsigned c = shist[k];
            if (c) atomicAdd(p.hist + k, (unsigned long long)c << p.hist_shift);
        }
    }
}

// ---------------------------------------------------------------------------------
// Split schedule: the events of every particle first (rt_events), then the observations
// (rt_observe).  In the two-cursor batch a warp's phase 1 runs an event only for the lanes
// whose particle has one left, so rounds late in a batch run with a few lanes and the
// latency of the table lookups is exposed; rt_events gives each thread a stream of
// particles and starts new ones whenever enough lanes are free, so events run with most
// lanes active, and writes each particle's trajectory segments (prepared for the
// observation path) to global memory.  rt_observe then bins every observation instant of
// 32 particles per warp in lockstep with no event code at all.  Same events, same
// segments, same bins as rt_transport.
// ---------------------------------------------------------------------------------

// A prepared segment in global memory: u = A (cartesian), x (radius-only, general);
// v = B (cartesian, radius-only) or d (general); the start sub-step with the mode in bit
// 30, and the direction offset.  32 bytes in FP32 (two 16-byte vectors), 64 in FP64.
// Records are stored evict-first (st.global.cs): they are read back only by a later kernel,
// after gigabytes of other traffic, and the L2 is better spent on the tables that every
// event looks up (rt_events on the 3D elastic workload: 2.37 -> 2.23 ms, with the clear
// stored the same way)
__device__ __forceinline__ void rec_store(float *r, const float u[3], const float v[3], int sm, int doff)
{
    float4 *q = reinterpret_cast<float4 *>(r);
    __stcs(q, make_float4(u[0], u[1], u[2], v[0]));
    __stcs(q + 1, make_float4(v[1], v[2], __int_as_float(sm), __int_as_float(doff)));
}
__device__ __forceinline__ void rec_store(double *r, const double u[3], const double v[3], int sm, int doff)
{
    double2 *q = reinterpret_cast<double2 *>(r);
    __stcs(q, make_double2(u[0], u[1]));
    __stcs(q + 1, make_double2(u[2], v[0]));
    __stcs(q + 2, make_double2(v[1], v[2]));
    __stcs(q + 3, make_double2(__longlong_as_double((long long)(((unsigned long long)(unsigned)doff << 32) | (unsigned)sm)), 0.0));
}
__device__ __forceinline__ void rec_load(const float *r, float u[3], float v[3], int &sm, int &doff)
{
    const float4 *q = reinterpret_cast<const float4 *>(r);
    const float4 a = __ldg(q), b = __ldg(q + 1);
    u[0] = a.x; u[1] = a.y; u[2] = a.z; v[0] = a.w;
    v[1] = b.x; v[2] = b.y; sm = __float_as_int(b.z); doff = __float_as_int(b.w);
}
__device__ __forceinline__ void rec_load(const double *r, double u[3], double v[3], int &sm, int &doff)
{
    const double2 *q = reinterpret_cast<const double2 *>(r);
    const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
    u[0] = a.x; u[1] = a.y; u[2] = b.x; v[0] = b.y; v[1] = c.x; v[2] = c.y;
    const unsigned long long w = (unsigned long long)__double_as_longlong(d.x);
    sm = (int)(unsigned)(w & 0xffffffffull);
    doff = (int)(unsigned)(w >> 32);
}
constexpr int kRecWords = 8; // R values per record

template <typename R, int OBS> __device__ __forceinline__ void rec_put(R *r, const Seg<R> &g)
{
    const R *u = OBS == OBS_CART ? g.A : g.x;
    const R *v = OBS == OBS_GENERAL ? g.d : g.B;
    rec_store(r, u, v, g.s0 | (g.mode << 30), g.doff);
}
template <typename R, int OBS> __device__ __forceinline__ void rec_get(const R *r, Seg<R> &g)
{
    R *u = OBS == OBS_CART ? g.A : g.x;
    R *v = OBS == OBS_GENERAL ? g.d : g.B;
    int sm;
    rec_load(r, u, v, sm, g.doff);
    g.s0 = sm & 0x3fffffff;
    g.mode = sm >> 30;
}

// A segment as rt_observe wants it: on the index path the mode sits in bit 30 of the
// direction offset; on the FP32 cartesian path the offsets lose a negative zero, a
// direction outside the grid becomes an infinite first offset, and the direction offset
// carries the 2^23 bias of the three bin patterns (see obs_offset_cart32).
template <typename R, int OBS> __device__ __forceinline__ void rec_put_seg(const DevParams<R> &p, R *r, Seg<R> g)
{
    if (p.sink == SINK_INDEX && g.doff >= 0) g.doff |= g.mode << 30;
    if (sizeof(R) == 4 && OBS == OBS_CART) {
#pragma unroll
        for (int a = 0; a < 3; ++a) g.A[a] = m_add(g.A[a], (R)0);
        if (g.doff < 0) g.A[0] = (R)INFINITY;
        g.doff = (int)((unsigned)g.doff - (unsigned)p.cart_bias);
    }
    rec_put<R, OBS>(r, g);
}

// The records after a particle's last segment: an end record at its death sub-step (it
// bins nothing: direction offset -1, infinite first offset), then a record that never
// comes into force (start 2^30 - 1, beyond every observation sub-step).  A particle that
// lives to the end gets the second only.
constexpr int kNeverStart = 0x3fffffff;
template <typename R> __device__ __forceinline__ void rec_put_end(R *r, int s0)
{
    const R u[3] = {(R)INFINITY, (R)0, (R)0}, v[3] = {(R)0, (R)0, (R)0};
    rec_store(r, u, v, s0, -1);
}

// The direction cell of a starting direction for the particle order: each component in 8
// slabs of [-1, 1] (kOrderCells = 512 cells, about 200 of them on the unit sphere).
template <typename R> __device__ __forceinline__ int32_t dir_cell(const R d[3])
{
    int q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) q[a] = min(7, max(0, (int)((d[a] + (R)1) * (R)4)));
    return (q[0] * 8 + q[1]) * 8 + q[2];
}

// lanes of a warp that start new particles together in rt_events (16 measured 3 % faster
// than 8 and 4 on the 3D elastic workload: fewer, fuller start rounds)
constexpr int kEventStartLanes = 16;

template <typename R, int OBS>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 2) rt_events(const DevParams<R> p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    for (int k = threadIdx.x; k < p.n_edges; k += blockDim.x) sedges[k] = p.edges[k];
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int K = p.seg_cap;
    R *segs = static_cast<R *>(p.segs);
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u}, c0 = cnt;
    bool bad = false;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool have = false;
    int nseg = 0;
    Part<R> s;
    Seg<R> g;
    // the histogram clear, fused: each thread zeroes its share in 16-byte evict-first stores,
    // a few per iteration (the event work is bound by instruction issue, the stores by HBM)
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t cw = t0;
    const int64_t cn = p.clear_words >> 1;
    ulonglong2 *cl = reinterpret_cast<ulonglong2 *>(p.clear);
    if (t0 == 0 && (p.clear_words & 1)) p.clear[p.clear_words - 1] = 0ull;
    for (;;) {
#pragma unroll 1
        for (int u = 0; u < 8 && cw < cn; ++u, cw += stride) __stcs(cl + cw, make_ulonglong2(0ull, 0ull));
        const bool idle = !have && i < p.n_particles;
        const unsigned idle_mask = __ballot_sync(full, idle), busy_mask = __ballot_sync(full, have);
        if (!(idle_mask | busy_mask)) break;
        // free lanes start their next particles together, once enough of them are free
        if (idle && (__popc(idle_mask) >= kEventStartLanes || !busy_mask)) {
            init_particle(p, (uint64_t)(p.pid0 + i), s);
            if (p.okey) p.okey[i] = dir_cell(s.d);
            c0 = cnt;
            seg_from(s, g);
            seg_prepare<R, OBS>(p, sedges, g);
            rec_put_seg<R, OBS>(p, segs + (size_t)i * K * kRecWords, g);
            if (p.seg_th) static_cast<R *>(p.seg_th)[(size_t)i * K] = (R)-1;
            nseg = 1;
            have = true;
        }
        if (!have) continue;
        int done = 0; // 1: the particle's run is over, 2: its segments overflow seg_cap - 2
        if (next_event(s) > p.s_end) {
            done = 1;
        } else {
            const int kind = process_event(p, (uint64_t)(p.pid0 + i), s, cnt);
            if ((int)s.k > p.max_events) { s.alive = 0; s.s_death = s.s0; bad = true; }
            if (!s.alive) {
                done = 1;
            } else if (nseg < K - 2) { // two records stay free for the end records
                seg_from(s, g);
                seg_prepare<R, OBS>(p, sedges, g);
                rec_put_seg<R, OBS>(p, segs + ((size_t)i * K + nseg) * kRecWords, g);
                if (p.seg_th) static_cast<R *>(p.seg_th)[(size_t)i * K + nseg] = kind == 0 ? s.th : (R)-1;
                ++nseg;
            } else {
                done = 2;
            }
        }
        if (done) {
            R *r = segs + (size_t)i * K * kRecWords;
            if (done == 1) {
                if (!s.alive) {
                    if (p.seg_th) static_cast<R *>(p.seg_th)[(size_t)i * K + nseg] = (R)-1;
                    rec_put_end(r + (size_t)nseg++ * kRecWords, s.s_death);
                }
                rec_put_end(r + (size_t)nseg * kRecWords, kNeverStart);
                if (p.trace) { // final state of the particle, the oracle's layout
                    double *f = p.trace + 16 * i;
#pragma unroll
                    for (int c = 0; c < 3; ++c) { f[c] = s.x[c]; f[3 + c] = s.d[c]; f[6 + c] = s.q[c]; }
                    f[9] = s.mode; f[10] = s.alive; f[11] = cnt.scat - c0.scat; f[12] = cnt.bnd - c0.bnd;
                    f[13] = s.s0; f[14] = s.s_death; f[15] = s.k;
                }
            } else { // rerun whole by rt_transport_list: its events are not counted here
                rec_put_end(r, 0); // nothing binned from sub-step 0
                rec_put_end(r + kRecWords, kNeverStart);
                cnt = c0;
                p.ovf_list[atomicAdd(p.ovf_count, 1u)] = (int32_t)i;
            }
            have = false;
            i += stride;
        }
    }
    for (; cw < cn; cw += stride) __stcs(cl + cw, make_ulonglong2(0ull, 0ull));
    unsigned v[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, v[c]);
        if (lane == 0 && t) atomicAdd(p.stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(p.status, 1);
}

// Observations of the particles rt_events traced: a warp takes 32 consecutive particles
// and walks the observation instants in lockstep, each lane on its own segment list (the
// segment after the one in force is loaded ahead, so a segment change finds its data
// in registers; loading the start of the one after that as well, so that the next bound
// needs no fresh load either, measured 5 % slower on the 3D elastic workload).
// Per instant a lane does one compare for a segment change or its end (rare, and then
// the offset from the segment start is set afresh), the binning, and one store; the
// offset is carried as a float counter while it stays an exact integer (below 2^24).
template <typename R, int SINK, int OBS>
__device__ __forceinline__ void observe_batch(const DevParams<R> &p, const R *sedges, unsigned *shist, int64_t base,
                                              Counters &cnt, bool &bad, const R *segs_in = nullptr, int64_t n_in = -1)
{
    // segs_in / n_in: another record array and particle count (a batch block's work item)
    constexpr bool SMEM = SINK == SINK_SMEM;
    constexpr bool INDEX = SINK == SINK_INDEX;
    const int lane = threadIdx.x & 31;
    const unsigned long long inc = 1ull << p.hist_shift;
    const int64_t col = base + lane; // the lane's column of the index array
    const bool have = col < (n_in >= 0 ? n_in : p.n_particles);
    const int64_t i = have && p.perm ? (int64_t)__ldg(p.perm + col) : col; // its particle
    // record k (in cur) is in force and record k + 1 waits in nxt; every particle's list
    // ends in records that bin nothing and never end (rec_put_end), so a change of segment
    // needs no count or limit checks
    const R *rec = (segs_in ? segs_in : static_cast<const R *>(p.segs)) + (size_t)(have ? i : 0) * p.seg_cap * kRecWords;
    constexpr bool C32 = sizeof(R) == 4 && OBS == OBS_CART;
    constexpr bool R64 = sizeof(R) == 8 && (OBS == OBS_RADIAL || OBS == OBS_CART); // FP64: FP32 estimates
    Seg<R> cur, nxt;
    SegF cf; // the segment in force in FP32 (R64)
    int k = 1, next_start = kNeverStart;
    if (have) {
        rec_get<R, OBS>(rec, cur);
        rec_get<R, OBS>(rec + kRecWords, nxt);
        next_start = nxt.s0;
    } else {
        cur.s0 = 0; cur.mode = 0; cur.doff = -1;
        cur.A[0] = (R)INFINITY; cur.A[1] = cur.A[2] = cur.B[0] = cur.B[1] = cur.B[2] = (R)0;
    }
    // the offset from the segment start is carried as a float counter while it stays an
    // exact integer (below 2^24), else converted afresh each instant
    const bool count_dl = sizeof(R) == 8 || p.s_end < (1 << 24);
    auto walk = [&](auto count_tag, auto est_tag) {
        constexpr bool CDL = decltype(count_tag)::value;
        constexpr bool EST = R64 && decltype(est_tag)::value;
        if (EST) segf_from<OBS>(cur, cf);
        // instants j0..j1 (all by default); the first pass of the loop moves the cursor to
        // the segment in force at j0
        const int j0 = p.obs_j0 > 1 ? p.obs_j0 : 1;
        const int s_last = (p.obs_j1 > 0 ? p.obs_j1 : p.n_obs) * p.n_sub;
        // FP64 with the FP32 estimates carries the offset as a float (an exact integer:
        // sub-steps stay below 2^24 there), so no FP64 instruction runs per instant
        using D = typename std::conditional<EST, float, R>::type;
        const D dstep = (D)p.n_sub;
        int so = j0 * p.n_sub;
        D dl = (D)(so - cur.s0);
        // every lane of a warp owns a column of the index array (rows are padded to 32
        // particles), so lanes past the last particle store their -1 there unconditionally
        int32_t *optr = INDEX ? p.obs_idx + (int64_t)(j0 - 1) * p.obs_rows + col : nullptr;
        int64_t toff = (int64_t)j0 * p.time_stride; // slice offset of instant j (shared and global sinks)
#pragma unroll 1
        for (; so <= s_last; so += p.n_sub) {
            if (so >= next_start) { // the next segment comes into force; load the one after it
                do {
                    cur = nxt;
                    ++k;
                    rec_get<R, OBS>(rec + (size_t)k * kRecWords, nxt);
                    next_start = nxt.s0;
                } while (so >= next_start);
                if (EST) segf_from<OBS>(cur, cf);
                dl = (D)(so - cur.s0);
            } else if (!CDL) {
                dl = (D)(so - cur.s0);
            }
            int v;
            if constexpr (C32) v = obs_offset_cart32(p, cur, dl, cur.doff);
            else if constexpr (EST && OBS == OBS_RADIAL) v = obs_offset_radial64(p, sedges, cur, cf, dl);
            else if constexpr (EST) v = obs_offset_cart64(p, sedges, cur, cf, dl);
            else v = obs_offset_dl<R, OBS>(p, sedges, cur, dl);
            if (CDL) dl += dstep;
            if (INDEX) {
                __stcs(optr, v); // evict-first: the fold reads it back from DRAM (4.15 -> 4.09 ms on the 3D elastic workload)
                optr += p.obs_rows;
                cnt.obs += v >= 0 ? 1u : 0u;
            } else {
                if (v >= 0) {
                    const int64_t idx = toff + (cur.mode ? p.mode_stride : 0) + v;
                    if (idx < p.hist_len) {
                        cnt.obs++;
                        if (SMEM) atomicAdd(shist + idx, 1u);
                        else atomicAdd(p.hist + idx, inc);
                    } else {
                        bad = true;
                    }
                }
                toff += p.time_stride;
            }
        }
    };
    if (R64 && p.bin32) walk(std::true_type{}, std::true_type{}); // FP64 counts dl exactly
    else if (count_dl) walk(std::true_type{}, std::false_type{});
    else walk(std::false_type{}, std::false_type{});
}

// the shared-memory sink holds one block per SM (the histogram fills the shared memory):
// FP32 takes 1024 threads so that 32 warps hide the latencies
template <typename R, int SINK> struct ObserveBounds {
    static constexpr int threads = SINK == SINK_SMEM ? (sizeof(R) == 4 ? 1024 : 512) : 256;
    static constexpr int min_blocks = SINK == SINK_SMEM ? 1 : (sizeof(R) == 4 ? 4 : 2);
};

template <typename R, int SINK, int OBS>
__global__ void __launch_bounds__(ObserveBounds<R, SINK>::threads, ObserveBounds<R, SINK>::min_blocks)
    rt_observe(const DevParams<R> p)
{
    constexpr bool SMEM = SINK == SINK_SMEM;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    const size_t off = (((size_t)p.n_edges * sizeof(R) + 15) / 16) * 16;
    unsigned *shist = reinterpret_cast<unsigned *>(smem_raw + off);
    const int T = blockDim.x;
    for (int k = threadIdx.x; k < p.n_edges; k += T) sedges[k] = p.edges[k];
    if (SMEM)
        for (int64_t k = threadIdx.x; k < p.hist_len; k += T) shist[k] = 0u;
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    const int64_t warps = ((int64_t)gridDim.x * T) >> 5;
    for (int64_t base = (((int64_t)blockIdx.x * T + threadIdx.x) >> 5) << 5; base < p.n_particles; base += warps * 32)
        observe_batch<R, SINK, OBS>(p, sedges, shist, base, cnt, bad);
    const unsigned t = __reduce_add_sync(full, cnt.obs);
    if (lane == 0 && t) atomicAdd(p.stats + 4, (unsigned long long)t);
    if (bad) atomicExch(p.status, 1);
    if (SMEM) {
        __syncthreads();
        for (int64_t k = threadIdx.x; k < p.hist_len; k += T) {
            const unsigned c = shist[k];
            if (c) atomicAdd(p.hist + k, (unsigned long long)c << p.hist_shift);
        }
    }
}

// The particles whose segments overflowed seg_cap in rt_events, rerun whole one per
// thread (the event-major schedule).  On the index path the rerun writes the particle's
// rows of the index array (rt_observe left them at -1), so the fold that follows sees
// every particle alike; otherwise its observations go to the histogram by 64-bit global
// atomics.  The list length is read on the device, so the launch needs no host
// synchronisation.
template <typename R, int SINK, int OBS>
__global__ void __launch_bounds__(256) rt_transport_list(const DevParams<R> p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    for (int k = threadIdx.x; k < p.n_edges; k += blockDim.x) sedges[k] = p.edges[k];
    __syncthreads();
    const unsigned n = *reinterpret_cast<volatile const uint32_t *>(p.ovf_count);
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        run_particle<R, SINK, OBS>(p, sedges, nullptr, p.ovf_list[t], cnt, bad);
    const unsigned full = 0xffffffffu;
    if (p.obs_j0 > 1) cnt.scat = cnt.bnd = cnt.kill = cnt.absorb = cnt.conv = 0u; // counted with the first range
    unsigned v[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned sum = __reduce_add_sync(full, v[c]);
        if ((threadIdx.x & 31) == 0 && sum) atomicAdd(p.stats + c, (unsigned long long)sum);
    }
    if (bad) atomicExch(p.status, 1);
}

// Batched transport: many independent problems (instances) sharing one observation
// grid, in one persistent launch.  Blocks pull (instance, particle range) work items,
// largest expected cost first, from a global counter; the instance's parameters are
// copied into shared memory and its histogram accumulates in the block's shared-memory
// copy, flushed to the instance's output whenever the block moves to another instance.
template <typename R, int OBS>
__global__ void __launch_bounds__(512, 1) rt_transport_batch(const BatchArgs<R> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ DevParams<R> sp;
    __shared__ int s_item;
    R *sedges = reinterpret_cast<R *>(smem_raw);
    size_t off = (((size_t)a.n_edges * sizeof(R) + 15) / 16) * 16;
    unsigned *shist = reinterpret_cast<unsigned *>(smem_raw + off);
    off += (((size_t)a.hist_len * 4 + 15) / 16) * 16;
    const int T = blockDim.x, C = a.ring_cap;
    Ring<R> ring;
    ring.cap = C;
    ring.stride = T;
    {
        R *r = reinterpret_cast<R *>(smem_raw + off);
        ring.x0 = r; ring.x1 = r + C * T; ring.x2 = r + 2 * C * T;
        ring.d0 = r + 3 * C * T; ring.d1 = r + 4 * C * T; ring.d2 = r + 5 * C * T;
        int *ri = reinterpret_cast<int *>(r + 6 * C * T);
        ring.s0 = ri; ring.mode = ri + C * T;
    }
    for (int k = threadIdx.x; k < a.n_edges; k += T) sedges[k] = a.edges[k];
    for (int64_t k = threadIdx.x; k < a.hist_len; k += T) shist[k] = 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = T >> 5;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    int cur = -1; // instance held in shared memory (the same in every thread)
    auto flush = [&](int inst) {
        unsigned long long *h = a.hists + (int64_t)inst * a.hist_len;
        const int sh = sp.hist_shift;
        for (int64_t k = threadIdx.x; k < a.hist_len; k += T) {
            const unsigned c = shist[k];
            if (c) {
                atomicAdd(h + k, (unsigned long long)c << sh);
                shist[k] = 0u;
            }
        }
    };
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
        const BatchItem bi = a.items[it];
        if (bi.inst != cur) {
            if (cur >= 0) flush(cur);
            __syncthreads();
            const uint32_t *src = reinterpret_cast<const uint32_t *>(a.params + bi.inst);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
            for (int k = threadIdx.x; k < (int)(sizeof(DevParams<R>) / 4); k += T) dst[k] = src[k];
            cur = bi.inst;
            __syncthreads();
        }
        const int64_t end = bi.first + bi.count;
        if (sp.event_major) {
            for (int64_t i = bi.first + threadIdx.x; i < end; i += T)
                run_particle<R, SINK_SMEM, OBS>(sp, sedges, shist, i, cnt, bad);
        } else {
            for (int64_t base = bi.first + 32 * warp; base < end; base += 32 * nwarps)
                run_batch<R, SINK_SMEM, OBS>(sp, sedges, shist, ring, base, end, cnt, bad);
        }
    }
    if (cur >= 0) flush(cur);
    const unsigned full = 0xffffffffu;
    unsigned v[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, v[c]);
        if (lane == 0 && t) atomicAdd(a.stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(a.status, 1);
}

// Batched transport of the event-heavy instances: the same work-item loop, one particle
// per thread (event-major).  SHIST: observations go to the block's shared-memory copy of
// the instance's histogram, flushed when the block moves to another instance (512 threads,
// one block per SM); else 64-bit atomics into the instance's histogram in device memory
// (no shared-memory copy, so three blocks fit on an SM).
template <typename R, bool SHIST> struct BatchEmBounds {
    static constexpr int threads = SHIST ? 512 : 256;
    static constexpr int min_blocks = SHIST ? 1 : (sizeof(R) == 4 ? 3 : 2);
};

template <typename R, int OBS, bool SHIST>
__global__ void __launch_bounds__(BatchEmBounds<R, SHIST>::threads, BatchEmBounds<R, SHIST>::min_blocks)
    rt_transport_batch_em(const BatchArgs<R> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ DevParams<R> sp;
    __shared__ int s_item;
    R *sedges = reinterpret_cast<R *>(smem_raw);
    unsigned *shist = SHIST ? reinterpret_cast<unsigned *>(smem_raw + (((size_t)a.n_edges * sizeof(R) + 15) / 16) * 16)
                            : nullptr;
    const int T = blockDim.x;
    for (int k = threadIdx.x; k < a.n_edges; k += T) sedges[k] = a.edges[k];
    if (SHIST)
        for (int64_t k = threadIdx.x; k < a.hist_len; k += T) shist[k] = 0u;
    const int lane = threadIdx.x & 31;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    int cur = -1;
    auto flush = [&](int inst) {
        unsigned long long *h = a.hists + (int64_t)inst * a.hist_len;
        const int sh = sp.hist_shift;
        for (int64_t k = threadIdx.x; k < a.hist_len; k += T) {
            const unsigned c = shist[k];
            if (c) {
                atomicAdd(h + k, (unsigned long long)c << sh);
                shist[k] = 0u;
            }
        }
    };
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
        const BatchItem bi = a.items[it];
        if (bi.inst != cur) {
            if (SHIST && cur >= 0) flush(cur);
            __syncthreads();
            const uint32_t *src = reinterpret_cast<const uint32_t *>(a.params + bi.inst);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
            for (int k = threadIdx.x; k < (int)(sizeof(DevParams<R>) / 4); k += T) dst[k] = src[k];
            __syncthreads();
            if (threadIdx.x == 0) sp.hist = a.hists + (int64_t)bi.inst * a.hist_len;
            cur = bi.inst;
            __syncthreads();
        }
        const int64_t end = bi.first + bi.count;
        for (int64_t i = bi.first + threadIdx.x; i < end; i += T)
            run_particle<R, SHIST ? SINK_SMEM : SINK_GLOBAL, OBS>(sp, sedges, shist, i, cnt, bad);
    }
    if (SHIST && cur >= 0) flush(cur);
    const unsigned full = 0xffffffffu;
    unsigned v[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, v[c]);
        if (lane == 0 && t) atomicAdd(a.stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(a.status, 1);
}

// Batched transport of the lockstep instances on the split schedule, inside one persistent
// launch: for each work item a block first runs its particles' events (a thread a particle
// at a time, new particles started by 16 lanes together as in rt_events), writing the
// prepared segment records to the block's scratch; after a barrier its warps walk the
// observation instants of 32 particles each in lockstep (observe_batch) into the
// instance's shared-memory histogram.  A particle with more segments than the instance's
// seg_cap - 2 gets end records and is run whole at once (run_particle).
template <typename R, int OBS>
__global__ void __launch_bounds__(kBatchSplitThreads, 1) rt_transport_batch_split(const BatchArgs<R> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ DevParams<R> sp;
    __shared__ int s_item;
    R *sedges = reinterpret_cast<R *>(smem_raw);
    const size_t off = (((size_t)a.n_edges * sizeof(R) + 15) / 16) * 16;
    unsigned *shist = reinterpret_cast<unsigned *>(smem_raw + off);
    R *scratch = static_cast<R *>(a.scratch) + (size_t)blockIdx.x * a.scratch_stride;
    const int T = blockDim.x;
    for (int k = threadIdx.x; k < a.n_edges; k += T) sedges[k] = a.edges[k];
    for (int64_t k = threadIdx.x; k < a.hist_len; k += T) shist[k] = 0u;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = T >> 5;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    int cur = -1; // instance held in shared memory
    auto flush = [&](int inst) {
        unsigned long long *h = a.hists + (int64_t)inst * a.hist_len;
        const int sh = sp.hist_shift;
        for (int64_t k = threadIdx.x; k < a.hist_len; k += T) {
            const unsigned c = shist[k];
            if (c) {
                atomicAdd(h + k, (unsigned long long)c << sh);
                shist[k] = 0u;
            }
        }
    };
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
        const BatchItem bi = a.items[it];
        if (bi.inst != cur) {
            if (cur >= 0) flush(cur);
            __syncthreads();
            const uint32_t *src = reinterpret_cast<const uint32_t *>(a.params + bi.inst);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
            for (int k = threadIdx.x; k < (int)(sizeof(DevParams<R>) / 4); k += T) dst[k] = src[k];
            cur = bi.inst;
            __syncthreads();
        }
        const int K = sp.seg_cap;
        const int64_t n = bi.count;
        // ---- events: local particle li (global bi.first + li) into scratch[li][K][8]
        {
            int64_t li = threadIdx.x;
            bool have = false;
            int nseg = 0;
            Part<R> s;
            Seg<R> g;
            Counters c0 = cnt;
            for (;;) {
                const bool idle = !have && li < n;
                const unsigned idle_mask = __ballot_sync(full, idle), busy_mask = __ballot_sync(full, have);
                if (!(idle_mask | busy_mask)) break;
                const uint64_t pid = (uint64_t)(sp.pid0 + bi.first + li);
                if (idle && (__popc(idle_mask) >= kEventStartLanes || !busy_mask)) {
                    init_particle(sp, pid, s);
                    c0 = cnt;
                    seg_from(s, g);
                    seg_prepare<R, OBS>(sp, sedges, g);
                    rec_put_seg<R, OBS>(sp, scratch + (size_t)li * K * kRecWords, g);
                    nseg = 1;
                    have = true;
                }
                if (!have) continue;
                int done = 0; // 1: the particle's run is over, 2: its segments overflow
                if (next_event(s) > sp.s_end) {
                    done = 1;
                } else {
                    process_event(sp, pid, s, cnt);
                    if ((int)s.k > sp.max_events) { s.alive = 0; s.s_death = s.s0; bad = true; }
                    if (!s.alive) {
                        done = 1;
                    } else if (nseg < K - 2) {
                        seg_from(s, g);
                        seg_prepare<R, OBS>(sp, sedges, g);
                        rec_put_seg<R, OBS>(sp, scratch + ((size_t)li * K + nseg) * kRecWords, g);
                        ++nseg;
                    } else {
                        done = 2;
                    }
                }
                if (done) {
                    R *r = scratch + (size_t)li * K * kRecWords;
                    if (done == 1) {
                        if (!s.alive) rec_put_end(r + (size_t)nseg++ * kRecWords, s.s_death);
                        rec_put_end(r + (size_t)nseg * kRecWords, kNeverStart);
                    } else { // run whole now; its list bins nothing
                        rec_put_end(r, 0);
                        rec_put_end(r + kRecWords, kNeverStart);
                        cnt = c0;
                        run_particle<R, SINK_SMEM, OBS>(sp, sedges, shist, bi.first + li, cnt, bad);
                    }
                    have = false;
                    li += T;
                }
            }
        }
        __syncthreads();
        // ---- observations: 32 particles per warp in lockstep
        for (int64_t base = 32 * warp; base < n; base += 32 * nwarps)
            observe_batch<R, SINK_SMEM, OBS>(sp, sedges, shist, base, cnt, bad, scratch, n);
    }
    if (cur >= 0) flush(cur);
    unsigned v[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, v[c]);
        if (lane == 0 && t) atomicAdd(a.stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(a.status, 1);
}

template <typename R, int SINK, int OBS> void *kernel_ptr() { return (void *)rt_transport<R, SINK, OBS>; }

template <typename R, int SINK> void *pick_obs(int obs)
{
    return obs == OBS_CART ? kernel_ptr<R, SINK, OBS_CART>()
                           : (obs == OBS_RADIAL ? kernel_ptr<R, SINK, OBS_RADIAL>() : kernel_ptr<R, SINK, OBS_GENERAL>());
}

// Score-function adjoint: replays each particle of rt_transport from its Philox key
// (one particle per thread; the path is recomputed, never stored) and accumulates, in
// FP64, adjoint[bin] * score over every observation instant.  Between two events the
// score is A + b_obs * j, so a segment only sums adjoint[bin] and j * adjoint[bin]; the
// scattering that ends it adds d log sigma(theta) / dp (table lookup) + a_inc to A.
template <typename R, int OBS>
__device__ __forceinline__ void adjoint_particle(const DevParams<R> &p, const AdjointArgs &a, const R *sedges,
                                                 const R *wts, const R *dls, int64_t i, double (&g)[RTMC_MAX_PARAMS],
                                                 Counters &cnt, bool &bad)
{
    const int np = a.n_params;
    const R tmax = (R)(a.n_theta - 1);
    const uint64_t pid = (uint64_t)(p.pid0 + i);
    Part<R> s;
    init_particle(p, pid, s);
    // this particle's score (scattering part) and sum of A * segment weights, in the
    // transport's precision; FP64 once per particle
    R A[RTMC_MAX_PARAMS], G[RTMC_MAX_PARAMS];
#pragma unroll
    for (int q = 0; q < RTMC_MAX_PARAMS; ++q) { A[q] = (R)0; G[q] = (R)0; }
    R SAJ = (R)0;
    int j = 1;
    for (;;) {
        const int e = next_event(s);
        const int lim = e <= p.s_end ? e : p.s_end + 1;
        Seg<R> sg;
        seg_from(s, sg);
        seg_prepare<R, OBS>(p, sedges, sg);
        R sa = (R)0, saj = (R)0;
        for (; j <= p.n_obs && j * p.n_sub < lim; ++j) { // observations strictly before the event
            const int v = obs_offset<R, OBS>(p, sedges, sg, j * p.n_sub);
            if (v < 0) continue;
            const int64_t idx = (int64_t)j * p.time_stride + (sg.mode ? p.mode_stride : 0) + v;
            if (idx >= p.hist_len) { bad = true; continue; }
            const R w = __ldg(wts + idx);
            sa += w;
            saj += w * (R)j;
            cnt.obs++;
        }
#pragma unroll
        for (int q = 0; q < RTMC_MAX_PARAMS; ++q)
            if (q < np) G[q] += A[q] * sa;
        SAJ += saj;
        if (j > p.n_obs || e > p.s_end) break;
        const int kind = process_event(p, pid, s, cnt);
        if ((int)s.k > p.max_events) { bad = true; break; }
        if (!s.alive) break;
        if (kind == 0) {
            R f = s.th < (R)0 ? (R)0 : (s.th > (R)1 ? (R)1 : s.th);
            f *= tmax;
            int k = (int)f;
            k = k > a.n_theta - 2 ? a.n_theta - 2 : k;
            const R w = f - (R)k;
#pragma unroll
            for (int q = 0; q < RTMC_MAX_PARAMS; ++q) {
                if (q < np) {
                    const R *t = dls + (size_t)q * a.n_theta + k;
                    const R t0 = __ldg(t), t1 = __ldg(t + 1);
                    A[q] += t0 + w * (t1 - t0) + (sizeof(R) == 4 ? (R)a.a_inc_f[q] : (R)a.a_inc[q]);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < RTMC_MAX_PARAMS; ++q)
        if (q < np) g[q] += (double)G[q] + a.b_obs[q] * (double)SAJ;
}

// A block's gradient sums in a fixed order (warp shuffles, then warp 0 over the warps) to
// out[blockIdx.x][n_params], and its counters and status; red holds a row per warp.
template <int NP>
__device__ __forceinline__ void adjoint_block_sums(const unsigned long long *, unsigned long long *stats, int32_t *status,
                                                   int np, double (&g)[NP], double (*red)[NP], double *out,
                                                   const Counters &cnt, bool bad)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        double v = g[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < NP && threadIdx.x < np) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
        out[(size_t)blockIdx.x * np + threadIdx.x] = v;
    }
    const unsigned full = 0xffffffffu;
    unsigned cv[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, cv[c]);
        if (lane == 0 && t) atomicAdd(stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(status, 1);
}

// Block sums go to a.partial in a fixed order, so the result is reproducible.
template <typename R, int OBS>
__global__ void __launch_bounds__(kAdjointThreads, sizeof(R) == 4 ? 3 : 2) rt_adjoint(const DevParams<R> p, const AdjointArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    __shared__ double red[kAdjointThreads / 32][RTMC_MAX_PARAMS];
    for (int k = threadIdx.x; k < p.n_edges; k += blockDim.x) sedges[k] = p.edges[k];
    __syncthreads();
    const R *wts = static_cast<const R *>(a.adjoint);
    const R *dls = sizeof(R) == 4 ? reinterpret_cast<const R *>(a.dlogsigma_f) : reinterpret_cast<const R *>(a.dlogsigma);
    double g[RTMC_MAX_PARAMS];
#pragma unroll
    for (int q = 0; q < RTMC_MAX_PARAMS; ++q) g[q] = 0.0;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_particles; i += stride)
        adjoint_particle<R, OBS>(p, a, sedges, wts, dls, i, g, cnt, bad);
    adjoint_block_sums<RTMC_MAX_PARAMS>(p.stats, p.stats, p.status, a.n_params, g, red, a.partial, cnt, bad);
}

// The split replay's particles whose segments overflowed, rerun whole one per thread;
// their block sums go to a.partial_list.  The list length is read on the device.
template <typename R, int OBS>
__global__ void __launch_bounds__(kAdjointThreads, sizeof(R) == 4 ? 3 : 2) rt_adjoint_list(const DevParams<R> p, const AdjointArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    __shared__ double red[kAdjointThreads / 32][RTMC_MAX_PARAMS];
    for (int k = threadIdx.x; k < p.n_edges; k += blockDim.x) sedges[k] = p.edges[k];
    __syncthreads();
    const R *wts = static_cast<const R *>(a.adjoint);
    const R *dls = sizeof(R) == 4 ? reinterpret_cast<const R *>(a.dlogsigma_f) : reinterpret_cast<const R *>(a.dlogsigma);
    double g[RTMC_MAX_PARAMS];
#pragma unroll
    for (int q = 0; q < RTMC_MAX_PARAMS; ++q) g[q] = 0.0;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    const unsigned n = *reinterpret_cast<volatile const uint32_t *>(p.ovf_count);
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        adjoint_particle<R, OBS>(p, a, sedges, wts, dls, p.ovf_list[t], g, cnt, bad);
    adjoint_block_sums<RTMC_MAX_PARAMS>(p.stats, p.stats, p.status, a.n_params, g, red, a.partial_list, cnt, bad);
}

// Split replay, observation side: rt_events has written every particle's segment records
// and the scattering angle that starts each segment (seg_th); like rt_observe, a warp walks
// the observation instants of 32 particles in lockstep, and instead of binning each lane
// sums the adjoint weights of its bins (AdjLane: the score of the segment in force is
// A + b_obs j, and a segment that a scattering starts adds d log sigma(theta) + a_inc to
// A).  Overflowing particles contribute nothing here (their lists hold only end records)
// and are replayed by rt_adjoint_list.
template <typename R, int OBS>
__global__ void __launch_bounds__(kAdjointThreads, sizeof(R) == 4 ? 4 : 2) rt_observe_adj(const DevParams<R> p, const AdjointArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    __shared__ double red[kAdjointThreads / 32][kAdjRingParams];
    for (int k = threadIdx.x; k < p.n_edges; k += blockDim.x) sedges[k] = p.edges[k];
    __syncthreads();
    constexpr bool C32 = sizeof(R) == 4 && OBS == OBS_CART;
    AdjLane<R> adj;
    adj.a = &a;
    adj.wts = static_cast<const R *>(a.adjoint);
    adj.dls = sizeof(R) == 4 ? reinterpret_cast<const R *>(a.dlogsigma_f) : reinterpret_cast<const R *>(a.dlogsigma);
#pragma unroll
    for (int q = 0; q < kAdjRingParams; ++q) adj.g[q] = 0.0;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    const int lane = threadIdx.x & 31;
    const int K = p.seg_cap;
    const bool count_dl = sizeof(R) == 8 || p.s_end < (1 << 24);
    const R dstep = (R)p.n_sub;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) << 5; base < p.n_particles;
         base += warps * 32) {
        const int64_t i = base + lane;
        const bool have = i < p.n_particles;
        const R *rec = static_cast<const R *>(p.segs) + (size_t)(have ? i : 0) * K * kRecWords;
        const R *th = static_cast<const R *>(p.seg_th) + (size_t)(have ? i : 0) * K;
        Seg<R> cur, nxt;
        R nth = (R)-1;
        int k = 1, next_start = kNeverStart;
        adj.start();
        if (have) {
            rec_get<R, OBS>(rec, cur);
            rec_get<R, OBS>(rec + kRecWords, nxt);
            next_start = nxt.s0;
            nth = __ldg(th + 1);
            adj.enter(__ldg(th));
        } else {
            cur.s0 = 0; cur.mode = 0; cur.doff = -1;
            cur.A[0] = (R)INFINITY; cur.A[1] = cur.A[2] = cur.B[0] = cur.B[1] = cur.B[2] = (R)0;
            cur.x[0] = (R)INFINITY; cur.x[1] = cur.x[2] = (R)0;
        }
        int so = p.n_sub;
        R dl = (R)(so - cur.s0);
        // the weights' index fits 32 bits (the host takes this replay only then); j is also
        // carried as a float, exact below 2^24
        int toff = (int)p.time_stride;
        const int tstep = (int)p.time_stride, mstep = (int)p.mode_stride, hlen = (int)p.hist_len;
        R fj = (R)1;
        // CDL: the offset dl is counted up per instant (an exact integer below 2^24), else
        // converted afresh; fixed per launch, so the loop has no test for it
        auto walk = [&](auto count_tag) {
            constexpr bool CDL = decltype(count_tag)::value;
#pragma unroll 1
            for (int j = 1; j <= p.n_obs; ++j, so += p.n_sub, toff += tstep, fj += (R)1) {
                if (so >= next_start) { // the next segment comes into force; load the one after it
                    do {
                        cur = nxt;
                        adj.enter(nth);
                        ++k;
                        rec_get<R, OBS>(rec + (size_t)k * kRecWords, nxt);
                        nth = __ldg(th + k);
                        next_start = nxt.s0;
                    } while (so >= next_start);
                    dl = (R)(so - cur.s0);
                } else if (!CDL) {
                    dl = (R)(so - cur.s0);
                }
                int v;
                if constexpr (C32) v = obs_offset_cart32(p, cur, dl, cur.doff);
                else v = obs_offset_dl<R, OBS>(p, sedges, cur, dl);
                dl += dstep;
                // branch-free: a lane without an observation adds a zero weight
                const int idx = toff + (cur.mode ? mstep : 0) + v;
                const bool take = v >= 0 && idx < hlen;
                bad |= v >= 0 && idx >= hlen;
                adj.observe_w(take ? __ldg(adj.wts + idx) : (R)0, fj);
                cnt.obs += take ? 1u : 0u;
            }
        };
        if (count_dl) walk(std::true_type{});
        else walk(std::false_type{});
        if (have) adj.finish();
    }
    double g[kAdjRingParams];
#pragma unroll
    for (int q = 0; q < kAdjRingParams; ++q) g[q] = adj.g[q];
    adjoint_block_sums<kAdjRingParams>(p.stats, p.stats, p.status, a.n_params, g, red, a.partial, cnt, bad);
}

// Adjoint replay on the converged two-phase transport (at most kAdjRingParams
// parameters): events run together in phase 1 and carry their scattering angle through
// the ring; phase 2 accumulates adjoint weights per observation in lockstep.
template <typename R, int OBS>
__global__ void __launch_bounds__(kAdjointThreads, sizeof(R) == 4 ? 3 : 1) rt_adjoint_ring(const DevParams<R> p, const AdjointArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[kAdjointThreads / 32][kAdjRingParams];
    R *sedges = reinterpret_cast<R *>(smem_raw);
    const size_t off = (((size_t)p.n_edges * sizeof(R) + 15) / 16) * 16;
    const int T = blockDim.x, C = p.ring_cap;
    Ring<R> ring;
    ring.cap = C;
    ring.stride = T;
    {
        R *r = reinterpret_cast<R *>(smem_raw + off);
        ring.x0 = r; ring.x1 = r + C * T; ring.x2 = r + 2 * C * T;
        ring.d0 = r + 3 * C * T; ring.d1 = r + 4 * C * T; ring.d2 = r + 5 * C * T;
        ring.th = r + 6 * C * T;
        int *ri = reinterpret_cast<int *>(r + 7 * C * T);
        ring.s0 = ri; ring.mode = ri + C * T;
    }
    for (int k = threadIdx.x; k < p.n_edges; k += T) sedges[k] = p.edges[k];
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Counters cnt = {0u, 0u, 0u, 0u, 0u, 0u};
    bool bad = false;
    AdjLane<R> adj;
    adj.a = &a;
    adj.wts = static_cast<const R *>(a.adjoint);
    if constexpr (sizeof(R) == 4) adj.dls = a.dlogsigma_f; else adj.dls = reinterpret_cast<const R *>(a.dlogsigma);
#pragma unroll
    for (int q = 0; q < kAdjRingParams; ++q) adj.g[q] = 0.0;
    const int64_t warps = ((int64_t)gridDim.x * T) >> 5;
    for (int64_t base = (((int64_t)blockIdx.x * T + threadIdx.x) >> 5) << 5; base < p.n_particles; base += warps * 32)
        run_batch<R, SINK_ADJOINT, OBS>(p, sedges, nullptr, ring, base, p.n_particles, cnt, bad, &adj);
    // block sums in a fixed order
#pragma unroll
    for (int q = 0; q < kAdjRingParams; ++q) {
        double v = adj.g[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(full, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < a.n_params) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
        a.partial[(size_t)blockIdx.x * a.n_params + threadIdx.x] = v;
    }
    unsigned cv[6] = {cnt.scat, cnt.bnd, cnt.kill, cnt.absorb, cnt.obs, cnt.conv};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const unsigned t = __reduce_add_sync(full, cv[c]);
        if (lane == 0 && t) atomicAdd(p.stats + c, (unsigned long long)t);
    }
    if (bad) atomicExch(p.status, 1);
}

template <typename R> void *pick_adjoint_ring(int obs)
{
    return obs == OBS_CART ? (void *)rt_adjoint_ring<R, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_adjoint_ring<R, OBS_RADIAL> : (void *)rt_adjoint_ring<R, OBS_GENERAL>);
}

template <typename R> void *pick_observe_adj(int obs)
{
    return obs == OBS_CART ? (void *)rt_observe_adj<R, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_observe_adj<R, OBS_RADIAL> : (void *)rt_observe_adj<R, OBS_GENERAL>);
}

template <typename R> void *pick_adjoint_list(int obs)
{
    return obs == OBS_CART ? (void *)rt_adjoint_list<R, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_adjoint_list<R, OBS_RADIAL> : (void *)rt_adjoint_list<R, OBS_GENERAL>);
}

template <typename R> void *pick_adjoint(int obs)
{
    return obs == OBS_CART ? (void *)rt_adjoint<R, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_adjoint<R, OBS_RADIAL> : (void *)rt_adjoint<R, OBS_GENERAL>);
}

template <typename R> void *pick_t(int sink, int obs)
{
    return sink == SINK_SMEM ? pick_obs<R, SINK_SMEM>(obs)
                             : (sink == SINK_GLOBAL ? pick_obs<R, SINK_GLOBAL>(obs) : pick_obs<R, SINK_INDEX>(obs));
}

} // namespace

// Launchers, instantiated per precision and kernel group by kernels.cu.
template <typename R> int launch_transport_t(const DevParams<R> &p, int grid, int block, size_t smem, void *stream)
{
    void *args[] = {(void *)&p};
    return (int)cudaLaunchKernel(pick_t<R>(p.sink, p.obs_kind), dim3(grid), dim3(block), args, smem, (cudaStream_t)stream);
}

template <typename R, bool SHIST> void *pick_batch_em(int obs)
{
    return obs == OBS_CART ? (void *)rt_transport_batch_em<R, OBS_CART, SHIST>
                           : (obs == OBS_RADIAL ? (void *)rt_transport_batch_em<R, OBS_RADIAL, SHIST>
                                                : (void *)rt_transport_batch_em<R, OBS_GENERAL, SHIST>);
}

template <typename R> void *pick_batch(int obs)
{
    return obs == OBS_CART ? (void *)rt_transport_batch<R, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_transport_batch<R, OBS_RADIAL> : (void *)rt_transport_batch<R, OBS_GENERAL>);
}

template <typename R> void *pick_batch_split(int obs)
{
    return obs == OBS_CART ? (void *)rt_transport_batch_split<R, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_transport_batch_split<R, OBS_RADIAL>
                                                : (void *)rt_transport_batch_split<R, OBS_GENERAL>);
}

// which: 0 the lockstep ring kernel, 1 the event-major kernel (device-memory histogram),
// 2 the split kernel, 3 the event-major kernel with the shared-memory histogram
template <typename R> void *pick_batch_kind(int which, int obs)
{
    switch (which) {
    case 1: return pick_batch_em<R, false>(obs);
    case 2: return pick_batch_split<R>(obs);
    case 3: return pick_batch_em<R, true>(obs);
    default: return pick_batch<R>(obs);
    }
}

template <typename R> int launch_batch_t(const BatchArgs<R> &a, int grid, int block, size_t smem, void *stream, int which)
{
    void *args[] = {(void *)&a};
    return (int)cudaLaunchKernel(pick_batch_kind<R>(which, a.obs_kind), dim3(grid), dim3(block), args, smem,
                                 (cudaStream_t)stream);
}

template <typename R> void *pick_events(int obs)
{
    return obs == OBS_CART ? (void *)rt_events<R, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_events<R, OBS_RADIAL> : (void *)rt_events<R, OBS_GENERAL>);
}

template <typename R, int SINK> void *pick_observe_obs(int obs)
{
    return obs == OBS_CART ? (void *)rt_observe<R, SINK, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_observe<R, SINK, OBS_RADIAL> : (void *)rt_observe<R, SINK, OBS_GENERAL>);
}

template <typename R> void *pick_observe(int sink, int obs)
{
    return sink == SINK_SMEM ? pick_observe_obs<R, SINK_SMEM>(obs)
                             : (sink == SINK_GLOBAL ? pick_observe_obs<R, SINK_GLOBAL>(obs) : pick_observe_obs<R, SINK_INDEX>(obs));
}

template <typename R, int SINK> void *pick_list_obs(int obs)
{
    return obs == OBS_CART ? (void *)rt_transport_list<R, SINK, OBS_CART>
                           : (obs == OBS_RADIAL ? (void *)rt_transport_list<R, SINK, OBS_RADIAL>
                                                : (void *)rt_transport_list<R, SINK, OBS_GENERAL>);
}

// the rerun of overflowing particles: index rows on the index path, else global atomics
template <typename R> void *pick_list(int sink, int obs)
{
    return sink == SINK_INDEX ? pick_list_obs<R, SINK_INDEX>(obs) : pick_list_obs<R, SINK_GLOBAL>(obs);
}

// the split schedule: rt_events, rt_observe, rt_transport_list, in stream order (l.part
// 1: the events and the order sort only; 2: the observations and the reruns only)
template <typename R>
int launch_split_t(const DevParams<R> &p, const SplitLaunch &l, void *stream)
{
    void *args[] = {(void *)&p};
    cudaError_t e = cudaSuccess;
    if (l.part != 2) {
        e = cudaLaunchKernel(pick_events<R>(p.obs_kind), dim3(l.grid_events), dim3(256), args, l.smem_events,
                             (cudaStream_t)stream);
        if (e == cudaSuccess && l.mid_event) e = cudaEventRecord((cudaEvent_t)l.mid_event, (cudaStream_t)stream);
    }
    if (l.part == 2) {
        // the particle order is in place already
    } else if (e == cudaSuccess && p.okey) {
        OrderParams o = l.order;
        o.key = p.okey;
        o.perm = p.perm;
        o.iperm = p.iperm;
        o.n = p.n_particles;
        e = (cudaError_t)launch_order(o, l.grid_order, stream);
    }
    if (l.part == 1) return (int)e;
    if (e == cudaSuccess)
        e = cudaLaunchKernel(pick_observe<R>(p.sink, p.obs_kind), dim3(l.grid_observe), dim3(l.block_observe), args,
                             l.smem_observe, (cudaStream_t)stream);
    if (e == cudaSuccess)
        e = cudaLaunchKernel(pick_list<R>(p.sink, p.obs_kind), dim3(l.grid_list), dim3(256), args, l.smem_events,
                             (cudaStream_t)stream);
    return (int)e;
}

template <typename R>
int launch_adjoint_t(const DevParams<R> &p, const AdjointArgs &a, int grid, int block, size_t smem, void *stream, bool ring)
{
    void *args[] = {(void *)&p, (void *)&a};
    void *fn = ring ? pick_adjoint_ring<R>(p.obs_kind) : pick_adjoint<R>(p.obs_kind);
    return (int)cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, (cudaStream_t)stream);
}

} // namespace rtmc
