/*
 * rtmc_oracle.c -- CPU FP64 oracle for the radiative-transfer Monte Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls this file;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, as the
 * checker.  The reference (cottereau/RadiativeTransferMonteCarlo) is MATLAB and cannot
 * run here; parity against it is therefore pinned by known answers (energy conservation,
 * Zoeppritz energy balance, the boundary energy partition, equipartition and P/S
 * conversion kinetics, Paasschens' 2D and 3D solutions and the diffusion limit, Sato's 3D
 * elastic solution) rather than by reference outputs: "parity unpinned" against
 * reference-produced vectors, which do not exist.
 *
 * Two restatements of the reference transport are provided:
 *
 *  scheme 0, "substep" -- a literal per-sub-step restatement of
 *      propagateParticleSmallDt.m:1-647 (Q-kill :100-138, move :141-143, plane
 *      boundaries :168-322 through MaterialClass.MaterialInterface
 *      (MaterialClass.m:1572-1756), Poisson scatter decision :591-601, azimuth :604-611,
 *      mode conversion :619-623, inverse-CDF angle :614-632, rotation :635-639),
 *      driven from radiativeTransfer.m:105-131 and observed by observeTime.m:1-146.
 *      poissrnd(lambda) > 0 is drawn as the equivalent Bernoulli u < 1 - exp(-lambda).
 *      This is the reference's own CPU algorithm (timed as the CPU baseline).
 *
 *  scheme 1, "event" (snap) -- the same Markov process advanced event by event: the
 *      number of sub-steps to the next scatter (or Q-kill) is geometric, so it is drawn
 *      as ceil(-log(u)/rate); plane-boundary crossings are solved in closed form on the
 *      sub-step grid; observations between events are straight-line extrapolations on
 *      that grid.  It consumes the Philox stream with exactly the slot layout the GPU
 *      kernels use, so GPU and oracle trajectories can be compared particle by particle.
 *
 * Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter =
 * (pid_lo, pid_hi, step, block), key = (seed_lo, seed_hi ^ stream).  A 32-bit output x
 * maps to u = (x + 0.5) * 2^-32 ("u32" mode) or, to reproduce the FP32 GPU path's
 * uniforms, u = ((x >> 9) + 0.5) * 2^-23 ("ufloat" mode: 24 significant bits, so the
 * value is exact in float and the FP32 kernels see the same number).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAX_BND 4
#define OR_NEVER ((int64_t)1 << 62)

/* ------------------------------------------------------------------------- */
/* Problem description (mirrored by oracle/oracle.py with ctypes)             */
/* ------------------------------------------------------------------------- */
typedef struct {
    int32_t d;            /* 2 or 3 */
    int32_t frame;        /* 0 cartesian, 1 cylindrical, 2 spherical */
    int32_t acoustics;    /* 1 acoustic, 0 elastic */
    int32_t scheme;       /* 0 substep, 1 event */
    int32_t ufloat;       /* 1: 23-bit uniforms exact in float (FP32 GPU stream) */
    int32_t src_dir;      /* 0 uniform, 1 outgoing, 2 upper */
    int32_t polarization; /* 0 P, 1 S */
    int32_t n_sub;        /* sub-steps per observation interval */
    int32_t n_obs;        /* observation instants (Nt - 1) */
    int32_t n_bnd;
    int32_t hist_shift;   /* fixed-point shift of a unit count */
    int32_t nthreads;
    int64_t n_particles;
    int64_t pid0;         /* first global particle id */
    uint64_t seed;
    double src_pos[3];
    double src_lambda;
    double v[2];          /* speed of mode P(0)/S(1) (acoustic: v[0]) */
    double mft[2];        /* mean free time per mode (INFINITY: no scattering) */
    double p2p, s2s;
    double qrate[2];      /* omega*h/Q per mode, 0 when Q = Inf */
    double h;             /* sub-step length */
    /* observation axes: 0 X, 1 Y, 2 Z, 3 PSI */
    int32_t axis_mode[4]; /* 0 ignored, 1 range check [lo,hi], 2 binned */
    int32_t axis_nedges[4];
    const double *axis_edges[4];
    int64_t axis_stride[4];
    int64_t time_stride;
    int64_t mode_stride;
    int64_t hist_len;
    /* boundaries */
    int32_t bnd_dir[OR_MAX_BND]; /* 1,2,3: planes x_dir = val; 4: cylinder sqrt(x^2+y^2) = val */
    int32_t bnd_absorb[OR_MAX_BND];
    double bnd_val[OR_MAX_BND];
    const double *zoe_rpp;   /* 181 values, 0:0.5:90 deg */
    const double *zoe_rsvsv; /* 181 values */
    /* inverse-CDF tables: index m*2+m' (acoustic: only 0) */
    int64_t tab_n[4];
    const double *tab_cdf[4];
    const double *tab_theta[4];
    /* source shape (initializeParticle.m:14-148) */
    int32_t src_type;     /* 0 point, 1 plane */
    int32_t src_aperture; /* plane: 0 rectangle, 1 circle */
    int64_t src_radial_n; /* point: knots of the radial inverse CDF, 0 = Gaussian radius */
    const double *src_radial_cdf;
    const double *src_radial_r;
    double src_normal[3], src_u[3], src_v[3];
    double src_extent[2];
    /* optional [n_particles] output of the event scheme: the smallest distance, over the
     * plane-crossing decisions that fix the particle's next event, between the sub-step
     * position that decides the crossing and the plane (length units).  A float
     * trajectory whose position error exceeds it may cross one sub-step earlier or later. */
    double *cross_margin;
} oracle_problem;

enum { ST_SCATTER = 0, ST_BOUNDARY, ST_KILL, ST_ABSORB, ST_OBS, ST_CONVERT, ST_N };

/* ------------------------------------------------------------------------- */
/* Philox4x32-10                                                              */
/* ------------------------------------------------------------------------- */
static inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void oracle_philox4x32_10(const uint32_t *ctr, const uint32_t *key, uint32_t *out)
{
    philox4x32_10(ctr, key, out);
}

typedef struct {
    uint32_t key[2];
    uint64_t pid;
    int ufloat;
} rng_t;

static inline void rng_block(const rng_t *g, uint32_t step, uint32_t block, double u[4])
{
    uint32_t ctr[4] = {(uint32_t)g->pid, (uint32_t)(g->pid >> 32), step, block};
    uint32_t o[4];
    philox4x32_10(ctr, g->key, o);
    for (int i = 0; i < 4; ++i) {
        if (g->ufloat)
            u[i] = ((double)(o[i] >> 9) + 0.5) * (1.0 / 8388608.0);
        else
            u[i] = ((double)o[i] + 0.5) * (1.0 / 4294967296.0);
    }
}

/* ------------------------------------------------------------------------- */
/* Inverse CDF: griddedInterpolant(cdf, theta) with linear interpolation and  */
/* linear extrapolation (MaterialClass.m:2462).                               */
/* ------------------------------------------------------------------------- */
static double invcdf_eval(const double *c, const double *th, int64_t n, double u)
{
    if (n < 2) return n == 1 ? th[0] : 0.0;
    int64_t lo = 0, hi = n - 1; /* find i with c[i] <= u < c[i+1], clamped to [0, n-2] */
    if (u < c[0]) lo = 0;
    else if (u >= c[n - 1]) lo = n - 2;
    else {
        while (hi - lo > 1) {
            int64_t mid = (lo + hi) >> 1;
            if (c[mid] <= u) lo = mid; else hi = mid;
        }
    }
    double t = (u - c[lo]) / (c[lo + 1] - c[lo]);
    return th[lo] + t * (th[lo + 1] - th[lo]);
}

double oracle_invcdf(const double *c, const double *th, int64_t n, double u)
{
    return invcdf_eval(c, th, n, u);
}

/* interp1(j1_deg, data, ang, 'linear', 'extrap') on the 0:0.5:90 grid (MaterialClass.m:1674) */
static double zoe_lookup(const double *tab, double ang_deg)
{
    double f = ang_deg * 2.0;
    int i = (int)floor(f);
    if (i < 0) i = 0;
    if (i > 179) i = 179;
    double w = f - (double)i;
    return tab[i] + w * (tab[i + 1] - tab[i]);
}

/* ------------------------------------------------------------------------- */
/* Small vector helpers                                                       */
/* ------------------------------------------------------------------------- */
static inline void cross3(const double a[3], const double b[3], double o[3])
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double norm3(const double a[3]) { return sqrt(dot3(a, a)); }
static inline void scale3(double a[3], double s) { a[0] *= s; a[1] *= s; a[2] *= s; }

/* ------------------------------------------------------------------------- */
/* Particle                                                                   */
/* ------------------------------------------------------------------------- */
typedef struct {
    double x[3], d[3], q[3];
    int mode;  /* 0 P, 1 S */
    int alive;
} particle_t;

/* griddedInterpolant(cdf, r, 'linear', 'nearest') of initializeParticle.m:201 */
static double radial_invcdf(const double *c, const double *r, int64_t n, double u)
{
    if (!(u > c[0])) return r[0];
    if (!(u < c[n - 1])) return r[n - 1];
    int64_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (c[mid] <= u) lo = mid; else hi = mid;
    }
    return r[lo] + (u - c[lo]) / (c[hi] - c[lo]) * (r[hi] - r[lo]);
}

/* initializeParticle.m:14-148,151-170.  Slots: step 0, block 0 = [r1, r2, phi0, theta0]
 * (plane source: [r1, r2, aperture 1, aperture 2]), block 1 = [phi, theta, alpha,
 * next-scatter], block 2 = [kill]. */
static void init_particle(const oracle_problem *P, const rng_t *g, particle_t *pt, double ub1[4])
{
    double a[4];
    rng_block(g, 0, 0, a);
    rng_block(g, 0, 1, ub1);
    if (P->src_type == 1) {
        /* plane wave (:61-148): Gaussian offset lambda/2 along n, aperture offsets along u, v */
        double c_long = sqrt(-2.0 * log(a[0])) * cos(2.0 * M_PI * a[1]) * P->src_lambda * 0.5;
        double c1, c2;
        if (P->src_aperture == 1) {
            double rho = P->src_extent[0] * sqrt(a[2]);
            double al = 2.0 * M_PI * a[3];
            c1 = rho * cos(al);
            c2 = rho * sin(al);
        } else {
            c1 = (a[2] - 0.5) * P->src_extent[0];
            c2 = (a[3] - 0.5) * P->src_extent[1];
        }
        double th = 2.0 * M_PI * ub1[1];
        double ct = cos(th), st = sin(th);
        for (int i = 0; i < 3; ++i) {
            pt->x[i] = P->src_pos[i] + c_long * P->src_normal[i] + c1 * P->src_u[i] + c2 * P->src_v[i];
            pt->d[i] = P->src_normal[i];
            pt->q[i] = ct * P->src_u[i] + st * P->src_v[i];
        }
        pt->mode = (!P->acoustics && P->polarization == 1) ? 1 : 0;
        pt->alive = 1;
        return;
    }
    double r = P->src_radial_n > 0 ? radial_invcdf(P->src_radial_cdf, P->src_radial_r, P->src_radial_n, a[0])
                                   : fabs(sqrt(-2.0 * log(a[0])) * cos(2.0 * M_PI * a[1])) * P->src_lambda;
    double cphi0, sphi0, cphi, sphi;
    double theta0 = 2.0 * M_PI * a[3];
    double theta = 2.0 * M_PI * ub1[1];
    if (P->d == 2) {
        cphi0 = cos(M_PI / 2); sphi0 = sin(M_PI / 2);
        cphi = cphi0; sphi = sphi0;
    } else {
        cphi0 = -1.0 + 2.0 * a[2];
        sphi0 = sqrt(fmax(0.0, (1.0 - cphi0) * (1.0 + cphi0)));
        if (P->src_dir == 2) { /* 'upper': phi = acos(rand) */
            cphi = ub1[0];
        } else {
            cphi = -1.0 + 2.0 * ub1[0];
        }
        sphi = sqrt(fmax(0.0, (1.0 - cphi) * (1.0 + cphi)));
    }
    if (P->src_dir == 1) { theta = theta0; cphi = cphi0; sphi = sphi0; }
    pt->d[0] = cos(theta) * sphi;
    pt->d[1] = sin(theta) * sphi;
    pt->d[2] = cphi;
    pt->q[0] = -sin(theta);
    pt->q[1] = cos(theta);
    pt->q[2] = 0.0;
    if (P->d == 3) {
        double al = 2.0 * M_PI * ub1[2];
        double c[3];
        cross3(pt->d, pt->q, c);
        double ca = cos(al), sa = sin(al);
        for (int i = 0; i < 3; ++i) pt->q[i] = pt->q[i] * ca + c[i] * sa;
    }
    pt->x[0] = P->src_pos[0] + r * cos(theta0) * sphi0;
    pt->x[1] = P->src_pos[1] + r * sin(theta0) * sphi0;
    pt->x[2] = P->src_pos[2] + r * cphi0;
    pt->mode = (!P->acoustics && P->polarization == 1) ? 1 : 0;
    pt->alive = 1;
}

/* Elastic reflection at a plane boundary with unit normal e_k (k = dir-1):
 * MaterialClass.MaterialInterface (MaterialClass.m:1587-1756) for the decisions and
 * propagateParticleSmallDt.m:197-321 for the updates.  u_split, u_coin are the two draws.
 * Returns 1 when the mode changed. */
static int elastic_plane_reflect(const oracle_problem *P, particle_t *pt, int k, double u_split, double u_coin,
                                 int64_t *stats)
{
    const double eps = 2.220446049250313e-16;
    double n[3] = {0, 0, 0};
    n[k] = 1.0;
    int mode0 = pt->mode;
    double adn = fabs(pt->d[k]);
    if (adn > 1.0) adn = 1.0;
    double ang = acos(adn) * (180.0 / M_PI);
    if (pt->mode == 0) {
        double rpp = zoe_lookup(P->zoe_rpp, ang);
        if (u_coin <= rpp) { /* P -> P */
            pt->d[k] = -pt->d[k];
            pt->q[k] = -pt->q[k];
        } else {             /* P -> SV, :212-248 */
            pt->mode = 1;
            double ratio = P->v[1] / P->v[0];
            double dn = pt->d[k];
            double nd[3] = {pt->d[0] * ratio, pt->d[1] * ratio, pt->d[2] * ratio};
            nd[k] = 0.0;
            double sin2 = dot3(nd, nd);
            double cv = sqrt(fmax(0.0, 1.0 - sin2));
            double sg = (dn > 0) - (dn < 0);
            nd[k] = -sg * cv;
            double nn = norm3(nd);
            scale3(nd, 1.0 / nn);
            memcpy(pt->d, nd, sizeof nd);
            double ax[3];
            cross3(pt->d, n, ax);
            scale3(ax, 1.0 / norm3(ax));
            cross3(ax, pt->d, pt->q);
        }
    } else {
        /* SV / SH split by polarisation energy, :1610-1646 */
        double eSH[3];
        cross3(pt->d, n, eSH);
        double nsh = norm3(eSH);
        if (nsh < eps) {
            double t[3] = {1.0, 0.0, 0.0};
            double tn = dot3(t, n);
            for (int i = 0; i < 3; ++i) t[i] -= tn * n[i];
            memcpy(eSH, t, sizeof t);
            nsh = norm3(t);
        }
        scale3(eSH, 1.0 / nsh);
        double eSV[3];
        cross3(eSH, pt->d, eSV);
        scale3(eSV, 1.0 / norm3(eSV));
        double aSV = dot3(pt->q, eSV), aSH = dot3(pt->q, eSH);
        double Esv = aSV * aSV, Esh = aSH * aSH;
        double probSV = Esv / (Esv + Esh + eps);
        int isSV = u_split < probSV;
        if (!isSV) { /* SH -> SH, :252-257 */
            pt->d[k] = -pt->d[k];
            pt->q[k] = -pt->q[k];
        } else {
            double rsvsv = zoe_lookup(P->zoe_rsvsv, ang);
            if (u_coin <= rsvsv) { /* SV -> SV, :260-271 */
                pt->d[k] = -pt->d[k];
                pt->q[k] = -pt->q[k];
            } else {               /* SV -> P, :274-321 */
                double ratio = P->v[0] / P->v[1];
                double dn = pt->d[k];
                double nd[3] = {pt->d[0] * ratio, pt->d[1] * ratio, pt->d[2] * ratio};
                nd[k] = 0.0;
                double sin2 = dot3(nd, nd);
                if (sin2 <= 1.0) {
                    pt->mode = 0;
                    double cv = sqrt(1.0 - sin2);
                    double sg = (dn > 0) - (dn < 0);
                    nd[k] = -sg * cv;
                    scale3(nd, 1.0 / norm3(nd));
                    memcpy(pt->d, nd, sizeof nd); /* perp is left unchanged, as in the reference */
                } else {
                    /* total internal reflection: stays SV, only dir mirrored (:313-319) */
                    pt->d[k] = -pt->d[k];
                }
            }
        }
    }
    if (pt->mode != mode0) stats[ST_CONVERT]++;
    return pt->mode != mode0;
}

static inline void mirror3(double v[3], const double n[3])
{
    double vn = 2.0 * dot3(v, n);
    for (int i = 0; i < 3; ++i) v[i] -= vn * n[i];
}

/* Elastic reflection at the cylinder wall with outward unit normal n,
 * propagateParticleSmallDt.m:356-571 (coefficients through griddedInterpolant 'linear',
 * 'nearest' on 0:0.5:90 degrees).  Returns 1 when the mode changed. */
static int elastic_cylinder_reflect(const oracle_problem *P, particle_t *pt, const double n[3], double u_split,
                                    double u_coin, int64_t *stats)
{
    int mode0 = pt->mode;
    double dn = dot3(pt->d, n);
    double ang = acos(fmin(1.0, fmax(-1.0, dn))) * (180.0 / M_PI);
    if (ang > 90.0) ang = 90.0;
    if (pt->mode == 0) {
        if (u_coin <= zoe_lookup(P->zoe_rpp, ang)) { /* P -> P, :392-405 */
            mirror3(pt->d, n);
            mirror3(pt->q, n);
        } else {                                     /* P -> SV, :409-451 */
            pt->mode = 1;
            double eta = P->v[1] / P->v[0];
            double nd[3];
            for (int i = 0; i < 3; ++i) nd[i] = eta * (pt->d[i] - dn * n[i]);
            double cv = sqrt(fmax(0.0, 1.0 - dot3(nd, nd)));
            for (int i = 0; i < 3; ++i) nd[i] -= cv * n[i];
            scale3(nd, 1.0 / norm3(nd));
            memcpy(pt->d, nd, sizeof nd);
            double ax[3];
            cross3(pt->d, n, ax);
            if (norm3(ax) < 1e-6) {
                const double ex[3] = {1.0, 0.0, 0.0};
                cross3(pt->d, ex, ax);
            }
            scale3(ax, 1.0 / norm3(ax));
            cross3(ax, pt->d, pt->q);
        }
    } else {
        double ax[3];
        cross3(pt->d, n, ax);
        double a2 = dot3(ax, ax);
        double sh = dot3(pt->q, ax);
        double prob_sh = a2 > 0 ? sh * sh / a2 : -1.0; /* NaN in the reference: never SH */
        if (u_split < prob_sh) {                                   /* SH, :474-485 */
            mirror3(pt->d, n);
            mirror3(pt->q, n);
        } else if (u_coin <= zoe_lookup(P->zoe_rsvsv, ang)) {      /* SV -> SV, :508-521 */
            mirror3(pt->d, n);
            mirror3(pt->q, n);
        } else {                                                   /* SV -> P, :523-566 */
            double eta = P->v[0] / P->v[1];
            double nd[3];
            for (int i = 0; i < 3; ++i) nd[i] = eta * (pt->d[i] - dn * n[i]);
            double sin2 = dot3(nd, nd);
            if (sin2 <= 1.0) {
                pt->mode = 0;
                double cv = sqrt(1.0 - sin2);
                for (int i = 0; i < 3; ++i) nd[i] -= cv * n[i];
                scale3(nd, 1.0 / norm3(nd));
                memcpy(pt->d, nd, sizeof nd); /* polarisation kept */
            } else {                          /* total internal reflection: SV mirror */
                mirror3(pt->d, n);
                mirror3(pt->q, n);
            }
        }
    }
    if (pt->mode != mode0) stats[ST_CONVERT]++;
    return pt->mode != mode0;
}

/* Cylinder test and update of one boundary pass (propagateParticleSmallDt.m:325-352):
 * 0 inside, 1 reflected, 2 absorbed. */
static int cylinder_hit(const oracle_problem *P, const rng_t *g, uint32_t step, uint32_t block, int b,
                        particle_t *pt, int *changed, int64_t *stats)
{
    double r = sqrt(pt->x[0] * pt->x[0] + pt->x[1] * pt->x[1]);
    double over = r - P->bnd_val[b];
    if (!(over > 0)) return 0;
    stats[ST_BOUNDARY]++;
    if (P->bnd_absorb[b]) { pt->alive = 0; stats[ST_ABSORB]++; return 2; }
    double n[3] = {pt->x[0] / r, pt->x[1] / r, 0.0};
    pt->x[0] -= 2.0 * over * n[0];
    pt->x[1] -= 2.0 * over * n[1];
    if (P->acoustics) {
        mirror3(pt->d, n);
    } else {
        double bb[4];
        rng_block(g, step, block, bb);
        *changed |= elastic_cylinder_reflect(P, pt, n, bb[0], bb[1], stats);
    }
    return 1;
}

/* Scattering: azimuth (:604-611), mode conversion (:619-623), theta (:614-632),
 * rotation and renormalisation (:635-639).  Returns the new mode. */
static double scatter(const oracle_problem *P, particle_t *pt, double u_phi, double u_mode, double u_theta)
{
    if (P->d == 2) {
        if (u_phi >= 0.5) scale3(pt->q, -1.0);
    } else {
        double ph = 2.0 * M_PI * u_phi;
        double c[3];
        cross3(pt->d, pt->q, c);
        double cp = cos(ph), sp = sin(ph);
        for (int i = 0; i < 3; ++i) pt->q[i] = cp * pt->q[i] + sp * c[i];
    }
    int m = pt->mode, m2 = m;
    if (!P->acoustics) {
        if (m == 0 && u_mode > P->p2p) m2 = 1;
        else if (m == 1 && u_mode > P->s2s) m2 = 0;
    }
    int ti = P->acoustics ? 0 : m * 2 + m2;
    double th = invcdf_eval(P->tab_cdf[ti], P->tab_theta[ti], P->tab_n[ti], u_theta);
    double ct = cos(th), st = sin(th);
    double nd[3], nq[3];
    for (int i = 0; i < 3; ++i) {
        nd[i] = ct * pt->d[i] + st * pt->q[i];
        nq[i] = -st * pt->d[i] + ct * pt->q[i];
    }
    scale3(nd, 1.0 / norm3(nd));
    scale3(nq, 1.0 / norm3(nq));
    memcpy(pt->d, nd, sizeof nd);
    memcpy(pt->q, nq, sizeof nq);
    pt->mode = m2;
    return th;
}

/* ------------------------------------------------------------------------- */
/* Observation: observeTime.m:14-144 with histcounts2 bin semantics.          */
/* ------------------------------------------------------------------------- */
static int64_t bin_index(const double *e, int ne, double v)
{
    /* histcounts: [e_i, e_{i+1}), last bin closed; outside or NaN -> -1 */
    if (!(v >= e[0]) || !(v <= e[ne - 1])) return -1;
    if (v == e[ne - 1]) return ne - 2;
    int lo = 0, hi = ne - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (e[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

static int64_t obs_index(const oracle_problem *P, const double x[3], const double dir[3], int mode, int it);

static void observe(const oracle_problem *P, const double x[3], const double dir[3], int mode, int it,
                    int64_t *hist, int use_atomic, int64_t *stats)
{
    int64_t idx = obs_index(P, x, dir, mode, it);
    if (idx < 0) return;
    int64_t inc = (int64_t)1 << P->hist_shift;
    if (use_atomic) __atomic_fetch_add(&hist[idx], inc, __ATOMIC_RELAXED);
    else hist[idx] += inc;
    stats[ST_OBS]++;
}

/* histogram index of an observation (observeTime.m:14-144), -1 outside the grid */
static int64_t obs_index(const oracle_problem *P, const double x[3], const double dir[3], int mode, int it)
{
    double c[4];
    double cz = dir[2];
    if (cz > 1.0) cz = 1.0;
    if (cz < -1.0) cz = -1.0;
    double psi = (P->d == 3) ? cz : acos(cz);
    if (P->frame == 0) {
        c[0] = x[0]; c[1] = x[1]; c[2] = x[2];
    } else {
        double rxy = hypot(x[0], x[1]);
        double th = atan2(x[1], x[0]);
        if (P->frame == 1 || P->d == 2) {
            c[0] = rxy; c[1] = th; c[2] = x[2];
        } else { /* 3D spherical: cart2sph, then sin(elevation) */
            double r = hypot(rxy, x[2]);
            double el = atan2(x[2], rxy);
            c[0] = r; c[1] = th; c[2] = sin(el);
        }
    }
    c[3] = psi;
    int64_t idx = 0;
    for (int a = 0; a < 4; ++a) {
        int am = P->axis_mode[a];
        if (am == 0) continue;
        const double *e = P->axis_edges[a];
        int ne = P->axis_nedges[a];
        if (am == 1) {
            if (!(c[a] >= e[0] && c[a] <= e[ne - 1])) return -1;
        } else {
            int64_t b = bin_index(e, ne, c[a]);
            if (b < 0) return -1;
            idx += b * P->axis_stride[a];
        }
    }
    return idx + (int64_t)it * P->time_stride + (int64_t)mode * P->mode_stride;
}

/* Score-function adjoint of an acoustic problem (see oracle_gradient): the score of
 * parameter q at observation j is A[q] + b_obs[q] j; a scattering at angle theta adds
 * dlogsigma_q(theta) (linear interpolation on a uniform grid of theta / pi) + a_inc[q]. */
typedef struct {
    const double *adjoint;
    const double *dlogsigma;
    int n_params, n_theta;
    const double *a_inc, *b_obs;
    double A[8];
    double g[8]; /* this thread's sums */
} adj_t;

/* ------------------------------------------------------------------------- */
/* Scheme 0: literal sub-step restatement                                     */
/* ------------------------------------------------------------------------- */
static void run_substep(const oracle_problem *P, int64_t pid, int64_t *hist, int use_atomic, int64_t *stats,
                        double *fstate)
{
    rng_t g;
    g.key[0] = (uint32_t)P->seed;
    g.key[1] = (uint32_t)(P->seed >> 32) ^ 0x5u; /* stream 5: sub-step scheme */
    g.pid = (uint64_t)pid;
    g.ufloat = P->ufloat;
    particle_t pt;
    double ub1[4];
    init_particle(P, &g, &pt, ub1);
    double pscat[2], pkill[2];
    for (int m = 0; m < 2; ++m) {
        pscat[m] = isinf(P->mft[m]) ? 0.0 : -expm1(-P->h / P->mft[m]);
        pkill[m] = P->qrate[m] > 0 ? -expm1(-P->qrate[m]) : 0.0;
    }
    int64_t nscat = 0;
    for (int it = 1; it <= P->n_obs && pt.alive; ++it) {
        for (int j = 1; j <= P->n_sub; ++j) {
            uint32_t sg = (uint32_t)((int64_t)(it - 1) * P->n_sub + j);
            double a[4];
            rng_block(&g, sg, 0, a); /* [kill, scatter, azimuth, theta] */
            int m = pt.mode;
            if (pkill[m] > 0 && a[0] < pkill[m]) { pt.alive = 0; stats[ST_KILL]++; break; }
            double x1[3] = {pt.x[0], pt.x[1], pt.x[2]};
            double step = P->v[m] * P->h;
            for (int i = 0; i < 3; ++i) pt.x[i] += step * pt.d[i];
            for (int b = 0; b < P->n_bnd && pt.alive; ++b) {
                if (P->bnd_dir[b] == 4) {
                    int ch = 0;
                    if (cylinder_hit(P, &g, sg, 2 + b, b, &pt, &ch, stats) == 2) break;
                    continue;
                }
                int k = P->bnd_dir[b] - 1;
                double val = P->bnd_val[b];
                if (!((pt.x[k] - val) * (x1[k] - val) < 0)) continue;
                stats[ST_BOUNDARY]++;
                if (P->bnd_absorb[b]) { pt.alive = 0; stats[ST_ABSORB]++; break; }
                pt.x[k] = 2.0 * val - pt.x[k];
                if (P->acoustics) {
                    pt.d[k] = -pt.d[k];
                } else {
                    double bb[4];
                    rng_block(&g, sg, 2 + b, bb);
                    elastic_plane_reflect(P, &pt, k, bb[0], bb[1], stats);
                }
            }
            if (!pt.alive) break;
            m = pt.mode;
            if (a[1] < pscat[m]) {
                double c[4];
                rng_block(&g, sg, 1, c); /* [mode, ...] */
                scatter(P, &pt, a[2], c[0], a[3]);
                stats[ST_SCATTER]++;
                nscat++;
            } else {
                /* theta = 0 rotation for non-scattered particles: renormalisation only */
                scale3(pt.d, 1.0 / norm3(pt.d));
                scale3(pt.q, 1.0 / norm3(pt.q));
            }
        }
        if (pt.alive) observe(P, pt.x, pt.d, pt.mode, it, hist, use_atomic, stats);
    }
    if (fstate) {
        double *f = fstate;
        for (int i = 0; i < 3; ++i) { f[i] = pt.x[i]; f[3 + i] = pt.d[i]; f[6 + i] = pt.q[i]; }
        f[9] = pt.mode; f[10] = pt.alive; f[11] = (double)nscat;
        f[12] = f[13] = f[14] = f[15] = 0.0;
    }
}

/* ------------------------------------------------------------------------- */
/* Scheme 1: event-driven (snap) restatement                                  */
/* ------------------------------------------------------------------------- */
/* number of sub-steps to the first success of a Bernoulli(1 - exp(-rate)) sequence */
static inline int64_t geom_steps(double u, double rate, int64_t cap)
{
    if (!(rate > 0)) return cap;
    const double inv_rate = 1.0 / rate; /* the GPU keeps the reciprocal rate */
    double k = ceil(-log(u) * inv_rate);
    if (k < 1.0) k = 1.0;
    if (k >= (double)cap) return cap;
    return (int64_t)k;
}

/* outside the cylinder after j sub-steps of the segment, placed as the event step does */
static inline int cyl_outside(const particle_t *pt, double step, int64_t j, double rad)
{
    double t = step * (double)j;
    double x = pt->x[0] + t * pt->d[0], y = pt->x[1] + t * pt->d[1];
    return sqrt(x * x + y * y) > rad;
}

/* first sub-step j in [1, lim) of a segment that ends outside the cylinder sqrt(x^2+y^2) =
 * rad, or lim: the larger root of |P + j V|^2 = rad^2, settled on the exact test */
static int64_t cyl_cross_steps(const particle_t *pt, double step, double rad, int64_t lim)
{
    if (cyl_outside(pt, step, 1, rad)) return 1;
    double vx = step * pt->d[0], vy = step * pt->d[1];
    double A = vx * vx + vy * vy;
    if (!(A > 0)) return lim;
    double B = pt->x[0] * vx + pt->x[1] * vy;
    double Cc = pt->x[0] * pt->x[0] + pt->x[1] * pt->x[1] - rad * rad;
    double sq = sqrt(fmax(0.0, B * B - A * Cc));
    double jr = B > 0 ? -Cc / (B + sq) : (sq - B) / A;
    if (!(jr < (double)lim)) return lim;
    int64_t j = jr < 1.0 ? 1 : (int64_t)floor(jr);
    for (int it = 0; it < 4 && j < lim && !cyl_outside(pt, step, j, rad); ++it) ++j;
    for (int it = 0; it < 4 && j > 1 && cyl_outside(pt, step, j - 1, rad); ++it) --j;
    return j < lim ? j : lim;
}

/* first sub-step j >= 1 of a segment at which the plane x_k = val is crossed */
static inline int64_t plane_cross_steps(double a, double b, int64_t cap)
{
    /* a = x0_k - val, b = per-sub-step displacement along k */
    if (a == 0.0 || b == 0.0 || (a > 0) == (b > 0)) return cap;
    double j = floor(fabs(a) / fabs(b)) + 1.0;
    if (j >= (double)cap) return cap;
    return (int64_t)j;
}

static void run_event(const oracle_problem *P, int64_t pid, int64_t *hist, int use_atomic, int64_t *stats,
                      double *fstate, adj_t *adj)
{
    if (adj)
        for (int q = 0; q < adj->n_params; ++q) adj->A[q] = 0.0;
    rng_t g;
    g.key[0] = (uint32_t)P->seed;
    g.key[1] = (uint32_t)(P->seed >> 32);
    g.pid = (uint64_t)pid;
    g.ufloat = P->ufloat;
    particle_t pt;
    double ub1[4], ub2[4];
    init_particle(P, &g, &pt, ub1);
    rng_block(&g, 0, 2, ub2);
    const int64_t s_end = (int64_t)P->n_obs * P->n_sub;
    const int64_t cap = s_end + 1; /* "never within the run" */
    double lam[2];
    for (int m = 0; m < 2; ++m) lam[m] = isinf(P->mft[m]) ? 0.0 : P->h / P->mft[m];
    int64_t s0 = 0;
    int64_t sS = geom_steps(ub1[3], lam[pt.mode], cap);
    int64_t sK = geom_steps(ub2[0], P->qrate[pt.mode], cap);
    int64_t s_death = cap;
    int next_obs = 1; /* observation j at sub-step j*n_sub */
    uint32_t k = 0;   /* event counter (step index of the Philox counter) */
    int64_t nscat = 0, nbnd = 0;
    double *margin = P->cross_margin ? P->cross_margin + (pid - P->pid0) : NULL;
    int64_t cand[OR_MAX_BND];
    double cmar[OR_MAX_BND];
    if (margin) *margin = INFINITY;
    for (;;) {
        int m = pt.mode;
        double step = P->v[m] * P->h;
        /* next boundary crossing on this segment */
        int64_t sB = cap;
        for (int b = 0; b < P->n_bnd; ++b) {
            if (P->bnd_dir[b] == 4) {
                int64_t j = cyl_cross_steps(&pt, step, P->bnd_val[b], cap - s0);
                if (j < cap - s0 && s0 + j < sB) sB = s0 + j;
                continue;
            }
            int kk = P->bnd_dir[b] - 1;
            int64_t j = plane_cross_steps(pt.x[kk] - P->bnd_val[b], step * pt.d[kk], cap);
            if (j < cap && s0 + j < sB) sB = s0 + j;
            if (margin && j < cap) {
                /* |a| - (j - 1) |b|: how far the position after j - 1 sub-steps is from the plane */
                double bb = fabs(step * pt.d[kk]), rem = fabs(pt.x[kk] - P->bnd_val[b]) - (double)(j - 1) * bb;
                double mg = rem < bb - rem ? rem : bb - rem;
                cand[b] = s0 + j;
                cmar[b] = mg;
            } else {
                cand[b] = cap + 1;
            }
        }
        int64_t e = sK;
        int kind = 2; /* 2 kill, 1 boundary, 0 scatter; ties resolve kill > boundary > scatter */
        if (sB < e) { e = sB; kind = 1; }
        if (sS < e) { e = sS; kind = 0; }
        if (margin)
            for (int b = 0; b < P->n_bnd; ++b) /* a crossing one sub-step off would change the event */
                if (P->bnd_dir[b] != 4 && cand[b] <= e + 1 && cand[b] <= s_end && cmar[b] < *margin) *margin = cmar[b];
        if (e > s_end) { e = cap; kind = -1; }
        /* observations strictly before the event */
        while (next_obs <= P->n_obs && (int64_t)next_obs * P->n_sub < e) {
            int64_t so = (int64_t)next_obs * P->n_sub;
            double dt = step * (double)(so - s0);
            double xo[3] = {pt.x[0] + dt * pt.d[0], pt.x[1] + dt * pt.d[1], pt.x[2] + dt * pt.d[2]};
            if (adj) {
                int64_t idx = obs_index(P, xo, pt.d, m, next_obs);
                if (idx >= 0) {
                    double w = adj->adjoint[idx];
                    for (int q = 0; q < adj->n_params; ++q)
                        adj->g[q] += w * (adj->A[q] + adj->b_obs[q] * (double)next_obs);
                    stats[ST_OBS]++;
                }
            } else {
                observe(P, xo, pt.d, m, next_obs, hist, use_atomic, stats);
            }
            next_obs++;
        }
        if (kind < 0) break;
        if (kind == 2) { pt.alive = 0; s_death = e; stats[ST_KILL]++; break; }
        double dt = step * (double)(e - s0);
        double xe[3] = {pt.x[0] + dt * pt.d[0], pt.x[1] + dt * pt.d[1], pt.x[2] + dt * pt.d[2]};
        k++;
        if (kind == 1) {
            double dt1 = step * (double)(e - 1 - s0);
            double x1[3] = {pt.x[0] + dt1 * pt.d[0], pt.x[1] + dt1 * pt.d[1], pt.x[2] + dt1 * pt.d[2]};
            memcpy(pt.x, xe, sizeof xe);
            int changed = 0;
            for (int b = 0; b < P->n_bnd && pt.alive; ++b) {
                if (P->bnd_dir[b] == 4) {
                    int hit = cylinder_hit(P, &g, k, 1 + b, b, &pt, &changed, stats);
                    nbnd += hit != 0;
                    if (hit == 2) break;
                    continue;
                }
                int kk = P->bnd_dir[b] - 1;
                double val = P->bnd_val[b];
                if (!((pt.x[kk] - val) * (x1[kk] - val) < 0)) continue;
                stats[ST_BOUNDARY]++;
                nbnd++;
                if (P->bnd_absorb[b]) { pt.alive = 0; stats[ST_ABSORB]++; break; }
                pt.x[kk] = 2.0 * val - pt.x[kk];
                if (P->acoustics) {
                    pt.d[kk] = -pt.d[kk];
                } else {
                    double bb[4];
                    rng_block(&g, k, 1 + b, bb);
                    changed |= elastic_plane_reflect(P, &pt, kk, bb[0], bb[1], stats);
                }
            }
            s0 = e;
            if (!pt.alive) { s_death = e; break; }
            if (changed) {
                double r0[4];
                rng_block(&g, k, 0, r0);
                int64_t js = geom_steps(r0[0], lam[pt.mode], cap);
                sS = (js >= cap) ? cap : e - 1 + js; /* the scatter test of this sub-step uses the new mode */
                int64_t jk = geom_steps(r0[1], P->qrate[pt.mode], cap);
                sK = (jk >= cap) ? cap : e + jk;
            }
        } else { /* scatter */
            double r0[4];
            rng_block(&g, k, 0, r0); /* [next, azimuth, mode, theta] */
            memcpy(pt.x, xe, sizeof xe);
            int m0 = pt.mode;
            double th = scatter(P, &pt, r0[1], r0[2], r0[3]);
            stats[ST_SCATTER]++;
            if (adj) {
                double f = th / M_PI;
                f = f < 0 ? 0 : (f > 1 ? 1 : f);
                f *= (double)(adj->n_theta - 1);
                int kk = (int)f;
                if (kk > adj->n_theta - 2) kk = adj->n_theta - 2;
                double w = f - (double)kk;
                for (int q = 0; q < adj->n_params; ++q) {
                    const double *t = adj->dlogsigma + (int64_t)q * adj->n_theta + kk;
                    adj->A[q] += t[0] + w * (t[1] - t[0]) + adj->a_inc[q];
                }
            }
            nscat++;
            s0 = e;
            int64_t js = geom_steps(r0[0], lam[pt.mode], cap);
            sS = (js >= cap) ? cap : e + js;
            if (pt.mode != m0) {
                double r1[4];
                rng_block(&g, k, 1, r1);
                int64_t jk = geom_steps(r1[0], P->qrate[pt.mode], cap);
                sK = (jk >= cap) ? cap : e + jk;
            }
        }
        if (sS > cap) sS = cap;
        if (sK > cap) sK = cap;
    }
    if (fstate) {
        double *f = fstate;
        for (int i = 0; i < 3; ++i) { f[i] = pt.x[i]; f[3 + i] = pt.d[i]; f[6 + i] = pt.q[i]; }
        f[9] = pt.mode; f[10] = pt.alive; f[11] = (double)nscat;
        f[12] = (double)nbnd; f[13] = (double)s0; f[14] = (double)(s_death < cap ? s_death : -1);
        f[15] = (double)k;
    }
}

/* ------------------------------------------------------------------------- */
/* Driver: radiativeTransfer.m:58-92 / :105-131 (packets -> particles)        */
/* ------------------------------------------------------------------------- */
int oracle_run(const oracle_problem *P, int64_t *hist, int64_t *stats_out, double *fstate)
{
    if (!P || !hist || P->n_obs < 1 || P->n_sub < 1 || (P->d != 2 && P->d != 3)) return 1;
    int nth = P->nthreads > 0 ? P->nthreads : 1;
    int64_t stats[ST_N];
    memset(stats, 0, sizeof stats);
    /* private histograms when they are small, shared atomics otherwise */
    int priv = (P->hist_len * (int64_t)nth * 8 <= ((int64_t)256 << 20));
#ifdef _OPENMP
#pragma omp parallel num_threads(nth)
#endif
    {
        int64_t ls[ST_N];
        memset(ls, 0, sizeof ls);
        int64_t *h = hist;
        if (priv && nth > 1) h = (int64_t *)calloc((size_t)P->hist_len, sizeof(int64_t));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t i = 0; i < P->n_particles; ++i) {
            double *fs = fstate ? fstate + 16 * i : NULL;
            if (P->scheme == 0) run_substep(P, P->pid0 + i, h, !(priv) && nth > 1, ls, fs);
            else run_event(P, P->pid0 + i, h, !(priv) && nth > 1, ls, fs, NULL);
        }
        if (h != hist) {
#ifdef _OPENMP
#pragma omp critical
#endif
            for (int64_t j = 0; j < P->hist_len; ++j) hist[j] += h[j];
            free(h);
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        for (int j = 0; j < ST_N; ++j) stats[j] += ls[j];
    }
    if (stats_out) memcpy(stats_out, stats, sizeof stats);
    return 0;
}

/* Score-function gradient of an acoustic problem (qrate = 0) by the event scheme:
 * grad[q] = sum over particles and observations of adjoint[bin] * (A_q + b_obs[q] j),
 * the replay that the GPU's rt_adjoint performs. */
int oracle_gradient(const oracle_problem *P, const double *adjoint, const double *dlogsigma, int n_params,
                    int n_theta, const double *a_inc, const double *b_obs, double *grad, int64_t *stats_out)
{
    if (!P || !adjoint || !dlogsigma || !grad || n_params < 1 || n_params > 8 || n_theta < 2 || !P->acoustics) return 1;
    int nth = P->nthreads > 0 ? P->nthreads : 1;
    int64_t stats[ST_N];
    memset(stats, 0, sizeof stats);
    for (int q = 0; q < n_params; ++q) grad[q] = 0.0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nth)
#endif
    {
        int64_t ls[ST_N];
        memset(ls, 0, sizeof ls);
        adj_t a;
        memset(&a, 0, sizeof a);
        a.adjoint = adjoint;
        a.dlogsigma = dlogsigma;
        a.n_params = n_params;
        a.n_theta = n_theta;
        a.a_inc = a_inc;
        a.b_obs = b_obs;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t i = 0; i < P->n_particles; ++i) run_event(P, P->pid0 + i, NULL, 0, ls, NULL, &a);
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            for (int q = 0; q < n_params; ++q) grad[q] += a.g[q];
            for (int j = 0; j < ST_N; ++j) stats[j] += ls[j];
        }
    }
    if (stats_out) memcpy(stats_out, stats, sizeof stats);
    return 0;
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Test entry: the elastic plane reflection (MaterialInterface decisions + the updates of
 * propagateParticleSmallDt.m:197-321) applied to n particles at the plane normal to
 * e_k, with draws u[2i] (SV/SH split) and u[2i+1] (reflection coin).  d, q are n x 3,
 * updated in place with mode.  Restates the energy-partition experiment of
 * Examples/BoundaryReflectionEnergyTests.m:110-193 without volume scattering. */
int oracle_reflect(const double *zoe_rpp, const double *zoe_rsvsv, double vp, double vs, int k, int64_t n,
                   double *d, double *q, int32_t *mode, const double *u)
{
    /* k = 0, 1, 2: plane normal to e_k; k = 3: cylinder wall with outward normal e_x */
    if (k < 0 || k > 3 || n < 0) return 1;
    const double ex[3] = {1.0, 0.0, 0.0};
    oracle_problem P;
    memset(&P, 0, sizeof P);
    P.v[0] = vp;
    P.v[1] = vs;
    P.zoe_rpp = zoe_rpp;
    P.zoe_rsvsv = zoe_rsvsv;
    int64_t stats[ST_N];
    for (int64_t i = 0; i < n; ++i) {
        particle_t pt;
        memcpy(pt.d, d + 3 * i, sizeof pt.d);
        memcpy(pt.q, q + 3 * i, sizeof pt.q);
        pt.mode = mode[i];
        pt.alive = 1;
        if (k == 3)
            elastic_cylinder_reflect(&P, &pt, ex, u[2 * i], u[2 * i + 1], stats);
        else
            elastic_plane_reflect(&P, &pt, k, u[2 * i], u[2 * i + 1], stats);
        memcpy(d + 3 * i, pt.d, sizeof pt.d);
        memcpy(q + 3 * i, pt.q, sizeof pt.q);
        mode[i] = pt.mode;
    }
    return 0;
}
