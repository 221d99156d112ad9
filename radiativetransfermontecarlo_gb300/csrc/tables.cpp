// Host FP64 table builders of librtmc.
//
// rtmc_tables_build restates MaterialClass.prepareSigma / prepareSigmaOne
// (@MaterialClass/MaterialClass.m:2379-2463) with the cross-sections of
// calcSigmaIsotropic (:172-359) and the PSDF families of :479-710.  Sigma and Sigma'
// use a globally adaptive Gauss-Kronrod (7,15) rule in place of MATLAB's `integral`;
// the pdf is sampled on n_theta points of [0, pi], the cdf is the running sum scaled by
// pi/n_theta and knots are kept where diff(cdf) > 1e-8 on either side, giving the
// linear griddedInterpolant (linear extrapolation) of :2459-2462.
//
// rtmc_zoeppritz_fluid restates ZoeppritzFluid.m:47-222 with complex arithmetic (the
// refraction angles turn complex beyond the critical angles).
#include "rtmc_internal.h"

#include <cuda_runtime_api.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <queue>
#include <thread>
#include <vector>

namespace rtmc {

thread_local std::string g_thread_error;

int fail(std::string *slot, int code, const std::string &msg)
{
    if (slot) *slot = msg;
    g_thread_error = msg;
    return code;
}

namespace {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------------
// Normalised power spectral densities Phi(z) (MaterialClass.m:479-710)
// ---------------------------------------------------------------------------------
struct Psdf {
    int kind = RTMC_PSDF_EXP;
    int d = 3;
    double a = 1.0, nu = 0.5;

    double operator()(double z) const
    {
        switch (kind) {
        case RTMC_PSDF_EXP:
            if (d == 2) return 1.0 / (4 * kPi * std::pow(1 + (z / a) * (z / a), 1.5));
            {
                double q = 1 + (z / a) * (z / a);
                return 1.0 / (6 * kPi * kPi * q * q);
            }
        case RTMC_PSDF_GAUSSIAN:
            if (d == 2) return 1.0 / (4 * kPi) * std::exp(-z * z / 4);
            return 1.0 / (6 * kPi * kPi) * std::exp(-z * z / (4 * a));
        case RTMC_PSDF_POWER_LAW:
            if (d == 2) return z * std::cyl_bessel_k(1.0, z) / (4 * kPi);
            return 1.0 / (6 * kPi * kPi) * std::exp(-z / a);
        case RTMC_PSDF_TRIANGULAR: {
            double hv = (2 * kPi - z) > 0 ? 1.0 : ((2 * kPi - z) == 0 ? 0.5 : 0.0);
            return (3.0 / 8.0 / (kPi * kPi * kPi * kPi)) * (1 - z / 2 / kPi) * hv;
        }
        case RTMC_PSDF_LOW_PASS: {
            double hv = (a - z) > 0 ? 1.0 : ((a - z) == 0 ? 0.5 : 0.0);
            return (2.0 / 9.0 / (kPi * kPi * kPi * kPi)) * hv;
        }
        case RTMC_PSDF_VON_KARMAN:
            if (d == 2) return 1.0 / (4 * kPi) / std::pow(1 + (z / a) * (z / a), nu + 1);
            return 1.0 / (6 * kPi * kPi) / std::pow(1 + (z / a) * (z / a), nu + 1.5);
        }
        return 0.0;
    }
};

int make_psdf(const rtmc_material &m, Psdf *p, std::string *err)
{
    p->kind = m.psdf;
    p->d = m.d;
    p->nu = m.nu;
    switch (m.psdf) {
    case RTMC_PSDF_EXP: p->a = (m.d == 2) ? std::sqrt(2.0) : std::cbrt(6.0); break;
    case RTMC_PSDF_GAUSSIAN: p->a = std::pow(3 * std::sqrt(kPi) / 4, 2.0 / 3.0); break;
    case RTMC_PSDF_POWER_LAW: p->a = std::cbrt(3 * kPi / 4); break;
    case RTMC_PSDF_TRIANGULAR:
        if (m.d != 3) return fail(err, RTMC_ERR_ARG, "triangular PSDF is defined for d = 3 only");
        break;
    case RTMC_PSDF_LOW_PASS:
        if (m.d != 3) return fail(err, RTMC_ERR_ARG, "low_pass PSDF is defined for d = 3 only");
        p->a = 3 * kPi / 2;
        break;
    case RTMC_PSDF_VON_KARMAN:
        if (!(m.nu > 0)) return fail(err, RTMC_ERR_ARG, "VonKarman PSDF needs a Hurst number nu > 0");
        p->a = (m.d == 2) ? 2 * std::sqrt(m.nu)
                          : std::cbrt(6 * std::sqrt(kPi) * std::tgamma(m.nu + 1.5) / std::tgamma(m.nu));
        break;
    default: return fail(err, RTMC_ERR_ARG, "unknown PSDF family");
    }
    return RTMC_OK;
}

// ---------------------------------------------------------------------------------
// Differential cross-sections sigma_ij(theta) (calcSigmaIsotropic, MaterialClass.m:172-359)
// ---------------------------------------------------------------------------------
struct Sigma {
    int which = 0;     // 0 acoustic, 1 PP, 2 PS, 3 SP, 4 SS, 5 constant
    int d = 3;
    Psdf phi;
    double omega = 0, zeta = 0, zP = 0, zS = 0, K = 1;
    double c1 = 0, c2 = 0, c3 = 0;         // acoustic: dkk, drr, rkr
    double dll = 0, dmm = 0, drr = 0, rlm = 0, rlr = 0, rmr = 0;
    double cst = 0;

    double operator()(double th) const
    {
        double c = std::cos(th);
        const double pi = kPi;
        switch (which) {
        case 0: {
            double p = (d == 2) ? zeta * zeta : zeta * zeta * zeta;
            return (pi / 2) * omega * p * (c * c * c2 * c2 + 2 * c * c3 * c1 * c2 + c1 * c1) *
                   phi(zeta * std::sqrt(2 * (1 - c)));
        }
        case 1: {
            double p = (d == 2) ? zP * zP : zP * zP * zP;
            double K2 = K * K, K4 = K2 * K2;
            double poly = (1 - 2 / K2) * (1 - 2 / K2) * dll * dll + 4 * (1 / K2 - 2 / K4) * rlm * dll * dmm * c * c +
                          (4 / K4) * dmm * dmm * c * c * c * c + drr * drr * c * c -
                          2 * (1 - 2 / K2) * rlr * dll * drr * c - (4 / K2) * rmr * dmm * drr * c * c * c;
            return (pi / 2) * omega * p * poly * phi(zP * std::sqrt(2 * (1 - c)));
        }
        case 2: {
            double poly = K * K * drr * drr + 4 * dmm * dmm * c * c - 4 * K * rmr * dmm * drr * c;
            double pre = (d == 2) ? (pi / 2) * omega * zP * zP : (pi / 2) * K * omega * zP * zP * zP;
            return pre * poly * (1 - c * c) * phi(zP * std::sqrt(1 + K * K - 2 * K * c));
        }
        case 3: {
            double poly = drr * drr + (4 / (K * K)) * dmm * dmm * c * c - (4 / K) * rmr * dmm * drr * c;
            double pre = (d == 2) ? (pi / 2) * omega * zP * zP : (pi / 4 / (K * K * K)) * omega * zS * zS * zS;
            return pre * poly * (1 - c * c) * phi(zS * std::sqrt(1 + 1 / (K * K) - 2 * c / K));
        }
        case 4: {
            double ph = phi(zS * std::sqrt(2 * (1 - c)));
            if (d == 2) {
                double G = 2 * c * c - 1;
                return (pi / 2) * omega * zS * zS *
                       (drr * drr * c * c + dmm * dmm * G * G - 2 * rmr * dmm * drr * c * G) * ph;
            }
            return (pi / 4) * omega * zS * zS * zS *
                   (drr * drr * (1 + c * c) + dmm * dmm * (4 * c * c * c * c - 3 * c * c + 1) -
                    rmr * dmm * drr * 4 * c * c * c) *
                   ph;
        }
        default: return cst;
        }
    }
};

// ---------------------------------------------------------------------------------
// Globally adaptive Gauss-Kronrod (7,15) quadrature
// ---------------------------------------------------------------------------------
const double kXgk[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                        0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                        0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                        0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
const double kWgk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                        0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                        0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                        0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
const double kWg[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                       0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

struct Piece {
    double a, b, val, err;
    bool operator<(const Piece &o) const { return err < o.err; }
};

Piece gk15(const std::function<double(double)> &f, double a, double b)
{
    double c = 0.5 * (a + b), hl = 0.5 * (b - a);
    double fc = f(c);
    double rk = fc * kWgk[7], rg = fc * kWg[3];
    for (int j = 0; j < 7; ++j) {
        double dx = hl * kXgk[j];
        double f1 = f(c - dx), f2 = f(c + dx);
        rk += kWgk[j] * (f1 + f2);
        if (j & 1) rg += kWg[j / 2] * (f1 + f2);
    }
    return Piece{a, b, rk * hl, std::fabs((rk - rg) * hl)};
}

double integrate(const std::function<double(double)> &f, double a, double b)
{
    std::priority_queue<Piece> q;
    double total = 0, err = 0;
    const int n0 = 10; // MATLAB's integral also starts from 10 subintervals
    for (int i = 0; i < n0; ++i) {
        double x0 = a + (b - a) * i / n0, x1 = (i == n0 - 1) ? b : a + (b - a) * (i + 1) / n0;
        Piece p = gk15(f, x0, x1);
        total += p.val;
        err += p.err;
        q.push(p);
    }
    for (int it = 0; it < 4000 && err > std::max(1e-15, 1e-13 * std::fabs(total)); ++it) {
        Piece p = q.top();
        q.pop();
        double m = 0.5 * (p.a + p.b);
        Piece l = gk15(f, p.a, m), r = gk15(f, m, p.b);
        total += l.val + r.val - p.val;
        err += l.err + r.err - p.err;
        q.push(l);
        q.push(r);
    }
    // re-sum to remove accumulated cancellation in the running total
    double s = 0;
    while (!q.empty()) {
        s += q.top().val;
        q.pop();
    }
    return s;
}

// total and momentum-transfer cross-sections (prepareSigmaOne, MaterialClass.m:2447-2452)
void sigma_totals(const Sigma &s, int d, double *S, double *Sp)
{
    const double pi = kPi;
    std::function<double(double)> f = [&](double t) { return s(t); };
    if (d == 2) {
        *S = 2 * integrate(f, 0, pi);
        *Sp = 2 * integrate([&](double t) { return s(t) * std::cos(t); }, 0, pi);
    } else {
        *S = 2 * pi * integrate([&](double t) { return s(t) * std::sin(t); }, 0, pi);
        *Sp = 2 * pi * integrate([&](double t) { return s(t) * std::sin(t) * std::cos(t); }, 0, pi);
    }
}

struct OneTable {
    double Sigma = 0, Sigmapr = 0;
    std::vector<double> cdf, theta;
};

// prepareSigmaOne (MaterialClass.m:2443-2463)
void prepare_one(const Sigma &s, int d, int64_t nth, OneTable *out)
{
    const double pi = kPi;
    double S, Sp;
    sigma_totals(s, d, &S, &Sp);
    out->Sigma = S;
    out->Sigmapr = Sp;
    const double dx = pi / (double)(nth - 1);
    const double scale = pi / (double)nth;
    std::vector<double> cdf((size_t)nth);
    double acc = 0;
    for (int64_t i = 0; i < nth; ++i) {
        double t = (i == nth - 1) ? pi : dx * (double)i;
        double p = (d == 2) ? (2 / S) * s(t) : (2 * pi / S) * std::sin(t) * s(t);
        if (!std::isnan(p)) acc += p; // cumsum(..., "omitnan")
        cdf[(size_t)i] = acc * scale;
    }
    std::vector<char> keep((size_t)nth, 0);
    for (int64_t i = 0; i + 1 < nth; ++i)
        if (cdf[(size_t)i + 1] - cdf[(size_t)i] > 1e-8) keep[(size_t)i] = keep[(size_t)i + 1] = 1;
    out->cdf.clear();
    out->theta.clear();
    for (int64_t i = 0; i < nth; ++i) {
        if (!keep[(size_t)i]) continue;
        double c = cdf[(size_t)i];
        if (!out->cdf.empty() && !(c > out->cdf.back())) continue; // strictly increasing knots
        out->cdf.push_back(c);
        out->theta.push_back((i == nth - 1) ? pi : dx * (double)i);
    }
}

} // namespace

int validate_tables(const rtmc_tables *t, std::string *err)
{
    if (!t) return fail(err, RTMC_ERR_NOTABLES, "tables handle is NULL");
    if (t->n_tables != 1 && t->n_tables != 4) return fail(err, RTMC_ERR_NOTABLES, "tables must hold 1 or 4 tables");
    for (int i = 0; i < t->n_tables; ++i) {
        if (t->cdf[i].size() < 2) return fail(err, RTMC_ERR_NOTABLES, "an inverse-CDF table has fewer than 2 knots");
        for (size_t j = 1; j < t->cdf[i].size(); ++j)
            if (!(t->cdf[i][j] > t->cdf[i][j - 1]))
                return fail(err, RTMC_ERR_NOTABLES, "inverse-CDF knots must be strictly increasing and finite");
        for (double th : t->theta[i])
            if (!std::isfinite(th)) return fail(err, RTMC_ERR_NOTABLES, "inverse-CDF angles must be finite");
    }
    return RTMC_OK;
}

} // namespace rtmc

using namespace rtmc;

namespace rtmc {
namespace {

// the cross-section of table i (0 for acoustics; PP, PS, SP, SS for elastics) of material m
int material_sigma(const rtmc_material *m, int i, Sigma *out)
{
    if (m->d != 2 && m->d != 3) return fail(nullptr, RTMC_ERR_ARG, "dimension must be 2 or 3");
    const bool ac = m->acoustics != 0;
    if (i < 0 || i >= (ac ? 1 : 4)) return fail(nullptr, RTMC_ERR_ARG, "table index out of range");
    Sigma base;
    base.d = m->d;
    if (m->psdf == RTMC_PSDF_CONST) {
        base.which = 5;
        base.cst = m->sigma_const[i];
        *out = base;
        return RTMC_OK;
    }
    if (!(m->freq > 0) || !(m->lc > 0)) return fail(nullptr, RTMC_ERR_ARG, "frequency and lc must be positive");
    int st = make_psdf(*m, &base.phi, nullptr);
    if (st) return st;
    base.omega = 2 * kPi * m->freq;
    if (ac) {
        if (!(m->v[0] > 0)) return fail(nullptr, RTMC_ERR_ARG, "acoustic speed must be positive");
        if (std::fabs(m->corr[0]) > 1)
            return fail(nullptr, RTMC_ERR_ARG, "Absolute value of corr(kappa,rho) should be less than 1!");
        base.zeta = base.omega / m->v[0] * m->lc;
        base.c1 = m->cv[0];
        base.c2 = m->cv[1];
        base.c3 = m->corr[0];
    } else {
        if (!(m->v[0] > 0) || !(m->v[1] > 0)) return fail(nullptr, RTMC_ERR_ARG, "vp and vs must be positive");
        for (int k = 0; k < 3; ++k)
            if (std::fabs(m->corr[k]) > 1)
                return fail(nullptr, RTMC_ERR_ARG, "Absolute values of correlation coefficients should be less than 1!");
        base.K = m->v[0] / m->v[1];
        base.zP = base.omega / m->v[0] * m->lc;
        base.zS = base.K * base.zP;
        base.dll = m->cv[0];
        base.dmm = m->cv[1];
        base.drr = m->cv[2];
        base.rlm = m->corr[0];
        base.rlr = m->corr[1];
        base.rmr = m->corr[2];
    }
    base.which = ac ? 0 : 1 + i;
    *out = base;
    return RTMC_OK;
}

} // namespace
} // namespace rtmc

extern "C" int rtmc_sigma_eval(const rtmc_material *m, int32_t table, int64_t n, const double *theta, double *sigma)
{
    if (!m || (n > 0 && (!theta || !sigma)) || n < 0) return fail(nullptr, RTMC_ERR_ARG, "rtmc_sigma_eval: bad argument");
    Sigma s;
    int st = material_sigma(m, table, &s);
    if (st) return st;
    for (int64_t k = 0; k < n; ++k) sigma[k] = s(theta[k]);
    return RTMC_OK;
}

extern "C" int rtmc_sigma_total(const rtmc_material *m, double *Sigma_out, double *Sigmapr_out)
{
    if (!m || !Sigma_out || !Sigmapr_out) return fail(nullptr, RTMC_ERR_ARG, "rtmc_sigma_total: NULL argument");
    const int nt = m->acoustics ? 1 : 4;
    for (int i = 0; i < nt; ++i) {
        Sigma s;
        int st = material_sigma(m, i, &s);
        if (st) return st;
        sigma_totals(s, m->d, Sigma_out + i, Sigmapr_out + i);
    }
    return RTMC_OK;
}

extern "C" int rtmc_tables_build(const rtmc_material *m, rtmc_tables **out)
{
    if (!m || !out) return fail(nullptr, RTMC_ERR_ARG, "rtmc_tables_build: NULL argument");
    *out = nullptr;
    if (m->d != 2 && m->d != 3) return fail(nullptr, RTMC_ERR_ARG, "dimension must be 2 or 3");
    int64_t nth = m->n_theta > 0 ? m->n_theta : 1000000;
    if (nth < 16) return fail(nullptr, RTMC_ERR_ARG, "n_theta must be at least 16");
    const bool ac = m->acoustics != 0;
    Sigma sig[4];
    for (int i = 0; i < (ac ? 1 : 4); ++i) {
        int st = material_sigma(m, i, &sig[i]);
        if (st) return st;
    }
    auto *t = new (std::nothrow) rtmc_tables();
    if (!t) return fail(nullptr, RTMC_ERR_ALLOC, "out of host memory");
    t->n_tables = ac ? 1 : 4;
    OneTable one[4];
    std::vector<std::thread> th;
    for (int i = 0; i < t->n_tables; ++i)
        th.emplace_back([s = sig[i], &one, i, d = m->d, nth]() { prepare_one(s, d, nth, &one[i]); });
    for (auto &x : th) x.join();
    for (int i = 0; i < t->n_tables; ++i) {
        t->cdf[i] = std::move(one[i].cdf);
        t->theta[i] = std::move(one[i].theta);
        t->info.Sigma[i] = one[i].Sigma;
        t->info.Sigmapr[i] = one[i].Sigmapr;
        t->info.n_knots[i] = (int64_t)t->cdf[i].size();
    }
    t->info.n_tables = t->n_tables;
    const double d = (double)m->d;
    rtmc_tables_info &I = t->info;
    if (ac) {
        double S = I.Sigma[0], Sp = I.Sigmapr[0], v = (m->psdf == RTMC_PSDF_CONST && !(m->v[0] > 0)) ? 1.0 : m->v[0];
        I.diffusivity = v * v / (d * (S - Sp));
        I.mean_free_time[0] = I.mean_free_time[1] = 1.0 / S;
        I.transport_mean_free_path[0] = I.transport_mean_free_path[1] = d * I.diffusivity / v;
        I.g = 1.0 - (v / S) / I.transport_mean_free_path[0];
        I.p2p = I.s2s = 1.0;
    } else {
        const double *S = I.Sigma, *Sp = I.Sigmapr;
        double vp = m->v[0], vs = m->v[1], K = vp / vs;
        I.mean_free_time[0] = 1.0 / (S[0] + S[1]);
        I.mean_free_time[1] = 1.0 / (S[2] + S[3]);
        double den = (S[0] + S[1] - Sp[0]) * (S[3] + S[2] - Sp[3]) - Sp[1] * Sp[2];
        double tP = (vp * (S[3] + S[2] - Sp[3]) + vs * Sp[1]) / den;
        double tS = (vs * (S[0] + S[1] - Sp[0]) + vp * Sp[2]) / den;
        I.transport_mean_free_path[0] = tP;
        I.transport_mean_free_path[1] = tS;
        double Dp = vp * tP / d, Ds = vs * tS / d;
        I.diffusivity = (Dp + 2 * K * K * K * Ds) / (1 + 2 * K * K * K);
        I.p2p = S[0] / (S[0] + S[1]);
        I.s2s = S[3] / (S[2] + S[3]);
    }
    // the knots are checked once here; the handle is immutable afterwards
    std::string err;
    const int st = validate_tables(t, &err);
    if (st) {
        delete t;
        return fail(nullptr, st, err);
    }
    t->gen = next_generation();
    *out = t;
    return RTMC_OK;
}

extern "C" int rtmc_tables_from_knots(int32_t n_tables, const int64_t *n_knots, const double *const *cdf,
                                      const double *const *theta, rtmc_tables **out)
{
    if (!out || !n_knots || !cdf || !theta) return fail(nullptr, RTMC_ERR_ARG, "rtmc_tables_from_knots: NULL argument");
    *out = nullptr;
    if (n_tables != 1 && n_tables != 4) return fail(nullptr, RTMC_ERR_ARG, "n_tables must be 1 or 4");
    auto *t = new (std::nothrow) rtmc_tables();
    if (!t) return fail(nullptr, RTMC_ERR_ALLOC, "out of host memory");
    t->n_tables = n_tables;
    t->info.n_tables = n_tables;
    for (int i = 0; i < n_tables; ++i) {
        if (n_knots[i] < 2 || !cdf[i] || !theta[i]) {
            delete t;
            return fail(nullptr, RTMC_ERR_ARG, "each table needs at least 2 knots");
        }
        t->cdf[i].assign(cdf[i], cdf[i] + n_knots[i]);
        t->theta[i].assign(theta[i], theta[i] + n_knots[i]);
        t->info.n_knots[i] = n_knots[i];
    }
    std::string err;
    int st = validate_tables(t, &err); // once: the handle is immutable afterwards
    if (st) {
        delete t;
        return fail(nullptr, st, err);
    }
    t->gen = next_generation();
    *out = t;
    return RTMC_OK;
}

extern "C" int rtmc_tables_get_info(const rtmc_tables *t, rtmc_tables_info *info)
{
    if (!t || !info) return fail(nullptr, RTMC_ERR_ARG, "rtmc_tables_get_info: NULL argument");
    *info = t->info;
    return RTMC_OK;
}

extern "C" int rtmc_tables_get_knots(const rtmc_tables *t, int32_t i, double *cdf, double *theta)
{
    if (!t || i < 0 || i >= t->n_tables) return fail(nullptr, RTMC_ERR_ARG, "rtmc_tables_get_knots: bad table index");
    if (cdf) std::memcpy(cdf, t->cdf[i].data(), t->cdf[i].size() * sizeof(double));
    if (theta) std::memcpy(theta, t->theta[i].data(), t->theta[i].size() * sizeof(double));
    return RTMC_OK;
}

extern "C" int rtmc_tables_eval(const rtmc_tables *t, int32_t i, int64_t n, const double *u, double *out)
{
    if (!t || i < 0 || i >= t->n_tables || n < 0 || (n > 0 && (!u || !out)))
        return fail(nullptr, RTMC_ERR_ARG, "rtmc_tables_eval: bad argument");
    const std::vector<double> &c = t->cdf[i], &th = t->theta[i];
    const int64_t nk = (int64_t)c.size();
    for (int64_t k = 0; k < n; ++k) {
        double x = u[k];
        int64_t lo = (int64_t)(std::upper_bound(c.begin(), c.end(), x) - c.begin()) - 1;
        lo = std::min<int64_t>(std::max<int64_t>(lo, 0), nk - 2);
        out[k] = th[(size_t)lo] + (x - c[(size_t)lo]) / (c[(size_t)lo + 1] - c[(size_t)lo]) *
                                      (th[(size_t)lo + 1] - th[(size_t)lo]);
    }
    return RTMC_OK;
}

extern "C" void rtmc_tables_free(rtmc_tables *t)
{
    if (!t) return;
    for (int k = 0; k < 2; ++k)
        if (t->image_pinned[k]) cudaHostUnregister(t->image[k].data());
    delete t;
}

// ---------------------------------------------------------------------------------
// Zoeppritz, solid over fluid (ZoeppritzFluid.m:47-222)
// ---------------------------------------------------------------------------------
namespace {
using cd = std::complex<double>;

bool solve3(cd A[3][3], cd b[3], cd x[3])
{
    int p[3] = {0, 1, 2};
    for (int c = 0; c < 3; ++c) {
        int piv = c;
        for (int r = c + 1; r < 3; ++r)
            if (std::abs(A[p[r]][c]) > std::abs(A[p[piv]][c])) piv = r;
        std::swap(p[c], p[piv]);
        if (std::abs(A[p[c]][c]) == 0.0) return false;
        for (int r = c + 1; r < 3; ++r) {
            cd f = A[p[r]][c] / A[p[c]][c];
            for (int k = c; k < 3; ++k) A[p[r]][k] -= f * A[p[c]][k];
            b[p[r]] -= f * b[p[c]];
        }
    }
    for (int c = 2; c >= 0; --c) {
        cd s = b[p[c]];
        for (int k = c + 1; k < 3; ++k) s -= A[p[c]][k] * x[k];
        x[c] = s / A[p[c]][c];
    }
    return true;
}

cd casin(double x) { return std::asin(cd(x, 0.0)); }
} // namespace

extern "C" int rtmc_zoeppritz_fluid(int32_t n, const double *ang, double vp1, double vs1, double rho1, double vp2,
                                    double vs2, double rho2, double *out)
{
    if (n < 0 || (n > 0 && (!ang || !out))) return fail(nullptr, RTMC_ERR_ARG, "rtmc_zoeppritz_fluid: bad argument");
    if (!(vp1 > 0) || !(vs1 > 0) || !(rho1 > 0) || !(vp2 > 0) || !(rho2 > 0) || vs2 != 0.0)
        return fail(nullptr, RTMC_ERR_ARG,
                    "rtmc_zoeppritz_fluid: needs vp1, vs1, rho1, vp2, rho2 > 0 and a fluid (vs2 = 0)");
    for (int i = 0; i < n; ++i) {
        const double a = ang[i] * kPi / 180.0;
        // P incidence
        double p = std::sin(a) / vp1;
        cd phi1 = a, psi1 = casin(vs1 * p), phi2 = casin(vp2 * p), psi2 = casin(vs2 * p);
        cd A[3][3] = {{std::cos(phi1), -std::sin(psi1), std::cos(phi2)},
                      {-std::cos(2.0 * psi1), vs1 / vp1 * std::sin(2.0 * psi1),
                       (rho2 * vp2 / (rho1 * vp1)) * std::cos(2.0 * psi2)},
                      {std::sin(2.0 * phi1), vp1 / vs1 * std::cos(2.0 * psi1),
                       (rho2 * vp1 * vs2 * vs2 / (rho1 * vp2 * vs1 * vs1)) * std::sin(2.0 * phi2)}};
        cd psi0 = casin(vs1 * std::sin(a) / vp1);
        cd b[3] = {std::cos(a), std::cos(2.0 * psi0), std::sin(2.0 * a)};
        cd x[3] = {0.0, 0.0, 0.0};
        if (!solve3(A, b, x)) return fail(nullptr, RTMC_ERR_ARG, "singular Zoeppritz system");
        double cphi1 = std::cos(phi1).real();
        out[0 * n + i] = std::norm(x[0]);
        out[1 * n + i] = (a == 0.0) ? 0.0 : (rho1 * vs1 * std::cos(psi1).real()) / (rho1 * vp1 * cphi1) * std::norm(x[1]);
        out[2 * n + i] = (rho2 * vp2 * std::cos(phi2).real()) / (rho1 * vp1 * cphi1) * std::norm(x[2]);
        // SV incidence
        p = std::sin(a) / vs1;
        phi1 = casin(vp1 * p);
        psi1 = a;
        phi2 = casin(vp2 * p);
        psi2 = casin(vs2 * p);
        cd B[3][3] = {{std::cos(phi1), -std::sin(psi1), std::cos(phi2)},
                      {-std::cos(2.0 * psi1), vs1 / vp1 * std::sin(2.0 * psi1),
                       (rho2 * vp2 / (rho1 * vp1)) * std::cos(2.0 * psi2)},
                      {std::sin(2.0 * phi1), (vp1 / vs1) * std::cos(2.0 * psi1),
                       (rho2 * vp1 * vs2 * vs2 / (rho1 * vp2 * vs1 * vs1)) * std::sin(2.0 * phi2)}};
        cd c[3] = {-std::sin(a), -vs1 * std::sin(2.0 * a) / vp1, vp1 * std::cos(2.0 * a) / vs1};
        if (!solve3(B, c, x)) return fail(nullptr, RTMC_ERR_ARG, "singular Zoeppritz system");
        double cpsi1 = std::cos(psi1).real();
        out[4 * n + i] = (a == 0.0) ? 0.0 : (rho1 * vp1 * std::cos(phi1).real()) / (rho1 * vs1 * cpsi1) * std::norm(x[0]);
        out[3 * n + i] = std::norm(x[1]);
        out[5 * n + i] = (rho2 * vp2 * std::cos(phi2).real()) / (rho1 * vs1 * cpsi1) * std::norm(x[2]);
        out[6 * n + i] = 1.0; // SH on a fluid: total reflection (ZoeppritzFluid.m:208-219)
    }
    return RTMC_OK;
}
