/*
 * rtmc_mex.c -- MATLAB / Octave gateway of librtmc.
 *
 * The seam of radiativeTransfer.m: its packet x time loop (radiativeTransfer.m:40-158)
 * becomes one call of this gateway, while initializeObservation, prepareSigma and the
 * normalisation (radiativeTransfer.m:161-191) stay in MATLAB (see radiativeTransfer.m,
 * rtmcProblem.m, rtmcKnots.m and rtmcEdges.m beside this file).
 *
 *   E          = rtmc_mex('forward', P, knots, edges)
 *   [E, stats] = rtmc_mex('forward', P, knots, edges)
 *   [g, stats] = rtmc_mex('gradient', P, knots, edges, W, S)
 *                rtmc_mex('reset')                         % releases the GPU context
 *
 *   P      1x1 struct with the fields of rtmc_problem (include/rtmc.h), as rtmcProblem.m
 *          fills them: scalars as doubles, fixed-size vectors as double vectors,
 *          bnd_dir / bnd_val / bnd_absorb as vectors of the boundaries (may be empty),
 *          zoe_rpp / zoe_rsvsv (181 values, elastic problems with a reflective boundary),
 *          src_radial_cdf / src_radial_r (a radial source profile, may be empty).
 *   knots  1x1 cell (acoustics) or 2x2 cell (elastics, {old mode, new mode}) of [cdf theta]
 *          matrices: the knots of material.invcdf (MaterialClass.m:2462), rtmcKnots.m.
 *   edges  1x4 cell {binX, binY, binZ, binPsi} of initializeObservation.m (rtmcEdges.m).
 *   E      uint32 column of P.hist_len counts, column-major [N1 N2 Nt modes] as the E of
 *          initializeObservation.m:133, saturating like MATLAB's uint32 additions
 *          (rtmc_forward_u32).
 *   W      P.hist_len adjoint weights dL/dcount (double); S struct with dlogsigma
 *          [n_theta x n_params] and dlogSigma [n_params] (rtmc_score); g the 1 x n_params
 *          gradient (rtmc_gradient; new: the reference has no gradient).
 *   stats  struct with the rtmc_stats fields.
 *
 * Build:  mex rtmc_mex.c -I<repo>/include -L<repo>/radiativetransfermontecarlo_gb300 -lrtmc
 *         (Octave: mkoctfile --mex with the same flags).
 *
 * All MATLAB API calls happen on the calling thread; the library returns a status and
 * never raises, so mexErrMsgIdAndTxt is called only after librtmc has returned.
 */
#include "mex.h"
#include "rtmc.h"

#include <math.h>
#include <stdint.h>
#include <string.h>

static rtmc_context *g_ctx = NULL;

static void release_context(void)
{
    if (g_ctx) rtmc_destroy(g_ctx);
    g_ctx = NULL;
}

static const mxArray *field(const mxArray *s, const char *name, int required)
{
    const mxArray *a = mxGetField(s, 0, name);
    if (required && (!a || mxIsEmpty(a))) mexErrMsgIdAndTxt("rtmc:field", "P.%s is required", name);
    return a && !mxIsEmpty(a) ? a : NULL;
}

static const double *doubles(const mxArray *a, const char *name)
{
    if (!mxIsDouble(a) || mxIsComplex(a)) mexErrMsgIdAndTxt("rtmc:type", "%s must be a real double array", name);
    return mxGetPr(a);
}

static double scalar(const mxArray *s, const char *name, double dflt, int required)
{
    const mxArray *a = field(s, name, required);
    if (!a) return dflt;
    if (mxGetNumberOfElements(a) != 1) mexErrMsgIdAndTxt("rtmc:type", "P.%s must be a scalar", name);
    return doubles(a, name)[0];
}

static int64_t integer(const mxArray *s, const char *name, int64_t dflt, int required)
{
    const double v = scalar(s, name, (double)dflt, required);
    if (!(v == floor(v)) || fabs(v) > 9007199254740992.0)
        mexErrMsgIdAndTxt("rtmc:type", "P.%s must be an integer below 2^53", name);
    return (int64_t)v;
}

/* the n values of P.<name> into out; the field must hold exactly n values */
static void vector(const mxArray *s, const char *name, double *out, size_t n, int required)
{
    const mxArray *a = field(s, name, required);
    if (!a) return;
    if (mxGetNumberOfElements(a) != n) mexErrMsgIdAndTxt("rtmc:type", "P.%s must hold %d values", name, (int)n);
    memcpy(out, doubles(a, name), n * sizeof(double));
}

/* the rtmc_problem of struct S and cell E (pointers into MATLAB-owned memory) */
static void read_problem(const mxArray *S, const mxArray *E, rtmc_problem *P)
{
    if (!mxIsStruct(S) || mxGetNumberOfElements(S) != 1) mexErrMsgIdAndTxt("rtmc:args", "P must be a 1x1 struct");
    if (!mxIsCell(E) || mxGetNumberOfElements(E) != 4) mexErrMsgIdAndTxt("rtmc:args", "edges must be a 1x4 cell");
    memset(P, 0, sizeof *P);
    P->d = (int32_t)integer(S, "d", 3, 1);
    P->frame = (int32_t)integer(S, "frame", RTMC_FRAME_SPHERICAL, 1);
    P->acoustics = (int32_t)integer(S, "acoustics", 1, 1);
    P->precision = (int32_t)integer(S, "precision", RTMC_FP32, 0);
    P->src_dir = (int32_t)integer(S, "src_dir", 0, 0);
    P->polarization = (int32_t)integer(S, "polarization", 0, 0);
    P->n_sub = (int32_t)integer(S, "n_sub", 1, 1);
    P->n_obs = (int32_t)integer(S, "n_obs", 1, 1);
    P->hist_shift = (int32_t)integer(S, "hist_shift", 0, 0);
    P->max_events = (int32_t)integer(S, "max_events", 0, 0);
    P->n_particles = integer(S, "n_particles", 0, 1);
    P->pid0 = integer(S, "pid0", 0, 0);
    P->seed = (uint64_t)integer(S, "seed", 0, 0);
    vector(S, "src_pos", P->src_pos, 3, 0);
    P->src_lambda = scalar(S, "src_lambda", 0.0, 0);
    vector(S, "v", P->v, 2, 1);
    vector(S, "mft", P->mft, 2, 1);
    P->p2p = scalar(S, "p2p", 1.0, 0);
    P->s2s = scalar(S, "s2s", 1.0, 0);
    vector(S, "qrate", P->qrate, 2, 0);
    P->h = scalar(S, "h", 0.0, 1);
    {
        double am[4] = {0, 0, 0, 0}, as[4] = {0, 0, 0, 0};
        vector(S, "axis_mode", am, 4, 1);
        vector(S, "axis_stride", as, 4, 1);
        for (int a = 0; a < 4; ++a) {
            P->axis_mode[a] = (int32_t)am[a];
            P->axis_stride[a] = (int64_t)as[a];
            const mxArray *e = mxGetCell(E, a);
            if (P->axis_mode[a] != RTMC_AXIS_IGNORED) {
                if (!e || mxIsEmpty(e)) mexErrMsgIdAndTxt("rtmc:edges", "edges{%d} is empty for an observed axis", a + 1);
                P->axis_edges[a] = doubles(e, "edges");
                P->axis_nedges[a] = (int32_t)mxGetNumberOfElements(e);
            }
        }
    }
    P->time_stride = integer(S, "time_stride", 0, 1);
    P->mode_stride = integer(S, "mode_stride", 0, 0);
    P->hist_len = integer(S, "hist_len", 0, 1);
    {
        const mxArray *bd = field(S, "bnd_dir", 0), *bv = field(S, "bnd_val", 0), *ba = field(S, "bnd_absorb", 0);
        const size_t nb = bd ? mxGetNumberOfElements(bd) : 0;
        if (nb > RTMC_MAX_BND) mexErrMsgIdAndTxt("rtmc:bnd", "at most %d boundaries", RTMC_MAX_BND);
        if (nb && (!bv || mxGetNumberOfElements(bv) != nb || (ba && mxGetNumberOfElements(ba) != nb)))
            mexErrMsgIdAndTxt("rtmc:bnd", "bnd_dir, bnd_val and bnd_absorb must have one value per boundary");
        P->n_bnd = (int32_t)nb;
        for (size_t b = 0; b < nb; ++b) {
            P->bnd_dir[b] = (int32_t)doubles(bd, "bnd_dir")[b];
            P->bnd_val[b] = doubles(bv, "bnd_val")[b];
            P->bnd_absorb[b] = ba ? (int32_t)doubles(ba, "bnd_absorb")[b] : 0;
        }
    }
    vector(S, "zoe_rpp", P->zoe_rpp, RTMC_ZOE_N, 0);
    vector(S, "zoe_rsvsv", P->zoe_rsvsv, RTMC_ZOE_N, 0);
    P->src_type = (int32_t)integer(S, "src_type", RTMC_SOURCE_POINT, 0);
    P->src_aperture = (int32_t)integer(S, "src_aperture", RTMC_APERTURE_RECTANGLE, 0);
    {
        const mxArray *rc = field(S, "src_radial_cdf", 0), *rr = field(S, "src_radial_r", 0);
        if (rc || rr) {
            if (!rc || !rr || mxGetNumberOfElements(rc) != mxGetNumberOfElements(rr))
                mexErrMsgIdAndTxt("rtmc:source", "src_radial_cdf and src_radial_r must have the same length");
            P->src_radial_n = (int32_t)mxGetNumberOfElements(rc);
            P->src_radial_cdf = doubles(rc, "src_radial_cdf");
            P->src_radial_r = doubles(rr, "src_radial_r");
        }
    }
    vector(S, "src_normal", P->src_normal, 3, 0);
    vector(S, "src_u", P->src_u, 3, 0);
    vector(S, "src_v", P->src_v, 3, 0);
    vector(S, "src_extent", P->src_extent, 2, 0);
}

/* tables handle wrapping the [cdf theta] matrices of a 1x1 or 2x2 cell */
static rtmc_tables *read_tables(const mxArray *K)
{
    if (!mxIsCell(K) || (mxGetNumberOfElements(K) != 1 && mxGetNumberOfElements(K) != 4))
        mexErrMsgIdAndTxt("rtmc:knots", "knots must be a 1x1 or 2x2 cell of [cdf theta] matrices");
    const int nt = (int)mxGetNumberOfElements(K);
    int64_t nk[4];
    const double *cdf[4], *th[4];
    for (int t = 0; t < nt; ++t) {
        /* table t = 2 * old + new; the cell is column-major: {old+1, new+1} at old + 2 new */
        const mxArray *c = mxGetCell(K, nt == 1 ? 0 : (t / 2) + 2 * (t % 2));
        if (!c || mxGetN(c) != 2 || mxGetM(c) < 2) mexErrMsgIdAndTxt("rtmc:knots", "each knot table is an n x 2 [cdf theta] matrix");
        nk[t] = (int64_t)mxGetM(c);
        cdf[t] = doubles(c, "knots");
        th[t] = cdf[t] + nk[t];
    }
    rtmc_tables *T = NULL;
    if (rtmc_tables_from_knots(nt, nk, cdf, th, &T) != RTMC_OK)
        mexErrMsgIdAndTxt("rtmc:knots", "%s", rtmc_last_error(NULL));
    return T;
}

static mxArray *stats_struct(const rtmc_stats *st)
{
    static const char *names[] = {"scatter_events", "boundary_hits", "kills", "absorbed", "observations",
                                  "conversions", "device_status", "launches", "kernel_ms", "fold_ms", "total_ms"};
    const double vals[] = {(double)st->scatter_events, (double)st->boundary_hits, (double)st->kills,
                           (double)st->absorbed, (double)st->observations, (double)st->conversions,
                           (double)st->device_status, (double)st->launches, st->kernel_ms, st->fold_ms, st->total_ms};
    const int n = (int)(sizeof names / sizeof names[0]);
    mxArray *s = mxCreateStructMatrix(1, 1, n, names);
    for (int i = 0; i < n; ++i) mxSetField(s, 0, names[i], mxCreateDoubleScalar(vals[i]));
    return s;
}

static void ensure_context(void)
{
    if (g_ctx) return;
    if (rtmc_create(0, &g_ctx) != RTMC_OK) {
        g_ctx = NULL;
        mexErrMsgIdAndTxt("rtmc:init", "%s", rtmc_last_error(NULL));
    }
    mexAtExit(release_context);
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    char cmd[16] = {0};
    if (nrhs < 1 || !mxIsChar(prhs[0]) || mxGetString(prhs[0], cmd, sizeof cmd) != 0)
        mexErrMsgIdAndTxt("rtmc:args", "usage: rtmc_mex('forward' | 'gradient' | 'reset', ...)");
    if (strcmp(cmd, "reset") == 0) {
        release_context();
        return;
    }
    const int forward = strcmp(cmd, "forward") == 0, gradient = strcmp(cmd, "gradient") == 0;
    if (!forward && !gradient) mexErrMsgIdAndTxt("rtmc:args", "unknown command '%s'", cmd);
    if ((forward && nrhs != 4) || (gradient && nrhs != 6))
        mexErrMsgIdAndTxt("rtmc:args", forward ? "rtmc_mex('forward', P, knots, edges)"
                                               : "rtmc_mex('gradient', P, knots, edges, W, S)");
    if (nlhs > 2) mexErrMsgIdAndTxt("rtmc:args", "at most two outputs");
    rtmc_problem P;
    read_problem(prhs[1], prhs[3], &P);
    if (P.hist_len <= 0) mexErrMsgIdAndTxt("rtmc:args", "P.hist_len must be positive");
    rtmc_score sc;
    const double *W = NULL;
    if (gradient) {
        if (!mxIsDouble(prhs[4]) || (int64_t)mxGetNumberOfElements(prhs[4]) != P.hist_len)
            mexErrMsgIdAndTxt("rtmc:args", "W must hold P.hist_len doubles");
        W = mxGetPr(prhs[4]);
        if (!mxIsStruct(prhs[5])) mexErrMsgIdAndTxt("rtmc:args", "S must be a struct with dlogsigma and dlogSigma");
        memset(&sc, 0, sizeof sc);
        const mxArray *D = field(prhs[5], "dlogsigma", 1), *dS = field(prhs[5], "dlogSigma", 1);
        sc.n_theta = (int32_t)mxGetM(D);
        sc.n_params = (int32_t)mxGetN(D);
        if (sc.n_params < 1 || sc.n_params > RTMC_MAX_PARAMS || (int)mxGetNumberOfElements(dS) != sc.n_params)
            mexErrMsgIdAndTxt("rtmc:args", "S.dlogsigma is n_theta x n_params (n_params <= %d), S.dlogSigma n_params",
                              RTMC_MAX_PARAMS);
        sc.dlogsigma = doubles(D, "S.dlogsigma"); /* column-major n_theta x n_params = [param][theta] */
        for (int q = 0; q < sc.n_params; ++q) sc.dlogSigma[q] = doubles(dS, "S.dlogSigma")[q];
    }
    ensure_context();
    rtmc_tables *T = read_tables(prhs[2]);
    rtmc_stats st;
    memset(&st, 0, sizeof st);
    mxArray *out;
    int status;
    if (forward) {
        out = mxCreateNumericMatrix((mwSize)P.hist_len, 1, mxUINT32_CLASS, mxREAL);
        status = rtmc_forward_u32(g_ctx, &P, T, (uint32_t *)mxGetData(out), &st);
    } else {
        out = mxCreateDoubleMatrix(1, (mwSize)sc.n_params, mxREAL);
        status = rtmc_gradient(g_ctx, &P, T, &sc, W, mxGetPr(out), &st);
    }
    rtmc_tables_free(T);
    if (status != RTMC_OK) {
        mxDestroyArray(out);
        mexErrMsgIdAndTxt(forward ? "rtmc:forward" : "rtmc:gradient", "%s", rtmc_last_error(g_ctx));
    }
    plhs[0] = out;
    if (nlhs > 1) plhs[1] = stats_struct(&st);
}
