/*
 * rtmc.h -- C ABI of librtmc, the GB300 radiative-transfer Monte Carlo engine.
 *
 * Plain C: fixed-width integers, doubles and pointers only.  Every entry point returns
 * an int status (RTMC_OK == 0); on failure rtmc_last_error() gives the message.  A
 * context is used by one host thread at a time; independent contexts may run side by
 * side (one per MATLAB parfor worker, say).
 *
 * Reference: cottereau/RadiativeTransferMonteCarlo (MATLAB).  Each entry point names
 * the reference code it replaces.
 */
#ifndef RTMC_H
#define RTMC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTMC_ABI_VERSION 2
#define RTMC_MAX_BND 4
#define RTMC_ZOE_N 181 /* Zoeppritz table on 0:0.5:90 degrees (MaterialClass.m:1809) */
#define RTMC_MAX_RADIAL 65536 /* knots of a radial source profile */

enum rtmc_status {
    RTMC_OK = 0,
    RTMC_ERR_ARG = 1,      /* invalid argument (message says which) */
    RTMC_ERR_CUDA = 2,     /* CUDA runtime error */
    RTMC_ERR_ALLOC = 3,    /* host or device allocation failed */
    RTMC_ERR_DEVICE = 4,   /* a kernel reported an error status (bounds, watchdog) */
    RTMC_ERR_NOTABLES = 5  /* tables handle missing or incompatible with the problem */
};

enum rtmc_psdf {
    RTMC_PSDF_EXP = 0,        /* MaterialClass.Exponential, MaterialClass.m:479-517 */
    RTMC_PSDF_GAUSSIAN = 1,   /* MaterialClass.Gaussian, :560-599 */
    RTMC_PSDF_POWER_LAW = 2,  /* MaterialClass.PowerLaw, :519-558 */
    RTMC_PSDF_TRIANGULAR = 3, /* MaterialClass.Triangular, :601-630 (3D only) */
    RTMC_PSDF_LOW_PASS = 4,   /* MaterialClass.LowPass, :632-662 (3D only) */
    RTMC_PSDF_VON_KARMAN = 5, /* MaterialClass.VonKarman, :664-710 */
    RTMC_PSDF_CONST = 6       /* isotropic constant sigma per table (MaterialClass.preset, :1765-1785) */
};

enum rtmc_frame { RTMC_FRAME_CARTESIAN = 0, RTMC_FRAME_CYLINDRICAL = 1, RTMC_FRAME_SPHERICAL = 2 };
enum rtmc_axis_mode { RTMC_AXIS_IGNORED = 0, RTMC_AXIS_RANGE = 1, RTMC_AXIS_BINNED = 2 };
enum rtmc_precision { RTMC_FP32 = 0, RTMC_FP64 = 1 };
enum rtmc_source { RTMC_SOURCE_POINT = 0, RTMC_SOURCE_PLANE = 1 };
enum rtmc_aperture { RTMC_APERTURE_RECTANGLE = 0, RTMC_APERTURE_CIRCLE = 1 };

/* ---------------------------------------------------------------------------------- */
/* Host FP64 table builders                                                            */
/* ---------------------------------------------------------------------------------- */

typedef struct rtmc_tables rtmc_tables; /* opaque, host-side FP64 inverse-CDF tables */

typedef struct {
    int32_t d;          /* 2 or 3 */
    int32_t acoustics;  /* 1 acoustic, 0 elastic */
    int32_t psdf;       /* enum rtmc_psdf */
    int32_t reserved;
    double freq;        /* Hz */
    double v[2];        /* acoustic: v[0]; elastic: vp, vs */
    double cv[3];       /* acoustic: CV kappa, CV rho; elastic: CV lambda, mu, rho */
    double corr[3];     /* acoustic: corr(kappa,rho); elastic: corr(l,m), corr(l,r), corr(m,r) */
    double lc;          /* correlation length */
    double nu;          /* Hurst number (Von Karman only) */
    double sigma_const[4]; /* RTMC_PSDF_CONST: sigma of table (i,j), row-major {PP,PS,SP,SS} */
    int64_t n_theta;    /* pdf grid size; the reference uses 1e6 (0 selects 1e6) */
} rtmc_material;

typedef struct {
    int32_t n_tables;   /* 1 acoustic, 4 elastic */
    int32_t reserved;
    int64_t n_knots[4];
    double Sigma[4];    /* row-major 2x2 for elastic, Sigma[0] for acoustic */
    double Sigmapr[4];
    double mean_free_time[2];
    double p2p, s2s;
    double diffusivity;
    double transport_mean_free_path[2];
    double g;           /* acoustic anisotropy coefficient */
} rtmc_tables_info;

/* Replaces MaterialClass.prepareSigma / prepareSigmaOne / calcSigmaIsotropic / getPSDF
 * (MaterialClass.m:2379-2463, :172-359, :381-455): cross-sections, Sigma and Sigma' by
 * adaptive Gauss-Kronrod quadrature, the pdf on n_theta points, cumsum cdf scaled by
 * pi/n_theta and the diff(cdf) > 1e-8 knot filter. */
int rtmc_tables_build(const rtmc_material *material, rtmc_tables **out);

/* Wraps caller-built knots, e.g. the GridVectors/Values of MATLAB griddedInterpolant
 * objects in material.invcdf (MaterialClass.m:2462); mean free times etc. come from the
 * caller, so the info block is filled with zeros apart from n_tables and n_knots. */
int rtmc_tables_from_knots(int32_t n_tables, const int64_t *n_knots, const double *const *cdf,
                           const double *const *theta, rtmc_tables **out);

int rtmc_tables_get_info(const rtmc_tables *tables, rtmc_tables_info *info);

/* copies knots of table t (0..n_tables-1) into caller buffers of n_knots[t] doubles */
int rtmc_tables_get_knots(const rtmc_tables *tables, int32_t t, double *cdf, double *theta);

/* host evaluation of invcdf{t}(u): griddedInterpolant linear, linear extrapolation */
int rtmc_tables_eval(const rtmc_tables *tables, int32_t t, int64_t n, const double *u, double *theta);

void rtmc_tables_free(rtmc_tables *tables);

/* sigma(theta) of table `table` of a material (calcSigmaIsotropic, MaterialClass.m:172-359),
 * at n angles; and the totals Sigma, Sigma' of every table (prepareSigmaOne,
 * MaterialClass.m:2447-2452; 1 value for acoustics, 4 for elastics).  Host FP64, used to
 * differentiate the tables with respect to material parameters. */
int rtmc_sigma_eval(const rtmc_material *material, int32_t table, int64_t n, const double *theta, double *sigma);
int rtmc_sigma_total(const rtmc_material *material, double *Sigma, double *Sigmapr);

/* Replaces MaterialClass.Zoeppritz + ZoeppritzFluid (MaterialClass.m:1786-1885,
 * ZoeppritzFluid.m:1-244): energy coefficients of a solid/fluid interface at n angles.
 * out is row-major [7][n]: E_Rpp, E_Rpsv, E_Tpp, E_Rsvsv, E_Rsp, E_Tsp, E_Rsh. */
int rtmc_zoeppritz_fluid(int32_t n, const double *angles_deg, double vp1, double vs1, double rho1,
                         double vp2, double vs2, double rho2, double *out);

/* ---------------------------------------------------------------------------------- */
/* Transport: the packet x time loop of radiativeTransfer.m:40-158                     */
/* ---------------------------------------------------------------------------------- */

typedef struct rtmc_context rtmc_context;

typedef struct {
    int32_t d;            /* 2 or 3 */
    int32_t frame;        /* enum rtmc_frame */
    int32_t acoustics;
    int32_t precision;    /* enum rtmc_precision */
    int32_t src_dir;      /* 0 'uniform', 1 'outgoing', 2 'upper' (initializeParticle.m:40-47) */
    int32_t polarization; /* 0 'P', 1 'S' */
    int32_t n_sub;        /* sub-steps per observation interval (propagateParticleSmallDt.m:4-7) */
    int32_t n_obs;        /* observation instants = Nt - 1 (t = 0 is never filled) */
    int32_t n_bnd;        /* plane boundaries, <= RTMC_MAX_BND */
    int32_t hist_shift;   /* a unit count adds 1 << hist_shift (64-bit fixed point); a bin of one
                             time slice holds at most n_particles counts, so n_particles must
                             stay below 2^(64 - hist_shift) (checked) */
    int32_t max_events;   /* per-particle event cap, a watchdog with no counterpart in the
                             reference: a particle reaching it stops and the call returns
                             RTMC_ERR_DEVICE (device_status bit 0); 0 = 4 n_sub n_obs + 64 */
    int32_t reserved;
    int64_t n_particles;
    int64_t pid0;         /* global id of the first particle (replica sharding) */
    uint64_t seed;
    double src_pos[3];
    double src_lambda;    /* Gaussian source radius (initializeParticle.m:23) */
    double v[2];          /* propagation speed of P (or acoustic) and S particles */
    double mft[2];        /* mean free time per mode; INFINITY disables scattering */
    double p2p, s2s;      /* mode-conservation probabilities (MaterialClass.m:2439-2440) */
    double qrate[2];      /* omega*h/Q per mode; 0 when Q = Inf (propagateParticleSmallDt.m:57-82) */
    double h;             /* sub-step length */
    /* observation axes 0..3 = X, Y, Z, PSI in the frame of observeTime.m:14-127 */
    int32_t axis_mode[4];    /* enum rtmc_axis_mode */
    int32_t axis_nedges[4];  /* edges of a binned axis; 2 for a range-checked axis */
    const double *axis_edges[4];
    int64_t axis_stride[4];  /* histogram stride of a binned axis */
    int64_t time_stride;
    int64_t mode_stride;
    int64_t hist_len;        /* int64 elements of the histogram */
    int32_t bnd_dir[RTMC_MAX_BND];    /* 1, 2, 3: plane x_dir = val; 4: cylinder sqrt(x^2 + y^2) = val */
    int32_t bnd_absorb[RTMC_MAX_BND]; /* 1 'absorbing', 0 'reflective' */
    double bnd_val[RTMC_MAX_BND];
    double zoe_rpp[RTMC_ZOE_N];       /* E_Rpp on 0:0.5:90 deg (elastic reflective boundary) */
    double zoe_rsvsv[RTMC_ZOE_N];     /* E_Rsvsv on 0:0.5:90 deg */
    /* source shape, initializeParticle.m:14-148; all zero is the Gaussian point source */
    int32_t src_type;       /* enum rtmc_source: point or plane (3D only) */
    int32_t src_aperture;   /* plane: enum rtmc_aperture */
    int32_t src_radial_n;   /* point: knots of the radial inverse CDF (0: Gaussian radius), <= RTMC_MAX_RADIAL */
    int32_t reserved2;
    const double *src_radial_cdf; /* [src_radial_n] strictly increasing CDF values (initializeParticle.m:175-203) */
    const double *src_radial_r;   /* [src_radial_n] radii at those CDF values */
    double src_normal[3];   /* plane: unit propagation direction n */
    double src_u[3];        /* plane: orthonormal basis (u, v) of the aperture plane, null(n) */
    double src_v[3];
    double src_extent[2];   /* plane: rectangle sides along u and v, or the circle radius in [0] */
} rtmc_problem;

typedef struct {
    int64_t scatter_events;  /* accepted scatterings (the throughput unit) */
    int64_t boundary_hits;
    int64_t kills;           /* Q-kills */
    int64_t absorbed;        /* absorbing-boundary deaths */
    int64_t observations;    /* counts added to the histogram */
    int64_t conversions;     /* P<->S changes at boundaries */
    int64_t device_status;   /* non-zero: a kernel guard tripped */
    int32_t launches;        /* kernel launches of the call */
    int32_t sink;            /* 0 shared-memory histogram, 1 global atomics, 2 index array + slice fold */
    double kernel_ms;        /* transport kernel(s), CUDA events on the context stream */
    double fold_ms;          /* slice-fold kernel(s) of the index path */
    double total_ms;         /* whole call, CUDA events (copies included) */
    double h2d_bytes;
    double d2h_bytes;
    double events_ms;        /* split schedule: the event kernel's share of kernel_ms */
    double convert_ms;       /* time-blocked fold without host copies: the conversion's share of fold_ms */
} rtmc_stats;

/* context on CUDA device `device` with its own stream */
int rtmc_create(int32_t device, rtmc_context **out);
void rtmc_destroy(rtmc_context *ctx);

/* last error message of ctx (or of the calling thread when ctx is NULL) */
const char *rtmc_last_error(const rtmc_context *ctx);
int32_t rtmc_abi_version(void);

/* sizeof of the ABI structs {rtmc_material, rtmc_tables_info, rtmc_problem, rtmc_stats},
 * for bindings that mirror them (ctypes, MEX) to check their layout */
int rtmc_abi_sizes(int64_t out[4]);

/* Replaces the packet loop radiativeTransfer.m:40-158 (initializeParticle +
 * propagateParticleSmallDt + observeTime for every packet and time instant).  hist_out
 * is a HOST buffer of problem->hist_len int64 (column-major [N1,N2,(..),Nt,modes], as the
 * uint32 array E of initializeObservation.m:133); the call uploads tables and edges,
 * runs on the GPU and copies the histogram back.  stats may be NULL. */
int rtmc_forward(rtmc_context *ctx, const rtmc_problem *problem, const rtmc_tables *tables,
                 int64_t *hist_out, rtmc_stats *stats);

/* rtmc_forward with the histogram in the reference's own type: hist_out is a HOST buffer
 * of problem->hist_len uint32, each bin's count (value >> hist_shift) saturated at
 * 4294967295 as MATLAB's uint32 additions saturate (initializeObservation.m:133,
 * observeTime.m:12, radiativeTransfer.m:88).  The narrowing runs on the device, so half
 * the bytes of rtmc_forward cross to the host. */
int rtmc_forward_u32(rtmc_context *ctx, const rtmc_problem *problem, const rtmc_tables *tables,
                     uint32_t *hist_out, rtmc_stats *stats);

/* Same, with the histogram left in device memory owned by ctx (no host copy);
 * rtmc_copy_histogram reads it back later. */
int rtmc_forward_device(rtmc_context *ctx, const rtmc_problem *problem, const rtmc_tables *tables,
                        rtmc_stats *stats);
int rtmc_copy_histogram(rtmc_context *ctx, int64_t *hist_out, int64_t n);

/* Device address and length (int64 elements) of the histogram rtmc_forward_device left
 * in ctx, valid until the next call on ctx or rtmc_destroy.  Lets a caller reduce replica
 * histograms in place on the device (the parfor sum E = E + E_local of
 * radiativeTransfer.m:88, across GPUs) before one rtmc_copy_histogram. */
int rtmc_histogram_device(rtmc_context *ctx, void **ptr, int64_t *n);

/* rtmc_forward plus the final state of every particle, for particle-by-particle checks:
 * state_out is a HOST buffer of n_particles x 16 doubles {x[3] at the last event, dir[3],
 * perp[3], mode (0 P, 1 S), alive, scatterings, boundary crossings, sub-step of the last
 * event, sub-step of death (-1 alive), event counter}.  No counterpart in the reference
 * (whose particle struct P, initializeParticle.m:163-170, is internal to the loop). */
int rtmc_forward_trace(rtmc_context *ctx, const rtmc_problem *problem, const rtmc_tables *tables,
                       int64_t *hist_out, double *state_out, rtmc_stats *stats);

/* ---------------------------------------------------------------------------------- */
/* Gradient of a histogram misfit (score-function adjoint with Philox path replay)     */
/* ---------------------------------------------------------------------------------- */

#define RTMC_MAX_PARAMS 8

/* How the path density of an acoustic problem depends on parameters p_q: the
 * differential cross-section sigma(theta; p) of the scattering table and its total
 * Sigma = 1 / mean free time.  The transport draws a scattering in each sub-step with
 * probability 1 - exp(-h Sigma) and its angle from sigma(theta) sin^(d-2)(theta) / Sigma,
 * so the score of a path up to sub-step S with scatterings at theta_1..theta_n is
 *   sum_i d log sigma(theta_i)/dp + d log Sigma/dp [n (kappa - 1) - (S - n) h Sigma],
 *   kappa = h Sigma / (exp(h Sigma) - 1). */
typedef struct {
    int32_t n_params;       /* 1 .. RTMC_MAX_PARAMS */
    int32_t n_theta;        /* >= 2 points of a uniform grid of theta on [0, pi] */
    const double *dlogsigma;              /* [n_params][n_theta] d log sigma(theta) / d p_q */
    double dlogSigma[RTMC_MAX_PARAMS];    /* d log Sigma / d p_q */
} rtmc_score;

/* New entry point, no counterpart in the reference (which has no gradient).  Replays the
 * particles of rtmc_forward (same problem, tables and Philox keys: recomputed, not
 * stored) and returns grad[q] = sum over particles and observation instants of
 * adjoint[bin] * score_q(path up to that instant), accumulated in FP64: the
 * score-function estimate of d L / d p_q when adjoint[b] = d L / d (count in bin b) of
 * the histogram rtmc_forward returns.  Acoustic problems only, with qrate = 0 (a
 * Q-dependence is carried as exp(-omega t / Q) weights on the host); adjoint is a HOST
 * array of hist_len doubles.  The launch shape is fixed per device, so repeated calls
 * return identical bits. */
int rtmc_gradient(rtmc_context *ctx, const rtmc_problem *problem, const rtmc_tables *tables,
                  const rtmc_score *score, const double *adjoint, double *grad, rtmc_stats *stats);

/* ---------------------------------------------------------------------------------- */
/* Batched runs: many independent problems in one persistent, CUDA-graph launch        */
/* ---------------------------------------------------------------------------------- */

typedef struct rtmc_batch rtmc_batch;

/* Stage n problems that share one observation grid (dimension, frame, acoustics,
 * precision, observation instants, axes, edges, strides, histogram length and shift;
 * the histogram must fit in shared memory, as the spherical 120 x 251 grid does) with
 * their own materials, tables, particle counts and seeds.  The tables and parameters go
 * to the device once; the launch (histogram clear + persistent kernel) is captured in a
 * CUDA graph.  Replaces n calls of radiativeTransfer (a parameter sweep driving
 * radiativeTransfer.m in a loop). */
int rtmc_batch_create(rtmc_context *ctx, int32_t n, const rtmc_problem *problems, const rtmc_tables *const *tables,
                      rtmc_batch **out);

/* Launch shape of the lockstep instances: threads per block (0: 512), ring capacity
 * (0: 8) and particles per work item (0: automatic) of the ring kernel
 * (rt_transport_batch).  block = 0 with ring_cap = -1 selects the split kernel instead
 * (rt_transport_batch_split): per work item, the events of its particles into
 * device-memory segment records, then the observations of 32 particles per warp in
 * lockstep.  Its segment records per particle follow the instance's expected events, or
 * the context's ring capacity (rtmc_set_launch) when one was set at rtmc_batch_create;
 * particles with more are run whole at once.  Rebuilds the work list and the graph,
 * keeps the staged tables. */
int rtmc_batch_set_launch(rtmc_batch *batch, int32_t block, int32_t ring_cap, int64_t chunk);

/* Where the event-major instances (rt_transport_batch_em) bin: 1 = the block's
 * shared-memory copy of the instance's histogram (512 threads, one block per SM, flushed
 * with 64-bit atomics when the block moves to another instance), 0 = 64-bit atomics into
 * the instance's histogram in device memory (256 threads, three blocks per SM; the
 * default, and -1), which hides more latency.  Rebuilds the graph. */
int rtmc_batch_set_em_histogram(rtmc_batch *batch, int32_t shared);

/* One replay of the graph; histograms stay on the device.  stats sums all instances. */
int rtmc_batch_run(rtmc_batch *batch, rtmc_stats *stats);

/* Which kernel runs each instance: event_major[i] = 1 for the event-major kernel
 * (rt_transport_batch_em: one particle per thread, 64-bit atomics into the instance's
 * histogram; event-heavy instances), 0 for the lockstep kernel with a shared-memory
 * histogram (rt_transport_batch).  event_major holds one int32 per instance.  A launch of
 * the batch runs one kernel per non-empty group (rtmc_stats.launches). */
int rtmc_batch_schedule(const rtmc_batch *batch, int32_t *event_major);

/* Sets which kernel runs each instance (event_major[i] = 1: rt_transport_batch_em, 0: the
 * lockstep kernel; both give the instance's histogram), or restores the automatic choice
 * (event_major = NULL: 1 when 4 x expected events per particle >= observation instants,
 * unless rtmc_set_schedule fixed the schedule when the batch was made).
 * Rebuilds the work lists and the graph. */
int rtmc_batch_set_schedule(rtmc_batch *batch, const int32_t *event_major);

/* Copies the int64 histograms of instances [first, first + count) into out (host),
 * instance-major, hist_len each. */
int rtmc_batch_histograms(rtmc_batch *batch, int32_t first, int32_t count, int64_t *out);

void rtmc_batch_destroy(rtmc_batch *batch);

/* Size of the static device scratch of rtmc_forward_noalloc (96 MB per GPU). */
#define RTMC_STATIC_SCRATCH_BYTES (96u << 20)

/* rtmc_forward for callers that cannot allocate device memory: code running where a
 * cudaMalloc is not allowed or not wanted, such as inside a host application whose
 * allocator owns the whole device, or a host that hands over only pre-allocated
 * buffers.  No counterpart in the reference (whose MATLAB loop allocates as it goes).
 *
 * The call allocates nothing: no cudaMalloc / cudaFree, no pinned host memory, no
 * streams or events, no heap memory on the host.  The caller passes the inputs
 * (problem, host tables) and the output: hist_device, a DEVICE buffer of
 * problem->hist_len int64 on the current device, which the call zeroes and fills.  The
 * staged tables, edges, counters and the time-major observation-index array (the
 * scratch of the index path, folded slice by slice as in rtmc_forward) live in one
 * file-scope __device__ array of RTMC_STATIC_SCRATCH_BYTES that every GPU loading the
 * library holds until exit; particles run in as many chunks as that array requires.
 * Problems whose tables, edges and one chunk of 32 particles do not fit are rejected
 * with RTMC_ERR_ARG and a message giving the sizes.
 *
 * The first call on a device looks the array up (cudaGetSymbolAddress with that device
 * current); make that first call before any stream capture.  stream may be NULL (the
 * legacy default stream); the call returns after the stream has finished its work.
 * All calls share the one array and it keeps the last call's contents (the call clears
 * what must start at zero): calls that overlap on the GPU, from several host threads or
 * streams, race and must be serialised by the caller.  On the host the call stages the
 * tables through a 2 MB file-scope buffer (no heap, no large stack frame) and holds a
 * library mutex while it runs, so calls from the threads of one process already run one
 * after another. */
int rtmc_forward_noalloc(const rtmc_problem *problem, const rtmc_tables *tables, int64_t *hist_device,
                         void *stream, rtmc_stats *stats);

/* pinned host memory for fast copies (cudaMallocHost); free with rtmc_host_free */
int rtmc_host_alloc(int64_t bytes, void **out);
int rtmc_host_free(void *p);

/* Launch shape of the transport (0 = automatic for each field): threads per block,
 * trajectory segments per lane in the shared-memory ring, and the device scratch budget
 * in MB for the time-major observation-index array of large histograms (-1: no index
 * array, observations go straight to the histogram with 64-bit global atomics). */
int rtmc_set_launch(rtmc_context *ctx, int32_t block, int32_t ring_cap, int32_t index_mb);

/* Pipelining of large histograms (index-array path): the particles run in `chunks`
 * launches over two index slots, and the fold of one chunk (bound by L2 atomics) runs on
 * a second stream while the transport of the next (bound by instruction issue) runs with
 * at most `transport_blocks_per_sm` blocks per SM, leaving room for the fold's blocks.
 * It also halves the index scratch.  0 = automatic (off; 2 blocks per SM when on);
 * chunks = 1: off. */
int rtmc_set_pipeline(rtmc_context *ctx, int32_t chunks, int32_t transport_blocks_per_sm);

/* Transport schedule: 0 = warps walk 32 particles' observation instants in lockstep
 * (events run ahead into a shared-memory ring; best when observations outnumber events);
 * 1 = one particle per thread, each event followed by its segment's observations (best
 * for event-heavy problems); 2 = split: one kernel runs every particle's events (each
 * thread a stream of particles) and writes its trajectory segments to device memory, a
 * second bins the observation instants of 32 particles per warp in lockstep (the segments
 * per particle follow the expected events, or the ring capacity of rtmc_set_launch when
 * one is set; particles with more are rerun one per thread); -1 = automatic (1 when 8 x
 * expected events per particle >= observation instants and the histogram does not go
 * through the index array, else 2).  All give the same histogram.  rtmc_gradient with
 * up to 4 parameters replays on the split schedule under -1 and 2, and with the lockstep
 * ring under 0 and 1 (the same sums up to rounding order). */
int rtmc_set_schedule(rtmc_context *ctx, int32_t event_major);

/* Fold of the index path (large histograms): 1 = each observation one 64-bit reduction
 * into its time slice of the histogram; 2 = time-blocked: FP32 counts with the 4
 * instants of a bin adjacent, a particle's run of instants in one bin added as one vector
 * reduction, then converted to the histogram (needs fewer than 2^24 particles, so that
 * FP32 counts are exact); 3 = time-blocked with a rolling accumulator when one particle
 * chunk covers the call: 64 MB of time blocks at a time, each turn converted (and zeroed)
 * right after its reductions (slower than 2 on the large grids measured; kept for
 * comparison); 0 = automatic (2 when it applies).  All give the same histogram. */
int rtmc_set_fold(rtmc_context *ctx, int32_t mode);

/* enable (1, default) or disable (0) reuse of the device copy of a tables handle across
 * calls; with 0 every call uploads its tables again (end-to-end timing) */
int rtmc_set_table_cache(rtmc_context *ctx, int32_t enable);

/* Calls that return the histogram to the host, on the split schedule with the time-blocked
 * fold and one particle chunk: rt_observe first bins the instants of the first copy groups
 * (at least first_percent of the instants), those groups are folded and their copies to
 * the host start, and then rt_observe bins the remaining instants, so that the host link
 * starts after a fraction of the observation pass.  0: one observation pass, then the
 * groups; -1: the default (40).  The histogram is the same; rtmc_stats.kernel_ms then
 * covers the events and the first instants, fold_ms the rest. */
int rtmc_set_early_copy(rtmc_context *ctx, int32_t first_percent);

/* FP64 problems on the radius-only observation path bin each observation through an FP32
 * estimate with a proven error bound, and in FP64 only when the estimate lies within that
 * bound of a bin edge: the same bins as the FP64 formula, at FP32 cost.  0 turns the
 * estimate off (every observation in FP64); 1, the default, turns it on. */
int rtmc_set_fp64_estimate(rtmc_context *ctx, int32_t enable);

/* On the index path of the split schedule, the particles are binned in the order of their
 * starting directions (a counting sort by direction cell between the event and the
 * observation kernels), so that the fold's blocks see particles that are close together
 * while they fly out and aggregate their counts in shared memory.  The histogram does not
 * depend on it.  0 keeps the particles in id order; 1, the default, sorts them. */
int rtmc_set_particle_order(rtmc_context *ctx, int32_t enable);

/* writes a device buffer larger than L2 (timing hygiene between measured runs) */
int rtmc_flush_l2(rtmc_context *ctx);

/* The L2's rate of 16-byte vector reductions (red.global.add.v4.f32, none awaited) into an
 * L2-resident 64 MB buffer at random slots, the bound of the time-blocked fold: the best of
 * three timed launches, in reductions per second (a measurement for the roofline) */
int rtmc_probe_l2_reductions(rtmc_context *ctx, double *reductions_per_s);

/* kernel time of the last forward call in ms (CUDA events) and its launch count */
int rtmc_last_timing(const rtmc_context *ctx, double *kernel_ms, int32_t *launches);

#ifdef __cplusplus
}
#endif

#endif /* RTMC_H */
