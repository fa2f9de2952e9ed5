/* cosmopp_gb300 -- GB300-native pixel-space CMB covariance and low-l TT
 * likelihood, the drop-in for Cosmo++'s CMatrixGenerator / CMatrix /
 * Likelihood path (plus the adjoint gradient that path lacks).
 *
 * C ABI: plain pointers and sizes, every call returns an int status
 * (CG_OK = 0), cg_last_error() gives the text.  One context per host thread;
 * calls on one context are serialised.  Host-pointer entry points block until
 * the result is on the host; *_device entry points take device pointers and
 * run asynchronously on the given CUDA stream.
 *
 * Packed storage is the reference's CMatrix layout: element (i, j), i <= j,
 * at j*(j+1)/2 + i (include/c_matrix.hpp:10-83, source/c_matrix.cpp:28-39),
 * identical to LAPACK 'U' packed.
 */
#ifndef COSMOPP_GB300_H
#define COSMOPP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CG_OK              0
#define CG_ERR_BAD_ARG     1  /* invalid argument (size, NULL, range) */
#define CG_ERR_NOT_PD      2  /* covariance not positive definite (per-element status) */
#define CG_ERR_NONFINITE   3  /* NaN / Inf in an input */
#define CG_ERR_TIMEOUT     4  /* a bounded device wait gave up */
#define CG_ERR_CUDA        5  /* CUDA runtime error */
#define CG_ERR_NO_DEVICE   6  /* no usable sm_103 device */
#define CG_ERR_ALLOC       7  /* device allocation failed */

#define CG_SCHEME_RING 0
#define CG_SCHEME_NEST 1      /* the reference's ordering (source/c_matrix_generator.cpp:182) */

#define CG_PREC_FP64   0      /* plain FP64 path */
#define CG_PREC_MIXED  1      /* batched mixed path: FP64 reference factor + FP32 whitened factors */

#define CG_RECENTER_FIXED 0   /* keep the reference point until cg_set_reference */
#define CG_RECENTER_BATCH 1   /* re-centre on every batch's geometric-mean C_l */
#define CG_RECENTER_AUTO  2   /* re-centre when a batch strays beyond recenter_radius */

typedef struct cg_ctx cg_ctx;
typedef struct cg_lik cg_lik;

typedef struct cg_config {
    int struct_size;           /* sizeof(cg_config) */
    /* pixels: either HEALPix (nside, scheme, good_pixels[n] or NULL = all) or dirs[n][3] */
    long nside;
    int scheme;
    const int* good_pixels;
    int n;
    const double* dirs;
    /* harmonic range and beam */
    int lmax;                  /* C_l vectors have lmax + 1 entries; l = 0, 1 are ignored */
    double fwhm_deg;           /* Gaussian beam FWHM in degrees (source/utils.cpp:54-64) */
    const double* beam;        /* optional B_l[lmax + 1] (e.g. pixel window x beam); overrides fwhm */
    /* white noise on the kept pixels: noise_var[n] or sigma^2 on every pixel */
    double noise_sigma;
    const double* noise_var;
    /* execution */
    int max_batch;             /* largest B a call may pass */
    int precision;             /* CG_PREC_FP64 or CG_PREC_MIXED */
    int device;                /* CUDA device ordinal */
    /* mixed path reference point */
    const double* cl_ref;      /* optional initial reference C_l[lmax + 1] */
    int recenter;              /* CG_RECENTER_* */
    double recenter_radius;    /* max |ln(C_l / Cref_l)| before an automatic re-centre (0 = 1.0) */
} cg_config;

/* Memory admission (no counterpart in the reference, whose covariance lives in host memory).
   The device bytes a context needs: bytes_fixed (the pixel geometry, the staging buffers of
   max_batch elements and, for the mixed path, the FP64 reference factor and the whitened
   Legendre table) plus bytes_per_element for every batch element in flight.  Planned against
   bytes_budget less a reserve of 256 MB + 1% (the CUDA context, allocator rounding):
   max_batch_fit elements fit; chunk = min(max_batch, max_batch_fit) is the piece a call's batch
   is evaluated in (one piece after another, each its own batch; with CG_RECENTER_BATCH each
   piece is re-centred on its own mean).  max_batch_fit = 0: nothing fits. */
typedef struct cg_memory_plan {
    size_t bytes_fixed;
    size_t bytes_per_element;
    size_t bytes_budget;
    size_t bytes_reserve;
    int max_batch_fit;
    int chunk;
} cg_memory_plan;

/* ---- context ----------------------------------------------------------- */
void cg_config_init(cg_config* cfg);
/* The plan for a configuration before any allocation: budget_bytes = 0 plans against the free
   memory of cfg->device (needs the device), otherwise against budget_bytes (no device needed). */
int cg_plan_memory(const cg_config* cfg, size_t budget_bytes, cg_memory_plan* plan);
/* The plan cg_create admitted this context with (against the device's free memory then).
   cg_create fails with CG_ERR_ALLOC, before allocating anything, when not one element fits. */
int cg_get_memory_plan(const cg_ctx* ctx, cg_memory_plan* plan);
int cg_create(cg_ctx** ctx, const cg_config* cfg);
void cg_destroy(cg_ctx* ctx);
const char* cg_last_error(const cg_ctx* ctx);   /* ctx may be NULL: last create error */
int cg_get_n(const cg_ctx* ctx);
int cg_unit_vectors(const cg_ctx* ctx, double* xyz);             /* [n][3] */

/* ---- covariance build --------------------------------------------------- */
/* CMatrixGenerator::clToCMatrix (include/c_matrix_generator.hpp:53,
   source/c_matrix_generator.cpp:164-232): packed C for one C_l vector, no noise.
   Same rounding order as the reference, so the result is bit-identical. */
int cg_build_cmatrix(cg_ctx* ctx, const double* cl, double* out_packed);
/* the same for B C_l vectors ([B][lmax+1] -> [B][n(n+1)/2]) */
int cg_build_cmatrix_batched(cg_ctx* ctx, int B, const double* cl, double* out_packed);
/* CMatrixGenerator::getFiducialMatrix (include/c_matrix_generator.hpp:126,
   source/c_matrix_generator.cpp:706-772): packed sum over l = lmax+1 .. lmax_max of
   C_l (2l+1)/(4pi) B_l^2 P_l(x_ij), plus the monopole/dipole marginalisation term
   100 C_2 (1 + x_ij) B_2^2, for this context's pixels.  The reference uses
   lmax_max = 4 nside; cl has lmax_max + 1 entries.  beam [lmax_max + 1] is nullable:
   NULL = the Gaussian beam of the context's fwhm_deg (unit pixel window).
   Bit-identical to the reference.  1 <= lmax < lmax_max <= CG_FIDUCIAL_LMAX_MAX. */
#define CG_FIDUCIAL_LMAX_MAX 4096
int cg_fiducial_matrix(cg_ctx* ctx, const double* cl, int lmax, int lmax_max, const double* beam,
                       double* out_packed);

/* LegendrePolynomialContainer's table (include/c_matrix_generator.hpp:10-36,
   source/c_matrix_generator.cpp:30-76) for this context's pixels: P_l(n_i . n_j) for
   l0 <= l < l1 at out[(l - l0) * n(n+1)/2 + j(j+1)/2 + i], i <= j -- the order of the
   reference's table file after its two int header fields (source/c_matrix_generator.cpp:136-162).
   Math::Legendre's recurrence and the reference's clamped dot product: bit-identical.
   0 <= l0 < l1 <= CG_FIDUCIAL_LMAX_MAX + 1. */
int cg_legendre_table(cg_ctx* ctx, int l0, int l1, double* out);
/* The averaging step of CMatrixGenerator::calculateNoiseMatrix
   (include/c_matrix_generator.hpp:161, source/c_matrix_generator.cpp:887-910): packed
   N_ij = (sum_k s_k[i] s_k[j]) / nsims from noise simulations sims [nsims][n] (each row one
   simulated map at the kept pixels), the sum over k in order with every product and sum
   rounded on its own, as the reference's loop: bit-identical to it.  max_abs_mean
   (nullable) receives the largest |mean over the simulations| of any pixel, the figure the
   reference prints.  Drawing and smoothing the simulations (HEALPix map2alm / alm2map)
   is the caller's.  Uses the context's device only; n need not be the context's n. */
int cg_noise_matrix_from_sims(cg_ctx* ctx, int nsims, int n, const double* sims, double* out_packed,
                              double* max_abs_mean);

/* ---- likelihood + gradient ---------------------------------------------- */
/* -2lnL = d^T C^-1 d + ln det C for B C_l vectors, C = C(cl_b) + noise
   (the reference's Likelihood(C, 0, N, goodPixels).calculate(d),
   include/likelihood.hpp:58,88; source/likelihood.cpp:69-180, without its
   hard-coded detOffset: logdet is the raw ln det C).
   d: one map (d_stride = 0) or B maps at stride d_stride (>= n).
   grad (nullable): [B][lmax+1] d(-2lnL)/dC_l (l < 2 are 0) -- new, no reference counterpart.
   chi2 / logdet / status nullable; status[b] = CG_OK or CG_ERR_NOT_PD / CG_ERR_NONFINITE, or
   (mixed path) CG_ERR_TIMEOUT when a bounded tensor-core wait gave up during the call.
   Returns CG_OK when the call ran, even if some elements carry a bad status. */
int cg_loglike(cg_ctx* ctx, int B, const double* cl, const double* d, int d_stride,
               double* m2lnl, double* chi2, double* logdet, double* grad, int* status);
/* device-pointer variant, asynchronous on `stream` (cudaStream_t, 0 = the context's stream) */
int cg_loglike_device(cg_ctx* ctx, int B, const double* d_cl, const double* d_d, int d_stride,
                      double* d_m2lnl, double* d_chi2, double* d_logdet, double* d_grad, int* d_status,
                      void* stream);
/* mixed path: set the reference point explicitly (C_l[lmax + 1]) */
int cg_set_reference(cg_ctx* ctx, const double* cl_ref);
/* number of reference (re)factorisations so far (mixed path) */
int cg_reference_count(const cg_ctx* ctx);

/* ---- batched HMC (Math::HMC::run, source/hmc.cpp:31-126, over many chains) ---- */
/* nchains chains on one map, parameters x = ln C_l for l = 2..lmax (lmax - 1 per chain),
   cl_template gives C_0, C_1 (ignored) and the layout; x0 [nchains][lmax-1].  Each
   iteration draws p ~ N(0, mass), runs nleap leapfrog steps of size tau with the
   derivative of -2lnL (halved, as the reference does), and accepts with
   exp(-dH/2), dH of -2lnL + p^2/m.  jitter != 0 draws tau in (0, tau] and
   ceil(nleap U) steps each iteration like the reference.  Every leapfrog step is
   one batched -2lnL + gradient call over all chains.  The leapfrog is resident on the
   device: positions, momenta and gradients stay in device memory through a trajectory,
   whose steps are launches only; per iteration the momenta go to the device and the
   proposals' dH, -2lnL and x come back for the acceptance draws.  Knob "hmc_device" = 0
   runs the same likelihood through cg_hmc_sample's host loop; the chains are the same
   bit for bit (C_l = exp(x) by one routine on both sides).  chain receives
   [niter+1][nchains][lmax]: -2lnL then x for every chain after every iteration
   (row 0 = the start); accept_rate [nchains] (nullable). */
int cg_hmc_run(cg_ctx* ctx, const double* map, int nchains, const double* x0, const double* cl_template,
               int niter, int nleap, double tau, const double* mass, int jitter, unsigned long long seed,
               double* chain, double* accept_rate);
/* A batched likelihood with gradient: -2lnL of nchains parameter vectors x [nchains][npar] into
   m2lnl [nchains] and d(-2lnL)/dx into grad [nchains][npar]; returns CG_OK or an error code that
   ends the run.  The batched form of LikelihoodWithDerivs (include/likelihood_function.hpp:30-47). */
typedef int (*cg_batch_like_grad_fn)(void* user, int nchains, const double* x, double* m2lnl, double* grad);
/* The sampler of cg_hmc_run over any batched likelihood with gradient (Math::HMC::run,
   source/hmc.cpp:31-126, over many chains): chain [niter+1][nchains][npar+1] holds -2lnL then x.
   Random numbers: std::mt19937(seed) through uniform_real_distribution(0, 1) and
   normal_distribution(0, 1) in the reference's order, so nchains = 1 with jitter != 0 reproduces
   Math::HMC(npar, like, root, tau, nleap, seed) with unit masses and the same start.  Needs no device. */
int cg_hmc_sample(int nchains, int npar, cg_batch_like_grad_fn like, void* user, const double* x0, int niter,
                  int nleap, double tau, const double* mass, int jitter, unsigned long long seed, double* chain,
                  double* accept_rate);

/* ---- batched Metropolis-Hastings (MetropolisHastings::run, source/mcmc.cpp:455-700) ---- */
#define CG_PRIOR_UNIFORM 0    /* 1/(max - min) on [p1 = min, p2 = max] (include/mcmc.hpp:350-357) */
#define CG_PRIOR_GAUSS   1    /* normal density, mean p1, sigma p2 (include/mcmc.hpp:360-365) */
/* A batched likelihood: -2lnL of nchains parameter vectors x [nchains][npar] into
   m2lnl [nchains]; returns CG_OK or an error code that ends the run.  The batched form
   of LikelihoodFunction::calculate (include/likelihood_function.hpp:7-17). */
typedef int (*cg_batch_like_fn)(void* user, int nchains, const double* x, double* m2lnl);
/* nchains chains from x0 [nchains][npar] for niter iterations.  Each iteration moves the
   parameter blocks in turn (blocks[b] = the index after block b's last parameter, as
   specifyParameterBlocks takes them; nblocks = 0 gives one block per parameter): the
   proposal is x_j + N(0,1) sampling_width[j] on the block, or, with adapt != 0 and the
   adaptive covariance ready, x + L g (g ~ N(0,1) on the block, L its Cholesky factor).
   Every block move is ONE like() call over all chains.  Priors per parameter
   (prior_mode CG_PRIOR_*, p1, p2; prior_mode NULL = flat); accept with
   min(1, prior ratio exp(-d(-2lnL)/2)).  The adaptive covariance is updated every
   100 iterations from all chains (factor 2.4^2/npar, diagonal epsilon 1e-7) and used once
   more than 100 states entered it.  chain [niter+1][nchains][npar+1]: -2lnL then x
   (row 0 = the start); accept_rate [nchains][nblocks'] (nullable) with nblocks' the
   block count used; proposal_cov [npar][npar] (nullable): the final adaptive covariance.
   Needs no device. */
int cg_mh_sample(int nchains, int npar, cg_batch_like_fn like, void* user, const double* x0, int niter,
                 const double* sampling_width, const int* prior_mode, const double* prior_p1,
                 const double* prior_p2, int nblocks, const int* blocks, int adapt, unsigned long long seed,
                 double* chain, double* accept_rate, double* proposal_cov);
/* cg_mh_sample over this context's pixel likelihood of `map`, parameters x = ln C_l for
   l = 2..lmax (npar = lmax - 1), the rest of C_l from cl_template; nchains <= max_batch.
   A proposal the likelihood cannot evaluate (not positive definite) is rejected. */
int cg_mh_run(cg_ctx* ctx, const double* map, int nchains, const double* x0, const double* cl_template,
              int niter, const double* sampling_width, const int* prior_mode, const double* prior_p1,
              const double* prior_p2, int nblocks, const int* blocks, int adapt, unsigned long long seed,
              double* chain, double* accept_rate, double* proposal_cov);

/* ---- instrumentation ------------------------------------------------------ */
/* self-test of the failure path of the device's bounded waits: one thread waits, with a short
   limit, on a barrier that nothing completes; *status receives CG_ERR_TIMEOUT when the wait
   gave up and reported as it should.  Nothing faults or hangs; the context stays usable. */
int cg_selftest_wait_timeout(cg_ctx* ctx, int* status);
/* Tensor-core rate probe: one CTA per SM issues iters x 4 tcgen05.mma kind::tf32 M128 N128 K8
   (A in tensor memory, B in shared memory: the form the factorisation kernels issue), reps
   timed launches after one warm-up, CUDA events on the context's stream.  *tflops = the TF32
   rate achieved (2 M N K per MMA), *ms = the mean launch time.  The FP32-accurate (3xTF32)
   peak of the factorisation kernels is a third of it.  No counterpart in the reference. */
int cg_probe_tf32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms);
/* FP32-pipe rate probe: 4 CTAs x 256 threads per SM, each thread 16 packed two-lane FMAs
   (fma.rn.f32x2, the FP32 contraction's instruction) per iteration on 8 independent chains;
   *tflops counts 2 flops per lane-FMA.  No counterpart in the reference. */
int cg_probe_fp32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms);
/* kernels this context has launched so far (a replayed graph counts its kernels) */
long long cg_launch_count(const cg_ctx* ctx);
/* Mixed calls with a fixed reference point (CG_RECENTER_FIXED, reference set) are captured into a
   CUDA graph on their first call with a given argument set (batch size, pointers, stream) and
   replayed with one graph launch on later calls with the same set; up to 8 sets are kept, and a
   knob change or a larger batch re-captures.  Calls from a stream that is already capturing, the
   legacy or per-thread default stream, or with profiling on, launch their kernels directly.  The
   knob "graph" = 0 turns replays off.  Returns the replays so far. */
long long cg_graph_replays(const cg_ctx* ctx);
/* record CUDA events between the stages of each cg_loglike* call */
int cg_set_profiling(cg_ctx* ctx, int enable);
/* per-stage device milliseconds of the last profiled call: ms[7] =
   {build/contraction, cholesky, trtri, lauum, solve+refine, adjoint, 0} */
int cg_stage_times(cg_ctx* ctx, double* ms);

/* ---- launch-shape tuning of the mixed path (no counterpart in the reference) ---- */
/* Knobs, by name.  Launch shapes (results change only in rounding order): "fwd_ctas",
   "chol_ctas", "panel_ctas" (persistent CTA counts of the tensor-core contraction, the Cholesky's
   off-diagonal work queue and its panel solve; 0 = one per SM, for the panel 7/8 of them while
   trtri runs beside the Cholesky), "adj" (tensor-core adjoint
   variant 0..3), "lauum" (2, the default: one CTA per block of C^-1 with the A operand split on
   chip; 0: A read pre-split; 1: persistent CTAs over a work queue, A split on chip; 0 differs from
   the others below 2^-22 of an entry), "trtri" (0, the default: one CTA per block of L^-1;
   1: persistent CTAs over a work queue with each block's two products chained on chip, identical
   results), "overlap" (1, the default: trtri's row launches run beside the Cholesky, which the
   call moves to a high-priority stream of the context, each row once its column's update is done;
   0: trtri after the Cholesky; identical results; with "trtri" = 1 the launches stay in sequence).  Accuracy choices, never changed by cg_autotune: "fwd" (forward contraction:
   0 = FP32 FMA, the default; 1 = tensor cores, faster, but its one-way accumulation rounding
   biases the whitened matrix by a few ulp of |A - I|, about 1e-3 in -2lnL at nside 16 for C_l
   a factor e from the reference point), "diag_sq" (1, the default: the Cholesky's diagonal
   blocks take their row sums of squares from the CUDA cores rather than the tensor core),
   "table_bf16" (0, the default; 1 rounds the whitened Legendre table to BF16 and rebuilds it at
   the current reference point: the BF16 table variant, whose error is measured, not a fast path).
   "graph" (1, the default: fixed-reference mixed calls replayed as one CUDA graph; 0 = direct launches). */
int cg_tune_set(cg_ctx* ctx, const char* knob, int value);
int cg_tune_get(const cg_ctx* ctx, const char* knob, int* value);
/* "fwd=1 fwd_ctas=0 ..." of the knobs in effect */
int cg_tune_describe(const cg_ctx* ctx, char* buf, int len);
/* One coordinate pass over the launch-shape knobs' candidate values on this context's shape at batch B
   (median of 3 timed calls per candidate, CUDA events), keeping a change only when it is
   faster by more than 0.5%; the result is applied and, if path is non-NULL, appended to that
   tuning file under "<device>|n=..|lmax=..|B=..|".  *best_ms = the chosen shape's time.
   Overwrites the context's staging buffers. */
int cg_autotune(cg_ctx* ctx, int B, const char* path, double* best_ms);
/* Apply the last entry of a tuning file for this device, n, lmax and B = max_batch (*found = 1),
   or keep the current knobs (*found = 0, also when the file does not exist).  cg_create does
   this for mixed contexts when the environment variable COSMOPP_GB300_TUNE_FILE names a file. */
int cg_tune_load(cg_ctx* ctx, const char* path, int* found);

/* ---- Likelihood drop-in (source/likelihood.cpp:38-41,69-180) ------------- */
/* construct from packed C, fiducial (nullable = 0) and noise, with optional
   foreground marginalisation; all host pointers, n(n+1)/2 doubles each */
int cg_likelihood_create(cg_lik** lik, int n, const double* c_packed, const double* fid_packed,
                         const double* noise_packed, const double* foreground, int device);
/* chi2 and logdet as the reference's calculate (logdet without detOffset) */
int cg_likelihood_calculate(cg_lik* lik, const double* t, double* chi2, double* logdet);
double cg_likelihood_logdet(const cg_lik* lik);
void cg_likelihood_destroy(cg_lik* lik);
const char* cg_likelihood_last_error(const cg_lik* lik);

/* The pixel-space part of LikelihoodPolarization (include/likelihood.hpp:137-224,
   source/likelihood.cpp:341-401,536-612).  c_packed: the (2 npix)-pixel Q-then-U covariance,
   packed; ninv: the (2 npix) x (2 npix) inverse noise matrix, row-major as n_inv.txt holds it,
   taken symmetric; good[ngood]: the kept pixels.  The construct keeps the Q and U rows and
   columns of the kept pixels and factors cInv = N^-1 + N^-1 C N^-1 (2 ngood pixels) on the
   device, FP64; cg_likelihood_logdet gives its raw ln det (the reference subtracts
   detOffset = 16078.083180 from it).  calculate: v [2 ngood] = N^-1 (Q, U) at the kept pixels,
   subtract [2 ngood] = the Q, U template correlated with T at the kept pixels (the reference
   forms it from the TT a_lm with alm2map_pol; that harmonic step is the caller's):
   chi2 = w^T cInv^-1 w with w = v - N^-1 subtract; logdet = the raw ln det. */
int cg_likelihood_pol_create(cg_lik** lik, int npix, const int* good, int ngood, const double* c_packed,
                             const double* ninv, int device);
int cg_likelihood_pol_calculate(cg_lik* lik, const double* v, const double* subtract, double* chi2,
                                double* logdet);

/* No counterpart in the reference.  The same construct + calculate as
   cg_likelihood_create / cg_likelihood_calculate, for one map, for callers
   that cannot allocate device memory (code running inside another framework's
   memory pool, plug-ins whose host owns every device allocation).  Inputs
   d_c_packed, d_fid_packed (nullable = 0), d_noise_packed (n(n+1)/2 doubles
   each) and d_t (n) and outputs d_out[2] = {chi2, raw ln det C} and d_status
   (nullable; CG_OK or CG_ERR_NOT_PD) are all device pointers owned by the
   caller; the call itself allocates nothing and runs asynchronously on
   `stream`.  d_out and d_status are written by the call's last kernel, so
   they hold results only when the call returned CG_OK (a host-side error
   returns before that kernel is queued).  Its workspace is one static device array sized for n <= 768
   (about 5.5 MB, held on every GPU that loads the library until exit); larger
   n is rejected with CG_ERR_BAD_ARG (text in cg_last_error(NULL)).  Every call
   shares that array: calls whose GPU work overlaps race and must be
   serialised.  The first call on a device looks up the array's address, so
   make it before capturing a CUDA graph on that device. */
int cg_likelihood_noalloc(int n, const double* d_c_packed, const double* d_fid_packed,
                          const double* d_noise_packed, const double* d_t, double* d_out, int* d_status,
                          void* stream);

/* ---- HEALPix geometry (host; Gorski et al. 2005) ------------------------ */
long cg_nside2npix(long nside);
long cg_ring2nest(long nside, long ipring);
long cg_nest2ring(long nside, long ipnest);
int cg_pix2vec(long nside, int scheme, const int* pix, int n, double* xyz);
/* Utils::beamFunction (source/utils.cpp:54-64), fwhm in degrees */
double cg_beam(int l, double fwhm_deg);

#ifdef __cplusplus
}
#endif
#endif
