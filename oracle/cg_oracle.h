/* Oracle: a plain-C restatement of the reference's pixel-space covariance and
 * low-l TT likelihood path (Cosmo++ 3.1), plus the FP64 adjoint gradient that
 * the reference lacks.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py use it, and only as the checker / the timed CPU
 * reference arm.  Nothing in the cosmopp_gb300 package links or calls it.
 *
 * Parity pinning: every function here is checked against the reference's own
 * code compiled from its sources (oracle/ref/, output in oracle/_ref/), via the
 * golden fixtures in tests/golden/ and the reference's own known-answer tests.
 *
 * Packed storage everywhere is the reference's: element (i, j), i <= j, at
 * j*(j+1)/2 + i (source/c_matrix.cpp:28-39), which is LAPACK 'U' packed.
 */
#ifndef CG_ORACLE_H
#define CG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

void orc_set_threads(int n);
int orc_get_threads(void);

/* Math::Legendre::calculate, include/legendre.hpp:26-37 */
double orc_legendre(int l, double x);
/* Utils::beamFunction, source/utils.cpp:54-64 (fwhm in degrees) */
double orc_beam(int l, double fwhm_deg);

/* pixel unit vectors, source/c_matrix_generator.cpp:178-185; scheme 0 = RING, 1 = NEST;
   good == NULL means all 12 nside^2 pixels */
void orc_unit_vectors(long nside, int scheme, const int* good, int n, double* xyz);

/* CMatrixGenerator::clToCMatrix, source/c_matrix_generator.cpp:164-232.
   beam2 == NULL: B_l = orc_beam(l, fwhm) (no pixel window).  restart != 0
   re-runs the Legendre recurrence from l = 1 for every l as the reference
   does (O(lmax^2) per pair); restart == 0 runs it once per pair, which gives
   the same values bit for bit. */
void orc_cl_to_cmatrix(const double* cl, int lmax, const double* xyz, int n, double fwhm_deg,
                       int restart, double* out_packed);

/* CMatrixGenerator::getFiducialMatrix, source/c_matrix_generator.cpp:705-772 */
void orc_fiducial_matrix(const double* cl, int lmax_max, const double* xyz, int n, int lmax,
                         double fwhm_deg, double* out_packed);

/* LAPACK dpptrf('U') and dpptri('U') (reference call sites source/matrix_impl.cpp:237-265),
   restated from the LAPACK reference algorithms; return LAPACK's info. */
int orc_dpptrf(int n, double* ap);
int orc_dpptri(int n, double* ap);
/* SymmetricMatrix::logDetFromCholeskyFactorization, source/matrix_impl.cpp:322-338 */
double orc_logdet_from_chol(int n, const double* ap, int* sign);
/* Likelihood::vmv, source/likelihood.cpp:137-152 */
double orc_vmv(int n, const double* a, const double* ap, const double* b);

/* Likelihood::construct (source/likelihood.cpp:69-134) with c, fid (may be NULL = 0) and noise
   packed; on return cinv holds the packed inverse and *logdet_raw = ln det (no offset).
   Returns 0, or the LAPACK info / -1 for a non-positive determinant. */
int orc_likelihood_construct(int n, const double* c, const double* fid, const double* noise,
                             double* cinv, double* logdet_raw);
/* Likelihood::calculate, source/likelihood.cpp:164-180; logdet_raw in, reference-style
   logdet (with foreground term, no offset) out; foreground may be NULL. Returns chi2 + logdet. */
double orc_likelihood_calculate(int n, const double* cinv, double logdet_raw, const double* t,
                                const double* foreground, double* chi2, double* logdet);

/* One -2lnL (+ gradient) evaluation on the reference's call sequence
   (source/test_like_low.cpp:183-193): C(cl) + diag(noise_var), zero fiducial.
   grad (nullable) receives d(-2lnL)/dC_l for l = 0..lmax (l < 2 are 0):
   tr[(C^-1 - a a^T) dC/dC_l], a = C^-1 d.  Returns 0 or a non-zero status. */
int orc_eval(const double* cl, int lmax, const double* xyz, int n, double fwhm_deg,
             const double* noise_var, const double* d, int restart,
             double* m2lnl, double* chi2, double* logdet_raw, double* grad);

/* The adjoint alone: grad_l = sum_ij W_ij (2l+1)/(4pi) B_l^2 P_l(x_ij) for a packed symmetric W */
void orc_adjoint(const double* w_packed, int lmax, const double* xyz, int n, double fwhm_deg, double* grad);

/* LegendrePolynomialContainer's table (source/c_matrix_generator.cpp:30-76):
   out[l * n(n+1)/2 + j(j+1)/2 + i] = P_l(clamped n_i . n_j), l = 0..lmax */
void orc_legendre_table(int lmax, const double* xyz, int n, double* out);

/* The averaging step of CMatrixGenerator::calculateNoiseMatrix
   (source/c_matrix_generator.cpp:887-910): packed N_ij = (sum_k s_k[i] s_k[j]) / nsims over
   noise simulations sims [nsims][n] at the kept pixels, k summed in order, and the largest
   |mean over simulations| of any pixel. */
void orc_noise_matrix(int nsims, int n, const double* sims, double* packed, double* max_abs_mean);

/* No reference counterpart: the exact-arithmetic yardstick for the FP64 noise floor.
   chi2 = d^T A^-1 d and ln det A for A = C (packed FP64) + diag(noise_var), computed in
   long double (x87 80-bit on x86-64: 64-bit significand, about 2000 times finer than FP64)
   by a dense Cholesky and a forward solve.  Returns 0, or j + 1 when pivot j is not
   positive.  On targets whose long double is IEEE quad it is software arithmetic and slow;
   the fixture script runs it in the x86 build container only. */
int orc_loglike_extended(int n, const double* c_packed, const double* noise_var, const double* d,
                         double* chi2, double* logdet_raw);

#ifdef __cplusplus
}
#endif
#endif
