/* Oracle: plain-C restatement of the reference's pixel covariance + low-l TT
 * likelihood path.  TEST INFRASTRUCTURE ONLY (see cg_oracle.h).
 *
 * Every routine keeps the reference's evaluation order where the reference
 * fixes one, so that with -ffp-contract=off the covariance matrix is bit for
 * bit the reference's.  The LAPACK routines follow the published LAPACK
 * reference algorithms (dpptrf/dtpsv/ddot, dpptri/dtptri/dtpmv/dspr).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "cg_oracle.h"
#include "healpix_pix.h"

static const double k_pi = 3.141592653589793; /* include/math_constants.hpp:8 */

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* include/legendre.hpp:26-37: vals[0] = 1, vals[1] = x,
   vals[l] = (2 - 1/l) x vals[l-1] - (1 - 1/l) vals[l-2] */
double orc_legendre(int l, double x)
{
    if (l == 0) return 1.0;
    double vm2 = 1.0, vm1 = x;
    for (int l1 = 2; l1 <= l; ++l1) {
        const double v = (2 - 1.0 / l1) * x * vm1 - (1 - 1.0 / l1) * vm2;
        vm2 = vm1;
        vm1 = v;
    }
    return vm1;
}

/* source/utils.cpp:54-64 */
double orc_beam(int l, double fwhm)
{
    if (fwhm == 0) return 1.0;
    const double sigma = sqrt(8 * log(2.0)) / (fwhm * k_pi / 180);
    return exp(-l * (l + 1) / (2 * sigma * sigma));
}

/* source/c_matrix_generator.cpp:178-185 (pix2ang + unit vector) */
void orc_unit_vectors(long nside, int scheme, const int* good, int n, double* xyz)
{
    for (int i = 0; i < n; ++i) {
        const long index = good ? good[i] : i;
        double theta, phi;
        if (scheme == 1) hp_pix2ang_nest(nside, index, &theta, &phi);
        else hp_pix2ang_ring(nside, index, &theta, &phi);
        xyz[3 * i + 0] = sin(theta) * cos(phi);
        xyz[3 * i + 1] = sin(theta) * sin(phi);
        xyz[3 * i + 2] = cos(theta);
    }
}

/* ThreeVector dot product (include/three_vector.hpp:37) and the clamp at
   source/c_matrix_generator.cpp:203-215 */
static double clamped_dot(const double* a, const double* b)
{
    double dot = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    if (dot > 1) dot = 1;
    if (dot < -1) dot = -1;
    return dot;
}

static void beam_table(int lmax, double fwhm, double* beam)
{
    /* Utils::readPixelWindowFunction with a unit pixel window: f[l] = 1 * B_l
       (source/utils.cpp:149-158) */
    for (int l = 0; l <= lmax; ++l) {
        double f = 1.0;
        f *= orc_beam(l, fwhm);
        beam[l] = f;
    }
}

/* source/c_matrix_generator.cpp:164-232 */
void orc_cl_to_cmatrix(const double* cl, int lmax, const double* xyz, int n, double fwhm,
                       int restart, double* out)
{
    double* beam = (double*)malloc(sizeof(double) * (lmax + 1));
    double* clc = (double*)calloc(lmax + 1, sizeof(double));
    beam_table(lmax, fwhm, beam);
    for (int l = 2; l <= lmax; ++l) clc[l] = cl[l] * (2 * l + 1) / (4 * k_pi);

#pragma omp parallel for schedule(dynamic, 8)
    for (int j = 0; j < n; ++j) {
        double* vals = (double*)malloc(sizeof(double) * (lmax + 2));
        for (int i = 0; i <= j; ++i) {
            const double dot = clamped_dot(xyz + 3 * i, xyz + 3 * j);
            double element = 0;
            if (restart) {
                for (int l = 2; l <= lmax; ++l) {
                    const double leg = orc_legendre(l, dot);
                    element += clc[l] * leg * beam[l] * beam[l];
                }
            } else {
                vals[0] = 1.0;
                vals[1] = dot;
                for (int l = 2; l <= lmax; ++l) {
                    vals[l] = (2 - 1.0 / l) * dot * vals[l - 1] - (1 - 1.0 / l) * vals[l - 2];
                    element += clc[l] * vals[l] * beam[l] * beam[l];
                }
            }
            out[(long)j * (j + 1) / 2 + i] = element;
        }
        free(vals);
    }
    free(beam);
    free(clc);
}

/* source/c_matrix_generator.cpp:705-772: terms lmax < l <= lmax_max plus the
   monopole/dipole marginalisation 100 C_2 (1 + x) B_2^2 */
void orc_fiducial_matrix(const double* cl, int lmax_max, const double* xyz, int n, int lmax,
                         double fwhm, double* out)
{
    double* beam = (double*)malloc(sizeof(double) * (lmax_max + 1));
    beam_table(lmax_max, fwhm, beam);
#pragma omp parallel for schedule(dynamic, 8)
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i <= j; ++i) {
            const double dot = clamped_dot(xyz + 3 * i, xyz + 3 * j);
            double element = 0;
            for (int l = lmax + 1; l <= lmax_max; ++l) {
                const double leg = orc_legendre(l, dot);
                element += cl[l] * ((2 * l + 1) / (4 * k_pi)) * leg * beam[l] * beam[l];
            }
            element += 100 * cl[2] * (1 + dot) * beam[2] * beam[2];
            out[(long)j * (j + 1) / 2 + i] = element;
        }
    }
    free(beam);
}

/* ---- LAPACK reference algorithms, upper packed (AP(i + j(j+1)/2), 0-based) ---- */

/* dpptrf 'U': for each column j, solve U(0:j,0:j)^T x = a(0:j, j) (dtpsv 'U','T','N'),
   then u_jj = sqrt(a_jj - x.x) (ddot). */
int orc_dpptrf(int n, double* ap)
{
    long jj = -1;
    for (int j = 0; j < n; ++j) {
        const long jc = jj + 1; /* start of column j */
        jj += j + 1;            /* diagonal of column j */
        if (j > 0) {
            long kk = 0;        /* dtpsv: x(jcol) for jcol = 0..j-1 */
            for (int c = 0; c < j; ++c) {
                double temp = ap[jc + c];
                long k = kk;
                for (int i = 0; i < c; ++i) { temp -= ap[k] * ap[jc + i]; ++k; }
                temp /= ap[kk + c];
                ap[jc + c] = temp;
                kk += c + 1;
            }
        }
        double dot = 0;
        for (int i = 0; i < j; ++i) dot += ap[jc + i] * ap[jc + i];
        const double ajj = ap[jj] - dot;
        if (ajj <= 0 || ajj != ajj) {
            ap[jj] = ajj;
            return j + 1;
        }
        ap[jj] = sqrt(ajj);
    }
    return 0;
}

/* dtptri 'U','N' followed by dpptri's U^-1 U^-T assembly (dspr + dscal) */
int orc_dpptri(int n, double* ap)
{
    /* dtptri */
    long jc = 0;
    for (int j = 0; j < n; ++j)
        if (ap[jc + j] == 0) return j + 1;
        else jc += j + 1;
    jc = 0;
    for (int j = 0; j < n; ++j) {
        ap[jc + j] = 1.0 / ap[jc + j];
        const double ajj = -ap[jc + j];
        /* dtpmv 'U','N' on the leading j x j block: x := T x, x = ap[jc .. jc+j-1] */
        long kk = 0;
        for (int c = 0; c < j; ++c) {
            if (ap[jc + c] != 0) {
                const double temp = ap[jc + c];
                long k = kk;
                for (int i = 0; i < c; ++i) { ap[jc + i] += temp * ap[k]; ++k; }
                ap[jc + c] *= ap[kk + c];
            }
            kk += c + 1;
        }
        for (int i = 0; i < j; ++i) ap[jc + i] *= ajj;
        jc += j + 1;
    }
    /* inv(U) * inv(U)^T */
    long jj = -1;
    for (int j = 0; j < n; ++j) {
        const long jcol = jj + 1;
        jj += j + 1;
        if (j > 0) { /* dspr 'U', alpha = 1, x = ap[jcol .. jcol+j-1], on the leading j x j block */
            long kk = 0;
            for (int c = 0; c < j; ++c) {
                const double xc = ap[jcol + c];
                if (xc != 0) {
                    const double temp = 1.0 * xc;
                    long k = kk;
                    for (int i = 0; i <= c; ++i) { ap[k] += ap[jcol + i] * temp; ++k; }
                }
                kk += c + 1;
            }
        }
        const double ajj = ap[jj];
        for (int i = 0; i <= j; ++i) ap[jcol + i] *= ajj;
    }
    return 0;
}

/* source/matrix_impl.cpp:322-338 */
double orc_logdet_from_chol(int n, const double* ap, int* sign)
{
    double logdet = 0;
    *sign = 1;
    for (int i = 0; i < n; ++i) {
        const double d = ap[(long)i * (i + 1) / 2 + i];
        logdet += log(fabs(d));
        if (d < 0) *sign *= -1;
    }
    return 2 * logdet;
}

static inline double sym_at(const double* ap, int i, int j)
{
    /* SymmetricMatrix::operator() (include/matrix_impl.hpp:494-502) */
    if (i < j) { const int t = i; i = j; j = t; }
    return ap[(long)i * (i + 1) / 2 + j];
}

/* source/likelihood.cpp:137-152 */
double orc_vmv(int n, const double* a, const double* ap, const double* b)
{
    double* res = (double*)calloc(n, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) res[i] += a[i] * sym_at(ap, i, j) * b[j];
    double result = 0;
    for (int i = 0; i < n; ++i) result += res[i];
    free(res);
    return result;
}

/* source/likelihood.cpp:69-134 (size checks are the caller's) */
int orc_likelihood_construct(int n, const double* c, const double* fid, const double* noise,
                             double* cinv, double* logdet_raw)
{
    const long np = (long)n * (n + 1) / 2;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < np; ++k) cinv[k] = c[k] + (fid ? fid[k] : 0.0) + noise[k];
    const int info = orc_dpptrf(n, cinv);
    if (info) return info;
    int sign = 1;
    *logdet_raw = orc_logdet_from_chol(n, cinv, &sign);
    if (sign != 1) return -1;
    return orc_dpptri(n, cinv);
}

/* source/likelihood.cpp:164-180 */
double orc_likelihood_calculate(int n, const double* cinv, double logdet_raw, const double* t,
                                const double* f, double* chi2, double* logdet)
{
    *chi2 = orc_vmv(n, t, cinv, t);
    *logdet = logdet_raw;
    if (f) {
        const double tCinvf = orc_vmv(n, t, cinv, f);
        const double fCinvf = orc_vmv(n, f, cinv, f);
        *logdet += log(fCinvf / n);
        *chi2 -= tCinvf * tCinvf / fCinvf;
    }
    return *chi2 + *logdet;
}

/* New (no reference counterpart): grad_l = sum_ij W_ij (2l+1)/(4pi) B_l^2 P_l(x_ij).
   Deterministic: fixed row chunks, partial sums combined in chunk order. */
void orc_adjoint(const double* w, int lmax, const double* xyz, int n, double fwhm, double* grad)
{
    enum { NCHUNK = 64 };
    double* beam = (double*)malloc(sizeof(double) * (lmax + 1));
    beam_table(lmax, fwhm, beam);
    double* part = (double*)calloc((size_t)NCHUNK * (lmax + 1), sizeof(double));
#pragma omp parallel for schedule(dynamic, 1)
    for (int ch = 0; ch < NCHUNK; ++ch) {
        double* acc = part + (size_t)ch * (lmax + 1);
        double* vals = (double*)malloc(sizeof(double) * (lmax + 2));
        for (int j = ch; j < n; j += NCHUNK) {
            for (int i = 0; i <= j; ++i) {
                const double wij = (i == j ? 1.0 : 2.0) * w[(long)j * (j + 1) / 2 + i];
                const double dot = clamped_dot(xyz + 3 * i, xyz + 3 * j);
                vals[0] = 1.0;
                vals[1] = dot;
                for (int l = 2; l <= lmax; ++l) {
                    vals[l] = (2 - 1.0 / l) * dot * vals[l - 1] - (1 - 1.0 / l) * vals[l - 2];
                    acc[l] += wij * vals[l];
                }
            }
        }
        free(vals);
    }
    for (int l = 0; l <= lmax; ++l) {
        double s = 0;
        for (int ch = 0; ch < NCHUNK; ++ch) s += part[(size_t)ch * (lmax + 1) + l];
        grad[l] = (l < 2) ? 0.0 : s * ((2 * l + 1) / (4 * k_pi)) * beam[l] * beam[l];
    }
    free(part);
    free(beam);
}

int orc_eval(const double* cl, int lmax, const double* xyz, int n, double fwhm,
             const double* noise_var, const double* d, int restart,
             double* m2lnl, double* chi2, double* logdet_raw, double* grad)
{
    const long np = (long)n * (n + 1) / 2;
    double* c = (double*)malloc(sizeof(double) * np);
    double* nz = (double*)calloc(np, sizeof(double));
    double* cinv = (double*)malloc(sizeof(double) * np);
    if (!c || !nz || !cinv) { free(c); free(nz); free(cinv); return -2; }
    orc_cl_to_cmatrix(cl, lmax, xyz, n, fwhm, restart, c);
    /* generateNoiseMatrix + maskMatrix (source/c_matrix_generator.cpp:774-787,
       source/c_matrix.cpp:183-201): diagonal noise variance on the kept pixels */
    for (int i = 0; i < n; ++i) nz[(long)i * (i + 1) / 2 + i] = noise_var[i];
    int st = orc_likelihood_construct(n, c, NULL, nz, cinv, logdet_raw);
    if (st == 0) {
        double ld;
        *m2lnl = orc_likelihood_calculate(n, cinv, *logdet_raw, d, NULL, chi2, &ld);
        if (grad) {
            /* W = C^-1 - a a^T, a = C^-1 d */
            double* a = (double*)calloc(n, sizeof(double));
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; ++i) {
                double s = 0;
                for (int j = 0; j < n; ++j) s += sym_at(cinv, i, j) * d[j];
                a[i] = s;
            }
#pragma omp parallel for schedule(dynamic, 16)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i <= j; ++i) cinv[(long)j * (j + 1) / 2 + i] -= a[i] * a[j];
            orc_adjoint(cinv, lmax, xyz, n, fwhm, grad);
            free(a);
        }
    }
    free(c);
    free(nz);
    free(cinv);
    return st;
}

/* source/c_matrix_generator.cpp:887-910: each element summed over k in order, every
   product and sum rounded on its own (-ffp-contract=off), then divided by nsims */
void orc_noise_matrix(int nsims, int n, const double* sims, double* packed, double* max_abs_mean)
{
    /* pixel-major copy so the k loop reads contiguously; the summation order is unchanged */
    double* st = (double*)malloc(sizeof(double) * (size_t)nsims * n);
    for (int k = 0; k < nsims; ++k)
        for (int i = 0; i < n; ++i) st[(size_t)i * nsims + k] = sims[(size_t)k * n + i];
#pragma omp parallel for schedule(dynamic, 8)
    for (int j = 0; j < n; ++j)
        for (int i = 0; i <= j; ++i) {
            const double* a = st + (size_t)i * nsims;
            const double* b = st + (size_t)j * nsims;
            double e = 0;
            for (int k = 0; k < nsims; ++k) e += a[k] * b[k];
            e /= nsims;
            packed[(long)j * (j + 1) / 2 + i] = e;
        }
    free(st);
    double mx = 0;
    for (int j = 0; j < n; ++j) {
        double avg = 0;
        for (int k = 0; k < nsims; ++k) avg += sims[(long)k * n + j];
        avg /= nsims;
        if (fabs(avg) > mx) mx = fabs(avg);
    }
    if (max_abs_mean) *max_abs_mean = mx;
}

/* LegendrePolynomialContainer(lMax, nSide, goodPixels) (source/c_matrix_generator.cpp:30-76):
   out[l * np + j(j+1)/2 + i] = Legendre::calculate(l, clamped dot), np = n(n+1)/2 */
void orc_legendre_table(int lmax, const double* xyz, int n, double* out)
{
    const long np = (long)n * (n + 1) / 2;
#pragma omp parallel for schedule(dynamic, 8)
    for (int j = 0; j < n; ++j)
        for (int i = 0; i <= j; ++i) {
            const double dot = clamped_dot(xyz + 3 * i, xyz + 3 * j);
            for (int l = 0; l <= lmax; ++l) out[(long)l * np + (long)j * (j + 1) / 2 + i] = orc_legendre(l, dot);
        }
}

/* Extended-precision -2lnL pieces (test infrastructure, no reference counterpart).  Dense
   row-major lower factor; left-looking: l_ij = (a_ij - sum_{k<j} l_ik l_jk) / l_jj, each row's
   dot products contiguous, rows of one column in parallel. */
int orc_loglike_extended(int n, const double* c_packed, const double* noise_var, const double* d,
                         double* chi2, double* logdet_raw)
{
    long double* L = (long double*)malloc(sizeof(long double) * (size_t)n * n);
    if (!L) return -2;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j)
            L[(size_t)i * n + j] = (long double)c_packed[(long)i * (i + 1) / 2 + j] +
                                   (i == j ? (long double)noise_var[i] : 0.0L);
    int info = 0;
    for (int j = 0; j < n && !info; ++j) {
        long double* rj = L + (size_t)j * n;
        long double s = rj[j];
        for (int k = 0; k < j; ++k) s -= rj[k] * rj[k];
        if (!(s > 0)) { info = j + 1; break; }
        const long double piv = sqrtl(s);
        rj[j] = piv;
#pragma omp parallel for schedule(static)
        for (int i = j + 1; i < n; ++i) {
            long double* ri = L + (size_t)i * n;
            long double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
            int k = 0;
            for (; k + 4 <= j; k += 4) {
                a0 += ri[k] * rj[k];
                a1 += ri[k + 1] * rj[k + 1];
                a2 += ri[k + 2] * rj[k + 2];
                a3 += ri[k + 3] * rj[k + 3];
            }
            for (; k < j; ++k) a0 += ri[k] * rj[k];
            ri[j] = (ri[j] - ((a0 + a1) + (a2 + a3))) / piv;
        }
    }
    if (!info) {
        long double ld = 0, c2 = 0;
        long double* y = (long double*)malloc(sizeof(long double) * n);
        for (int i = 0; i < n; ++i) {
            const long double* ri = L + (size_t)i * n;
            long double s = d[i];
            for (int k = 0; k < i; ++k) s -= ri[k] * y[k];
            y[i] = s / ri[i];
            c2 += y[i] * y[i];
            ld += logl(ri[i]);
        }
        free(y);
        *chi2 = (double)c2;
        *logdet_raw = (double)(2 * ld);
    }
    free(L);
    return info;
}
