/* C entry points over the reference's own, unmodified classes
   (CMatrixGenerator, CMatrix, Likelihood, Math::Legendre and the reference's
   TestLegendre / TestMatrix known-answer subtests).  Test infrastructure: the
   fixture generator under tests/golden/ calls these through ctypes to pin the
   oracle restatement to the reference's real code. */
#include <vector>
#include <string>
#include <exception>
#include <cstring>

#include <c_matrix.hpp>
#include <c_matrix_generator.hpp>
#include <likelihood.hpp>
#include <legendre.hpp>
#include <utils.hpp>
#include <test_legendre.hpp>
#include <test_matrix.hpp>
#include <hmc.hpp>
#include <alm_healpix_tools.h>
#include <whole_matrix.hpp>
#include <fstream>
#include <unistd.h>

static std::string g_err;

extern "C" const char* ref_last_error() { return g_err.c_str(); }

static void copy_packed(const CMatrix& m, double* out)
{
    const int n = m.getNPix();
    for (int j = 0; j < n; ++j)
        for (int i = 0; i <= j; ++i)
            out[(long)j * (j + 1) / 2 + i] = m.element(i, j);
}

/* CMatrixGenerator::clToCMatrix (source/c_matrix_generator.cpp:164-232);
   good_nest == NULL means all pixels. */
extern "C" int ref_cl_to_cmatrix(const double* cl, int lmax, long nside, double fwhm_deg,
                                 const int* good_nest, int n, double* out_packed)
{
    try {
        std::vector<double> c(cl, cl + lmax + 1);
        std::vector<int> good;
        if (good_nest) good.assign(good_nest, good_nest + n);
        CMatrix* m = CMatrixGenerator::clToCMatrix(c, nside, fwhm_deg, good_nest ? &good : NULL);
        copy_packed(*m, out_packed);
        delete m;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* The reference's low-l call sequence (source/test_like_low.cpp:183-193):
   clToCMatrix -> generateNoiseMatrix + maskMatrix -> Likelihood(C, 0, N, good, {})
   -> calculate(d).  logdet is the reference's value (with its detOffset). */
extern "C" int ref_likelihood(const double* cl, int lmax, long nside, double fwhm_deg,
                              const int* good_nest, int n, double noise_sigma, const double* d,
                              double* chi2, double* logdet, double* like)
{
    try {
        std::vector<double> c(cl, cl + lmax + 1);
        std::vector<int> good(good_nest, good_nest + n);
        CMatrix* cm = CMatrixGenerator::clToCMatrix(c, nside, fwhm_deg, &good);
        CMatrix* noise = CMatrixGenerator::generateNoiseMatrix(nside, noise_sigma);
        noise->maskMatrix(good);
        CMatrix fid(n);
        Likelihood like_obj(*cm, fid, *noise, good, std::vector<double>());
        std::vector<double> t(d, d + n);
        *like = like_obj.calculate(t, *chi2, *logdet);
        delete cm;
        delete noise;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* Likelihood from caller-supplied packed matrices (fiducial may be NULL = 0),
   with optional foreground marginalisation (source/likelihood.cpp:69-180). */
extern "C" int ref_likelihood_packed(const double* c_packed, const double* fid_packed, const double* noise_packed,
                                     int n, const double* d, const double* foreground,
                                     double* chi2, double* logdet, double* like)
{
    try {
        CMatrix c(n), f(n), nm(n);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i <= j; ++i) {
                const long k = (long)j * (j + 1) / 2 + i;
                c.element(i, j) = c_packed[k];
                if (fid_packed) f.element(i, j) = fid_packed[k];
                nm.element(i, j) = noise_packed[k];
            }
        std::vector<int> good(n);
        for (int i = 0; i < n; ++i) good[i] = i;
        std::vector<double> fg;
        if (foreground) fg.assign(foreground, foreground + n);
        Likelihood like_obj(c, f, nm, good, fg);
        std::vector<double> t(d, d + n);
        *like = like_obj.calculate(t, *chi2, *logdet);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* CMatrixGenerator::getFiducialMatrix (source/c_matrix_generator.cpp:705-772) */
extern "C" int ref_fiducial_matrix(const double* cl, int cl_size, long nside, int lmax, double fwhm_deg,
                                   const int* good_nest, int n, double* out_packed)
{
    try {
        std::vector<double> c(cl, cl + cl_size);
        std::vector<int> good(good_nest, good_nest + n);
        CMatrix* m = CMatrixGenerator::getFiducialMatrix(c, nside, lmax, fwhm_deg, &good);
        copy_packed(*m, out_packed);
        delete m;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* LegendrePolynomialContainer(lMax, nSide, goodPixels) written by its own writeIntoFile
   (source/c_matrix_generator.cpp:30-76,136-162) */
extern "C" int ref_legendre_table_write(int lmax, long nside, const int* good_nest, int n, const char* path)
{
    try {
        std::vector<int> good(good_nest, good_nest + n);
        LegendrePolynomialContainer lp(lmax, nside, &good);
        lp.writeIntoFile(path);
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* clToCMatrix with a LegendrePolynomialContainer read back by its file constructor
   (source/c_matrix_generator.cpp:89-134,164-232) */
extern "C" int ref_cl_to_cmatrix_lp_file(const double* cl, int lmax, long nside, double fwhm_deg,
                                         const int* good_nest, int n, const char* path, double* out_packed)
{
    try {
        std::vector<double> c(cl, cl + lmax + 1);
        std::vector<int> good(good_nest, good_nest + n);
        LegendrePolynomialContainer lp(path);
        CMatrix* m = CMatrixGenerator::clToCMatrix(c, nside, fwhm_deg, &good, &lp);
        copy_packed(*m, out_packed);
        delete m;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* clToCMatrix's matrix with a comment, written by CMatrix's own writeIntoFile and
   writeIntoTextFile (source/c_matrix.cpp:67-107) */
extern "C" int ref_cmatrix_write_files(const double* cl, int lmax, long nside, double fwhm_deg, const int* good_nest,
                                       int n, const char* comment, const char* bin_path, const char* txt_path)
{
    try {
        std::vector<double> c(cl, cl + lmax + 1);
        std::vector<int> good(good_nest, good_nest + n);
        CMatrix* m = CMatrixGenerator::clToCMatrix(c, nside, fwhm_deg, &good);
        m->comment() = comment;
        m->writeIntoFile(bin_path);
        m->writeIntoTextFile(txt_path);
        delete m;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* Utils::readClFromFile (source/utils.cpp:173-217): up to max values into out, count returned */
extern "C" int ref_read_cl(const char* path, int has_l, int is_dl, double* out, int max)
{
    try {
        std::vector<double> cl;
        Utils::readClFromFile(path, cl, has_l != 0, is_dl != 0);
        const int k = (int)cl.size() < max ? (int)cl.size() : max;
        for (int i = 0; i < k; ++i) out[i] = cl[i];
        return (int)cl.size();
    } catch (std::exception& e) { g_err = e.what(); return -1; }
}

/* Utils::beamFunction (source/utils.cpp:54-64) and the pixel-window reader
   with the unit window the shim serves (source/utils.cpp:66-170). */
extern "C" double ref_beam(int l, double fwhm_deg) { return Utils::beamFunction(l, fwhm_deg); }
extern "C" int ref_pixel_window(long nside, int lmax, double fwhm_deg, double* out)
{
    try {
        std::vector<double> f;
        Utils::readPixelWindowFunction(f, nside, lmax, fwhm_deg);
        for (int l = 0; l <= lmax; ++l) out[l] = f[l];
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* Math::Legendre::calculate (include/legendre.hpp:26-37) */
extern "C" double ref_legendre(int l, double x) { Math::Legendre leg; return leg.calculate(l, x); }

/* The reference's own known-answer subtests (source/test_legendre.cpp:27-51,
   source/test_matrix.cpp:417-488), run through their protected runSubTest. */
class CgTestLegendre : public TestLegendre { public: using TestLegendre::runSubTest; };
class CgTestMatrix : public TestMatrix { public: using TestMatrix::runSubTest; };

extern "C" int ref_run_subtest(const char* which, int i, double* res, double* expected)
{
    try {
        std::string name;
        if (std::strcmp(which, "legendre") == 0) { CgTestLegendre t; t.runSubTest(i, *res, *expected, name); }
        else if (std::strcmp(which, "matrix") == 0) { CgTestMatrix t; t.runSubTest(i, *res, *expected, name); }
        else return 2;
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* Math::HMC::run (source/hmc.cpp:31-126), unmodified, on an analytic Gaussian
   -2lnL = sum_i ((x_i - mu_i) / sig_i)^2 with unit masses and starting point `start`.  Records,
   at full precision, every point where the reference evaluated the derivative, except the
   re-evaluation at the current point that opens each iteration (the batched sampler keeps
   that gradient from the previous step instead): the leapfrog positions in order, into
   pts [max_pts][n].  Returns their count (or -1); the chain file the reference writes is
   root + ".txt". */
namespace {
class RefGauss : public Math::LikelihoodWithDerivs {
public:
    RefGauss(int n, const double* mu, const double* sig) : mu_(mu, mu + n), sig_(sig, sig + n) {}
    double calculate(double* p, int n) override
    {
        after_calc_ = true;
        double s = 0;
        for (int i = 0; i < n; ++i) {
            const double d = (p[i] - mu_[i]) / sig_[i];
            s += d * d;
        }
        return s;
    }
    double calculateDeriv(double* p, int n, int i) override
    {
        if (i == 0) {
            if (!after_calc_) pts.insert(pts.end(), p, p + n);
            after_calc_ = false;
        }
        return 2 * (p[i] - mu_[i]) / (sig_[i] * sig_[i]);
    }
    std::vector<double> pts;

private:
    std::vector<double> mu_, sig_;
    bool after_calc_ = true;  // the first derivative call (at the start) follows the first calculate
};
}  // namespace

extern "C" int ref_hmc_gaussian(int n, const double* mu, const double* sig, const double* start, double tau_max,
                                int n_max, unsigned int seed, int iters, const char* root, double* pts, int max_pts)
{
    try {
        RefGauss like(n, mu, sig);
        Math::HMC hmc(n, like, root, tau_max, n_max, (time_t)seed);
        for (int i = 0; i < n; ++i) hmc.setParam(i, "x" + std::to_string(i), 1.0, start[i]);
        hmc.run(iters);
        const int cnt = (int)(like.pts.size() / n);
        for (int k = 0; k < cnt && k < max_pts; ++k)
            for (int i = 0; i < n; ++i) pts[(size_t)k * n + i] = like.pts[(size_t)k * n + i];
        return cnt;
    } catch (std::exception& e) { g_err = e.what(); return -1; }
}

/* LikelihoodPolarization (source/likelihood.cpp:341-401, 536-612), unmodified: the constructor
   reads n_inv.txt (written here, in directory `dir`, from ninv [size][size] row-major) and
   factors cInv = N^-1 + N^-1 C N^-1 over the Q and U rows of the kept pixels; calculate() is
   then run with all-zero TT a_lm, so its E-mode template is zero (the shim's rotation and
   synthesis map zero coefficients to zero maps and refuse anything else): chi2 = v^T cInv^-1 v,
   logdet = the reference's (with its detOffset).  size = 2 npix; lmax >= 2 sizes the unused
   ET(TT)^-1 matrix. */
extern "C" int ref_likelihood_pol(int size, const double* c_packed, const double* ninv, const int* good, int ngood,
                                  long nside, int lmax, const double* v, const char* dir, double* chi2, double* logdet)
{
    try {
        const std::string path = std::string(dir) + "/n_inv.txt";
        {
            std::ofstream out(path.c_str());
            out.precision(17);
            for (int i = 0; i < size; ++i) {
                for (int j = 0; j < size; ++j) out << ninv[(size_t)i * size + j] << (j + 1 < size ? " " : "\n");
            }
        }
        char cwd[4096];
        if (!getcwd(cwd, sizeof cwd)) { g_err = "getcwd"; return 1; }
        if (chdir(dir) != 0) { g_err = "chdir"; return 1; }
        CMatrix c(size);
        for (int j = 0; j < size; ++j)
            for (int i = 0; i <= j; ++i) c.element(i, j) = c_packed[(long)j * (j + 1) / 2 + i];
        std::vector<int> g(good, good + ngood);
        WholeMatrix ettt(2, lmax);
        int rc = 0;
        try {
            LikelihoodPolarization like(c, nside, g, lmax, ettt);
            LikelihoodPolarization::AlmType alm(lmax, lmax);
            alm.SetToZero();
            std::vector<double> vv(v, v + 2 * ngood);
            like.calculate(vv, alm, *chi2, *logdet);
        } catch (std::exception& e) { g_err = e.what(); rc = 1; }
        if (chdir(cwd) != 0) { g_err = "chdir back"; return 1; }
        return rc;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

/* CMatrixGenerator::calculateNoiseMatrix (source/c_matrix_generator.cpp:789-929), unmodified, at
   one resolution and beam (nSideOriginal = nSide, fwhmOriginal = fwhm), where the shim's harmonic
   round trip hands each simulated map on unchanged and records it.  mask [12 nside^2] (NEST,
   kept where > 0.5) and nobs [12 nside^2] go into the text files the reference reads (in `dir`);
   out_packed receives the reference's noise matrix over the kept pixels, sims [nsims][12 nside^2]
   (RING order, as synthesised) the maps it averaged; returns the number of maps (or -1). */
extern "C" int ref_noise_matrix(long nside, const double* mask, const double* nobs, double sigma0, double fwhm_deg,
                                const char* dir, double* out_packed, double* sims, int max_sims)
{
    try {
        const long npix = 12 * nside * nside;
        const std::string mpath = std::string(dir) + "/mask.txt", npath = std::string(dir) + "/noise.txt";
        {
            std::ofstream m(mpath.c_str());
            m.precision(17);
            m << nside << " 1\n";
            for (long i = 0; i < npix; ++i) m << mask[i] << "\n";
            std::ofstream nf(npath.c_str());
            nf.precision(17);
            for (long i = 0; i < npix; ++i) nf << i << " 0 " << nobs[i] << "\n";
        }
        cg_shim_synthesised_maps().clear();
        CMatrix* nm = CMatrixGenerator::calculateNoiseMatrix(mpath.c_str(), npath.c_str(), sigma0, fwhm_deg, nside, fwhm_deg);
        copy_packed(*nm, out_packed);
        delete nm;
        const std::vector<std::vector<double> >& rec = cg_shim_synthesised_maps();
        for (size_t k = 0; k < rec.size() && (int)k < max_sims; ++k)
            for (long i = 0; i < npix; ++i) sims[k * npix + i] = rec[k][i];
        return (int)rec.size();
    } catch (std::exception& e) { g_err = e.what(); return -1; }
}
