// Header-only C++ drop-in for Cosmo++'s pixel-likelihood classes, over the
// C ABI of libcosmopp_gb300.so (include/cosmopp_gb300.h).
//
// Same class names, signatures, argument meaning and error behaviour as the
// reference (Cosmo++ 3.1):
//   CMatrix           include/c_matrix.hpp:10-83, source/c_matrix.cpp
//   LegendrePolynomialContainer include/c_matrix_generator.hpp:10-36, source/c_matrix_generator.cpp:30-162
//   CMatrixGenerator  include/c_matrix_generator.hpp:40-160 (clToCMatrix, getFiducialMatrix,
//                     generateNoiseMatrix, the noise matrix's averaging step)
//   Utils::readClFromFile source/utils.cpp:173-217
//   LikelihoodResult  include/likelihood.hpp:18-30
//   Likelihood        include/likelihood.hpp:36-132, source/likelihood.cpp:38-328
//   StandardException include/exception_handler.hpp:10-30
// plus the gradient adaptors the reference's samplers consume:
//   PixelLikelihoodWithDerivs : Math::LikelihoodWithDerivs (include/likelihood_function.hpp:30-47)
//   PixelLikelihoodLBFGS (value / gradient as Math::RealFunctionMultiDim / RealFunctionMultiToMulti,
//                        include/function.hpp:113-179)
//   PixelLikelihoodFunction<LargeVector> (set / value / derivative, include/hmc_general.hpp:49-62)
//
// The interface headers are shared with the reference through its own include
// guards: if the reference's header was included first, its definitions are
// used; otherwise identical ones are declared here.
#ifndef COSMOPP_GB300_COSMOPP_HPP
#define COSMOPP_GB300_COSMOPP_HPP

#include <cmath>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../cosmopp_gb300.h"

#ifndef COSMO_PP_EXCEPTION_HANDLER_HPP
#define COSMO_PP_EXCEPTION_HANDLER_HPP
#include <exception>
class StandardException : public std::exception
{
public:
    ~StandardException() throw() {}
    virtual const char* what() const throw() { return s_.c_str(); }
    void set(const std::string& s) { s_ = s; }

private:
    std::string s_;
};
#endif

#ifndef COSMO_PP_LIKELIHOOD_FUNCTION_HPP
#define COSMO_PP_LIKELIHOOD_FUNCTION_HPP
namespace Math
{
class LikelihoodFunction
{
public:
    virtual ~LikelihoodFunction() {}
    virtual double calculate(double* params, int nParams) = 0;
    virtual double calculateExact(double* params, int nParams) { return calculate(params, nParams); }
};
class LikelihoodWithDerivs : public LikelihoodFunction
{
public:
    virtual ~LikelihoodWithDerivs() {}
    virtual double calculate(double* params, int nParams) = 0;
    virtual double calculateDeriv(double* params, int nParams, int i) = 0;
};
}  // namespace Math
#endif

namespace cosmopp_gb300_detail
{
inline void raise(const std::string& msg)
{
    StandardException exc;
    exc.set(msg);
    throw exc;
}
inline void check(int rc, const std::string& what, const char* detail)
{
    if (rc != CG_OK) raise(what + ": " + (detail ? detail : "") + " (status " + std::to_string(rc) + ")");
}
}  // namespace cosmopp_gb300_detail

/// Covariance matrix in pixel space, packed upper storage j(j+1)/2 + i.
class CMatrix
{
public:
    CMatrix(int nPix) : nPix_(nPix) { initialize(); }
    CMatrix(const char* fileName) { readFromFile(fileName); }
    double& element(int i, int j) { return matrix_[getIndex(i, j)]; }
    double element(int i, int j) const { return matrix_[getIndex(i, j)]; }
    int getNPix() const { return nPix_; }
    const std::string& comment() const { return comment_; }
    std::string& comment() { return comment_; }
    /// the packed array (n(n+1)/2 doubles), as the C ABI takes it
    const double* data() const { return matrix_.data(); }
    double* data() { return matrix_.data(); }

    /// binary format of source/c_matrix.cpp:42-85: [int nPix][doubles][int len][chars]
    void readFromFile(const char* fileName)
    {
        std::ifstream in(fileName, std::ios::in | std::ios::binary);
        if (!in) cosmopp_gb300_detail::raise(std::string("Covariance matrix file ") + fileName + " cannot be read.");
        in.read((char*)&nPix_, sizeof(int));
        initialize();
        in.read((char*)matrix_.data(), matrix_.size() * sizeof(double));
        int len = 0;
        in.read((char*)&len, sizeof(int));
        comment_.resize(len);
        if (len) in.read(&comment_[0], len);
    }
    void writeIntoFile(const char* fileName) const
    {
        std::ofstream out(fileName, std::ios::binary | std::ios::out);
        if (!out) cosmopp_gb300_detail::raise(std::string("Cannot write into output file ") + fileName + ".");
        out.write((const char*)&nPix_, sizeof(int));
        out.write((const char*)matrix_.data(), matrix_.size() * sizeof(double));
        const int len = (int)comment_.size();
        out.write((const char*)&len, sizeof(int));
        if (len) out.write(comment_.data(), len);
    }
    /// text format of source/c_matrix.cpp:87-107: nPix, the comment, then "i<TAB>j<TAB>value" for
    /// i <= j, column by column, at the stream's default precision
    void writeIntoTextFile(const char* fileName) const
    {
        std::ofstream out(fileName);
        if (!out) cosmopp_gb300_detail::raise(std::string("Cannot write into output file ") + fileName + ".");
        out << nPix_ << std::endl;
        out << comment_ << std::endl;
        for (int j = 0; j < nPix_; ++j)
            for (int i = 0; i <= j; ++i) out << i << '\t' << j << '\t' << element(i, j) << std::endl;
    }
    /// reads what writeIntoTextFile writes (source/c_matrix.cpp:109-154 takes the same layout; it
    /// reads one whitespace-separated token per entry, so here the i, j, value triples are read
    /// as written); an index outside the matrix raises, as there
    void readFromTextFile(const char* fileName)
    {
        std::ifstream in(fileName);
        if (!in) cosmopp_gb300_detail::raise(std::string("Cannot read the input file ") + fileName + ".");
        in >> nPix_;
        initialize();
        std::string rest;
        std::getline(in, rest);
        std::getline(in, comment_);
        int i, j;
        double val;
        while (in >> i >> j >> val) {
            if (i < 0 || i >= nPix_) cosmopp_gb300_detail::raise("Invalid index i = " + std::to_string(i) + ".");
            if (j < 0 || j >= nPix_) cosmopp_gb300_detail::raise("Invalid index j = " + std::to_string(j) + ".");
            element(i, j) = val;
        }
    }
    /// source/c_matrix.cpp:183-201
    void maskMatrix(const std::vector<int>& goodPixels)
    {
        const int g = (int)goodPixels.size();
        std::vector<double> m((size_t)g * (g + 1) / 2);
        for (int j = 0; j < g; ++j)
            for (int i = 0; i <= j; ++i) m[(size_t)j * (j + 1) / 2 + i] = element(goodPixels[i], goodPixels[j]);
        nPix_ = g;
        matrix_.swap(m);
    }

private:
    size_t getIndex(int i, int j) const
    {
        if (i > j) std::swap(i, j);
        return (size_t)j * (j + 1) / 2 + i;
    }
    void initialize()
    {
        if (nPix_ <= 0) cosmopp_gb300_detail::raise("the number of pixels must be positive.");
        matrix_.assign((size_t)nPix_ * (nPix_ + 1) / 2, 0.0);
    }
    int nPix_ = 0;
    std::vector<double> matrix_;
    std::string comment_;
};

/// Table of P_l(n_i . n_j), l = 0..lMax, i <= j, for a pixel set
/// (include/c_matrix_generator.hpp:10-36).  Built on the GPU with the reference's
/// recurrence and dot product (bit-identical values); the file format is the
/// reference's (int lMax, int nPix, then the packed table of every l).
class LegendrePolynomialContainer
{
public:
    /// source/c_matrix_generator.cpp:30-76; goodPixels in NEST ordering (NULL = all pixels)
    LegendrePolynomialContainer(int lMax, long nSide, const std::vector<int>* goodPixels = NULL, int device = 0)
        : lMax_(lMax)
    {
        if (lMax < 0 || lMax > CG_FIDUCIAL_LMAX_MAX) cosmopp_gb300_detail::raise("LegendrePolynomialContainer: invalid lMax");
        cg_config cfg;
        cg_config_init(&cfg);
        cfg.nside = nSide;
        cfg.scheme = CG_SCHEME_NEST;
        if (goodPixels) {
            cfg.good_pixels = goodPixels->data();
            cfg.n = (int)goodPixels->size();
        }
        cfg.lmax = lMax < 2 ? 2 : lMax;
        cfg.fwhm_deg = 1.0;
        cfg.device = device;
        cg_ctx* ctx = NULL;
        cosmopp_gb300_detail::check(cg_create(&ctx, &cfg), "LegendrePolynomialContainer", cg_last_error(NULL));
        nPix_ = cg_get_n(ctx);
        data_.resize((size_t)(lMax + 1) * pairs());
        const int rc = cg_legendre_table(ctx, 0, lMax + 1, data_.data());
        std::string err = rc ? cg_last_error(ctx) : "";
        cg_destroy(ctx);
        cosmopp_gb300_detail::check(rc, "LegendrePolynomialContainer", err.c_str());
    }
    /// source/c_matrix_generator.cpp:89-134
    explicit LegendrePolynomialContainer(const char* fileName)
    {
        std::ifstream in(fileName, std::ios::in | std::ios::binary);
        if (!in) cosmopp_gb300_detail::raise(std::string("Cannot open input file ") + fileName + ".");
        int lMax = -1, nPix = -1;
        in.read((char*)&lMax, sizeof(int));
        if (lMax < 0) cosmopp_gb300_detail::raise("Invalid lMax = " + std::to_string(lMax) + " read from file " + fileName + ".");
        in.read((char*)&nPix, sizeof(int));
        if (nPix < 0) cosmopp_gb300_detail::raise("Invalid nPix = " + std::to_string(nPix) + " read from file " + fileName + ".");
        lMax_ = lMax;
        nPix_ = nPix;
        data_.resize((size_t)(lMax + 1) * pairs());
        in.read((char*)data_.data(), (std::streamsize)(sizeof(double) * data_.size()));
        if (!in) cosmopp_gb300_detail::raise(std::string("Truncated Legendre table in ") + fileName + ".");
    }
    /// P_l(n_i . n_j) for i <= j (source/c_matrix_generator.cpp:78-87)
    double value(int l, int j, int i) const { return data_[(size_t)l * pairs() + (size_t)j * (j + 1) / 2 + i]; }
    /// source/c_matrix_generator.cpp:136-162
    void writeIntoFile(const char* fileName) const
    {
        std::ofstream out(fileName, std::ios::binary | std::ios::out);
        if (!out) cosmopp_gb300_detail::raise(std::string("Cannot write into file ") + fileName + ".");
        out.write((const char*)&lMax_, sizeof(int));
        out.write((const char*)&nPix_, sizeof(int));
        out.write((const char*)data_.data(), (std::streamsize)(sizeof(double) * data_.size()));
    }
    int lMax() const { return lMax_; }
    int nPix() const { return nPix_; }

private:
    size_t pairs() const { return (size_t)nPix_ * (nPix_ + 1) / 2; }
    int lMax_ = -1, nPix_ = 0;
    std::vector<double> data_;  // [l][j(j+1)/2 + i]
};

namespace Utils
{
/// source/utils.cpp:173-217: one C_l per line from l = 0 (hasL: each line starts with l;
/// isDl: the values are D_l = l(l+1) C_l / (2 pi) for l > 0); stops at the first empty line
inline void readClFromFile(const char* fileName, std::vector<double>& cl, bool hasL = false, bool isDl = false)
{
    std::ifstream in(fileName);
    if (!in) cosmopp_gb300_detail::raise(std::string("Cannot open the input file ") + fileName + ".");
    cl.clear();
    int l = 0;
    while (!in.eof()) {
        std::string s;
        std::getline(in, s);
        if (s == "") break;
        std::stringstream str(s);
        int dummyL;
        double val;
        if (hasL) {
            str >> dummyL;
            if (dummyL != l)
                cosmopp_gb300_detail::raise(std::string("Invalid format of the input file ") + fileName +
                                            ". Expected to read l = " + std::to_string(l) + " but found l = " +
                                            std::to_string(dummyL) + ".");
        }
        str >> val;
        if (isDl && l) val *= (2 * M_PI / (l * (l + 1)));
        cl.push_back(val);
        ++l;
    }
}
}  // namespace Utils

/// Converts C_l to pixel-space covariance matrices on the GPU.
class CMatrixGenerator
{
public:
    /// source/c_matrix_generator.cpp:164-232; goodPixels in NEST ordering (NULL = all pixels),
    /// fwhm in degrees, lmax = cl.size() - 1.  Bit-identical to the reference.  Returns a new
    /// CMatrix the caller deletes, as the reference does.  A table lp is checked against the
    /// pixel count and lmax but not read: its values are the ones the device's recurrence
    /// computes, so the matrix is the same with or without it.
    static CMatrix* clToCMatrix(const std::vector<double>& cl, long nSide, double fwhm,
                                const std::vector<int>* goodPixels = NULL, const LegendrePolynomialContainer* lp = NULL,
                                int device = 0)
    {
        if (cl.size() < 3) cosmopp_gb300_detail::raise("clToCMatrix: cl must reach at least l = 2");
        if (lp) {
            const long nPix = goodPixels ? (long)goodPixels->size() : (long)cg_nside2npix(nSide);
            if (lp->nPix() != nPix || lp->lMax() < (int)cl.size() - 1)
                cosmopp_gb300_detail::raise("clToCMatrix: the Legendre table does not cover these pixels and l");
        }
        cg_config cfg;
        cg_config_init(&cfg);
        cfg.nside = nSide;
        cfg.scheme = CG_SCHEME_NEST;
        if (goodPixels) {
            cfg.good_pixels = goodPixels->data();
            cfg.n = (int)goodPixels->size();
        }
        cfg.lmax = (int)cl.size() - 1;
        cfg.fwhm_deg = fwhm;
        cfg.device = device;
        cg_ctx* ctx = NULL;
        cosmopp_gb300_detail::check(cg_create(&ctx, &cfg), "clToCMatrix", cg_last_error(NULL));
        CMatrix* m = new CMatrix(cg_get_n(ctx));
        const int rc = cg_build_cmatrix(ctx, cl.data(), m->data());
        std::string err = rc ? cg_last_error(ctx) : "";
        cg_destroy(ctx);
        if (rc) {
            delete m;
            cosmopp_gb300_detail::check(rc, "clToCMatrix", err.c_str());
        }
        return m;
    }
    /// source/c_matrix_generator.cpp:234-240: C_l read from a text file (Utils::readClFromFile,
    /// one value per line from l = 0); lMax is not used, as in the reference
    static CMatrix* clToCMatrix(const char* clFileName, long nSide, int /*lMax*/, double fwhm,
                                const std::vector<int>* goodPixels = NULL, const LegendrePolynomialContainer* lp = NULL,
                                int device = 0)
    {
        std::vector<double> cl;
        Utils::readClFromFile(clFileName, cl);
        return clToCMatrix(cl, nSide, fwhm, goodPixels, lp, device);
    }
    /// source/c_matrix_generator.cpp:706-772: sum over l = lMax+1 .. 4 nSide plus the
    /// monopole/dipole term 100 C_2 (1 + x) B_2^2; cl must reach l = 4 nSide.  Bit-identical
    /// to the reference.  Returns a new CMatrix the caller deletes.
    static CMatrix* getFiducialMatrix(const std::vector<double>& cl, long nSide, int lMax, double fwhm,
                                      const std::vector<int>* goodPixels = NULL,
                                      const LegendrePolynomialContainer* lp = NULL, int device = 0)
    {
        const int lMaxMax = (int)(4 * nSide);
        if ((long)cl.size() < lMaxMax + 1) cosmopp_gb300_detail::raise("getFiducialMatrix: cl must reach l = 4 nSide");
        if (lp) {
            const long nPix = goodPixels ? (long)goodPixels->size() : (long)cg_nside2npix(nSide);
            if (lp->nPix() != nPix || lp->lMax() < lMaxMax)
                cosmopp_gb300_detail::raise("getFiducialMatrix: the Legendre table does not cover these pixels and l");
        }
        cg_config cfg;
        cg_config_init(&cfg);
        cfg.nside = nSide;
        cfg.scheme = CG_SCHEME_NEST;
        if (goodPixels) {
            cfg.good_pixels = goodPixels->data();
            cfg.n = (int)goodPixels->size();
        }
        cfg.lmax = lMax;
        cfg.fwhm_deg = fwhm;
        cfg.device = device;
        cg_ctx* ctx = NULL;
        cosmopp_gb300_detail::check(cg_create(&ctx, &cfg), "getFiducialMatrix", cg_last_error(NULL));
        CMatrix* m = new CMatrix(cg_get_n(ctx));
        m->comment() = "fiducial matrix";
        const int rc = cg_fiducial_matrix(ctx, cl.data(), lMax, lMaxMax, NULL, m->data());
        std::string err = rc ? cg_last_error(ctx) : "";
        cg_destroy(ctx);
        if (rc) {
            delete m;
            cosmopp_gb300_detail::check(rc, "getFiducialMatrix", err.c_str());
        }
        return m;
    }
    /// source/c_matrix_generator.cpp:697-703: C_l read from a text file
    static CMatrix* getFiducialMatrix(const char* clFileName, long nSide, int lMax, double fwhm,
                                      const std::vector<int>* goodPixels = NULL,
                                      const LegendrePolynomialContainer* lp = NULL, int device = 0)
    {
        std::vector<double> cl;
        Utils::readClFromFile(clFileName, cl);
        return getFiducialMatrix(cl, nSide, lMax, fwhm, goodPixels, lp, device);
    }
    /// source/c_matrix_generator.cpp:774-787 (full sky, noise^2 on the diagonal)
    static CMatrix* generateNoiseMatrix(long nSide, double noise = 1e-3)
    {
        const int nPix = (int)cg_nside2npix(nSide);
        CMatrix* m = new CMatrix(nPix);
        m->comment() = "noise matrix";
        for (int i = 0; i < nPix; ++i) m->element(i, i) = noise * noise;
        return m;
    }
};

struct LikelihoodResult
{
    std::string mapName;
    double logDet;
    double chi2;
    double like;
    inline bool operator<(const LikelihoodResult& other) const { return like < other.like; }
};

/// Likelihood for temperature maps (source/likelihood.cpp:38-328), factorised on the GPU.
class Likelihood
{
public:
    Likelihood(const CMatrix& cMatrix, const CMatrix& fiducialMatrix, const CMatrix& noiseMatrix,
               const std::vector<int>& goodPixels, const std::vector<double>& foreground, int device = 0)
        : goodPixels_(goodPixels)
    {
        const size_t g = goodPixels.size();
        sizeCheck(cMatrix, g, "c.dat");
        sizeCheck(fiducialMatrix, g, "c_fiducial.dat");
        sizeCheck(noiseMatrix, g, "c_noise.dat");
        const int rc = cg_likelihood_create(&lik_, (int)g, cMatrix.data(), fiducialMatrix.data(), noiseMatrix.data(),
                                            foreground.empty() ? NULL : foreground.data(), device);
        if (rc == CG_ERR_NOT_PD)
            cosmopp_gb300_detail::raise("The determinant of the covariance matrix is not positive. The covariance "
                                        "matrix must be positive definite.");
        cosmopp_gb300_detail::check(rc, "Likelihood", cg_likelihood_last_error(NULL));
    }
    ~Likelihood() { cg_likelihood_destroy(lik_); }
    Likelihood(const Likelihood&) = delete;
    Likelihood& operator=(const Likelihood&) = delete;

    /// source/likelihood.cpp:164-180; logDet includes the reference's detOffset
    double calculate(const std::vector<double>& t, double& chi2, double& logDet) const
    {
        if (t.size() != goodPixels_.size()) cosmopp_gb300_detail::raise("calculate: map size differs from goodPixels");
        cosmopp_gb300_detail::check(cg_likelihood_calculate(lik_, t.data(), &chi2, &logDet), "Likelihood::calculate",
                                    cg_likelihood_last_error(lik_));
        const double detOffset = -29677.0566;  // source/likelihood.cpp:127
        logDet -= detOffset;
        return chi2 + logDet;
    }
    /// source/likelihood.cpp:285-328
    void calculateAll(const std::vector<std::vector<double> >& t, const std::vector<std::string>& mapNames,
                      std::vector<LikelihoodResult>& results) const
    {
        if (mapNames.size() != t.size()) cosmopp_gb300_detail::raise("calculateAll: names and maps differ in number");
        for (size_t i = 0; i < t.size(); ++i) {
            LikelihoodResult r;
            r.mapName = mapNames[i];
            r.like = calculate(t[i], r.chi2, r.logDet);
            results.push_back(r);
        }
    }

private:
    static void sizeCheck(const CMatrix& m, size_t g, const char* what)
    {
        if ((size_t)m.getNPix() != g) {
            std::stringstream s;
            s << "There are " << g << " unmasked pixels, however the covariance matrix in " << what
              << " corresponds to " << m.getNPix() << ". Please generate the covariance matrix with the same mask.";
            cosmopp_gb300_detail::raise(s.str());
        }
    }
    cg_lik* lik_ = NULL;
    std::vector<int> goodPixels_;
};

/// -2lnL and its gradient for one data map, parameters ln C_l (or C_l) for
/// l = lMin .. lMin + nParams - 1, as the reference's HMC consumes them
/// (Math::LikelihoodWithDerivs; all derivatives are of -2 ln L).  One GPU
/// evaluation gives -2lnL and the whole gradient, cached for the last point,
/// so HMC's n_par calculateDeriv calls (source/hmc.cpp:158-163) cost one call.
class PixelLikelihoodWithDerivs : public Math::LikelihoodWithDerivs
{
public:
    PixelLikelihoodWithDerivs(cg_ctx* ctx, const std::vector<double>& map, const std::vector<double>& clTemplate,
                              int lMin = 2, bool logParams = true)
        : ctx_(ctx), map_(map), cl_(clTemplate), lMin_(lMin), log_(logParams), grad_(clTemplate.size())
    {
    }
    double calculate(double* params, int nParams) override
    {
        eval(params, nParams);
        return value_;
    }
    double calculateDeriv(double* params, int nParams, int i) override
    {
        eval(params, nParams);
        return dparam_[i];
    }
    /// full gradient of -2lnL w.r.t. the parameters at x
    void gradient(const std::vector<double>& x, std::vector<double>* g)
    {
        eval(const_cast<double*>(x.data()), (int)x.size());
        *g = dparam_;
    }

private:
    void eval(double* params, int nParams)
    {
        if ((int)last_.size() == nParams && std::equal(last_.begin(), last_.end(), params)) return;
        std::vector<double> cl = cl_;
        for (int k = 0; k < nParams; ++k) cl[lMin_ + k] = log_ ? std::exp(params[k]) : params[k];
        int st = 0;
        double chi2, logdet;
        cosmopp_gb300_detail::check(cg_loglike(ctx_, 1, cl.data(), map_.data(), 0, &value_, &chi2, &logdet,
                                               grad_.data(), &st),
                                    "PixelLikelihoodWithDerivs", cg_last_error(ctx_));
        if (st != CG_OK) cosmopp_gb300_detail::raise("PixelLikelihoodWithDerivs: covariance not positive definite");
        dparam_.resize(nParams);
        for (int k = 0; k < nParams; ++k) {
            const int l = lMin_ + k;
            dparam_[k] = log_ ? grad_[l] * cl[l] : grad_[l];
        }
        last_.assign(params, params + nParams);
    }
    cg_ctx* ctx_;
    std::vector<double> map_, cl_;
    int lMin_;
    bool log_;
    std::vector<double> grad_, dparam_, last_;
    double value_ = 0;
};

/// set / value / derivative Function for HMCGeneral and LBFGS_General
/// (include/hmc_general.hpp:49-62, include/lbfgs_general.hpp:43-52), over any
/// LargeVector with contents() -> std::vector<double>& (BasicLargeVector).
template <typename LargeVector>
class PixelLikelihoodFunction
{
public:
    explicit PixelLikelihoodFunction(PixelLikelihoodWithDerivs& like) : like_(like) {}
    void set(const LargeVector& x) { x_ = x.contents(); }
    double value() { return like_.calculate(x_.data(), (int)x_.size()); }
    void derivative(LargeVector* res)
    {
        std::vector<double> g;
        like_.gradient(x_, &g);
        res->contents() = g;
    }

private:
    PixelLikelihoodWithDerivs& like_;
    std::vector<double> x_;
};

#endif
