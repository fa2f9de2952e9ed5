// The reference's own low-l flow (source/test_like_low.cpp:183-193) through the
// C++ drop-in classes: clToCMatrix -> generateNoiseMatrix + maskMatrix ->
// Likelihood(C, zero fiducial, N, goodPixels, {}) -> calculate(d), then a few
// HMC-style leapfrog steps on PixelLikelihoodWithDerivs (source/hmc.cpp:78-96).
// Input (argv[1]): nside lmax fwhm sigma n, goodPixels[n], cl[lmax+1], d[n], and
// optionally lmaxmax clFull[lmaxmax+1]: then the fiducial matrix is
// getFiducialMatrix(clFull, nside, lmax, fwhm, &goodPixels) as the reference's
// test builds it (written raw into argv[3]), else zero.
// Output: the packed C as raw doubles into argv[2], then one line
// "like chi2 logDet" and "hmc <final -2lnL> <accepted>" on stdout.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include <cosmopp_gb300/cosmopp.hpp>

int main(int argc, char** argv)
{
    if (argc < 3) return 2;
    std::ifstream in(argv[1]);
    long nside;
    int lmax, n;
    double fwhm, sigma;
    in >> nside >> lmax >> fwhm >> sigma >> n;
    std::vector<int> good(n);
    for (int& g : good) in >> g;
    std::vector<double> cl(lmax + 1), d(n);
    for (double& c : cl) in >> c;
    for (double& v : d) in >> v;
    int lmaxmax = 0;
    std::vector<double> clFull;
    if (in >> lmaxmax) {
        clFull.resize(lmaxmax + 1);
        for (double& c : clFull) in >> c;
    }
    try {
        CMatrix* c = CMatrixGenerator::clToCMatrix(cl, nside, fwhm, &good);
        {
            std::ofstream out(argv[2], std::ios::binary);
            out.write((const char*)c->data(), sizeof(double) * (size_t)n * (n + 1) / 2);
        }
        CMatrix* noise = CMatrixGenerator::generateNoiseMatrix(nside, sigma);
        noise->maskMatrix(good);
        CMatrix* fid = clFull.empty() ? new CMatrix(n)
                                      : CMatrixGenerator::getFiducialMatrix(clFull, nside, lmax, fwhm, &good);
        if (!clFull.empty() && argc > 3) {
            std::ofstream out(argv[3], std::ios::binary);
            out.write((const char*)fid->data(), sizeof(double) * (size_t)n * (n + 1) / 2);
        }
        Likelihood like(*c, *fid, *noise, good, std::vector<double>());
        delete fid;
        double chi2, logDet;
        const double l = like.calculate(d, chi2, logDet);
        std::printf("%.17g %.17g %.17g\n", l, chi2, logDet);
        delete c;
        delete noise;

        // leapfrog on ln C_l, l = 2..lmax, as Math::HMC drives a LikelihoodWithDerivs
        cg_config cfg;
        cg_config_init(&cfg);
        cfg.nside = nside;
        cfg.scheme = CG_SCHEME_NEST;
        cfg.good_pixels = good.data();
        cfg.n = n;
        cfg.lmax = lmax;
        cfg.fwhm_deg = fwhm;
        cfg.noise_sigma = sigma;
        cg_ctx* ctx = NULL;
        if (cg_create(&ctx, &cfg) != CG_OK) return 3;
        PixelLikelihoodWithDerivs f(ctx, d, cl, 2, true);
        const int np = lmax - 1;
        std::vector<double> x(np), p(np, 0.0);
        for (int k = 0; k < np; ++k) x[k] = std::log(cl[2 + k]);
        const double tau = 0.01;
        double h0 = f.calculate(x.data(), np);
        for (int k = 0; k < np; ++k) p[k] = (k % 2 ? 0.5 : -0.5);
        double k0 = 0;
        for (double v : p) k0 += v * v;
        for (int s = 0; s < 10; ++s) {
            for (int k = 0; k < np; ++k) p[k] -= tau / 2 * f.calculateDeriv(x.data(), np, k) / 2;
            for (int k = 0; k < np; ++k) x[k] += tau * p[k];
            for (int k = 0; k < np; ++k) p[k] -= tau / 2 * f.calculateDeriv(x.data(), np, k) / 2;
        }
        double k1 = 0;
        for (double v : p) k1 += v * v;
        const double h1 = f.calculate(x.data(), np);
        // energy conservation of the leapfrog: -2lnL/2 + p^2/2 (source/hmc.cpp:98-104)
        std::printf("hmc %.17g %.17g\n", h1, (h1 / 2 + k1 / 2) - (h0 / 2 + k0 / 2));
        cg_destroy(ctx);
    } catch (std::exception& e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 1;
    }
    return 0;
}
