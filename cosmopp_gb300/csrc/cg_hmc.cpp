// Batched Hamiltonian Monte Carlo over the pixel likelihood: many chains
// advance together, every leapfrog step one batched -2lnL + gradient call.
//
// Same update rules as the reference's Math::HMC::run (source/hmc.cpp:31-126):
//   p ~ N(0, m);  H = -2lnL(x) + sum p^2 / m
//   leapfrog: p -= tau/2 * g/2;  x += tau/m * p;  p -= tau/2 * g/2
//             (g is the derivative of -2lnL, hence the /2, source/hmc.cpp:84,91)
//   accept with probability exp(-(H_new - H_old) / 2)   (source/hmc.cpp:98-118)
// with parameters x_l = ln C_l for l = 2 .. lmax.  The reference draws tau
// uniformly in (0, tauMax] and the step count as ceil(nMax U) every iteration
// (source/hmc.cpp:59-60); jitter = 0 keeps them fixed at tau and nleap.
#include <cmath>
#include <random>
#include <vector>

#include "cg_internal.h"

extern "C" int cg_hmc_run(cg_ctx* ctx, const double* map, int nchains, const double* x0, const double* cl_template,
                          int niter, int nleap, double tau, const double* mass, int jitter, unsigned long long seed,
                          double* chain, double* accept_rate)
{
    if (!ctx || !map || !x0 || !cl_template || !chain || nchains < 1 || nchains > ctx->max_batch || niter < 1 ||
        nleap < 1 || !(tau > 0)) {
        if (ctx) ctx->err = "bad arguments to cg_hmc_run";
        return CG_ERR_BAD_ARG;
    }
    const int lmax = ctx->lmax, L1 = lmax + 1, np = lmax - 1;
    std::vector<double> m(np, 1.0);
    if (mass)
        for (int k = 0; k < np; ++k) {
            if (!(mass[k] > 0)) { ctx->err = "HMC masses must be positive"; return CG_ERR_BAD_ARG; }
            m[k] = mass[k];
        }
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    std::normal_distribution<double> gauss(0.0, 1.0);
    std::vector<double> x(x0, x0 + (size_t)nchains * np), xn(x), p((size_t)nchains * np);
    std::vector<double> cl((size_t)nchains * L1), u(nchains), un(nchains), g((size_t)nchains * L1), gn(g);
    std::vector<double> gx((size_t)nchains * np), gxn(gx);
    std::vector<int> st(nchains), acc(nchains, 0);

    // -2lnL and d(-2lnL)/d ln C_l at parameter vectors xs
    auto evaluate = [&](const std::vector<double>& xs, std::vector<double>& uu, std::vector<double>& gg,
                        std::vector<double>& gxx) -> int {
        for (int c = 0; c < nchains; ++c) {
            for (int l = 0; l < L1; ++l) cl[(size_t)c * L1 + l] = cl_template[l];
            for (int k = 0; k < np; ++k) cl[(size_t)c * L1 + 2 + k] = std::exp(xs[(size_t)c * np + k]);
        }
        const int rc = cg_loglike(ctx, nchains, cl.data(), map, 0, uu.data(), nullptr, nullptr, gg.data(), st.data());
        if (rc) return rc;
        for (int c = 0; c < nchains; ++c) {
            if (st[c] != CG_OK) uu[c] = INFINITY;  // a proposal the likelihood cannot evaluate is rejected
            for (int k = 0; k < np; ++k)
                gxx[(size_t)c * np + k] = gg[(size_t)c * L1 + 2 + k] * cl[(size_t)c * L1 + 2 + k];
        }
        return CG_OK;
    };
    auto record = [&](int it) {
        for (int c = 0; c < nchains; ++c) {
            double* row = chain + ((size_t)it * nchains + c) * (np + 1);
            row[0] = u[c];
            for (int k = 0; k < np; ++k) row[1 + k] = x[(size_t)c * np + k];
        }
    };
    int rc = evaluate(x, u, g, gx);
    if (rc) return rc;
    record(0);
    for (int it = 1; it <= niter; ++it) {
        double t = tau;
        int nsteps = nleap;
        if (jitter) {
            t = uni(gen) * tau;
            nsteps = (int)std::ceil(nleap * uni(gen));
            if (nsteps < 1) nsteps = 1;
        }
        std::vector<double> h0(nchains, 0.0);
        for (int c = 0; c < nchains; ++c) {
            double kin = 0;
            for (int k = 0; k < np; ++k) {
                const double v = std::sqrt(m[k]) * gauss(gen);
                p[(size_t)c * np + k] = v;
                kin += v * v / m[k];
            }
            h0[c] = u[c] + kin;
        }
        xn = x;
        gxn = gx;
        for (int s = 0; s < nsteps; ++s) {
            for (size_t i = 0; i < p.size(); ++i) {
                const int k = (int)(i % np);
                p[i] -= t / 2 * gxn[i] / 2;
                xn[i] += t / m[k] * p[i];
            }
            if ((rc = evaluate(xn, un, gn, gxn))) return rc;
            for (size_t i = 0; i < p.size(); ++i) p[i] -= t / 2 * gxn[i] / 2;
        }
        for (int c = 0; c < nchains; ++c) {
            double kin = 0;
            for (int k = 0; k < np; ++k) kin += p[(size_t)c * np + k] * p[(size_t)c * np + k] / m[k];
            const double dh = un[c] + kin - h0[c];
            const double q = uni(gen);
            if (std::isfinite(dh) && q <= std::exp(-dh / 2)) {
                ++acc[c];
                for (int k = 0; k < np; ++k) {
                    x[(size_t)c * np + k] = xn[(size_t)c * np + k];
                    gx[(size_t)c * np + k] = gxn[(size_t)c * np + k];
                }
                u[c] = un[c];
            }
        }
        record(it);
    }
    if (accept_rate)
        for (int c = 0; c < nchains; ++c) accept_rate[c] = (double)acc[c] / niter;
    return CG_OK;
}
