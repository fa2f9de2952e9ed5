// Batched Hamiltonian Monte Carlo: many chains advance together, every leapfrog
// step one batched -2lnL + gradient call.
//
// Same update rules as the reference's Math::HMC::run (source/hmc.cpp:31-126):
//   p ~ N(0, m);  H = -2lnL(x) + sum p^2 / m
//   leapfrog: p -= tau/2 * g/2;  x += tau/m * p;  p -= tau/2 * g/2
//             (g is the derivative of -2lnL, hence the /2, source/hmc.cpp:84,91)
//   accept with probability exp(-(H_new - H_old) / 2)   (source/hmc.cpp:98-118)
// The reference draws tau uniformly in (0, tauMax] and the step count as
// ceil(nMax U) every iteration (source/hmc.cpp:59-60); jitter = 0 keeps them
// fixed at tau and nleap.  The random numbers come from one std::mt19937 seeded
// with `seed` through std::uniform_real_distribution<double>(0, 1) and
// std::normal_distribution<double>(0, 1), drawn in the reference's order (tau,
// step count, the momenta chain by chain, then one acceptance draw per chain),
// so one chain with jitter reproduces Math::HMC's chain for the same seed.
//
// cg_hmc_sample runs over any batched likelihood with gradient (a callback);
// cg_hmc_run is the pixel likelihood of a context, parameters x_l = ln C_l.
#include <cmath>
#include <random>
#include <vector>

#include "cg_internal.h"

extern "C" int cg_hmc_sample(int nchains, int npar, cg_batch_like_grad_fn like, void* user, const double* x0,
                             int niter, int nleap, double tau, const double* mass, int jitter,
                             unsigned long long seed, double* chain, double* accept_rate)
{
    if (!like || !x0 || !chain || nchains < 1 || npar < 1 || niter < 1 || nleap < 1 || !(tau > 0))
        return CG_ERR_BAD_ARG;
    const int np = npar;
    std::vector<double> m(np, 1.0);
    if (mass)
        for (int k = 0; k < np; ++k) {
            if (!(mass[k] > 0)) return CG_ERR_BAD_ARG;
            m[k] = mass[k];
        }
    std::mt19937 gen((std::mt19937::result_type)seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    std::normal_distribution<double> gauss(0.0, 1.0);
    std::vector<double> x(x0, x0 + (size_t)nchains * np), xn(x), p((size_t)nchains * np);
    std::vector<double> u(nchains), un(nchains), gx((size_t)nchains * np), gxn(gx), kin0(nchains);
    std::vector<int> acc(nchains, 0);

    auto record = [&](int it) {
        for (int c = 0; c < nchains; ++c) {
            double* row = chain + ((size_t)it * nchains + c) * (np + 1);
            row[0] = u[c];
            for (int k = 0; k < np; ++k) row[1 + k] = x[(size_t)c * np + k];
        }
    };
    int rc = like(user, nchains, x.data(), u.data(), gx.data());
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
        for (int c = 0; c < nchains; ++c) {
            double kin = 0;
            for (int k = 0; k < np; ++k) {
                const double v = std::sqrt(m[k]) * gauss(gen);
                p[(size_t)c * np + k] = v;
                kin += v * v / m[k];
            }
            kin0[c] = kin;
        }
        xn = x;
        gxn = gx;
        for (int s = 0; s < nsteps; ++s) {
            for (size_t i = 0; i < p.size(); ++i) {
                const int k = (int)(i % np);
                p[i] -= t / 2 * gxn[i] / 2;
                xn[i] += t / m[k] * p[i];
            }
            if ((rc = like(user, nchains, xn.data(), un.data(), gxn.data()))) return rc;
            for (size_t i = 0; i < p.size(); ++i) p[i] -= t / 2 * gxn[i] / 2;
        }
        for (int c = 0; c < nchains; ++c) {
            double kin = 0;
            for (int k = 0; k < np; ++k) kin += p[(size_t)c * np + k] * p[(size_t)c * np + k] / m[k];
            // deltaLike = newLike + newPLike - currentLike - oldPLike, in the reference's order
            const double dh = un[c] + kin - u[c] - kin0[c];
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

namespace {

// the pixel likelihood of a context over parameters x = ln C_l (l = 2 .. lmax), the rest of C_l
// from a template: -2lnL and d(-2lnL)/d ln C_l = C_l d(-2lnL)/dC_l; a proposal the likelihood
// cannot evaluate (a bad status) gets -2lnL = +inf and is rejected
struct PixelTarget {
    cg_ctx* ctx;
    const double* map;
    const double* cl_template;
    std::vector<double> cl, g;
    std::vector<int> st;
};

int pixel_like_grad(void* user, int nchains, const double* x, double* m2lnl, double* grad)
{
    PixelTarget& T = *static_cast<PixelTarget*>(user);
    const int L1 = T.ctx->lmax + 1, np = L1 - 2;
    for (int c = 0; c < nchains; ++c) {
        for (int l = 0; l < L1; ++l) T.cl[(size_t)c * L1 + l] = T.cl_template[l];
        for (int k = 0; k < np; ++k) T.cl[(size_t)c * L1 + 2 + k] = std::exp(x[(size_t)c * np + k]);
    }
    const int rc = cg_loglike(T.ctx, nchains, T.cl.data(), T.map, 0, m2lnl, nullptr, nullptr, T.g.data(), T.st.data());
    if (rc) return rc;
    for (int c = 0; c < nchains; ++c) {
        if (T.st[c] != CG_OK) m2lnl[c] = INFINITY;
        for (int k = 0; k < np; ++k)
            grad[(size_t)c * np + k] = T.g[(size_t)c * L1 + 2 + k] * T.cl[(size_t)c * L1 + 2 + k];
    }
    return CG_OK;
}

}  // namespace

extern "C" int cg_hmc_run(cg_ctx* ctx, const double* map, int nchains, const double* x0, const double* cl_template,
                          int niter, int nleap, double tau, const double* mass, int jitter, unsigned long long seed,
                          double* chain, double* accept_rate)
{
    if (!ctx || !map || !x0 || !cl_template || !chain || nchains < 1 || nchains > ctx->max_batch || niter < 1 ||
        nleap < 1 || !(tau > 0)) {
        if (ctx) ctx->err = "bad arguments to cg_hmc_run";
        return CG_ERR_BAD_ARG;
    }
    const int L1 = ctx->lmax + 1, np = ctx->lmax - 1;
    if (mass)
        for (int k = 0; k < np; ++k)
            if (!(mass[k] > 0)) { ctx->err = "HMC masses must be positive"; return CG_ERR_BAD_ARG; }
    PixelTarget T{ctx, map, cl_template, std::vector<double>((size_t)nchains * L1),
                  std::vector<double>((size_t)nchains * L1), std::vector<int>(nchains)};
    return cg_hmc_sample(nchains, np, pixel_like_grad, &T, x0, niter, nleap, tau, mass, jitter, seed, chain,
                         accept_rate);
}
