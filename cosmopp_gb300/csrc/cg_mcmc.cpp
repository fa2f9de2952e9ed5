// Batched Metropolis-Hastings: many chains advance together, and every block
// update is one batched likelihood call over all chains.
//
// Same rules as the reference's MetropolisHastings::run (source/mcmc.cpp:455-700):
//   * parameters move block by block (specifyParameterBlocks; one block per
//     parameter by default, source/mcmc.cpp:58,548-651);
//   * the proposal is x_j + N(0,1) samplingWidth_j for j in the block
//     (generateNewPoint, include/mcmc.hpp:138), or, once the adaptive covariance
//     is ready, x + L g with g ~ N(0,1) on the block's entries and zero elsewhere
//     and L the lower Cholesky factor of the proposal covariance
//     (source/mcmc.cpp:555-572);
//   * the prior is a product of uniform 1/(max-min) on [min, max] and Gaussian
//     densities (include/mcmc.hpp:350-392); a proposal outside the prior is not
//     evaluated and keeps the old likelihood (source/mcmc.cpp:590-595);
//   * p = prior_new/prior_old exp(-(like_new - like_old)/2), capped at 1, accept
//     when U <= p (source/mcmc.cpp:605-650);
//   * the adaptive covariance (Haario et al.) is updated every 100 iterations
//     from every chain's sums of x and x x^T since the last update, chain by
//     chain, with factor 2.4^2/n and epsilon 1e-7 on the diagonal
//     (updateCovarianceMatrix, include/mcmc.hpp:660-699, pooled the way the MPI
//     master pools its chains, source/mcmc.cpp:226-340); it is used once more
//     than 100 states have entered it.
// The reference's forced move for approximate likelihoods, its resume files and
// its stopping rules are not part of this driver: it runs a fixed number of
// iterations and returns the chains (Gelman-Rubin R is in diagnostics.py).
#include <cmath>
#include <random>
#include <vector>

#include "cg_internal.h"

namespace {

double prior_of(int np, const int* mode, const double* p1, const double* p2, const double* x)
{
    if (!mode) return 1.0;
    double r = 1.0;
    for (int i = 0; i < np; ++i) {
        if (mode[i] == CG_PRIOR_UNIFORM) {
            r *= (x[i] >= p1[i] && x[i] <= p2[i]) ? 1.0 / (p2[i] - p1[i]) : 0.0;
        } else {
            const double d = x[i] - p1[i];
            r *= 1.0 / (std::sqrt(2 * M_PI) * p2[i]) * std::exp(-d * d / (2 * p2[i] * p2[i]));
        }
    }
    return r;
}

// Lower Cholesky factor of a symmetric matrix (row-major, in place below the
// diagonal); false if a pivot is not positive.
bool cholesky_lower(int n, std::vector<double>& a)
{
    for (int j = 0; j < n; ++j) {
        double s = a[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) s -= a[(size_t)j * n + k] * a[(size_t)j * n + k];
        if (!(s > 0)) return false;
        const double d = std::sqrt(s);
        a[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double t = a[(size_t)i * n + j];
            for (int k = 0; k < j; ++k) t -= a[(size_t)i * n + k] * a[(size_t)j * n + k];
            a[(size_t)i * n + j] = t / d;
        }
        for (int k = j + 1; k < n; ++k) a[(size_t)j * n + k] = 0.0;
    }
    return true;
}

struct Adaptive {
    int n;
    double factor, eps = 1e-7;
    unsigned long count = 0;           // covarianceElementsNum_
    std::vector<double> mean, mean_new, cov, chol;
    bool ready = false;
    explicit Adaptive(int np) : n(np), factor(2.4 * 2.4 / np), mean(np, 0.0), mean_new(np), cov((size_t)np * np, 0.0),
                                chol((size_t)np * np, 0.0) {}

    // include/mcmc.hpp:660-686 for one chain's sums over k states
    void update(unsigned long k, const double* sum, const double* msum)
    {
        const double c = (double)count, t = (double)(count + k);
        for (int i = 0; i < n; ++i) mean_new[i] = c / t * mean[i] + sum[i] / t;
        for (int i = 0; i < n; ++i)
            for (int j = i; j < n; ++j) {
                double& v = cov[(size_t)i * n + j];
                v = (c - 1) / (t - 1) * v +
                    factor / (t - 1) *
                        (c * mean[i] * mean[j] - t * mean_new[i] * mean_new[j] + msum[(size_t)i * n + j] +
                         (double)k * (i == j ? eps : 0.0));
                cov[(size_t)j * n + i] = v;
            }
        mean = mean_new;
        count += k;
    }
    // include/mcmc.hpp:688-698
    void refactor()
    {
        std::vector<double> a = cov;
        if (cholesky_lower(n, a)) {
            chol = a;
            if (count > 100) ready = true;
        }
    }
};

}  // namespace

extern "C" int cg_mh_sample(int nchains, int npar, cg_batch_like_fn like, void* user, const double* x0, int niter,
                            const double* sampling_width, const int* prior_mode, const double* prior_p1,
                            const double* prior_p2, int nblocks, const int* blocks, int adapt,
                            unsigned long long seed, double* chain, double* accept_rate, double* proposal_cov)
{
    if (nchains < 1 || npar < 1 || !like || !x0 || niter < 1 || !sampling_width || !chain) return CG_ERR_BAD_ARG;
    if (prior_mode) {
        if (!prior_p1 || !prior_p2) return CG_ERR_BAD_ARG;
        for (int i = 0; i < npar; ++i) {
            if (prior_mode[i] == CG_PRIOR_UNIFORM && !(prior_p2[i] > prior_p1[i])) return CG_ERR_BAD_ARG;
            if (prior_mode[i] == CG_PRIOR_GAUSS && !(prior_p2[i] > 0)) return CG_ERR_BAD_ARG;
            if (prior_mode[i] != CG_PRIOR_UNIFORM && prior_mode[i] != CG_PRIOR_GAUSS) return CG_ERR_BAD_ARG;
        }
    }
    std::vector<int> ends;
    if (nblocks > 0 && blocks) {
        int prev = 0;
        for (int b = 0; b < nblocks; ++b) {
            if (blocks[b] <= prev || blocks[b] > npar) return CG_ERR_BAD_ARG;
            ends.push_back(prev = blocks[b]);
        }
        if (prev != npar) return CG_ERR_BAD_ARG;
    } else {
        for (int i = 1; i <= npar; ++i) ends.push_back(i);  // one block per parameter, source/mcmc.cpp:58
    }
    const int nb = (int)ends.size();
    const size_t nx = (size_t)nchains * npar;

    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    std::normal_distribution<double> gauss(0.0, 1.0);
    std::vector<double> x(x0, x0 + nx), xold(nx), like_cur(nchains), like_new(nchains), prior_cur(nchains),
        prior_new(nchains), g(npar);
    std::vector<long> acc((size_t)nchains * nb, 0);

    int rc = like(user, nchains, x.data(), like_cur.data());
    if (rc) return rc;
    for (int c = 0; c < nchains; ++c) prior_cur[c] = prior_of(npar, prior_mode, prior_p1, prior_p2, &x[(size_t)c * npar]);

    Adaptive ad(npar);
    std::vector<unsigned long> win_n(nchains, 0);
    std::vector<double> win_sum(nx, 0.0), win_msum((size_t)nchains * npar * npar, 0.0);

    auto record = [&](int it) {
        for (int c = 0; c < nchains; ++c) {
            double* row = chain + ((size_t)it * nchains + c) * (npar + 1);
            row[0] = like_cur[c];
            for (int k = 0; k < npar; ++k) row[1 + k] = x[(size_t)c * npar + k];
        }
    };
    record(0);
    for (int it = 1; it <= niter; ++it) {
        int begin = 0;
        for (int b = 0; b < nb; ++b) {
            const int end = ends[b];
            xold = x;
            for (int c = 0; c < nchains; ++c) {
                double* xc = &x[(size_t)c * npar];
                if (adapt && ad.ready) {
                    for (int j = 0; j < npar; ++j) g[j] = 0.0;
                    for (int j = begin; j < end; ++j) g[j] = gauss(gen);
                    for (int i = 0; i < npar; ++i) {
                        double r = 0.0;
                        for (int j = 0; j <= i; ++j) r += ad.chol[(size_t)i * npar + j] * g[j];
                        xc[i] += r;
                    }
                } else {
                    for (int j = begin; j < end; ++j) xc[j] += gauss(gen) * sampling_width[j];
                }
                prior_new[c] = prior_of(npar, prior_mode, prior_p1, prior_p2, xc);
            }
            if ((rc = like(user, nchains, x.data(), like_new.data()))) return rc;
            for (int c = 0; c < nchains; ++c) {
                if (prior_new[c] == 0) like_new[c] = like_cur[c];
                double p = prior_new[c] / prior_cur[c];
                p *= std::exp(-(like_new[c] - like_cur[c]) / 2.0);
                if (!(p == p)) p = 0;  // a likelihood that could not be evaluated rejects
                if (p > 1) p = 1;
                const double q = uni(gen);
                if (q <= p) {
                    prior_cur[c] = prior_new[c];
                    like_cur[c] = like_new[c];
                    ++acc[(size_t)c * nb + b];
                } else {
                    for (int k = 0; k < npar; ++k) x[(size_t)c * npar + k] = xold[(size_t)c * npar + k];
                }
            }
            begin = end;
        }
        record(it);
        if (adapt) {
            for (int c = 0; c < nchains; ++c) {
                const double* xc = &x[(size_t)c * npar];
                ++win_n[c];
                for (int i = 0; i < npar; ++i) {
                    win_sum[(size_t)c * npar + i] += xc[i];
                    for (int j = 0; j < npar; ++j) win_msum[((size_t)c * npar + i) * npar + j] += xc[i] * xc[j];
                }
            }
            if (it % 100 == 0) {
                for (int c = 0; c < nchains; ++c) {
                    if (win_n[c] >= 2)
                        ad.update(win_n[c], &win_sum[(size_t)c * npar], &win_msum[(size_t)c * npar * npar]);
                    win_n[c] = 0;
                }
                std::fill(win_sum.begin(), win_sum.end(), 0.0);
                std::fill(win_msum.begin(), win_msum.end(), 0.0);
                ad.refactor();
            }
        }
    }
    if (accept_rate)
        for (size_t i = 0; i < acc.size(); ++i) accept_rate[i] = (double)acc[i] / niter;
    if (proposal_cov)
        for (size_t i = 0; i < ad.cov.size(); ++i) proposal_cov[i] = ad.cov[i];
    return CG_OK;
}

namespace {
struct PixelLike {
    cg_ctx* ctx;
    const double* map;
    const double* cl_template;
    std::vector<double> cl;
    std::vector<int> st;
};

// -2lnL at x = ln C_l (l = 2..lmax) for every chain, one batched call
int pixel_like(void* user, int nchains, const double* x, double* m2lnl)
{
    PixelLike& P = *static_cast<PixelLike*>(user);
    const int L1 = P.ctx->lmax + 1, np = P.ctx->lmax - 1;
    for (int c = 0; c < nchains; ++c) {
        for (int l = 0; l < L1; ++l) P.cl[(size_t)c * L1 + l] = P.cl_template[l];
        for (int k = 0; k < np; ++k) P.cl[(size_t)c * L1 + 2 + k] = std::exp(x[(size_t)c * np + k]);
    }
    const int rc = cg_loglike(P.ctx, nchains, P.cl.data(), P.map, 0, m2lnl, nullptr, nullptr, nullptr, P.st.data());
    if (rc) return rc;
    for (int c = 0; c < nchains; ++c)
        if (P.st[c] != CG_OK) m2lnl[c] = INFINITY;  // rejected
    return CG_OK;
}
}  // namespace

extern "C" int cg_mh_run(cg_ctx* ctx, const double* map, int nchains, const double* x0, const double* cl_template,
                         int niter, const double* sampling_width, const int* prior_mode, const double* prior_p1,
                         const double* prior_p2, int nblocks, const int* blocks, int adapt, unsigned long long seed,
                         double* chain, double* accept_rate, double* proposal_cov)
{
    if (!ctx || !map || !cl_template || nchains < 1 || nchains > ctx->max_batch) {
        if (ctx) ctx->err = "bad arguments to cg_mh_run";
        return CG_ERR_BAD_ARG;
    }
    PixelLike P{ctx, map, cl_template, std::vector<double>((size_t)nchains * (ctx->lmax + 1)),
                std::vector<int>(nchains)};
    const int rc = cg_mh_sample(nchains, ctx->lmax - 1, pixel_like, &P, x0, niter, sampling_width, prior_mode,
                                prior_p1, prior_p2, nblocks, blocks, adapt, seed, chain, accept_rate, proposal_cov);
    if (rc == CG_ERR_BAD_ARG && ctx->err.empty()) ctx->err = "bad arguments to cg_mh_run";
    return rc;
}
