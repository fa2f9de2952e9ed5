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
// cg_hmc_run is the pixel likelihood of a context, parameters x_l = ln C_l: by default with the
// leapfrog resident on the device (k_hmc.cu), the host drawing the random numbers and deciding the
// acceptances once per trajectory; knob "hmc_device" = 0 runs the same pixel likelihood through
// cg_hmc_sample's host loop instead.  Both give the same chains bit for bit.
#include <cmath>
#include <random>
#include <vector>

#include "cg_exp.h"
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
        for (int k = 0; k < np; ++k) T.cl[(size_t)c * L1 + 2 + k] = cg::exp_same(x[(size_t)c * np + k]);
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

// The device-resident driver: the same random numbers, drawn in the same order, and the same
// arithmetic as cg_hmc_sample over pixel_like_grad.  Per iteration one copy to the device (the
// momenta) and one back (the proposals' dH, positions and -2lnL, for the acceptance draws and the
// record); the leapfrog steps in between are launches only.
int hmc_run_device(cg_ctx* ctx, const double* map, int B, const double* x0, const double* cl_template, int niter,
                   int nleap, double tau, const std::vector<double>& m, int jitter, unsigned long long seed,
                   double* chain, double* accept_rate)
{
    const int L1 = ctx->lmax + 1, np = ctx->lmax - 1, n = ctx->n;
    const size_t bp = (size_t)B * np, bl = (size_t)B * L1;
    cudaStream_t s = ctx->stream;
    // x, xn, p, g, gn [B np]; cl, gcl [B L1]; u, un, kin0, dh [B]; mass [np]; template [L1]; map [n];
    // status, flags [B] (ints, at the end)
    const size_t nd = 5 * bp + 2 * bl + 4 * (size_t)B + np + L1 + n;
    double* buf = nullptr;
    CG_CUDA_TRY(ctx, cudaMalloc((void**)&buf, sizeof(double) * nd + sizeof(int) * 2 * (size_t)B));
    double *x = buf, *xn = x + bp, *p = xn + bp, *g = p + bp, *gn = g + bp, *cl = gn + bp, *gcl = cl + bl;
    double *u = gcl + bl, *un = u + B, *kin0 = un + B, *dh = kin0 + B, *mass = dh + B, *tmpl = mass + np;
    double* dmap = tmpl + L1;
    int* st = reinterpret_cast<int*>(buf + nd);
    int* flag = st + B;
    std::mt19937 gen((std::mt19937::result_type)seed);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    std::normal_distribution<double> gauss(0.0, 1.0);
    std::vector<double> hx(x0, x0 + bp), hxn(bp), hp(bp), hu(B), hun(B), hkin0(B), hdh(B);
    std::vector<int> hflag(B), acc(B, 0);
    auto record = [&](int it) {
        for (int c = 0; c < B; ++c) {
            double* row = chain + ((size_t)it * B + c) * (np + 1);
            row[0] = hu[c];
            for (int k = 0; k < np; ++k) row[1 + k] = hx[(size_t)c * np + k];
        }
    };
    int rc = CG_OK;
    auto cp = [&](void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
        if (!rc && cudaMemcpyAsync(dst, src, bytes, kind, s) != cudaSuccess) {
            ctx->err = "cg_hmc_run: device copy failed";
            rc = CG_ERR_CUDA;
        }
    };
    // the likelihood at xn (the positions p and x passed to drift are already advanced): C_l, the
    // call, the gradient in ln C_l and the closing half kick
    auto evaluate = [&](double t, int kick) {
        if (!rc) rc = cg_loglike_device(ctx, B, cl, dmap, 0, un, nullptr, nullptr, gcl, st, s);
        if (!rc) rc = cg::hmc_launch_kick(ctx, B, np, t, kick, p, gn, gcl, cl, st, un, s);
    };
    cp(mass, m.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
    cp(tmpl, cl_template, sizeof(double) * L1, cudaMemcpyHostToDevice);
    cp(dmap, map, sizeof(double) * n, cudaMemcpyHostToDevice);
    cp(xn, x0, sizeof(double) * bp, cudaMemcpyHostToDevice);
    CG_CUDA_TRY(ctx, cudaMemsetAsync(p, 0, sizeof(double) * bp, s));
    CG_CUDA_TRY(ctx, cudaMemsetAsync(gn, 0, sizeof(double) * bp, s));
    // the start: C_l from x0 (a zero step leaves x0 unchanged), -2lnL and the gradient
    if (!rc) rc = cg::hmc_launch_drift(ctx, B, np, 0.0, p, gn, xn, mass, tmpl, cl, s);
    evaluate(0.0, 0);
    cp(x, xn, sizeof(double) * bp, cudaMemcpyDeviceToDevice);
    cp(g, gn, sizeof(double) * bp, cudaMemcpyDeviceToDevice);
    cp(u, un, sizeof(double) * B, cudaMemcpyDeviceToDevice);
    cp(hu.data(), un, sizeof(double) * B, cudaMemcpyDeviceToHost);
    if (!rc && cudaStreamSynchronize(s) != cudaSuccess) { ctx->err = "cg_hmc_run: stream failed"; rc = CG_ERR_CUDA; }
    if (!rc) record(0);
    for (int it = 1; it <= niter && !rc; ++it) {
        double t = tau;
        int nsteps = nleap;
        if (jitter) {
            t = uni(gen) * tau;
            nsteps = (int)std::ceil(nleap * uni(gen));
            if (nsteps < 1) nsteps = 1;
        }
        for (int c = 0; c < B; ++c) {
            double kin = 0;
            for (int k = 0; k < np; ++k) {
                const double v = std::sqrt(m[k]) * gauss(gen);
                hp[(size_t)c * np + k] = v;
                kin += v * v / m[k];
            }
            hkin0[c] = kin;
        }
        cp(p, hp.data(), sizeof(double) * bp, cudaMemcpyHostToDevice);
        cp(kin0, hkin0.data(), sizeof(double) * B, cudaMemcpyHostToDevice);
        cp(xn, x, sizeof(double) * bp, cudaMemcpyDeviceToDevice);
        cp(gn, g, sizeof(double) * bp, cudaMemcpyDeviceToDevice);
        for (int st_ = 0; st_ < nsteps && !rc; ++st_) {
            rc = cg::hmc_launch_drift(ctx, B, np, t, p, gn, xn, mass, tmpl, cl, s);
            evaluate(t, 1);
        }
        if (!rc) rc = cg::hmc_launch_energy(ctx, B, np, p, mass, un, u, kin0, dh, s);
        cp(hdh.data(), dh, sizeof(double) * B, cudaMemcpyDeviceToHost);
        cp(hxn.data(), xn, sizeof(double) * bp, cudaMemcpyDeviceToHost);
        cp(hun.data(), un, sizeof(double) * B, cudaMemcpyDeviceToHost);
        if (!rc && cudaStreamSynchronize(s) != cudaSuccess) { ctx->err = "cg_hmc_run: stream failed"; rc = CG_ERR_CUDA; }
        if (rc) break;
        for (int c = 0; c < B; ++c) {
            const double q = uni(gen);
            hflag[c] = std::isfinite(hdh[c]) && q <= std::exp(-hdh[c] / 2);
            if (hflag[c]) {
                ++acc[c];
                for (int k = 0; k < np; ++k) hx[(size_t)c * np + k] = hxn[(size_t)c * np + k];
                hu[c] = hun[c];
            }
        }
        cp(flag, hflag.data(), sizeof(int) * B, cudaMemcpyHostToDevice);
        if (!rc) rc = cg::hmc_launch_accept(ctx, B, np, flag, xn, gn, un, x, g, u, s);
        record(it);
    }
    if (!rc && cudaStreamSynchronize(s) != cudaSuccess) { ctx->err = "cg_hmc_run: stream failed"; rc = CG_ERR_CUDA; }
    cudaFree(buf);
    if (rc) return rc;
    if (accept_rate)
        for (int c = 0; c < B; ++c) accept_rate[c] = (double)acc[c] / niter;
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
    std::vector<double> m(np, 1.0);
    if (mass) m.assign(mass, mass + np);
    if (ctx->tune.hmc_device) {
        CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
        return hmc_run_device(ctx, map, nchains, x0, cl_template, niter, nleap, tau, m, jitter, seed, chain,
                              accept_rate);
    }
    PixelTarget T{ctx, map, cl_template, std::vector<double>((size_t)nchains * L1),
                  std::vector<double>((size_t)nchains * L1), std::vector<int>(nchains)};
    return cg_hmc_sample(nchains, np, pixel_like_grad, &T, x0, niter, nleap, tau, mass, jitter, seed, chain,
                         accept_rate);
}
