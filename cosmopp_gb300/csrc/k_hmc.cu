// Device-resident leapfrog of the batched HMC over the pixel likelihood (cg_hmc_run): the positions,
// momenta and gradients of all chains stay in device memory for a whole trajectory, and each
// leapfrog step is three launches on the context's stream (half kick + drift + C_l = exp(x), the
// batched -2lnL + gradient call, half kick) with no host synchronisation in between.  The
// arithmetic is the host loop's (cg_hmc_sample, after Math::HMC::run in source/hmc.cpp:78-96) with
// every product and sum rounded separately, so the two drivers produce the same chains bit for bit.
#include "cg_exp.h"
#include "cg_internal.h"

namespace cg {
namespace {

// p -= t/2 * g/2;  x += t/m * p;  cl = [template l < 2, exp(x)] for every chain c and parameter k
__global__ void hmc_drift(int B, int np, int L1, double t, double* __restrict__ p, const double* __restrict__ g,
                          double* __restrict__ x, const double* __restrict__ mass, const double* __restrict__ tmpl,
                          double* __restrict__ cl)
{
    const int c = blockIdx.x;
    for (int k = threadIdx.x; k < np; k += blockDim.x) {
        const size_t i = (size_t)c * np + k;
        const double pk = __dsub_rn(p[i], __ddiv_rn(__dmul_rn(__ddiv_rn(t, 2.0), g[i]), 2.0));
        const double xk = __dadd_rn(x[i], __dmul_rn(__ddiv_rn(t, mass[k]), pk));
        p[i] = pk;
        x[i] = xk;
        cl[(size_t)c * L1 + 2 + k] = exp_same(xk);
    }
    if (threadIdx.x < 2) cl[(size_t)c * L1 + threadIdx.x] = tmpl[threadIdx.x];
}

// g = d(-2lnL)/dC_l * C_l (the gradient in x = ln C_l); -2lnL = +inf where the call flagged the
// element; then p -= t/2 * g/2 (with kick = 0 only the gradient: the trajectory's start)
__global__ void hmc_kick(int B, int np, int L1, double t, int kick, double* __restrict__ p, double* __restrict__ g,
                         const double* __restrict__ gcl, const double* __restrict__ cl, const int* __restrict__ st,
                         double* __restrict__ m2lnl)
{
    const int c = blockIdx.x;
    for (int k = threadIdx.x; k < np; k += blockDim.x) {
        const size_t i = (size_t)c * np + k;
        const double gk = __dmul_rn(gcl[(size_t)c * L1 + 2 + k], cl[(size_t)c * L1 + 2 + k]);
        g[i] = gk;
        if (kick) p[i] = __dsub_rn(p[i], __ddiv_rn(__dmul_rn(__ddiv_rn(t, 2.0), gk), 2.0));
    }
    if (threadIdx.x == 0 && st[c] != CG_OK) m2lnl[c] = INFINITY;
}

// dH_c = u_new + sum_k p^2 / m - u_old - kin0, in the host loop's order (one thread per chain)
__global__ void hmc_energy(int B, int np, const double* __restrict__ p, const double* __restrict__ mass,
                           const double* __restrict__ un, const double* __restrict__ u,
                           const double* __restrict__ kin0, double* __restrict__ dh)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= B) return;
    double kin = 0.0;
    for (int k = 0; k < np; ++k) {
        const double v = p[(size_t)c * np + k];
        kin = __dadd_rn(kin, __ddiv_rn(__dmul_rn(v, v), mass[k]));
    }
    dh[c] = __dsub_rn(__dsub_rn(__dadd_rn(un[c], kin), u[c]), kin0[c]);
}

// the accepted chains take the proposal: x, g, u <- xn, gn, un
__global__ void hmc_accept(int B, int np, const int* __restrict__ flag, const double* __restrict__ xn,
                           const double* __restrict__ gn, const double* __restrict__ un, double* __restrict__ x,
                           double* __restrict__ g, double* __restrict__ u)
{
    const int c = blockIdx.x;
    if (!flag[c]) return;
    for (int k = threadIdx.x; k < np; k += blockDim.x) {
        const size_t i = (size_t)c * np + k;
        x[i] = xn[i];
        g[i] = gn[i];
    }
    if (threadIdx.x == 0) u[c] = un[c];
}

}  // namespace

int hmc_launch_drift(cg_ctx* ctx, int B, int np, double t, double* p, const double* g, double* x, const double* mass,
                     const double* tmpl, double* cl, cudaStream_t s)
{
    hmc_drift<<<B, 64, 0, s>>>(B, np, ctx->lmax + 1, t, p, g, x, mass, tmpl, cl);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int hmc_launch_kick(cg_ctx* ctx, int B, int np, double t, int kick, double* p, double* g, const double* gcl,
                    const double* cl, const int* st, double* m2lnl, cudaStream_t s)
{
    hmc_kick<<<B, 64, 0, s>>>(B, np, ctx->lmax + 1, t, kick, p, g, gcl, cl, st, m2lnl);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int hmc_launch_energy(cg_ctx* ctx, int B, int np, const double* p, const double* mass, const double* un,
                      const double* u, const double* kin0, double* dh, cudaStream_t s)
{
    hmc_energy<<<(B + 63) / 64, 64, 0, s>>>(B, np, p, mass, un, u, kin0, dh);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int hmc_launch_accept(cg_ctx* ctx, int B, int np, const int* flag, const double* xn, const double* gn,
                      const double* un, double* x, double* g, double* u, cudaStream_t s)
{
    hmc_accept<<<B, 64, 0, s>>>(B, np, flag, xn, gn, un, x, g, u);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
