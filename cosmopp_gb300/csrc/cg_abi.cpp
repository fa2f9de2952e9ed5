// C ABI of cosmopp_gb300: context set-up, staging of host buffers, dispatch
// to the plain FP64 and mixed paths, and the Likelihood drop-in.
//
// Entry points and the reference interfaces they replace are declared in
// include/cosmopp_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>

#include <cstdlib>

#include "cg_internal.h"

namespace {

thread_local std::string g_create_error;

bool device_ok(int device, int* sm_count, std::string& why)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        why = "no CUDA device available";
        return false;
    }
    if (device < 0 || device >= count) {
        why = "device ordinal out of range";
        return false;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        why = "cudaGetDeviceProperties failed";
        return false;
    }
    if (prop.major != 10 || prop.minor != 3) {
        why = std::string("cosmopp_gb300 is built for sm_103 (GB300); device is ") + prop.name + " sm_" +
              std::to_string(prop.major) + std::to_string(prop.minor);
        return false;
    }
    *sm_count = prop.multiProcessorCount;
    return true;
}

template <typename T>
bool dalloc(T** p, size_t count)
{
    if (count == 0) count = 1;
    if (cudaMalloc((void**)p, sizeof(T) * count) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return false;
    }
    return true;
}

}  // namespace

namespace cg {
// error text for entry points that have no context (read with cg_last_error(NULL))
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace cg

extern "C" void cg_config_init(cg_config* cfg)
{
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->struct_size = (int)sizeof(cg_config);
    cfg->scheme = CG_SCHEME_NEST;
    cfg->noise_sigma = 1e-3;  // CMatrixGenerator::generateNoiseMatrix default (include/c_matrix_generator.hpp:147)
    cfg->max_batch = 1;
    cfg->precision = CG_PREC_FP64;
    cfg->recenter = CG_RECENTER_AUTO;
}

extern "C" const char* cg_last_error(const cg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }
extern "C" int cg_get_n(const cg_ctx* ctx) { return ctx ? ctx->n : 0; }

extern "C" int cg_unit_vectors(const cg_ctx* ctx, double* xyz)
{
    if (!ctx || !xyz) return CG_ERR_BAD_ARG;
    std::memcpy(xyz, ctx->xyz.data(), sizeof(double) * ctx->xyz.size());
    return CG_OK;
}

extern "C" void cg_destroy(cg_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (cg_ctx::Graph& gr : ctx->graphs)
        if (gr.exec) cudaGraphExecDestroy(gr.exec);
    cg::fp64_free(ctx);
    cg::mixed_free(ctx);
    cudaFree(ctx->d_xyz); cudaFree(ctx->d_noise); cudaFree(ctx->d_lega); cudaFree(ctx->d_legb);
    cudaFree(ctx->d_beam); cudaFree(ctx->d_cl); cudaFree(ctx->d_out);
    for (cudaEvent_t e : ctx->marks)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {ctx->ev_fork, ctx->ev_col, ctx->ev_join})
        if (e) cudaEventDestroy(e);
    if (ctx->hi) {
        cudaStreamSynchronize(ctx->hi);
        cudaStreamDestroy(ctx->hi);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// ---- memory admission ----------------------------------------------------------

namespace {

// the context's own allocations of cg_create: geometry, beam tables, staging for max_batch elements
size_t staging_bytes(int N, int lmax, int max_batch)
{
    const size_t L1 = (size_t)lmax + 1, Bm = (size_t)max_batch;
    return sizeof(double) * (3 * (size_t)N + N + 3 * L1 + Bm * L1) + sizeof(double) * (Bm * (3 + L1) + Bm * N) +
           sizeof(int) * Bm;
}

void fill_plan(const cg_ctx* shape, size_t budget, cg_memory_plan* p)
{
    size_t fixed = staging_bytes(shape->N, shape->lmax, shape->max_batch), per = 0;
    if (shape->precision == CG_PREC_MIXED) {
        size_t f = 0;
        cg::mixed_bytes(shape, &f, &per);
        fixed += f;
    } else {
        per = cg::fp64_bytes_per_element(shape);
    }
    p->bytes_fixed = fixed;
    p->bytes_per_element = per;
    p->bytes_budget = budget;
    p->bytes_reserve = ((size_t)256 << 20) + budget / 100;
    const size_t avail = budget > p->bytes_reserve + fixed ? budget - p->bytes_reserve - fixed : 0;
    const size_t fit = per ? avail / per : 0;
    p->max_batch_fit = (int)std::min<size_t>(fit, (size_t)1 << 30);
    p->chunk = std::min(shape->max_batch, p->max_batch_fit);
}

// pixel count, padded size and l range of a configuration (the checks cg_create repeats)
int shape_of(const cg_config* cfg, cg_ctx* shape)
{
    if (!cfg || cfg->struct_size != (int)sizeof(cg_config)) return CG_ERR_BAD_ARG;
    if (cfg->lmax < 2 || cfg->lmax > 255 || cfg->max_batch < 1) return CG_ERR_BAD_ARG;
    if (cfg->precision != CG_PREC_FP64 && cfg->precision != CG_PREC_MIXED) return CG_ERR_BAD_ARG;
    int n;
    if (cfg->dirs) {
        n = cfg->n;
    } else {
        if (cfg->nside <= 0 || cfg->nside > 8192) return CG_ERR_BAD_ARG;
        const long npix = cg_nside2npix(cfg->nside);
        n = cfg->good_pixels ? cfg->n : (int)npix;
        if (n > npix) return CG_ERR_BAD_ARG;
    }
    if (n <= 0) return CG_ERR_BAD_ARG;
    shape->n = n;
    shape->nt = 2 * ((n + 2 * cg::TS - 1) / (2 * cg::TS));
    shape->N = shape->nt * cg::TS;
    shape->lmax = cfg->lmax;
    shape->max_batch = cfg->max_batch;
    shape->precision = cfg->precision;
    return CG_OK;
}

}  // namespace

extern "C" int cg_plan_memory(const cg_config* cfg, size_t budget_bytes, cg_memory_plan* plan)
{
    if (!plan) return CG_ERR_BAD_ARG;
    cg_ctx shape;
    int rc = shape_of(cfg, &shape);
    if (rc) { g_create_error = "cg_plan_memory: invalid configuration"; return rc; }
    if (budget_bytes == 0) {
        if (cudaSetDevice(cfg->device) != cudaSuccess) { g_create_error = "cg_plan_memory: no such device"; return CG_ERR_NO_DEVICE; }
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { g_create_error = "cg_plan_memory: cudaMemGetInfo failed"; return CG_ERR_CUDA; }
        budget_bytes = fr;
    }
    fill_plan(&shape, budget_bytes, plan);
    return CG_OK;
}

extern "C" int cg_get_memory_plan(const cg_ctx* ctx, cg_memory_plan* plan)
{
    if (!ctx || !plan) return CG_ERR_BAD_ARG;
    *plan = ctx->plan;
    return CG_OK;
}

extern "C" int cg_create(cg_ctx** out, const cg_config* cfg)
{
    g_create_error.clear();
    if (!out || !cfg) { g_create_error = "NULL argument"; return CG_ERR_BAD_ARG; }
    *out = nullptr;
    if (cfg->struct_size != (int)sizeof(cg_config)) { g_create_error = "cg_config.struct_size mismatch"; return CG_ERR_BAD_ARG; }
    if (cfg->lmax < 2 || cfg->lmax > 255) { g_create_error = "lmax must be in [2, 255]"; return CG_ERR_BAD_ARG; }
    if (cfg->max_batch < 1) { g_create_error = "max_batch must be >= 1"; return CG_ERR_BAD_ARG; }
    if (cfg->precision != CG_PREC_FP64 && cfg->precision != CG_PREC_MIXED) { g_create_error = "unknown precision"; return CG_ERR_BAD_ARG; }
    std::unique_ptr<cg_ctx> ctx(new (std::nothrow) cg_ctx());
    if (!ctx) { g_create_error = "out of host memory"; return CG_ERR_ALLOC; }

    // pixel directions
    if (cfg->dirs) {
        if (cfg->n <= 0) { g_create_error = "n must be > 0 with dirs"; return CG_ERR_BAD_ARG; }
        ctx->n = cfg->n;
        ctx->xyz.assign(cfg->dirs, cfg->dirs + 3 * (size_t)cfg->n);
    } else {
        if (cfg->nside <= 0 || cfg->nside > 8192) { g_create_error = "invalid nside"; return CG_ERR_BAD_ARG; }
        const long npix = cg_nside2npix(cfg->nside);
        ctx->n = cfg->good_pixels ? cfg->n : (int)npix;
        if (ctx->n <= 0 || ctx->n > npix) { g_create_error = "invalid number of kept pixels"; return CG_ERR_BAD_ARG; }
        ctx->xyz.resize(3 * (size_t)ctx->n);
        if (cg_pix2vec(cfg->nside, cfg->scheme, cfg->good_pixels, ctx->n, ctx->xyz.data()) != CG_OK) {
            g_create_error = "invalid pixel index or scheme";
            return CG_ERR_BAD_ARG;
        }
    }
    for (double v : ctx->xyz)
        if (!std::isfinite(v)) { g_create_error = "non-finite direction"; return CG_ERR_NONFINITE; }
    ctx->lmax = cfg->lmax;
    // an even number of 64-tiles, so the tensor-core kernels can work on 128x128 supertiles
    ctx->nt = 2 * ((ctx->n + 2 * cg::TS - 1) / (2 * cg::TS));
    ctx->N = ctx->nt * cg::TS;
    ctx->max_batch = cfg->max_batch;
    ctx->precision = cfg->precision;
    ctx->recenter = cfg->recenter;
    ctx->recenter_radius = cfg->recenter_radius > 0 ? cfg->recenter_radius : 1.0;
    ctx->device = cfg->device;

    // beam: Utils::readPixelWindowFunction with a unit window (f[l] = 1, f[l] *= B_l)
    ctx->leg.beam.resize(ctx->lmax + 1);
    ctx->leg.a.assign(ctx->lmax + 1, 0.0);
    ctx->leg.b.assign(ctx->lmax + 1, 0.0);
    for (int l = 0; l <= ctx->lmax; ++l) {
        if (cfg->beam) ctx->leg.beam[l] = cfg->beam[l];
        else {
            double f = 1.0;
            f *= cg_beam(l, cfg->fwhm_deg);
            ctx->leg.beam[l] = f;
        }
        if (l >= 1) {
            ctx->leg.a[l] = 2 - 1.0 / l;  // include/legendre.hpp:34
            ctx->leg.b[l] = 1 - 1.0 / l;
        }
    }
    if (cfg->fwhm_deg < 0 && !cfg->beam) { g_create_error = "invalid fwhm"; return CG_ERR_BAD_ARG; }
    ctx->fwhm_deg = cfg->beam ? -1.0 : cfg->fwhm_deg;
    // noise: generateNoiseMatrix puts noise * noise on the diagonal (source/c_matrix_generator.cpp:774-787)
    ctx->noise.resize(ctx->n);
    for (int i = 0; i < ctx->n; ++i) {
        ctx->noise[i] = cfg->noise_var ? cfg->noise_var[i] : cfg->noise_sigma * cfg->noise_sigma;
        if (!std::isfinite(ctx->noise[i])) { g_create_error = "non-finite noise"; return CG_ERR_NONFINITE; }
    }

    std::string why;
    if (!device_ok(ctx->device, &ctx->sm_count, why)) { g_create_error = why; return CG_ERR_NO_DEVICE; }
    if (cudaSetDevice(ctx->device) != cudaSuccess) { g_create_error = "cudaSetDevice failed"; return CG_ERR_CUDA; }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        g_create_error = "cudaStreamCreate failed";
        return CG_ERR_CUDA;
    }
    // admission: plan the device bytes against the free memory before allocating anything
    {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { g_create_error = "cudaMemGetInfo failed"; cg_destroy(ctx.release()); return CG_ERR_CUDA; }
        fill_plan(ctx.get(), fr, &ctx->plan);
        if (ctx->plan.max_batch_fit < 1) {
            char msg[256];
            std::snprintf(msg, sizeof msg,
                          "admission: %.2f GB fixed + %.2f GB per batch element do not fit in %.2f GB free "
                          "(reserve %.2f GB)",
                          ctx->plan.bytes_fixed / 1e9, ctx->plan.bytes_per_element / 1e9, fr / 1e9,
                          ctx->plan.bytes_reserve / 1e9);
            g_create_error = msg;
            cg_destroy(ctx.release());
            return CG_ERR_ALLOC;
        }
        ctx->chunk = ctx->plan.chunk;
    }
    const int N = ctx->N, L1 = ctx->lmax + 1, Bm = ctx->max_batch;
    std::vector<double> soa(3 * (size_t)N, 0.0), nz(N, 0.0);
    for (int i = 0; i < ctx->n; ++i) {
        for (int c = 0; c < 3; ++c) soa[(size_t)c * N + i] = ctx->xyz[3 * (size_t)i + c];
        nz[i] = ctx->noise[i];
    }
    // staging: cl [Bm][L1], then outputs m2lnl, chi2, logdet [Bm], grad [Bm][L1], data [Bm][N], status
    ctx->d_out_bytes = sizeof(double) * ((size_t)Bm * (3 + L1) + (size_t)Bm * N) + sizeof(int) * Bm;
    if (!dalloc(&ctx->d_xyz, soa.size()) || !dalloc(&ctx->d_noise, (size_t)N) || !dalloc(&ctx->d_lega, (size_t)L1) ||
        !dalloc(&ctx->d_legb, (size_t)L1) || !dalloc(&ctx->d_beam, (size_t)L1) || !dalloc(&ctx->d_cl, (size_t)Bm * L1) ||
        !dalloc((unsigned char**)&ctx->d_out, ctx->d_out_bytes)) {
        g_create_error = "device allocation failed";
        cg_destroy(ctx.release());
        return CG_ERR_ALLOC;
    }
    cudaMemcpy(ctx->d_xyz, soa.data(), sizeof(double) * soa.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_noise, nz.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_lega, ctx->leg.a.data(), sizeof(double) * L1, cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_legb, ctx->leg.b.data(), sizeof(double) * L1, cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->d_beam, ctx->leg.beam.data(), sizeof(double) * L1, cudaMemcpyHostToDevice);
    if (cudaGetLastError() != cudaSuccess) { g_create_error = "upload failed"; cg_destroy(ctx.release()); return CG_ERR_CUDA; }
    if (ctx->precision == CG_PREC_MIXED && cfg->cl_ref) {
        const int rc = cg::mixed_prepare_reference(ctx.get(), cfg->cl_ref);
        if (rc) { g_create_error = ctx->err; cg_destroy(ctx.release()); return rc; }
    }
    // launch shapes tuned earlier for this device, pixel count, l range and batch size
    if (ctx->precision == CG_PREC_MIXED) {
        const char* tf = std::getenv("COSMOPP_GB300_TUNE_FILE");
        if (tf && *tf) cg_tune_load(ctx.get(), tf, nullptr);
    }
    *out = ctx.release();
    return CG_OK;
}

// ---- covariance build ------------------------------------------------------

extern "C" int cg_build_cmatrix_batched(cg_ctx* ctx, int B, const double* cl, double* out_packed)
{
    if (!ctx || !cl || !out_packed || B < 1 || B > ctx->max_batch) {
        if (ctx) ctx->err = "bad arguments to cg_build_cmatrix_batched";
        return CG_ERR_BAD_ARG;
    }
    for (size_t k = 0; k < (size_t)B * (ctx->lmax + 1); ++k)
        if (!std::isfinite(cl[k])) { ctx->err = "non-finite C_l"; return CG_ERR_NONFINITE; }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t np = (size_t)ctx->n * (ctx->n + 1) / 2;
    double* d_out = nullptr;
    CG_CUDA_TRY(ctx, cudaMalloc((void**)&d_out, sizeof(double) * np * B));
    cudaMemcpyAsync(ctx->d_cl, cl, sizeof(double) * B * (ctx->lmax + 1), cudaMemcpyHostToDevice, ctx->stream);
    int rc = cg::fp64_build_packed(ctx, B, ctx->d_cl, d_out, ctx->stream);
    if (rc == CG_OK) {
        cudaMemcpyAsync(out_packed, d_out, sizeof(double) * np * B, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    }
    cudaFree(d_out);
    return rc;
}

extern "C" int cg_build_cmatrix(cg_ctx* ctx, const double* cl, double* out_packed)
{
    return cg_build_cmatrix_batched(ctx, 1, cl, out_packed);
}

extern "C" int cg_fiducial_matrix(cg_ctx* ctx, const double* cl, int lmax, int lmax_max, const double* beam,
                                  double* out_packed)
{
    if (!ctx || !cl || !out_packed || lmax < 1 || lmax_max <= lmax || lmax_max > CG_FIDUCIAL_LMAX_MAX) {
        if (ctx) ctx->err = "bad arguments to cg_fiducial_matrix (need 1 <= lmax < lmax_max <= 4096)";
        return CG_ERR_BAD_ARG;
    }
    if (!beam && ctx->fwhm_deg < 0) {
        ctx->err = "cg_fiducial_matrix: the context has a caller-given beam table; pass beam[0..lmax_max]";
        return CG_ERR_BAD_ARG;
    }
    const int L1 = lmax_max + 1;
    for (int l = 0; l < L1; ++l)
        if (!std::isfinite(cl[l]) || (beam && !std::isfinite(beam[l]))) {
            ctx->err = "non-finite C_l or beam";
            return CG_ERR_NONFINITE;
        }
    // tables as source/c_matrix_generator.cpp:706-772 forms its terms: Bonnet coefficients
    // (include/legendre.hpp:34), cl[l] * ((2l+1)/(4 pi)), the beam (unit pixel window), 100 cl[2]
    std::vector<double> tab((size_t)4 * L1, 0.0);
    double* a = tab.data();
    double* b = a + L1;
    double* fc = b + L1;
    double* bm = fc + L1;
    for (int l = 0; l < L1; ++l) {
        if (l >= 1) {
            a[l] = 2 - 1.0 / l;
            b[l] = 1 - 1.0 / l;
        }
        fc[l] = cl[l] * ((2 * l + 1) / (4 * cg::kPiHost));
        double f = 1.0;
        f *= beam ? beam[l] : cg_beam(l, ctx->fwhm_deg);
        bm[l] = f;
    }
    const double m0 = 100 * cl[2];
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t np = (size_t)ctx->n * (ctx->n + 1) / 2;
    double *d_tab = nullptr, *d_out = nullptr;
    CG_CUDA_TRY(ctx, cudaMalloc((void**)&d_tab, sizeof(double) * tab.size()));
    if (cudaMalloc((void**)&d_out, sizeof(double) * np) != cudaSuccess) {
        cudaFree(d_tab);
        ctx->err = "cg_fiducial_matrix: out of device memory";
        return CG_ERR_CUDA;
    }
    cudaMemcpyAsync(d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, ctx->stream);
    int rc = cg::fp64_build_fiducial(ctx, lmax + 1, lmax_max, d_tab, m0, d_out, ctx->stream);
    if (rc == CG_OK) {
        cudaMemcpyAsync(out_packed, d_out, sizeof(double) * np, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    }
    cudaFree(d_tab);
    cudaFree(d_out);
    return rc;
}

extern "C" int cg_legendre_table(cg_ctx* ctx, int l0, int l1, double* out)
{
    if (!ctx || !out || l0 < 0 || l1 <= l0 || l1 > CG_FIDUCIAL_LMAX_MAX + 1) {
        if (ctx) ctx->err = "bad arguments to cg_legendre_table (need 0 <= l0 < l1 <= 4097)";
        return CG_ERR_BAD_ARG;
    }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t np = (size_t)ctx->n * (ctx->n + 1) / 2;
    // the l range goes through a device buffer of at most 1 GiB, a slab of l values at a time
    const int slab = (int)std::max<size_t>(1, std::min<size_t>((size_t)(l1 - l0), ((size_t)1 << 30) / (8 * np)));
    std::vector<double> ab((size_t)2 * l1, 0.0);
    for (int l = 1; l < l1; ++l) {  // include/legendre.hpp:34
        ab[l] = 2 - 1.0 / l;
        ab[l1 + l] = 1 - 1.0 / l;
    }
    double *d_ab = nullptr, *d_out = nullptr;
    CG_CUDA_TRY(ctx, cudaMalloc((void**)&d_ab, sizeof(double) * ab.size()));
    if (cudaMalloc((void**)&d_out, sizeof(double) * np * slab) != cudaSuccess) {
        cudaFree(d_ab);
        ctx->err = "cg_legendre_table: out of device memory";
        return CG_ERR_ALLOC;
    }
    cudaMemcpyAsync(d_ab, ab.data(), sizeof(double) * ab.size(), cudaMemcpyHostToDevice, ctx->stream);
    int rc = CG_OK;
    for (int a = l0; a < l1 && rc == CG_OK; a += slab) {
        const int b = std::min(l1, a + slab);
        rc = cg::fp64_legendre_table(ctx, a, b, d_ab, d_ab + l1, d_out, ctx->stream);
        if (rc == CG_OK) {
            cudaMemcpyAsync(out + (size_t)(a - l0) * np, d_out, sizeof(double) * np * (b - a), cudaMemcpyDeviceToHost,
                            ctx->stream);
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
        }
    }
    cudaFree(d_ab);
    cudaFree(d_out);
    return rc;
}

extern "C" int cg_noise_matrix_from_sims(cg_ctx* ctx, int nsims, int n, const double* sims, double* out_packed,
                                         double* max_abs_mean)
{
    if (!ctx || nsims < 1 || n < 1 || !sims || !out_packed) {
        if (ctx) ctx->err = "bad arguments to cg_noise_matrix_from_sims";
        return CG_ERR_BAD_ARG;
    }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t ns = (size_t)nsims * n, np = (size_t)n * (n + 1) / 2;
    double *d_sims = nullptr, *d_out = nullptr, *d_mean = nullptr;
    if (cudaMalloc((void**)&d_sims, sizeof(double) * ns) != cudaSuccess ||
        cudaMalloc((void**)&d_out, sizeof(double) * np) != cudaSuccess ||
        cudaMalloc((void**)&d_mean, sizeof(double) * n) != cudaSuccess) {
        cudaFree(d_sims);
        cudaFree(d_out);
        cudaFree(d_mean);
        ctx->err = "cg_noise_matrix_from_sims: out of device memory";
        return CG_ERR_ALLOC;
    }
    std::vector<double> mean(n);
    cudaMemcpyAsync(d_sims, sims, sizeof(double) * ns, cudaMemcpyHostToDevice, ctx->stream);
    int rc = cg::fp64_noise_matrix(ctx, nsims, n, d_sims, d_out, d_mean, ctx->stream);
    if (rc == CG_OK) {
        cudaMemcpyAsync(out_packed, d_out, sizeof(double) * np, cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(mean.data(), d_mean, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    }
    if (rc == CG_OK && max_abs_mean) {
        double mx = 0;
        for (int j = 0; j < n; ++j) mx = std::max(mx, std::fabs(mean[j]));
        *max_abs_mean = mx;
    }
    cudaFree(d_sims);
    cudaFree(d_out);
    cudaFree(d_mean);
    return rc;
}

// ---- likelihood ------------------------------------------------------------

static int loglike_chunks(cg_ctx* ctx, int B, const double* d_cl, const double* d_d, int d_stride, double* d_m2lnl,
                          double* d_chi2, double* d_logdet, double* d_grad, int* d_status, cudaStream_t s);

extern "C" int cg_loglike_device(cg_ctx* ctx, int B, const double* d_cl, const double* d_d, int d_stride,
                                 double* d_m2lnl, double* d_chi2, double* d_logdet, double* d_grad, int* d_status,
                                 void* stream)
{
    if (!ctx) return CG_ERR_BAD_ARG;
    if (B < 1 || B > ctx->max_batch || !d_cl || !d_d || !d_m2lnl || (d_stride != 0 && d_stride < ctx->n)) {
        ctx->err = "bad arguments to cg_loglike";
        return CG_ERR_BAD_ARG;
    }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    ctx->nmarks = 0;
    // A mixed call with a fixed reference point makes no host decision that depends on the data, so
    // its ~80 launches are captured once into a CUDA graph and replayed with one launch while the
    // arguments, the knobs and the workspace stay the same.  Anything that stops a capture (the
    // caller's stream already capturing, the legacy stream, profiling marks) runs the launches
    // directly instead.
    if (ctx->precision == CG_PREC_MIXED && ctx->tune.graph && ctx->recenter == CG_RECENTER_FIXED &&
        ctx->wmx.have_ref && !ctx->profiling && s != cudaStreamLegacy && s != cudaStreamPerThread) {
        cg::GraphKey key;
        key.B = B;
        key.d_stride = d_stride;
        key.stream = s;
        const void* p[8] = {d_cl, d_d, d_m2lnl, d_chi2, d_logdet, d_grad, d_status, nullptr};
        for (int i = 0; i < 8; ++i) key.ptr[i] = p[i];
        ++ctx->graph_uses;
        cg_ctx::Graph* slot = nullptr;
        for (cg_ctx::Graph& gr : ctx->graphs)
            if (gr.exec && gr.epoch == ctx->epoch && gr.key == key) slot = &gr;
        if (slot) {
            slot->last_use = ctx->graph_uses;
            CG_CUDA_TRY(ctx, cudaGraphLaunch(slot->exec, s));
            cg::count_launch(ctx, slot->launches);
            ++ctx->graph_replays;
            return CG_OK;
        }
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
            const int rc0 = cg::mixed_ensure(ctx, std::min(B, ctx->chunk > 0 ? ctx->chunk : B));
            if (rc0) return rc0;
            // relaxed: a kernel's module may still be loaded lazily on its first launch
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
                const long long l0 = ctx->launches;
                const int rc = loglike_chunks(ctx, B, d_cl, d_d, d_stride, d_m2lnl, d_chi2, d_logdet, d_grad,
                                              d_status, s);
                cudaGraph_t g = nullptr;
                const cudaError_t ec = cudaStreamEndCapture(s, &g);
                cudaGraphExec_t ex = nullptr;
                // node priorities: the overlapped Cholesky's launches keep their stream's priority
                if (!rc && ec == cudaSuccess && g &&
                    cudaGraphInstantiate(&ex, g, cudaGraphInstantiateFlagUseNodePriority) == cudaSuccess) {
                    cudaGraphDestroy(g);
                    // the stale or least recently used slot takes it
                    cg_ctx::Graph* victim = &ctx->graphs[0];
                    for (cg_ctx::Graph& gr : ctx->graphs) {
                        if (!gr.exec || gr.epoch != ctx->epoch) { victim = &gr; break; }
                        if (gr.last_use < victim->last_use) victim = &gr;
                    }
                    if (victim->exec) cudaGraphExecDestroy(victim->exec);
                    victim->exec = ex;
                    victim->key = key;
                    victim->epoch = ctx->epoch;
                    victim->launches = ctx->launches - l0;
                    victim->last_use = ctx->graph_uses;
                    CG_CUDA_TRY(ctx, cudaGraphLaunch(ex, s));
                    return CG_OK;
                }
                // the capture did not take: forget it and run the launches directly
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                ctx->launches = l0;
                if (rc && rc != CG_ERR_CUDA) return rc;
            } else {
                cudaGetLastError();
            }
        }
    }
    return loglike_chunks(ctx, B, d_cl, d_d, d_stride, d_m2lnl, d_chi2, d_logdet, d_grad, d_status, s);
}

// the batch in pieces of the admitted chunk (one piece when the whole batch fits)
static int loglike_chunks(cg_ctx* ctx, int B, const double* d_cl, const double* d_d, int d_stride, double* d_m2lnl,
                          double* d_chi2, double* d_logdet, double* d_grad, int* d_status, cudaStream_t s)
{
    const int chunk = ctx->chunk > 0 ? ctx->chunk : B;
    const size_t L1 = (size_t)ctx->lmax + 1;
    for (int b0 = 0; b0 < B; b0 += chunk) {
        const int nb = std::min(chunk, B - b0);
        const double* cl = d_cl + b0 * L1;
        const double* dd = d_d + (d_stride ? (size_t)b0 * d_stride : 0);
        double* m2 = d_m2lnl + b0;
        double* c2 = d_chi2 ? d_chi2 + b0 : nullptr;
        double* ld = d_logdet ? d_logdet + b0 : nullptr;
        double* gr = d_grad ? d_grad + b0 * L1 : nullptr;
        int* st = d_status ? d_status + b0 : nullptr;
        const int rc = ctx->precision == CG_PREC_MIXED
                           ? cg::mixed_loglike(ctx, nb, cl, nullptr, dd, d_stride, m2, c2, ld, gr, st, s)
                           : cg::fp64_loglike(ctx, nb, cl, dd, d_stride, m2, c2, ld, gr, st, s);
        if (rc) return rc;
    }
    return CG_OK;
}

extern "C" int cg_loglike(cg_ctx* ctx, int B, const double* cl, const double* d, int d_stride, double* m2lnl,
                          double* chi2, double* logdet, double* grad, int* status)
{
    if (!ctx) return CG_ERR_BAD_ARG;
    if (B < 1 || B > ctx->max_batch || !cl || !d || !m2lnl || (d_stride != 0 && d_stride < ctx->n)) {
        ctx->err = "bad arguments to cg_loglike";
        return CG_ERR_BAD_ARG;
    }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int L1 = ctx->lmax + 1, n = ctx->n, Bm = ctx->max_batch;
    double* o_m2 = ctx->d_out;
    double* o_chi2 = o_m2 + Bm;
    double* o_ld = o_chi2 + Bm;
    double* o_grad = o_ld + Bm;
    double* o_d = o_grad + (size_t)Bm * L1;
    int* o_st = (int*)(o_d + (size_t)Bm * ctx->N);
    cudaStream_t s = ctx->stream;
    CG_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_cl, cl, sizeof(double) * B * L1, cudaMemcpyHostToDevice, s));
    const int nmaps = d_stride ? B : 1;
    if (d_stride == 0 || d_stride == n) {
        CG_CUDA_TRY(ctx, cudaMemcpyAsync(o_d, d, sizeof(double) * (size_t)nmaps * n, cudaMemcpyHostToDevice, s));
    } else {
        CG_CUDA_TRY(ctx, cudaMemcpy2DAsync(o_d, sizeof(double) * n, d, sizeof(double) * d_stride, sizeof(double) * n,
                                           nmaps, cudaMemcpyHostToDevice, s));
    }
    int rc = cg_loglike_device(ctx, B, ctx->d_cl, o_d, d_stride ? n : 0, o_m2, o_chi2, o_ld, grad ? o_grad : nullptr,
                               o_st, s);
    if (rc) return rc;
    CG_CUDA_TRY(ctx, cudaMemcpyAsync(m2lnl, o_m2, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
    if (chi2) CG_CUDA_TRY(ctx, cudaMemcpyAsync(chi2, o_chi2, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
    if (logdet) CG_CUDA_TRY(ctx, cudaMemcpyAsync(logdet, o_ld, sizeof(double) * B, cudaMemcpyDeviceToHost, s));
    if (grad) CG_CUDA_TRY(ctx, cudaMemcpyAsync(grad, o_grad, sizeof(double) * B * L1, cudaMemcpyDeviceToHost, s));
    if (status) CG_CUDA_TRY(ctx, cudaMemcpyAsync(status, o_st, sizeof(int) * B, cudaMemcpyDeviceToHost, s));
    CG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return CG_OK;
}

extern "C" int cg_set_reference(cg_ctx* ctx, const double* cl_ref)
{
    if (!ctx || !cl_ref) return CG_ERR_BAD_ARG;
    if (ctx->precision != CG_PREC_MIXED) { ctx->err = "cg_set_reference needs a CG_PREC_MIXED context"; return CG_ERR_BAD_ARG; }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return cg::mixed_prepare_reference(ctx, cl_ref);
}

extern "C" int cg_reference_count(const cg_ctx* ctx) { return ctx ? ctx->wmx.ref_count : 0; }

extern "C" long long cg_launch_count(const cg_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" long long cg_graph_replays(const cg_ctx* ctx) { return ctx ? ctx->graph_replays : 0; }

extern "C" int cg_set_profiling(cg_ctx* ctx, int enable)
{
    if (!ctx) return CG_ERR_BAD_ARG;
    ctx->profiling = enable != 0;
    return CG_OK;
}

extern "C" int cg_stage_times(cg_ctx* ctx, double* ms)
{
    if (!ctx || !ms) return CG_ERR_BAD_ARG;
    for (int k = 0; k < cg::ST_COUNT; ++k) ms[k] = 0.0;
    if (ctx->nmarks > 0) CG_CUDA_TRY(ctx, cudaEventSynchronize(ctx->marks[ctx->nmarks - 1]));
    for (int k = 0; k + 1 < ctx->nmarks; ++k) {
        float t = 0.f;
        CG_CUDA_TRY(ctx, cudaEventElapsedTime(&t, ctx->marks[k], ctx->marks[k + 1]));
        ms[ctx->mark_stage[k]] += t;
    }
    ctx->nmarks = 0;
    return CG_OK;
}

// ---- Likelihood drop-in ------------------------------------------------------

struct cg_lik {
    cg_ctx ctx;                  // device, sizes, stream and error text
    double* A = nullptr;         // tiled C + F + N, then L, then C^-1
    double* M = nullptr;
    double* Dinv = nullptr;
    double* diag = nullptr;
    double* tmp = nullptr;       // [4][N] vectors + scalars
    int* st = nullptr;
    double logdet = 0;
    std::vector<double> fg;
    double* Ninv = nullptr;      // polarisation likelihood: dense N^-1 (ld x ld, column-major)
    int ld = 0;
};

extern "C" void cg_likelihood_destroy(cg_lik* lik)
{
    if (!lik) return;
    cudaSetDevice(lik->ctx.device);
    if (lik->ctx.stream) cudaStreamSynchronize(lik->ctx.stream);
    cudaFree(lik->A); cudaFree(lik->M); cudaFree(lik->Dinv); cudaFree(lik->diag); cudaFree(lik->tmp); cudaFree(lik->st);
    cudaFree(lik->Ninv);
    if (lik->ctx.stream) cudaStreamDestroy(lik->ctx.stream);
    delete lik;
}

extern "C" const char* cg_likelihood_last_error(const cg_lik* lik) { return lik ? lik->ctx.err.c_str() : g_create_error.c_str(); }
extern "C" double cg_likelihood_logdet(const cg_lik* lik) { return lik ? lik->logdet : 0.0; }

extern "C" int cg_likelihood_create(cg_lik** out, int n, const double* c_packed, const double* fid_packed,
                                    const double* noise_packed, const double* foreground, int device)
{
    g_create_error.clear();
    if (!out || n <= 0 || !c_packed || !noise_packed) { g_create_error = "bad arguments to cg_likelihood_create"; return CG_ERR_BAD_ARG; }
    *out = nullptr;
    std::unique_ptr<cg_lik> lik(new (std::nothrow) cg_lik());
    if (!lik) return CG_ERR_ALLOC;
    cg_ctx& ctx = lik->ctx;
    std::string why;
    if (!device_ok(device, &ctx.sm_count, why)) { g_create_error = why; return CG_ERR_NO_DEVICE; }
    ctx.device = device;
    ctx.n = n;
    ctx.nt = (n + cg::TS - 1) / cg::TS;
    ctx.N = ctx.nt * cg::TS;
    cudaSetDevice(device);
    if (cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking) != cudaSuccess) { g_create_error = "stream"; return CG_ERR_CUDA; }
    const size_t np = (size_t)n * (n + 1) / 2, tiled = cg::tiled_elems(ctx.nt);
    double* dpk = nullptr;
    if (!dalloc(&lik->A, tiled) || !dalloc(&lik->M, tiled) || !dalloc(&lik->Dinv, (size_t)ctx.nt * cg::TILE_ELEMS) ||
        !dalloc(&lik->diag, (size_t)ctx.N) || !dalloc(&lik->tmp, 4 * (size_t)ctx.N + 8) || !dalloc(&lik->st, 1) ||
        !dalloc(&dpk, 3 * np)) {
        cudaFree(dpk);
        g_create_error = "device allocation failed";
        cg_likelihood_destroy(lik.release());
        return CG_ERR_ALLOC;
    }
    for (size_t k = 0; k < np; ++k)
        if (!std::isfinite(c_packed[k]) || !std::isfinite(noise_packed[k]) || (fid_packed && !std::isfinite(fid_packed[k]))) {
            cudaFree(dpk);
            g_create_error = "non-finite matrix entry";
            cg_likelihood_destroy(lik.release());
            return CG_ERR_NONFINITE;
        }
    cudaStream_t s = ctx.stream;
    cudaMemcpyAsync(dpk, c_packed, sizeof(double) * np, cudaMemcpyHostToDevice, s);
    if (fid_packed) cudaMemcpyAsync(dpk + np, fid_packed, sizeof(double) * np, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dpk + 2 * np, noise_packed, sizeof(double) * np, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(lik->st, 0, sizeof(int), s);
    cg::fp64_packed_to_tiled(n, ctx.nt, dpk, fid_packed ? dpk + np : nullptr, dpk + 2 * np, lik->A, s);
    int rc = cg::tiled_cholesky<double>(&ctx, 1, ctx.nt, lik->A, lik->Dinv, lik->diag, lik->st, tiled, s);
    if (!rc) {
        cg::fp64_logdet(1, n, ctx.N, lik->diag, lik->tmp + 4 * (size_t)ctx.N, s);
        rc = cg::tiled_trtri<double>(&ctx, 1, ctx.nt, lik->A, lik->Dinv, lik->M, tiled, s);
    }
    if (!rc) rc = cg::tiled_lauum<double>(&ctx, 1, ctx.nt, lik->M, lik->A, tiled, s);
    int st = 0;
    if (!rc) {
        cudaMemcpyAsync(&lik->logdet, lik->tmp + 4 * (size_t)ctx.N, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&st, lik->st, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { ctx.err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    }
    cudaFree(dpk);
    if (!rc && st) {
        // source/likelihood.cpp:120-125: "The covariance matrix must be positive definite."
        ctx.err = "The covariance matrix is not positive definite.";
        rc = CG_ERR_NOT_PD;
    }
    if (rc) {
        g_create_error = ctx.err;
        cg_likelihood_destroy(lik.release());
        return rc;
    }
    if (foreground) lik->fg.assign(foreground, foreground + n);
    *out = lik.release();
    return CG_OK;
}

// chi2 (and the foreground terms) for the padded vector already in lik->tmp[0 .. N)
static int lik_finish(cg_lik* lik, double* chi2, double* logdet)
{
    cg_ctx& ctx = lik->ctx;
    const int n = ctx.n, N = ctx.N;
    cudaStream_t s = ctx.stream;
    double* tv = lik->tmp;          // padded t
    double* ta = tv + N;            // C^-1 t
    double* fv = ta + N;            // padded f
    double* fa = fv + N;            // C^-1 f
    double* sc = fa + N;            // scalars
    cg::fp64_symv(1, ctx.nt, N, lik->A, tv, ta, s);
    cg::fp64_dot(n, tv, ta, sc + 1, s);  // chi2 = t^T C^-1 t (Likelihood::vmv, source/likelihood.cpp:137-152)
    const bool fgm = !lik->fg.empty();
    if (fgm) {
        cudaMemcpyAsync(fv, lik->fg.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
        cg::fp64_symv(1, ctx.nt, N, lik->A, fv, fa, s);
        cg::fp64_dot(n, tv, fa, sc + 2, s);
        cg::fp64_dot(n, fv, fa, sc + 3, s);
    }
    double h[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(h, sc, sizeof(double) * 4, cudaMemcpyDeviceToHost, s);
    CG_CUDA_TRY(&ctx, cudaStreamSynchronize(s));
    *chi2 = h[1];
    *logdet = lik->logdet;
    if (fgm) {
        // foreground marginalisation, source/likelihood.cpp:171-177
        const double tCinvf = h[2], fCinvf = h[3];
        *logdet += std::log(fCinvf / n);
        *chi2 -= tCinvf * tCinvf / fCinvf;
    }
    return CG_OK;
}

extern "C" int cg_likelihood_calculate(cg_lik* lik, const double* t, double* chi2, double* logdet)
{
    if (!lik || !t || !chi2 || !logdet) return CG_ERR_BAD_ARG;
    cg_ctx& ctx = lik->ctx;
    const int n = ctx.n, N = ctx.N;
    if (lik->Ninv) { ctx.err = "a polarisation likelihood takes cg_likelihood_pol_calculate"; return CG_ERR_BAD_ARG; }
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(t[i])) { ctx.err = "non-finite map value"; return CG_ERR_NONFINITE; }
    CG_CUDA_TRY(&ctx, cudaSetDevice(ctx.device));
    cudaStream_t s = ctx.stream;
    cudaMemsetAsync(lik->tmp, 0, sizeof(double) * 4 * N, s);
    cudaMemcpyAsync(lik->tmp, t, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    return lik_finish(lik, chi2, logdet);
}

extern "C" int cg_likelihood_pol_create(cg_lik** out, int npix, const int* good, int ngood, const double* c_packed,
                                        const double* ninv, int device)
{
    g_create_error.clear();
    if (!out || npix <= 0 || !good || ngood <= 0 || ngood > npix || !c_packed || !ninv) {
        g_create_error = "bad arguments to cg_likelihood_pol_create";
        return CG_ERR_BAD_ARG;
    }
    *out = nullptr;
    for (int i = 0; i < ngood; ++i)
        if (good[i] < 0 || good[i] >= npix) { g_create_error = "good pixel index out of range"; return CG_ERR_BAD_ARG; }
    // source/likelihood.cpp:371-384: the Q and U rows and columns of the kept pixels
    const int n = 2 * ngood, size = 2 * npix, ld = (n + 63) / 64 * 64;
    auto full = [&](int k) { return k < ngood ? good[k] : npix + good[k - ngood]; };
    const size_t np = (size_t)n * (n + 1) / 2;
    std::vector<double> cg_packed(np), nd((size_t)ld * ld, 0.0);
    for (int j = 0; j < n; ++j) {
        const long fj = full(j);
        for (int i = 0; i <= j; ++i) {
            const long fi = full(i), a = std::min(fi, fj), b = std::max(fi, fj);
            cg_packed[(size_t)j * (j + 1) / 2 + i] = c_packed[(size_t)b * (b + 1) / 2 + a];
        }
        for (int i = 0; i < n; ++i) nd[(size_t)j * ld + i] = ninv[(size_t)full(i) * size + fj];
    }
    for (double v : cg_packed)
        if (!std::isfinite(v)) { g_create_error = "non-finite matrix entry"; return CG_ERR_NONFINITE; }
    for (double v : nd)
        if (!std::isfinite(v)) { g_create_error = "non-finite matrix entry"; return CG_ERR_NONFINITE; }
    cg_ctx tmpctx;
    std::string why;
    if (!device_ok(device, &tmpctx.sm_count, why)) { g_create_error = why; return CG_ERR_NO_DEVICE; }
    tmpctx.device = device;
    cudaSetDevice(device);
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { g_create_error = "stream"; return CG_ERR_CUDA; }
    const size_t nel = (size_t)ld * ld;
    double *d_c = nullptr, *d_n = nullptr, *d_cd = nullptr, *d_t = nullptr, *d_m = nullptr, *d_mp = nullptr;
    int rc = CG_OK;
    if (!dalloc(&d_c, np) || !dalloc(&d_n, nel) || !dalloc(&d_cd, nel) || !dalloc(&d_t, nel) || !dalloc(&d_m, nel) ||
        !dalloc(&d_mp, np)) {
        g_create_error = "device allocation failed";
        rc = CG_ERR_ALLOC;
    }
    std::vector<double> m_packed(np), zero(np, 0.0);
    if (rc == CG_OK) {
        cudaMemcpyAsync(d_c, cg_packed.data(), sizeof(double) * np, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_n, nd.data(), sizeof(double) * nel, cudaMemcpyHostToDevice, s);
        // source/likelihood.cpp:386-387: cInv = N^-1 + N^-1 C N^-1
        rc = cg::fp64_pol_matrix(&tmpctx, n, ld, d_c, d_n, d_cd, d_t, d_m, d_mp, s);
        if (rc == CG_OK) {
            cudaMemcpyAsync(m_packed.data(), d_mp, sizeof(double) * np, cudaMemcpyDeviceToHost, s);
            if (cudaStreamSynchronize(s) != cudaSuccess) { g_create_error = "polarisation matrix build failed"; rc = CG_ERR_CUDA; }
        } else {
            g_create_error = tmpctx.err;
        }
    }
    cudaFree(d_c); cudaFree(d_cd); cudaFree(d_t); cudaFree(d_m); cudaFree(d_mp);
    cudaStreamDestroy(s);
    if (rc == CG_OK) rc = cg_likelihood_create(out, n, m_packed.data(), nullptr, zero.data(), nullptr, device);
    if (rc != CG_OK) {
        cudaFree(d_n);
        return rc;
    }
    (*out)->Ninv = d_n;
    (*out)->ld = ld;
    return CG_OK;
}

extern "C" int cg_likelihood_pol_calculate(cg_lik* lik, const double* v, const double* subtract, double* chi2,
                                           double* logdet)
{
    if (!lik || !v || !subtract || !chi2 || !logdet) return CG_ERR_BAD_ARG;
    cg_ctx& ctx = lik->ctx;
    if (!lik->Ninv) { ctx.err = "not a polarisation likelihood"; return CG_ERR_BAD_ARG; }
    const int n = ctx.n, N = ctx.N;
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(v[i]) || !std::isfinite(subtract[i])) { ctx.err = "non-finite map value"; return CG_ERR_NONFINITE; }
    CG_CUDA_TRY(&ctx, cudaSetDevice(ctx.device));
    cudaStream_t s = ctx.stream;
    double* w = lik->tmp;           // padded w = v - N^-1 s
    double* vv = w + N;             // v, then s, in the C^-1 slots that lik_finish overwrites
    double* sv = vv + N;
    cudaMemsetAsync(lik->tmp, 0, sizeof(double) * 4 * N, s);
    cudaMemcpyAsync(vv, v, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(sv, subtract, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    // source/likelihood.cpp:595-600: vCopy -= N^-1 subtractMap
    int rc = cg::fp64_dense_residual(&ctx, n, lik->ld, lik->Ninv, vv, sv, w, s);
    if (rc) return rc;
    cudaMemsetAsync(vv, 0, sizeof(double) * 2 * N, s);
    return lik_finish(lik, chi2, logdet);   // chi2 = w^T cInv w (source/likelihood.cpp:602-609)
}

extern "C" int cg_selftest_wait_timeout(cg_ctx* ctx, int* status)
{
    if (!ctx || !status) return CG_ERR_BAD_ARG;
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return cg::selftest_wait_timeout(ctx, status);
}

extern "C" int cg_probe_fp32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms)
{
    if (!ctx || !tflops || !ms) return CG_ERR_BAD_ARG;
    if (iters > (1 << 24) || reps > 10000) { ctx->err = "cg_probe_fp32_rate: iters <= 2^24, reps <= 10000"; return CG_ERR_BAD_ARG; }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return cg::probe_fp32_rate(ctx, iters, reps, tflops, ms);
}

extern "C" int cg_probe_tf32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms)
{
    if (!ctx || !tflops || !ms) return CG_ERR_BAD_ARG;
    if (iters > (1 << 22) || reps > 10000) { ctx->err = "cg_probe_tf32_rate: iters <= 2^22, reps <= 10000"; return CG_ERR_BAD_ARG; }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return cg::probe_tf32_rate(ctx, iters, reps, tflops, ms);
}
