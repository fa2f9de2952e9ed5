// Launch-shape tuning of the batched mixed path: named knobs (cg_tune_set / cg_tune_get), a
// coordinate search timed with CUDA events on the context's own shape (cg_autotune), and a text
// file of the results per device, pixel count, l range and batch size (cg_tune_load), which
// cg_create reads when COSMOPP_GB300_TUNE_FILE names one.  The reference has no counterpart: its
// covariance and likelihood run on the CPU with no launch shapes to choose.
//
// File format, one entry per line (later lines for the same key win):
//   <device name>|n=<n>|lmax=<lmax>|B=<B>| fwd=0 fwd_ctas=0 chol_ctas=0 panel_ctas=0 adj=0 diag_sq=1 ms=31.5
// The search covers the launch-shape knobs only (CTA counts, the adjoint's fetch variant); the
// knobs that change rounding (fwd, diag_sq, table_bf16) keep the values they have.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <vector>

#include "cg_internal.h"

namespace {

struct Knob {
    const char* name;
    int cg::Tune::*field;
};

const Knob kKnobs[] = {
    {"fwd", &cg::Tune::fwd},
    {"fwd_ctas", &cg::Tune::fwd_ctas},
    {"chol_ctas", &cg::Tune::chol_ctas},
    {"panel_ctas", &cg::Tune::panel_ctas},
    {"adj", &cg::Tune::adj},
    {"diag_sq", &cg::Tune::diag_sq},
    {"table_bf16", &cg::Tune::table_bf16},
    {"graph", &cg::Tune::graph},
    {"lauum", &cg::Tune::lauum},
    {"trtri", &cg::Tune::trtri},
    {"hmc_device", &cg::Tune::hmc_device},
    {"overlap", &cg::Tune::overlap},
};

const Knob* find_knob(const char* name)
{
    if (!name) return nullptr;
    for (const Knob& k : kKnobs)
        if (std::strcmp(k.name, name) == 0) return &k;
    return nullptr;
}

// the values a knob may take on this context (also the autotuner's candidates)
std::vector<int> candidates(const cg_ctx* ctx, const Knob& k)
{
    const int sm = ctx->sm_count;
    const int lp = ((ctx->lmax + 1 + 15) / 16) * 16;
    (void)lp;
    if (k.field == &cg::Tune::fwd_ctas) return {0, sm * 3 / 4, sm / 2};
    if (k.field == &cg::Tune::chol_ctas) return {0, sm / 2, 2 * sm};
    if (k.field == &cg::Tune::panel_ctas) return {0, sm / 2, sm, 2 * sm};
    if (k.field == &cg::Tune::adj) return {0, 1, 2, 3};
    if (k.field == &cg::Tune::lauum) return {0, 1, 2};
    if (k.field == &cg::Tune::trtri) return {0, 1};
    if (k.field == &cg::Tune::overlap) return {1, 0};
    return {ctx->tune.*(k.field)};  // accuracy knobs (fwd, diag_sq, table_bf16) and switches (graph, hmc_device): not searched
}

bool valid_value(const cg_ctx* ctx, const Knob& k, int v)
{
    if (k.field == &cg::Tune::fwd) return v == 0 || v == 1;
    if (k.field == &cg::Tune::adj) return v >= 0 && v <= 3;
    if (k.field == &cg::Tune::lauum) return v >= 0 && v <= 2;
    if (k.field == &cg::Tune::diag_sq || k.field == &cg::Tune::table_bf16 || k.field == &cg::Tune::graph ||
        k.field == &cg::Tune::trtri || k.field == &cg::Tune::hmc_device || k.field == &cg::Tune::overlap)
        return v == 0 || v == 1;
    return v >= 0 && v <= 64 * std::max(1, ctx->sm_count);  // CTA counts; 0 = one per SM
}

std::string device_name(int device)
{
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return "unknown";
    std::string s = p.name;
    std::replace(s.begin(), s.end(), '|', '_');
    return s;
}

std::string key_of(const cg_ctx* ctx, int B)
{
    std::ostringstream o;
    o << device_name(ctx->device) << "|n=" << ctx->n << "|lmax=" << ctx->lmax << "|B=" << B << "|";
    return o.str();
}

std::string describe(const cg::Tune& t)
{
    std::ostringstream o;
    bool first = true;
    for (const Knob& k : kKnobs) {
        o << (first ? "" : " ") << k.name << "=" << t.*(k.field);
        first = false;
    }
    return o.str();
}

// knob=value pairs of a line's tail into t (unknown names are skipped); false if nothing parsed
bool parse_values(const cg_ctx* ctx, const std::string& tail, cg::Tune& t)
{
    std::istringstream in(tail);
    std::string tok;
    int got = 0;
    while (in >> tok) {
        const size_t eq = tok.find('=');
        if (eq == std::string::npos) continue;
        const Knob* k = find_knob(tok.substr(0, eq).c_str());
        if (!k) continue;
        char* end = nullptr;
        const long v = std::strtol(tok.c_str() + eq + 1, &end, 10);
        if (!end || *end || !valid_value(ctx, *k, (int)v)) return false;
        t.*(k->field) = (int)v;
        ++got;
    }
    return got > 0;
}

// median device time of `reps` mixed-path calls on the staging buffers (after one warm-up call)
int time_calls(cg_ctx* ctx, int B, int reps, double* ms)
{
    const int L1 = ctx->lmax + 1, Bm = ctx->max_batch;
    double* o_m2 = ctx->d_out;
    double* o_grad = o_m2 + 3 * (size_t)Bm;
    double* o_d = o_grad + (size_t)Bm * L1;
    int* o_st = (int*)(o_d + (size_t)Bm * ctx->N);
    cudaStream_t s = ctx->stream;
    cudaEvent_t e0, e1;
    CG_CUDA_TRY(ctx, cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); ctx->err = "cudaEventCreate"; return CG_ERR_CUDA; }
    std::vector<float> t;
    int rc = CG_OK;
    for (int r = 0; r <= reps && !rc; ++r) {
        cudaEventRecord(e0, s);
        rc = cg_loglike_device(ctx, B, ctx->d_cl, o_d, 0, o_m2, nullptr, nullptr, o_grad, o_st, s);
        cudaEventRecord(e1, s);
        if (!rc && cudaEventSynchronize(e1) != cudaSuccess) { ctx->err = "cudaEventSynchronize"; rc = CG_ERR_CUDA; }
        float x = 0;
        if (!rc && r > 0) {
            cudaEventElapsedTime(&x, e0, e1);
            t.push_back(x);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return CG_OK;
}

}  // namespace

extern "C" int cg_tune_set(cg_ctx* ctx, const char* knob, int value)
{
    if (!ctx) return CG_ERR_BAD_ARG;
    const Knob* k = find_knob(knob);
    if (!k || !valid_value(ctx, *k, value)) { ctx->err = std::string("cg_tune_set: bad knob or value: ") + (knob ? knob : "NULL"); return CG_ERR_BAD_ARG; }
    const int old = ctx->tune.*(k->field);
    ctx->tune.*(k->field) = value;
    if (old != value) ++ctx->epoch;  // a captured call baked the old launch shapes in
    // the table is built at the reference point: rebuild it in the new precision
    if (k->field == &cg::Tune::table_bf16 && old != value && ctx->precision == CG_PREC_MIXED && ctx->wmx.have_ref) {
        CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
        const std::vector<double> ref = ctx->wmx.cl_ref;
        return cg::mixed_prepare_reference(ctx, ref.data());
    }
    return CG_OK;
}

extern "C" int cg_tune_get(const cg_ctx* ctx, const char* knob, int* value)
{
    const Knob* k = find_knob(knob);
    if (!ctx || !k || !value) return CG_ERR_BAD_ARG;
    *value = ctx->tune.*(k->field);
    return CG_OK;
}

extern "C" int cg_tune_describe(const cg_ctx* ctx, char* buf, int len)
{
    if (!ctx || !buf || len <= 0) return CG_ERR_BAD_ARG;
    const std::string s = describe(ctx->tune);
    std::snprintf(buf, (size_t)len, "%s", s.c_str());
    return (int)s.size() < len ? CG_OK : CG_ERR_BAD_ARG;
}

extern "C" int cg_tune_load(cg_ctx* ctx, const char* path, int* found)
{
    if (!ctx || !path) return CG_ERR_BAD_ARG;
    if (found) *found = 0;
    std::ifstream in(path);
    if (!in) return CG_OK;  // no file yet: keep the defaults
    const std::string key = key_of(ctx, ctx->max_batch);
    std::string line;
    cg::Tune best = ctx->tune;
    bool hit = false;
    while (std::getline(in, line)) {
        if (line.compare(0, key.size(), key) != 0) continue;
        cg::Tune t = ctx->tune;
        if (parse_values(ctx, line.substr(key.size()), t)) {
            best = t;
            hit = true;
        }
    }
    if (hit) {
        ctx->tune = best;
        ++ctx->epoch;
    }
    if (found) *found = hit ? 1 : 0;
    return CG_OK;
}

extern "C" int cg_autotune(cg_ctx* ctx, int B, const char* path, double* best_ms)
{
    if (!ctx) return CG_ERR_BAD_ARG;
    if (ctx->precision != CG_PREC_MIXED) { ctx->err = "cg_autotune: the knobs belong to the mixed path"; return CG_ERR_BAD_ARG; }
    if (B < 1 || B > ctx->max_batch) { ctx->err = "cg_autotune: 1 <= B <= max_batch"; return CG_ERR_BAD_ARG; }
    CG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    // inputs: the reference point's C_l (or the smooth law) perturbed by +-5% per element and l,
    // deterministic; one map of unit values.  The launch shapes do not depend on the values.
    const int L1 = ctx->lmax + 1, Bm = ctx->max_batch;
    std::vector<double> base(L1, 0.0), cl((size_t)B * L1, 0.0), d((size_t)ctx->n, 1.0);
    for (int l = 2; l < L1; ++l)
        base[l] = ctx->wmx.have_ref ? ctx->wmx.cl_ref[l] : 1e3 * 2.0 * cg::kPiHost / (l * (l + 1.0));
    for (int b = 0; b < B; ++b)
        for (int l = 2; l < L1; ++l) cl[(size_t)b * L1 + l] = base[l] * (1.0 + 0.05 * std::sin(0.7 * b + 1.3 * l));
    double* o_d = ctx->d_out + 3 * (size_t)Bm + (size_t)Bm * L1;
    CG_CUDA_TRY(ctx, cudaMemcpy(ctx->d_cl, cl.data(), sizeof(double) * cl.size(), cudaMemcpyHostToDevice));
    CG_CUDA_TRY(ctx, cudaMemcpy(o_d, d.data(), sizeof(double) * d.size(), cudaMemcpyHostToDevice));
    const cg::Tune saved = ctx->tune;
    ++ctx->epoch;
    const bool prof = ctx->profiling;
    ctx->profiling = false;
    const int reps = 3;
    double best = 0;
    int rc = time_calls(ctx, B, reps, &best);
    // one coordinate pass: each knob in turn over its candidates, the others at their best so far
    for (const Knob& k : kKnobs) {
        if (rc) break;
        if (k.field == &cg::Tune::fwd_ctas && ctx->tune.fwd != 1) continue;
        const int keep = ctx->tune.*(k.field);
        int pick = keep;
        for (int v : candidates(ctx, k)) {
            if (v == keep) continue;
            ctx->tune.*(k.field) = v;
            ++ctx->epoch;
            double ms = 0;
            if ((rc = time_calls(ctx, B, reps, &ms))) break;
            if (ms < best * 0.995) {  // a change must win by more than the timing noise
                best = ms;
                pick = v;
            }
        }
        ctx->tune.*(k.field) = pick;
        ++ctx->epoch;
    }
    ctx->profiling = prof;
    if (rc) {
        ctx->tune = saved;
        ++ctx->epoch;
        return rc;
    }
    if (best_ms) *best_ms = best;
    if (path && *path) {
        std::ofstream out(path, std::ios::app);
        if (!out) { ctx->err = std::string("cg_autotune: cannot append to ") + path; return CG_ERR_BAD_ARG; }
        out << key_of(ctx, B) << " " << describe(ctx->tune) << " ms=" << best << "\n";
    }
    return CG_OK;
}
