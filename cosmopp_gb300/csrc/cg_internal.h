// Internal declarations shared by the cosmopp_gb300 translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/cosmopp_gb300.h"

namespace cg {

// ---- tiled symmetric layout ---------------------------------------------
// An N x N symmetric matrix (N = nt * TS) is kept as its lower-triangular
// tiles: tile (I, J), J <= I, at tile index I(I+1)/2 + J, each tile TS x TS
// column-major (element (r, c) at r + c*TS).  Padding rows/columns n..N-1 hold
// the identity, which changes neither ln det nor any solve.
constexpr int TS = 64;
constexpr int TILE_ELEMS = TS * TS;
constexpr double kPiHost = 3.141592653589793;  // Math::pi, include/math_constants.hpp:8

__host__ __device__ inline int tile_index(int I, int J) { return I * (I + 1) / 2 + J; }
__host__ __device__ inline int ntiles_lower(int nt) { return nt * (nt + 1) / 2; }
inline size_t tiled_elems(int nt) { return (size_t)ntiles_lower(nt) * TILE_ELEMS; }

// inverse of tile_index for the lower triangle: t -> (I, J)
__host__ __device__ inline void tile_coords(int t, int& I, int& J)
{
    int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while (i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    I = i;
    J = t - i * (i + 1) / 2;
}

// ---- constants uploaded per context --------------------------------------
struct LegConsts {
    // Bonnet recurrence coefficients exactly as include/legendre.hpp:34 forms
    // them: a_l = 2 - 1.0/l, b_l = 1 - 1.0/l
    std::vector<double> a, b;
    std::vector<double> beam;   // B_l (pixel window x beam), source/utils.cpp:149-158
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// ---- plain FP64 path workspace -------------------------------------------
struct Fp64Work {
    int cap = 0;                 // batch capacity
    double* A = nullptr;         // [cap][tiled]  C, then L, then C^-1
    double* M = nullptr;         // [cap][tiled]  L^-1
    double* Dinv = nullptr;      // [cap][nt][TS*TS] inverses of the diagonal L tiles
    double* diag = nullptr;      // [cap][N] diagonal of L
    double* clc = nullptr;       // [cap][lmax+1] cl_l (2l+1)/(4 pi)
    double* dvec = nullptr;      // [cap][N] data maps (padded)
    double* alpha = nullptr;     // [cap][N]
    double* gpart = nullptr;     // [cap][nblk][lmax+1] adjoint partial sums
    int* st = nullptr;           // [cap] status
    double* ld = nullptr;        // [cap] ln det
};

// ---- mixed path workspace ------------------------------------------------
struct MixedWork {
    int cap = 0;
    bool have_ref = false;
    std::vector<double> cl_ref;  // current reference C_l (host copy)
    int ref_count = 0;
    int lpad = 0;                // l extent of the table rows (lmax + 1 rounded up to 16)
    // reference point, FP64
    double* Lref = nullptr;      // [tiled] Cholesky factor of C_ref
    double* Mref = nullptr;      // [tiled] L_ref^-1
    double* Dinv_ref = nullptr;  // [nt][TS*TS]
    double* diag_ref = nullptr;  // [N]
    double* cref = nullptr;      // [lmax+1] reference C_l on the device
    double* ldref = nullptr;     // [1] ln det C_ref
    double* Y = nullptr;         // [nharm_pad][N] real spherical harmonics x B_l at the pixels
    double* Z = nullptr;         // [nharm_pad][N] L_ref^-1 Y
    float* U = nullptr;          // [tiles][TS*TS][lpad] whitened Legendre table
    float* Zf = nullptr;         // [nharm_pad][N] Z in FP32 (the x^T Ubar x term of the gradient)
    // per batch element
    float* A = nullptr;          // [cap][tiled] I + K_b (kept for the refinement residual)
    float* V = nullptr;          // [cap][tiled] V_b = (I + K_b)^-1
    float* Ls = nullptr;         // [cap][tc_split_elems] L_b, split canonical storage
    float* Ms = nullptr;         // [cap][tc_split_elems] (L_b^-1)^T blocks, split canonical storage
    float* Lc = nullptr;         // [cap][tc_c1_elems] L_b (and S before the panel solve), FP32 canonical
    float* Mc = nullptr;         // [cap][tc_c1_elems] (L_b^-1)^T blocks, FP32 canonical
    float* Linv = nullptr;       // [cap][tc_linv_elems] inverses of the 128x128 diagonal blocks of L_b
    float* diag = nullptr;       // [cap][N]
    float* eps = nullptr;        // [cap][lpad] C_l / Cref_l - 1
    double* y = nullptr;         // [cap][N] L_ref^-1 d
    double* x = nullptr;         // [cap][N] (I+K)^-1 y
    double* r = nullptr;         // [cap][N] refinement residual
    double* part = nullptr;      // [cap][tiles][2][TS] matvec partials (FP64 for trmv, float2 pairs for symv)
    float* gpart = nullptr;      // [tiles][cap][lpad] adjoint partials
    float* proj = nullptr;       // [cap][nharm_pad] Z^T x_b
    double* ld = nullptr;        // [cap] ln det C_b
    int* st = nullptr;           // [cap]
    int* tcerr = nullptr;        // [1 + tc_queue_slots] tensor-core error flag and work-queue counters
};

// ---- launch-shape knobs of the mixed path (set by cg_tune_set / cg_autotune / a tuning file) ----
struct Tune {
    // forward contraction: 0 = FP32 FMA (contract_fwd, round to nearest), 1 = tensor cores
    // (contract_fwd_tc): faster, but the tensor core's one-way FP32 accumulation biases A's entries
    // by a few ulp of |A - I|, which grows with |C_l / C_ref,l - 1| (1.3e-3 in -2lnL at nside 16
    // for C_l = C_ref / e); an accuracy choice, not searched by the autotuner
    int fwd = 0;
    int fwd_ctas = 0;     // persistent CTAs of the tensor-core contraction (0 = one per SM)
    int chol_ctas = 0;    // persistent CTAs of the Cholesky's off-diagonal work queue, column blocks J > 0 (0 = one per SM)
    int panel_ctas = 0;   // persistent CTAs of the Cholesky's panel solve (0 = one per SM; 7/8 of them when
                          // trtri's rows run beside the Cholesky)
    int adj = 0;          // tensor-core adjoint variant (fetch groups / buffers), 0 .. 3
    int diag_sq = 1;      // Cholesky diagonal blocks: row sums of squares on the CUDA cores (accuracy, not speed)
    int table_bf16 = 0;   // the whitened Legendre table rounded to BF16 (8-bit significand) when it is built:
                          // the BF16 table variant, for its measured error; storage stays FP32
    int graph = 1;        // mixed calls with a fixed reference point replayed as one CUDA graph
    int lauum = 2;        // lauum: one CTA per block with the A operand from the FP32 copy, split on chip (2),
                          // or from the split copy (0); persistent CTAs over a work queue (1)
    int trtri = 0;        // 0 = one CTA per trtri block, 1 = persistent CTAs over a work queue (same results)
    int hmc_device = 1;   // cg_hmc_run: 1 = leapfrog resident on the device, 0 = the host loop (same chains)
    int overlap = 1;      // 1 = trtri's row launches run beside the Cholesky (which moves to a high-priority
                          // stream of the context), row I2 once column I2's update is done; 0 = after it.
                          // With the work-queue trtri (trtri = 1) the launches stay in sequence
};

// the argument set a captured mixed call was recorded for
struct GraphKey {
    int B = 0, d_stride = 0;
    const void* ptr[8] = {};
    cudaStream_t stream = nullptr;
    bool operator==(const GraphKey& o) const
    {
        if (B != o.B || d_stride != o.d_stride || stream != o.stream) return false;
        for (int i = 0; i < 8; ++i)
            if (ptr[i] != o.ptr[i]) return false;
        return true;
    }
};

}  // namespace cg

struct cg_ctx {
    int device = 0;
    int n = 0, nt = 0, N = 0;    // kept pixels, tiles per side, padded size
    int lmax = 0;
    double fwhm_deg = -1;        // Gaussian beam FWHM (degrees); -1 when the caller gave the beam table
    int max_batch = 1;
    int precision = CG_PREC_FP64;
    int recenter = CG_RECENTER_AUTO;
    double recenter_radius = 1.0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    // the overlapped Cholesky + trtri (Tune::overlap): the Cholesky's stream, at the device's highest
    // priority, and the events that fork it from the caller's stream, hand each column to trtri and join
    cudaStream_t hi = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_col = nullptr, ev_join = nullptr;
    std::vector<double> xyz;     // [n][3]
    std::vector<double> noise;   // [n]
    cg::LegConsts leg;
    double* d_xyz = nullptr;     // [3][N] SoA, padding rows = 0
    double* d_noise = nullptr;   // [N]
    double* d_lega = nullptr;    // [lmax+1]
    double* d_legb = nullptr;
    double* d_beam = nullptr;
    double* d_cl = nullptr;      // staging [max_batch][lmax+1]
    double* d_out = nullptr;     // staging for outputs
    size_t d_out_bytes = 0;
    cg::Fp64Work w64;
    cg::MixedWork wmx;
    cg::Tune tune;
    // one captured mixed call (cg_loglike_device), replayed while its arguments, the knobs and the
    // workspace stay the same; epoch counts changes to the latter two
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        cg::GraphKey key;
        long long epoch = -1;
        long long launches = 0;     // kernels in the captured call
        long long last_use = 0;
    };
    static constexpr int kGraphs = 8;  // argument sets kept (a caller cycling a few buffers)
    Graph graphs[kGraphs];
    long long epoch = 0, graph_uses = 0, graph_replays = 0;
    // memory admission (cg_plan_memory): a call's batch runs in pieces of `chunk` elements
    int chunk = 0;
    cg_memory_plan plan = {};
    std::string err;
    // instrumentation: kernel launch counter and optional per-stage CUDA events
    long long launches = 0;
    bool profiling = false;
    int nmarks = 0;
    cudaEvent_t marks[16] = {};
    int mark_stage[16] = {};
};

// helpers shared by the translation units
#define CG_CUDA_TRY(ctx, expr)                                                           \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            (ctx)->err = std::string(#expr) + ": " + cudaGetErrorString(e_);            \
            return CG_ERR_CUDA;                                                          \
        }                                                                                \
    } while (0)

namespace cg {
// stage ids reported by cg_stage_times
enum Stage { ST_BUILD = 0, ST_CHOL, ST_TRTRI, ST_LAUUM, ST_SOLVE, ST_ADJOINT, ST_END, ST_COUNT };
inline void stage_mark(cg_ctx* ctx, int stage, cudaStream_t s)
{
    if (!ctx->profiling || ctx->nmarks >= 16) return;
    if (!ctx->marks[ctx->nmarks]) cudaEventCreate(&ctx->marks[ctx->nmarks]);
    ctx->mark_stage[ctx->nmarks] = stage;
    cudaEventRecord(ctx->marks[ctx->nmarks], s);
    ++ctx->nmarks;
}
inline void count_launch(cg_ctx* ctx, long long k = 1) { ctx->launches += k; }
// plain FP64 path (k_fp64.cu)
int fp64_ensure(cg_ctx* ctx, int B);
size_t fp64_bytes_per_element(const cg_ctx* ctx);
// mixed path device bytes: reference point + table, and one batch element's workspace
void mixed_bytes(const cg_ctx* ctx, size_t* fixed, size_t* per_element);
int fp64_build_tiled(cg_ctx* ctx, int B, const double* d_cl, bool add_noise, cudaStream_t s);
int fp64_build_tiled_into(cg_ctx* ctx, int B, const double* d_cl, bool add_noise, double* A, cudaStream_t s);
int fp64_build_packed(cg_ctx* ctx, int B, const double* d_cl, double* d_out, cudaStream_t s);
// polarisation likelihood set-up: M = N^-1 + N^-1 C N^-1 for packed C and dense N^-1 (ld x ld,
// column-major, zero padded), packed into d_m_packed; d_cd, d_t, d_m are ld x ld scratch
int fp64_pol_matrix(cg_ctx* ctx, int n, int ld, const double* d_c_packed, const double* d_ninv, double* d_cd,
                    double* d_t, double* d_m, double* d_m_packed, cudaStream_t s);
// w = v - N^-1 s for the dense N^-1 above
int fp64_dense_residual(cg_ctx* ctx, int n, int ld, const double* d_ninv, const double* d_v, const double* d_s,
                        double* d_w, cudaStream_t s);
// P_l(x_ij) for l0 <= l < l1 into d_out [(l1 - l0)][n(n+1)/2]; d_a, d_b = the recurrence
// coefficients, at least l1 entries each (device pointers)
int fp64_legendre_table(cg_ctx* ctx, int l0, int l1, const double* d_a, const double* d_b, double* d_out,
                        cudaStream_t s);
// packed noise covariance from simulations [nsims][n] and per-pixel means (device pointers)
int fp64_noise_matrix(cg_ctx* ctx, int nsims, int n, const double* d_sims, double* d_out, double* d_mean,
                      cudaStream_t s);
int fp64_build_fiducial(cg_ctx* ctx, int lo, int hi, const double* d_tables, double m0, double* d_out,
                        cudaStream_t s);
int fp64_loglike(cg_ctx* ctx, int B, const double* d_cl, const double* d_d, int d_stride, double* d_m2lnl,
                 double* d_chi2, double* d_logdet, double* d_grad, int* d_status, cudaStream_t s);
// generic tiled FP64 / FP32 factorisation entry points (k_chol.cu)
template <typename T>
int tiled_cholesky(cg_ctx* ctx, int B, int nt, T* A, T* Dinv, T* diag, int* status, size_t strideA, cudaStream_t s);
template <typename T>
int tiled_trtri(cg_ctx* ctx, int B, int nt, const T* L, const T* Dinv, T* M, size_t strideA, cudaStream_t s);
template <typename T>
int tiled_lauum(cg_ctx* ctx, int B, int nt, const T* M, T* V, size_t strideA, cudaStream_t s);
// tensor-core FP32 (3xTF32) versions (k_tc.cu); d_err is set if a bounded wait gave up
// tensor-core FP32 kernels (k_tc.cu): L, M^T and Linv in the split canonical storage
size_t tc_split_elems(int nt);   // floats per matrix of the split (hi/lo) L / M^T storage
size_t tc_c1_elems(int nt);      // floats per matrix of the FP32 canonical L / M^T copies
size_t tc_linv_elems(int nt);    // floats per matrix of the Linv blocks
// The tensor-core entry points take d_err = [0] the error flag (set when a bounded wait gave up),
// then tc_queue_slots(nt) work-queue counters, all zero before the call.
int tc_queue_slots(int nt);

// device-resident leapfrog of cg_hmc_run (k_hmc.cu): half kick + drift + C_l = exp(x); gradient in
// ln C_l + half kick; dH per chain; accepted proposals into the chains' state
int hmc_launch_drift(cg_ctx* ctx, int B, int np, double t, double* p, const double* g, double* x, const double* mass,
                     const double* tmpl, double* cl, cudaStream_t s);
int hmc_launch_kick(cg_ctx* ctx, int B, int np, double t, int kick, double* p, double* g, const double* gcl,
                    const double* cl, const int* st, double* m2lnl, cudaStream_t s);
int hmc_launch_energy(cg_ctx* ctx, int B, int np, const double* p, const double* mass, const double* un,
                      const double* u, const double* kin0, double* dh, cudaStream_t s);
int hmc_launch_accept(cg_ctx* ctx, int B, int np, const int* flag, const double* xn, const double* gn,
                      const double* un, double* x, double* g, double* u, cudaStream_t s);
int tiled_cholesky_tc(cg_ctx* ctx, int B, int nt, const float* A, float* Ls, float* Lc, float* Linv, float* Ms,
                      float* Mc, float* diag, int* status, int* d_err, cudaStream_t s);
// the tensor-core Cholesky with trtri's row launches beside it (Tune::overlap = 1): the Cholesky on
// ctx->hi, forked from s; row I2 on s once column I2's update is done; s joins the Cholesky at the end
int tiled_chol_trtri_tc(cg_ctx* ctx, int B, int nt, const float* A, float* Ls, float* Lc, float* Linv, float* Ms,
                        float* Mc, float* diag, int* status, int* d_err, cudaStream_t s);
int tiled_trtri_tc(cg_ctx* ctx, int B, int nt, const float* Ls, const float* Linv, float* Ms, float* Mc,
                   int* d_err, cudaStream_t s);
int tiled_lauum_tc(cg_ctx* ctx, int B, int nt, const float* Ms, const float* Mc, float* V, int* d_err,
                   const double* y, int ystride, float2* part, cudaStream_t s);
// part[t][b][l] = sum_e w_e V_b[e] Ubar_l[e] over lower tile t (k_tc.cu), for lp % 16 == 0, lp <= 96
bool adjoint_tc_ok(int lp);
int adjoint_contract_tc(cg_ctx* ctx, int B, int nt, int lp, const float* U, const float* V, size_t strideA,
                        float* part, int* d_err, cudaStream_t s);
// A_b = I + sum_l eps_bl Ubar_l on the tensor cores (k_tc.cu), for lp % 16 == 0, lp <= 64; ctas = the
// persistent grid (0 = one CTA per SM)
bool contract_fwd_tc_ok(int lp);
int contract_fwd_tc_launch(cg_ctx* ctx, int B, int nt, int lp, const float* U, const float* eps, float* A,
                           size_t strideA, int* d_err, int ctas, cudaStream_t s);
int selftest_wait_timeout(cg_ctx* ctx, int* host_status);
// achieved rate of the factorisation kernels' MMA form (kind::tf32 M128 N128 K8, A in tensor memory)
int probe_tf32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms_per_launch);
// achieved FP32 rate of packed two-lane FMAs (fma.rn.f32x2), the FP32 contraction's instruction
int probe_fp32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms_per_launch);
// mixed path (k_mixed.cu)
int mixed_prepare_reference(cg_ctx* ctx, const double* cl_ref_host);
int mixed_loglike(cg_ctx* ctx, int B, const double* d_cl, const double* h_cl, const double* d_d, int d_stride,
                  double* d_m2lnl, double* d_chi2, double* d_logdet, double* d_grad, int* d_status, cudaStream_t s);
void mixed_free(cg_ctx* ctx);
// the mixed path's per-element workspace for B elements (allocated before a graph capture)
int mixed_ensure(cg_ctx* ctx, int B);
void fp64_free(cg_ctx* ctx);
// small FP64 launchers used by the Likelihood drop-in (k_fp64.cu)
void fp64_packed_to_tiled(int n, int nt, const double* c, const double* f, const double* nz, double* A, cudaStream_t s);
void fp64_symv(int B, int nt, int N, const double* V, const double* dv, double* alpha, cudaStream_t s);
void fp64_logdet(int B, int n, int N, const double* diag, double* out, cudaStream_t s);
void fp64_dot(int n, const double* a, const double* b, double* out, cudaStream_t s);
}  // namespace cg
