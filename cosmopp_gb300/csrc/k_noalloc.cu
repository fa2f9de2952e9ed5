// Allocation-free variant of the Likelihood drop-in's construct + calculate
// (FP64 Cholesky of C + fiducial + noise, ln det, explicit inverse, chi2 of one
// map) for callers that may not call cudaMalloc: code running inside another
// framework's memory pool or allocator, plug-ins loaded into a host process
// that owns every device allocation, or hosts whose policy forbids device
// allocations after start-up.  The caller passes inputs and outputs in device
// memory; the workspace is a fixed static device array in this file.
//
// The array holds the workspace of one matrix of up to CG_NOALLOC_MAX_N
// pixels (about 5.5 MB) and stays resident on every GPU that loads the
// library until the process exits.  All calls share it: two calls whose GPU
// work overlaps (different streams, or different host threads on one device)
// race on it and give wrong results; serialise them.  Each call clears what
// must start at zero, so the contents a previous call left behind do not
// matter.
//
// The outputs (d_out, d_status) are written by the last kernel the call queues, so
// they are meaningful only when the call returned CG_OK; a host-side error returns
// before that kernel is queued and leaves them as they were.
//
// The first call on each device resolves the array's device address with
// cudaGetSymbolAddress (with that device current).  Make that first call
// before capturing a CUDA graph on the device.
#include <mutex>

#include "cg_internal.h"

#define CG_NOALLOC_MAX_N 768

namespace {

constexpr int kMaxNt = (CG_NOALLOC_MAX_N + cg::TS - 1) / cg::TS;
constexpr size_t kTiled = (size_t)kMaxNt * (kMaxNt + 1) / 2 * cg::TILE_ELEMS;
constexpr size_t kN = (size_t)kMaxNt * cg::TS;
// layout (in doubles): A, M (tiled), Dinv, diag, t, C^-1 t, scalars[8], status
constexpr size_t kOffA = 0;
constexpr size_t kOffM = kOffA + kTiled;
constexpr size_t kOffDinv = kOffM + kTiled;
constexpr size_t kOffDiag = kOffDinv + (size_t)kMaxNt * cg::TILE_ELEMS;
constexpr size_t kOffT = kOffDiag + kN;
constexpr size_t kOffTa = kOffT + kN;
constexpr size_t kOffSc = kOffTa + kN;
constexpr size_t kOffSt = kOffSc + 8;
constexpr size_t kScratchDoubles = kOffSt + 8;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// once per device, with that device current
int scratch_for_device(int device, double** out, std::string& err)
{
    if (device < 0 || device >= kMaxDevices) { err = "device ordinal out of range"; return CG_ERR_BAD_ARG; }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return CG_ERR_CUDA;
        }
        g_scratch_addr[device] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[device];
    return CG_OK;
}

__global__ void noalloc_finish(int n, const double* __restrict__ sc, const int* __restrict__ st,
                               double* __restrict__ out, int* __restrict__ status)
{
    if (threadIdx.x != 0) return;
    out[0] = sc[1];  // chi2 = t^T C^-1 t
    out[1] = sc[0];  // raw ln det C
    if (status) *status = *st;
}

}  // namespace

namespace cg {
void set_global_error(const std::string& msg);
}

extern "C" int cg_likelihood_noalloc(int n, const double* d_c_packed, const double* d_fid_packed,
                                     const double* d_noise_packed, const double* d_t, double* d_out, int* d_status,
                                     void* stream)
{
    if (n <= 0 || !d_c_packed || !d_noise_packed || !d_t || !d_out) {
        cg::set_global_error("cg_likelihood_noalloc: NULL pointer or n <= 0");
        return CG_ERR_BAD_ARG;
    }
    if (n > CG_NOALLOC_MAX_N) {
        cg::set_global_error("cg_likelihood_noalloc: n = " + std::to_string(n) + " exceeds the static workspace limit of " +
                             std::to_string(CG_NOALLOC_MAX_N) + " pixels; use cg_likelihood_create");
        return CG_ERR_BAD_ARG;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cg::set_global_error("cg_likelihood_noalloc: no current CUDA device");
        return CG_ERR_NO_DEVICE;
    }
    std::string err;
    double* base = nullptr;
    int rc = scratch_for_device(device, &base, err);
    if (rc) { cg::set_global_error("cg_likelihood_noalloc: " + err); return rc; }

    cg_ctx ctx;  // sizes and error text only; owns no device memory
    ctx.device = device;
    ctx.n = n;
    ctx.nt = (n + cg::TS - 1) / cg::TS;
    ctx.N = ctx.nt * cg::TS;
    const size_t tiled = cg::tiled_elems(ctx.nt);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* A = base + kOffA;
    double* M = base + kOffM;
    double* Dinv = base + kOffDinv;
    double* diag = base + kOffDiag;
    double* tv = base + kOffT;
    double* ta = base + kOffTa;
    double* sc = base + kOffSc;
    int* st = reinterpret_cast<int*>(base + kOffSt);

    // what must start at zero: the status word and the padded map
    if (cudaMemsetAsync(st, 0, sizeof(int), s) != cudaSuccess ||
        cudaMemsetAsync(tv, 0, sizeof(double) * ctx.N, s) != cudaSuccess ||
        cudaMemcpyAsync(tv, d_t, sizeof(double) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        cg::set_global_error("cg_likelihood_noalloc: cudaMemsetAsync / cudaMemcpyAsync failed");
        return CG_ERR_CUDA;
    }
    cg::fp64_packed_to_tiled(n, ctx.nt, d_c_packed, d_fid_packed, d_noise_packed, A, s);
    rc = cg::tiled_cholesky<double>(&ctx, 1, ctx.nt, A, Dinv, diag, st, tiled, s);
    if (!rc) {
        cg::fp64_logdet(1, n, ctx.N, diag, sc, s);
        rc = cg::tiled_trtri<double>(&ctx, 1, ctx.nt, A, Dinv, M, tiled, s);
    }
    if (!rc) rc = cg::tiled_lauum<double>(&ctx, 1, ctx.nt, M, A, tiled, s);
    if (!rc) {
        cg::fp64_symv(1, ctx.nt, ctx.N, A, tv, ta, s);
        cg::fp64_dot(n, tv, ta, sc + 1, s);
        noalloc_finish<<<1, 32, 0, s>>>(n, sc, st, d_out, d_status);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { ctx.err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    }
    if (rc) cg::set_global_error("cg_likelihood_noalloc: " + ctx.err);
    return rc;
}
