// Batched mixed-precision path: -2lnL and d(-2lnL)/dC_l for many C_l vectors.
//
// The reference evaluates one C_l at a time: clToCMatrix, then Likelihood's
// dpptrf/dpptri in FP64 (source/c_matrix_generator.cpp:164-232,
// source/likelihood.cpp:69-180).  On GB300 FP64 runs at ~1/64 of FP32, so
// this path keeps FP64 only where the ill-conditioning of C needs it:
//
//   reference point (FP64, once per re-centre):
//     Cref = C(cl_ref) + N = Lref Lref^T,  Mref = Lref^-1,  ln det Cref
//     Y    = real spherical harmonics x B_l at the pixels (sum_m Y_lm Y_lm^T
//            = (2l+1)/(4pi) B_l^2 P_l(x), the addition theorem)
//     Z    = Mref Y,  Ubar_l = cref_l Z_l Z_l^T   (whitened Legendre table,
//            stored FP32 as [tile][entry][l])
//     y    = Mref d
//   per batch element b (FP32 O(n^3), FP64 accumulations):
//     eps_bl = C_bl / cref_l - 1
//     A_b = I + K_b,  K_b = sum_l eps_bl Ubar_l   (= Lref^-1 (C_b - Cref) Lref^-T)
//         -- the [pairs x l] x [l x batch] contraction
//     A_b = L_b L_b^T (FP32), V_b = A_b^-1 (FP32)
//     ln det C_b = ln det Cref + 2 sum ln diag(L_b)           (FP64 sum)
//     x_b = V_b y, one refinement step r = y - A_b x_b, x_b += V_b r (FP64)
//     chi2_b = y^T x_b
//     d(-2lnL)/dC_l = sum_ij (V_b - x_b x_b^T)_ij Ubar_l,ij / cref_l
//         -- the transposed contraction against the same table.
// A_b is well conditioned (eigenvalues in [min_l C_bl/cref_l, max_l C_bl/cref_l]),
// which is what makes FP32 factors accurate to ~1e-6 in -2lnL.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cuda_bf16.h>

#include "cg_internal.h"
#include "cg_tc.cuh"
#include "cg_tile.cuh"

namespace cg {

using namespace tile;

namespace {

constexpr double kPi = 3.141592653589793;

inline int lpad_of(int lmax) { return ((lmax + 1 + 15) / 16) * 16; }
inline int nharm_of(int lmax) { return (lmax + 1) * (lmax + 1) - 4; }  // l = 2..lmax
inline int nharm_pad(int lmax) { return ((nharm_of(lmax) + TS - 1) / TS) * TS; }

// Real orthonormal spherical harmonics times B_l at every pixel, rows h =
// (l^2 - 4) + {0: m=0, 2m-1: cos, 2m: sin}; normalised associated Legendre
// functions by the standard three-term recurrence in l at fixed m.
__global__ void ylm_basis(int n, int N, int lmax, const double* __restrict__ xyz, const double* __restrict__ beam,
                          double* __restrict__ Y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (i >= N) return;
    const bool real = i < n;
    double x = 0, sth = 0, phi = 0;
    if (real) {
        const double px = xyz[i], py = xyz[N + i], pz = xyz[2 * N + i];
        x = pz;
        sth = sqrt(px * px + py * py);
        phi = atan2(py, px);
    }
    double pmm = 1.0 / sqrt(4.0 * kPi);  // Pbar_0^0
    for (int k = 1; k <= m; ++k) pmm *= -sqrt((2.0 * k + 1.0) / (2.0 * k)) * sth;
    double sm, cm;
    sincos((double)m * phi, &sm, &cm);
    const double fac = (m == 0) ? 1.0 : sqrt(2.0);
    double p2 = 0.0, p1 = pmm;  // P_{l-2}, P_{l-1}
    for (int l = m; l <= lmax; ++l) {
        double p;
        if (l == m) p = pmm;
        else if (l == m + 1) p = sqrt(2.0 * m + 3.0) * x * pmm;
        else {
            const double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            const double bb = sqrt(((double)(l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
            p = a * (x * p1 - bb * p2);
        }
        if (l > m) { p2 = p1; p1 = p; }
        if (l >= 2) {
            const int base = l * l - 4;
            const double v = real ? fac * p * beam[l] : 0.0;
            if (m == 0) Y[(size_t)base * N + i] = v;
            else {
                Y[(size_t)(base + 2 * m - 1) * N + i] = v * cm;
                Y[(size_t)(base + 2 * m) * N + i] = v * sm;
            }
        }
    }
}

// Z[h][I-block] = sum_{J <= I} Mref_IJ Y[h][J-block]; grid (nt, nharm_pad / TS)
__global__ void __launch_bounds__(256) whiten_basis(int nt, int N, const double* __restrict__ Mref,
                                                    const double* __restrict__ Y, double* __restrict__ Z)
{
    extern __shared__ unsigned char smem_raw[];
    constexpr int L = SmemLd<double>::v;
    double* sX = reinterpret_cast<double*>(smem_raw);
    double* sY = sX + TS * L;
    const int I = blockIdx.x, H = blockIdx.y;
    int r0, c0;
    micro_coords(r0, c0);
    double acc[4][4] = {};
    for (int J = 0; J <= I; ++J) {
        load_direct(sX, Mref + (size_t)tile_index(I, J) * TILE_ELEMS);
        for (int e = threadIdx.x; e < TILE_ELEMS; e += blockDim.x) {
            const int m = e % TS, c = e / TS;  // sY[m][c] = Y[H*TS + c][J*TS + m]
            sY[m * L + c] = Y[(size_t)(H * TS + c) * N + J * TS + m];
        }
        __syncthreads();
        tile_mma(sX, sY, acc, r0, c0);
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) Z[(size_t)(H * TS + c0 + q) * N + I * TS + r0 + a] = acc[a][q];
}

// Ubar[t][e][l] = cref_l sum_{h in l} Z[h][i] Z[h][j] (FP64 sums, FP32 store);
// grid (tiles, TS / CC): each block covers CC columns (CC*TS entries) of one tile.
template <int CC>
__global__ void __launch_bounds__(256) build_ubar(int N, int lmax, int lp, const double* __restrict__ Z,
                                                  const double* __restrict__ cref, float* __restrict__ U)
{
    extern __shared__ unsigned char smem_raw[];
    constexpr int HB = 32;                                   // harmonics per sub-batch
    double* zi = reinterpret_cast<double*>(smem_raw);        // [HB][TS]
    double* zj = zi + HB * TS;                               // [HB][CC]
    float* out = reinterpret_cast<float*>(zj + HB * CC);     // [lp][CC*TS]
    int I, J;
    tile_coords(blockIdx.x, I, J);
    const int c_begin = blockIdx.y * CC;
    constexpr int NE = CC * TS;                              // entries in this block
    constexpr int PER = NE / 256;                            // entries per thread
    for (int k = threadIdx.x; k < NE * lp; k += blockDim.x) out[k] = 0.f;
    __syncthreads();
    for (int l = 2; l <= lmax; ++l) {
        const int h0 = l * l - 4, h1 = (l + 1) * (l + 1) - 4;
        double acc[PER];
#pragma unroll
        for (int p = 0; p < PER; ++p) acc[p] = 0.0;
        for (int hb = h0; hb < h1; hb += HB) {
            const int nh = min(HB, h1 - hb);
            for (int k = threadIdx.x; k < nh * TS; k += blockDim.x)
                zi[k] = Z[(size_t)(hb + k / TS) * N + I * TS + k % TS];
            for (int k = threadIdx.x; k < nh * CC; k += blockDim.x)
                zj[k] = Z[(size_t)(hb + k / CC) * N + J * TS + c_begin + k % CC];
            __syncthreads();
#pragma unroll
            for (int p = 0; p < PER; ++p) {
                const int e = threadIdx.x + 256 * p;  // e = r + TS * cc
                const int r = e % TS, cc = e / TS;
                double s = acc[p];
                for (int h = 0; h < nh; ++h) s += zi[h * TS + r] * zj[h * CC + cc];
                acc[p] = s;
            }
            __syncthreads();
        }
#pragma unroll
        for (int p = 0; p < PER; ++p) out[l * NE + threadIdx.x + 256 * p] = (float)(cref[l] * acc[p]);
    }
    __syncthreads();
    // table layout [tile][l][entry]: each l row of this block's entries is contiguous
    float* dst = U + (size_t)blockIdx.x * TILE_ELEMS * lp + (size_t)c_begin * TS;
    for (int k = threadIdx.x; k < NE * lp; k += blockDim.x) dst[(size_t)(k / NE) * TILE_ELEMS + k % NE] = out[k];
}

// y = M d for the lower-triangular tiled FP64 M, one CTA per tile (I, J <= I) and map:
// part[t][r] = (M_IJ d_J)[r] (four partial sums per row, fixed order), then trmv_reduce sums the
// row's tiles in order.  One CTA per tile spreads the FP64 products over every SM (a CTA per row
// block left 40 SMs to do them at this GPU's FP64 rate).
__global__ void __launch_bounds__(256) trmv_partials(int nt, int n, const double* __restrict__ M,
                                                     const double* __restrict__ d, int d_stride,
                                                     double* __restrict__ part)
{
    __shared__ double red[4][TS];
    const int t = blockIdx.x, b = blockIdx.y, ntile = ntiles_lower(nt);
    int I, J;
    tile_coords(t, I, J);
    const int r = threadIdx.x % TS, q = threadIdx.x / TS;
    const double* tl = M + (size_t)t * TILE_ELEMS;
    const double* db = d + (size_t)b * d_stride;
    double s = 0.0;
    for (int c = q; c < TS; c += 4) {
        const int j = J * TS + c;
        if (j < n) s = fma(tl[r + TS * c], db[j], s);
    }
    red[q][r] = s;
    __syncthreads();
    if (q == 0) part[((size_t)b * ntile + t) * TS + r] = ((red[0][r] + red[1][r]) + red[2][r]) + red[3][r];
}

__global__ void __launch_bounds__(64) trmv_reduce(int nt, int N, const double* __restrict__ part,
                                                  double* __restrict__ y)
{
    const int I = blockIdx.x, b = blockIdx.y, r = threadIdx.x, ntile = ntiles_lower(nt);
    const double* pb = part + (size_t)b * ntile * TS;
    double s = 0.0;
    for (int J = 0; J <= I; ++J) s += pb[(size_t)tile_index(I, J) * TS + r];
    y[(size_t)b * N + I * TS + r] = s;
}

// eps[l][b] = C_bl / cref_l - 1 (0 for l < 2 and padding)
__global__ void make_eps(int B, int lmax, int lp, const double* __restrict__ cl, const double* __restrict__ cref,
                         float* __restrict__ eps)
{
    const int b = blockIdx.x;
    for (int l = threadIdx.x; l < lp; l += blockDim.x) {
        float v = 0.f;
        if (l >= 2 && l <= lmax) {
            const double c = cl[(size_t)b * (lmax + 1) + l];
            v = (float)(c / cref[l] - 1.0);
        }
        eps[(size_t)l * B + b] = v;  // [l][b]: the contraction stages a row of batch elements per l
    }
}

__global__ void init_status(int B, const double* __restrict__ cl, int lmax, int* __restrict__ status)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    int st = CG_OK;
    for (int l = 0; l <= lmax; ++l)
        if (!isfinite(cl[(size_t)b * (lmax + 1) + l])) st = CG_ERR_NONFINITE;
    status[b] = st;
}

// Forward contraction: A_b[t][e] = [e on the diagonal] + sum_l Ubar[t][l][e] eps[l][b], written
// to A.  A CTA covers BB batch elements and FWD_NBLK consecutive blocks of EB = 16384 / BB entries
// (blocks never straddle a tile); thread (te, tb) computes 8 entries x 8 batch elements: entries
// 4 te .. 4 te + 3 and EB/2 + 4 te .. + 3, so that the threads of a warp read 16-byte pieces that
// are 16 bytes apart (conflict-free 128-bit shared-memory loads; 8-entry runs 32 bytes apart were a
// two-way conflict on every load, which made the loop shared-memory bound).  Rows l = 0, 1 are zero
// in the table and in eps (C_0, C_1 do not enter) and are skipped.  The
// next block's table rows (lp rows of EB floats, 4096 floats apart) arrive by bulk copies into a
// double buffer while the current block is computed; eps is staged once.  A bounded wait that
// gives up sets *err (reported as CG_ERR_TIMEOUT).
// grid (tiles * TILE_ELEMS / (EB * FWD_NBLK), ceil(B / BB)).
constexpr int FWD_NBLK = 8;
template <int BB>
__global__ void __launch_bounds__(256) contract_fwd(int B, int lp, const float* __restrict__ U,
                                                    const float* __restrict__ eps, float* __restrict__ A,
                                                    size_t strideA, int* __restrict__ err)
{
    constexpr int EB = 128 * 128 / BB, TE = EB / 8;  // entries per block, threads along entries
    extern __shared__ __align__(128) float fsm[];
    float* sE = fsm;                       // [lp][BB]
    float* sU = fsm + lp * BB;             // [2][lp][EB]
    __shared__ uint64_t full[2];
    const int b_begin = blockIdx.y * BB;
    const size_t blk0 = (size_t)blockIdx.x * FWD_NBLK;  // first entry block of this CTA
    const uint32_t bytes = (uint32_t)(lp * EB * sizeof(float));
    auto issue = [&](int i) {  // table rows of block blk0 + i into buffer i & 1 (thread 0)
        const size_t e_begin = (blk0 + i) * EB;
        const float* src = U + (e_begin / TILE_ELEMS) * TILE_ELEMS * lp + e_begin % TILE_ELEMS;
        float* dst = sU + (i & 1) * lp * EB;
        tc::mbar_arrive_expect_tx(&full[i & 1], bytes);
        for (int l = 0; l < lp; ++l)
            tc::bulk_g2s(tc::smem_u32(dst + l * EB), src + (size_t)l * TILE_ELEMS, EB * sizeof(float), &full[i & 1]);
    };
    if (threadIdx.x == 0) {
        tc::mbar_init(&full[0], 1);
        tc::mbar_init(&full[1], 1);
        tc::fence_mbar_init();
        issue(0);
        issue(1);
    }
    for (int k = threadIdx.x; k < lp * BB; k += 256) {
        const int l = k / BB, bb = k % BB, b = b_begin + bb;
        sE[l * BB + bb] = (b < B) ? eps[(size_t)l * B + b] : 0.f;
    }
    __syncthreads();
    const int te = threadIdx.x % TE, tb = threadIdx.x / TE;
    const int e0 = te * 4, e1 = EB / 2 + te * 4, b0 = tb * 8;
    bool ok = true;
    for (int i = 0; i < FWD_NBLK; ++i) {
        if (ok && !tc::mbar_wait(&full[i & 1], (i >> 1) & 1, 1u << 22, err)) {
            ok = false;
            atomicExch(err, 1);
        }
        const float* bu = sU + (i & 1) * lp * EB;
        float acc[8][8];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[a][q] = 0.f;
        if (b_begin + b0 < B) {
#pragma unroll 2
            for (int l = 2; l < lp; ++l) {
                const float4 u0 = *reinterpret_cast<const float4*>(&bu[l * EB + e0]);
                const float4 u1 = *reinterpret_cast<const float4*>(&bu[l * EB + e1]);
                const float4 w0 = *reinterpret_cast<const float4*>(&sE[l * BB + b0]);
                const float4 w1 = *reinterpret_cast<const float4*>(&sE[l * BB + b0 + 4]);
                const float u[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
                const float w[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
                for (int a = 0; a < 8; ++a)
#pragma unroll
                    for (int q = 0; q < 8; q += 2) tc::fma2(acc[a][q], acc[a][q + 1], u[a], u[a], w[q], w[q + 1]);
            }
        }
        __syncthreads();  // buffer i & 1 is read: refill it with block i + 2
        if (threadIdx.x == 0 && i + 2 < FWD_NBLK) issue(i + 2);
        const size_t e_begin = (blk0 + i) * EB;
        int I, J;
        tile_coords((int)(e_begin / TILE_ELEMS), I, J);
        const int eoff = (int)(e_begin % TILE_ELEMS);  // the block's entry offset within the tile
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int bb = b_begin + b0 + q;
            if (bb >= B) continue;
            float v[8];
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                const int e = eoff + (a < 4 ? e0 + a : e1 + a - 4);
                const bool dg = (I == J) && (e % TS == e / TS);
                v[a] = acc[a][q] + (dg ? 1.f : 0.f);
            }
            float* pb = A + (size_t)bb * strideA + e_begin;
            *reinterpret_cast<float4*>(pb + e0) = make_float4(v[0], v[1], v[2], v[3]);
            *reinterpret_cast<float4*>(pb + e1) = make_float4(v[4], v[5], v[6], v[7]);
        }
    }
}

// ln det C_b = ln det Cref + 2 sum ln diag(L_b), FP64 sums; grid B
__global__ void __launch_bounds__(256) logdet_mixed(int n, int N, const float* __restrict__ diag,
                                                    const double* __restrict__ logdet_ref, double* __restrict__ out)
{
    __shared__ double red[256];
    const int b = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += log((double)diag[(size_t)b * N + i]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[b] = *logdet_ref + 2.0 * red[0];
}

// chi2_b = y_b . x_b, m2lnl_b = chi2_b + logdet_b; grid B
__global__ void __launch_bounds__(256) chi2_mixed(int n, int N, int ystride, const double* __restrict__ y,
                                                  const double* __restrict__ x, const double* __restrict__ logdet,
                                                  double* __restrict__ m2lnl, double* __restrict__ chi2,
                                                  double* __restrict__ logdet_out)
{
    __shared__ double red[256];
    const int b = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += y[(size_t)b * ystride + i] * x[(size_t)b * N + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (chi2) chi2[b] = red[0];
        if (logdet_out) logdet_out[b] = logdet[b];
        m2lnl[b] = red[0] + logdet[b];
    }
}

// a tensor-core kernel whose bounded wait gave up marks every element of the batch
__global__ void merge_tc_status(int B, int* __restrict__ err, int* __restrict__ status)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B && *err) status[b] = CG_ERR_TIMEOUT;
}

// broadcast y (one map) to every batch element: yb[b][i] = y[i]
__global__ void broadcast_vec(int B, int N, const double* __restrict__ y, double* __restrict__ yb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (i < N && b < B) yb[(size_t)b * N + i] = y[i];
}

// Adjoint gradient, d(-2lnL)/dC_l = tr((V - x x^T) Ubar_l) / cref_l, in two parts:
//   tr(V Ubar_l)   = sum over stored entries e of w_e V[e] Ubar[e][l], w_e = 2 below the
//                    diagonal, 1 on it, 0 above it (the tiles hold the lower triangle);
//   x^T Ubar_l x   = cref_l |Z_l^T x|^2, Ubar_l = cref_l Z_l Z_l^T (Z_l: the 2l+1 rows of Z).

// part[t][b][l] = sum_{e in tile t} w_e V_b[t][e] Ubar[t][l][e]: one CTA per tile and 32 NA batch
// elements (the tile's table block is read once per 48 l); grid (tiles, ceil(B / (32 NA)),
// ceil(lp / 48)).  Thread (bg = t % 32, lg = t / 32) holds batch elements bg + 32 a (a < NA) and
// l = lbase + 6 lg .. + 5.  NA = 8 for large batches, 2 when B <= 64.  V chunks are staged [b][entry] with row
// stride ADJ_LD (16-byte rows; the 8 lanes of each 128-bit phase hit different banks).
constexpr int ADJ_KE = 64;       // entries per chunk
constexpr int ADJ_LD = ADJ_KE + 4;
template <int NA>
__global__ void __launch_bounds__(256, 2) contract_adj(int B, int lp, const float* __restrict__ U,
                                                       const float* __restrict__ V, size_t strideA,
                                                       float* __restrict__ part)
{
    extern __shared__ float asm_[];
    float* sV = asm_;                      // [32 NA][ADJ_LD]
    float* sU = asm_ + 32 * NA * ADJ_LD;   // [48][ADJ_KE]
    const int t = blockIdx.x, b_begin = blockIdx.y * 32 * NA, lbase = 48 * blockIdx.z;
    int I, J;
    tile_coords(t, I, J);
    const int bg = threadIdx.x % 32, lg = threadIdx.x / 32, l0 = 6 * lg;
    float acc[NA][6];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int q = 0; q < 6; ++q) acc[a][q] = 0.f;
    const float* Ut = U + (size_t)t * TILE_ELEMS * lp;
    // batch rows present; staging skips the 32-row groups beyond them (their sums are never stored)
    const int nrow = min(32 * NA, B - b_begin), na = (nrow + 31) / 32;
    for (int e0 = 0; e0 < TILE_ELEMS; e0 += ADJ_KE) {
        __syncthreads();
        // V: up to 256 rows x 64 entries, 16 threads per row (coalesced), weights applied
        for (int k = threadIdx.x; k < 32 * na * (ADJ_KE / 4); k += 256) {
            const int bb = k / (ADJ_KE / 4), e4 = k % (ADJ_KE / 4), b = b_begin + bb;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (b < B) {
                v = __ldg(reinterpret_cast<const float4*>(V + (size_t)b * strideA + (size_t)t * TILE_ELEMS + e0 + 4 * e4));
                float w[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int ee = e0 + 4 * e4 + i, r = ee % TS, c = ee / TS;
                    w[i] = (I != J || r > c) ? 2.f : (r == c ? 1.f : 0.f);
                }
                v = make_float4(w[0] * v.x, w[1] * v.y, w[2] * v.z, w[3] * v.w);
            }
            *reinterpret_cast<float4*>(&sV[bb * ADJ_LD + 4 * e4]) = v;
        }
        // table: 48 l rows x 64 entries (rows contiguous in the [tile][l][entry] layout)
        for (int k = threadIdx.x; k < 48 * (ADJ_KE / 4); k += 256) {
            const int l = k / (ADJ_KE / 4), e4 = k % (ADJ_KE / 4);
            float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lbase + l < lp)
                u = __ldg(reinterpret_cast<const float4*>(Ut + (size_t)(lbase + l) * TILE_ELEMS + e0 + 4 * e4));
            *reinterpret_cast<float4*>(&sU[l * ADJ_KE + 4 * e4]) = u;
        }
        __syncthreads();
#pragma unroll 2
        for (int e4 = 0; e4 < ADJ_KE / 4; ++e4) {
            float4 v[NA], u4[6];
#pragma unroll
            for (int a = 0; a < NA; ++a) v[a] = *reinterpret_cast<const float4*>(&sV[(bg + 32 * a) * ADJ_LD + 4 * e4]);
#pragma unroll
            for (int q = 0; q < 6; ++q) u4[q] = *reinterpret_cast<const float4*>(&sU[(l0 + q) * ADJ_KE + 4 * e4]);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                    const float va = (j == 0) ? v[a].x : (j == 1) ? v[a].y : (j == 2) ? v[a].z : v[a].w;
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const float uq = (j == 0) ? u4[q].x : (j == 1) ? u4[q].y : (j == 2) ? u4[q].z : u4[q].w;
                        acc[a][q] = fmaf(va, uq, acc[a][q]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const int b = b_begin + bg + 32 * a;
        if (b >= B) continue;
#pragma unroll
        for (int q = 0; q < 6; ++q)
            if (lbase + l0 + q < lp) part[((size_t)t * B + b) * lp + lbase + l0 + q] = acc[a][q];
    }
}

// proj[b][h] = sum_i Z[h][i] x_b[i] (FP32); 64 x 64 output per CTA, 4 x 4 per thread;
// grid (nharm_pad / 64, ceil(B / 64))
// Z^T x_b in K slices: slice z = blockIdx.z covers pixels [z ks, (z + 1) ks) and writes
// proj_part[z][b][h]; project_reduce sums the slices in order (deterministic).  One 64 x 64 output
// tile per CTA over all N pixels gave only nhp / 64 x B / 64 CTAs (144 at the benchmark point, fewer
// than the SMs), each walking 80 K steps alone.
constexpr int PROJ_KSPLIT = 4;
__global__ void __launch_bounds__(256) project_x(int B, int N, int nhp, int ks, const float* __restrict__ Zf,
                                                 const double* __restrict__ x, float* __restrict__ proj_part)
{
    __shared__ float sx[64][33], sz[64][33];
    const int h_begin = blockIdx.x * 64, b_begin = blockIdx.y * 64;
    const int th = threadIdx.x % 16, tb = threadIdx.x / 16;
    const int kb = blockIdx.z * ks, ke = min(N, kb + ks);
    float acc[4][4] = {};
    for (int k0 = kb; k0 < ke; k0 += 32) {
        __syncthreads();
        for (int k = threadIdx.x; k < 64 * 32; k += 256) {
            const int row = k / 32, kk = k % 32, b = b_begin + row;
            sx[row][kk] = (b < B && k0 + kk < ke) ? (float)x[(size_t)b * N + k0 + kk] : 0.f;
            sz[row][kk] = (k0 + kk < ke) ? Zf[(size_t)(h_begin + row) * N + k0 + kk] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; ++kk) {
            float xv[4], zv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) { xv[i] = sx[tb + 16 * i][kk]; zv[i] = sz[th + 16 * i][kk]; }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(xv[i], zv[j], acc[i][j]);
        }
    }
    float* out = proj_part + (size_t)blockIdx.z * B * nhp;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int b = b_begin + tb + 16 * i;
        if (b >= B) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) out[(size_t)b * nhp + h_begin + th + 16 * j] = acc[i][j];
    }
}

__global__ void project_reduce(size_t n, const float* __restrict__ part, float* __restrict__ proj)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = part[i];
#pragma unroll
        for (int z = 1; z < PROJ_KSPLIT; ++z) v += part[(size_t)z * n + i];
        proj[i] = v;
    }
}

// grad_bl = (sum over tiles of part) / cref_l - sum_{h in l} proj_bh^2, with the rows of Z for l
// at h = l^2 - 4 .. l^2 + 2l - 4; grid B.  The tile sums are
// double-float in FP32, four threads per l over interleaved tiles merged in a fixed order, and
// converted to FP64 once: summing 820 partials per l in FP64 ran at this GPU's FP64 rate.
__global__ void __launch_bounds__(256) adj_finish(int B, int ntile, int lmax, int lp, int nhp,
                                                  const float* __restrict__ part, const float* __restrict__ proj,
                                                  const double* __restrict__ cref, double* __restrict__ grad)
{
    __shared__ float sh[4][64], sl[4][64];
    const int b = blockIdx.x, li = threadIdx.x % 64, ch = threadIdx.x / 64;
    for (int base = 0; base <= lmax; base += 64) {
        const int l = base + li;
        float h = 0.f, lo = 0.f;
        if (l >= 2 && l <= lmax)
            for (int t = ch; t < ntile; t += 4) df_add(h, lo, part[((size_t)t * B + b) * lp + l]);
        sh[ch][li] = h;
        sl[ch][li] = lo;
        __syncthreads();
        if (ch == 0 && l <= lmax) {
            double g = 0.0;
            if (l >= 2) {
#pragma unroll
                for (int k = 1; k < 4; ++k) df_merge(h, lo, sh[k][li], sl[k][li]);
                const double sum = (double)h + (double)lo;
                double xx = 0.0;
                for (int hh = l * l - 4; hh < (l + 1) * (l + 1) - 4; ++hh) {
                    const double p = (double)proj[(size_t)b * nhp + hh];
                    xx += p * p;
                }
                g = sum / cref[l] - xx;
            }
            grad[(size_t)b * (lmax + 1) + l] = g;
        }
        __syncthreads();
    }
}

// the table's values rounded to the nearest BF16 (round to nearest even), kept in FP32
__global__ void round_to_bf16(size_t n, float* __restrict__ u)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        u[i] = __bfloat162float(__float2bfloat16_rn(u[i]));
}

// Z in FP32
__global__ void to_f32(size_t n, const double* __restrict__ src, float* __restrict__ dst)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

template <typename T>
int dalloc(cg_ctx* ctx, T** p, size_t count)
{
    if (cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        ctx->err = "device allocation failed (mixed path workspace)";
        return CG_ERR_ALLOC;
    }
    return CG_OK;
}

}  // namespace

void mixed_free(cg_ctx* ctx)
{
    MixedWork& w = ctx->wmx;
    cudaFree(w.Lref); cudaFree(w.Mref); cudaFree(w.Dinv_ref); cudaFree(w.diag_ref); cudaFree(w.Y); cudaFree(w.Z);
    cudaFree(w.U); cudaFree(w.A); cudaFree(w.Ms); cudaFree(w.Linv); cudaFree(w.diag); cudaFree(w.eps); cudaFree(w.y);
    cudaFree(w.x); cudaFree(w.r); cudaFree(w.gpart); cudaFree(w.st); cudaFree(w.V); cudaFree(w.Ls); cudaFree(w.cref);
    cudaFree(w.ldref); cudaFree(w.part); cudaFree(w.ld); cudaFree(w.tcerr); cudaFree(w.Zf); cudaFree(w.proj);
    cudaFree(w.Lc); cudaFree(w.Mc);
    w = MixedWork();
}

// Device bytes of the mixed path: *fixed = the reference point's buffers and the whitened table
// (ensure_ref_bufs), *per_element = one batch element's workspace (ensure_batch_bufs), in their order
void mixed_bytes(const cg_ctx* ctx, size_t* fixed, size_t* per_element)
{
    const size_t tiled = tiled_elems(ctx->nt);
    const size_t N = (size_t)ctx->N, nt = (size_t)ctx->nt, lp = (size_t)lpad_of(ctx->lmax);
    const size_t nhp = (size_t)nharm_pad(ctx->lmax), ntile = (size_t)ntiles_lower(ctx->nt);
    *fixed = sizeof(double) * (2 * tiled + nt * TILE_ELEMS + N + 2 * nhp * N) + sizeof(float) * (tiled * lp + nhp * N) +
             sizeof(double) * ((size_t)ctx->lmax + 2) + sizeof(int) * (1 + (size_t)tc_queue_slots(ctx->nt));
    *per_element = sizeof(float) * (2 * tiled + 2 * tc_split_elems(ctx->nt) + tc_linv_elems(ctx->nt) +
                                    2 * tc_c1_elems(ctx->nt) + N + lp + ntile * lp + (1 + PROJ_KSPLIT) * nhp) +
                   sizeof(double) * (3 * N + ntile * 2 * TS + 1) + sizeof(int);
}

static int ensure_ref_bufs(cg_ctx* ctx)
{
    MixedWork& w = ctx->wmx;
    if (w.Lref) return CG_OK;
    const size_t tiled = tiled_elems(ctx->nt);
    const int N = ctx->N, nt = ctx->nt, lp = lpad_of(ctx->lmax), nhp = nharm_pad(ctx->lmax);
    int rc = dalloc(ctx, &w.Lref, tiled);
    if (!rc) rc = dalloc(ctx, &w.Mref, tiled);
    if (!rc) rc = dalloc(ctx, &w.Dinv_ref, (size_t)nt * TILE_ELEMS);
    if (!rc) rc = dalloc(ctx, &w.diag_ref, (size_t)N);
    if (!rc) rc = dalloc(ctx, &w.Y, (size_t)nhp * N);
    if (!rc) rc = dalloc(ctx, &w.Z, (size_t)nhp * N);
    if (!rc) rc = dalloc(ctx, &w.U, tiled * lp);
    if (!rc) rc = dalloc(ctx, &w.Zf, (size_t)nhp * N);
    if (!rc) rc = dalloc(ctx, &w.cref, (size_t)ctx->lmax + 1);
    if (!rc) rc = dalloc(ctx, &w.ldref, 1);
    if (!rc) rc = dalloc(ctx, &w.tcerr, 1 + (size_t)tc_queue_slots(nt));
    if (!rc) CG_CUDA_TRY(ctx, cudaMemset(w.tcerr, 0, sizeof(int) * (1 + tc_queue_slots(nt))));
    if (rc) { mixed_free(ctx); return rc; }
    w.lpad = lp;
    return CG_OK;
}

static int ensure_batch_bufs(cg_ctx* ctx, int B)
{
    MixedWork& w = ctx->wmx;
    if (w.cap >= B) return CG_OK;
    ++ctx->epoch;  // a captured call refers to the buffers freed below
    cudaFree(w.A); cudaFree(w.V); cudaFree(w.Ls); cudaFree(w.Ms); cudaFree(w.Linv); cudaFree(w.diag); cudaFree(w.eps);
    cudaFree(w.y); cudaFree(w.x); cudaFree(w.r); cudaFree(w.part); cudaFree(w.gpart); cudaFree(w.st); cudaFree(w.ld);
    cudaFree(w.proj); cudaFree(w.Lc); cudaFree(w.Mc);
    w.A = w.V = w.Ls = w.Ms = w.Linv = w.diag = w.eps = w.gpart = w.proj = w.Lc = w.Mc = nullptr;
    w.y = w.x = w.r = w.part = w.ld = nullptr;
    w.st = nullptr;
    w.cap = 0;
    const size_t tiled = tiled_elems(ctx->nt);
    const int N = ctx->N, nt = ctx->nt, lp = lpad_of(ctx->lmax), ntile = ntiles_lower(nt);
    int rc = dalloc(ctx, &w.A, tiled * B);
    if (!rc) rc = dalloc(ctx, &w.V, tiled * B);
    if (!rc) rc = dalloc(ctx, &w.Ls, tc_split_elems(nt) * B);
    if (!rc) rc = dalloc(ctx, &w.Ms, tc_split_elems(nt) * B);
    if (!rc) rc = dalloc(ctx, &w.Linv, tc_linv_elems(nt) * B);
    if (!rc) rc = dalloc(ctx, &w.Lc, tc_c1_elems(nt) * B);
    if (!rc) rc = dalloc(ctx, &w.Mc, tc_c1_elems(nt) * B);
    if (!rc) rc = dalloc(ctx, &w.diag, (size_t)B * N);
    if (!rc) rc = dalloc(ctx, &w.eps, (size_t)B * lp);
    if (!rc) rc = dalloc(ctx, &w.y, (size_t)B * N);
    if (!rc) rc = dalloc(ctx, &w.x, (size_t)B * N);
    if (!rc) rc = dalloc(ctx, &w.r, (size_t)B * N);
    if (!rc) rc = dalloc(ctx, &w.part, (size_t)B * ntile * 2 * TS);
    if (!rc) rc = dalloc(ctx, &w.gpart, (size_t)ntile * B * lp);
    if (!rc) rc = dalloc(ctx, &w.proj, (size_t)(1 + PROJ_KSPLIT) * B * nharm_pad(ctx->lmax));  // + K-slice partials
    if (!rc) rc = dalloc(ctx, &w.st, (size_t)B);
    if (!rc) rc = dalloc(ctx, &w.ld, (size_t)B);
    if (rc) return rc;
    w.cap = B;
    return CG_OK;
}

int mixed_ensure(cg_ctx* ctx, int B) { return ensure_batch_bufs(ctx, B); }

int mixed_prepare_reference(cg_ctx* ctx, const double* cl_ref_host)
{
    int rc = ensure_ref_bufs(ctx);
    if (rc) return rc;
    MixedWork& w = ctx->wmx;
    const int nt = ctx->nt, N = ctx->N, n = ctx->n, lmax = ctx->lmax, lp = w.lpad;
    const size_t tiled = tiled_elems(nt);
    for (int l = 2; l <= lmax; ++l)
        if (!(cl_ref_host[l] > 0) || !std::isfinite(cl_ref_host[l])) {
            ctx->err = "reference C_l must be positive and finite for l >= 2";
            return CG_ERR_BAD_ARG;
        }
    cudaStream_t s = ctx->stream;
    w.cl_ref.assign(cl_ref_host, cl_ref_host + lmax + 1);
    CG_CUDA_TRY(ctx, cudaMemcpyAsync(w.cref, cl_ref_host, sizeof(double) * (lmax + 1), cudaMemcpyHostToDevice, s));
    // Cref = C(cl_ref) + N in FP64, factor and invert the factor
    if ((rc = fp64_build_tiled_into(ctx, 1, w.cref, true, w.Lref, s))) return rc;
    int* st = nullptr;
    if ((rc = dalloc(ctx, &st, 1))) return rc;
    cudaMemsetAsync(st, 0, sizeof(int), s);
    rc = tiled_cholesky<double>(ctx, 1, nt, w.Lref, w.Dinv_ref, w.diag_ref, st, tiled, s);
    if (!rc) rc = tiled_trtri<double>(ctx, 1, nt, w.Lref, w.Dinv_ref, w.Mref, tiled, s);
    int hst = 0;
    if (!rc) {
        fp64_logdet(1, n, N, w.diag_ref, w.ldref, s);
        cudaMemcpyAsync(&hst, st, sizeof(int), cudaMemcpyDeviceToHost, s);
    }
    // whitened harmonic basis and table
    const int nhp = nharm_pad(lmax);
    if (!rc) {
        CG_CUDA_TRY(ctx, cudaMemsetAsync(w.Y, 0, sizeof(double) * (size_t)nhp * N, s));
        ylm_basis<<<dim3((N + 127) / 128, lmax + 1), 128, 0, s>>>(n, N, lmax, ctx->d_xyz, ctx->d_beam, w.Y);
        const size_t smz = 2 * (size_t)TS * SmemLd<double>::v * sizeof(double);
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(whiten_basis, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz));
        whiten_basis<<<dim3(nt, nhp / TS), 256, smz, s>>>(nt, N, w.Mref, w.Y, w.Z);
        to_f32<<<1024, 256, 0, s>>>((size_t)nhp * N, w.Z, w.Zf);
        if (lp <= 48) {
            constexpr int CC = 8;
            const size_t smu = sizeof(double) * 32 * (TS + CC) + sizeof(float) * (size_t)CC * TS * lp;
            CG_CUDA_TRY(ctx, cudaFuncSetAttribute(build_ubar<CC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smu));
            build_ubar<CC><<<dim3(ntiles_lower(nt), TS / CC), 256, smu, s>>>(N, lmax, lp, w.Z, w.cref, w.U);
        } else {
            constexpr int CC = 4;
            const size_t smu = sizeof(double) * 32 * (TS + CC) + sizeof(float) * (size_t)CC * TS * lp;
            CG_CUDA_TRY(ctx, cudaFuncSetAttribute(build_ubar<CC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smu));
            build_ubar<CC><<<dim3(ntiles_lower(nt), TS / CC), 256, smu, s>>>(N, lmax, lp, w.Z, w.cref, w.U);
        }
        if (ctx->tune.table_bf16) round_to_bf16<<<1024, 256, 0, s>>>(tiled * lp, w.U);
        CG_CUDA_TRY(ctx, cudaGetLastError());
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    }
    cudaFree(st);
    if (!rc && hst) {
        ctx->err = "reference covariance is not positive definite";
        rc = CG_ERR_NOT_PD;
    }
    if (rc) { w.have_ref = false; return rc; }
    w.have_ref = true;
    ++w.ref_count;
    return CG_OK;
}

static void geometric_mean(int B, int lmax, const double* cl, std::vector<double>& out)
{
    out.assign(lmax + 1, 0.0);
    for (int l = 2; l <= lmax; ++l) {
        double s = 0.0;
        int cnt = 0;
        for (int b = 0; b < B; ++b) {
            const double v = cl[(size_t)b * (lmax + 1) + l];
            if (v > 0 && std::isfinite(v)) { s += std::log(v); ++cnt; }
        }
        out[l] = cnt ? std::exp(s / cnt) : 1.0;
    }
}

int mixed_loglike(cg_ctx* ctx, int B, const double* d_cl, const double* h_cl, const double* d_d, int d_stride,
                  double* d_m2lnl, double* d_chi2, double* d_logdet, double* d_grad, int* d_status, cudaStream_t s)
{
    MixedWork& w = ctx->wmx;
    const int nt = ctx->nt, N = ctx->N, n = ctx->n, lmax = ctx->lmax;
    int rc = ensure_batch_bufs(ctx, B);
    if (rc) return rc;
    // decide the reference point on the host
    std::vector<double> hcl;
    const bool need_host = !w.have_ref || ctx->recenter != CG_RECENTER_FIXED;
    if (need_host && !h_cl) {
        hcl.resize((size_t)B * (lmax + 1));
        CG_CUDA_TRY(ctx, cudaMemcpyAsync(hcl.data(), d_cl, sizeof(double) * hcl.size(), cudaMemcpyDeviceToHost, s));
        CG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        h_cl = hcl.data();
    }
    if (need_host) {
        bool recentre = !w.have_ref || ctx->recenter == CG_RECENTER_BATCH;
        if (!recentre) {
            double dev = 0.0;
            for (int b = 0; b < B; ++b)
                for (int l = 2; l <= lmax; ++l) {
                    const double v = h_cl[(size_t)b * (lmax + 1) + l];
                    if (v > 0 && std::isfinite(v)) dev = std::max(dev, std::fabs(std::log(v / w.cl_ref[l])));
                }
            recentre = dev > ctx->recenter_radius;
        }
        if (recentre) {
            std::vector<double> gm;
            geometric_mean(B, lmax, h_cl, gm);
            if ((rc = mixed_prepare_reference(ctx, gm.data()))) return rc;
        }
    }
    const int lp = w.lpad, ntile = ntiles_lower(nt);
    const size_t tiled = tiled_elems(nt);
    stage_mark(ctx, ST_BUILD, s);
    // a timeout reports on its own call only; the work queues start empty
    CG_CUDA_TRY(ctx, cudaMemsetAsync(w.tcerr, 0, sizeof(int) * (1 + tc_queue_slots(nt)), s));
    init_status<<<(B + 127) / 128, 128, 0, s>>>(B, d_cl, lmax, w.st);
    make_eps<<<B, 64, 0, s>>>(B, lmax, lp, d_cl, w.cref, w.eps);
    count_launch(ctx, d_stride == 0 ? 6 : 5);
    // y = Mref d: one map (broadcast) or one per element
    if (d_stride == 0) {
        trmv_partials<<<dim3(ntile, 1), 256, 0, s>>>(nt, n, w.Mref, d_d, 0, w.part);
        trmv_reduce<<<dim3(nt, 1), 64, 0, s>>>(nt, N, w.part, w.r);
        broadcast_vec<<<dim3((N + 255) / 256, B), 256, 0, s>>>(B, N, w.r, w.y);
    } else {
        trmv_partials<<<dim3(ntile, B), 256, 0, s>>>(nt, n, w.Mref, d_d, d_stride, w.part);
        trmv_reduce<<<dim3(nt, B), 64, 0, s>>>(nt, N, w.part, w.y);
    }
    // A_b = I + sum_l eps_bl Ubar_l; small batches use 32-element CTA tiles (more entries per block)
    // when the double-buffered table rows fit in shared memory
    // (64-element tiles where the 32-element tile's buffers do not fit, e.g. lp = 96)
    const size_t smem32 = sizeof(float) * lp * (32 + 2 * 512), smem128 = sizeof(float) * lp * (128 + 2 * 128);
    const size_t smem64 = sizeof(float) * lp * (64 + 2 * 256);
    if (ctx->tune.fwd == 1 && contract_fwd_tc_ok(lp)) {
        if ((rc = contract_fwd_tc_launch(ctx, B, nt, lp, w.U, w.eps, w.A, tiled, w.tcerr, ctx->tune.fwd_ctas, s)))
            return rc;
    } else if (B <= 48 && smem32 <= 200 * 1024) {
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(contract_fwd<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem32));
        contract_fwd<32><<<dim3((unsigned)(tiled / (512 * FWD_NBLK)), (B + 31) / 32), 256, smem32, s>>>(
            B, lp, w.U, w.eps, w.A, tiled, w.tcerr);
    } else if (B <= 64 && smem64 <= 224 * 1024) {
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(contract_fwd<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem64));
        contract_fwd<64><<<dim3((unsigned)(tiled / (256 * FWD_NBLK)), (B + 63) / 64), 256, smem64, s>>>(
            B, lp, w.U, w.eps, w.A, tiled, w.tcerr);
    } else {
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(contract_fwd<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem128));
        contract_fwd<128><<<dim3((unsigned)(tiled / (128 * FWD_NBLK)), (B + 127) / 128), 256, smem128, s>>>(
            B, lp, w.U, w.eps, w.A, tiled, w.tcerr);
    }
    stage_mark(ctx, ST_CHOL, s);
    if (ctx->tune.overlap && ctx->tune.trtri != 1) {
        // trtri's rows beside the Cholesky (which marks the trtri stage's start where it ends); the
        // work-queue trtri runs after it (beside it, one call in about three hundred gave results that
        // differed in the last bits)
        if ((rc = tiled_chol_trtri_tc(ctx, B, nt, w.A, w.Ls, w.Lc, w.Linv, w.Ms, w.Mc, w.diag, w.st, w.tcerr, s)))
            return rc;
        logdet_mixed<<<B, 256, 0, s>>>(n, N, w.diag, w.ldref, w.ld);
        count_launch(ctx);
    } else {
        if ((rc = tiled_cholesky_tc(ctx, B, nt, w.A, w.Ls, w.Lc, w.Linv, w.Ms, w.Mc, w.diag, w.st, w.tcerr, s)))
            return rc;
        logdet_mixed<<<B, 256, 0, s>>>(n, N, w.diag, w.ldref, w.ld);
        count_launch(ctx);
        stage_mark(ctx, ST_TRTRI, s);
        if ((rc = tiled_trtri_tc(ctx, B, nt, w.Ls, w.Linv, w.Ms, w.Mc, w.tcerr, s))) return rc;
    }
    // x = V y; r = y - A x; x += V r  (the partials buffer holds double-float pairs here); the first
    // pass's tile partials come from lauum's epilogue, which still holds each block of V in registers
    // (not from the work-queue lauum, whose epilogues run beside the next block's K loop)
    float2* pf = reinterpret_cast<float2*>(w.part);
    const bool fused = ctx->tune.lauum != 1;
    stage_mark(ctx, ST_LAUUM, s);
    if ((rc = tiled_lauum_tc(ctx, B, nt, w.Ms, w.Mc, w.V, w.tcerr, fused ? w.y : nullptr, N, pf, s))) return rc;
    stage_mark(ctx, ST_SOLVE, s);
    if (!fused) {
        symv_partials<false><<<dim3((ntile + SYMV_TPB - 1) / SYMV_TPB, B), 256, 0, s>>>(nt, w.V, tiled, w.y, N, pf);
        count_launch(ctx);
    }
    symv_reduce<<<dim3(nt, B), 64, 0, s>>>(nt, pf, w.x, N, nullptr, 1.0);
    symv_partials<true><<<dim3((ntile + SYMV_TPB - 1) / SYMV_TPB, B), 256, 0, s>>>(nt, w.A, tiled, w.x, N, pf);
    symv_reduce<<<dim3(nt, B), 64, 0, s>>>(nt, pf, w.r, N, w.y, -1.0);
    symv_partials<false><<<dim3((ntile + SYMV_TPB - 1) / SYMV_TPB, B), 256, 0, s>>>(nt, w.V, tiled, w.r, N, pf);
    symv_reduce<<<dim3(nt, B), 64, 0, s>>>(nt, pf, w.x, N, w.x, 1.0);
    chi2_mixed<<<B, 256, 0, s>>>(n, N, N, w.y, w.x, w.ld, d_m2lnl, d_chi2, d_logdet);
    count_launch(ctx, 6);
    stage_mark(ctx, ST_ADJOINT, s);
    if (d_grad) {
        if (adjoint_tc_ok(lp)) {
            if ((rc = adjoint_contract_tc(ctx, B, nt, lp, w.U, w.V, tiled, w.gpart, w.tcerr, s))) return rc;
        } else if (B <= 64) {
            const size_t sma = sizeof(float) * (64 * ADJ_LD + 48 * ADJ_KE);
            CG_CUDA_TRY(ctx, cudaFuncSetAttribute(contract_adj<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sma));
            contract_adj<2><<<dim3(ntile, (B + 63) / 64, (lp + 47) / 48), 256, sma, s>>>(B, lp, w.U, w.V, tiled, w.gpart);
            count_launch(ctx);
        } else {
            const size_t sma = sizeof(float) * (256 * ADJ_LD + 48 * ADJ_KE);
            CG_CUDA_TRY(ctx, cudaFuncSetAttribute(contract_adj<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sma));
            contract_adj<8><<<dim3(ntile, (B + 255) / 256, (lp + 47) / 48), 256, sma, s>>>(B, lp, w.U, w.V, tiled, w.gpart);
            count_launch(ctx);
        }
        const int nhp = nharm_pad(lmax);
        const int ks = ((N + PROJ_KSPLIT * 32 - 1) / (PROJ_KSPLIT * 32)) * 32;
        float* proj_part = w.proj + (size_t)B * nhp;
        project_x<<<dim3(nhp / 64, (B + 63) / 64, PROJ_KSPLIT), 256, 0, s>>>(B, N, nhp, ks, w.Zf, w.x, proj_part);
        project_reduce<<<(unsigned)std::min<size_t>(((size_t)B * nhp + 255) / 256, 4096), 256, 0, s>>>(
            (size_t)B * nhp, proj_part, w.proj);
        adj_finish<<<B, 256, 0, s>>>(B, ntile, lmax, lp, nhp, w.gpart, w.proj, w.cref, d_grad);
        count_launch(ctx, 3);
    }
    merge_tc_status<<<(B + 127) / 128, 128, 0, s>>>(B, w.tcerr, w.st);
    count_launch(ctx);
    if (d_status) CG_CUDA_TRY(ctx, cudaMemcpyAsync(d_status, w.st, sizeof(int) * B, cudaMemcpyDeviceToDevice, s));
    stage_mark(ctx, ST_END, s);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
