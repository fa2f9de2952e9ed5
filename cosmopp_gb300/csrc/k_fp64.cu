// Plain FP64 path: covariance build, likelihood and adjoint gradient.
//
// build_c_tiled / build_c_packed replace CMatrixGenerator::clToCMatrix
// (source/c_matrix_generator.cpp:164-232).  Each thread runs the Bonnet
// recurrence once per pixel pair in registers; the reference restarts it for
// every l (include/legendre.hpp:26-37) but produces the same P_l values bit for
// bit, and the element sum keeps the reference's operation order
//   element += ((clCopy_l * P_l) * B_l) * B_l
// with explicitly rounded (non-fused) FP64 operations, so C is bit-identical
// to the reference's.
//
// The likelihood follows Likelihood::construct / calculate
// (source/likelihood.cpp:69-180): C + N, Cholesky (k_chol.cu), ln det from
// the factor's diagonal, explicit inverse, chi2 = d^T C^-1 d.  The adjoint
// gradient (no reference counterpart) is
//   d(-2lnL)/dC_l = sum_ij (C^-1 - a a^T)_ij (2l+1)/(4pi) B_l^2 P_l(x_ij),  a = C^-1 d.
#include "cg_internal.h"

namespace cg {

namespace {

constexpr double kPi = 3.141592653589793;  // include/math_constants.hpp:8
constexpr int kThreads = 256;
constexpr int kAdjChunk = 48;               // l values accumulated per adjoint pass

// ThreeVector dot (include/three_vector.hpp:37) + clamp (c_matrix_generator.cpp:203-215)
__device__ __forceinline__ double pair_dot(const double* __restrict__ xyz, int N, int i, int j)
{
    double d = __dadd_rn(__dadd_rn(__dmul_rn(xyz[i], xyz[j]), __dmul_rn(xyz[N + i], xyz[N + j])),
                         __dmul_rn(xyz[2 * N + i], xyz[2 * N + j]));
    if (d > 1.0) d = 1.0;
    if (d < -1.0) d = -1.0;
    return d;
}

// sum_{l=2}^{lmax} ((clc_l * P_l) * B_l) * B_l in the reference's order, 4 pairs at once
__device__ __forceinline__ void cmat_sum4(const double x[4], double out[4], int lmax, const double* sa,
                                          const double* sb, const double* sc, const double* sbeam)
{
    double p0[4], p1[4], acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) { p0[q] = 1.0; p1[q] = x[q]; acc[q] = 0.0; }
    for (int l = 2; l <= lmax; ++l) {
        const double a = sa[l], b = sb[l], c = sc[l], bm = sbeam[l];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double p = __dsub_rn(__dmul_rn(__dmul_rn(a, x[q]), p1[q]), __dmul_rn(b, p0[q]));
            acc[q] = __dadd_rn(acc[q], __dmul_rn(__dmul_rn(__dmul_rn(c, p), bm), bm));
            p0[q] = p1[q];
            p1[q] = p;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) out[q] = acc[q];
}

__device__ __forceinline__ void load_consts(double* sa, double* sb, double* sc, double* sbeam, int lmax,
                                            const double* lega, const double* legb, const double* beam,
                                            const double* cl_b)
{
    for (int l = threadIdx.x; l <= lmax; l += blockDim.x) {
        sa[l] = lega[l];
        sb[l] = legb[l];
        sbeam[l] = beam[l];
        // clCopy[l] = cl[l] * (2 l + 1) / (4 pi)   (c_matrix_generator.cpp:190-193)
        sc[l] = (l >= 2) ? __ddiv_rn(__dmul_rn(cl_b[l], (double)(2 * l + 1)), 4.0 * kPi) : 0.0;
    }
}

// C (+ noise on the diagonal, identity padding) into the tiled layout, grid (tiles, B)
__global__ void __launch_bounds__(kThreads) build_c_tiled(int n, int N, int lmax, const double* __restrict__ xyz,
                                                          const double* __restrict__ noise,
                                                          const double* __restrict__ lega,
                                                          const double* __restrict__ legb,
                                                          const double* __restrict__ beam,
                                                          const double* __restrict__ cl, int add_noise,
                                                          double* __restrict__ A, size_t strideA)
{
    extern __shared__ double sconst[];
    double* sa = sconst;
    double* sb = sa + (lmax + 1);
    double* sc = sb + (lmax + 1);
    double* sbeam = sc + (lmax + 1);
    const int b = blockIdx.y;
    load_consts(sa, sb, sc, sbeam, lmax, lega, legb, beam, cl + (size_t)b * (lmax + 1));
    __syncthreads();
    int I, J;
    tile_coords(blockIdx.x, I, J);
    double* tile = A + (size_t)b * strideA + (size_t)blockIdx.x * TILE_ELEMS;
    for (int g = 0; g < TILE_ELEMS / (kThreads * 4); ++g) {
        double x[4], v[4];
        int e[4];
        bool real[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            e[q] = threadIdx.x + kThreads * (4 * g + q);
            const int i = I * TS + e[q] % TS, j = J * TS + e[q] / TS;
            real[q] = (i < n && j < n);
            x[q] = real[q] ? pair_dot(xyz, N, i, j) : 0.0;
        }
        cmat_sum4(x, v, lmax, sa, sb, sc, sbeam);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = I * TS + e[q] % TS, j = J * TS + e[q] / TS;
            double val;
            if (real[q]) {
                val = v[q];
                // cInv_(i,j) = c + fiducial(0) + noise  (source/likelihood.cpp:102-110)
                if (add_noise && i == j) val = __dadd_rn(__dadd_rn(val, 0.0), noise[i]);
            } else {
                val = (i == j) ? 1.0 : 0.0;
            }
            tile[e[q]] = val;
        }
    }
}

// packed output (i <= j at j(j+1)/2 + i), one thread per entry, grid (ceil(np/256), B)
__global__ void __launch_bounds__(kThreads) build_c_packed(int n, int N, int lmax, const double* __restrict__ xyz,
                                                           const double* __restrict__ lega,
                                                           const double* __restrict__ legb,
                                                           const double* __restrict__ beam,
                                                           const double* __restrict__ cl, double* __restrict__ out)
{
    extern __shared__ double sconst[];
    double* sa = sconst;
    double* sb = sa + (lmax + 1);
    double* sc = sb + (lmax + 1);
    double* sbeam = sc + (lmax + 1);
    const int b = blockIdx.y;
    load_consts(sa, sb, sc, sbeam, lmax, lega, legb, beam, cl + (size_t)b * (lmax + 1));
    __syncthreads();
    const long np = (long)n * (n + 1) / 2;
    const long k0 = 4 * ((long)blockIdx.x * kThreads + threadIdx.x);
    if (k0 >= np) return;
    long j = (long)((sqrt(8.0 * (double)k0 + 1.0) - 1.0) * 0.5);
    while (j * (j + 1) / 2 > k0) --j;
    while ((j + 1) * (j + 2) / 2 <= k0) ++j;
    long i = k0 - j * (j + 1) / 2;
    double x[4], v[4];
    long kk[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // four consecutive packed entries: walk i, wrap to the next column
        kk[q] = k0 + q;
        x[q] = (kk[q] < np) ? pair_dot(xyz, N, (int)i, (int)j) : 0.0;
        if (++i > j) { ++j; i = 0; }
    }
    cmat_sum4(x, v, lmax, sa, sb, sc, sbeam);
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (kk[q] < np) out[(size_t)b * np + kk[q]] = v[q];
}

// CMatrixGenerator::getFiducialMatrix (source/c_matrix_generator.cpp:706-772), packed i <= j:
//   element = sum_{l=lo}^{hi} (((fc_l * P_l) * B_l) * B_l) + (((m0 * (1 + x)) * B_2) * B_2)
// with fc_l = cl_l * ((2l+1)/(4 pi)) and m0 = 100 cl_2 formed on the host as the reference
// forms them; tab = [a | b | fc | beam], hi + 1 entries each; lo >= 2.
__global__ void __launch_bounds__(kThreads) build_fid_packed(int n, int N, int lo, int hi,
                                                             const double* __restrict__ xyz,
                                                             const double* __restrict__ tab, double m0,
                                                             double* __restrict__ out)
{
    extern __shared__ double sconst[];
    const int L1 = hi + 1;
    for (int e = threadIdx.x; e < 4 * L1; e += blockDim.x) sconst[e] = tab[e];
    __syncthreads();
    const double* sa = sconst;
    const double* sb = sa + L1;
    const double* sf = sb + L1;
    const double* sbeam = sf + L1;
    const long np = (long)n * (n + 1) / 2;
    const long k0 = 4 * ((long)blockIdx.x * kThreads + threadIdx.x);
    if (k0 >= np) return;
    long j = (long)((sqrt(8.0 * (double)k0 + 1.0) - 1.0) * 0.5);
    while (j * (j + 1) / 2 > k0) --j;
    while ((j + 1) * (j + 2) / 2 <= k0) ++j;
    long i = k0 - j * (j + 1) / 2;
    double x[4], p0[4], p1[4], acc[4];
    long kk[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        kk[q] = k0 + q;
        x[q] = (kk[q] < np) ? pair_dot(xyz, N, (int)i, (int)j) : 0.0;
        if (++i > j) { ++j; i = 0; }
        p0[q] = 1.0;
        p1[q] = x[q];
        acc[q] = 0.0;
    }
    for (int l = 2; l < lo; ++l) {  // recurrence only (include/legendre.hpp:34)
        const double a = sa[l], b = sb[l];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double p = __dsub_rn(__dmul_rn(__dmul_rn(a, x[q]), p1[q]), __dmul_rn(b, p0[q]));
            p0[q] = p1[q];
            p1[q] = p;
        }
    }
    for (int l = lo; l <= hi; ++l) {
        const double a = sa[l], b = sb[l], f = sf[l], bm = sbeam[l];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double p = __dsub_rn(__dmul_rn(__dmul_rn(a, x[q]), p1[q]), __dmul_rn(b, p0[q]));
            acc[q] = __dadd_rn(acc[q], __dmul_rn(__dmul_rn(__dmul_rn(f, p), bm), bm));
            p0[q] = p1[q];
            p1[q] = p;
        }
    }
    const double b2 = sbeam[2];
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (kk[q] < np)
            out[kk[q]] = __dadd_rn(acc[q], __dmul_rn(__dmul_rn(__dmul_rn(m0, __dadd_rn(1.0, x[q])), b2), b2));
}

// ln det = 2 sum_i ln L_ii over the n real pixels (source/matrix_impl.cpp:322-338), grid B
__global__ void __launch_bounds__(kThreads) logdet_reduce(int n, int N, const double* __restrict__ diag,
                                                          double* __restrict__ logdet)
{
    __shared__ double red[kThreads];
    const int b = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) s += log(fabs(diag[(size_t)b * N + i]));
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) logdet[b] = 2.0 * red[0];
}

// padded copy of the data maps into dvec[b][N]
__global__ void pad_data(int n, int N, int B, const double* __restrict__ d, int d_stride, double* __restrict__ dv)
{
    const int b = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || b >= B) return;
    dv[(size_t)b * N + i] = (i < n) ? d[(size_t)b * d_stride + i] : 0.0;
}

// alpha = V d with V symmetric in lower tiles; grid (nt, B); thread (row r, part q)
template <typename T>
__global__ void __launch_bounds__(kThreads) symv_tiled(int nt, int N, const T* __restrict__ V, size_t strideA,
                                                       const double* __restrict__ dv, double* __restrict__ alpha)
{
    __shared__ double part[4][TS];
    const int I = blockIdx.x, b = blockIdx.y;
    const int r = threadIdx.x % TS, q = threadIdx.x / TS;
    const T* Vb = V + (size_t)b * strideA;
    const double* db = dv + (size_t)b * N;
    double s = 0.0;
    for (int J = 0; J < nt; ++J) {
        if (J <= I) {
            const T* t = Vb + (size_t)tile_index(I, J) * TILE_ELEMS;
            for (int c = q; c < TS; c += 4) s += (double)t[r + TS * c] * db[J * TS + c];
        } else {
            const T* t = Vb + (size_t)tile_index(J, I) * TILE_ELEMS;
            for (int c = q; c < TS; c += 4) s += (double)t[c + TS * r] * db[J * TS + c];
        }
    }
    part[q][r] = s;
    __syncthreads();
    if (q == 0) alpha[(size_t)b * N + I * TS + r] = ((part[0][r] + part[1][r]) + part[2][r]) + part[3][r];
}

// chi2 = d . alpha, m2lnl = chi2 + logdet; grid B
__global__ void __launch_bounds__(kThreads) chi2_finish(int n, int N, const double* __restrict__ dv,
                                                        const double* __restrict__ alpha,
                                                        const double* __restrict__ logdet, double* __restrict__ m2lnl,
                                                        double* __restrict__ chi2)
{
    __shared__ double red[kThreads];
    const int b = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) s += dv[(size_t)b * N + i] * alpha[(size_t)b * N + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (chi2) chi2[b] = red[0];
        m2lnl[b] = red[0] + logdet[b];
    }
}

// Adjoint partial sums: for every lower tile, sum over its pairs of
// w_ij P_l(x_ij) for l in [l0, l1), w_ij = mult (V_ij - a_i a_j); grid (tiles, B)
__global__ void __launch_bounds__(kThreads) adjoint_tiles(int n, int N, int l0, int l1, const double* __restrict__ xyz,
                                                          const double* __restrict__ lega,
                                                          const double* __restrict__ legb,
                                                          const double* __restrict__ V, size_t strideA,
                                                          const double* __restrict__ alpha,
                                                          double* __restrict__ gpart, int ntile, int lstride)
{
    __shared__ double sa[256], sb[256];
    __shared__ double red[kThreads / 32][kAdjChunk];
    for (int l = threadIdx.x; l < l1 && l < 256; l += kThreads) { sa[l] = lega[l]; sb[l] = legb[l]; }
    __syncthreads();
    int I, J;
    tile_coords(blockIdx.x, I, J);
    const int b = blockIdx.y;
    const double* tile = V + (size_t)b * strideA + (size_t)blockIdx.x * TILE_ELEMS;
    const double* al = alpha + (size_t)b * N;
    double acc[kAdjChunk];
#pragma unroll
    for (int c = 0; c < kAdjChunk; ++c) acc[c] = 0.0;
    for (int e = threadIdx.x; e < TILE_ELEMS; e += kThreads) {
        const int i = I * TS + e % TS, j = J * TS + e / TS;
        if (i >= n || j >= n || j > i) continue;
        const double w = (i == j ? 1.0 : 2.0) * (tile[e] - al[i] * al[j]);
        const double x = pair_dot(xyz, N, i, j);
        double p0 = 1.0, p1 = x;
        for (int l = 2; l < l0; ++l) {  // advance to P_{l0-1}, P_{l0-2}
            const double p = (sa[l] * x) * p1 - sb[l] * p0;
            p0 = p1;
            p1 = p;
        }
#pragma unroll
        for (int c = 0; c < kAdjChunk; ++c) {
            const int l = l0 + c;
            if (l < l1) {
                const double p = (sa[l] * x) * p1 - sb[l] * p0;
                acc[c] += w * p;
                p0 = p1;
                p1 = p;
            }
        }
    }
    // deterministic block reduction: warp shuffles, then warps in order
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
#pragma unroll
    for (int c = 0; c < kAdjChunk; ++c) {
        double v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < kAdjChunk && l0 + (int)threadIdx.x < l1) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w][threadIdx.x];
        gpart[((size_t)b * ntile + blockIdx.x) * lstride + l0 + threadIdx.x] = s;
    }
}

// grad_l = (sum over tiles) * ((2l+1)/(4 pi)) * B_l * B_l; grid B
__global__ void adjoint_finish(int lmax, int ntile, const double* __restrict__ gpart, const double* __restrict__ beam,
                               double* __restrict__ grad)
{
    const int b = blockIdx.x;
    for (int l = threadIdx.x; l <= lmax; l += blockDim.x) {
        double s = 0.0;
        if (l >= 2)
            for (int t = 0; t < ntile; ++t) s += gpart[((size_t)b * ntile + t) * (lmax + 1) + l];
        grad[(size_t)b * (lmax + 1) + l] = (l < 2) ? 0.0 : s * ((2 * l + 1) / (4 * kPi)) * beam[l] * beam[l];
    }
}

// input check: non-finite C_l -> status NONFINITE, else OK
__global__ void check_inputs(int B, int lmax, const double* __restrict__ cl, int* __restrict__ status)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    int st = CG_OK;
    for (int l = 0; l <= lmax; ++l)
        if (!isfinite(cl[(size_t)b * (lmax + 1) + l])) st = CG_ERR_NONFINITE;
    status[b] = st;
}

__global__ void copy_status(int B, const int* __restrict__ src, int* __restrict__ dst)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < B) dst[b] = src[b];
}

// A = c + fid + noise from packed host-layout arrays into the tiled layout,
// in the reference's summation order (source/likelihood.cpp:102-110); grid tiles
__global__ void __launch_bounds__(kThreads) packed_sum_to_tiled(int n, const double* __restrict__ c,
                                                                const double* __restrict__ f,
                                                                const double* __restrict__ nz, double* __restrict__ A)
{
    int I, J;
    tile_coords(blockIdx.x, I, J);
    double* tile = A + (size_t)blockIdx.x * TILE_ELEMS;
    for (int e = threadIdx.x; e < TILE_ELEMS; e += kThreads) {
        const int i = I * TS + e % TS, j = J * TS + e / TS;
        double v;
        if (i < n && j < n) {
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            const size_t k = (size_t)hi * (hi + 1) / 2 + lo;
            v = __dadd_rn(__dadd_rn(c[k], f ? f[k] : 0.0), nz[k]);
        } else {
            v = (i == j) ? 1.0 : 0.0;
        }
        tile[e] = v;
    }
}

__global__ void dot_kernel(int n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out)
{
    __shared__ double red[kThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) s += a[i] * b[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// Dense FP64 helpers of the polarisation likelihood's set-up (column-major, leading dimension
// ld, a multiple of 64, zero padding beyond n).
// out = add + A B: one 64 x 64 output tile per CTA, 16-deep K slices of A and B in shared memory,
// 4 x 4 outputs per thread at rows tx + 16 p and columns ty + 16 q
__global__ void __launch_bounds__(kThreads) dense_gemm64(int ld, const double* __restrict__ A,
                                                         const double* __restrict__ Bm,
                                                         const double* __restrict__ add, double* __restrict__ out)
{
    __shared__ double As[16][65], Bs[16][65];
    const int bi = blockIdx.x * 64, bj = blockIdx.y * 64;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    double acc[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = 0.0;
    for (int k0 = 0; k0 < ld; k0 += 16) {
        for (int e = threadIdx.x; e < 1024; e += kThreads) {
            const int r = e % 64, kk = e / 64;
            As[kk][r] = A[(size_t)(k0 + kk) * ld + bi + r];
            const int kb = e % 16, c = e / 16;
            Bs[kb][c] = Bm[(size_t)(bj + c) * ld + k0 + kb];
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int p = 0; p < 4; ++p) a[p] = As[kk][tx + 16 * p];
#pragma unroll
            for (int q = 0; q < 4; ++q) b[q] = Bs[kk][ty + 16 * q];
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const size_t o = (size_t)(bj + ty + 16 * q) * ld + bi + tx + 16 * p;
            out[o] = (add ? add[o] : 0.0) + acc[p][q];
        }
}

// packed symmetric (i <= j at j(j+1)/2 + i) to dense, zero outside n x n; grid covers ld x ld
__global__ void packed_to_dense(int n, int ld, const double* __restrict__ pk, double* __restrict__ d)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)ld * ld) return;
    const int r = (int)(e % ld), c = (int)(e / ld);
    const int i = min(r, c), j = max(r, c);
    d[e] = (j < n) ? pk[(size_t)j * (j + 1) / 2 + i] : 0.0;
}

// the upper triangle of a dense symmetric matrix, packed
__global__ void dense_to_packed(int n, int ld, const double* __restrict__ d, double* __restrict__ pk)
{
    const long np = (long)n * (n + 1) / 2;
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    long j = (long)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
    while (j * (j + 1) / 2 > k) --j;
    while ((j + 1) * (j + 2) / 2 <= k) ++j;
    const long i = k - j * (j + 1) / 2;
    pk[k] = d[(size_t)j * ld + i];
}

// w = v - N s for a dense symmetric N (row i read as column i, coalesced over i)
__global__ void dense_residual(int n, int ld, const double* __restrict__ Nm, const double* __restrict__ v,
                               const double* __restrict__ sv, double* __restrict__ w)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
    for (int j = 0; j < n; ++j) acc = fma(Nm[(size_t)j * ld + i], sv[j], acc);
    w[i] = v[i] - acc;
}

// LegendrePolynomialContainer's table (source/c_matrix_generator.cpp:30-76): P_l(x_ij) for
// l0 <= l < l1 at out[(l - l0) np + j(j+1)/2 + i], i <= j, by Math::Legendre's recurrence
// (include/legendre.hpp:26-37: P_0 = 1, P_1 = x, P_l = ((2 - 1/l) x) P_{l-1} - (1 - 1/l) P_{l-2},
// coefficients a_l, b_l from the host) with the reference's dot product and clamp, so the
// table is bit-identical.  One thread per pair; stores of one l are coalesced over pairs.
__global__ void __launch_bounds__(kThreads) legendre_table(int n, int N, int l0, int l1,
                                                           const double* __restrict__ xyz,
                                                           const double* __restrict__ a,
                                                           const double* __restrict__ b,
                                                           double* __restrict__ out)
{
    const long np = (long)n * (n + 1) / 2;
    const long k = (long)blockIdx.x * kThreads + threadIdx.x;
    if (k >= np) return;
    long j = (long)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
    while (j * (j + 1) / 2 > k) --j;
    while ((j + 1) * (j + 2) / 2 <= k) ++j;
    const int i = (int)(k - j * (j + 1) / 2);
    const double x = pair_dot(xyz, N, i, (int)j);
    double p0 = 1.0, p1 = x;
    for (int l = 0; l < l1; ++l) {
        double p;
        if (l == 0) {
            p = 1.0;
        } else if (l == 1) {
            p = x;
        } else {
            p = __dsub_rn(__dmul_rn(__dmul_rn(a[l], x), p1), __dmul_rn(b[l], p0));
            p0 = p1;
            p1 = p;
        }
        if (l >= l0) out[(size_t)(l - l0) * np + k] = p;
    }
}

// Averaging step of CMatrixGenerator::calculateNoiseMatrix (source/c_matrix_generator.cpp:887-910):
// N_ij = (sum_k s_k[i] s_k[j]) / nsims, k in order, every product and sum rounded on its own
// (the reference's loop, compiled without contraction), so the packed result is
// bit-identical.  A CTA computes one 64x64 tile (I <= J) of the upper triangle; 16-deep
// slices of the two 64-pixel panels are staged in shared memory; each thread keeps a
// 4x4 block of sums at rows ty + 16a and columns tx + 16b.
constexpr int kNoiseT = 64, kNoiseK = 16;

__global__ void __launch_bounds__(kThreads, 2) noise_syrk_packed(int nsims, int n, const double* __restrict__ sims,
                                                              double* __restrict__ out)
{
    const long t = blockIdx.x;
    int J = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((long)J * (J + 1) / 2 > t) --J;
    while ((long)(J + 1) * (J + 2) / 2 <= t) ++J;
    const int I = (int)(t - (long)J * (J + 1) / 2);
    __shared__ double si[kNoiseK][kNoiseT], sj[kNoiseK][kNoiseT];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    for (int k0 = 0; k0 < nsims; k0 += kNoiseK) {
#pragma unroll
        for (int r = 0; r < kNoiseK * kNoiseT / kThreads; ++r) {
            const int e = threadIdx.x + r * kThreads, kk = e / kNoiseT, c = e % kNoiseT, k = k0 + kk;
            const int gi = I * kNoiseT + c, gj = J * kNoiseT + c;
            si[kk][c] = (k < nsims && gi < n) ? sims[(size_t)k * n + gi] : 0.0;
            sj[kk][c] = (k < nsims && gj < n) ? sims[(size_t)k * n + gj] : 0.0;
        }
        __syncthreads();
        const int kend = min(kNoiseK, nsims - k0);
        for (int kk = 0; kk < kend; ++kk) {
            double x[4], y[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) x[a] = si[kk][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) y[b] = sj[kk][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = __dadd_rn(acc[a][b], __dmul_rn(x[a], y[b]));
        }
        __syncthreads();
    }
    const double dn = (double)nsims;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int i = I * kNoiseT + ty + 16 * a, j = J * kNoiseT + tx + 16 * b;
            if (i <= j && j < n) out[(size_t)j * (j + 1) / 2 + i] = __ddiv_rn(acc[a][b], dn);
        }
}

// per-pixel mean over the simulations, summed in order (source/c_matrix_generator.cpp:901-910)
__global__ void sim_means(int nsims, int n, const double* __restrict__ sims, double* __restrict__ mean)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0.0;
    for (int k = 0; k < nsims; ++k) s = __dadd_rn(s, sims[(size_t)k * n + j]);
    mean[j] = __ddiv_rn(s, (double)nsims);
}

}  // namespace

void fp64_packed_to_tiled(int n, int nt, const double* c, const double* f, const double* nz, double* A, cudaStream_t s)
{
    packed_sum_to_tiled<<<ntiles_lower(nt), kThreads, 0, s>>>(n, c, f, nz, A);
}

void fp64_symv(int B, int nt, int N, const double* V, const double* dv, double* alpha, cudaStream_t s)
{
    symv_tiled<double><<<dim3(nt, B), kThreads, 0, s>>>(nt, N, V, tiled_elems(nt), dv, alpha);
}

void fp64_logdet(int B, int n, int N, const double* diag, double* out, cudaStream_t s)
{
    logdet_reduce<<<B, kThreads, 0, s>>>(n, N, diag, out);
}

void fp64_dot(int n, const double* a, const double* b, double* out, cudaStream_t s)
{
    dot_kernel<<<1, kThreads, 0, s>>>(n, a, b, out);
}

void fp64_free(cg_ctx* ctx)
{
    Fp64Work& w = ctx->w64;
    cudaFree(w.A); cudaFree(w.M); cudaFree(w.Dinv); cudaFree(w.diag); cudaFree(w.clc);
    cudaFree(w.dvec); cudaFree(w.alpha); cudaFree(w.gpart); cudaFree(w.st); cudaFree(w.ld);
    w = Fp64Work();
}

// Device bytes of one batch element's FP64 workspace: the allocations of fp64_ensure, in its order
size_t fp64_bytes_per_element(const cg_ctx* ctx)
{
    const size_t tiled = tiled_elems(ctx->nt);
    const int ntile = ntiles_lower(ctx->nt);
    return sizeof(double) * tiled * 2 + sizeof(double) * (size_t)ctx->nt * TILE_ELEMS +
           sizeof(double) * (size_t)ctx->N * 3 + sizeof(double) * (size_t)ntile * (ctx->lmax + 1) + sizeof(int) +
           sizeof(double);
}

int fp64_ensure(cg_ctx* ctx, int B)
{
    Fp64Work& w = ctx->w64;
    if (w.cap >= B) return CG_OK;
    fp64_free(ctx);
    const size_t tiled = tiled_elems(ctx->nt);
    const int ntile = ntiles_lower(ctx->nt);
    auto alloc = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, bytes) == cudaSuccess; };
    bool ok = alloc((void**)&w.A, sizeof(double) * tiled * B) && alloc((void**)&w.M, sizeof(double) * tiled * B) &&
              alloc((void**)&w.Dinv, sizeof(double) * (size_t)B * ctx->nt * TILE_ELEMS) &&
              alloc((void**)&w.diag, sizeof(double) * (size_t)B * ctx->N) &&
              alloc((void**)&w.dvec, sizeof(double) * (size_t)B * ctx->N) &&
              alloc((void**)&w.alpha, sizeof(double) * (size_t)B * ctx->N) &&
              alloc((void**)&w.gpart, sizeof(double) * (size_t)B * ntile * (ctx->lmax + 1)) &&
              alloc((void**)&w.st, sizeof(int) * (size_t)B) && alloc((void**)&w.ld, sizeof(double) * (size_t)B);
    if (!ok) {
        fp64_free(ctx);
        cudaGetLastError();
        ctx->err = "device allocation failed for the FP64 workspace";
        return CG_ERR_ALLOC;
    }
    w.cap = B;
    return CG_OK;
}

static size_t const_smem(int lmax) { return sizeof(double) * 4 * (size_t)(lmax + 1); }

int fp64_build_tiled_into(cg_ctx* ctx, int B, const double* d_cl, bool add_noise, double* A, cudaStream_t s)
{
    const int ntile = ntiles_lower(ctx->nt);
    build_c_tiled<<<dim3(ntile, B), kThreads, const_smem(ctx->lmax), s>>>(
        ctx->n, ctx->N, ctx->lmax, ctx->d_xyz, ctx->d_noise, ctx->d_lega, ctx->d_legb, ctx->d_beam, d_cl,
        add_noise ? 1 : 0, A, tiled_elems(ctx->nt));
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int fp64_build_tiled(cg_ctx* ctx, int B, const double* d_cl, bool add_noise, cudaStream_t s)
{
    return fp64_build_tiled_into(ctx, B, d_cl, add_noise, ctx->w64.A, s);
}

int fp64_build_packed(cg_ctx* ctx, int B, const double* d_cl, double* d_out, cudaStream_t s)
{
    const long np = (long)ctx->n * (ctx->n + 1) / 2;
    build_c_packed<<<dim3((unsigned)((np + 4 * kThreads - 1) / (4 * kThreads)), B), kThreads, const_smem(ctx->lmax), s>>>(
        ctx->n, ctx->N, ctx->lmax, ctx->d_xyz, ctx->d_lega, ctx->d_legb, ctx->d_beam, d_cl, d_out);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int fp64_build_fiducial(cg_ctx* ctx, int lo, int hi, const double* d_tab, double m0, double* d_out, cudaStream_t s)
{
    const long np = (long)ctx->n * (ctx->n + 1) / 2;
    const int smem = (int)(sizeof(double) * 4 * (hi + 1));
    if (smem > 48 * 1024)
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(build_fid_packed, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    build_fid_packed<<<(unsigned)((np + 4 * kThreads - 1) / (4 * kThreads)), kThreads, smem, s>>>(
        ctx->n, ctx->N, lo, hi, ctx->d_xyz, d_tab, m0, d_out);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int fp64_pol_matrix(cg_ctx* ctx, int n, int ld, const double* d_c_packed, const double* d_ninv, double* d_cd,
                    double* d_t, double* d_m, double* d_m_packed, cudaStream_t s)
{
    const size_t nel = (size_t)ld * ld;
    packed_to_dense<<<(unsigned)((nel + kThreads - 1) / kThreads), kThreads, 0, s>>>(n, ld, d_c_packed, d_cd);
    const dim3 grid(ld / 64, ld / 64);
    dense_gemm64<<<grid, kThreads, 0, s>>>(ld, d_cd, d_ninv, nullptr, d_t);   // T = C N^-1
    dense_gemm64<<<grid, kThreads, 0, s>>>(ld, d_ninv, d_t, d_ninv, d_m);     // M = N^-1 + N^-1 T
    const long np = (long)n * (n + 1) / 2;
    dense_to_packed<<<(unsigned)((np + kThreads - 1) / kThreads), kThreads, 0, s>>>(n, ld, d_m, d_m_packed);
    count_launch(ctx, 4);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int fp64_dense_residual(cg_ctx* ctx, int n, int ld, const double* d_ninv, const double* d_v, const double* d_s,
                        double* d_w, cudaStream_t s)
{
    dense_residual<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(n, ld, d_ninv, d_v, d_s, d_w);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int fp64_legendre_table(cg_ctx* ctx, int l0, int l1, const double* d_a, const double* d_b, double* d_out,
                        cudaStream_t s)
{
    const long np = (long)ctx->n * (ctx->n + 1) / 2;
    legendre_table<<<(unsigned)((np + kThreads - 1) / kThreads), kThreads, 0, s>>>(ctx->n, ctx->N, l0, l1, ctx->d_xyz,
                                                                                 d_a, d_b, d_out);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int fp64_noise_matrix(cg_ctx* ctx, int nsims, int n, const double* d_sims, double* d_out, double* d_mean,
                      cudaStream_t s)
{
    const long nt = (n + kNoiseT - 1) / kNoiseT;
    noise_syrk_packed<<<(unsigned)(nt * (nt + 1) / 2), kThreads, 0, s>>>(nsims, n, d_sims, d_out);
    sim_means<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(nsims, n, d_sims, d_mean);
    count_launch(ctx, 2);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int fp64_loglike(cg_ctx* ctx, int B, const double* d_cl, const double* d_d, int d_stride, double* d_m2lnl,
                 double* d_chi2, double* d_logdet, double* d_grad, int* d_status, cudaStream_t s)
{
    int rc = fp64_ensure(ctx, B);
    if (rc) return rc;
    Fp64Work& w = ctx->w64;
    const int nt = ctx->nt, N = ctx->N, n = ctx->n, lmax = ctx->lmax;
    const size_t strideA = tiled_elems(nt);
    const int ntile = ntiles_lower(nt);
    stage_mark(ctx, ST_BUILD, s);
    check_inputs<<<(B + 127) / 128, 128, 0, s>>>(B, lmax, d_cl, w.st);
    count_launch(ctx);
    if ((rc = fp64_build_tiled(ctx, B, d_cl, true, s))) return rc;
    stage_mark(ctx, ST_CHOL, s);
    if ((rc = tiled_cholesky<double>(ctx, B, nt, w.A, w.Dinv, w.diag, w.st, strideA, s))) return rc;
    logdet_reduce<<<B, kThreads, 0, s>>>(n, N, w.diag, w.ld);
    count_launch(ctx);
    stage_mark(ctx, ST_TRTRI, s);
    if ((rc = tiled_trtri<double>(ctx, B, nt, w.A, w.Dinv, w.M, strideA, s))) return rc;
    stage_mark(ctx, ST_LAUUM, s);
    if ((rc = tiled_lauum<double>(ctx, B, nt, w.M, w.A, strideA, s))) return rc;
    stage_mark(ctx, ST_SOLVE, s);
    pad_data<<<dim3((N + 255) / 256, B), 256, 0, s>>>(n, N, B, d_d, d_stride, w.dvec);
    symv_tiled<double><<<dim3(nt, B), kThreads, 0, s>>>(nt, N, w.A, strideA, w.dvec, w.alpha);
    chi2_finish<<<B, kThreads, 0, s>>>(n, N, w.dvec, w.alpha, w.ld, d_m2lnl, d_chi2);
    count_launch(ctx, 3);
    stage_mark(ctx, ST_ADJOINT, s);
    if (d_logdet) CG_CUDA_TRY(ctx, cudaMemcpyAsync(d_logdet, w.ld, sizeof(double) * B, cudaMemcpyDeviceToDevice, s));
    if (d_grad) {
        for (int l0 = 2; l0 <= lmax; l0 += kAdjChunk) {
            const int l1 = (l0 + kAdjChunk <= lmax + 1) ? l0 + kAdjChunk : lmax + 1;
            adjoint_tiles<<<dim3(ntile, B), kThreads, 0, s>>>(n, N, l0, l1, ctx->d_xyz, ctx->d_lega, ctx->d_legb, w.A,
                                                              strideA, w.alpha, w.gpart, ntile, lmax + 1);
            count_launch(ctx);
        }
        adjoint_finish<<<B, 64, 0, s>>>(lmax, ntile, w.gpart, ctx->d_beam, d_grad);
        count_launch(ctx);
    }
    if (d_status) { copy_status<<<(B + 127) / 128, 128, 0, s>>>(B, w.st, d_status); count_launch(ctx); }
    stage_mark(ctx, ST_END, s);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
