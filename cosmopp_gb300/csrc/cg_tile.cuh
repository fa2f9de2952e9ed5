// Shared 64x64 tile helpers for the tiled kernels (k_chol.cu, k_mixed.cu).
// A tile in global memory is column-major, element (r, c) at r + TS*c; in
// shared memory an operand is kept as s[m * SmemLd + row] so that a 256-thread
// block can run 4x4 register micro-tiles over the m (reduction) index.
#pragma once

#include "cg_internal.h"

namespace cg {
namespace tile {

constexpr int NT_THREADS = 256;

// smem tile stored as s[m * SLD + row]
template <typename T>
struct SmemLd {
    static constexpr int v = TS + (sizeof(T) == 4 ? 4 : 2);
};

// sX[m][r] = G(r, m) with G column-major (r + TS*m): contiguous copy
template <typename T>
__device__ __forceinline__ void load_direct(T* s, const T* __restrict__ g)
{
    constexpr int L = SmemLd<T>::v;
    for (int e = threadIdx.x; e < TILE_ELEMS; e += blockDim.x) {
        const int r = e % TS, m = e / TS;
        s[m * L + r] = g[e];
    }
}

// sX[m][r] = G(m, r): transposed copy
template <typename T>
__device__ __forceinline__ void load_trans(T* s, const T* __restrict__ g)
{
    constexpr int L = SmemLd<T>::v;
    for (int e = threadIdx.x; e < TILE_ELEMS; e += blockDim.x) {
        const int m = e % TS, r = e / TS;  // G(m, r) at m + TS*r = e
        s[m * L + r] = g[e];
    }
}

// acc(r0+a, c0+b) += sum_m X(r0+a, m) Y(c0+b, m), sX[m][r], sY[m][c]
template <typename T>
__device__ __forceinline__ void tile_mma(const T* sX, const T* sY, T acc[4][4], int r0, int c0)
{
    constexpr int L = SmemLd<T>::v;
#pragma unroll 8
    for (int m = 0; m < TS; ++m) {
        T x[4], y[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) x[a] = sX[m * L + r0 + a];
#pragma unroll
        for (int b = 0; b < 4; ++b) y[b] = sY[m * L + c0 + b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = fma(x[a], y[b], acc[a][b]);
    }
}

__device__ __forceinline__ void micro_coords(int& r0, int& c0)
{
    r0 = (threadIdx.x % 16) * 4;
    c0 = (threadIdx.x / 16) * 4;
}

}  // namespace tile
}  // namespace cg

namespace cg {
namespace tile {

// Symmetric matvec on the tiled lower storage, two deterministic passes:
// symv_partials: per lower tile (I, J): part[t][0][r] = (V_IJ v_J)[r],
//                part[t][1][c] = (V_IJ^T v_I)[c] (I != J), each as a double-float pair (hi, lo);
// symv_reduce:   out_I = sum_J (row-I pieces) in a fixed order, double-float, one FP64 conversion.
// DF = false: FP32 products and in-tile sums (a solve, whose error is then
// refined away).  DF = true: the vector is split into two FP32 words
// (hi + lo) and every product is formed exactly with an FMA, the in-tile sums
// carried as double-float pairs (Dekker / Knuth error-free transformations) --
// ~44-bit residuals y - A x at FP32 issue rate instead of the 1/64-rate FP64 pipe.
__device__ __forceinline__ void df_add(float& hi, float& lo, float v)
{
    const float t = hi + v;
    const float z = t - hi;
    lo += (hi - (t - z)) + (v - z);
    hi = t;
}

// two double-float partial sums combined (Knuth's TwoSum on the high words, the low words added)
__device__ __forceinline__ void df_merge(float& hi, float& lo, float h2, float l2)
{
    const float t = hi + h2;
    const float z = t - hi;
    lo = (lo + l2) + ((hi - (t - z)) + (h2 - z));
    hi = t;
}

// Packed two-lane FP32 operations (each lane rounded to nearest on its own, as the scalar operation
// would be, and never contracted into a fused operation): the residual pass keeps its row and
// column double-float sums as the two lanes of one pair, so each operation serves both.
__device__ __forceinline__ float2 pk_add(float2 a, float2 b)
{
    asm("{\n\t.reg .b64 ra, rb;\n\tmov.b64 ra, {%0, %1};\n\tmov.b64 rb, {%2, %3};\n\t"
        "add.rn.f32x2 ra, ra, rb;\n\tmov.b64 {%0, %1}, ra;\n\t}"
        : "+f"(a.x), "+f"(a.y)
        : "f"(b.x), "f"(b.y));
    return a;
}
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b)
{
    asm("{\n\t.reg .b64 ra, rb;\n\tmov.b64 ra, {%0, %1};\n\tmov.b64 rb, {%2, %3};\n\t"
        "sub.rn.f32x2 ra, ra, rb;\n\tmov.b64 {%0, %1}, ra;\n\t}"
        : "+f"(a.x), "+f"(a.y)
        : "f"(b.x), "f"(b.y));
    return a;
}
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b)
{
    asm("{\n\t.reg .b64 ra, rb;\n\tmov.b64 ra, {%0, %1};\n\tmov.b64 rb, {%2, %3};\n\t"
        "mul.rn.f32x2 ra, ra, rb;\n\tmov.b64 {%0, %1}, ra;\n\t}"
        : "+f"(a.x), "+f"(a.y)
        : "f"(b.x), "f"(b.y));
    return a;
}
// a * b + c, one rounding per lane
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c)
{
    asm("{\n\t.reg .b64 ra, rb, rc;\n\tmov.b64 ra, {%0, %1};\n\tmov.b64 rb, {%2, %3};\n\t"
        "mov.b64 rc, {%4, %5};\n\tfma.rn.f32x2 ra, ra, rb, rc;\n\tmov.b64 {%0, %1}, ra;\n\t}"
        : "+f"(a.x), "+f"(a.y)
        : "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return a;
}
// (hi, lo) += a * (bh + bl) in double-float arithmetic: the product a bh exactly as p + (a bh - p)
// (one fused operation), p added to hi by Knuth's two-sum, every error term folded into lo
__device__ __forceinline__ void pk_df_madd(float2& hi, float2& lo, float2 a, float2 bh, float2 bl)
{
    const float2 p = pk_mul(a, bh);
    const float2 t = pk_add(hi, p);
    const float2 z = pk_sub(t, hi);
    const float2 e = pk_add(pk_sub(hi, pk_sub(t, z)), pk_sub(p, z));
    const float2 perr = pk_fma(a, bh, make_float2(-p.x, -p.y));
    lo = pk_add(lo, pk_add(e, pk_fma(a, bl, perr)));
    hi = t;
}

// One CTA walks SYMV_TPB consecutive tiles of one batch element: 128-bit loads, the next tile
// prefetched into registers while the current one is reduced.  grid (ceil(tiles / SYMV_TPB), B).
// The four partial sums of a row are combined in FP32 (double-float for DF) and converted to FP64
// once: this GPU's FP64 rate is about two operations per clock per SM, and converting every
// thread's partials cost more than reading the tile.
constexpr int SYMV_TPB = 8;
template <bool DF>
__global__ void __launch_bounds__(256) symv_partials(int nt, const float* __restrict__ V, size_t strideA,
                                                     const double* __restrict__ v, int vstride,
                                                     float2* __restrict__ part)
{
    __shared__ float s[TS][TS + 1];
    __shared__ float svh[2][TS], svl[2][TS];
    __shared__ float redh[4][2][TS], redl[4][2][TS];
    const int b = blockIdx.y, ntile = ntiles_lower(nt);
    const int t0 = blockIdx.x * SYMV_TPB;
    const int tn = min(SYMV_TPB, ntile - t0);
    const float* base = V + (size_t)b * strideA;
    // thread's share of a tile: float4 k at element 4 (threadIdx.x + 256 k), k < 4
    auto load = [&](int t, float4 (&d)[4]) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            d[k] = __ldg(reinterpret_cast<const float4*>(base + (size_t)t * TILE_ELEMS + 4 * (threadIdx.x + 256 * k)));
    };
    float4 cur[4], nxt[4];
    load(t0, cur);
    const int r = threadIdx.x % TS, q = threadIdx.x / TS;
    for (int i = 0; i < tn; ++i) {
        const int t = t0 + i;
        int I, J;
        tile_coords(t, I, J);
        if (i + 1 < tn) load(t + 1, nxt);
        __syncthreads();  // the previous tile's shared-memory reads are done
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int e = 4 * (threadIdx.x + 256 * k);  // s[c][r] = tile(r, c), e = r + TS c
            const float w[4] = {cur[k].x, cur[k].y, cur[k].z, cur[k].w};
#pragma unroll
            for (int j = 0; j < 4; ++j) s[(e + j) / TS][(e + j) % TS] = w[j];
        }
        if (threadIdx.x < 2 * TS) {
            const int w = threadIdx.x / TS, k = threadIdx.x % TS;
            const double x = v[(size_t)b * vstride + (w == 0 ? J : I) * TS + k];
            const float h = (float)x;
            svh[w][k] = h;
            svl[w][k] = (float)(x - (double)h);
        }
        __syncthreads();
        float ah = 0.f, al = 0.f, th = 0.f, tl = 0.f;
        if (DF) {
            // row (lane x) and column (lane y) sums as packed pairs, in two interleaved chains
            // (columns q + 8i and q + 8i + 4) merged at the end: half the dependent additions in a row
            float2 H1 = make_float2(0.f, 0.f), L1 = H1, H2 = H1, L2 = H1;
#pragma unroll
            for (int c = q; c < TS; c += 8) {
                pk_df_madd(H1, L1, make_float2(s[c][r], s[r][c]), make_float2(svh[0][c], svh[1][c]),
                           make_float2(svl[0][c], svl[1][c]));
                pk_df_madd(H2, L2, make_float2(s[c + 4][r], s[r][c + 4]),
                           make_float2(svh[0][c + 4], svh[1][c + 4]), make_float2(svl[0][c + 4], svl[1][c + 4]));
            }
            ah = H1.x; al = L1.x; th = H1.y; tl = L1.y;
            df_merge(ah, al, H2.x, L2.x);
            df_merge(th, tl, H2.y, L2.y);
        } else {
            float2 H = make_float2(0.f, 0.f);  // (row, column) sums, one packed FMA per column
#pragma unroll
            for (int c = q; c < TS; c += 4)
                H = pk_fma(make_float2(s[c][r], s[r][c]), make_float2(svh[0][c], svh[1][c]), H);
            ah = H.x;
            th = H.y;
        }
        redh[q][0][r] = ah;
        redl[q][0][r] = al;
        redh[q][1][r] = th;
        redl[q][1][r] = tl;
        __syncthreads();
        if (q == 0) {
            float2* p = part + ((size_t)b * ntile + t) * 2 * TS;
            float h0 = redh[0][0][r], l0 = redl[0][0][r], h1 = redh[0][1][r], l1 = redl[0][1][r];
#pragma unroll
            for (int k = 1; k < 4; ++k) {
                if (DF) {
                    df_merge(h0, l0, redh[k][0][r], redl[k][0][r]);
                    df_merge(h1, l1, redh[k][1][r], redl[k][1][r]);
                } else {
                    h0 += redh[k][0][r];
                    h1 += redh[k][1][r];
                }
            }
            p[r] = make_float2(h0, DF ? l0 : 0.f);
            p[TS + r] = (I != J) ? make_float2(h1, DF ? l1 : 0.f) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) cur[k] = nxt[k];
    }
}

static __global__ void __launch_bounds__(64) symv_reduce(int nt, const float2* __restrict__ part, double* __restrict__ out,
                                                  int ostride, const double* __restrict__ add, double sign)
{
    const int I = blockIdx.x, b = blockIdx.y, r = threadIdx.x, ntile = ntiles_lower(nt);
    const float2* pb = part + (size_t)b * ntile * 2 * TS;
    float h = 0.f, l = 0.f;
    for (int J = 0; J <= I; ++J) {
        const float2 x = pb[(size_t)tile_index(I, J) * 2 * TS + r];
        df_merge(h, l, x.x, x.y);
    }
    for (int J = I + 1; J < nt; ++J) {
        const float2 x = pb[(size_t)tile_index(J, I) * 2 * TS + TS + r];
        df_merge(h, l, x.x, x.y);
    }
    const size_t o = (size_t)b * ostride + I * TS + r;
    out[o] = (add ? add[o] : 0.0) + sign * ((double)h + (double)l);
}

}  // namespace tile
}  // namespace cg
