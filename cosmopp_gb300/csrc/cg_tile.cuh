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
            // two interleaved double-float chains per direction (columns q + 8i and q + 8i + 4), merged
            // at the end: half the dependent additions in a row
            float bh = 0.f, bl = 0.f, uh = 0.f, ul = 0.f;
#pragma unroll
            for (int c = q; c < TS; c += 8) {
                const float va = s[c][r], vt = s[r][c], wa = s[c + 4][r], wt = s[r][c + 4];
                const float p = va * svh[0][c], pw = wa * svh[0][c + 4];
                df_add(ah, al, p);
                df_add(bh, bl, pw);
                al += fmaf(va, svh[0][c], -p) + va * svl[0][c];
                bl += fmaf(wa, svh[0][c + 4], -pw) + wa * svl[0][c + 4];
                const float pt = vt * svh[1][c], ptw = wt * svh[1][c + 4];
                df_add(th, tl, pt);
                df_add(uh, ul, ptw);
                tl += fmaf(vt, svh[1][c], -pt) + vt * svl[1][c];
                ul += fmaf(wt, svh[1][c + 4], -ptw) + wt * svl[1][c + 4];
            }
            df_merge(ah, al, bh, bl);
            df_merge(th, tl, uh, ul);
        } else {
            for (int c = q; c < TS; c += 4) {
                ah = fmaf(s[c][r], svh[0][c], ah);
                th = fmaf(s[r][c], svh[1][c], th);
            }
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
