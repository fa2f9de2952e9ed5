// Tensor-core (tcgen05, kind::tf32) tile products for the FP32 whitened
// matrices of the mixed path, at FP32 accuracy by the 3xTF32 split
// a*b ~ a_hi*b_hi + a_hi*b_lo + a_lo*b_hi (a_hi = the 19 bits the tensor core
// reads, a_lo = a - a_hi), accumulated in FP32 in tensor memory.
//
// One CTA (128 threads) owns a 128x128 output supertile (2x2 of the 64x64
// storage tiles) and runs a K loop over 32-wide chunks: every thread loads
// one row of the A and B chunks into registers, the chunk is split hi/lo into
// a double-buffered shared-memory stage in the K-major canonical layout, and
// one thread issues 12 MMAs (M128 N128 K8) per chunk and commits them to the
// stage's mbarrier; the next chunk's global loads overlap those MMAs.
//
//   chol_tc_update: left-looking Cholesky, column block J: S_IJ = A_IJ - sum_{k<J} L_Ik L_Jk^T;
//                   the diagonal CTA factors S_JJ = L_JJ L_JJ^T and inverts L_JJ in shared memory
//   chol_tc_panel:  L_IJ = S_IJ L_JJ^-T                        (I > J)
//   trtri_tc_row:   M_IJ = -L_II^-1 sum_{k=J}^{I-1} L_Ik M_kJ, M_II = L_II^-1   (M = L^-1)
//   lauum_tc:       V_IJ = sum_{k >= row} M_kI^T M_kJ = (L L^T)^-1
// (I, J in 128-row blocks; every matrix in 64x64 column-major storage tiles; the
// 128x128 inverses of the diagonal blocks of L are kept row-major in Linv.)
#include "cg_internal.h"
#include "cg_tc.cuh"

namespace cg {

using namespace tc;

namespace {

constexpr int KC = 32;                     // K columns per chunk
constexpr int STAGE_FLOATS = 128 * KC;     // one operand half (hi or lo) per stage
constexpr uint32_t LBO = 128, SBO = KC / 4 * 128;
constexpr uint32_t IDESC = idesc_tf32(128, 128);

struct TcSmem {
    float buf[2][4][STAGE_FLOATS];         // [stage][a_hi, a_lo, b_hi, b_lo]
};

// stores one float4 (row r, K columns 4q..4q+3 of the chunk) as hi and lo parts
__device__ __forceinline__ void put4(float* hi, float* lo, int r, int q, float4 v)
{
    const uint32_t o = kmajor_offset(r, 4 * q, KC) / 4;
    float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w));
    *reinterpret_cast<float4*>(hi + o) = v;
    *reinterpret_cast<float4*>(lo + o) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
}

// Tensor-memory columns: R (running sum) at 0, segment accumulators S0 / S1 at 128 / 256.
constexpr uint32_t COL_R = 0, COL_S0 = 128, COL_S1 = 256, TMEM_COLS = 512;
constexpr int SEG = 2;  // chunks per segment: 24 MMAs accumulate in TMEM before a drain

// R (+)= S for this warp's 32 lanes: FP32 adds with round-to-nearest on the CUDA cores.  The
// tensor core's own FP32 accumulation is not round-to-nearest, so long K loops drift; short
// segments drained this way keep the sum at FP32 accuracy.
__device__ __forceinline__ void drain(uint32_t tm, uint32_t scol, bool first)
{
    const uint32_t lane_off = (uint32_t)(32 * (threadIdx.x / 32)) << 16;
#pragma unroll 1
    for (uint32_t cc = 0; cc < 128; cc += 32) {
        float sv[32];
        tmem_ld32(tm + lane_off + scol + cc, sv);
        if (!first) {
            float rv[32];
            tmem_ld32(tm + lane_off + COL_R + cc, rv);
#pragma unroll
            for (int i = 0; i < 32; ++i) sv[i] += rv[i];
        }
        tmem_st32(tm + lane_off + COL_R + cc, sv);
    }
}

// K loop: nchunks chunks; fa(c, r, q) / fb(c, r, q) return the float4 of row r, K columns
// 4q..4q+3 of chunk c.  The result is left in tensor-memory columns COL_R .. COL_R + 127.
// Returns false if an mbarrier wait gave up (the caller flags an error).
template <class FA, class FB>
__device__ bool tc_kloop(int nchunks, FA fa, FB fb, TcSmem& sm, uint64_t* bars, uint32_t tm)
{
    const int r = threadIdx.x;  // this thread's row of A and of B
    float4 ra[KC / 4], rb[KC / 4];
    bool ok = true;
    if (nchunks > 0) {
#pragma unroll
        for (int q = 0; q < KC / 4; ++q) { ra[q] = fa(0, r, q); rb[q] = fb(0, r, q); }
    }
    for (int c = 0; c < nchunks; ++c) {
        const int st = c & 1, seg = c / SEG, pos = c % SEG;
        if (c >= 2) ok &= mbar_wait(&bars[st], ((c - 2) >> 1) & 1);  // MMAs of chunk c-2 done: stage free
        if (pos == 1 && seg >= 1) {
            // chunk c-2 closed segment seg-1 (SEG == 2): fold it into R while segment seg runs
            fence_after();
            drain(tm, (seg - 1) & 1 ? COL_S1 : COL_S0, seg == 1);
            fence_before();
        }
#pragma unroll
        for (int q = 0; q < KC / 4; ++q) {
            put4(sm.buf[st][0], sm.buf[st][1], r, q, ra[q]);
            put4(sm.buf[st][2], sm.buf[st][3], r, q, rb[q]);
        }
        if (c + 1 < nchunks) {
#pragma unroll
            for (int q = 0; q < KC / 4; ++q) { ra[q] = fa(c + 1, r, q); rb[q] = fb(c + 1, r, q); }
        }
        fence_proxy_async();
        __syncthreads();
        if (threadIdx.x == 0) {
            fence_after();
            const uint32_t acc_col = (seg & 1) ? COL_S1 : COL_S0;
            const uint32_t ah = smem_u32(sm.buf[st][0]), al = smem_u32(sm.buf[st][1]);
            const uint32_t bh = smem_u32(sm.buf[st][2]), bl = smem_u32(sm.buf[st][3]);
#pragma unroll
            for (int kk = 0; kk < KC / 8; ++kk) {
                const uint32_t off = kk * 2 * LBO;
                const uint32_t first = (pos == 0 && kk == 0) ? 0u : 1u;
                mma_tf32(tm + acc_col, smem_desc(al + off, LBO, SBO), smem_desc(bh + off, LBO, SBO), IDESC, first);
                mma_tf32(tm + acc_col, smem_desc(ah + off, LBO, SBO), smem_desc(bl + off, LBO, SBO), IDESC, 1u);
                mma_tf32(tm + acc_col, smem_desc(ah + off, LBO, SBO), smem_desc(bh + off, LBO, SBO), IDESC, 1u);
            }
            mma_commit(&bars[st]);
        }
    }
    // wait for the last chunk (its commit tracks every earlier MMA too) and fold the open segment(s)
    if (nchunks > 0) {
        ok &= mbar_wait(&bars[(nchunks - 1) & 1], ((nchunks - 1) >> 1) & 1);
        fence_after();
        const int last_seg = (nchunks - 1) / SEG;
        const int last_pos = (nchunks - 1) % SEG;
        if (last_seg >= 1 && last_pos == 0) {
            // segment last_seg-1 was closed by chunk nchunks-2 but not drained yet (no chunk at pos 1 followed)
            drain(tm, (last_seg - 1) & 1 ? COL_S1 : COL_S0, last_seg == 1);
        }
        drain(tm, last_seg & 1 ? COL_S1 : COL_S0, last_seg == 0);
        fence_before();
    }
    return ok;
}

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// element (r, m..m+3) of a column-major 64x64 tile: four loads, each coalesced across the warp's rows
__device__ __forceinline__ float4 ld4_col(const float* t, int r, int m)
{
    return make_float4(t[r + TS * m], t[r + TS * (m + 1)], t[r + TS * (m + 2)], t[r + TS * (m + 3)]);
}

constexpr float4 kZero4 = {0.f, 0.f, 0.f, 0.f};
constexpr int LINV = 128 * 128;  // floats per 128x128 diagonal-block inverse

// the accumulator row this thread holds in TMEM (warp w: lanes 32w..32w+31)
__device__ __forceinline__ uint32_t lane_base() { return (uint32_t)(32 * (threadIdx.x / 32)) << 16; }

// write the 128x128 result in R (times sgn) into the four column-major tiles of supertile (I2, J2)
// (skipping the tile above the diagonal of a diagonal supertile)
__device__ __forceinline__ void store_block(uint32_t tm, float* base, int I2, int J2, float sgn)
{
    const int row = threadIdx.x;
    for (int cc = 0; cc < 128; cc += 32) {
        float v[32];
        tmem_ld32(tm + lane_base() + COL_R + cc, v);
        const int ti = 2 * I2 + row / 64, tj = 2 * J2 + cc / 64;
        if (tj > ti) continue;
        float* t = base + (size_t)tile_index(ti, tj) * TILE_ELEMS;
#pragma unroll
        for (int i = 0; i < 32; ++i) t[(row % 64) + TS * ((cc % 64) + i)] = sgn * v[i];
    }
}

struct TcCtl {
    uint64_t bars[2];
    uint32_t tbase;
    int bad;
};

__device__ __forceinline__ uint32_t tc_begin(TcCtl& ctl)
{
    if (threadIdx.x < 32) tmem_alloc(&ctl.tbase, TMEM_COLS);
    if (threadIdx.x == 0) {
        mbar_init(&ctl.bars[0], 1);
        mbar_init(&ctl.bars[1], 1);
        ctl.bad = 0;
    }
    fence_before();
    __syncthreads();
    fence_after();
    return ctl.tbase;
}

__device__ __forceinline__ void tc_end(uint32_t tm)
{
    fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tmem_dealloc(tm, TMEM_COLS);
}

// re-arm the two stage barriers for a second K loop in the same CTA (all earlier MMAs completed)
__device__ __forceinline__ void tc_rearm(TcCtl& ctl)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&ctl.bars[0])));
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&ctl.bars[1])));
        mbar_init(&ctl.bars[0], 1);
        mbar_init(&ctl.bars[1], 1);
    }
    __syncthreads();
}

// Cholesky of the 128x128 block in s (column-major, leading dimension 129, lower part used)
// and the inverse of its factor into inv (same layout); 128 threads.  Sets *bad on a
// non-positive pivot.
__device__ void factor_block128(float* s, float* inv, int* bad)
{
    constexpr int L = 129;
    const int t = threadIdx.x;
    for (int c = 0; c < 128; ++c) {
        if (t == 0) {
            float v = s[c * L + c];
            if (!(v > 0.f)) { *bad = 1; v = 1.f; }
            s[c * L + c] = sqrtf(v);
        }
        __syncthreads();
        const float piv = s[c * L + c];
        if (t > c) s[c * L + t] /= piv;
        __syncthreads();
        if (t > c) {  // column q = t of the trailing block: rows r >= q
            const float lq = s[c * L + t];
            for (int r = t; r < 128; ++r) s[t * L + r] -= s[c * L + r] * lq;
        }
        __syncthreads();
    }
    // column t of the inverse by forward substitution
    for (int r = 0; r < 128; ++r) {
        if (r < t) { inv[t * L + r] = 0.f; continue; }
        float acc = (r == t) ? 1.f : 0.f;
        for (int m = t; m < r; ++m) acc -= s[m * L + r] * inv[t * L + m];
        inv[t * L + r] = acc / s[r * L + r];
    }
    __syncthreads();
}

// Left-looking Cholesky, column block J2, row block I2 = J2 + blockIdx.x; grid (nt2 - J2, B).
// Off-diagonal blocks: A_IJ <- A_IJ - sum_{k < 2 J2} L_I,k L_J,k^T (S, stored in place).
// Diagonal block: S_JJ factorised to L_JJ (in place), its diagonal to diag, its inverse to Linv.
__global__ void __launch_bounds__(128) chol_tc_update(int J2, int nt, float* __restrict__ A, size_t strideA,
                                                      float* __restrict__ Linv, float* __restrict__ diag,
                                                      int* __restrict__ status, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
    __shared__ TcCtl ctl;
    const int I2 = J2 + blockIdx.x, b = blockIdx.y, nt2 = nt / 2;
    float* Ab = A + (size_t)b * strideA;
    const uint32_t tm = tc_begin(ctl);
    const int nchunks = 2 * J2 * (TS / KC);
    auto fa = [&](int c, int r, int q) -> float4 {
        const float* t = Ab + (size_t)tile_index(2 * I2 + r / 64, c / 2) * TILE_ELEMS;
        return ld4_col(t, r % 64, (c % 2) * KC + 4 * q);
    };
    auto fb = [&](int c, int r, int q) -> float4 {
        const float* t = Ab + (size_t)tile_index(2 * J2 + r / 64, c / 2) * TILE_ELEMS;
        return ld4_col(t, r % 64, (c % 2) * KC + 4 * q);
    };
    bool ok = true;
    if (nchunks > 0) ok = tc_kloop(nchunks, fa, fb, sm, ctl.bars, tm);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    const int row = threadIdx.x;
    if (I2 > J2) {
        if (nchunks > 0) {
            for (int cc = 0; cc < 128; cc += 32) {
                float v[32];
                tmem_ld32(tm + lane_base() + COL_R + cc, v);
                float* t = Ab + (size_t)tile_index(2 * I2 + row / 64, 2 * J2 + cc / 64) * TILE_ELEMS;
#pragma unroll
                for (int i = 0; i < 32; ++i) t[(row % 64) + TS * ((cc % 64) + i)] -= v[i];
            }
        }
        tc_end(tm);
        return;
    }
    // diagonal block: S = A_JJ - P into shared memory (column-major, ld 129), lower part
    float* s = reinterpret_cast<float*>(smem_raw);
    float* inv = s + 128 * 129;
    __syncthreads();
    for (int cc = 0; cc < 128; cc += 32) {
        float v[32];
        if (nchunks > 0) tmem_ld32(tm + lane_base() + COL_R + cc, v);
        else {
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = 0.f;
        }
        const int ti = 2 * J2 + row / 64, tj = 2 * J2 + cc / 64;
        if (tj > ti) continue;
        const float* t = Ab + (size_t)tile_index(ti, tj) * TILE_ELEMS;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            const int col = cc + i;
            s[col * 129 + row] = t[(row % 64) + TS * (col % 64)] - v[i];
        }
    }
    __syncthreads();
    factor_block128(s, inv, &ctl.bad);
    // L_JJ into the three lower tiles (strict upper of the diagonal tiles zeroed), diag, Linv row-major
    for (int col = 0; col < 128; ++col) {
        const int ti = 2 * J2 + row / 64, tj = 2 * J2 + col / 64;
        if (tj > ti) continue;
        float* t = Ab + (size_t)tile_index(ti, tj) * TILE_ELEMS;
        t[(row % 64) + TS * (col % 64)] = (row >= col) ? s[col * 129 + row] : 0.f;
    }
    diag[(size_t)b * nt * TS + J2 * 128 + row] = s[row * 129 + row];
    float* li = Linv + ((size_t)b * nt2 + J2) * LINV;
    for (int col = 0; col < 128; ++col) li[row * 128 + col] = inv[col * 129 + row];
    if (threadIdx.x == 0 && ctl.bad && status && status[b] == CG_OK) status[b] = CG_ERR_NOT_PD;
    tc_end(tm);
}

// L_IJ = S_IJ Linv_J^T for I2 = J2 + 1 + blockIdx.x; grid (nt2 - J2 - 1, B)
__global__ void __launch_bounds__(128) chol_tc_panel(int J2, int nt, float* __restrict__ A, size_t strideA,
                                                     const float* __restrict__ Linv, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
    __shared__ TcCtl ctl;
    const int I2 = J2 + 1 + blockIdx.x, b = blockIdx.y, nt2 = nt / 2;
    float* Ab = A + (size_t)b * strideA;
    const float* li = Linv + ((size_t)b * nt2 + J2) * LINV;
    const uint32_t tm = tc_begin(ctl);
    // A(r, m) = S(r, m): block column m/64 of row block I2; B(c, m) = Linv(c, m) row-major
    auto fa = [&](int c, int r, int q) -> float4 {
        const int m = c * KC + 4 * q;
        const float* t = Ab + (size_t)tile_index(2 * I2 + r / 64, 2 * J2 + m / 64) * TILE_ELEMS;
        return ld4_col(t, r % 64, m % 64);
    };
    auto fb = [&](int c, int r, int q) -> float4 { return ld4(li + r * 128 + c * KC + 4 * q); };
    const bool ok = tc_kloop(128 / KC, fa, fb, sm, ctl.bars, tm);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    __syncthreads();  // every S read is done before the tiles are overwritten
    store_block(tm, Ab, I2, J2, 1.f);
    tc_end(tm);
}

// Row block I2 of M = L^-1; CTA J2 = blockIdx.x <= I2; grid (I2 + 1, B)
__global__ void __launch_bounds__(128) trtri_tc_row(int I2, int nt, const float* __restrict__ Lm,
                                                    const float* __restrict__ Linv, float* __restrict__ M,
                                                    size_t strideA, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
    __shared__ TcCtl ctl;
    const int J2 = blockIdx.x, b = blockIdx.y, nt2 = nt / 2;
    const float* Lb = Lm + (size_t)b * strideA;
    float* Mb = M + (size_t)b * strideA;
    const float* li = Linv + ((size_t)b * nt2 + I2) * LINV;
    const int row = threadIdx.x;
    if (J2 == I2) {  // M_II = Linv_I, into the three lower column-major tiles
        for (int col = 0; col < 128; ++col) {
            const int ti = 2 * I2 + row / 64, tj = 2 * I2 + col / 64;
            if (tj > ti) continue;
            Mb[(size_t)tile_index(ti, tj) * TILE_ELEMS + (row % 64) + TS * (col % 64)] = li[row * 128 + col];
        }
        return;
    }
    const uint32_t tm = tc_begin(ctl);
    // S = sum_{k=2 J2}^{2 I2 - 1} L_{I,k} M_{k,J}: A(r, m) = L tile (2 I2 + r/64, k)(r%64, m) column-major,
    // B(c, m) = M tile (k, 2 J2 + c/64)(m, c%64) column-major -> contiguous in m for fixed c
    const int k0 = 2 * J2;
    const int nchunks = (2 * I2 - k0) * (TS / KC);
    auto fa = [&](int c, int r, int q) -> float4 {
        const int k = k0 + c / 2;
        const float* t = Lb + (size_t)tile_index(2 * I2 + r / 64, k) * TILE_ELEMS;
        return ld4_col(t, r % 64, (c % 2) * KC + 4 * q);
    };
    auto fb = [&](int c, int r, int q) -> float4 {
        const int k = k0 + c / 2, col = 2 * J2 + r / 64;
        if (k < col) return kZero4;
        const float* t = Mb + (size_t)tile_index(k, col) * TILE_ELEMS;
        return ld4(t + (r % 64) * TS + (c % 2) * KC + 4 * q);
    };
    bool ok = tc_kloop(nchunks, fa, fb, sm, ctl.bars, tm);
    // S into the M tiles of block (I2, J2) (not read by any other block of this launch)
    store_block(tm, Mb, I2, J2, 1.f);
    __syncthreads();
    tc_rearm(ctl);
    // M_IJ = -Linv_I S: A(r, m) = Linv(r, m) row-major; B(c, m) = S(m, c) column-major tiles
    auto fa2 = [&](int c, int r, int q) -> float4 { return ld4(li + r * 128 + c * KC + 4 * q); };
    auto fb2 = [&](int c, int r, int q) -> float4 {
        // S was written by this kernel: coherent L2 loads, not the read-only path
        const int m = c * KC + 4 * q;
        const float* t = Mb + (size_t)tile_index(2 * I2 + m / 64, 2 * J2 + r / 64) * TILE_ELEMS;
        return __ldcg(reinterpret_cast<const float4*>(t + (r % 64) * TS + (m % 64)));
    };
    ok &= tc_kloop(128 / KC, fa2, fb2, sm, ctl.bars, tm);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    __syncthreads();
    store_block(tm, Mb, I2, J2, -1.f);
    tc_end(tm);
}


// V_IJ (128x128 supertile, lower) = sum over k of M_k,I^T M_k,J with M column-major tiles.
// grid (supertiles of the lower triangle, B), 128 threads.
__global__ void __launch_bounds__(128) lauum_tc(int nt, const float* __restrict__ M, float* __restrict__ V,
                                                size_t strideA, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
    __shared__ uint64_t bars[2];
    __shared__ uint32_t tbase;
    int I2, J2;
    tile_coords(blockIdx.x, I2, J2);
    const int b = blockIdx.y;
    const float* Mb = M + (size_t)b * strideA;
    if (threadIdx.x < 32) tmem_alloc(&tbase, TMEM_COLS);
    if (threadIdx.x == 0) { mbar_init(&bars[0], 1); mbar_init(&bars[1], 1); }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = tbase;
    const int k0 = 2 * I2;                     // first tile row with a non-zero M_k,row
    const int nchunks = (nt - k0) * (TS / KC);
    // A(r, m) = M_{k, 2I2 + r/64}(m, r%64): tile (k, col) column-major, element (m, r') at m + 64 r'
    auto fa = [&](int c, int r, int q) -> float4 {
        const int k = k0 + c / 2, col = 2 * I2 + r / 64;
        if (k < col) return make_float4(0.f, 0.f, 0.f, 0.f);
        const float* t = Mb + (size_t)tile_index(k, col) * TILE_ELEMS;
        return ld4(t + (r % 64) * TS + (c % 2) * KC + 4 * q);
    };
    auto fb = [&](int c, int r, int q) -> float4 {
        const int k = k0 + c / 2, col = 2 * J2 + r / 64;
        if (k < col) return make_float4(0.f, 0.f, 0.f, 0.f);
        const float* t = Mb + (size_t)tile_index(k, col) * TILE_ELEMS;
        return ld4(t + (r % 64) * TS + (c % 2) * KC + 4 * q);
    };
    const bool ok = tc_kloop(nchunks, fa, fb, sm, bars, tm);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    // epilogue: warp w holds rows 32w..32w+31; write column-major tiles (coalesced per column)
    const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int row = 32 * w + lane;
    float* Vb = V + (size_t)b * strideA;
    for (int cc = 0; cc < 128; cc += 32) {
        float v[32];
        tmem_ld32(tm + ((uint32_t)(32 * w) << 16) + COL_R + cc, v);
        const int ti = 2 * I2 + row / 64, tj = 2 * J2 + cc / 64;
        if (tj > ti) continue;  // above the diagonal of a diagonal supertile
        float* t = Vb + (size_t)tile_index(ti, tj) * TILE_ELEMS;
#pragma unroll
        for (int i = 0; i < 32; ++i) t[(row % 64) + TS * ((cc % 64) + i)] = v[i];
    }
    fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tmem_dealloc(tm, TMEM_COLS);
}

}  // namespace

static size_t tc_smem() { return sizeof(TcSmem) > 2 * 128 * 129 * 4 ? sizeof(TcSmem) : 2 * 128 * 129 * 4; }

int tiled_cholesky_tc(cg_ctx* ctx, int B, int nt, float* A, float* Linv, float* diag, int* status, size_t strideA,
                      int* d_err, cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core Cholesky needs an even tile count"; return CG_ERR_BAD_ARG; }
    const int smem = (int)tc_smem() + 1024;
    static bool attr = false;
    if (!attr) {
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(chol_tc_update, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(chol_tc_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const int nt2 = nt / 2;
    for (int J2 = 0; J2 < nt2; ++J2) {
        chol_tc_update<<<dim3(nt2 - J2, B), 128, smem, s>>>(J2, nt, A, strideA, Linv, diag, status, d_err);
        count_launch(ctx);
        if (J2 + 1 < nt2) {
            chol_tc_panel<<<dim3(nt2 - J2 - 1, B), 128, smem, s>>>(J2, nt, A, strideA, Linv, d_err);
            count_launch(ctx);
        }
    }
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int tiled_trtri_tc(cg_ctx* ctx, int B, int nt, const float* L, const float* Linv, float* M, size_t strideA, int* d_err,
                   cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core trtri needs an even tile count"; return CG_ERR_BAD_ARG; }
    const int smem = (int)tc_smem() + 1024;
    static bool attr = false;
    if (!attr) {
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(trtri_tc_row, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const int nt2 = nt / 2;
    for (int I2 = 0; I2 < nt2; ++I2) {
        trtri_tc_row<<<dim3(I2 + 1, B), 128, smem, s>>>(I2, nt, L, Linv, M, strideA, d_err);
        count_launch(ctx);
    }
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int tiled_lauum_tc(cg_ctx* ctx, int B, int nt, const float* M, float* V, size_t strideA, int* d_err, cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core lauum needs an even tile count"; return CG_ERR_BAD_ARG; }
    const int smem = (int)sizeof(TcSmem) + 1024;
    static bool attr = false;
    if (!attr) {
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(lauum_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const int nt2 = nt / 2;
    lauum_tc<<<dim3(nt2 * (nt2 + 1) / 2, B), 128, smem, s>>>(nt, M, V, strideA, d_err);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
