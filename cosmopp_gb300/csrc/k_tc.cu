// Tensor-core (tcgen05, kind::tf32) tile products for the FP32 whitened
// matrices of the mixed path, at FP32 accuracy by the 3xTF32 split
// a*b ~ a_hi*b_hi + a_hi*b_lo + a_lo*b_hi with a_hi = a rounded to nearest TF32
// and a_lo = a - a_hi rounded to nearest TF32 (unbiased; truncating instead
// biases sums of squares).  The tensor core's FP32 accumulation is not
// round-to-nearest and drifts by ~0.4 ulp per instruction, always the same
// way, so each chunk's hi*hi products (4 MMAs) go to a fresh tensor-memory
// accumulator that is folded into a per-thread FP32 register sum
// (round-to-nearest) one chunk later.  The correction products (8 MMAs per
// chunk) are ~2^-11 of the sum, so their drift is negligible and they
// accumulate in one tensor-memory accumulator over the whole K loop.
//
// One CTA (256 threads) owns a 128x128 output supertile (2x2 of the 64x64
// storage tiles) and runs a K loop over 32-wide chunks.  Thread t loads row
// t % 128, K half t / 128 of the A and B chunks into registers two chunks
// ahead; A is split hi/lo straight into tensor memory (tcgen05.st, lane = row),
// B into a double-buffered shared-memory stage in the K-major canonical layout.
// One thread issues the 12 MMAs (M128 N128 K8, A from tensor memory) of a chunk
// and commits them to the stage's mbarrier.  Keeping A out of shared memory
// removes its stores and the MMAs' re-reads of it there (shared-memory bandwidth
// bounds this loop).
//
//   chol_tc_update: left-looking Cholesky, column block J: S_IJ = A_IJ - sum_{k<J} L_Ik L_Jk^T;
//                   the diagonal CTA factors S_JJ = L_JJ L_JJ^T and inverts L_JJ in shared memory
//   chol_tc_panel:  L_IJ = S_IJ L_JJ^-T                        (I > J)
//   trtri_tc_row:   M_IJ = -L_II^-1 sum_{k=J}^{I-1} L_Ik M_kJ, M_II = L_II^-1   (M = L^-1)
//   lauum_tc:       V_IJ = sum_{k >= row} M_kI^T M_kJ = (L L^T)^-1
// (I, J in 128-row blocks; A, L and V in 64x64 column-major storage tiles, M in
// transposed (row-major) tiles and the 128x128 inverses of L's diagonal blocks
// column-major in Linv.  With these layouts every operand the K loops read has
// element (r, k) at r + ld k: consecutive threads (rows) read consecutive words.)
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
    float buf[2][2][STAGE_FLOATS];         // [stage][b_hi, b_lo]
};

// stores one float4 (row r, K columns 4q..4q+3 of the chunk) as hi and lo parts
__device__ __forceinline__ void put4(float* hi, float* lo, int r, int q, float4 v)
{
    const uint32_t o = kmajor_offset(r, 4 * q, KC) / 4;
    const float4 h = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
    *reinterpret_cast<float4*>(hi + o) = h;
    *reinterpret_cast<float4*>(lo + o) =
        make_float4(tf32_rn(v.x - h.x), tf32_rn(v.y - h.y), tf32_rn(v.z - h.z), tf32_rn(v.w - h.w));
}

// Tensor-memory columns (512): hi*hi accumulators for the two chunk parities, the correction
// accumulator, and the A operand (hi, lo) of the two stages.
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_CORR = 256;
__device__ __forceinline__ uint32_t col_main(int set) { return 128u * set; }
__device__ __forceinline__ uint32_t col_a_hi(int st) { return 384u + 64u * st; }
__device__ __forceinline__ uint32_t col_a_lo(int st) { return 384u + 64u * st + 32u; }

// the accumulator row this thread holds in TMEM (warp w: lanes 32 (w % 4) .. + 31)
__device__ __forceinline__ uint32_t lane_base() { return (uint32_t)(32 * ((threadIdx.x / 32) % 4)) << 16; }

// R[j] += accumulator at column col of this thread's row, columns 64 (t / 128) + j
__device__ __forceinline__ void drain(uint32_t tm, uint32_t col, float (&R)[64])
{
    const uint32_t c0 = 64 * (threadIdx.x / 128);
#pragma unroll
    for (int part = 0; part < 4; ++part) {
        float m[16];
        tmem_ld16(tm + lane_base() + col + c0 + 16 * part, m);
#pragma unroll
        for (int i = 0; i < 16; ++i) R[16 * part + i] += m[i];
    }
}

constexpr int NTH = 256;  // threads per CTA: row r = t % 128, K half h = t / 128 (q in 4h .. 4h+3)

// K loop: nchunks chunks; fa(c, r, q) / fb(c, r, q) return the float4 of row r, K columns
// 4q..4q+3 of chunk c.  Loads run two chunks ahead of the MMAs.  On return R[j] holds the
// product for row t % 128, column 64 (t / 128) + j (0 if nchunks == 0).  Returns false if an
// mbarrier wait gave up.
template <class FA, class FB>
__device__ bool tc_kloop(int nchunks, FA fa, FB fb, TcSmem& sm, uint64_t* bars, uint32_t tm, float (&R)[64])
{
    const int r = threadIdx.x % 128, h = threadIdx.x / 128;
#pragma unroll
    for (int j = 0; j < 64; ++j) R[j] = 0.f;
    float4 pa0[4], pb0[4], pa1[4], pb1[4];
    bool ok = true;
    if (nchunks > 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) { pa0[q] = fa(0, r, 4 * h + q); pb0[q] = fb(0, r, 4 * h + q); }
    }
    if (nchunks > 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q) { pa1[q] = fa(1, r, 4 * h + q); pb1[q] = fb(1, r, 4 * h + q); }
    }
    auto step = [&](int c, float4 (&qa)[4], float4 (&qb)[4]) {
        const int st = c & 1;
        if (c >= 2) {
            // MMAs of chunk c-2 done: its A columns and B stage are free, its hi*hi sum goes to R
            ok &= mbar_wait(&bars[st], ((c - 2) >> 1) & 1);
            fence_after();
            drain(tm, col_main(st), R);
        }
        {
            float ahi[16], alo[16];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float v[4] = {qa[q].x, qa[q].y, qa[q].z, qa[q].w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    ahi[4 * q + i] = tf32_rn(v[i]);
                    alo[4 * q + i] = tf32_rn(v[i] - ahi[4 * q + i]);
                }
            }
            tmem_st16(tm + lane_base() + col_a_hi(st) + 16 * h, ahi);
            tmem_st16(tm + lane_base() + col_a_lo(st) + 16 * h, alo);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) put4(sm.buf[st][0], sm.buf[st][1], r, 4 * h + q, qb[q]);
        if (c + 2 < nchunks) {
#pragma unroll
            for (int q = 0; q < 4; ++q) { qa[q] = fa(c + 2, r, 4 * h + q); qb[q] = fb(c + 2, r, 4 * h + q); }
        }
        tmem_wait_st();
        fence_proxy_async();
        fence_before();
        __syncthreads();
        if (threadIdx.x == 0) {
            fence_after();
            const uint32_t bh = smem_u32(sm.buf[st][0]), bl = smem_u32(sm.buf[st][1]);
            const uint32_t ah = tm + col_a_hi(st), al = tm + col_a_lo(st);
#pragma unroll
            for (int kk = 0; kk < KC / 8; ++kk) {
                const uint32_t off = kk * 2 * LBO;
                mma_tf32_ta(tm + COL_CORR, al + 8 * kk, smem_desc(bh + off, LBO, SBO), IDESC, (c | kk) ? 1u : 0u);
                mma_tf32_ta(tm + COL_CORR, ah + 8 * kk, smem_desc(bl + off, LBO, SBO), IDESC, 1u);
                mma_tf32_ta(tm + col_main(st), ah + 8 * kk, smem_desc(bh + off, LBO, SBO), IDESC, kk ? 1u : 0u);
            }
            mma_commit(&bars[st]);
        }
    };
    for (int c = 0; c < nchunks; c += 2) {
        step(c, pa0, pb0);
        if (c + 1 < nchunks) step(c + 1, pa1, pb1);
    }
    // the last one or two chunks and the corrections: wait for the last commit (it tracks every
    // earlier MMA) and fold
    if (nchunks > 0) {
        ok &= mbar_wait(&bars[(nchunks - 1) & 1], ((nchunks - 1) >> 1) & 1);
        fence_after();
        if (nchunks >= 2) drain(tm, col_main((nchunks - 2) & 1), R);
        drain(tm, col_main((nchunks - 1) & 1), R);
        drain(tm, COL_CORR, R);
        fence_before();
    }
    return ok;
}

// element (r, m..m+3) of a column-major 64x64 tile (or of the transpose of a row-major one): four
// loads, each coalesced across the warp's rows
__device__ __forceinline__ float4 ld4_col(const float* t, int r, int m)
{
    return make_float4(t[r + TS * m], t[r + TS * (m + 1)], t[r + TS * (m + 2)], t[r + TS * (m + 3)]);
}

// the same for data written earlier in the same kernel: coherent L2 loads, not the read-only path
__device__ __forceinline__ float4 ld4_col_cg(const float* t, int r, int m)
{
    return make_float4(__ldcg(t + r + TS * m), __ldcg(t + r + TS * (m + 1)), __ldcg(t + r + TS * (m + 2)),
                       __ldcg(t + r + TS * (m + 3)));
}

// element (r, m..m+3) of a column-major 128x128 block (Linv)
__device__ __forceinline__ float4 ld4_linv(const float* li, int r, int m)
{
    return make_float4(li[r + 128 * m], li[r + 128 * (m + 1)], li[r + 128 * (m + 2)], li[r + 128 * (m + 3)]);
}

constexpr float4 kZero4 = {0.f, 0.f, 0.f, 0.f};
constexpr int LINV = 128 * 128;  // floats per 128x128 diagonal-block inverse


// write the 128x128 result (this thread: row t % 128, columns 64 (t / 128) + j in R) times sgn
// into the column-major tiles of supertile (I2, J2), skipping the tile above the diagonal
__device__ __forceinline__ void store_block(const float (&R)[64], float* base, int I2, int J2, float sgn)
{
    const int row = threadIdx.x % 128, h = threadIdx.x / 128;
    const int ti = 2 * I2 + row / 64, tj = 2 * J2 + h;
    if (tj > ti) return;
    float* t = base + (size_t)tile_index(ti, tj) * TILE_ELEMS;
#pragma unroll
    for (int j = 0; j < 64; ++j) t[(row % 64) + TS * j] = sgn * R[j];
}

// the same into row-major (transposed) tiles: this thread's row is 64 contiguous floats
__device__ __forceinline__ void store_block_t(const float (&R)[64], float* base, int I2, int J2, float sgn)
{
    const int row = threadIdx.x % 128, h = threadIdx.x / 128;
    const int ti = 2 * I2 + row / 64, tj = 2 * J2 + h;
    if (tj > ti) return;
    float4* t = reinterpret_cast<float4*>(base + (size_t)tile_index(ti, tj) * TILE_ELEMS + (row % 64) * TS);
#pragma unroll
    for (int j = 0; j < 16; ++j)
        t[j] = make_float4(sgn * R[4 * j], sgn * R[4 * j + 1], sgn * R[4 * j + 2], sgn * R[4 * j + 3]);
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
// and the inverse of its factor into inv (same layout); 256 threads.  Panels of 8 columns
// factorised column by column, then one rank-8 update of the trailing block.  The inverse is
// block-recursive: inv11 = L11^-1, inv22 = L22^-1 (in parallel), inv21 = -inv22 (L21 inv11),
// with tmp a 64x65 scratch block.  Sets *bad on a non-positive pivot.
__device__ void factor_block128(float* s, float* inv, float* tmp, int* bad)
{
    constexpr int L = 129;
    const int t = threadIdx.x;
    // Trailing updates are summed in u (inv's storage, free until the inverse) and subtracted
    // once per column: subtracting each term from s directly drops the terms below half an
    // ulp of the diagonal (about 1 after whitening) and biases the log-determinant upwards.
    float* u = inv;
    for (int e = t; e < 128 * 128; e += NTH) u[(e / 128) * L + e % 128] = 0.f;
    __syncthreads();
    for (int kb = 0; kb < 128; kb += 8) {
        for (int c = kb; c < kb + 8; ++c) {
            if (t == 0) {
                float v = s[c * L + c] - u[c * L + c];
                if (!(v > 0.f)) { *bad = 1; v = 1.f; }
                s[c * L + c] = sqrtf(v);
            }
            __syncthreads();
            const float piv = s[c * L + c];
            if (t > c && t < 128) s[c * L + t] = (s[c * L + t] - u[c * L + t]) / piv;
            __syncthreads();
            const int nq = kb + 7 - c;  // remaining panel columns c+1 .. kb+7
            for (int e = t; e < nq * 128; e += NTH) {
                const int q = c + 1 + e / 128, rr = e % 128;
                if (rr >= q) u[q * L + rr] += s[c * L + rr] * s[c * L + q];
            }
            __syncthreads();
        }
        const int q0 = kb + 8;
        for (int e = t; e < (128 - q0) * 128; e += NTH) {
            const int q = q0 + e / 128, rr = e % 128;
            if (rr < q) continue;
            float acc = u[q * L + rr];
#pragma unroll
            for (int c = 0; c < 8; ++c) acc += s[(kb + c) * L + rr] * s[(kb + c) * L + q];
            u[q * L + rr] = acc;
        }
        __syncthreads();
    }
    // diagonal 64-blocks: thread t < 64 -> column t of L11^-1, 128 <= t < 192 -> column t-128 of L22^-1
    if (t < 64 || (t >= 128 && t < 192)) {
        const int off = (t < 64) ? 0 : 64;
        const int col = off + (t % 64);
        for (int r = off; r < off + 64; ++r) {
            if (r < col) { inv[col * L + r] = 0.f; continue; }
            float acc = (r == col) ? 1.f : 0.f;
            for (int m = col; m < r; ++m) acc -= s[m * L + r] * inv[col * L + m];
            inv[col * L + r] = acc / s[r * L + r];
        }
    }
    __syncthreads();
    // tmp = L21 inv11 (rows 64..127, cols 0..63 of L times inv11)
    for (int e = t; e < 64 * 64; e += NTH) {
        const int rr = e % 64, cc = e / 64;
        float acc = 0.f;
        for (int m = cc; m < 64; ++m) acc += s[m * L + 64 + rr] * inv[cc * L + m];
        tmp[cc * 65 + rr] = acc;
    }
    __syncthreads();
    // inv21 = -inv22 tmp; inv12 = 0
    for (int e = t; e < 64 * 64; e += NTH) {
        const int rr = e % 64, cc = e / 64;
        float acc = 0.f;
        for (int m = 0; m <= rr; ++m) acc += inv[(64 + m) * L + 64 + rr] * tmp[cc * 65 + m];
        inv[cc * L + 64 + rr] = -acc;
        inv[(64 + cc) * L + rr] = 0.f;
    }
    __syncthreads();
}

// Left-looking Cholesky, column block J2, row block I2 = J2 + blockIdx.x; grid (nt2 - J2, B).
// Off-diagonal blocks: A_IJ <- A_IJ - sum_{k < 2 J2} L_I,k L_J,k^T (S, stored in place).
// Diagonal block: S_JJ factorised to L_JJ (in place), its diagonal to diag, its inverse to Linv.
__global__ void __launch_bounds__(NTH) chol_tc_update(int J2, int nt, float* __restrict__ A, size_t strideA,
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
    float R[64];
    const bool ok = tc_kloop(nchunks, fa, fb, sm, ctl.bars, tm, R);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    const int row = threadIdx.x % 128, c0 = 64 * (threadIdx.x / 128);
    if (I2 > J2) {
        if (nchunks > 0) {
            float* t = Ab + (size_t)tile_index(2 * I2 + row / 64, 2 * J2 + c0 / 64) * TILE_ELEMS;
#pragma unroll
            for (int j = 0; j < 64; ++j) t[(row % 64) + TS * j] -= R[j];
        }
        tc_end(tm);
        return;
    }
    // diagonal block: S = A_JJ - P into shared memory (column-major, ld 129), lower part
    float* s = reinterpret_cast<float*>(smem_raw);
    float* inv = s + 128 * 129;
    float* tmp = inv + 128 * 129;
    __syncthreads();
    {
        const int ti = 2 * J2 + row / 64, tj = 2 * J2 + c0 / 64;
        if (tj <= ti) {
            const float* t = Ab + (size_t)tile_index(ti, tj) * TILE_ELEMS;
#pragma unroll
            for (int j = 0; j < 64; ++j) s[(c0 + j) * 129 + row] = t[(row % 64) + TS * j] - R[j];
        }
    }
    __syncthreads();
    factor_block128(s, inv, tmp, &ctl.bad);
    // L_JJ into the three lower tiles (strict upper of the diagonal tiles zeroed), diag, Linv column-major
    for (int col = c0; col < c0 + 64; ++col) {
        const int ti = 2 * J2 + row / 64, tj = 2 * J2 + col / 64;
        if (tj > ti) continue;
        float* t = Ab + (size_t)tile_index(ti, tj) * TILE_ELEMS;
        t[(row % 64) + TS * (col % 64)] = (row >= col) ? s[col * 129 + row] : 0.f;
    }
    if (threadIdx.x < 128) diag[(size_t)b * nt * TS + J2 * 128 + row] = s[row * 129 + row];
    float* li = Linv + ((size_t)b * nt2 + J2) * LINV;
    for (int col = c0; col < c0 + 64; ++col) li[col * 128 + row] = inv[col * 129 + row];
    if (threadIdx.x == 0 && ctl.bad && status && status[b] == CG_OK) status[b] = CG_ERR_NOT_PD;
    tc_end(tm);
}

// L_IJ = S_IJ Linv_J^T for I2 = J2 + 1 + blockIdx.x; grid (nt2 - J2 - 1, B)
__global__ void __launch_bounds__(NTH) chol_tc_panel(int J2, int nt, float* __restrict__ A, size_t strideA,
                                                     const float* __restrict__ Linv, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
    __shared__ TcCtl ctl;
    const int I2 = J2 + 1 + blockIdx.x, b = blockIdx.y, nt2 = nt / 2;
    float* Ab = A + (size_t)b * strideA;
    const float* li = Linv + ((size_t)b * nt2 + J2) * LINV;
    const uint32_t tm = tc_begin(ctl);
    // A(r, m) = S(r, m): block column m/64 of row block I2; B(c, m) = Linv(c, m) column-major
    auto fa = [&](int c, int r, int q) -> float4 {
        const int m = c * KC + 4 * q;
        const float* t = Ab + (size_t)tile_index(2 * I2 + r / 64, 2 * J2 + m / 64) * TILE_ELEMS;
        return ld4_col(t, r % 64, m % 64);
    };
    auto fb = [&](int c, int r, int q) -> float4 { return ld4_linv(li, r, c * KC + 4 * q); };
    float R[64];
    const bool ok = tc_kloop(128 / KC, fa, fb, sm, ctl.bars, tm, R);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    __syncthreads();  // every S read is done before the tiles are overwritten
    store_block(R, Ab, I2, J2, 1.f);
    tc_end(tm);
}

// Row block I2 of M = L^-1; CTA J2 = blockIdx.x <= I2; grid (I2 + 1, B)
__global__ void __launch_bounds__(NTH) trtri_tc_row(int I2, int nt, const float* __restrict__ Lm,
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
    const int row = threadIdx.x % 128, c0 = 64 * (threadIdx.x / 128);
    if (J2 == I2) {  // M_II = Linv_I, into the three lower row-major tiles
        for (int col = c0; col < c0 + 64; ++col) {
            const int ti = 2 * I2 + row / 64, tj = 2 * I2 + col / 64;
            if (tj > ti) continue;
            Mb[(size_t)tile_index(ti, tj) * TILE_ELEMS + (row % 64) * TS + (col % 64)] = li[col * 128 + row];
        }
        return;
    }
    const uint32_t tm = tc_begin(ctl);
    // S = sum_{k=2 J2}^{2 I2 - 1} L_{I,k} M_{k,J}: A(r, m) = L tile (2 I2 + r/64, k)(r%64, m) column-major,
    // B(c, m) = M tile (k, 2 J2 + c/64)(m, c%64) row-major, at c%64 + 64 m
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
        return ld4_col(t, r % 64, (c % 2) * KC + 4 * q);
    };
    float R[64];
    bool ok = tc_kloop(nchunks, fa, fb, sm, ctl.bars, tm, R);
    // S into the M tiles of block (I2, J2) (not read by any other block of this launch)
    store_block_t(R, Mb, I2, J2, 1.f);
    __syncthreads();
    tc_rearm(ctl);
    // M_IJ = -Linv_I S: A(r, m) = Linv(r, m) column-major; B(c, m) = S(m, c), row-major tiles
    auto fa2 = [&](int c, int r, int q) -> float4 { return ld4_linv(li, r, c * KC + 4 * q); };
    auto fb2 = [&](int c, int r, int q) -> float4 {
        const int m = c * KC + 4 * q;
        const float* t = Mb + (size_t)tile_index(2 * I2 + m / 64, 2 * J2 + r / 64) * TILE_ELEMS;
        return ld4_col_cg(t, r % 64, m % 64);
    };
    ok &= tc_kloop(128 / KC, fa2, fb2, sm, ctl.bars, tm, R);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    __syncthreads();
    store_block_t(R, Mb, I2, J2, -1.f);
    tc_end(tm);
}


// V_IJ (128x128 supertile, lower) = sum over k of M_k,I^T M_k,J with M in row-major tiles; V in
// column-major tiles.
// grid (supertiles of the lower triangle, B), 256 threads.
__global__ void __launch_bounds__(NTH) lauum_tc(int nt, const float* __restrict__ M, float* __restrict__ V,
                                                size_t strideA, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TcSmem& sm = *reinterpret_cast<TcSmem*>(smem_raw);
    __shared__ TcCtl ctl;
    int I2, J2;
    tile_coords(blockIdx.x, I2, J2);
    const int b = blockIdx.y;
    const float* Mb = M + (size_t)b * strideA;
    const uint32_t tm = tc_begin(ctl);
    const int k0 = 2 * I2;                     // first tile row with a non-zero M_k,row
    const int nchunks = (nt - k0) * (TS / KC);
    // A(r, m) = M_{k, 2I2 + r/64}(m, r%64): tile (k, col) row-major, element (m, r') at r' + 64 m
    auto fa = [&](int c, int r, int q) -> float4 {
        const int k = k0 + c / 2, col = 2 * I2 + r / 64;
        if (k < col) return make_float4(0.f, 0.f, 0.f, 0.f);
        const float* t = Mb + (size_t)tile_index(k, col) * TILE_ELEMS;
        return ld4_col(t, r % 64, (c % 2) * KC + 4 * q);
    };
    auto fb = [&](int c, int r, int q) -> float4 {
        const int k = k0 + c / 2, col = 2 * J2 + r / 64;
        if (k < col) return make_float4(0.f, 0.f, 0.f, 0.f);
        const float* t = Mb + (size_t)tile_index(k, col) * TILE_ELEMS;
        return ld4_col(t, r % 64, (c % 2) * KC + 4 * q);
    };
    float R[64];
    const bool ok = tc_kloop(nchunks, fa, fb, sm, ctl.bars, tm, R);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    store_block(R, V + (size_t)b * strideA, I2, J2, 1.f);
    tc_end(tm);
}

}  // namespace

static size_t tc_smem()
{
    const size_t fac = (2 * 128 * 129 + 64 * 65) * sizeof(float);  // block, its inverse, scratch
    return sizeof(TcSmem) > fac ? sizeof(TcSmem) : fac;
}

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
        chol_tc_update<<<dim3(nt2 - J2, B), NTH, smem, s>>>(J2, nt, A, strideA, Linv, diag, status, d_err);
        count_launch(ctx);
        if (J2 + 1 < nt2) {
            chol_tc_panel<<<dim3(nt2 - J2 - 1, B), NTH, smem, s>>>(J2, nt, A, strideA, Linv, d_err);
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
        trtri_tc_row<<<dim3(I2 + 1, B), NTH, smem, s>>>(I2, nt, L, Linv, M, strideA, d_err);
        count_launch(ctx);
    }
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int tiled_lauum_tc(cg_ctx* ctx, int B, int nt, const float* M, float* V, size_t strideA, int* d_err, cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core lauum needs an even tile count"; return CG_ERR_BAD_ARG; }
    const int smem = (int)tc_smem() + 1024;
    static bool attr = false;
    if (!attr) {
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(lauum_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const int nt2 = nt / 2;
    lauum_tc<<<dim3(nt2 * (nt2 + 1) / 2, B), NTH, smem, s>>>(nt, M, V, strideA, d_err);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

}  // namespace cg
