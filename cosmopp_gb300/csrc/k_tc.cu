// Tensor-core (tcgen05, kind::tf32) tile products for the FP32 whitened
// matrices of the mixed path, at FP32 accuracy by the 3xTF32 split
// a*b ~ a_hi*b_hi + a_hi*b_lo + a_lo*b_hi with a_hi = a rounded to nearest TF32
// and a_lo = a - a_hi rounded to nearest TF32 (unbiased; truncating instead
// biases sums of squares).  The tensor core's FP32 accumulation is not
// round-to-nearest and drifts by ~0.4 ulp per instruction, always the same
// way, so the 24 MMAs of each chunk pair (one 64-wide K tile) go to a fresh
// tensor-memory accumulator that is folded into a per-thread FP32 register sum
// (round-to-nearest) once the pair is done: the drift stays bounded by one
// tile's.  (Every K loop covers whole tiles, so its chunk count is even.)
//
// Operand storage ("split canonical", SC): every factor these kernels consume
// is stored already split, hi and lo planes, each 64-row x 32-K block in the
// MMA's K-major no-swizzle canonical layout (8-row x 16-byte core matrices,
// LBO 128 B along K, SBO 1024 B between row groups).  An SC tile (64 x 64) is
// [plane][K chunk][64 x 32 block] = 32 KB; two tiles stacked vertically give
// the 128-row operand block of one chunk.  So the B operand of a chunk is four
// (or two) contiguous bulk copies (cp.async.bulk) straight into shared memory,
// and the A operand is eight coalesced 16-byte loads per thread that go
// unchanged into tensor memory (tcgen05.st, lane = row): no per-element split
// or layout work in the K loop.
//
// One CTA owns a 128x128 output supertile (2x2 storage tiles) and runs a
// warp-specialised K loop over 32-wide chunks, the roles handing off through
// mbarriers only:
//   warps 0-7  (producers): when chunk c's MMAs are done, store the A operand of
//              chunk c + 4 into the tensor-memory stage chunk c used (four stages)
//              and, at the end of a chunk pair, fold the pair's accumulator into
//              registers and release it; thread t handles row t % 128, K half t / 128;
//   warps 8,10 (MMA issue): one thread each, for alternate chunk pairs (chunks
//              4k, 4k + 1 and 4k + 2, 4k + 3), issues a chunk's 12 MMAs (M128 N128
//              K8, A from tensor memory, B from shared memory) once its A, its B and
//              its accumulator are ready, and commits them to the stage's mbarriers.
//              Issue blocks while the tensor pipe is busy, so with one issuer the pipe
//              idled during every barrier wait; with two, one issuer waits while the
//              other's MMAs run;
//   warps 9,11 (copies): one thread each keeps a ring filled with bulk copies,
//              refilling a stage when its readers are done: warp 9 the NSTB
//              shared-memory B stages, warp 11 the NSTA A stages (for A streamed
//              through shared memory).  With one thread for both, every A copy
//              waited behind the previous chunk's B stage, which frees only when that
//              stage's MMAs complete, so A ran only a chunk or two ahead of use, short
//              of DRAM latency, and the producers waited for it (clock64 trace).
//
//   chol_tc_update: left-looking Cholesky, column block J: S_IJ = A_IJ - sum_{k<J} L_Ik L_Jk^T;
//                   the diagonal CTA factors S_JJ = L_JJ L_JJ^T, inverts L_JJ in shared memory and
//                   writes L_JJ, Linv_J = L_JJ^-1 and (M_JJ)^T = Linv_J^T
//   chol_tc_panel:  L_IJ = S_IJ Linv_J^T                       (I > J)
//   trtri_tc_row:   (M_IJ)^T = -(sum_{k=J}^{I-1} M_kJ^T L_Ik^T) Linv_I^T    (M = L^-1, I > J)
//   lauum_tc:       V_IJ = sum_{k >= I} M_kI^T M_kJ = (L L^T)^-1
// A operands that are streamed from DRAM (each read by one CTA per launch: L's row
// panels in the Cholesky, M^T's column panels in trtri) come instead from an FP32
// copy in the same canonical layout (C1: one plane, 16 KB per tile) and are split
// in registers, which halves their bytes; the producer warps have the time for it.
// Layouts: A (input, I + K_b) and V (output) in FP32 64x64 column-major tiles;
// L in SC and C1 tiles (rows = L's rows, K = L's columns), S (L before the panel
// solve) in C1 only; M in SC and C1 tiles of M^T (tile (I, J) holds (M_IJ)^T:
// rows = M's columns in tile J, K = M's rows in tile I); Linv_J as a 128x128 SC
// block [K chunk][plane][128 x 32].
#include <algorithm>

#include "cg_internal.h"
#include "cg_tc.cuh"

namespace cg {

using namespace tc;

namespace {

constexpr int KC = 32;                          // K columns per chunk
constexpr uint32_t LBO = 128, SBO = KC / 4 * 128;
constexpr uint32_t IDESC = idesc_tf32(128, 128);
constexpr int NPROD = 256;                      // producers (warps 0-7)
constexpr int NTH = NPROD + 128;                // + the MMA issuers (warps 8, 10) and the copy warps (9: B, 11: A)
constexpr int NAST = 4;                         // A stages in tensor memory
constexpr int NIQ = 8;                          // item ids in flight in a CTA's stream
constexpr int NSTB = 4;                         // B stages in shared memory
constexpr uint32_t STB_BYTES = 2u * 128 * KC * 4;  // one B stage: hi + lo, 128 rows x 32 K (32 KB)
constexpr int NSTA = 4;                         // A stages in shared memory (FP32 canonical chunks)
constexpr uint32_t STA_BYTES = 128u * KC * 4;   // one A stage: 128 rows x 32 K FP32 (16 KB)
constexpr int SC_PLANE = TS * TS;               // floats per plane of an SC tile
constexpr int SC_CHUNK = TS * KC;               // floats per 64 x 32 block
constexpr int SC_TILE = 2 * SC_PLANE;           // floats per SC tile (32 KB)
constexpr int C1_TILE = SC_PLANE;               // floats per FP32 canonical tile (16 KB)
constexpr int LI_CHUNK = 2 * 128 * KC;          // floats per K chunk of a Linv block (hi + lo)
constexpr int LINV_SC = 4 * LI_CHUNK;           // floats per Linv block (128 KB)

static_assert(SC_CHUNK * 4 == 8192 && LI_CHUNK * 4 == (int)STB_BYTES, "layout sizes");
// Chunk c goes to B stage c % NSTB and tensor-memory A stage c % NAST, and is issued by the issuer
// of pair parity (c / 2) % 2.  Stage counts of 4 give every stage to one issuer, which then waits
// on the stage's barriers phase by phase in order.  Otherwise the issuer that is ahead could wait
// for a phase two ahead of the barrier, which a parity wait reports as complete: it would read a
// stage whose copy is still in flight.
static_assert(NSTB == 4 && NAST == 4, "one issuer per stage");

// zero 64 x 32 block: the source of bulk copies for operand tiles above the diagonal
__device__ __align__(128) float g_zero_block[SC_CHUNK];

// Tensor-memory columns (512): the accumulators of the two chunk parities and the A operand
// (hi, lo) of the four stages
constexpr uint32_t TMEM_COLS = 512;
__device__ __forceinline__ uint32_t col_main(int set) { return 128u * set; }
__device__ __forceinline__ uint32_t col_a_hi(int st) { return 256u + 64u * st; }
__device__ __forceinline__ uint32_t col_a_lo(int st) { return 256u + 64u * st + 32u; }

// the accumulator row this thread holds in TMEM (warp w: lanes 32 (w % 4) .. + 31)
__device__ __forceinline__ uint32_t lane_base() { return (uint32_t)(32 * ((threadIdx.x / 32) % 4)) << 16; }

// R[j] += accumulator at column col of this thread's row, columns 64 (t / 128) + j
__device__ __forceinline__ void drain(uint32_t tm, uint32_t col, float (&R)[64])
{
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        float m[32];
        tmem_ld32w(tm + lane_base() + col + 64 * (threadIdx.x / 128) + 32 * half, m);
#pragma unroll
        for (int i = 0; i < 32; i += 2) add2(R[32 * half + i], R[32 * half + i + 1], m[i], m[i + 1]);
    }
}

struct TcCtl {
    uint64_t mma_bar[NAST];   // stage: the MMAs of its chunk completed (its A and B stages are free)
    uint64_t acc_free[2];     // pair parity: the pair's accumulator was drained (one arrival per producer warp)
    uint64_t a_full[NAST];    // stage: the chunk's A is in tensor memory (one arrival per producer warp) and,
                              // where a copy thread fills the B stage, its B landed (that thread's arrival
                              // with the copies' bytes), so the issuer polls one barrier per chunk
    uint64_t b_full[NSTB];    // B_PRE: the stage's B, copied ahead of its K loop, landed (B_COPY copies complete on a_full)
    uint64_t b_empty[NSTB];   // B stage's MMAs completed
    uint64_t as_full[NSTA];   // A shared-memory stage landed
    uint64_t as_empty[NSTA];  // A shared-memory stage read by every producer warp
    uint64_t iq_full[NIQ];    // item slot written by the copy thread
    uint64_t iq_empty[NIQ];   // item slot released by every producer warp, both issuers and the A copy thread
    int iq[NIQ];              // item ids of the stream, -1 = end
    uint32_t tbase;
    int bad;
};

// bcopy: a copy thread fills the B stages (B_COPY), so a_full also counts its arrival; bfull: b_full
// is initialised too (not when a second K loop's B copies may already be counting on it)
__device__ __forceinline__ void init_bars(TcCtl& ctl, bool bcopy = true, bool bfull = true)
{
    for (int i = 0; i < NAST; ++i) mbar_init(&ctl.mma_bar[i], 1);
    for (int i = 0; i < 2; ++i) mbar_init(&ctl.acc_free[i], NPROD / 32);
    for (int i = 0; i < NAST; ++i) mbar_init(&ctl.a_full[i], NPROD / 32 + (bcopy ? 1 : 0));
    for (int i = 0; i < NSTB; ++i) {
        if (bfull) mbar_init(&ctl.b_full[i], 1);
        mbar_init(&ctl.b_empty[i], 1);
    }
    for (int i = 0; i < NSTA; ++i) {
        mbar_init(&ctl.as_full[i], 1);
        mbar_init(&ctl.as_empty[i], NPROD / 32);
    }
    for (int i = 0; i < NIQ; ++i) {
        mbar_init(&ctl.iq_full[i], 1);
        mbar_init(&ctl.iq_empty[i], NPROD / 32 + 3);
        ctl.iq[i] = -1;
    }
    fence_mbar_init();
}

__device__ __forceinline__ uint32_t tc_begin(TcCtl& ctl, bool bcopy = true)
{
    if (threadIdx.x < 32) tmem_alloc(&ctl.tbase, TMEM_COLS);
    if (threadIdx.x == 0) {
        init_bars(ctl, bcopy);
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

// re-arm the barriers for a second K loop in the same CTA whose B stages were filled ahead (B_PRE):
// every MMA of the first loop completed; b_full, which the second loop's B copies (issued by the
// first loop's B copy thread as the stages were freed) count on, is left as it is
__device__ __forceinline__ void tc_rearm_pre(TcCtl& ctl)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t* all = &ctl.mma_bar[0];  // every barrier of TcCtl, contiguous
        for (int i = 0; i < 2 * NAST + 2 + 2 * NSTB + 2 * NSTA + 2 * NIQ; ++i)
            if (all + i < ctl.b_full || all + i >= ctl.b_full + NSTB)
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(all + i)));
        init_bars(ctl, false, false);
    }
    __syncthreads();
}

// ---- operand access --------------------------------------------------------

// A operand: row rr of SC tile t, K chunk kc, K columns 16h .. 16h+15, hi and lo.  Across a warp
// (32 consecutive rows) every load covers four whole 128-byte core-matrix rows.
__device__ __forceinline__ void ld_sc(const float* t, int rr, int kc, int h, float4 (&hi)[4], float4 (&lo)[4])
{
    const float* p = t + kc * SC_CHUNK + (rr >> 3) * 256 + (rr & 7) * 4 + 4 * h * 32;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        hi[i] = __ldg(reinterpret_cast<const float4*>(p + i * 32));
        lo[i] = __ldg(reinterpret_cast<const float4*>(p + SC_PLANE + i * 32));
    }
}

// A operand: row rr, K chunk kc, K columns 16h .. 16h+15 of an FP32 canonical tile (split into
// hi and lo only when it is stored to tensor memory, so that the load's latency stays hidden)
template <bool COHERENT>
__device__ __forceinline__ void ld_c1(const float* t, int rr, int kc, int h, float4 (&x)[4])
{
    const float* p = t + kc * SC_CHUNK + (rr >> 3) * 256 + (rr & 7) * 4 + 4 * h * 32;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4* px = reinterpret_cast<const float4*>(p + i * 32);
        x[i] = COHERENT ? __ldcg(px) : __ldg(px);
    }
}

// x = hi + lo with hi = x rounded to nearest TF32 and lo = x - hi (exact; formed as packed two-lane
// adds of -hi).  lo is left for the tensor core to truncate to TF32: its sign is that of the
// rounding of hi, so the truncation is as often up as down, and the error (below 2^-21 of x) is of
// the size of the a_lo * b_lo term the 3xTF32 split drops anyway.  (Truncating hi instead would make
// lo always of x's sign and bias sums of squares.)
__device__ __forceinline__ void split1(const float4& x, float4& hi, float4& lo)
{
    hi = make_float4(tf32_rn(x.x), tf32_rn(x.y), tf32_rn(x.z), tf32_rn(x.w));
    float d0 = x.x, d1 = x.y, d2 = x.z, d3 = x.w;
    add2(d0, d1, -hi.x, -hi.y);
    add2(d2, d3, -hi.z, -hi.w);
    lo = make_float4(d0, d1, d2, d3);
}

__device__ __forceinline__ void split4(const float4 (&x)[4], float4 (&hi)[4], float4 (&lo)[4])
{
#pragma unroll
    for (int i = 0; i < 4; ++i) split1(x[i], hi[i], lo[i]);
}

// B operand of one chunk from two stacked SC tiles (rows 0-63: top, 64-127: bot; nullptr = zero)
__device__ __forceinline__ void bulk_tiles(const float* top, const float* bot, int kc, uint32_t dst, uint64_t* bar)
{
    mbar_arrive_expect_tx(bar, STB_BYTES);
    const float* z = g_zero_block;
    const uint32_t blk = SC_CHUNK * 4;
    bulk_g2s(dst, top ? top + kc * SC_CHUNK : z, blk, bar);
    bulk_g2s(dst + blk, bot ? bot + kc * SC_CHUNK : z, blk, bar);
    bulk_g2s(dst + 2 * blk, top ? top + SC_PLANE + kc * SC_CHUNK : z, blk, bar);
    bulk_g2s(dst + 3 * blk, bot ? bot + SC_PLANE + kc * SC_CHUNK : z, blk, bar);
}

// B operand of one chunk from a Linv block (K chunk kc: hi then lo, 16 KB each)
__device__ __forceinline__ void bulk_linv(const float* li, int kc, uint32_t dst, uint64_t* bar)
{
    mbar_arrive_expect_tx(bar, STB_BYTES);
    bulk_g2s(dst, li + kc * LI_CHUNK, STB_BYTES / 2, bar);
    bulk_g2s(dst + STB_BYTES / 2, li + kc * LI_CHUNK + LI_CHUNK / 2, STB_BYTES / 2, bar);
}

// A operand of one chunk from two stacked FP32 canonical tiles (rows 0-63: top, 64-127: bot;
// nullptr = zero) into an A stage
__device__ __forceinline__ void bulk_a_c1(const float* top, const float* bot, int kc, uint32_t dst, uint64_t* bar)
{
    mbar_arrive_expect_tx(bar, STA_BYTES);
    const float* z = g_zero_block;
    const uint32_t blk = SC_CHUNK * 4;
    bulk_g2s(dst, top ? top + kc * SC_CHUNK : z, blk, bar);
    bulk_g2s(dst + blk, bot ? bot + kc * SC_CHUNK : z, blk, bar);
}

// split row rr (K values v[0..63] times sgn) into a split canonical store: element (rr, k) at
// base + (k / 32) * chunk_stride + plane * plane_stride + canon_off(rr, k % 32)
__device__ __forceinline__ void st_split_row(float* base, int chunk_stride, int plane_stride, int rr,
                                             const float (&v)[64], float sgn)
{
#pragma unroll
    for (int kc = 0; kc < 2; ++kc)
#pragma unroll
        for (int k4 = 0; k4 < 8; ++k4) {
            const int k = 32 * kc + 4 * k4;
            const float4 x = make_float4(sgn * v[k], sgn * v[k + 1], sgn * v[k + 2], sgn * v[k + 3]);
            const float4 h = make_float4(tf32_rn(x.x), tf32_rn(x.y), tf32_rn(x.z), tf32_rn(x.w));
            const float4 l = make_float4(tf32_rn(x.x - h.x), tf32_rn(x.y - h.y), tf32_rn(x.z - h.z), tf32_rn(x.w - h.w));
            float* p = base + kc * chunk_stride + (rr >> 3) * 256 + k4 * 32 + (rr & 7) * 4;
            *reinterpret_cast<float4*>(p) = h;
            *reinterpret_cast<float4*>(p + plane_stride) = l;
        }
}

__device__ __forceinline__ void st_sc_row(float* tile, int rr, const float (&v)[64], float sgn)
{
    st_split_row(tile, SC_CHUNK, SC_PLANE, rr, v, sgn);
}

// row rr (K values v[0..63] times sgn) of an FP32 canonical tile
__device__ __forceinline__ void st_c1_row(float* tile, int rr, const float (&v)[64], float sgn)
{
#pragma unroll
    for (int kc = 0; kc < 2; ++kc)
#pragma unroll
        for (int k4 = 0; k4 < 8; ++k4) {
            const int k = 32 * kc + 4 * k4;
            *reinterpret_cast<float4*>(tile + kc * SC_CHUNK + (rr >> 3) * 256 + k4 * 32 + (rr & 7) * 4) =
                make_float4(sgn * v[k], sgn * v[k + 1], sgn * v[k + 2], sgn * v[k + 3]);
        }
}

// ---- the K loop --------------------------------------------------------------

// How the A operand of chunk c reaches the producers (the item stream passes the item's geometry
// first: fa(gm, c, ...)):
//   A_REG_SC  fa(c, r, h, x[8]) loads row r, K half h of the chunk as hi (x[0..3]) and lo (x[4..7]);
//   A_REG_C1  fa(c, r, h, x[4]) loads it as FP32, split when stored to tensor memory;
//   A_SMEM_C1 fa(c, top, bot, kc) names the two FP32 canonical tiles (rows 0-63, 64-127; nullptr =
//             zero) and the K chunk within them; the copy warp brings them into a ring of NSTA
//             shared-memory stages by bulk copies, ahead of the producers;
//   A_SMEM_PRE (at most NSTA chunks) the producers wrote the FP32 chunks into the ring stages
//             themselves before the loop (fa unused).
enum { A_REG_SC = 0, A_REG_C1 = 1, A_SMEM_C1 = 2, A_SMEM_PRE = 3 };
// How the B operand reaches its shared-memory stage:
//   B_COPY    fb(c, dst, bar) issues bulk copies of the split chunk into the stage;
//   B_FROM_A  (A_SMEM_C1 only, fb unused) B is the same matrix as A (a diagonal block's L_J L_J^T):
//             the producers write the A chunk they split into the B stage too, so the rows are read
//             from memory once, in FP32, instead of twice.
//   B_PRE     (at most NSTB chunks) the stages were filled before the loop, each copy completing on
//             the stage's b_full (phase 0); the loop copies nothing.
enum { B_COPY = 0, B_FROM_A = 1, B_PRE = 2 };

// ---- pieces shared by the single-item K loop and the item stream -----------------------------

constexpr uint32_t kMaxIter = 1u << 22;  // try_wait attempts before a wait gives up

// chunk g's A (row r, K half h: from qx, or for A_SMEM_C1 from the shared-memory ring) into
// tensor-memory stage g % NAST, then one arrival per warp on the stage's a_full barrier
// ssq (nullable, B_FROM_A only): the chunk's sum of squares of this thread's 16 values, summed in
// FP32 (round to nearest) and added to the double-float (ssq->x, ssq->y) by an exact two-sum
// ga (>= 0): the chunk's place in the A ring's own sequence, where not every chunk passes the ring
template <int AMODE, int BMODE = B_COPY, int NX, class W>
__device__ __forceinline__ void put_a(int g, float4 (&qx)[NX], W& wait, const float* sa_f, TcCtl& ctl, uint32_t tm,
                                      float2* ssq = nullptr, int ga = -1)
{
    const int r = threadIdx.x % 128, h = threadIdx.x / 128, lane = threadIdx.x % 32, st = g % NAST;
    if constexpr (AMODE == A_SMEM_C1 || AMODE == A_SMEM_PRE) {
        // this thread's 16 values of the staged chunk (row r, K columns 16h .. 16h+15)
        const int gi = ga >= 0 ? ga : g;
        const int si = gi % NSTA;
        if constexpr (AMODE == A_SMEM_C1) wait(&ctl.as_full[si], (gi / NSTA) & 1);
        const float* p = sa_f + si * (STA_BYTES / 4) + (r >> 3) * 256 + (r & 7) * 4 + 4 * h * 32;
#pragma unroll
        for (int i = 0; i < 4; ++i) qx[i] = *reinterpret_cast<const float4*>(p + i * 32);
        if constexpr (AMODE == A_SMEM_C1) {
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctl.as_empty[si]);
        }
        if constexpr (BMODE == B_FROM_A) {
            if (ssq) {
                float p = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    p = fmaf(qx[i].x, qx[i].x, p);
                    p = fmaf(qx[i].y, qx[i].y, p);
                    p = fmaf(qx[i].z, qx[i].z, p);
                    p = fmaf(qx[i].w, qx[i].w, p);
                }
                const float t = __fadd_rn(ssq->x, p), bp = __fsub_rn(t, ssq->x);
                const float e = __fadd_rn(__fsub_rn(ssq->x, __fsub_rn(t, bp)), __fsub_rn(p, bp));
                ssq->x = t;
                ssq->y = __fadd_rn(ssq->y, e);
            }
        }
    }
    float4 qh[4], ql[4];
    if constexpr (AMODE == A_REG_SC) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            qh[i] = qx[i];
            ql[i] = qx[4 + i];
        }
    } else {
        split4(reinterpret_cast<const float4(&)[4]>(qx), qh, ql);
    }
    tmem_st16x2_wait(tm + lane_base() + col_a_hi(st) + 16 * h, qh, tm + lane_base() + col_a_lo(st) + 16 * h, ql);
    if constexpr (BMODE == B_FROM_A) {
        // the same piece into B stage g % NSTB (free: the caller retired chunk g - 4), hi and lo planes
        float* stage = const_cast<float*>(sa_f) - (NSTB * STB_BYTES) / 4 + (g % NSTB) * (STB_BYTES / 4) +
                       (r >> 3) * 256 + (r & 7) * 4 + 4 * h * 32;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            *reinterpret_cast<float4*>(stage + i * 32) = qh[i];
            *reinterpret_cast<float4*>(stage + STB_BYTES / 8 + i * 32) = ql[i];
        }
        fence_proxy_async();  // the MMA reads the stage through the async proxy
    }
    fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&ctl.a_full[st]);
}

// chunk g's MMAs are done (its stages are free); with `fold` (g ends its pair) fold the pair's
// accumulator into R and release it (one arrival per warp).  With `last` the wait ignores the abort
// flag: every MMA that was issued completes, and none may still run when tensor memory is freed.
template <class W>
__device__ __forceinline__ void retire_acc(int g, bool last, bool fold, W& wait, bool& ok, int* err, TcCtl& ctl,
                                           uint32_t tm, float (&R)[64])
{
    if (!last) {
        wait(&ctl.mma_bar[g % NAST], (g / NAST) & 1);
    } else if (!mbar_wait(&ctl.mma_bar[g % NAST], (g / NAST) & 1, kMaxIter)) {
        ok = false;
        atomicExch(err, 1);
    }
    if (!fold) return;
    fence_after();
    drain(tm, col_main((g >> 1) & 1), R);
    fence_before();
    __syncwarp();
    if (threadIdx.x % 32 == 0) mbar_arrive(&ctl.acc_free[(g >> 1) & 1]);
}

// one issuer thread: chunk g's 12 MMAs (M128 N128 K8, A from tensor-memory stage g % NAST, B from
// shared-memory stage g % NSTB) into the accumulator of its pair's parity (fresh at the pair's first
// chunk), once its A, its B and its accumulator are ready, committed to the stage's mbarriers
template <int BMODE = B_COPY, class W>
__device__ __forceinline__ void issue_chunk(int g, W& wait, TcCtl& ctl, uint32_t tm, uint32_t sb)
{
    const int st = g % NAST, sbi = g % NSTB, pr = g >> 1;
    wait(&ctl.a_full[st], (g / NAST) & 1);  // A put and (B_COPY) B landed: one barrier
    if constexpr (BMODE == B_PRE) wait(&ctl.b_full[sbi], 0);
    if ((g & 1) == 0 && pr >= 2) wait(&ctl.acc_free[pr & 1], ((pr - 2) >> 1) & 1);
    fence_after();
    const uint32_t bh = sb + sbi * STB_BYTES, bl = bh + STB_BYTES / 2;
    const uint32_t ah = tm + col_a_hi(st), al = tm + col_a_lo(st), d = tm + col_main(pr & 1);
#pragma unroll
    for (int kk = 0; kk < KC / 8; ++kk) {
        const uint32_t off = kk * 2 * LBO;
        mma_tf32_ta(d, al + 8 * kk, smem_desc(bh + off, LBO, SBO), IDESC, ((g & 1) || kk) ? 1u : 0u);
        mma_tf32_ta(d, ah + 8 * kk, smem_desc(bh + off, LBO, SBO), IDESC, 1u);
        mma_tf32_ta(d, ah + 8 * kk, smem_desc(bl + off, LBO, SBO), IDESC, 1u);
    }
    mma_commit(&ctl.mma_bar[st]);
    if constexpr (BMODE == B_COPY) mma_commit(&ctl.b_empty[sbi]);
}

// the A copy thread's share of chunk g (A_SMEM_C1: fa(..., top, bot, kc) names the tiles): into the A
// ring once its stage is free
template <int AMODE, class W, class FA>
__device__ __forceinline__ void copy_a(int g, W& wait, TcCtl& ctl, uint32_t sb, FA&& fa)
{
    if constexpr (AMODE == A_SMEM_C1) {
        const int si = g % NSTA;
        if (g >= NSTA) wait(&ctl.as_empty[si], ((g / NSTA) - 1) & 1);
        const float *top, *bot;
        int kc;
        fa(top, bot, kc);
        bulk_a_c1(top, bot, kc, sb + NSTB * STB_BYTES + si * STA_BYTES, &ctl.as_full[si]);
    }
}

// the B copy thread's share of chunk g (fb(..., dst, bar)): into the B ring once its stage's MMAs are done
template <int BMODE, class W, class FB>
__device__ __forceinline__ void copy_b(int g, W& wait, TcCtl& ctl, uint32_t sb, FB&& fb)
{
    if constexpr (BMODE == B_COPY) {
        const int sbi = g % NSTB;
        if (g >= NSTB) wait(&ctl.b_empty[sbi], ((g / NSTB) - 1) & 1);
        fb(sb + sbi * STB_BYTES, &ctl.a_full[sbi]);  // stage sbi == the chunk's A stage (NSTB == NAST)
    }
}

// ---- the K loop of one item ------------------------------------------------------------------

// nchunks chunks (even); fb(c, dst, bar) issues the B chunk's bulk copies into shared memory at dst.
// Called by every thread of the CTA.  On return the producer threads (t < NPROD) hold in R[j] the
// product for row t % 128, column 64 (t / 128) + j (0 if nchunks == 0).  Returns false if an
// mbarrier wait gave up; waits give up early once *err is set (by this or any other CTA), and a
// thread whose wait gave up skips its later waits, so a failure ends the launch quickly.
// tc_kloop's default `tail`: nothing after the B copy thread's last copy
struct NoTail {
    template <class W>
    __device__ __forceinline__ void operator()(W&, TcCtl&, uint32_t) const {}
};

template <int AMODE, int BMODE = B_COPY, class FA, class FB, class FT = NoTail>
__device__ bool tc_kloop(int nchunks, FA fa, FB fb, unsigned char* sbuf, TcCtl& ctl, uint32_t tm, float (&R)[64],
                         int* err, float2* ssq = nullptr, FT tail = FT())
{
    static_assert(BMODE != B_FROM_A || AMODE == A_SMEM_C1, "B_FROM_A needs the A chunk staged in shared memory");
    bool ok = true;
    auto wait = [&](uint64_t* bar, uint32_t parity) {
        if (!ok) return;
        ok = mbar_wait(bar, parity, kMaxIter, err);
        if (!ok) atomicExch(err, 1);
    };
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t sb = smem_u32(sbuf);
    const float* sa_f = reinterpret_cast<const float*>(sbuf + NSTB * STB_BYTES);
#pragma unroll
    for (int j = 0; j < 64; ++j) R[j] = 0.f;
    if (warp < NPROD / 32) {
        // ---- producers
        const int r = threadIdx.x % 128, h = threadIdx.x / 128;
        constexpr int NX = (AMODE == A_REG_SC) ? 8 : 4;
        constexpr bool REG = (AMODE == A_REG_SC || AMODE == A_REG_C1);
        float4 a0[NX], a1[NX];  // register modes: the loaded A of two chunks (slot = chunk & 1)
        // chunks 0 and 1 into the empty stages 0 and 1; register modes load two chunks ahead of the store
        if constexpr (REG) {
            if (nchunks > 0) fa(0, r, h, a0);
            if (nchunks > 1) fa(1, r, h, a1);
        }
        if (nchunks > 0) {
            put_a<AMODE, BMODE>(0, a0, wait, sa_f, ctl, tm, ssq);
            if constexpr (REG) { if (nchunks > 2) fa(2, r, h, a0); }
        }
        if (nchunks > 1) {
            put_a<AMODE, BMODE>(1, a1, wait, sa_f, ctl, tm, ssq);
            if constexpr (REG) { if (nchunks > 3) fa(3, r, h, a1); }
        }
        // step c: chunk c - 2 is retired and its A stage takes chunk c + 2 (held in slot qx = c & 1)
        auto step = [&](int c, float4 (&qx)[NX]) {
            if (c >= 2) retire_acc(c - 2, false, (c & 1) != 0, wait, ok, err, ctl, tm, R);
            if (c + 2 < nchunks) {
                put_a<AMODE, BMODE>(c + 2, qx, wait, sa_f, ctl, tm, ssq);
                if constexpr (REG) { if (c + 4 < nchunks) fa(c + 4, r, h, qx); }
            }
        };
        for (int c = 0; c < nchunks; c += 2) {
            step(c, a0);
            if (c + 1 < nchunks) step(c + 1, a1);
        }
        for (int c = (nchunks >= 2 ? nchunks - 2 : 0); c < nchunks; ++c)
            retire_acc(c, true, (c & 1) || c == nchunks - 1, wait, ok, err, ctl, tm, R);
    } else if (warp == NPROD / 32 || warp == NPROD / 32 + 2) {
        // ---- MMA issue: chunk pairs 0, 2, 4, ... from warp 8, pairs 1, 3, 5, ... from warp 10
        if (lane == 0)
            for (int c = (warp == NPROD / 32) ? 0 : 2; c < nchunks; c += 4) {
                issue_chunk<BMODE>(c, wait, ctl, tm, sb);
                if (c + 1 < nchunks) issue_chunk<BMODE>(c + 1, wait, ctl, tm, sb);
            }
        __syncwarp();
    } else if (warp == NPROD / 32 + 1) {
        // ---- B copies, then tail(wait, ctl, sb) (e.g. a next loop's B copies as the stages free up)
        if (lane == 0) {
            for (int c = 0; c < nchunks; ++c)
                copy_b<BMODE>(c, wait, ctl, sb, [&](uint32_t dst, uint64_t* bar) { fb(c, dst, bar); });
            tail(wait, ctl, sb);
        }
        __syncwarp();
    } else {
        // ---- A copies
        if (lane == 0)
            for (int c = 0; c < nchunks; ++c)
                copy_a<AMODE>(c, wait, ctl, sb, [&](auto& top, auto& bot, auto& kc) { fa(c, top, bot, kc); });
        __syncwarp();
    }
    return ok;
}

// ---- the K loop over a stream of items -------------------------------------------------------

// Items taken in order from a counter shared by the CTAs of a launch (zero before the launch): the
// B copy thread takes them and publishes the ids, in order, through a ring of NIQ shared-memory slots
// (-1 = no more items); every role walks the same sequence of (item, chunk) pairs, and the chunks
// of all the items pass through the stages as one sequence, so an item's copies and A stores start
// while the previous item is still in the tensor pipe and a CTA pays its set-up and its first
// loads' latency once, not per item.  Taking items in order keeps the CTAs running together on
// neighbouring items (a static share per CTA lets them drift apart).
// geo(it) gives item it's geometry (a struct whose member n, even and >= 2, is its chunk count), worked out
// once per item by each role; fa(gm, c, ...) (as for tc_kloop) and fb(gm, c, dst, bar) receive it.
// Once the last chunk of an item is folded in, the producer threads (t < NPROD) call epi(gm, R)
// with R[j] its product at row t % 128, column 64 (t / 128) + j, then clear R.  Called by every
// thread of the CTA.  Failure handling as tc_kloop; a thread whose wait gave up also takes no new
// items, and item ids outside [0, nitems) end the stream.
template <int AMODE, class GEO, class FA, class FB, class FE>
__device__ bool tc_stream(int nitems, int* queue, GEO geo, FA fa, FB fb, FE epi, unsigned char* sbuf, TcCtl& ctl,
                          uint32_t tm, float (&R)[64], int* err)
{
    bool ok = true;
    auto wait = [&](uint64_t* bar, uint32_t parity) {
        if (!ok) return;
        ok = mbar_wait(bar, parity, kMaxIter, err);
        if (!ok) atomicExch(err, 1);
    };
    // a reader's position in the stream: chunk c of the item in queue slot k % NIQ, of geometry gm;
    // gm.n = 0 at the end
    using Geo = decltype(geo(0));
    struct Cur {
        int k, c;
        Geo gm;
    };
    auto enter = [&](Cur& q) {
        wait(&ctl.iq_full[q.k % NIQ], (q.k / NIQ) & 1);
        const int it = ctl.iq[q.k % NIQ];
        q.c = 0;
        if (ok && it >= 0 && it < nitems) {
            q.gm = geo(it);
        } else {
            q.gm.n = 0;
        }
    };
    // to the next chunk; on leaving an item a releasing reader frees its slot: REL_WARP for a whole
    // warp (one arrival after every lane is done), REL_ONE for a single thread (the issuers)
    enum { REL_NONE, REL_WARP, REL_ONE };
    auto next = [&](Cur& q, int release) {
        if (++q.c < q.gm.n) return;
        if (release == REL_WARP) {
            __syncwarp();
            if ((threadIdx.x % 32) == 0) mbar_arrive(&ctl.iq_empty[q.k % NIQ]);
        } else if (release == REL_ONE) {
            mbar_arrive(&ctl.iq_empty[q.k % NIQ]);
        }
        ++q.k;
        enter(q);
    };
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t sb = smem_u32(sbuf);
    const float* sa_f = reinterpret_cast<const float*>(sbuf + NSTB * STB_BYTES);
#pragma unroll
    for (int j = 0; j < 64; ++j) R[j] = 0.f;
    if (warp < NPROD / 32) {
        // ---- producers
        const int r = threadIdx.x % 128, h = threadIdx.x / 128;
        constexpr int NX = (AMODE == A_REG_SC) ? 8 : 4;
        float4 a0[NX], a1[NX];  // register modes: the loaded A of two chunks (slot = chunk & 1)
        // the next chunk to load (register modes), to put into tensor memory, to retire
        Cur lq{}, pq{}, dq{};
        if constexpr (AMODE != A_SMEM_C1) enter(lq);
        enter(pq);
        enter(dq);
        auto load = [&](float4 (&x)[NX]) {
            if constexpr (AMODE != A_SMEM_C1) {
                if (lq.gm.n) {
                    fa(lq.gm, lq.c, r, h, x);
                    next(lq, REL_NONE);
                }
            }
        };
        auto put = [&](int g, float4 (&qx)[NX]) {
            put_a<AMODE>(g, qx, wait, sa_f, ctl, tm);
            next(pq, REL_NONE);
        };
        auto retire = [&](int g, bool last) {
            const bool item_end = dq.c == dq.gm.n - 1;
            retire_acc(g, last, (g & 1) || item_end, wait, ok, err, ctl, tm, R);
            if (item_end) epi(dq.gm, R);
            next(dq, REL_WARP);
            if (item_end) {
#pragma unroll
                for (int j = 0; j < 64; ++j) R[j] = 0.f;
            }
        };
        // chunks 0 and 1 into the empty stages 0 and 1; register modes load two chunks ahead of the store
        int nput = 0;  // chunks put so far; while any remain, chunk g + 2 is put at step g
        load(a0);
        load(a1);
        if (pq.gm.n) {
            put(nput++, a0);
            load(a0);
        }
        if (pq.gm.n) {
            put(nput++, a1);
            load(a1);
        }
        // step g: chunk g - 2 is retired and its A stage takes chunk g + 2 (held in slot qx = g & 1)
        auto step = [&](int g, float4 (&qx)[NX]) {
            if (g >= 2) retire(g - 2, false);
            if (pq.gm.n) {
                put(nput++, qx);
                load(qx);
            }
        };
        for (int g = 0; g < nput; g += 2) {
            step(g, a0);
            if (g + 1 < nput) step(g + 1, a1);
        }
        for (int g = (nput >= 2 ? nput - 2 : 0); g < nput; ++g) retire(g, true);
    } else if (warp == NPROD / 32 || warp == NPROD / 32 + 2) {
        // ---- MMA issue: chunk pairs 0, 2, 4, ... of the stream from warp 8, pairs 1, 3, ... from warp 10
        const int par = (warp == NPROD / 32) ? 0 : 1;
        if (lane == 0) {
            Cur q{};
            enter(q);
            for (int g = 0; q.gm.n; ++g) {
                if (((g >> 1) & 1) == par) issue_chunk(g, wait, ctl, tm, sb);
                next(q, REL_ONE);
            }
        }
        __syncwarp();
    } else if (warp == NPROD / 32 + 3) {
        // ---- A copies, following the published items
        if (lane == 0) {
            Cur q{};
            enter(q);
            for (int g = 0; q.gm.n; ++g) {
                copy_a<AMODE>(g, wait, ctl, sb, [&](auto& top, auto& bot, auto& kc) { fa(q.gm, q.c, top, bot, kc); });
                next(q, REL_ONE);
            }
        }
        __syncwarp();
    } else {
        // ---- B copies: this thread takes the items and publishes them
        if (lane == 0) {
            int g = 0;
            for (int k = 0;; ++k) {
                const int slot = k % NIQ;
                if (k >= NIQ) wait(&ctl.iq_empty[slot], ((k / NIQ) - 1) & 1);
                const int got = ok ? atomicAdd(queue, 1) : -1;
                const int it = (got >= 0 && got < nitems) ? got : -1;
                ctl.iq[slot] = it;
                mbar_arrive(&ctl.iq_full[slot]);
                if (it < 0) break;
                const Geo gm = geo(it);
                for (int c = 0; c < gm.n; ++c, ++g)
                    copy_b<B_COPY>(g, wait, ctl, sb, [&](uint32_t dst, uint64_t* bar) { fb(gm, c, dst, bar); });
            }
        }
        __syncwarp();
    }
    return ok;
}

// ---- a stream of chained items ---------------------------------------------------------------

// Chunks g .. g + 3 of a chained item: the A operand is the item's first product, held in R (this
// thread: row t % 128, K columns 64 h + j of the four chunks' 128, i.e. chunks 2 h and 2 h + 1),
// split into hi and lo as put_a splits (so the result is the one a ring round trip would give) and
// stored to the tensor-memory stages (g + q) % NAST, which the caller freed by retiring every earlier
// chunk.  Every producer warp arrives once on each of the four stages' a_full.
__device__ __forceinline__ void put_chain(int g, const float (&R)[64], TcCtl& ctl, uint32_t tm)
{
    const int h = threadIdx.x / 128, lane = threadIdx.x % 32;
#pragma unroll
    for (int qq = 0; qq < 2; ++qq) {
        const int st = (g + 2 * h + qq) % NAST;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            float4 x[4], qh[4], ql[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int j = 32 * qq + 16 * half + 4 * i;
                x[i] = make_float4(R[j], R[j + 1], R[j + 2], R[j + 3]);
            }
            split4(x, qh, ql);
            tmem_st16x2_wait(tm + lane_base() + col_a_hi(st) + 16 * half, qh, tm + lane_base() + col_a_lo(st) + 16 * half,
                             ql);
        }
    }
    fence_before();
    __syncwarp();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) mbar_arrive(&ctl.a_full[(g + q) % NAST]);
}

// tc_stream for items that are two chained products, R1 = sum over its first n1 chunks (A from the
// FP32 canonical ring, A_SMEM_C1) and R = R1 x (four more chunks of B): the last four chunks' A is
// R1 itself, which the producers move from their registers to tensor memory (put_chain) once every
// chunk of the first product is folded in, so the intermediate product never leaves the SM and the
// CTA goes on to the next item without a barrier or a pipeline restart.  geo(it) gives a struct with
// members n (all chunks, n1 + 4) and n1 (even, >= 2); fa(gm, c, top, bot, kc) names chunk c < n1's
// A tiles; fb(gm, c, dst, bar) issues the B copies of every chunk; epi(gm, R) as for tc_stream.
template <class GEO, class FA, class FB, class FE>
__device__ bool tc_stream_chain(int nitems, int* queue, GEO geo, FA fa, FB fb, FE epi, unsigned char* sbuf,
                                TcCtl& ctl, uint32_t tm, float (&R)[64], int* err)
{
    bool ok = true;
    auto wait = [&](uint64_t* bar, uint32_t parity) {
        if (!ok) return;
        ok = mbar_wait(bar, parity, kMaxIter, err);
        if (!ok) atomicExch(err, 1);
    };
    using Geo = decltype(geo(0));
    struct Cur {
        int k, c;
        Geo gm;
    };
    auto enter = [&](Cur& q) {
        wait(&ctl.iq_full[q.k % NIQ], (q.k / NIQ) & 1);
        const int it = ctl.iq[q.k % NIQ];
        q.c = 0;
        if (ok && it >= 0 && it < nitems) {
            q.gm = geo(it);
        } else {
            q.gm.n = 0;
        }
    };
    enum { REL_NONE, REL_WARP, REL_ONE };
    auto next = [&](Cur& q, int release) {
        if (++q.c < q.gm.n) return;
        if (release == REL_WARP) {
            __syncwarp();
            if ((threadIdx.x % 32) == 0) mbar_arrive(&ctl.iq_empty[q.k % NIQ]);
        } else if (release == REL_ONE) {
            mbar_arrive(&ctl.iq_empty[q.k % NIQ]);
        }
        ++q.k;
        enter(q);
    };
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t sb = smem_u32(sbuf);
    const float* sa_f = reinterpret_cast<const float*>(sbuf + NSTB * STB_BYTES);
#pragma unroll
    for (int j = 0; j < 64; ++j) R[j] = 0.f;
    if (warp < NPROD / 32) {
        // ---- producers: chunks put (np), retired (nr), taken from the A ring (ga), in stream order
        Cur pq{}, dq{};
        enter(pq);
        enter(dq);
        int np = 0, nr = 0, ga = 0;
        float4 qx[4];
        auto retire = [&](bool last) {
            const bool item_end = dq.c == dq.gm.n - 1;
            retire_acc(nr, last, (nr & 1) || item_end, wait, ok, err, ctl, tm, R);
            if (item_end) {
                epi(dq.gm, R);
#pragma unroll
                for (int j = 0; j < 64; ++j) R[j] = 0.f;
            }
            ++nr;
            next(dq, REL_WARP);
        };
        while (pq.gm.n) {
            if (pq.c < pq.gm.n1) {
                // a ring chunk into tensor-memory stage np % NAST, once chunk np - NAST has retired
                while (nr <= np - NAST) retire(false);
                put_a<A_SMEM_C1>(np, qx, wait, sa_f, ctl, tm, nullptr, ga);
                ++ga;
                ++np;
                next(pq, REL_NONE);
            } else {
                // the item's first product complete in R: the four chained chunks from it
                while (nr < np) retire(false);
                put_chain(np, R, ctl, tm);
#pragma unroll
                for (int j = 0; j < 64; ++j) R[j] = 0.f;
                np += 4;
                for (int q = 0; q < 4; ++q) next(pq, REL_NONE);
            }
        }
        while (nr < np) retire(true);
    } else if (warp == NPROD / 32 || warp == NPROD / 32 + 2) {
        // ---- MMA issue: chunk pairs 0, 2, 4, ... of the stream from warp 8, pairs 1, 3, ... from warp 10
        const int par = (warp == NPROD / 32) ? 0 : 1;
        if (lane == 0) {
            Cur q{};
            enter(q);
            for (int g = 0; q.gm.n; ++g) {
                if (((g >> 1) & 1) == par) issue_chunk(g, wait, ctl, tm, sb);
                next(q, REL_ONE);
            }
        }
        __syncwarp();
    } else if (warp == NPROD / 32 + 3) {
        // ---- A copies of the ring chunks, following the published items
        if (lane == 0) {
            Cur q{};
            enter(q);
            for (int ga = 0; q.gm.n;) {
                if (q.c < q.gm.n1) {
                    copy_a<A_SMEM_C1>(ga, wait, ctl, sb, [&](auto& top, auto& bot, auto& kc) { fa(q.gm, q.c, top, bot, kc); });
                    ++ga;
                }
                next(q, REL_ONE);
            }
        }
        __syncwarp();
    } else {
        // ---- B copies: this thread takes the items and publishes them
        if (lane == 0) {
            int g = 0;
            for (int k = 0;; ++k) {
                const int slot = k % NIQ;
                if (k >= NIQ) wait(&ctl.iq_empty[slot], ((k / NIQ) - 1) & 1);
                const int got = ok ? atomicAdd(queue, 1) : -1;
                const int it = (got >= 0 && got < nitems) ? got : -1;
                ctl.iq[slot] = it;
                mbar_arrive(&ctl.iq_full[slot]);
                if (it < 0) break;
                const Geo gm = geo(it);
                for (int c = 0; c < gm.n; ++c, ++g)
                    copy_b<B_COPY>(g, wait, ctl, sb, [&](uint32_t dst, uint64_t* bar) { fb(gm, c, dst, bar); });
            }
        }
        __syncwarp();
    }
    return ok;
}

// write the 128x128 result (this thread: row t % 128, columns 64 (t / 128) + j in R) times sgn
// into the FP32 column-major tiles of supertile (I2, J2), skipping the tile above the diagonal
__device__ __forceinline__ void store_block(const float (&R)[64], float* base, int I2, int J2, float sgn)
{
    if (threadIdx.x >= NPROD) return;
    const int row = threadIdx.x % 128, h = threadIdx.x / 128;
    const int ti = 2 * I2 + row / 64, tj = 2 * J2 + h;
    if (tj > ti) return;
    float* t = base + (size_t)tile_index(ti, tj) * TILE_ELEMS;
#pragma unroll
    for (int j = 0; j < 64; ++j) t[(row % 64) + TS * j] = sgn * R[j];
}

// Cholesky of the 64x64 diagonal block at (o, o) of s (column-major, leading dimension 129, lower
// part), in place.  The updates from factorised panels are summed in u (the same positions of u's
// storage) and subtracted from a column once, when its panel is reached: subtracting each term
// from s directly drops the terms below half an ulp of the diagonal (about 1 after whitening) and
// biases the log-determinant upwards.  Panels of 8 columns: each of the 64 threads that own the
// block's rows factors the panel's 8x8 diagonal block itself (same operands and operation order in
// every thread, so the same values) and then its own row's 8 values, so a panel needs no barrier
// until its columns are written; the trailing sums are then updated four threads per row, from the
// written columns.  All NTH threads take part (every barrier is reached by all).  Sets *bad on a
// non-positive pivot.
__device__ void factor_block64(float* s, float* u, int o, int* bad)
{
    constexpr int L = 129;
    const int t = threadIdx.x;
    for (int e = t; e < 64 * 64; e += NTH) u[(o + e / 64) * L + o + e % 64] = 0.f;
    __syncthreads();
    const int r = o + t % 64, part = t / 64;  // parts 0-3 share the row's trailing sums; t >= 256 idle
    for (int kb = o; kb < o + 64; kb += 8) {
        float lb[8][8], rv[8], lr[8];
        // the panel's 8x8 diagonal block, in the two warps that own the panel's rows (t < 64;
        // the same operands and operation order in every thread, so the same values); a
        // non-positive pivot is recorded in a register and stored after the loop, so no store
        // to shared memory holds back the block's loads
        if (t < 64) {
        bool notpd = false;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
#pragma unroll
            for (int j = 0; j <= i; ++j) {
                const float a = s[(kb + j) * L + kb + i] - u[(kb + j) * L + kb + i];
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < j; ++k) acc = fmaf(lb[i][k], lb[j][k], acc);
                if (j < i) {
                    lb[i][j] = (a - acc) * rv[j];
                } else {
                    float v = a - acc;
                    if (!(v > 0.f)) {  // not positive definite (or NaN): flag, go on with a benign pivot
                        notpd = true;
                        v = 1.f;
                    }
                    lb[i][i] = sqrtf(v);
                    rv[i] = 1.f / lb[i][i];
                }
            }
        }
        // this thread's row r: below the block from its own column entries, inside it from lb
#pragma unroll
        for (int j = 0; j < 8; ++j) lr[j] = 0.f;
        if (r >= kb + 8) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < j; ++k) acc = fmaf(lr[k], lb[j][k], acc);
                lr[j] = ((s[(kb + j) * L + r] - u[(kb + j) * L + r]) - acc) * rv[j];
            }
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (r == kb + i) {
#pragma unroll
                    for (int j = 0; j <= i; ++j) lr[j] = lb[i][j];
                }
        }
        if (notpd && t == 0) *bad = 1;
        }
        __syncthreads();  // every read of the panel's columns is done
        if (t < 64) {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (r >= kb + j) s[(kb + j) * L + r] = lr[j];
        }
        __syncthreads();
        // u[q][r] += sum_j L[r][kb+j] L[q][kb+j] for kb + 8 <= q <= r; q = kb + 8 + part (mod 4),
        // two q at a time so that their loads and sums overlap (each entry's sum in the same order);
        // the row's panel values come back from shared memory
        if (t < 256 && r >= kb + 8) {
#pragma unroll
            for (int j = 0; j < 8; ++j) lr[j] = s[(kb + j) * L + r];
            int q = kb + 8 + part;
            for (; q + 4 <= r; q += 8) {
                float a0 = u[q * L + r], a1 = u[(q + 4) * L + r], x0[8], x1[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    x0[j] = s[(kb + j) * L + q];
                    x1[j] = s[(kb + j) * L + q + 4];
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    a0 = fmaf(lr[j], x0[j], a0);
                    a1 = fmaf(lr[j], x1[j], a1);
                }
                u[q * L + r] = a0;
                u[(q + 4) * L + r] = a1;
            }
            if (q <= r) {
                float acc = u[q * L + r];
#pragma unroll
                for (int j = 0; j < 8; ++j) acc = fmaf(lr[j], s[(kb + j) * L + q], acc);
                u[q * L + r] = acc;
            }
        }
        __syncthreads();
    }
}

// inverse of the lower-triangular 64x64 block at (o, o) of s into the same block of inv (zero above
// its diagonal), blocked by 8: the eight 8x8 diagonal blocks by forward substitution (one thread per
// column), then the block diagonals d = 1..7 below it in turn, M_IJ = -M_II (sum_{k=J}^{I-1} L_Ik M_kJ)
// for I - J = d: the sums one thread per element into tmp, a barrier, the products with M_II one
// thread per element.  All NTH threads take part (every barrier is reached by all).  A forward
// substitution per column (one thread per column, row blocks in turn) took 2.7 times as long: its
// 64 threads ran one long dependent chain each.
__device__ void invert_block64(const float* s, float* inv, float* tmp, int o)
{
    constexpr int L = 129;
    const int t = threadIdx.x;
    for (int e = t; e < 64 * 64; e += NTH) {
        const int r = e % 64, c = e / 64;
        if (r < c) inv[(o + c) * L + o + r] = 0.f;
    }
    if (t < 64) {
        const int base = o + 8 * (t / 8), j = t % 8;
        float y[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            float v = (i == j) ? 1.f : 0.f;
#pragma unroll
            for (int k = 0; k < i; ++k) v = fmaf(-s[(base + k) * L + base + i], y[k], v);
            y[i] = (i < j) ? 0.f : v / s[(base + i) * L + base + i];
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (i >= j) inv[(base + j) * L + base + i] = y[i];
    }
    __syncthreads();
    for (int d = 1; d < 8; ++d) {
        const int nel = 64 * (8 - d);  // blocks (J + d, J), J < 8 - d: element e = 64 J + 8 j + r
        for (int e = t; e < nel; e += NTH) {
            const int J = e / 64, I = J + d, r = e % 8, j = (e / 8) % 8;
            const int c = o + 8 * J + j, row = o + 8 * I + r;
            float acc = 0.f;
            for (int kb = o + 8 * J; kb < o + 8 * I; kb += 8) {
#pragma unroll
                for (int k = 0; k < 8; ++k) acc = fmaf(s[(kb + k) * L + row], inv[c * L + kb + k], acc);
            }
            tmp[e] = acc;
        }
        __syncthreads();
        for (int e = t; e < nel; e += NTH) {
            const int J = e / 64, I = J + d, r = e % 8, j = (e / 8) % 8;
            const int c = o + 8 * J + j, rb = o + 8 * I;
            float acc = 0.f;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q <= r) acc = fmaf(inv[(rb + q) * L + rb + r], tmp[64 * J + 8 * j + q], acc);
            inv[c * L + rb + r] = -acc;
        }
        __syncthreads();
    }
}

// Cholesky of the 128x128 block in s (column-major, leading dimension 129, lower part used) and
// the inverse of its factor into inv (same layout, zero above the diagonal); all NTH threads take
// part (every __syncthreads is reached by all).  Sets *bad on a non-positive pivot.  Blocked in
// 64x64 halves, so that most of the work is in register-blocked 64x64 products (4x4 outputs per
// thread, t < 256) rather than in the latency-bound panel steps:
//   L11 = chol(S11), L11^-1;  L21 = S21 L11^-T;  S22' = S22 - L21 L21^T (one subtraction per
//   element, the sum formed first);  L22 = chol(S22'), L22^-1;  (L^-1)21 = -L22^-1 (L21 L11^-1).
__device__ void factor_block128(float* s, float* inv, float* tmp, int* bad)
{
    constexpr int L = 129;
    const int t = threadIdx.x;
    const int i0 = 4 * (t % 16), j0 = 4 * ((t / 16) % 16);  // this thread's 4x4 outputs of a 64x64 product
    factor_block64(s, inv, 0, bad);
    invert_block64(s, inv, tmp, 0);
    for (int e = t; e < 64 * 64; e += NTH) inv[(64 + e / 64) * L + e % 64] = 0.f;  // upper-right block
    __syncthreads();
    // L21 = S21 L11^-T: L21[i][j] = sum_{k <= j} S21[i][k] L11^-1[j][k]
    float acc[4][4] = {};
    if (t < 256) {
        for (int k = 0; k < j0 + 4; ++k) {
            float a4[4], b4[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a4[q] = s[k * L + 64 + i0 + q];
                b4[q] = inv[k * L + j0 + q];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a4[p], b4[q], acc[p][q]);
        }
    }
    __syncthreads();  // every read of S21 is done
    if (t < 256) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) s[(j0 + q) * L + 64 + i0 + p] = acc[p][q];
    }
    __syncthreads();
    // S22' = S22 - L21 L21^T on the lower part (each thread reads and writes only its own outputs of S22)
    if (t < 256 && i0 + 3 >= j0) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[p][q] = 0.f;
        for (int k = 0; k < 64; ++k) {
            float a4[4], b4[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a4[q] = s[k * L + 64 + i0 + q];
                b4[q] = s[k * L + 64 + j0 + q];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a4[p], b4[q], acc[p][q]);
        }
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (i0 + p >= j0 + q) {
                    float* x = &s[(64 + j0 + q) * L + 64 + i0 + p];
                    *x = *x - acc[p][q];
                }
    }
    __syncthreads();
    factor_block64(s, inv, 64, bad);
    invert_block64(s, inv, tmp, 64);
    __syncthreads();
    // T = L21 L11^-1 into tmp (tmp[j * 65 + i] = T[i][j]); L11^-1[k][j] = 0 for k < j
    if (t < 256) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[p][q] = 0.f;
        for (int k = j0; k < 64; ++k) {
            float a4[4], b4[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a4[q] = s[k * L + 64 + i0 + q];
                b4[q] = inv[(j0 + q) * L + k];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a4[p], b4[q], acc[p][q]);
        }
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) tmp[(j0 + q) * 65 + i0 + p] = acc[p][q];
    }
    __syncthreads();
    // (L^-1)21 = -L22^-1 T into inv rows 64..127, columns 0..63; L22^-1[i][k] = 0 for k > i
    if (t < 256) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[p][q] = 0.f;
        for (int k = 0; k <= i0 + 3; ++k) {
            float a4[4], b4[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a4[q] = inv[(64 + k) * L + 64 + i0 + q];
                b4[q] = tmp[(j0 + q) * 65 + k];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a4[p], b4[q], acc[p][q]);
        }
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) inv[(j0 + q) * L + 64 + i0 + p] = -acc[p][q];
    }
    __syncthreads();
}

// Left-looking Cholesky, column block J2.  The first B CTAs of the 1-D grid are the diagonal blocks
// (one per batch element), which also factorise, so they start first and their factorisation
// overlaps the off-diagonal blocks.  Off-diagonal blocks: S_IJ = A_IJ - sum_{k < 2 J2} L_I,k L_J,k^T
// into the L storage (C1); for J2 > 0 the CTAs after the first B are persistent and take them from
// the work queue, batch element by batch element (the blocks of one element share its L_J panel
// in L2); for J2 = 0 (no K loop, S = A) they copy the blocks, grid-stride, without tensor memory.
// Diagonal block: S_JJ factorised, L_JJ into the L storage, its inverse into Linv and, transposed,
// into the M storage, its diagonal into diag.
__global__ void __launch_bounds__(NTH, 1) chol_tc_update(int J2, int nt, int B, const float* __restrict__ A,
                                                         float* __restrict__ Ls, float* __restrict__ Lc,
                                                         float* __restrict__ Linv, float* __restrict__ Ms,
                                                         float* __restrict__ Mc, float* __restrict__ diag,
                                                         int* __restrict__ status, int* __restrict__ queue,
                                                         int* __restrict__ err, int diag_sq)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ TcCtl ctl;
    __shared__ float2 sq[2][128];   // diagonal blocks: sum over K of L_rk^2, per row and K half
    const int nt2 = nt / 2, noff = nt2 - J2 - 1;
    const size_t ntile = (size_t)ntiles_lower(nt);
    const int row = threadIdx.x % 128, h = threadIdx.x / 128;
    const bool prod = threadIdx.x < NPROD;
    const int nchunks = 2 * J2 * (TS / KC);
    float R[64];
    // S = A - R for the block's rows row, 64 h .. 64 h + 63 into the C1 tile
    auto store_s = [&](size_t boff, int I2) {
        const int ti = 2 * I2 + row / 64, tj = 2 * J2 + h;
        const size_t tix = boff + tile_index(ti, tj);
        const float* a = A + tix * TILE_ELEMS + row % 64;
#pragma unroll
        for (int j = 0; j < 64; ++j) R[j] = a[TS * j] - R[j];
        st_c1_row(Lc + tix * C1_TILE, row % 64, R, 1.f);
    };
    if ((int)blockIdx.x >= B && J2 > 0) {
        const uint32_t tm = tc_begin(ctl);
        struct Item {
            int n, I2;
            size_t boff;  // the batch element's first tile
        };
        auto geo = [&](int it) { return Item{nchunks, J2 + 1 + it % noff, (size_t)(it / noff) * ntile}; };
        auto fa = [&](const Item& q, int c, const float*& top, const float*& bot, int& kc) {
            top = Lc + (q.boff + tile_index(2 * q.I2, c / 2)) * C1_TILE;
            bot = Lc + (q.boff + tile_index(2 * q.I2 + 1, c / 2)) * C1_TILE;
            kc = c % 2;
        };
        auto fb = [&](const Item& q, int c, uint32_t dst, uint64_t* bar) {
            bulk_tiles(Ls + (q.boff + tile_index(2 * J2, c / 2)) * SC_TILE,
                       Ls + (q.boff + tile_index(2 * J2 + 1, c / 2)) * SC_TILE, c % 2, dst, bar);
        };
        auto epi = [&](const Item& q, float (&)[64]) { store_s(q.boff, q.I2); };
        tc_stream<A_SMEM_C1>(noff * B, queue, geo, fa, fb, epi, smem_raw, ctl, tm, R, err);
        tc_end(tm);
        return;
    }
    if ((int)blockIdx.x >= B) {
        // J2 = 0: no K loop, S = A; the CTAs after the first B stride over the off-diagonal blocks
        for (int k = blockIdx.x - B; k < noff * B; k += gridDim.x - B) {
#pragma unroll
            for (int j = 0; j < 64; ++j) R[j] = 0.f;
            if (prod) store_s((size_t)(k / noff) * ntile, J2 + 1 + k % noff);
        }
        return;
    }
    // a diagonal block
    const int I2 = J2, b = blockIdx.x;
    const float* Ab = A + (size_t)b * ntile * TILE_ELEMS;
    float* Lcb = Lc + (size_t)b * ntile * C1_TILE;
    const uint32_t tm = tc_begin(ctl, false);  // B_FROM_A: the producers fill the B stages themselves
    auto fa = [&](int c, const float*& top, const float*& bot, int& kc) {
        top = Lcb + (size_t)tile_index(2 * I2, c / 2) * C1_TILE;
        bot = Lcb + (size_t)tile_index(2 * I2 + 1, c / 2) * C1_TILE;
        kc = c % 2;
    };
    // B = A (S_JJ = A_JJ - L_J L_J^T): the producers copy the split A chunk into the B stage.  The
    // tensor core's FP32 accumulation rounds one way, so its sums of squares on the diagonal of
    // L_J L_J^T come out low by a fraction of an ulp per MMA, every one in the same direction; over
    // the n pivots that biases ln det upwards, by up to ~1e-3 at nside 16 for C_l far from the
    // reference point.  With diag_sq the producers also sum each row's squares on the CUDA cores
    // (round to nearest, double-float across chunks) and those sums replace the diagonal.
    auto fb = [](int, uint32_t, uint64_t*) {};
    float2 ssq = make_float2(0.f, 0.f);
    tc_kloop<A_SMEM_C1, B_FROM_A>(nchunks, fa, fb, smem_raw, ctl, tm, R, err, diag_sq ? &ssq : nullptr);
    if (prod) sq[h][row] = ssq;
    // diagonal block: S = A_JJ - P into shared memory (column-major, ld 129), lower part
    float* s = reinterpret_cast<float*>(smem_raw);
    float* inv = s + 128 * 129;
    float* tmp = inv + 128 * 129;
    __syncthreads();  // every MMA and copy of the K loop is complete: the stages may be reused
    if (prod) {
        const int ti = 2 * J2 + row / 64, tj = 2 * J2 + h;
        if (tj <= ti) {
            const float* t = Ab + (size_t)tile_index(ti, tj) * TILE_ELEMS;
#pragma unroll
            for (int j = 0; j < 64; ++j) s[(64 * h + j) * 129 + row] = t[(row % 64) + TS * j] - R[j];
            if (diag_sq && h == row / 64) {
                const double p = ((double)sq[0][row].x + (double)sq[1][row].x) +
                                 ((double)sq[0][row].y + (double)sq[1][row].y);
                s[row * 129 + row] = (float)((double)t[(row % 64) + TS * (row % 64)] - p);
            }
        }
    }
    __syncthreads();
    factor_block128(s, inv, tmp, &ctl.bad);
    float v[64];
    // L_JJ itself is not stored: no later step reads L's diagonal blocks (the updates and trtri
    // take L's off-diagonal panels, the panel solves and trtri the inverse Linv_J)
    if (threadIdx.x < 128) diag[(size_t)b * nt * TS + J2 * 128 + row] = s[row * 129 + row];
    if (prod) {   // Linv_J: row `row`, K columns 64h .. 64h+63 (chunks 2h, 2h+1)
        float* li = Linv + ((size_t)b * nt2 + J2) * LINV_SC;
#pragma unroll
        for (int j = 0; j < 64; ++j) v[j] = inv[(64 * h + j) * 129 + row];
        st_split_row(li + 2 * h * LI_CHUNK, LI_CHUNK, LI_CHUNK / 2, row, v, 1.f);
    }
    if (prod) {   // (M_JJ)^T = Linv_J^T: SC tile (2J2 + h, 2J2 + cc/64), row cc % 64 (M's column), K = M's rows
        const int cc = row;
        const int ti = 2 * J2 + h, tj = 2 * J2 + cc / 64;
        if (tj <= ti) {
            float* Mb = Ms + (size_t)b * ntile * SC_TILE;
            float* Mcb = Mc + (size_t)b * ntile * C1_TILE;
#pragma unroll
            for (int j = 0; j < 64; ++j) v[j] = inv[cc * 129 + 64 * h + j];
            st_sc_row(Mb + (size_t)tile_index(ti, tj) * SC_TILE, cc % 64, v, 1.f);
            st_c1_row(Mcb + (size_t)tile_index(ti, tj) * C1_TILE, cc % 64, v, 1.f);
        }
    }
    if (threadIdx.x == 0 && ctl.bad && status && status[b] == CG_OK) status[b] = CG_ERR_NOT_PD;
    tc_end(tm);
}

// L_IJ = S_IJ Linv_J^T for every I2 > J2 and batch element: items it = b (nt2 - J2 - 1) + I2 - J2 - 1,
// taken in order from the work queue by persistent CTAs
__global__ void __launch_bounds__(NTH, 1) chol_tc_panel(int J2, int nt, int B, float* __restrict__ Ls,
                                                        float* __restrict__ Lc, const float* __restrict__ Linv,
                                                        int* __restrict__ queue, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ TcCtl ctl;
    const int nt2 = nt / 2, m = nt2 - J2 - 1;
    const size_t ntile = (size_t)ntiles_lower(nt);
    const uint32_t tm = tc_begin(ctl);
    struct Item {
        int n, I2;
        const float* Lcb;  // the batch element's S / L (C1)
        const float* li;   // its Linv_J
        size_t boff;       // its first tile
    };
    auto geo = [&](int it) {
        const size_t b = it / m;
        return Item{128 / KC, J2 + 1 + it % m, Lc + b * ntile * C1_TILE, Linv + (b * nt2 + J2) * LINV_SC, b * ntile};
    };
    // A(r, m) = S_IJ(r, m), C1 tiles (2 I2 + r/64, 2 J2 + m/64); B(c, m) = Linv_J(c, m)
    auto fa = [&](const Item& q, int c, const float*& top, const float*& bot, int& kc) {
        top = q.Lcb + (size_t)tile_index(2 * q.I2, 2 * J2 + c / 2) * C1_TILE;
        bot = q.Lcb + (size_t)tile_index(2 * q.I2 + 1, 2 * J2 + c / 2) * C1_TILE;
        kc = c % 2;
    };
    auto fb = [&](const Item& q, int c, uint32_t dst, uint64_t* bar) { bulk_linv(q.li, c, dst, bar); };
    // the item's S tiles were all read (its MMAs are done) before they are overwritten
    auto epi = [&](const Item& q, float (&R)[64]) {
        const int row = threadIdx.x % 128, h = threadIdx.x / 128;
        const size_t tix = q.boff + tile_index(2 * q.I2 + row / 64, 2 * J2 + h);
        st_sc_row(Ls + tix * SC_TILE, row % 64, R, 1.f);
        st_c1_row(Lc + tix * C1_TILE, row % 64, R, 1.f);
    };
    float R[64];
    tc_stream<A_SMEM_C1>(m * B, queue, geo, fa, fb, epi, smem_raw, ctl, tm, R, err);
    tc_end(tm);
}

// Row block I2 of M = L^-1, off-diagonal blocks J2 = blockIdx.x < I2; grid (I2, B).  Computes
// the transposes: S^T = sum_{k=2 J2}^{2 I2 - 1} M_kJ^T L_Ik^T, then (M_IJ)^T = -S^T Linv_I^T with
// S^T kept in shared memory.
__global__ void __launch_bounds__(NTH, 1) trtri_tc_row(int I2, int nt, const float* __restrict__ Ls,
                                                       const float* __restrict__ Linv, float* __restrict__ Ms,
                                                       float* __restrict__ Mc, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ TcCtl ctl;
    const int J2 = blockIdx.x, b = blockIdx.y, nt2 = nt / 2;
    const size_t ntile = (size_t)ntiles_lower(nt);
    const float* Lb = Ls + (size_t)b * ntile * SC_TILE;
    float* Mb = Ms + (size_t)b * ntile * SC_TILE;
    float* Mcb = Mc + (size_t)b * ntile * C1_TILE;
    const float* li = Linv + ((size_t)b * nt2 + I2) * LINV_SC;
    const int row = threadIdx.x % 128, h = threadIdx.x / 128;
    const uint32_t tm = tc_begin(ctl);
    // A(c, m) = M_kJ(m, c): C1 tile (k, 2 J2 + c/64) of M^T (zero above the diagonal);
    // B(r, m) = L_Ik(r, m): SC tiles (2 I2, k), (2 I2 + 1, k)
    const int k0 = 2 * J2;
    const int nchunks = (2 * I2 - k0) * (TS / KC);
    auto fa = [&](int c, const float*& top, const float*& bot, int& kc) {
        const int k = k0 + c / 2;
        top = (k >= 2 * J2) ? Mcb + (size_t)tile_index(k, 2 * J2) * C1_TILE : nullptr;
        bot = (k >= 2 * J2 + 1) ? Mcb + (size_t)tile_index(k, 2 * J2 + 1) * C1_TILE : nullptr;
        kc = c % 2;
    };
    auto fb = [&](int c, uint32_t dst, uint64_t* bar) {
        const int k = k0 + c / 2;
        bulk_tiles(Lb + (size_t)tile_index(2 * I2, k) * SC_TILE, Lb + (size_t)tile_index(2 * I2 + 1, k) * SC_TILE,
                   c % 2, dst, bar);
    };
    // the second product's B, Linv_I's four chunks, copied into the B stages by the first loop's B copy
    // thread as each stage's last MMAs complete, so that it lands while the first product finishes
    auto tail = [&](auto& wait, TcCtl& c, uint32_t sb) {
        for (int q = 0; q < NSTB; ++q) {
            const int cq = nchunks - 1 - ((nchunks - 1 - q) % NSTB);  // the first loop's last chunk in stage q
            wait(&c.b_empty[q], (cq / NSTB) & 1);
            bulk_linv(li, q, sb + q * STB_BYTES, &c.b_full[q]);
        }
    };
    float R[64];
    tc_kloop<A_SMEM_C1>(nchunks, fa, fb, smem_raw, ctl, tm, R, err, nullptr, tail);
    // S^T stays on chip: into the A ring as the four FP32 canonical K chunks of the second product
    // (row = M's column, K = M's rows 64h .. 64h+63: chunks 2h, 2h+1).  Every producer's last ring
    // read came before the last chunk's MMAs, which any producer leaving the loop has waited for.
    if (threadIdx.x < NPROD) {
        float* ring = reinterpret_cast<float*>(smem_raw + NSTB * STB_BYTES);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int k = 64 * h + 4 * q;
            *reinterpret_cast<float4*>(ring + (k / KC) * (STA_BYTES / 4) + (row >> 3) * 256 + ((k % KC) >> 2) * 32 +
                                       (row & 7) * 4) = make_float4(R[4 * q], R[4 * q + 1], R[4 * q + 2], R[4 * q + 3]);
        }
    }
    tc_rearm_pre(ctl);  // its __syncthreads also makes the ring writes visible to all producers
    // A(c, m) = S^T(c, m) from the ring; B(r, m) = Linv_I(r, m), already in (or on its way to) the B stages
    static_assert(128 / KC == NSTB, "the second product's B fills the B stages exactly");
    auto fa2 = [](int, const float*&, const float*&, int&) {};
    auto fb2 = [](int, uint32_t, uint64_t*) {};
    tc_kloop<A_SMEM_PRE, B_PRE>(128 / KC, fa2, fb2, smem_raw, ctl, tm, R, err);
    if (threadIdx.x < NPROD) {
        const size_t tix = tile_index(2 * I2 + h, 2 * J2 + row / 64);
        st_sc_row(Mb + tix * SC_TILE, row % 64, R, -1.f);
        st_c1_row(Mcb + tix * C1_TILE, row % 64, R, -1.f);
    }
    tc_end(tm);
}

// Row block I2 of M = L^-1 as a stream of items it = b * I2 + J2 (J2 < I2) taken in order from the
// work queue by persistent CTAs: each item is trtri_tc_row's two products, S^T = sum_k M_kJ^T L_Ik^T
// (A from M^T's FP32 canonical copy through the ring) and (M_IJ)^T = -S^T Linv_I^T, chained on chip
// (tc_stream_chain), with the same operands, splits and summation order, so the same results.  The
// items of one batch element share its L row panel I in L2.
__global__ void __launch_bounds__(NTH, 1) trtri_tc_stream(int I2, int nt, int B, const float* __restrict__ Ls,
                                                          const float* __restrict__ Linv, float* __restrict__ Ms,
                                                          float* __restrict__ Mc, int* __restrict__ queue,
                                                          int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ TcCtl ctl;
    const int nt2 = nt / 2;
    const size_t ntile = (size_t)ntiles_lower(nt);
    const uint32_t tm = tc_begin(ctl);
    struct Item {
        int n, n1, J2, b;
    };
    auto geo = [&](int it) {
        const int J2 = it % I2, n1 = (2 * I2 - 2 * J2) * (TS / KC);
        return Item{n1 + 128 / KC, n1, J2, it / I2};
    };
    // A(c, m) = M_kJ(m, c): C1 tiles (k, 2 J2), (k, 2 J2 + 1) of M^T, k >= 2 J2 (zero above the diagonal)
    auto fa = [&](const Item& q, int c, const float*& top, const float*& bot, int& kc) {
        const float* Mcb = Mc + (size_t)q.b * ntile * C1_TILE;
        const int k = 2 * q.J2 + c / 2;
        top = Mcb + (size_t)tile_index(k, 2 * q.J2) * C1_TILE;
        bot = (k >= 2 * q.J2 + 1) ? Mcb + (size_t)tile_index(k, 2 * q.J2 + 1) * C1_TILE : nullptr;
        kc = c % 2;
    };
    // B: L_Ik (SC tiles (2 I2, k), (2 I2 + 1, k)) for the first product, then Linv_I's four chunks
    auto fb = [&](const Item& q, int c, uint32_t dst, uint64_t* bar) {
        if (c < q.n1) {
            const float* Lb = Ls + (size_t)q.b * ntile * SC_TILE;
            const int k = 2 * q.J2 + c / 2;
            bulk_tiles(Lb + (size_t)tile_index(2 * I2, k) * SC_TILE, Lb + (size_t)tile_index(2 * I2 + 1, k) * SC_TILE,
                       c % 2, dst, bar);
        } else {
            bulk_linv(Linv + ((size_t)q.b * nt2 + I2) * LINV_SC, c - q.n1, dst, bar);
        }
    };
    auto epi = [&](const Item& q, float (&R)[64]) {
        const int row = threadIdx.x % 128, h = threadIdx.x / 128;
        const size_t tix = (size_t)q.b * ntile + tile_index(2 * I2 + h, 2 * q.J2 + row / 64);
        st_sc_row(Ms + tix * SC_TILE, row % 64, R, -1.f);
        st_c1_row(Mc + tix * C1_TILE, row % 64, R, -1.f);
    };
    float R[64];
    tc_stream_chain(I2 * B, queue, geo, fa, fb, epi, smem_raw, ctl, tm, R, err);
    tc_end(tm);
}

// V_IJ (128x128 supertile, lower) = sum over k of M_k,I^T M_k,J from the M^T storage; V in FP32
// column-major tiles.  grid (supertiles of the lower triangle, B).  One CTA per supertile: the
// hardware's in-order CTA dispatch keeps the CTAs running together on one batch element, whose M
// stays in L2 (a persistent stream over a work queue, lauum_tc_stream, measured slower at nside 16
// and level at nside 32).
// AM = A_SMEM_C1 (the default): the A operand from the FP32 canonical copy Mc through the
// shared-memory ring, split on chip, its low parts left unrounded for the tensor core; A_REG_SC: from
// the split copy Ms, low parts rounded to TF32 when it was written.
// y (nullable): the solve's first pass x = V y folded into the epilogue, from the block still in
// registers: for each stored 64x64 tile (I, J) of V, part[t][0][r] = (V_IJ y_J)[r] and, for I != J,
// part[t][1][c] = (V_IJ^T y_I)[c] (zero on diagonal tiles), as FP32 sums with a zero low word: the
// layout and meaning of tile::symv_partials<false>, whose read of V it saves.
template <int AM>
__global__ void __launch_bounds__(NTH, 1) lauum_tc(int nt, const float* __restrict__ Ms, const float* __restrict__ Mc,
                                                   float* __restrict__ V, int* __restrict__ err,
                                                   const double* __restrict__ y, int ystride, float2* __restrict__ part)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ TcCtl ctl;
    __shared__ __align__(16) float ys[2][128];  // y at the block's columns (J) and rows (I), fused solve pass
    int I2, J2;
    tile_coords(blockIdx.x, I2, J2);
    const int b = blockIdx.y;
    const size_t ntile = (size_t)ntiles_lower(nt);
    const float* Mb = Ms + (size_t)b * ntile * SC_TILE;
    float ypre = 0.f;  // this thread's y entry for the epilogue, loaded before the K loop hides its latency
    if (y && threadIdx.x < 256)
        ypre = (float)__ldg(y + (size_t)b * ystride + (threadIdx.x < 128 ? 2 * J2 : 2 * I2) * TS + threadIdx.x % 128);
    const uint32_t tm = tc_begin(ctl);
    const int k0 = 2 * I2;  // first tile row with a non-zero M_k,I
    const int nchunks = (nt - k0) * (TS / KC);
    // A(r, m) = M_{k, 2I2 + r/64}(m, r%64); B(c, m) = M_{k, 2J2 + c/64}(m, c%64); zero above the diagonal.
    // AM = A_REG_SC: A loaded pre-split by the producers, two chunks ahead in registers; A_SMEM_C1:
    // A from the FP32 copy through the four-stage ring (half the bytes, further ahead), split on
    // chip: 5.85 against 6.19 ms at nside 16, batch 256.
    auto fa = [&](int c, int r, int h, float4 (&x)[8]) {
        const int k = k0 + c / 2, col = 2 * I2 + r / 64;
        if (k < col) {
#pragma unroll
            for (int i = 0; i < 8; ++i) x[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            float4 hi[4], lo[4];
            ld_sc(Mb + (size_t)tile_index(k, col) * SC_TILE, r % 64, c % 2, h, hi, lo);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                x[i] = hi[i];
                x[4 + i] = lo[i];
            }
        }
    };
    auto fb = [&](int c, uint32_t dst, uint64_t* bar) {
        const int k = k0 + c / 2;
        const float* top = (k >= 2 * J2) ? Mb + (size_t)tile_index(k, 2 * J2) * SC_TILE : nullptr;
        const float* bot = (k >= 2 * J2 + 1) ? Mb + (size_t)tile_index(k, 2 * J2 + 1) * SC_TILE : nullptr;
        bulk_tiles(top, bot, c % 2, dst, bar);
    };
    float R[64];
    if constexpr (AM == A_SMEM_C1) {
        const float* Mcb = Mc + (size_t)b * ntile * C1_TILE;
        auto fa1 = [&](int c, const float*& top, const float*& bot, int& kc) {
            const int k = k0 + c / 2;
            top = Mcb + (size_t)tile_index(k, 2 * I2) * C1_TILE;
            bot = (k >= 2 * I2 + 1) ? Mcb + (size_t)tile_index(k, 2 * I2 + 1) * C1_TILE : nullptr;
            kc = c % 2;
        };
        tc_kloop<A_SMEM_C1>(nchunks, fa1, fb, smem_raw, ctl, tm, R, err);
    } else {
        tc_kloop<A_REG_SC>(nchunks, fa, fb, smem_raw, ctl, tm, R, err);
    }
    store_block(R, V + (size_t)b * ntile * TILE_ELEMS, I2, J2, 1.f);
    if (y) {
        if (threadIdx.x < 256) ys[threadIdx.x / 128][threadIdx.x % 128] = ypre;
        __syncthreads();  // every MMA and copy of the K loop is done: the ring is free for the column sums
        float(*red)[64] = reinterpret_cast<float(*)[64]>(smem_raw);  // [producer warp][column]: warp column sums
        float2* pb = part + (size_t)b * ntile * 2 * TS;
        if (threadIdx.x < NPROD) {
            const int row = threadIdx.x % 128, h = threadIdx.x / 128, lane = threadIdx.x % 32;
            const int ti = 2 * I2 + row / 64, tj = 2 * J2 + h;  // the same for the whole warp
            if (tj <= ti) {
                // row sum V_IJ(row, :) y_J in four interleaved chains
                float a[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int j = 0; j < 64; j += 4) {
                    const float4 yv = *reinterpret_cast<const float4*>(&ys[0][64 * h + j]);
                    a[0] = fmaf(R[j], yv.x, a[0]);
                    a[1] = fmaf(R[j + 1], yv.y, a[1]);
                    a[2] = fmaf(R[j + 2], yv.z, a[2]);
                    a[3] = fmaf(R[j + 3], yv.w, a[3]);
                }
                pb[(size_t)tile_index(ti, tj) * 2 * TS + row % 64] = make_float2((a[0] + a[1]) + (a[2] + a[3]), 0.f);
                if (ti != tj) {
                    // column sums y_I(rows)^T V_IJ over the warp's 32 rows: five halving exchange steps,
                    // after which lane L holds the sums of columns 2L and 2L + 1
                    const float yr = ys[1][row];
#pragma unroll
                    for (int j = 0; j < 64; ++j) R[j] *= yr;
#pragma unroll
                    for (int st = 0; st < 5; ++st) {
                        const int H = 32 >> st, xm = 16 >> st;
                        const bool up = (lane & xm) != 0;  // keeps the upper half of the columns
#pragma unroll
                        for (int i = 0; i < H; ++i) {
                            const float send = up ? R[i] : R[H + i];
                            const float keep = up ? R[H + i] : R[i];
                            R[i] = keep + __shfl_xor_sync(0xffffffffu, send, xm);
                        }
                    }
                    *reinterpret_cast<float2*>(&red[threadIdx.x / 32][2 * lane]) = make_float2(R[0], R[1]);
                }
            }
        }
        __syncthreads();
        if (threadIdx.x < NPROD) {
            const int hh = threadIdx.x / 128, half = (threadIdx.x / 64) % 2, c = threadIdx.x % 64;
            const int ti = 2 * I2 + half, tj = 2 * J2 + hh;
            if (tj <= ti) {
                // the tile's 64 rows are producer warps 4 hh + 2 half and 4 hh + 2 half + 1
                const float sum = (ti != tj) ? red[4 * hh + 2 * half][c] + red[4 * hh + 2 * half + 1][c] : 0.f;
                pb[(size_t)tile_index(ti, tj) * 2 * TS + TS + c] = make_float2(sum, 0.f);
            }
        }
    }
    tc_end(tm);
}

// lauum_tc as a stream of items it = b * (supertiles) + t (t in tile_coords order) taken in order
// from the work queue by persistent CTAs, so that a CTA's set-up and the first loads of an item
// overlap the previous item's MMAs.  The A operand (M^T's column panel I) comes from the FP32
// canonical copy through the shared-memory ring and is split on chip (its low part left unrounded
// for the tensor core to truncate, where lauum_tc reads the split copy's rounded one: the two differ
// by under 2^-22 of an entry); the B operand from the split copy, as in lauum_tc.
__global__ void __launch_bounds__(NTH, 1) lauum_tc_stream(int nt, int B, const float* __restrict__ Ms,
                                                          const float* __restrict__ Mc, float* __restrict__ V,
                                                          int* __restrict__ queue, int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ TcCtl ctl;
    const int nt2 = nt / 2, nsup = nt2 * (nt2 + 1) / 2;
    const size_t ntile = (size_t)ntiles_lower(nt);
    const uint32_t tm = tc_begin(ctl);
    struct Item {
        int n, I2, J2;
        size_t boff;  // the batch element's first tile
    };
    auto geo = [&](int it) {
        int I2, J2;
        tile_coords(it % nsup, I2, J2);
        return Item{(nt - 2 * I2) * (TS / KC), I2, J2, (size_t)(it / nsup) * ntile};
    };
    // A(r, m) = M_{k, 2I2 + r/64}(m, r%64): C1 tiles (k, 2 I2), (k, 2 I2 + 1) of M^T, k >= 2 I2
    auto fa = [&](const Item& q, int c, const float*& top, const float*& bot, int& kc) {
        const int k = 2 * q.I2 + c / 2;
        top = Mc + (q.boff + tile_index(k, 2 * q.I2)) * C1_TILE;
        bot = (k >= 2 * q.I2 + 1) ? Mc + (q.boff + tile_index(k, 2 * q.I2 + 1)) * C1_TILE : nullptr;
        kc = c % 2;
    };
    auto fb = [&](const Item& q, int c, uint32_t dst, uint64_t* bar) {
        const int k = 2 * q.I2 + c / 2;
        const float* top = (k >= 2 * q.J2) ? Ms + (q.boff + tile_index(k, 2 * q.J2)) * SC_TILE : nullptr;
        const float* bot = (k >= 2 * q.J2 + 1) ? Ms + (q.boff + tile_index(k, 2 * q.J2 + 1)) * SC_TILE : nullptr;
        bulk_tiles(top, bot, c % 2, dst, bar);
    };
    auto epi = [&](const Item& q, float (&R)[64]) { store_block(R, V + q.boff * TILE_ELEMS, q.I2, q.J2, 1.f); };
    float R[64];
    tc_stream<A_SMEM_C1>(nsup * B, queue, geo, fa, fb, epi, smem_raw, ctl, tm, R, err);
    tc_end(tm);
}

// ---- adjoint contraction ---------------------------------------------------------------------

// part[t][b][l] = sum over the entries e of lower tile t of w_e V_b[e] Ubar_l[e], w_e = 2 below the
// matrix diagonal, 1 on it, 0 above (V symmetric, stored lower): the per-tile terms of
// Tr(V dA/dC_l).  One GEMM per tile and 128 batch elements: M = 128 (b), N = lp (l), K = the tile's
// 4096 entries in 32-wide chunks, 3xTF32.  The operand rows (128 rows of V, lp of Ubar) are 16 KB
// apart or more, so they are fetched in groups of G chunks: each warp copies (cp.async) G x 128
// contiguous bytes of a row at a time into one of NB group buffers, NB - 1 groups ahead (fetching
// 128 bytes of every row per chunk left HBM at a third of its bandwidth, and one group of 512-byte
// runs in flight at about 40%).  The producers then store their
// pieces split: V (A, weighted) into tensor memory, Ubar (B) into a shared-memory stage (K-major
// canonical, lp rows), so the FP32 table needs no split copy.  One thread issues the MMAs; each
// chunk pair's accumulator is folded into round-to-nearest registers (the tensor core's FP32
// accumulation drifts one way).  The weight 2 of the off-diagonal tiles is applied to the sums
// at the end.  RC >= lp / 2: the accumulator columns a producer drains.
// grid (tiles, ceil(B / 128)).
constexpr int ADJ_NTH = NPROD + 32;

template <int RC, int G, int NB>
__global__ void __launch_bounds__(ADJ_NTH, 1) contract_adj_tc(int B, int lp, const float* __restrict__ U,
                                                              const float* __restrict__ V, size_t strideA,
                                                              float* __restrict__ part, int* __restrict__ err)
{
    constexpr int NBP = (8 * RC + NPROD - 1) / NPROD;  // B pieces (8 K values) per producer and chunk
    constexpr int P = 8 * G;                            // 16-byte pieces of a row in a group
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t mma_bar[NAST], acc_free[2], ab_full[NAST];
    __shared__ uint32_t tbase;
    const int t = blockIdx.x, b0 = blockIdx.y * 128;
    int I, J;
    tile_coords(t, I, J);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (warp == 0) tmem_alloc(&tbase, TMEM_COLS);
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) mbar_init(&acc_free[i], NPROD / 32);
        for (int i = 0; i < NAST; ++i) {
            mbar_init(&mma_bar[i], 1);
            mbar_init(&ab_full[i], NPROD / 32);
        }
        fence_mbar_init();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = tbase, sb = smem_u32(smem_raw);
    const uint32_t plane = (uint32_t)lp * KC * 4, stb = 2 * plane;  // B stage: lp rows x 32 K, hi then lo
    constexpr int NCH = TILE_ELEMS / KC;
    bool ok = true;
    auto wait = [&](uint64_t* bar, uint32_t parity) {
        if (!ok) return;
        ok = mbar_wait(bar, parity, kMaxIter, err);
        if (!ok) atomicExch(err, 1);
    };
    if (warp < NPROD / 32) {
        const int r = threadIdx.x % 128, h = threadIdx.x / 128, b = b0 + r;
        float R[RC];
#pragma unroll
        for (int j = 0; j < RC; ++j) R[j] = 0.f;
        // NB group buffers after the B stages: 128 V rows then lp Ubar rows of P pieces, piece j of
        // row q at physical piece j ^ (q % P), so that the producers' reads (one row per lane) and
        // the warps' copies (one row per warp) both spread over the banks
        const uint32_t gbuf = (uint32_t)(128 + lp) * P * 16;
        auto gpiece = [&](int k, int q, int j) {
            return (uint32_t)(NAST * stb + (k % NB) * gbuf + (q * P + (j ^ (q % P))) * 16);
        };
        // group k (chunks G k .. G k + G - 1): consecutive threads copy consecutive pieces of a row
        auto fetch = [&](int k) {
            if (G * k < NCH) {
                for (int idx = threadIdx.x; idx < (128 + lp) * P; idx += NPROD) {
                    const int q = idx / P, j = idx % P;
                    // rows past B copy row B - 1: their products are never stored, and a row only
                    // touches its own outputs
                    const float* src = (q < 128)
                                           ? V + (size_t)min(b0 + q, B - 1) * strideA + (size_t)t * TILE_ELEMS
                                           : U + ((size_t)t * lp + (q - 128)) * TILE_ELEMS;
                    cp_async16(sb + gpiece(k, q, j), src + KC * G * k + 4 * j);
                }
            }
            cp_async_commit();
        };
        auto rd = [&](int k, int q, int j) {
            return *reinterpret_cast<const float4*>(smem_raw + gpiece(k, q, j));
        };
        // chunk c into stage c % NAST: weighted, split V into tensor memory, split Ubar into shared
        // memory.  At the first chunk of group k, its copies are waited for (the NB - 2 later groups
        // may still be in flight) and published to all producers (named barrier), which also frees
        // group k - 1's buffer for group k + NB - 1.
        auto put = [&](int c) {
            const int st = c % NAST, k = c / G, cl = c % G;
            if (cl == 0) {
                cp_async_wait<NB - 2>();
                asm volatile("bar.sync 1, %0;" ::"n"(NPROD) : "memory");
                fetch(k + NB - 1);
            }
            float4 x[4], qh[4], ql[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) x[i] = rd(k, r, 8 * cl + 4 * h + i);
            if (I == J) {  // diagonal tile: weight 2 below the diagonal, 1 on it, 0 above (1/2 of that here)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float* xi = reinterpret_cast<float*>(&x[i]);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const int e = KC * c + 16 * h + 4 * i + kk, rr = e % TS, cc = e / TS;
                        xi[kk] *= (rr > cc) ? 1.f : (rr == cc ? 0.5f : 0.f);
                    }
                }
            }
            split4(x, qh, ql);
            tmem_st16x2_wait(tm + lane_base() + col_a_hi(st) + 16 * h, qh, tm + lane_base() + col_a_lo(st) + 16 * h, ql);
            unsigned char* stage = smem_raw + st * stb;
#pragma unroll
            for (int p = 0; p < NBP; ++p) {
                const int i = threadIdx.x + NPROD * p;
                if (i < 4 * lp) {
                    const int l = i / 4, k0 = 8 * (i % 4);
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        float4 hi, lo;
                        split1(rd(k, 128 + l, 8 * cl + k0 / 4 + q), hi, lo);
                        const uint32_t off = (l / 8) * 1024 + ((k0 / 4) + q) * 128 + (l % 8) * 16;
                        *reinterpret_cast<float4*>(stage + off) = hi;
                        *reinterpret_cast<float4*>(stage + plane + off) = lo;
                    }
                }
            }
            fence_proxy_async();
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ab_full[st]);
        };
        // chunk c's MMAs are done: fold its lp / 2 columns of this thread into R and release the
        // accumulator (the last chunks' waits ignore the abort flag: no MMA may outlive tensor memory)
        // chunk c's MMAs are done (its stages are free); at the end of a chunk pair, fold the pair's
        // lp / 2 columns of this thread into R and release the accumulator (the last chunks' waits
        // ignore the abort flag: no MMA may outlive tensor memory)
        auto retire = [&](int c, bool last) {
            if (!last) {
                wait(&mma_bar[c % NAST], (c / NAST) & 1);
            } else if (!mbar_wait(&mma_bar[c % NAST], (c / NAST) & 1, kMaxIter)) {
                ok = false;
                atomicExch(err, 1);
            }
            if (!(c & 1)) return;
            fence_after();
#pragma unroll
            for (int j = 0; j < (RC + 7) / 8; ++j) {
                if (8 * j < lp / 2) {
                    float m[8];
                    tmem_ld8w(tm + lane_base() + col_main((c >> 1) & 1) + h * (lp / 2) + 8 * j, m);
#pragma unroll
                    for (int i = 0; i < 8; i += 2) add2(R[8 * j + i], R[8 * j + i + 1], m[i], m[i + 1]);
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_free[(c >> 1) & 1]);
        };
        // groups are fetched NB - 1 ahead of the stores, the stores run two chunks ahead of the MMAs:
        // step c retires chunk c - 2 and stores chunk c + 2 into its stage
        for (int k = 0; k < NB - 1; ++k) fetch(k);
        put(0);
        put(1);
        for (int c = 0; c < NCH; ++c) {
            if (c >= 2) retire(c - 2, false);
            if (c + 2 < NCH) put(c + 2);
        }
        cp_async_wait<0>();
        retire(NCH - 2, true);
        retire(NCH - 1, true);
        if (b < B) {
            float* dst = part + ((size_t)t * B + b) * lp + h * (lp / 2);
#pragma unroll
            for (int j = 0; j < RC; ++j)
                if (j < lp / 2) dst[j] = 2.f * R[j];
        }
    } else if (lane == 0) {
        // MMA issue: chunk c's 12 MMAs (M128 N lp K8) once its operands and its accumulator are ready
        const uint32_t idesc = idesc_tf32(128, lp);
        for (int c = 0; c < NCH; ++c) {
            const int st = c % NAST, pr = c >> 1;
            wait(&ab_full[st], (c / NAST) & 1);
            if ((c & 1) == 0 && pr >= 2) wait(&acc_free[pr & 1], ((pr - 2) >> 1) & 1);
            fence_after();
            const uint32_t bh = sb + st * stb, bl = bh + plane;
            const uint32_t ah = tm + col_a_hi(st), al = tm + col_a_lo(st), d = tm + col_main(pr & 1);
#pragma unroll
            for (int kk = 0; kk < KC / 8; ++kk) {
                const uint32_t off = kk * 2 * LBO;
                mma_tf32_ta(d, al + 8 * kk, smem_desc(bh + off, LBO, SBO), idesc, ((c & 1) || kk) ? 1u : 0u);
                mma_tf32_ta(d, ah + 8 * kk, smem_desc(bh + off, LBO, SBO), idesc, 1u);
                mma_tf32_ta(d, ah + 8 * kk, smem_desc(bl + off, LBO, SBO), idesc, 1u);
            }
            mma_commit(&mma_bar[st]);
        }
    }
    __syncwarp();
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tm, TMEM_COLS);
}

// ---- forward contraction on the tensor cores ---------------------------------------------------
// A_b = I + sum_l eps_bl Ubar_l for every entry e of every lower tile and every batch element b:
// D[e][b] = sum_l Ubar[e][l] E[b][l] with M = 128 entries (a row block of a tile), N = the batch
// chunk (16 .. 256, zero-padded), K = lp.  3xTF32 as everywhere here; the two cross products go
// into the accumulator first, while it is still small, and the hi*hi products last, so the tensor
// core's one-way accumulation drift acts on the main term over only lp / 8 instructions.  The
// identity is added in FP32 by the epilogue.  Persistent CTAs (one per SM) walk the row blocks in
// steps of the grid; per CTA the batch chunk's E (hi and lo planes) stays in shared memory:
//   warps 0-3 (producers): load a row block's table rows (lane = entry, coalesced per l), split them
//              and write the K-major canonical A operand into one of two shared-memory stages;
//   warp 8    (MMA issue): one thread issues the block's 3 lp / 8 MMAs (A and B from shared memory)
//              into one of two tensor-memory accumulators and commits them;
//   warps 4-7 (epilogue): drain the accumulator (lane = entry, 32 batch columns per load), add the
//              identity on the diagonal and store A[b][e] (each warp store 128 contiguous bytes).
constexpr int FWD_PROD = 128;
constexpr int FWD_NTH = 2 * FWD_PROD + 32;
constexpr int FWD_NBMAX = 256;

struct FwdCtl {
    uint64_t a_full[2];   // A stage written (one arrival per producer warp)
    uint64_t a_empty[2];  // A stage's MMAs completed
    uint64_t d_full[2];   // accumulator's MMAs completed
    uint64_t d_empty[2];  // accumulator drained (one arrival per epilogue warp)
    uint64_t fin;         // the issuer's last commit
    uint32_t tbase;
};

template <int LP>
__global__ void __launch_bounds__(FWD_NTH) contract_fwd_tc(int B, int nblk, int nb, const float* __restrict__ U,
                                                           const float* __restrict__ eps, float* __restrict__ A,
                                                           size_t strideA, int* err)
{
    static_assert(LP % 16 == 0 && LP <= 64, "lp");
    constexpr uint32_t SBO_A = LP / 4 * 128;                 // row-group stride of the K-major operands
    constexpr uint32_t A_PLANE = 128u * LP * 4;              // one plane of an A stage
    extern __shared__ __align__(1024) unsigned char fsm_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(fsm_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t b_plane = (uint32_t)nb * LP * 4;
    unsigned char* sB = sm;                                   // [hi, lo][nb x LP]
    unsigned char* sA = sm + 2 * b_plane;                     // [stage][hi, lo][128 x LP]
    __shared__ FwdCtl ctl;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int b_begin = blockIdx.y * nb;
    bool ok = true;
    auto wait = [&](uint64_t* bar, uint32_t parity) {
        if (!ok) return;
        ok = mbar_wait(bar, parity, kMaxIter, err);
        if (!ok) atomicExch(err, 1);
    };
    // E's split planes, K-major canonical (row = batch element of the chunk, K = l)
    for (int k = threadIdx.x; k < nb * LP; k += blockDim.x) {
        const int r = k / LP, l = k % LP, b = b_begin + r;
        const float v = (b < B) ? eps[(size_t)l * B + b] : 0.f;
        const float hi = tf32_rn(v), lo = tf32_rn(v - hi);
        const uint32_t off = (uint32_t)((r >> 3) * SBO_A + (l >> 2) * 128 + (r & 7) * 16 + (l & 3) * 4);
        *reinterpret_cast<float*>(sB + off) = hi;
        *reinterpret_cast<float*>(sB + b_plane + off) = lo;
    }
    // two accumulators of nb <= 256 columns, acc apart (a power of two >= 32): 2 acc <= 512 columns
    uint32_t acc = 32;
    while (acc < (uint32_t)nb) acc *= 2;
    if (warp == 8) tmem_alloc(&ctl.tbase, 2 * acc);
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&ctl.a_full[i], FWD_PROD / 32);
            mbar_init(&ctl.a_empty[i], 1);
            mbar_init(&ctl.d_full[i], 1);
            mbar_init(&ctl.d_empty[i], FWD_PROD / 32);
        }
        mbar_init(&ctl.fin, 1);
        fence_mbar_init();
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = ctl.tbase;
    if (warp < 4) {
        // producers: row p of every row block this CTA takes
        const int p = threadIdx.x;
        int i = 0;
        for (int m = blockIdx.x; m < nblk && ok; m += gridDim.x, ++i) {
            const int t = m / (TILE_ELEMS / 128), e = (m % (TILE_ELEMS / 128)) * 128 + p;
            const float* src = U + (size_t)t * TILE_ELEMS * LP + e;
            float v[LP];
#pragma unroll
            for (int l = 0; l < LP; ++l) v[l] = __ldg(src + (size_t)l * TILE_ELEMS);
            const int st = i & 1;
            wait(&ctl.a_empty[st], ((i >> 1) & 1) ^ 1);
            if (!ok) break;
            unsigned char* hi = sA + st * 2 * A_PLANE;
            const uint32_t row = (uint32_t)((p >> 3) * SBO_A + (p & 7) * 16);
#pragma unroll
            for (int k4 = 0; k4 < LP / 4; ++k4) {
                float4 h, lo;
                split1(make_float4(v[4 * k4], v[4 * k4 + 1], v[4 * k4 + 2], v[4 * k4 + 3]), h, lo);
                *reinterpret_cast<float4*>(hi + row + k4 * 128) = h;
                *reinterpret_cast<float4*>(hi + A_PLANE + row + k4 * 128) = lo;
            }
            fence_proxy_async();  // the MMA reads the stage through the async proxy
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctl.a_full[st]);
        }
    } else if (warp < 8) {
        // epilogue: row (entry) 32 (warp % 4) + lane of every row block
        const int p = (warp - 4) * 32 + lane;
        int i = 0;
        for (int m = blockIdx.x; m < nblk; m += gridDim.x, ++i) {
            const int dsel = i & 1;
            wait(&ctl.d_full[dsel], (i >> 1) & 1);
            if (!ok) break;
            fence_after();
            const int t = m / (TILE_ELEMS / 128), e = (m % (TILE_ELEMS / 128)) * 128 + p;
            int I, J;
            tile_coords(t, I, J);
            const float one = (I == J && (e % TS) == (e / TS)) ? 1.f : 0.f;
            float* dst = A + (size_t)t * TILE_ELEMS + e;
            for (int c0 = 0; c0 < nb; c0 += 32) {
                float v[32];
                tmem_ld32w(tm + lane_base() + acc * dsel + c0, v);  // columns past nb: unused
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int b = b_begin + c0 + j;
                    if (c0 + j < nb && b < B) dst[(size_t)b * strideA] = v[j] + one;
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctl.d_empty[dsel]);
        }
    } else if (lane == 0) {
        // the MMA issuer
        const uint32_t idesc = idesc_tf32(128, nb);
        const uint32_t a0 = smem_u32(sA), bh = smem_u32(sB), bl = bh + b_plane;
        int i = 0;
        for (int m = blockIdx.x; m < nblk; m += gridDim.x, ++i) {
            const int st = i & 1, dsel = i & 1;
            wait(&ctl.a_full[st], (i >> 1) & 1);
            wait(&ctl.d_empty[dsel], ((i >> 1) & 1) ^ 1);
            if (!ok) break;
            fence_after();
            const uint32_t ah = a0 + st * 2 * A_PLANE, al = ah + A_PLANE, d = tm + acc * dsel;
#pragma unroll
            for (int kk = 0; kk < LP / 8; ++kk) {
                const uint32_t off = kk * 2 * LBO;
                mma_tf32(d, smem_desc(al + off, LBO, SBO_A), smem_desc(bh + off, LBO, SBO_A), idesc, kk ? 1u : 0u);
                mma_tf32(d, smem_desc(ah + off, LBO, SBO_A), smem_desc(bl + off, LBO, SBO_A), idesc, 1u);
            }
#pragma unroll
            for (int kk = 0; kk < LP / 8; ++kk) {
                const uint32_t off = kk * 2 * LBO;
                mma_tf32(d, smem_desc(ah + off, LBO, SBO_A), smem_desc(bh + off, LBO, SBO_A), idesc, 1u);
            }
            mma_commit(&ctl.a_empty[st]);
            mma_commit(&ctl.d_full[dsel]);
        }
        // every MMA issued so far completes before tensor memory is freed (bounded, ignores the abort flag)
        mma_commit(&ctl.fin);
        if (!mbar_wait(&ctl.fin, 0, kMaxIter)) atomicExch(err, 1);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 8) tmem_dealloc(tm, 2 * acc);
}

// Self-test of the bounded-wait path: one thread waits, with a short limit, on an mbarrier
// that nothing arrives on; the wait must give up and report CG_ERR_TIMEOUT.
__global__ void wait_timeout_probe(int* status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        *status = mbar_wait(&bar, 0, 1u << 12) ? CG_OK : CG_ERR_TIMEOUT;
    }
}

// Rate probe for the MMA form the factorisation kernels issue: tcgen05.mma kind::tf32, M128 N128 K8,
// A from tensor memory, B from shared memory (K-major, no swizzle), one issuing thread per CTA and
// one CTA per SM.  The operands hold arbitrary finite values; the accumulator is never read.  The
// issuing thread commits its MMAs to an mbarrier and waits for them with a time limit (2 s of
// %globaltimer); a wait that gives up sets *err.  Tensor memory is freed after the wait either way.
__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void __launch_bounds__(128) mma_rate_probe(int iters, int* err)
{
    constexpr int KC_P = 32;                     // K extent of the B operand in shared memory
    constexpr uint32_t LBO_P = 128, SBO_P = KC_P / 4 * 128;
    __shared__ __align__(1024) float sb[128 * KC_P];
    __shared__ uint64_t done;
    __shared__ uint32_t tbase;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int e = threadIdx.x; e < 128 * KC_P; e += blockDim.x) sb[e] = 1.0f + 1e-3f * (float)((e * 37) % 101);
    if (warp == 0) tmem_alloc(&tbase, 256);  // D: columns 0-127, A: 128-159
    if (threadIdx.x == 0) {
        mbar_init(&done, 1);
        fence_mbar_init();
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = tbase;
    {
        float v[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = 0.5f + 1e-3f * (float)((lane * 13 + i * 7 + warp) % 97);
        tmem_st32(tm + ((uint32_t)(warp * 32) << 16) + 128, v);
    }
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        fence_after();
        const uint32_t idesc = idesc_tf32(128, 128);
        const uint32_t b0 = smem_u32(sb);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int kk = 0; kk < KC_P / 8; ++kk)
                mma_tf32_ta(tm, tm + 128 + 8 * kk, smem_desc(b0 + kk * 2 * LBO_P, LBO_P, SBO_P), idesc,
                            (it || kk) ? 1u : 0u);
        }
        mma_commit(&done);
        const uint64_t t0 = global_ns();
        bool ok = false;
        while (!ok) {
            uint32_t d;
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(d)
                : "r"(smem_u32(&done)), "r"(0u)
                : "memory");
            ok = d != 0;
            if (!ok && global_ns() - t0 > 2000000000ull) break;
        }
        if (!ok) atomicExch(err, 1);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tm, 256);
}

// FP32-pipe probe: 8 independent packed two-lane FMA chains (fma.rn.f32x2, the form the FP32
// contraction issues) per thread, 8 warps per CTA, 4 CTAs per SM; the chains stay bounded
// (a += c m with |c m| = 1e-7) and the result is kept live by a store that never happens
__global__ void __launch_bounds__(256) fma2_rate_probe(int iters, float seed, float* sink)
{
    float a[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) a[i] = seed * (float)(threadIdx.x + i);
    const float m0 = 0.999f, m1 = 1.0001f, c0 = 1e-7f, c1 = -1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int i = 0; i < 16; i += 2) fma2(a[i], a[i + 1], c0, c1, m0, m1);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 16; ++i) s += a[i];
    if (s == 12345.678f) sink[threadIdx.x] = s;
}

}  // namespace

int probe_fp32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms_per_launch)
{
    if (iters <= 0 || reps <= 0) { ctx->err = "probe: iters and reps must be positive"; return CG_ERR_BAD_ARG; }
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CG_CUDA_TRY(ctx, cudaMalloc((void**)&sink, 256 * sizeof(float)));
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int grid = 4 * ctx->sm_count;
    if (e == cudaSuccess) {
        fma2_rate_probe<<<grid, 256, 0, ctx->stream>>>(iters, 1e-3f, sink);  // warm-up
        count_launch(ctx);
        e = cudaEventRecord(e0, ctx->stream);
    }
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
        fma2_rate_probe<<<grid, 256, 0, ctx->stream>>>(iters, 1e-3f, sink);
        count_launch(ctx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    int rc = CG_OK;
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    else {
        // 16 packed FMAs (32 lane-FMAs, 64 flops) per thread and iteration
        const double flops = 64.0 * iters * 256.0 * grid * reps;
        *tflops = flops / (ms * 1e-3) / 1e12;
        *ms_per_launch = ms / reps;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    return rc;
}

int probe_tf32_rate(cg_ctx* ctx, int iters, int reps, double* tflops, double* ms_per_launch)
{
    if (iters <= 0 || reps <= 0) { ctx->err = "probe: iters and reps must be positive"; return CG_ERR_BAD_ARG; }
    int* d_err = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CG_CUDA_TRY(ctx, cudaMalloc((void**)&d_err, sizeof(int)));
    int rc = CG_OK;
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        mma_rate_probe<<<ctx->sm_count, 128, 0, ctx->stream>>>(iters, d_err);  // warm-up
        count_launch(ctx);
        e = cudaEventRecord(e0, ctx->stream);
    }
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
        mma_rate_probe<<<ctx->sm_count, 128, 0, ctx->stream>>>(iters, d_err);
        count_launch(ctx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    float ms = 0;
    int herr = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = CG_ERR_CUDA; }
    else if (herr) { ctx->err = "probe: a bounded wait gave up"; rc = CG_ERR_TIMEOUT; }
    else {
        const double flops = 2.0 * 128 * 128 * 8 * 4.0 * iters * (double)ctx->sm_count * reps;
        *tflops = flops / (ms * 1e-3) / 1e12;
        *ms_per_launch = ms / reps;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d_err);
    return rc;
}

static int tc_smem()
{
    const int fac = (2 * 128 * 129 + 64 * 65) * (int)sizeof(float);  // block, its inverse, scratch
    const int ring = NSTB * (int)STB_BYTES + NSTA * (int)STA_BYTES;
    return (ring > fac ? ring : fac) + 1024;
}

template <class K>
static int set_smem(cg_ctx* ctx, K kern)
{
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem()));
    return CG_OK;
}

size_t tc_split_elems(int nt) { return (size_t)ntiles_lower(nt) * SC_TILE; }
size_t tc_c1_elems(int nt) { return (size_t)ntiles_lower(nt) * C1_TILE; }
size_t tc_linv_elems(int nt) { return (size_t)(nt / 2) * LINV_SC; }
// work-queue counters after the error flag: one per panel launch of the Cholesky (slots 0 .. nt/2 - 1),
// one per update launch (nt/2 .. nt - 1), the streamed lauum's (nt), one per streamed trtri row
// (nt + 1 + I2, I2 < nt/2)
int tc_queue_slots(int nt) { return nt + 1 + nt / 2; }

// the Cholesky's column block J2: the update (with the diagonal blocks' factorisation) and the panel solve
static void chol_column(cg_ctx* ctx, int J2, int B, int nt, const float* A, float* Ls, float* Lc, float* Linv,
                        float* Ms, float* Mc, float* diag, int* status, int* d_err, cudaStream_t s)
{
    const int nt2 = nt / 2;
    // diagonal CTAs, then one CTA per off-diagonal block (J2 = 0) or persistent CTAs
    const int noff = (nt2 - J2 - 1) * B;
    const int cap = J2 == 0 ? 4 * ctx->sm_count : (ctx->tune.chol_ctas > 0 ? ctx->tune.chol_ctas : ctx->sm_count);
    const int grid = B + (noff < cap ? noff : cap);
    chol_tc_update<<<grid, NTH, tc_smem(), s>>>(J2, nt, B, A, Ls, Lc, Linv, Ms, Mc, diag, status,
                                                d_err + 1 + nt2 + J2, d_err, ctx->tune.diag_sq);
    count_launch(ctx);
}

// pc_default: the persistent CTA count when the knob panel_ctas is 0
static void chol_panel(cg_ctx* ctx, int J2, int B, int nt, float* Ls, float* Lc, const float* Linv, int* d_err,
                       cudaStream_t s, int pc_default)
{
    const int nt2 = nt / 2;
    if (J2 + 1 >= nt2) return;
    const int items = (nt2 - J2 - 1) * B;
    const int pc = ctx->tune.panel_ctas > 0 ? ctx->tune.panel_ctas : pc_default;
    chol_tc_panel<<<items < pc ? items : pc, NTH, tc_smem(), s>>>(J2, nt, B, Ls, Lc, Linv, d_err + 1 + J2, d_err);
    count_launch(ctx);
}

// trtri's row block I2 >= 1 (the diagonal blocks M_II come from the Cholesky): its blocks J2 < I2
// read L's row panel I2 (final once the Cholesky's panel I2 - 1 is done), Linv_I2 (from column I2's
// update) and M's rows above I2 (earlier rows), and write M's row I2, which no later Cholesky step reads
static void trtri_row(cg_ctx* ctx, int I2, int B, int nt, const float* Ls, const float* Linv, float* Ms, float* Mc,
                      int* d_err, cudaStream_t s)
{
    if (ctx->tune.trtri == 1) {
        const int items = I2 * B;
        trtri_tc_stream<<<items < ctx->sm_count ? items : ctx->sm_count, NTH, tc_smem(), s>>>(
            I2, nt, B, Ls, Linv, Ms, Mc, d_err + 1 + nt + 1 + I2, d_err);
    } else {
        trtri_tc_row<<<dim3(I2, B), NTH, tc_smem(), s>>>(I2, nt, Ls, Linv, Ms, Mc, d_err);
    }
    count_launch(ctx);
}

static int trtri_smem(cg_ctx* ctx)
{
    return ctx->tune.trtri == 1 ? set_smem(ctx, trtri_tc_stream) : set_smem(ctx, trtri_tc_row);
}

int tiled_cholesky_tc(cg_ctx* ctx, int B, int nt, const float* A, float* Ls, float* Lc, float* Linv, float* Ms,
                      float* Mc, float* diag, int* status, int* d_err, cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core Cholesky needs an even tile count"; return CG_ERR_BAD_ARG; }
    int rc;
    if ((rc = set_smem(ctx, chol_tc_update)) || (rc = set_smem(ctx, chol_tc_panel))) return rc;
    for (int J2 = 0; J2 < nt / 2; ++J2) {
        chol_column(ctx, J2, B, nt, A, Ls, Lc, Linv, Ms, Mc, diag, status, d_err, s);
        chol_panel(ctx, J2, B, nt, Ls, Lc, Linv, d_err, s, ctx->sm_count);
    }
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int tiled_trtri_tc(cg_ctx* ctx, int B, int nt, const float* Ls, const float* Linv, float* Ms, float* Mc,
                   int* d_err, cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core trtri needs an even tile count"; return CG_ERR_BAD_ARG; }
    int rc;
    if ((rc = trtri_smem(ctx))) return rc;
    for (int I2 = 1; I2 < nt / 2; ++I2) trtri_row(ctx, I2, B, nt, Ls, Linv, Ms, Mc, d_err, s);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

// The Cholesky on the context's high-priority stream and trtri's rows on s, each row after its
// column's update (the block scheduler then gives free SMs to the Cholesky's CTAs first, and
// trtri's fill the rest: the panel solves' HBM-bound launches, the update's tails); s waits for
// the whole Cholesky at the end.  Same launches, same results as tiled_cholesky_tc + tiled_trtri_tc.
int tiled_chol_trtri_tc(cg_ctx* ctx, int B, int nt, const float* A, float* Ls, float* Lc, float* Linv, float* Ms,
                        float* Mc, float* diag, int* status, int* d_err, cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core Cholesky needs an even tile count"; return CG_ERR_BAD_ARG; }
    int rc;
    if ((rc = set_smem(ctx, chol_tc_update)) || (rc = set_smem(ctx, chol_tc_panel)) || (rc = trtri_smem(ctx)))
        return rc;
    if (!ctx->hi) {
        int least = 0, greatest = 0;
        CG_CUDA_TRY(ctx, cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CG_CUDA_TRY(ctx, cudaStreamCreateWithPriority(&ctx->hi, cudaStreamNonBlocking, greatest));
    }
    for (cudaEvent_t* e : {&ctx->ev_fork, &ctx->ev_col, &ctx->ev_join})
        if (!*e) CG_CUDA_TRY(ctx, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    CG_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_fork, s));
    CG_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->hi, ctx->ev_fork, 0));
    for (int J2 = 0; J2 < nt / 2; ++J2) {
        chol_column(ctx, J2, B, nt, A, Ls, Lc, Linv, Ms, Mc, diag, status, d_err, ctx->hi);
        if (J2 >= 1) {
            CG_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_col, ctx->hi));
            CG_CUDA_TRY(ctx, cudaStreamWaitEvent(s, ctx->ev_col, 0));
            trtri_row(ctx, J2, B, nt, Ls, Linv, Ms, Mc, d_err, s);
        }
        // the panel solve is bound by its writes of L: 7/8 of the SMs keep that rate and leave the
        // rest to trtri's rows (at nside 16, batch 256: 29.51 -> 29.35 ms per call; half of them: 29.75)
        chol_panel(ctx, J2, B, nt, Ls, Lc, Linv, d_err, ctx->hi, ctx->sm_count * 7 / 8);
    }
    stage_mark(ctx, ST_TRTRI, ctx->hi);  // the Cholesky's end: the trtri stage is the rows left after it
    CG_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_join, ctx->hi));
    CG_CUDA_TRY(ctx, cudaStreamWaitEvent(s, ctx->ev_join, 0));
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int tiled_lauum_tc(cg_ctx* ctx, int B, int nt, const float* Ms, const float* Mc, float* V, int* d_err,
                   const double* y, int ystride, float2* part, cudaStream_t s)
{
    if (nt % 2) { ctx->err = "tensor-core lauum needs an even tile count"; return CG_ERR_BAD_ARG; }
    int rc;
    const int nt2 = nt / 2, nsup = nt2 * (nt2 + 1) / 2;
    if (ctx->tune.lauum == 1) {
        if ((rc = set_smem(ctx, lauum_tc_stream))) return rc;
        const int items = nsup * B;
        lauum_tc_stream<<<items < ctx->sm_count ? items : ctx->sm_count, NTH, tc_smem(), s>>>(
            nt, B, Ms, Mc, V, d_err + 1 + nt, d_err);
    } else if (ctx->tune.lauum == 2) {
        if ((rc = set_smem(ctx, lauum_tc<A_SMEM_C1>))) return rc;
        lauum_tc<A_SMEM_C1><<<dim3(nsup, B), NTH, tc_smem(), s>>>(nt, Ms, Mc, V, d_err, y, ystride, part);
    } else {
        if ((rc = set_smem(ctx, lauum_tc<A_REG_SC>))) return rc;
        lauum_tc<A_REG_SC><<<dim3(nsup, B), NTH, tc_smem(), s>>>(nt, Ms, Mc, V, d_err, y, ystride, part);
    }
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

bool adjoint_tc_ok(int lp) { return lp % 16 == 0 && lp >= 16 && lp <= 96; }

// G chunks per fetch group, NB group buffers: buffers and B stages within 224 KB
template <int RC, int G, int NB>
static int launch_adj_tc(cg_ctx* ctx, dim3 grid, int B, int lp, const float* U, const float* V, size_t strideA,
                         float* part, int* d_err, cudaStream_t s)
{
    static_assert(NB >= 2 && NAST * 2 * 2 * RC * KC * 4 + NB * (128 + 2 * RC) * G * 128 <= 224 * 1024, "shared memory");
    const int smem = NAST * 2 * lp * KC * 4 + NB * (128 + lp) * G * 128;
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(contract_adj_tc<RC, G, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          smem));
    contract_adj_tc<RC, G, NB><<<grid, ADJ_NTH, smem, s>>>(B, lp, U, V, strideA, part, d_err);
    return CG_OK;
}

int adjoint_contract_tc(cg_ctx* ctx, int B, int nt, int lp, const float* U, const float* V, size_t strideA,
                        float* part, int* d_err, cudaStream_t s)
{
    if (!adjoint_tc_ok(lp)) { ctx->err = "tensor-core adjoint contraction needs lp % 16 == 0, lp <= 96"; return CG_ERR_BAD_ARG; }
    const dim3 grid(ntiles_lower(nt), (B + 127) / 128);
    // tuning variants: fetch groups G of two chunks with NB group buffers (default), or shallower rings
    const int v = ctx->tune.adj;
    int rc;
    if (lp <= 48)
        rc = v == 1   ? launch_adj_tc<24, 2, 3>(ctx, grid, B, lp, U, V, strideA, part, d_err, s)
             : v == 2 ? launch_adj_tc<24, 1, 4>(ctx, grid, B, lp, U, V, strideA, part, d_err, s)
             : v == 3 ? launch_adj_tc<24, 4, 2>(ctx, grid, B, lp, U, V, strideA, part, d_err, s)  // 512-byte row runs
                      : launch_adj_tc<24, 2, 4>(ctx, grid, B, lp, U, V, strideA, part, d_err, s);
    else if (lp <= 64)
        rc = v == 2 ? launch_adj_tc<32, 1, 4>(ctx, grid, B, lp, U, V, strideA, part, d_err, s)
                    : launch_adj_tc<32, 2, 3>(ctx, grid, B, lp, U, V, strideA, part, d_err, s);
    else
        rc = v == 2 ? launch_adj_tc<48, 1, 3>(ctx, grid, B, lp, U, V, strideA, part, d_err, s)
                    : launch_adj_tc<48, 2, 2>(ctx, grid, B, lp, U, V, strideA, part, d_err, s);
    if (rc) return rc;
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

bool contract_fwd_tc_ok(int lp) { return lp % 16 == 0 && lp >= 16 && lp <= 64; }

static size_t fwd_tc_smem(int lp, int nb) { return (size_t)2 * nb * lp * 4 + (size_t)2 * 2 * 128 * lp * 4 + 1024; }

int contract_fwd_tc_launch(cg_ctx* ctx, int B, int nt, int lp, const float* U, const float* eps, float* A,
                           size_t strideA, int* d_err, int ctas, cudaStream_t s)
{
    if (!contract_fwd_tc_ok(lp)) { ctx->err = "tensor-core forward contraction needs lp % 16 == 0, lp <= 64"; return CG_ERR_BAD_ARG; }
    // batch chunk: the whole batch up to 256 (rounded up to the MMA's N step of 16), smaller where
    // E's two planes and two A stages would not fit in shared memory
    int nb = ((std::min(B, FWD_NBMAX) + 15) / 16) * 16;
    while (nb > 16 && fwd_tc_smem(lp, nb) > 227 * 1024) nb -= 16;
    const size_t smem = fwd_tc_smem(lp, nb);
    const int nblk = ntiles_lower(nt) * (TILE_ELEMS / 128);
    const int grid_x = std::max(1, std::min(nblk, ctas > 0 ? ctas : ctx->sm_count));
    const dim3 grid(grid_x, (B + nb - 1) / nb);
    switch (lp) {
#define CG_FWD_CASE(LPV)                                                                                          \
    case LPV:                                                                                                      \
        CG_CUDA_TRY(ctx, cudaFuncSetAttribute(contract_fwd_tc<LPV>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                              (int)smem));                                                          \
        contract_fwd_tc<LPV><<<grid, FWD_NTH, smem, s>>>(B, nblk, nb, U, eps, A, strideA, d_err);                   \
        break;
        CG_FWD_CASE(16)
        CG_FWD_CASE(32)
        CG_FWD_CASE(48)
        CG_FWD_CASE(64)
#undef CG_FWD_CASE
    }
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

int selftest_wait_timeout(cg_ctx* ctx, int* host_status)
{
    int* d = nullptr;
    CG_CUDA_TRY(ctx, cudaMalloc((void**)&d, sizeof(int)));
    wait_timeout_probe<<<1, 32, 0, ctx->stream>>>(d);
    count_launch(ctx);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_status, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    if (e != cudaSuccess) {
        ctx->err = cudaGetErrorString(e);
        return CG_ERR_CUDA;
    }
    return CG_OK;
}

}  // namespace cg
