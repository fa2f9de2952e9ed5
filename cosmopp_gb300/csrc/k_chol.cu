// Batched tiled Cholesky, triangular inverse and inverse assembly on the
// lower-tile layout of cg_internal.h, templated on FP64 (plain path) and FP32
// (whitened matrices of the mixed path).
//
// Replaces the reference's packed LAPACK calls dpptrf_ / dpptri_
// (source/matrix_impl.cpp:237-265, called from source/likelihood.cpp:113,132)
// and logDetFromCholeskyFactorization (source/matrix_impl.cpp:322-338).
//
//   per step k:  chol_diag   L_kk = chol(A_kk), Dinv_kk = L_kk^-1, diag, status
//                chol_panel  L_ik = A_ik Dinv_kk^T               (i > k)
//                chol_update A_ij -= L_ik L_jk^T                 (k < j <= i)
//   trtri rows:  M_ii = Dinv_ii, M_ij = -Dinv_ii sum_{k=j}^{i-1} L_ik M_kj, the sums
//                accumulated right-looking (one tile product per block)
//   lauum:       V_ij = sum_{k>=i} M_ki^T M_kj  (= C^-1, lower tiles)
//
// Every grid has a batch dimension; nothing waits on another block.
#include "cg_internal.h"
#include "cg_tile.cuh"

namespace cg {

namespace {

using namespace tile;

template <typename T>
__device__ __forceinline__ T my_sqrt(T v);
template <>
__device__ __forceinline__ double my_sqrt<double>(double v) { return sqrt(v); }
template <>
__device__ __forceinline__ float my_sqrt<float>(float v) { return sqrtf(v); }

// ---- step kernels ----------------------------------------------------------

// Factor the diagonal tile of step k for every batch element, write L_kk
// (strict upper zeroed), its inverse Dinv_kk and the diagonal of L.
template <typename T>
__global__ void __launch_bounds__(NT_THREADS) chol_diag(int k, int nt, T* A, size_t strideA, T* Dinv,
                                                        T* diag, int* status)
{
    constexpr int L = TS + 1;
    extern __shared__ unsigned char smem_raw[];
    T* s = reinterpret_cast<T*>(smem_raw);  // s[c*L + r] = A(r, c)
    T* sinv = s + TS * L;
    __shared__ int bad;
    const int b = blockIdx.x;
    T* tile = A + (size_t)b * strideA + (size_t)tile_index(k, k) * TILE_ELEMS;
    // The trailing updates are summed in u (sinv's storage, unused until the inverse) and
    // subtracted from the column once, when it is reached.  Subtracting each rank-1 term
    // from A directly loses every term below half an ulp of A's diagonal (about 1 for a
    // whitened matrix), which biases L's diagonal, hence the log-determinant, upwards.
    T* u = sinv;
    for (int e = threadIdx.x; e < TILE_ELEMS; e += blockDim.x) {
        s[(e / TS) * L + (e % TS)] = tile[e];
        u[(e / TS) * L + (e % TS)] = T(0);
    }
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int c = 0; c < TS; ++c) {
        if (threadIdx.x == 0) {
            T v = s[c * L + c] - u[c * L + c];
            if (!(v > T(0))) {  // not positive definite (or NaN): flag, keep going on a benign value
                bad = 1;
                v = T(1);
            }
            s[c * L + c] = my_sqrt(v);
        }
        __syncthreads();
        const T piv = s[c * L + c];
        for (int r = c + 1 + threadIdx.x; r < TS; r += blockDim.x) s[c * L + r] = (s[c * L + r] - u[c * L + r]) / piv;
        __syncthreads();
        const int m = TS - c - 1;  // trailing triangle of size m
        const int cnt = m * (m + 1) / 2;
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            int rr, ss;
            tile_coords(e, rr, ss);  // rr >= ss within the trailing block
            const int r = c + 1 + rr, q = c + 1 + ss;
            u[q * L + r] += s[c * L + r] * s[c * L + q];
        }
        __syncthreads();
    }
    // inverse of the lower-triangular factor: one column per thread
    if (threadIdx.x < TS) {
        const int c = threadIdx.x;
        for (int r = 0; r < TS; ++r) {
            if (r < c) { sinv[c * L + r] = T(0); continue; }
            T acc = (r == c) ? T(1) : T(0);
            for (int m = c; m < r; ++m) acc -= s[m * L + r] * sinv[c * L + m];
            sinv[c * L + r] = acc / s[r * L + r];
        }
    }
    __syncthreads();
    T* dinv = Dinv + ((size_t)b * nt + k) * TILE_ELEMS;
    for (int e = threadIdx.x; e < TILE_ELEMS; e += blockDim.x) {
        const int r = e % TS, c = e / TS;
        tile[e] = (r >= c) ? s[c * L + r] : T(0);
        dinv[e] = sinv[c * L + r];
    }
    if (threadIdx.x < TS) diag[(size_t)b * nt * TS + k * TS + threadIdx.x] = s[threadIdx.x * L + threadIdx.x];
    if (threadIdx.x == 0 && bad && status && status[b] == CG_OK) status[b] = CG_ERR_NOT_PD;
}

// L_ik = A_ik Dinv_kk^T for i = k+1 .. nt-1
template <typename T>
__global__ void __launch_bounds__(NT_THREADS) chol_panel(int k, int nt, T* A, size_t strideA, const T* Dinv)
{
    extern __shared__ unsigned char smem_raw[];
    constexpr int L = SmemLd<T>::v;
    T* sX = reinterpret_cast<T*>(smem_raw);
    T* sY = sX + TS * L;
    const int i = k + 1 + blockIdx.x, b = blockIdx.y;
    T* tile = A + (size_t)b * strideA + (size_t)tile_index(i, k) * TILE_ELEMS;
    load_direct(sX, tile);
    load_direct(sY, Dinv + ((size_t)b * nt + k) * TILE_ELEMS);  // sY[m][c] = Dinv(c, m)
    __syncthreads();
    int r0, c0;
    micro_coords(r0, c0);
    T acc[4][4] = {};
    tile_mma(sX, sY, acc, r0, c0);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) tile[(r0 + a) + TS * (c0 + q)] = acc[a][q];
}

// A_ij -= L_ik L_jk^T over the trailing lower triangle of step k
template <typename T>
__global__ void __launch_bounds__(NT_THREADS) chol_update(int k, int nt, T* A, size_t strideA)
{
    extern __shared__ unsigned char smem_raw[];
    constexpr int L = SmemLd<T>::v;
    T* sX = reinterpret_cast<T*>(smem_raw);
    T* sY = sX + TS * L;
    int ii, jj;
    tile_coords(blockIdx.x, ii, jj);
    const int i = k + 1 + ii, j = k + 1 + jj, b = blockIdx.y;
    T* base = A + (size_t)b * strideA;
    load_direct(sX, base + (size_t)tile_index(i, k) * TILE_ELEMS);
    load_direct(sY, base + (size_t)tile_index(j, k) * TILE_ELEMS);
    __syncthreads();
    int r0, c0;
    micro_coords(r0, c0);
    T acc[4][4] = {};
    tile_mma(sX, sY, acc, r0, c0);
    T* out = base + (size_t)tile_index(i, j) * TILE_ELEMS;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) out[(r0 + a) + TS * (c0 + q)] -= acc[a][q];
}

// Right-looking triangular inverse M = L^-1.  Before row i is finalised, the
// slot of M_ij holds S_ij = sum_{k=j}^{i-1} L_ik M_kj (accumulated by
// trtri_update); trtri_finish turns it into M_ij = -Dinv_ii S_ij (M_ii = Dinv_ii).
template <typename T>
__global__ void __launch_bounds__(NT_THREADS) trtri_finish(int i, int nt, const T* Dinv, T* M, size_t strideA)
{
    extern __shared__ unsigned char smem_raw[];
    constexpr int L = SmemLd<T>::v;
    T* sX = reinterpret_cast<T*>(smem_raw);
    T* sY = sX + TS * L;
    const int j = blockIdx.x, b = blockIdx.y;
    const T* dinv_i = Dinv + ((size_t)b * nt + i) * TILE_ELEMS;
    T* out = M + (size_t)b * strideA + (size_t)tile_index(i, j) * TILE_ELEMS;
    if (j == i) {
        for (int e = threadIdx.x; e < TILE_ELEMS; e += blockDim.x) out[e] = dinv_i[e];
        return;
    }
    load_direct(sX, dinv_i);  // X(r, m) = Dinv(r, m)
    load_trans(sY, out);      // Y(c, m) = S(m, c)
    __syncthreads();
    int r0, c0;
    micro_coords(r0, c0);
    T acc[4][4] = {};
    tile_mma(sX, sY, acc, r0, c0);
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) out[(r0 + a) + TS * (c0 + q)] = -acc[a][q];
}

// S_kj += L_ki M_ij for k = i+1 .. nt-1, j = 0 .. i; grid ((nt-i-1)*(i+1), B)
template <typename T>
__global__ void __launch_bounds__(NT_THREADS) trtri_update(int i, int nt, const T* Lm, T* M, size_t strideA)
{
    extern __shared__ unsigned char smem_raw[];
    constexpr int L = SmemLd<T>::v;
    T* sX = reinterpret_cast<T*>(smem_raw);
    T* sY = sX + TS * L;
    const int k = i + 1 + blockIdx.x / (i + 1), j = blockIdx.x % (i + 1), b = blockIdx.y;
    const T* Lb = Lm + (size_t)b * strideA;
    T* Mb = M + (size_t)b * strideA;
    load_direct(sX, Lb + (size_t)tile_index(k, i) * TILE_ELEMS);  // X(r, m) = L_ki(r, m)
    load_trans(sY, Mb + (size_t)tile_index(i, j) * TILE_ELEMS);   // Y(c, m) = M_ij(m, c)
    __syncthreads();
    int r0, c0;
    micro_coords(r0, c0);
    T acc[4][4] = {};
    tile_mma(sX, sY, acc, r0, c0);
    T* out = Mb + (size_t)tile_index(k, j) * TILE_ELEMS;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) out[(r0 + a) + TS * (c0 + q)] += acc[a][q];
}

// V_ij = sum_{k >= i} M_ki^T M_kj for every lower tile (i, j)
template <typename T>
__global__ void __launch_bounds__(NT_THREADS) lauum_tiles(int nt, const T* M, T* V, size_t strideA)
{
    extern __shared__ unsigned char smem_raw[];
    constexpr int L = SmemLd<T>::v;
    T* sX = reinterpret_cast<T*>(smem_raw);
    T* sY = sX + TS * L;
    int i, j;
    tile_coords(blockIdx.x, i, j);
    const int b = blockIdx.y;
    const T* Mb = M + (size_t)b * strideA;
    int r0, c0;
    micro_coords(r0, c0);
    T acc[4][4] = {};
    for (int k = i; k < nt; ++k) {
        load_trans(sX, Mb + (size_t)tile_index(k, i) * TILE_ELEMS);  // X(r, m) = M_ki(m, r)
        load_trans(sY, Mb + (size_t)tile_index(k, j) * TILE_ELEMS);  // Y(c, m) = M_kj(m, c)
        __syncthreads();
        tile_mma(sX, sY, acc, r0, c0);
        __syncthreads();
    }
    T* out = V + (size_t)b * strideA + (size_t)tile_index(i, j) * TILE_ELEMS;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) out[(r0 + a) + TS * (c0 + q)] = acc[a][q];
}

template <typename T>
size_t pair_smem() { return 2 * (size_t)TS * SmemLd<T>::v * sizeof(T); }
template <typename T>
size_t diag_smem() { return 2 * (size_t)TS * (TS + 1) * sizeof(T); }

// The attribute belongs to the device that is current when it is set, and the FP64 kernels
// need more than the default 48 KB, so it is set on every call (a few host microseconds):
// a context on another device, or the allocation-free entry point on another GPU, then
// launches with it too, and no process-wide flag is shared between threads.
template <typename T>
int set_smem_attrs(cg_ctx* ctx)
{
    const int bytes = (int)pair_smem<T>();
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(chol_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)diag_smem<T>()));
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(chol_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(chol_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(trtri_finish<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(trtri_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    CG_CUDA_TRY(ctx, cudaFuncSetAttribute(lauum_tiles<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return CG_OK;
}

}  // namespace

template <typename T>
int tiled_cholesky(cg_ctx* ctx, int B, int nt, T* A, T* Dinv, T* diag, int* status, size_t strideA, cudaStream_t s)
{
    int rc = set_smem_attrs<T>(ctx);
    if (rc) return rc;
    const size_t sm = pair_smem<T>();
    for (int k = 0; k < nt; ++k) {
        chol_diag<T><<<B, NT_THREADS, diag_smem<T>(), s>>>(k, nt, A, strideA, Dinv, diag, status);
        const int m = nt - k - 1;
        count_launch(ctx, m > 0 ? 3 : 1);
        if (m > 0) {
            chol_panel<T><<<dim3(m, B), NT_THREADS, sm, s>>>(k, nt, A, strideA, Dinv);
            chol_update<T><<<dim3(m * (m + 1) / 2, B), NT_THREADS, sm, s>>>(k, nt, A, strideA);
        }
    }
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

template <typename T>
int tiled_trtri(cg_ctx* ctx, int B, int nt, const T* Lm, const T* Dinv, T* M, size_t strideA, cudaStream_t s)
{
    int rc = set_smem_attrs<T>(ctx);
    if (rc) return rc;
    const size_t sm = pair_smem<T>();
    CG_CUDA_TRY(ctx, cudaMemsetAsync(M, 0, sizeof(T) * strideA * B, s));
    for (int i = 0; i < nt; ++i) {
        trtri_finish<T><<<dim3(i + 1, B), NT_THREADS, sm, s>>>(i, nt, Dinv, M, strideA);
        count_launch(ctx, i + 1 < nt ? 2 : 1);
        if (i + 1 < nt) trtri_update<T><<<dim3((nt - i - 1) * (i + 1), B), NT_THREADS, sm, s>>>(i, nt, Lm, M, strideA);
    }
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

template <typename T>
int tiled_lauum(cg_ctx* ctx, int B, int nt, const T* M, T* V, size_t strideA, cudaStream_t s)
{
    int rc = set_smem_attrs<T>(ctx);
    if (rc) return rc;
    lauum_tiles<T><<<dim3(ntiles_lower(nt), B), NT_THREADS, pair_smem<T>(), s>>>(nt, M, V, strideA);
    count_launch(ctx);
    CG_CUDA_TRY(ctx, cudaGetLastError());
    return CG_OK;
}

template int tiled_cholesky<double>(cg_ctx*, int, int, double*, double*, double*, int*, size_t, cudaStream_t);
template int tiled_cholesky<float>(cg_ctx*, int, int, float*, float*, float*, int*, size_t, cudaStream_t);
template int tiled_trtri<double>(cg_ctx*, int, int, const double*, const double*, double*, size_t, cudaStream_t);
template int tiled_trtri<float>(cg_ctx*, int, int, const float*, const float*, float*, size_t, cudaStream_t);
template int tiled_lauum<double>(cg_ctx*, int, int, const double*, double*, size_t, cudaStream_t);
template int tiled_lauum<float>(cg_ctx*, int, int, const float*, float*, size_t, cudaStream_t);

}  // namespace cg
