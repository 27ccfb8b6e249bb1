// fs_mlp_tc.cu -- batched forward pass of the learned proposal's network (16 -> 128 -> 128 ->
// 128 -> 16, ReLU, BF16 weights and activations, FP32 accumulation) on the fifth-generation
// tensor cores: tcgen05.mma with both operands in shared memory and the FP32 accumulator in
// tensor memory (TMEM), read back with tcgen05.ld for the bias / ReLU / BF16 epilogue.  No
// counterpart in the reference.  Used by fs_mlp_infer (the held-out gate, predictions); the
// sampler evaluates the network per warp inside the sweep (fs_mlp.cuh).
//
// One CTA = 4 warps = one 128-row tile at a time (persistent over tiles).  Row r of the tile
// is TMEM lane r; warp w reads lanes 32w..32w+31, so each thread owns one row in the
// epilogue.  Operands use the no-swizzle K-major canonical layout: 8 x 8 BF16 core matrices
// of 128 contiguous bytes, core matrices adjacent along K 128 bytes apart (leading byte
// offset), 8-row groups (K / 8) * 128 bytes apart (stride byte offset).  The weights come
// from the sampler's fragment-ordered blob (fs_mlp_pack) and are scattered into that layout
// once per CTA.
//
// Every wait on the MMA completion barrier is bounded; a CTA that gives up writes NaN to its
// rows, releases its tensor memory and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/feynsimul.h"
#include "fs_mlp.cuh"
#include "fs_tc.cuh"

#define TC_M 128                  // rows per tile (the MMA's M)
#define TC_THREADS 128            // 4 warps
#define TC_TMEM_COLS 128          // FP32 accumulator columns (N <= 128)

extern int fsi_thread_error(int code, const char *msg);

struct TcSmem {
    alignas(128) fs_bf16 w1[FS_MLP_H * FS_MLP_IN];   // B operands, [N = out][K = in]
    alignas(128) fs_bf16 w2[FS_MLP_H * FS_MLP_H];
    alignas(128) fs_bf16 w3[FS_MLP_H * FS_MLP_H];
    alignas(128) fs_bf16 w4[FS_MLP_OUT * FS_MLP_H];
    alignas(128) fs_bf16 act[TC_M * FS_MLP_H];        // A operand, [M = row][K]
    float bias[FS_MLP_NBIAS];
    alignas(8) unsigned long long mbar;
    unsigned tmem_base;
    int give_up;
};

// one layer's weights, fragment order -> canonical K-major layout [N][K]
__device__ __forceinline__ void tc_unpack(fs_bf16 *w, const uint2 *__restrict__ frag, int K, int N)
{
    const int NT = N / 8, n_entries = (K / 16) * NT * 32;
    for (int e = threadIdx.x; e < n_entries; e += TC_THREADS) {
        const int lane = e & 31, t = e >> 5;
        const int kt = t / NT, nt = t % NT;
        const int n = nt * 8 + (lane >> 2), k = kt * 16 + (lane & 3) * 2;
        const uint2 u = frag[e];
        *(unsigned *)(w + tc_off(n, k, K)) = u.x;       // W[n][k], W[n][k+1]
        *(unsigned *)(w + tc_off(n, k + 8, K)) = u.y;   // W[n][k+8], W[n][k+9]
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1) fs_mlp_infer_tc_kernel(const uint2 *__restrict__ frag,
                                                                       const float *__restrict__ bias,
                                                                       const float *__restrict__ x,
                                                                       float *__restrict__ y, int n_rows)
{
    extern __shared__ __align__(1024) unsigned char tc_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(tc_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_tiles = (n_rows + TC_M - 1) / TC_M;
    const uint32_t mbar = tc_smem(&S.mbar);

    tc_unpack(S.w1, frag + FS_MLP_OFF_W1, FS_MLP_IN, FS_MLP_H);
    tc_unpack(S.w2, frag + FS_MLP_OFF_W2, FS_MLP_H, FS_MLP_H);
    tc_unpack(S.w3, frag + FS_MLP_OFF_W3, FS_MLP_H, FS_MLP_H);
    tc_unpack(S.w4, frag + FS_MLP_OFF_W4, FS_MLP_H, FS_MLP_OUT);
    for (int i = tid; i < FS_MLP_NBIAS; i += TC_THREADS) S.bias[i] = bias[i];
    if (tid == 0) {
        S.give_up = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&S.tmem_base)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t t_row = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's TMEM lanes
    uint32_t phase = 0;
    bool ok = true;

    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int row = tile * TC_M + tid;  // this thread's row (TMEM lane tid)
        // ---- layer-1 input: 16 features -> BF16, K = 16 ----
        {
            float h[16];
#pragma unroll
            for (int c = 0; c < 16; c++) h[c] = row < n_rows ? x[(size_t)row * 16 + c] : 0.f;
            tc_st8(S.act + tc_off(tid, 0, FS_MLP_IN), h);
            tc_st8(S.act + tc_off(tid, 8, FS_MLP_IN), h + 8);
        }
#pragma unroll 1
        for (int layer = 0; layer < 4 && ok; layer++) {
            const int K = layer == 0 ? FS_MLP_IN : FS_MLP_H;
            const int N = layer == 3 ? FS_MLP_OUT : FS_MLP_H;
            const fs_bf16 *W = layer == 0 ? S.w1 : layer == 1 ? S.w2 : layer == 2 ? S.w3 : S.w4;
            tc_fence_async();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                const uint32_t idesc = tc_idesc(TC_M, N);
#pragma unroll 1
                for (int kk = 0; kk < K / 16; kk++)
                    tc_mma(tmem, tc_desc(S.act + kk * 128, K), tc_desc(W + kk * 128, K), idesc, kk > 0);
                tc_commit(mbar);
            }
            if (!tc_wait(mbar, phase)) S.give_up = 1;
            phase ^= 1u;
            tc_fence_after();
            __syncthreads();
            if (S.give_up) {
                ok = false;
                break;
            }
            const float *b = S.bias + (layer == 0 ? FS_MLP_OFF_B1 : layer == 1 ? FS_MLP_OFF_B2
                                                                  : layer == 2 ? FS_MLP_OFF_B3 : FS_MLP_OFF_B4);
            if (layer < 3) {
                // bias, ReLU, BF16: the next layer's A operand (K = 128)
#pragma unroll 1
                for (int c0 = 0; c0 < FS_MLP_H; c0 += 16) {
                    float v[16];
                    tc_ld16(t_row + (uint32_t)c0, v);
#pragma unroll
                    for (int i = 0; i < 16; i++) v[i] = fmaxf(v[i] + b[c0 + i], 0.f);
                    tc_st8(S.act + tc_off(tid, c0, FS_MLP_H), v);
                    tc_st8(S.act + tc_off(tid, c0 + 8, FS_MLP_H), v + 8);
                }
            } else {
                float v[16];
                tc_ld16(t_row, v);
                if (row < n_rows)
#pragma unroll
                    for (int i = 0; i < 16; i++) y[(size_t)row * 16 + i] = v[i] + b[i];
            }
        }
        if (!ok) {
            for (int t2 = tile; t2 < n_tiles; t2 += gridDim.x) {
                const int r2 = t2 * TC_M + tid;
                if (r2 < n_rows)
                    for (int i = 0; i < 16; i++) y[(size_t)r2 * 16 + i] = __int_as_float(0x7FC00000);
            }
        }
    }
    // release the tensor memory once no MMA is in flight: after a give-up, wait (bounded)
    // for the last commit's phase before freeing the columns
    if (!ok) tc_wait(mbar, phase ^ 1u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
    (void)lane;
}

// Launched by fs_mlp_infer (fs_mlp_train.cu): one CTA per SM pair at most, persistent over
// the 128-row tiles.
int fsi_mlp_infer_tc(const void *frag, const float *bias, const float *x, float *y, int n_rows, cudaStream_t s)
{
    // per call: the attribute belongs to the current device (a process may use several)
    {
        cudaError_t e = cudaFuncSetAttribute(fs_mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(TcSmem));
        if (e != cudaSuccess) return fsi_thread_error(FS_ERR_CUDA, cudaGetErrorString(e));
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
    const int n_tiles = (n_rows + TC_M - 1) / TC_M;
    const int grid = n_tiles < 2 * sms ? n_tiles : 2 * sms;
    fs_mlp_infer_tc_kernel<<<grid, TC_THREADS, sizeof(TcSmem), s>>>((const uint2 *)frag, bias, x, y, n_rows);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fsi_thread_error(FS_ERR_LAUNCH, cudaGetErrorString(e));
    return FS_OK;
}
