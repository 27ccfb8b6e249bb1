// fs_mlp_train.cu -- training of the learned bisection proposal's network on the tcgen05
// tensor cores (BF16 operands, FP32 accumulation in tensor memory), its Adam step and weight
// packing, and the C ABI of training and batched inference.  No counterpart in the
// reference.
//
// Parameters (FP32 master copy, one flat array, FS_MLP_NPARAM floats):
//   W1[128][16] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] W4[16][128] b4[16]
// The forward pass keeps the BF16 activations in shared memory; the loss gradient is formed
// per row; the backward pass runs dA = dZ W and dW = dZ^T A and adds the weight / bias
// gradients to an FP32 gradient array with atomics (the Adam kernel divides nothing: the
// loss is already a batch mean).
//
// Loss (per row, D degrees of freedom, z the midpoint's displacement from the endpoints'
// mean in units of sigma_1): sum_d 0.5 (z_d - o_d)^2 exp(-s_d) + 0.5 s_d with
// s_d = 4 tanh(o_{D+d} / 4): the Gaussian negative log-likelihood of z under N(o, exp(s)).
#include <cuda_runtime.h>

#include <stddef.h>

#include "../../include/feynsimul.h"
#include "fs_mlp.cuh"
#include "fs_tc.cuh"

#define FS_MLP_NPARAM (128 * 16 + 128 + 128 * 128 + 128 + 128 * 128 + 128 + 16 * 128 + 16)
#define P_W1 0
#define P_B1 (P_W1 + 128 * 16)
#define P_W2 (P_B1 + 128)
#define P_B2 (P_W2 + 128 * 128)
#define P_W3 (P_B2 + 128)
#define P_B3 (P_W3 + 128 * 128)
#define P_W4 (P_B3 + 128)
#define P_B4 (P_W4 + 16 * 128)
static_assert(P_W1 % 4 == 0 && P_W2 % 4 == 0 && P_W3 % 4 == 0, "16-byte gradient rows");

// BF16 weight copy used by training (row-major, same order as the FP32 weights, no biases)
#define Q_W1 0
#define Q_W2 (Q_W1 + 128 * 16)
#define Q_W3 (Q_W2 + 128 * 128)
#define Q_W4 (Q_W3 + 128 * 128)
#define Q_N (Q_W4 + 16 * 128)

extern int fsi_thread_error(int code, const char *msg);

__device__ __forceinline__ fs_bf16 f2bf(float x)
{
    unsigned r = fs_pack_bf16(x, 0.f);
    return (fs_bf16)(r & 0xFFFFu);
}

// ---------------------------------------------------------------- tcgen05 training
// The same forward pass, loss and backward pass on the fifth-generation tensor cores, with
// the same BF16 rounding points.  One CTA = 4 warps, persistent over 128-row tiles; thread t
// owns row t of a tile (tensor-memory lane t) in every epilogue.  Tensor memory (512 FP32
// columns): the layer accumulator F (a forward layer's output or a hidden gradient dA), and
// the weight gradients summed over the CTA's tiles: dW2 and dW3 (128 columns each), dW1 (16)
// and dW4 transposed (16; its M is the 128 inputs).  Shared memory holds BF16 tiles in the
// canonical layout of fs_tc.cuh: the activations a1..a3 and the hidden gradient g (128 x
// 128, rows = the tile's rows), the input x and the output gradient dz4 (128 x 16), and the
// weights W1..W4 ([out][in]).  The forward GEMMs read them K-major; dA = dZ W reads W
// MN-major, and dW = dZ^T A reads dZ and A MN-major (K = the tile's rows), so no tile is
// transposed.  The six 128-wide tiles come first and the allocation is padded, so every
// byte a descriptor can reach lies inside it under either reading of its byte offsets.
// Bias gradients are FP32 column sums of the unrounded gradients (warp butterflies, then
// shared-memory atomics).
#define TT_THREADS 128
#define TT_TMEM_COLS 512
#define TT_F 0u
#define TT_DW2 128u
#define TT_DW3 256u
#define TT_DW1 384u
#define TT_DW4 400u

struct TtSmem {
    alignas(1024) fs_bf16 a1[128 * 128];
    alignas(128) fs_bf16 a2[128 * 128];
    alignas(128) fs_bf16 w2[128 * 128];
    alignas(128) fs_bf16 w3[128 * 128];
    alignas(128) fs_bf16 w4[16 * 128];
    alignas(128) fs_bf16 a3[128 * 128];
    alignas(128) fs_bf16 g[128 * 128];
    alignas(128) fs_bf16 x[128 * 16];
    alignas(128) fs_bf16 dz4[128 * 16];
    alignas(128) fs_bf16 w1[128 * 16];
    float bias[128 * 3 + 16];
    float db[128 * 3 + 16];
    float loss;
    alignas(8) unsigned long long mbar;
    unsigned tmem_base;
    int give_up;
};
// farthest byte a read of a 128-wide tile can reach from the tile's start: 8 K-steps of 16
// rows (4096 bytes each) plus 15 column blocks and one row block at the larger offset
#define TT_REACH (7 * 4096 + 15 * 2048 + 256)
#define TT_SMEM_BYTES \
    (offsetof(TtSmem, g) + TT_REACH > sizeof(TtSmem) ? offsetof(TtSmem, g) + TT_REACH : sizeof(TtSmem))

// column sums over the warp's 32 lanes of v[0..32) (one value per column and lane), added to
// dst[lane] for lane < ncols; v is consumed
__device__ __forceinline__ void tt_colsum32(float (&v)[32], float *dst, int lane, int ncols)
{
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const bool up = (lane & w) != 0;
#pragma unroll
        for (int i = 0; i < w; i++) {
            const float send = up ? v[i] : v[i + w];
            const float keep = up ? v[i + w] : v[i];
            v[i] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, w);
        }
    }
    if (lane < ncols) atomicAdd(dst + lane, v[0]);
}

__global__ void __launch_bounds__(TT_THREADS, 1) fs_mlp_train_tc_kernel(
    const float *__restrict__ params, const fs_bf16 *__restrict__ wq, float *__restrict__ grad,
    const float *__restrict__ xin, const float *__restrict__ zin, int n_rows, int dof, float inv_batch,
    float *loss_out)
{
    extern __shared__ __align__(1024) unsigned char tt_raw[];
    TtSmem &S = *reinterpret_cast<TtSmem *>(tt_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_tiles = (n_rows + 127) / 128;
    const uint32_t mbar = tc_smem(&S.mbar);

    // ---- weights (the BF16 training copy, [out][in]) into canonical tiles, eight
    // consecutive inputs (one core-matrix row, 16 bytes) per load and store; biases ----
    {
        const uint4 *q = reinterpret_cast<const uint4 *>(wq);
        for (int i = tid; i < 128 * 16 / 8; i += TT_THREADS)
            *reinterpret_cast<uint4 *>(S.w1 + tc_off(i / 2, (i % 2) * 8, 16)) = q[Q_W1 / 8 + i];
        for (int i = tid; i < 128 * 128 / 8; i += TT_THREADS) {
            *reinterpret_cast<uint4 *>(S.w2 + tc_off(i / 16, (i % 16) * 8, 128)) = q[Q_W2 / 8 + i];
            *reinterpret_cast<uint4 *>(S.w3 + tc_off(i / 16, (i % 16) * 8, 128)) = q[Q_W3 / 8 + i];
        }
        for (int i = tid; i < 16 * 128 / 8; i += TT_THREADS)
            *reinterpret_cast<uint4 *>(S.w4 + tc_off(i / 16, (i % 16) * 8, 128)) = q[Q_W4 / 8 + i];
    }
    for (int i = tid; i < 128; i += TT_THREADS) {
        S.bias[i] = params[P_B1 + i];
        S.bias[128 + i] = params[P_B2 + i];
        S.bias[256 + i] = params[P_B3 + i];
    }
    if (tid < 16) S.bias[384 + tid] = params[P_B4 + tid];
    for (int i = tid; i < 128 * 3 + 16; i += TT_THREADS) S.db[i] = 0.f;
    if (tid == 0) {
        S.loss = 0.f;
        S.give_up = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&S.tmem_base)),
                     "r"(TT_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t t_row = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's lanes
    uint32_t phase = 0;
    bool ok = true, first = true;

    // one step: the operands made visible to the tensor cores, thread 0 issues the MMAs and
    // commits, every thread waits (bounded) for them
    auto step = [&](auto &&issue) {
        tc_fence_async();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            issue();
            tc_commit(mbar);
        }
        if (!tc_wait(mbar, phase)) S.give_up = 1;
        phase ^= 1u;
        tc_fence_after();
        __syncthreads();
        ok = S.give_up == 0;
        return ok;
    };
    // forward epilogue: act = BF16(relu(F + b))
    auto relu_out = [&](fs_bf16 *act, const float *b) {
#pragma unroll 1
        for (int c0 = 0; c0 < 128; c0 += 16) {
            float v[16];
            tc_ld16(t_row + TT_F + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) v[i] = fmaxf(v[i] + b[c0 + i], 0.f);
            tc_st8(act + tc_off(tid, c0, 128), v);
            tc_st8(act + tc_off(tid, c0 + 8, 128), v + 8);
        }
    };
    // backward epilogue: dZ = F * (act > 0) -> g as BF16, its FP32 column sums into dbl
    auto grad_out = [&](const fs_bf16 *act, float *dbl) {
#pragma unroll 1
        for (int c0 = 0; c0 < 128; c0 += 32) {
            float v[32];
            tc_ld16(t_row + TT_F + (uint32_t)c0, *reinterpret_cast<float(*)[16]>(v));
            tc_ld16(t_row + TT_F + (uint32_t)c0 + 16u, *reinterpret_cast<float(*)[16]>(v + 16));
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const uint4 u = *reinterpret_cast<const uint4 *>(act + tc_off(tid, c0 + 8 * q, 128));
                const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    if (!(__uint_as_float(w[e] << 16) > 0.f)) v[8 * q + 2 * e] = 0.f;
                    if (!(__uint_as_float(w[e] & 0xFFFF0000u) > 0.f)) v[8 * q + 2 * e + 1] = 0.f;
                }
                tc_st8(S.g + tc_off(tid, c0 + 8 * q, 128), v + 8 * q);
            }
            tt_colsum32(v, dbl + c0, lane, 32);
        }
    };

    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int row = tile * 128 + tid;
        const bool valid = row < n_rows;
        {
            float h[16];
            const float4 *xr = reinterpret_cast<const float4 *>(xin + (size_t)row * 16);
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float4 f = valid ? xr[c] : make_float4(0.f, 0.f, 0.f, 0.f);
                h[4 * c] = f.x;
                h[4 * c + 1] = f.y;
                h[4 * c + 2] = f.z;
                h[4 * c + 3] = f.w;
            }
            tc_st8(S.x + tc_off(tid, 0, 16), h);
            tc_st8(S.x + tc_off(tid, 8, 16), h + 8);
        }
        // ---- forward ----
        if (!step([&] { tc_mma(tmem + TT_F, tc_desc(S.x, 16), tc_desc(S.w1, 16), tc_idesc(128, 128), 0); }))
            break;
        relu_out(S.a1, S.bias);
        if (!step([&] {
                for (int kk = 0; kk < 8; kk++)
                    tc_mma(tmem + TT_F, tc_desc(S.a1 + kk * 128, 128), tc_desc(S.w2 + kk * 128, 128),
                           tc_idesc(128, 128), kk > 0);
            }))
            break;
        relu_out(S.a2, S.bias + 128);
        if (!step([&] {
                for (int kk = 0; kk < 8; kk++)
                    tc_mma(tmem + TT_F, tc_desc(S.a2 + kk * 128, 128), tc_desc(S.w3 + kk * 128, 128),
                           tc_idesc(128, 128), kk > 0);
            }))
            break;
        relu_out(S.a3, S.bias + 256);
        if (!step([&] {
                for (int kk = 0; kk < 8; kk++)
                    tc_mma(tmem + TT_F, tc_desc(S.a3 + kk * 128, 128), tc_desc(S.w4 + kk * 128, 128),
                           tc_idesc(128, 16), kk > 0);
            }))
            break;
        // ---- loss and its gradient for this thread's row ----
        {
            float z4[16], g[32];
            tc_ld16(t_row + TT_F, z4);
#pragma unroll
            for (int c = 0; c < 16; c++) z4[c] += S.bias[384 + c];
#pragma unroll
            for (int c = 0; c < 32; c++) g[c] = 0.f;
            float l = 0.f;
            if (valid) {
#pragma unroll
                for (int d = 0; d < 8; d++) {
                    if (d >= dof) break;
                    float sr = 0.f;
#pragma unroll
                    for (int c = 0; c < 16; c++) sr = c == dof + d ? z4[c] : sr;
                    const float o = z4[d];
                    const float th = tanhf(0.25f * sr);
                    const float s = 4.f * th;
                    const float e = expf(-s);
                    const float z = zin[(size_t)row * 8 + d];
                    const float df = z - o;
                    l += 0.5f * df * df * e + 0.5f * s;
                    g[d] = -df * e * inv_batch;
                    const float gs = (0.5f - 0.5f * df * df * e) * (1.f - th * th) * inv_batch;
#pragma unroll
                    for (int c = 0; c < 16; c++) g[c] = c == dof + d ? gs : g[c];
                }
            }
            tc_st8(S.dz4 + tc_off(tid, 0, 16), g);
            tc_st8(S.dz4 + tc_off(tid, 8, 16), g + 8);
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, off);
            if (lane == 0) atomicAdd(&S.loss, l);
            tt_colsum32(g, S.db + 384, lane, 16);
        }
        // ---- backward ----
        const uint32_t acc0 = first ? 0u : 1u;
        if (!step([&] {
                for (int kk = 0; kk < 8; kk++)  // dW4^T += A3^T dZ4 (M = inputs, N = outputs)
                    tc_mma(tmem + TT_DW4, tc_desc_mn(S.a3 + kk * 2048, 128), tc_desc_mn(S.dz4 + kk * 256, 16),
                           tc_idesc(128, 16, true, true), acc0 | (kk > 0));
                // dA3 = dZ4 W4
                tc_mma(tmem + TT_F, tc_desc(S.dz4, 16), tc_desc_mn(S.w4, 128), tc_idesc(128, 128, false, true), 0);
            }))
            break;
        grad_out(S.a3, S.db + 256);
        if (!step([&] {
                for (int kk = 0; kk < 8; kk++)  // dW3 += dZ3^T A2
                    tc_mma(tmem + TT_DW3, tc_desc_mn(S.g + kk * 2048, 128), tc_desc_mn(S.a2 + kk * 2048, 128),
                           tc_idesc(128, 128, true, true), acc0 | (kk > 0));
                for (int kk = 0; kk < 8; kk++)  // dA2 = dZ3 W3
                    tc_mma(tmem + TT_F, tc_desc(S.g + kk * 128, 128), tc_desc_mn(S.w3 + kk * 2048, 128),
                           tc_idesc(128, 128, false, true), kk > 0);
            }))
            break;
        grad_out(S.a2, S.db + 128);
        if (!step([&] {
                for (int kk = 0; kk < 8; kk++)  // dW2 += dZ2^T A1
                    tc_mma(tmem + TT_DW2, tc_desc_mn(S.g + kk * 2048, 128), tc_desc_mn(S.a1 + kk * 2048, 128),
                           tc_idesc(128, 128, true, true), acc0 | (kk > 0));
                for (int kk = 0; kk < 8; kk++)  // dA1 = dZ2 W2
                    tc_mma(tmem + TT_F, tc_desc(S.g + kk * 128, 128), tc_desc_mn(S.w2 + kk * 2048, 128),
                           tc_idesc(128, 128, false, true), kk > 0);
            }))
            break;
        grad_out(S.a1, S.db);
        if (!step([&] {
                for (int kk = 0; kk < 8; kk++)  // dW1 += dZ1^T X
                    tc_mma(tmem + TT_DW1, tc_desc_mn(S.g + kk * 2048, 128), tc_desc_mn(S.x + kk * 256, 16),
                           tc_idesc(128, 16, true, true), acc0 | (kk > 0));
            }))
            break;
        first = false;
    }
    if (ok && !first) {
        // the CTA's weight gradients out of tensor memory: thread t = lane t is output row t
        // of dW1..dW3 and input column t of dW4
        // (16-byte vector atomics: the parameter offsets of W1..W3 are multiples of 4 floats)
        auto add4 = [](float *dst, const float *v) {
            atomicAdd(reinterpret_cast<float4 *>(dst), make_float4(v[0], v[1], v[2], v[3]));
        };
#pragma unroll 1
        for (int c0 = 0; c0 < 128; c0 += 16) {
            float v[16];
            tc_ld16(t_row + TT_DW2 + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; i += 4) add4(grad + P_W2 + tid * 128 + c0 + i, v + i);
            tc_ld16(t_row + TT_DW3 + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; i += 4) add4(grad + P_W3 + tid * 128 + c0 + i, v + i);
        }
        {
            float v[16];
            tc_ld16(t_row + TT_DW1, v);
#pragma unroll
            for (int i = 0; i < 16; i += 4) add4(grad + P_W1 + tid * 16 + i, v + i);
            tc_ld16(t_row + TT_DW4, v);
#pragma unroll
            for (int o = 0; o < 16; o++) atomicAdd(grad + P_W4 + o * 128 + tid, v[o]);
        }
        for (int i = tid; i < 128; i += TT_THREADS) {
            atomicAdd(grad + P_B1 + i, S.db[i]);
            atomicAdd(grad + P_B2 + i, S.db[128 + i]);
            atomicAdd(grad + P_B3 + i, S.db[256 + i]);
        }
        if (tid < 16) atomicAdd(grad + P_B4 + tid, S.db[384 + tid]);
        if (tid == 0 && loss_out) atomicAdd(loss_out, S.loss);
    }
    if (!ok && tid == 0 && loss_out) atomicAdd(loss_out, __int_as_float(0x7FC00000));  // gave up: NaN loss
    // release the tensor memory once no MMA is in flight: after a give-up, wait (bounded)
    // for the last commit's phase before freeing the columns
    if (!ok) tc_wait(mbar, phase ^ 1u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TT_TMEM_COLS)
                     : "memory");
}

// Adam step on the FP32 master weights; writes the BF16 training copy and clears the
// gradient.
__global__ void fs_mlp_adam_kernel(float *params, float *m, float *v, float *grad, fs_bf16 *wq, float lr,
                                   float b1c, float b2c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= FS_MLP_NPARAM) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float w = params[i] - lr * (mi / b1c) / (sqrtf(vi / b2c) + eps);
    params[i] = w;
    grad[i] = 0.f;
    int q = -1;
    if (i < P_B1) q = Q_W1 + (i - P_W1);
    else if (i >= P_W2 && i < P_B2) q = Q_W2 + (i - P_W2);
    else if (i >= P_W3 && i < P_B3) q = Q_W3 + (i - P_W3);
    else if (i >= P_W4 && i < P_B4) q = Q_W4 + (i - P_W4);
    if (q >= 0) wq[q] = f2bf(w);
}

// FP32 master weights -> BF16 training copy + inference fragments + biases
__global__ void fs_mlp_pack_kernel(const float *params, fs_bf16 *wq, uint2 *frag, float *bias)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Q_N) {
        int p;
        if (i < Q_W2) p = P_W1 + i;
        else if (i < Q_W3) p = P_W2 + (i - Q_W2);
        else if (i < Q_W4) p = P_W3 + (i - Q_W3);
        else p = P_W4 + (i - Q_W4);
        wq[i] = f2bf(params[p]);
    }
    if (i < FS_MLP_FRAG_U2) {
        // which layer / tile / lane this fragment entry belongs to
        int off, K, N, pw;
        if (i < FS_MLP_OFF_W2) { off = FS_MLP_OFF_W1; K = 16; N = 128; pw = P_W1; }
        else if (i < FS_MLP_OFF_W3) { off = FS_MLP_OFF_W2; K = 128; N = 128; pw = P_W2; }
        else if (i < FS_MLP_OFF_W4) { off = FS_MLP_OFF_W3; K = 128; N = 128; pw = P_W3; }
        else { off = FS_MLP_OFF_W4; K = 128; N = 16; pw = P_W4; }
        const int e = i - off, lane = e & 31, t = e >> 5, NT = N / 8;
        const int kt = t / NT, nt = t % NT;
        const int n = nt * 8 + (lane >> 2), k = kt * 16 + (lane & 3) * 2;
        const float *W = params + pw;  // W[n][k], row stride K
        uint2 u;
        u.x = fs_pack_bf16(W[n * K + k], W[n * K + k + 1]);
        u.y = fs_pack_bf16(W[n * K + k + 8], W[n * K + k + 9]);
        frag[i] = u;
    }
    if (i < FS_MLP_NBIAS) {
        int p;
        if (i < FS_MLP_OFF_B2) p = P_B1 + i;
        else if (i < FS_MLP_OFF_B3) p = P_B2 + (i - FS_MLP_OFF_B2);
        else if (i < FS_MLP_OFF_B4) p = P_B3 + (i - FS_MLP_OFF_B3);
        else p = P_B4 + (i - FS_MLP_OFF_B4);
        bias[i] = params[p];
    }
}

// ------------------------------------------------------------------ C ABI
static int launch_check(const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fsi_thread_error(FS_ERR_LAUNCH, cudaGetErrorString(e));
    (void)what;
    return FS_OK;
}

extern "C" int fs_mlp_sizes(int64_t *n_param, int64_t *n_bf16, int64_t *n_frag_u2, int64_t *n_bias)
{
    if (n_param) *n_param = FS_MLP_NPARAM;
    if (n_bf16) *n_bf16 = Q_N;
    if (n_frag_u2) *n_frag_u2 = FS_MLP_FRAG_U2;
    if (n_bias) *n_bias = FS_MLP_NBIAS;
    return FS_OK;
}

extern "C" int fs_mlp_train_step(const float *params, const uint16_t *wq, float *grad, const float *x,
                                 const float *z, int32_t n_rows, int32_t dof, float inv_batch, float *loss,
                                 void *stream)
{
    if (dof < 1 || dof > 8 || n_rows < 1)
        return fsi_thread_error(FS_ERR_CONFIG, "fs_mlp_train_step: need 1 <= dof <= 8 and n_rows >= 1");
    if (((uintptr_t)wq | (uintptr_t)x | (uintptr_t)grad) & 15u)
        return fsi_thread_error(FS_ERR_CONFIG, "fs_mlp_train_step: wq, x and grad must be 16-byte aligned");
    // per call: the attribute belongs to the current device (a process may use several)
    cudaError_t e = cudaFuncSetAttribute(fs_mlp_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)TT_SMEM_BYTES);
    if (e != cudaSuccess) return fsi_thread_error(FS_ERR_CUDA, cudaGetErrorString(e));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
    const int n_tiles = (n_rows + 127) / 128;
    fs_mlp_train_tc_kernel<<<n_tiles < sms ? n_tiles : sms, TT_THREADS, TT_SMEM_BYTES, (cudaStream_t)stream>>>(
        params, (const fs_bf16 *)wq, grad, x, z, n_rows, dof, inv_batch, loss);
    return launch_check("fs_mlp_train_tc_kernel");
}

extern "C" int fs_mlp_adam(float *params, float *m, float *v, float *grad, uint16_t *wq, int32_t step, float lr,
                           void *stream)
{
    if (step < 1) return fsi_thread_error(FS_ERR_CONFIG, "fs_mlp_adam: step counts from 1");
    const float b1c = 1.f - powf(0.9f, (float)step), b2c = 1.f - powf(0.999f, (float)step);
    fs_mlp_adam_kernel<<<(FS_MLP_NPARAM + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        params, m, v, grad, (fs_bf16 *)wq, lr, b1c, b2c);
    return launch_check("fs_mlp_adam_kernel");
}

extern "C" int fs_mlp_pack(const float *params, uint16_t *wq, void *frag, float *bias, void *stream)
{
    int n = FS_MLP_FRAG_U2 > Q_N ? FS_MLP_FRAG_U2 : Q_N;
    fs_mlp_pack_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, (fs_bf16 *)wq, (uint2 *)frag,
                                                                           bias);
    return launch_check("fs_mlp_pack_kernel");
}

// batched inference on the tcgen05 tensor cores (fs_mlp_tc.cu)
extern int fsi_mlp_infer_tc(const void *frag, const float *bias, const float *x, float *y, int n_rows,
                            cudaStream_t s);

extern "C" int fs_mlp_infer(const void *frag, const float *bias, const float *x, float *y, int32_t n_rows,
                            void *stream)
{
    if (n_rows < 1) return FS_OK;
    return fsi_mlp_infer_tc(frag, bias, x, y, n_rows, (cudaStream_t)stream);
}
