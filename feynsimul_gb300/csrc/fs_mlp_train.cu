// fs_mlp_train.cu -- training and inference kernels of the learned bisection proposal
// (BF16 tensor-core mma.sync, FP32 accumulation).  No counterpart in the reference.
//
// Parameters (FP32 master copy, one flat array, FS_MLP_NPARAM floats):
//   W1[128][16] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] W4[16][128] b4[16]
// Training tile: 64 rows per CTA, 8 warps.  Forward keeps the BF16 activations in shared
// memory; the loss gradient is formed per row; backward runs dW = dZ^T A and dA = dZ W with
// transposed ldmatrix loads and adds the CTA's weight / bias gradients to an FP32 gradient
// array with atomics (the Adam kernel divides nothing: the loss is already a batch mean).
//
// Loss (per row, D degrees of freedom, z the midpoint's displacement from the endpoints'
// mean in units of sigma_1): sum_d 0.5 (z_d - o_d)^2 exp(-s_d) + 0.5 s_d with
// s_d = 4 tanh(o_{D+d} / 4): the Gaussian negative log-likelihood of z under N(o, exp(s)).
#include <cuda_runtime.h>

#include "../../include/feynsimul.h"
#include "fs_mlp.cuh"

#define FS_MLP_NPARAM (128 * 16 + 128 + 128 * 128 + 128 + 128 * 128 + 128 + 16 * 128 + 16)
#define P_W1 0
#define P_B1 (P_W1 + 128 * 16)
#define P_W2 (P_B1 + 128)
#define P_B2 (P_W2 + 128 * 128)
#define P_W3 (P_B2 + 128)
#define P_B3 (P_W3 + 128 * 128)
#define P_W4 (P_B3 + 128)
#define P_B4 (P_W4 + 16 * 128)

// BF16 weight copy used by training (row-major, same order as the FP32 weights, no biases)
#define Q_W1 0
#define Q_W2 (Q_W1 + 128 * 16)
#define Q_W3 (Q_W2 + 128 * 128)
#define Q_W4 (Q_W3 + 128 * 128)
#define Q_N (Q_W4 + 16 * 128)

typedef unsigned short fs_bf16;  // raw BF16 bits

#define ROWS 64
#define LDH 136  // padded row stride (elements) of 128-wide tiles
#define LDS 24   // padded row stride of 16-wide tiles

extern int fsi_thread_error(int code, const char *msg);

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const fs_bf16 *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}

__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], const fs_bf16 *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}

__device__ __forceinline__ fs_bf16 f2bf(float x)
{
    unsigned r = fs_pack_bf16(x, 0.f);
    return (fs_bf16)(r & 0xFFFFu);
}

__device__ __forceinline__ float bf2f(fs_bf16 x) { return __uint_as_float(((unsigned)x) << 16); }

// acc[MT][NT] += A * B over K for one warp.
//   TA = false: A stored A[m][k] (k contiguous);  TA = true: stored At[k][m].
//   TB = false: B stored Bt[n][k] (k contiguous); TB = true: stored B[k][n].
// NT must be even (two n-tiles per ldmatrix.x4).
template <int MT, int NT, bool TA, bool TB>
__device__ __forceinline__ void warp_gemm(float (&acc)[MT][NT][4], const fs_bf16 *A, int lda, int m0,
                                          const fs_bf16 *B, int ldb, int n0, int K, int lane)
{
    const int j = lane >> 3, r8 = lane & 7;
    for (int k0 = 0; k0 < K; k0 += 16) {
        unsigned a[MT][4];
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
            if (!TA)
                ldsm_x4(a[mt], A + (m0 + mt * 16 + r8 + (j & 1) * 8) * lda + k0 + (j >> 1) * 8);
            else
                ldsm_x4_t(a[mt], A + (k0 + (j >> 1) * 8 + r8) * lda + m0 + mt * 16 + (j & 1) * 8);
        }
#pragma unroll
        for (int nt = 0; nt < NT; nt += 2) {
            unsigned b[4];
            if (!TB)
                ldsm_x4(b, B + (n0 + nt * 8 + (j >> 1) * 8 + r8) * ldb + k0 + (j & 1) * 8);
            else
                ldsm_x4_t(b, B + (k0 + (j & 1) * 8 + r8) * ldb + n0 + nt * 8 + (j >> 1) * 8);
#pragma unroll
            for (int mt = 0; mt < MT; mt++) {
                fs_mma_bf16(acc[mt][nt], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b[0], b[1]);
                fs_mma_bf16(acc[mt][nt + 1], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b[2], b[3]);
            }
        }
    }
}

template <int MT, int NT>
__device__ __forceinline__ void zero_acc(float (&acc)[MT][NT][4])
{
#pragma unroll
    for (int i = 0; i < MT; i++)
#pragma unroll
        for (int j = 0; j < NT; j++) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
}

// forward epilogue: out = relu(acc + bias) as BF16 into a [ROWS][LDH] tile
template <int NT>
__device__ __forceinline__ void store_relu(const float (&acc)[1][NT][4], const float *bias, fs_bf16 *out, int m0,
                                           int n0, int lane)
{
    const int r = m0 + (lane >> 2), c = (lane & 3) * 2;
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        const int col = n0 + nt * 8 + c;
        const float b0 = bias[col], b1 = bias[col + 1];
        out[r * LDH + col] = f2bf(fmaxf(acc[0][nt][0] + b0, 0.f));
        out[r * LDH + col + 1] = f2bf(fmaxf(acc[0][nt][1] + b1, 0.f));
        out[(r + 8) * LDH + col] = f2bf(fmaxf(acc[0][nt][2] + b0, 0.f));
        out[(r + 8) * LDH + col + 1] = f2bf(fmaxf(acc[0][nt][3] + b1, 0.f));
    }
}

// backward epilogue: dZ = acc * (A > 0) as BF16, column sums of dZ into the bias gradient
template <int NT>
__device__ __forceinline__ void store_dz(const float (&acc)[1][NT][4], const fs_bf16 *act, fs_bf16 *out,
                                         float *s_db, int m0, int n0, int lane)
{
    const int r = m0 + (lane >> 2), c = (lane & 3) * 2;
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        const int col = n0 + nt * 8 + c;
        float v[4];
        v[0] = bf2f(act[r * LDH + col]) > 0.f ? acc[0][nt][0] : 0.f;
        v[1] = bf2f(act[r * LDH + col + 1]) > 0.f ? acc[0][nt][1] : 0.f;
        v[2] = bf2f(act[(r + 8) * LDH + col]) > 0.f ? acc[0][nt][2] : 0.f;
        v[3] = bf2f(act[(r + 8) * LDH + col + 1]) > 0.f ? acc[0][nt][3] : 0.f;
        out[r * LDH + col] = f2bf(v[0]);
        out[r * LDH + col + 1] = f2bf(v[1]);
        out[(r + 8) * LDH + col] = f2bf(v[2]);
        out[(r + 8) * LDH + col + 1] = f2bf(v[3]);
        // sum the 16 rows of this fragment column: lanes with equal (lane & 3)
        float s0 = v[0] + v[2], s1 = v[1] + v[3];
#pragma unroll
        for (int off = 4; off < 32; off <<= 1) {
            s0 += __shfl_xor_sync(0xFFFFFFFFu, s0, off);
            s1 += __shfl_xor_sync(0xFFFFFFFFu, s1, off);
        }
        if (lane < 4) {
            atomicAdd(s_db + col, s0);
            atomicAdd(s_db + col + 1, s1);
        }
    }
}

// weight-gradient epilogue: atomically add a warp tile of dW[o][i] (row stride ld)
template <int MT, int NT>
__device__ __forceinline__ void add_dw(const float (&acc)[MT][NT][4], float *g, int ld, int m0, int n0, int lane)
{
    const int r = lane >> 2, c = (lane & 3) * 2;
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
            const int row = m0 + mt * 16 + r, col = n0 + nt * 8 + c;
            atomicAdd(g + row * ld + col, acc[mt][nt][0]);
            atomicAdd(g + row * ld + col + 1, acc[mt][nt][1]);
            atomicAdd(g + (row + 8) * ld + col, acc[mt][nt][2]);
            atomicAdd(g + (row + 8) * ld + col + 1, acc[mt][nt][3]);
        }
}

struct __align__(16) MlpSmem {
    fs_bf16 w1[128 * LDS];
    fs_bf16 w2[128 * LDH];
    fs_bf16 w3[128 * LDH];
    fs_bf16 w4[16 * LDH];
    fs_bf16 x[ROWS * LDS];
    fs_bf16 a1[ROWS * LDH];
    fs_bf16 a2[ROWS * LDH];
    fs_bf16 a3[ROWS * LDH];
    fs_bf16 g1[ROWS * LDH];
    fs_bf16 g2[ROWS * LDH];
    fs_bf16 dz4[ROWS * LDS];
    float z4[ROWS * 16];
    float db[128 * 3 + 16];
    float loss;
};

__global__ void __launch_bounds__(256) fs_mlp_train_kernel(const float *__restrict__ params,
                                                           const fs_bf16 *__restrict__ wq, float *__restrict__ grad,
                                                           const float *__restrict__ xin, const float *__restrict__ zin,
                                                           int n_rows, int dof, float inv_batch, float *loss_out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    MlpSmem &S = *reinterpret_cast<MlpSmem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.x * ROWS;

    // ---- stage weights (BF16) and the input tile ----
    for (int i = tid; i < 128 * 16; i += 256) S.w1[(i / 16) * LDS + i % 16] = wq[Q_W1 + i];
    for (int i = tid; i < 128 * 128; i += 256) {
        S.w2[(i / 128) * LDH + i % 128] = wq[Q_W2 + i];
        S.w3[(i / 128) * LDH + i % 128] = wq[Q_W3 + i];
    }
    for (int i = tid; i < 16 * 128; i += 256) S.w4[(i / 128) * LDH + i % 128] = wq[Q_W4 + i];
    for (int i = tid; i < ROWS * 16; i += 256) {
        const int r = i / 16, c = i % 16;
        const float v = (row0 + r < n_rows) ? xin[(size_t)(row0 + r) * 16 + c] : 0.f;
        S.x[r * LDS + c] = f2bf(v);
    }
    for (int i = tid; i < 128 * 3 + 16; i += 256) S.db[i] = 0.f;
    if (tid == 0) S.loss = 0.f;
    __syncthreads();

    const int wm = warp & 3, wn = warp >> 2;  // 4 row tiles x 2 column halves
    // ---- forward ----
    {
        float acc[1][8][4];
        zero_acc(acc);
        warp_gemm<1, 8, false, false>(acc, S.x, LDS, wm * 16, S.w1, LDS, wn * 64, 16, lane);
        store_relu<8>(acc, params + P_B1, S.a1, wm * 16, wn * 64, lane);
    }
    __syncthreads();
    {
        float acc[1][8][4];
        zero_acc(acc);
        warp_gemm<1, 8, false, false>(acc, S.a1, LDH, wm * 16, S.w2, LDH, wn * 64, 128, lane);
        store_relu<8>(acc, params + P_B2, S.a2, wm * 16, wn * 64, lane);
    }
    __syncthreads();
    {
        float acc[1][8][4];
        zero_acc(acc);
        warp_gemm<1, 8, false, false>(acc, S.a2, LDH, wm * 16, S.w3, LDH, wn * 64, 128, lane);
        store_relu<8>(acc, params + P_B3, S.a3, wm * 16, wn * 64, lane);
    }
    __syncthreads();
    if (warp < 4) {
        float acc[1][2][4];
        zero_acc(acc);
        warp_gemm<1, 2, false, false>(acc, S.a3, LDH, warp * 16, S.w4, LDH, 0, 128, lane);
        const int r = warp * 16 + (lane >> 2), c = (lane & 3) * 2;
#pragma unroll
        for (int nt = 0; nt < 2; nt++) {
            const int col = nt * 8 + c;
            S.z4[r * 16 + col] = acc[0][nt][0] + params[P_B4 + col];
            S.z4[r * 16 + col + 1] = acc[0][nt][1] + params[P_B4 + col + 1];
            S.z4[(r + 8) * 16 + col] = acc[0][nt][2] + params[P_B4 + col];
            S.z4[(r + 8) * 16 + col + 1] = acc[0][nt][3] + params[P_B4 + col + 1];
        }
    }
    __syncthreads();
    // ---- loss and its gradient per row ----
    if (tid < ROWS) {
        const int r = tid;
        const bool valid = row0 + r < n_rows;
        float l = 0.f;
        float g[16];
#pragma unroll
        for (int c = 0; c < 16; c++) g[c] = 0.f;
        if (valid) {
            for (int d = 0; d < dof; d++) {
                const float o = S.z4[r * 16 + d], sr = S.z4[r * 16 + dof + d];
                const float th = tanhf(0.25f * sr);
                const float s = 4.f * th;
                const float e = expf(-s);
                const float z = zin[(size_t)(row0 + r) * 8 + d];
                const float df = z - o;
                l += 0.5f * df * df * e + 0.5f * s;
                g[d] = -df * e * inv_batch;
                g[dof + d] = (0.5f - 0.5f * df * df * e) * (1.f - th * th) * inv_batch;
            }
        }
#pragma unroll
        for (int c = 0; c < 16; c++) {
            S.dz4[r * LDS + c] = f2bf(g[c]);
            atomicAdd(&S.db[384 + c], g[c]);
        }
        atomicAdd(&S.loss, l);
    }
    __syncthreads();
    // ---- backward ----
    {   // dW4 += dZ4^T A3: [16 x 128]
        float acc[1][2][4];
        zero_acc(acc);
        warp_gemm<1, 2, true, true>(acc, S.dz4, LDS, 0, S.a3, LDH, warp * 16, ROWS, lane);
        add_dw<1, 2>(acc, grad + P_W4, 128, 0, warp * 16, lane);
    }
    {   // dA3 = dZ4 W4 -> dZ3 (g1)
        float acc[1][8][4];
        zero_acc(acc);
        warp_gemm<1, 8, false, true>(acc, S.dz4, LDS, wm * 16, S.w4, LDH, wn * 64, 16, lane);
        store_dz<8>(acc, S.a3, S.g1, S.db + 256, wm * 16, wn * 64, lane);
    }
    __syncthreads();
    {   // dW3 += dZ3^T A2
        float acc[2][8][4];
        zero_acc(acc);
        warp_gemm<2, 8, true, true>(acc, S.g1, LDH, wm * 32, S.a2, LDH, wn * 64, ROWS, lane);
        add_dw<2, 8>(acc, grad + P_W3, 128, wm * 32, wn * 64, lane);
    }
    {   // dA2 = dZ3 W3 -> dZ2 (g2)
        float acc[1][8][4];
        zero_acc(acc);
        warp_gemm<1, 8, false, true>(acc, S.g1, LDH, wm * 16, S.w3, LDH, wn * 64, 128, lane);
        store_dz<8>(acc, S.a2, S.g2, S.db + 128, wm * 16, wn * 64, lane);
    }
    __syncthreads();
    {   // dW2 += dZ2^T A1
        float acc[2][8][4];
        zero_acc(acc);
        warp_gemm<2, 8, true, true>(acc, S.g2, LDH, wm * 32, S.a1, LDH, wn * 64, ROWS, lane);
        add_dw<2, 8>(acc, grad + P_W2, 128, wm * 32, wn * 64, lane);
    }
    __syncthreads();  // g1 is rewritten next
    {   // dA1 = dZ2 W2 -> dZ1 (g1)
        float acc[1][8][4];
        zero_acc(acc);
        warp_gemm<1, 8, false, true>(acc, S.g2, LDH, wm * 16, S.w2, LDH, wn * 64, 128, lane);
        store_dz<8>(acc, S.a1, S.g1, S.db, wm * 16, wn * 64, lane);
    }
    __syncthreads();
    {   // dW1 += dZ1^T X: [128 x 16]
        float acc[1][2][4];
        zero_acc(acc);
        warp_gemm<1, 2, true, true>(acc, S.g1, LDH, warp * 16, S.x, LDS, 0, ROWS, lane);
        add_dw<1, 2>(acc, grad + P_W1, 16, warp * 16, 0, lane);
    }
    __syncthreads();
    for (int i = tid; i < 128; i += 256) {
        atomicAdd(grad + P_B1 + i, S.db[i]);
        atomicAdd(grad + P_B2 + i, S.db[128 + i]);
        atomicAdd(grad + P_B3 + i, S.db[256 + i]);
    }
    if (tid < 16) atomicAdd(grad + P_B4 + tid, S.db[384 + tid]);
    if (tid == 0 && loss_out) atomicAdd(loss_out, S.loss);
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
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(fs_mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(MlpSmem));
        if (e != cudaSuccess) return fsi_thread_error(FS_ERR_CUDA, cudaGetErrorString(e));
        attr_done = true;
    }
    fs_mlp_train_kernel<<<(n_rows + ROWS - 1) / ROWS, 256, sizeof(MlpSmem), (cudaStream_t)stream>>>(
        params, (const fs_bf16 *)wq, grad, x, z, n_rows, dof, inv_batch, loss);
    return launch_check("fs_mlp_train_kernel");
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
