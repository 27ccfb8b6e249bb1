// fs_mlp.cuh -- the learned bisection proposal's network evaluated per warp on the tensor
// cores (BF16 inputs, FP32 accumulation, mma.sync.m16n8k16) inside the sweep, pasted into
// the NVRTC module when the learned proposal is on; its sizes and BF16 packing are shared
// with the tcgen05 training and batched-inference kernels (fs_mlp_train.cu, fs_mlp_tc.cu).
// No counterpart in the reference.
//
// Network: 4 linear layers 16 -> 128 -> 128 -> 128 -> 16 with ReLU between them.
//   input  (16): the segment's endpoint midpoint and half-difference per degree of freedom,
//                divided by a length scale, zero padded;
//   output (16): o[0..D) the mean shift and o[D..2D) the log-variance change of the
//                level-1 bisection midpoint, in units of the free-particle width sigma_1.
//
// Inference weight layout ("fragment order"): for a layer with W[out][in] (B operand
// B[k=in][n=out]) the BF16 pairs each lane needs for mma.sync's B fragment of k-tile kt
// and n-tile nt are stored as uint2 at frag[(kt * NT + nt) * 32 + lane], so a warp reads
// 256 contiguous bytes per fragment.  Layers are stored one after another (FS_MLP_OFF_*).
#pragma once

#define FS_MLP_IN 16
#define FS_MLP_H 128
#define FS_MLP_OUT 16
// uint2 offsets of the layers in the fragment-ordered weight blob
#define FS_MLP_OFF_W1 0
#define FS_MLP_OFF_W2 (FS_MLP_OFF_W1 + (FS_MLP_IN / 16) * (FS_MLP_H / 8) * 32)
#define FS_MLP_OFF_W3 (FS_MLP_OFF_W2 + (FS_MLP_H / 16) * (FS_MLP_H / 8) * 32)
#define FS_MLP_OFF_W4 (FS_MLP_OFF_W3 + (FS_MLP_H / 16) * (FS_MLP_H / 8) * 32)
#define FS_MLP_FRAG_U2 (FS_MLP_OFF_W4 + (FS_MLP_H / 16) * (FS_MLP_OUT / 8) * 32)
// float offsets of the biases (after the fragments, in a separate float array)
#define FS_MLP_OFF_B1 0
#define FS_MLP_OFF_B2 (FS_MLP_OFF_B1 + FS_MLP_H)
#define FS_MLP_OFF_B3 (FS_MLP_OFF_B2 + FS_MLP_H)
#define FS_MLP_OFF_B4 (FS_MLP_OFF_B3 + FS_MLP_H)
#define FS_MLP_NBIAS (FS_MLP_OFF_B4 + FS_MLP_OUT)

__device__ __forceinline__ unsigned fs_pack_bf16(float lo, float hi)
{
    unsigned r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ void fs_mma_bf16(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                            unsigned b0, unsigned b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// One hidden layer for a 16-row tile: out = relu(in * W^T + b) with in / out as A
// fragments (8 k-tiles of 16 columns, 4 registers each).  The C fragment of two adjacent
// n-tiles is exactly the A fragment of the next layer's k-tile, so layers chain in
// registers.
__device__ __forceinline__ void fs_mlp_hidden(const uint2 *__restrict__ frag, const float *__restrict__ bias,
                                              const unsigned (&in)[FS_MLP_H / 16][4],
                                              unsigned (&out)[FS_MLP_H / 16][4], int lane)
{
#pragma unroll
    for (int j = 0; j < FS_MLP_H / 16; j++) {  // output k-tile j = n-tiles 2j, 2j+1
        float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < FS_MLP_H / 16; kt++) {
            const uint2 b0 = frag[(kt * (FS_MLP_H / 8) + 2 * j) * 32 + lane];
            const uint2 b1 = frag[(kt * (FS_MLP_H / 8) + 2 * j + 1) * 32 + lane];
            fs_mma_bf16(c0, in[kt][0], in[kt][1], in[kt][2], in[kt][3], b0.x, b0.y);
            fs_mma_bf16(c1, in[kt][0], in[kt][1], in[kt][2], in[kt][3], b1.x, b1.y);
        }
        const int col = (lane & 3) * 2;
        const float2 bb0 = *(const float2 *)(bias + 16 * j + col);
        const float2 bb1 = *(const float2 *)(bias + 16 * j + 8 + col);
        out[j][0] = fs_pack_bf16(fmaxf(c0[0] + bb0.x, 0.f), fmaxf(c0[1] + bb0.y, 0.f));
        out[j][1] = fs_pack_bf16(fmaxf(c0[2] + bb0.x, 0.f), fmaxf(c0[3] + bb0.y, 0.f));
        out[j][2] = fs_pack_bf16(fmaxf(c1[0] + bb1.x, 0.f), fmaxf(c1[1] + bb1.y, 0.f));
        out[j][3] = fs_pack_bf16(fmaxf(c1[2] + bb1.x, 0.f), fmaxf(c1[3] + bb1.y, 0.f));
    }
}

// Warp-collective inference: every lane passes its 16 input features and receives its 16
// outputs.  All 32 lanes must call (rows 0-15 and 16-31 form two 16-row tiles).
__device__ __forceinline__ void fs_mlp_eval_warp(const uint2 *__restrict__ frag, const float *__restrict__ bias,
                                                 const float (&x)[FS_MLP_IN], float (&y)[FS_MLP_OUT])
{
    const int lane = threadIdx.x & 31;
    unsigned f[8];
#pragma unroll
    for (int j = 0; j < 8; j++) f[j] = fs_pack_bf16(x[2 * j], x[2 * j + 1]);
#pragma unroll
    for (int j = 0; j < FS_MLP_OUT; j++) y[j] = 0.f;
#pragma unroll 1
    for (int q = 0; q < 2; q++) {
        // input A fragment: rows lane/4 and lane/4+8 of tile q, columns (lane%4)*2 (+8)
        const int src0 = q * 16 + (lane >> 2), src1 = src0 + 8, c = lane & 3;
        unsigned a[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int cc = 0; cc < 4; cc++) {
            const unsigned v0 = __shfl_sync(0xFFFFFFFFu, f[cc], src0);
            const unsigned v1 = __shfl_sync(0xFFFFFFFFu, f[cc], src1);
            const unsigned v2 = __shfl_sync(0xFFFFFFFFu, f[4 + cc], src0);
            const unsigned v3 = __shfl_sync(0xFFFFFFFFu, f[4 + cc], src1);
            if (c == cc) {
                a[0] = v0;
                a[1] = v1;
                a[2] = v2;
                a[3] = v3;
            }
        }
        // layer 1 (K = 16): straight into the A fragments of layer 2
        unsigned h1[FS_MLP_H / 16][4], h2[FS_MLP_H / 16][4];
#pragma unroll
        for (int j = 0; j < FS_MLP_H / 16; j++) {
            float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
            const uint2 b0 = frag[FS_MLP_OFF_W1 + (2 * j) * 32 + lane];
            const uint2 b1 = frag[FS_MLP_OFF_W1 + (2 * j + 1) * 32 + lane];
            fs_mma_bf16(c0, a[0], a[1], a[2], a[3], b0.x, b0.y);
            fs_mma_bf16(c1, a[0], a[1], a[2], a[3], b1.x, b1.y);
            const int col = (lane & 3) * 2;
            const float2 bb0 = *(const float2 *)(bias + FS_MLP_OFF_B1 + 16 * j + col);
            const float2 bb1 = *(const float2 *)(bias + FS_MLP_OFF_B1 + 16 * j + 8 + col);
            h1[j][0] = fs_pack_bf16(fmaxf(c0[0] + bb0.x, 0.f), fmaxf(c0[1] + bb0.y, 0.f));
            h1[j][1] = fs_pack_bf16(fmaxf(c0[2] + bb0.x, 0.f), fmaxf(c0[3] + bb0.y, 0.f));
            h1[j][2] = fs_pack_bf16(fmaxf(c1[0] + bb1.x, 0.f), fmaxf(c1[1] + bb1.y, 0.f));
            h1[j][3] = fs_pack_bf16(fmaxf(c1[2] + bb1.x, 0.f), fmaxf(c1[3] + bb1.y, 0.f));
        }
        fs_mlp_hidden(frag + FS_MLP_OFF_W2, bias + FS_MLP_OFF_B2, h1, h2, lane);
        fs_mlp_hidden(frag + FS_MLP_OFF_W3, bias + FS_MLP_OFF_B3, h2, h1, lane);
        // layer 4 (N = 16, no activation)
        float o0[4] = {0.f, 0.f, 0.f, 0.f}, o1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < FS_MLP_H / 16; kt++) {
            const uint2 b0 = frag[FS_MLP_OFF_W4 + (kt * 2) * 32 + lane];
            const uint2 b1 = frag[FS_MLP_OFF_W4 + (kt * 2 + 1) * 32 + lane];
            fs_mma_bf16(o0, h1[kt][0], h1[kt][1], h1[kt][2], h1[kt][3], b0.x, b0.y);
            fs_mma_bf16(o1, h1[kt][0], h1[kt][1], h1[kt][2], h1[kt][3], b1.x, b1.y);
        }
        // output fragment -> rows: lane (q*16 + r) takes row r from lanes 4*(r%8)+c
        const int r = lane - q * 16;
        const bool mine = (r >= 0 && r < 16);
        const int hi = (r >> 3) & 1;
#pragma unroll
        for (int cc = 0; cc < 4; cc++) {
            const int src = 4 * (r & 7) + cc;
            const float v00 = __shfl_sync(0xFFFFFFFFu, o0[0], src), v01 = __shfl_sync(0xFFFFFFFFu, o0[1], src);
            const float v02 = __shfl_sync(0xFFFFFFFFu, o0[2], src), v03 = __shfl_sync(0xFFFFFFFFu, o0[3], src);
            const float v10 = __shfl_sync(0xFFFFFFFFu, o1[0], src), v11 = __shfl_sync(0xFFFFFFFFu, o1[1], src);
            const float v12 = __shfl_sync(0xFFFFFFFFu, o1[2], src), v13 = __shfl_sync(0xFFFFFFFFu, o1[3], src);
            if (mine) {
                y[2 * cc] = (hi ? v02 : v00) + bias[FS_MLP_OFF_B4 + 2 * cc];
                y[2 * cc + 1] = (hi ? v03 : v01) + bias[FS_MLP_OFF_B4 + 2 * cc + 1];
                y[8 + 2 * cc] = (hi ? v12 : v10) + bias[FS_MLP_OFF_B4 + 8 + 2 * cc];
                y[8 + 2 * cc + 1] = (hi ? v13 : v11) + bias[FS_MLP_OFF_B4 + 8 + 2 * cc + 1];
            }
        }
    }
}
