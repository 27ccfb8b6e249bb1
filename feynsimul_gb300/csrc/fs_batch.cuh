// fs_batch.cuh -- many independent systems of different sizes in one persistent launch.
// No counterpart in the reference (which runs one system per OpenCL program).
//
// fs_api.cu pastes the RNG header, then for every system type k (one per distinct DOF
// value / plugin) the plugin's code inside `namespace fs_type_k` plus a functor with the
// potential and operators, then this file and a generated dispatcher kernel.
//
// A work item is a tile of walkers of one system.  CTAs pull items from a global counter
// (largest first, so the ragged tail is short) and run all the launch's sweeps on the
// tile: the same Metropolis-bisection move as fs_pimc.cuh (kernel.c:258-399, with the
// fixed-mode xorshift or RANLUX streams), but N, S, epsilon, the bisection widths and the walker
// counts are runtime values of the system, the path tile lives in shared memory while the
// saved old segments go to the CTA's slice of a global scratch buffer (a 27-DOF,
// 1024-slice walker's path alone takes 117 KB), and a walker wider than a warp
// synchronises with a named barrier of its own.
#pragma once

#define FS_BATCH_MAX_S 10
#ifndef FSB_RANLUX
#define FSB_RANLUX 0
#endif

// the batch's random streams: per segment thread (node draws, acceptance) and per walker
// (the segment offset; every thread of the walker advances its own identical copy), as the
// sweep's fixed mode: xorshift rows or RANLUX tables (luxury FS_NSKIP for the whole batch)
#if FSB_RANLUX
typedef FsRanluxStream<FS_NSKIP> FsbStream;
__device__ __forceinline__ float fsb_uniform(FsbStream &g) { return g.next(); }
__device__ __forceinline__ fs_u32 fsb_offset(FsbStream &g, fs_u32 range)
{
    return ((fs_u32)__fmul_rn(g.next(), (float)range)) & (range - 1u);  // kernel.c:715-718, fixed mode
}
#define FSB_DRAW_UNROLL _Pragma("unroll 1")  // one inlined generator per move loop
#else
typedef FsXorshift FsbStream;
__device__ __forceinline__ float fsb_uniform(FsbStream &g) { return fs_xs_float(g); }
__device__ __forceinline__ fs_u32 fsb_offset(FsbStream &g, fs_u32 range) { return fs_xs_next(g) & (range - 1u); }
#define FSB_DRAW_UNROLL _Pragma("unroll")
#endif

struct FsBatchSys {
    float *paths;            // [walkers][DOF][N]
    float *old_scratch;      // per CTA slot: saved segments [(seg-1)*DOF][tile threads], then
                             // with the potential cache their cached V [(seg-1)][tile threads]
    float *vcache;           // potential cache: V of every slice [walkers][N] (3 or more DOF)
    fs_u32 *seeds;           // [threads][4]  (thread = walker * tpw + t)
    fs_u32 *wseeds;          // [walkers][4]
    fs_u32 *rtab;            // RANLUX: [threads][28] (the reference's table layout)
    fs_u32 *gtab;            // RANLUX: [walkers][28]
    fs_u32 *accepts;         // [threads]
    double *op_sums;         // [walkers][nops], accumulated over launches
    int n_walkers, N, S, tpw, wpb, nops, type, n_tiles;
    int op_runs, msteps;
    int global;              // 1: the tile works on its walkers' rows of `paths` in place
    float eps;
    float sigma[FS_BATCH_MAX_S + 1];
};

struct FsBatchItem {
    int sys, tile;
};

__device__ __forceinline__ void fs_walker_sync(int tpw, int wl)
{
    if (tpw <= 32) {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned m = tpw == 32 ? 0xFFFFFFFFu : (((1u << tpw) - 1u) << (lane / tpw * tpw));
        __syncwarp(m);
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(1 + wl), "r"(tpw) : "memory");
    }
}

// One tile: walkers [tile*wpb, ...) of system sd.  All threads of the CTA call it.
// Systems of 3 or more DOF keep V of every slice in device memory between moves (as the
// sweep's potential cache: slice s of a walker at (s mod 2^S) * (N / 2^S) + s / 2^S, so a
// walker's segment threads touch consecutive words): the old action is a sum of cached
// values, the same products and sums as evaluating V again, and a move evaluates V only at
// its proposed nodes.  The old values are saved beside the old segment and written back if
// the move is rejected.
// GLOBAL: the walkers' paths stay in device memory (L1/L2) and are worked on in place, for
// walkers too large to put enough of them in shared memory to fill the CTA (the same
// arithmetic as the shared-memory tile, like the sweep's global-path mode).
template <int DOF, class Sys, bool GLOBAL>
__device__ __forceinline__ void fs_batch_tile(const FsBatchSys &sd, int tile, float *smem, size_t old_slot_floats)
{
    const int tid = threadIdx.x;
    const int N = sd.N, S = sd.S, seg = 1 << S, tpw = sd.tpw;
    const int dstride = N + (N >> S);
    int wstride = DOF * dstride;
    wstride = ((wstride + 15) / 16) * 16;
    if ((wstride / 16) % 2 == 0) wstride += 16;
    const int w0 = tile * sd.wpb;
    const int n_here = min(sd.wpb, sd.n_walkers - w0);
    const int wl = tid / tpw, t = tid % tpw;
    const bool active = wl < n_here;
    const int nthr = sd.wpb * tpw;
    // saved old segments: this CTA's slice of the global scratch, [(seg-1)*DOF][tile threads]
    float *s_old = sd.old_scratch + (size_t)blockIdx.x * old_slot_floats;
    double *s_op = (double *)(GLOBAL ? smem : smem + sd.wpb * wstride);  // [wpb][nops]
    constexpr bool VC = DOF >= 3;
    float *s_oldv = s_old + (size_t)(seg - 1) * DOF * nthr;  // [(seg-1)][tile threads]

#define FSB_AT(P, d, s) (GLOBAL ? (P)[(d) * N + (s)] : (P)[(d) * dstride + (s) + ((s) >> S)])
    {
        if (!GLOBAL) {
            const size_t base = (size_t)w0 * DOF * N;
            const int count = n_here * DOF * N;
            for (int i = tid; i < count; i += blockDim.x) {
                const int wi = i / (DOF * N), r = i - wi * (DOF * N);
                const int d = r / N, sl = r - d * N;
                FSB_AT(smem + wi * wstride, d, sl) = sd.paths[base + i];
            }
        }
        for (int i = tid; i < sd.wpb * sd.nops; i += blockDim.x) s_op[i] = 0.0;
    }
    __syncthreads();

    if (active) {
        const int w = w0 + wl;
        float *P = GLOBAL ? sd.paths + (size_t)w * DOF * N : smem + wl * wstride;
        const int th = w * tpw + t;
        FsbStream g, ws;
        {
#if FSB_RANLUX
            fs_rl_load(g.st, sd.rtab + (size_t)th * 28);
            g.count = 0u;
            fs_rl_load(ws.st, sd.gtab + (size_t)w * 28);
            ws.count = 0u;
#else
            const uint4 s4 = *(const uint4 *)(sd.seeds + (size_t)th * 4);
            g.x = s4.x; g.y = s4.y; g.z = s4.z; g.w = s4.w;
            const uint4 g4 = *(const uint4 *)(sd.wseeds + (size_t)w * 4);
            ws.x = g4.x; ws.y = g4.y; ws.z = g4.z; ws.w = g4.w;
#endif
        }
        float *Vc = VC ? sd.vcache + (size_t)w * N : nullptr;
#define FSB_VIDX(s) ((((s) & (seg - 1)) * tpw) + ((s) >> S))
        if (VC) {
#pragma unroll 1
            for (int s = t * seg; s < (t + 1) * seg; s++) {
                float x[DOF];
#pragma unroll
                for (int d = 0; d < DOF; d++) x[d] = FSB_AT(P, d, s);
                Vc[FSB_VIDX(s)] = Sys::pot(x);
            }
            fs_walker_sync(tpw, wl);
        }
        fs_u32 n_acc = 0u;
        double opd[Sys::NOPS > 0 ? Sys::NOPS : 1];
#pragma unroll
        for (int k = 0; k < Sys::NOPS; k++) opd[k] = 0.0;
        const float eps = sd.eps;
#pragma unroll 1
        for (int run = 0; run < sd.op_runs; run++) {
#pragma unroll 1
            for (int step = 0; step < sd.msteps; step++) {
                const fs_u32 off = fsb_offset(ws, (fs_u32)seg);
                const int start = (int)((off + (fs_u32)(seg * t)) & (fs_u32)(N - 1));
                // ---- bisection move (kernel.c:258-399) ----
                float aOld = 0.f, aNew = 0.f;
                float x[DOF];
#pragma unroll 1
                for (int i = 1; i < seg; i++) {
                    const int p = (start + i) & (N - 1);
#pragma unroll
                    for (int d = 0; d < DOF; d++) {
                        x[d] = FSB_AT(P, d, p);
                        s_old[((i - 1) * DOF + d) * nthr + tid] = x[d];
                    }
                    if (!VC) aOld = __fadd_rn(aOld, __fmul_rn(eps, Sys::pot(x)));
                }
                if (VC) {
#pragma unroll 4
                    for (int i = 1; i < seg; i++) {
                        const float v = Vc[FSB_VIDX((start + i) & (N - 1))];
                        s_oldv[(i - 1) * nthr + tid] = v;
                        aOld = __fadd_rn(aOld, __fmul_rn(eps, v));
                    }
                }
#pragma unroll 1
                for (int n = 1; n <= S; n++) {
                    const int half = 1 << (S - n);
                    const float sig = sd.sigma[n];
#pragma unroll 1
                    for (int i = 0; i < (1 << (n - 1)); i++) {
                        const int m = ((1 + 2 * i) * half + start) & (N - 1);
                        const int l = (i * 2 * half + start) & (N - 1);
                        const int r = ((i + 1) * 2 * half + start) & (N - 1);
                        FSB_DRAW_UNROLL
                        for (int d = 0; d < DOF; d++) {
                            const float u = fsb_uniform(g);
                            const float v = fsb_uniform(g);
                            // evaluated for every degree of freedom and replaced by 0 where
                            // v == 0 (kernel.c:349-353): no branch, so the compiler
                            // interleaves the degrees of freedom
                            float rz = __fmul_rn(__fmul_rn(sig, sqrtf(__fmul_rn(-2.f, __logf(v)))),
                                                 __sinf(__fmul_rn(6.28318548f, u)));
                            rz = v != 0.f ? rz : 0.f;
                            FSB_AT(P, d, m) = __fadd_rn(__fmul_rn(0.5f, __fadd_rn(FSB_AT(P, d, l), FSB_AT(P, d, r))), rz);
                        }
                    }
                }
#pragma unroll 1
                for (int i = 1; i < seg; i++) {
                    const int p = (start + i) & (N - 1);
#pragma unroll
                    for (int d = 0; d < DOF; d++) x[d] = FSB_AT(P, d, p);
                    const float v = Sys::pot(x);
                    if (VC) Vc[FSB_VIDX(p)] = v;
                    aNew = __fadd_rn(aNew, __fmul_rn(eps, v));
                }
                if (__expf(__fsub_rn(aOld, aNew)) < fsb_uniform(g)) {
#pragma unroll 1
                    for (int i = 1; i < seg; i++) {
                        const int p = (start + i) & (N - 1);
#pragma unroll
                        for (int d = 0; d < DOF; d++) FSB_AT(P, d, p) = s_old[((i - 1) * DOF + d) * nthr + tid];
                        if (VC) Vc[FSB_VIDX(p)] = s_oldv[(i - 1) * nthr + tid];
                    }
                } else {
                    n_acc++;
                }
                fs_walker_sync(tpw, wl);
            }
            // ---- measurement: the thread's slices (kernel.c:734-745), summed in FP32 in
            // slice order and then added once to the FP64 sums (a chain of FP64 adds per
            // slice is slow on GB300's narrow FP64 pipe) ----
            if (Sys::NOPS > 0) {
                float opp[Sys::NOPS > 0 ? Sys::NOPS : 1];
#pragma unroll
                for (int k = 0; k < Sys::NOPS; k++) opp[k] = 0.0f;
#pragma unroll 1
                for (int s = t * seg; s < (t + 1) * seg; s++) {
                    float x[DOF], ov[Sys::NOPS > 0 ? Sys::NOPS : 1];
#pragma unroll
                    for (int d = 0; d < DOF; d++) x[d] = FSB_AT(P, d, s);
                    Sys::ops(x, ov);
#pragma unroll
                    for (int k = 0; k < Sys::NOPS; k++) opp[k] = __fadd_rn(opp[k], ov[k]);
                }
#pragma unroll
                for (int k = 0; k < Sys::NOPS; k++) opd[k] += (double)opp[k];
            }
            fs_walker_sync(tpw, wl);
        }
        sd.accepts[th] = n_acc;
#if FSB_RANLUX
        fs_rl_store(g.st, sd.rtab + (size_t)th * 28);
        if (t == 0) fs_rl_store(ws.st, sd.gtab + (size_t)w * 28);
#else
        *(uint4 *)(sd.seeds + (size_t)th * 4) = make_uint4(g.x, g.y, g.z, g.w);
        if (t == 0) *(uint4 *)(sd.wseeds + (size_t)w * 4) = make_uint4(ws.x, ws.y, ws.z, ws.w);
#endif
#pragma unroll
        for (int k = 0; k < Sys::NOPS; k++) atomicAdd(s_op + wl * Sys::NOPS + k, opd[k]);
    }
    __syncthreads();
    {
        if (!GLOBAL) {
            const size_t base = (size_t)w0 * DOF * N;
            const int count = n_here * DOF * N;
            for (int i = tid; i < count; i += blockDim.x) {
                const int wi = i / (DOF * N), r = i - wi * (DOF * N);
                const int d = r / N, sl = r - d * N;
                sd.paths[base + i] = FSB_AT(smem + wi * wstride, d, sl);
            }
        }
        for (int i = tid; i < n_here * sd.nops; i += blockDim.x) sd.op_sums[(size_t)w0 * sd.nops + i] += s_op[i];
    }
    __syncthreads();  // the next tile reuses the shared-memory tile
#undef FSB_VIDX
#undef FSB_AT
}
