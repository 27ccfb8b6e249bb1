// fs_pimc.cuh -- the Metropolis-bisection path-integral sweep (sm_103a, NVRTC-specialised).
//
// fs_api.cu builds one module per run configuration, exactly as the reference rebuilds
// its OpenCL program per configuration (FeynSimul/kernel.py:215-381): the FS_* macros,
// the RNG header and the plugin's userCode / potential / operator / correlator strings are
// pasted in front of this file.
//
// Work decomposition (kernel.py:192-211 semantics, GB300 layout):
//   * one CUDA thread per reference work-item: a walker's N/2^S "segment threads" bisect
//     their own 2^S-slice segment of the walker's path at a per-step random offset shared
//     by the walker (kernel.c:709-721); walker mode is one thread per walker;
//   * FS_WPB walkers per CTA; a walker's threads sit in one warp (TPW <= 32, synchronised
//     by __syncwarp on the walker's lanes) or fill the CTA (TPW > 32, __syncthreads);
//   * the walker's whole path [DOF][N] lives in shared memory for the whole launch (padded
//     so the segment threads' accesses are free of bank conflicts), loaded and stored once
//     with coalesced reads and writes of the reference's walker-major layout;
//   * RNG state in registers; global accepts / seeds / operator means keep the
//     reference's thread-id layout (kernel.c:541) so the host reductions are unchanged;
//   * operator and correlator running sums in registers (FP64 unless the
//     reference-order FP32 mode is selected), histogram counts privatised per CTA in
//     shared memory.
#pragma once

#define FS_HALF_N (FS_N / 2)
#define FS_THREADS (FS_NWALKERS * FS_TPW)
// Correlator helpers (FS_MX > 1, set by the host for correlator runs whose walkers have few
// segment threads): the CTA holds FS_MX groups of FS_WPB x FS_TPW threads.  Group 0 runs the
// moves and the per-slice measurement; every group sums correlator lags, so a walker's N/2
// lags spread over FS_TPW x FS_MX threads instead of its FS_TPW segment threads.  Each lag is
// still summed by one thread in slice order, so the sums are the same bit for bit.
// FS_PIPE (the host sets it where the movers fill whole warps): the movers measure the
// operators and copy their slices into a double-buffered path snapshot (FS_SNSTRIDE words
// each, the padded slice layout); the helper groups evaluate the correlator values on the
// snapshot and sum the lags, for measurement m while the movers sweep towards measurement
// m + 1.  One CTA barrier per measurement hands a snapshot over; the movers sync among
// themselves on named barrier 1 and the helpers on named barrier 2.  Every sum is formed in
// the same order as without the pipeline, so the results are the same bit for bit.
#ifndef FS_MX
#define FS_MX 1
#endif
#ifndef FS_PIPE
#define FS_PIPE 0
#endif
#ifndef FS_SNSTRIDE
#define FS_SNSTRIDE 0
#endif
#define FS_MBLOCK (FS_WPB * FS_TPW)          // threads that run the moves
#define FS_BLOCK (FS_MBLOCK * FS_MX)
#define FS_CTPW (FS_TPW * (FS_MX - FS_PIPE))  // correlator threads per walker
#if FS_PIPE
#define FS_LPT 4                             // lags 4 lt .. 4 lt + 3
#define FS_LAG(j) (4 * lt + (j))
#else
#define FS_LPT ((FS_HALF_N + FS_CTPW - 1) / FS_CTPW)  // correlator lags owned per thread
#define FS_LAG(j) (lt + (j) * FS_CTPW)
#endif
#if FS_MX > 1 && (!FS_PARALLEL || FS_TPW > 32 || FS_GLOBAL || FS_NCOR == 0 || FS_NWALKERS % FS_WPB != 0)
#error "correlator helpers need parallel-path walkers of at most 32 threads in shared memory, correlators, and full CTAs"
#endif
#if FS_PIPE && (FS_MX < 2 || FS_MBLOCK % 32 != 0 || FS_LEARNED || FS_SNSTRIDE < FS_DOF * (FS_N + (FS_N >> FS_S)) || FS_SNSTRIDE % 16 != 0 || FS_N % 8 != 0 || FS_CTPW < FS_N / 8)
#error "pipelined correlator helpers need helper groups, whole warps of movers and a path snapshot"
#endif
#define FS_COR_REGS (FS_ACCUM != 3 && FS_LPT * FS_NCOR <= 16)
#define FS_CSTEP (FS_N % 4 == 0 ? 4 : 1)  // FP64 correlator: partial sums over s1 mod 4
// Correlator FP64 sums of FP32 builds (FP64, Kahan and study modes): one measurement's
// products of a lag are summed in FP32, then added to the lag's FP64 running sum.  The FP32
// partial (FS_PARTIALS, fs_config.partials) is either four fused multiply-add chains
// over the slices s1 mod 4, added pairwise (FS_COR_FMA; 0, the default), or the rounded
// products in float-float (FS_COR_FF, fs_ff_add; 1, and always in the study mode, whose FP32
// and Kahan columns sum the same products in slice order).  The FMA partial of an N-slice
// lag sum is within gamma(N/4 + 2) * sum_s |x_s x_(s+tau)| <= gamma(N/4 + 2) * C(0) of the
// exact sum (gamma(n) = n u / (1 - n u), u = 2^-24; sum_s |x_s x_(s+tau)| <= sum_s x_s^2 by
// Cauchy-Schwarz).  FS_COR_ILV (set by the host, which sizes shared memory for it): a thread
// owning at most 4 lags sums them in one pass over the slice values, which are stored twice
// in a row (FS_CSTRIDE = 2N words per correlator) so that slice s1 + tau is read without a
// wrap.
#ifndef FS_PARTIALS
#define FS_PARTIALS 0
#endif
#define FS_COR_FMA ((FS_ACCUM == 1 || FS_ACCUM == 2) && !FS_DOUBLE && FS_PARTIALS == 0)
// Operator FP64 sums of FP32 builds ("fp64" accumulation, FS_PARTIALS 0, parallel-path
// mode): a segment thread's 2^S values of one measurement summed in FP32 in slice order,
// within gamma(2^S) * sum |value| of the exact sum, then one FP64 add (GB300's FP64 pipe is
// narrow: a chain of FP64 adds per slice made the measurement latency bound)
#define FS_OP_PART (FS_ACCUM == 1 && !FS_DOUBLE && FS_PARTIALS == 0 && FS_PARALLEL)
#define FS_COR_FF (FS_ACCUM != 0 && !FS_DOUBLE && !FS_COR_FMA)
#ifndef FS_COR_ILV
#define FS_COR_ILV 0
#endif
#if FS_COR_ILV && !((FS_COR_FF || FS_COR_FMA) && FS_LPT <= 4 && (FS_PIPE || FS_LPT * FS_CTPW <= FS_N))
#error "FS_COR_ILV needs FP32 correlator partials and at most 4 lags per thread"
#endif
#if FS_PIPE && !(FS_COR_FMA && FS_COR_ILV)
#error "pipelined correlator helpers sum FP32 partials over doubled slice values"
#endif
#define FS_CSTRIDE (FS_COR_ILV ? 2 * FS_N : FS_N)
#ifndef FS_CWSTRIDE
#define FS_CWSTRIDE (FS_NCOR * FS_CSTRIDE)  // per-walker correlator buffer (the host pads it)
#endif
#if FS_CWSTRIDE < 2 * FS_SNSTRIDE + FS_NCOR * FS_CSTRIDE
#error "per-walker correlator buffer smaller than its slice values"
#endif

// Shared-memory path layout.  Slice s of degree d of a walker sits at d * FS_DSTRIDE +
// FS_PHYS(s) with one padding word after every 2^S slices: the segment threads of a walker
// read slices 2^S apart, which the padding turns into 2^S + 1 words apart, an odd stride,
// so the threads of a warp hit distinct banks.  FS_WSTRIDE (walker stride, from the host)
// is an odd multiple of 16 words so two walkers sharing a warp use opposite bank halves.
//
// Global-path mode (FS_GLOBAL, the reference's ENABLE_GLOBAL_PATH, kernel.c:62-70 and
// :582-588): the walker's threads work in place on its [DOF][N] rows of the paths array
// (cached in L1/L2), for paths larger than shared memory; same arithmetic, same results.
#if FS_GLOBAL
#define FS_PHYS(s) (s)
#define FS_DSTRIDE FS_N
#else
#define FS_PHYS(s) ((s) + ((s) >> FS_S))
#define FS_DSTRIDE (FS_N + (FS_N >> FS_S))
#endif
#define FS_AT(P, d, s) (P)[(d) * FS_DSTRIDE + FS_PHYS(s)]
#ifndef FS_VCACHE
#define FS_VCACHE 0
#define FS_VSTRIDE 0
#endif
// The potential cache lives in shared memory (FS_VSTRIDE words per walker, the path's padded
// slice layout) or, with FS_VGLOBAL, in device memory: N values per walker, slice s at
// (s mod 2^S) * (N / 2^S) + s / 2^S, so the segment threads of a walker, whose slices lie
// 2^S apart, touch consecutive words.  It costs no shared memory there, only L1/L2 traffic.
#ifndef FS_VGLOBAL
#define FS_VGLOBAL 0
#endif
#if FS_VGLOBAL
#define FS_VIDX(s) ((((s) & (FS_SEG - 1)) * (FS_N / FS_SEG)) + ((s) >> FS_S))
#else
#define FS_VIDX(s) FS_PHYS(s)
#endif
// a move keeps its old cached values (FS_SEG - 1 of them) for a rejection
#ifndef FS_VKEEP
#define FS_VKEEP (FS_SEG <= 33)
#endif

#if FS_DOUBLE
#define FS_ADD __dadd_rn
#define FS_SUB __dsub_rn
#define FS_MUL __dmul_rn
#define FS_DIV __ddiv_rn
#define FS_SQRT_RN __dsqrt_rn
#define FS_LOG log
#define FS_SQRT sqrt
#define FS_SIN sin
#define FS_EXP exp
#define FS_TWO_PI 6.283185307179586
#else
#define FS_ADD __fadd_rn
#define FS_SUB __fsub_rn
#define FS_MUL __fmul_rn
#define FS_DIV __fdiv_rn
#define FS_SQRT_RN __fsqrt_rn
#if FS_FAST
#define FS_LOG __logf
#define FS_SIN __sinf
#define FS_EXP __expf
#else
#define FS_LOG logf
#define FS_SIN sinf
#define FS_EXP expf
#endif
#define FS_SQRT sqrtf
#define FS_TWO_PI 6.28318548f  // 2 * float(pi), as the reference's single-precision constant
#endif

// ---------------------------------------------------------------- streams
#if FS_RANLUX
#if FS_DOUBLE
typedef FsRanluxStream64<FS_NSKIP> FsUStream;
#else
typedef FsRanluxStream<FS_NSKIP> FsUStream;
#endif
__device__ __forceinline__ FT fs_uniform(FsUStream &g) { return g.next(); }
typedef FsUStream FsIStream;
#else
typedef FsXorshift FsUStream;
typedef FsXorshift FsIStream;
__device__ __forceinline__ FT fs_uniform(FsXorshift &g)
{
#if FS_DOUBLE
    return fs_xs_double(g);
#else
    return fs_xs_float(g);
#endif
}
#endif

// offset of the walker's segment grid for one Metropolis step (kernel.c:715, :718)
__device__ __forceinline__ fs_u32 fs_offset(FsIStream &g, fs_u32 range)
{
#if FS_RANLUX
    FT f = g.next();
#if FS_COMPAT
    // (uint)(f * (ranluxIntMax+1)) (kernel.c:206): low 8 bits are zero
    return ((fs_u32)FS_MUL(f, (FT)FS_RIM)) & (range - 1u);
#else
    return ((fs_u32)FS_MUL(f, (FT)range)) & (range - 1u);
#endif
#else
    return fs_xs_next(g) & (range - 1u);
#endif
}

#if FS_SEG > 1
#define FS_OLD_N ((FS_SEG - 1) * FS_DOF)
#else
#define FS_OLD_N 1
#endif

// Rolled move loops for RANLUX (its generator calls are large) and for big plugins (a
// fully unrolled move repeats the potential 2 * (2^S - 1) times, which for a 10-atom
// cluster costs minutes of compilation and overflows the instruction cache)
#if FS_RANLUX || FS_DOF > 8
#define FS_MOVE_UNROLL _Pragma("unroll 1")
#else
#define FS_MOVE_UNROLL _Pragma("unroll")
#endif
// The old- and new-action loops (2^S - 1 potential evaluations each)
#ifndef FS_ACT_UNROLL
#define FS_ACT_UNROLL FS_MOVE_UNROLL
#endif

// kernel.c:258-399 on a shared-memory path P[DOF][N].
// With the learned proposal (FS_LEARNED) the level-1 midpoint is drawn from N(lmu, lsd^2)
// instead of the free-particle bridge N(mid, sigma_1^2).  Both the forward and the reverse
// proposal condition on the segment's endpoints, which the move does not change, and the
// other nodes keep the free-particle proposal, whose density ratio cancels the kinetic
// action exactly; the Metropolis-Hastings log-ratio therefore gains only, per degree of
// freedom of that node, [(x_old - mid)^2 - (x_new - mid)^2] / (2 sigma_1^2)
// + [z_new^2 - ((x_old - lmu) / lsd)^2] / 2, with z_new the standard normal drawn.
//
// Potential cache (FS_VCACHE): Vc holds V(x_s) of every slice of the walker's current path
// (FS_VIDX: shared or device memory).  The old action is then a sum of cached values
// -- the same products and sums as evaluating V again, so bit for bit the same aOld --
// and only the proposed nodes are evaluated; an accepted move leaves their new values in
// the cache, a rejected one restores the path and writes the kept old values back
// (FS_VKEEP), or re-evaluates its nodes.
__device__ __forceinline__ int fs_bisect(FT *P, FT *Vc, fs_u32 start, FsUStream &g, const FT *sigma,
                                         const FT *lmu, const FT *lsd)
{
    FT corr = (FT)0;
    FT old[FS_OLD_N];
    FT aOld = (FT)0;
#pragma unroll
    for (int i = 1; i < FS_SEG; i++) {
        const fs_u32 p = (start + (fs_u32)i) & (FS_N - 1);
#pragma unroll
        for (int d = 0; d < FS_DOF; d++) old[(i - 1) * FS_DOF + d] = FS_AT(P, d, p);
    }
#if FS_VCACHE
    // cached values: the loads are independent, so they are issued together; with at most
    // 32 interior slices they are kept and written back if the move is rejected (a
    // re-evaluation there would cost the warp the potential of every slice whenever one of
    // its lanes rejects)
#if FS_VKEEP
    FT vold[FS_SEG - 1];
#pragma unroll
    for (int i = 1; i < FS_SEG; i++) {
        const fs_u32 p = (start + (fs_u32)i) & (FS_N - 1);
        vold[i - 1] = Vc[FS_VIDX(p)];
        aOld = FS_ADD(aOld, FS_MUL((FT)FS_EPS, vold[i - 1]));
    }
#else
#pragma unroll 16
    for (int i = 1; i < FS_SEG; i++) {
        const fs_u32 p = (start + (fs_u32)i) & (FS_N - 1);
        aOld = FS_ADD(aOld, FS_MUL((FT)FS_EPS, Vc[FS_VIDX(p)]));
    }
#endif
#else
    FS_ACT_UNROLL
    for (int i = 1; i < FS_SEG; i++) {
        const fs_u32 p = (start + (fs_u32)i) & (FS_N - 1);
        aOld = FS_ADD(aOld, FS_MUL((FT)FS_EPS, fs_pot(FS_ARGS_AT(P, p))));
    }
#endif
    FS_MOVE_UNROLL
    for (int n = 1; n <= FS_S; n++) {
        const int half = 1 << (FS_S - n);
        const FT sig = sigma[n];
        FS_MOVE_UNROLL
        for (int i = 0; i < (1 << (n - 1)); i++) {
            const fs_u32 m = ((fs_u32)((1 + 2 * i) * half) + start) & (FS_N - 1);
            const fs_u32 l = ((fs_u32)(i * 2 * half) + start) & (FS_N - 1);
            const fs_u32 r = ((fs_u32)((i + 1) * 2 * half) + start) & (FS_N - 1);
#if FS_RANLUX && !FS_DOUBLE && (2 * FS_DOF) % 4 == 0
            // the node's 2*DOF uniforms (u, v per degree) in whole generator calls
            float uv[2 * FS_DOF];
            g.template next_k<2 * FS_DOF>(uv);
#pragma unroll
            for (int d = 0; d < FS_DOF; d++) {
                const FT u = uv[2 * d];
                const FT v = uv[2 * d + 1];
#else
            FS_MOVE_UNROLL
            for (int d = 0; d < FS_DOF; d++) {
                const FT u = fs_uniform(g);
                const FT v = fs_uniform(g);
#endif
#if FS_LEARNED
                if (n == 1) {
                    FT z = (FT)0;
                    if (v != (FT)0) z = FS_MUL(FS_SQRT(FS_MUL((FT)-2, FS_LOG(v))), FS_SIN(FS_MUL((FT)FS_TWO_PI, u)));
                    const FT mid = FS_MUL((FT)0.5, FS_ADD(FS_AT(P, d, l), FS_AT(P, d, r)));
                    const FT xo = FS_AT(P, d, m);
                    const FT xn = lmu[d] + lsd[d] * z;
                    const FT dn = xn - mid, dov = xo - mid, zo = (xo - lmu[d]) / lsd[d];
                    corr += (dov * dov - dn * dn) / (2 * sig * sig) + (FT)0.5 * (z * z - zo * zo);
                    FS_AT(P, d, m) = xn;
                    continue;
                }
#endif
                // sigma_n * sqrt(-2 log v) * sin(2 pi u), left to right (kernel.c:352-353), or 0
                // for v == 0 (kernel.c:349-351).  Evaluated unconditionally and selected: log 0
                // is -inf, so that lane's product is infinite or NaN and is discarded, and no
                // branch is taken per degree of freedom.
                FT rz = FS_MUL(FS_MUL(sig, FS_SQRT(FS_MUL((FT)-2, FS_LOG(v)))),
                               FS_SIN(FS_MUL((FT)FS_TWO_PI, u)));
                rz = v != (FT)0 ? rz : (FT)0;
                FS_AT(P, d, m) = FS_ADD(FS_MUL((FT)0.5, FS_ADD(FS_AT(P, d, l), FS_AT(P, d, r))), rz);
            }
        }
    }
    FT aNew = (FT)0;
    FS_ACT_UNROLL
    for (int i = 1; i < FS_SEG; i++) {
        const fs_u32 p = (start + (fs_u32)i) & (FS_N - 1);
        const FT v = fs_pot(FS_ARGS_AT(P, p));
#if FS_VCACHE
        Vc[FS_VIDX(p)] = v;
#endif
        aNew = FS_ADD(aNew, FS_MUL((FT)FS_EPS, v));
    }
    const FT acc = fs_uniform(g);
#if FS_LEARNED
    if (FS_EXP(FS_SUB(aOld, aNew) + corr) < acc) {
#else
    (void)corr;
    (void)lmu;
    (void)lsd;
    if (FS_EXP(FS_SUB(aOld, aNew)) < acc) {
#endif
#pragma unroll
        for (int i = 1; i < FS_SEG; i++) {
            const fs_u32 p = (start + (fs_u32)i) & (FS_N - 1);
#pragma unroll
            for (int d = 0; d < FS_DOF; d++) FS_AT(P, d, p) = old[(i - 1) * FS_DOF + d];
        }
#if FS_VCACHE && FS_VKEEP
#pragma unroll
        for (int i = 1; i < FS_SEG; i++) Vc[FS_VIDX((start + (fs_u32)i) & (FS_N - 1))] = vold[i - 1];
#elif FS_VCACHE
        FS_MOVE_UNROLL
        for (int i = 1; i < FS_SEG; i++) {
            const fs_u32 p = (start + (fs_u32)i) & (FS_N - 1);
            Vc[FS_VIDX(p)] = fs_pot(FS_ARGS_AT(P, p));
        }
#else
        (void)Vc;
#endif
        return 0;
    }
    return 1;
}

#ifndef FS_BISECT
#define FS_BISECT 1
#endif
#ifndef FS_PATH_SHIFT
#define FS_PATH_SHIFT 0
#endif
#ifndef FS_SNM
#define FS_SNM 0
#endif

#if FS_PATH_SHIFT || FS_SNM
// kernel.c:245-249: half the squared step over epsilon^2
__device__ __forceinline__ FT fs_kin(FT a, FT b)
{
    const FT d = FS_SUB(a, b);
    return FS_MUL(FS_MUL((FT)0.5, FS_MUL(d, d)), (FT)FS_EPS_INV2);
}
#endif

#if FS_PATH_SHIFT
// kernel.c:407-473: shift slices left..right (cyclically) of one degree of freedom by
// offset; returns the change of the kinetic + potential sum.  left == right shifts nothing.
__device__ __forceinline__ FT fs_shift(FT *P, int degree, FT offset, fs_u32 left, fs_u32 right)
{
    if (left == right) return (FT)0;
    FT kinDiff = (FT)0, potDiff = (FT)0;
    fs_u32 ll, rr;
    if (left < right) {
        ll = left == 0 ? FS_N - 1 : left - 1;
        rr = right == FS_N - 1 ? 0 : right + 1;
    } else {
        ll = left - 1;
        rr = right + 1;
    }
    kinDiff = FS_SUB(kinDiff, fs_kin(FS_AT(P, degree, left), FS_AT(P, degree, ll)));
    kinDiff = FS_SUB(kinDiff, fs_kin(FS_AT(P, degree, right), FS_AT(P, degree, rr)));
    // slices left, left+1, ... right (mod N), in the reference's order
    const fs_u32 count = left < right ? right - left + 1 : FS_N - left + right + 1;
#pragma unroll 1
    for (fs_u32 j = 0; j < count; j++) {
        const fs_u32 i = (left + j) & (FS_N - 1);
        potDiff = FS_SUB(potDiff, fs_pot(FS_ARGS_AT(P, i)));
        FS_AT(P, degree, i) = FS_ADD(FS_AT(P, degree, i), offset);
        potDiff = FS_ADD(potDiff, fs_pot(FS_ARGS_AT(P, i)));
    }
    kinDiff = FS_ADD(kinDiff, fs_kin(FS_AT(P, degree, left), FS_AT(P, degree, ll)));
    kinDiff = FS_ADD(kinDiff, fs_kin(FS_AT(P, degree, right), FS_AT(P, degree, rr)));
    return FS_ADD(kinDiff, potDiff);
}

// kernel.c:640-666: one path-shift move of degree k % DOF; saved holds N values of scratch
__device__ __forceinline__ int fs_path_shift_move(FT *P, unsigned long long k, FsIStream &is, FsUStream &g,
                                                  FT *saved)
{
    const int degree = (int)(k % FS_DOF);
    const fs_u32 left = fs_offset(is, FS_N);
    const fs_u32 right = fs_offset(is, FS_N);
    const FT offset = FS_MUL((FT)FS_PSALPHA, FS_SUB(FS_MUL((FT)2, fs_uniform(g)), (FT)1));
#if !FS_COMPAT
#pragma unroll 1
    for (int i = 0; i < FS_N; i++) saved[i] = FS_AT(P, degree, i);
#else
    (void)saved;
#endif
    const FT diff = fs_shift(P, degree, offset, left, right);
    if (FS_EXP(FS_MUL((FT)(-FS_EPS), diff)) < fs_uniform(g)) {
#if FS_COMPAT
        // the reference reverts by shifting again by -offset (kernel.c:654-656), which
        // leaves the rounding of x + offset - offset in the path
        if (left != right) {
            const fs_u32 count = left < right ? right - left + 1 : FS_N - left + right + 1;
#pragma unroll 1
            for (fs_u32 j = 0; j < count; j++) {
                const fs_u32 i = (left + j) & (FS_N - 1);
                FS_AT(P, degree, i) = FS_ADD(FS_AT(P, degree, i), -offset);
            }
        }
#else
#pragma unroll 1
        for (int i = 0; i < FS_N; i++) FS_AT(P, degree, i) = saved[i];
#endif
        return 0;
    }
    return 1;
}
#endif

#if FS_SNM
// kernel.c:668-705: single-node move of node k mod (N * DOF), uniform in +-alpha
__device__ __forceinline__ int fs_single_node_move(FT *P, unsigned long long k, FsUStream &g)
{
    const fs_u32 modPoint = (fs_u32)(k % FS_N);
    const int degree = (int)((k % ((unsigned long long)FS_N * FS_DOF)) / FS_N);
    const fs_u32 l = modPoint == 0 ? FS_N - 1 : modPoint - 1;
    const fs_u32 r = modPoint == FS_N - 1 ? 0 : modPoint + 1;
    const FT oldX = FS_AT(P, degree, modPoint);
    const FT xl = FS_AT(P, degree, l), xr = FS_AT(P, degree, r);
    const FT modX = FS_ADD(oldX, FS_MUL(FS_SUB(FS_MUL((FT)2, fs_uniform(g)), (FT)1), (FT)FS_ALPHA));
    FT dE = FS_SUB(FS_SUB(FS_ADD(fs_kin(modX, xr), fs_kin(modX, xl)), fs_kin(oldX, xl)), fs_kin(oldX, xr));
    dE = FS_SUB(dE, fs_pot(FS_ARGS_AT(P, modPoint)));
    FS_AT(P, degree, modPoint) = modX;
    dE = FS_ADD(dE, fs_pot(FS_ARGS_AT(P, modPoint)));
    FS_AT(P, degree, modPoint) = oldX;
    if (FS_EXP(FS_MUL((FT)(-FS_EPS), dE)) > fs_uniform(g)) {
        FS_AT(P, degree, modPoint) = modX;
        return 1;
    }
    return 0;
}
#endif

struct FsArgs {
    FT *paths;                 // [walkers][DOF][N]
    fs_u32 *accepts;           // [threads]
    fs_u32 *seeds;             // xorshift [threads+1][4]
    const fs_u32 *seed_snap;   // xorshift, reference-compatible mode: table at launch start
    fs_u32 *walker_seeds;      // xorshift, fixed mode: [walkers][4]
    fs_u32 *rtab;              // RANLUX [threads][28]
    fs_u32 *gtab;              // RANLUX compat [threads][28], fixed [walkers][28]
    void *op_means;            // [threads][nOps] (study mode: [threads][nOps][3] double)
    void *cor_means;           // [walkers][nCorr][N/2]
    fs_u32 *bins;              // [res^DOF]
    fs_u64 *hist;              // [hist bins]
    int *status;               // [0] flags (FS_STATUS_*), [1] 1 + a walker that raised one
    double opnorm;
    FT *shift_old;             // path shift, fixed mode: the shifted row before the move [walkers][N]
    unsigned long long step_base;  // fixed mode: Metropolis steps of earlier launches
    const uint2 *mlp_frag;     // learned proposal: network fragments and biases
    const float *mlp_bias;
    float mlp_inv_scale;       // features = endpoint coordinates * mlp_inv_scale
    int block_offset;          // first CTA of this launch (chunked launches of fs_run_host)
    FT *vcache;                // potential cache in device memory (FS_VGLOBAL): [walkers][N]
};

__device__ __forceinline__ int fs_thread_id(int w, int t)
{
#if FS_PARALLEL
    const int g = w / FS_WPG, l1 = w % FS_WPG;
    return g * FS_TPW + t + l1 * FS_NWG * FS_TPW;  // kernel.c:539-541
#else
    return w;
#endif
}

#if FS_ACCUM == 0
typedef FT FsCorAcc;
#elif FS_ACCUM == 3
// precision study: the same products summed in plain FP32, Kahan FP32 and FP64 (24 bytes)
struct FsCorAcc {
    double d;
    float f, ks, kc, pad;
};
#else
typedef double FsCorAcc;
#endif

// FP32 -> FP64 on the integer pipe (GB300's FP64 pipe is narrow, and the FP64 sums spend
// one conversion per term there): exact for every value a flush-to-zero build produces --
// normal numbers and signed zeros; infinities and NaNs kept.  The sign moves to bit 63, the
// exponent is rebiased by 1023 - 127, the mantissa moves up by 29 bits.  IEEE builds (which
// can produce denormals) convert in hardware.
__device__ __forceinline__ double fs_f2d(float x)
{
#if FS_FAST && !FS_DOUBLE
    const unsigned u = __float_as_uint(x);
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned sign = u & 0x80000000u;
    unsigned hi;
    if (e == 0u) hi = sign;
    else if (e == 0xFFu) hi = sign | 0x7FF00000u | ((u & 0x7FFFFFu) >> 3);
    else hi = sign | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
#else
    return (double)x;
#endif
}
__device__ __forceinline__ double fs_f2d(double x) { return x; }

// float-float accumulation: Knuth's TwoSum yields the exact rounding error of s + q, and the
// errors are summed on the side (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM
// J. Sci. Comput. 26 (2005), Algorithm 4.4 "Sum2"); s + e then carries about 48 significant
// bits.  Explicitly rounded adds, so no contraction or reassociation can touch the steps.
__device__ __forceinline__ void fs_ff_add(float &s, float &e, float q)
{
    const float t = __fadd_rn(s, q);
    const float bp = __fsub_rn(t, s);
    const float ap = __fsub_rn(t, bp);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, ap), __fsub_rn(q, bp)));
    s = t;
}

__device__ __forceinline__ void fs_kahan(float &s, float &c, float x)
{
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// 16-byte path staging: FS_VEC values of one degree of freedom at slices s .. s + FS_VEC - 1
// (s a multiple of FS_VEC) are consecutive in global memory and, when 2^S >= FS_VEC, in the
// padded shared layout.  Every walker's block starts at a multiple of N values, and the
// paths array is allocated 256-byte aligned, so the 16-byte global accesses are aligned.
#if FS_DOUBLE
typedef double2 FsVec;
#define FS_VEC_N 2
#else
typedef float4 FsVec;
#define FS_VEC_N 4
#endif
#if !FS_GLOBAL && FS_N % FS_VEC_N == 0 && (1 << FS_S) >= FS_VEC_N
#define FS_VEC FS_VEC_N
#else
#define FS_VEC 1
#endif
__device__ __forceinline__ void fs_vec_scatter(FT *d, const FsVec v)
{
#if FS_DOUBLE
    d[0] = v.x; d[1] = v.y;
#else
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
#endif
}
__device__ __forceinline__ FsVec fs_vec_gather(const FT *d)
{
#if FS_DOUBLE
    return make_double2(d[0], d[1]);
#else
    return make_float4(d[0], d[1], d[2], d[3]);
#endif
}
__device__ __forceinline__ bool fs_vec_finite(const FsVec v)
{
#if FS_DOUBLE
    return isfinite(v.x) && isfinite(v.y);
#else
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w);
#endif
}

// Status word: a path value that is not finite (NaN or infinity) at the end of a launch.
// Every path value passes through the launch's path-out copy (or, for global paths, the
// owner's final check), so one compare per value per launch finds any walker whose
// proposals or potential blew up; the host reads the word at fs_sync.
#define FS_STATUS_NONFINITE 1
__device__ __forceinline__ void fs_flag_nonfinite(int *status, int walker)
{
    atomicOr(status, FS_STATUS_NONFINITE);
    atomicCAS(status + 1, 0, walker + 1);
}

// Per-launch segment offsets (RANLUX, parallel-path mode): the walker's offset stream feeds
// only the bisection's segment offsets there (kernel.c:715-718), one draw per Metropolis
// step, independent of the path.  So one lane draws the launch's FS_OPRUNS * FS_MSTEPS
// offsets up front into shared memory (one byte each, segments of at most 256 slices), and
// the steps read them: the same draws in the same order, and the generator's code for that
// stream stays out of the move loop.
#define FS_NSTEPS_LAUNCH (FS_OPRUNS * FS_MSTEPS)
#if FS_RANLUX && FS_PARALLEL && FS_BISECT && FS_SEG <= 256 && FS_NSTEPS_LAUNCH <= 256
#define FS_OFF_PRE 1
#else
#define FS_OFF_PRE 0
#endif

#ifndef FS_RNG_ONLY
#if FS_MINB > 0
#define FS_LAUNCH_BOUNDS __launch_bounds__(FS_BLOCK, FS_MINB)
#else
#define FS_LAUNCH_BOUNDS __launch_bounds__(FS_BLOCK)
#endif
extern "C" __global__ void FS_LAUNCH_BOUNDS fs_metropolis(FsArgs a)
{
    extern __shared__ __align__(16) unsigned char fs_smem[];
#if FS_RANLUX
    __shared__ FsIStream s_istream[FS_WPB];
#if FS_OFF_PRE
    __shared__ unsigned char s_offs[FS_WPB][FS_NSTEPS_LAUNCH];
#else
    __shared__ fs_u32 s_off[FS_WPB];
#endif
#endif
#if FS_GLOBAL
    FT *s_v = (FT *)fs_smem;                                     // [WPB][VSTRIDE] (FS_VCACHE)
#else
    FT *s_path = (FT *)fs_smem;                                  // [WPB][DOF*N]
    FT *s_v = s_path + FS_WPB * FS_WSTRIDE;                      // [WPB][VSTRIDE] (FS_VCACHE)
#endif
    FT *s_cor = s_v + FS_WPB * FS_VSTRIDE;                     // [WPB][CWSTRIDE >= NCOR * CSTRIDE]
    fs_u32 *s_hist = (fs_u32 *)(s_cor + FS_WPB * FS_CWSTRIDE);  // [HBINS]

    const int tid_b = threadIdx.x;
    const int grp = tid_b / FS_MBLOCK;             // 0: movers; 1..FS_MX-1: correlator helpers
    const int wl = (tid_b - grp * FS_MBLOCK) / FS_TPW;
    const int t = tid_b % FS_TPW;
    const bool mover = FS_MX == 1 || grp == 0;
    // this thread's lags FS_LAG(j): lt + j * FS_CTPW; with FS_PIPE the helper lanes lt < N/8
    // own lags 4 lt + j
    const int lt = (grp - FS_PIPE) * FS_TPW + t;
    const bool lagger = FS_PIPE ? !mover && lt < FS_N / 8 : true;
    const int w0 = (blockIdx.x + a.block_offset) * FS_WPB;
    const int w = w0 + wl;
    const int n_here = min(FS_WPB, FS_NWALKERS - w0);
    const bool active = wl < n_here;

    // ---- path in (coalesced global reads; padded shared layout) ----
    {
#if !FS_GLOBAL
        const size_t base = (size_t)w0 * FS_DOF * FS_N;
        const int count = n_here * FS_DOF * FS_N;
#if FS_VEC > 1
        // 16-byte loads of FS_VEC consecutive slices; they lie in one 2^S block of the padded
        // layout, so their shared-memory words are consecutive too
        const FsVec *src = (const FsVec *)(a.paths + base);
        for (int i4 = tid_b; i4 < count / FS_VEC; i4 += FS_BLOCK) {
            const int i = i4 * FS_VEC;
            const int wi = i / (FS_DOF * FS_N), r = i - wi * (FS_DOF * FS_N);
            const int d = r / FS_N, sl = r - d * FS_N;
            FT *dst = &FS_AT(s_path + wi * FS_WSTRIDE, d, sl);
            const FsVec v = src[i4];
            fs_vec_scatter(dst, v);
        }
#else
        for (int i = tid_b; i < count; i += FS_BLOCK) {
            const int wi = i / (FS_DOF * FS_N), r = i - wi * (FS_DOF * FS_N);
            const int d = r / FS_N, sl = r - d * FS_N;
            FS_AT(s_path + wi * FS_WSTRIDE, d, sl) = a.paths[base + i];
        }
#endif
#endif
#if FS_NHIST > 0
        for (int i = tid_b; i < FS_HBINS; i += FS_BLOCK) s_hist[i] = 0u;
#endif
    }
    __syncthreads();

    if (active) {
#if FS_PIPE
        // the movers' own barrier (whole warps; the helpers never wait on it)
#if FS_MBLOCK == 32
#define FS_WSYNC() do { if (mover) __syncwarp(); } while (0)
#else
#define FS_WSYNC() do { if (mover) asm volatile("bar.sync 1, %0;" ::"n"(FS_MBLOCK) : "memory"); } while (0)
#endif
#elif FS_TPW <= 32 && FS_MX == 1
        const unsigned lane = threadIdx.x & 31u;
        const unsigned wmask = FS_TPW == 32 ? 0xFFFFFFFFu
                                            : (((1u << FS_TPW) - 1u) << (lane / FS_TPW * FS_TPW));
#define FS_WSYNC() __syncwarp(wmask)
#else
#define FS_WSYNC() __syncthreads()
#endif
#if FS_GLOBAL
        FT *P = a.paths + (size_t)w * FS_DOF * FS_N;
#else
        FT *P = s_path + wl * FS_WSTRIDE;
#endif
#if FS_VGLOBAL
        FT *Vc = a.vcache + (size_t)w * FS_N;
#else
        FT *Vc = s_v + wl * FS_VSTRIDE;
#endif
        const int tid = fs_thread_id(w, t);
        // sigma table (kernel.c:608-618), computed on the host with the same FP operations
        const FT *sigma = fs_sigma;

        // ---- RNG state ----
        FsUStream fs;
#if FS_RANLUX
        if (mover) {
            fs_rl_load(fs.st, a.rtab + (size_t)tid * 28);
            fs.count = 0u;
        }
        // The walker's offset stream: every reference work-item of the walker advances an
        // identical copy; here one lane advances it in shared memory for the walker.
        FsIStream &is = s_istream[wl];
        if (mover && t == 0) {
#if FS_COMPAT
            fs_rl_load(is.st, a.gtab + (size_t)tid * 28);
#else
            fs_rl_load(is.st, a.gtab + (size_t)w * 28);
#endif
            is.count = 0u;
#if FS_OFF_PRE
#pragma unroll 1
            for (int k = 0; k < FS_NSTEPS_LAUNCH; k++) s_offs[wl][k] = (unsigned char)fs_offset(is, FS_SEG);
#endif
        }
        FS_WSYNC();
#else
        FsIStream is;
        if (mover) {
            const uint4 s4 = *(const uint4 *)(a.seeds + (size_t)tid * 4);
            fs.x = s4.x; fs.y = s4.y; fs.z = s4.z; fs.w = s4.w;
#if FS_COMPAT
#if FS_PARALLEL
            const int row = (w / FS_WPG) + (w % FS_WPG) * FS_NWG;  // kernel.c:568
#else
            const int row = w;  // local size 1
#endif
            const uint4 g4 = *(const uint4 *)(a.seed_snap + (size_t)row * 4);
#else
            const uint4 g4 = *(const uint4 *)(a.walker_seeds + (size_t)w * 4);
#endif
            is.x = g4.x; is.y = g4.y; is.z = g4.z; is.w = g4.w;
        }
#endif
        fs_u32 n_acc = 0u;

#if FS_NOPS > 0
        FT opr[FS_NOPS];
        double opd[FS_NOPS];
        float opf[FS_NOPS], opks[FS_NOPS], opkc[FS_NOPS], opp[FS_NOPS];
#pragma unroll
        for (int i = 0; i < FS_NOPS; i++) {
            opr[i] = (FT)0; opd[i] = 0.0; opf[i] = 0.0f; opks[i] = 0.0f; opkc[i] = 0.0f; opp[i] = 0.0f;
        }
#endif
#if FS_NCOR > 0
        FsCorAcc *g_cor = (FsCorAcc *)a.cor_means + (size_t)w * FS_NCOR * FS_HALF_N;
        // FS_PIPE: two path snapshots ahead of the correlator values
        FT *const C = s_cor + wl * FS_CWSTRIDE + 2 * FS_SNSTRIDE;  // one measurement's values
#if FS_PIPE
        FT *const SN0 = s_cor + wl * FS_CWSTRIDE;
        FT *SN = SN0;  // the movers' next snapshot
#endif
#if FS_COR_REGS
        FsCorAcc cacc[FS_NCOR][FS_LPT];
#pragma unroll
        for (int c = 0; c < FS_NCOR; c++)
#pragma unroll
            for (int j = 0; j < FS_LPT; j++) {
                const int tau = FS_LAG(j);
                cacc[c][j] = lagger && tau < FS_HALF_N ? g_cor[c * FS_HALF_N + tau] : (FsCorAcc)0;
            }
#endif
#endif

#if FS_VCACHE
        // potential cache: V of each of the walker's slices at launch start
        {
#if FS_PARALLEL
            const int v_lo = t * FS_SEG, v_hi = (t + 1) * FS_SEG;
#else
            const int v_lo = 0, v_hi = FS_N;
#endif
#pragma unroll 1
            for (int s = v_lo; s < (mover ? v_hi : v_lo); s++) Vc[FS_VIDX(s)] = fs_pot(FS_ARGS_AT(P, s));
        }
        FS_WSYNC();
#endif

#if FS_NOPS > 0
        // the operators of slice s of path Q, added to this thread's sums
        auto fs_op_add = [&](const FT *Q, int s) {
            FT ov[FS_NOPS];
            fs_ops(FS_ARGS_AT(Q, s), ov);
#pragma unroll
            for (int i = 0; i < FS_NOPS; i++) {
#if FS_ACCUM == 0
                opr[i] = FS_ADD(opr[i], ov[i]);
#elif FS_OP_PART
                opp[i] = __fadd_rn(opp[i], (float)ov[i]);
#elif FS_ACCUM == 1
                opd[i] = __dadd_rn(opd[i], fs_f2d(ov[i]));
#elif FS_ACCUM == 2
                fs_kahan(opks[i], opkc[i], (float)ov[i]);
#else
                opf[i] = __fadd_rn(opf[i], (float)ov[i]);
                fs_kahan(opks[i], opkc[i], (float)ov[i]);
                opd[i] = __dadd_rn(opd[i], fs_f2d(ov[i]));
#endif
            }
        };
        // end of one measurement's operator values: the FP32 partials into the FP64 sums
        auto fs_op_flush = [&]() {
#if FS_OP_PART
#pragma unroll
            for (int i = 0; i < FS_NOPS; i++) {
                opd[i] = __dadd_rn(opd[i], fs_f2d(opp[i]));
                opp[i] = 0.0f;
            }
#endif
        };
#endif
#if FS_NCOR > 0
        // the correlator values of slice s of path Q into the measurement's buffer C
        auto fs_cor_put = [&](const FT *Q, int s) {
            FT cv[FS_NCOR];
            fs_cors(FS_ARGS_AT(Q, s), cv);
#pragma unroll
            for (int c = 0; c < FS_NCOR; c++) {
                C[c * FS_CSTRIDE + s] = cv[c];
#if FS_COR_ILV
                C[c * FS_CSTRIDE + s + FS_N] = cv[c];
#endif
            }
        };
#if !FS_PIPE
        // one measurement's lag sums of the slice values in Cm, added to the lags this thread
        // owns: tau = lt + j * FS_CTPW
        auto fs_cor_lags = [&](const FT *Cm) {
#pragma unroll
            for (int c = 0; c < FS_NCOR; c++) {
                const FT *Cc = Cm + c * FS_CSTRIDE;
#if FS_COR_ILV
                // every lag this thread owns in one pass over the slices: 2 x FS_LPT independent
                // float-float chains, and Cc[s1] loaded once for all lags.  Unrolled by 8 (HO,
                // N=128, 4 lags: 0.78 / 0.61 / 0.53 / 0.47 ms per launch for 1 / 2 / 4 / 8;
                // a full unroll, 0.81 ms, misses the instruction cache); by 2 in the study mode,
                // whose three sums per product make the loop body large (10-atom cluster: 2.08
                // against 1.80-1.87e9 node updates/s at 8).  Lags past N/2 (when
                // FS_CTPW does not divide N/2) are summed and dropped; s1 + tau < N + LPT * CTPW
                // <= 2N stays inside the doubled slice values.
#if FS_COR_FMA
                {
                    // four FMA chains per lag (slices s1 mod 4); the slice values s1..s1+3
                    // in one 16-byte load (Cc is 16-byte aligned: the host pads every
                    // stride to 64 bytes), shared by all lags of the thread
                    float pa[FS_LPT][4];
#pragma unroll
                    for (int j = 0; j < FS_LPT; j++)
#pragma unroll
                        for (int k = 0; k < 4; k++) pa[j][k] = 0.0f;
#if FS_N % 4 == 0
#pragma unroll 2
                    for (int s1 = 0; s1 < FS_N; s1 += 4) {
                        const float4 c4 = *reinterpret_cast<const float4 *>(Cc + s1);
#pragma unroll
                        for (int j = 0; j < FS_LPT; j++) {
                            const float *cj = Cc + s1 + lt + j * FS_CTPW;
                            pa[j][0] = __fmaf_rn(c4.x, cj[0], pa[j][0]);
                            pa[j][1] = __fmaf_rn(c4.y, cj[1], pa[j][1]);
                            pa[j][2] = __fmaf_rn(c4.z, cj[2], pa[j][2]);
                            pa[j][3] = __fmaf_rn(c4.w, cj[3], pa[j][3]);
                        }
                    }
#else
#pragma unroll
                    for (int s1 = 0; s1 < FS_N; s1++)
#pragma unroll
                        for (int j = 0; j < FS_LPT; j++)
                            pa[j][s1 & 3] = __fmaf_rn(Cc[s1], Cc[s1 + lt + j * FS_CTPW], pa[j][s1 & 3]);
#endif
#pragma unroll
                    for (int j = 0; j < FS_LPT; j++) {
                        const double m =
                            fs_f2d(__fadd_rn(__fadd_rn(pa[j][0], pa[j][1]), __fadd_rn(pa[j][2], pa[j][3])));
#if FS_COR_REGS
                        cacc[c][j] = __dadd_rn(cacc[c][j], m);
#else
                        const int tau = lt + j * FS_CTPW;
                        if (tau < FS_HALF_N) g_cor[c * FS_HALF_N + tau] = __dadd_rn(g_cor[c * FS_HALF_N + tau], m);
#endif
                    }
                }
#else
                {
                    float fs[FS_LPT], fe[FS_LPT];
#if FS_ACCUM == 3
                    float af[FS_LPT], aks[FS_LPT], akc[FS_LPT];
#endif
#pragma unroll
                    for (int j = 0; j < FS_LPT; j++) {
                        fs[j] = 0.0f;
                        fe[j] = 0.0f;
#if FS_ACCUM == 3
                        const int tau = lt + j * FS_CTPW;
                        const FsCorAcc a0 = tau < FS_HALF_N ? g_cor[c * FS_HALF_N + tau] : FsCorAcc{};
                        af[j] = a0.f; aks[j] = a0.ks; akc[j] = a0.kc;
#endif
                    }
#if FS_ACCUM == 3
#pragma unroll 2
#else
#pragma unroll 8
#endif
                    for (int s1 = 0; s1 < FS_N; s1++) {
                        const FT c0 = Cc[s1];
#pragma unroll
                        for (int j = 0; j < FS_LPT; j++) {
                            const FT q = FS_MUL(c0, Cc[s1 + lt + j * FS_CTPW]);
                            fs_ff_add(fs[j], fe[j], q);
#if FS_ACCUM == 3
                            af[j] = __fadd_rn(af[j], q);
                            fs_kahan(aks[j], akc[j], q);
#endif
                        }
                    }
#pragma unroll
                    for (int j = 0; j < FS_LPT; j++) {
                        const double m = __dadd_rn(fs_f2d(fs[j]), fs_f2d(fe[j]));
#if FS_COR_REGS
                        cacc[c][j] = __dadd_rn(cacc[c][j], m);
#else
                        const int tau = lt + j * FS_CTPW;
                        if (tau < FS_HALF_N) {
#if FS_ACCUM == 3
                            FsCorAcc *g = g_cor + c * FS_HALF_N + tau;
                            g->d = __dadd_rn(g->d, m);
                            g->f = af[j]; g->ks = aks[j]; g->kc = akc[j];
#else
                            g_cor[c * FS_HALF_N + tau] = __dadd_rn(g_cor[c * FS_HALF_N + tau], m);
#endif
                        }
#endif
                    }
                }
#endif  // FS_COR_FMA
#else
#if FS_COR_REGS
#pragma unroll
#else
#pragma unroll 1
#endif
                for (int j = 0; j < FS_LPT; j++) {
                    const int tau = lt + j * FS_CTPW;
                    if (tau >= FS_HALF_N) continue;
#if FS_COR_REGS
                    FsCorAcc acc = cacc[c][j];
#else
                    FsCorAcc acc = g_cor[c * FS_HALF_N + tau];
#endif
#if FS_COR_FMA
                    {
                        float p[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#if FS_N % 4 == 0
#pragma unroll 2
                        for (int s1 = 0; s1 < FS_N; s1 += 4)
#pragma unroll
                            for (int k = 0; k < 4; k++)
                                p[k] = __fmaf_rn(Cc[s1 + k], Cc[(s1 + k + tau) & (FS_N - 1)], p[k]);
#else
#pragma unroll
                        for (int s1 = 0; s1 < FS_N; s1++)
                            p[s1 & 3] = __fmaf_rn(Cc[s1], Cc[(s1 + tau) & (FS_N - 1)], p[s1 & 3]);
#endif
                        acc = __dadd_rn(acc, fs_f2d(__fadd_rn(__fadd_rn(p[0], p[1]), __fadd_rn(p[2], p[3]))));
                    }
#elif FS_COR_FF
                    {
                        float fs = 0.0f, fe = 0.0f;
#pragma unroll 4
                        for (int s1 = 0; s1 < FS_N; s1++) {
                            const FT q = FS_MUL(Cc[s1], Cc[(s1 + tau) & (FS_N - 1)]);
                            fs_ff_add(fs, fe, q);
#if FS_ACCUM == 3
                            acc.f = __fadd_rn(acc.f, q);
                            fs_kahan(acc.ks, acc.kc, q);
#endif
                        }
#if FS_ACCUM == 3
                        acc.d = __dadd_rn(acc.d, __dadd_rn(fs_f2d(fs), fs_f2d(fe)));
#else
                        acc = __dadd_rn(acc, __dadd_rn(fs_f2d(fs), fs_f2d(fe)));
#endif
                    }
#elif FS_ACCUM == 0 && FS_PARALLEL
                    // the reference's summation order (kernel.c:736-793)
#pragma unroll 1
                    for (int k = 0; k < FS_SEG; k++)
#pragma unroll 1
                        for (int cti = 0; cti < FS_HALF_N; cti++) {
                            const int tp = (tau - cti + FS_HALF_N) % FS_HALF_N;
                            if (tp >= FS_TPW) continue;
                            const int s1 = tp * FS_SEG + k;
                            acc = FS_ADD(acc, FS_MUL(Cc[s1], Cc[(s1 + tau) & (FS_N - 1)]));
                        }
#else
#if FS_ACCUM == 0
#pragma unroll 4
                    for (int s1 = 0; s1 < FS_N; s1++)
                        acc = FS_ADD(acc, FS_MUL(Cc[s1], Cc[(s1 + tau) & (FS_N - 1)]));
#else
                    // FP64 sums: four partial sums over s1 mod 4, combined at the end as
                    // (p0 + p1) + (p2 + p3), p0 starting from the running sum.  Four
                    // independent chains keep the FP64 pipe busy (a single chain of N
                    // dependent adds made the lag loop latency bound).
#if FS_ACCUM == 3
                    double p0 = acc.d, p1 = 0.0, p2 = 0.0, p3 = 0.0;
#else
                    double p0 = acc, p1 = 0.0, p2 = 0.0, p3 = 0.0;
#endif
#pragma unroll 2
                    for (int s1 = 0; s1 < FS_N; s1 += FS_CSTEP) {
                        const FT q0 = FS_MUL(Cc[s1], Cc[(s1 + tau) & (FS_N - 1)]);
                        p0 = __dadd_rn(p0, fs_f2d(q0));
#if FS_CSTEP == 4
                        const FT q1 = FS_MUL(Cc[s1 + 1], Cc[(s1 + 1 + tau) & (FS_N - 1)]);
                        const FT q2 = FS_MUL(Cc[s1 + 2], Cc[(s1 + 2 + tau) & (FS_N - 1)]);
                        const FT q3 = FS_MUL(Cc[s1 + 3], Cc[(s1 + 3 + tau) & (FS_N - 1)]);
                        p1 = __dadd_rn(p1, fs_f2d(q1));
                        p2 = __dadd_rn(p2, fs_f2d(q2));
                        p3 = __dadd_rn(p3, fs_f2d(q3));
#endif
#if FS_ACCUM == 3
                        // the study's FP32 columns: the same products in slice order
                        acc.f = __fadd_rn(acc.f, (float)q0);
                        fs_kahan(acc.ks, acc.kc, (float)q0);
#if FS_CSTEP == 4
                        acc.f = __fadd_rn(acc.f, (float)q1);
                        fs_kahan(acc.ks, acc.kc, (float)q1);
                        acc.f = __fadd_rn(acc.f, (float)q2);
                        fs_kahan(acc.ks, acc.kc, (float)q2);
                        acc.f = __fadd_rn(acc.f, (float)q3);
                        fs_kahan(acc.ks, acc.kc, (float)q3);
#endif
#endif
                    }
#if FS_ACCUM == 3
                    acc.d = __dadd_rn(__dadd_rn(p0, p1), __dadd_rn(p2, p3));
#else
                    acc = __dadd_rn(__dadd_rn(p0, p1), __dadd_rn(p2, p3));
#endif
#endif
#endif
#if FS_COR_REGS
                    cacc[c][j] = acc;
#else
                    g_cor[c * FS_HALF_N + tau] = acc;
#endif
                }
#endif
            }
        };
#else
        // pipelined helpers: helper lane lt < N/8 sums lags 4 lt .. 4 lt + 3 of one
        // measurement with the same four chains per lag (slices s1 mod 4, in slice order) and
        // the same pairwise combination as the lag sums above, so the same bits; the slice
        // values s1..s1+3 and the window s1 + 4 lt .. s1 + 4 lt + 7 come in 16-byte loads (2
        // per 16 products), the window's upper half carried to the next step.  Reads stop at
        // slice 4 lt + N + 3 < 3N/2 of the doubled values.
        auto fs_cor_lags4 = [&](const FT *Cm) {
            if (!(lt < FS_N / 8)) return;
#pragma unroll
            for (int c = 0; c < FS_NCOR; c++) {
                const float4 *cv4 = reinterpret_cast<const float4 *>(Cm + c * FS_CSTRIDE);
                const float4 *wv4 = cv4 + lt;
                float pa[4][4];
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int k = 0; k < 4; k++) pa[j][k] = 0.0f;
                float4 w0 = wv4[0];
#pragma unroll 16
                for (int q = 0; q < FS_N / 4; q++) {
                    const float4 a4 = cv4[q];
                    const float4 w1 = wv4[q + 1];
                    const float av[4] = {a4.x, a4.y, a4.z, a4.w};
                    const float wv[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
                    for (int j = 0; j < 4; j++)
#pragma unroll
                        for (int k = 0; k < 4; k++) pa[j][k] = __fmaf_rn(av[k], wv[k + j], pa[j][k]);
                    w0 = w1;
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const double m =
                        fs_f2d(__fadd_rn(__fadd_rn(pa[j][0], pa[j][1]), __fadd_rn(pa[j][2], pa[j][3])));
#if FS_COR_REGS
                    cacc[c][j] = __dadd_rn(cacc[c][j], m);
#else
                    g_cor[c * FS_HALF_N + FS_LAG(j)] = __dadd_rn(g_cor[c * FS_HALF_N + FS_LAG(j)], m);
#endif
                }
            }
        };
#endif
#endif

        // ---- sweeps (kernel.c:628-799) ----
#if FS_PIPE
        if (!mover) {
            // helpers: measurement run on its snapshot while the movers sweep towards the
            // next one
#pragma unroll 1
            for (int run = 0; run < FS_OPRUNS; run++) {
                __syncthreads();
                const FT *Q = SN0 + (run & 1) * FS_SNSTRIDE;
#pragma unroll 1
                for (int s = lt; s < FS_N; s += FS_CTPW) fs_cor_put(Q, s);
                asm volatile("bar.sync 2, %0;" ::"n"(FS_BLOCK - FS_MBLOCK) : "memory");
                fs_cor_lags4(C);
            }
        } else
#endif
        {
#pragma unroll 1
        for (int run = 0; run < FS_OPRUNS; run++) {
#pragma unroll 1
            for (int step = 0; step < FS_MSTEPS; step++) {
#if !FS_PARALLEL && (FS_PATH_SHIFT || FS_SNM)
                {
                    // walker-mode moves ahead of the bisection (kernel.c:640-705).  The
                    // reference's step counter i*mSteps + j restarts every launch; the fixed
                    // mode continues it across launches.
#if FS_COMPAT
                    const unsigned long long k = (unsigned long long)run * FS_MSTEPS + step;
#else
                    const unsigned long long k = a.step_base + (unsigned long long)run * FS_MSTEPS + step;
#endif
#if FS_PATH_SHIFT
                    n_acc += (fs_u32)fs_path_shift_move(P, k, is, fs, a.shift_old + (size_t)w * FS_N);
#endif
#if FS_SNM
                    n_acc += (fs_u32)fs_single_node_move(P, k, fs);
#endif
                }
#endif
#if FS_BISECT
#if FS_RANLUX
#if FS_OFF_PRE
                const fs_u32 off = s_offs[wl][run * FS_MSTEPS + step];
#else
                if (mover && t == 0) s_off[wl] = fs_offset(is, FS_PARALLEL ? FS_SEG : FS_N);
                FS_WSYNC();
                const fs_u32 off = s_off[wl];
#endif
#else
                const fs_u32 off = mover ? fs_offset(is, FS_PARALLEL ? FS_SEG : FS_N) : 0u;
#endif
#if FS_PARALLEL
                const fs_u32 start = (off + (fs_u32)(FS_SEG * t)) & (FS_N - 1);
#else
                const fs_u32 start = off;
#endif
#if FS_LEARNED
                // level-1 proposal from the segment's endpoints (warp-wide network evaluation)
                FT lmu[FS_DOF], lsd[FS_DOF];
                {
                    float feat[FS_MLP_IN], out[FS_MLP_OUT];
#pragma unroll
                    for (int k = 0; k < FS_MLP_IN; k++) feat[k] = 0.f;
                    const fs_u32 e1 = (start + FS_SEG) & (FS_N - 1);
#pragma unroll
                    for (int d = 0; d < FS_DOF; d++) {
                        const FT x0 = FS_AT(P, d, start), x1 = FS_AT(P, d, e1);
                        feat[d] = 0.5f * (x0 + x1) * a.mlp_inv_scale;
                        feat[FS_DOF + d] = 0.5f * (x1 - x0) * a.mlp_inv_scale;
                    }
                    fs_mlp_eval_warp(a.mlp_frag, a.mlp_bias, feat, out);
                    const FT s1 = sigma[1];
#pragma unroll
                    for (int d = 0; d < FS_DOF; d++) {
                        const FT mid = 0.5f * (FS_AT(P, d, start) + FS_AT(P, d, e1));
                        float o = out[d], sv = 4.f * tanhf(0.25f * out[FS_DOF + d]);
                        if (!(fabsf(o) < 64.f) || !(fabsf(sv) <= 4.f)) {  // non-finite: free proposal
                            o = 0.f;
                            sv = 0.f;
                        }
                        lmu[d] = mid + s1 * o;
                        lsd[d] = s1 * __expf(0.5f * sv);
                    }
                }
                n_acc += (fs_u32)fs_bisect(P, Vc, start, fs, sigma, lmu, lsd);
#else
                if (mover) n_acc += (fs_u32)fs_bisect(P, Vc, start, fs, sigma, nullptr, nullptr);
#endif
#endif  // FS_BISECT
                FS_WSYNC();
            }
            // ---- measurement (kernel.c:734-797) ----
#if FS_PARALLEL
            const int s_lo = t * FS_SEG, s_hi = (t + 1) * FS_SEG;
#else
            const int s_lo = 0, s_hi = FS_N;
#endif
#pragma unroll 1
            for (int s = s_lo; s < (mover ? s_hi : s_lo); s++) {
#if FS_NOPS > 0
                fs_op_add(P, s);
#endif
#if FS_PIPE
#pragma unroll
                for (int d = 0; d < FS_DOF; d++) FS_AT(SN, d, s) = FS_AT(P, d, s);
#elif FS_NCOR > 0
                fs_cor_put(P, s);
#endif
#if FS_BINS
                {
                    int ok = 1, inc = 1, bi = 0;
#pragma unroll
                    for (int d = 0; d < FS_DOF; d++) {
                        const FT x = FS_AT(P, d, s);
                        if (x < (FT)FS_XMIN || x >= (FT)FS_XMAX) ok = 0;
                        bi += (int)((fs_u32)FS_MUL(FS_SUB(x, (FT)FS_XMIN), (FT)FS_INVBIN)) * inc;
                        inc *= FS_BINRES;
                    }
                    if (ok) atomicAdd(a.bins + bi, 1u);
                }
#endif
#if FS_NHIST > 0
                {
                    FT hv[FS_NHIST];
                    fs_hist(FS_ARGS_AT(P, s), hv);
#pragma unroll
                    for (int h = 0; h < FS_NHIST; h++) {
                        const FT x = hv[h];
                        if (x >= (FT)FS_HLO && x < (FT)FS_HHI) {
                            const int b = (int)FS_MUL(FS_SUB(x, (FT)FS_HLO), (FT)FS_HINVW);
                            if (b >= 0 && b < FS_HBINS) atomicAdd(s_hist + b, 1u);
                        }
                    }
                }
#endif
            }
#if FS_NOPS > 0
            if (mover) fs_op_flush();
#endif
#if FS_PIPE
            __syncthreads();  // the snapshot goes to the helper threads
            SN = SN == SN0 ? SN0 + FS_SNSTRIDE : SN0;
#elif FS_NCOR > 0
            FS_WSYNC();
            fs_cor_lags(C);
#endif
            FS_WSYNC();
        }
        }

        // ---- epilogue (kernel.c:801-836) ----
        if (mover) a.accepts[tid] = n_acc;
#if FS_NOPS > 0
#pragma unroll
        for (int i = 0; i < (mover ? FS_NOPS : 0); i++) {
            const size_t o = (size_t)tid * FS_NOPS + i;
#if FS_ACCUM == 0
            ((FT *)a.op_means)[o] = FS_MUL(opr[i], (FT)FS_OPNORM);
#elif FS_ACCUM == 1
            ((double *)a.op_means)[o] = __dmul_rn(opd[i], a.opnorm);
#elif FS_ACCUM == 2
            ((float *)a.op_means)[o] = __fmul_rn(opks[i], (float)FS_OPNORM);
#else
            ((double *)a.op_means)[3 * o + 0] = (double)__fmul_rn(opf[i], (float)FS_OPNORM);
            ((double *)a.op_means)[3 * o + 1] = (double)__fmul_rn(opks[i], (float)FS_OPNORM);
            ((double *)a.op_means)[3 * o + 2] = __dmul_rn(opd[i], a.opnorm);
#endif
        }
#endif
#if FS_NCOR > 0 && FS_COR_REGS
#pragma unroll
        for (int c = 0; c < FS_NCOR; c++)
#pragma unroll
            for (int j = 0; j < FS_LPT; j++) {
                const int tau = FS_LAG(j);
                if (lagger && tau < FS_HALF_N) g_cor[c * FS_HALF_N + tau] = cacc[c][j];
            }
#endif
#if FS_GLOBAL
        {
            // the walker's slices this thread owns, checked in place (the shared-memory
            // mode checks every value in its path-out copy instead)
#if FS_PARALLEL
            const int c_lo = t * FS_SEG, c_hi = (t + 1) * FS_SEG;
#else
            const int c_lo = 0, c_hi = FS_N;
#endif
            bool bad = false;
#pragma unroll 1
            for (int s = c_lo; s < c_hi; s++)
#pragma unroll
                for (int d = 0; d < FS_DOF; d++) bad |= !isfinite(FS_AT(P, d, s));
            if (bad) fs_flag_nonfinite(a.status, w);
        }
#endif
#if FS_RANLUX
        if (mover) fs_rl_store(fs.st, a.rtab + (size_t)tid * 28);
        FS_WSYNC();
#if FS_COMPAT
        if (mover) fs_rl_store(is.st, a.gtab + (size_t)tid * 28);
#else
        if (mover && t == 0) fs_rl_store(is.st, a.gtab + (size_t)w * 28);
#endif
#else
        if (mover) *(uint4 *)(a.seeds + (size_t)tid * 4) = make_uint4(fs.x, fs.y, fs.z, fs.w);
#if !FS_COMPAT
        if (mover && t == 0) *(uint4 *)(a.walker_seeds + (size_t)w * 4) = make_uint4(is.x, is.y, is.z, is.w);
#endif
#endif
#undef FS_WSYNC
    }
    __syncthreads();

    // ---- path out (coalesced global writes) ----
    {
#if !FS_GLOBAL
        const size_t base = (size_t)w0 * FS_DOF * FS_N;
        const int count = n_here * FS_DOF * FS_N;
#if FS_VEC > 1
        FsVec *dstv = (FsVec *)(a.paths + base);
        for (int i4 = tid_b; i4 < count / FS_VEC; i4 += FS_BLOCK) {
            const int i = i4 * FS_VEC;
            const int wi = i / (FS_DOF * FS_N), r = i - wi * (FS_DOF * FS_N);
            const int d = r / FS_N, sl = r - d * FS_N;
            const FsVec v = fs_vec_gather(&FS_AT(s_path + wi * FS_WSTRIDE, d, sl));
            dstv[i4] = v;
            if (!fs_vec_finite(v)) fs_flag_nonfinite(a.status, w0 + wi);
        }
#else
        for (int i = tid_b; i < count; i += FS_BLOCK) {
            const int wi = i / (FS_DOF * FS_N), r = i - wi * (FS_DOF * FS_N);
            const int d = r / FS_N, sl = r - d * FS_N;
            const FT v = FS_AT(s_path + wi * FS_WSTRIDE, d, sl);
            a.paths[base + i] = v;
            if (!isfinite(v)) fs_flag_nonfinite(a.status, w0 + wi);
        }
#endif
#endif
#if FS_NHIST > 0
        for (int i = tid_b; i < FS_HBINS; i += FS_BLOCK)
            if (s_hist[i]) atomicAdd(a.hist + i, (fs_u64)s_hist[i]);
#endif
    }
}
#endif  // FS_RNG_ONLY

// RANLUX state-table seeding: row i from the 64-bit value xs[i] (ranluxcl_init)
extern "C" __global__ void fs_ranlux_init(fs_u32 *tab, const fs_u64 *xs, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    FsRanlux r;
    fs_rl_seed(r, xs[i]);
    fs_rl_store(r, tab + (size_t)i * 28);
}

// stream dumps used by the RNG parity tests
extern "C" __global__ void fs_ranlux_dump(const fs_u64 *xs, int n, int n_calls, float *out, fs_u32 *states)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    FsRanlux r;
    fs_rl_seed(r, xs[i]);
#pragma unroll 1
    for (int c = 0; c < n_calls; c++) {
        float o0, o1, o2, o3;
        fs_rl_next4<FS_NSKIP>(r, o0, o1, o2, o3);
        float *o = out + ((size_t)i * n_calls + c) * 4;
        o[0] = o0; o[1] = o1; o[2] = o2; o[3] = o3;
    }
    fs_rl_store(r, states + (size_t)i * 28);
}

extern "C" __global__ void fs_ranlux_dump64(const fs_u64 *xs, int n, int n_calls, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    FsRanluxStream64<FS_NSKIP> g;
    fs_rl_seed(g.st, xs[i]);
    g.count = 0u;
#pragma unroll 1
    for (int c = 0; c < 4 * n_calls; c++) out[(size_t)i * 4 * n_calls + c] = g.next();
}

extern "C" __global__ void fs_xorshift_dump(fs_u32 *states, int n, int n_draws, fs_u32 *out, float *fout)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    FsXorshift s;
    s.x = states[4 * i]; s.y = states[4 * i + 1]; s.z = states[4 * i + 2]; s.w = states[4 * i + 3];
#pragma unroll 1
    for (int k = 0; k < n_draws; k++) {
        FsXorshift c = s;
        fout[(size_t)i * n_draws + k] = fs_xs_float(c);
        out[(size_t)i * n_draws + k] = fs_xs_next(s);
    }
    states[4 * i] = s.x; states[4 * i + 1] = s.y; states[4 * i + 2] = s.z; states[4 * i + 3] = s.w;
}
