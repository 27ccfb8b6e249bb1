// fs_rng.cuh -- device random number generators, bit-identical to the reference's.
//
// Included into every NVRTC module built by fs_api.cu (kept free of host headers).
//
//  * xorshift128 exactly as FeynSimul/GPUsrc/kernel.c:214-239: float = float(w) * 2^-32
//    (the constant 2.328306437080797e-10 is 2^-32 once rounded to FP32, which is what the
//    reference's -cl-single-precision-constant build uses).
//  * RANLUX in the RANLUXCL v1.3.1 formulation the reference vendors
//    (examples/pyopencl-ranluxcl.cl): subtract-with-borrow on 24 lags with the p-skip
//    schedule, xorshift64 seeding and 32-cycle warm-up.  The lags are multiples of 2^-24 in
//    [0, 1), so this file keeps them as integers (k << 8 for value k * 2^-24) and runs the
//    subtract-with-borrow as a hardware borrow chain (see FsRanlux); the results are
//    identical because every float operation of the reference on these values is exact.
//    Output floats are formed exactly as the reference forms them (small values get the
//    next lag's bits, zero maps to 2^-48).
//  * State tables in global memory keep the reference's 28-word float layout
//    (pyopencl-ranluxcl.cl:264-277), converted on load and store.
#pragma once

typedef unsigned int fs_u32;
typedef unsigned long long fs_u64;

// ---------------------------------------------------------------- xorshift128
struct FsXorshift {
    fs_u32 x, y, z, w;
};

__device__ __forceinline__ fs_u32 fs_xs_next(FsXorshift &s)
{
    fs_u32 t = s.x ^ (s.x << 11);
    s.x = s.y;
    s.y = s.z;
    s.z = s.w;
    s.w = s.w ^ (s.w >> 19) ^ (t ^ (t >> 8));
    return s.w;
}

__device__ __forceinline__ float fs_xs_float(FsXorshift &s)
{
    return __fmul_rn(__uint2float_rn(fs_xs_next(s)), 0x1p-32f);
}

__device__ __forceinline__ double fs_xs_double(FsXorshift &s)
{
    // ENABLE_DOUBLE build of kernel.c:229: double(w) * 2.328306437080797e-10 in FP64
    return __dmul_rn((double)fs_xs_next(s), 2.328306437080797e-10);
}

// ---------------------------------------------------------------- RANLUX
// Lag value k (0 <= k < 2^24, value k * 2^-24) is held as k << 8.  Then one
// subtract-with-borrow step s_a = s_j - s_a - c is a single `subc.cc.u32` on the shifted
// words: the hardware borrow-out equals the digit borrow (the low bytes are zero) and the
// top 24 bits of the difference are the new digit; an `and` clears the low byte.  Steps are
// chained through the carry flag inside one asm block, so a step costs two instructions and
// its critical path is one.  The borrow enters the chain as `0 - c` and leaves it as
// `0 - 0 - borrow` (so c is 0 or 0xFFFFFFFF), i.e. only through subtractions, whichever
// polarity the flag has.
struct FsRanlux {
    fs_u32 s[24];   // k << 8; s[0] is the reference's s01
    fs_u32 carry;   // 0 or 0xFFFFFFFF (the reference stores 0 or 2^-24)
    fs_u32 in24;
    fs_u32 stepnr;
    fs_u32 dummy;   // padding word of the table, carried through unchanged
};

// cycle position p updates lag a = 23 - p from lag (a + 10) % 24.  A chunk names only the
// eight lag words it reads or writes (the 24-step cycle needs all of them).
__device__ __forceinline__ void fs_rl_chunk4_p0(FsRanlux &r)
{
    asm("{\n\t.reg .u32 fsz;\n\tmov.u32 fsz, 0;\n\t" "sub.cc.u32 fsz, fsz, %4;\n\t"
        "subc.cc.u32 %0, %5, %0;\n\t" "and.b32 %0, %0, -256;\n\t"
        "subc.cc.u32 %1, %6, %1;\n\t" "and.b32 %1, %1, -256;\n\t"
        "subc.cc.u32 %2, %7, %2;\n\t" "and.b32 %2, %2, -256;\n\t"
        "subc.cc.u32 %3, %8, %3;\n\t" "and.b32 %3, %3, -256;\n\t"
        "mov.u32 fsz, 0;\n\t" "subc.u32 %4, fsz, fsz;\n\t" "}"
        : "+r"(r.s[23]), "+r"(r.s[22]), "+r"(r.s[21]), "+r"(r.s[20]), "+r"(r.carry)
        : "r"(r.s[9]), "r"(r.s[8]), "r"(r.s[7]), "r"(r.s[6]));
}

__device__ __forceinline__ void fs_rl_chunk4_p4(FsRanlux &r)
{
    asm("{\n\t.reg .u32 fsz;\n\tmov.u32 fsz, 0;\n\t" "sub.cc.u32 fsz, fsz, %4;\n\t"
        "subc.cc.u32 %0, %5, %0;\n\t" "and.b32 %0, %0, -256;\n\t"
        "subc.cc.u32 %1, %6, %1;\n\t" "and.b32 %1, %1, -256;\n\t"
        "subc.cc.u32 %2, %7, %2;\n\t" "and.b32 %2, %2, -256;\n\t"
        "subc.cc.u32 %3, %8, %3;\n\t" "and.b32 %3, %3, -256;\n\t"
        "mov.u32 fsz, 0;\n\t" "subc.u32 %4, fsz, fsz;\n\t" "}"
        : "+r"(r.s[19]), "+r"(r.s[18]), "+r"(r.s[17]), "+r"(r.s[16]), "+r"(r.carry)
        : "r"(r.s[5]), "r"(r.s[4]), "r"(r.s[3]), "r"(r.s[2]));
}

__device__ __forceinline__ void fs_rl_chunk4_p8(FsRanlux &r)
{
    asm("{\n\t.reg .u32 fsz;\n\tmov.u32 fsz, 0;\n\t" "sub.cc.u32 fsz, fsz, %4;\n\t"
        "subc.cc.u32 %0, %5, %0;\n\t" "and.b32 %0, %0, -256;\n\t"
        "subc.cc.u32 %1, %6, %1;\n\t" "and.b32 %1, %1, -256;\n\t"
        "subc.cc.u32 %2, %7, %2;\n\t" "and.b32 %2, %2, -256;\n\t"
        "subc.cc.u32 %3, %8, %3;\n\t" "and.b32 %3, %3, -256;\n\t"
        "mov.u32 fsz, 0;\n\t" "subc.u32 %4, fsz, fsz;\n\t" "}"
        : "+r"(r.s[15]), "+r"(r.s[14]), "+r"(r.s[13]), "+r"(r.s[12]), "+r"(r.carry)
        : "r"(r.s[1]), "r"(r.s[0]), "r"(r.s[23]), "r"(r.s[22]));
}

__device__ __forceinline__ void fs_rl_chunk4_p12(FsRanlux &r)
{
    asm("{\n\t.reg .u32 fsz;\n\tmov.u32 fsz, 0;\n\t" "sub.cc.u32 fsz, fsz, %4;\n\t"
        "subc.cc.u32 %0, %5, %0;\n\t" "and.b32 %0, %0, -256;\n\t"
        "subc.cc.u32 %1, %6, %1;\n\t" "and.b32 %1, %1, -256;\n\t"
        "subc.cc.u32 %2, %7, %2;\n\t" "and.b32 %2, %2, -256;\n\t"
        "subc.cc.u32 %3, %8, %3;\n\t" "and.b32 %3, %3, -256;\n\t"
        "mov.u32 fsz, 0;\n\t" "subc.u32 %4, fsz, fsz;\n\t" "}"
        : "+r"(r.s[11]), "+r"(r.s[10]), "+r"(r.s[9]), "+r"(r.s[8]), "+r"(r.carry)
        : "r"(r.s[21]), "r"(r.s[20]), "r"(r.s[19]), "r"(r.s[18]));
}

__device__ __forceinline__ void fs_rl_chunk4_p16(FsRanlux &r)
{
    asm("{\n\t.reg .u32 fsz;\n\tmov.u32 fsz, 0;\n\t" "sub.cc.u32 fsz, fsz, %4;\n\t"
        "subc.cc.u32 %0, %5, %0;\n\t" "and.b32 %0, %0, -256;\n\t"
        "subc.cc.u32 %1, %6, %1;\n\t" "and.b32 %1, %1, -256;\n\t"
        "subc.cc.u32 %2, %7, %2;\n\t" "and.b32 %2, %2, -256;\n\t"
        "subc.cc.u32 %3, %8, %3;\n\t" "and.b32 %3, %3, -256;\n\t"
        "mov.u32 fsz, 0;\n\t" "subc.u32 %4, fsz, fsz;\n\t" "}"
        : "+r"(r.s[7]), "+r"(r.s[6]), "+r"(r.s[5]), "+r"(r.s[4]), "+r"(r.carry)
        : "r"(r.s[17]), "r"(r.s[16]), "r"(r.s[15]), "r"(r.s[14]));
}

__device__ __forceinline__ void fs_rl_chunk4_p20(FsRanlux &r)
{
    asm("{\n\t.reg .u32 fsz;\n\tmov.u32 fsz, 0;\n\t" "sub.cc.u32 fsz, fsz, %4;\n\t"
        "subc.cc.u32 %0, %5, %0;\n\t" "and.b32 %0, %0, -256;\n\t"
        "subc.cc.u32 %1, %6, %1;\n\t" "and.b32 %1, %1, -256;\n\t"
        "subc.cc.u32 %2, %7, %2;\n\t" "and.b32 %2, %2, -256;\n\t"
        "subc.cc.u32 %3, %8, %3;\n\t" "and.b32 %3, %3, -256;\n\t"
        "mov.u32 fsz, 0;\n\t" "subc.u32 %4, fsz, fsz;\n\t" "}"
        : "+r"(r.s[3]), "+r"(r.s[2]), "+r"(r.s[1]), "+r"(r.s[0]), "+r"(r.carry)
        : "r"(r.s[13]), "r"(r.s[12]), "r"(r.s[11]), "r"(r.s[10]));
}

__device__ __forceinline__ void fs_rl_cycle(FsRanlux &r)
{
    asm("{\n\t.reg .u32 fsz;\n\tmov.u32 fsz, 0;\n\t" "sub.cc.u32 fsz, fsz, %24;\n\t"
        "subc.cc.u32 %23, %9, %23;\n\t" "and.b32 %23, %23, -256;\n\t"
        "subc.cc.u32 %22, %8, %22;\n\t" "and.b32 %22, %22, -256;\n\t"
        "subc.cc.u32 %21, %7, %21;\n\t" "and.b32 %21, %21, -256;\n\t"
        "subc.cc.u32 %20, %6, %20;\n\t" "and.b32 %20, %20, -256;\n\t"
        "subc.cc.u32 %19, %5, %19;\n\t" "and.b32 %19, %19, -256;\n\t"
        "subc.cc.u32 %18, %4, %18;\n\t" "and.b32 %18, %18, -256;\n\t"
        "subc.cc.u32 %17, %3, %17;\n\t" "and.b32 %17, %17, -256;\n\t"
        "subc.cc.u32 %16, %2, %16;\n\t" "and.b32 %16, %16, -256;\n\t"
        "subc.cc.u32 %15, %1, %15;\n\t" "and.b32 %15, %15, -256;\n\t"
        "subc.cc.u32 %14, %0, %14;\n\t" "and.b32 %14, %14, -256;\n\t"
        "subc.cc.u32 %13, %23, %13;\n\t" "and.b32 %13, %13, -256;\n\t"
        "subc.cc.u32 %12, %22, %12;\n\t" "and.b32 %12, %12, -256;\n\t"
        "subc.cc.u32 %11, %21, %11;\n\t" "and.b32 %11, %11, -256;\n\t"
        "subc.cc.u32 %10, %20, %10;\n\t" "and.b32 %10, %10, -256;\n\t"
        "subc.cc.u32 %9, %19, %9;\n\t" "and.b32 %9, %9, -256;\n\t"
        "subc.cc.u32 %8, %18, %8;\n\t" "and.b32 %8, %8, -256;\n\t"
        "subc.cc.u32 %7, %17, %7;\n\t" "and.b32 %7, %7, -256;\n\t"
        "subc.cc.u32 %6, %16, %6;\n\t" "and.b32 %6, %6, -256;\n\t"
        "subc.cc.u32 %5, %15, %5;\n\t" "and.b32 %5, %5, -256;\n\t"
        "subc.cc.u32 %4, %14, %4;\n\t" "and.b32 %4, %4, -256;\n\t"
        "subc.cc.u32 %3, %13, %3;\n\t" "and.b32 %3, %3, -256;\n\t"
        "subc.cc.u32 %2, %12, %2;\n\t" "and.b32 %2, %2, -256;\n\t"
        "subc.cc.u32 %1, %11, %1;\n\t" "and.b32 %1, %1, -256;\n\t"
        "subc.cc.u32 %0, %10, %0;\n\t" "and.b32 %0, %0, -256;\n\t"
        "mov.u32 fsz, 0;\n\t" "subc.u32 %24, fsz, fsz;\n\t" "}"
        : "+r"(r.s[0]), "+r"(r.s[1]), "+r"(r.s[2]), "+r"(r.s[3]), "+r"(r.s[4]), "+r"(r.s[5]), "+r"(r.s[6]), "+r"(r.s[7]), "+r"(r.s[8]), "+r"(r.s[9]), "+r"(r.s[10]), "+r"(r.s[11]), "+r"(r.s[12]), "+r"(r.s[13]), "+r"(r.s[14]), "+r"(r.s[15]), "+r"(r.s[16]), "+r"(r.s[17]), "+r"(r.s[18]), "+r"(r.s[19]), "+r"(r.s[20]), "+r"(r.s[21]), "+r"(r.s[22]), "+r"(r.s[23]), "+r"(r.carry));
}

// output of the step that just updated lag A (pyopencl-ranluxcl.cl:363-378)
template <int A>
__device__ __forceinline__ float fs_rl_value(const FsRanlux &r)
{
    const fs_u32 v = r.s[A];
    const float hi = __fmul_rn(__uint2float_rn(v), 0x1p-32f);
    const float lo = __fmul_rn(__uint2float_rn(r.s[(A + 9) % 24]), 0x1p-56f);
    float out = v < (4096u << 8) ? __fadd_rn(hi, lo) : hi;
    return out == 0.0f ? 0x1p-48f : out;
}

// NSKIP steps starting at cycle position pos (a multiple of 4); returns the new position
template <int NSKIP>
__device__ __forceinline__ fs_u32 fs_rl_skip(FsRanlux &r, fs_u32 pos)
{
    if (NSKIP == 0) return pos;
    // up to the cycle boundary (falls through on purpose)
    switch (pos) {
    case 4: fs_rl_chunk4_p4(r);
    case 8: fs_rl_chunk4_p8(r);
    case 12: fs_rl_chunk4_p12(r);
    case 16: fs_rl_chunk4_p16(r);
    case 20: fs_rl_chunk4_p20(r);
    default: break;
    }
    const int initial = pos ? 24 - (int)pos : 0;
    const int bulk = (NSKIP - initial) / 24;
    const int rem = NSKIP - initial - bulk * 24;
#pragma unroll 1
    for (int i = 0; i < bulk; i++) fs_rl_cycle(r);
    if (rem > 0) fs_rl_chunk4_p0(r);
    if (rem > 4) fs_rl_chunk4_p4(r);
    if (rem > 8) fs_rl_chunk4_p8(r);
    if (rem > 12) fs_rl_chunk4_p12(r);
    if (rem > 16) fs_rl_chunk4_p16(r);
    return (fs_u32)rem;
}

// Four outputs: the plain conversion, and the small-value correction of fs_rl_value only
// when some lane of the warp drew a value below 2^-12 (probability 2^-12 per value).
#define FS_RL_OUT4(P)                                                                      \
    fs_rl_chunk4_p##P(r);                                                                  \
    o0 = __fmul_rn(__uint2float_rn(r.s[23 - P]), 0x1p-32f);                                \
    o1 = __fmul_rn(__uint2float_rn(r.s[22 - P]), 0x1p-32f);                                \
    o2 = __fmul_rn(__uint2float_rn(r.s[21 - P]), 0x1p-32f);                                \
    o3 = __fmul_rn(__uint2float_rn(r.s[20 - P]), 0x1p-32f);                                \
    if (__any_sync(__activemask(),                                                         \
                   min(min(r.s[23 - P], r.s[22 - P]), min(r.s[21 - P], r.s[20 - P])) < (4096u << 8))) { \
        o0 = fs_rl_value<23 - P>(r);                                                       \
        o1 = fs_rl_value<22 - P>(r);                                                       \
        o2 = fs_rl_value<21 - P>(r);                                                       \
        o3 = fs_rl_value<20 - P>(r);                                                       \
    }

// four outputs (ranluxcl32), then the skip after every 24 outputs
template <int NSKIP>
__device__ __forceinline__ void fs_rl_next4(FsRanlux &r, float &o0, float &o1, float &o2, float &o3)
{
    switch (r.stepnr) {
    case 0: FS_RL_OUT4(0) break;
    case 4: FS_RL_OUT4(4) break;
    case 8: FS_RL_OUT4(8) break;
    case 12: FS_RL_OUT4(12) break;
    case 16: FS_RL_OUT4(16) break;
    default: FS_RL_OUT4(20) break;
    }
    fs_u32 pos = r.stepnr + 4u;
    if (NSKIP % 24 == 0) {
        // planar scheme: skip whenever a cycle completes; in24 stays untouched
        if (pos == 24u) pos = fs_rl_skip<NSKIP>(r, 0u);
        r.stepnr = pos;
    } else {
        r.stepnr = pos == 24u ? 0u : pos;
        r.in24 += 4u;
        if (r.in24 == 24u) {
            r.in24 = 0u;
            r.stepnr = fs_rl_skip<NSKIP>(r, r.stepnr);
        }
    }
}

// ranluxcl_init: three xorshift64 words give eight 24-bit lags, three times; 32 cycles
// of warm-up (pyopencl-ranluxcl.cl:597-725)
__device__ __forceinline__ void fs_rl_seed(FsRanlux &r, fs_u64 x)
{
#pragma unroll
    for (int b = 0; b < 3; b++) {
        fs_u64 w[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            w[k] = x;
        }
        // 192 bits w0|w1|w2, most significant first, in chunks of 24
        r.s[b * 8 + 0] = (fs_u32)(w[0] >> 40) << 8;
        r.s[b * 8 + 1] = ((fs_u32)(w[0] >> 16) & 0xFFFFFFu) << 8;
        r.s[b * 8 + 2] = (((fs_u32)(w[0] & 0xFFFFu) << 8) | (fs_u32)(w[1] >> 56)) << 8;
        r.s[b * 8 + 3] = ((fs_u32)(w[1] >> 32) & 0xFFFFFFu) << 8;
        r.s[b * 8 + 4] = ((fs_u32)(w[1] >> 8) & 0xFFFFFFu) << 8;
        r.s[b * 8 + 5] = (((fs_u32)(w[1] & 0xFFu) << 16) | (fs_u32)(w[2] >> 48)) << 8;
        r.s[b * 8 + 6] = ((fs_u32)(w[2] >> 24) & 0xFFFFFFu) << 8;
        r.s[b * 8 + 7] = ((fs_u32)w[2] & 0xFFFFFFu) << 8;
    }
    r.in24 = 0u;
    r.stepnr = 0u;
    r.carry = r.s[23] == 0u ? 0xFFFFFFFFu : 0u;
    r.dummy = 0u;
#pragma unroll 1
    for (int i = 0; i < 32; i++) fs_rl_cycle(r);
}

// reference table layout <-> integer state
__device__ __forceinline__ void fs_rl_load(FsRanlux &r, const fs_u32 *t)
{
#pragma unroll
    for (int i = 0; i < 24; i++) r.s[i] = (fs_u32)__fmul_rn(__uint_as_float(t[i]), 4294967296.0f);
    r.carry = t[24] != 0u ? 0xFFFFFFFFu : 0u;
    r.dummy = t[25];
    r.in24 = t[26];
    r.stepnr = t[27];
}

__device__ __forceinline__ void fs_rl_store(const FsRanlux &r, fs_u32 *t)
{
#pragma unroll
    for (int i = 0; i < 24; i++) t[i] = __float_as_uint(__fmul_rn(__uint2float_rn(r.s[i]), 0x1p-32f));
    t[24] = r.carry ? __float_as_uint(0x1p-24f) : 0u;
    t[25] = r.dummy;
    t[26] = r.in24;
    t[27] = r.stepnr;
}

// kernel.c:180-190: four buffered values per generator call; the counter starts at 0
// in every launch (kernel.c:557-558)
template <int NSKIP>
struct FsRanluxStream {
    FsRanlux st;
    float b0, b1, b2, b3;
    fs_u32 count;

    __device__ __forceinline__ float next()
    {
        fs_u32 c = count & 3u;
        if (c == 0u) fs_rl_next4<NSKIP>(st, b0, b1, b2, b3);
        count++;
        return c == 0u ? b0 : (c == 1u ? b1 : (c == 2u ? b2 : b3));
    }

    // K consecutive values (K a multiple of 4), the same values next() would return K
    // times: the rem still-buffered values first, then K/4 fresh quadruples, the last rem
    // of which stay buffered.  One branch per K values instead of one per value.
    template <int K>
    __device__ __forceinline__ void next_k(float (&u)[K])
    {
        static_assert(K % 4 == 0, "K must be a multiple of 4");
        const fs_u32 rem = (4u - (count & 3u)) & 3u;
        // one inlined generator call in a rolled loop (the generator is large; K/4 inlined
        // copies cost instruction-cache misses): each quadruple is shifted in at the end
        float c[K];
#pragma unroll 1
        for (int q = 0; q < K / 4; q++) {
            float o0, o1, o2, o3;
            fs_rl_next4<NSKIP>(st, o0, o1, o2, o3);
#pragma unroll
            for (int k = 0; k < K - 4; k++) c[k] = c[k + 4];
            c[K - 4] = o0; c[K - 3] = o1; c[K - 2] = o2; c[K - 1] = o3;
        }
        switch (rem) {
        case 0:
#pragma unroll
            for (int k = 0; k < K; k++) u[k] = c[k];
            b0 = c[K - 4]; b1 = c[K - 3]; b2 = c[K - 2]; b3 = c[K - 1];
            break;
        case 1:
            u[0] = b3;
#pragma unroll
            for (int k = 1; k < K; k++) u[k] = c[k - 1];
            b3 = c[K - 1];
            break;
        case 2:
            u[0] = b2; u[1] = b3;
#pragma unroll
            for (int k = 2; k < K; k++) u[k] = c[k - 2];
            b2 = c[K - 2]; b3 = c[K - 1];
            break;
        default:
            u[0] = b1; u[1] = b2; u[2] = b3;
#pragma unroll
            for (int k = 3; k < K; k++) u[k] = c[k - 3];
            b1 = c[K - 3]; b2 = c[K - 2]; b3 = c[K - 1];
            break;
        }
        count += K;
    }
};

// ranluxcl64 (pyopencl-ranluxcl.cl:893-920) with the same four-value buffering
template <int NSKIP>
struct FsRanluxStream64 {
    FsRanlux st;
    double b0, b1, b2, b3;
    fs_u32 count;

    __device__ __forceinline__ void pair(double &a, double &b)
    {
        float v0, v1, v2, v3;
        fs_rl_next4<NSKIP>(st, v0, v1, v2, v3);
        if (v0 == 0x1p-48f) v0 = 0.0f;
        if (v2 == 0x1p-48f) v2 = 0.0f;
        a = __dadd_rn((double)v0, __ddiv_rn((double)v1, 16777216.0));
        b = __dadd_rn((double)v2, __ddiv_rn((double)v3, 16777216.0));
    }

    __device__ __forceinline__ double next()
    {
        fs_u32 c = count & 3u;
        if (c == 0u) {
            pair(b0, b1);
            pair(b2, b3);
        }
        count++;
        return c == 0u ? b0 : (c == 1u ? b1 : (c == 2u ? b2 : b3));
    }
};
