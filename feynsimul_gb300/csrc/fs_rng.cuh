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
//    [0, 1), so this file keeps them as 24-bit integers k (value k * 2^-24): one step is
//    d = a - b - carry; carry = sign(d); k = d mod 2^24, three integer ops instead of the
//    reference's five float ops, with identical results because every float operation of
//    the reference on these values is exact.  Output floats are formed exactly as the
//    reference forms them (small values get the next lag's bits, zero maps to 2^-48).
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
struct FsRanlux {
    fs_u32 s[24];   // lag value k, s[0] is the reference's s01
    fs_u32 carry;   // 0 or 1 (the reference stores 0 or 2^-24)
    fs_u32 in24;
    fs_u32 stepnr;
    fs_u32 dummy;   // padding word of the table, carried through unchanged
};

// one subtract-with-borrow step on lag A (cycle position 23-A)
template <int A>
__device__ __forceinline__ void fs_rl_swb(FsRanlux &r)
{
    fs_u32 d = r.s[(A + 10) % 24] - r.s[A] - r.carry;
    r.carry = d >> 31;
    r.s[A] = d & 0xFFFFFFu;
}

template <int A>
__device__ __forceinline__ float fs_rl_out(FsRanlux &r)
{
    fs_rl_swb<A>(r);
    fs_u32 v = r.s[A];
    float out = __fmul_rn(__uint2float_rn(v), 0x1p-24f);
    if (v < 4096u) {  // value below 2^-12: add the next lag scaled by 2^-24
        out = __fadd_rn(out, __fmul_rn(__uint2float_rn(r.s[(A + 9) % 24]), 0x1p-48f));
        if (out == 0.0f) out = 0x1p-48f;
    }
    return out;
}

// steps at cycle positions P..P+3 (no outputs)
template <int P>
__device__ __forceinline__ void fs_rl_skip4(FsRanlux &r)
{
    fs_rl_swb<23 - P>(r);
    fs_rl_swb<22 - P>(r);
    fs_rl_swb<21 - P>(r);
    fs_rl_swb<20 - P>(r);
}

__device__ __forceinline__ void fs_rl_cycle(FsRanlux &r)
{
    fs_rl_skip4<0>(r);
    fs_rl_skip4<4>(r);
    fs_rl_skip4<8>(r);
    fs_rl_skip4<12>(r);
    fs_rl_skip4<16>(r);
    fs_rl_skip4<20>(r);
}

// NSKIP steps starting at cycle position pos (a multiple of 4); returns the new position
template <int NSKIP>
__device__ __forceinline__ fs_u32 fs_rl_skip(FsRanlux &r, fs_u32 pos)
{
    if (NSKIP == 0) return pos;
    // up to the cycle boundary (falls through on purpose)
    switch (pos) {
    case 4: fs_rl_skip4<4>(r);
    case 8: fs_rl_skip4<8>(r);
    case 12: fs_rl_skip4<12>(r);
    case 16: fs_rl_skip4<16>(r);
    case 20: fs_rl_skip4<20>(r);
    default: break;
    }
    const int initial = pos ? 24 - (int)pos : 0;
    const int bulk = (NSKIP - initial) / 24;
    const int rem = NSKIP - initial - bulk * 24;
#pragma unroll 1
    for (int i = 0; i < bulk; i++) fs_rl_cycle(r);
    if (rem > 0) fs_rl_skip4<0>(r);
    if (rem > 4) fs_rl_skip4<4>(r);
    if (rem > 8) fs_rl_skip4<8>(r);
    if (rem > 12) fs_rl_skip4<12>(r);
    if (rem > 16) fs_rl_skip4<16>(r);
    return (fs_u32)rem;
}

// four outputs (ranluxcl32), then the skip after every 24 outputs
template <int NSKIP>
__device__ __forceinline__ void fs_rl_next4(FsRanlux &r, float &o0, float &o1, float &o2, float &o3)
{
    switch (r.stepnr) {
    case 0: o0 = fs_rl_out<23>(r); o1 = fs_rl_out<22>(r); o2 = fs_rl_out<21>(r); o3 = fs_rl_out<20>(r); break;
    case 4: o0 = fs_rl_out<19>(r); o1 = fs_rl_out<18>(r); o2 = fs_rl_out<17>(r); o3 = fs_rl_out<16>(r); break;
    case 8: o0 = fs_rl_out<15>(r); o1 = fs_rl_out<14>(r); o2 = fs_rl_out<13>(r); o3 = fs_rl_out<12>(r); break;
    case 12: o0 = fs_rl_out<11>(r); o1 = fs_rl_out<10>(r); o2 = fs_rl_out<9>(r); o3 = fs_rl_out<8>(r); break;
    case 16: o0 = fs_rl_out<7>(r); o1 = fs_rl_out<6>(r); o2 = fs_rl_out<5>(r); o3 = fs_rl_out<4>(r); break;
    default: o0 = fs_rl_out<3>(r); o1 = fs_rl_out<2>(r); o2 = fs_rl_out<1>(r); o3 = fs_rl_out<0>(r); break;
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
        r.s[b * 8 + 0] = (fs_u32)(w[0] >> 40);
        r.s[b * 8 + 1] = (fs_u32)(w[0] >> 16) & 0xFFFFFFu;
        r.s[b * 8 + 2] = ((fs_u32)(w[0] & 0xFFFFu) << 8) | (fs_u32)(w[1] >> 56);
        r.s[b * 8 + 3] = (fs_u32)(w[1] >> 32) & 0xFFFFFFu;
        r.s[b * 8 + 4] = (fs_u32)(w[1] >> 8) & 0xFFFFFFu;
        r.s[b * 8 + 5] = ((fs_u32)(w[1] & 0xFFu) << 16) | (fs_u32)(w[2] >> 48);
        r.s[b * 8 + 6] = (fs_u32)(w[2] >> 24) & 0xFFFFFFu;
        r.s[b * 8 + 7] = (fs_u32)w[2] & 0xFFFFFFu;
    }
    r.in24 = 0u;
    r.stepnr = 0u;
    r.carry = r.s[23] == 0u ? 1u : 0u;
    r.dummy = 0u;
#pragma unroll 1
    for (int i = 0; i < 32; i++) fs_rl_cycle(r);
}

// reference table layout <-> integer state
__device__ __forceinline__ void fs_rl_load(FsRanlux &r, const fs_u32 *t)
{
#pragma unroll
    for (int i = 0; i < 24; i++) r.s[i] = (fs_u32)__fmul_rn(__uint_as_float(t[i]), 16777216.0f);
    r.carry = t[24] != 0u ? 1u : 0u;
    r.dummy = t[25];
    r.in24 = t[26];
    r.stepnr = t[27];
}

__device__ __forceinline__ void fs_rl_store(const FsRanlux &r, fs_u32 *t)
{
#pragma unroll
    for (int i = 0; i < 24; i++) t[i] = __float_as_uint(__fmul_rn(__uint2float_rn(r.s[i]), 0x1p-24f));
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
