/*
 * rng_oracle.h -- TEST INFRASTRUCTURE ONLY (oracle). CPU restatement of the reference's
 * random number generators; never linked into the product.
 *
 *  - xorshift128 (Marsaglia) as in FeynSimul/GPUsrc/kernel.c:214-239;
 *  - RANLUX in the RANLUXCL v1.3.1 formulation (third-party, MIT, vendored by the
 *    reference as examples/pyopencl-ranluxcl.cl; upstream version unpinned because the
 *    reference took it from its installed PyOpenCL): one subtract-with-borrow step
 *    (pyopencl-ranluxcl.cl:363-378), 4-value generation with the p-skipping schedule
 *    (:384-557), xorshift64 seeding + warm-up (:597-725), the double variant (:893-920);
 *  - the kernel's buffering wrappers (kernel.c:171-207).
 *
 * The state struct keeps the reference's 28-word layout (24 lag values, carry, dummy,
 * in24, stepnr; pyopencl-ranluxcl.cl:264-277) so state tables compare word for word.
 * Compile with -fsingle-precision-constant (float build) like the reference.
 */
#ifndef FS_RNG_ORACLE_H
#define FS_RNG_ORACLE_H

#include <stdint.h>

typedef struct {
    float s[24];   /* s[0] is the reference's s01 ... s[23] is s24 */
    float carry;   /* 0 or 2^-24 */
    float dummy;   /* padding word; never read */
    int in24;
    int stepnr;
} fso_ranlux_t;

#define FSO_TWOM24 (1.0f / 16777216.0f)
#define FSO_TWOM12 (1.0f / 4096.0f)

/* p-skip count per luxury level (pyopencl-ranluxcl.cl:304-317) */
static inline int fso_nskip(int lux)
{
    switch (lux) {
    case 0: return 0;
    case 1: return 24;
    case 2: return 76;
    case 3: return 200;
    case 4: return 380;
    default: return lux - 24;
    }
}

/* One subtract-with-borrow step on lag value s[a]; returns the output value. */
static inline float fso_swb(fso_ranlux_t *r, int a)
{
    float sj24 = r->s[(a + 10) % 24], sj24m1 = r->s[(a + 9) % 24];
    float uni = sj24 - r->s[a] - r->carry;
    if (uni < 0.0f) {
        uni += 1.0f;
        r->carry = FSO_TWOM24;
    } else {
        r->carry = 0.0f;
    }
    r->s[a] = uni;
    float out = uni;
    if (uni < FSO_TWOM12) {        /* fill the low bits of tiny outputs */
        out += FSO_TWOM24 * sj24m1;
        if (out == 0.0f) out = FSO_TWOM24 * FSO_TWOM24;
    }
    return out;
}

/* Cycle position p (0..23) updates lag index 23-p. */
static inline float fso_step(fso_ranlux_t *r, int p) { return fso_swb(r, 23 - p); }

static inline void fso_ranlux_skip(fso_ranlux_t *r, int pos, int count)
{
    for (int i = 0; i < count; i++) fso_step(r, (pos + i) % 24);
}

/* Four consecutive outputs, then the p-skip after every 24 outputs. */
static inline void fso_ranlux32(fso_ranlux_t *r, int nskip, float out[4])
{
    int pos = r->stepnr;
    for (int i = 0; i < 4; i++) out[i] = fso_step(r, pos + i);
    pos += 4;
    if (nskip % 24 == 0) {
        /* planar scheme: in24 is not used; skip whenever a 24-cycle completes */
        if (pos == 24) {
            fso_ranlux_skip(r, 0, nskip);
            pos = 0;
        }
        r->stepnr = pos;
    } else {
        r->stepnr = pos % 24;
        r->in24 += 4;
        if (r->in24 == 24) {
            r->in24 = 0;
            fso_ranlux_skip(r, r->stepnr, nskip);
            r->stepnr = (r->stepnr + nskip) % 24;
        }
    }
}

/* Double outputs from two float quadruples (pyopencl-ranluxcl.cl:893-920). */
static inline void fso_ranlux64(fso_ranlux_t *r, int nskip, double out[4])
{
    for (int h = 0; h < 2; h++) {
        float v[4];
        fso_ranlux32(r, nskip, v);
        if (v[0] == FSO_TWOM24 * FSO_TWOM24) v[0] = 0.0f;
        if (v[2] == FSO_TWOM24 * FSO_TWOM24) v[2] = 0.0f;
        out[2 * h + 0] = (double)v[0] + (double)v[1] / 16777216.0;
        out[2 * h + 1] = (double)v[2] + (double)v[3] / 16777216.0;
    }
}

/* Seeding: three xorshift64 words -> eight 24-bit lag values, three times, then
 * 32 full cycles of warm-up. */
static inline void fso_ranlux_init(fso_ranlux_t *r, uint64_t x)
{
    for (int blk = 0; blk < 3; blk++) {
        uint64_t w[3];
        for (int k = 0; k < 3; k++) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            w[k] = x;
        }
        /* the 192 bits w0|w1|w2 (most significant first) cut into 8 chunks of 24 */
        for (int c = 0; c < 8; c++) {
            int bit = c * 24; /* offset from the top of the 192-bit string */
            uint32_t v = 0;
            for (int b = 0; b < 24; b++) {
                int pos = bit + b, word = pos / 64, sh = 63 - (pos % 64);
                v = (v << 1) | (uint32_t)((w[word] >> sh) & 1u);
            }
            r->s[blk * 8 + c] = (float)v * FSO_TWOM24;
        }
    }
    r->in24 = 0;
    r->stepnr = 0;
    r->carry = (r->s[23] == 0.0f) ? FSO_TWOM24 : 0.0f;
    r->dummy = 0.0f;
    for (int i = 0; i < 32 * 24; i++) fso_step(r, i % 24);
}

/* kernel.c:171-207: four buffered values per generator call; the counter restarts
 * at 0 in every launch (kernel.c:557-558), dropping any unread buffered values. */
typedef struct {
    fso_ranlux_t st;
    float buf[4];
    double dbuf[4];
    uint32_t count;
} fso_ranlux_stream_t;

static inline float fso_ranlux_float(fso_ranlux_stream_t *g, int nskip)
{
    if ((g->count & 3u) == 0) fso_ranlux32(&g->st, nskip, g->buf);
    return g->buf[(g->count++) & 3u];
}

static inline double fso_ranlux_double(fso_ranlux_stream_t *g, int nskip)
{
    if ((g->count & 3u) == 0) fso_ranlux64(&g->st, nskip, g->dbuf);
    return g->dbuf[(g->count++) & 3u];
}

/* xorshift128, kernel.c:214-220 */
static inline uint32_t fso_xorshift(uint32_t s[4])
{
    uint32_t t = s[0] ^ (s[0] << 11);
    s[0] = s[1];
    s[1] = s[2];
    s[2] = s[3];
    s[3] = s[3] ^ (s[3] >> 19) ^ (t ^ (t >> 8));
    return s[3];
}

#endif
