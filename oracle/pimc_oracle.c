/*
 * pimc_oracle.c -- TEST INFRASTRUCTURE ONLY (oracle). CPU restatement of the reference's
 * Metropolis-bisection sweep; never linked into the product.  It is the checker for the
 * CUDA kernels in tests/, in __graft_entry__.smoke() and in bench.py's CPU baseline.
 *
 * Pinned against the reference's own kernel.c compiled on the CPU (oracle/build_ref.py)
 * through the golden fixtures in tests/golden/ (tests/test_oracle.py).
 *
 * Template: oracle/oracle.py prepends the FS_* configuration macros and replaces the
 * user marker below with the plugin's userCode and the generated potential / operator /
 * correlator / histogram functions, then compiles with
 *   gcc -std=gnu11 -O2 -ffp-contract=off -fgnu89-inline -fopenmp [-fsingle-precision-constant]
 *
 * Follows (reference file:line):
 *   RNG draws ............ FeynSimul/GPUsrc/kernel.c:76-101, :180-239
 *   sigma table .......... kernel.c:605-619
 *   bisection move ....... kernel.c:258-399
 *   sweep driver ......... kernel.c:538-737 (parallel-path and walker modes)
 *   measurement .......... kernel.c:734-797 (operator, histogram, correlator)
 *   epilogue ............. kernel.c:801-836
 * Parallel-path mode runs the walker's work-items in lock-step: within one Metropolis
 * step their segments have disjoint interiors and fixed endpoints, so executing them one
 * after another between the reference's barriers gives the barrier semantics exactly.
 *
 * Modes (identical meaning in the CUDA kernels):
 *   FS_COMPAT 1  reference-compatible RNG use: per-thread xorshift rows, the walker's
 *                integer stream read from seed row (group + lid1*nWG) at call start and not
 *                written back (kernel.c:568-572); RANLUX integers (uint)(f*ranluxIntMax)
 *                whose low 8 bits are zero, so the segment offset is 0 (kernel.c:206, :715).
 *   FS_COMPAT 0  fixed: each walker owns an integer stream that is written back;
 *                RANLUX offsets are (uint)(f * range).
 *   FS_ACCUM 0   operator / correlator sums in FP32, in the reference's order.
 *   FS_ACCUM 1   FP64 sums.  FS_ACCUM 2: compensated (Kahan) FP32 sums.
 *   FS_ACCUM 3   precision study: FP32, Kahan-FP32 and FP64 sums of the same values.
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <tgmath.h>
/* OpenCL's rsqrt for plugin code (type-generic through tgmath's sqrt) */
#ifndef rsqrt
#define rsqrt(x) (1 / sqrt(x))
#endif

#include "rng_oracle.h"

#if FS_DOUBLE
typedef double FT;
#else
typedef float FT;
#endif
#define FLOAT_TYPE FT
/* OpenCL spellings the plugin strings may use */
#define native_exp exp
#define native_log log
#define native_sqrt sqrt
#define native_sin sin
#define native_cos cos
#define native_divide(a, b) ((a) / (b))
#define native_recip(a) (1.0 / (a))
#define native_powr pow

/*@USER@*/

#define FS_HALF_N (FS_N / 2)
#define FS_THREADS (FS_NWALKERS * FS_TPW)

typedef struct {
    uint32_t xs[4];
    fso_ranlux_stream_t rl;
} fso_stream_t;

static inline FT fso_uniform(fso_stream_t *g)
{
#if FS_RANLUX
#if FS_DOUBLE
    return fso_ranlux_double(&g->rl, FS_NSKIP);
#else
    return fso_ranlux_float(&g->rl, FS_NSKIP);
#endif
#else
    uint32_t w = fso_xorshift(g->xs);
    return (FT)w * (FT)2.328306437080797e-10;
#endif
}

/* Offset of the walker's segment grid for one Metropolis step. */
static inline uint32_t fso_offset(fso_stream_t *g, uint32_t range)
{
#if FS_RANLUX
    FT f = fso_uniform(g);
#if FS_COMPAT
    uint32_t r = (uint32_t)(f * (FT)FS_RIM);
    return r & (range - 1u);
#else
    return ((uint32_t)(f * (FT)range)) & (range - 1u);
#endif
#else
    return fso_xorshift(g->xs) & (range - 1u);
#endif
}

/* kernel.c:258-399 */
static int fso_bisect(FT *path, uint32_t start, fso_stream_t *g, const FT *sigma)
{
    FT old[(FS_SEG > 1 ? FS_SEG - 1 : 1) * FS_DOF];
    FT actionOld = 0.0;
    for (int i = 1; i < FS_SEG; i++) {
        uint32_t p = (start + (uint32_t)i) % FS_N;
        for (int d = 0; d < FS_DOF; d++) old[(i - 1) * FS_DOF + d] = path[d * FS_N + p];
        FT v = fs_pot(FS_ARGS_AT(path, p));
        FT t = (FT)FS_EPS * v;
        actionOld = actionOld + t;
    }
    for (int n = 1; n <= FS_S; n++) {
        int half = 1 << (FS_S - n);
        for (int i = 0; i < (1 << (n - 1)); i++) {
            uint32_t m = ((uint32_t)((1 + 2 * i) * half) + start) % FS_N;
            uint32_t l = ((uint32_t)(i * 2 * half) + start) % FS_N;
            uint32_t r = ((uint32_t)((i + 1) * 2 * half) + start) % FS_N;
            for (int d = 0; d < FS_DOF; d++) {
                FT u = fso_uniform(g);
                FT v = fso_uniform(g);
                FT rz;
                if (v == 0.0)
                    rz = 0.0;
                else
                    rz = sigma[n] * sqrt(-2.0 * log(v)) * sin(2.0 * M_PI * u);
                path[d * FS_N + m] = 0.5 * (path[d * FS_N + l] + path[d * FS_N + r]) + rz;
            }
        }
    }
    FT actionNew = 0.0;
    for (int i = 1; i < FS_SEG; i++) {
        uint32_t p = (start + (uint32_t)i) % FS_N;
        FT v = fs_pot(FS_ARGS_AT(path, p));
        FT t = (FT)FS_EPS * v;
        actionNew = actionNew + t;
    }
    FT acc = fso_uniform(g);
    if (exp(actionOld - actionNew) < acc) {
        for (int i = 1; i < FS_SEG; i++) {
            uint32_t p = (start + (uint32_t)i) % FS_N;
            for (int d = 0; d < FS_DOF; d++) path[d * FS_N + p] = old[(i - 1) * FS_DOF + d];
        }
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
/* kernel.c:245-249: half the squared step over epsilon^2 */
static inline FT fso_kin(FT a, FT b)
{
    FT d = a - b;
    return (FT)0.5 * (d * d) * (FT)FS_EPS_INV2;
}
#endif

#if FS_PATH_SHIFT
/* kernel.c:407-473: shift slices left..right (cyclically) of one degree of freedom by
 * offset and return the change of the kinetic + potential sum.  left == right shifts
 * nothing. */
static FT fso_shift(FT *path, int degree, FT offset, uint32_t left, uint32_t right)
{
    if (left == right) return 0.0;
    FT kinDiff = 0.0, potDiff = 0.0;
    FT *x = path + (size_t)degree * FS_N;
    if (left < right) {
        uint32_t rr = right + 1, ll = left - 1;
        if (left == 0) ll = FS_N - 1;
        if (right == FS_N - 1) rr = 0;
        kinDiff -= fso_kin(x[left], x[ll]);
        kinDiff -= fso_kin(x[right], x[rr]);
        for (uint32_t i = left; i <= right; i++) {
            potDiff -= fs_pot(FS_ARGS_AT(path, i));
            x[i] = x[i] + offset;
            potDiff += fs_pot(FS_ARGS_AT(path, i));
        }
        kinDiff += fso_kin(x[left], x[ll]);
        kinDiff += fso_kin(x[right], x[rr]);
    } else {
        kinDiff -= fso_kin(x[left], x[left - 1]);
        kinDiff -= fso_kin(x[right], x[right + 1]);
        for (uint32_t i = left; i < FS_N; i++) {
            potDiff -= fs_pot(FS_ARGS_AT(path, i));
            x[i] += offset;
            potDiff += fs_pot(FS_ARGS_AT(path, i));
        }
        for (uint32_t i = 0; i <= right; i++) {
            potDiff -= fs_pot(FS_ARGS_AT(path, i));
            x[i] += offset;
            potDiff += fs_pot(FS_ARGS_AT(path, i));
        }
        kinDiff += fso_kin(x[left], x[left - 1]);
        kinDiff += fso_kin(x[right], x[right + 1]);
    }
    return kinDiff + potDiff;
}

/* the reference's revert (kernel.c:654-656): the same shift by -offset */
static void fso_shift_back(FT *path, int degree, FT offset, uint32_t left, uint32_t right)
{
    if (left == right) return;
    FT *x = path + (size_t)degree * FS_N;
    if (left < right) {
        for (uint32_t i = left; i <= right; i++) x[i] = x[i] + -offset;
    } else {
        for (uint32_t i = left; i < FS_N; i++) x[i] += -offset;
        for (uint32_t i = 0; i <= right; i++) x[i] += -offset;
    }
}
#endif

typedef struct {
    FT *paths;               /* [walkers][DOF][N] */
    uint32_t *accepts;       /* [threads] */
    uint32_t *seeds;         /* xorshift: [threads+1][4] */
    uint32_t *walker_seeds;  /* xorshift, fixed mode: [walkers][4] */
    uint32_t *ranlux_tab;    /* RANLUX: [threads][28] */
    uint32_t *group_tab;     /* RANLUX: compat [threads][28], fixed [walkers][28] */
    void *op_means;          /* [threads][nOps] (FS_ACCUM 3: [threads][nOps][3] double) */
    void *cor_means;         /* [walkers or threads][nCorr][N/2] */
    uint32_t *bins;          /* [res^DOF] */
    unsigned long long *hist;/* [nbins] */
    int walker_begin, walker_end, omp_threads;
    double opnorm;           /* 1 / (operatorRuns * slices per thread), as a double */
    unsigned long long step_base; /* fixed mode: Metropolis steps of earlier launches */
} fso_args_t;

/* reference thread id of segment t of walker w (kernel.c:539-541) */
static inline int fso_thread_id(int w, int t)
{
#if FS_PARALLEL
    int g = w / FS_WPG, l1 = w % FS_WPG;
    return g * FS_TPW + t + l1 * FS_NWG * FS_TPW;
#else
    (void)t;
    return w;
#endif
}

typedef struct {
    float s, c; /* Kahan sum and compensation */
} fso_kahan_t;

static inline void fso_kahan_add(fso_kahan_t *k, float x)
{
    float y = x - k->c;
    float t = k->s + y;
    k->c = (t - k->s) - y;
    k->s = t;
}

/* Correlator sums of the FP64 and Kahan modes in FP32 builds: one measurement's N products of
 * a lag are summed in float-float -- Knuth's TwoSum gives the rounding error of every add
 * exactly, and the errors are summed on the side (Ogita, Rump and Oishi, "Accurate sum and
 * dot product", SIAM J. Sci. Comput. 26 (2005), Algorithm 4.4 "Sum2") -- and s + e joins the
 * lag's FP64 running sum (the study's FP64 column likewise; its FP32 and Kahan columns
 * sum the same products in slice order).  The error of the measurement's sum is bounded by
 * about N * 2^-48 * sum |products|, far below the FP32 rounding of the products themselves. */
#define FSO_COR_FF (FS_ACCUM != 0 && !FS_DOUBLE)
static inline void fso_ff_add(float *s, float *e, float q)
{
    const float t = *s + q;
    const float bp = t - *s;
    const float ap = t - bp;
    *e = *e + ((*s - ap) + (q - bp));
    *s = t;
}

/* precision-study correlator accumulator (FS_ACCUM 3): the same products summed in
 * plain FP32, Kahan-compensated FP32 and FP64; 24 bytes, the device's layout */
typedef struct {
    double d;
    float f, ks, kc, pad;
} fso_cor_study_t;

#if FS_NCOR > 0
static inline FT fso_cor_prod(const FT *path, uint32_t s1, uint32_t s2, int c)
{
    FT a[FS_NCOR], b[FS_NCOR];
    fs_cors(FS_ARGS_AT(path, s1), a);
    fs_cors(FS_ARGS_AT(path, s2), b);
    FT prod = 1.0;
    prod *= a[c];
    prod *= b[c];
    return prod;
}
#endif

int fso_run(fso_args_t *A)
{
    /* sigma table, kernel.c:608-618 */
    FT sigma[FS_S + 1];
    {
        int twoPow = 1;
        sigma[0] = ((FT)FS_SEG) * (FT)FS_EPS;
        for (int i = 1; i <= FS_S; i++) {
            twoPow *= 2;
            sigma[i] = sqrt(((FT)FS_SEG * (FT)FS_EPS / (2.0 * (FT)twoPow)));
        }
    }
#if !FS_RANLUX && FS_COMPAT
    /* the walker integer stream is read from the table as it was at launch start */
    uint32_t *snap = (uint32_t *)malloc(sizeof(uint32_t) * 4 * (FS_THREADS + 1));
    memcpy(snap, A->seeds, sizeof(uint32_t) * 4 * (FS_THREADS + 1));
#endif
    int wb = A->walker_begin, we = A->walker_end;
#pragma omp parallel for schedule(dynamic, 1) num_threads(A->omp_threads)
    for (int w = wb; w < we; w++) {
        FT *path = A->paths + (size_t)w * FS_DOF * FS_N;
        fso_stream_t fs[FS_TPW];
        fso_stream_t is;
        uint32_t acc[FS_TPW];
        memset(&is, 0, sizeof(is));
        for (int t = 0; t < FS_TPW; t++) {
            int tid = fso_thread_id(w, t);
            memset(&fs[t], 0, sizeof(fs[t]));
            acc[t] = 0;
#if FS_RANLUX
            memcpy(&fs[t].rl.st, A->ranlux_tab + (size_t)tid * 28, 112);
#else
            memcpy(fs[t].xs, A->seeds + (size_t)tid * 4, 16);
#endif
        }
#if FS_RANLUX
#if FS_COMPAT
        memcpy(&is.rl.st, A->group_tab + (size_t)fso_thread_id(w, 0) * 28, 112);
#else
        memcpy(&is.rl.st, A->group_tab + (size_t)w * 28, 112);
#endif
#else
#if FS_COMPAT
#if FS_PARALLEL
        {
            int row = (w / FS_WPG) + (w % FS_WPG) * FS_NWG;
            memcpy(is.xs, snap + (size_t)row * 4, 16);
        }
#else
        memcpy(is.xs, snap + (size_t)w * 4, 16);
#endif
#else
        memcpy(is.xs, A->walker_seeds + (size_t)w * 4, 16);
#endif
#endif

#if FS_NOPS > 0
        FT opr[FS_TPW][FS_NOPS];      /* the reference's FLOAT_TYPE sum (kernel.c:622) */
        float opf[FS_TPW][FS_NOPS];   /* plain FP32 sum (precision study) */
        double opd[FS_TPW][FS_NOPS];
        fso_kahan_t opk[FS_TPW][FS_NOPS];
        memset(opr, 0, sizeof(opr));
        memset(opf, 0, sizeof(opf));
        memset(opd, 0, sizeof(opd));
        memset(opk, 0, sizeof(opk));
#endif
#if FS_NCOR > 0
        /* correlator sums for this walker, continuing the stored values (never reset
         * on the device, kernel.c:784-788) */
        double cord[FS_NCOR][FS_HALF_N];
        FT corf[FS_NCOR][FS_HALF_N];
        float cor32[FS_NCOR][FS_HALF_N];
        fso_kahan_t cork[FS_NCOR][FS_HALF_N];
        {
            size_t crow = (size_t)w;
            for (int c = 0; c < FS_NCOR; c++)
                for (int tau = 0; tau < FS_HALF_N; tau++) {
                    size_t idx = (crow * FS_NCOR + c) * FS_HALF_N + tau;
#if FS_ACCUM == 0
                    corf[c][tau] = ((FT *)A->cor_means)[idx];
#elif FS_ACCUM == 3
                    const fso_cor_study_t *cs = (const fso_cor_study_t *)A->cor_means + idx;
                    cord[c][tau] = cs->d;
                    cor32[c][tau] = cs->f;
                    cork[c][tau].s = cs->ks;
                    cork[c][tau].c = cs->kc;
#else
                    cord[c][tau] = ((double *)A->cor_means)[idx];
#endif
                }
        }
        (void)cor32;
        (void)cork;
#endif
        for (int run = 0; run < FS_OPRUNS; run++) {
            for (int step = 0; step < FS_MSTEPS; step++) {
#if FS_PARALLEL
                uint32_t off = fso_offset(&is, FS_SEG);
                for (int t = 0; t < FS_TPW; t++) {
                    uint32_t start = (off + (uint32_t)(FS_SEG * t)) % FS_N;
                    acc[t] += (uint32_t)fso_bisect(path, start, &fs[t], sigma);
                }
#else
                /* kernel.c:640-705: the step counter i*mSteps + j restarts every launch in
                 * the reference; the fixed mode continues it across launches */
#if FS_COMPAT
                const unsigned long long k = (unsigned long long)run * FS_MSTEPS + step;
#else
                const unsigned long long k = A->step_base + (unsigned long long)run * FS_MSTEPS + step;
#endif
                (void)k;
#if FS_PATH_SHIFT
                {
                    const int degree = (int)(k % FS_DOF);
                    const uint32_t left = fso_offset(&is, FS_N);
                    const uint32_t right = fso_offset(&is, FS_N);
                    const FT offset = (FT)FS_PSALPHA * ((FT)2.0 * fso_uniform(&fs[0]) - (FT)1.0);
#if !FS_COMPAT
                    FT saved[FS_N];
                    memcpy(saved, path + (size_t)degree * FS_N, sizeof(saved));
#endif
                    const FT diff = fso_shift(path, degree, offset, left, right);
                    if (exp(-(FT)FS_EPS * diff) < fso_uniform(&fs[0])) {
#if FS_COMPAT
                        fso_shift_back(path, degree, offset, left, right);
#else
                        memcpy(path + (size_t)degree * FS_N, saved, sizeof(saved));
#endif
                    } else {
                        acc[0]++;
                    }
                }
#endif
#if FS_SNM
                {
                    const uint32_t modPoint = (uint32_t)(k % FS_N);
                    const uint32_t modPathPoint = (uint32_t)(k % ((unsigned long long)FS_N * FS_DOF));
                    uint32_t ri = modPathPoint + 1, li = modPathPoint - 1;
                    if (modPoint == 0) li += FS_N;
                    else if (modPoint == FS_N - 1) ri -= FS_N;
                    const FT oldX = path[modPathPoint];
                    const FT modX = oldX + ((FT)2.0 * fso_uniform(&fs[0]) - (FT)1.0) * (FT)FS_ALPHA;
                    FT diffE = fso_kin(modX, path[ri]) + fso_kin(modX, path[li]) - fso_kin(path[modPathPoint], path[li]) -
                               fso_kin(path[modPathPoint], path[ri]);
                    diffE -= fs_pot(FS_ARGS_AT(path, modPoint));
                    path[modPathPoint] = modX;
                    diffE += fs_pot(FS_ARGS_AT(path, modPoint));
                    path[modPathPoint] = oldX;
                    if (exp(-(FT)FS_EPS * diffE) > fso_uniform(&fs[0])) {
                        path[modPathPoint] = modX;
                        acc[0]++;
                    }
                }
#endif
#if FS_BISECT
                uint32_t start = fso_offset(&is, FS_N) % FS_N;
                acc[0] += (uint32_t)fso_bisect(path, start, &fs[0], sigma);
#endif
#endif
            }
            /* measurement, kernel.c:734-797 */
            for (int t = 0; t < FS_TPW; t++) {
#if FS_PARALLEL
                int s0 = t * FS_SEG, s1 = (t + 1) * FS_SEG;
#else
                int s0 = 0, s1 = FS_N;
#endif
                for (int s = s0; s < s1; s++) {
#if FS_NOPS > 0
                    FT ov[FS_NOPS];
                    fs_ops(FS_ARGS_AT(path, s), ov);
                    for (int i = 0; i < FS_NOPS; i++) {
                        opr[t][i] = opr[t][i] + ov[i];
                        opf[t][i] = opf[t][i] + (float)ov[i];
                        opd[t][i] += (double)ov[i];
                        fso_kahan_add(&opk[t][i], (float)ov[i]);
                    }
#endif
#if FS_BINS
                    {
                        int ok = 1, inc = 1, bi = 0;
                        for (int d = 0; d < FS_DOF; d++) {
                            FT x = path[d * FS_N + s];
                            if (x < (FT)FS_XMIN || x >= (FT)FS_XMAX) {
                                ok = 0;
                                break;
                            }
                            bi += (int)((uint32_t)((x - (FT)FS_XMIN) * (FT)FS_INVBIN)) * inc;
                            inc *= FS_BINRES;
                        }
                        if (ok) __atomic_fetch_add(A->bins + bi, 1u, __ATOMIC_RELAXED);
                    }
#endif
#if FS_NHIST > 0
                    {
                        FT hv[FS_NHIST];
                        fs_hist(FS_ARGS_AT(path, s), hv);
                        for (int h = 0; h < FS_NHIST; h++) {
                            FT x = hv[h];
                            if (x >= (FT)FS_HLO && x < (FT)FS_HHI) {
                                int b = (int)((x - (FT)FS_HLO) * (FT)FS_HINVW);
                                if (b >= 0 && b < FS_HBINS)
                                    __atomic_fetch_add(A->hist + b, 1ull, __ATOMIC_RELAXED);
                            }
                        }
                    }
#endif
                }
            }
#if FS_NCOR > 0
#if FS_PARALLEL
            for (int c = 0; c < FS_NCOR; c++)
                for (int tau = 0; tau < FS_HALF_N; tau++) {
#if FS_ACCUM == 0
                    /* the reference's order: slice k of every work-item, then the lag
                     * rotation of kernel.c:751-757 */
                    for (int k = 0; k < FS_SEG; k++)
                        for (int cti = 0; cti < FS_HALF_N; cti++) {
                            int tp = ((tau - cti) % FS_HALF_N + FS_HALF_N) % FS_HALF_N;
                            if (tp >= FS_TPW) continue;
                            uint32_t s1 = (uint32_t)(tp * FS_SEG + k);
                            uint32_t s2 = (s1 + (uint32_t)tau) % FS_N;
                            corf[c][tau] = corf[c][tau] + fso_cor_prod(path, s1, s2, c);
                        }
#elif FSO_COR_FF
                    {
                        float fs = 0.0f, fe = 0.0f;
                        for (uint32_t s1 = 0; s1 < FS_N; s1++) {
                            const FT pr = fso_cor_prod(path, s1, (s1 + (uint32_t)tau) % FS_N, c);
                            fso_ff_add(&fs, &fe, pr);
#if FS_ACCUM == 3
                            cor32[c][tau] = cor32[c][tau] + (float)pr;
                            fso_kahan_add(&cork[c][tau], (float)pr);
#endif
                        }
                        cord[c][tau] = cord[c][tau] + ((double)fs + (double)fe);
                    }
#else
                    {
                        /* FP64 sums: partial sums over s1 mod 4, combined as (p0 + p1) + (p2 + p3)
                         * (p0 from the running sum); the FP32 study columns in slice order */
                        double p[4] = {cord[c][tau], 0.0, 0.0, 0.0};
                        const uint32_t step = (FS_N % 4 == 0) ? 4u : 1u;
                        for (uint32_t s1 = 0; s1 < FS_N; s1++) {
                            const FT pr = fso_cor_prod(path, s1, (s1 + (uint32_t)tau) % FS_N, c);
                            p[s1 % step] += (double)pr;
#if FS_ACCUM == 3
                            cor32[c][tau] = cor32[c][tau] + (float)pr;
                            fso_kahan_add(&cork[c][tau], (float)pr);
#endif
                        }
                        cord[c][tau] = (p[0] + p[1]) + (p[2] + p[3]);
                    }
#endif
                }
#else
#if FS_ACCUM == 0
            for (uint32_t s1 = 0; s1 < FS_N; s1++)
                for (int tau = 0; tau < FS_HALF_N; tau++)
                    for (int c = 0; c < FS_NCOR; c++)
                        corf[c][tau] = corf[c][tau] + fso_cor_prod(path, s1, (s1 + (uint32_t)tau) % FS_N, c);
#elif FSO_COR_FF
            /* one lag at a time, float-float as in the parallel mode */
            for (int c = 0; c < FS_NCOR; c++)
                for (int tau = 0; tau < FS_HALF_N; tau++) {
                    float fs = 0.0f, fe = 0.0f;
                    for (uint32_t s1 = 0; s1 < FS_N; s1++) {
                        const FT pr = fso_cor_prod(path, s1, (s1 + (uint32_t)tau) % FS_N, c);
                        fso_ff_add(&fs, &fe, pr);
#if FS_ACCUM == 3
                        cor32[c][tau] = cor32[c][tau] + (float)pr;
                        fso_kahan_add(&cork[c][tau], (float)pr);
#endif
                    }
                    cord[c][tau] = cord[c][tau] + ((double)fs + (double)fe);
                }
#else
            /* one lag at a time, the FP64 sums in the four-way order of the parallel mode */
            for (int c = 0; c < FS_NCOR; c++)
                for (int tau = 0; tau < FS_HALF_N; tau++) {
                    double p[4] = {cord[c][tau], 0.0, 0.0, 0.0};
                    const uint32_t step = (FS_N % 4 == 0) ? 4u : 1u;
                    for (uint32_t s1 = 0; s1 < FS_N; s1++) {
                        const FT pr = fso_cor_prod(path, s1, (s1 + (uint32_t)tau) % FS_N, c);
                        p[s1 % step] += (double)pr;
#if FS_ACCUM == 3
                        cor32[c][tau] = cor32[c][tau] + (float)pr;
                        fso_kahan_add(&cork[c][tau], (float)pr);
#endif
                    }
                    cord[c][tau] = (p[0] + p[1]) + (p[2] + p[3]);
                }
#endif
#endif
#endif
        }
        /* epilogue, kernel.c:801-836 */
        for (int t = 0; t < FS_TPW; t++) {
            int tid = fso_thread_id(w, t);
            A->accepts[tid] = acc[t];
#if FS_NOPS > 0
            for (int i = 0; i < FS_NOPS; i++) {
                size_t o = (size_t)tid * FS_NOPS + i;
#if FS_ACCUM == 0
                ((FT *)A->op_means)[o] = opr[t][i] * (FT)FS_OPNORM;
#elif FS_ACCUM == 1
                ((double *)A->op_means)[o] = opd[t][i] * A->opnorm;
#elif FS_ACCUM == 2
                ((float *)A->op_means)[o] = opk[t][i].s * (float)FS_OPNORM;
#else
                ((double *)A->op_means)[3 * o + 0] = (double)(opf[t][i] * (float)FS_OPNORM);
                ((double *)A->op_means)[3 * o + 1] = (double)(opk[t][i].s * (float)FS_OPNORM);
                ((double *)A->op_means)[3 * o + 2] = opd[t][i] * A->opnorm;
#endif
            }
#endif
#if FS_RANLUX
            memcpy(A->ranlux_tab + (size_t)tid * 28, &fs[t].rl.st, 112);
#if FS_COMPAT
            memcpy(A->group_tab + (size_t)tid * 28, &is.rl.st, 112);
#endif
#else
            memcpy(A->seeds + (size_t)tid * 4, fs[t].xs, 16);
#endif
        }
#if FS_RANLUX && !FS_COMPAT
        memcpy(A->group_tab + (size_t)w * 28, &is.rl.st, 112);
#endif
#if !FS_RANLUX && !FS_COMPAT
        memcpy(A->walker_seeds + (size_t)w * 4, is.xs, 16);
#endif
#if FS_NCOR > 0
        for (int c = 0; c < FS_NCOR; c++)
            for (int tau = 0; tau < FS_HALF_N; tau++) {
                size_t idx = ((size_t)w * FS_NCOR + c) * FS_HALF_N + tau;
#if FS_ACCUM == 0
                ((FT *)A->cor_means)[idx] = corf[c][tau];
#elif FS_ACCUM == 3
                fso_cor_study_t *cs = (fso_cor_study_t *)A->cor_means + idx;
                cs->d = cord[c][tau];
                cs->f = cor32[c][tau];
                cs->ks = cork[c][tau].s;
                cs->kc = cork[c][tau].c;
                cs->pad = 0.f;
#else
                ((double *)A->cor_means)[idx] = cord[c][tau];
#endif
            }
#endif
    }
#if !FS_RANLUX && FS_COMPAT
    free(snap);
#endif
    return 0;
}

/* RANLUX state-table seeding (ranluxcl_init for each row's 64-bit seed value). */
void fso_ranlux_init_rows(uint32_t *tab, int n, const uint64_t *xs)
{
    for (int i = 0; i < n; i++) {
        fso_ranlux_t st;
        fso_ranlux_init(&st, xs[i]);
        memcpy(tab + (size_t)i * 28, &st, 112);
    }
}
