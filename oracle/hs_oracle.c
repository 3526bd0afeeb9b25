/*
 * hs_oracle.c -- CPU restatement of helioselene's variable-time MSM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the test suite,
 * the smoke check and the CPU-baseline leg of the benchmark load it; the
 * product (helioselene_gb300) never does.
 *
 * What it restates (helioselene sources):
 *   field arithmetic mod p = 2^255-19 and q = 2^255-gamma ...... hs_field_impl.h
 *   Jacobian dbl/add/add_safe, encoding, decoding, SWU map ..... hs_curve_impl.h
 *   signed-digit recode, Straus (n<=16), Pippenger, dispatcher . hs_curve_impl.h
 *     (helios/src/x64/helios_msm_vartime.cpp:110-416)
 *   Montgomery batch inversion (fp/include/fp_batch_invert.h:61-114)
 *   batch Jacobian->affine (helios/include/helios_batch_affine.h:55-98)
 *   Pedersen r*H + sum v_i*G_i (helios/include/helios_pedersen.h:55-86)
 *
 * keep_carry = 0 reproduces the reference bit for bit, including its w = 8
 * recode defect (864 <= n < 2592 drops the carry out of digit 31);
 * keep_carry = 1 is the mathematically exact MSM.
 *
 * Exchange formats (all little endian):
 *   scalar   32 bytes, any 256-bit value
 *   affine   64 bytes, x || y canonical; 64 zero bytes = identity
 *   jacobian 96 bytes, X || Y || Z (any value < 2^256); Z == 0 = identity
 *   encoded  32 bytes, the reference's point serialization
 */

#include "hs_oracle.h"

#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

typedef struct
{
    uint64_t v[4];
} fe;

/* ---------------- F_p, p = 2^255 - 19, c = 38 ---------------- */
#define FE(name) fp_##name
#define FE_M0 0xffffffffffffffedULL
#define FE_M1 0xffffffffffffffffULL
#define FE_M2 0xffffffffffffffffULL
#define FE_M3 0x7fffffffffffffffULL
#define FE_C0 38ULL
#define FE_C1 0ULL
#include "hs_field_impl.h"
#undef FE
#undef FE_M0
#undef FE_M1
#undef FE_M2
#undef FE_M3
#undef FE_C0
#undef FE_C1

/* ---------------- F_q, q = 2^255 - gamma, c = 2*gamma ---------------- */
/* gamma = 85737960593035654572250192257530476641 (fq/include/x64/fq51.h:38-40) */
#define FE(name) fq_##name
#define FE_M0 0x6eb6d2727927c79fULL
#define FE_M1 0xbf7f782cb7656b58ULL
#define FE_M2 0xffffffffffffffffULL
#define FE_M3 0x7fffffffffffffffULL
#define FE_C0 0x22925b1b0db070c2ULL
#define FE_C1 0x81010fa69135294fULL
#include "hs_field_impl.h"
#undef FE
#undef FE_M0
#undef FE_M1
#undef FE_M2
#undef FE_M3
#undef FE_C0
#undef FE_C1

/* sqrt in F_p (p = 5 mod 8): r = a^((p+3)/8), times sqrt(-1) when r^2 = -a.
 * Returns 0 when a is a square (fp/src/x64/fp_sqrt.cpp). */
static int fp_sqrt(fe *r, const fe *a)
{
    static const uint64_t e[4] = {0xfffffffffffffffeULL, 0xffffffffffffffffULL, 0xffffffffffffffffULL,
                                  0x0fffffffffffffffULL};
    /* sqrt(-1) = 2^((p-1)/4) */
    static const uint64_t e4[4] = {0xfffffffffffffffbULL, 0xffffffffffffffffULL, 0xffffffffffffffffULL,
                                   0x1fffffffffffffffULL};
    fe x, chk, na;
    fp_pow(&x, a, e);
    fp_sq(&chk, &x);
    if (!fp_eq(&chk, a))
    {
        fp_neg(&na, a);
        if (!fp_eq(&chk, &na))
            return -1;
        fe two, i;
        fp_set_u64(&two, 2);
        fp_pow(&i, &two, e4);
        fp_mul(&x, &x, &i);
    }
    *r = x;
    return 0;
}

/* sqrt in F_q (q = 3 mod 4): r = a^((q+1)/4) (fq/src/x64/fq_sqrt.cpp:45) */
static int fq_sqrt(fe *r, const fe *a)
{
    /* (q+1)/4 */
    static const uint64_t e[4] = {0x1badb49c9e49f1e8ULL, 0xefdfde0b2dd95ad6ULL, 0xffffffffffffffffULL,
                                  0x1fffffffffffffffULL};
    fe x, chk;
    fq_pow(&x, a, e);
    fq_sq(&chk, &x);
    if (!fq_eq(&chk, a))
        return -1;
    *r = x;
    return 0;
}

static fe HELIOS_B_FE, SELENE_B_FE;

/* b constants from the decimal values in helios/include/helios_constants.h:38 and
 * selene/include/selene_constants.h:38 */
static const uint8_t HELIOS_B_BYTES[32] = {
    0xd4, 0x3a, 0xd7, 0xed, 0xe1, 0x9e, 0xb4, 0x22, 0x35, 0xbf, 0x13, 0x41, 0x38, 0x6f, 0x3f, 0x04,
    0x3b, 0x7b, 0xbb, 0x3e, 0x6b, 0xa7, 0x94, 0xbe, 0xb8, 0x70, 0xea, 0xb0, 0x39, 0xc7, 0xe8, 0x22};
static const uint8_t SELENE_B_BYTES[32] = {
    0x58, 0x45, 0x5a, 0xcb, 0x83, 0x09, 0xde, 0x68, 0x0e, 0x90, 0xae, 0x06, 0xdf, 0x4b, 0x94, 0xf3,
    0x79, 0xe2, 0xff, 0x95, 0xa5, 0xbb, 0x51, 0x7f, 0xc1, 0x76, 0x58, 0x69, 0x13, 0x77, 0x12, 0x70};

static pthread_once_t g_once = PTHREAD_ONCE_INIT;
static void init_consts(void)
{
    fp_load32(&HELIOS_B_FE, HELIOS_B_BYTES);
    fq_load32(&SELENE_B_FE, SELENE_B_BYTES);
}

/* ---------------- Helios over F_p ---------------- */
#define CV(name) helios_##name
#define F(name) fp_##name
#define CV_B (&HELIOS_B_FE)
#define CV_SSWU_Z 7
#include "hs_curve_impl.h"
#undef CV
#undef F
#undef CV_B
#undef CV_SSWU_Z

/* ---------------- Selene over F_q ---------------- */
#define CV(name) selene_##name
#define F(name) fq_##name
#define CV_B (&SELENE_B_FE)
#define CV_SSWU_Z (-4)
#include "hs_curve_impl.h"
#undef CV
#undef F
#undef CV_B
#undef CV_SSWU_Z

/* ===================================================================== */
/* exported API: one generic body per curve, selected by a small table     */
/* ===================================================================== */

#define GEN_API(C, FF)                                                                                        \
    static void C##_load_affine(C##_jac *p, const uint8_t *b64)                                               \
    {                                                                                                         \
        int z = 1;                                                                                            \
        for (int i = 0; i < 64; i++)                                                                          \
            if (b64[i])                                                                                       \
            {                                                                                                 \
                z = 0;                                                                                        \
                break;                                                                                        \
            }                                                                                                 \
        if (z)                                                                                                \
        {                                                                                                     \
            C##_identity(p);                                                                                  \
            return;                                                                                           \
        }                                                                                                     \
        FF##_load32(&p->X, b64);                                                                              \
        FF##_load32(&p->Y, b64 + 32);                                                                         \
        FF##_set_u64(&p->Z, 1);                                                                               \
    }                                                                                                         \
    static void C##_load_jac(C##_jac *p, const uint8_t *b96)                                                  \
    {                                                                                                         \
        FF##_load32(&p->X, b96);                                                                              \
        FF##_load32(&p->Y, b96 + 32);                                                                         \
        FF##_load32(&p->Z, b96 + 64);                                                                         \
    }                                                                                                         \
    static void C##_store_affine(uint8_t *b64, const C##_jac *p)                                              \
    {                                                                                                         \
        fe x, y;                                                                                              \
        C##_to_affine(&x, &y, p);                                                                             \
        FF##_tobytes(b64, &x);                                                                                \
        FF##_tobytes(b64 + 32, &y);                                                                           \
    }                                                                                                         \
    typedef struct                                                                                            \
    {                                                                                                         \
        const uint8_t *scalars;                                                                               \
        const C##_jac *pts;                                                                                   \
        size_t n;                                                                                             \
        C##_jac out;                                                                                          \
    } C##_task;                                                                                               \
    static void *C##_worker(void *arg)                                                                        \
    {                                                                                                         \
        C##_task *t = (C##_task *)arg;                                                                        \
        C##_msm(&t->out, t->scalars, t->pts, t->n, 1);                                                        \
        return NULL;                                                                                          \
    }

GEN_API(helios, fp)
GEN_API(selene, fq)

#define DISPATCH(curve, call_h, call_s) \
    do                                  \
    {                                   \
        if ((curve) == HSO_HELIOS)      \
        {                               \
            call_h;                     \
        }                               \
        else if ((curve) == HSO_SELENE) \
        {                               \
            call_s;                     \
        }                               \
        else                            \
            return -1;                  \
    } while (0)

#define BODY_MSM(C)                                                       \
    {                                                                     \
        C##_jac *pts = (C##_jac *)malloc((n ? n : 1) * sizeof(C##_jac));  \
        if (!pts)                                                         \
            return -2;                                                    \
        for (size_t i = 0; i < n; i++)                                    \
            if (jac)                                                      \
                C##_load_jac(&pts[i], points + 96 * i);                   \
            else                                                          \
                C##_load_affine(&pts[i], points + 64 * i);                \
        C##_jac r;                                                        \
        if (window > 0)                                                   \
            C##_pippenger(&r, scalars, pts, n, keep_carry, window);       \
        else                                                              \
            C##_msm(&r, scalars, pts, n, keep_carry);                     \
        C##_tobytes(out32, &r);                                           \
        if (out64)                                                        \
            C##_store_affine(out64, &r);                                  \
        free(pts);                                                        \
    }

static int msm_common(int curve, uint8_t *out32, uint8_t *out64, const uint8_t *scalars, const uint8_t *points,
                      size_t n, int keep_carry, int jac, int window)
{
    pthread_once(&g_once, init_consts);
    if (window > 0 && (window < 2 || window > 16))
        return -1;
    DISPATCH(curve, BODY_MSM(helios), BODY_MSM(selene));
    return 0;
}

int hso_msm(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n, int keep_carry)
{
    return msm_common(curve, out32, NULL, scalars, pts64, n, keep_carry, 0, 0);
}

int hso_msm_affine_out(int curve, uint8_t out32[32], uint8_t out64[64], const uint8_t *scalars,
                       const uint8_t *pts64, size_t n, int keep_carry)
{
    return msm_common(curve, out32, out64, scalars, pts64, n, keep_carry, 0, 0);
}

int hso_msm_jac(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *jac96, size_t n,
                int keep_carry)
{
    return msm_common(curve, out32, NULL, scalars, jac96, n, keep_carry, 1, 0);
}

int hso_pippenger_w(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n, int w,
                    int keep_carry)
{
    return msm_common(curve, out32, NULL, scalars, pts64, n, keep_carry, 0, w);
}

#define BODY_NAIVE(C)                                 \
    {                                                 \
        C##_jac acc, p, t;                            \
        C##_identity(&acc);                           \
        for (size_t i = 0; i < n; i++)                \
        {                                             \
            C##_load_affine(&p, pts64 + 64 * i);      \
            C##_scalar_mul(&t, scalars + 32 * i, &p); \
            C##_add_safe(&acc, &acc, &t);             \
        }                                             \
        C##_tobytes(out32, &acc);                     \
    }

int hso_msm_naive(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n)
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_NAIVE(helios), BODY_NAIVE(selene));
    return 0;
}

#define BODY_MT(C)                                                                   \
    {                                                                                \
        C##_jac *pts = (C##_jac *)malloc((n ? n : 1) * sizeof(C##_jac));             \
        C##_task *tasks = (C##_task *)calloc((size_t)nthreads, sizeof(C##_task));    \
        pthread_t *tids = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));  \
        if (!pts || !tasks || !tids)                                                 \
        {                                                                            \
            free(pts);                                                               \
            free(tasks);                                                             \
            free(tids);                                                              \
            return -2;                                                               \
        }                                                                            \
        for (size_t i = 0; i < n; i++)                                               \
            C##_load_affine(&pts[i], pts64 + 64 * i);                                \
        size_t chunk = (n + (size_t)nthreads - 1) / (size_t)nthreads;                \
        for (int t = 0; t < nthreads; t++)                                           \
        {                                                                            \
            size_t lo = (size_t)t * chunk, hi = lo + chunk;                          \
            if (lo > n)                                                              \
                lo = n;                                                              \
            if (hi > n)                                                              \
                hi = n;                                                              \
            tasks[t].scalars = scalars + 32 * lo;                                    \
            tasks[t].pts = pts + lo;                                                 \
            tasks[t].n = hi - lo;                                                    \
            pthread_create(&tids[t], NULL, C##_worker, &tasks[t]);                   \
        }                                                                            \
        C##_jac acc;                                                                 \
        C##_identity(&acc);                                                          \
        for (int t = 0; t < nthreads; t++)                                           \
        {                                                                            \
            pthread_join(tids[t], NULL);                                             \
            C##_add_safe(&acc, &acc, &tasks[t].out);                                 \
        }                                                                            \
        C##_tobytes(out32, &acc);                                                    \
        free(pts);                                                                   \
        free(tasks);                                                                 \
        free(tids);                                                                  \
    }

int hso_msm_mt(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n, int nthreads)
{
    pthread_once(&g_once, init_consts);
    if (nthreads < 1)
        nthreads = 1;
    DISPATCH(curve, BODY_MT(helios), BODY_MT(selene));
    return 0;
}

/* Many independent MSMs on a pool of threads (each MSM exact-mode hso_msm on
 * one thread; the threads take MSMs in index order from a shared counter).
 * MSM i reads sizes[i] scalars / affine points from where MSM i-1 ended. */
typedef struct
{
    int curve;
    uint8_t *out32s;
    const uint8_t *scalars, *pts64;
    const uint64_t *sizes, *offs;
    size_t count;
    size_t *next;
    int rc;
} many_task;

static void *many_worker(void *arg)
{
    many_task *t = (many_task *)arg;
    for (;;)
    {
        size_t i = __atomic_fetch_add(t->next, 1, __ATOMIC_RELAXED);
        if (i >= t->count)
            break;
        const uint64_t o = t->offs[i];
        if (hso_msm(t->curve, t->out32s + 32 * i, t->scalars + 32 * o, t->pts64 + 64 * o, (size_t)t->sizes[i], 1))
            t->rc = -1;
    }
    return NULL;
}

int hso_msm_many(int curve, uint8_t *out32s, const uint8_t *scalars, const uint8_t *pts64, const uint64_t *sizes,
                 size_t count, int nthreads)
{
    pthread_once(&g_once, init_consts);
    if (nthreads < 1)
        nthreads = 1;
    uint64_t *offs = (uint64_t *)malloc((count ? count : 1) * sizeof(uint64_t));
    many_task *tasks = (many_task *)calloc((size_t)nthreads, sizeof(many_task));
    pthread_t *tids = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!offs || !tasks || !tids)
    {
        free(offs);
        free(tasks);
        free(tids);
        return -2;
    }
    uint64_t o = 0;
    for (size_t i = 0; i < count; i++)
    {
        offs[i] = o;
        o += sizes[i];
    }
    size_t next = 0;
    for (int t = 0; t < nthreads; t++)
    {
        tasks[t] = (many_task){curve, out32s, scalars, pts64, sizes, offs, count, &next, 0};
        pthread_create(&tids[t], NULL, many_worker, &tasks[t]);
    }
    int rc = 0;
    for (int t = 0; t < nthreads; t++)
    {
        pthread_join(tids[t], NULL);
        if (tasks[t].rc)
            rc = tasks[t].rc;
    }
    free(offs);
    free(tasks);
    free(tids);
    return rc;
}

#define BODY_PED(C)                                                          \
    {                                                                        \
        size_t m = n + 1;                                                    \
        uint8_t *sc = (uint8_t *)malloc(32 * m);                             \
        C##_jac *pts = (C##_jac *)malloc(m * sizeof(C##_jac));               \
        if (!sc || !pts)                                                     \
        {                                                                    \
            free(sc);                                                        \
            free(pts);                                                       \
            return -2;                                                       \
        }                                                                    \
        memcpy(sc, blinding, 32);                                            \
        if (n)                                                               \
            memcpy(sc + 32, values, 32 * n);                                 \
        C##_load_affine(&pts[0], H64);                                       \
        for (size_t i = 0; i < n; i++)                                       \
            C##_load_affine(&pts[i + 1], gens64 + 64 * i);                   \
        C##_jac r;                                                           \
        C##_msm(&r, sc, pts, m, keep_carry);                                 \
        C##_tobytes(out32, &r);                                              \
        free(sc);                                                            \
        free(pts);                                                           \
    }

int hso_pedersen(int curve, uint8_t out32[32], const uint8_t blinding[32], const uint8_t H64[64],
                 const uint8_t *values, const uint8_t *gens64, size_t n, int keep_carry)
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_PED(helios), BODY_PED(selene));
    return 0;
}

#define BODY_MAP(C)                                \
    for (size_t i = 0; i < n; i++)                 \
    {                                              \
        C##_jac p;                                 \
        C##_map_to_curve(&p, u32s + 32 * i);       \
        C##_store_affine(out64 + 64 * i, &p);      \
    }

int hso_map_to_curve(int curve, uint8_t *out64, const uint8_t *u32s, size_t n)
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_MAP(helios), BODY_MAP(selene));
    return 0;
}

typedef struct
{
    int curve;
    uint8_t *out64;
    const uint8_t *u32s;
    size_t n;
} map_task;

static void *map_worker(void *arg)
{
    map_task *t = (map_task *)arg;
    hso_map_to_curve(t->curve, t->out64, t->u32s, t->n);
    return NULL;
}

int hso_map_to_curve_mt(int curve, uint8_t *out64, const uint8_t *u32s, size_t n, int nthreads)
{
    pthread_once(&g_once, init_consts);
    if (curve != HSO_HELIOS && curve != HSO_SELENE)
        return -1;
    if (nthreads < 1)
        nthreads = 1;
    map_task *tasks = (map_task *)calloc((size_t)nthreads, sizeof(map_task));
    pthread_t *tids = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!tasks || !tids)
    {
        free(tasks);
        free(tids);
        return -2;
    }
    size_t chunk = (n + (size_t)nthreads - 1) / (size_t)nthreads;
    for (int t = 0; t < nthreads; t++)
    {
        size_t lo = (size_t)t * chunk, hi = lo + chunk;
        if (lo > n)
            lo = n;
        if (hi > n)
            hi = n;
        tasks[t].curve = curve;
        tasks[t].out64 = out64 + 64 * lo;
        tasks[t].u32s = u32s + 32 * lo;
        tasks[t].n = hi - lo;
        pthread_create(&tids[t], NULL, map_worker, &tasks[t]);
    }
    for (int t = 0; t < nthreads; t++)
        pthread_join(tids[t], NULL);
    free(tasks);
    free(tids);
    return 0;
}

#define BODY_DEC(C)                                  \
    for (size_t i = 0; i < n; i++)                   \
    {                                                \
        C##_jac p;                                   \
        if (C##_frombytes(&p, in32 + 32 * i) != 0)   \
        {                                            \
            memset(out64 + 64 * i, 0, 64);           \
            bad++;                                   \
            continue;                                \
        }                                            \
        C##_store_affine(out64 + 64 * i, &p);        \
    }

int hso_decompress(int curve, uint8_t *out64, const uint8_t *in32, size_t n)
{
    pthread_once(&g_once, init_consts);
    int bad = 0;
    DISPATCH(curve, BODY_DEC(helios), BODY_DEC(selene));
    return bad;
}

#define BODY_ENC(C)                                  \
    for (size_t i = 0; i < n; i++)                   \
    {                                                \
        C##_jac p;                                   \
        C##_load_affine(&p, in64 + 64 * i);          \
        C##_tobytes(out32 + 32 * i, &p);             \
    }

int hso_compress(int curve, uint8_t *out32, const uint8_t *in64, size_t n)
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_ENC(helios), BODY_ENC(selene));
    return 0;
}

#define BODY_ENCJ(C)                                 \
    for (size_t i = 0; i < n; i++)                   \
    {                                                \
        C##_jac p;                                   \
        C##_load_jac(&p, in96 + 96 * i);             \
        C##_tobytes(out32 + 32 * i, &p);             \
    }

int hso_compress_jac(int curve, uint8_t *out32, const uint8_t *in96, size_t n)
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_ENCJ(helios), BODY_ENCJ(selene));
    return 0;
}

/* Montgomery batch inversion with zero -> zero (fp/include/fp_batch_invert.h:61-114) */
#define BODY_BINV(FF)                                                   \
    {                                                                   \
        fe *in = (fe *)malloc((n ? n : 1) * sizeof(fe));                \
        fe *acc = (fe *)malloc((n ? n : 1) * sizeof(fe));               \
        if (!in || !acc)                                                \
        {                                                               \
            free(in);                                                   \
            free(acc);                                                  \
            return -2;                                                  \
        }                                                               \
        for (size_t i = 0; i < n; i++)                                  \
            FF##_load32(&in[i], in32 + 32 * i);                         \
        fe run;                                                         \
        FF##_set_u64(&run, 1);                                          \
        for (size_t i = 0; i < n; i++)                                  \
        {                                                               \
            if (!FF##_iszero(&in[i]))                                   \
                FF##_mul(&run, &run, &in[i]);                           \
            acc[i] = run;                                               \
        }                                                               \
        fe inv;                                                         \
        FF##_inv(&inv, &run);                                           \
        for (size_t i = n; i-- > 0;)                                    \
        {                                                               \
            fe r;                                                       \
            if (FF##_iszero(&in[i]))                                    \
            {                                                           \
                FF##_set_u64(&r, 0);                                    \
            }                                                           \
            else                                                        \
            {                                                           \
                fe prev;                                                \
                if (i)                                                  \
                    prev = acc[i - 1];                                  \
                else                                                    \
                    FF##_set_u64(&prev, 1);                             \
                FF##_mul(&r, &inv, &prev);                              \
                FF##_mul(&inv, &inv, &in[i]);                           \
            }                                                           \
            FF##_tobytes(out32 + 32 * i, &r);                           \
        }                                                               \
        free(in);                                                       \
        free(acc);                                                      \
    }

int hso_batch_invert(int field, uint8_t *out32, const uint8_t *in32, size_t n)
{
    pthread_once(&g_once, init_consts);
    if (field == HSO_FIELD_P)
        BODY_BINV(fp)
    else if (field == HSO_FIELD_Q)
        BODY_BINV(fq)
    else
        return -1;
    return 0;
}

/* batch Jacobian -> affine, identity -> (0,0) (helios/include/helios_batch_affine.h:55-98) */
#define BODY_B2A(C)                                  \
    for (size_t i = 0; i < n; i++)                   \
    {                                                \
        C##_jac p;                                   \
        C##_load_jac(&p, in96 + 96 * i);             \
        C##_store_affine(out64 + 64 * i, &p);        \
    }

int hso_batch_to_affine(int curve, uint8_t *out64, const uint8_t *in96, size_t n)
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_B2A(helios), BODY_B2A(selene));
    return 0;
}

#define BODY_SMUL(C)                                 \
    {                                                \
        C##_jac p, r;                                \
        C##_load_affine(&p, pt64);                   \
        C##_scalar_mul(&r, scalar, &p);              \
        C##_store_affine(out64, &r);                 \
    }

int hso_scalar_mul(int curve, uint8_t out64[64], const uint8_t scalar[32], const uint8_t pt64[64])
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_SMUL(helios), BODY_SMUL(selene));
    return 0;
}

#define BODY_ADD(C)                                  \
    {                                                \
        C##_jac a, b, r;                             \
        C##_load_affine(&a, a64);                    \
        C##_load_affine(&b, b64);                    \
        C##_add_safe(&r, &a, &b);                    \
        C##_store_affine(out64, &r);                 \
    }

int hso_point_add(int curve, uint8_t out64[64], const uint8_t a64[64], const uint8_t b64[64])
{
    pthread_once(&g_once, init_consts);
    DISPATCH(curve, BODY_ADD(helios), BODY_ADD(selene));
    return 0;
}

/* radix-2^51 limbs (the reference's fp_fe / fq_fe on 64-bit hosts, fp/include/fp.h:42-46)
 * -> canonical bytes.  Limbs may be lazy (above 2^51). */
int hso_fe51_to_bytes(int field, uint8_t out32[32], const uint64_t limbs[5])
{
    uint64_t w[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 5; i++)
    {
        int bit = 51 * i;
        int word = bit >> 6, off = bit & 63;
        u128 v = (u128)limbs[i] << off;
        for (int k = word; k < 5 && v; k++)
        {
            u128 s = (u128)w[k] + (uint64_t)v;
            w[k] = (uint64_t)s;
            v = (v >> 64) + (s >> 64);
        }
    }
    fe r = {{w[0], w[1], w[2], w[3]}};
    if (field == HSO_FIELD_P)
    {
        fp_carry_c(&r, w[4]);
        fp_tobytes(out32, &r);
    }
    else if (field == HSO_FIELD_Q)
    {
        /* w[4] < 2^12: fold it with repeated single-step carries */
        for (uint64_t k = w[4]; k > 0;)
        {
            uint64_t step = k > 255 ? 255 : k;
            fq_carry_c(&r, step);
            k -= step;
        }
        fq_tobytes(out32, &r);
    }
    else
        return -1;
    return 0;
}

int hso_abi_version(void) { return 1; }
