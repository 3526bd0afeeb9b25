/*
 * Field arithmetic template for the oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * Included twice by hs_oracle.c, once per field of the Helios/Selene cycle:
 *   F_p, p = 2^255 - 19            (Helios coordinates, Selene scalars)
 *   F_q, q = 2^255 - gamma         (Selene coordinates, Helios scalars)
 * Both moduli satisfy 2^256 == c (mod m) with a small c < 2^128
 * (c = 38 for p, c = 2*gamma for q; the reference folds the same way:
 * fp/include/x64/fp51_inline.h:46-146 folds by 19 at 2^255,
 * fq/include/x64/fq51.h:53-62 states 2^256 == 2*gamma mod q).
 *
 * Representation: four 64-bit limbs, little endian, value in [0, 2^256)
 * ("weakly reduced": congruent to the field element, not necessarily < m).
 * Canonical form (< m) is produced only where bytes leave the field,
 * mirroring fp_tobytes / fq_tobytes (fp/src/x64/fp_tobytes.cpp:31-114,
 * fq/src/x64/fq_tobytes.cpp:44-143).
 *
 * Required macros: FE(name) -> prefixed function name, FE_M0..FE_M3 (modulus
 * limbs), FE_C0, FE_C1 (c = 2^256 mod m, two limbs).
 */

static inline void FE(carry_c)(fe *r, uint64_t k)
{
    /* r += k * c, k small (< 2^8); wraps once at most, handled by caller */
    u128 t;
    uint64_t carry;
    t = (u128)r->v[0] + (u128)k * FE_C0;
    r->v[0] = (uint64_t)t;
    t = (u128)r->v[1] + (u128)k * FE_C1 + (t >> 64);
    r->v[1] = (uint64_t)t;
    t = (u128)r->v[2] + (t >> 64);
    r->v[2] = (uint64_t)t;
    t = (u128)r->v[3] + (t >> 64);
    r->v[3] = (uint64_t)t;
    carry = (uint64_t)(t >> 64);
    if (carry)
    {
        /* value wrapped past 2^256: the low part is < k*c, adding c again cannot wrap */
        t = (u128)r->v[0] + FE_C0;
        r->v[0] = (uint64_t)t;
        t = (u128)r->v[1] + FE_C1 + (t >> 64);
        r->v[1] = (uint64_t)t;
        t = (u128)r->v[2] + (t >> 64);
        r->v[2] = (uint64_t)t;
        r->v[3] += (uint64_t)(t >> 64);
    }
}

static inline void FE(add)(fe *r, const fe *a, const fe *b)
{
    u128 t = 0;
    for (int i = 0; i < 4; i++)
    {
        t = (u128)a->v[i] + b->v[i] + (t >> 64);
        r->v[i] = (uint64_t)t;
    }
    FE(carry_c)(r, (uint64_t)(t >> 64));
}

static inline void FE(sub)(fe *r, const fe *a, const fe *b)
{
    /* a - b; on borrow the wrapped value is a - b + 2^256 == a - b + c, so subtract c */
    uint64_t borrow = 0;
    for (int i = 0; i < 4; i++)
    {
        u128 t = (u128)a->v[i] - b->v[i] - borrow;
        r->v[i] = (uint64_t)t;
        borrow = (uint64_t)(t >> 64) & 1;
    }
    for (int round = 0; round < 2 && borrow; round++)
    {
        u128 t = (u128)r->v[0] - FE_C0;
        r->v[0] = (uint64_t)t;
        uint64_t bw = (uint64_t)(t >> 64) & 1;
        t = (u128)r->v[1] - FE_C1 - bw;
        r->v[1] = (uint64_t)t;
        bw = (uint64_t)(t >> 64) & 1;
        t = (u128)r->v[2] - bw;
        r->v[2] = (uint64_t)t;
        bw = (uint64_t)(t >> 64) & 1;
        t = (u128)r->v[3] - bw;
        r->v[3] = (uint64_t)t;
        borrow = (uint64_t)(t >> 64) & 1;
    }
}

static inline void FE(mul)(fe *r, const fe *a, const fe *b)
{
    uint64_t t[8] = {0};
    for (int i = 0; i < 4; i++)
    {
        u128 acc = 0;
        for (int j = 0; j < 4; j++)
        {
            acc = (u128)a->v[i] * b->v[j] + t[i + j] + (acc >> 64);
            t[i + j] = (uint64_t)acc;
        }
        t[i + 4] = (uint64_t)(acc >> 64);
    }
    /* fold 1: s = lo + hi * c.  hi < 2^256 and c < 2^128 (for q, c = 2*gamma < 2^127.02),
       so s < 2^384: six limbs. */
    uint64_t s[6];
    u128 acc = 0;
    for (int i = 0; i < 4; i++)
    {
        acc = (u128)t[4 + i] * FE_C0 + t[i] + (acc >> 64);
        s[i] = (uint64_t)acc;
    }
    s[4] = (uint64_t)(acc >> 64);
    s[5] = 0;
    if (FE_C1)
    {
        acc = 0;
        for (int i = 0; i < 4; i++)
        {
            acc = (u128)t[4 + i] * FE_C1 + s[i + 1] + (acc >> 64);
            s[i + 1] = (uint64_t)acc;
        }
        s[5] += (uint64_t)(acc >> 64);
    }
    /* fold 2: o = s[0..3] + H * c with H = s[4] + s[5]*2^64 < 2^128, so o < 2^257 */
    uint64_t o[5] = {s[0], s[1], s[2], s[3], 0};
    acc = 0;
    for (int i = 0; i < 2; i++)
    {
        acc = (u128)s[4 + i] * FE_C0 + o[i] + (acc >> 64);
        o[i] = (uint64_t)acc;
    }
    for (int i = 2; i < 5; i++)
    {
        acc = (u128)o[i] + (acc >> 64);
        o[i] = (uint64_t)acc;
    }
    if (FE_C1)
    {
        acc = 0;
        for (int i = 0; i < 2; i++)
        {
            acc = (u128)s[4 + i] * FE_C1 + o[i + 1] + (acc >> 64);
            o[i + 1] = (uint64_t)acc;
        }
        for (int i = 3; i < 5; i++)
        {
            acc = (u128)o[i] + (acc >> 64);
            o[i] = (uint64_t)acc;
        }
    }
    fe res = {{o[0], o[1], o[2], o[3]}};
    /* fold 3: o[4] <= 1 */
    FE(carry_c)(&res, o[4]);
    *r = res;
}

static inline void FE(sq)(fe *r, const fe *a) { FE(mul)(r, a, a); }

/* canonical representative in [0, m).  m < 2^255 and 2m = 2^256 - c, so a value
 * below 2^256 lies in [0, 2m + c): subtract 2m when a + c carries, then m once more. */
static inline void FE(canon)(fe *r, const fe *a)
{
    static const uint64_t M[4] = {FE_M0, FE_M1, FE_M2, FE_M3};
    fe v, t;
    u128 acc = (u128)a->v[0] + FE_C0;
    t.v[0] = (uint64_t)acc;
    acc = (u128)a->v[1] + FE_C1 + (acc >> 64);
    t.v[1] = (uint64_t)acc;
    acc = (u128)a->v[2] + (acc >> 64);
    t.v[2] = (uint64_t)acc;
    acc = (u128)a->v[3] + (acc >> 64);
    t.v[3] = (uint64_t)acc;
    v = ((uint64_t)(acc >> 64)) ? t : *a;
    uint64_t borrow = 0;
    for (int i = 0; i < 4; i++)
    {
        u128 d = (u128)v.v[i] - M[i] - borrow;
        t.v[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 64) & 1;
    }
    *r = borrow ? v : t;
}

static inline int FE(iszero)(const fe *a)
{
    fe c;
    FE(canon)(&c, a);
    return (c.v[0] | c.v[1] | c.v[2] | c.v[3]) == 0;
}

static inline int FE(eq)(const fe *a, const fe *b)
{
    fe d;
    FE(sub)(&d, a, b);
    return FE(iszero)(&d);
}

static inline void FE(neg)(fe *r, const fe *a)
{
    fe z = {{0, 0, 0, 0}};
    FE(sub)(r, &z, a);
}

static inline void FE(set_u64)(fe *r, uint64_t v)
{
    r->v[0] = v;
    r->v[1] = r->v[2] = r->v[3] = 0;
}

/* canonical 32-byte little-endian encoding */
static inline void FE(tobytes)(uint8_t s[32], const fe *a)
{
    fe c;
    FE(canon)(&c, a);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 8; j++)
            s[8 * i + j] = (uint8_t)(c.v[i] >> (8 * j));
}

/* 32 bytes -> element, bit 255 masked, no reduction (fp/src/x64/fp_frombytes.cpp:31-54) */
static inline void FE(frombytes)(fe *r, const uint8_t s[32])
{
    for (int i = 0; i < 4; i++)
    {
        uint64_t w = 0;
        for (int j = 0; j < 8; j++)
            w |= (uint64_t)s[8 * i + j] << (8 * j);
        r->v[i] = w;
    }
    r->v[3] &= 0x7fffffffffffffffULL;
}

/* full 256-bit load (no masking), used for canonical-affine exchange buffers */
static inline void FE(load32)(fe *r, const uint8_t s[32])
{
    for (int i = 0; i < 4; i++)
    {
        uint64_t w = 0;
        for (int j = 0; j < 8; j++)
            w |= (uint64_t)s[8 * i + j] << (8 * j);
        r->v[i] = w;
    }
}

static inline int FE(isnegative)(const fe *a)
{
    fe c;
    FE(canon)(&c, a);
    return (int)(c.v[0] & 1);
}

/* r = a^e for a 256-bit exponent e (square-and-multiply, 4-bit fixed window) */
static inline void FE(pow)(fe *r, const fe *a, const uint64_t e[4])
{
    fe tab[16];
    FE(set_u64)(&tab[0], 1);
    tab[1] = *a;
    for (int i = 2; i < 16; i++)
        FE(mul)(&tab[i], &tab[i - 1], a);
    fe acc;
    FE(set_u64)(&acc, 1);
    for (int i = 63; i >= 0; i--)
    {
        for (int k = 0; k < 4; k++)
            FE(sq)(&acc, &acc);
        unsigned nib = (unsigned)(e[i / 16] >> (4 * (i % 16))) & 15;
        if (nib)
            FE(mul)(&acc, &acc, &tab[nib]);
    }
    *r = acc;
}

/* inversion by Fermat: a^(m-2); 0 maps to 0 (the reference's inv0 semantics,
 * helios/src/x64/helios_map_to_curve.cpp:127 relies on it) */
static inline void FE(inv)(fe *r, const fe *a)
{
    static const uint64_t e[4] = {FE_M0 - 2, FE_M1, FE_M2, FE_M3};
    FE(pow)(r, a, e);
}
