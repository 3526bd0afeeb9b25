/*
 * Curve template for the oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * Included once per curve by hs_oracle.c.  Required macros:
 *   CV(name)  -> curve-prefixed name (helios_/selene_)
 *   F(name)   -> coordinate-field function (fp_/fq_)
 *   CV_B      -> pointer to the curve constant b (fe)
 *   CV_SSWU_Z -> small signed integer Z of the SWU map
 *
 * Both curves are y^2 = x^3 - 3x + b (helios/include/helios_constants.h:36-41,
 * selene/include/selene_constants.h:36-41).  Points are Jacobian (X:Y:Z),
 * x = X/Z^2, y = Y/Z^3, identity has Z == 0 (helios/include/helios_ops.h:45-64).
 */

typedef struct
{
    fe X, Y, Z;
} CV(jac);

static inline void CV(identity)(CV(jac) * r)
{
    F(set_u64)(&r->X, 1);
    F(set_u64)(&r->Y, 1);
    F(set_u64)(&r->Z, 0);
}

static inline int CV(is_identity)(const CV(jac) * p) { return F(iszero)(&p->Z); }

static inline void CV(neg)(CV(jac) * r, const CV(jac) * p)
{
    r->X = p->X;
    F(neg)(&r->Y, &p->Y);
    r->Z = p->Z;
}

/* dbl-2001-b with a = -3, 3M+5S (helios/src/x64/helios_dbl.cpp:45-88) */
static void CV(dbl)(CV(jac) * r, const CV(jac) * p)
{
    fe delta, gamma, beta, alpha, t0, t1, t2;
    F(sq)(&delta, &p->Z);
    F(sq)(&gamma, &p->Y);
    F(mul)(&beta, &p->X, &gamma);
    F(sub)(&t0, &p->X, &delta);
    F(add)(&t1, &p->X, &delta);
    F(mul)(&alpha, &t0, &t1);
    F(add)(&t0, &alpha, &alpha);
    F(add)(&alpha, &t0, &alpha);
    fe X3, Y3, Z3;
    F(sq)(&X3, &alpha);
    F(add)(&t0, &beta, &beta);
    F(add)(&t0, &t0, &t0);
    F(sub)(&X3, &X3, &t0);
    F(sub)(&X3, &X3, &t0);
    F(add)(&t1, &p->Y, &p->Z);
    F(sq)(&t2, &t1);
    F(sub)(&t2, &t2, &gamma);
    F(sub)(&Z3, &t2, &delta);
    F(sub)(&t1, &t0, &X3);
    F(mul)(&t2, &alpha, &t1);
    F(sq)(&t0, &gamma);
    F(add)(&t0, &t0, &t0);
    F(add)(&t0, &t0, &t0);
    F(sub)(&Y3, &t2, &t0);
    F(sub)(&Y3, &Y3, &t0);
    r->X = X3;
    r->Y = Y3;
    r->Z = Z3;
}

/* add-2007-bl, 11M+5S, incomplete (helios/src/x64/helios_add.cpp:52-107) */
static void CV(add_raw)(CV(jac) * r, const CV(jac) * p, const CV(jac) * q)
{
    fe Z1Z1, Z2Z2, U1, U2, S1, S2, H, I, J, rr, V, t0, t1;
    F(sq)(&Z1Z1, &p->Z);
    F(sq)(&Z2Z2, &q->Z);
    F(mul)(&U1, &p->X, &Z2Z2);
    F(mul)(&U2, &q->X, &Z1Z1);
    F(mul)(&t0, &q->Z, &Z2Z2);
    F(mul)(&S1, &p->Y, &t0);
    F(mul)(&t0, &p->Z, &Z1Z1);
    F(mul)(&S2, &q->Y, &t0);
    F(sub)(&H, &U2, &U1);
    F(add)(&t0, &H, &H);
    F(sq)(&I, &t0);
    F(mul)(&J, &H, &I);
    F(sub)(&rr, &S2, &S1);
    F(add)(&rr, &rr, &rr);
    F(mul)(&V, &U1, &I);
    fe X3, Y3, Z3;
    F(sq)(&X3, &rr);
    F(sub)(&X3, &X3, &J);
    F(add)(&t0, &V, &V);
    F(sub)(&X3, &X3, &t0);
    F(sub)(&t0, &V, &X3);
    F(mul)(&t1, &rr, &t0);
    F(mul)(&t0, &S1, &J);
    F(add)(&t0, &t0, &t0);
    F(sub)(&Y3, &t1, &t0);
    F(add)(&t0, &p->Z, &q->Z);
    F(sq)(&t1, &t0);
    F(sub)(&t1, &t1, &Z1Z1);
    F(sub)(&t1, &t1, &Z2Z2);
    F(mul)(&Z3, &t1, &H);
    r->X = X3;
    r->Y = Y3;
    r->Z = Z3;
}

/* complete variable-time addition: identity, P == Q, P == -Q
 * (helios/src/x64/helios_msm_vartime.cpp:59-104) */
static void CV(add_safe)(CV(jac) * r, const CV(jac) * p, const CV(jac) * q)
{
    if (CV(is_identity)(p))
    {
        *r = *q;
        return;
    }
    if (CV(is_identity)(q))
    {
        *r = *p;
        return;
    }
    fe z1z1, z2z2, u1, u2, d;
    F(sq)(&z1z1, &p->Z);
    F(sq)(&z2z2, &q->Z);
    F(mul)(&u1, &p->X, &z2z2);
    F(mul)(&u2, &q->X, &z1z1);
    F(sub)(&d, &u1, &u2);
    if (F(iszero)(&d))
    {
        fe s1, s2, t;
        F(mul)(&t, &q->Z, &z2z2);
        F(mul)(&s1, &p->Y, &t);
        F(mul)(&t, &p->Z, &z1z1);
        F(mul)(&s2, &q->Y, &t);
        F(sub)(&d, &s1, &s2);
        if (F(iszero)(&d))
            CV(dbl)(r, p);
        else
            CV(identity)(r);
        return;
    }
    CV(add_raw)(r, p, q);
}

/* Jacobian -> canonical affine; identity -> (0,0) (helios/include/helios_batch_affine.h:55-98) */
static void CV(to_affine)(fe *x, fe *y, const CV(jac) * p)
{
    if (CV(is_identity)(p))
    {
        F(set_u64)(x, 0);
        F(set_u64)(y, 0);
        return;
    }
    fe zi, zi2, zi3;
    F(inv)(&zi, &p->Z);
    F(sq)(&zi2, &zi);
    F(mul)(&zi3, &zi2, &zi);
    F(mul)(x, &p->X, &zi2);
    F(mul)(y, &p->Y, &zi3);
    F(canon)(x, x);
    F(canon)(y, y);
}

/* 32-byte encoding: x LE, bit 255 = parity of y, identity = zeros
 * (helios/src/x64/helios_tobytes.cpp:42-66) */
static void CV(tobytes)(uint8_t s[32], const CV(jac) * p)
{
    if (CV(is_identity)(p))
    {
        memset(s, 0, 32);
        return;
    }
    fe x, y;
    CV(to_affine)(&x, &y, p);
    F(tobytes)(s, &x);
    s[31] |= (uint8_t)(F(isnegative)(&y) << 7);
}

/* rhs = x^3 - 3x + b */
static void CV(rhs)(fe *r, const fe *x)
{
    fe x2, x3, t;
    F(sq)(&x2, x);
    F(mul)(&x3, &x2, x);
    F(add)(&t, x, x);
    F(add)(&t, &t, x);
    F(sub)(r, &x3, &t);
    F(add)(r, r, CV_B);
}

/* decode (helios/src/x64/helios_frombytes.cpp:59-109): returns 0 / -1 */
static int CV(frombytes)(CV(jac) * r, const uint8_t s[32])
{
    unsigned parity = (s[31] >> 7) & 1;
    uint8_t xb[32], chk[32];
    memcpy(xb, s, 32);
    xb[31] &= 0x7f;
    fe x;
    F(frombytes)(&x, xb);
    F(tobytes)(chk, &x);
    if (memcmp(chk, xb, 32) != 0)
        return -1;
    fe rhs, y;
    CV(rhs)(&rhs, &x);
    if (F(sqrt)(&y, &rhs) != 0)
        return -1;
    if ((unsigned)F(isnegative)(&y) != parity)
        F(neg)(&y, &y);
    r->X = x;
    r->Y = y;
    F(set_u64)(&r->Z, 1);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Signed-digit recoding (helios/src/x64/helios_msm_vartime.cpp:110-162)
 * ------------------------------------------------------------------------- */

/* 64 signed radix-16 digits; the top digit keeps the final carry */
static void CV(encode_signed_w4)(int16_t *digits, const uint8_t *scalar)
{
    int carry = 0;
    for (int i = 0; i < 31; i++)
    {
        carry += scalar[i];
        int c2 = (carry + 8) >> 4;
        digits[2 * i] = (int16_t)(carry - (c2 << 4));
        carry = (c2 + 8) >> 4;
        digits[2 * i + 1] = (int16_t)(c2 - (carry << 4));
    }
    carry += scalar[31];
    int c2 = (carry + 8) >> 4;
    digits[62] = (int16_t)(carry - (c2 << 4));
    digits[63] = (int16_t)c2;
}

#ifndef HS_CURVE_COMMON_BITS
#define HS_CURVE_COMMON_BITS
static int scalar_bits(const uint8_t *s, int pos, int w)
{
    int v = 0;
    for (int b = 0; b < w; b++)
    {
        int bit = pos + b;
        if (bit < 256)
            v |= ((s[bit >> 3] >> (bit & 7)) & 1) << b;
    }
    return v;
}

#endif

/* ceil(256/w) signed digits in [-2^(w-1), 2^(w-1)).  The reference drops the
 * carry out of the last digit; with keep_carry the carry becomes one extra
 * digit, which makes the recoding exact for every w. Returns the digit count. */
static int CV(encode_signed_wbit)(int16_t *digits, const uint8_t *scalar, int w, int keep_carry)
{
    const int half = 1 << (w - 1);
    const int mask = (1 << w) - 1;
    const int nd = (256 + w - 1) / w;
    int carry = 0;
    for (int i = 0; i < nd; i++)
    {
        int val = (scalar_bits(scalar, i * w, w) & mask) + carry;
        carry = val >> w;
        val &= mask;
        if (val >= half)
        {
            val -= (1 << w);
            carry = 1;
        }
        digits[i] = (int16_t)val;
    }
    if (keep_carry)
    {
        digits[nd] = (int16_t)carry;
        return nd + 1;
    }
    return nd;
}

#ifndef HS_CURVE_COMMON_WINDOW
#define HS_CURVE_COMMON_WINDOW
/* window rule (helios/src/x64/helios_msm_vartime.cpp:248-263) */
static int pippenger_window(size_t n)
{
    if (n < 96)
        return 5;
    if (n < 288)
        return 6;
    if (n < 864)
        return 7;
    if (n < 2592)
        return 8;
    if (n < 7776)
        return 9;
    if (n < 23328)
        return 10;
    return 11;
}

#endif

/* Straus, n <= 16 (helios/src/x64/helios_msm_vartime.cpp:168-242).  The table
 * holds 16 multiples instead of 8 so that a top digit of up to 16 (scalars with
 * byte 31 >= 0x78, i.e. not reduced) stays in bounds; for reduced scalars the
 * extra entries are never read. */
static void CV(straus)(CV(jac) * result, const uint8_t *scalars, const CV(jac) * points, size_t n)
{
    int16_t *dig = (int16_t *)malloc(n * 64 * sizeof(int16_t));
    CV(jac) *tab = (CV(jac) *)malloc(n * 16 * sizeof(CV(jac)));
    for (size_t i = 0; i < n; i++)
    {
        CV(encode_signed_w4)(dig + i * 64, scalars + i * 32);
        CV(jac) *T = tab + i * 16;
        T[0] = points[i];
        CV(dbl)(&T[1], &points[i]);
        for (int j = 1; j < 15; j++)
            CV(add_safe)(&T[j + 1], &T[j], &points[i]);
    }
    CV(jac) acc;
    CV(identity)(&acc);
    int acc_id = 1;
    for (int d = 63; d >= 0; d--)
    {
        if (!acc_id)
            for (int k = 0; k < 4; k++)
                CV(dbl)(&acc, &acc);
        for (size_t i = 0; i < n; i++)
        {
            int dg = dig[i * 64 + (size_t)d];
            if (dg == 0)
                continue;
            CV(jac) pt;
            if (dg > 0)
                pt = tab[i * 16 + (size_t)(dg - 1)];
            else
                CV(neg)(&pt, &tab[i * 16 + (size_t)(-dg - 1)]);
            if (acc_id)
            {
                acc = pt;
                acc_id = 0;
            }
            else
                CV(add_safe)(&acc, &acc, &pt);
        }
    }
    free(dig);
    free(tab);
    if (acc_id)
        CV(identity)(result);
    else
        *result = acc;
}

/* Pippenger (helios/src/x64/helios_msm_vartime.cpp:265-388): per window,
 * MSB first, Horner doubling, bucket fill, running-sum reduction. */
static void CV(pippenger)(CV(jac) * result, const uint8_t *scalars, const CV(jac) * points, size_t n, int keep_carry, int w_override)
{
    const int w = w_override > 0 ? w_override : pippenger_window(n);
    const size_t nb = (size_t)1 << (w - 1);
    const int maxd = (256 + w - 1) / w + 1;
    int16_t *dig = (int16_t *)malloc(n * (size_t)maxd * sizeof(int16_t));
    int nw = 0;
    for (size_t i = 0; i < n; i++)
        nw = CV(encode_signed_wbit)(dig + i * (size_t)maxd, scalars + i * 32, w, keep_carry);
    CV(jac) *bk = (CV(jac) *)malloc(nb * sizeof(CV(jac)));
    unsigned char *bk_id = (unsigned char *)malloc(nb);
    CV(jac) total;
    CV(identity)(&total);
    int total_id = 1;
    for (int win = nw - 1; win >= 0; win--)
    {
        if (!total_id)
            for (int d = 0; d < w; d++)
                CV(dbl)(&total, &total);
        memset(bk_id, 1, nb);
        for (size_t i = 0; i < n; i++)
        {
            int dg = dig[i * (size_t)maxd + (size_t)win];
            if (dg == 0)
                continue;
            size_t b;
            CV(jac) ep;
            if (dg > 0)
            {
                b = (size_t)(dg - 1);
                ep = points[i];
            }
            else
            {
                b = (size_t)(-dg - 1);
                CV(neg)(&ep, &points[i]);
            }
            if (bk_id[b])
            {
                bk[b] = ep;
                bk_id[b] = 0;
            }
            else
                CV(add_safe)(&bk[b], &bk[b], &ep);
        }
        CV(jac) run, part;
        int run_id = 1, part_id = 1;
        for (size_t j = nb; j-- > 0;)
        {
            if (!bk_id[j])
            {
                if (run_id)
                {
                    run = bk[j];
                    run_id = 0;
                }
                else
                    CV(add_safe)(&run, &run, &bk[j]);
            }
            if (!run_id)
            {
                if (part_id)
                {
                    part = run;
                    part_id = 0;
                }
                else
                    CV(add_safe)(&part, &part, &run);
            }
        }
        if (!part_id)
        {
            if (total_id)
            {
                total = part;
                total_id = 0;
            }
            else
                CV(add_safe)(&total, &total, &part);
        }
    }
    free(dig);
    free(bk);
    free(bk_id);
    if (total_id)
        CV(identity)(result);
    else
        *result = total;
}

/* dispatcher (helios/src/x64/helios_msm_vartime.cpp:394-416) */
static void CV(msm)(CV(jac) * result, const uint8_t *scalars, const CV(jac) * points, size_t n, int keep_carry)
{
    if (n == 0)
    {
        CV(identity)(result);
        return;
    }
    if (n <= 16)
        CV(straus)(result, scalars, points, n);
    else
        CV(pippenger)(result, scalars, points, n, keep_carry, 0);
}

/* double-and-add scalar multiple, any 256-bit scalar; used for naive sums */
static void CV(scalar_mul)(CV(jac) * r, const uint8_t s[32], const CV(jac) * p)
{
    CV(jac) acc;
    CV(identity)(&acc);
    for (int bit = 255; bit >= 0; bit--)
    {
        CV(dbl)(&acc, &acc);
        if ((s[bit >> 3] >> (bit & 7)) & 1)
            CV(add_safe)(&acc, &acc, p);
    }
    *r = acc;
}

/* Simplified SWU, RFC 9380 6.6.2 (helios/src/x64/helios_map_to_curve.cpp:98-198):
 * x1 = (-B/A)(1 + 1/(Z^2u^4 + Zu^2)), or B/(ZA) when the denominator is 0;
 * x = x1 if g(x1) is square else Z u^2 x1; sgn0(y) = sgn0(u).  Output Z = 1. */
static void CV(map_to_curve)(CV(jac) * r, const uint8_t ub[32])
{
    fe u, A, Z, Zabs, u2, Zu2, den, t, inv_den, x1, x2, gx1, gx2, y1, y2 = {{0, 0, 0, 0}}, one;
    F(frombytes)(&u, ub);
    F(set_u64)(&one, 1);
    F(set_u64)(&A, 3);
    F(neg)(&A, &A);
    int zs = CV_SSWU_Z;
    F(set_u64)(&Zabs, (uint64_t)(zs < 0 ? -zs : zs));
    if (zs < 0)
        F(neg)(&Z, &Zabs);
    else
        Z = Zabs;
    F(sq)(&u2, &u);
    F(mul)(&Zu2, &Z, &u2);
    F(sq)(&t, &Zu2);
    F(add)(&den, &t, &Zu2);
    if (F(iszero)(&den))
    {
        /* x1 = B / (Z*A) */
        F(mul)(&t, &Z, &A);
        F(inv)(&t, &t);
        F(mul)(&x1, CV_B, &t);
    }
    else
    {
        /* x1 = (-B/A) * (1 + 1/den) */
        F(inv)(&inv_den, &den);
        F(add)(&inv_den, &inv_den, &one);
        F(inv)(&t, &A);
        F(mul)(&t, &t, CV_B);
        F(neg)(&t, &t);
        F(mul)(&x1, &t, &inv_den);
    }
    CV(rhs)(&gx1, &x1);
    fe x, y;
    if (F(sqrt)(&y1, &gx1) == 0)
    {
        x = x1;
        y = y1;
    }
    else
    {
        F(mul)(&x2, &Zu2, &x1);
        CV(rhs)(&gx2, &x2);
        F(sqrt)(&y2, &gx2);
        x = x2;
        y = y2;
    }
    if (F(isnegative)(&u) != F(isnegative)(&y))
        F(neg)(&y, &y);
    F(canon)(&r->X, &x);
    F(canon)(&r->Y, &y);
    F(set_u64)(&r->Z, 1);
}
