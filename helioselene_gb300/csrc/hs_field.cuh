// hs_field.cuh -- F_p and F_q arithmetic for sm_103a on the integer-multiply pipe.
//
//   F_p, p = 2^255 - 19      (Helios coordinates)   2^256 == 38       (mod p)
//   F_q, q = 2^255 - gamma   (Selene coordinates)   2^256 == 2*gamma  (mod q)
//
// The reference keeps radix-2^51 limbs and folds by 19 / gamma
// (fp/include/x64/fp51_inline.h:46-243, fq/include/x64/fq51_inline.h:1087-1225,
// constants fq/include/x64/fq51.h:38-86).  Here an element is eight 32-bit
// limbs (little endian) holding any value in [0, 2^256) congruent to it
// ("weakly reduced"); the canonical value < m is produced only at the edges.
// Products are 8x8 schoolbook rows of mad.lo/madc.hi carry chains (even and
// odd partial products in separate chains so no carry has to be spilled),
// followed by a fold of the high half by c = 2^256 mod m.

#pragma once
#include <cstdint>

namespace hs {

struct Fe {
    uint32_t w[8];
};

// ---------------------------------------------------------------------------
// field parameter sets
// ---------------------------------------------------------------------------
struct FpParams {
    // p = 2^255 - 19
    static constexpr uint32_t M[8] = {0xffffffedu, 0xffffffffu, 0xffffffffu, 0xffffffffu,
                                      0xffffffffu, 0xffffffffu, 0xffffffffu, 0x7fffffffu};
    // c = 2^256 mod p = 38 (one limb)
    static constexpr int NC = 1;
    static constexpr uint32_t C[4] = {38u, 0u, 0u, 0u};
};

struct FqParams {
    // q = 2^255 - gamma, gamma = 85737960593035654572250192257530476641
    static constexpr uint32_t M[8] = {0x7927c79fu, 0x6eb6d272u, 0xb7656b58u, 0xbf7f782cu,
                                      0xffffffffu, 0xffffffffu, 0xffffffffu, 0x7fffffffu};
    // c = 2^256 mod q = 2*gamma (four limbs)
    static constexpr int NC = 4;
    static constexpr uint32_t C[4] = {0x0db070c2u, 0x22925b1bu, 0x9135294fu, 0x81010fa6u};
};

// ---------------------------------------------------------------------------
// raw 256-bit helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mul_wide_8x8(uint32_t t[16], const uint32_t a[8], const uint32_t b[8])
{
    // row 0: even products straight into t[0..7], odd products chained on top
    asm("mul.lo.u32 %0, %2, %3;\n\tmul.hi.u32 %1, %2, %3;" : "=r"(t[0]), "=r"(t[1]) : "r"(a[0]), "r"(b[0]));
    asm("mul.lo.u32 %0, %2, %3;\n\tmul.hi.u32 %1, %2, %3;" : "=r"(t[2]), "=r"(t[3]) : "r"(a[2]), "r"(b[0]));
    asm("mul.lo.u32 %0, %2, %3;\n\tmul.hi.u32 %1, %2, %3;" : "=r"(t[4]), "=r"(t[5]) : "r"(a[4]), "r"(b[0]));
    asm("mul.lo.u32 %0, %2, %3;\n\tmul.hi.u32 %1, %2, %3;" : "=r"(t[6]), "=r"(t[7]) : "r"(a[6]), "r"(b[0]));
    asm("{\n\t"
        "mad.lo.cc.u32  %0, %8, %12, %0;\n\t"
        "madc.hi.cc.u32 %1, %8, %12, %1;\n\t"
        "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"
        "madc.hi.cc.u32 %3, %9, %12, %3;\n\t"
        "madc.lo.cc.u32 %4, %10, %12, %4;\n\t"
        "madc.hi.cc.u32 %5, %10, %12, %5;\n\t"
        "madc.lo.cc.u32 %6, %11, %12, %6;\n\t"
        "madc.hi.u32    %7, %11, %12, 0;\n\t"
        "}"
        : "+r"(t[1]), "+r"(t[2]), "+r"(t[3]), "+r"(t[4]), "+r"(t[5]), "+r"(t[6]), "+r"(t[7]), "=r"(t[8])
        : "r"(a[1]), "r"(a[3]), "r"(a[5]), "r"(a[7]), "r"(b[0]));
#pragma unroll
    for (int i = 1; i < 8; i++) {
        // even chain: t[i..i+7] += a[0,2,4,6] * b[i]; carry -> fresh t[i+8]
        asm("{\n\t"
            "mad.lo.cc.u32  %0, %9, %13, %0;\n\t"
            "madc.hi.cc.u32 %1, %9, %13, %1;\n\t"
            "madc.lo.cc.u32 %2, %10, %13, %2;\n\t"
            "madc.hi.cc.u32 %3, %10, %13, %3;\n\t"
            "madc.lo.cc.u32 %4, %11, %13, %4;\n\t"
            "madc.hi.cc.u32 %5, %11, %13, %5;\n\t"
            "madc.lo.cc.u32 %6, %12, %13, %6;\n\t"
            "madc.hi.cc.u32 %7, %12, %13, %7;\n\t"
            "addc.u32       %8, 0, 0;\n\t"
            "}"
            : "+r"(t[i]), "+r"(t[i + 1]), "+r"(t[i + 2]), "+r"(t[i + 3]), "+r"(t[i + 4]), "+r"(t[i + 5]),
              "+r"(t[i + 6]), "+r"(t[i + 7]), "=r"(t[i + 8])
            : "r"(a[0]), "r"(a[2]), "r"(a[4]), "r"(a[6]), "r"(b[i]));
        // odd chain: t[i+1..i+8] += a[1,3,5,7] * b[i].  The partial sum after row i is
        // below 2^(32(i+9)), so nothing carries out of t[i+8].
        asm("{\n\t"
            "mad.lo.cc.u32  %0, %8, %12, %0;\n\t"
            "madc.hi.cc.u32 %1, %8, %12, %1;\n\t"
            "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"
            "madc.hi.cc.u32 %3, %9, %12, %3;\n\t"
            "madc.lo.cc.u32 %4, %10, %12, %4;\n\t"
            "madc.hi.cc.u32 %5, %10, %12, %5;\n\t"
            "madc.lo.cc.u32 %6, %11, %12, %6;\n\t"
            "madc.hi.u32    %7, %11, %12, %7;\n\t"
            "}"
            : "+r"(t[i + 1]), "+r"(t[i + 2]), "+r"(t[i + 3]), "+r"(t[i + 4]), "+r"(t[i + 5]), "+r"(t[i + 6]),
              "+r"(t[i + 7]), "+r"(t[i + 8])
            : "r"(a[1]), "r"(a[3]), "r"(a[5]), "r"(a[7]), "r"(b[i]));
    }
}

// Squaring: the 28 cross products a_i a_j (i < j) once, doubled, plus the 8
// squares -- 72 half-products instead of 128.  Cross products go in rows
// (row i: a_i * a_j, j > i), split by the parity of j so that each chain
// covers contiguous words; the partial sum after row i is below 2^(32(i+9)),
// so carries are propagated only up to word i+8.  Single-instruction asm
// statements are volatile to keep the carry chains in order.
__device__ __forceinline__ void sqr_wide_8(uint32_t t[16], const uint32_t a[8])
{
#pragma unroll
    for (int k = 0; k < 16; k++)
        t[k] = 0;
#pragma unroll
    for (int i = 0; i < 7; i++) {
#pragma unroll
        for (int par = 1; par <= 2; par++) {
            const int j0 = i + par;
            if (j0 > 7)
                continue;
            int top = 0;
#pragma unroll
            for (int j = j0; j <= 7; j += 2) {
                if (j == j0)
                    asm volatile("mad.lo.cc.u32 %0, %1, %2, %0;" : "+r"(t[i + j]) : "r"(a[i]), "r"(a[j]));
                else
                    asm volatile("madc.lo.cc.u32 %0, %1, %2, %0;" : "+r"(t[i + j]) : "r"(a[i]), "r"(a[j]));
                asm volatile("madc.hi.cc.u32 %0, %1, %2, %0;" : "+r"(t[i + j + 1]) : "r"(a[i]), "r"(a[j]));
                top = i + j + 1;
            }
#pragma unroll
            for (int k = top + 1; k <= i + 8; k++) {
                if (k < i + 8)
                    asm volatile("addc.cc.u32 %0, %0, 0;" : "+r"(t[k]));
                else
                    asm volatile("addc.u32 %0, %0, 0;" : "+r"(t[k]));
            }
        }
    }
    // double the cross sum (< 2^511, so nothing leaves word 15)
#pragma unroll
    for (int k = 15; k > 0; k--)
        t[k] = __funnelshift_l(t[k - 1], t[k], 1);
    t[0] <<= 1;
    // add the squares a_i^2 at words 2i, 2i+1
    asm("{\n\t"
        "mad.lo.cc.u32  %0, %16, %16, %0;\n\t"
        "madc.hi.cc.u32 %1, %16, %16, %1;\n\t"
        "madc.lo.cc.u32 %2, %17, %17, %2;\n\t"
        "madc.hi.cc.u32 %3, %17, %17, %3;\n\t"
        "madc.lo.cc.u32 %4, %18, %18, %4;\n\t"
        "madc.hi.cc.u32 %5, %18, %18, %5;\n\t"
        "madc.lo.cc.u32 %6, %19, %19, %6;\n\t"
        "madc.hi.cc.u32 %7, %19, %19, %7;\n\t"
        "madc.lo.cc.u32 %8, %20, %20, %8;\n\t"
        "madc.hi.cc.u32 %9, %20, %20, %9;\n\t"
        "madc.lo.cc.u32 %10, %21, %21, %10;\n\t"
        "madc.hi.cc.u32 %11, %21, %21, %11;\n\t"
        "madc.lo.cc.u32 %12, %22, %22, %12;\n\t"
        "madc.hi.cc.u32 %13, %22, %22, %13;\n\t"
        "madc.lo.cc.u32 %14, %23, %23, %14;\n\t"
        "madc.hi.u32    %15, %23, %23, %15;\n\t"
        "}"
        : "+r"(t[0]), "+r"(t[1]), "+r"(t[2]), "+r"(t[3]), "+r"(t[4]), "+r"(t[5]), "+r"(t[6]), "+r"(t[7]),
          "+r"(t[8]), "+r"(t[9]), "+r"(t[10]), "+r"(t[11]), "+r"(t[12]), "+r"(t[13]), "+r"(t[14]), "+r"(t[15])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]));
}

template <class P>
struct Field {
    using Params = P;
    static constexpr uint32_t M0 = P::M[0], M1 = P::M[1], M2 = P::M[2], M3 = P::M[3];
    static constexpr uint32_t M4 = P::M[4], M5 = P::M[5], M6 = P::M[6], M7 = P::M[7];
    static constexpr uint32_t C0 = P::C[0], C1 = P::C[1], C2 = P::C[2], C3 = P::C[3];

    __device__ __forceinline__ static Fe zero()
    {
        Fe r;
#pragma unroll
        for (int i = 0; i < 8; i++)
            r.w[i] = 0;
        return r;
    }
    __device__ __forceinline__ static Fe one()
    {
        Fe r = zero();
        r.w[0] = 1;
        return r;
    }
    __device__ __forceinline__ static Fe from_u32(uint32_t v)
    {
        Fe r = zero();
        r.w[0] = v;
        return r;
    }

    // r += k*c for k in {0,1}-like masks: adds (c & mask), returns carry out
    __device__ __forceinline__ static uint32_t add_c_masked(Fe &r, uint32_t mask)
    {
        uint32_t cy;
        asm("{\n\t"
            "add.cc.u32  %0, %0, %9;\n\t"
            "addc.cc.u32 %1, %1, %10;\n\t"
            "addc.cc.u32 %2, %2, %11;\n\t"
            "addc.cc.u32 %3, %3, %12;\n\t"
            "addc.cc.u32 %4, %4, 0;\n\t"
            "addc.cc.u32 %5, %5, 0;\n\t"
            "addc.cc.u32 %6, %6, 0;\n\t"
            "addc.cc.u32 %7, %7, 0;\n\t"
            "addc.u32    %8, 0, 0;\n\t"
            "}"
            : "+r"(r.w[0]), "+r"(r.w[1]), "+r"(r.w[2]), "+r"(r.w[3]), "+r"(r.w[4]), "+r"(r.w[5]), "+r"(r.w[6]),
              "+r"(r.w[7]), "=r"(cy)
            : "r"(C0 & mask), "r"(C1 & mask), "r"(C2 & mask), "r"(C3 & mask));
        return cy;
    }

    __device__ __forceinline__ static uint32_t sub_c_masked(Fe &r, uint32_t mask)
    {
        uint32_t bw;
        asm("{\n\t"
            "sub.cc.u32  %0, %0, %9;\n\t"
            "subc.cc.u32 %1, %1, %10;\n\t"
            "subc.cc.u32 %2, %2, %11;\n\t"
            "subc.cc.u32 %3, %3, %12;\n\t"
            "subc.cc.u32 %4, %4, 0;\n\t"
            "subc.cc.u32 %5, %5, 0;\n\t"
            "subc.cc.u32 %6, %6, 0;\n\t"
            "subc.cc.u32 %7, %7, 0;\n\t"
            "subc.u32    %8, 0, 0;\n\t"
            "}"
            : "+r"(r.w[0]), "+r"(r.w[1]), "+r"(r.w[2]), "+r"(r.w[3]), "+r"(r.w[4]), "+r"(r.w[5]), "+r"(r.w[6]),
              "+r"(r.w[7]), "=r"(bw)
            : "r"(C0 & mask), "r"(C1 & mask), "r"(C2 & mask), "r"(C3 & mask));
        return bw;  // 0 or 0xffffffff
    }

    // a + b; a carry out of 2^256 is worth c
    __device__ __forceinline__ static Fe add(const Fe &a, const Fe &b)
    {
        Fe r;
        uint32_t cy;
        asm("{\n\t"
            "add.cc.u32  %0, %9, %17;\n\t"
            "addc.cc.u32 %1, %10, %18;\n\t"
            "addc.cc.u32 %2, %11, %19;\n\t"
            "addc.cc.u32 %3, %12, %20;\n\t"
            "addc.cc.u32 %4, %13, %21;\n\t"
            "addc.cc.u32 %5, %14, %22;\n\t"
            "addc.cc.u32 %6, %15, %23;\n\t"
            "addc.cc.u32 %7, %16, %24;\n\t"
            "addc.u32    %8, 0, 0;\n\t"
            "}"
            : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3]), "=r"(r.w[4]), "=r"(r.w[5]), "=r"(r.w[6]),
              "=r"(r.w[7]), "=r"(cy)
            : "r"(a.w[0]), "r"(a.w[1]), "r"(a.w[2]), "r"(a.w[3]), "r"(a.w[4]), "r"(a.w[5]), "r"(a.w[6]),
              "r"(a.w[7]), "r"(b.w[0]), "r"(b.w[1]), "r"(b.w[2]), "r"(b.w[3]), "r"(b.w[4]), "r"(b.w[5]),
              "r"(b.w[6]), "r"(b.w[7]));
        uint32_t cy2 = add_c_masked(r, 0u - cy);
        if (cy2)  // wrapped again: the low part is < c, adding c once more cannot carry
            add_c_masked(r, 0xffffffffu);
        return r;
    }

    // a - b; a borrow out of 2^256 is worth -c
    __device__ __forceinline__ static Fe sub(const Fe &a, const Fe &b)
    {
        Fe r;
        uint32_t bw;
        asm("{\n\t"
            "sub.cc.u32  %0, %9, %17;\n\t"
            "subc.cc.u32 %1, %10, %18;\n\t"
            "subc.cc.u32 %2, %11, %19;\n\t"
            "subc.cc.u32 %3, %12, %20;\n\t"
            "subc.cc.u32 %4, %13, %21;\n\t"
            "subc.cc.u32 %5, %14, %22;\n\t"
            "subc.cc.u32 %6, %15, %23;\n\t"
            "subc.cc.u32 %7, %16, %24;\n\t"
            "subc.u32    %8, 0, 0;\n\t"
            "}"
            : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3]), "=r"(r.w[4]), "=r"(r.w[5]), "=r"(r.w[6]),
              "=r"(r.w[7]), "=r"(bw)
            : "r"(a.w[0]), "r"(a.w[1]), "r"(a.w[2]), "r"(a.w[3]), "r"(a.w[4]), "r"(a.w[5]), "r"(a.w[6]),
              "r"(a.w[7]), "r"(b.w[0]), "r"(b.w[1]), "r"(b.w[2]), "r"(b.w[3]), "r"(b.w[4]), "r"(b.w[5]),
              "r"(b.w[6]), "r"(b.w[7]));
        uint32_t bw2 = sub_c_masked(r, bw);
        if (bw2)  // wrapped again: the value is now >= 2^256 - c, one more -c cannot borrow
            sub_c_masked(r, 0xffffffffu);
        return r;
    }

    __device__ __forceinline__ static Fe neg(const Fe &a) { return sub(zero(), a); }
    __device__ __forceinline__ static Fe dbl(const Fe &a) { return add(a, a); }

    // fold a 512-bit product t[0..15] to a weakly reduced element
    __device__ __forceinline__ static Fe reduce_wide(const uint32_t t[16])
    {
        Fe r;
        if (P::NC == 1) {
            // r = t_lo + 38 * t_hi: even/odd chains, top word r8 <= 38
            uint32_t r8;
            asm("{\n\t"
                "mad.lo.cc.u32  %0, %9, %17, %13;\n\t"
                "madc.hi.cc.u32 %1, %9, %17, %14;\n\t"
                "madc.lo.cc.u32 %2, %10, %17, %15;\n\t"
                "madc.hi.cc.u32 %3, %10, %17, %16;\n\t"
                "madc.lo.cc.u32 %4, %11, %17, %18;\n\t"
                "madc.hi.cc.u32 %5, %11, %17, %19;\n\t"
                "madc.lo.cc.u32 %6, %12, %17, %20;\n\t"
                "madc.hi.cc.u32 %7, %12, %17, %21;\n\t"
                "addc.u32       %8, 0, 0;\n\t"
                "}"
                : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3]), "=r"(r.w[4]), "=r"(r.w[5]),
                  "=r"(r.w[6]), "=r"(r.w[7]), "=r"(r8)
                : "r"(t[8]), "r"(t[10]), "r"(t[12]), "r"(t[14]), "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]),
                  "r"(C0), "r"(t[4]), "r"(t[5]), "r"(t[6]), "r"(t[7]));
            asm("{\n\t"
                "mad.lo.cc.u32  %0, %8, %12, %0;\n\t"
                "madc.hi.cc.u32 %1, %8, %12, %1;\n\t"
                "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"
                "madc.hi.cc.u32 %3, %9, %12, %3;\n\t"
                "madc.lo.cc.u32 %4, %10, %12, %4;\n\t"
                "madc.hi.cc.u32 %5, %10, %12, %5;\n\t"
                "madc.lo.cc.u32 %6, %11, %12, %6;\n\t"
                "madc.hi.u32    %7, %11, %12, %7;\n\t"
                "}"
                : "+r"(r.w[1]), "+r"(r.w[2]), "+r"(r.w[3]), "+r"(r.w[4]), "+r"(r.w[5]), "+r"(r.w[6]),
                  "+r"(r.w[7]), "+r"(r8)
                : "r"(t[9]), "r"(t[11]), "r"(t[13]), "r"(t[15]), "r"(C0));
            // r8 * 38 back into the low words; a wrap leaves < 2^11 in r, so +38 is safe
            uint32_t cy;
            asm("{\n\t"
                "mad.lo.cc.u32 %0, %9, %10, %0;\n\t"
                "addc.cc.u32   %1, %1, 0;\n\t"
                "addc.cc.u32   %2, %2, 0;\n\t"
                "addc.cc.u32   %3, %3, 0;\n\t"
                "addc.cc.u32   %4, %4, 0;\n\t"
                "addc.cc.u32   %5, %5, 0;\n\t"
                "addc.cc.u32   %6, %6, 0;\n\t"
                "addc.cc.u32   %7, %7, 0;\n\t"
                "addc.u32      %8, 0, 0;\n\t"
                "}"
                : "+r"(r.w[0]), "+r"(r.w[1]), "+r"(r.w[2]), "+r"(r.w[3]), "+r"(r.w[4]), "+r"(r.w[5]),
                  "+r"(r.w[6]), "+r"(r.w[7]), "=r"(cy)
                : "r"(r8), "r"(C0));
            r.w[0] += C0 & (0u - cy);
        } else {
            // fold 1: s[0..11] = t_lo + t_hi * G (G = 2*gamma, 4 limbs); s < 2^384
            uint32_t s[12];
#pragma unroll
            for (int i = 0; i < 8; i++)
                s[i] = t[i];
            const uint32_t G[4] = {C0, C1, C2, C3};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                asm("{\n\t"
                    "mad.lo.cc.u32  %0, %9, %13, %0;\n\t"
                    "madc.hi.cc.u32 %1, %9, %13, %1;\n\t"
                    "madc.lo.cc.u32 %2, %10, %13, %2;\n\t"
                    "madc.hi.cc.u32 %3, %10, %13, %3;\n\t"
                    "madc.lo.cc.u32 %4, %11, %13, %4;\n\t"
                    "madc.hi.cc.u32 %5, %11, %13, %5;\n\t"
                    "madc.lo.cc.u32 %6, %12, %13, %6;\n\t"
                    "madc.hi.cc.u32 %7, %12, %13, %7;\n\t"
                    "addc.u32       %8, 0, 0;\n\t"
                    "}"
                    : "+r"(s[k]), "+r"(s[k + 1]), "+r"(s[k + 2]), "+r"(s[k + 3]), "+r"(s[k + 4]), "+r"(s[k + 5]),
                      "+r"(s[k + 6]), "+r"(s[k + 7]), "=r"(s[k + 8])
                    : "r"(t[8]), "r"(t[10]), "r"(t[12]), "r"(t[14]), "r"(G[k]));
                asm("{\n\t"
                    "mad.lo.cc.u32  %0, %8, %12, %0;\n\t"
                    "madc.hi.cc.u32 %1, %8, %12, %1;\n\t"
                    "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"
                    "madc.hi.cc.u32 %3, %9, %12, %3;\n\t"
                    "madc.lo.cc.u32 %4, %10, %12, %4;\n\t"
                    "madc.hi.cc.u32 %5, %10, %12, %5;\n\t"
                    "madc.lo.cc.u32 %6, %11, %12, %6;\n\t"
                    "madc.hi.u32    %7, %11, %12, %7;\n\t"
                    "}"
                    : "+r"(s[k + 1]), "+r"(s[k + 2]), "+r"(s[k + 3]), "+r"(s[k + 4]), "+r"(s[k + 5]),
                      "+r"(s[k + 6]), "+r"(s[k + 7]), "+r"(s[k + 8])
                    : "r"(t[9]), "r"(t[11]), "r"(t[13]), "r"(t[15]), "r"(G[k]));
            }
            // fold 2: p[0..7] = h * G with h = s[8..11] (< 2^128), so p < 2^255.02.
            // Row k adds h * G[k] at word k: even limbs of h in one chain (carry into the
            // fresh word p[k+4]), odd limbs in a second chain ending in p[k+4].
            uint32_t p[8];
            asm("mul.lo.u32 %0, %2, %3;\n\tmul.hi.u32 %1, %2, %3;" : "=r"(p[0]), "=r"(p[1]) : "r"(s[8]), "r"(G[0]));
            asm("mul.lo.u32 %0, %2, %3;\n\tmul.hi.u32 %1, %2, %3;" : "=r"(p[2]), "=r"(p[3]) : "r"(s[10]), "r"(G[0]));
            asm("{\n\t"
                "mad.lo.cc.u32  %0, %4, %6, %0;\n\t"
                "madc.hi.cc.u32 %1, %4, %6, %1;\n\t"
                "madc.lo.cc.u32 %2, %5, %6, %2;\n\t"
                "madc.hi.u32    %3, %5, %6, 0;\n\t"
                "}"
                : "+r"(p[1]), "+r"(p[2]), "+r"(p[3]), "=r"(p[4])
                : "r"(s[9]), "r"(s[11]), "r"(G[0]));
#pragma unroll
            for (int k = 1; k < 4; k++) {
                asm("{\n\t"
                    "mad.lo.cc.u32  %0, %5, %7, %0;\n\t"
                    "madc.hi.cc.u32 %1, %5, %7, %1;\n\t"
                    "madc.lo.cc.u32 %2, %6, %7, %2;\n\t"
                    "madc.hi.cc.u32 %3, %6, %7, %3;\n\t"
                    "addc.u32       %4, 0, 0;\n\t"
                    "}"
                    : "+r"(p[k]), "+r"(p[k + 1]), "+r"(p[k + 2]), "+r"(p[k + 3]), "=r"(p[k + 4])
                    : "r"(s[8]), "r"(s[10]), "r"(G[k]));
                asm("{\n\t"
                    "mad.lo.cc.u32  %0, %4, %6, %0;\n\t"
                    "madc.hi.cc.u32 %1, %4, %6, %1;\n\t"
                    "madc.lo.cc.u32 %2, %5, %6, %2;\n\t"
                    "madc.hi.u32    %3, %5, %6, %3;\n\t"
                    "}"
                    : "+r"(p[k + 1]), "+r"(p[k + 2]), "+r"(p[k + 3]), "+r"(p[k + 4])
                    : "r"(s[9]), "r"(s[11]), "r"(G[k]));
            }
            uint32_t cy;
            asm("{\n\t"
                "add.cc.u32  %0, %9, %17;\n\t"
                "addc.cc.u32 %1, %10, %18;\n\t"
                "addc.cc.u32 %2, %11, %19;\n\t"
                "addc.cc.u32 %3, %12, %20;\n\t"
                "addc.cc.u32 %4, %13, %21;\n\t"
                "addc.cc.u32 %5, %14, %22;\n\t"
                "addc.cc.u32 %6, %15, %23;\n\t"
                "addc.cc.u32 %7, %16, %24;\n\t"
                "addc.u32    %8, 0, 0;\n\t"
                "}"
                : "=r"(r.w[0]), "=r"(r.w[1]), "=r"(r.w[2]), "=r"(r.w[3]), "=r"(r.w[4]), "=r"(r.w[5]),
                  "=r"(r.w[6]), "=r"(r.w[7]), "=r"(cy)
                : "r"(s[0]), "r"(s[1]), "r"(s[2]), "r"(s[3]), "r"(s[4]), "r"(s[5]), "r"(s[6]), "r"(s[7]),
                  "r"(p[0]), "r"(p[1]), "r"(p[2]), "r"(p[3]), "r"(p[4]), "r"(p[5]), "r"(p[6]), "r"(p[7]));
            // fold 3: one carry bit worth G
            uint32_t cy2 = add_c_masked(r, 0u - cy);
            if (cy2)
                add_c_masked(r, 0xffffffffu);
        }
        return r;
    }

    __device__ __forceinline__ static Fe mul(const Fe &a, const Fe &b)
    {
        uint32_t t[16];
        mul_wide_8x8(t, a.w, b.w);
        return reduce_wide(t);
    }

    __device__ __forceinline__ static Fe sqr(const Fe &a)
    {
        uint32_t t[16];
        sqr_wide_8(t, a.w);
        return reduce_wide(t);
    }

    // canonical representative in [0, m): a < 2^256 = 2m + c
    __device__ __forceinline__ static Fe canon(const Fe &a)
    {
        Fe t = a;
        uint32_t cy = add_c_masked(t, 0xffffffffu);  // t = a + c; carry <=> a >= 2m
        Fe v = cy ? t : a;
        Fe d;
        uint32_t bw;
        asm("{\n\t"
            "sub.cc.u32  %0, %9, %17;\n\t"
            "subc.cc.u32 %1, %10, %18;\n\t"
            "subc.cc.u32 %2, %11, %19;\n\t"
            "subc.cc.u32 %3, %12, %20;\n\t"
            "subc.cc.u32 %4, %13, %21;\n\t"
            "subc.cc.u32 %5, %14, %22;\n\t"
            "subc.cc.u32 %6, %15, %23;\n\t"
            "subc.cc.u32 %7, %16, %24;\n\t"
            "subc.u32    %8, 0, 0;\n\t"
            "}"
            : "=r"(d.w[0]), "=r"(d.w[1]), "=r"(d.w[2]), "=r"(d.w[3]), "=r"(d.w[4]), "=r"(d.w[5]), "=r"(d.w[6]),
              "=r"(d.w[7]), "=r"(bw)
            : "r"(v.w[0]), "r"(v.w[1]), "r"(v.w[2]), "r"(v.w[3]), "r"(v.w[4]), "r"(v.w[5]), "r"(v.w[6]),
              "r"(v.w[7]), "r"(M0), "r"(M1), "r"(M2), "r"(M3), "r"(M4), "r"(M5), "r"(M6), "r"(M7));
        return bw ? v : d;
    }

    __device__ __forceinline__ static bool is_zero(const Fe &a)
    {
        // a == 0 (mod m) <=> a in {0, m, 2m}; the top word screens the common case
        uint32_t top = a.w[7];
        if (top != 0u && top != M7 && top != ((M7 << 1) | (M6 >> 31)))
            return false;
        Fe c = canon(a);
        uint32_t o = 0;
#pragma unroll
        for (int i = 0; i < 8; i++)
            o |= c.w[i];
        return o == 0;
    }

    __device__ __forceinline__ static bool is_exact_zero(const Fe &a)
    {
        uint32_t o = 0;
#pragma unroll
        for (int i = 0; i < 8; i++)
            o |= a.w[i];
        return o == 0;
    }

    __device__ __forceinline__ static bool eq(const Fe &a, const Fe &b) { return is_zero(sub(a, b)); }

    // a^e for e given as eight 32-bit words (4-bit fixed window)
    __device__ static Fe pow(const Fe &a, const uint32_t e[8])
    {
        Fe tab[16];
        tab[0] = one();
        tab[1] = a;
#pragma unroll 1
        for (int i = 2; i < 16; i++)
            tab[i] = mul(tab[i - 1], a);
        Fe acc = one();
#pragma unroll 1
        for (int i = 63; i >= 0; i--) {
            acc = sqr(acc);
            acc = sqr(acc);
            acc = sqr(acc);
            acc = sqr(acc);
            uint32_t nib = (e[i >> 3] >> (4 * (i & 7))) & 15u;
            if (nib) {
                Fe m = tab[0];
#pragma unroll
                for (int k = 1; k < 16; k++)
                    if (k == (int)nib)
                        m = tab[k];
                acc = mul(acc, m);
            }
        }
        return acc;
    }

    // ---- inversion by batched divsteps ----------------------------------------
    // The variable-time binary-GCD inversion of Bernstein and Yang ("Fast
    // constant-time gcd computation and modular inversion", 2019), with the
    // half-delta divstep: starting from (f, g) = (m, a), each divstep maps
    //     delta > 0 and g odd:  (delta, f, g) -> (1 - delta, g, (g - f) / 2)
    //     g odd:                (delta, f, g) -> (1 + delta, f, (g + f) / 2)
    //     g even:               (delta, f, g) -> (1 + delta, f, g / 2)
    // until g = 0, where f = +-gcd = +-1.  Steps run in batches of 30 on the low
    // 32 bits of f and g, which give a transition matrix T (entries at most 2^30)
    // with 2^30 (f', g') = T (f, g); T is then applied to the full f and g, held
    // in nine signed 30-bit limbs, and to (d, e) with f = d a, g = e a (mod m),
    // where the division by 2^30 is made exact by adding a multiple of m.  At the
    // end a^-1 = +-d.  A 256-bit input needs at most 590 divsteps (20 batches);
    // the loop is capped at 40.  Against Fermat's a^(m-2) (255 dependent
    // squarings) the dependent chain is about a tenth as long.
    struct L30 {
        int32_t l[9];  // value = sum l[i] 2^(30 i); l[0..7] in [0, 2^30), l[8] signed
    };

    __device__ __forceinline__ static L30 to_l30(const Fe &a)
    {
        L30 r;
#pragma unroll
        for (int i = 0; i < 9; i++) {
            const int b = 30 * i, k = b >> 5, sh = b & 31;
            const uint64_t lo = a.w[k], hi = k + 1 < 8 ? a.w[k + 1] : 0u;
            r.l[i] = (int32_t)(((lo | (hi << 32)) >> sh) & 0x3fffffffu);
        }
        return r;
    }

    // (x, y) <- (s x + t y + k m) / 2^30 for one row; the low 30 bits vanish
    __device__ __forceinline__ static void l30_row(L30 &out, const L30 &x, const L30 &y, int32_t s, int32_t t,
                                                   int32_t k, const L30 &m)
    {
        int64_t c = (int64_t)s * x.l[0] + (int64_t)t * y.l[0] + (int64_t)k * m.l[0];
        c >>= 30;
#pragma unroll
        for (int i = 1; i < 9; i++) {
            c += (int64_t)s * x.l[i] + (int64_t)t * y.l[i] + (int64_t)k * m.l[i];
            out.l[i - 1] = (int32_t)(c & 0x3fffffff);
            c >>= 30;
        }
        out.l[8] = (int32_t)c;
    }

    __device__ static Fe inv(const Fe &a)
    {
        const Fe x = canon(a);
        if (is_exact_zero(x))
            return zero();  // 0 -> 0
        const Fe mf = {{M0, M1, M2, M3, M4, M5, M6, M7}};
        const L30 m = to_l30(mf);
        L30 zero30;
#pragma unroll
        for (int i = 0; i < 9; i++)
            zero30.l[i] = 0;
        // m^-1 mod 2^32 by Newton's iteration (m odd: m m = 1 mod 8 to start)
        uint32_t minv = M0;
#pragma unroll
        for (int i = 0; i < 4; i++)
            minv *= 2u - M0 * minv;
        L30 f = m, g = to_l30(x), d = zero30, e = zero30;
        e.l[0] = 1;
        int32_t D = 1;  // 2 delta, delta = 1/2
        for (int batch = 0; batch < 40; batch++) {
            uint32_t any = 0;
#pragma unroll
            for (int i = 0; i < 9; i++)
                any |= (uint32_t)g.l[i];
            if (!any)
                break;
            uint32_t fl = (uint32_t)f.l[0] | ((uint32_t)f.l[1] << 30);
            uint32_t gl = (uint32_t)g.l[0] | ((uint32_t)g.l[1] << 30);
            int32_t u = 1, v = 0, q = 0, r = 1;
#pragma unroll 1
            for (int i = 0; i < 30; i++) {
                if (D > 0 && (gl & 1u)) {
                    D = 2 - D;
                    const uint32_t t = fl;
                    fl = gl;
                    gl -= t;
                    const int32_t tu = u, tv = v;
                    u = q;
                    v = r;
                    q -= tu;
                    r -= tv;
                } else if (gl & 1u) {
                    D = 2 + D;
                    gl += fl;
                    q += u;
                    r += v;
                } else {
                    D = 2 + D;
                }
                gl >>= 1;
                u *= 2;
                v *= 2;
            }
            L30 nf, ng, nd, ne;
            l30_row(nf, f, g, u, v, 0, m);
            l30_row(ng, f, g, q, r, 0, m);
            const uint32_t td = (uint32_t)u * (uint32_t)d.l[0] + (uint32_t)v * (uint32_t)e.l[0];
            const uint32_t te = (uint32_t)q * (uint32_t)d.l[0] + (uint32_t)r * (uint32_t)e.l[0];
            const int32_t md = (int32_t)(((0u - td) * minv) << 2) >> 2;  // in [-2^29, 2^29)
            const int32_t me = (int32_t)(((0u - te) * minv) << 2) >> 2;
            l30_row(nd, d, e, u, v, md, m);
            l30_row(ne, d, e, q, r, me, m);
            f = nf;
            g = ng;
            d = nd;
            e = ne;
        }
        // d + 16 m > 0 (|d| < m here), packed into nine 32-bit words, folded mod m
        int64_t c = 0;
        uint32_t w[9];
        {
            L30 t;
#pragma unroll
            for (int i = 0; i < 9; i++) {
                c += (int64_t)d.l[i] + 16 * (int64_t)m.l[i];
                t.l[i] = i < 8 ? (int32_t)(c & 0x3fffffff) : (int32_t)c;
                c >>= 30;
            }
            uint64_t acc = 0;
            int bits = 0, k = 0;
#pragma unroll
            for (int i = 0; i < 9; i++) {
                acc |= (uint64_t)(uint32_t)t.l[i] << bits;
                bits += 30;
                while (bits >= 32 && k < 9) {
                    w[k++] = (uint32_t)acc;
                    acc >>= 32;
                    bits -= 32;
                }
            }
            while (k < 9) {
                w[k++] = (uint32_t)acc;
                acc >>= 32;
            }
        }
        Fe lo;
#pragma unroll
        for (int i = 0; i < 8; i++)
            lo.w[i] = w[i];
        Fe cfe = zero();
        add_c_masked(cfe, 0xffffffffu);  // 2^256 mod m
        Fe res = add(lo, mul(from_u32(w[8]), cfe));
        return f.l[8] < 0 ? neg(res) : res;
    }
};

using Fp = Field<FpParams>;
using Fq = Field<FqParams>;

}  // namespace hs
