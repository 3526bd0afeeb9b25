// hs_curve.cuh -- Helios / Selene group law on the device.
//
// Both curves are y^2 = x^3 - 3x + b (helios/include/helios_constants.h:36-41 over
// F_p, selene/include/selene_constants.h:36-41 over F_q).  The reference adds in
// Jacobian coordinates (add-2007-bl, dbl-2001-b, helios/src/x64/helios_add.cpp:52-107,
// helios_dbl.cpp:45-88) behind an edge-case wrapper (helios_msm_vartime.cpp:59-104).
//
// Bucket arithmetic here uses extended Jacobian "XYZZ" coordinates
// (x = X/ZZ, y = Y/ZZZ, ZZ^3 = ZZZ^2): mixed addition of an affine base costs
// 8M+2S instead of 7M+4S, and the doubling / inverse cases are detected from
// the same intermediate values.  The identity is ZZ = 0 exactly (a non-identity
// point never has ZZ congruent to 0, and the identity is only ever produced by
// an explicit store of zeros).

#pragma once
#include "hs_field.cuh"

namespace hs {

struct HeliosCurve {
    using F = Fp;
    static constexpr int ID = 0;
    // b = 15789920373731020205926570676277057129217619222203920395806844808978996083412
    __device__ __forceinline__ static Fe b()
    {
        return Fe{{0xedd73ad4u, 0x22b49ee1u, 0x4113bf35u, 0x043f6f38u, 0x3ebb7b3bu, 0xbe94a76bu, 0xb0ea70b8u,
                   0x22e8c739u}};
    }
    static constexpr int SSWU_Z = 7;  // helios/src/x64/helios_map_to_curve.cpp:54
};

struct SeleneCurve {
    using F = Fq;
    static constexpr int ID = 1;
    // b = 50691664119640283727448954162351551669994268339720539671652090628799494505816
    __device__ __forceinline__ static Fe b()
    {
        return Fe{{0xcb5a4558u, 0x68de0983u, 0x06ae900eu, 0xf3944bdfu, 0x95ffe279u, 0x7f51bba5u, 0x695876c1u,
                   0x70127713u}};
    }
    static constexpr int SSWU_Z = -4;  // selene/src/x64/selene_map_to_curve.cpp
};

struct Affine {
    Fe x, y;
};

struct Xyzz {
    Fe X, Y, ZZ, ZZZ;
};

template <class C>
struct Group {
    using F = typename C::F;

    __device__ __forceinline__ static Fe b() { return C::b(); }

    __device__ __forceinline__ static Xyzz inf()
    {
        Xyzz r;
        r.X = F::zero();
        r.Y = F::zero();
        r.ZZ = F::zero();
        r.ZZZ = F::zero();
        return r;
    }

    __device__ __forceinline__ static bool is_inf(const Xyzz &p) { return F::is_exact_zero(p.ZZ); }

    __device__ __forceinline__ static Xyzz from_affine(const Fe &x, const Fe &y)
    {
        Xyzz r;
        r.X = x;
        r.Y = y;
        r.ZZ = F::one();
        r.ZZZ = F::one();
        return r;
    }

    // dbl-2008-s-1 for a = -3: M = 3(X - ZZ)(X + ZZ).  7M + 2S.
    __device__ static Xyzz dbl(const Xyzz &p)
    {
        if (is_inf(p))
            return p;
        Fe U = F::dbl(p.Y);
        Fe V = F::sqr(U);
        Fe W = F::mul(U, V);
        Fe S = F::mul(p.X, V);
        Fe t0 = F::sub(p.X, p.ZZ);
        Fe t1 = F::add(p.X, p.ZZ);
        Fe M = F::mul(t0, t1);
        M = F::add(F::dbl(M), M);
        Xyzz r;
        r.X = F::sub(F::sqr(M), F::dbl(S));
        r.Y = F::sub(F::mul(M, F::sub(S, r.X)), F::mul(W, p.Y));
        r.ZZ = F::mul(V, p.ZZ);
        r.ZZZ = F::mul(W, p.ZZZ);
        if (F::is_zero(r.ZZ))  // y == 0 (no such point on a prime-order curve; kept complete)
            return inf();
        return r;
    }

    // mdbl-2008-s-1: doubling of an affine point, M = 3x^2 - 3.
    __device__ static Xyzz dbl_affine(const Fe &x, const Fe &y)
    {
        Fe U = F::dbl(y);
        Fe V = F::sqr(U);
        Fe W = F::mul(U, V);
        Fe S = F::mul(x, V);
        Fe M = F::sub(F::sqr(x), F::one());
        M = F::add(F::dbl(M), M);
        Xyzz r;
        r.X = F::sub(F::sqr(M), F::dbl(S));
        r.Y = F::sub(F::mul(M, F::sub(S, r.X)), F::mul(W, y));
        r.ZZ = V;
        r.ZZZ = W;
        if (F::is_zero(r.ZZ))
            return inf();
        return r;
    }

    // acc += (x2, y2), the affine point never being the identity.  madd-2008-s.
    __device__ __forceinline__ static void add_affine(Xyzz &acc, const Fe &x2, const Fe &y2)
    {
        if (is_inf(acc)) {
            acc = from_affine(x2, y2);
            return;
        }
        Fe U2 = F::mul(x2, acc.ZZ);
        Fe S2 = F::mul(y2, acc.ZZZ);
        Fe P = F::sub(U2, acc.X);
        Fe R = F::sub(S2, acc.Y);
        if (F::is_zero(P)) {
            if (F::is_zero(R))
                acc = dbl_affine(x2, y2);  // same point: double
            else
                acc = inf();  // opposite points
            return;
        }
        Fe PP = F::sqr(P);
        Fe PPP = F::mul(P, PP);
        Fe Q = F::mul(acc.X, PP);
        Fe X3 = F::sub(F::sub(F::sqr(R), PPP), F::dbl(Q));
        Fe Y3 = F::sub(F::mul(R, F::sub(Q, X3)), F::mul(acc.Y, PPP));
        acc.ZZ = F::mul(acc.ZZ, PP);
        acc.ZZZ = F::mul(acc.ZZZ, PPP);
        acc.X = X3;
        acc.Y = Y3;
    }

    // p + q, complete.  add-2008-s: 12M + 2S.
    __device__ static Xyzz add(const Xyzz &p, const Xyzz &q)
    {
        if (is_inf(p))
            return q;
        if (is_inf(q))
            return p;
        Fe U1 = F::mul(p.X, q.ZZ);
        Fe U2 = F::mul(q.X, p.ZZ);
        Fe S1 = F::mul(p.Y, q.ZZZ);
        Fe S2 = F::mul(q.Y, p.ZZZ);
        Fe P = F::sub(U2, U1);
        Fe R = F::sub(S2, S1);
        if (F::is_zero(P)) {
            if (F::is_zero(R))
                return dbl(p);
            return inf();
        }
        Fe PP = F::sqr(P);
        Fe PPP = F::mul(P, PP);
        Fe Q = F::mul(U1, PP);
        Xyzz r;
        r.X = F::sub(F::sub(F::sqr(R), PPP), F::dbl(Q));
        r.Y = F::sub(F::mul(R, F::sub(Q, r.X)), F::mul(S1, PPP));
        r.ZZ = F::mul(F::mul(p.ZZ, q.ZZ), PP);
        r.ZZZ = F::mul(F::mul(p.ZZZ, q.ZZZ), PPP);
        return r;
    }

    __device__ __forceinline__ static Xyzz neg(const Xyzz &p)
    {
        Xyzz r = p;
        if (!is_inf(p))
            r.Y = F::neg(p.Y);
        return r;
    }

    // XYZZ -> Jacobian without inversion: Z = ZZ*ZZZ, X = X*ZZ*ZZZ^2, Y = Y*ZZ^3*ZZZ^2.
    // Identity -> (1:1:0), the reference's encoding (helios/include/helios_ops.h:45-50).
    __device__ static void to_jacobian(Fe &X, Fe &Y, Fe &Z, const Xyzz &p)
    {
        if (is_inf(p)) {
            X = F::one();
            Y = F::one();
            Z = F::zero();
            return;
        }
        Fe zzz2 = F::sqr(p.ZZZ);
        Fe zz2 = F::sqr(p.ZZ);
        Z = F::mul(p.ZZ, p.ZZZ);
        X = F::mul(F::mul(p.X, p.ZZ), zzz2);
        Y = F::mul(F::mul(p.Y, F::mul(zz2, p.ZZ)), zzz2);
    }

    // XYZZ -> canonical affine (one inversion); identity -> (0,0)
    __device__ static Affine to_affine(const Xyzz &p)
    {
        Affine a;
        if (is_inf(p)) {
            a.x = F::zero();
            a.y = F::zero();
            return a;
        }
        Fe inv = F::inv(F::mul(p.ZZ, p.ZZZ));
        a.x = F::canon(F::mul(F::mul(p.X, p.ZZZ), inv));
        a.y = F::canon(F::mul(F::mul(p.Y, p.ZZ), inv));
        return a;
    }
};

}  // namespace hs
