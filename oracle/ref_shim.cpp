// ref_shim.cpp -- flat C entry points over the reference's own x64 code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/Makefile, target `ref`)
// together with the unmodified helioselene sources into oracle/_ref/libhsref.so,
// which the test suite uses to pin the C restatement (hs_oracle.c) to the
// reference bit for bit.  It is built only where the reference tree exists.
//
// Calls: helios_msm_vartime / selene_msm_vartime (x64 static binding,
// helios/include/helios_msm_vartime.h:50-60), *_tobytes, *_frombytes,
// *_map_to_curve, and the header-only *_pedersen_commit / *_batch_to_affine.

#include "fp_frombytes.h"
#include "fp_tobytes.h"
#include "fq_frombytes.h"
#include "fq_tobytes.h"
#include "helios.h"
#include "helios_batch_affine.h"
#include "helios_frombytes.h"
#include "helios_map_to_curve.h"
#include "helios_msm_vartime.h"
#include "helios_ops.h"
#include "helios_pedersen.h"
#include "helios_tobytes.h"
#include "selene.h"
#include "selene_batch_affine.h"
#include "selene_frombytes.h"
#include "selene_map_to_curve.h"
#include "selene_msm_vartime.h"
#include "selene_ops.h"
#include "selene_pedersen.h"
#include "selene_tobytes.h"

#include <cstdint>
#include <cstring>
#include <vector>

namespace
{
    template <class J, class FB> void load_affine(J *p, const uint8_t *b64, FB frombytes, void (*one)(J *))
    {
        bool z = true;
        for (int i = 0; i < 64; i++)
            z = z && b64[i] == 0;
        if (z)
        {
            one(p);
            return;
        }
        frombytes(p->X, b64);
        frombytes(p->Y, b64 + 32);
        std::memset(p->Z, 0, sizeof(p->Z));
        p->Z[0] = 1;
    }

    void h_ident(helios_jacobian *p) { helios_identity(p); }
    void s_ident(selene_jacobian *p) { selene_identity(p); }
} // namespace

extern "C"
{
    // points: n x 64 bytes canonical affine (zeros = identity); out: 32-byte encoding
    int ref_msm(int curve, uint8_t *out32, const uint8_t *scalars, const uint8_t *pts64, size_t n)
    {
        if (curve == 0)
        {
            std::vector<helios_jacobian> p(n ? n : 1);
            for (size_t i = 0; i < n; i++)
                load_affine(&p[i], pts64 + 64 * i, fp_frombytes, h_ident);
            helios_jacobian r;
            helios_msm_vartime(&r, scalars, p.data(), n);
            helios_tobytes(out32, &r);
            return 0;
        }
        if (curve == 1)
        {
            std::vector<selene_jacobian> p(n ? n : 1);
            for (size_t i = 0; i < n; i++)
                load_affine(&p[i], pts64 + 64 * i, fq_frombytes, s_ident);
            selene_jacobian r;
            selene_msm_vartime(&r, scalars, p.data(), n);
            selene_tobytes(out32, &r);
            return 0;
        }
        return -1;
    }

    // points: n x 15 uint64 (X[5], Y[5], Z[5] radix-2^51, the reference's own struct)
    int ref_msm_jac51(int curve, uint8_t *out32, const uint8_t *scalars, const uint64_t *jac51, size_t n)
    {
        if (curve == 0)
        {
            helios_jacobian r;
            helios_msm_vartime(&r, scalars, reinterpret_cast<const helios_jacobian *>(jac51), n);
            helios_tobytes(out32, &r);
            return 0;
        }
        if (curve == 1)
        {
            selene_jacobian r;
            selene_msm_vartime(&r, scalars, reinterpret_cast<const selene_jacobian *>(jac51), n);
            selene_tobytes(out32, &r);
            return 0;
        }
        return -1;
    }

    int ref_encode_jac51(int curve, uint8_t *out32, const uint64_t *jac51)
    {
        if (curve == 0)
            helios_tobytes(out32, reinterpret_cast<const helios_jacobian *>(jac51));
        else if (curve == 1)
            selene_tobytes(out32, reinterpret_cast<const selene_jacobian *>(jac51));
        else
            return -1;
        return 0;
    }

    int ref_map_to_curve(int curve, uint8_t *out32, const uint8_t *u)
    {
        if (curve == 0)
        {
            helios_jacobian r;
            helios_map_to_curve(&r, u);
            helios_tobytes(out32, &r);
        }
        else if (curve == 1)
        {
            selene_jacobian r;
            selene_map_to_curve(&r, u);
            selene_tobytes(out32, &r);
        }
        else
            return -1;
        return 0;
    }

    int ref_pedersen(int curve, uint8_t *out32, const uint8_t *blinding, const uint8_t *H64, const uint8_t *values,
                     const uint8_t *gens64, size_t n)
    {
        if (curve == 0)
        {
            helios_jacobian H, r;
            load_affine(&H, H64, fp_frombytes, h_ident);
            std::vector<helios_jacobian> g(n ? n : 1);
            for (size_t i = 0; i < n; i++)
                load_affine(&g[i], gens64 + 64 * i, fp_frombytes, h_ident);
            helios_pedersen_commit(&r, blinding, &H, values, g.data(), n);
            helios_tobytes(out32, &r);
        }
        else if (curve == 1)
        {
            selene_jacobian H, r;
            load_affine(&H, H64, fq_frombytes, s_ident);
            std::vector<selene_jacobian> g(n ? n : 1);
            for (size_t i = 0; i < n; i++)
                load_affine(&g[i], gens64 + 64 * i, fq_frombytes, s_ident);
            selene_pedersen_commit(&r, blinding, &H, values, g.data(), n);
            selene_tobytes(out32, &r);
        }
        else
            return -1;
        return 0;
    }

    // jac51 in, canonical affine bytes out (identity -> zeros)
    int ref_batch_to_affine(int curve, uint8_t *out64, const uint64_t *jac51, size_t n)
    {
        if (curve == 0)
        {
            std::vector<helios_affine> a(n ? n : 1);
            helios_batch_to_affine(a.data(), reinterpret_cast<const helios_jacobian *>(jac51), n);
            for (size_t i = 0; i < n; i++)
            {
                fp_tobytes(out64 + 64 * i, a[i].x);
                fp_tobytes(out64 + 64 * i + 32, a[i].y);
            }
        }
        else if (curve == 1)
        {
            std::vector<selene_affine> a(n ? n : 1);
            selene_batch_to_affine(a.data(), reinterpret_cast<const selene_jacobian *>(jac51), n);
            for (size_t i = 0; i < n; i++)
            {
                fq_tobytes(out64 + 64 * i, a[i].x);
                fq_tobytes(out64 + 64 * i + 32, a[i].y);
            }
        }
        else
            return -1;
        return 0;
    }
}
