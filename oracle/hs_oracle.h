/*
 * hs_oracle.h -- CPU restatement of helioselene's vartime MSM path.
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).
 * Formats and semantics are documented in hs_oracle.c.
 */
#ifndef HS_ORACLE_H
#define HS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HSO_HELIOS 0
#define HSO_SELENE 1
#define HSO_FIELD_P 0
#define HSO_FIELD_Q 1

int hso_abi_version(void);
int hso_msm(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n, int keep_carry);
int hso_msm_affine_out(int curve, uint8_t out32[32], uint8_t out64[64], const uint8_t *scalars,
                       const uint8_t *pts64, size_t n, int keep_carry);
int hso_msm_jac(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *jac96, size_t n,
                int keep_carry);
int hso_pippenger_w(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n, int w,
                    int keep_carry);
int hso_msm_naive(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n);
int hso_msm_mt(int curve, uint8_t out32[32], const uint8_t *scalars, const uint8_t *pts64, size_t n, int nthreads);
int hso_msm_many(int curve, uint8_t *out32s, const uint8_t *scalars, const uint8_t *pts64, const uint64_t *sizes,
                 size_t count, int nthreads);
int hso_pedersen(int curve, uint8_t out32[32], const uint8_t blinding[32], const uint8_t H64[64],
                 const uint8_t *values, const uint8_t *gens64, size_t n, int keep_carry);
int hso_map_to_curve(int curve, uint8_t *out64, const uint8_t *u32s, size_t n);
int hso_map_to_curve_mt(int curve, uint8_t *out64, const uint8_t *u32s, size_t n, int nthreads);
int hso_decompress(int curve, uint8_t *out64, const uint8_t *in32, size_t n);
int hso_compress(int curve, uint8_t *out32, const uint8_t *in64, size_t n);
int hso_compress_jac(int curve, uint8_t *out32, const uint8_t *in96, size_t n);
int hso_batch_invert(int field, uint8_t *out32, const uint8_t *in32, size_t n);
int hso_batch_to_affine(int curve, uint8_t *out64, const uint8_t *in96, size_t n);
int hso_scalar_mul(int curve, uint8_t out64[64], const uint8_t scalar[32], const uint8_t pt64[64]);
int hso_point_add(int curve, uint8_t out64[64], const uint8_t a64[64], const uint8_t b64[64]);
int hso_fe51_to_bytes(int field, uint8_t out32[32], const uint64_t limbs[5]);

#ifdef __cplusplus
}
#endif
#endif
