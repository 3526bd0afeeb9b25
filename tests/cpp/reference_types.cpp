// Compile-time check of include/helioselene_gb300.hpp against the reference's
// own headers: the reference's point records must have the layout of
// hs_jacobian51 / hs_affine51 (static assertions in the header), and every
// binding with the reference's signatures, and the point-API adapters over
// helioselene::HeliosPoint / SelenePoint, must compile.  Built with -c only.
#include "helios.h"
#include "selene.h"
#include "helioselene_point.h"
#include "helioselene_scalar.h"

#include "helioselene_gb300.hpp"

namespace hg = helioselene_gb300;

// the bindings take exactly the reference's signatures
void (*const bind_helios_msm)(helios_jacobian *, const unsigned char *, const helios_jacobian *, size_t) =
    &hg::helios_msm_vartime;
void (*const bind_selene_msm)(selene_jacobian *, const unsigned char *, const selene_jacobian *, size_t) =
    &hg::selene_msm_vartime;
void (*const bind_helios_ped)(helios_jacobian *, const unsigned char *, const helios_jacobian *, const unsigned char *,
                              const helios_jacobian *, size_t) = &hg::helios_pedersen_commit;
void (*const bind_selene_ped)(selene_jacobian *, const unsigned char *, const selene_jacobian *, const unsigned char *,
                              const selene_jacobian *, size_t) = &hg::selene_pedersen_commit;
void (*const bind_helios_aff)(helios_affine *, const helios_jacobian *, size_t) = &hg::helios_batch_to_affine;
void (*const bind_selene_aff)(selene_affine *, const selene_jacobian *, size_t) = &hg::selene_batch_to_affine;
void (*const bind_helios_smul)(helios_jacobian *, const unsigned char *, const helios_jacobian *) =
    &hg::helios_scalarmult_vartime;
void (*const bind_selene_smul)(selene_jacobian *, const unsigned char *, const selene_jacobian *) =
    &hg::selene_scalarmult_vartime;

helioselene::HeliosPoint point_api_helios(const helioselene::HeliosScalar *s, const helioselene::HeliosPoint *p,
                                          size_t n)
{
    return hg::multi_scalar_mul(s, p, n);
}

helioselene::SelenePoint point_api_selene(const helioselene::SeleneScalar &b, const helioselene::SelenePoint &H,
                                          const helioselene::SeleneScalar *v, const helioselene::SelenePoint *g,
                                          size_t n)
{
    return hg::pedersen_commit(b, H, v, g, n);
}
