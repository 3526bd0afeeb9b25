// hs_curve_selene.cu -- instantiates the MSM kernels for the Selene curve.
#include "hs_msm_impl.cuh"

namespace hs {
const CurveOps selene_ops = make_ops<SeleneCurve>();
}  // namespace hs
