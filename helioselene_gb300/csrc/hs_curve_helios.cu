// hs_curve_helios.cu -- instantiates the MSM kernels for the Helios curve.
#include "hs_msm_impl.cuh"

namespace hs {
const CurveOps helios_ops = make_ops<HeliosCurve>();
}  // namespace hs
