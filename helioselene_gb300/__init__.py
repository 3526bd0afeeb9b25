"""helioselene_gb300 -- GB300-native variable-time MSM for the Helios/Selene cycle.

The compute path is libhelioselene_gb300.so (hand-written sm_103a CUDA behind
the C ABI in include/helioselene_gb300.h); this package loads it and mirrors the
reference's point API for the MSM path.  There is no CPU implementation.
"""

from ._lib import (FMT_AFFINE, FMT_AFFINE51, FMT_BYTES, FMT_COMPRESSED, FMT_JACOBIAN51, HELIOS, SELENE,
                   HsError, LIB_PATH, load)
from .api import (Context, FixedBase, HeliosPoint, Server, SelenePoint, affine64_to_jac51, default_context, fe51_to_int,
                  helios_batch_to_affine, int_to_fe51, jac51_from_ints, selene_batch_to_affine)

__all__ = [
    "Context", "FixedBase", "Server", "HeliosPoint", "SelenePoint", "HsError", "load", "LIB_PATH", "default_context",
    "helios_batch_to_affine", "selene_batch_to_affine", "affine64_to_jac51", "jac51_from_ints",
    "int_to_fe51", "fe51_to_int",
    "HELIOS", "SELENE", "FMT_JACOBIAN51", "FMT_AFFINE51", "FMT_AFFINE", "FMT_COMPRESSED", "FMT_BYTES",
]
