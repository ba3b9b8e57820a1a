// inst_parity_cross_embedded.cu — crossing-detection kernels of the adaptive methods (RKF45,
// Cash-Karp), FP64 parity arithmetic (compiled with -fmad=false like every inst_parity_*
// translation unit).
#include "registry.cuh"

namespace degpu {

void register_cross_embedded_parity() {
    register_cross_embedded_methods<RhsVanDerPol, PrecParity>();
    register_cross_embedded_methods<RhsPendulum, PrecParity>();
    register_cross_embedded_methods<RhsLorenz, PrecParity>();
    register_cross_embedded_methods<RhsHarmonic, PrecParity>();
    register_cross_embedded_methods<RhsBrusselator, PrecParity>();
    register_cross_embedded_methods<RhsCr3bp, PrecParity>();
    register_cross_embedded_methods<RhsLogistic, PrecParity>();
    register_cross_embedded_methods<RhsExpGrowth, PrecParity>();
}

}  // namespace degpu
