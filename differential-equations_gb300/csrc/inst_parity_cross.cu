// inst_parity_cross.cu — crossing- and event-detection kernels, FP64 parity arithmetic (compiled with
// -fmad=false like every inst_parity_* translation unit).
#include "registry.cuh"

namespace degpu {

void register_cross_parity() {
    register_cross_all_methods<RhsVanDerPol, PrecParity>();
    register_cross_all_methods<RhsPendulum, PrecParity>();
    register_cross_all_methods<RhsLorenz, PrecParity>();
    register_cross_all_methods<RhsHarmonic, PrecParity>();
    register_cross_all_methods<RhsBrusselator, PrecParity>();
    register_cross_all_methods<RhsCr3bp, PrecParity>();
    register_cross_all_methods<RhsLogistic, PrecParity>();
    register_cross_all_methods<RhsExpGrowth, PrecParity>();
}

}  // namespace degpu
