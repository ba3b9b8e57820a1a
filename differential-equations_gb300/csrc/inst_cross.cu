// inst_cross.cu — crossing- and event-detection kernels, FP64 fast and mixed arithmetic.
#include "registry.cuh"

namespace degpu {

void register_cross_fast_mixed() {
    register_cross_all_methods<RhsVanDerPol, PrecFast>();
    register_cross_all_methods<RhsPendulum, PrecFast>();
    register_cross_all_methods<RhsLorenz, PrecFast>();
    register_cross_all_methods<RhsHarmonic, PrecFast>();
    register_cross_all_methods<RhsBrusselator, PrecFast>();
    register_cross_all_methods<RhsCr3bp, PrecFast>();
    register_cross_all_methods<RhsLogistic, PrecFast>();
    register_cross_all_methods<RhsExpGrowth, PrecFast>();
    register_cross_all_methods<RhsVanDerPol, PrecMixed>();
    register_cross_all_methods<RhsPendulum, PrecMixed>();
    register_cross_all_methods<RhsLorenz, PrecMixed>();
    register_cross_all_methods<RhsHarmonic, PrecMixed>();
    register_cross_all_methods<RhsBrusselator, PrecMixed>();
    register_cross_all_methods<RhsCr3bp, PrecMixed>();
    register_cross_all_methods<RhsLogistic, PrecMixed>();
    register_cross_all_methods<RhsExpGrowth, PrecMixed>();
    // DOPRI5's tight class (FP32-pair stages) for the production families, as in the
    // multi-family kernel; the other families' tight class runs FP64 fast
    cross_registry()[VariantKey{DEGPU_DOPRI5, RhsVanDerPol::ID, PrecMixedPair::ID, 1}] =
        &launch_cross<TabDopri5, RhsVanDerPol, PrecMixedPair>;
    cross_registry()[VariantKey{DEGPU_DOPRI5, RhsPendulum::ID, PrecMixedPair::ID, 1}] =
        &launch_cross<TabDopri5, RhsPendulum, PrecMixedPair>;
    cross_registry()[VariantKey{DEGPU_DOPRI5, RhsLorenz::ID, PrecMixedPair::ID, 1}] =
        &launch_cross<TabDopri5, RhsLorenz, PrecMixedPair>;
}

}  // namespace degpu
