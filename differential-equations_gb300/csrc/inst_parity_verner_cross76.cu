// inst_parity_verner_cross76.cu — crossing, hyperplane and event detection with Verner's pairs
// RKV766E/RKV767E (FP64 parity arithmetic, compiled with -fmad=false like every inst_parity_*
// translation unit).
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg() {
    cross_registry()[VariantKey{DEGPU_RKV766E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV766E, Rhs, PrecParity>;
    cross_registry()[VariantKey{DEGPU_RKV767E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV767E, Rhs, PrecParity>;
}

void register_verner_cross76_parity() {
    reg<RhsHarmonic>();
    reg<RhsVanDerPol>();
    reg<RhsPendulum>();
    reg<RhsLorenz>();
}

}  // namespace degpu
