// inst_parity_verner_cross65.cu — crossing, hyperplane and event detection with Verner's pairs
// RKV655E/RKV656E (FP64 parity arithmetic, compiled with -fmad=false like every inst_parity_*
// translation unit).
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg() {
    cross_registry()[VariantKey{DEGPU_RKV655E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV655E, Rhs, PrecParity>;
    cross_registry()[VariantKey{DEGPU_RKV656E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV656E, Rhs, PrecParity>;
}

void register_verner_cross65_parity() {
    reg<RhsHarmonic>();
    reg<RhsVanDerPol>();
    reg<RhsPendulum>();
    reg<RhsLorenz>();
}

}  // namespace degpu
