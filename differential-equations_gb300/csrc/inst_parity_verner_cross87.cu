// inst_parity_verner_cross87.cu — crossing, hyperplane and event detection with Verner's pairs
// RKV877E/RKV878E (FP64 parity arithmetic, compiled with -fmad=false like every inst_parity_*
// translation unit).
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg() {
    cross_registry()[VariantKey{DEGPU_RKV877E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV877E, Rhs, PrecParity>;
    cross_registry()[VariantKey{DEGPU_RKV878E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV878E, Rhs, PrecParity>;
}

void register_verner_cross87_parity() {
    reg<RhsHarmonic>();
    reg<RhsVanDerPol>();
    reg<RhsPendulum>();
    reg<RhsLorenz>();
}

}  // namespace degpu
