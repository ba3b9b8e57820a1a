// inst_parity_verner_cross98.cu — crossing, hyperplane and event detection with Verner's pairs
// RKV988E/RKV989E (FP64 parity arithmetic, compiled with -fmad=false like every inst_parity_*
// translation unit).
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg() {
    cross_registry()[VariantKey{DEGPU_RKV988E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV988E, Rhs, PrecParity>;
    cross_registry()[VariantKey{DEGPU_RKV989E, Rhs::ID, PrecParity::ID, 1}] = &launch_cross<TabRKV989E, Rhs, PrecParity>;
}

void register_verner_cross98_parity() {
    reg<RhsHarmonic>();
    reg<RhsVanDerPol>();
    reg<RhsPendulum>();
    reg<RhsLorenz>();
}

}  // namespace degpu
