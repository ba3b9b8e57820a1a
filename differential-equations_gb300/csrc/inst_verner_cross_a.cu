// inst_verner_cross_a.cu — crossing, hyperplane and event detection with Verner's pairs
// RKV655E, RKV656E, RKV766E and RKV767E in FP64 fast arithmetic (what a mixed solve of these pairs runs).
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg() {
    cross_registry()[VariantKey{DEGPU_RKV655E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV655E, Rhs, PrecFast>;
    cross_registry()[VariantKey{DEGPU_RKV656E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV656E, Rhs, PrecFast>;
    cross_registry()[VariantKey{DEGPU_RKV766E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV766E, Rhs, PrecFast>;
    cross_registry()[VariantKey{DEGPU_RKV767E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV767E, Rhs, PrecFast>;
}

void register_verner_cross6576_fast() {
    reg<RhsVanDerPol>();
    reg<RhsPendulum>();
    reg<RhsLorenz>();
}

}  // namespace degpu
