// inst_verner_cross_b.cu — crossing, hyperplane and event detection with Verner's pairs
// RKV877E, RKV878E, RKV988E and RKV989E in FP64 fast arithmetic (what a mixed solve of these pairs runs).
#include "registry.cuh"

namespace degpu {

template <class Rhs>
static void reg() {
    cross_registry()[VariantKey{DEGPU_RKV877E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV877E, Rhs, PrecFast>;
    cross_registry()[VariantKey{DEGPU_RKV878E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV878E, Rhs, PrecFast>;
    cross_registry()[VariantKey{DEGPU_RKV988E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV988E, Rhs, PrecFast>;
    cross_registry()[VariantKey{DEGPU_RKV989E, Rhs::ID, PrecFast::ID, 1}] = &launch_cross<TabRKV989E, Rhs, PrecFast>;
}

void register_verner_cross8798_fast() {
    reg<RhsVanDerPol>();
    reg<RhsPendulum>();
    reg<RhsLorenz>();
}

}  // namespace degpu
