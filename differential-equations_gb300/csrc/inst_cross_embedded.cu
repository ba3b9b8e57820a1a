// inst_cross_embedded.cu — crossing-detection kernels of the adaptive methods (RKF45,
// Cash-Karp), FP64 fast and mixed arithmetic.
#include "registry.cuh"

namespace degpu {

void register_cross_embedded_fast_mixed() {
    register_cross_embedded_methods<RhsVanDerPol, PrecFast>();
    register_cross_embedded_methods<RhsPendulum, PrecFast>();
    register_cross_embedded_methods<RhsLorenz, PrecFast>();
    register_cross_embedded_methods<RhsVanDerPol, PrecMixed>();
    register_cross_embedded_methods<RhsPendulum, PrecMixed>();
    register_cross_embedded_methods<RhsLorenz, PrecMixed>();
}

}  // namespace degpu
