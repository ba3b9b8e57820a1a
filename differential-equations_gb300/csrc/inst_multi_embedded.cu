// inst_multi_embedded.cu — multi-family persistent kernels of the order-5 embedded pairs (RKF45,
// Cash-Karp), FP64 fast and mixed, with and without output times.
#include "registry.cuh"

namespace degpu {
void register_multi_embedded() {
    register_multi<TabRKF45, PrecFast>();
    register_multi<TabRKF45, PrecMixed>();
    register_multi<TabCashKarp, PrecFast>();
    register_multi<TabCashKarp, PrecMixed>();
}
}  // namespace degpu
