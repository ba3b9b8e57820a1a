// mol.cu — entry points of the general method-of-lines path (degpu_mol_rhs, degpu_mol_rk4) and
// its FP64 (contracted) and FP32 drivers; the parity drivers are in inst_parity_mol.cu.
#include <mutex>

#include "mol.cuh"

namespace degpu {

std::map<std::tuple<int, int, int, int>, MolOps>& mol_registry() {
    static std::map<std::tuple<int, int, int, int>, MolOps> m;
    return m;
}

void register_mol_fast() {
    register_mol_all<double>(1);
    register_mol_all<float>(2);
}

static const MolOps* mol_ops(const degpu_mol* m, int32_t precision) {
    static std::once_flag once;
    std::call_once(once, []() {
        register_mol_parity();
        register_mol_fast();
    });
    int cls;
    switch (precision) {
        case DEGPU_FP64_PARITY: cls = 0; break;
        case DEGPU_FP64_FAST:
        case DEGPU_FP64_PLAIN: cls = 1; break;
        case DEGPU_MIXED: cls = 2; break;
        default: return nullptr;
    }
    auto it = mol_registry().find({m->pde_id, m->dims, m->fields, cls});
    return it == mol_registry().end() ? nullptr : &it->second;
}

}  // namespace degpu

using namespace degpu;

extern "C" {

degpu_status degpu_mol_rhs(const degpu_mol* mol, int32_t precision, double t, const void* y, void* dydt,
                           void* stream) {
    if (!mol_valid(mol) || !y || !dydt) return DEGPU_BAD_INPUT;
    const MolOps* ops = mol_ops(mol, precision);
    if (!ops) return precision < DEGPU_FP64_PARITY || precision > DEGPU_MIXED_FP64_CTRL ? DEGPU_BAD_INPUT
                                                                                         : DEGPU_UNSUPPORTED;
    return ops->rhs(mol, t, y, dydt, (cudaStream_t)stream);
}

degpu_status degpu_mol_rk4(const degpu_mol* mol, int32_t precision, double t0, double tf, double h, void* y,
                           int64_t* steps, void* stream) {
    if (!mol_valid(mol) || !y) return DEGPU_BAD_INPUT;
    // validate_step_size_parameters (src/utils.rs:60-157): a non-zero step no longer than the
    // interval, pointing from t0 to tf
    if (!(tf != t0) || !(h != 0.0) || !isfinite(h) || (h > 0.0) != (tf > t0) || fabs(h) > fabs(tf - t0))
        return DEGPU_BAD_INPUT;
    const MolOps* ops = mol_ops(mol, precision);
    if (!ops) return precision < DEGPU_FP64_PARITY || precision > DEGPU_MIXED_FP64_CTRL ? DEGPU_BAD_INPUT
                                                                                         : DEGPU_UNSUPPORTED;
    return ops->rk4(mol, t0, tf, h, y, steps, (cudaStream_t)stream);
}

}  // extern "C"
