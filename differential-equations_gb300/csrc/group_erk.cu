// group_erk.cu — dispatch of the group-per-system kernels (FP64_FAST and MIXED variants are
// instantiated here; the parity variants in inst_parity_group.cu, compiled with -fmad=false).
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <mutex>
#include <tuple>
#include <vector>

#include "group_erk.cuh"

namespace degpu {

std::map<GroupKey, GroupLaunch>& group_registry() {
    static std::map<GroupKey, GroupLaunch> m;
    return m;
}
std::map<GroupKey, GroupRoundOps>& group_round_registry() {
    static std::map<GroupKey, GroupRoundOps> m;
    return m;
}

void register_groups() {
    static std::once_flag once;
    std::call_once(once, []() {
        register_group_parity();
        register_group_fast();
        register_group_pair853();
        register_group_pair853_rounds();
        register_group_pair5();
        register_group_rounds();
    });
}

void register_group_fast() {
    reg_group<TabDop853, PrecFast, 8, 1>();
    reg_group<TabDop853, PrecFast, 16, 1>();
    reg_group<TabDop853, PrecFast, 32, 1>();
    reg_group<TabDop853, PrecFast, 16, 2>();
    reg_group<TabDop853, PrecFast, 16, 4>();
    reg_group<TabDop853, PrecFast, 32, 2>();
    reg_group<TabDop853, PrecFast, 32, 4>();
    reg_group<TabDop853, PrecFast, 32, 8>();
    reg_group<TabDop853, PrecMixed, 8, 1>();
    reg_group<TabDop853, PrecMixed, 16, 1>();
    reg_group<TabDop853, PrecMixed, 32, 1>();
    reg_group<TabDop853, PrecMixed, 16, 2>();
    reg_group<TabDop853, PrecMixed, 16, 4>();
    reg_group<TabDop853, PrecMixed, 32, 2>();
    reg_group<TabDop853, PrecMixed, 32, 4>();
    reg_group<TabDop853, PrecMixed, 32, 8>();
    reg_group<TabDopri5, PrecFast, 8, 1>();
    reg_group<TabDopri5, PrecFast, 16, 1>();
    reg_group<TabDopri5, PrecMixed, 8, 1>();
    reg_group<TabDopri5, PrecMixed, 16, 1>();
    reg_group<TabDopri5, PrecMixed, 32, 1>();
    reg_group<TabDopri5, PrecMixed, 32, 2>();
    reg_group<TabDopri5, PrecMixed, 32, 4>();
    reg_group<TabDopri5, PrecMixed, 32, 8>();
    reg_group<TabDopri5, PrecFast, 32, 1>();
    reg_group<TabDopri5, PrecFast, 32, 2>();
    reg_group<TabDopri5, PrecFast, 32, 4>();
    reg_group<TabDopri5, PrecFast, 32, 8>();
}

}  // namespace degpu

namespace degpu {

// (G lanes per system, CPL components per lane) by dimension bucket; the autotuner
// (degpu/autotune.py) may replace entries through degpu_internal_group_config or a tuning file
// named by DEGPU_TUNE_FILE with lines "method precision dense dmax G CPL".
struct GroupChoice {
    int dmax, g, cpl;
};

static std::map<std::tuple<int, int, int>, std::vector<GroupChoice>>& tune_table() {
    static std::map<std::tuple<int, int, int>, std::vector<GroupChoice>> m;
    return m;
}

static std::vector<GroupChoice> default_choices() {
    return {{8, 8, 1}, {16, 16, 1}, {32, 32, 1}, {64, 32, 2}, {128, 32, 4}, {256, 32, 8}};
}

static void load_tune_file() {
    static std::once_flag once;
    std::call_once(once, []() {
        const char* path = getenv("DEGPU_TUNE_FILE");
        if (!path) return;
        FILE* f = fopen(path, "r");
        if (!f) return;
        int m, p, dn, dmax, g, cpl;
        while (fscanf(f, "%d %d %d %d %d %d", &m, &p, &dn, &dmax, &g, &cpl) == 6) {
            auto& v = tune_table()[{m, p, dn}];
            if (v.empty()) v = default_choices();
            for (auto& c : v)
                if (c.dmax == dmax) c = {dmax, g, cpl};
        }
        fclose(f);
    });
}

static GroupChoice choose(int method, int prec, int dense, int d) {
    load_tune_file();
    auto it = tune_table().find({method, prec, dense});
    const std::vector<GroupChoice>& v = it != tune_table().end() ? it->second : default_choices();
    for (const auto& c : v)
        if (d <= c.dmax) return c;
    return {-1, 0, 0};
}

degpu_status group_solve(const degpu_problem* pb, const degpu_method_cfg* cfg, const EnsArgs& a, const int32_t* dims,
                        cudaStream_t s) {
    register_groups();
    if (!dims) return DEGPU_BAD_INPUT;
    if (cfg->method == DEGPU_RK4) return DEGPU_UNSUPPORTED;
    const int64_t n = a.n;
    std::vector<int32_t> hd(n);
    if (cudaMemcpyAsync(hd.data(), dims, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return DEGPU_CUDA_ERROR;
    const int dense = a.n_eval > 0 ? 1 : 0;
    // a mixed solve sends instances with rtol below the mixed-precision bound to its tight class
    const double split = mixed_split(cfg);
    std::vector<double> rtol_host;
    if (split > 0.0) {
        rtol_host.resize(n);
        if (cudaMemcpyAsync(rtol_host.data(), a.rtol, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
    }
    // buckets keyed by (precision, G, CPL)
    std::map<std::tuple<int, int, int>, std::vector<int64_t>> buckets;
    for (int64_t i = 0; i < n; ++i) {
        int d = hd[i];
        if (d <= 0 || d > pb->dim || (d & 1)) return DEGPU_BAD_INPUT;
        int prec = cfg->precision;
        GroupChoice c{};
        if (split > 0.0 && rtol_host[i] < split) {
            // the tight class: FP32-pair stages where built for this layout, else FP64 fast
            prec = mixed_low_precision(cfg);
            c = choose(cfg->method, prec, dense, d);
            if (c.dmax < 0 || !group_registry().count(GroupKey{cfg->method, prec, dense, c.g, c.cpl}))
                prec = DEGPU_FP64_FAST;
        }
        if (prec != PrecMixedPair::ID) c = choose(cfg->method, prec, dense, d);
        if (c.dmax < 0) return DEGPU_UNSUPPORTED;
        buckets[{prec, c.g, c.cpl}].push_back(i);
    }
    // longest first inside a bucket: the largest systems start first, the tail holds small ones
    for (auto& b : buckets)
        std::stable_sort(b.second.begin(), b.second.end(), [&](int64_t x, int64_t y) { return hd[x] > hd[y]; });
    std::vector<void*> to_free;
    degpu_status st = DEGPU_OK;
    for (auto& b : buckets) {
        const int prec = std::get<0>(b.first);
        auto it = group_registry().find(GroupKey{cfg->method, prec, dense, std::get<1>(b.first), std::get<2>(b.first)});
        if (it == group_registry().end()) {
            st = DEGPU_UNSUPPORTED;
            break;
        }
        int64_t* d_idx = nullptr;
        unsigned long long* d_tk = nullptr;
        if (cudaMallocAsync((void**)&d_idx, b.second.size() * sizeof(int64_t), s) != cudaSuccess ||
            cudaMallocAsync((void**)&d_tk, sizeof(unsigned long long), s) != cudaSuccess) {
            st = DEGPU_OOM;
            break;
        }
        to_free.push_back(d_idx);
        to_free.push_back(d_tk);
        if (cudaMemcpyAsync(d_idx, b.second.data(), b.second.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemsetAsync(d_tk, 0, sizeof(unsigned long long), s) != cudaSuccess) {
            st = DEGPU_CUDA_ERROR;
            break;
        }
        GroupArgs ga;
        ga.a = a;
        ga.a.index = d_idx;
        ga.a.count = (int64_t)b.second.size();
        ga.a.ticket = d_tk;
        ga.dims = dims;
        if (it->second(ga, s) != cudaSuccess) {
            st = DEGPU_CUDA_ERROR;
            break;
        }
    }
    // the index lists come from host vectors that die with this call
    if (cudaStreamSynchronize(s) != cudaSuccess && st == DEGPU_OK) st = DEGPU_CUDA_ERROR;
    for (void* p : to_free) cudaFreeAsync(p, s);
    return st;
}

}  // namespace degpu

namespace degpu {

degpu_status group_round_parts(const degpu_problem* pb, const degpu_method_cfg* cfg, const int32_t* dims_host,
                               const double* rtol_host, int64_t n, int dense, std::vector<GroupRoundPart>& parts) {
    parts.clear();
    if (!dims_host || cfg->method == DEGPU_RK4) return DEGPU_UNSUPPORTED;
    const double split = mixed_split(cfg);
    std::map<std::tuple<int, int, int>, size_t> slot;
    for (int64_t i = 0; i < n; ++i) {
        const int d = dims_host[i];
        if (d <= 0 || d > pb->dim || (d & 1)) return DEGPU_BAD_INPUT;
        int prec = cfg->precision;
        GroupChoice c{};
        if (split > 0.0 && rtol_host[i] < split) {
            prec = mixed_low_precision(cfg);  // as in group_solve
            c = choose(cfg->method, prec, dense, d);
            if (c.dmax < 0 || !group_round_registry().count(GroupKey{cfg->method, prec, dense, c.g, c.cpl}) ||
                !group_registry().count(GroupKey{cfg->method, prec, dense, c.g, c.cpl}))
                prec = DEGPU_FP64_FAST;
        }
        if (prec != PrecMixedPair::ID) c = choose(cfg->method, prec, dense, d);
        if (c.dmax < 0) return DEGPU_UNSUPPORTED;
        const auto key = std::make_tuple(prec, c.g, c.cpl);
        auto it = slot.find(key);
        if (it == slot.end()) {
            auto r = group_round_registry().find(GroupKey{cfg->method, prec, dense, c.g, c.cpl});
            if (r == group_round_registry().end()) return DEGPU_UNSUPPORTED;
            it = slot.emplace(key, parts.size()).first;
            parts.push_back(GroupRoundPart{r->second, {}});
        }
        parts[it->second].idx.push_back(i);
    }
    // the largest systems first inside a part, as in group_solve
    for (auto& p : parts)
        std::stable_sort(p.idx.begin(), p.idx.end(), [&](int64_t x, int64_t y) { return dims_host[x] > dims_host[y]; });
    return DEGPU_OK;
}

}  // namespace degpu

extern "C" int degpu_internal_group_config(int method, int prec, int dense, int dmax, int g, int cpl) {
    using namespace degpu;
    auto& v = tune_table()[{method, prec, dense}];
    if (v.empty()) v = default_choices();
    for (auto& c : v)
        if (c.dmax == dmax) {
            c = {dmax, g, cpl};
            return 0;
        }
    return 1;
}
