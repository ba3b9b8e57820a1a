// nvrtc_rhs.cu — right-hand sides supplied as CUDA source at run time (degpu_register_rhs_nvrtc).
//
// The user source defines
//     template <class R> __device__ void NAME(R t, const R* y, R* dydt, const double* p);
// the CUDA twin of `ODE::diff(&self, t, &y, &mut dydt)` (src/ode/ode.rs:20-44) with the
// system's fields in p[0..n_params).  Registration compiles the integrator headers plus that
// source with NVRTC for this GPU: once with -fmad=false (the parity variants), once with
// contraction (FP64_FAST / MIXED), and once more for DOPRI5's FP32-pair stages (the tight class
// of a MIXED solve) with R = degpu::df.  The last build is optional: a source that does not
// compile for pairs (it calls a function with no pair overload) runs its tight class in
// FP64_FAST.  The kernels load through the runtime's library API.

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "side_paths.cuh"

namespace degpu {
int device_sm_count();
double mixed_split(const degpu_method_cfg* cfg);
}

namespace degpu {

struct NvrtcRhs {
    int dim, n_params;
    cudaLibrary_t mod[3] = {nullptr, nullptr, nullptr};  // parity, contracted and pair builds
    // [method][prec: parity, fast, mixed, pair][dense][kernel: 0 thread, 1 persistent]
    cudaKernel_t fn[3][4][2][2] = {};
};

static std::mutex g_mu;
static std::vector<NvrtcRhs*> g_rhs;

static std::string csrc_dir() {
    Dl_info info;
    if (dladdr((void*)&csrc_dir, &info) && info.dli_fname) {
        std::string p(info.dli_fname);
        auto s = p.rfind('/');
        if (s != std::string::npos) return p.substr(0, s);
    }
    return ".";
}

static const char* kMethods[3] = {"TabRK4", "TabDopri5", "TabDop853"};
static const char* kPrecs[4] = {"PrecParity", "PrecFast", "PrecMixed", "PrecMixedPair"};
// the build that holds (method m, precision slot p): 0 parity, 1 contracted, 2 pair stages
static int build_of(int m, int p) { return p == 0 ? 0 : p == 3 ? (m == 1 ? 2 : -1) : 1; }

static std::string kernel_name(int m, int p, int dense, int persistent) {
    return std::string("degpu::") + (persistent ? "erk_persistent_kernel<" : "erk_thread_kernel<") + "degpu::" +
           kMethods[m] + ", degpu::RhsUser, degpu::" + kPrecs[p] + ", " + (dense ? "true" : "false") + ">";
}

static degpu_status compile_module(const std::string& src, int build, NvrtcRhs* r, std::string& log) {
    const bool parity = build == 0;
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "degpu_user_rhs.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        return DEGPU_CUDA_ERROR;
    std::vector<std::string> names;
    for (int m = 0; m < 3; ++m)
        for (int p = 0; p < 4; ++p) {
            if (build_of(m, p) != build) continue;
            for (int d = 0; d < 2; ++d)
                for (int k = 0; k < 2; ++k) {
                    names.push_back(kernel_name(m, p, d, k));
                    nvrtcAddNameExpression(prog, names.back().c_str());
                }
        }
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    std::string arch = "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor) + "a";
    std::string inc1 = "-I" + csrc_dir();
    std::string inc2 = "-I" + csrc_dir() + "/../../include";
    std::vector<const char*> opts = {arch.c_str(), "-std=c++17", inc1.c_str(), inc2.c_str(), "-default-device",
                                     parity ? "-fmad=false" : "-fmad=true"};
    nvrtcResult rc = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    if (ls > 1) {
        std::string l(ls, '\0');
        nvrtcGetProgramLog(prog, &l[0]);
        log += l;
    }
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return DEGPU_BAD_INPUT;
    }
    size_t cs = 0;
    nvrtcGetCUBINSize(prog, &cs);
    std::vector<char> cubin(cs);
    nvrtcGetCUBIN(prog, cubin.data());
    cudaLibrary_t mod;
    if (cudaLibraryLoadData(&mod, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
        nvrtcDestroyProgram(&prog);
        return DEGPU_CUDA_ERROR;
    }
    r->mod[build] = mod;
    for (int m = 0; m < 3; ++m)
        for (int p = 0; p < 4; ++p) {
            if (build_of(m, p) != build) continue;
            for (int d = 0; d < 2; ++d)
                for (int k = 0; k < 2; ++k) {
                    std::string nm = kernel_name(m, p, d, k);
                    const char* lowered = nullptr;
                    if (nvrtcGetLoweredName(prog, nm.c_str(), &lowered) != NVRTC_SUCCESS ||
                        cudaLibraryGetKernel(&r->fn[m][p][d][k], mod, lowered) != cudaSuccess) {
                        nvrtcDestroyProgram(&prog);
                        return DEGPU_CUDA_ERROR;
                    }
                }
        }
    nvrtcDestroyProgram(&prog);
    return DEGPU_OK;
}

degpu_status nvrtc_rhs_info(int32_t id, int32_t* dim, int32_t* n_params) {
    std::lock_guard<std::mutex> g(g_mu);
    int k = id - DEGPU_RHS_NVRTC_BASE;
    if (k < 0 || k >= (int)g_rhs.size()) return DEGPU_BAD_INPUT;
    if (dim) *dim = g_rhs[k]->dim;
    if (n_params) *n_params = g_rhs[k]->n_params;
    return DEGPU_OK;
}

degpu_status nvrtc_solve(const degpu_problem* pb, const degpu_method_cfg* cfg, const degpu_batch_in* in,
                         degpu_batch_out* out, cudaStream_t s) {
    NvrtcRhs* r;
    {
        std::lock_guard<std::mutex> g(g_mu);
        int k = pb->rhs_id - DEGPU_RHS_NVRTC_BASE;
        if (k < 0 || k >= (int)g_rhs.size()) return DEGPU_BAD_INPUT;
        r = g_rhs[k];
    }
    if (in->family || in->dims || pb->dim != r->dim || pb->n_params < r->n_params) return DEGPU_BAD_INPUT;
    const int64_t n = in->n;
    EnsArgs a{};
    a.n = n;
    a.count = n;
    a.t0 = in->t0;
    a.tf = in->tf;
    a.y0 = in->y0;
    a.params = in->params;
    a.rtol = in->rtol;
    a.atol = in->atol;
    a.rtol_vec = in->rtol_vec;
    a.atol_vec = in->atol_vec;
    a.dmax = pb->dim;
    a.y_final = out->y_final;
    a.t_final = out->t_final;
    a.accepted = out->accepted;
    a.rejected = out->rejected;
    a.fevals = out->fevals;
    a.status = out->status;
    a.h0 = cfg->h0;
    a.h_min = cfg->h_min;
    a.h_max = cfg->h_max;
    a.max_steps = cfg->max_steps;
    a.safety = cfg->safety_factor;
    a.min_scale = cfg->min_scale;
    a.max_scale = cfg->max_scale;
    a.safety_f = (float)a.safety;
    a.min_scale_f = (float)a.min_scale;
    a.max_scale_f = (float)a.max_scale;
    a.dense_mode = cfg->dense_mode;
    a.n_params = pb->n_params;
    if (in->n_eval > 0) return DEGPU_UNSUPPORTED;  // dense output for run-time systems: not built
    // run-time systems have RK4, DOPRI5 and DOP853 in the parity, FP64_FAST and MIXED forms
    if (cfg->method < DEGPU_RK4 || cfg->method > DEGPU_DOP853) return DEGPU_UNSUPPORTED;
    if (cfg->precision != DEGPU_FP64_PARITY && cfg->precision != DEGPU_FP64_FAST && cfg->precision != DEGPU_MIXED)
        return DEGPU_UNSUPPORTED;
    const int m = cfg->method, persistent = cfg->kernel == DEGPU_KERNEL_PERSISTENT ? 1 : 0;
    // a MIXED solve sends the instances with rtol below the bound to the pair stages (DOPRI5,
    // when the source built for pairs) or to FP64_FAST, like a built-in system's
    struct Part {
        int prec;
        std::vector<int64_t> idx;
    };
    std::vector<Part> parts;
    const double split = mixed_split(cfg);
    if (split > 0.0) {
        std::vector<double> rt(n);
        if (cudaMemcpyAsync(rt.data(), in->rtol, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return DEGPU_CUDA_ERROR;
        const int low = r->fn[m][3][0][persistent] ? 3 : DEGPU_FP64_FAST;
        parts.push_back(Part{low, {}});
        parts.push_back(Part{DEGPU_MIXED, {}});
        for (int64_t i = 0; i < n; ++i) parts[rt[i] < split ? 0 : 1].idx.push_back(i);
    } else {
        parts.push_back(Part{cfg->precision, {}});
    }
    std::vector<void*> scratch;
    degpu_status st = DEGPU_OK;
    for (const Part& pt : parts) {
        if (split > 0.0 && pt.idx.empty()) continue;
        cudaKernel_t f = r->fn[m][pt.prec][0][persistent];
        if (!f) {
            st = DEGPU_UNSUPPORTED;
            break;
        }
        EnsArgs ga = a;
        if (split > 0.0) {
            int64_t* d_idx = nullptr;
            if (cudaMallocAsync((void**)&d_idx, pt.idx.size() * sizeof(int64_t), s) != cudaSuccess) {
                st = DEGPU_OOM;
                break;
            }
            scratch.push_back(d_idx);
            if (cudaMemcpyAsync(d_idx, pt.idx.data(), pt.idx.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s) !=
                cudaSuccess) {
                st = DEGPU_CUDA_ERROR;
                break;
            }
            ga.index = d_idx;
            ga.count = (int64_t)pt.idx.size();
        }
        unsigned grid;
        if (persistent) {
            unsigned long long* tk = nullptr;
            if (cudaMallocAsync((void**)&tk, sizeof(unsigned long long), s) != cudaSuccess) {
                st = DEGPU_OOM;
                break;
            }
            scratch.push_back(tk);
            if (cudaMemsetAsync(tk, 0, sizeof(unsigned long long), s) != cudaSuccess) {
                st = DEGPU_CUDA_ERROR;
                break;
            }
            ga.ticket = tk;
            int bps = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)f, 128, 0);
            long long g = (long long)(bps > 0 ? bps : 1) * device_sm_count();
            long long need = (ga.count + 127) / 128;
            grid = (unsigned)(g < need ? g : need);
        } else {
            grid = (unsigned)((ga.count + 127) / 128);
        }
        void* args[] = {&ga};
        if (cudaLaunchKernel((const void*)f, dim3(grid), dim3(128), args, 0, s) != cudaSuccess) {
            st = DEGPU_CUDA_ERROR;
            break;
        }
    }
    // the index lists come from host vectors that die with this call
    if (split > 0.0 && cudaStreamSynchronize(s) != cudaSuccess && st == DEGPU_OK) st = DEGPU_CUDA_ERROR;
    for (void* q : scratch) cudaFreeAsync(q, s);
    return st;
}

}  // namespace degpu

using namespace degpu;

extern "C" degpu_status degpu_register_rhs_nvrtc(const char* source, const char* name, int32_t dim, int32_t n_params,
                                                 int32_t* rhs_id, char* log, size_t log_size) {
    if (!source || !name || !rhs_id || dim <= 0 || dim > 64 || n_params < 0 || n_params > 64) return DEGPU_BAD_INPUT;
    cudaFree(nullptr);  // make sure a context exists for the driver API
    std::string src;
    src += "#include \"erk_core.cuh\"\n";
    src += source;
    src += "\nnamespace degpu {\nstruct RhsUser {\n";
    src += "  static constexpr int ID = 1000, D = " + std::to_string(dim) + ", NP = " + std::to_string(n_params) + ";\n";
    src += "  template <class P> __device__ static __forceinline__ void diff(double t, const typename P::S* y, "
           "typename P::S* dydt, const double* p) {\n";
    src += "    ::" + std::string(name) + "<typename P::S>((typename P::S)t, y, dydt, p);\n  }\n};\n}\n";
    NvrtcRhs* r = new NvrtcRhs();
    r->dim = dim;
    r->n_params = n_params;
    std::string lg;
    degpu_status st = compile_module(src, 0, r, lg);
    if (st == DEGPU_OK) st = compile_module(src, 1, r, lg);
    if (st == DEGPU_OK) {
        std::string plog;
        if (compile_module(src, 2, r, plog) != DEGPU_OK) {
            // optional: the tight class of a MIXED solve then runs in FP64_FAST
            if (r->mod[2]) cudaLibraryUnload(r->mod[2]);
            r->mod[2] = nullptr;
            for (auto& fm : r->fn)
                for (auto& fd : fm[3])
                    for (auto& fk : fd) fk = nullptr;
            lg += "note: no FP32-pair build of this source (the tight class of MIXED solves runs in FP64_FAST)\n";
        }
    }
    if (log && log_size) {
        size_t k = lg.size() < log_size - 1 ? lg.size() : log_size - 1;
        memcpy(log, lg.data(), k);
        log[k] = 0;
    }
    if (st != DEGPU_OK) {
        for (cudaLibrary_t m : r->mod)
            if (m) cudaLibraryUnload(m);
        delete r;
        return st;
    }
    std::lock_guard<std::mutex> g(g_mu);
    g_rhs.push_back(r);
    *rhs_id = DEGPU_RHS_NVRTC_BASE + (int32_t)g_rhs.size() - 1;
    return DEGPU_OK;
}
