// server.cu — continuous-batching server over the ensemble kernels (degpu_server_*).
//
// One scheduler thread owns the device side.  Each loop:
//   1. admits queued requests in arrival order while the memory budget and the active-slot
//      count allow (first-come first-served: a request that does not fit waits, later ones wait
//      behind it, so none starves);
//   2. for every admitted request on its own stream: copies its inputs in, clears its resident
//      state, and launches the first round;
//   3. for every request whose last round has completed (an event): if all instances are done it
//      copies the outputs back, otherwise it launches the next round; the resident state
//      (Parked lanes: t, h, y, derivative, counters, controller state) never leaves the device.
// Rounds are bounded (`round_budget` driver iterations per instance), so the GPU is shared
// between the requests in flight and a new request starts within one round of being admitted.
// Requests with output times run round kernels that also write them (the times sorted once, as
// TEvalSolout::new sorts them).  Ragged FPU-beta requests run the resumable group kernels, one
// round kernel per (precision, layout) bucket.  Requests the round kernels do not cover (run-time
// families, family maps, parity-form chains) are solved with one degpu_solve_ensemble call on the
// request's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "group_erk.cuh"
#include "registry.cuh"

namespace degpu {

using Clock = std::chrono::steady_clock;

struct SrvRequest {
    uint64_t id;
    degpu_problem pb;
    degpu_method_cfg cfg;
    degpu_batch_in in;    // host
    degpu_batch_out out;  // host
    Clock::time_point t_submit, t_done;
    int state = 0;  // 0 queued, 1 rounds running, 2 copying out, 3 done
    degpu_status result = DEGPU_OK;
    size_t bytes = 0;
    bool resumable = false;
    // The round kernels of a resumable request, each over its own instances with its own
    // resident state and work ticket: one part for a plain request; a mixed request whose rtol
    // values straddle the mixed-precision bound has a second part (the tight class); a ragged
    // request has one part per (precision, layout) bucket of the group kernels.  An empty index
    // list means every instance.
    struct Part {
        RoundOps ops{};
        std::vector<int64_t> idx;
        EnsArgs args{};
        void* park = nullptr;
        unsigned long long* ticket = nullptr;
    };
    std::vector<Part> parts;
    // device side
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    char* dblock = nullptr;
    degpu_batch_in din{};
    degpu_batch_out dout{};
    unsigned long long* done_dev = nullptr;
    unsigned long long* done_host = nullptr;  // pinned
    // output times of a resumable request: ascending, with the permutation to the caller's order
    std::vector<double> te_sorted;
    std::vector<int32_t> te_perm;
};

struct ServerImpl {
    degpu_server_cfg cfg;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::shared_ptr<SrvRequest>> queue;
    std::map<uint64_t, std::shared_ptr<SrvRequest>> all;
    std::vector<std::shared_ptr<SrvRequest>> active;
    std::vector<cudaStream_t> free_streams;
    std::atomic<bool> stop{false};
    uint64_t next_id = 1;
    size_t used = 0;
    std::thread th;

    static size_t align(size_t x) { return (x + 255) & ~(size_t)255; }

    size_t footprint(const SrvRequest& r) const {
        const size_t n = (size_t)r.in.n, d = (size_t)r.pb.dim, np = (size_t)(r.pb.n_params > 0 ? r.pb.n_params : 1);
        const size_t m = (size_t)(r.in.n_eval > 0 ? r.in.n_eval : 0);
        size_t b = align(n * 8) * 6 + align(d * n * 8) * 2 + align(np * n * 8) + align(n * 4) * 3 + align(n * 8) * 3;
        b += align(m * 8) + align(m * d * n * 8) + align(m * 4);
        if (r.in.rtol_vec) b += align(d * n * 8);
        if (r.in.atol_vec) b += align(d * n * 8);
        if (r.resumable) {
            b += 512;  // done counter
            for (const auto& pt : r.parts) {
                const size_t cnt = pt.idx.empty() ? n : pt.idx.size();
                b += align(pt.idx.size() * 8) + align(cnt * pt.ops.park_bytes) + 256;
            }
        }
        return b;
    }

    bool start_request(SrvRequest& r) {
        const size_t n = (size_t)r.in.n, d = (size_t)r.pb.dim, np = (size_t)(r.pb.n_params > 0 ? r.pb.n_params : 1);
        const size_t m = (size_t)(r.in.n_eval > 0 ? r.in.n_eval : 0);
        cudaStream_t s = r.stream;
        if (cudaMallocAsync((void**)&r.dblock, r.bytes, s) != cudaSuccess) return false;
        char* p = r.dblock;
        auto take = [&](size_t bytes) {
            char* q = p;
            p += align(bytes);
            return q;
        };
        auto up = [&](const void* src, size_t bytes) -> void* {
            if (!src) return nullptr;
            void* dst = take(bytes);
            cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
            return dst;
        };
        r.din = r.in;
        r.din.t0 = (const double*)up(r.in.t0, n * 8);
        r.din.tf = (const double*)up(r.in.tf, n * 8);
        r.din.y0 = (const double*)up(r.in.y0, d * n * 8);
        r.din.params = r.pb.n_params > 0 ? (const double*)up(r.in.params, np * n * 8) : nullptr;
        r.din.rtol = (const double*)up(r.in.rtol, n * 8);
        r.din.atol = (const double*)up(r.in.atol, n * 8);
        r.din.rtol_vec = (const double*)up(r.in.rtol_vec, d * n * 8);
        r.din.atol_vec = (const double*)up(r.in.atol_vec, d * n * 8);
        r.din.dims = r.in.dims ? (const int32_t*)up(r.in.dims, n * 4) : nullptr;
        r.din.family = r.in.family ? (const int32_t*)up(r.in.family, n * 4) : nullptr;
        r.din.t_eval = m ? (const double*)up(r.in.t_eval, m * 8) : nullptr;
        r.dout.y_final = (double*)take(d * n * 8);
        r.dout.t_final = (double*)take(n * 8);
        r.dout.dense = (m && r.out.dense) ? (double*)take(m * d * n * 8) : nullptr;
        r.dout.accepted = (int64_t*)take(n * 8);
        r.dout.rejected = (int64_t*)take(n * 8);
        r.dout.fevals = (int64_t*)take(n * 8);
        r.dout.status = (int32_t*)take(n * 4);
        if (!r.resumable) {
            degpu_status st = degpu_solve_ensemble(&r.pb, &r.cfg, &r.din, &r.dout, s);
            if (st != DEGPU_OK) {
                r.result = st;
                return false;
            }
            return true;
        }
        r.done_dev = (unsigned long long*)take(16);
        cudaMemsetAsync(r.done_dev, 0, 8, s);
        EnsArgs a{};
        a.n = (int64_t)n;
        a.count = (int64_t)n;
        a.t0 = r.din.t0;
        a.tf = r.din.tf;
        a.y0 = r.din.y0;
        a.params = r.din.params;
        a.rtol = r.din.rtol;
        a.atol = r.din.atol;
        a.rtol_vec = r.din.rtol_vec;
        a.atol_vec = r.din.atol_vec;
        a.dmax = r.pb.dim;
        a.y_final = r.dout.y_final;
        a.t_final = r.dout.t_final;
        a.accepted = r.dout.accepted;
        a.rejected = r.dout.rejected;
        a.fevals = r.dout.fevals;
        a.status = r.dout.status;
        a.h0 = r.cfg.h0;
        a.h_min = r.cfg.h_min;
        a.h_max = r.cfg.h_max;
        a.max_steps = r.cfg.max_steps;
        a.safety = r.cfg.safety_factor;
        a.min_scale = r.cfg.min_scale;
        a.max_scale = r.cfg.max_scale;
        a.safety_f = (float)a.safety;
        a.min_scale_f = (float)a.min_scale;
        a.max_scale_f = (float)a.max_scale;
        a.dense_mode = r.cfg.dense_mode;
        a.n_params = r.pb.n_params;
        a.dims = r.din.dims;
        if (!r.te_sorted.empty()) {
            // the sorted output times over the caller's copy, their permutation, NaN outputs
            a.n_eval = (int32_t)m;
            a.t_eval = (const double*)r.din.t_eval;
            cudaMemcpyAsync((void*)a.t_eval, r.te_sorted.data(), m * 8, cudaMemcpyHostToDevice, s);
            a.eval_perm = (const int32_t*)up(r.te_perm.data(), m * 4);
            a.dense = r.dout.dense;
            cudaMemsetAsync(a.dense, 0xFF, m * d * n * 8, s);  // 0xFF bytes form a quiet NaN
        }
        for (auto& pt : r.parts) {
            const size_t cnt = pt.idx.empty() ? n : pt.idx.size();
            pt.args = a;
            if (!pt.idx.empty()) pt.args.index = (const int64_t*)up(pt.idx.data(), cnt * 8);
            pt.args.count = (int64_t)cnt;
            pt.park = take(cnt * pt.ops.park_bytes);
            pt.ticket = (unsigned long long*)take(16);
            pt.args.ticket = pt.ticket;
            cudaMemsetAsync(pt.park, 0, cnt * pt.ops.park_bytes, s);  // phase 0: not started
        }
        return launch_round(r);
    }

    bool launch_round(SrvRequest& r) {
        cudaStream_t s = r.stream;
        for (auto& pt : r.parts) {
            if (cudaMemsetAsync(pt.ticket, 0, 8, s) != cudaSuccess) return false;
            if (pt.ops.launch(pt.args, pt.park, cfg.round_budget, r.done_dev, 0, s) != cudaSuccess) return false;
        }
        cudaMemcpyAsync(r.done_host, r.done_dev, 8, cudaMemcpyDeviceToHost, s);
        cudaEventRecord(r.ev, s);
        return true;
    }

    void copy_out(SrvRequest& r) {
        const size_t n = (size_t)r.in.n, d = (size_t)r.pb.dim;
        const size_t m = (size_t)(r.in.n_eval > 0 ? r.in.n_eval : 0);
        cudaStream_t s = r.stream;
        auto down = [&](void* dst, const void* src, size_t bytes) {
            if (dst && src) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
        };
        down(r.out.y_final, r.dout.y_final, d * n * 8);
        down(r.out.t_final, r.dout.t_final, n * 8);
        down(r.out.dense, r.dout.dense, m * d * n * 8);
        down(r.out.accepted, r.dout.accepted, n * 8);
        down(r.out.rejected, r.dout.rejected, n * 8);
        down(r.out.fevals, r.dout.fevals, n * 8);
        down(r.out.status, r.dout.status, n * 4);
        cudaEventRecord(r.ev, s);
    }

    void finish(const std::shared_ptr<SrvRequest>& r, degpu_status st) {
        if (r->dblock) cudaFreeAsync(r->dblock, r->stream);
        cudaStreamSynchronize(r->stream);
        std::lock_guard<std::mutex> g(mu);
        r->result = st;
        r->state = 3;
        r->t_done = Clock::now();
        used -= r->bytes;
        free_streams.push_back(r->stream);
        r->stream = nullptr;
        cv.notify_all();
    }

    void loop() {
        cudaSetDevice(device);
        for (;;) {
            bool progressed = false;
            std::vector<std::shared_ptr<SrvRequest>> admit;
            {
                std::lock_guard<std::mutex> g(mu);
                while (!queue.empty() && (int)active.size() + (int)admit.size() < cfg.max_active &&
                       !free_streams.empty()) {
                    auto& r = queue.front();
                    if (used + r->bytes > cfg.memory_budget_bytes && !(active.empty() && admit.empty())) break;
                    used += r->bytes;
                    r->stream = free_streams.back();
                    free_streams.pop_back();
                    admit.push_back(r);
                    queue.pop_front();
                }
                if (stop && queue.empty() && active.empty() && admit.empty()) return;
            }
            for (auto& r : admit) {
                progressed = true;
                if (start_request(*r)) {
                    if (!r->resumable) {
                        copy_out(*r);
                        r->state = 2;
                    } else {
                        r->state = 1;
                    }
                    active.push_back(r);
                } else {
                    finish(r, r->result != DEGPU_OK ? r->result : DEGPU_CUDA_ERROR);
                }
            }
            for (size_t k = 0; k < active.size();) {
                auto r = active[k];
                cudaError_t q = cudaEventQuery(r->ev);
                if (q == cudaErrorNotReady) {
                    ++k;
                    continue;
                }
                progressed = true;
                if (q != cudaSuccess) {
                    active.erase(active.begin() + k);
                    finish(r, DEGPU_CUDA_ERROR);
                    continue;
                }
                if (r->state == 1) {
                    if (*r->done_host >= (unsigned long long)r->in.n) {
                        copy_out(*r);
                        r->state = 2;
                    } else if (!launch_round(*r)) {
                        active.erase(active.begin() + k);
                        finish(r, DEGPU_CUDA_ERROR);
                        continue;
                    }
                    ++k;
                } else {
                    active.erase(active.begin() + k);
                    finish(r, DEGPU_OK);
                }
            }
            if (!progressed) {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait_for(lk, std::chrono::microseconds(active.empty() ? 2000 : 50));
            }
        }
    }
};

}  // namespace degpu

using namespace degpu;

struct degpu_server {
    ServerImpl impl;
};

extern "C" {

degpu_status degpu_server_create(const degpu_server_cfg* cfg, degpu_server** server) {
    if (!server) return DEGPU_BAD_INPUT;
    ensure_registered();
    auto* s = new degpu_server();
    ServerImpl& I = s->impl;
    I.cfg.memory_budget_bytes = (cfg && cfg->memory_budget_bytes) ? cfg->memory_budget_bytes : (uint64_t)150 << 30;
    I.cfg.max_active = (cfg && cfg->max_active > 0) ? cfg->max_active : 64;
    I.cfg.round_budget = (cfg && cfg->round_budget > 0) ? cfg->round_budget : 512;
    cudaGetDevice(&I.device);
    for (int k = 0; k < I.cfg.max_active; ++k) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            delete s;
            return DEGPU_CUDA_ERROR;
        }
        I.free_streams.push_back(st);
    }
    I.th = std::thread([&I]() { I.loop(); });
    *server = s;
    return DEGPU_OK;
}

degpu_status degpu_server_submit(degpu_server* server, const degpu_problem* pb, const degpu_method_cfg* cfg,
                                 const degpu_batch_in* in, degpu_batch_out* out, uint64_t* request_id) {
    if (!server || !pb || !cfg || !in || !out || !request_id || in->n <= 0 || !out->y_final) return DEGPU_BAD_INPUT;
    if (!in->t0 || !in->tf || !in->y0 || !in->rtol || !in->atol || pb->dim <= 0) return DEGPU_BAD_INPUT;
    ServerImpl& I = server->impl;
    auto r = std::make_shared<SrvRequest>();
    r->pb = *pb;
    r->cfg = *cfg;
    r->in = *in;
    r->out = *out;
    r->t_submit = Clock::now();
    const bool plain = !in->family && !in->dims && pb->rhs_id < DEGPU_RHS_NVRTC_BASE;
    const bool ragged = !in->family && in->dims && pb->rhs_id == DEGPU_RHS_FPU_BETA;
    const int dense = (in->n_eval > 0 && in->t_eval && out->dense) ? 1 : 0;
    if (plain) {
        auto it = round_registry().find(VariantKey{cfg->method, pb->rhs_id, cfg->precision, dense});
        if (it != round_registry().end()) {
            r->resumable = true;
            r->parts.resize(1);
            r->parts[0].ops = it->second;
        }
        // a mixed request whose rtol values straddle the mixed-precision bound: the instances
        // below it run the FP32-pair round kernels where built, else the FP64_FAST ones
        const double bound = mixed_split(cfg);
        auto it64 = round_registry().find(VariantKey{cfg->method, pb->rhs_id, mixed_low_precision(cfg), dense});
        if (it64 == round_registry().end())
            it64 = round_registry().find(VariantKey{cfg->method, pb->rhs_id, DEGPU_FP64_FAST, dense});
        if (r->resumable && bound > 0.0) {
            if (it64 == round_registry().end()) return DEGPU_UNSUPPORTED;
            std::vector<int64_t> idx[2];
            for (int64_t i = 0; i < in->n; ++i) idx[in->rtol[i] < bound ? 1 : 0].push_back(i);
            if (idx[0].empty()) {
                r->parts[0].ops = it64->second;  // every instance below the bound
            } else if (!idx[1].empty()) {
                r->parts[0].idx = std::move(idx[0]);
                r->parts.push_back(SrvRequest::Part{});
                r->parts[1].ops = it64->second;
                r->parts[1].idx = std::move(idx[1]);
            }
        }
    } else if (ragged) {
        // FPU-beta chains: resumable group kernels, one part per (precision, layout) bucket;
        // anything the round kernels do not cover is solved in one piece instead
        std::vector<GroupRoundPart> gp;
        if (group_round_parts(pb, cfg, in->dims, in->rtol, in->n, dense, gp) == DEGPU_OK) {
            r->resumable = true;
            for (auto& g : gp) {
                SrvRequest::Part pt;
                pt.ops = RoundOps{g.ops.park_bytes, g.ops.launch};
                if (gp.size() > 1 || g.idx.size() != (size_t)in->n) pt.idx = std::move(g.idx);
                r->parts.push_back(std::move(pt));
            }
        }
    }
    if (r->resumable && dense) {
        // TEvalSolout::new's stable ascending sort (src/solout/t_eval.rs:154-171), done once
        const int32_t m = in->n_eval;
        r->te_perm.resize(m);
        for (int32_t e = 0; e < m; ++e) r->te_perm[e] = e;
        std::stable_sort(r->te_perm.begin(), r->te_perm.end(),
                         [&](int32_t x, int32_t y) { return in->t_eval[x] < in->t_eval[y]; });
        r->te_sorted.resize(m);
        for (int32_t e = 0; e < m; ++e) r->te_sorted[e] = in->t_eval[r->te_perm[e]];
    }
    r->bytes = I.footprint(*r);
    if (cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming) != cudaSuccess) return DEGPU_CUDA_ERROR;
    if (cudaMallocHost((void**)&r->done_host, 16) != cudaSuccess) return DEGPU_OOM;
    *r->done_host = 0;
    {
        std::lock_guard<std::mutex> g(I.mu);
        if (I.stop) return DEGPU_BAD_INPUT;
        r->id = I.next_id++;
        I.all[r->id] = r;
        I.queue.push_back(r);
    }
    I.cv.notify_all();
    *request_id = r->id;
    return DEGPU_OK;
}

degpu_status degpu_server_poll(degpu_server* server, uint64_t id, int32_t* done, double* latency_ms) {
    if (!server || !done) return DEGPU_BAD_INPUT;
    ServerImpl& I = server->impl;
    std::lock_guard<std::mutex> g(I.mu);
    auto it = I.all.find(id);
    if (it == I.all.end()) return DEGPU_BAD_INPUT;
    auto& r = it->second;
    *done = r->state == 3 ? 1 : 0;
    if (r->state == 3 && latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    return r->state == 3 ? r->result : DEGPU_OK;
}

degpu_status degpu_server_wait(degpu_server* server, uint64_t id, double* latency_ms) {
    if (!server) return DEGPU_BAD_INPUT;
    ServerImpl& I = server->impl;
    std::unique_lock<std::mutex> lk(I.mu);
    auto it = I.all.find(id);
    if (it == I.all.end()) return DEGPU_BAD_INPUT;
    auto r = it->second;
    I.cv.wait(lk, [&]() { return r->state == 3; });
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    return r->result;
}

degpu_status degpu_server_destroy(degpu_server* server) {
    if (!server) return DEGPU_BAD_INPUT;
    ServerImpl& I = server->impl;
    I.stop = true;
    I.cv.notify_all();
    if (I.th.joinable()) I.th.join();
    for (auto& kv : I.all) {
        if (kv.second->ev) cudaEventDestroy(kv.second->ev);
        if (kv.second->done_host) cudaFreeHost(kv.second->done_host);
    }
    for (cudaStream_t s : I.free_streams) cudaStreamDestroy(s);
    delete server;
    return DEGPU_OK;
}

}  // extern "C"
