// Batched SIMPLE cases in one CUDA graph with an SM-share autotuner (batch.hpp).
#include "batch.hpp"

#include <algorithm>

namespace sysu {

namespace {
int device_sms() {
    int dev = 0, n = 0;
    SYSU_CUDA(cudaGetDevice(&dev));
    SYSU_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    return n;
}

double elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    SYSU_CUDA(cudaEventElapsedTime(&ms, a, b));
    return ms;
}
}  // namespace

CaseBatch::CaseBatch(const std::vector<std::string> &params) {
    try {
        for (const std::string &p : params) cases.push_back(new sysu_solver{new SimpleSolver(p)});
        SYSU_CUDA(cudaStreamCreateWithFlags(&main_, cudaStreamNonBlocking));
        SYSU_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
        SYSU_CUDA(cudaEventCreate(&t0_));
        SYSU_CUDA(cudaEventCreate(&t1_));
        join_.resize(cases.size());
        for (cudaEvent_t &e : join_) SYSU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    } catch (...) {
        for (sysu_solver *s : cases) {
            delete s->impl;
            delete s;
        }
        cases.clear();
        throw;
    }
}

CaseBatch::~CaseBatch() {
    if (main_) cudaStreamSynchronize(main_);
    if (exec_) cudaGraphExecDestroy(exec_);
    for (cudaEvent_t e : join_)
        if (e) cudaEventDestroy(e);
    if (fork_) cudaEventDestroy(fork_);
    if (t0_) cudaEventDestroy(t0_);
    if (t1_) cudaEventDestroy(t1_);
    if (main_) cudaStreamDestroy(main_);
    for (sysu_solver *s : cases) {
        try {
            delete s->impl;
        } catch (...) {
        }
        delete s;
    }
}

void CaseBatch::set_caps(const std::vector<int> &caps) {
    if (caps.size() != cases.size()) throw CaseError{"one SM cap per case"};
    for (size_t k = 0; k < cases.size(); ++k) at((int)k).kw.sm_cap = std::max(0, caps[k]);
    if (exec_) {
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
    }
}

TuneResult CaseBatch::tune(const std::vector<int> &candidates) {
    std::vector<int> cand(candidates);
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    if (cand.empty() || cand[0] < 1) throw CaseError{"tune: candidate SM caps must be >= 1"};
    const int S = device_sms();
    const int nc = size();
    TuneResult r;
    std::vector<std::vector<double>> t(nc, std::vector<double>(cand.size(), 0.0));
    r.ms_full.assign(nc, 0.0);
    for (int k = 0; k < nc; ++k) {
        SimpleSolver &c = at(k);
        auto one = [&](int cap) {
            c.kw.sm_cap = cap;
            c.enqueue_iteration();  // warm (grids, caches)
            SYSU_CUDA(cudaEventRecord(t0_, c.st));
            c.enqueue_iteration();
            SYSU_CUDA(cudaEventRecord(t1_, c.st));
            SYSU_CUDA(cudaEventSynchronize(t1_));
            return elapsed_ms(t0_, t1_);
        };
        r.ms_full[k] = one(0);
        for (size_t j = 0; j < cand.size(); ++j) t[k][j] = one(std::min(cand[j], S));
        c.kw.sm_cap = 0;
        c.reset();
    }
    // greedy on the model makespan J = max(slowest case alone, SM-time / SMs):
    // start every case at the smallest cap and keep applying the single
    // one-step cap increase that lowers J most, while the caps fit the GPU
    std::vector<size_t> pick(nc, 0);
    auto model = [&](const std::vector<size_t> &pk, long *used) {
        double tmax = 0.0, area = 0.0;
        long u = 0;
        for (int k = 0; k < nc; ++k) {
            double tk = t[k][pk[k]];
            tmax = std::max(tmax, tk);
            area += tk * cand[pk[k]];
            u += cand[pk[k]];
        }
        if (used) *used = u;
        return std::max(tmax, area / S);
    };
    double J = model(pick, nullptr);
    for (;;) {
        int best = -1;
        double bestJ = J;
        for (int k = 0; k < nc; ++k) {
            if (pick[k] + 1 >= cand.size()) continue;
            std::vector<size_t> trial(pick);
            ++trial[k];
            long u = 0;
            double j = model(trial, &u);
            if (u <= S && j < bestJ - 1e-9) {
                bestJ = j;
                best = k;
            }
        }
        if (best < 0) break;
        ++pick[best];
        J = bestJ;
    }
    r.sm_cap.resize(nc);
    r.ms_alone.resize(nc);
    r.makespan_ms = J;
    for (int k = 0; k < nc; ++k) {
        r.sm_cap[k] = cand[pick[k]];
        r.ms_alone[k] = t[k][pick[k]];
    }
    // the graph issues the longest cases first
    order_.resize(nc);
    for (int k = 0; k < nc; ++k) order_[k] = k;
    std::stable_sort(order_.begin(), order_.end(), [&](int a, int b) { return r.ms_alone[a] > r.ms_alone[b]; });
    // the model ignores contention between branches: measure the real makespan of
    // the greedy caps scaled by 1/2, 1, 2, 4 and 8 and keep the fastest
    std::vector<int> best = r.sm_cap;
    double best_ms = -1.0;
    for (double fct : {1.0, 0.5, 2.0, 4.0, 8.0}) {
        std::vector<int> caps(nc);
        for (int k = 0; k < nc; ++k) {
            double want = r.sm_cap[k] * fct;
            int c = cand[0];
            for (int x : cand)
                if (x <= want + 1e-9) c = x;
            caps[k] = std::min(c, S);
        }
        set_caps(caps);
        capture();
        replay(1);
        double ms = replay(2) / 2.0;
        for (int k = 0; k < nc; ++k) at(k).reset();
        if (best_ms < 0.0 || ms < best_ms) {
            best_ms = ms;
            best = caps;
        }
    }
    r.sm_cap = best;
    r.measured_ms = best_ms;
    for (int k = 0; k < nc; ++k) {
        size_t j = 0;
        while (j + 1 < cand.size() && cand[j] < best[k]) ++j;
        r.ms_alone[k] = t[k][j];
    }
    set_caps(r.sm_cap);
    return r;
}

void CaseBatch::capture() {
    if (exec_) {
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
    }
    // every allocation and one-time set-up happens in an eager iteration
    for (int k = 0; k < size(); ++k) {
        at(k).enqueue_iteration();
        at(k).sync();
        at(k).reset();
    }
    long before = g_launches.load();
    cudaGraph_t g;
    SYSU_CUDA(cudaStreamBeginCapture(main_, cudaStreamCaptureModeThreadLocal));
    try {
        SYSU_CUDA(cudaEventRecord(fork_, main_));
        if ((int)order_.size() != size()) {
            order_.resize(size());
            for (int k = 0; k < size(); ++k) order_[k] = k;
        }
        for (int k : order_) {
            SimpleSolver &c = at(k);
            SYSU_CUDA(cudaStreamWaitEvent(c.st, fork_, 0));
            c.enqueue_iteration();
            SYSU_CUDA(cudaEventRecord(join_[k], c.st));
            SYSU_CUDA(cudaStreamWaitEvent(main_, join_[k], 0));
        }
    } catch (...) {
        cudaGraph_t junk;
        cudaStreamEndCapture(main_, &junk);
        if (junk) cudaGraphDestroy(junk);
        throw;
    }
    SYSU_CUDA(cudaStreamEndCapture(main_, &g));
    graph_launches_ = g_launches.load() - before;
    g_launches -= graph_launches_;
    cudaError_t e = cudaGraphInstantiate(&exec_, g, 0);
    cudaGraphDestroy(g);
    SYSU_CUDA(e);
}

double CaseBatch::replay(int n) {
    if (!exec_) throw CaseError{"batch: capture() first"};
    SYSU_CUDA(cudaEventRecord(t0_, main_));
    for (int i = 0; i < n; ++i) {
        SYSU_CUDA(cudaGraphLaunch(exec_, main_));
        g_launches += graph_launches_;
    }
    SYSU_CUDA(cudaEventRecord(t1_, main_));
    SYSU_CUDA(cudaEventSynchronize(t1_));
    for (int k = 0; k < size(); ++k) at(k).iter_done += n;
    return elapsed_ms(t0_, t1_);
}

std::string CaseBatch::check() {
    for (int k = 0; k < size(); ++k) {
        std::string m = at(k).check_iteration();
        if (!m.empty()) return "case " + std::to_string(k) + ": " + m;
    }
    return "";
}

double CaseBatch::run_sequential(int n) {
    SYSU_CUDA(cudaEventRecord(t0_, main_));
    for (int k = 0; k < size(); ++k) {
        SimpleSolver &c = at(k);
        SYSU_CUDA(cudaStreamWaitEvent(c.st, t0_, 0));
        for (int i = 0; i < n; ++i) {
            c.enqueue_iteration();
            ++c.iter_done;
        }
        SYSU_CUDA(cudaEventRecord(join_[k], c.st));
        SYSU_CUDA(cudaStreamWaitEvent(main_, join_[k], 0));
        // one case at a time: the next case starts when this one is done
        SYSU_CUDA(cudaEventSynchronize(join_[k]));
    }
    SYSU_CUDA(cudaEventRecord(t1_, main_));
    SYSU_CUDA(cudaEventSynchronize(t1_));
    return elapsed_ms(t0_, t1_);
}

}  // namespace sysu
