// Many independent SIMPLE cases advanced together: one CUDA graph holds one
// outer iteration of every case (each case's kernels on its own branch, so the
// cases run concurrently), and an autotuner sizes each case's persistent Krylov
// grids (SMs per case, i.e. rows per warp) so that the cases share the GPU.
#pragma once

#include <string>
#include <vector>

#include "handles.hpp"

namespace sysu {

struct TuneResult {
    std::vector<int> sm_cap;        // chosen SMs per case
    std::vector<double> ms_alone;   // one outer iteration at that cap, case alone
    std::vector<double> ms_full;    // one outer iteration with no cap, case alone
    double makespan_ms = 0.0;       // the model's makespan: max(slowest case, SM-time / SMs)
    double measured_ms = 0.0;       // graph replay time of the chosen caps
};

class CaseBatch {
  public:
    explicit CaseBatch(const std::vector<std::string> &params);
    ~CaseBatch();
    CaseBatch(const CaseBatch &) = delete;
    CaseBatch &operator=(const CaseBatch &) = delete;

    int size() const { return (int)cases.size(); }
    sysu_solver *handle(int k) { return cases[k]; }
    SimpleSolver &at(int k) { return *cases[k]->impl; }

    // Time one outer iteration of every case alone for each candidate SM cap,
    // then choose caps greedily against the makespan model max(slowest case,
    // SM-time / SMs) while the caps fit the GPU; the graph issues the longest
    // cases first.  The model's caps scaled by 1/2, 1, 2, 4 and 8 are then replayed
    // and the fastest kept.  The cases are reset to their initial state afterwards.
    TuneResult tune(const std::vector<int> &candidates);
    void set_caps(const std::vector<int> &caps);
    // One eager iteration per case (allocates every buffer), a reset, then the
    // capture of one outer iteration of all cases into the graph.
    void capture();
    // n replays of the graph (n outer iterations of every case); device ms.
    double replay(int n);
    // check_iteration of every case ("" or the first failure, prefixed by the case).
    std::string check();
    // each case alone, one after the other, n eager iterations; device ms
    double run_sequential(int n);

  private:
    std::vector<sysu_solver *> cases;
    cudaStream_t main_ = nullptr;
    cudaEvent_t fork_ = nullptr, t0_ = nullptr, t1_ = nullptr;
    std::vector<cudaEvent_t> join_;
    std::vector<int> order_;  // capture order of the cases (longest first after tune)
    cudaGraphExec_t exec_ = nullptr;
    long graph_launches_ = 0;
};

}  // namespace sysu
