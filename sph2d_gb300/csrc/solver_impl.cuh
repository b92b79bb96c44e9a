// solver_impl.cuh — the state behind an rrsph_solver handle (private to the library).
#pragma once

#include <vector>

#include "kernels.cuh"

namespace rrsph_impl {

constexpr int kPhases = 6;
inline const char* const kPhaseNames[kPhases] = {"keys", "sort", "reorder", "density", "forces", "whole"};
constexpr uint32_t kFlagNeverEnding = RRSPH_FLAG_NEVER_ENDING;
// Default skins of the candidate lists, in units of hsml. In 2D a wider skin
// rebuilds less often for a few more candidates per particle: on the 409k
// flume 0.5 h gave 0.1235 ms per step over 200 steps (8 rebuilds) against
// 0.1280 ms at 0.3 h (15 rebuilds), and 0.138 against 0.160 ms over steps
// 6-25 (3 against 6 rebuilds); 0.3 h in 3D, where the candidate count grows
// with the cube of the radius.
constexpr double kDefaultSkin2 = 0.5;
constexpr double kDefaultSkin3 = 0.3;
// Steps per graph launch when a call asks for at least that many (even: a run
// ends on the parity it started on); fewer run one single-step graph each.
constexpr int kRunSteps = 10;

struct AdjointRun;  // a forward run recorded for the reverse sweep (adjoint.cu)

}  // namespace rrsph_impl

using rrsph_impl::kPhases;
using rrsph_impl::kPhaseNames;
using rrsph_impl::kFlagNeverEnding;
using rrsph_impl::kDefaultSkin2;
using rrsph_impl::kDefaultSkin3;
using rrsph_impl::kRunSteps;

struct rrsph_solver {
    rrsph_params params{};
    rrsph::DevParams P{};
    int precision = RRSPH_PRECISION_FP64;
    int dim = 2;
    int device = 0;
    cudaStream_t stream = nullptr;
    rrsph::State S{};
    rrsph::Sorted G{};
    rrsph::StepScalars* scal = nullptr;  // [2] on the device
    uint32_t* flags = nullptr;
    rrsph::StepScalars* h_scal = nullptr;  // pinned
    uint32_t* h_flags = nullptr;           // pinned
    rrsph::HostReport* h_report = nullptr;  // mapped pinned mailbox of k_report
    rrsph::HostReport* d_report = nullptr;  // its device address
    double* diag = nullptr;                 // rrsph_diagnostics_get: block partials, then the sums
    double* staging = nullptr;
    size_t staging_words = 0;
    std::vector<void*> allocations;
    int sort_bits = 0;
    bool graphs = true;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};      // one step, starting at parity 0 / 1
    cudaGraphExec_t graph_run[2] = {nullptr, nullptr};  // kRunSteps steps, starting at parity 0 / 1
    cudaGraphExec_t graph_mark[2] = {nullptr, nullptr}; // one step recording ev_density after its density pass
    unsigned long long launches = 0;
    unsigned long long launches_in_graph[2] = {0, 0};
    unsigned long long launches_in_run[2] = {0, 0};
    unsigned long long launches_in_mark[2] = {0, 0};
    // rrsph_step_host: the copy stream that brings back what the last density
    // pass finished while the force gather runs, and its events
    cudaStream_t dl_stream = nullptr;
    cudaEvent_t ev_density = nullptr;  // recorded (external) after the marked step's density pass
    cudaEvent_t ev_dl = nullptr;       // the copy stream's work done
    bool mark_density = false;         // capturing: record ev_density after the density launch
    uint64_t step_index = 0;
    bool keys_ready = false;  // the next step's predict + keys were computed by the last whole step
    bool timing = false;
    cudaEvent_t ev[kPhases + 1] = {};
    double phase_ms[kPhases] = {};
    uint64_t timed_steps = 0;
    rrsph_impl::AdjointRun* adj = nullptr;
    int gather_threads[2] = {rrsph::kGatherThreads, rrsph::kGatherThreads};  // density, forces block sizes
    // neighbour reuse of the FP32-mixed step
    bool verlet = false;
    double verlet_skin = kDefaultSkin3;        // skin, in units of hsml (set at creation by dimension)
    cudaStream_t aux = nullptr;                // captures the rebuild / reuse bodies of a step graph
    unsigned long long* vl_builds = nullptr;   // device: list builds since creation
    uint32_t* h_vl = nullptr;                  // pinned: the rebuild flag, read with direct launches
    cudaGraph_t vl_body = nullptr;  // rebuild body of the graph being captured
    bool vl_pending = false;
    // neighbour reuse: the two P4 / V4 (/ VD4) buffers (a step reads [parity], its key
    // pass writes the next step's into [parity ^ 1])
    float4* p4buf[2] = {nullptr, nullptr};
    float4* v4buf[2] = {nullptr, nullptr};
    float4* vd4buf[2] = {nullptr, nullptr};  // continuity density
    unsigned long long vl_extra_launches = 0;  // launches a rebuild adds to a reuse step
    bool nlist_valid = false;  // nlist / ncount hold the last step's neighbours on the current grid
};

namespace rrsph_impl {
// Frees the recorded adjoint run of s, if any (adjoint.cu).
void adjoint_release(rrsph_solver* s);
// The status (and error message) the device flags f mean for s (solver.cu).
int flags_status(const rrsph_solver* s, uint32_t f);
}  // namespace rrsph_impl


namespace rrsph_impl {
// Every captured step graph (the caller synchronises the stream first).
inline void destroy_step_graphs(rrsph_solver* s) {
    for (cudaGraphExec_t* set : {s->graph, s->graph_run, s->graph_mark}) {
        for (int i = 0; i < 2; i++) {
            if (set[i]) cudaGraphExecDestroy(set[i]);
            set[i] = nullptr;
        }
    }
}
}  // namespace rrsph_impl
