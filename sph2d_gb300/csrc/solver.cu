// solver.cu — the C ABI of the GPU step: solver handles, upload/download,
// the captured step graphs and the loop-piece entry points.
//
// One step is the loop body of time_integration
// (sources/RRSPH_OMP/src/TimeIntegration.cpp:60-100):
//   keys      predict_half_step + cell keys      (PredictHalfStep.cpp:4-23, GridFind.cpp:55-75)
//   sort      stable radix sort by (cell, id)    (GridFind.cpp:53-87)
//   reorder   cell-order copies + cell table     (GridFind.cpp:77-87)
//   density   density_sum | density_con          (Density.h:25-114)
//   forces    update_acceleration                (UpdateAcceleration.cpp:33-125)
//   whole     piston + whole_step + bounds check (WaveMaker.cpp:34-82, WholeStep.cpp:19-62)
// The sequence is captured once per step parity into a CUDA graph and replayed;
// the scalars that change between steps (time, dt, step counter) live on the
// device, double-buffered by parity, and are advanced by the whole-step kernel.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../host/error.hpp"
#include "kernels.cuh"
#include "sort.cuh"

using rrsph::set_error;

#include "solver_impl.cuh"

namespace {

#define RRSPH_CUDA_TRY(call)                                                                       \
    do {                                                                                           \
        cudaError_t err_ = (call);                                                                 \
        if (err_ != cudaSuccess)                                                                   \
            return set_error(err_ == cudaErrorMemoryAllocation ? RRSPH_ERR_OUT_OF_MEMORY : RRSPH_ERR_CUDA, \
                             std::string(#call) + ": " + cudaGetErrorString(err_));                \
    } while (0)

template <typename T>
int dev_alloc(rrsph_solver* s, T** ptr, size_t count) {
    *ptr = nullptr;
    if (count == 0) return RRSPH_OK;
    void* p = nullptr;
    RRSPH_CUDA_TRY(cudaMalloc(&p, count * sizeof(T)));
    s->allocations.push_back(p);
    *ptr = static_cast<T*>(p);
    return RRSPH_OK;
}

// Host copies of the smoothing-kernel factors and W (SmoothingKernel.h).
double host_factor(const rrsph_params& p, int skf) {
    const double h = p.hsml, pi = p.pi;
    const bool d3 = p.dim == 3;
    switch (skf) {
    case 2: return d3 ? 1 / (pi * std::sqrt(pi) * h * h * h) : 1 / (pi * (h * h));
    case 3: return d3 ? 21 / (16 * pi * (h * h * h)) : 7 / (4 * pi * (h * h));
    case 4: return d3 ? 15 / (pi * ((4 * h) * (4 * h) * (4 * h))) : 5 / (16 * pi * (h * h));
    default: return d3 ? 3.0 / (2.0 * pi * (h * h * h)) : 15.0 / (7.0 * pi * (h * h));
    }
}
double host_w(const rrsph_params& p, double dist, int skf) {
    const double q = dist / p.hsml, f = host_factor(p, skf);
    switch (skf) {
    case 2: return f * std::exp(-q * q);
    case 3: { if (q <= 2) { const double t = 1 - 0.5 * q; return f * t * t * t * t * (2 * q + 1); } return 0; }
    case 4: { if (q <= 2) { const double t = 2 - q; return f * t * t * t; } return 0; }
    default:
        if (q <= 1) return f * (2.0 / 3.0 - q * q + q * q * q * 0.5);
        if (q <= 2) { const double t = 2.0 - q; return f * (1.0 / 6.0 * (t * t * t)); }
        return 0;
    }
}

int fill_dev_params(const rrsph_params& p, rrsph::DevParams& P) {
    std::memset(&P, 0, sizeof(P));
    P.dim = (int)p.dim;
    P.n = (uint32_t)p.ntotal;
    P.nfluid = (uint32_t)p.nfluid;
    if (p.max_cells == 0 || p.max_cells > (1ull << 32))
        return set_error(RRSPH_ERR_UNSUPPORTED, "max_cells out of range; derive the params first");
    P.max_cells = (uint32_t)std::min<uint64_t>(p.max_cells, 0xFFFFFFFFull);
    P.max_nb = p.max_neighbours;
    P.type_non_existent = p.type_non_existent;
    P.xmin = p.x_mingeom; P.ymin = p.y_mingeom; P.zmin = p.z_mingeom;
    P.oxmin = rrsph::dorder(p.x_mingeom); P.oymin = rrsph::dorder(p.y_mingeom); P.ozmin = rrsph::dorder(p.z_mingeom);
    P.oxmax = rrsph::dorder(p.x_maxgeom); P.oymax = rrsph::dorder(p.y_maxgeom); P.ozmax = rrsph::dorder(p.z_maxgeom);
    P.xmax = p.x_maxgeom; P.ymax = p.y_maxgeom; P.zmax = p.z_maxgeom;
    P.cell = p.cell_scale_k * p.hsml;
    P.inv_cell = 1.0 / P.cell;
    P.cut2 = P.cell * P.cell;
    P.h = p.hsml;
    P.inv_h = 1.0 / p.hsml;
    P.mass = p.mass;
    P.g = p.g;
    P.rho0 = p.rho0;
    const double c_sqr = p.eos_sound_vel_method == 0 ? 200 * p.g * p.depth * p.eos_sound_vel_coef : p.eos_sound_vel;
    P.c_eos = std::sqrt(c_sqr);
    P.B = c_sqr * p.rho0 / 7;
    P.c_av = p.eos_sound_vel;
    P.etq_h2 = (p.hsml * (double)0.1f) * (p.hsml * (double)0.1f);
    for (int s = 1; s <= 4; s++) P.kf[s] = host_factor(p, s);
    P.kf[0] = P.kf[1];
    auto skf = [](uint32_t v) { return (v >= 1 && v <= 4) ? (int)v : 1; };
    P.density_skf = skf(p.density_skf);
    P.intf_skf = skf(p.intf_skf);
    P.av_skf = skf(p.artificial_viscosity_skf);
    P.avel_skf = skf(p.average_velocity_skf);
    P.ap_skf = skf(p.artificial_pressure_skf);
    P.w0_density = host_w(p, 0, P.density_skf);
    P.density_treatment = (int)p.density_treatment;
    P.delta_sph_dhc = p.density_delta_sph_coef * p.hsml * P.c_eos;
    P.intf_form = p.intf_sph_approximation == 1 ? 1 : 2;
    P.art_pressure = p.artificial_pressure ? 1 : 0;
    P.ap_index = p.artificial_pressure_index;
    P.ap_coef = p.artificial_pressure_coef;
    P.ap_wdelta = host_w(p, p.delta, P.ap_skf);
    P.art_visc = p.artificial_viscosity ? 1 : 0;
    P.av_alpha = p.artificial_shear_visc;
    P.av_beta = p.artificial_bulk_visc;
    P.avg_vel = p.average_velocity ? 1 : 0;
    P.avg_vel_coef = p.average_velocity_coef;
    P.repulsive = p.boundary_treatment == 1;
    P.lj_rr0 = 2 * p.hsml;
    P.lj_D = 5 * p.g * p.depth;
    P.consistency_check = p.consistency_check ? 1 : 0;
    P.consistency_treatment = (int)p.consistency_treatment;
    P.nwm = (int)p.nwm;
    P.nwm_start = (uint32_t)std::min<uint64_t>(p.nwm_particles_start, 0xFFFFFFFFull);
    P.nwm_end = (uint32_t)std::min<uint64_t>(p.nwm_particles_end, 0xFFFFFFFFull);
    P.nwm_valid = !(p.nwm_particles_start < p.nfluid || p.nwm_particles_end < p.nfluid ||
                    p.nwm_particles_end < p.nwm_particles_start || p.nwm_particles_end > p.ntotal);
    P.nwm_time_start = p.nwm_time_start;
    P.nwm_phase = p.nwm_phase;
    P.nwm_freq = p.nwm_freq;
    P.nwm_H = p.nwm_wave_magnitude;
    P.nwm_k = p.nwm_wave_number;
    P.depth = p.depth;
    P.dt_method = (int)p.dt_correction_method;
    P.dt_reduce = p.dt_dynamic_reduce ? 1 : 0;
    P.cfl = p.CFL_coef;
    P.never_ending_dt = (p.hsml / P.c_eos) * 1.E-6;
    P.all_cubic = P.density_skf == 1 && P.intf_skf == 1 && P.av_skf == 1 && P.avel_skf == 1 && P.ap_skf == 1;
    rrsph::MixedF& M = P.mf;
    M.cell = (float)P.cell;
    M.h = (float)P.h;
    M.inv_h = (float)P.inv_h;
    M.mass = (float)P.mass;
    M.rho0 = (float)P.rho0;
    M.cut2_lo = (float)(P.cut2 * (1.0 - 1e-5));
    M.cut2_hi = (float)(P.cut2 * (1.0 + 1e-5));
    for (int k = 0; k < 5; k++) M.kf[k] = (float)P.kf[k];
    M.w0_density = (float)(P.mass * P.w0_density);
    {
        const double d = P.rho0 - P.mass * P.w0_density;
        M.rho0_minus_w0_hi = (float)d;
        M.rho0_minus_w0_lo = (float)(d - (double)M.rho0_minus_w0_hi);
    }
    M.B = (float)P.B;
    M.inv_rho0 = (float)(1.0 / P.rho0);
    M.lj_rr0 = (float)P.lj_rr0;
    M.lj_D = (float)P.lj_D;
    M.etq_h2 = (float)P.etq_h2;
    M.av_alpha_c = (float)(P.av_alpha * P.c_av);
    M.av_beta = (float)P.av_beta;
    M.ap_coef = (float)P.ap_coef;
    M.ap_index = (float)P.ap_index;
    M.ap_inv_wdelta = (float)(1.0 / P.ap_wdelta);
    M.avel_coef2 = (float)(2.0 * P.avg_vel_coef);
    M.dhc = (float)P.delta_sph_dhc;
    return RRSPH_OK;
}

int key_bits(uint64_t max_cells) {
    int b = 0;
    while ((1ull << b) < max_cells) b++;
    return b < 1 ? 1 : b;
}

void drop_graphs(rrsph_solver* s) {
    cudaStreamSynchronize(s->stream);
    rrsph_impl::destroy_step_graphs(s);
}

// Candidate-list cutoff (cell + skin, widened a little: a list may hold more
// than the pairs within it, never fewer), (skin / 2)^2 slightly narrowed, the
// edge band that looks two cells away, and the launches a rebuild adds.
void set_verlet_params(rrsph_solver* s) {
    const double skin = s->verlet_skin * s->params.hsml;
    const double c = s->P.cell + skin;
    s->P.vl_cut2 = (float)(c * c * (1.0 + 1e-4));
    s->P.vl_half_skin2 = (float)(0.25 * skin * skin * (1.0 - 1e-4));
    s->P.vl_skin_edge = (float)(skin * 1.01);
    // reset + sort (3 per 8-bit pass) + reorder + build (a step that reuses the
    // lists launches nothing for them: the key pass wrote its cell-order copies)
    s->vl_extra_launches = 3ull + 3ull * (unsigned long long)((s->sort_bits + 7) / 8);
}

int check_handle(rrsph_solver* s, const char* fn) {
    if (!s) return set_error(RRSPH_ERR_INVALID_ARGUMENT, std::string(fn) + ": null solver");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return set_error(RRSPH_ERR_CUDA, std::string(fn) + ": cudaSetDevice: " + cudaGetErrorString(e));
    return RRSPH_OK;
}

// The stable sort of the key pass's (cell, id) pairs into (keys_a, ids_a),
// whatever the number of passes: the grid stays there after the step, while
// the whole step's key pass rewrites (keys_in, ids_in) for the next one.
void sort_grid(rrsph_solver* s, cudaStream_t st) {
    rrsph::radix_sort_pairs_into(s->G.keys_in, s->G.ids_in, s->G.keys_a, s->G.ids_a, s->G.keys_b, s->G.ids_b,
                                 s->G.sort_scratch, s->P.n, s->sort_bits, st, &s->launches);
    s->G.key = s->G.keys_a;
    s->G.id = s->G.ids_a;
}

// Builds the grid on the current state: keys (optionally with the predictor),
// sort, reorder with the given force-side sources.
template <int DIM>
void enqueue_grid(rrsph_solver* s, int predict, rrsph::StepScalars* scal, rrsph::GatherSrc fsrc) {
    rrsph::launch_keys<DIM>(s->P, s->S, s->G, scal, predict, s->flags, s->stream);
    sort_grid(s, s->stream);
    rrsph::launch_reorder<DIM>(s->P, s->S, s->G, fsrc, s->precision == RRSPH_PRECISION_MIXED, s->stream);
    s->launches += 2;
}

template <int DIM>
void enqueue_density(rrsph_solver* s, rrsph::StepScalars* scal) {
    const int th = s->gather_threads[0];
    if (s->precision == RRSPH_PRECISION_MIXED) rrsph::launch_density_mixed<DIM>(s->P, s->S, s->G, scal, s->flags, s->stream, th);
    else rrsph::launch_density_fp64<DIM>(s->P, s->S, s->G, scal, s->flags, s->stream, th);
    s->launches++;
}

template <int DIM>
void enqueue_forces(rrsph_solver* s, uint32_t terms, rrsph::StepScalars* scal, int write_mu, int use_masks = 0) {
    const int th = s->gather_threads[1];
    if (s->precision == RRSPH_PRECISION_MIXED)
        rrsph::launch_forces_mixed<DIM>(s->P, s->S, s->G, terms, scal, s->flags, write_mu, use_masks, s->stream, th);
    else rrsph::launch_forces_fp64<DIM>(s->P, s->S, s->G, terms, scal, s->flags, write_mu, s->stream, th, use_masks);
    s->launches++;
}

// One loop step on parity `par`; events[i] (if non-null) are recorded between
// phases. with_keys runs the predict + key pass first; otherwise the previous
// step's whole-step kernel has done it. The whole-step kernel always prepares
// the next step's predict + keys.
// Neighbour reuse: the grid + list rebuild on stream st (a step that reuses
// the lists has its cell-order copies from the key pass). The rebuilt grid
// stays in (keys_a, ids_a) while the lists are reused: the key pass of every
// step rewrites keys_in.
// Neighbour reuse: the step of parity `read` reads P4 / V4 [read]; the key
// pass writes its copies into [write].
void set_verlet_copies(rrsph_solver* s, int read, int write) {
    s->G.P4 = s->p4buf[read];
    s->G.V4 = s->v4buf[read];
    s->G.P4n = s->p4buf[write];
    s->G.V4n = s->v4buf[write];
    if (s->G.VD4n) {
        s->G.VD4 = s->vd4buf[read];
        s->G.VD4n = s->vd4buf[write];
    }
}

// Whether the cell-tile density pass runs (compile-time variant: 2D summation
// density with the cubic kernel), which reads the last build's cell table.
bool tiles_active(const rrsph_solver* s) {
    return RRSPH_DENSITY_CELL_TILES && s->verlet && s->dim == 2 && s->P.density_treatment == 0 && s->P.all_cubic;
}
// The key pass keeps or clears cell-table entries as the density pass needs;
// on a change the table is cleared wholesale (no entry of another grid stays).
int set_keep_cells(rrsph_solver* s) {
    const int keep = tiles_active(s) ? 1 : 0;
    if (keep != s->P.keep_cells) {
        s->P.keep_cells = keep;
        RRSPH_CUDA_TRY(cudaMemsetAsync(s->G.cell_start, 0xFF, (size_t)s->P.max_cells * sizeof(uint32_t), s->stream));
    }
    return RRSPH_OK;
}

void enqueue_verlet_rebuild(rrsph_solver* s, cudaStream_t st) {
    rrsph::launch_verlet_reset(s->S.vl_rebuild, s->S.vl_gone, s->vl_builds, st);
    if (s->P.keep_cells) {  // the previous build's table stayed in place: clear it for the reorder
        rrsph::launch_clear_cells(s->G.cell_start, s->P.max_cells, st);
        s->launches++;
    }
    rrsph::radix_sort_pairs_into(s->G.keys_in, s->G.ids_in, s->G.keys_a, s->G.ids_a, s->G.keys_b, s->G.ids_b,
                                 s->G.sort_scratch, s->P.n, s->sort_bits, st, &s->launches);
    s->G.key = s->G.keys_a;
    s->G.id = s->G.ids_a;
    const bool cont = s->P.density_treatment != 0;
    rrsph::GatherSrc fsrc{s->S.vpx, s->S.vpy, s->S.vpz, cont ? s->S.rho_pred : s->S.rho, nullptr, 1};
    if (s->dim == 3) {
        rrsph::launch_reorder<3>(s->P, s->S, s->G, fsrc, 1, st);
        rrsph::launch_verlet_build<3>(s->P, s->S, s->G, st);
    } else {
        rrsph::launch_reorder<2>(s->P, s->S, s->G, fsrc, 1, st);
        rrsph::launch_verlet_build<2>(s->P, s->S, s->G, st);
    }
    s->launches += 3;
}

// One step of the mixed loop with neighbour reuse. In a captured graph the
// rebuild is a conditional node that a kernel sets from the flag the last key
// pass raised; with direct launches the host reads the flag.
int enqueue_step_verlet(rrsph_solver* s, int par, cudaEvent_t* events, bool with_keys) {
    rrsph::StepScalars* cur = s->scal + par;
    rrsph::StepScalars* nxt = s->scal + (par ^ 1);
    cudaStream_t st = s->stream;
    s->G.key = s->G.keys_a;  // the grid of the last rebuild
    s->G.id = s->G.ids_a;
    if (events) cudaEventRecord(events[0], st);
    if (with_keys) set_verlet_copies(s, par, par);  // this step's copies from its own key pass
    if (with_keys) {
        if (s->dim == 3) rrsph::launch_keys<3>(s->P, s->S, s->G, cur, 1, s->flags, st);
        else rrsph::launch_keys<2>(s->P, s->S, s->G, cur, 1, s->flags, st);
        s->launches++;
    }
    set_verlet_copies(s, par, par ^ 1);
    if (events) cudaEventRecord(events[1], st);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    RRSPH_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusActive) {
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        RRSPH_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
        cudaGraphConditionalHandle h;
        RRSPH_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
        rrsph::launch_verlet_decide(h, s->S.vl_rebuild, st);
        s->launches++;
        RRSPH_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 1;
        cudaGraphNode_t cnode;
        RRSPH_CUDA_TRY(cudaGraphAddNode(&cnode, g, deps, nullptr, nd, &np));
        s->vl_body = np.conditional.phGraph_out[0];
        s->vl_pending = true;
        RRSPH_CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    } else {
        RRSPH_CUDA_TRY(cudaMemcpyAsync(s->h_vl, s->S.vl_rebuild, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
        if (*s->h_vl) {
            const unsigned long long before = s->launches;
            enqueue_verlet_rebuild(s, st);
            s->launches = before;  // a rebuild's launches are counted from vl_builds
        }
    }
    if (events) {
        cudaEventRecord(events[2], st);
        cudaEventRecord(events[3], st);
    }
    const bool d3 = s->dim == 3;
    if (d3) rrsph::launch_density_verlet<3>(s->P, s->S, s->G, cur, s->flags, st, s->gather_threads[0]);
    else rrsph::launch_density_verlet<2>(s->P, s->S, s->G, cur, s->flags, st, s->gather_threads[0]);
    if (s->mark_density) RRSPH_CUDA_TRY(cudaEventRecordWithFlags(s->ev_density, st, cudaEventRecordExternal));
    if (events) cudaEventRecord(events[4], st);
    // the whole step runs inside the force gather unless dt waits for the step's
    // maxima or a particle may have more neighbours than a list holds
    const bool fuse = !(s->P.dt_method == 2 && s->P.dt_reduce) &&
                      s->P.max_nb <= (uint32_t)rrsph::verlet_cap(s->dim) + 1u;
    if (d3) rrsph::launch_forces_verlet<3>(s->P, s->S, s->G, cur, nxt, s->flags, st, s->gather_threads[1], fuse ? 1 : 0);
    else rrsph::launch_forces_verlet<2>(s->P, s->S, s->G, cur, nxt, s->flags, st, s->gather_threads[1], fuse ? 1 : 0);
    if (events) cudaEventRecord(events[5], st);
    if (!fuse) {
        if (d3) rrsph::launch_whole_step<3>(s->P, s->S, s->G, cur, nxt, s->flags, 1, st);
        else rrsph::launch_whole_step<2>(s->P, s->S, s->G, cur, nxt, s->flags, 1, st);
    }
    if (events) cudaEventRecord(events[6], st);
    s->launches += fuse ? 2 : 3;
    return RRSPH_OK;
}

// Fills the rebuild body of the conditional node of a just-captured step (its
// launches are counted from vl_builds).
int capture_verlet_body(rrsph_solver* s) {
    s->vl_pending = false;
    const unsigned long long before = s->launches;
    RRSPH_CUDA_TRY(cudaStreamBeginCaptureToGraph(s->aux, s->vl_body, nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal));
    enqueue_verlet_rebuild(s, s->aux);
    cudaGraph_t out = nullptr;
    RRSPH_CUDA_TRY(cudaStreamEndCapture(s->aux, &out));
    s->launches = before;
    return RRSPH_OK;
}

template <int DIM>
void enqueue_step(rrsph_solver* s, int par, cudaEvent_t* events, bool with_keys) {
    rrsph::StepScalars* cur = s->scal + par;
    rrsph::StepScalars* nxt = s->scal + (par ^ 1);
    const bool cont = s->P.density_treatment != 0;
    rrsph::GatherSrc fsrc{s->S.vpx, s->S.vpy, s->S.vpz, cont ? s->S.rho_pred : s->S.rho, nullptr, 1};
    if (events) cudaEventRecord(events[0], s->stream);
    if (with_keys) {
        rrsph::launch_keys<DIM>(s->P, s->S, s->G, cur, 1, s->flags, s->stream);
        s->launches++;
    }
    if (events) cudaEventRecord(events[1], s->stream);
    sort_grid(s, s->stream);
    if (events) cudaEventRecord(events[2], s->stream);
    rrsph::launch_reorder<DIM>(s->P, s->S, s->G, fsrc, s->precision == RRSPH_PRECISION_MIXED, s->stream);
    if (events) cudaEventRecord(events[3], s->stream);
    enqueue_density<DIM>(s, cur);
    if (s->mark_density) cudaEventRecordWithFlags(s->ev_density, s->stream, cudaEventRecordExternal);
    if (events) cudaEventRecord(events[4], s->stream);
    enqueue_forces<DIM>(s, RRSPH_TERM_ALL, cur, 0, 1);
    if (events) cudaEventRecord(events[5], s->stream);
    rrsph::launch_whole_step<DIM>(s->P, s->S, s->G, cur, nxt, s->flags, 1, s->stream);
    if (events) cudaEventRecord(events[6], s->stream);
    s->launches += 2;
}

int enqueue_step_dim(rrsph_solver* s, int par, cudaEvent_t* events, bool with_keys) {
    if (s->verlet) return enqueue_step_verlet(s, par, events, with_keys);
    if (s->dim == 3) enqueue_step<3>(s, par, events, with_keys);
    else enqueue_step<2>(s, par, events, with_keys);
    return RRSPH_OK;
}

void enqueue_keys_dim(rrsph_solver* s, int par) {
    if (s->verlet) set_verlet_copies(s, par, par);
    if (s->dim == 3) rrsph::launch_keys<3>(s->P, s->S, s->G, s->scal + par, 1, s->flags, s->stream);
    else rrsph::launch_keys<2>(s->P, s->S, s->G, s->scal + par, 1, s->flags, s->stream);
    s->launches++;
}

int ensure_staging(rrsph_solver* s, size_t words) {
    if (s->staging_words >= words) return RRSPH_OK;
    if (s->staging) {
        cudaFree(s->staging);
        for (auto& a : s->allocations)
            if (a == s->staging) a = nullptr;
        s->staging = nullptr;
    }
    int rc = dev_alloc(s, &s->staging, words);
    if (rc) return rc;
    s->staging_words = words;
    return RRSPH_OK;
}

int flags_to_status(const rrsph_solver* s, uint32_t f) {
    // the per-step bounds check of update_step comes before the next step's grid
    // find, whose key pass the whole-step kernel already ran
    if ((f & RRSPH_FLAG_OUTSIDE_GEOMETRY) && s->params.consistency_check && s->params.consistency_treatment == 1)
        return set_error(RRSPH_ERR_OUTSIDE_GEOMETRY, "Encounter particle outside boundaries");
    if (f & RRSPH_FLAG_OUT_OF_DOMAIN) return set_error(RRSPH_ERR_OUT_OF_DOMAIN, "cell_idx was >= params.max_cells");
    if (f & RRSPH_FLAG_NEIGHBOUR_OVERFLOW) return set_error(RRSPH_ERR_NEIGHBOUR_OVERFLOW, "making neighbours grid: error occured");
    if (f & kFlagNeverEnding) return set_error(RRSPH_ERR_NEVER_ENDING, "never ending simulation");
    if ((f & RRSPH_FLAG_OUTSIDE_GEOMETRY) && s->params.consistency_check && s->params.consistency_treatment == 1)
        return set_error(RRSPH_ERR_OUTSIDE_GEOMETRY, "Encounter particle outside boundaries");
    return RRSPH_OK;
}

}  // namespace

int rrsph_impl::flags_status(const rrsph_solver* s, uint32_t f) { return flags_to_status(s, f); }

// ============================================================== C ABI ======

extern "C" int rrsph_create(const rrsph_params* p, int precision, rrsph_solver** out) {
    if (!p || !out) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_create: null argument");
    *out = nullptr;
    if (p->struct_size != sizeof(rrsph_params))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_create: params not initialised by rrsph_params_defaults");
    if (p->dim != 2 && p->dim != 3) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_create: dim must be 2 or 3");
    if (p->ntotal == 0 || p->ntotal >= (1ull << 31)) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_create: bad ntotal");
    if (p->hsml <= 0 || p->mass <= 0) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_create: derive the params first");
    if (precision != RRSPH_PRECISION_FP64 && precision != RRSPH_PRECISION_MIXED)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_create: unknown precision");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(RRSPH_ERR_NO_DEVICE, "rrsph_create: no CUDA device");
    }
    rrsph_solver* s = new rrsph_solver();
    s->params = *p;
    s->precision = precision;
    s->dim = (int)p->dim;
    cudaGetDevice(&s->device);
    int rc = fill_dev_params(*p, s->P);
    auto fail = [&](int code) {
        rrsph_destroy(s);
        return code;
    };
    if (rc) return fail(rc);
    s->sort_bits = key_bits(p->max_cells);
    const size_t n = p->ntotal;
    const bool d3 = s->dim == 3;
    const bool cont = p->density_treatment != 0;
    const bool mixed = precision == RRSPH_PRECISION_MIXED;
    auto& S = s->S;
    auto& G = s->G;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(set_error(RRSPH_ERR_CUDA, "rrsph_create: cudaStreamCreate failed"));
#define A(ptr, count) \
    do {                                                 \
        if ((rc = dev_alloc(s, &(ptr), (count))) != 0) return fail(rc); \
    } while (0)
    A(S.rx, n); A(S.ry, n); A(S.vx, n); A(S.vy, n); A(S.ax, n); A(S.ay, n); A(S.vpx, n); A(S.vpy, n);
    if (d3) { A(S.rz, n); A(S.vz, n); A(S.az, n); A(S.vpz, n); }
    if (p->average_velocity) { A(S.avx, n); A(S.avy, n); if (d3) A(S.avz, n); }
    A(S.rho, n); A(S.p, n); A(S.drho, n); A(S.rho_pred, n); A(S.mu, n);
    A(S.itype, n); A(S.key_of, n); A(S.itype_changed, 1);
    A(G.keys_in, n); A(G.ids_in, n); A(G.keys_a, n); A(G.ids_a, n); A(G.keys_b, n); A(G.ids_b, n);
    A(G.sort_scratch, rrsph::sort_scratch_words((uint32_t)n));
    A(G.cell_start, (size_t)s->P.max_cells); A(G.cell_end, (size_t)s->P.max_cells);
    A(G.rx, n); A(G.ry, n); if (d3) A(G.rz, n);
    A(G.itype, n);
    if (!mixed) {
        A(G.vx, n); A(G.vy, n); if (d3) A(G.vz, n);
        A(G.rho, n); A(G.p, n); A(G.pr2, n);
        // the density pass's pairs for the force pass: [3^dim + 1][n] masks, 64-bit in 3D
        A(G.nbmask, (size_t)(d3 ? 2 * 28 : 10) * n);
        // cell-relative float offsets (key pass) and their cell-order copy: the
        // density pass's float test rejects the stencil particles beyond the cutoff
        if (d3) A(S.coff4, n); else A(S.coff2, n);
        A(G.P4, n);
        if (cont) { A(G.vdx, n); A(G.vdy, n); if (d3) A(G.vdz, n); A(G.rhod, n); }
    } else {
        if (d3) { A(S.coff4, n); A(S.vpf4, n); } else { A(S.coff2, n); A(S.vpf2, n); }
        if (n < rrsph::verlet_max_particles(s->dim)) {  // neighbour reuse
            const size_t cap = (size_t)rrsph::verlet_cap(s->dim);
            A(S.cxy, n); A(S.bcxy, n); A(S.slot, n); A(S.vl_rebuild, 2); A(s->vl_builds, 1);
            if (d3) {
                A(S.boff4, n);
            } else {
                A(S.boff, n);
            }
            S.vl_gone = S.vl_rebuild + 1;
            A(G.vlist, cap * n); A(G.vcount, n); A(G.nlist, cap * n); A(G.ncount, n);
        }
        A(G.P4, n); A(G.V4, n); A(G.PR, n);
        if (cont) A(G.VD4, n);
        s->p4buf[0] = s->p4buf[1] = G.P4;
        s->v4buf[0] = s->v4buf[1] = G.V4;
        s->vd4buf[0] = s->vd4buf[1] = G.VD4;
        if (G.vlist) {
            A(s->p4buf[1], n); A(s->v4buf[1], n);
            if (cont) A(s->vd4buf[1], n);
        }
        G.P4n = s->p4buf[1];
        G.V4n = s->v4buf[1];
        G.VD4n = cont ? s->vd4buf[1] : nullptr;
        if (!d3) A(G.nbmask, 10 * n);
    }
    A(s->scal, 2);
    A(s->flags, 1);
#undef A
    if (S.vl_rebuild) {
        if (cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking) != cudaSuccess ||
            cudaMallocHost(&s->h_vl, sizeof(uint32_t)) != cudaSuccess)
            return fail(set_error(RRSPH_ERR_CUDA, "rrsph_create: neighbour-reuse stream"));
        // no lists yet: empty lists, masks and grid until the first build (which the flag forces)
        const struct {
            void* ptr;
            int value;
            size_t bytes;
            const char* name;
        } zero[] = {{S.vl_rebuild, 0xFF, sizeof(uint32_t), "rebuild flag"},
                    {S.vl_gone, 0, sizeof(uint32_t), "build flags"},
                    {s->vl_builds, 0, sizeof(unsigned long long), "build count"},
                    {G.vcount, 0, n * sizeof(uint32_t), "candidate counts"},
                    {G.ncount, 0, n * sizeof(uint32_t), "neighbour counts"},
                    {S.bcxy, 0, n * sizeof(uint32_t), "build cells"},
                    {S.slot, 0, n * sizeof(uint32_t), "build slots"},
                    {d3 ? (void*)S.boff4 : (void*)S.boff, 0, n * (d3 ? sizeof(float4) : sizeof(float2)), "build offsets"},
                    {G.keys_a, 0, n * sizeof(uint32_t), "grid keys"},
                    {G.ids_a, 0, n * sizeof(uint32_t), "grid ids"}};
        for (const auto& z : zero) {
            const cudaError_t e = cudaMemsetAsync(z.ptr, z.value, z.bytes, s->stream);
            if (e != cudaSuccess)
                return fail(set_error(RRSPH_ERR_CUDA, std::string("rrsph_create: memset of the ") + z.name +
                                                          " failed: " + cudaGetErrorString(e)));
        }
        s->verlet = true;
        s->verlet_skin = s->dim == 3 ? kDefaultSkin3 : kDefaultSkin2;
        set_verlet_params(s);
        s->P.keep_cells = tiles_active(s) ? 1 : 0;  // the table is cleared wholesale below
    }
    if (cudaMallocHost(&s->h_scal, sizeof(rrsph::StepScalars)) != cudaSuccess ||
        cudaMallocHost(&s->h_flags, sizeof(uint32_t)) != cudaSuccess ||
        cudaHostAlloc(&s->h_report, sizeof(rrsph::HostReport), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&s->d_report, s->h_report, 0) != cudaSuccess)
        return fail(set_error(RRSPH_ERR_OUT_OF_MEMORY, "rrsph_create: pinned host allocation failed"));
    std::memset(s->h_report, 0, sizeof(rrsph::HostReport));
    // empty cell table, zeroed state
    if (cudaMemsetAsync(G.cell_start, 0xFF, (size_t)s->P.max_cells * sizeof(uint32_t), s->stream) != cudaSuccess ||
        cudaMemsetAsync(S.key_of, 0xFF, n * sizeof(uint32_t), s->stream) != cudaSuccess ||
        cudaMemsetAsync(s->scal, 0, 2 * sizeof(rrsph::StepScalars), s->stream) != cudaSuccess ||
        cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), s->stream) != cudaSuccess ||
        cudaMemsetAsync(S.itype_changed, 0, sizeof(uint32_t), s->stream) != cudaSuccess)
        return fail(set_error(RRSPH_ERR_CUDA, std::string("rrsph_create: memset failed: ") +
                                                  cudaGetErrorString(cudaGetLastError())));
    for (int i = 0; i <= kPhases; i++) {
        if (cudaEventCreate(&s->ev[i]) != cudaSuccess) return fail(set_error(RRSPH_ERR_CUDA, "rrsph_create: event"));
    }
    if (cudaStreamSynchronize(s->stream) != cudaSuccess)
        return fail(set_error(RRSPH_ERR_CUDA, "rrsph_create: synchronize failed"));
    *out = s;
    return RRSPH_OK;
}

extern "C" void rrsph_destroy(rrsph_solver* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    rrsph_impl::adjoint_release(s);
    rrsph_impl::destroy_step_graphs(s);
    if (s->ev_density) cudaEventDestroy(s->ev_density);
    if (s->ev_dl) cudaEventDestroy(s->ev_dl);
    if (s->dl_stream) cudaStreamDestroy(s->dl_stream);
    for (int i = 0; i <= kPhases; i++)
        if (s->ev[i]) cudaEventDestroy(s->ev[i]);
    for (void* a : s->allocations)
        if (a) cudaFree(a);
    if (s->h_scal) cudaFreeHost(s->h_scal);
    if (s->h_flags) cudaFreeHost(s->h_flags);
    if (s->h_report) cudaFreeHost(s->h_report);
    if (s->h_vl) cudaFreeHost(s->h_vl);
    if (s->aux) cudaStreamDestroy(s->aux);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

extern "C" int rrsph_get_stream(rrsph_solver* s, void** stream) {
    if (!s || !stream) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_get_stream: null argument");
    *stream = (void*)s->stream;
    return RRSPH_OK;
}

namespace {
// The device address of a host array the device can reach (page-locked host
// memory: cudaMallocHost / cudaHostAlloc / cudaHostRegister), else null.
// Null in, null out.
const void* device_view(const void* host) {
    if (!host) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}
int finish_upload(rrsph_solver* s, bool wait);

// rrsph_upload without the checks; wait: return after the caller's arrays
// were read (else they are read in stream order). rho may be null with
// summation density (rrsph_step_host: the step recomputes it before any read).
int upload_impl(rrsph_solver* s, const double* r, uint32_t stride, const double* v, const double* rho,
                const double* pres, const int32_t* itype, bool wait) {
    int rc;
    const size_t n = s->P.n;
    auto& S = s->S;
    cudaStream_t st = s->stream;
    // page-locked caller arrays: one kernel reads them over the host link (and
    // clears itype_changed: the uploaded types are the reference)
    const double* dr = static_cast<const double*>(device_view(r));
    const double* dv = static_cast<const double*>(device_view(v));
    const double* drho = static_cast<const double*>(device_view(rho));
    const double* dp = static_cast<const double*>(device_view(pres));
    const int32_t* dit = static_cast<const int32_t*>(device_view(itype));
    if (dr && dv && (drho || !rho) && dit && (dp || !pres)) {
        if (s->verlet) set_verlet_copies(s, 0, 0);  // step 0 reads the copies its key pass writes
        if (S.vl_rebuild) {  // before the key pass below, which may raise the flag again
            rrsph::launch_verlet_upload_check(S.vl_rebuild, S.vl_gone, st);
            s->launches++;
        }
        if (s->dim == 3)
            rrsph::launch_upload_direct<3>(s->P, S, s->G, dr, dv, drho, dp, dit, stride, s->scal, s->params.dt,
                                           s->flags, st);
        else
            rrsph::launch_upload_direct<2>(s->P, S, s->G, dr, dv, drho, dp, dit, stride, s->scal, s->params.dt,
                                           s->flags, st);
        s->launches++;
        if (wait) RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
        s->step_index = 0;
        s->nlist_valid = false;
        s->keys_ready = true;  // the upload kernel ran the first step's key pass
        return RRSPH_OK;
    }
    if ((rc = ensure_staging(s, 2 * n * stride)) != 0) return rc;
    RRSPH_CUDA_TRY(cudaMemsetAsync(S.itype_changed, 0, sizeof(uint32_t), st));  // the uploaded types are the reference
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->staging, r, n * stride * sizeof(double), cudaMemcpyHostToDevice, st));
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->staging + n * stride, v, n * stride * sizeof(double), cudaMemcpyHostToDevice, st));
    if (s->dim == 3) rrsph::launch_unpack<3>(s->P, S, s->staging, s->staging + n * stride, stride, st);
    else rrsph::launch_unpack<2>(s->P, S, s->staging, s->staging + n * stride, stride, st);
    s->launches++;
    if (rho) RRSPH_CUDA_TRY(cudaMemcpyAsync(S.rho, rho, n * sizeof(double), cudaMemcpyHostToDevice, st));
    if (pres) RRSPH_CUDA_TRY(cudaMemcpyAsync(S.p, pres, n * sizeof(double), cudaMemcpyHostToDevice, st));
    else RRSPH_CUDA_TRY(cudaMemsetAsync(S.p, 0, n * sizeof(double), st));
    RRSPH_CUDA_TRY(cudaMemcpyAsync(S.itype, itype, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    // fresh work arrays of time_integration (TimeIntegration.cpp:35-50)
    RRSPH_CUDA_TRY(cudaMemsetAsync(S.ax, 0, n * sizeof(double), st));
    RRSPH_CUDA_TRY(cudaMemsetAsync(S.ay, 0, n * sizeof(double), st));
    if (S.az) RRSPH_CUDA_TRY(cudaMemsetAsync(S.az, 0, n * sizeof(double), st));
    if (S.avx) {
        RRSPH_CUDA_TRY(cudaMemsetAsync(S.avx, 0, n * sizeof(double), st));
        RRSPH_CUDA_TRY(cudaMemsetAsync(S.avy, 0, n * sizeof(double), st));
        if (S.avz) RRSPH_CUDA_TRY(cudaMemsetAsync(S.avz, 0, n * sizeof(double), st));
    }
    RRSPH_CUDA_TRY(cudaMemsetAsync(S.drho, 0, n * sizeof(double), st));
    return finish_upload(s, wait);
}
}  // namespace

extern "C" int rrsph_upload(rrsph_solver* s, const double* r, uint32_t stride, const double* v, const double* rho,
                            const double* pres, const int32_t* itype) {
    int rc = check_handle(s, "rrsph_upload");
    if (rc) return rc;
    if (!r || !v || !rho || !itype) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_upload: null array");
    if (stride < (uint32_t)s->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_upload: stride < dim");
    return upload_impl(s, r, stride, v, rho, pres, itype, true);
}

namespace {
// The rest of rrsph_upload after the state is on the device: the step
// scalars, the neighbour-list check, and (wait) the wait for the caller's arrays.
int finish_upload(rrsph_solver* s, bool wait) {
    auto& S = s->S;
    cudaStream_t st = s->stream;
    rrsph::StepScalars init{};
    init.dt = s->params.dt;
    std::memcpy(s->h_scal, &init, sizeof(init));
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->scal, s->h_scal, sizeof(init), cudaMemcpyHostToDevice, st));
    if (S.vl_rebuild) {  // the next key pass checks the uploaded positions against the last build
        rrsph::launch_verlet_upload_check(S.vl_rebuild, S.vl_gone, st);
        s->launches++;
    }
    if (wait) RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
    s->step_index = 0;
    s->nlist_valid = false;
    s->keys_ready = false;
    return RRSPH_OK;
}
}  // namespace

namespace {
// rrsph_download without the checks; wait: return after the arrays were written;
// itype_if_changed: page-locked itype holds the uploaded types (rrsph_step_host),
// so it is rewritten only if a step changed a type since.
int download_impl(rrsph_solver* s, double* r, uint32_t stride, double* v, double* rho, double* pres, int32_t* itype,
                  bool wait, bool itype_if_changed = false) {
    int rc;
    const size_t n = s->P.n;
    cudaStream_t st = s->stream;
    // page-locked caller arrays: one kernel writes them over the host link
    double* dr = const_cast<double*>(static_cast<const double*>(device_view(r)));
    double* dv = const_cast<double*>(static_cast<const double*>(device_view(v)));
    double* drho = const_cast<double*>(static_cast<const double*>(device_view(rho)));
    double* dp = const_cast<double*>(static_cast<const double*>(device_view(pres)));
    int32_t* dit = const_cast<int32_t*>(static_cast<const int32_t*>(device_view(itype)));
    if ((dr || !r) && (dv || !v) && (drho || !rho) && (dp || !pres) && (dit || !itype)) {
        const uint32_t* itype_if = itype_if_changed ? s->S.itype_changed : nullptr;
        if (s->dim == 3) rrsph::launch_download_direct<3>(s->P, s->S, dr, dv, drho, dp, dit, stride, st, itype_if);
        else rrsph::launch_download_direct<2>(s->P, s->S, dr, dv, drho, dp, dit, stride, st, itype_if);
        s->launches++;
        if (wait) RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
        return RRSPH_OK;
    }
    if (r || v) {
        if ((rc = ensure_staging(s, 2 * n * stride)) != 0) return rc;
        if (s->dim == 3) rrsph::launch_pack<3>(s->P, s->S, r ? s->staging : nullptr, v ? s->staging + n * stride : nullptr, stride, st);
        else rrsph::launch_pack<2>(s->P, s->S, r ? s->staging : nullptr, v ? s->staging + n * stride : nullptr, stride, st);
        s->launches++;
        if (r) RRSPH_CUDA_TRY(cudaMemcpyAsync(r, s->staging, n * stride * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (v) RRSPH_CUDA_TRY(cudaMemcpyAsync(v, s->staging + n * stride, n * stride * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    if (rho) RRSPH_CUDA_TRY(cudaMemcpyAsync(rho, s->S.rho, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (pres) RRSPH_CUDA_TRY(cudaMemcpyAsync(pres, s->S.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (itype) RRSPH_CUDA_TRY(cudaMemcpyAsync(itype, s->S.itype, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    if (wait) RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
    return RRSPH_OK;
}
}  // namespace

extern "C" int rrsph_download(rrsph_solver* s, double* r, uint32_t stride, double* v, double* rho, double* pres,
                              int32_t* itype) {
    int rc = check_handle(s, "rrsph_download");
    if (rc) return rc;
    if ((r || v) && stride < (uint32_t)s->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_download: stride < dim");
    return download_impl(s, r, stride, v, rho, pres, itype, true);
}

namespace {

// Captures `count` steps, the first of parity par0, as one executable graph.
// A step of the reuse loop adds a conditional node whose body (the rebuild)
// is captured after the main capture, with the step's own buffer set.
int capture_steps(rrsph_solver* s, int par0, int count, cudaGraphExec_t* out, unsigned long long* launches_out) {
    cudaStream_t st = s->stream;
    cudaGraph_t g = nullptr;
    const unsigned long long before = s->launches;
    std::vector<std::pair<cudaGraph_t, rrsph::Sorted>> bodies;
    RRSPH_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = RRSPH_OK;
    for (int j = 0; j < count && rc == RRSPH_OK; j++) {
        rc = enqueue_step_dim(s, (par0 + j) & 1, nullptr, false);
        if (rc == RRSPH_OK && s->vl_pending) {
            bodies.emplace_back(s->vl_body, s->G);
            s->vl_pending = false;
        }
    }
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (rc == RRSPH_OK && ce != cudaSuccess)
        rc = set_error(RRSPH_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    const rrsph::Sorted keep = s->G;
    for (size_t b = 0; b < bodies.size() && rc == RRSPH_OK; b++) {
        s->G = bodies[b].second;
        s->vl_body = bodies[b].first;
        rc = capture_verlet_body(s);
    }
    s->G = keep;
    if (rc == RRSPH_OK) {
        const cudaError_t e = cudaGraphInstantiate(out, g, 0);
        if (e != cudaSuccess) rc = set_error(RRSPH_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    if (g) cudaGraphDestroy(g);
    *launches_out = s->launches - before;
    s->launches = before;
    return rc;
}

// The single-step graphs of both parities and the kRunSteps-step graphs
// starting at either parity, captured together on first use.
int ensure_graphs(rrsph_solver* s) {
    for (int par = 0; par < 2; par++) {
        int rc;
        if (!s->graph[par] && (rc = capture_steps(s, par, 1, &s->graph[par], &s->launches_in_graph[par])) != 0)
            return rc;
        if (!s->graph_run[par] &&
            (rc = capture_steps(s, par, kRunSteps, &s->graph_run[par], &s->launches_in_run[par])) != 0)
            return rc;
    }
    return RRSPH_OK;
}

// nsteps steps on the handle's stream; mark_last: the last step records
// ev_density after its density pass (graph replay only).
int enqueue_steps(rrsph_solver* s, uint64_t nsteps, bool mark_last = false) {
    cudaStream_t st = s->stream;
    for (uint64_t k = 0; k < nsteps;) {
        const int par = (int)(s->step_index & 1);
        const bool with_keys = !s->keys_ready;
        s->keys_ready = true;
        uint64_t done = 1;
        if (s->timing) {
            int rc = enqueue_step_dim(s, par, s->ev, with_keys);
            if (rc) return rc;
            RRSPH_CUDA_TRY(cudaEventSynchronize(s->ev[kPhases]));
            for (int i = 0; i < kPhases; i++) {
                float ms = 0;
                cudaEventElapsedTime(&ms, s->ev[i], s->ev[i + 1]);
                s->phase_ms[i] += ms;
            }
            s->timed_steps++;
        } else if (s->graphs) {
            const int rc = ensure_graphs(s);
            if (rc) return rc;
            if (with_keys) enqueue_keys_dim(s, par);
            // whole runs of kRunSteps steps as one graph launch, the rest one step each
            if (nsteps - k - (mark_last ? 1 : 0) >= (uint64_t)kRunSteps) {
                RRSPH_CUDA_TRY(cudaGraphLaunch(s->graph_run[par], st));
                s->launches += s->launches_in_run[par];
                done = kRunSteps;
            } else if (mark_last && k + 1 == nsteps) {
                if (!s->graph_mark[par]) {
                    s->mark_density = true;
                    const int rm = capture_steps(s, par, 1, &s->graph_mark[par], &s->launches_in_mark[par]);
                    s->mark_density = false;
                    if (rm) return rm;
                }
                RRSPH_CUDA_TRY(cudaGraphLaunch(s->graph_mark[par], st));
                s->launches += s->launches_in_mark[par];
            } else {
                RRSPH_CUDA_TRY(cudaGraphLaunch(s->graph[par], st));
                s->launches += s->launches_in_graph[par];
            }
        } else {
            int rc = enqueue_step_dim(s, par, nullptr, with_keys);
            if (rc) return rc;
        }
        s->step_index += done;
        k += done;
        s->nlist_valid = s->verlet;  // the step's density pass wrote nlist on the current grid
    }
    return RRSPH_OK;
}

}  // namespace

extern "C" int rrsph_set_time(rrsph_solver* s, double time) {
    int rc = check_handle(s, "rrsph_set_time");
    if (rc) return rc;
    const int par = (int)(s->step_index & 1);
    rrsph::launch_set_time(&s->scal[par], time, nullptr, s->stream);
    RRSPH_CUDA_TRY(cudaGetLastError());
    s->launches++;
    return RRSPH_OK;
}

extern "C" int rrsph_step_async(rrsph_solver* s, uint64_t nsteps) {
    int rc = check_handle(s, "rrsph_step_async");
    if (rc) return rc;
    return enqueue_steps(s, nsteps);
}

extern "C" int rrsph_sync(rrsph_solver* s, double* time_out) {
    int rc = check_handle(s, "rrsph_sync");
    if (rc) return rc;
    cudaStream_t st = s->stream;
    const int parn = (int)(s->step_index & 1);
    rrsph::launch_report(&s->scal[parn], s->step_index ? &s->scal[parn ^ 1] : nullptr, s->flags, s->d_report, st);
    s->launches++;
    RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
    RRSPH_CUDA_TRY(cudaGetLastError());
    if (time_out) *time_out = s->h_report->time;
    return flags_to_status(s, s->h_report->flags);
}

extern "C" int rrsph_step(rrsph_solver* s, uint64_t nsteps, double* time_io) {
    int rc = check_handle(s, "rrsph_step");
    if (rc) return rc;
    if (!time_io) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step: null time");
    rrsph::launch_set_time(&s->scal[s->step_index & 1], *time_io, s->flags, s->stream);  // time, flags cleared
    RRSPH_CUDA_TRY(cudaGetLastError());
    s->launches++;
    if ((rc = enqueue_steps(s, nsteps)) != 0) return rc;
    return rrsph_sync(s, time_io);
}

namespace {
// rrsph_step_host (upload first) and rrsph_step_download (the state on the
// device); the arguments are checked by the callers.
int steps_and_download(rrsph_solver* s, uint64_t nsteps, double* time_io, double* r, uint32_t stride, double* v,
                       double* rho, double* pres, int32_t* itype, bool upload) {
    int rc;
    cudaStream_t st = s->stream;
    const size_t n = s->P.n;
    // with graph replay the last step marks the end of its density pass: p, and
    // rho with summation density (the whole step leaves it), come back on a
    // copy stream while the force gather runs
    const bool mark = s->graphs && !s->timing;
    if (mark && !s->dl_stream) {
        if (cudaStreamCreateWithFlags(&s->dl_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_density, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_dl, cudaEventDisableTiming) != cudaSuccess)
            return set_error(RRSPH_ERR_CUDA, "rrsph_step_host: copy stream");
    }
    // with summation density the step recomputes rho before reading it: not uploaded
    const double* rho_in = s->P.density_treatment == 0 ? nullptr : rho;
    if (upload && (rc = upload_impl(s, r, stride, v, rho_in, nullptr, itype, false)) != 0) return rc;
    rrsph::launch_set_time(&s->scal[s->step_index & 1], *time_io, s->flags, st);  // time, flags cleared
    RRSPH_CUDA_TRY(cudaGetLastError());
    s->launches++;
    if ((rc = enqueue_steps(s, nsteps, mark)) != 0) return rc;
    const bool early_rho = mark && rho && s->P.density_treatment == 0;
    if (mark) {
        RRSPH_CUDA_TRY(cudaStreamWaitEvent(s->dl_stream, s->ev_density, 0));
        if (pres) RRSPH_CUDA_TRY(cudaMemcpyAsync(pres, s->S.p, n * sizeof(double), cudaMemcpyDeviceToHost, s->dl_stream));
        if (early_rho)
            RRSPH_CUDA_TRY(cudaMemcpyAsync(rho, s->S.rho, n * sizeof(double), cudaMemcpyDeviceToHost, s->dl_stream));
        RRSPH_CUDA_TRY(cudaEventRecord(s->ev_dl, s->dl_stream));
    }
    if ((rc = download_impl(s, r, stride, v, early_rho ? nullptr : rho, mark ? nullptr : pres, itype, false, upload)) != 0)
        return rc;
    if (mark) RRSPH_CUDA_TRY(cudaStreamWaitEvent(st, s->ev_dl, 0));
    return rrsph_sync(s, time_io);
}
}  // namespace

extern "C" int rrsph_step_host(rrsph_solver* s, uint64_t nsteps, double* time_io, double* r, uint32_t stride,
                               double* v, double* rho, double* pres, int32_t* itype) {
    int rc = check_handle(s, "rrsph_step_host");
    if (rc) return rc;
    if (!time_io || !r || !v || !rho || !itype) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_host: null argument");
    if (stride < (uint32_t)s->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_host: stride < dim");
    if (nsteps == 0) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_host: no steps");
    return steps_and_download(s, nsteps, time_io, r, stride, v, rho, pres, itype, true);
}

extern "C" int rrsph_step_download(rrsph_solver* s, uint64_t nsteps, double* time_io, double* r, uint32_t stride,
                                   double* v, double* rho, double* pres, int32_t* itype) {
    int rc = check_handle(s, "rrsph_step_download");
    if (rc) return rc;
    if (!time_io) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_download: null time");
    if ((r || v) && stride < (uint32_t)s->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_download: stride < dim");
    if (nsteps == 0) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_download: no steps");
    return steps_and_download(s, nsteps, time_io, r, stride, v, rho, pres, itype, false);
}

extern "C" int rrsph_last_report(rrsph_solver* s, double* time, uint32_t* flags, uint64_t* pairs_last,
                                 uint64_t* pairs_total) {
    int rc = check_handle(s, "rrsph_last_report");
    if (rc) return rc;
    const rrsph::HostReport r = *s->h_report;  // written by the last rrsph_sync's report kernel
    if (time) *time = r.time;
    if (flags) *flags = r.flags;
    if (pairs_last) *pairs_last = r.pairs_last;
    if (pairs_total) *pairs_total = r.pairs_total;
    return RRSPH_OK;
}

extern "C" int rrsph_status(rrsph_solver* s, uint32_t* flags, int clear) {
    int rc = check_handle(s, "rrsph_status");
    if (rc) return rc;
    if (!flags) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_status: null flags");
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->h_flags, s->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    if (clear) RRSPH_CUDA_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    *flags = *s->h_flags;
    return RRSPH_OK;
}

extern "C" int rrsph_diagnostics_get(rrsph_solver* s, rrsph_diagnostics* out) {
    int rc = check_handle(s, "rrsph_diagnostics_get");
    if (rc) return rc;
    if (!out) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_diagnostics_get: null output");
    constexpr int kBlocks = 608;  // fixed: the summation order does not depend on the device
    if (!s->diag) {
        if ((rc = dev_alloc(s, &s->diag, (size_t)(kBlocks + 1) * rrsph::kDiagQuantities)) != 0) return rc;
    }
    double* sums = s->diag + (size_t)kBlocks * rrsph::kDiagQuantities;
    if (s->dim == 3) rrsph::launch_diagnostics<3>(s->P, s->S, s->diag, kBlocks, sums, s->stream);
    else rrsph::launch_diagnostics<2>(s->P, s->S, s->diag, kBlocks, sums, s->stream);
    s->launches += 2;
    double h[rrsph::kDiagQuantities];
    RRSPH_CUDA_TRY(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    out->mass = h[0];
    out->kinetic = h[1];
    out->potential = h[2];
    out->internal = h[3];
    out->momentum[0] = h[4];
    out->momentum[1] = h[5];
    out->momentum[2] = h[6];
    out->mass_boundary = h[7];
    out->fluid = (uint64_t)h[8];
    out->boundary = (uint64_t)h[9];
    return RRSPH_OK;
}

extern "C" int rrsph_pair_count(rrsph_solver* s, uint64_t* last_step, uint64_t* total) {
    int rc = check_handle(s, "rrsph_pair_count");
    if (rc) return rc;
    const int cur = (int)(s->step_index & 1);  // scalars the next step will use
    rrsph::StepScalars h[2];
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->h_scal, s->scal + cur, sizeof(rrsph::StepScalars), cudaMemcpyDeviceToHost, s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    h[0] = *s->h_scal;
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->h_scal, s->scal + (cur ^ 1), sizeof(rrsph::StepScalars), cudaMemcpyDeviceToHost, s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    h[1] = *s->h_scal;
    if (last_step) *last_step = s->step_index ? h[1].pairs : 0;
    if (total) *total = h[0].pairs_total;
    return RRSPH_OK;
}

extern "C" int rrsph_get_dt(rrsph_solver* s, double* dt) {
    int rc = check_handle(s, "rrsph_get_dt");
    if (rc) return rc;
    if (!dt) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_get_dt: null dt");
    const int par = (int)(s->step_index & 1);
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->h_scal, &s->scal[par], sizeof(rrsph::StepScalars), cudaMemcpyDeviceToHost, s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    *dt = s->h_scal->dt;
    return RRSPH_OK;
}

// ---------------------------------------------------------- loop pieces ----

namespace {

template <int DIM>
void enqueue_component_grid(rrsph_solver* s, bool with_p) {
    s->keys_ready = false;  // this grid's keys were made without the predictor
    s->nlist_valid = false;  // and it replaces the grid the last step's list refers to
    if (s->P.keep_cells)     // the last build's table is still in place
        cudaMemsetAsync(s->G.cell_start, 0xFF, (size_t)s->P.max_cells * sizeof(uint32_t), s->stream);
    if (s->S.vl_rebuild) cudaMemsetAsync(s->S.vl_rebuild, 0xFF, sizeof(uint32_t), s->stream);
    rrsph::GatherSrc fsrc{s->S.vx, s->S.vy, s->S.vz, s->S.rho, with_p ? s->S.p : nullptr, 0};
    enqueue_grid<DIM>(s, 0, s->scal, fsrc);
}
void enqueue_component_grid_dim(rrsph_solver* s, bool with_p) {
    if (s->dim == 3) enqueue_component_grid<3>(s, with_p);
    else enqueue_component_grid<2>(s, with_p);
}

int finish_component(rrsph_solver* s, const char* fn) {
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->h_flags, s->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(RRSPH_ERR_CUDA, std::string(fn) + ": " + cudaGetErrorString(e));
    const uint32_t f = *s->h_flags;
    if (f & RRSPH_FLAG_OUT_OF_DOMAIN) return set_error(RRSPH_ERR_OUT_OF_DOMAIN, "cell_idx was >= params.max_cells");
    if (f & RRSPH_FLAG_NEIGHBOUR_OVERFLOW) return set_error(RRSPH_ERR_NEIGHBOUR_OVERFLOW, "making neighbours grid: error occured");
    return RRSPH_OK;
}

}  // namespace

extern "C" int rrsph_grid_find(rrsph_solver* s, uint32_t* keys, uint32_t* grid, uint32_t* cells_start) {
    int rc = check_handle(s, "rrsph_grid_find");
    if (rc) return rc;
    cudaStream_t st = s->stream;
    RRSPH_CUDA_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), st));
    enqueue_component_grid_dim(s, false);
    const size_t n = s->P.n;
    uint32_t* d_cs = nullptr;
    if (cells_start) {
        RRSPH_CUDA_TRY(cudaMallocAsync(&d_cs, ((size_t)s->P.max_cells + 1) * sizeof(uint32_t), st));
        rrsph::launch_cells_start(s->P, s->G, d_cs, st);
        s->launches++;
        RRSPH_CUDA_TRY(cudaMemcpyAsync(cells_start, d_cs, ((size_t)s->P.max_cells + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        RRSPH_CUDA_TRY(cudaFreeAsync(d_cs, st));
    }
    if (keys) RRSPH_CUDA_TRY(cudaMemcpyAsync(keys, s->S.key_of, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (grid) RRSPH_CUDA_TRY(cudaMemcpyAsync(grid, s->G.id, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    return finish_component(s, "rrsph_grid_find");
}

extern "C" int rrsph_neighbours(rrsph_solver* s, uint32_t* counts, uint32_t* list, uint32_t max_per,
                                uint64_t* total_pairs) {
    int rc = check_handle(s, "rrsph_neighbours");
    if (rc) return rc;
    if (!counts || !list || max_per == 0) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_neighbours: bad arguments");
    cudaStream_t st = s->stream;
    const size_t n = s->P.n;
    RRSPH_CUDA_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), st));
    enqueue_component_grid_dim(s, false);
    uint32_t *d_counts = nullptr, *d_list = nullptr;
    RRSPH_CUDA_TRY(cudaMallocAsync(&d_counts, n * sizeof(uint32_t), st));
    RRSPH_CUDA_TRY(cudaMallocAsync(&d_list, n * (size_t)max_per * sizeof(uint32_t), st));
    if (s->dim == 3) rrsph::launch_neighbour_list<3>(s->P, s->G, d_counts, d_list, max_per, s->flags, st);
    else rrsph::launch_neighbour_list<2>(s->P, s->G, d_counts, d_list, max_per, s->flags, st);
    s->launches++;
    RRSPH_CUDA_TRY(cudaMemcpyAsync(counts, d_counts, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    RRSPH_CUDA_TRY(cudaMemcpyAsync(list, d_list, n * (size_t)max_per * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    RRSPH_CUDA_TRY(cudaFreeAsync(d_counts, st));
    RRSPH_CUDA_TRY(cudaFreeAsync(d_list, st));
    rc = finish_component(s, "rrsph_neighbours");
    if (total_pairs) {
        uint64_t t = 0;
        for (size_t j = 0; j < n; j++) t += counts[j];
        *total_pairs = t;
    }
    return rc;
}

extern "C" int rrsph_step_neighbours(rrsph_solver* s, uint32_t* counts, uint32_t* list, uint32_t max_per,
                                     uint64_t* total_pairs) {
    int rc = check_handle(s, "rrsph_step_neighbours");
    if (rc) return rc;
    if (!counts || !list || max_per == 0)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_neighbours: bad arguments");
    if (!s->verlet)
        return set_error(RRSPH_ERR_UNSUPPORTED, "rrsph_step_neighbours: needs the FP32-mixed step with neighbour reuse");
    if (!s->nlist_valid)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_step_neighbours: no step has run since the last upload, "
                                                     "grid call or reuse setting");
    cudaStream_t st = s->stream;
    const size_t n = s->P.n;
    RRSPH_CUDA_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), st));
    uint32_t *d_counts = nullptr, *d_list = nullptr;
    RRSPH_CUDA_TRY(cudaMallocAsync(&d_counts, n * sizeof(uint32_t), st));
    RRSPH_CUDA_TRY(cudaMallocAsync(&d_list, n * (size_t)max_per * sizeof(uint32_t), st));
    s->G.key = s->G.keys_a;  // the grid of the last rebuild, which the list refers to
    s->G.id = s->G.ids_a;
    if (s->dim == 3) rrsph::launch_nlist_export<3>(s->P, s->G, d_counts, d_list, max_per, s->flags, st);
    else rrsph::launch_nlist_export<2>(s->P, s->G, d_counts, d_list, max_per, s->flags, st);
    s->launches++;
    RRSPH_CUDA_TRY(cudaMemcpyAsync(counts, d_counts, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    RRSPH_CUDA_TRY(cudaMemcpyAsync(list, d_list, n * (size_t)max_per * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    RRSPH_CUDA_TRY(cudaFreeAsync(d_counts, st));
    RRSPH_CUDA_TRY(cudaFreeAsync(d_list, st));
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->h_flags, s->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
    RRSPH_CUDA_TRY(cudaGetLastError());
    if (*s->h_flags & RRSPH_FLAG_NEIGHBOUR_OVERFLOW)
        return set_error(RRSPH_ERR_NEIGHBOUR_OVERFLOW, "rrsph_step_neighbours: a particle has more than max_per "
                                                       "neighbours, or more than a list holds");
    if (total_pairs) {
        uint64_t t = 0;
        for (size_t j = 0; j < n; j++) t += counts[j];
        *total_pairs = t;
    }
    return RRSPH_OK;
}

extern "C" int rrsph_density(rrsph_solver* s, double* out_rho_or_drho, double* out_p) {
    int rc = check_handle(s, "rrsph_density");
    if (rc) return rc;
    cudaStream_t st = s->stream;
    const size_t n = s->P.n;
    RRSPH_CUDA_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), st));
    enqueue_component_grid_dim(s, false);
    if (s->dim == 3) enqueue_density<3>(s, s->scal);
    else enqueue_density<2>(s, s->scal);
    const bool cont = s->P.density_treatment != 0;
    if (out_rho_or_drho)
        RRSPH_CUDA_TRY(cudaMemcpyAsync(out_rho_or_drho, cont ? s->S.drho : s->S.rho, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (out_p) RRSPH_CUDA_TRY(cudaMemcpyAsync(out_p, s->S.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    return finish_component(s, "rrsph_density");
}

extern "C" int rrsph_forces(rrsph_solver* s, uint32_t terms, double* a, uint32_t stride, double* av, double* mu) {
    int rc = check_handle(s, "rrsph_forces");
    if (rc) return rc;
    if (!a || stride < (uint32_t)s->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_forces: bad a/stride");
    if (av && !s->S.avx) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_forces: average_velocity is off");
    cudaStream_t st = s->stream;
    const size_t n = s->P.n;
    RRSPH_CUDA_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), st));
    enqueue_component_grid_dim(s, true);
    if (s->dim == 3) enqueue_forces<3>(s, terms, s->scal, 1);
    else enqueue_forces<2>(s, terms, s->scal, 1);
    if ((rc = ensure_staging(s, 2 * n * stride)) != 0) return rc;
    // pack a (and av) through the staging buffer with the pack kernel's layout
    rrsph::State tmp = s->S;
    tmp.rx = s->S.ax; tmp.ry = s->S.ay; tmp.rz = s->S.az;
    tmp.vx = s->S.avx; tmp.vy = s->S.avy; tmp.vz = s->S.avz;
    double* dv = av ? s->staging + n * stride : nullptr;
    if (s->dim == 3) rrsph::launch_pack<3>(s->P, tmp, s->staging, dv, stride, st);
    else rrsph::launch_pack<2>(s->P, tmp, s->staging, dv, stride, st);
    s->launches++;
    RRSPH_CUDA_TRY(cudaMemcpyAsync(a, s->staging, n * stride * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (av) RRSPH_CUDA_TRY(cudaMemcpyAsync(av, dv, n * stride * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (mu) RRSPH_CUDA_TRY(cudaMemcpyAsync(mu, s->S.mu, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    return finish_component(s, "rrsph_forces");
}

extern "C" int rrsph_download_rates(rrsph_solver* s, double* a, uint32_t stride, double* drho) {
    int rc = check_handle(s, "rrsph_download_rates");
    if (rc) return rc;
    if (a && stride < (uint32_t)s->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_download_rates: stride < dim");
    cudaStream_t st = s->stream;
    const size_t n = s->P.n;
    if (a) {
        if ((rc = ensure_staging(s, n * stride)) != 0) return rc;
        rrsph::State tmp = s->S;
        tmp.rx = s->S.ax; tmp.ry = s->S.ay; tmp.rz = s->S.az;
        if (s->dim == 3) rrsph::launch_pack<3>(s->P, tmp, s->staging, nullptr, stride, st);
        else rrsph::launch_pack<2>(s->P, tmp, s->staging, nullptr, stride, st);
        s->launches++;
        RRSPH_CUDA_TRY(cudaMemcpyAsync(a, s->staging, n * stride * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    if (drho) RRSPH_CUDA_TRY(cudaMemcpyAsync(drho, s->S.drho, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(st));
    RRSPH_CUDA_TRY(cudaGetLastError());
    return RRSPH_OK;
}

// ------------------------------------------------------------- timing ------

extern "C" int rrsph_phase_count(rrsph_solver* s, int* count) {
    if (!s || !count) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_phase_count: null argument");
    *count = kPhases;
    return RRSPH_OK;
}
extern "C" const char* rrsph_phase_name(rrsph_solver* s, int phase) {
    (void)s;
    return (phase >= 0 && phase < kPhases) ? kPhaseNames[phase] : "";
}
extern "C" int rrsph_set_phase_timing(rrsph_solver* s, int enable) {
    if (!s) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_phase_timing: null solver");
    s->timing = enable != 0;
    return RRSPH_OK;
}
extern "C" int rrsph_phase_times(rrsph_solver* s, double* ms_per_phase, int count, uint64_t* steps, int reset) {
    if (!s || !ms_per_phase) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_phase_times: null argument");
    for (int i = 0; i < count && i < kPhases; i++) ms_per_phase[i] = s->phase_ms[i];
    if (steps) *steps = s->timed_steps;
    if (reset) {
        for (double& v : s->phase_ms) v = 0;
        s->timed_steps = 0;
    }
    return RRSPH_OK;
}
extern "C" int rrsph_kernel_launches(rrsph_solver* s, uint64_t* launches) {
    if (!s || !launches) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_kernel_launches: null argument");
    uint64_t builds = 0;
    if (s->vl_builds) {  // a step counts its reuse branch; add what each rebuild launched on top
        int rc = rrsph_neighbour_rebuilds(s, &builds);
        if (rc) return rc;
    }
    *launches = s->launches + builds * (s->vl_extra_launches + (s->P.keep_cells ? 1ull : 0ull));
    return RRSPH_OK;
}

extern "C" int rrsph_neighbour_rebuilds(rrsph_solver* s, uint64_t* rebuilds) {
    int rc = check_handle(s, "rrsph_neighbour_rebuilds");
    if (rc) return rc;
    if (!rebuilds) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_neighbour_rebuilds: null argument");
    *rebuilds = 0;
    if (!s->vl_builds) return RRSPH_OK;
    unsigned long long v = 0;
    RRSPH_CUDA_TRY(cudaMemcpyAsync(&v, s->vl_builds, sizeof(v), cudaMemcpyDeviceToHost, s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    *rebuilds = v;
    return RRSPH_OK;
}

extern "C" int rrsph_set_neighbour_reuse(rrsph_solver* s, int enable, double skin_over_h) {
    int rc = check_handle(s, "rrsph_set_neighbour_reuse");
    if (rc) return rc;
    if (enable && !s->S.vl_rebuild)
        return set_error(RRSPH_ERR_UNSUPPORTED, "neighbour reuse needs an FP32-mixed solver (at most 2^27 particles "
                                                "in 2D, 2^25 in 3D)");
    if (enable && !(skin_over_h >= 0 && skin_over_h <= 1))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_neighbour_reuse: skin must be in (0, 1] hsml, or 0");
    if (skin_over_h == 0) skin_over_h = s->verlet_skin;  // keep the current skin
    drop_graphs(s);
    s->verlet = enable != 0;
    s->nlist_valid = false;
    if (enable) {
        s->verlet_skin = skin_over_h;
        set_verlet_params(s);
    }
    if ((rc = set_keep_cells(s)) != 0) return rc;
    if (s->S.vl_rebuild) RRSPH_CUDA_TRY(cudaMemsetAsync(s->S.vl_rebuild, 0xFF, sizeof(uint32_t), s->stream));
    s->keys_ready = false;
    return RRSPH_OK;
}

// ------------------------------------------------- ensembles and tuning ----

namespace {


// A device copy of the particle state and step scalars (the autotuner runs
// trial steps on the uploaded state and puts it back).
struct Backup {
    std::vector<std::pair<void*, size_t>> fields;
    void* buf = nullptr;
    rrsph::StepScalars scal[2];
    uint64_t step_index = 0;
};

int backup_state(rrsph_solver* s, Backup& b) {
    const size_t n = s->P.n, d = n * sizeof(double);
    auto& S = s->S;
    double* dbl[] = {S.rx, S.ry, S.rz, S.vx, S.vy, S.vz, S.ax, S.ay, S.az, S.avx, S.avy, S.avz,
                     S.rho, S.p, S.drho, S.rho_pred};
    for (double* f : dbl)
        if (f) b.fields.emplace_back(f, d);
    b.fields.emplace_back(S.itype, n * sizeof(int32_t));
    size_t total = 0;
    for (auto& f : b.fields) total += f.second;
    RRSPH_CUDA_TRY(cudaMalloc(&b.buf, total));
    char* dst = static_cast<char*>(b.buf);
    for (auto& f : b.fields) {
        RRSPH_CUDA_TRY(cudaMemcpyAsync(dst, f.first, f.second, cudaMemcpyDeviceToDevice, s->stream));
        dst += f.second;
    }
    RRSPH_CUDA_TRY(cudaMemcpyAsync(b.scal, s->scal, sizeof(b.scal), cudaMemcpyDeviceToHost, s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    b.step_index = s->step_index;
    return RRSPH_OK;
}

int restore_state(rrsph_solver* s, const Backup& b) {
    const char* src = static_cast<const char*>(b.buf);
    for (auto& f : b.fields) {
        RRSPH_CUDA_TRY(cudaMemcpyAsync(f.first, src, f.second, cudaMemcpyDeviceToDevice, s->stream));
        src += f.second;
    }
    RRSPH_CUDA_TRY(cudaMemcpyAsync(s->scal, b.scal, sizeof(b.scal), cudaMemcpyHostToDevice, s->stream));
    if (s->S.vl_rebuild) RRSPH_CUDA_TRY(cudaMemsetAsync(s->S.vl_rebuild, 0xFF, sizeof(uint32_t), s->stream));
    RRSPH_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->step_index = b.step_index;
    s->keys_ready = false;
    s->nlist_valid = false;
    return RRSPH_OK;
}

}  // namespace

extern "C" int rrsph_set_wave_makers(rrsph_solver* s, uint32_t count, const rrsph_wave_maker* makers) {
    int rc = check_handle(s, "rrsph_set_wave_makers");
    if (rc) return rc;
    if (count && !makers) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_wave_makers: null makers");
    const size_t n = s->P.n;
    std::vector<int32_t> owner(n, -1);
    std::vector<rrsph::PistonLaw> laws(count);
    const double g = s->params.g, pi = s->params.pi;
    for (uint32_t w = 0; w < count; w++) {
        const rrsph_wave_maker& m = makers[w];
        if ((m.nwm != 2 && m.nwm != 3) || m.particles_end < m.particles_start || m.particles_end > n ||
            !(m.wave_length > 0) || !(m.depth > 0))
            return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_wave_makers: bad wave maker " + std::to_string(w));
        for (uint64_t i = m.particles_start; i < m.particles_end; i++) {
            if (owner[i] >= 0)
                return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_wave_makers: overlapping particle ranges");
            owner[i] = (int32_t)w;
        }
        // nwm_wave_number and nwm_freq as fillInComputingParams derives them (Input.cpp:125-137)
        const double k = 2. * pi / m.wave_length;
        const double kd = k * m.depth;
        laws[w] = rrsph::PistonLaw{(int)m.nwm, m.time_start, m.phase, std::sqrt(k * g * std::tanh(kd)),
                                   m.wave_magnitude, k, m.depth};
    }
    drop_graphs(s);  // the step graphs hold the state pointers by value
    if (!s->S.wave_tank) {
        if ((rc = dev_alloc(s, &s->S.wave_tank, n)) != 0) return rc;
    }
    rrsph::PistonLaw* table = nullptr;
    if ((rc = dev_alloc(s, &table, std::max<size_t>(count, 1))) != 0) return rc;
    RRSPH_CUDA_TRY(cudaMemcpy(s->S.wave_tank, owner.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (count) RRSPH_CUDA_TRY(cudaMemcpy(table, laws.data(), count * sizeof(rrsph::PistonLaw), cudaMemcpyHostToDevice));
    s->S.wave_law = table;
    if (!count) s->S.wave_tank = nullptr;  // an empty table restores the params' wave maker
    return RRSPH_OK;
}

extern "C" int rrsph_set_gather_threads(rrsph_solver* s, uint32_t density_threads, uint32_t force_threads) {
    int rc = check_handle(s, "rrsph_set_gather_threads");
    if (rc) return rc;
    for (uint32_t t : {density_threads, force_threads})
        if (t == 0 || t % 32 || t > (uint32_t)rrsph::kMaxGatherThreads)
            return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_gather_threads: block size must be a multiple of "
                                                         "32 in [32, 256]");
    drop_graphs(s);
    s->gather_threads[0] = (int)density_threads;
    s->gather_threads[1] = (int)force_threads;
    return RRSPH_OK;
}

extern "C" int rrsph_autotune(rrsph_solver* s, uint32_t steps, uint32_t* threads_out) {
    int rc = check_handle(s, "rrsph_autotune");
    if (rc) return rc;
    if (steps == 0) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_autotune: steps must be positive");
    uint32_t flags_before = 0;
    RRSPH_CUDA_TRY(cudaMemcpy(&flags_before, s->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    Backup b;
    if ((rc = backup_state(s, b)) != 0) {
        if (b.buf) cudaFree(b.buf);
        return rc;
    }
    const int cand[] = {64, 128, 256};
    float best = 0;
    int best_d = s->gather_threads[0], best_f = s->gather_threads[1];
    cudaEvent_t e0 = s->ev[0], e1 = s->ev[1];
    const bool timing = s->timing;
    s->timing = false;
    for (int td : cand) {
        for (int tf : cand) {
            drop_graphs(s);
            s->gather_threads[0] = td;
            s->gather_threads[1] = tf;
            rc = enqueue_steps(s, 1);  // captures the candidate's graphs
            if (!rc) {
                cudaEventRecord(e0, s->stream);
                rc = enqueue_steps(s, steps);
                cudaEventRecord(e1, s->stream);
            }
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(RRSPH_ERR_CUDA, "rrsph_autotune: event");
            float ms = 0;
            if (!rc) cudaEventElapsedTime(&ms, e0, e1);
            if (!rc) rc = restore_state(s, b);
            if (rc) break;
            if (best == 0 || ms < best) {
                best = ms;
                best_d = td;
                best_f = tf;
            }
        }
        if (rc) break;
    }
    s->timing = timing;
    cudaFree(b.buf);
    drop_graphs(s);
    s->gather_threads[0] = best_d;
    s->gather_threads[1] = best_f;
    if (rc) return rc;
    if (threads_out) {
        threads_out[0] = (uint32_t)best_d;
        threads_out[1] = (uint32_t)best_f;
    }
    // flags the trial steps raised belong to no step the caller ran
    RRSPH_CUDA_TRY(cudaMemcpy(s->flags, &flags_before, sizeof(uint32_t), cudaMemcpyHostToDevice));
    return RRSPH_OK;
}

extern "C" int rrsph_autotune_skin(rrsph_solver* s, uint32_t steps, double* skin_out) {
    int rc = check_handle(s, "rrsph_autotune_skin");
    if (rc) return rc;
    if (steps == 0) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_autotune_skin: steps must be positive");
    if (!s->verlet) return set_error(RRSPH_ERR_UNSUPPORTED, "rrsph_autotune_skin: needs the mixed step with neighbour reuse");
    uint32_t flags_before = 0;
    RRSPH_CUDA_TRY(cudaMemcpy(&flags_before, s->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    Backup b;
    if ((rc = backup_state(s, b)) != 0) {
        if (b.buf) cudaFree(b.buf);
        return rc;
    }
    // each trial starts from a fresh build of the same state (two untimed
    // steps, which also capture the step graphs) and times `steps` steps with
    // the rebuilds its skin asks for: a wider skin rebuilds less often and
    // tests more candidates per step
    const double cand[] = {0.2, 0.3, 0.4, 0.5, 0.6, 0.8};
    const double current = s->verlet_skin;
    double best_skin = current;
    float best = 0;
    cudaEvent_t e0 = s->ev[0], e1 = s->ev[1];
    const bool timing = s->timing;
    s->timing = false;
    for (double skin : cand) {
        drop_graphs(s);
        s->verlet_skin = skin;
        set_verlet_params(s);
        if (cudaMemsetAsync(s->S.vl_rebuild, 0xFF, sizeof(uint32_t), s->stream) != cudaSuccess) {
            rc = set_error(RRSPH_ERR_CUDA, "rrsph_autotune_skin: memset");
            break;
        }
        rc = enqueue_steps(s, 2);
        if (!rc) {
            cudaEventRecord(e0, s->stream);
            rc = enqueue_steps(s, steps);
            cudaEventRecord(e1, s->stream);
        }
        if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(RRSPH_ERR_CUDA, "rrsph_autotune_skin: event");
        float ms = 0;
        if (!rc) cudaEventElapsedTime(&ms, e0, e1);
        if (!rc) rc = restore_state(s, b);
        if (rc) break;
        if (best == 0 || ms < best) {
            best = ms;
            best_skin = skin;
        }
    }
    s->timing = timing;
    cudaFree(b.buf);
    drop_graphs(s);
    s->verlet_skin = rc ? current : best_skin;
    set_verlet_params(s);
    s->nlist_valid = false;
    RRSPH_CUDA_TRY(cudaMemsetAsync(s->S.vl_rebuild, 0xFF, sizeof(uint32_t), s->stream));
    if (rc) return rc;
    if (skin_out) *skin_out = best_skin;
    RRSPH_CUDA_TRY(cudaMemcpy(s->flags, &flags_before, sizeof(uint32_t), cudaMemcpyHostToDevice));
    return RRSPH_OK;
}
