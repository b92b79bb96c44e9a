// ref_driver.cpp — runs the reference's own RRSPH_OMP compute core on a case
// written by the test harness (TEST INFRASTRUCTURE: builds only where the
// reference sources are present; see oracle/build_ref.sh).
//
// The reference's full executable cannot be built here (fmt and googletest are
// not vendored), so this driver stands in for fileInput()/time_integration():
// it sets the global ExperimentParams from a key/value file whose values were
// derived by the caller, and calls the reference's functions:
//   grid        make_grid + find_neighbours           (RRSPH_OMP/src/GridFind.cpp:47-189)
//   density     density_sum | density_con             (RRSPH_COMMON/include/Density.h:25-114)
//   terms:M     the per-pair parts summed per particle as the reference's unit tests
//               do (RRSPH_COMMON/tests/test*OMP.cpp): M bit mask of RRSPH_TERM_*
//   accel       update_acceleration                   (RRSPH_OMP/src/UpdateAcceleration.cpp:33-125)
//   run:N       N iterations of the loop body of TimeIntegration.cpp:60-100 with the
//               piston call enabled (dynamic_boundaries, WaveMaker.cpp:34-82),
//               reporting wall time per phase and per step (step_ms.f64; phase_ms.f64:
//               per step predict, grid, density, accel, whole) and the
//               directed pairs of every step's find_neighbours (pairs.u64, counted
//               outside the timed phases); when
//               case_dir holds gauges.txt ("every search_n type_filter" then the gauge
//               x positions), the WaterProfile free-surface elevation at those
//               positions is sampled before the first step and after every `every`
//               steps into gauges.f64 (samples x gauges)
//
// Usage: rrsph_ref <case_dir> <mode> [threads]
// Inputs in case_dir: params.txt, r.f64, v.f64, rho.f64, p.f64, itype.i32
// (r, v: ntotal x dim doubles). Outputs are written into case_dir.
#include "CommonIncl.h"
#include "GridUtils.h"
#include "GridFind.h"
#include "Density.h"
#include "InternalForce.h"
#include "ArtificialViscosity.h"
#include "ExtForce.h"
#include "AverageVelocity.h"
#include "UpdateAcceleration.h"
#include "PredictHalfStep.h"
#include "WholeStep.h"
#include "WaveMaker.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iomanip>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

// Symbols the reference's libraries would provide (version queries, logging of dt).
rr_uint RRSPH_GetSpecificVersionMajor() { return 0; }
rr_uint RRSPH_GetSpecificVersionMinor() { return 0; }
rr_uint RRSPH_GetSpecificVersionPatch() { return 0; }
std::string RRSPH_GetSpecificVersionName() { return "RRSPH_OMP"; }
std::string format_save_time(rr_float time, rr_float) { return std::to_string(time); }

namespace {

std::string g_dir;

template <typename T>
std::vector<T> read_array(const std::string& name, size_t count) {
    std::vector<T> out(count);
    std::ifstream f(g_dir + "/" + name, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + name);
    f.read(reinterpret_cast<char*>(out.data()), count * sizeof(T));
    if ((size_t)f.gcount() != count * sizeof(T)) throw std::runtime_error("short read " + name);
    return out;
}
template <typename T>
void write_array(const std::string& name, const T* data, size_t count) {
    std::ofstream f(g_dir + "/" + name, std::ios::binary);
    f.write(reinterpret_cast<const char*>(data), count * sizeof(T));
}

void load_params() {
    std::map<std::string, std::function<void(double)>> set = {
#define F(name) {#name, [](double x) { params.name = (decltype(params.name))x; }}
        F(dim), F(ntotal), F(nfluid), F(nvirt), F(x_mingeom), F(x_maxgeom), F(y_mingeom),
        F(y_maxgeom), F(z_mingeom), F(z_maxgeom), F(delta), F(rho0), F(depth),
        F(nwm_particles_start), F(nwm_particles_end), F(density_treatment), F(density_skf),
        F(density_delta_sph_coef), F(eos_sound_vel_method), F(eos_sound_vel),
        F(eos_sound_vel_coef), F(intf_hsml_coef), F(intf_sph_approximation), F(intf_skf),
        F(artificial_pressure), F(artificial_pressure_skf), F(artificial_pressure_index),
        F(artificial_pressure_coef), F(artificial_viscosity), F(artificial_shear_visc),
        F(artificial_bulk_visc), F(artificial_viscosity_skf), F(average_velocity),
        F(average_velocity_coef), F(average_velocity_skf), F(consistency_check),
        F(consistency_treatment), F(boundary_treatment), F(nwm), F(nwm_direction),
        F(nwm_time_start), F(nwm_wave_length), F(nwm_wave_magnitude), F(nwm_phase),
        F(simulation_time), F(dt_correction_method), F(dt), F(CFL_coef), F(max_neighbours),
        F(local_threads), F(start_simulation_time), F(hsml), F(mass), F(cell_scale_k), F(maxn),
        F(max_cells), F(nwm_wave_number), F(nwm_freq), F(nwm_piston_magnitude),
#undef F
    };
    std::ifstream f(g_dir + "/params.txt");
    if (!f) throw std::runtime_error("cannot open params.txt");
    std::string key;
    std::string value;
    while (f >> key >> value) {
        auto it = set.find(key);
        if (it != set.end()) it->second(std::strtod(value.c_str(), nullptr));
    }
}

struct State {
    vheap_darray_floatn r, v;
    heap_darray<rr_float> rho, p;
    heap_darray<rr_int> itype;
};

State load_state() {
    const size_t n = params.ntotal, dim = params.dim, maxn = params.maxn;
    vheap_darray_floatn::set_dimenstions(dim);
    vheap_darray_floatn_md::set_dimenstions(dim);
    State s{vheap_darray_floatn(maxn), vheap_darray_floatn(maxn), heap_darray<rr_float>(maxn),
            heap_darray<rr_float>(maxn), heap_darray<rr_int>(maxn)};
    auto r = read_array<double>("r.f64", n * dim);
    auto v = read_array<double>("v.f64", n * dim);
    auto rho = read_array<double>("rho.f64", n);
    auto p = read_array<double>("p.f64", n);
    auto it = read_array<int32_t>("itype.i32", n);
    for (size_t i = 0; i < n; i++) {
        if (dim == 3) {
            auto& R = s.r.get_flt3();
            auto& V = s.v.get_flt3();
            R(i).x = r[i * 3]; R(i).y = r[i * 3 + 1]; R(i).z = r[i * 3 + 2];
            V(i).x = v[i * 3]; V(i).y = v[i * 3 + 1]; V(i).z = v[i * 3 + 2];
        } else {
            auto& R = s.r.get_flt2();
            auto& V = s.v.get_flt2();
            R(i).x = r[i * 2]; R(i).y = r[i * 2 + 1];
            V(i).x = v[i * 2]; V(i).y = v[i * 2 + 1];
        }
        s.rho(i) = rho[i];
        s.p(i) = p[i];
        s.itype(i) = it[i];
    }
    return s;
}

std::vector<double> flat(const vheap_darray_floatn& a) {
    const size_t n = params.ntotal, dim = params.dim;
    std::vector<double> out(n * dim);
    for (size_t i = 0; i < n; i++) {
        if (dim == 3) {
            const auto& A = a.get_flt3();
            out[i * 3] = A(i).x; out[i * 3 + 1] = A(i).y; out[i * 3 + 2] = A(i).z;
        } else {
            const auto& A = a.get_flt2();
            out[i * 2] = A(i).x; out[i * 2 + 1] = A(i).y;
        }
    }
    return out;
}

void write_neighbours(const heap_darray_md<rr_uint>& nb) {
    const size_t n = params.ntotal;
    std::vector<uint32_t> counts(n), list;
    for (size_t j = 0; j < n; j++) {
        size_t k = 0;
        for (; k < params.max_neighbours; k++) {
            rr_uint i = nb(k, j);
            if (i == params.ntotal) break;
            list.push_back((uint32_t)i);
        }
        counts[j] = (uint32_t)k;
    }
    write_array("counts.u32", counts.data(), n);
    write_array("list.u32", list.data(), list.size());
}

template <typename F2, typename F3>
void for_pairs(const State& s, const heap_darray_md<rr_uint>& nb, F2 f2, F3 f3) {
    const rr_iter n = (rr_iter)params.ntotal;
#pragma omp parallel for
    for (rr_iter j = 0; j < n; j++) {
        for (rr_iter k = 0;; k++) {
            rr_uint i = nb(k, j);
            if (i == params.ntotal) break;
            if (params.dim == 3) f3((rr_uint)j, i);
            else f2((rr_uint)j, i);
        }
    }
}

// Per-term sums as in testExternalForceOMP.cpp:30-52, testInternalForceOMP.cpp:48-80,
// testArtificialViscosityOMP.cpp:38-60, testAverageVelocityOMP.cpp:40-62 (all j).
template <typename V, typename GetR, typename GetV>
void terms_impl(const State& s, const heap_darray_md<rr_uint>& nb, unsigned mask, GetR R,
                GetV Vv, heap_darray<V>& a, heap_darray<V>& av, heap_darray<rr_float>& mu) {
    const rr_iter n = (rr_iter)params.ntotal;
#pragma omp parallel for
    for (rr_iter jj = 0; jj < n; jj++) {
        const rr_uint j = (rr_uint)jj;
        V acc = 0.;
        if (mask & 1u) acc.y = -params.g;
        V avt = 0.;
        rr_float arvmu = 0;
        for (rr_iter k = 0;; k++) {
            rr_uint i = nb(k, j);
            if (i == params.ntotal) break;
            V diff_ij = R(i) - R(j);
            rr_float dist_ij = length(diff_ij);
            if (mask & 2u) acc += external_force_part(dist_ij, R(j), R(i), s.itype(j), s.itype(i));
            if (mask & 4u)
                acc += find_internal_changes_part(diff_ij, dist_ij, s.p(j), s.p(i), s.rho(j), s.rho(i));
            if (mask & 8u)
                acc += artificial_viscosity_part(R(j), R(i), Vv(j), Vv(i), s.rho(j), s.rho(i), &arvmu);
            if (mask & 16u)
                avt += average_velocity_part(dist_ij, s.itype(i), Vv(j), Vv(i), s.rho(j), s.rho(i));
        }
        a(j) = acc;
        av(j) = avt;
        mu(j) = arvmu;
    }
}

void mode_terms(State& s, unsigned mask) {
    heap_darray_md<rr_uint> nb(params.max_neighbours, params.maxn);
    grid_find(s.r, s.itype, nb);
    heap_darray<rr_float> mu(params.maxn);
    const size_t n = params.ntotal, dim = params.dim;
    std::vector<double> a_out(n * dim), av_out(n * dim);
    if (dim == 3) {
        const auto& R = s.r.get_flt3();
        const auto& Vv = s.v.get_flt3();
        heap_darray<rr_float3> a(params.maxn), av(params.maxn);
        terms_impl(s, nb, mask, [&](rr_uint i) { return R(i); }, [&](rr_uint i) { return Vv(i); }, a, av, mu);
        for (size_t i = 0; i < n; i++) {
            a_out[i * 3] = a(i).x; a_out[i * 3 + 1] = a(i).y; a_out[i * 3 + 2] = a(i).z;
            av_out[i * 3] = av(i).x; av_out[i * 3 + 1] = av(i).y; av_out[i * 3 + 2] = av(i).z;
        }
    } else {
        const auto& R = s.r.get_flt2();
        const auto& Vv = s.v.get_flt2();
        heap_darray<rr_float2> a(params.maxn), av(params.maxn);
        terms_impl(s, nb, mask, [&](rr_uint i) { return R(i); }, [&](rr_uint i) { return Vv(i); }, a, av, mu);
        for (size_t i = 0; i < n; i++) {
            a_out[i * 2] = a(i).x; a_out[i * 2 + 1] = a(i).y;
            av_out[i * 2] = av(i).x; av_out[i * 2 + 1] = av(i).y;
        }
    }
    write_array("a.f64", a_out.data(), a_out.size());
    write_array("av.f64", av_out.data(), av_out.size());
    write_array("mu.f64", &mu(0), n);
}

// HeightTesting::maxInLayer (tools/WaterProfile/include/HeightTesting.h:25-54): the
// largest y over the particles (of type `type_filter` when it is non-zero) with
// |x - x_gauge| < search_n * hsml; 0 when none is near.
double gauge_max_in_layer(const State& s, double x_gauge, double search_n, int type_filter) {
    const double radius = search_n * params.hsml;
    const auto& r = s.r.get_flt2();
    double best = 0;
    for (size_t i = 0; i < params.ntotal; i++) {
        if (type_filter && s.itype(i) != type_filter) continue;
        if (std::fabs(r(i).x - x_gauge) < radius) best = std::max(best, r(i).y);
    }
    return best;
}

struct GaugeSpec {
    unsigned long every = 0;
    double search_n = 3;
    int type_filter = 0;
    std::vector<double> xs;
};

GaugeSpec load_gauges() {
    GaugeSpec g;
    std::ifstream f(g_dir + "/gauges.txt");
    if (!f) return g;
    f >> g.every >> g.search_n >> g.type_filter;
    double x;
    while (f >> x) g.xs.push_back(x);
    if (params.dim != 2) throw std::runtime_error("gauges: 2D only");
    return g;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <case_dir> <mode> [threads]\n", argv[0]);
        return 2;
    }
    g_dir = argv[1];
    const std::string mode = argv[2];
    try {
        load_params();
#ifdef _OPENMP
        int threads = argc > 3 ? std::atoi(argv[3]) : (int)params.local_threads;
        if (threads > 0) omp_set_num_threads(threads);
#endif
        State s = load_state();
        const size_t n = params.ntotal;

        if (mode == "grid") {
            heap_darray<rr_uint> grid(params.maxn), cells(params.max_cells);
            std::vector<uint32_t> keys(n);
            for (size_t i = 0; i < n; i++) {
                keys[i] = (uint32_t)(params.dim == 3 ? get_cell_idx3(s.r.get_flt3()(i))
                                                     : get_cell_idx2(s.r.get_flt2()(i)));
            }
            make_grid(s.r, grid, cells);
            std::vector<uint32_t> g(n), cs(params.max_cells + 1);
            for (size_t i = 0; i < n; i++) g[i] = (uint32_t)grid(i);
            for (size_t c = 0; c < params.max_cells; c++) cs[c] = (uint32_t)cells(c);
            cs[params.max_cells] = (uint32_t)n;
            heap_darray_md<rr_uint> nb(params.max_neighbours, params.maxn);
            find_neighbours(s.r, s.itype, grid, cells, nb);
            write_array("keys.u32", keys.data(), n);
            write_array("grid.u32", g.data(), n);
            write_array("cells_start.u32", cs.data(), cs.size());
            write_neighbours(nb);
        } else if (mode == "density") {
            heap_darray_md<rr_uint> nb(params.max_neighbours, params.maxn);
            grid_find(s.r, s.itype, nb);
            heap_darray<rr_float> out(params.maxn), p(params.maxn);
            if (density_is_using_continuity()) density_con(s.r, s.v, nb, s.rho, out, p);
            else density_sum(s.r, nb, out, p);
            write_array("density.f64", &out(0), n);
            write_array("pout.f64", &p(0), n);
        } else if (mode.rfind("terms:", 0) == 0) {
            mode_terms(s, (unsigned)std::strtoul(mode.c_str() + 6, nullptr, 0));
        } else if (mode == "accel") {
            heap_darray_md<rr_uint> nb(params.max_neighbours, params.maxn);
            grid_find(s.r, s.itype, nb);
            vheap_darray_floatn a(params.maxn), av(params.maxn);
            heap_darray<rr_float> drho(params.maxn);
            update_acceleration(s.itype, s.r, s.v, nb, s.rho, s.p, a, drho, av);
            auto fa = flat(a);
            write_array("a.f64", fa.data(), fa.size());
        } else if (mode.rfind("run:", 0) == 0) {
            const unsigned long nsteps = std::strtoul(mode.c_str() + 4, nullptr, 10);
            const bool cont = density_is_using_continuity();
            heap_darray<rr_float> rho_predict(params.maxn), drho(params.maxn);
            vheap_darray_floatn v_predict(params.maxn), a(params.maxn), av(params.maxn);
            heap_darray_md<rr_uint> nb(params.max_neighbours, params.maxn);
            rr_float time = params.start_simulation_time;
            double t_predict = 0, t_grid = 0, t_density = 0, t_accel = 0, t_whole = 0, t_aside = 0;
            const GaugeSpec gs = load_gauges();
            std::vector<double> gauges;
            auto sample = [&]() {
                for (double x : gs.xs) gauges.push_back(gauge_max_in_layer(s, x, gs.search_n, gs.type_filter));
            };
            std::vector<uint64_t> pairs(nsteps);
            std::vector<double> step_ms(nsteps);
            std::vector<double> phase_ms(5 * nsteps);  // per step: predict, grid, density, accel, whole
            if (gs.every) sample();
            auto t_all = std::chrono::steady_clock::now();
            for (unsigned long step = 0; step < nsteps; step++) {
                const double phases_before = t_predict + t_grid + t_density + t_accel + t_whole;
                const double before[5] = {t_predict, t_grid, t_density, t_accel, t_whole};
                auto t0 = std::chrono::steady_clock::now();
                predict_half_step(s.itype, s.rho, drho, s.v, a, rho_predict, v_predict);
                t_predict += ms_since(t0);
                t0 = std::chrono::steady_clock::now();
                grid_find(s.r, s.itype, nb);
                t_grid += ms_since(t0);
                t0 = std::chrono::steady_clock::now();
                {
                    uint64_t cnt = 0;
                    const rr_iter nn = (rr_iter)params.ntotal;
#pragma omp parallel for reduction(+ : cnt)
                    for (rr_iter j = 0; j < nn; j++) {
                        for (rr_iter k = 0; nb(k, j) != params.ntotal; k++) cnt++;
                    }
                    pairs[step] = cnt;
                }
                t_aside += ms_since(t0);
                t0 = std::chrono::steady_clock::now();
                if (cont) density_con(s.r, s.v, nb, s.rho, drho, s.p);
                else density_sum(s.r, nb, s.rho, s.p);
                t_density += ms_since(t0);
                t0 = std::chrono::steady_clock::now();
                update_acceleration(s.itype, s.r, v_predict, nb, cont ? rho_predict : s.rho, s.p, a,
                                    drho, av);
                t_accel += ms_since(t0);
                t0 = std::chrono::steady_clock::now();
                if (params.nwm && time >= params.nwm_time_start && params.dim == 2) {
                    make_waves(s.r.get_flt2(), s.v.get_flt2(), a.get_flt2(), s.itype, params.nfluid,
                               params.ntotal, time);
                }
                whole_step(step, drho, a, av, s.itype, s.rho, s.v, s.r);
                t_whole += ms_since(t0);
                step_ms[step] = t_predict + t_grid + t_density + t_accel + t_whole - phases_before;
                const double after[5] = {t_predict, t_grid, t_density, t_accel, t_whole};
                for (int q = 0; q < 5; q++) phase_ms[5 * step + q] = after[q] - before[q];
                time += params.dt;
                if (gs.every && (step + 1) % gs.every == 0) {
                    t0 = std::chrono::steady_clock::now();
                    sample();
                    t_aside += ms_since(t0);
                }
            }
            const double total = ms_since(t_all) - t_aside;
            write_array("pairs.u64", pairs.data(), pairs.size());
            write_array("step_ms.f64", step_ms.data(), step_ms.size());
            write_array("phase_ms.f64", phase_ms.data(), phase_ms.size());
            if (gs.every) write_array("gauges.f64", gauges.data(), gauges.size());
            auto fr = flat(s.r), fv = flat(s.v), fa = flat(a);
            write_array("r_out.f64", fr.data(), fr.size());
            write_array("v_out.f64", fv.data(), fv.size());
            write_array("a_out.f64", fa.data(), fa.size());
            write_array("rho_out.f64", &s.rho(0), n);
            write_array("p_out.f64", &s.p(0), n);
            std::vector<int32_t> it(n);
            for (size_t i = 0; i < n; i++) it[i] = (int32_t)s.itype(i);
            write_array("itype_out.i32", it.data(), n);
            std::ofstream t(g_dir + "/timing.txt");
            t << std::setprecision(17);
            int threads_used = 1;
#ifdef _OPENMP
            threads_used = omp_get_max_threads();
#endif
            t << "total_ms " << total << "\npredict_ms " << t_predict << "\ngrid_ms " << t_grid
              << "\ndensity_ms " << t_density << "\naccel_ms " << t_accel << "\nwhole_ms "
              << t_whole << "\nsteps " << nsteps << "\ntime " << time << "\nthreads "
              << threads_used << "\n";
        } else {
            std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
            return 2;
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "reference error: %s\n", e.what());
        return 1;
    }
    return 0;
}
