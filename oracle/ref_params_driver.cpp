// ref_params_driver.cpp — checks the RRSPH_CUDA binding's parameter mapping
// (sph2d_gb300/integration/rrsph_cuda_params.cpp) with the reference's own
// parameter loaders (TEST INFRASTRUCTURE; built by oracle/build_ref.sh from
// the staged reference sources).
//
// Usage:
//   ref_params <experiment_dir>   the reference's load_particle_params +
//                                 load_model_params + apply_*_params
//                                 (ParticleParams.cpp:22-149, ModelParams.cpp:110-311)
//                                 on the experiment, then fill_rrsph_params_from;
//                                 prints every rrsph_params field as "name value"
//   ref_params --mapping          gives each ExperimentParams field that has a
//                                 counterpart a distinct value (each bool alone
//                                 set) and checks that fill_rrsph_params_from puts
//                                 it into the field of the same name; prints
//                                 "mapping ok" or the fields that differ
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "ModelParams.h"
#include "Params.h"
#include "ParticleParams.h"
#include "rrsph_cuda_params.h"

// the reference's loaders (declared in its ParamsIO.h, which also pulls in the
// experiment-directory tooling this driver does not build)
ParticleParams load_particle_params(const std::filesystem::path& experiment_directory);
void apply_particle_params(ExperimentParams& experiment_params, const ParticleParams& particle_params);
ModelParams load_model_params(const std::filesystem::path& experiment_directory);
void apply_model_params(ExperimentParams& experiment_params, const ModelParams& model_params);

namespace {

template <typename T>
void put(const char* name, T v) {
    if constexpr (std::is_floating_point_v<T>) std::printf("%s %.17g\n", name, (double)v);
    else if constexpr (std::is_signed_v<T>) std::printf("%s %lld\n", name, (long long)v);
    else std::printf("%s %llu\n", name, (unsigned long long)v);
}

rrsph_params fresh() {
    rrsph_params p;
    std::memset(&p, 0, sizeof(p));
    p.struct_size = (uint32_t)sizeof(rrsph_params);
    return p;
}

void print_all(const rrsph_params& p) {
#define RRSPH_FIELD(name) put(#name, p.name);
#include "params_fields.def"
#undef RRSPH_FIELD
}

// Fields of both structs with a numeric (non-bool) type in ExperimentParams.
#define NUMERIC_FIELDS(X)                                                                            \
    X(dim) X(ntotal) X(nfluid) X(nvirt) X(x_mingeom) X(x_maxgeom) X(y_mingeom) X(y_maxgeom)           \
    X(z_mingeom) X(z_maxgeom) X(delta) X(rho0) X(depth) X(nwm_particles_start) X(nwm_particles_end)   \
    X(density_treatment) X(density_skf) X(density_delta_sph_coef) X(eos_sound_vel_method)             \
    X(intf_sph_approximation) X(eos_sound_vel) X(eos_sound_vel_coef) X(intf_hsml_coef) X(intf_skf)    \
    X(artificial_pressure_skf) X(artificial_pressure_index) X(artificial_pressure_coef)               \
    X(artificial_shear_visc) X(artificial_bulk_visc) X(artificial_viscosity_skf)                      \
    X(average_velocity_coef) X(average_velocity_skf) X(consistency_treatment) X(boundary_treatment)   \
    X(nwm) X(nwm_direction) X(nwm_time_start) X(nwm_wave_length) X(nwm_wave_magnitude) X(nwm_phase)   \
    X(simulation_time) X(dt_correction_method) X(dt) X(CFL_coef) X(max_neighbours) X(local_threads)   \
    X(save_time) X(dump_time) X(start_simulation_time) X(hsml) X(mass) X(cell_scale_k) X(maxn)        \
    X(max_cells) X(nwm_wave_number) X(nwm_freq) X(nwm_piston_magnitude)
#define BOOL_FIELDS(X)                                                                               \
    X(artificial_pressure) X(artificial_viscosity) X(average_velocity) X(consistency_check) X(use_dump) \
    X(save_every_step) X(save_velocity) X(save_pressure) X(save_density) X(use_crash_dump)

int mapping() {
    std::vector<std::string> bad;
    ExperimentParams e;
    unsigned k = 0;
#define SET(name) e.name = (decltype(e.name))(3 + k++);
    NUMERIC_FIELDS(SET)
#undef SET
#define CLEAR(name) e.name = false;
    BOOL_FIELDS(CLEAR)
#undef CLEAR
    rrsph_params p = fresh();
    if (fill_rrsph_params_from(e, &p) != RRSPH_OK) bad.push_back("fill failed");
    k = 0;
#define CHECK(name)                                                                    \
    if ((double)p.name != (double)(decltype(e.name))(3 + k)) bad.push_back(#name);    \
    k++;
    NUMERIC_FIELDS(CHECK)
#undef CHECK
#define CHECK_OFF(name) if (p.name != 0) bad.push_back(#name " (off)");
    BOOL_FIELDS(CHECK_OFF)
#undef CHECK_OFF
    // each switch alone: exactly its own field turns on
#define ONE(name)                                                                      \
    {                                                                                  \
        ExperimentParams f = e;                                                        \
        f.name = true;                                                                 \
        rrsph_params q = fresh();                                                      \
        fill_rrsph_params_from(f, &q);                                                 \
        int on = q.artificial_pressure + q.artificial_viscosity + q.average_velocity +   \
                 q.consistency_check + q.use_dump + q.save_every_step + q.save_velocity + \
                 q.save_pressure + q.save_density + q.use_crash_dump;                  \
        if (q.name != 1 || on != 1) bad.push_back(#name " (on)");                      \
    }
    BOOL_FIELDS(ONE)
#undef ONE
    if (p.pi != ExperimentParams::pi || p.g != ExperimentParams::g || p.type_boundary != -2 ||
        p.type_non_existent != 0 || p.type_water != 2 || p.dt_dynamic_reduce != 0)
        bad.push_back("constants");
    rrsph_params u;
    std::memset(&u, 0, sizeof(u));
    if (fill_rrsph_params_from(e, &u) != RRSPH_ERR_INVALID_ARGUMENT) bad.push_back("uninitialised params accepted");
    if (bad.empty()) {
        std::printf("mapping ok\n");
        return 0;
    }
    for (const auto& b : bad) std::printf("mapping differs: %s\n", b.c_str());
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <experiment_dir> | --mapping\n", argv[0]);
        return 2;
    }
    try {
        if (std::string(argv[1]) == "--mapping") return mapping();
        ExperimentParams e;
        apply_particle_params(e, load_particle_params(argv[1]));
        apply_model_params(e, load_model_params(argv[1]));
        rrsph_params p = fresh();
        if (fill_rrsph_params_from(e, &p) != RRSPH_OK) throw std::runtime_error("fill_rrsph_params_from failed");
        print_all(p);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "reference error: %s\n", ex.what());
        return 1;
    }
    return 0;
}
