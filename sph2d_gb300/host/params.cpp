// params.cpp — experiment parameters for the C ABI: defaults, the JSON files of
// an experiment directory, and the values fileInput() derives from them.
//
// Mirrors, in this library's own code:
//   ExperimentParams defaults        sources/RRSPH_PARAMS/include/Params.h:8-196
//   ModelParams defaults / loading   sources/RRSPH_PARAMS/include/ModelParams.h:11-78,
//                                    sources/RRSPH_PARAMS/src/ModelParams.cpp:12-311
//   ParticleParams loading           sources/RRSPH_PARAMS/src/ParticleParams.cpp:51-149
//   fillInComputingParams et al.     sources/RRSPH_COMMON/src/Input.cpp:17-138, 238-331
#include "../../include/rrsph_cuda.h"
#include "error.hpp"
#include "json_lite.hpp"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

namespace rrsph {

static thread_local std::string g_last_error = "no error";

int set_error(int code, const std::string& msg) {
    if (code != RRSPH_OK) g_last_error = msg;
    return code;
}

}  // namespace rrsph

using rrsph::set_error;

extern "C" int rrsph_abi_version(void) { return RRSPH_ABI_VERSION; }
extern "C" size_t rrsph_params_sizeof(void) { return sizeof(rrsph_params); }
extern "C" const char* rrsph_last_error(void) { return rrsph::g_last_error.c_str(); }

extern "C" int rrsph_params_offsetof(const char* field, size_t* offset) {
    if (!field || !offset) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_params_offsetof: null argument");
#define RRSPH_FIELD(name)                          \
    if (std::strcmp(field, #name) == 0) {          \
        *offset = offsetof(rrsph_params, name);    \
        return RRSPH_OK;                           \
    }
#include "params_fields.def"
#undef RRSPH_FIELD
    return set_error(RRSPH_ERR_INVALID_ARGUMENT, std::string("rrsph_params_offsetof: unknown field ") + field);
}

extern "C" int rrsph_params_defaults(rrsph_params* p) {
    if (!p) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_params_defaults: null params");
    std::memset(p, 0, sizeof(*p));
    p->struct_size = (uint32_t)sizeof(rrsph_params);
    p->dim = 2;
    p->rho0 = 1000;
    // ModelParams member initialisers (ModelParams.h:17-77); optionals without
    // a value resolve to 0 through value_or(T{}) (ModelParams.cpp:117-120).
    p->density_treatment = 1;        // DENSITY_CONTINUITY
    p->density_skf = 1;
    p->intf_hsml_coef = 1;
    p->intf_sph_approximation = 2;
    p->intf_skf = 1;
    p->artificial_pressure = 0;
    p->artificial_pressure_skf = 1;
    p->artificial_pressure_index = 4;
    p->artificial_pressure_coef = 0.2;
    p->artificial_viscosity = 0;
    p->artificial_viscosity_skf = 1;
    p->average_velocity = 0;
    p->average_velocity_skf = 1;
    p->use_crash_dump = 1;
    p->consistency_check = 1;
    p->consistency_treatment = 1;    // CONSISTENCY_STOP
    p->nwm = 0;
    p->dt_correction_method = 2;     // DT_CORRECTION_DYNAMIC
    p->dt_dynamic_reduce = 0;
    p->max_neighbours = 64;
    p->save_velocity = 1;
    p->save_pressure = 1;
    p->save_density = 1;
    // ExperimentParams values fileInput() uses before it sets them (Params.h)
    p->cell_scale_k = 2;
    p->eos_sound_vel_coef = 0;
    p->local_threads = 0;
    p->pi = 3.14159265358979323846;
    p->g = 9.81;
    p->type_boundary = -2;
    p->type_non_existent = 0;
    p->type_water = 2;
    return RRSPH_OK;
}

namespace {

bool read_file(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

struct Loader {
    const rrsph::JsonObject& js;
    std::string missing;
    // load(param): mandatory (ModelParams.cpp:240-245)
    bool mandatory(const char* k, double& dst) {
        if (!js.contains(k)) { missing = k; return false; }
        dst = js.number(k);
        return true;
    }
    template <typename T>
    bool mandatory_u(const char* k, T& dst) {
        double d;
        if (!mandatory(k, d)) return false;
        dst = (T)d;
        return true;
    }
    // load_default / load_optional: keep the current value when absent
    void opt(const char* k, double& dst) { if (js.contains(k)) dst = js.number(k); }
    template <typename T>
    void opt_u(const char* k, T& dst) { if (js.contains(k)) dst = (T)js.number(k); }
};

}  // namespace

extern "C" int rrsph_experiment_load_params(const char* experiment_dir, rrsph_params* p) {
    if (!experiment_dir || !p) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_experiment_load_params: null argument");
    if (p->struct_size != sizeof(rrsph_params))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_experiment_load_params: params not initialised by rrsph_params_defaults");
    const std::string dir(experiment_dir);
    std::string text;
    try {
        // ---- ParticleParams.json (ParticleParams.cpp:51-149)
        if (!read_file(dir + "/ParticleParams.json", text))
            return set_error(RRSPH_ERR_IO, "No params file provided: '" + dir + "/ParticleParams.json' expected");
        {
            const auto js = rrsph::JsonObject::parse(text);
            Loader L{js, {}};
            L.opt_u("dim", p->dim);
            bool ok = L.mandatory("x_mingeom", p->x_mingeom) && L.mandatory("x_maxgeom", p->x_maxgeom) &&
                      L.mandatory("y_mingeom", p->y_mingeom) && L.mandatory("y_maxgeom", p->y_maxgeom);
            if (ok && p->dim == 3) ok = L.mandatory("z_mingeom", p->z_mingeom) && L.mandatory("z_maxgeom", p->z_maxgeom);
            if (ok && p->dim != 3) { p->z_mingeom = 0; p->z_maxgeom = 0; }
            ok = ok && L.mandatory("delta", p->delta) && L.mandatory_u("ntotal", p->ntotal) &&
                 L.mandatory_u("nfluid", p->nfluid) && L.mandatory_u("nvirt", p->nvirt);
            if (!ok) return set_error(RRSPH_ERR_PARSE, "Mandatory param not specified: " + L.missing);
            p->rho0 = 1000;
            L.opt("rho0", p->rho0);
            p->nwm_particles_start = p->ntotal;
            p->nwm_particles_end = p->ntotal;
            L.opt_u("nwm_particles_start", p->nwm_particles_start);
            L.opt_u("nwm_particles_end", p->nwm_particles_end);
            p->depth = 0;
            L.opt("depth", p->depth);
            if (p->dim != 2 && p->dim != 3) return set_error(RRSPH_ERR_PARSE, "invalid params.dim value: " + std::to_string(p->dim));
        }
        // ---- ModelParams.json (ModelParams.cpp:185-311)
        if (!read_file(dir + "/ModelParams.json", text))
            return set_error(RRSPH_ERR_IO, "No params file provided: '" + dir + "/ModelParams.json' expected");
        {
            const auto js = rrsph::JsonObject::parse(text);
            Loader L{js, {}};
            double ver[3] = {0, 0, 0};
            L.opt("params_target_version_major", ver[0]);
            L.opt("params_target_version_minor", ver[1]);
            L.opt("params_target_version_patch", ver[2]);
            // target < current (3.1.4) as the reference's ParamsVersion::operator< has it
            // (RRSPH_PARAMS/src/Version.h:17-21): every component compared on its own
            // (major <= 3, minor <= 1, patch < 4), not lexicographically
            const bool old = ver[0] <= 3 && ver[1] <= 1 && ver[2] < 4;

            L.opt_u("density_treatment", p->density_treatment);
            uint32_t density_normalization = 0;
            L.opt_u("density_normalization", density_normalization);
            L.opt_u("density_skf", p->density_skf);
            L.opt("density_delta_sph_coef", p->density_delta_sph_coef);
            if (!L.mandatory_u("eos_sound_vel_method", p->eos_sound_vel_method))
                return set_error(RRSPH_ERR_PARSE, "Mandatory param not specified: eos_sound_vel_method");
            const bool has_eos_vel = js.contains("eos_sound_vel"), has_eos_coef = js.contains("eos_sound_vel_coef");
            L.opt("eos_sound_vel", p->eos_sound_vel);
            L.opt("eos_sound_vel_coef", p->eos_sound_vel_coef);
            L.opt("intf_hsml_coef", p->intf_hsml_coef);
            L.opt_u("intf_sph_approximation", p->intf_sph_approximation);
            L.opt_u("intf_skf", p->intf_skf);
            L.opt_u("artificial_pressure", p->artificial_pressure);
            L.opt_u("artificial_pressure_skf", p->artificial_pressure_skf);
            L.opt("artificial_pressure_index", p->artificial_pressure_index);
            L.opt("artificial_pressure_coef", p->artificial_pressure_coef);
            uint32_t visc = 1;
            L.opt_u("visc", visc);
            L.opt_u("artificial_viscosity", p->artificial_viscosity);
            const bool has_shear = js.contains("artificial_shear_visc"), has_bulk = js.contains("artificial_bulk_visc");
            L.opt("artificial_shear_visc", p->artificial_shear_visc);
            L.opt("artificial_bulk_visc", p->artificial_bulk_visc);
            L.opt_u("artificial_viscosity_skf", p->artificial_viscosity_skf);
            L.opt_u("average_velocity", p->average_velocity);
            const bool has_avc = js.contains("average_velocity_coef");
            L.opt("average_velocity_coef", p->average_velocity_coef);
            L.opt_u("average_velocity_skf", p->average_velocity_skf);
            L.opt_u("save_every_step", p->save_every_step);
            if (!L.mandatory("save_time", p->save_time))
                return set_error(RRSPH_ERR_PARSE, "Mandatory param not specified: save_time");
            const bool has_dump_time = js.contains("dump_time");
            L.opt("dump_time", p->dump_time);
            L.opt_u("use_dump", p->use_dump);
            L.opt_u("use_crash_dump", p->use_crash_dump);
            L.opt_u("consistency_check", p->consistency_check);
            L.opt_u("consistency_treatment", p->consistency_treatment);
            if (!L.mandatory_u("boundary_treatment", p->boundary_treatment))
                return set_error(RRSPH_ERR_PARSE, "Mandatory param not specified: boundary_treatment");
            L.opt_u("nwm", p->nwm);
            L.opt("nwm_time_start", p->nwm_time_start);
            const bool has_wl = js.contains("nwm_wave_length"), has_wm = js.contains("nwm_wave_magnitude");
            L.opt("nwm_wave_length", p->nwm_wave_length);
            L.opt("nwm_wave_magnitude", p->nwm_wave_magnitude);
            bool has_dir = js.contains("nwm_direction");
            L.opt_u("nwm_direction", p->nwm_direction);
            if (old) { p->nwm_direction = 1; has_dir = true; } // backward_compatibility_model_params (:162-167)
            L.opt("nwm_phase", p->nwm_phase);
            if (!L.mandatory("simulation_time", p->simulation_time))
                return set_error(RRSPH_ERR_PARSE, "Mandatory param not specified: simulation_time");
            L.opt_u("dt_correction_method", p->dt_correction_method);
            const bool has_dt = js.contains("dt"), has_cfl = js.contains("CFL_coef");
            L.opt("dt", p->dt);
            L.opt("CFL_coef", p->CFL_coef);
            L.opt_u("max_neighbours", p->max_neighbours);
            L.opt_u("local_threads", p->local_threads);
            L.opt_u("save_velocity", p->save_velocity);
            L.opt_u("save_pressure", p->save_pressure);
            L.opt_u("save_density", p->save_density);
            L.opt_u("dt_dynamic_reduce", p->dt_dynamic_reduce);

            // check_optional_params (ModelParams.cpp:12-95)
            if (visc) return set_error(RRSPH_ERR_UNSUPPORTED, "Not implemented: visc");
            if (density_normalization) return set_error(RRSPH_ERR_UNSUPPORTED, "Not implemented: density_normalization");
            if (p->eos_sound_vel_method == 1 && !has_eos_vel) return set_error(RRSPH_ERR_PARSE, "Need optional param: eos_sound_vel");
            if (p->eos_sound_vel_method == 0 && !has_eos_coef) return set_error(RRSPH_ERR_PARSE, "Need optional param: eos_sound_vel_coef");
            if (p->eos_sound_vel_method > 1) return set_error(RRSPH_ERR_PARSE, "Invalid enum value: eos_sound_vel_method");
            if (p->density_treatment == 2 && !js.contains("density_delta_sph_coef"))
                return set_error(RRSPH_ERR_PARSE, "Need optional param: density_delta_sph_coef");
            if (p->artificial_viscosity && (!has_shear || !has_bulk))
                return set_error(RRSPH_ERR_PARSE, std::string("Need optional param: ") + (!has_shear ? "artificial_shear_visc" : "artificial_bulk_visc"));
            if (p->average_velocity && !has_avc) return set_error(RRSPH_ERR_PARSE, "Need optional param: average_velocity_coef");
            if (p->use_dump && !has_dump_time) return set_error(RRSPH_ERR_PARSE, "Need optional param: dump_time");
            switch (p->nwm) {
            case 0: case 4: break;
            case 2: case 3:
                if (!has_wl) return set_error(RRSPH_ERR_PARSE, "Need optional param: nwm_wave_length");
                if (!has_wm) return set_error(RRSPH_ERR_PARSE, "Need optional param: nwm_wave_magnitude");
                if (!has_dir) return set_error(RRSPH_ERR_PARSE, "Need optional param: nwm_direction");
                break;
            case 5:
                if (!has_wm) return set_error(RRSPH_ERR_PARSE, "Need optional param: nwm_wave_magnitude");
                break;
            default: return set_error(RRSPH_ERR_PARSE, "Invalid enum value: nwm");
            }
            switch (p->dt_correction_method) {
            case 0: if (!has_dt) return set_error(RRSPH_ERR_PARSE, "Need optional param: dt"); break;
            case 1: case 2: if (!has_cfl) return set_error(RRSPH_ERR_PARSE, "Need optional param: CFL_coef"); break;
            default: return set_error(RRSPH_ERR_PARSE, "Invalid enum value: dt_correction_method");
            }
        }
    } catch (const std::exception& e) {
        return set_error(RRSPH_ERR_PARSE, std::string("params json: ") + e.what());
    }
    return RRSPH_OK;
}

namespace {

uint64_t intlog2(uint64_t v) { // CommonIncl.h:69-77
    uint64_t passes = 0;
    while (v > 1) { v >>= 1; ++passes; }
    return passes;
}
uint64_t split2(uint64_t x) {
    x = (x | x << 16) & 0x0000FFFFull;
    x = (x | x << 8) & 0x00FF00FFull;
    x = (x | x << 4) & 0x0F0F0F0Full;
    x = (x | x << 2) & 0x33333333ull;
    x = (x | x << 1) & 0x55555555ull;
    return x;
}
uint64_t split3(uint64_t a) {
    uint64_t x = a & 0x000003ffull;
    x = (x | x << 16) & 0x30000ffull;
    x = (x | x << 8) & 0x0300f00full;
    x = (x | x << 4) & 0x30c30c3ull;
    x = (x | x << 2) & 0x9249249ull;
    return x;
}
uint64_t coord(double r, double rmin, double cell) {
    const double c = (r - rmin) / cell;
    return c > 0 ? (uint64_t)c : 0;
}
int cell_scale_of(uint32_t skf, double* k) { // Input.cpp:17-26
    switch (skf) {
    case 1: *k = 2; return 0;
    case 2: *k = 3; return 0;
    case 3: *k = 2; return 0;
    case 4: *k = 2; return 0;
    default: return -1;
    }
}

}  // namespace

extern "C" int rrsph_params_derive(rrsph_params* p, const double* r, uint32_t stride) {
    if (!p) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_params_derive: null params");
    if (p->struct_size != sizeof(rrsph_params))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_params_derive: params not initialised by rrsph_params_defaults");
    if (p->dim != 2 && p->dim != 3) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "invalid params.dim value: " + std::to_string(p->dim));
    if (p->ntotal == 0 || p->nfluid > p->ntotal) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_params_derive: bad particle counts");
    if (p->ntotal >= (1ull << 31)) return set_error(RRSPH_ERR_UNSUPPORTED, "rrsph_params_derive: ntotal must be < 2^31");
    if (p->nfluid > 0 && p->depth == 0 && (!r || stride < p->dim))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_params_derive: positions needed to find the depth");

    // fillInComputingParams (Input.cpp:93-110)
    p->hsml = p->delta * p->intf_hsml_coef;
    p->maxn = 1ull << (1 + intlog2(p->ntotal));
    {   // countCells (Input.cpp:45-75) runs before cell_scale_k is updated, so it
        // uses the value cell_scale_k held at that point (2 by default).
        const double cell = p->cell_scale_k * p->hsml;
        const uint64_t x_id = coord(p->x_maxgeom, p->x_mingeom, cell);
        const uint64_t y_id = coord(p->y_maxgeom, p->y_mingeom, cell);
        uint64_t z_id, max_id, id;
        if (p->dim == 3) {
            z_id = coord(p->z_maxgeom, p->z_mingeom, cell);
            max_id = 1ull << 10;
            id = split3(x_id) | (split3(y_id) << 1) | (split3(z_id) << 2);
        } else {
            z_id = 0;
            max_id = 1ull << 16;
            id = split2(x_id) | (split2(y_id) << 1);
        }
        if (x_id > max_id || y_id > max_id || z_id >= max_id) {
            return set_error(RRSPH_ERR_UNSUPPORTED,
                             "can't make grid with so many cells: (" + std::to_string(x_id) + "/" + std::to_string(max_id) + "; " +
                                 std::to_string(y_id) + "/" + std::to_string(max_id) + "; " + std::to_string(z_id) + "/" +
                                 std::to_string(max_id) + ")");
        }
        p->max_cells = 1ull << (intlog2(id) + 1);
    }
    {   // mass = rho0 * delta^dim (powun)
        double m = 1;
        for (uint32_t i = 0; i < p->dim; i++) m *= p->delta;
        p->mass = p->rho0 * m;
    }
    {   // get_cell_scale_k over all kernel choices must agree (Input.cpp:28-43)
        const uint32_t skfs[5] = {p->artificial_pressure_skf, p->artificial_viscosity_skf, p->average_velocity_skf,
                                  p->intf_skf, p->density_skf};
        double kmin = 1e300, kmax = -1e300;
        for (uint32_t s : skfs) {
            double k;
            if (cell_scale_of(s, &k)) return set_error(RRSPH_ERR_PARSE, "get_cell_scale_k: unknown skf " + std::to_string(s));
            kmin = std::fmin(kmin, k);
            kmax = std::fmax(kmax, k);
        }
        if (kmin != kmax) return set_error(RRSPH_ERR_UNSUPPORTED, "selected incompatible skf");
        p->cell_scale_k = kmax;
    }
    // find_depth (Input.cpp:77-91): only when depth is not given
    if (p->depth == 0) {
        double ymin = FLT_MAX, ymax = -FLT_MAX;
        for (uint64_t i = 0; i < p->nfluid; i++) {
            const double y = r[i * stride + 1];
            ymax = std::fmax(y, ymax);
            ymin = std::fmin(y, ymin);
        }
        p->depth = ymax - ymin;
    }
    // postFillInModelParams (Input.cpp:112-138)
    if (p->eos_sound_vel_method == 0) p->eos_sound_vel = std::sqrt(200 * p->g * p->depth * p->eos_sound_vel_coef);
    if (p->dt_correction_method == 1) {
        p->dt = p->CFL_coef * p->hsml / (p->eos_sound_vel * (1 + 1.2 * p->artificial_shear_visc));
    }
    if (p->nwm == 2 || p->nwm == 3) {
        p->nwm_wave_number = 2. * p->pi / p->nwm_wave_length;
        const double kd = p->nwm_wave_number * p->depth;
        p->nwm_freq = std::sqrt(p->nwm_wave_number * p->g * std::tanh(kd));
        p->nwm_piston_magnitude =
            p->nwm_wave_magnitude * 0.5 / (std::sinh(kd) * std::sinh(kd)) * (std::sinh(kd) * std::cosh(kd) + kd);
    }
    if (p->max_neighbours < 2) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "max_neighbours must be >= 2");
    return RRSPH_OK;
}
