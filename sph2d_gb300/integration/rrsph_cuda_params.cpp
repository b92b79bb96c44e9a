// rrsph_cuda_params.cpp — ExperimentParams (the reference's global params) to
// the C ABI's rrsph_params. Part of the RRSPH_CUDA backend; compiled with the
// reference's headers.
#include "rrsph_cuda_params.h"

int fill_rrsph_params_from(const ExperimentParams& e, rrsph_params* p) {
    if (!p || p->struct_size != sizeof(rrsph_params)) return RRSPH_ERR_INVALID_ARGUMENT;
    p->dim = (uint32_t)e.dim;
    // ParticleParams.json (apply_particle_params, ParticleParams.cpp:22-44)
    p->ntotal = e.ntotal;
    p->nfluid = e.nfluid;
    p->nvirt = e.nvirt;
    p->x_mingeom = e.x_mingeom;
    p->x_maxgeom = e.x_maxgeom;
    p->y_mingeom = e.y_mingeom;
    p->y_maxgeom = e.y_maxgeom;
    p->z_mingeom = e.z_mingeom;
    p->z_maxgeom = e.z_maxgeom;
    p->delta = e.delta;
    p->rho0 = e.rho0;
    p->depth = e.depth;
    p->nwm_particles_start = e.nwm_particles_start;
    p->nwm_particles_end = e.nwm_particles_end;
    // ModelParams.json (apply_model_params, ModelParams.cpp:110-173)
    p->density_treatment = (uint32_t)e.density_treatment;
    p->density_skf = (uint32_t)e.density_skf;
    p->density_delta_sph_coef = e.density_delta_sph_coef;
    p->eos_sound_vel_method = (uint32_t)e.eos_sound_vel_method;
    p->intf_sph_approximation = (uint32_t)e.intf_sph_approximation;
    p->eos_sound_vel = e.eos_sound_vel;
    p->eos_sound_vel_coef = e.eos_sound_vel_coef;
    p->intf_hsml_coef = e.intf_hsml_coef;
    p->intf_skf = (uint32_t)e.intf_skf;
    p->artificial_pressure = e.artificial_pressure ? 1u : 0u;
    p->artificial_pressure_skf = (uint32_t)e.artificial_pressure_skf;
    p->artificial_viscosity = e.artificial_viscosity ? 1u : 0u;
    p->artificial_pressure_index = e.artificial_pressure_index;
    p->artificial_pressure_coef = e.artificial_pressure_coef;
    p->artificial_shear_visc = e.artificial_shear_visc;
    p->artificial_bulk_visc = e.artificial_bulk_visc;
    p->artificial_viscosity_skf = (uint32_t)e.artificial_viscosity_skf;
    p->average_velocity = e.average_velocity ? 1u : 0u;
    p->average_velocity_coef = e.average_velocity_coef;
    p->average_velocity_skf = (uint32_t)e.average_velocity_skf;
    p->consistency_check = e.consistency_check ? 1u : 0u;
    p->consistency_treatment = (uint32_t)e.consistency_treatment;
    p->boundary_treatment = (uint32_t)e.boundary_treatment;
    p->nwm = (uint32_t)e.nwm;
    p->nwm_direction = (uint32_t)e.nwm_direction;
    p->nwm_time_start = e.nwm_time_start;
    p->nwm_wave_length = e.nwm_wave_length;
    p->nwm_wave_magnitude = e.nwm_wave_magnitude;
    p->nwm_phase = e.nwm_phase;
    p->simulation_time = e.simulation_time;
    p->dt_correction_method = (uint32_t)e.dt_correction_method;
    p->dt = e.dt;
    p->CFL_coef = e.CFL_coef;
    p->max_neighbours = (uint32_t)e.max_neighbours;
    p->local_threads = (uint32_t)e.local_threads;
    p->save_time = e.save_time;
    p->dump_time = e.dump_time;
    p->use_dump = e.use_dump ? 1u : 0u;
    p->save_every_step = e.save_every_step ? 1u : 0u;
    p->save_velocity = e.save_velocity ? 1u : 0u;
    p->save_pressure = e.save_pressure ? 1u : 0u;
    p->save_density = e.save_density ? 1u : 0u;
    p->use_crash_dump = e.use_crash_dump ? 1u : 0u;
    p->start_simulation_time = e.start_simulation_time;
    // derived by fileInput (fillInComputingParams, find_depth,
    // postFillInModelParams: Input.cpp:77-138)
    p->hsml = e.hsml;
    p->mass = e.mass;
    p->cell_scale_k = e.cell_scale_k;
    p->maxn = e.maxn;
    p->max_cells = e.max_cells;
    p->nwm_wave_number = e.nwm_wave_number;
    p->nwm_freq = e.nwm_freq;
    p->nwm_piston_magnitude = e.nwm_piston_magnitude;
    // constants (Params.h:176-193)
    p->pi = ExperimentParams::pi;
    p->g = ExperimentParams::g;
    p->type_boundary = ExperimentParams::TYPE_BOUNDARY;
    p->type_non_existent = ExperimentParams::TYPE_NON_EXISTENT;
    p->type_water = ExperimentParams::TYPE_WATER;
    return RRSPH_OK;
}
