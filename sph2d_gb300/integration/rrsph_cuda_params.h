// rrsph_cuda_params.h — part of the RRSPH_CUDA backend, the binding that the
// reference's build adds beside RRSPH_OMP and RRSPH_CL (compiled against the
// reference's headers, linked with librrsph_cuda.so).
//
// fill_rrsph_params_from copies the global ExperimentParams that the
// reference's fileInput fills (sources/RRSPH_PARAMS/include/Params.h:8-196,
// Input.cpp:238-331) into the POD rrsph_params of the C ABI
// (include/rrsph_cuda.h): the loaded fields, the method switches and the
// values fileInput derives (hsml, mass, maxn, max_cells, cell_scale_k, the
// speed of sound, dt, the piston's wave number, frequency and stroke).
#pragma once

#include "Params.h"
#include "rrsph_cuda.h"

// p must come from rrsph_params_defaults (struct_size set); fields without a
// counterpart in ExperimentParams keep their defaults (dt_dynamic_reduce = 0:
// the OpenMP build's dt). Returns RRSPH_OK, or RRSPH_ERR_INVALID_ARGUMENT for
// a null or uninitialised p.
int fill_rrsph_params_from(const ExperimentParams& e, rrsph_params* p);
