// TimeIntegration.cpp — the RRSPH_CUDA backend of the reference's time loop:
// time_integration with the signature of RRSPH_OMP/include/TimeIntegration.h:4-9,
// built inside the reference's tree (with its headers and RRSPH_COMMON for
// RRSPHOutput) and linked with librrsph_cuda.so. SPH.cpp selects it as it
// selects the OpenMP and OpenCL backends (SPH.cpp:1-10, 64-68).
//
// The reference's loop (TimeIntegration.cpp:21-102) allocates its work arrays,
// runs predict / grid / density / forces / whole step per step and hands the
// host arrays to RRSPHOutput::update_step after each step. Here the state lives
// on the GPU for the whole run: one rrsph_step_download per step (the loop
// body, with the piston call the OpenMP loop leaves commented out enabled, as
// the OpenCL backend has it, and the download into the caller's arrays) so that
// update_step writes its data and dump layers and runs its boundary check from
// host copies exactly as it does for RRSPH_OMP. A step whose device check
// fails still downloads first, so update_step writes the crash dump and throws
// the reference's own error.
//
// The precision is the FP32-mixed step unless RRSPH_CUDA_PRECISION=fp64.
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "CommonIncl.h"
#include "Output.h"
#include "TimeIntegration.h"
#include "rrsph_cuda_params.h"

namespace {

void ok(int rc) {
    if (rc != RRSPH_OK) throw std::runtime_error{rrsph_last_error()};
}

struct SolverHandle {
    rrsph_solver* s = nullptr;
    ~SolverHandle() {
        if (s) rrsph_destroy(s);
    }
};

int precision_from_env() {
    const char* v = std::getenv("RRSPH_CUDA_PRECISION");
    return v && std::string(v) == "fp64" ? RRSPH_PRECISION_FP64 : RRSPH_PRECISION_MIXED;
}

}  // namespace

void time_integration(vheap_darray_floatn& r_var, vheap_darray_floatn& v_var, heap_darray<rr_float>& rho,
                      heap_darray<rr_float>& p, heap_darray<rr_int>& itype) {
    rrsph_params prm;
    ok(rrsph_params_defaults(&prm));
    ok(fill_rrsph_params_from(params, &prm));

    // the caller's AoS arrays: rr_float2 is two doubles, rr_float3 four (a pad, RRFloat3.h:5)
    const bool d3 = params.dim == 3;
    double* r = d3 ? &r_var.get_flt3()(0).x : &r_var.get_flt2()(0).x;
    double* v = d3 ? &v_var.get_flt3()(0).x : &v_var.get_flt2()(0).x;
    const uint32_t stride = d3 ? 4u : 2u;
    const rr_uint n = params.ntotal;
    std::vector<int32_t> it(n);  // rr_int is 64-bit; the ABI takes int32
    for (rr_uint i = 0; i < n; ++i) it[i] = (int32_t)itype(i);

    SolverHandle h;
    ok(rrsph_create(&prm, precision_from_env(), &h.s));
    ok(rrsph_upload(h.s, r, stride, v, &rho(0), &p(0), it.data()));

    RRSPHOutput::instance().setup_output(
        std::bind(make_shared_vheap_darray_floatn, std::cref(r_var)),
        std::bind(make_shared_darray_copy<rr_int>, std::cref(itype)),
        std::bind(make_shared_vheap_darray_floatn, std::cref(v_var)),
        std::bind(make_shared_darray_copy<rr_float>, std::cref(p)),
        std::bind(make_shared_darray_copy<rr_float>, std::cref(rho)));

    rr_float time = params.start_simulation_time;
    rr_uint itimestep = 0;
    while (time <= params.simulation_time) {
        RRSPHOutput::instance().start_step(time);
        // the step and the download of its state (time += dt also when the step's check fails)
        const int rc = rrsph_step_download(h.s, 1, &time, r, stride, v, &rho(0), &p(0), it.data());
        const std::string step_error = rc == RRSPH_OK ? std::string() : rrsph_last_error();
        if (rc != RRSPH_OK) ok(rrsph_download(h.s, r, stride, v, &rho(0), &p(0), it.data()));
        for (rr_uint i = 0; i < n; ++i) itype(i) = it[i];
        itimestep++;
        RRSPHOutput::instance().update_step(time, itimestep);  // layers; its check throws on a failed step
        RRSPHOutput::instance().finish_step();
        if (rc != RRSPH_OK) throw std::runtime_error{step_error};
    }
}
