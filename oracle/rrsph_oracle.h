/*
 * rrsph_oracle.h — CPU oracle for the WCSPH step (TEST INFRASTRUCTURE).
 *
 * A plain-C (C11 + OpenMP, FP64) restatement of RRSPH_OMP's hot path, used only
 * as the checker by the tests, by the smoke check and as the CPU baseline of the
 * benchmark. The product (the CUDA library) never links or calls it.
 *
 * Parity of this restatement is pinned two ways:
 *   - against the golden CSVs and known-answer values of the reference's own
 *     tests (sources/RRSPH_COMMON/tests/caseDamBreak/test/OMP/ golden CSV files,
 *     testEOS.cpp, testSmoothingKernel.cpp, testGridUtils.cpp);
 *   - against the reference's own OMP compute core, compiled from its sources by
 *     oracle/build_ref.sh into oracle/_ref/ and run on the same inputs.
 *
 * Layouts: vectors are particle-major with a stride in doubles (2D: x,y;
 * 3D: x,y,z[,pad]); neighbour lists are list[j*max_per + n] with counts[j],
 * the reference's heap_darray_md layout (RR/include/RR/Memory/HeapDArray.h:78-84)
 * without the sentinel.
 */
#ifndef RRSPH_ORACLE_H
#define RRSPH_ORACLE_H

#include <stdint.h>
#include "../include/rrsph_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Smoothing kernels (SmoothingKernel.h:20-274). skf: 1 cubic, 2 Gauss,
 * 3 Wendland, 4 Desbrun. grad receives dim components. */
double orc_kernel_factor(const rrsph_params* p, uint32_t skf);
double orc_kernel_w(const rrsph_params* p, double dist, uint32_t skf);
void orc_kernel_dwdr(const rrsph_params* p, double dist, const double* diff,
                     uint32_t skf, double* grad);

/* EOS.cpp:3-44 */
double orc_eos_c_sqr(const rrsph_params* p);
double orc_eos_c(const rrsph_params* p);
double orc_eos_p(const rrsph_params* p, double rho);
double orc_eos_rho(const rrsph_params* p, double pres);

/* GridUtils.h:50-150: Morton code of a cell coordinate / of a position. */
uint32_t orc_morton2(uint32_t x, uint32_t y);
uint32_t orc_morton3(uint32_t x, uint32_t y, uint32_t z);
void orc_morton2_decode(uint32_t m, uint32_t* x, uint32_t* y);
void orc_morton3_decode(uint32_t m, uint32_t* x, uint32_t* y, uint32_t* z);
uint32_t orc_cell_idx(const rrsph_params* p, const double* r);
/* get_neighbouring_cells2/3 (GridUtils.h:190-250); cells gets 9 or 27 entries,
 * 0xFFFFFFFF for an invalid cell. */
void orc_neighbouring_cells(const rrsph_params* p, uint32_t idx, uint32_t* cells);

/* make_grid (GridFind.cpp:47-88). keys[ntotal], grid[ntotal],
 * cells_start[max_cells + 1]. Returns RRSPH_ERR_OUT_OF_DOMAIN if a key is
 * >= max_cells (with consistency_check) — then nothing is written. */
int orc_cell_keys(const rrsph_params* p, const double* r, uint32_t stride,
                  uint32_t* keys);
int orc_make_grid(const rrsph_params* p, const uint32_t* keys, uint32_t* grid,
                  uint32_t* cells_start);
/* find_neighbours (GridFind.cpp:112-189). */
int orc_find_neighbours(const rrsph_params* p, const double* r, uint32_t stride,
                        const int32_t* itype, const uint32_t* grid,
                        const uint32_t* cells_start, uint32_t* counts,
                        uint32_t* list, uint32_t max_per);

/* density_sum (Density.h:25-61) / density_con (Density.h:63-114). */
void orc_density_sum(const rrsph_params* p, const double* r, uint32_t stride,
                     const uint32_t* counts, const uint32_t* list, uint32_t max_per,
                     double* rho, double* pres);
void orc_density_con(const rrsph_params* p, const double* r, const double* v,
                     uint32_t stride, const double* rho, const uint32_t* counts,
                     const uint32_t* list, uint32_t max_per, double* drho,
                     double* pres);

/* update_acceleration (UpdateAcceleration.cpp:33-125) restricted to the terms
 * in `terms` (RRSPH_TERM_*). mu[j] = max |mu_ij| of the artificial viscosity
 * (ArtificialViscosity.h:41-45), may be NULL; av may be NULL. */
void orc_forces(const rrsph_params* p, uint32_t terms, const int32_t* itype,
                const double* r, const double* v, uint32_t stride,
                const double* rho, const double* pres, const uint32_t* counts,
                const uint32_t* list, uint32_t max_per, double* a, double* av,
                double* mu);

/* Piston / wave makers (WaveMaker.cpp:4-157) on the state at `time`. */
void orc_make_waves(rrsph_params* p, double* r, double* v, uint32_t stride,
                    int32_t* itype, double time);

/* The whole time loop body (TimeIntegration.cpp:60-100) for nsteps steps with
 * the piston call enabled. State arrays are read and updated in place; a and
 * drho (ntotal rows each) carry the previous step's values (zero at the start,
 * as the loop's fresh work arrays). itimestep is the loop counter of the first
 * step (0 => dt/2 velocity update, WholeStep.cpp:33). Returns 0 or an RRSPH_ERR_*
 * code. pair_counts (may be NULL) receives the directed pairs of each step
 * (nsteps entries). */
int orc_run(rrsph_params* p, double* r, double* v, uint32_t stride, double* rho,
            double* pres, int32_t* itype, double* a, double* drho,
            uint64_t itimestep, uint64_t nsteps, double* time_io,
            uint64_t* pair_counts);

/* Gauge elevation: HeightTesting::maxInLayer (tools/WaterProfile/include/
 * HeightTesting.h:25-54) — max y of particles with |x - x_gauge| < search_n*h
 * and itype == type_filter (type_filter == 0: any type); 0 if none. */
double orc_gauge(const rrsph_params* p, const double* r, uint32_t stride,
                 const int32_t* itype, double x_gauge, double search_n,
                 int32_t type_filter);

/* Forward run of the loop with a Fourier piston, X(t) = sum_k coef[k-1]
 * sin(k omega t) on the nwm particle range, and its forward-mode derivatives
 * (rrsph_tangent.c). Gauges of the states after sample_from, sample_from +
 * sample_every, ... <= nsteps steps go to gauges[s]; their derivatives by the
 * coefficients to dgauges[s * ncoef + k]. Method set: 2D, summation density,
 * cubic kernel, no artificial pressure / XSPH, constant dt, nwm == 2; otherwise
 * RRSPH_ERR_UNSUPPORTED. */
int orc_piston_tangent_run(rrsph_params* p, double* r, double* v, uint32_t stride, double* rho, double* pres,
                           int32_t* itype, double* a, uint64_t nsteps, double* time_io, uint32_t ncoef,
                           double omega, const double* coef, double gauge_x, double search_n, int32_t gauge_type,
                           uint64_t sample_from, uint64_t sample_every, double* gauges, double* dgauges,
                           uint64_t max_samples, uint64_t* nsamples);

/* Threads the oracle uses (OpenMP); <= 0 keeps the runtime default. */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
