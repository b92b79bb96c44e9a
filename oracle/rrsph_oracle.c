/*
 * rrsph_oracle.c — CPU oracle for the WCSPH step (TEST INFRASTRUCTURE ONLY).
 *
 * Restates the FP64 arithmetic of RRSPH_OMP operation by operation (same
 * evaluation order, no FMA contraction: build with -ffp-contract=off) so that it
 * agrees with the reference's compiled code to rounding. Each function names the
 * reference lines it follows (paths relative to the reference's sources/).
 * Only tests/, the smoke check and the benchmark's CPU-baseline leg use it.
 */
#include "rrsph_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define INVALID_CELL 0xFFFFFFFFu              /* GRID_INVALID_CELL = UINT_MAX (GridUtils.h:8) */
#define MAX_CELL_COORD2 ((1u << 16) - 1u)     /* GRID_MAX_CELL_COORD2 (GridUtils.h:9)          */

static double sqr(double v) { return v * v; }
static double cube(double v) { return v * v * v; }
/* powun (RRSPH_COMMON/include/CommonIncl.h:38-44): repeated multiplication from 1 */
static double powun(double v, unsigned n) {
    double r = 1;
    for (unsigned i = n; i > 0; i--) r *= v;
    return r;
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------- kernels -- */
/* SmoothingKernel.h:22-23, 92-93, 135-136, 193-194 */
double orc_kernel_factor(const rrsph_params* p, uint32_t skf) {
    const double h = p->hsml, pi = p->pi;
    const int d3 = p->dim == 3;
    switch (skf) {
    case 2: return d3 ? 1 / (pi * sqrt(pi) * cube(h)) : 1 / (pi * sqr(h));
    case 3: return d3 ? 21 / (16 * pi * cube(h)) : 7 / (4 * pi * sqr(h));
    case 4: return d3 ? 15 / (pi * cube(4 * h)) : 5 / (16 * pi * sqr(h));
    default: return d3 ? 3.0 / (2.0 * pi * cube(h)) : 15.0 / (7.0 * pi * sqr(h));
    }
}

/* smoothing_kernel_w (SmoothingKernel.h:244-252) */
double orc_kernel_w(const rrsph_params* p, double dist, uint32_t skf) {
    const double q = dist / p->hsml; /* get_kernel_q (:14-16) */
    const double f = orc_kernel_factor(p, skf);
    switch (skf) {
    case 2: /* gauss_kernel_q3 (:107-109) */
        return f * exp(-q * q);
    case 3: /* wendland_kernel_q2 (:152-154) */
        if (q <= 2) return f * powun(1 - 0.5 * q, 4) * (2 * q + 1);
        return 0;
    case 4: /* desbrun_kernel_q2 (:209-211) */
        if (q <= 2) return f * cube(2 - q);
        return 0;
    default: /* cubic_kernel_w (:58-69) */
        if (q <= 1) return f * (2.0 / 3.0 - sqr(q) + cube(q) * 0.5);
        if (q <= 2) return f * (1.0 / 6.0 * cube(2.0 - q));
        return 0;
    }
}

/* smoothing_kernel_dwdr (SmoothingKernel.h:266-274); grad has dim entries */
void orc_kernel_dwdr(const rrsph_params* p, double dist, const double* diff,
                     uint32_t skf, double* grad) {
    const int dim = (int)p->dim;
    const double h = p->hsml;
    const double q = dist / h;
    const double f = orc_kernel_factor(p, skf);
    int k;
    switch (skf) {
    case 2: { /* gauss_kernel_q3_grad (:114-116) with w = gauss_kernel_w */
        const double w = f * exp(-q * q);
        for (k = 0; k < dim; k++) grad[k] = diff[k] / sqr(h) * (-2) * w;
        return;
    }
    case 3: /* wendland_kernel_dwdr (:174-186) */
        if (q < (double)1.e-6f || !(q < 2)) {
            for (k = 0; k < dim; k++) grad[k] = 0;
            return;
        }
        for (k = 0; k < dim; k++) {
            const double fk = diff[k] / h / dist * f * 2;
            grad[k] = fk * (powun(1 - 0.5 * q, 4) - (2 * q + 1) * powun(1 - 0.5 * q, 3));
        }
        return;
    case 4: /* desbrun_kernel_dwdr (:230-240) */
        if (q < 2) {
            for (k = 0; k < dim; k++) grad[k] = diff[k] / dist / h * f * (-3 * sqr(2 - q));
        } else {
            for (k = 0; k < dim; k++) grad[k] = 0;
        }
        return;
    default: /* cubic_kernel_dwdr (:75-85) with the q1/q2 gradients (:42-56) */
        if (q <= 1) {
            for (k = 0; k < dim; k++) grad[k] = diff[k] / sqr(h) * f * (-2.0 + 3.0 * 0.5 * q);
        } else if (q <= 2) {
            for (k = 0; k < dim; k++) grad[k] = -diff[k] / dist / h * f * (sqr(2.0 - q) * 0.5);
        } else {
            for (k = 0; k < dim; k++) grad[k] = 0;
        }
        return;
    }
}

/* -------------------------------------------------------------------- EOS -- */
/* get_sound_velocity_sqr (RRSPH_COMMON/src/EOS.cpp:3-10). Method 1 returns the
 * user's eos_sound_vel as c^2 (the reference's behaviour, kept as is). */
double orc_eos_c_sqr(const rrsph_params* p) {
    if (p->eos_sound_vel_method == 0) return 200 * p->g * p->depth * p->eos_sound_vel_coef;
    return p->eos_sound_vel;
}
double orc_eos_c(const rrsph_params* p) { return sqrt(orc_eos_c_sqr(p)); }
static double eos_B(const rrsph_params* p) { return orc_eos_c_sqr(p) * p->rho0 / 7; } /* EOS.cpp:25-28 */
/* eos_art_p (EOS.cpp:31-34) */
double orc_eos_p(const rrsph_params* p, double rho) {
    return eos_B(p) * (powun(rho / p->rho0, 7) - 1);
}
/* eos_art_rho (EOS.cpp:36-44) */
double orc_eos_rho(const rrsph_params* p, double pres) {
    const double val = pres / eos_B(p) + 1;
    if (val >= 0) return p->rho0 * pow(val, 1.0 / 7);
    return NAN;
}

/* ------------------------------------------------------------------- grid -- */
/* morton2D_SplitBy2bits / m2D_e_magicbits (GridUtils.h:92-104); the 64-bit
 * rr_uint arithmetic keeps the low 16 bits of each coordinate. */
static uint64_t split2(uint64_t x) {
    x = (x | x << 16) & 0x0000FFFFull;
    x = (x | x << 8) & 0x00FF00FFull;
    x = (x | x << 4) & 0x0F0F0F0Full;
    x = (x | x << 2) & 0x33333333ull;
    x = (x | x << 1) & 0x55555555ull;
    return x;
}
/* morton3D_SplitBy3bits / m3D_e_magicbits (GridUtils.h:50-64): 10 bits/axis */
static uint64_t split3(uint64_t a) {
    uint64_t x = a & 0x000003ffull;
    x = (x | x << 16) & 0x30000ffull;
    x = (x | x << 8) & 0x0300f00full;
    x = (x | x << 4) & 0x30c30c3ull;
    x = (x | x << 2) & 0x9249249ull;
    return x;
}
static uint64_t second_bits(uint64_t m) { /* GridUtils.h:107-114 */
    uint64_t x = m & 0x55555555ull;
    x = (x ^ (x >> 1)) & 0x33333333ull;
    x = (x ^ (x >> 2)) & 0x0F0F0F0Full;
    x = (x ^ (x >> 4)) & 0x00FF00FFull;
    x = (x ^ (x >> 8)) & 0x0000FFFFull;
    return x;
}
static uint64_t third_bits(uint64_t m) { /* GridUtils.h:67-74 */
    uint64_t x = m & 0x9249249ull;
    x = (x ^ (x >> 2)) & 0x30c30c3ull;
    x = (x ^ (x >> 4)) & 0x0300f00full;
    x = (x ^ (x >> 8)) & 0x30000ffull;
    x = (x ^ (x >> 16)) & 0x000003ffull;
    return x;
}
uint32_t orc_morton2(uint32_t x, uint32_t y) { return (uint32_t)(split2(x) | (split2(y) << 1)); }
uint32_t orc_morton3(uint32_t x, uint32_t y, uint32_t z) {
    return (uint32_t)(split3(x) | (split3(y) << 1) | (split3(z) << 2));
}
void orc_morton2_decode(uint32_t m, uint32_t* x, uint32_t* y) {
    *x = (uint32_t)second_bits(m);
    *y = (uint32_t)second_bits((uint64_t)m >> 1);
}
void orc_morton3_decode(uint32_t m, uint32_t* x, uint32_t* y, uint32_t* z) {
    *x = (uint32_t)third_bits(m);
    *y = (uint32_t)third_bits((uint64_t)m >> 1);
    *z = (uint32_t)third_bits((uint64_t)m >> 2);
}

/* get_cell_coord_from_particle_coord (GridUtils.h:135-137): (rr_uint) truncation
 * of (r - r_min) / (cell_scale_k * h). Positions below r_min are outside the
 * geometry; they map to coordinate 0 here (the reference's cast is undefined). */
static uint64_t cell_coord(double r, double rmin, double cell) {
    const double c = (r - rmin) / cell;
    if (!(c >= 0)) return 0;
    if (c >= 18446744073709551615.0) return UINT64_MAX;
    return (uint64_t)c;
}

/* get_cell_idx2/3 (GridUtils.h:139-150) */
uint32_t orc_cell_idx(const rrsph_params* p, const double* r) {
    const double cell = p->cell_scale_k * p->hsml; /* grid_cell_size (GridUtils.h:30-32) */
    const uint64_t x = cell_coord(r[0], p->x_mingeom, cell);
    const uint64_t y = cell_coord(r[1], p->y_mingeom, cell);
    if (p->dim == 3) {
        const uint64_t z = cell_coord(r[2], p->z_mingeom, cell);
        return (uint32_t)(split3(x) | (split3(y) << 1) | (split3(z) << 2));
    }
    return (uint32_t)(split2(x) | (split2(y) << 1));
}

/* inc/dec_cell_coord and get_neighbouring_cells2/3 (GridUtils.h:158-250) */
static uint64_t inc_coord(uint64_t r) { return r == MAX_CELL_COORD2 ? INVALID_CELL : r + 1; }
static uint64_t dec_coord(uint64_t r) { return r == 0 ? INVALID_CELL : r - 1; }
void orc_neighbouring_cells(const rrsph_params* p, uint32_t idx, uint32_t* cells) {
    const int d3 = p->dim == 3;
    const int count = d3 ? 27 : 9;
    int i;
    if (idx == INVALID_CELL) {
        for (i = 0; i < count; i++) cells[i] = INVALID_CELL;
        return;
    }
    if (!d3) {
        uint32_t cx, cy;
        uint64_t xs[3], ys[3];
        orc_morton2_decode(idx, &cx, &cy);
        xs[0] = dec_coord(cx); xs[1] = cx; xs[2] = inc_coord(cx);
        ys[0] = dec_coord(cy); ys[1] = cy; ys[2] = inc_coord(cy);
        i = 0;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                cells[i++] = (xs[a] == INVALID_CELL || ys[b] == INVALID_CELL)
                                 ? INVALID_CELL
                                 : (uint32_t)(split2(xs[a]) | (split2(ys[b]) << 1));
    } else {
        uint32_t cx, cy, cz;
        uint64_t xs[3], ys[3], zs[3];
        orc_morton3_decode(idx, &cx, &cy, &cz);
        xs[0] = dec_coord(cx); xs[1] = cx; xs[2] = inc_coord(cx);
        ys[0] = dec_coord(cy); ys[1] = cy; ys[2] = inc_coord(cy);
        zs[0] = dec_coord(cz); zs[1] = cz; zs[2] = inc_coord(cz);
        i = 0;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                for (int c = 0; c < 3; c++)
                    cells[i++] = (xs[a] == INVALID_CELL || ys[b] == INVALID_CELL || zs[c] == INVALID_CELL)
                                     ? INVALID_CELL
                                     : (uint32_t)(split3(xs[a]) | (split3(ys[b]) << 1) | (split3(zs[c]) << 2));
    }
}

/* make_grid, first loop (GridFind.cpp:55-75) */
int orc_cell_keys(const rrsph_params* p, const double* r, uint32_t stride, uint32_t* keys) {
    const uint64_t n = p->ntotal;
    for (uint64_t i = 0; i < n; i++) {
        const uint32_t c = orc_cell_idx(p, r + i * stride);
        if (p->consistency_check && c >= p->max_cells) return RRSPH_ERR_OUT_OF_DOMAIN;
        keys[i] = c;
    }
    return RRSPH_OK;
}

/* make_grid, counting sort (GridFind.cpp:53-87): histogram, serial inclusive
 * prefix over max_cells, reverse scatter so ids ascend within a cell. The result
 * cells_start[c] is the lower bound of cell c in grid; one extra entry
 * cells_start[max_cells] = ntotal closes the last cell. */
int orc_make_grid(const rrsph_params* p, const uint32_t* keys, uint32_t* grid, uint32_t* cells_start) {
    const uint64_t n = p->ntotal, mc = p->max_cells;
    memset(cells_start, 0, (size_t)(mc + 1) * sizeof(uint32_t));
    for (uint64_t i = 0; i < n; i++) {
        if (keys[i] >= mc) return RRSPH_ERR_OUT_OF_DOMAIN;
        cells_start[keys[i]]++;
    }
    for (uint64_t c = 1; c < mc; c++) cells_start[c] += cells_start[c - 1];
    for (uint64_t i = n; i > 0; --i) {
        const uint64_t j = i - 1;
        const uint32_t c = keys[j];
        grid[cells_start[c] - 1] = (uint32_t)j;
        cells_start[c]--;
    }
    cells_start[mc] = (uint32_t)n;
    return RRSPH_OK;
}

/* find_neighbours (GridFind.cpp:112-189). Overflow (a particle with
 * max_neighbours - 1 or more neighbours, or more than max_per) is an error, as
 * with consistency_check on. */
int orc_find_neighbours(const rrsph_params* p, const double* r, uint32_t stride,
                        const int32_t* itype, const uint32_t* grid,
                        const uint32_t* cells_start, uint32_t* counts,
                        uint32_t* list, uint32_t max_per) {
    const int64_t n = (int64_t)p->ntotal;
    const int dim = (int)p->dim;
    const int ncells = dim == 3 ? 27 : 9;
    const double cell = p->cell_scale_k * p->hsml;
    const double max_dist = sqr(cell);
    uint32_t cap = p->max_neighbours ? p->max_neighbours - 1 : 0;
    if (cap > max_per) cap = max_per;
    int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int64_t j = 0; j < n; j++) {
        uint32_t cnt = 0;
        if (itype[j] != p->type_non_existent) {
            uint32_t cells[27];
            const double* rj = r + j * stride;
            orc_neighbouring_cells(p, orc_cell_idx(p, rj), cells);
            for (int ci = 0; ci < ncells; ci++) {
                const uint32_t c = cells[ci];
                if (c == INVALID_CELL) continue;
                if (c >= p->max_cells) continue; /* no particle can have such a key */
                for (uint32_t g = cells_start[c]; g < cells_start[c + 1]; g++) {
                    const uint32_t i = grid[g];
                    if ((int64_t)i == j) continue;
                    if (itype[i] == p->type_non_existent) continue;
                    const double* ri = r + (size_t)i * stride;
                    double d2;
                    if (dim == 3) {
                        const double dx = ri[0] - rj[0], dy = ri[1] - rj[1], dz = ri[2] - rj[2];
                        d2 = dx * dx + dy * dy + dz * dz;
                    } else {
                        const double dx = ri[0] - rj[0], dy = ri[1] - rj[1];
                        d2 = dx * dx + dy * dy;
                    }
                    if (d2 < max_dist) {
                        if (cnt >= cap) {
                            err = 1;
                            continue;
                        }
                        list[(size_t)j * max_per + cnt] = i;
                        cnt++;
                    }
                }
            }
        }
        counts[j] = cnt;
    }
    return err ? RRSPH_ERR_NEIGHBOUR_OVERFLOW : RRSPH_OK;
}

/* --------------------------------------------------------------- density -- */
static double dist_of(const double* a, const double* b, int dim, double* diff /* b - a */) {
    double s;
    diff[0] = b[0] - a[0];
    diff[1] = b[1] - a[1];
    s = diff[0] * diff[0] + diff[1] * diff[1];
    if (dim == 3) {
        diff[2] = b[2] - a[2];
        s = diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2];
    }
    return sqrt(s);
}

/* density_sum (Density.h:25-61) */
void orc_density_sum(const rrsph_params* p, const double* r, uint32_t stride,
                     const uint32_t* counts, const uint32_t* list, uint32_t max_per,
                     double* rho, double* pres) {
    const int64_t n = (int64_t)p->ntotal;
    const int dim = (int)p->dim;
    const double wjj = orc_kernel_w(p, 0, p->density_skf);
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
        double rho_temp = p->mass * wjj;
        for (uint32_t k = 0; k < counts[j]; k++) {
            const uint32_t i = list[(size_t)j * max_per + k];
            double diff[3];
            const double dist = dist_of(r + j * stride, r + (size_t)i * stride, dim, diff);
            rho_temp += p->mass * orc_kernel_w(p, dist, p->density_skf);
        }
        rho[j] = rho_temp;
        pres[j] = orc_eos_p(p, rho_temp);
    }
}

/* density_con (Density.h:63-114) */
void orc_density_con(const rrsph_params* p, const double* r, const double* v,
                     uint32_t stride, const double* rho, const uint32_t* counts,
                     const uint32_t* list, uint32_t max_per, double* drho,
                     double* pres) {
    const int64_t n = (int64_t)p->ntotal;
    const int dim = (int)p->dim;
    const double c = orc_eos_c(p);
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
        double drho_temp = 0;
        const double* rj = r + j * stride;
        const double* vj = v + j * stride;
        for (uint32_t k = 0; k < counts[j]; k++) {
            const uint32_t i = list[(size_t)j * max_per + k];
            const double* ri = r + (size_t)i * stride;
            const double* vi = v + (size_t)i * stride;
            double diff[3], dwdr[3], r_ab[3], dvx[3];
            const double dist = dist_of(rj, ri, dim, diff); /* diff = ri - rj */
            orc_kernel_dwdr(p, dist, diff, p->density_skf, dwdr);
            double vcc;
            for (int d = 0; d < dim; d++) {
                r_ab[d] = rj[d] - ri[d];
                dvx[d] = vi[d] - vj[d];
            }
            if (dim == 3) vcc = dvx[0] * dwdr[0] + dvx[1] * dwdr[1] + dvx[2] * dwdr[2];
            else vcc = dvx[0] * dwdr[0] + dvx[1] * dwdr[1];
            drho_temp += p->mass * vcc;
            if (p->density_treatment == 2) {
                double rd, rl;
                if (dim == 3) {
                    rd = r_ab[0] * dwdr[0] + r_ab[1] * dwdr[1] + r_ab[2] * dwdr[2];
                    rl = r_ab[0] * r_ab[0] + r_ab[1] * r_ab[1] + r_ab[2] * r_ab[2];
                } else {
                    rd = r_ab[0] * dwdr[0] + r_ab[1] * dwdr[1];
                    rl = r_ab[0] * r_ab[0] + r_ab[1] * r_ab[1];
                }
                const double r_factor = rd / rl;
                const double rho_factor = (rho[i] - rho[j]) / rho[i];
                const double delta_rho = rho_factor * r_factor;
                const double dhc = p->density_delta_sph_coef * p->hsml * c;
                drho_temp += 2 * dhc * delta_rho * p->mass;
            }
        }
        drho[j] = drho_temp;
        pres[j] = orc_eos_p(p, rho[j]);
    }
}

/* ----------------------------------------------------------------- forces -- */
/* calc_art_pressure (InternalForce.h:24-48) */
static double art_pressure(const rrsph_params* p, double w_ij, double p_i, double p_j,
                           double rho_i, double rho_j) {
    const double delta_r_kernel = orc_kernel_w(p, p->delta, p->artificial_pressure_skf);
    const int neg_i = p_i < 0, neg_j = p_j < 0;
    double ap = 0;
    if (neg_i || neg_j) {
        const double f_ij = w_ij / delta_r_kernel;
        const double api = neg_i ? (-p->artificial_pressure_coef * p_i / sqr(rho_i)) : 0;
        const double apj = neg_j ? (-p->artificial_pressure_coef * p_j / sqr(rho_j)) : 0;
        ap = (api + apj) * pow(f_ij, p->artificial_pressure_index);
    }
    return ap;
}

/* update_acceleration (UpdateAcceleration.cpp:33-125) and the per-pair terms:
 * external_force_part (ExtForce.h:15-60), find_internal_changes_part
 * (InternalForce.h:53-141), artificial_viscosity_part (ArtificialViscosity.h:29-65),
 * average_velocity_part (AverageVelocity.h:20-37). */
void orc_forces(const rrsph_params* p, uint32_t terms, const int32_t* itype,
                const double* r, const double* v, uint32_t stride,
                const double* rho, const double* pres, const uint32_t* counts,
                const uint32_t* list, uint32_t max_per, double* a, double* av,
                double* mu) {
    const int64_t n = (int64_t)p->ntotal;
    const int dim = (int)p->dim;
    const double rr0 = 2 * p->hsml;                 /* ExtForce.h:26 */
    const double D = 5 * p->g * p->depth;           /* ExtForce.h:27 */
    const double etq = (double)0.1f;                /* art_visc_etq (ArtificialViscosity.h:22) */
    const double c_av = p->eos_sound_vel;           /* params_eos_sound_vel (ArtificialViscosity.h:57) */
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
        double at[3] = {0, 0, 0}, avt[3] = {0, 0, 0}, arvmu = 0;
        const double* rj = r + j * stride;
        const double* vj = v + j * stride;
        if (terms & RRSPH_TERM_GRAVITY) at[1] = -p->g;
        for (uint32_t k = 0; k < counts[j]; k++) {
            const uint32_t i = list[(size_t)j * max_per + k];
            const double* ri = r + (size_t)i * stride;
            const double* vi = v + (size_t)i * stride;
            double diff[3];
            const double dist = dist_of(rj, ri, dim, diff); /* diff_ij = r(i) - r(j) */

            if ((terms & RRSPH_TERM_EXTERNAL) && p->boundary_treatment == 1) {
                if (itype[j] > 0 && itype[i] < 0 && dist < rr0) {
                    const double rr_norm = rr0 / dist;
                    const double f = D * (powun(rr_norm, 12) - powun(rr_norm, 4)) / sqr(dist);
                    for (int d = 0; d < dim; d++) at[d] += (rj[d] - ri[d]) * f;
                }
            }
            if (terms & RRSPH_TERM_INTERNAL) {
                double dw[3], pf;
                orc_kernel_dwdr(p, dist, diff, p->intf_skf, dw);
                if (p->intf_sph_approximation == 1) {
                    pf = (pres[j] + pres[i]) / (rho[j] * rho[i]);
                } else {
                    pf = (pres[i] / sqr(rho[i]) + pres[j] / sqr(rho[j]));
                }
                if (p->artificial_pressure) {
                    pf += art_pressure(p, orc_kernel_w(p, dist, p->artificial_pressure_skf),
                                       pres[i], pres[j], rho[i], rho[j]);
                }
                for (int d = 0; d < dim; d++) at[d] += (dw[d] * pf) * p->mass;
            }
            if ((terms & RRSPH_TERM_ART_VISC) && p->artificial_viscosity) {
                double dv[3], dr[3], vr, rr;
                for (int d = 0; d < dim; d++) {
                    dv[d] = vj[d] - vi[d];
                    dr[d] = rj[d] - ri[d];
                }
                if (dim == 3) {
                    vr = dv[0] * dr[0] + dv[1] * dr[1] + dv[2] * dr[2];
                    rr = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
                } else {
                    vr = dv[0] * dr[0] + dv[1] * dr[1];
                    rr = dr[0] * dr[0] + dr[1] * dr[1];
                }
                if (vr < 0) {
                    const double mu_ij = p->hsml * vr / (rr + sqr(p->hsml * etq));
                    if (fabs(mu_ij) > arvmu) arvmu = fabs(mu_ij);
                    const double rho_ij = 0.5 * (rho[i] + rho[j]);
                    const double piv = (p->artificial_bulk_visc * mu_ij -
                                        p->artificial_shear_visc * c_av) * mu_ij / rho_ij;
                    double dw[3];
                    orc_kernel_dwdr(p, dist, diff, p->artificial_viscosity_skf, dw);
                    for (int d = 0; d < dim; d++) at[d] += (dw[d] * piv) * p->mass;
                }
            }
            if ((terms & RRSPH_TERM_AVERAGE_VELOCITY) && p->average_velocity) {
                if (itype[i] > 0) {
                    const double w = orc_kernel_w(p, dist, p->average_velocity_skf);
                    for (int d = 0; d < dim; d++)
                        avt[d] += (vi[d] - vj[d]) * p->mass / (rho[i] + rho[j]) * w * 2 *
                                  p->average_velocity_coef;
                }
            }
        }
        for (int d = 0; d < dim; d++) a[j * stride + d] = at[d];
        if (av)
            for (int d = 0; d < dim; d++) av[j * stride + d] = avt[d];
        if (mu) mu[j] = arvmu;
    }
}

/* ------------------------------------------------------------ wave makers -- */
/* dynamic_boundaries (WaveMaker.cpp:34-82); the OMP code moves x only. */
static void dynamic_boundaries(const rrsph_params* p, double* r, double* v, uint32_t stride,
                               double time) {
    if (p->nwm_particles_start < p->nfluid || p->nwm_particles_end < p->nfluid ||
        p->nwm_particles_end < p->nwm_particles_start || p->nwm_particles_end > p->ntotal)
        return;
    const double generator_phase = p->nwm_phase - p->nwm_freq * p->nwm_time_start;
    const double delta = generator_phase;
    const double omega = p->nwm_freq;
    const double H = p->nwm_wave_magnitude;
    const double kd = p->nwm_wave_number * p->depth;
    const double m1 = 2 * sqr(sinh(kd)) / (sinh(kd) * cosh(kd) + kd);
    const double S0 = H / m1;
    double vx = 0.5 * S0 * omega * cos(omega * time + delta);
    if (p->nwm == 3) {
        const double e2_1 = sqr(H) / (32 * p->depth);
        const double e2_2 = 3 * cosh(kd) / cube(sinh(kd)) - 2 / m1;
        const double e2_coef = e2_1 + e2_2;
        vx += 2 * omega * e2_coef * cos(2 * omega * time + 2 * delta);
    }
    for (uint64_t i = p->nwm_particles_start; i < p->nwm_particles_end; i++) {
        r[i * stride] = r[i * stride] + vx * p->dt;
        v[i * stride] = vx;
    }
}

/* nwm_solitary_rayleigh (WaveMaker.cpp:84-134) */
static void solitary_rayleigh(const rrsph_params* p, double* r, double* v, uint32_t stride,
                              double time) {
    if (p->nwm_particles_start < p->nfluid || p->nwm_particles_end < p->nfluid ||
        p->nwm_particles_end < p->nwm_particles_start || p->nwm_particles_end > p->ntotal)
        return;
    const double H = p->nwm_wave_magnitude, h = p->depth, g = p->g;
    const double k = sqrt(3 * H / (4 * sqr(h) * (H + h)));
    const double c = sqrt(g * (H + h));
    const double Tf = 2 / (k * c) * (3.8 + H / h);
    const double tau = k * c * (time - Tf);
    const double u = tanh(tau);
    const double top_left = k * H * (h + H - H * sqr(u));
    const double top_right = 2 * k * sqr(H * u);
    const double top = top_left + top_right;
    const double bottom = sqr(k * (h + H - H * sqr(u)));
    const double dxdu = top / bottom;
    const double dudtau = 1 - sqr(tanh(tau));
    const double dtaudt = k * c;
    const double dxdt = dxdu * dudtau * dtaudt;
    for (uint64_t i = p->nwm_particles_start; i < p->nwm_particles_end; i++) {
        r[i * stride] = r[i * stride] + dxdt * p->dt;
        v[i * stride] = dxdt;
    }
}

/* make_waves (WaveMaker.cpp:4-32) incl. disappear_wall (:136-157) */
void orc_make_waves(rrsph_params* p, double* r, double* v, uint32_t stride, int32_t* itype,
                    double time) {
    switch (p->nwm) {
    case 2:
    case 3:
        dynamic_boundaries(p, r, v, stride, time);
        break;
    case 4:
        if (!(p->nwm_particles_start < p->nfluid || p->nwm_particles_end < p->nfluid ||
              p->nwm_particles_end < p->nwm_particles_start)) {
            for (uint64_t i = p->nwm_particles_start; i < p->nwm_particles_end && i < p->ntotal; i++)
                itype[i] = p->type_non_existent;
        }
        p->nwm = 0;
        break;
    case 5:
        solitary_rayleigh(p, r, v, stride, time);
        break;
    default:
        break;
    }
}

/* ------------------------------------------------------------- time loop -- */
static int within_geometry(const rrsph_params* p, const double* q) { /* WholeStep.cpp:4-17 */
    int in = q[0] < p->x_maxgeom && q[0] > p->x_mingeom && q[1] < p->y_maxgeom && q[1] > p->y_mingeom;
    if (p->dim == 3) in = in && q[2] < p->z_maxgeom && q[2] > p->z_mingeom;
    return in;
}

/* time_integration loop body (TimeIntegration.cpp:60-100) with
 * predict_half_step (PredictHalfStep.cpp:4-23), grid_find (GridFind.cpp:215-236),
 * density_sum/density_con, update_acceleration, the piston call that the OMP
 * loop leaves commented out (TimeIntegration.cpp:90-92) enabled, whole_step
 * (WholeStep.cpp:19-62) and the per-step boundary check (Output.cpp:395-416). */
int orc_run(rrsph_params* p, double* r, double* v, uint32_t stride, double* rho,
            double* pres, int32_t* itype, double* a, double* drho,
            uint64_t itimestep, uint64_t nsteps, double* time_io,
            uint64_t* pair_counts) {
    const uint64_t n = p->ntotal;
    const int dim = (int)p->dim;
    const int cont = p->density_treatment != 0;
    const uint32_t max_per = p->max_neighbours ? p->max_neighbours : 1;
    int rc = RRSPH_OK;
    double time = *time_io;
    double* v_pred = (double*)malloc(n * stride * sizeof(double));
    double* rho_pred = (double*)malloc(n * sizeof(double));
    double* av = (double*)calloc(n * stride, sizeof(double));
    double* mu = (double*)calloc(n, sizeof(double));
    uint32_t* keys = (uint32_t*)malloc(n * sizeof(uint32_t));
    uint32_t* grid = (uint32_t*)malloc(n * sizeof(uint32_t));
    uint32_t* cells = (uint32_t*)malloc((p->max_cells + 1) * sizeof(uint32_t));
    uint32_t* counts = (uint32_t*)malloc(n * sizeof(uint32_t));
    uint32_t* list = (uint32_t*)malloc(n * (size_t)max_per * sizeof(uint32_t));
    if (!v_pred || !rho_pred || !av || !mu || !keys || !grid || !cells || !counts || !list) {
        rc = RRSPH_ERR_OUT_OF_MEMORY;
        goto done;
    }
    for (uint64_t s = 0; s < nsteps; s++, itimestep++) {
        /* predict_half_step */
        for (uint64_t i = 0; i < n; i++) {
            if (cont) rho_pred[i] = rho[i] + drho[i] * p->dt * 0.5;
            for (int d = 0; d < dim; d++)
                v_pred[i * stride + d] = v[i * stride + d] + a[i * stride + d] * p->dt * 0.5;
        }
        /* grid_find */
        for (uint64_t i = 0; i < n; i++) keys[i] = orc_cell_idx(p, r + i * stride);
        if (p->consistency_check) {
            for (uint64_t i = 0; i < n; i++)
                if (keys[i] >= p->max_cells) { rc = RRSPH_ERR_OUT_OF_DOMAIN; goto done; }
        }
        rc = orc_make_grid(p, keys, grid, cells);
        if (rc) goto done;
        rc = orc_find_neighbours(p, r, stride, itype, grid, cells, counts, list, max_per);
        if (rc) goto done;
        if (pair_counts) {
            uint64_t tot = 0;
            for (uint64_t i = 0; i < n; i++) tot += counts[i];
            pair_counts[s] = tot;
        }
        /* density */
        if (cont) orc_density_con(p, r, v, stride, rho, counts, list, max_per, drho, pres);
        else orc_density_sum(p, r, stride, counts, list, max_per, rho, pres);
        /* update_acceleration: v_predict, rho_predict (continuity) or rho */
        orc_forces(p, RRSPH_TERM_ALL, itype, r, v_pred, stride, cont ? rho_pred : rho, pres,
                   counts, list, max_per, a, p->average_velocity ? av : NULL, mu);
        /* update_dt (UpdateAcceleration.cpp:15-29, 104-121) under DT_CORRECTION_DYNAMIC:
         * the OpenMP build compiles the maxima out (both stay 0); with
         * dt_dynamic_reduce they are the serial build's max |a_j| and max arvmu_j. */
        if (p->dt_correction_method == 2) {
            double amax = 0, mumax = 0;
            if (p->dt_dynamic_reduce) {
                for (uint64_t j = 0; j < n; j++) {
                    const double* aj = a + j * stride;
                    double l2 = aj[0] * aj[0] + aj[1] * aj[1];
                    if (dim == 3) l2 += aj[2] * aj[2];
                    const double am = sqrt(l2);
                    if (am > amax) amax = am;
                    if (mu[j] > mumax) mumax = mu[j];
                }
            }
            const double c0 = orc_eos_c(p);
            const double min_dt_a = sqrt(p->hsml / amax);
            const double min_dt_mu = p->hsml / (c0 + mumax);
            p->dt = p->CFL_coef * (min_dt_mu < min_dt_a ? min_dt_mu : min_dt_a);
            if (p->dt <= (p->hsml / c0) * 1.E-6) { rc = RRSPH_ERR_NEVER_ENDING; goto done; }
        }
        /* piston */
        if (p->nwm && time >= p->nwm_time_start) orc_make_waves(p, r, v, stride, itype, time);
        /* whole_step */
        {
            const double r_dt = p->dt;
            const double v_dt = itimestep ? p->dt : p->dt * 0.5;
            for (uint64_t i = 0; i < n; i++) {
                if (cont) rho[i] = rho[i] + drho[i] * v_dt;
                if (itype[i] > 0) {
                    double* vi = v + i * stride;
                    double* ri = r + i * stride;
                    for (int d = 0; d < dim; d++) vi[d] += a[i * stride + d] * v_dt;
                    if (p->average_velocity)
                        for (int d = 0; d < dim; d++) vi[d] += av[i * stride + d];
                    if (p->consistency_treatment == 2) {
                        double nr[3];
                        for (int d = 0; d < dim; d++) nr[d] = ri[d] + vi[d] * r_dt;
                        if (within_geometry(p, nr)) {
                            for (int d = 0; d < dim; d++) ri[d] = nr[d];
                        } else {
                            itype[i] = p->type_non_existent;
                        }
                    } else {
                        for (int d = 0; d < dim; d++) ri[d] += vi[d] * r_dt;
                    }
                }
            }
        }
        time += p->dt;
        /* update_step consistency check (Output.cpp:395-416) */
        if (p->consistency_check) {
            for (uint64_t i = 0; i < n; i++) {
                const double* ri = r + i * stride;
                int ok = within_geometry(p, ri) && isfinite(ri[0]) && isfinite(ri[1]);
                if (dim == 3) ok = ok && isfinite(ri[2]);
                if (!ok && p->consistency_treatment == 1) {
                    rc = RRSPH_ERR_OUTSIDE_GEOMETRY;
                    goto done;
                }
            }
        }
    }
done:
    *time_io = time;
    free(v_pred); free(rho_pred); free(av); free(mu); free(keys); free(grid); free(cells);
    free(counts); free(list);
    return rc;
}

/* HeightTesting::maxInLayer (tools/WaterProfile/include/HeightTesting.h:25-54) */
double orc_gauge(const rrsph_params* p, const double* r, uint32_t stride,
                 const int32_t* itype, double x_gauge, double search_n, int32_t type_filter) {
    const double radius = search_n * p->hsml;
    double best = 0;
    for (uint64_t i = 0; i < p->ntotal; i++) {
        if (type_filter && itype[i] != type_filter) continue;
        const double x = r[i * stride], y = r[i * stride + 1];
        if (fabs(x - x_gauge) < radius && y > best) best = y;
    }
    return best;
}
