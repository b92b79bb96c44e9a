/*
 * rrsph_tangent.c — forward-mode (tangent-linear) derivatives of the time loop
 * with respect to the coefficients of a Fourier piston (TEST INFRASTRUCTURE:
 * the FP64 forward-mode reference that the GPU adjoint is checked against; the
 * product never links it).
 *
 * The loop is orc_run's (TimeIntegration.cpp:60-100 with the piston call
 * enabled) for the method set of the piston flume: 2D, summation density
 * (Density.h:25-61), cubic spline kernel for density, pressure and viscosity
 * (SmoothingKernel.h:20-85), pressure form 1 or 2 (InternalForce.h:121-141),
 * Monaghan artificial viscosity (ArtificialViscosity.h:29-65), Lennard-Jones
 * boundary (ExtForce.h:15-60), constant dt, whole_step with CONSISTENCY_FIX or
 * STOP (WholeStep.cpp:19-62). The forward values come from the same oracle
 * functions as orc_run, so they are bit-identical to orc_run's.
 *
 * The piston particles [nwm_particles_start, nwm_particles_end) move with the
 * displacement X(t) = sum_k coef[k-1] sin(k omega t), k = 1..ncoef, i.e. the
 * velocity vx(t) = sum_k coef[k-1] k omega cos(k omega t) takes the place of
 * dynamic_boundaries' law (WaveMaker.cpp:34-82): r.x += vx dt, v.x = vx.
 *
 * Tangents, per coefficient direction d (all ncoef at once):
 *   v*'   = v' + a'_prev dt/2
 *   rho'_j = sum_i m sc (e . e'),           e = r_i - r_j, dW/dr = e sc
 *   p'_j   = c^2 (rho_j/rho0)^6 rho'_j
 *   a'_j   = sum_i [e' S + e S'] - LJ',     S = m sc (PF + Pi)
 *   piston: r'.x += phi_d dt, v'.x = phi_d,  phi_d(t) = k omega cos(k omega t)
 *   whole:  v' += a' v_dt, r' += v' dt      (fluid)
 * and the gauge tangent is y' of the particle that attains the gauge maximum
 * (HeightTesting.h:25-54; the first such id in ascending order).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "rrsph_oracle.h"

#define MAXC 16

/* cubic spline: sc with dW/dr = e*sc (SmoothingKernel.h:42-56) and sc1d = (dsc/ddist)/dist */
static void cubic_sc(double f, double h, double dist, double* sc, double* sc1d) {
    const double q = dist / h;
    if (q <= 1) {
        *sc = f / (h * h) * (-2.0 + 1.5 * q);
        *sc1d = 1.5 * f / (h * h * h * dist);
    } else if (q <= 2) {
        const double t = 2 - q;
        *sc = -f * t * t * 0.5 / (h * dist);
        *sc1d = f / (2 * h) * (2 * t / (h * dist * dist) + t * t / (dist * dist * dist));
    } else {
        *sc = 0;
        *sc1d = 0;
    }
}

static int in_geometry(const rrsph_params* p, double x, double y) {
    return x < p->x_maxgeom && x > p->x_mingeom && y < p->y_maxgeom && y > p->y_mingeom;
}

/* gauge maximum and its particle (HeightTesting::maxInLayer); id = -1 if none */
static double gauge_arg(const rrsph_params* p, const double* r, uint32_t stride, const int32_t* itype,
                        double xg, double radius, int32_t type, int64_t* id) {
    double best = 0;
    *id = -1;
    for (uint64_t i = 0; i < p->ntotal; i++) {
        if (type && itype[i] != type) continue;
        const double x = r[i * stride], y = r[i * stride + 1];
        if (fabs(x - xg) < radius && y > best) {
            best = y;
            *id = (int64_t)i;
        }
    }
    return best;
}

int orc_piston_tangent_run(rrsph_params* p, double* r, double* v, uint32_t stride, double* rho, double* pres,
                           int32_t* itype, double* a, uint64_t nsteps, double* time_io, uint32_t ncoef,
                           double omega, const double* coef, double gauge_x, double search_n, int32_t gauge_type,
                           uint64_t sample_from, uint64_t sample_every, double* gauges, double* dgauges,
                           uint64_t max_samples, uint64_t* nsamples) {
    const uint64_t n = p->ntotal;
    const uint32_t nc = ncoef;
    if (p->dim != 2 || stride < 2 || p->density_treatment != 0 || p->density_skf != 1 || p->intf_skf != 1 ||
        (p->artificial_viscosity && p->artificial_viscosity_skf != 1) || p->artificial_pressure ||
        p->average_velocity || p->dt_correction_method == 2 || p->nwm != 2 || nc == 0 || nc > MAXC ||
        sample_every == 0)
        return RRSPH_ERR_UNSUPPORTED;
    if (p->nwm_particles_start < p->nfluid || p->nwm_particles_end < p->nwm_particles_start ||
        p->nwm_particles_end > n)
        return RRSPH_ERR_UNSUPPORTED;
    const uint32_t max_per = p->max_neighbours ? p->max_neighbours : 1;
    const double h = p->hsml, m = p->mass, dt = p->dt;
    const double f = orc_kernel_factor(p, 1);
    const double c2 = orc_eos_c_sqr(p);
    const double rr0 = 2 * h, D = 5 * p->g * p->depth;
    const double eta = (h * (double)0.1f) * (h * (double)0.1f);
    const double alpha = p->artificial_shear_visc, beta = p->artificial_bulk_visc, c_av = p->eos_sound_vel;
    const double radius = search_n * h;
    int rc = RRSPH_OK;
    double time = *time_io;
    uint64_t ns = 0;

    const size_t vec = (size_t)n * 2 * nc, sca = (size_t)n * nc;
    double* rt = calloc(vec, sizeof(double));
    double* vt = calloc(vec, sizeof(double));
    double* at = calloc(vec, sizeof(double));
    double* vpt = calloc(vec, sizeof(double));
    double* rhot = calloc(sca, sizeof(double));
    double* pt = calloc(sca, sizeof(double));
    double* vp = malloc((size_t)n * stride * sizeof(double));
    uint32_t* keys = malloc(n * sizeof(uint32_t));
    uint32_t* grid = malloc(n * sizeof(uint32_t));
    uint32_t* cells = malloc((p->max_cells + 1) * sizeof(uint32_t));
    uint32_t* counts = malloc(n * sizeof(uint32_t));
    uint32_t* list = malloc(n * (size_t)max_per * sizeof(uint32_t));
    if (!rt || !vt || !at || !vpt || !rhot || !pt || !vp || !keys || !grid || !cells || !counts || !list) {
        rc = RRSPH_ERR_OUT_OF_MEMORY;
        goto done;
    }
#define T2(arr, i, c, d) arr[((size_t)(i) * 2 + (c)) * nc + (d)]

    for (uint64_t step = 0;; step++) {
        /* gauge sample of the state after `step` steps */
        if (step >= sample_from && (step - sample_from) % sample_every == 0) {
            if (ns < max_samples) {
                int64_t id;
                gauges[ns] = gauge_arg(p, r, stride, itype, gauge_x, radius, gauge_type, &id);
                for (uint32_t d = 0; d < nc; d++) dgauges[ns * nc + d] = id >= 0 ? T2(rt, id, 1, d) : 0.0;
            }
            ns++;
        }
        if (step == nsteps) break;
        /* predict_half_step */
        for (uint64_t i = 0; i < n; i++) {
            for (int c = 0; c < 2; c++) {
                vp[i * stride + c] = v[i * stride + c] + a[i * stride + c] * dt * 0.5;
                for (uint32_t d = 0; d < nc; d++) T2(vpt, i, c, d) = T2(vt, i, c, d) + T2(at, i, c, d) * dt * 0.5;
            }
        }
        /* grid_find */
        for (uint64_t i = 0; i < n; i++) keys[i] = orc_cell_idx(p, r + i * stride);
        if (p->consistency_check) {
            for (uint64_t i = 0; i < n; i++)
                if (keys[i] >= p->max_cells) { rc = RRSPH_ERR_OUT_OF_DOMAIN; goto done; }
        }
        if ((rc = orc_make_grid(p, keys, grid, cells)) != 0) goto done;
        if ((rc = orc_find_neighbours(p, r, stride, itype, grid, cells, counts, list, max_per)) != 0) goto done;
        /* density_sum and its tangent */
        orc_density_sum(p, r, stride, counts, list, max_per, rho, pres);
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < (int64_t)n; j++) {
            double acc[MAXC] = {0};
            const double* rj = r + j * stride;
            for (uint32_t k = 0; k < counts[j]; k++) {
                const uint32_t i = list[(size_t)j * max_per + k];
                const double* ri = r + (size_t)i * stride;
                const double ex = ri[0] - rj[0], ey = ri[1] - rj[1];
                const double dist = sqrt(ex * ex + ey * ey);
                double sc, sc1d;
                cubic_sc(f, h, dist, &sc, &sc1d);
                for (uint32_t d = 0; d < nc; d++) {
                    const double edx = T2(rt, i, 0, d) - T2(rt, j, 0, d), edy = T2(rt, i, 1, d) - T2(rt, j, 1, d);
                    acc[d] += m * sc * (ex * edx + ey * edy);
                }
            }
            const double x = rho[j] / p->rho0, x2 = x * x;
            const double dp = c2 * (x2 * x2 * x2);
            for (uint32_t d = 0; d < nc; d++) {
                rhot[j * nc + d] = acc[d];
                pt[j * nc + d] = dp * acc[d];
            }
        }
        /* update_acceleration and its tangent */
        orc_forces(p, RRSPH_TERM_ALL, itype, r, vp, stride, rho, pres, counts, list, max_per, a, NULL, NULL);
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < (int64_t)n; j++) {
            double ax[MAXC] = {0}, ay[MAXC] = {0};
            const double* rj = r + j * stride;
            const double* vj = vp + j * stride;
            const double rhoj = rho[j], pj = pres[j];
            for (uint32_t k = 0; k < counts[j]; k++) {
                const uint32_t i = list[(size_t)j * max_per + k];
                const double* ri = r + (size_t)i * stride;
                const double* vi = vp + (size_t)i * stride;
                const double rhoi = rho[i], pi = pres[i];
                const double ex = ri[0] - rj[0], ey = ri[1] - rj[1];
                const double s = ex * ex + ey * ey;
                const double dist = sqrt(s);
                double sc, sc1d;
                cubic_sc(f, h, dist, &sc, &sc1d);
                const int form1 = p->intf_sph_approximation == 1;
                const double PF = form1 ? (pj + pi) / (rhoj * rhoi) : pi / (rhoi * rhoi) + pj / (rhoj * rhoj);
                /* artificial viscosity, vr = (v_j - v_i).(r_j - r_i) */
                const double dvx = vj[0] - vi[0], dvy = vj[1] - vi[1];
                const double vr = -(dvx * ex + dvy * ey);
                const int av = p->artificial_viscosity && vr < 0;
                double Pi = 0, Pimu = 0, den = 0, mu = 0, rbar = 0;
                if (av) {
                    den = 1.0 / (s + eta);
                    mu = h * vr * den;
                    rbar = 0.5 * (rhoi + rhoj);
                    Pi = (beta * mu - alpha * c_av) * mu / rbar;
                    Pimu = (2 * beta * mu - alpha * c_av) / rbar;
                }
                const double S = m * sc * (PF + Pi);
                const int lj = p->boundary_treatment == 1 && itype[j] > 0 && itype[i] < 0 && dist < rr0;
                double fl = 0, fls = 0;
                if (lj) {
                    const double rn = rr0 / dist, rn2 = rn * rn, rn4 = rn2 * rn2, rn12 = rn4 * rn4 * rn4;
                    fl = D * (rn12 - rn4) / s;
                    fls = D * (-7 * rn12 + 3 * rn4) / (s * s);
                }
                for (uint32_t d = 0; d < nc; d++) {
                    const double edx = T2(rt, i, 0, d) - T2(rt, j, 0, d), edy = T2(rt, i, 1, d) - T2(rt, j, 1, d);
                    const double esd = ex * edx + ey * edy;
                    const double rj_t = rhot[j * nc + d], ri_t = rhot[i * nc + d];
                    const double pj_t = pt[j * nc + d], pi_t = pt[i * nc + d];
                    double PFd;
                    if (form1)
                        PFd = (pj_t + pi_t) / (rhoj * rhoi) - PF * (rj_t / rhoj + ri_t / rhoi);
                    else
                        PFd = pi_t / (rhoi * rhoi) - 2 * pi * ri_t / (rhoi * rhoi * rhoi) + pj_t / (rhoj * rhoj) -
                              2 * pj * rj_t / (rhoj * rhoj * rhoj);
                    double Pid = 0;
                    if (av) {
                        const double dvdx = T2(vpt, j, 0, d) - T2(vpt, i, 0, d);
                        const double dvdy = T2(vpt, j, 1, d) - T2(vpt, i, 1, d);
                        const double vrd = -(dvdx * ex + dvdy * ey) - (dvx * edx + dvy * edy);
                        const double mud = h * (vrd * den - vr * den * den * 2 * esd);
                        Pid = Pimu * mud - Pi / rbar * 0.5 * (ri_t + rj_t);
                    }
                    const double Sd = m * (sc1d * esd * (PF + Pi) + sc * (PFd + Pid));
                    ax[d] += edx * S + ex * Sd;
                    ay[d] += edy * S + ey * Sd;
                    if (lj) {
                        const double fld = fls * 2 * esd;
                        ax[d] -= edx * fl + ex * fld;
                        ay[d] -= edy * fl + ey * fld;
                    }
                }
            }
            for (uint32_t d = 0; d < nc; d++) {
                T2(at, j, 0, d) = ax[d];
                T2(at, j, 1, d) = ay[d];
            }
        }
        /* Fourier piston */
        if (time >= p->nwm_time_start) {
            double vx = 0, phi[MAXC];
            for (uint32_t k = 1; k <= nc; k++) {
                phi[k - 1] = k * omega * cos(k * omega * time);
                vx += coef[k - 1] * phi[k - 1];
            }
            for (uint64_t i = p->nwm_particles_start; i < p->nwm_particles_end; i++) {
                r[i * stride] = r[i * stride] + vx * dt;
                v[i * stride] = vx;
                for (uint32_t d = 0; d < nc; d++) {
                    T2(rt, i, 0, d) += phi[d] * dt;
                    T2(vt, i, 0, d) = phi[d];
                }
            }
        }
        /* whole_step */
        {
            const double v_dt = step ? dt : dt * 0.5;
            for (uint64_t i = 0; i < n; i++) {
                if (itype[i] <= 0) continue;
                double* vi = v + i * stride;
                double* ri = r + i * stride;
                vi[0] += a[i * stride] * v_dt;
                vi[1] += a[i * stride + 1] * v_dt;
                for (int c = 0; c < 2; c++)
                    for (uint32_t d = 0; d < nc; d++) T2(vt, i, c, d) += T2(at, i, c, d) * v_dt;
                const double nx = ri[0] + vi[0] * dt, ny = ri[1] + vi[1] * dt;
                if (p->consistency_treatment == 2 && !in_geometry(p, nx, ny)) {
                    itype[i] = p->type_non_existent;
                    continue;
                }
                ri[0] = nx;
                ri[1] = ny;
                for (int c = 0; c < 2; c++)
                    for (uint32_t d = 0; d < nc; d++) T2(rt, i, c, d) += T2(vt, i, c, d) * dt;
            }
        }
        time += dt;
        if (p->consistency_check && p->consistency_treatment == 1) {
            for (uint64_t i = 0; i < n; i++) {
                const double* ri = r + i * stride;
                if (!(in_geometry(p, ri[0], ri[1]) && isfinite(ri[0]) && isfinite(ri[1]))) {
                    rc = RRSPH_ERR_OUTSIDE_GEOMETRY;
                    goto done;
                }
            }
        }
    }
#undef T2
done:
    *time_io = time;
    if (nsamples) *nsamples = ns;
    free(rt); free(vt); free(at); free(vpt); free(rhot); free(pt); free(vp);
    free(keys); free(grid); free(cells); free(counts); free(list);
    return rc;
}
