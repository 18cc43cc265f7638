/* Oracle -- TEST INFRASTRUCTURE ONLY (see pdpd_oracle.h).
 *
 * Restates, in plain C and in the same floating-point operation order, the reference's
 * FP64 half-step engine:
 *   step_impl            include/dpd/engines/naive/naive_dpd_engine_half_step.hpp:239-356
 *   update_cell_forces   naive_dpd_engine_half_step.hpp:358-424
 *   update_hookean_bond  naive_dpd_engine_half_step.hpp:426-446
 *   update_angle_bond    naive_dpd_engine_half_step.hpp:448-483
 *   update_pos/update_mom/calc_force/calc_angle_force
 *                        include/dpd/maths/dpd_maths_core_half_step.hpp:22-230
 *   hash RNG             include/dpd/core/hash.hpp:20-30,61-65,81-88
 *   default_hash         include/dpd/maths/dpd_maths_core.hpp:55-79
 * Build with -ffp-contract=off so no multiply-add is fused on any host.
 */
#include "pdpd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- hash RNG */

uint64_t pdo_mix64_m2(uint64_t x)
{
    const uint64_t C = 0xd392d2a7u;
    x = x ^ (x >> 32);
    x = x * C;
    x = x ^ (x >> 32);
    x = x * C;
    x = x ^ (x >> 32);
    return x;
}

uint64_t pdo_t_hash(uint32_t t, uint64_t seed)
{
    uint64_t base = seed + pdo_mix64_m2(t);
    return pdo_mix64_m2(base);
}

uint32_t pdo_hash_rng_sym(uint64_t t_hash, uint32_t a, uint32_t b)
{
    if (a > b) {
        uint32_t tmp = a;
        a = b;
        b = tmp;
    }
    return (uint32_t)pdo_mix64_m2(((uint64_t)a | ((uint64_t)b << 32)) ^ t_hash);
}

float pdo_default_hash(uint64_t t_hash, uint32_t a, uint32_t b)
{
    uint32_t ru = pdo_hash_rng_sym(t_hash, a, b);
    int32_t rs;
    memcpy(&rs, &ru, 4); /* two's complement reinterpretation, as uint32_to_int32 */
    const float scale = 0.00000000023283064365386962890625f; /* 2^-32 */
    return (float)rs * scale;
}

void pdo_hash_batch(size_t n, const uint32_t *t, const uint64_t *seed, const uint32_t *a,
                    const uint32_t *b, uint64_t *t_hash_out, uint32_t *h_out, float *u_out)
{
    for (size_t i = 0; i < n; i++) {
        uint64_t th = pdo_t_hash(t[i], seed[i]);
        if (t_hash_out) t_hash_out[i] = th;
        if (h_out) h_out[i] = pdo_hash_rng_sym(th, a[i], b[i]);
        if (u_out) u_out[i] = pdo_default_hash(th, a[i], b[i]);
    }
}

/* ---------------------------------------------------------------- cells */

/* dpd_state.hpp:138-139: computed in single precision, compared in double. */
static const float MIN_DISTANCE_CUTOFF = 0.000000001f;

static double min_dist_cutoff_sqr(void)
{
    volatile float m = MIN_DISTANCE_CUTOFF;
    float sq = m * m;
    return (double)sq;
}

void pdo_cell_index(const pdo_world *w, uint32_t *cell_out)
{
    const int Ly = w->box[1], Lz = w->box[2];
    for (uint32_t i = 0; i < w->n_beads; i++) {
        int c0 = (int)floor(w->x[3 * i + 0]);
        int c1 = (int)floor(w->x[3 * i + 1]);
        int c2 = (int)floor(w->x[3 * i + 2]);
        cell_out[i] = (uint32_t)(c0 * Ly * Lz + c1 * Lz + c2);
    }
}

typedef struct cell_list {
    uint32_t n_cells;
    uint32_t *start; /* n_cells+1 */
    uint32_t *beads; /* bead ids, grouped by cell, ascending id inside a cell */
} cell_list;

/* Counting sort by cell, stable in bead id: the same per-cell order as the reference's
 * push_back over beads in id order (naive_dpd_engine_half_step.hpp:276-293). */
static int build_cells(const pdo_world *w, cell_list *cl, uint32_t *cell_of)
{
    const uint32_t n_cells = (uint32_t)w->box[0] * (uint32_t)w->box[1] * (uint32_t)w->box[2];
    cl->n_cells = n_cells;
    cl->start = (uint32_t *)calloc((size_t)n_cells + 1, sizeof(uint32_t));
    cl->beads = (uint32_t *)malloc(sizeof(uint32_t) * (w->n_beads ? w->n_beads : 1));
    if (!cl->start || !cl->beads) return -1;
    pdo_cell_index(w, cell_of);
    for (uint32_t i = 0; i < w->n_beads; i++) cl->start[cell_of[i] + 1]++;
    for (uint32_t c = 0; c < n_cells; c++) cl->start[c + 1] += cl->start[c];
    uint32_t *fill = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)n_cells + 1));
    if (!fill) return -1;
    memcpy(fill, cl->start, sizeof(uint32_t) * ((size_t)n_cells + 1));
    for (uint32_t i = 0; i < w->n_beads; i++) cl->beads[fill[cell_of[i]]++] = i;
    free(fill);
    return 0;
}

static void free_cells(cell_list *cl)
{
    free(cl->start);
    free(cl->beads);
    cl->start = cl->beads = NULL;
}

/* ---------------------------------------------------------------- pair forces */

typedef struct force_job {
    pdo_world *w;
    const cell_list *cl;
    uint64_t t_hash;
    double scale_inv_sqrt_dt;
    double min_dr2;
    uint32_t cell_begin, cell_end;
} force_job;

/* naive_dpd_engine_half_step.hpp:181-196 */
static void relative_cell(const int32_t *box, const int *base, const int *dir, int *pos,
                          double *delta)
{
    for (int i = 0; i < 3; i++) {
        int raw = base[i] + dir[i];
        int is_left = raw < 0;
        int is_right = raw == box[i];
        pos[i] = raw + (is_left - is_right) * box[i];
        delta[i] = (double)(is_right - is_left) * (double)box[i];
    }
}

/* Full-shell gather for every bead of cells [cell_begin, cell_end): for each of the 27
 * directions in (-1..1)^3 lexicographic order, for each bead of that neighbour cell in
 * id order, add the pair force to the home bead (naive_dpd_engine_half_step.hpp:300-315,
 * 358-424; calc_force dpd_maths_core_half_step.hpp:69-157). */
static void *force_worker(void *arg)
{
    force_job *job = (force_job *)arg;
    pdo_world *w = job->w;
    const cell_list *cl = job->cl;
    const int32_t *box = w->box;
    const uint32_t nt = w->n_types;
    for (uint32_t c = job->cell_begin; c < job->cell_end; c++) {
        int pos[3];
        pos[0] = (int)(c / ((uint32_t)box[1] * (uint32_t)box[2]));
        pos[1] = (int)((c / (uint32_t)box[2]) % (uint32_t)box[1]);
        pos[2] = (int)(c % (uint32_t)box[2]);
        int dir[3];
        for (dir[0] = -1; dir[0] <= 1; dir[0]++)
            for (dir[1] = -1; dir[1] <= 1; dir[1]++)
                for (dir[2] = -1; dir[2] <= 1; dir[2]++) {
                    int opos[3];
                    double delta[3];
                    relative_cell(box, pos, dir, opos, delta);
                    uint32_t oc = (uint32_t)(opos[0] * box[1] * box[2] + opos[1] * box[2] + opos[2]);
                    for (uint32_t ko = cl->start[oc]; ko < cl->start[oc + 1]; ko++) {
                        uint32_t o = cl->beads[ko];
                        double ob_x[3];
                        for (int d = 0; d < 3; d++) ob_x[d] = w->x[3 * o + d] + delta[d];
                        for (uint32_t kh = cl->start[c]; kh < cl->start[c + 1]; kh++) {
                            uint32_t h = cl->beads[kh];
                            /* two stationary beads do not interact
                               (naive_dpd_engine_half_merge.hpp:440-449, 516-522) */
                            if ((w->stationary >> (w->hash[h] >> 28)) & (w->stationary >> (w->hash[o] >> 28)) & 1u)
                                continue;
                            double dx[3];
                            for (int d = 0; d < 3; d++) dx[d] = w->x[3 * h + d] - ob_x[d];
                            double dr2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
                            if (dr2 >= 1 || dr2 < job->min_dr2) continue;
                            double dr = sqrt(dr2);

                            /* calc_force with kappa = 0, r0 = 0.5 */
                            const double kappa = 0.0, r0 = 0.5;
                            double inv_dr = 1.0 / dr;
                            uint32_t hh = w->hash[h], ho = w->hash[o];
                            uint32_t th = hh >> 28, to = ho >> 28;
                            double con_strength, sqrt_diss;
                            if (w->cell_conservative) {
                                /* per-cell strengths, averaged over the two beads' cells
                                   (naive_dpd_engine_half_merge.hpp:221-236, 570-583) */
                                const size_t n2 = (size_t)nt * nt, k = (size_t)th * nt + to;
                                con_strength = (w->cell_conservative[c * n2 + k] + w->cell_conservative[oc * n2 + k]) * 0.5;
                                sqrt_diss = (sqrt(w->cell_dissipative[c * n2 + k]) + sqrt(w->cell_dissipative[oc * n2 + k])) * 0.5;
                            } else {
                                con_strength = w->conservative[th * nt + to];
                                sqrt_diss = sqrt(w->dissipative[th * nt + to]);
                            }
                            double dv[3];
                            for (int d = 0; d < 3; d++) dv[d] = w->v[3 * h + d] - w->v[3 * o + d];
                            double wr = 1.0 - dr;
                            double con_force = con_strength * wr;
                            double e[3];
                            for (int d = 0; d < 3; d++) e[d] = dx[d] * inv_dr;
                            double rdotv = e[0] * dv[0] + e[1] * dv[1] + e[2] * dv[2];
                            double sqrt_gammap = sqrt_diss * wr;
                            double diss_force = -sqrt_gammap * sqrt_gammap * rdotv;
                            double u = (double)pdo_default_hash(job->t_hash, hh, ho);
                            double rand_scale = sqrt_gammap * job->scale_inv_sqrt_dt;
                            double rand_force = rand_scale * u;
                            double dr0 = r0 - dr;
                            double hookean_force = kappa * dr0;
                            double scaled = con_force + diss_force + rand_force + hookean_force;
                            for (int d = 0; d < 3; d++) w->f[3 * h + d] = w->f[3 * h + d] + e[d] * scaled;
                        }
                    }
                }
    }
    return NULL;
}

/* ---------------------------------------------------------------- bonds */

/* naive_dpd_engine_half_step.hpp:198-209 */
static void distance_from_to(const int32_t *box, const double *base, const double *other,
                             double *res)
{
    for (int i = 0; i < 3; i++) {
        double len = (double)box[i];
        double dx = other[i] - base[i];
        int wrap_neg = dx > len * 0.5;
        int wrap_pos = dx < -len * 0.5;
        res[i] = dx + (double)(wrap_pos - wrap_neg) * len;
    }
}

static double l2_norm(const double *d)
{
    return sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

/* naive_dpd_engine_half_step.hpp:426-446 */
static int hookean_bond(pdo_world *w, uint32_t k, char *err, size_t errlen)
{
    uint32_t h = w->bond_beads[2 * k], t = w->bond_beads[2 * k + 1];
    double dx[3];
    distance_from_to(w->box, &w->x[3 * h], &w->x[3 * t], dx);
    double dr = l2_norm(dx);
    if (dr > 2.0) {
        if (err) snprintf(err, errlen, "an angle bond has snapped (bond %u, r=%g)", k, dr);
        return -1;
    }
    double dr0 = w->bond_r0[k] - dr;
    double hookean_force = w->bond_kappa[k] * dr0;
    double s = hookean_force / dr;
    for (int d = 0; d < 3; d++) {
        double fd = dx[d] * s;
        w->f[3 * h + d] = w->f[3 * h + d] - fd;
        w->f[3 * t + d] = w->f[3 * t + d] + fd;
    }
    return 0;
}

/* naive_dpd_engine_half_step.hpp:448-483 and calc_angle_force
 * (dpd_maths_core_half_step.hpp:177-229) */
static void angle_bond(pdo_world *w, uint32_t k)
{
    uint32_t h = w->angle_beads[3 * k], m = w->angle_beads[3 * k + 1], t = w->angle_beads[3 * k + 2];
    double first[3], second[3];
    distance_from_to(w->box, &w->x[3 * h], &w->x[3 * m], first);
    distance_from_to(w->box, &w->x[3 * m], &w->x[3 * t], second);
    double r01 = l2_norm(first), r12 = l2_norm(second);
    double kappa = w->angle_kappa[k];
    double cos_theta0 = cos(w->angle_theta0[k]);
    double sin_theta0 = sin(w->angle_theta0[k]);
    double hf[3] = {0, 0, 0}, mf[3] = {0, 0, 0}, tf[3] = {0, 0, 0};
    double mag_product = r01 * r12;
    if (mag_product > 0.0001) {
        double b1_mag_sq = r01 * r01;
        double b2_mag_sq = r12 * r12;
        double b1_dot_b2 = first[0] * second[0] + first[1] * second[1] + first[2] * second[2];
        double b1b2_over_b1sq = b1_dot_b2 / b1_mag_sq;
        double b1b2_over_b2sq = b1_dot_b2 / b2_mag_sq;
        double cos_phi_sq = b1b2_over_b1sq * b1b2_over_b2sq;
        double force_mag = kappa / mag_product;
        if (fabs(b1_dot_b2) > 0.000001 && sin_theta0 > 0) {
            double inv_prefactor = 1.0 / sqrt(1.0 / cos_phi_sq - 1.0);
            force_mag = force_mag * (cos_theta0 - sin_theta0 * inv_prefactor);
        }
        for (int d = 0; d < 3; d++) {
            hf[d] = (first[d] * b1b2_over_b1sq - second[d]) * force_mag;
            tf[d] = (first[d] - second[d] * b1b2_over_b2sq) * force_mag;
            mf[d] = -(hf[d] + tf[d]);
        }
    }
    for (int d = 0; d < 3; d++) {
        w->f[3 * h + d] = w->f[3 * h + d] + hf[d];
        w->f[3 * t + d] = w->f[3 * t + d] + tf[d];
        w->f[3 * m + d] = w->f[3 * m + d] + mf[d];
    }
}

/* ---------------------------------------------------------------- step */

static int run_parallel(force_job *jobs, int nthreads)
{
    if (nthreads <= 1) {
        force_worker(&jobs[0]);
        return 0;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    if (!th) return -1;
    int started = 0;
    for (int i = 1; i < nthreads; i++) {
        if (pthread_create(&th[i], NULL, force_worker, &jobs[i]) != 0) break;
        started = i;
    }
    force_worker(&jobs[0]);
    for (int i = started + 1; i < nthreads; i++) force_worker(&jobs[i]); /* not started */
    for (int i = 1; i <= started; i++) pthread_join(th[i], NULL);
    free(th);
    return 0;
}

int pdo_run(pdo_world *w, uint32_t nsteps, int nthreads, char *err, size_t errlen)
{
    for (int i = 0; i < 3; i++) {
        if (w->box[i] < 2) {
            if (err) snprintf(err, errlen, "Distance in each direction must be at least 2");
            return -1;
        }
    }
    if (nthreads < 1) nthreads = 1;
    const double dt = w->dt;
    const double scale_inv_sqrt_dt = sqrt(24 * 1.0 / dt);
    const double min_dr2 = min_dist_cutoff_sqr();
    uint32_t *cell_of = (uint32_t *)malloc(sizeof(uint32_t) * (w->n_beads ? w->n_beads : 1));
    force_job *jobs = (force_job *)malloc(sizeof(force_job) * (size_t)nthreads);
    if (!cell_of || !jobs) return -1;
    int rc = 0;
    for (uint32_t s = 0; s < nsteps && rc == 0; s++) {
        uint64_t t_hash = pdo_t_hash((uint32_t)w->t, w->seed);

        /* update_pos (dpd_maths_core_half_step.hpp:22-49) */
        const double hdt2 = (dt * dt) * 0.5, hdt = dt * 0.5;
        for (uint32_t i = 0; i < w->n_beads; i++) {
            /* stationary bead types are not moved (naive_dpd_engine_half_merge.hpp:329-333) */
            if ((w->stationary >> (w->hash[i] >> 28)) & 1u) continue;
            for (int d = 0; d < 3; d++) {
                double L = (double)w->box[d];
                double x = w->x[3 * i + d] + w->v[3 * i + d] * dt + w->f[3 * i + d] * hdt2;
                if (x < 0) {
                    x += L;
                    if (x == L) x = 0;
                } else if (x >= L) {
                    x -= L;
                }
                if (!(0 <= x && x < L)) {
                    if (err) snprintf(err, errlen, "bead %u left the box", i);
                    rc = -1;
                }
                w->x[3 * i + d] = x;
            }
            for (int d = 0; d < 3; d++) {
                w->v[3 * i + d] = w->v[3 * i + d] + w->f[3 * i + d] * hdt;
                w->f[3 * i + d] = 0;
            }
        }
        if (rc) break;

        cell_list cl;
        if (build_cells(w, &cl, cell_of) != 0) {
            rc = -1;
            break;
        }
        uint32_t per = (cl.n_cells + (uint32_t)nthreads - 1) / (uint32_t)nthreads;
        for (int i = 0; i < nthreads; i++) {
            jobs[i].w = w;
            jobs[i].cl = &cl;
            jobs[i].t_hash = t_hash;
            jobs[i].scale_inv_sqrt_dt = scale_inv_sqrt_dt;
            jobs[i].min_dr2 = min_dr2;
            uint32_t b = per * (uint32_t)i;
            uint32_t e = b + per;
            jobs[i].cell_begin = b < cl.n_cells ? b : cl.n_cells;
            jobs[i].cell_end = e < cl.n_cells ? e : cl.n_cells;
        }
        run_parallel(jobs, nthreads);
        free_cells(&cl);

        for (uint32_t k = 0; k < w->n_bonds && rc == 0; k++) rc = hookean_bond(w, k, err, errlen);
        if (rc) break;
        for (uint32_t k = 0; k < w->n_angles; k++) angle_bond(w, k);

        /* update_mom (dpd_maths_core_half_step.hpp:51-61); a stationary bead's v and f are
           cleared instead (naive_dpd_engine_half_merge.hpp:387-394) */
        for (uint32_t i = 0; i < w->n_beads; i++) {
            if ((w->stationary >> (w->hash[i] >> 28)) & 1u) {
                for (int d = 0; d < 3; d++) w->v[3 * i + d] = w->f[3 * i + d] = 0.0;
                continue;
            }
            for (int d = 0; d < 3; d++) w->v[3 * i + d] = w->v[3 * i + d] + w->f[3 * i + d] * hdt;
        }

        w->t += 1;
    }
    free(cell_of);
    free(jobs);
    return rc;
}

/* ---------------------------------------------------------------- observables */

typedef struct obs_job {
    const pdo_world *w;
    const cell_list *cl;
    uint32_t cell_begin, cell_end;
    uint32_t n_bins;
    double virial;
    uint64_t *rdf;
} obs_job;

static void *obs_worker(void *arg)
{
    obs_job *job = (obs_job *)arg;
    const pdo_world *w = job->w;
    const cell_list *cl = job->cl;
    const int32_t *box = w->box;
    const uint32_t nt = w->n_types;
    double vir = 0;
    for (uint32_t c = job->cell_begin; c < job->cell_end; c++) {
        int pos[3];
        pos[0] = (int)(c / ((uint32_t)box[1] * (uint32_t)box[2]));
        pos[1] = (int)((c / (uint32_t)box[2]) % (uint32_t)box[1]);
        pos[2] = (int)(c % (uint32_t)box[2]);
        int dir[3];
        for (dir[0] = -1; dir[0] <= 1; dir[0]++)
            for (dir[1] = -1; dir[1] <= 1; dir[1]++)
                for (dir[2] = -1; dir[2] <= 1; dir[2]++) {
                    int opos[3];
                    double delta[3];
                    relative_cell(box, pos, dir, opos, delta);
                    uint32_t oc = (uint32_t)(opos[0] * box[1] * box[2] + opos[1] * box[2] + opos[2]);
                    for (uint32_t ko = cl->start[oc]; ko < cl->start[oc + 1]; ko++) {
                        uint32_t o = cl->beads[ko];
                        for (uint32_t kh = cl->start[c]; kh < cl->start[c + 1]; kh++) {
                            uint32_t h = cl->beads[kh];
                            if (h >= o) continue; /* each unordered pair once */
                            double dx[3];
                            for (int d = 0; d < 3; d++) dx[d] = w->x[3 * h + d] - (w->x[3 * o + d] + delta[d]);
                            double dr2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
                            if (dr2 >= 1 || dr2 <= 0) continue;
                            double dr = sqrt(dr2);
                            uint32_t th = w->hash[h] >> 28, to = w->hash[o] >> 28;
                            double a = w->conservative[th * nt + to];
                            if (w->cell_conservative) { /* spatial: mean of the two cells' values */
                                const size_t n2 = (size_t)nt * nt, k = (size_t)th * nt + to;
                                a = (w->cell_conservative[c * n2 + k] + w->cell_conservative[oc * n2 + k]) * 0.5;
                            }
                            vir += a * (1.0 - dr) * dr; /* r . F^C = a (1-r) r */
                            if (job->rdf) {
                                uint32_t lo = th < to ? th : to, hi = th < to ? to : th;
                                uint32_t bin = (uint32_t)(dr * job->n_bins);
                                if (bin >= job->n_bins) bin = job->n_bins - 1;
                                job->rdf[(size_t)(lo * nt + hi) * job->n_bins + bin]++;
                            }
                        }
                    }
                }
    }
    job->virial = vir;
    return NULL;
}

void pdo_observe(const pdo_world *w, int nthreads, pdo_observables *obs,
                 uint32_t n_bins, uint64_t *rdf, uint32_t n_bond_bins, uint64_t *bond_hist)
{
    if (nthreads < 1) nthreads = 1;
    double ke2 = 0, mom[3] = {0, 0, 0};
    for (uint32_t i = 0; i < w->n_beads; i++) {
        for (int d = 0; d < 3; d++) {
            double v = w->v[3 * i + d];
            ke2 += v * v;
            mom[d] += v;
        }
    }
    uint32_t *cell_of = (uint32_t *)malloc(sizeof(uint32_t) * (w->n_beads ? w->n_beads : 1));
    cell_list cl;
    build_cells(w, &cl, cell_of);
    size_t rdf_len = (size_t)w->n_types * w->n_types * n_bins;
    obs_job *jobs = (obs_job *)calloc((size_t)nthreads, sizeof(obs_job));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    uint32_t per = (cl.n_cells + (uint32_t)nthreads - 1) / (uint32_t)nthreads;
    for (int i = 0; i < nthreads; i++) {
        jobs[i].w = w;
        jobs[i].cl = &cl;
        uint32_t b = per * (uint32_t)i, e = b + per;
        jobs[i].cell_begin = b < cl.n_cells ? b : cl.n_cells;
        jobs[i].cell_end = e < cl.n_cells ? e : cl.n_cells;
        jobs[i].n_bins = n_bins;
        jobs[i].rdf = rdf ? (uint64_t *)calloc(rdf_len ? rdf_len : 1, sizeof(uint64_t)) : NULL;
    }
    for (int i = 1; i < nthreads; i++) pthread_create(&th[i], NULL, obs_worker, &jobs[i]);
    obs_worker(&jobs[0]);
    for (int i = 1; i < nthreads; i++) pthread_join(th[i], NULL);
    double vir = 0;
    if (rdf) memset(rdf, 0, rdf_len * sizeof(uint64_t));
    for (int i = 0; i < nthreads; i++) {
        vir += jobs[i].virial;
        if (rdf) {
            for (size_t k = 0; k < rdf_len; k++) rdf[k] += jobs[i].rdf[k];
            free(jobs[i].rdf);
        }
    }
    if (bond_hist) memset(bond_hist, 0, sizeof(uint64_t) * n_bond_bins);
    for (uint32_t k = 0; k < w->n_bonds; k++) {
        uint32_t h = w->bond_beads[2 * k], t = w->bond_beads[2 * k + 1];
        double dx[3];
        distance_from_to(w->box, &w->x[3 * h], &w->x[3 * t], dx);
        double dr = l2_norm(dx);
        double fmag = w->bond_kappa[k] * (w->bond_r0[k] - dr); /* along +dx on the tail */
        vir += fmag * dr;
        if (bond_hist && n_bond_bins) {
            uint32_t bin = (uint32_t)(dr / 2.0 * n_bond_bins);
            if (bin >= n_bond_bins) bin = n_bond_bins - 1;
            bond_hist[bin]++;
        }
    }
    if (obs) {
        obs->ke2 = ke2;
        obs->virial = vir;
        for (int d = 0; d < 3; d++) obs->momentum[d] = mom[d];
    }
    free(jobs);
    free(th);
    free(cell_of);
    free_cells(&cl);
}
