/* Oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's FP64 half-step DPD integrator
 * (NaiveDPDEngineHalfStep, include/dpd/engines/naive/naive_dpd_engine_half_step.hpp) and of
 * the hash RNG it draws from (include/dpd/core/hash.hpp).  Only tests/, the smoke check and
 * bench.py's CPU-baseline / reference arm may load it, and only as the checker or as the
 * timed CPU baseline.  The GPU engine never calls it.
 *
 * Parity is pinned against the reference itself: tests/golden/ holds outputs of the
 * reference's own engines (compiled unchanged from the reference headers by
 * oracle/ref/Makefile) and tests/test_oracle.py requires this file to reproduce them
 * bit for bit.
 */
#ifndef PDPD_ORACLE_H
#define PDPD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A world in flat form: the same information the engine's C ABI receives. */
typedef struct pdo_world {
    int32_t box[3];
    double dt;
    double lambda;
    uint64_t seed;
    int64_t t;
    uint32_t n_types;
    const double *conservative;  /* n_types*n_types, row-major a_ij */
    const double *dissipative;   /* n_types*n_types, gamma_ij */
    uint32_t n_beads;
    const uint32_t *hash;        /* BeadHash of each bead, by bead id */
    double *x, *v, *f;           /* 3*n_beads, xyz per bead, by bead id */
    uint32_t n_bonds;
    const uint32_t *bond_beads;  /* 2*n_bonds: head, tail */
    const double *bond_kappa, *bond_r0;
    uint32_t n_angles;
    const uint32_t *angle_beads; /* 3*n_angles: head, middle, tail */
    const double *angle_kappa, *angle_theta0;
    uint32_t stationary;         /* bit k set: bead type k is stationary (BeadType::stationary) */
    /* Spatially varying strengths (NULL: the matrices above everywhere): per cell (x-major, z
       fastest) n_types^2 values of a_ij and of gamma_ij. */
    const double *cell_conservative, *cell_dissipative;
} pdo_world;

/* hash.hpp:20-30 */
uint64_t pdo_mix64_m2(uint64_t x);
/* hash.hpp:61-65 */
uint64_t pdo_t_hash(uint32_t t, uint64_t seed);
/* hash.hpp:81-88 */
uint32_t pdo_hash_rng_sym(uint64_t t_hash, uint32_t a, uint32_t b);
/* dpd_maths_core.hpp:55-79 */
float pdo_default_hash(uint64_t t_hash, uint32_t a, uint32_t b);

/* Bulk versions for the known-answer tests: n records. */
void pdo_hash_batch(size_t n, const uint32_t *t, const uint64_t *seed, const uint32_t *a,
                    const uint32_t *b, uint64_t *t_hash_out, uint32_t *h_out, float *u_out);

/* Advance the world by nsteps with the half-step integrator.  nthreads <= 1 runs serially.
 * Returns 0, or -1 with a message in err (a snapped bond, a bead outside the box, an invalid
 * box).  The results do not depend on nthreads. */
int pdo_run(pdo_world *w, uint32_t nsteps, int nthreads, char *err, size_t errlen);

/* Cell index of every bead: floor(x) per dimension, cx*Ly*Lz + cy*Lz + cz
 * (naive_dpd_engine_half_step.hpp:155-168). */
void pdo_cell_index(const pdo_world *w, uint32_t *cell_out);

/* Observables of the current state (FP64), for the statistical comparisons:
 *   ke2        = sum over beads of |v|^2
 *   virial     = sum over interacting pairs i<j of r_ij . F^C_ij (conservative part only)
 *                + sum over Hookean bonds of r . F + angle-bond virial
 *   rdf        = pair-distance histogram for r < 1, n_bins bins, per unordered type pair
 *                (index ti*n_types+tj with ti<=tj), layout [n_types*n_types][n_bins]
 *   bond_hist  = Hookean bond-length histogram over [0, 2), n_bond_bins bins
 *   momentum   = total momentum (3)
 * Any output pointer may be NULL. */
typedef struct pdo_observables {
    double ke2;
    double virial;
    double momentum[3];
} pdo_observables;
void pdo_observe(const pdo_world *w, int nthreads, pdo_observables *obs,
                 uint32_t n_bins, uint64_t *rdf, uint32_t n_bond_bins, uint64_t *bond_hist);

#ifdef __cplusplus
}
#endif

#endif
