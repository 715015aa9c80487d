/* CPU oracle for gdock's scoring and FCC clustering: a plain-C, FP64
 * restatement of the reference algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker the GPU path is
 * compared against, and the timed CPU baseline; no product code path links,
 * loads or calls it.  Each function cites the gdock source (file:line) whose
 * arithmetic it restates, in the reference's own operation order so that
 * per-pair values and every cutoff decision are reproduced exactly.
 */
#ifndef GD_ORACLE_H
#define GD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element classes (same codes as the C ABI) */
enum { ORC_ELEM_OTHER = 0, ORC_ELEM_H = 1, ORC_ELEM_C = 2, ORC_ELEM_N = 3, ORC_ELEM_O = 4, ORC_ELEM_S = 5 };

typedef struct {
  int32_t n;
  const double *x, *y, *z;
  const double *epsilon, *rmin2, *charge, *vdw_radius;
  const int32_t *serial;
  const int16_t *resseq;
  const uint8_t *chain;
  const uint8_t *element;
  const uint8_t *is_ca;
} orc_mol;

typedef struct { double vdw, elec, desolv, air; } orc_weights;

/* energies of one pose, in the order of gd_pose_energy */
typedef struct { double fitness, vdw, elec, desolv, air, restraint_penalty; } orc_energy;

void orc_center_of_mass(const orc_mol *m, double out[3]);
void orc_apply_genes(const orc_mol *lig, const double genes[6], double *x, double *y, double *z);

double orc_vdw_energy(const orc_mol *rec, const orc_mol *lig);
double orc_elec_energy(const orc_mol *rec, const orc_mol *lig);
double orc_desolv_energy(const orc_mol *rec, const orc_mol *lig);
/* restraints given as residue-number pairs (receptor resseq, ligand resseq) */
double orc_air_energy(const int32_t *pairs, int32_t k, const orc_mol *rec, const orc_mol *lig);
double orc_satisfaction_ratio(const int32_t *pairs, int32_t k, const orc_mol *rec, const orc_mol *lig);
int32_t orc_count_restraints(const int32_t *pairs, int32_t k, const orc_mol *rec, const orc_mol *lig,
                             int32_t *kept_pairs);

/* Chromosome::fitness for one set of genes (restraints already filtered) */
void orc_fitness(const orc_mol *rec, const orc_mol *lig, const int32_t *pairs, int32_t k,
                 const orc_weights *w, const double genes[6], orc_energy *out);
/* Population::eval_fitness over n genes, on nthreads worker threads */
void orc_score_poses(const orc_mol *rec, const orc_mol *lig, const int32_t *pairs, int32_t k,
                     const orc_weights *w, const double *genes, int32_t n, orc_energy *out,
                     int32_t nthreads);
/* score of explicitly given ligand coordinates (the `score` command path) */
void orc_score_models(const orc_mol *rec, const orc_mol *lig, const int32_t *pairs, int32_t k,
                      const orc_weights *w, const double *xyz, int32_t n_models, orc_energy *out,
                      int32_t nthreads);

/* calculate_contacts on a complex (any atom list with chain ids).  Keys are
 * (chainA<<48)|(uint16 resA<<32)|(chainB<<16)|uint16 resB with chainA<chainB,
 * returned sorted ascending.  Returns the number of keys (<= cap). */
int32_t orc_contacts(const orc_mol *complex_, double cutoff, int64_t *keys, int32_t cap);
/* contacts of receptor + ligand moved by genes (the clustering input) */
int32_t orc_pose_contacts(const orc_mol *rec, const orc_mol *lig, const double genes[6], double cutoff,
                          int64_t *keys, int32_t cap);

/* cluster_structures over n sorted contact sets given as offsets into keys.
 * Writes clusters in output order: centers[c], sizes[c], member lists
 * concatenated in members (ascending within each cluster).  Returns the
 * number of clusters kept (size >= min_size). */
int32_t orc_cluster(const int64_t *keys, const int64_t *offsets, int32_t n, double fcc_cutoff,
                    double strictness, int32_t min_size, int32_t *centers, int32_t *sizes,
                    int32_t *members);
/* pairwise FCC values (n*n, row i col j) */
void orc_pairwise_fcc(const int64_t *keys, const int64_t *offsets, int32_t n, double *fcc, double *fcc_v);

/* Population::evolve (src/population.rs:74-121) with every random draw given
 * explicitly, in the order the reference consumes them:
 *   tour[3n]      tournament indices (tournament_selection, :124-158)
 *   perm[n]       the shuffled order: shuffled[k] = selected[perm[k]] (:88)
 *   cross_u[6(n/2)] uniform draws of ga::crossover (src/ga.rs:7-39)
 *   mut_u[6m], mut_z[6m] uniform draws of Chromosome::mutate and the normal
 *                 perturbation drawn when one triggers (src/chromosome.rs:56-77),
 *                 m = 2(n/2).
 * genes_out/fit_out receive m individuals (genes and the stale fitness the
 * reference carries), elites written over the first `elitism` slots. */
void orc_evolve(int32_t n, const double *genes, const double *fitness, int32_t elitism,
                const int32_t *tour, int32_t tour_size, const int32_t *perm, const double *cross_u,
                double crossover_rate, const double *mut_u, const double *mut_z, double mutation_rate,
                double max_displacement, double *genes_out, double *fit_out);
#ifdef __cplusplus
}
#endif
#endif
