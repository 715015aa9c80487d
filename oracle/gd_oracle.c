/* CPU oracle for gdock's scoring and FCC clustering (FP64 restatement).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path and the timed CPU
 * baseline.  Built with -ffp-contract=off so that every a*b+c is two
 * roundings, as in the reference (Rust never fuses multiply-adds).
 * Expression shapes follow the reference line by line; comments cite the
 * gdock source (path:line) each function restates.
 */
#include "gd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define PI_F64 3.141592653589793 /* std::f64::consts::PI */

/* constants: src/constants.rs:59-64 */
static const double VDW_CUTOFF = 12.0;
static const double SOFTCORE_ALPHA = 0.5;
static const double DESOLV_CUTOFF = 8.0;
static const double ELEC_CUTOFF = 15.0;
static const double ELEC_MIN_DISTANCE = 1.0;
static const double AIR_FORCE_CONSTANT = 10.0;

/* structure::distance, src/structure.rs:312-317 */
static inline double distance_xyz(double ax, double ay, double az, double bx, double by, double bz) {
  double dx = ax - bx;
  double dy = ay - by;
  double dz = az - bz;
  return sqrt(dx * dx + dy * dy + dz * dz);
}

/* f64::powi(x, 6) as LLVM expands it: x^2 * (x^2)^2 */
static inline double powi6(double x) {
  double x2 = x * x;
  double x4 = x2 * x2;
  return x2 * x4;
}

/* Molecule::center_of_mass, src/structure.rs:63-69 (left fold, then / n) */
void orc_center_of_mass(const orc_mol *m, double out[3]) {
  double sx = -0.0, sy = -0.0, sz = -0.0;
  for (int32_t i = 0; i < m->n; i++) sx += m->x[i];
  for (int32_t i = 0; i < m->n; i++) sy += m->y[i];
  for (int32_t i = 0; i < m->n; i++) sz += m->z[i];
  double n = (double)m->n;
  out[0] = sx / n;
  out[1] = sy / n;
  out[2] = sz / n;
}

/* Chromosome::apply_genes (src/chromosome.rs:79-83) =
 * Molecule::rotate (src/structure.rs:80-117) then displace (:119-131). */
void orc_apply_genes(const orc_mol *lig, const double g[6], double *ox, double *oy, double *oz) {
  double c[3];
  orc_center_of_mass(lig, c);
  double alpha = g[0], beta = g[1], gamma = g[2];
  for (int32_t i = 0; i < lig->n; i++) {
    double x = lig->x[i] - c[0];
    double y = lig->y[i] - c[1];
    double z = lig->z[i] - c[2];
    double new_x = x * cos(alpha) * cos(beta) +
                   y * (-sin(alpha) * cos(gamma) + cos(alpha) * sin(beta) * sin(gamma)) +
                   z * (sin(alpha) * sin(gamma) + cos(alpha) * sin(beta) * cos(gamma));
    double new_y = x * sin(alpha) * cos(beta) +
                   y * (cos(alpha) * cos(gamma) + sin(alpha) * sin(beta) * sin(gamma)) +
                   z * (-cos(alpha) * sin(gamma) + sin(alpha) * sin(beta) * cos(gamma));
    double new_z = -x * sin(beta) + y * cos(beta) * sin(gamma) + z * cos(beta) * cos(gamma);
    x = new_x + c[0];
    y = new_y + c[1];
    z = new_z + c[2];
    ox[i] = x + g[3];
    oy[i] = y + g[4];
    oz[i] = z + g[5];
  }
}

/* softcore_lj_potential, src/fitness.rs:57-70 */
static inline double softcore_lj(double e1, double r1, double e2, double r2, double distance, double alpha) {
  double epsilon_ij = sqrt(e1 * e2);
  double rmin_ij = r1 + r2;
  double rmin6 = powi6(rmin_ij);
  double r6 = powi6(distance);
  double r_eff6 = r6 + alpha * rmin6;
  double ratio = rmin6 / r_eff6;
  return epsilon_ij * (ratio * ratio - 2.0 * ratio);
}

/* f64::clamp */
static inline double clamp_f64(double v, double lo, double hi) {
  if (v < lo) return lo;
  if (v > hi) return hi;
  return v;
}

/* vdw_energy, src/fitness.rs:86-105 (pairs with equal serials are skipped) */
double orc_vdw_energy(const orc_mol *rec, const orc_mol *lig) {
  double energy = 0.0;
  for (int32_t i = 0; i < rec->n; i++) {
    for (int32_t j = 0; j < lig->n; j++) {
      if (rec->serial[i] != lig->serial[j]) {
        double dist = distance_xyz(rec->x[i], rec->y[i], rec->z[i], lig->x[j], lig->y[j], lig->z[j]);
        if (dist > 0.0 && dist < VDW_CUTOFF) {
          double vdw = softcore_lj(rec->epsilon[i], rec->rmin2[i], lig->epsilon[j], lig->rmin2[j], dist,
                                   SOFTCORE_ALPHA);
          energy += clamp_f64(vdw, -50.0, 500.0);
        }
      }
    }
  }
  return energy;
}

/* elec_energy, src/fitness.rs:284-302 (epsilon = r dielectric) */
double orc_elec_energy(const orc_mol *rec, const orc_mol *lig) {
  const double k = 332.0636;
  double energy = 0.0;
  for (int32_t i = 0; i < rec->n; i++) {
    for (int32_t j = 0; j < lig->n; j++) {
      double dist = distance_xyz(rec->x[i], rec->y[i], rec->z[i], lig->x[j], lig->y[j], lig->z[j]);
      if (dist > ELEC_MIN_DISTANCE && dist < ELEC_CUTOFF) {
        energy += k * (rec->charge[i] * lig->charge[j]) / (dist * dist);
      }
    }
  }
  return energy;
}

/* get_asp closure, src/fitness.rs:129-138 */
static inline double asp_of(uint8_t elem) {
  switch (elem) {
    case ORC_ELEM_C: return 0.012;
    case ORC_ELEM_N: return -0.160;
    case ORC_ELEM_O: return -0.160;
    case ORC_ELEM_S: return 0.012;
    default: return 0.0;
  }
}

/* desolv_energy, src/fitness.rs:122-184 */
double orc_desolv_energy(const orc_mol *rec, const orc_mol *lig) {
  double energy = 0.0;
  for (int32_t i = 0; i < rec->n; i++) {
    double asp1 = asp_of(rec->element[i]);
    if (fabs(asp1) < 0.001) continue;
    int64_t burial_count = 0;
    for (int32_t j = 0; j < lig->n; j++) {
      double dist = distance_xyz(rec->x[i], rec->y[i], rec->z[i], lig->x[j], lig->y[j], lig->z[j]);
      if (dist < DESOLV_CUTOFF) burial_count += 1;
    }
    double burial = (double)burial_count / 10.0;
    if (!(burial < 1.0)) burial = 1.0; /* f64::min(1.0) for finite values */
    energy -= asp1 * burial * rec->vdw_radius[i] * rec->vdw_radius[i] * 4.0 * PI_F64;
  }
  for (int32_t j = 0; j < lig->n; j++) {
    double asp2 = asp_of(lig->element[j]);
    if (fabs(asp2) < 0.001) continue;
    int64_t burial_count = 0;
    for (int32_t i = 0; i < rec->n; i++) {
      double dist = distance_xyz(rec->x[i], rec->y[i], rec->z[i], lig->x[j], lig->y[j], lig->z[j]);
      if (dist < DESOLV_CUTOFF) burial_count += 1;
    }
    double burial = (double)burial_count / 10.0;
    if (!(burial < 1.0)) burial = 1.0;
    energy -= asp2 * burial * lig->vdw_radius[j] * lig->vdw_radius[j] * 4.0 * PI_F64;
  }
  return energy;
}

/* the first atom named CA with a residue number (src/fitness.rs:219-227,
 * src/restraints.rs:20-29) */
static int32_t find_ca(const orc_mol *m, int32_t resseq) {
  for (int32_t i = 0; i < m->n; i++)
    if ((int32_t)m->resseq[i] == resseq && m->is_ca[i]) return i;
  return -1;
}

/* create_restraints_from_pairs, src/restraints.rs:44-77: keep the pairs whose
 * two CAs exist.  kept_pairs may be NULL. */
int32_t orc_count_restraints(const int32_t *pairs, int32_t k, const orc_mol *rec, const orc_mol *lig,
                             int32_t *kept_pairs) {
  int32_t m = 0;
  for (int32_t r = 0; r < k; r++) {
    if (find_ca(rec, pairs[2 * r]) >= 0 && find_ca(lig, pairs[2 * r + 1]) >= 0) {
      if (kept_pairs) {
        kept_pairs[2 * m] = pairs[2 * r];
        kept_pairs[2 * m + 1] = pairs[2 * r + 1];
      }
      m++;
    }
  }
  return m;
}

/* air_energy, src/fitness.rs:205-249 (flat bottom [0, 7], k = 10) */
double orc_air_energy(const int32_t *pairs, int32_t k, const orc_mol *rec, const orc_mol *lig) {
  double energy = 0.0;
  const double lower_bound = 0.0, upper_bound = 7.0;
  for (int32_t r = 0; r < k; r++) {
    int32_t a = find_ca(rec, pairs[2 * r]);
    int32_t b = find_ca(lig, pairs[2 * r + 1]);
    if (a >= 0 && b >= 0) {
      double dist = distance_xyz(rec->x[a], rec->y[a], rec->z[a], lig->x[b], lig->y[b], lig->z[b]);
      double violation;
      if (dist < lower_bound) violation = lower_bound - dist;
      else if (dist > upper_bound) violation = dist - upper_bound;
      else violation = 0.0;
      energy += AIR_FORCE_CONSTANT * violation * violation;
    }
  }
  return energy;
}

/* satisfaction_ratio + Restraint::is_satisfied (src/fitness.rs:251-267,
 * src/restraints.rs:11-40) */
double orc_satisfaction_ratio(const int32_t *pairs, int32_t k, const orc_mol *rec, const orc_mol *lig) {
  int32_t satisfied = 0;
  for (int32_t r = 0; r < k; r++) {
    int32_t a = find_ca(rec, pairs[2 * r]);
    int32_t b = find_ca(lig, pairs[2 * r + 1]);
    if (a >= 0 && b >= 0) {
      double dist = distance_xyz(rec->x[a], rec->y[a], rec->z[a], lig->x[b], lig->y[b], lig->z[b]);
      if (dist <= 7.0) satisfied++;
    }
  }
  if (k > 0) return (double)satisfied / (double)k;
  return 0.0;
}

static void score_lig(const orc_mol *rec, const orc_mol *moved, const int32_t *pairs, int32_t k,
                      const orc_weights *w, orc_energy *o) {
  o->vdw = orc_vdw_energy(rec, moved);
  o->elec = orc_elec_energy(rec, moved);
  o->desolv = orc_desolv_energy(rec, moved);
  o->air = orc_air_energy(pairs, k, rec, moved);
  double ratio = orc_satisfaction_ratio(pairs, k, rec, moved);
  o->restraint_penalty = (1.0 - ratio) * (double)k;
  /* src/chromosome.rs:121-124 */
  o->fitness = w->vdw * o->vdw + w->elec * o->elec + w->desolv * o->desolv + w->air * o->air;
}

/* Chromosome::fitness, src/chromosome.rs:85-128 (energy mode) */
void orc_fitness(const orc_mol *rec, const orc_mol *lig, const int32_t *pairs, int32_t k,
                 const orc_weights *w, const double genes[6], orc_energy *out) {
  double *buf = (double *)malloc(sizeof(double) * 3 * (size_t)(lig->n > 0 ? lig->n : 1));
  double *x = buf, *y = buf + lig->n, *z = buf + 2 * lig->n;
  orc_apply_genes(lig, genes, x, y, z);
  orc_mol moved = *lig;
  moved.x = x;
  moved.y = y;
  moved.z = z;
  score_lig(rec, &moved, pairs, k, w, out);
  free(buf);
}

typedef struct {
  const orc_mol *rec, *lig;
  const int32_t *pairs;
  int32_t k;
  const orc_weights *w;
  const double *genes; /* or model coordinates */
  int32_t n, models;
  orc_energy *out;
  int32_t next;
  pthread_mutex_t mu;
} pool_job;

static void *pool_worker(void *arg) {
  pool_job *j = (pool_job *)arg;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    int32_t p = j->next++;
    pthread_mutex_unlock(&j->mu);
    if (p >= j->n) break;
    if (j->models) {
      int32_t nl = j->lig->n;
      const double *xyz = j->genes + (size_t)p * 3 * (size_t)nl;
      double *buf = (double *)malloc(sizeof(double) * 3 * (size_t)(nl > 0 ? nl : 1));
      for (int32_t a = 0; a < nl; a++) {
        buf[a] = xyz[3 * a];
        buf[nl + a] = xyz[3 * a + 1];
        buf[2 * nl + a] = xyz[3 * a + 2];
      }
      orc_mol moved = *j->lig;
      moved.x = buf;
      moved.y = buf + nl;
      moved.z = buf + 2 * nl;
      score_lig(j->rec, &moved, j->pairs, j->k, j->w, &j->out[p]);
      free(buf);
    } else {
      orc_fitness(j->rec, j->lig, j->pairs, j->k, j->w, j->genes + 6 * (size_t)p, &j->out[p]);
    }
  }
  return NULL;
}

static void run_pool(pool_job *job, int32_t nthreads) {
  if (nthreads < 1) nthreads = 1;
  pthread_mutex_init(&job->mu, NULL);
  job->next = 0;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
  for (int32_t t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, pool_worker, job);
  for (int32_t t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&job->mu);
}

/* Population::eval_fitness, src/population.rs:48-61 (a parallel map) */
void orc_score_poses(const orc_mol *rec, const orc_mol *lig, const int32_t *pairs, int32_t k,
                     const orc_weights *w, const double *genes, int32_t n, orc_energy *out,
                     int32_t nthreads) {
  pool_job job;
  memset(&job, 0, sizeof job);
  job.rec = rec; job.lig = lig; job.pairs = pairs; job.k = k; job.w = w;
  job.genes = genes; job.n = n; job.models = 0; job.out = out;
  run_pool(&job, nthreads);
}

/* commands::score::score, src/commands/score.rs:32-79: each model's
 * coordinates scored as given (xyz: n_models x n_lig x 3) */
void orc_score_models(const orc_mol *rec, const orc_mol *lig, const int32_t *pairs, int32_t k,
                      const orc_weights *w, const double *xyz, int32_t n_models, orc_energy *out,
                      int32_t nthreads) {
  pool_job job;
  memset(&job, 0, sizeof job);
  job.rec = rec; job.lig = lig; job.pairs = pairs; job.k = k; job.w = w;
  job.genes = xyz; job.n = n_models; job.models = 1; job.out = out;
  run_pool(&job, nthreads);
}

/* ---------------------------------------------------------------- FCC -- */

static int cmp_i64(const void *a, const void *b) {
  int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}

typedef struct { uint8_t chain; int16_t resseq; int32_t first; int32_t count; } residue_grp;

static int cmp_atom_key(const void *a, const void *b) {
  const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}

/* calculate_contacts, src/clustering.rs:62-115.  Residues are keyed by
 * (chain, resseq) over non-hydrogen atoms; a contact is any atom pair of two
 * residues on different chains within cutoff (<=). */
int32_t orc_contacts(const orc_mol *m, double cutoff, int64_t *keys, int32_t cap) {
  int32_t n = m->n;
  /* sort heavy atoms by residue key, stable by index */
  int64_t *ak = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  int32_t nh = 0;
  for (int32_t i = 0; i < n; i++) {
    if (m->element[i] == ORC_ELEM_H) continue;
    int64_t key = ((int64_t)m->chain[i] << 16) | (int64_t)(uint16_t)m->resseq[i];
    ak[nh++] = (key << 32) | (int64_t)i;
  }
  qsort(ak, (size_t)nh, sizeof(int64_t), cmp_atom_key);
  residue_grp *g = (residue_grp *)malloc(sizeof(residue_grp) * (size_t)(nh > 0 ? nh : 1));
  int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nh > 0 ? nh : 1));
  int32_t ng = 0;
  for (int32_t a = 0; a < nh; a++) {
    int64_t key = ak[a] >> 32;
    idx[a] = (int32_t)(ak[a] & 0xffffffff);
    if (ng == 0 || (((int64_t)g[ng - 1].chain << 16) | (uint16_t)g[ng - 1].resseq) != key) {
      g[ng].chain = (uint8_t)(key >> 16);
      g[ng].resseq = (int16_t)(uint16_t)(key & 0xffff);
      g[ng].first = a;
      g[ng].count = 0;
      ng++;
    }
    g[ng - 1].count++;
  }
  int32_t nk = 0;
  for (int32_t i = 0; i < ng; i++) {
    for (int32_t j = i + 1; j < ng; j++) {
      if (g[i].chain == g[j].chain) continue;
      int found = 0;
      for (int32_t a = 0; a < g[i].count && !found; a++) {
        int32_t ia = idx[g[i].first + a];
        for (int32_t b = 0; b < g[j].count; b++) {
          int32_t ib = idx[g[j].first + b];
          double dx = m->x[ia] - m->x[ib], dy = m->y[ia] - m->y[ib], dz = m->z[ia] - m->z[ib];
          double dist = sqrt(dx * dx + dy * dy + dz * dz);
          if (dist <= cutoff) {
            found = 1;
            break;
          }
        }
      }
      if (found) {
        const residue_grp *lo = g[i].chain < g[j].chain ? &g[i] : &g[j];
        const residue_grp *hi = g[i].chain < g[j].chain ? &g[j] : &g[i];
        int64_t key = ((int64_t)lo->chain << 48) | ((int64_t)(uint16_t)lo->resseq << 32) |
                      ((int64_t)hi->chain << 16) | (int64_t)(uint16_t)hi->resseq;
        if (nk < cap) keys[nk] = key;
        nk++;
      }
    }
  }
  free(ak);
  free(g);
  free(idx);
  int32_t out = nk < cap ? nk : cap;
  qsort(keys, (size_t)out, sizeof(int64_t), cmp_i64);
  return nk;
}

/* the complex of receptor + ligand moved by the genes
 * (src/commands/run.rs:666-684 then combine_molecules) */
int32_t orc_pose_contacts(const orc_mol *rec, const orc_mol *lig, const double genes[6], double cutoff,
                          int64_t *keys, int32_t cap) {
  int32_t n = rec->n + lig->n;
  double *buf = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  double *x = buf, *y = buf + n, *z = buf + 2 * n;
  memcpy(x, rec->x, sizeof(double) * (size_t)rec->n);
  memcpy(y, rec->y, sizeof(double) * (size_t)rec->n);
  memcpy(z, rec->z, sizeof(double) * (size_t)rec->n);
  orc_apply_genes(lig, genes, x + rec->n, y + rec->n, z + rec->n);
  uint8_t *chain = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
  uint8_t *elem = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
  int16_t *resseq = (int16_t *)malloc(sizeof(int16_t) * (size_t)(n > 0 ? n : 1));
  memcpy(chain, rec->chain, (size_t)rec->n);
  memcpy(chain + rec->n, lig->chain, (size_t)lig->n);
  memcpy(elem, rec->element, (size_t)rec->n);
  memcpy(elem + rec->n, lig->element, (size_t)lig->n);
  memcpy(resseq, rec->resseq, sizeof(int16_t) * (size_t)rec->n);
  memcpy(resseq + rec->n, lig->resseq, sizeof(int16_t) * (size_t)lig->n);
  orc_mol cx;
  memset(&cx, 0, sizeof cx);
  cx.n = n;
  cx.x = x;
  cx.y = y;
  cx.z = z;
  cx.chain = chain;
  cx.element = elem;
  cx.resseq = resseq;
  int32_t r = orc_contacts(&cx, cutoff, keys, cap);
  free(buf);
  free(chain);
  free(elem);
  free(resseq);
  return r;
}

/* |X intersect Y| of two sorted key lists */
static int64_t common_count(const int64_t *a, int64_t na, const int64_t *b, int64_t nb) {
  int64_t i = 0, j = 0, c = 0;
  while (i < na && j < nb) {
    if (a[i] < b[j]) i++;
    else if (a[i] > b[j]) j++;
    else {
      c++;
      i++;
      j++;
    }
  }
  return c;
}

/* calculate_fcc, src/clustering.rs:122-132 */
static void fcc_pair(const int64_t *keys, const int64_t *off, int32_t i, int32_t j, double *fcc, double *fcc_v) {
  int64_t ni = off[i + 1] - off[i], nj = off[j + 1] - off[j];
  if (ni == 0 || nj == 0) {
    *fcc = 0.0;
    *fcc_v = 0.0;
    return;
  }
  double common = (double)common_count(keys + off[i], ni, keys + off[j], nj);
  *fcc = common / (double)ni;
  *fcc_v = common / (double)nj;
}

void orc_pairwise_fcc(const int64_t *keys, const int64_t *offsets, int32_t n, double *fcc, double *fcc_v) {
  for (int32_t i = 0; i < n; i++)
    for (int32_t j = 0; j < n; j++)
      fcc_pair(keys, offsets, i, j, &fcc[(size_t)i * n + j], &fcc_v[(size_t)i * n + j]);
}

typedef struct { int32_t center, size, first; } cl_rec;

/* create_elements + cluster_elements + the size filter of cluster_structures
 * (src/clustering.rs:151-254, 265-293) */
int32_t orc_cluster(const int64_t *keys, const int64_t *offsets, int32_t n, double fcc_cutoff,
                    double strictness, int32_t min_size, int32_t *centers, int32_t *sizes,
                    int32_t *members) {
  if (n <= 0) return 0;
  uint8_t *nb = (uint8_t *)calloc((size_t)n * (size_t)n, 1);
  for (int32_t i = 0; i < n; i++) {
    for (int32_t j = 0; j < n; j++) {
      double fcc, fcc_v;
      fcc_pair(keys, offsets, i, j, &fcc, &fcc_v);
      if (fcc >= fcc_cutoff && fcc_v >= fcc_cutoff * strictness) nb[(size_t)i * n + j] = 1;
      if (fcc_v >= fcc_cutoff && fcc >= fcc_cutoff * strictness) nb[(size_t)j * n + i] = 1;
    }
  }
  uint8_t *used = (uint8_t *)calloc((size_t)n, 1);
  cl_rec *cl = (cl_rec *)malloc(sizeof(cl_rec) * (size_t)n);
  int32_t *mem = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  int32_t ncl = 0, nmem = 0;
  for (;;) {
    int32_t center = -1;
    int64_t best = -1;
    for (int32_t e = 0; e < n; e++) {
      if (used[e]) continue;
      int64_t cnt = 0;
      for (int32_t f = 0; f < n; f++)
        if (nb[(size_t)e * n + f] && !used[f]) cnt++;
      if (cnt > best) { /* strict: ties keep the lower index */
        best = cnt;
        center = e;
      }
    }
    if (center < 0) break;
    int32_t first = nmem;
    mem[nmem++] = center;
    for (int32_t f = 0; f < n; f++) {
      if (f != center && nb[(size_t)center * n + f] && !used[f]) {
        mem[nmem++] = f;
        used[f] = 1;
      }
    }
    used[center] = 1;
    /* members sorted ascending */
    for (int32_t a = first + 1; a < nmem; a++) {
      int32_t v = mem[a], b = a - 1;
      while (b >= first && mem[b] > v) {
        mem[b + 1] = mem[b];
        b--;
      }
      mem[b + 1] = v;
    }
    cl[ncl].center = center;
    cl[ncl].size = nmem - first;
    cl[ncl].first = first;
    ncl++;
  }
  /* stable sort by size descending */
  for (int32_t a = 1; a < ncl; a++) {
    cl_rec v = cl[a];
    int32_t b = a - 1;
    while (b >= 0 && cl[b].size < v.size) {
      cl[b + 1] = cl[b];
      b--;
    }
    cl[b + 1] = v;
  }
  int32_t kept = 0, mo = 0;
  for (int32_t c = 0; c < ncl; c++) {
    if (cl[c].size < min_size) continue;
    centers[kept] = cl[c].center;
    sizes[kept] = cl[c].size;
    memcpy(members + mo, mem + cl[c].first, sizeof(int32_t) * (size_t)cl[c].size);
    mo += cl[c].size;
    kept++;
  }
  free(nb);
  free(used);
  free(cl);
  free(mem);
  return kept;
}

/* ------------------------------------------------------------------ GA -- */

/* stable ascending order of fitness (slice::sort_by with partial_cmp) */
static void stable_order(int32_t n, const double *f, int descending, int32_t *order) {
  for (int32_t i = 0; i < n; i++) order[i] = i;
  /* insertion sort: stable */
  for (int32_t i = 1; i < n; i++) {
    int32_t v = order[i], j = i - 1;
    while (j >= 0 && (descending ? (f[order[j]] < f[v]) : (f[order[j]] > f[v]))) {
      order[j + 1] = order[j];
      j--;
    }
    order[j + 1] = v;
  }
}

void orc_evolve(int32_t n, const double *genes, const double *fitness, int32_t elitism,
                const int32_t *tour, int32_t tour_size, const int32_t *perm, const double *cross_u,
                double crossover_rate, const double *mut_u, const double *mut_z, double mutation_rate,
                double max_displacement, double *genes_out, double *fit_out) {
  const double TWO_PI = 2.0 * PI_F64;
  int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  int32_t *sel = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  /* elitism: stable sort ascending, take the first `elitism` (:76-82) */
  stable_order(n, fitness, 0, order);
  int32_t ne = elitism < n ? elitism : n;
  int32_t elite[64];
  for (int32_t i = 0; i < ne && i < 64; i++) elite[i] = order[i];
  /* tournament: the first minimum of tour_size draws (:136-156) */
  for (int32_t k = 0; k < n; k++) {
    int32_t best = tour[tour_size * k];
    for (int32_t t = 1; t < tour_size; t++) {
      int32_t c = tour[tour_size * k + t];
      if (fitness[best] > fitness[c]) best = c;
    }
    sel[k] = best;
  }
  /* shuffle then pairwise crossover; an odd last individual is dropped (:88-99) */
  int32_t m = 2 * (n / 2);
  double *g2 = (double *)malloc(sizeof(double) * 6 * (size_t)(m > 0 ? m : 1));
  double *f2 = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
  for (int32_t p = 0; p < n / 2; p++) {
    int32_t a = sel[perm[2 * p]], b = sel[perm[2 * p + 1]];
    for (int32_t g = 0; g < 6; g++) {
      double ga = genes[6 * a + g], gb = genes[6 * b + g];
      if (cross_u[6 * p + g] <= crossover_rate) {
        g2[6 * (2 * p) + g] = gb;
        g2[6 * (2 * p + 1) + g] = ga;
      } else {
        g2[6 * (2 * p) + g] = ga;
        g2[6 * (2 * p + 1) + g] = gb;
      }
    }
    f2[2 * p] = fitness[a];
    f2[2 * p + 1] = fitness[b];
  }
  /* creep mutation (src/chromosome.rs:56-77) */
  for (int32_t k = 0; k < m; k++) {
    for (int32_t g = 0; g < 6; g++) {
      if (mut_u[6 * k + g] <= mutation_rate) {
        double v = g2[6 * k + g] + mut_z[6 * k + g];
        if (g < 3) {
          double r = fmod(v, TWO_PI); /* f64::rem_euclid */
          if (r < 0.0) r = r + fabs(TWO_PI);
          v = r;
        } else {
          if (v < -max_displacement) v = -max_displacement;
          if (v > max_displacement) v = max_displacement;
        }
        g2[6 * k + g] = v;
      }
    }
  }
  /* stable sort descending by the carried fitness, elites over the first
   * slots (:110-118) */
  stable_order(m, f2, 1, order);
  for (int32_t k = 0; k < m; k++) {
    for (int32_t g = 0; g < 6; g++) genes_out[6 * k + g] = g2[6 * order[k] + g];
    fit_out[k] = f2[order[k]];
  }
  for (int32_t i = 0; i < ne && i < m; i++) {
    for (int32_t g = 0; g < 6; g++) genes_out[6 * i + g] = genes[6 * elite[i] + g];
    fit_out[i] = fitness[elite[i]];
  }
  free(order);
  free(sel);
  free(g2);
  free(f2);
}
