/* gdock_gb300 — GB300 (sm_103a) engine for gdock's population fitness
 * evaluation and FCC clustering, behind a plain C ABI.
 *
 * The entry points replace these functions of the gdock (Rust) reference, so
 * that its host code can call one GPU through a thin FFI crate:
 *
 *   Population::eval_fitness          src/population.rs:48-61   -> gd_score_poses
 *   Chromosome::fitness (one pose)    src/chromosome.rs:85-128  -> gd_score_poses (n = 1)
 *   Chromosome::apply_genes           src/chromosome.rs:79-83   -> inside gd_score_poses / gd_cluster
 *   fitness::{vdw,elec,desolv}_energy src/fitness.rs:86-184,284-302 -> gd_score_models
 *   fitness::air_energy, satisfaction_ratio src/fitness.rs:205-267 -> gd_score_* (air, restraint_penalty)
 *   commands::score::score loop       src/commands/score.rs:32-79 -> gd_score_models
 *   restraints::create_restraints_from_pairs src/restraints.rs:44-77 -> gd_complex_create
 *   clustering::calculate_contacts    src/clustering.rs:62-115  -> gd_pose_contacts
 *   clustering::cluster_structures    src/clustering.rs:265-293 -> gd_cluster
 *   Evaluator::new / calc_metrics     src/evaluator.rs:50-144   -> gd_evaluator_create / gd_evaluate_poses
 *   Population::eval_metrics          src/population.rs:63-71   -> gd_evaluate_poses
 *
 * Conventions: every call returns a gd_status; nothing throws or aborts
 * across the ABI.  The library copies all inputs; callers keep ownership of
 * their buffers.  A context belongs to one host thread at a time (serialise
 * externally to share one).  All floating-point outputs are FP64.
 */
#ifndef GDOCK_GB300_H
#define GDOCK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GD_ABI_VERSION 1

typedef enum gd_status {
  GD_OK = 0,
  GD_ERR_INVALID_ARG = 1, /* bad pointer, size or value */
  GD_ERR_OOM = 2,         /* device allocation failed or HBM budget exceeded */
  GD_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  GD_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  GD_ERR_CAPACITY = 5,    /* an output buffer is too small */
  GD_ERR_STATE = 6        /* call not valid in the object's current state */
} gd_status;

typedef enum gd_precision {
  GD_PREC_F64 = 0, /* plain form: FP64 throughout (the correctness reference) */
  GD_PREC_F32 = 1  /* FP32 pair terms, compensated partials, FP64 per-pose reduction,
                      FP64 recheck of every pair near a cutoff */
} gd_precision;

/* element classes, from the trimmed PDB element column (src/structure.rs:241-256) */
enum { GD_ELEM_OTHER = 0, GD_ELEM_H = 1, GD_ELEM_C = 2, GD_ELEM_N = 3, GD_ELEM_O = 4, GD_ELEM_S = 5 };

/* One molecule as structure-of-arrays; the fields of gdock's Atom that the
 * scoring and clustering read (src/structure.rs:27-49). */
typedef struct gd_atoms {
  int32_t n;
  const double *x, *y, *z;
  const double *epsilon;    /* toppar epsilon (kcal/mol, <= 0 for OPLS types) */
  const double *rmin2;      /* toppar Rmin/2 (A) */
  const double *charge;     /* partial charge (e) */
  const double *vdw_radius; /* radius by element (A) */
  const int32_t *serial;    /* PDB serial: equal receptor/ligand serials skip the vdW pair */
  const int16_t *resseq;    /* residue number */
  const uint8_t *chain;     /* chain id character */
  const uint8_t *element;   /* GD_ELEM_* */
  const uint8_t *is_ca;     /* 1 when the atom name is "CA" */
} gd_atoms;

/* EnergyWeights, src/constants.rs:28-56 (defaults 0.4, 0.05, 3.4, 1.0) */
typedef struct gd_weights { double vdw, elec, desolv, air; } gd_weights;

/* The six fields Chromosome::fitness writes (src/chromosome.rs:111-127). */
typedef struct gd_pose_energy {
  double fitness, vdw, elec, desolv, air, restraint_penalty;
} gd_pose_energy;

/* ClusteringConfig, src/clustering.rs:14-35 (defaults 5.0, 0.60, 0.75, 4) */
typedef struct gd_cluster_cfg {
  double contact_distance, fcc_cutoff, strictness;
  int32_t min_cluster_size;
} gd_cluster_cfg;

/* Rotation/translation of one pose as the host precomputes it from its genes
 * (cosines and sines of the three angles with the host's libm, the composite
 * matrix entries in the reference's operation order, the displacement). */
typedef struct gd_pose_frame {
  double ca, sa, cb, sb, cg, sg;
  double m01, m02, m11, m12;
  double dx, dy, dz;
  double pad[3];
} gd_pose_frame;

typedef struct gd_context gd_context;
typedef struct gd_complex gd_complex;

int32_t gd_abi_version(void);
const char *gd_status_string(gd_status s);

/* Context on one CUDA device.  hbm_budget_bytes = 0 means "no limit beyond
 * the device's memory". */
gd_status gd_context_create(int32_t device, uint64_t hbm_budget_bytes, gd_context **out);
gd_status gd_context_destroy(gd_context *ctx);
/* Tuning knobs of the context's kernels (the autotuner sets these).
 *   GD_TUNE_F32_SLOTS: variant of the FP32 scoring kernel: ligand slots per
 *                      lane (2 or 4), plus 16 / 64 to evaluate two / four
 *                      receptor rows per inner step, plus 256 for the
 *                      register cap of five resident CTAs per SM; valid: 4,
 *                      20, 66, 68, 322, 324; 0 = automatic (324).
 *   GD_TUNE_SPLIT:     work items of the FP32 scoring kernel: 0 = automatic
 *                      (the ligand chunks of each pose when their scratch fits
 *                      in 4 GiB and the context's HBM budget, else whole
 *                      poses), 1 = whole poses, 2 = chunks whenever possible.
 *                      Energies are bit-identical either way.
 *   GD_TUNE_FAULT:     failure-detection test only: 1 = the FP32 scoring
 *                      kernel issues no copy for one receptor stage, so that
 *                      stage's bounded wait (2 s) runs out, the kernel drains
 *                      its other copies (bounded) and the call reports
 *                      GD_ERR_TIMEOUT; the context stays usable.  0 = off.
 *   GD_TUNE_FCC:       pair counts of the device FCC: 0 = automatic (by the
 *                      estimated work of each), 1 = popcount over the
 *                      compacted contact bitsets of every pose pair, 2 =
 *                      per-contact lists of the poses that make it (the
 *                      pairs of each list counted with atomics: little work
 *                      when the contacts are spread over many poses, at most
 *                      16,384 poses).  Clusters are identical either way.
 *   GD_TUNE_CONTACTS:  contact pass of gd_pose_contacts: 0 = automatic (the
 *                      per-pose residue-pair bitmaps of the clustering path
 *                      whenever receptor and ligand are single chains that
 *                      share no residue, else per-residue contact lists),
 *                      1 = per-residue contact lists always.  Both decide
 *                      every atom pair exactly; the keys are identical.
 *   GD_TUNE_RPARTS:    receptor parts per ligand chunk of a split FP32
 *                      launch: 0 = automatic (more than one only when the
 *                      launch has too few (pose, chunk) items to fill the
 *                      GPU), 1..8 = that many.  The energies do not depend
 *                      on it (per-segment fixed-point sums).
 * Read-only (gd_context_get_tuning; set_tuning refuses them):
 *   GD_INFO_LAST_FCC:      pair counts of the context's last device
 *                          clustering: 1 bitsets, 2 postings, 0 none yet.
 *   GD_INFO_LAST_CONTACTS: contact pass of the last gd_pose_contacts or
 *                          gd_cluster: 1 lists, 2 bitmaps, 0 none yet. */
enum { GD_TUNE_F32_SLOTS = 0, GD_TUNE_SPLIT = 1, GD_TUNE_FAULT = 2, GD_TUNE_FCC = 3, GD_TUNE_CONTACTS = 4,
       GD_TUNE_RPARTS = 5,
       GD_INFO_LAST_FCC = 16, GD_INFO_LAST_CONTACTS = 17 };
gd_status gd_context_set_tuning(gd_context *ctx, int32_t knob, int32_t value);
/* The FP32 scoring autotuner: times every candidate (GD_TUNE_F32_SLOTS,
 * GD_TUNE_SPLIT) = (20,1) (66,1) (68,1) (322,1) (324,1) (324,2) on n
 * device-resident poses of cx (two launches each, CUDA events on `stream`,
 * NULL = the context's stream) and sets both knobs to the fastest.  rates
 * (may be NULL) receives poses/s per candidate in that order; *best (may be
 * NULL) the index of the chosen one.  The complex's own size and the pose
 * count matter: tune on a sample of the real workload. */
#define GD_AUTOTUNE_CANDIDATES 6
gd_status gd_autotune_f32(gd_complex *cx, const gd_pose_frame *d_frames, int32_t n, double max_displacement,
                          gd_pose_energy *d_out, void *stream, double *rates, int32_t *best);
int32_t gd_context_get_tuning(const gd_context *ctx, int32_t knob);

/* Message of the last failing call on this context ("" if none). */
const char *gd_last_error(const gd_context *ctx);
/* Bytes of device memory the context's objects hold. */
uint64_t gd_context_bytes_in_use(const gd_context *ctx);

/* Upload a receptor and a ligand that is already centred on the receptor
 * (utils::position_ligand, src/utils.rs:77-95).  restraint_pairs holds
 * n_pairs (receptor resseq, ligand resseq) pairs; as in
 * create_restraints_from_pairs, a pair is kept when both molecules contain
 * an atom named CA with that residue number (the first such atom is used)
 * and dropped otherwise.  w may be NULL for the default weights. */
gd_status gd_complex_create(gd_context *ctx, const gd_atoms *receptor, const gd_atoms *ligand,
                            const int32_t *restraint_pairs, int32_t n_pairs, const gd_weights *w,
                            gd_complex **out);
gd_status gd_complex_destroy(gd_complex *cx);
/* number of restraints kept at upload */
int32_t gd_complex_num_restraints(const gd_complex *cx);
gd_status gd_complex_set_weights(gd_complex *cx, const gd_weights *w);

/* Host-side frame of each pose from its 6 genes (alpha, beta, gamma, dx, dy, dz). */
gd_status gd_make_frames(const double *genes, int32_t n, gd_pose_frame *frames);

/* Population::eval_fitness: score n poses given as genes (n x 6, host
 * memory); writes n gd_pose_energy records (host memory).  Synchronous. */
gd_status gd_score_poses(gd_complex *cx, const double *genes, int32_t n, gd_precision prec,
                         gd_pose_energy *out);

/* Same, on device-resident frames and outputs, enqueued on `stream`
 * (a cudaStream_t; NULL = the context's stream).  max_displacement bounds
 * |dx|, |dy|, |dz| over the frames (it sizes the FP32 guard bands).  Returns
 * after the launch; errors of the device run are reported by gd_sync. */
gd_status gd_score_frames_device(gd_complex *cx, const gd_pose_frame *d_frames, int32_t n,
                                 gd_precision prec, double max_displacement, gd_pose_energy *d_out,
                                 void *stream);
/* gd_score_frames_device in the FP32 form, for callers that must not
 * allocate device memory while they score (for example a host whose GPU
 * memory is handed to its own pool allocator at start-up, or a real-time loop
 * that cannot take an allocation's latency).  No counterpart in the
 * reference.  It allocates nothing: its argument block lives in a 4 KiB
 * file-scope device array that every GPU loading the library keeps until the
 * process exits.  The first call on a device looks that array's address up
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * Receptors of more than 4096 atoms are rejected with GD_ERR_INVALID_ARG.
 * All calls share the one array: calls that overlap on the GPU (different
 * streams, or contexts on the same device) race and must be serialised by
 * the caller.  Errors of the device run are reported by gd_sync. */
gd_status gd_score_frames_device_noalloc(gd_complex *cx, const gd_pose_frame *d_frames, int32_t n,
                                         double max_displacement, gd_pose_energy *d_out, void *stream);

/* Wait for the context's work and report any device-side error. */
gd_status gd_sync(gd_context *ctx);

/* The `score` command: score n_models ligand coordinate sets as given
 * (lig_xyz: n_models x n_lig x 3, host memory); no transform is applied. */
gd_status gd_score_models(gd_complex *cx, const double *lig_xyz, int32_t n_models, gd_precision prec,
                          gd_pose_energy *out);

/* calculate_contacts for the complex receptor + ligand moved by each pose's
 * genes.  Contact keys are (chainA<<48)|(uint16(resA)<<32)|(chainB<<16)|uint16(resB)
 * with chainA < chainB, ascending per pose.  offsets has n+1 entries; keys
 * holds up to cap keys.  GD_ERR_CAPACITY (with offsets[n] = keys needed) if
 * cap is too small. */
gd_status gd_pose_contacts(gd_complex *cx, const double *genes, int32_t n, int64_t *keys, int64_t cap,
                           int64_t *offsets);

/* cluster_structures over the n poses given as genes: contacts, all-pairs
 * FCC, neighbour graph and greedy clustering, clusters of at least
 * min_cluster_size in gdock's output order.  centers/sizes hold up to n
 * entries, members up to n; *n_clusters receives the count. cfg may be NULL
 * for the defaults. */
gd_status gd_cluster(gd_complex *cx, const double *genes, int32_t n, const gd_cluster_cfg *cfg,
                     int32_t *n_clusters, int32_t *centers, int32_t *sizes, int32_t *members);

/* cluster_structures on caller-supplied contact sets (keys/offsets as
 * gd_pose_contacts writes them); the FCC and neighbour graph run on the GPU. */
gd_status gd_cluster_sets(gd_context *ctx, const int64_t *keys, const int64_t *offsets, int32_t n,
                          const gd_cluster_cfg *cfg, int32_t *n_clusters, int32_t *centers,
                          int32_t *sizes, int32_t *members);

/* ----------------------------------------------------------- DockQ --
 * evaluator::Evaluator (src/evaluator.rs:50-186): quality of poses against
 * a reference ligand structure.  Metrics as src/evaluator.rs:29-35. */
typedef struct gd_dock_metrics { double rmsd, irmsd, fnat, dockq; } gd_dock_metrics;
typedef struct gd_evaluator gd_evaluator;

/* Evaluator::new(receptor, reference) (src/evaluator.rs:51-66) for the
 * complex's receptor; the ligand of the complex is the moving structure.
 * Atom names (trimmed, at most 4 characters) are packed little-endian into
 * one uint32 per atom: byte k = character k, zero-padded.  Only the fields
 * x, y, z, resseq and chain of `reference` are read.  The complex must
 * outlive the evaluator. */
gd_status gd_evaluator_create(gd_complex *cx, const gd_atoms *reference, const uint32_t *rec_names,
                              const uint32_t *lig_names, const uint32_t *ref_names, gd_evaluator **out);
gd_status gd_evaluator_destroy(gd_evaluator *ev);
/* Sizes fixed at creation, into counts[GD_EVAL_COUNTS]: receptor interface
 * residues, reference interface residues, native contacts, ligand atoms read
 * per pose, L-RMSD pairs, i-RMSD pairs, native-identity (receptor, ligand)
 * atom pairs tested per pose. */
#define GD_EVAL_COUNTS 7
gd_status gd_evaluator_counts(const gd_evaluator *ev, int64_t *counts);

/* Population::eval_metrics (src/population.rs:63-71): calc_metrics of the
 * ligand moved by each of n gene vectors (6 doubles each), FP64 on the GPU;
 * out[n].  Contact decisions and fnat are exact; rmsd and irmsd differ from
 * the reference's sequential sums only by summation order. */
gd_status gd_evaluate_poses(gd_evaluator *ev, const double *genes, int32_t n, gd_dock_metrics *out);
/* gd_evaluate_poses on device-resident frames (gd_make_frames layout) into
 * device-resident metrics, asynchronously on `stream` (NULL = the context's
 * stream).  Errors of the device run are reported by gd_sync. */
gd_status gd_evaluate_frames_device(gd_evaluator *ev, const gd_pose_frame *d_frames, int32_t n,
                                    gd_dock_metrics *d_out, void *stream);

/* ----------------------------------------------------------------- GA --
 * gdock's generation loop (src/commands/run.rs:381-531: evaluate, track the
 * best, stop after convergence_window stagnant generations, evolve) with
 * Population::evolve (src/population.rs:74-121) on the GPU, for many jobs at
 * once.  The random draws of each generation are made on the host in the
 * reference's order from a seeded xoshiro256** stream (not rand's StdRng). */
typedef struct gd_ga_cfg {
  int32_t pop_size;             /* POPULATION_SIZE (150); even */
  int32_t elitism;              /* ELITISM_COUNT (5) */
  int32_t tournament_size;      /* TOURNAMENT_SIZE (3) */
  double crossover_rate;        /* CROSSOVER_RATE (0.6) */
  double mutation_rate;         /* MUTATION_RATE (0.1) */
  double max_displacement;      /* MAX_DISPLACEMENT (50 A) */
  double rot_sigma;             /* creep sigma of the angles (0.174 rad) */
  double trans_sigma;           /* creep sigma of the displacement (1 A) */
  int32_t max_generations;      /* MAX_GENERATIONS (250) */
  int32_t early_stopping;       /* ENABLE_EARLY_STOPPING (1) */
  double convergence_threshold; /* CONVERGENCE_THRESHOLD (0.001) */
  int32_t convergence_window;   /* CONVERGENCE_WINDOW (10) */
  uint64_t seed;                /* job j uses seed + j */
  int32_t hof_max_size;         /* HALL_OF_FAME_MAX_SIZE (500); 0 = no Hall of Fame */
  int32_t hof_top_k;            /* HALL_OF_FAME_TOP_K (10) */
} gd_ga_cfg;

/* One Hall of Fame entry (src/commands/run.rs:64-73). */
typedef struct gd_hof_entry {
  double genes[6];
  double fitness;
  int32_t generation;
  int32_t pad;
} gd_hof_entry;

/* The reference's constants (src/constants.rs:2-16, src/chromosome.rs:64-71). */
gd_status gd_ga_default_cfg(gd_ga_cfg *cfg);
/* The host draws of one job: initial genes (pop_size x 6) and, per
 * generation, tournament indices, the shuffled order, crossover and mutation
 * uniforms and the mutation perturbations (any pointer may be NULL). */
gd_status gd_ga_draw(const gd_ga_cfg *cfg, uint64_t seed, int32_t generations, double *init_genes, int32_t *tour,
                     int32_t *perm, double *cross_u, double *mut_u, double *mut_z);
/* DockQ metrics of every generation (src/commands/run.rs:387-388,449-450):
 * for each job with an evaluator (created on that job's complex), the
 * metrics of the generation's first best-fitness pose and the mean DockQ of
 * the population, computed on the device after each evaluation inside the
 * generation loop.  best and mean_dockq are jobs x max_generations; entries
 * of generations a job did not reach, or of jobs without an evaluator, are
 * left as they were. */
typedef struct gd_ga_metrics {
  gd_evaluator *const *evaluators; /* [jobs], NULL entries allowed */
  gd_dock_metrics *best;           /* [jobs][max_generations] */
  double *mean_dockq;              /* [jobs][max_generations] */
} gd_ga_metrics;

/* Run the GA of `jobs` complexes to completion on the device; with
 * use_graph (FP32 form) one generation is a captured CUDA graph replayed.
 * Outputs: final populations (jobs x pop x 6), their energies
 * (jobs x pop), generations evolved per job, best fitness per generation
 * (jobs x max_generations, may be NULL), and each job's Hall of Fame
 * (HallOfFame::add_from_population after every evaluation inside the
 * generation loop, src/commands/run.rs:99-213,385; kept on the device):
 * out_hof receives jobs x hof_max_size entries in the reference's order,
 * out_hof_count the entries per job.  Both NULL (or hof_max_size 0) = no
 * Hall of Fame.  metrics may be NULL (no per-generation DockQ). */
gd_status gd_ga_run(gd_context *ctx, gd_complex *const *complexes, int32_t jobs, const gd_ga_cfg *cfg,
                    gd_precision prec, int32_t use_graph, double *out_genes, gd_pose_energy *out_energies,
                    int32_t *out_generations, double *out_history, gd_hof_entry *out_hof,
                    int32_t *out_hof_count, const gd_ga_metrics *metrics);

/* ------------------------------------------------------------- serving --
 * A request loop for docking jobs (gdock's `run` GA per job): jobs are
 * admitted first-come first-served into resident slots as slots and the HBM
 * budget allow; every tick advances all resident jobs by one generation in
 * shared launches (continuous batching), keeping each job's coordinates,
 * parameters and population on the device; finished jobs leave their slot to
 * the next queued job.  A job's result does not depend on the other jobs. */
typedef struct gd_server gd_server;
typedef struct gd_server_cfg {
  int32_t max_slots;    /* jobs resident at once */
  uint64_t hbm_budget;  /* device bytes resident complexes may hold (0: the context's budget only) */
  gd_ga_cfg ga;         /* GA settings of every job (seed ignored: per job) */
  int32_t precision;    /* gd_precision */
} gd_server_cfg;
enum { GD_JOB_QUEUED = 0, GD_JOB_RUNNING = 1, GD_JOB_DONE = 2, GD_JOB_FAILED = 3 };
typedef struct gd_job_result {
  int32_t status, error, generations;
  double latency_s; /* submit -> done (or -> now) */
  double queue_s;   /* submit -> admitted */
} gd_job_result;
typedef struct gd_server_stats {
  int64_t completed, queued, resident, generations_run, poses_scored;
  uint64_t device_bytes;
  double latency_p50_s, latency_p99_s, latency_max_s;
  double gpu_busy_s;  /* device time of the generations run (CUDA events) */
  double elapsed_s;   /* since the first submission */
} gd_server_stats;

gd_status gd_server_default_cfg(gd_server_cfg *cfg);
gd_status gd_server_create(gd_context *ctx, const gd_server_cfg *cfg, gd_server **out);
gd_status gd_server_destroy(gd_server *s);
/* Queue a job (inputs copied); thread-safe.  Refused with GD_ERR_STATE once
 * the server's own thread has stopped on an error (gd_last_error names it). */
gd_status gd_server_submit(gd_server *s, const gd_atoms *receptor, const gd_atoms *ligand,
                           const int32_t *restraint_pairs, int32_t n_pairs, const gd_weights *w, uint64_t seed,
                           int64_t *job_id);
/* One tick on the caller's thread (admit, one generation, retire). */
gd_status gd_server_step(gd_server *s, int32_t *resident_jobs);
/* Run ticks on the server's own thread until gd_server_stop (which drains
 * queued and resident jobs first).  A tick that fails stops the thread: every
 * resident and queued job ends GD_JOB_FAILED with the tick's status. */
gd_status gd_server_start(gd_server *s);
gd_status gd_server_stop(gd_server *s);
gd_status gd_server_wait(gd_server *s, int64_t job_id, double timeout_s, int32_t *status);
/* Status and, when done, final population (pop x 6), its energies and the
 * best fitness per generation (max_generations); pointers may be NULL. */
gd_status gd_server_result(gd_server *s, int64_t job_id, gd_job_result *res, double *genes,
                           gd_pose_energy *energies, double *history);
/* The Hall of Fame of a finished job (the server keeps one per job when the
 * GA config's hof_max_size and hof_top_k are positive; the defaults are
 * 500 and 10): *count receives the entries; up to cap of them go to
 * entries, GD_ERR_CAPACITY when cap is too small, GD_ERR_STATE before the
 * job is done. */
gd_status gd_server_hall_of_fame(gd_server *s, int64_t job_id, gd_hof_entry *entries, int32_t cap, int32_t *count);
gd_status gd_server_release(gd_server *s, int64_t job_id);
gd_status gd_server_get_stats(gd_server *s, gd_server_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* GDOCK_GB300_H */
