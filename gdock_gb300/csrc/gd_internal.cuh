// Internal declarations shared by the gdock_gb300 CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "gdock_gb300.h"
#include <nvtx3/nvToolsExt.h>

namespace gd {

// Four doubles, 32-byte aligned (one receptor atom of the FP64 tiles).
struct alignas(32) D4 {
  double x, y, z, w;
};

// Receptor atoms per tile staged in shared memory by one bulk (TMA) copy.
constexpr int kTile = 256;
// Receptor atoms per segment of the FP32 kernel's ring: the receptor is
// stored as spatially compact segments of this many atoms, each with a
// bounding sphere.
constexpr int kRecSeg = 64;
constexpr int kStages = 3;
// Upper bounds of a device-side wait before it gives up: polls and wall time.
constexpr uint32_t kSpinLimit = 1u << 26;
constexpr uint64_t kWaitLimitNs = 2000000000ull;
// Distinct (epsilon, Rmin/2) atom types a complex may hold.
constexpr int kMaxTypes = 64;
// FP32 scoring variant when none is set: 4 ligand slots per lane, 4 receptor
// rows per step, five resident CTAs per SM (GD_TUNE_F32_SLOTS encoding)
constexpr int kDefaultF32Tune = 256 + 64 + 4;

// device error codes written to the context's error word
enum : int { kDevOk = 0, kDevTimeout = 1, kDevCapacity = 2, kDevRange = 3, kDevBoundsBase = 1000 };
// Index checks of the library's debug variant (built with -DGD_DEBUG_CHECKS:
// libgdock_gb300_debug.so).  A failed check records kDevBoundsBase + site in
// the context's error word (the first failure stays) and the caller skips or
// clamps the access; the call then reports the site.  In the release library
// every check is the constant true.
#ifdef GD_DEBUG_CHECKS
#define GD_DCHECK(errp, cond, site) ((cond) || (atomicCAS((errp), 0, kDevBoundsBase + (site)), false))
#else
#define GD_DCHECK(errp, cond, site) true
#endif

// Per-job state of the device GA (the reference loop's counters,
// src/commands/run.rs:371-425).  stop: 0 running, 1 converged, 2 done.
struct GaJobState {
  int gen, stop, stagnant, hof_n;  // hof_n: Hall of Fame entries held
  double last_best;
  int hof_sorted, pad;             // 1 once a prune has sorted the Hall of Fame
};

// Per-pair parameters of one type pair, FP32 form, for the soft-core LJ
// rewritten as eps (q^2 - 2q) = 4 eps x (x - 1) with q = 2x and
// x = 1 / (r^6 * 2/R6 + 1), R6 = (Rmin_i + Rmin_j)^6, eps = sqrt(eps_i eps_j).
struct TypePair32 { float inv2, eps4; };  // 2/R6 (FLT_MAX when R6 = 0), 4 eps
// FP64 form: R6, alpha*R6 (alpha = 0.5), eps.
struct TypePair64 { double r6, hr6, eps, pad; };

// Exact FP64 thresholds on the squared distance d2 = dx*dx + dy*dy + dz*dz,
// so that d2-comparisons make the same decisions as the reference's
// comparisons of sqrt(d2) against its cutoffs.
struct Thresholds {
  double vdw_lt;    // dist < 12   <=>  d2 < vdw_lt
  double elec_gt;   // dist > 1    <=>  d2 > elec_gt
  double elec_lt;   // dist < 15   <=>  d2 < elec_lt
  double desolv_lt; // dist < 8    <=>  d2 < desolv_lt
  double contact_le;// dist <= 5   <=>  d2 <= contact_le (per call's cutoff)
};

struct ScoreParams {
  // receptor, sorted by atom type, padded to a multiple of kTile
  const float4 *rec_pos32;  // (x-O, y-O, z-O, 332.0636*q) FP32
  const D4 *rec_pos64; // (x, y, z, q) FP64
  const int2 *rec_meta;     // (type, serial)
  const int4 *rec_meta16;   // (type, serial, 0, 0): the FP32 kernel's copy, as wide as a position
  const double *rec_desolv; // [nr * 11] energy contribution at burial count 0..10
  const float4 *rec_seg;    // per kRecSeg-atom segment: bounding sphere (centre - O, radius) FP32
  int nr, n_tiles, nseg;
  // ligand in slot order (spatially compact runs of 32 atoms)
  const int *lig_perm;      // slot position -> original atom index
  const D4 *lig_slot_sph;   // per 32-atom slot: bounding sphere in the positioned frame (centre, radius)
  const double *lig_x, *lig_y, *lig_z;
  const double *lig_q;
  const int *lig_type, *lig_serial;
  const double *lig_desolv; // [nl * 11]
  int nl;
  double cx, cy, cz;        // rotation centre (centroid of the positioned ligand)
  double ox, oy, oz;        // FP32 coordinate origin
  const TypePair32 *tab32;
  const TypePair64 *tab64;
  int nt;
  int need_clamp;           // some |eps_ij| may exceed the [-50, 500] clamp
  // restraints: receptor CA coordinates and ligand CA atom index
  const D4 *restr_rec; // (x, y, z, -) of the receptor CA
  const int *restr_lig;     // ligand CA index (slot order)
  int K;
  double wv, we, wd, wa;
  Thresholds thr;
  float guard_v, guard_e, guard_d; // FP32 guard half-widths on d2
  // poses
  const gd_pose_frame *frames;
  const double *models;     // explicit ligand coordinates (n x nl x 3) or null
  int n_poses;
  gd_pose_energy *out;
  int *err;
  const int *skip;          // when non-null and nonzero, the complex's poses are not scored
};

}  // namespace gd

using gd::D4;

struct gd_context {
  int device = 0;
  uint64_t budget = 0;
  uint64_t in_use = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  int *d_err = nullptr;
  std::string last_error;
  // grow-only scratch: device and pinned host staging
  void *d_scratch = nullptr;
  size_t d_scratch_bytes = 0;
  void *h_pinned = nullptr;
  size_t h_pinned_bytes = 0;
  // argument blocks of batched launches (descriptors, queue, counters)
  void *d_batch = nullptr;
  size_t d_batch_bytes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int tune_f32_slots = 0;  // 0: automatic (kDefaultF32Tune)
  int tune_split = 0;      // GD_TUNE_SPLIT: 0 automatic, 1 whole poses, 2 always split
  int tune_fault = 0;      // GD_TUNE_FAULT: 1 = drop one stage copy (failure-detection tests)
  int tune_fcc = 0;        // GD_TUNE_FCC: 0 automatic, 1 bitsets, 2 contact postings
  int tune_contacts = 0;   // GD_TUNE_CONTACTS: 0 automatic (bitmaps where possible), 1 per-residue lists
  int tune_rparts = 0;     // GD_TUNE_RPARTS: 0 automatic, 1..8 receptor parts per ligand chunk (split mode)
  int last_fcc = 0;        // GD_INFO_LAST_FCC: pair counts of the last device clustering (1 bitsets, 2 postings)
  int last_contacts = 0;   // GD_INFO_LAST_CONTACTS: kernel of the last contact pass (1 lists, 2 bitmaps)
};

struct gd_complex {
  gd_context *ctx = nullptr;
  int nr = 0, nl = 0, nr_pad = 0, nt = 0, K = 0;
  gd_weights w{};
  bool serial_overlap = false;
  bool need_clamp = false;
  double cx = 0, cy = 0, cz = 0, ox = 0, oy = 0, oz = 0;
  double rec_extent = 0;  // max |x - O| over receptor atoms (inf-norm)
  double lig_radius = 0;  // max |x - c| over ligand atoms (Euclidean)
  // device arrays
  float4 *rec_pos32 = nullptr;
  D4 *rec_pos64 = nullptr;
  int2 *rec_meta = nullptr;
  int4 *rec_meta16 = nullptr;
  double *rec_desolv = nullptr;
  double *lig_x = nullptr, *lig_y = nullptr, *lig_z = nullptr, *lig_q = nullptr;
  int *lig_type = nullptr, *lig_serial = nullptr;
  double *lig_desolv = nullptr;
  gd::TypePair32 *tab32 = nullptr;
  gd::TypePair64 *tab64 = nullptr;
  D4 *restr_rec = nullptr;
  int *restr_lig = nullptr;
  int *lig_perm = nullptr;  // slot position -> original ligand atom index
  float4 *rec_seg = nullptr;  // receptor segment spheres (FP32, relative to O)
  D4 *lig_slot_sph = nullptr;  // ligand slot spheres (positioned frame)
  int nseg = 0;
  std::vector<void *> allocs;
  uint64_t bytes = 0;
  // host copies used by clustering
  std::vector<double> h_rx, h_ry, h_rz, h_lx, h_ly, h_lz;
  std::vector<uint8_t> h_rchain, h_lchain, h_relem, h_lelem;
  std::vector<int16_t> h_rres, h_lres;
  std::vector<int> h_lig_slot;  // original ligand atom index -> slot position on the device
  void *cluster_cache = nullptr;  // gd::ClusterTopo*, built on first use
};

namespace gd {
// Host-side phase trace, printed to stderr when GD_TRACE is set in the
// environment (off by default).
bool trace_on();
void trace(const char *phase, double seconds);
// NVTX range over a scope, named after the ABI call or phase (seen by ncu and
// nsys; without a tool attached a push/pop is a null-pointer check).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};
gd_status fail(gd_context *ctx, gd_status s, const std::string &msg);
gd_status cuda_fail(gd_context *ctx, cudaError_t e, const char *what);
gd_status dev_alloc(gd_context *ctx, uint64_t bytes, void **p);
void dev_free(gd_context *ctx, void *p, uint64_t bytes);
gd_status ensure_scratch(gd_context *ctx, size_t dev_bytes, size_t pinned_bytes);
gd_status check_device_error(gd_context *ctx);
Thresholds make_thresholds(double contact_cutoff);
void make_frame(const double *g, gd_pose_frame *f);
void guard_widths(const gd_complex *cx, double max_disp, float *gv, float *ge, float *gd);
gd_status launch_score(gd_complex *cx, const gd_pose_frame *d_frames, const double *d_models, int n,
                       gd_precision prec, gd_pose_energy *d_out, cudaStream_t stream, double max_disp);
void free_cluster_cache(gd_complex *cx);
// A small sphere enclosing n points (x[i], y[i], z[i]) for i = idx[k], or
// i = k when idx is null; the radius is the largest distance from the
// returned centre, so every point is enclosed (gd_api.cu).
void enclosing_ball(const double *x, const double *y, const double *z, const int *idx, int n, double c[3],
                    double &r);
gd_status ensure_batch_scratch(gd_context *ctx, size_t dev_bytes);
ScoreParams make_params(gd_complex *cx, const gd_pose_frame *d_frames, const double *d_models, int n,
                        gd_pose_energy *d_out, double max_disp);
gd_status launch_score_batch_f32(gd_context *ctx, const std::vector<ScoreParams> &descs, bool serial, bool clamp,
                                 int slots, cudaStream_t stream);
struct BatchLaunch;
gd_status batch_prepare(gd_context *ctx, const std::vector<ScoreParams> &descs, bool serial, bool clamp, int slots,
                        BatchLaunch **out);
gd_status batch_launch(gd_context *ctx, BatchLaunch *b, cudaStream_t stream);
// DockQ metrics of n device-resident frames of the evaluator's complex
// (gd_eval.cu); skip (may be null) is read on the device: nonzero = no work.
gd_status launch_dockq(gd_evaluator *ev, const gd_pose_frame *d_frames, int n, gd_dock_metrics *d_out,
                       const int *skip, cudaStream_t stream);
gd_complex *evaluator_complex(const gd_evaluator *ev);
void batch_free(gd_context *ctx, BatchLaunch *b);
}  // namespace gd
