// Batched FP32 scoring: a persistent kernel in which every warp owns whole
// work items taken from a global queue, so that poses of many complexes of
// uneven sizes share one launch and no warp ever waits for another.  A work
// item is one pose, or (split mode, the default) one 128-atom ligand chunk of
// a pose, or for launches with few poses one receptor part of such a chunk
// (the receptor segments g with g mod R = part).
//
// Per work item a warp
//   1. copies the complex's descriptor and the pose frame to its shared memory;
//   2. for each chunk of 32*S ligand atoms: transforms them exactly (FP64, the
//      reference's operation order, src/structure.rs:80-131), keeps FP32
//      copies in registers (S slots of 32 atoms, one per lane; the ligand is
//      stored in spatially compact slot order) and a bounding sphere and box
//      per slot;
//   3. streams the receptor through its own two-stage shared-memory ring,
//      each stage filled by one bulk (TMA) copy of a 64-atom segment and
//      guarded by a per-warp mbarrier with a bounded wait; the receptor is
//      stored as spatially compact segments with bounding spheres, and only
//      the segments within reach of the chunk's slot spheres are copied and
//      tested (the slot spheres are precomputed and move rigidly with the
//      pose);
//   4. row test: each lane takes one (receptor atom, slot) row of an 8 x 4
//      round; a row whose atom lies beyond the 15 A reach of the slot's
//      sphere or box is dropped (every pair of it contributes exactly
//      nothing), one beyond the 12 A reach is a far row (Coulomb only); kept
//      rows go to per-slot lists in shared memory;
//   5. evaluates the kept rows four at a time (independent FP32 chains):
//      soft-core LJ, Coulomb, burial counts and guard-band tests for near
//      rows, Coulomb and its band for far rows;
//   6. re-decides in FP64, once per segment, the pairs of flagged steps whose
//      FP32 d2 lies within the guard band of a cutoff (1, 8, 12, 15 A), so
//      all decisions equal the FP64 ones;
//   7. reduces exactly: each segment's FP32 vdW and Coulomb partials become
//      2^-32 fixed-point integers summed per lane (integer sums do not depend
//      on their order, so neither do the energies on how segments, chunks and
//      receptor parts are grouped into work items), desolvation from the
//      exact burial counts in FP64 in a fixed order, AIR in restraint order
//      (bit-identical), and writes the six-field record
//      (src/chromosome.rs:110-127).  Split mode: the item that completes a
//      pose adds the items' partials.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gd_device.cuh"

namespace gd {
namespace {

constexpr int kWarps = 4;      // warps per CTA (independent)
constexpr int kSeg = 64;       // receptor atoms per ring stage
constexpr int kWS = 2;         // ring stages per warp (a stage takes microseconds to process: two hide the copy)
constexpr int kBlk = 8;        // receptor atoms per row-test round (lane = slot * 8 + atom)
constexpr int kMaxS = 4;       // ligand slots per lane, at most (one row-test round covers 8 atoms x 4 slots)
constexpr int kList = kSeg + 8;  // row-list entries per slot: a segment's atoms + two paddings of 4 rows
constexpr int kFar = kWS * kSeg; // shared-memory index of the far-away dummy receptor atom
constexpr int kCntSmemMax = 4096;  // burial counters kept in shared memory up to this many receptor atoms
constexpr int kSegListMax = 512;   // receptor segments a chunk's culled list holds (more: every segment)
static_assert(kSeg == kRecSeg, "the ring stage is one receptor segment");

struct BatchParams {
  const ScoreParams *descs;       // one per complex
  const long long *item_start;    // prefix sums of work items, ncx + 1 entries
  int ncx;
  long long total;
  unsigned long long *queue;      // work counter, zero at launch
  uint8_t *gcounts;               // per-warp burial counters in global memory (when not in smem)
  int gcount_stride;              // bytes per warp in gcounts
  int smem_cnt;                   // bytes per warp of shared-memory counters (0: use gcounts)
  int max_nr;                     // largest receptor of the batch
  int warp_smem;                  // bytes of shared memory per warp
  int *err;
  // split mode: a work item is one ligand chunk of a pose; the chunk that
  // finishes a pose last reduces its per-chunk partials
  int split;
  const long long *pose_start;    // first batch-wide pose index of each complex
  int max_chunks;                 // partial slots per pose (chunks x rparts)
  double *part;                   // [pose][chunk * rparts + part][vdw, elec (fixed point), ligand desolvation][32 lanes]
  unsigned *pcount;               // [pose][(max_nr + 1) / 2] receptor burial counts, two 16-bit counts a word
  int *pdone;                     // [pose] items finished
  int rparts;                     // receptor parts per chunk (split mode; 1: whole receptor)
  unsigned *lcount;               // [pose][max_nl] ligand burial counts (rparts > 1)
  int max_nl;
  // failure-detection test (GD_TUNE_FAULT): the warp that takes work item 0
  // issues no copy for its first ring stage, so its bounded wait runs out
  int drop_copy;
};

struct WarpSmem {
  size_t pos, meta, list, fixq, cmask, cidx, lfix, bars, desc, frame, blob, box, rc, ssph, segl, cnt, total;
};

__host__ __device__ inline WarpSmem warp_layout(int smem_cnt) {
  WarpSmem L;
  size_t o = 0;
  auto al = [&](size_t a) { o = (o + a - 1) / a * a; };
  L.pos = o;
  o += sizeof(float4) * (kWS * kSeg + 1);  // + the far dummy atom
  al(16);
  L.meta = o;  // at a fixed distance from pos: one address serves both
  o += sizeof(int4) * (kWS * kSeg + 1);
  al(16);
  L.list = o;
  o += sizeof(uint16_t) * kMaxS * kList;
  al(16);
  L.fixq = o;
  o += sizeof(uint16_t) * kMaxS * kList;  // at most one entry per step of a segment
  al(16);
  L.cmask = o;  // per near row of the segment: lanes with d2 < 64 (ballot)
  o += sizeof(unsigned) * kMaxS * kList;
  al(16);
  L.cidx = o;   // ... and its receptor atom (stage index)
  o += sizeof(uint16_t) * kMaxS * kList;
  al(16);
  L.lfix = o;
  o += sizeof(int) * kMaxS * 32;
  al(16);
  L.bars = o;
  o += 8 * kWS;
  al(16);
  L.desc = o;
  o += sizeof(ScoreParams);
  al(16);
  L.frame = o;
  o += sizeof(gd_pose_frame);
  L.blob = o;
  o += sizeof(float4) * 8;
  L.box = o;
  o += sizeof(float4) * 2 * kMaxS;
  L.rc = o;
  o += sizeof(int) * kSeg;
  L.ssph = o;  // the chunk's slot spheres (culling test of the receptor segments)
  o += sizeof(float4) * kMaxS;
  L.segl = o;  // the chunk's receptor segments within reach
  o += sizeof(uint16_t) * kSegListMax;
  al(16);
  L.cnt = o;
  o += smem_cnt;
  al(128);
  L.total = o;
  return L;
}

__device__ __forceinline__ void issue_seg(long long q, int seg, const ScoreParams &p, float4 *s_pos, int4 *s_meta,
                                          uint64_t *s_bar) {
  const int st = static_cast<int>(q % kWS);
  constexpr uint32_t kBytes = kSeg * (sizeof(float4) + sizeof(int4));
  mbar_expect_tx(&s_bar[st], kBytes);
  bulk_g2s(&s_pos[st * kSeg], p.rec_pos32 + static_cast<size_t>(seg) * kSeg, kSeg * sizeof(float4), &s_bar[st]);
  bulk_g2s(&s_meta[st * kSeg], p.rec_meta16 + static_cast<size_t>(seg) * kSeg, kSeg * sizeof(int4), &s_bar[st]);
}

// acc += v when t < 0 (one predicated add)
__device__ __forceinline__ void add_if_lt0(float &acc, float t, float v) {
  asm("{\n\t.reg .pred p;\n\tsetp.lt.f32 p, %1, 0f00000000;\n\t@p add.f32 %0, %0, %2;\n\t}" : "+f"(acc)
      : "f"(t), "f"(v));
}
// acc = a * b + acc (one rounding) when t < 0
__device__ __forceinline__ void fma_if_lt0(float &acc, float t, float a, float b) {
  asm("{\n\t.reg .pred p;\n\tsetp.lt.f32 p, %1, 0f00000000;\n\t@p fma.rn.f32 %0, %2, %3, %0;\n\t}" : "+f"(acc)
      : "f"(t), "f"(a), "f"(b));
}
// acc = a * b + acc (one rounding) when |t| < lim
__device__ __forceinline__ void fma_if_abs_lt(float &acc, float t, float lim, float a, float b) {
  asm("{\n\t.reg .pred p;\n\tsetp.lt.f32 p, %1, %2;\n\t@p fma.rn.f32 %0, %3, %4, %0;\n\t}" : "+f"(acc)
      : "f"(fabsf(t)), "f"(lim), "f"(a), "f"(b));
}
// a += 1 and b += 1 when d2 < 64
__device__ __forceinline__ void count_if_lt64(int &a, int &b, float d2) {
  asm("{\n\t.reg .pred p;\n\tsetp.lt.f32 p, %2, 0f42800000;\n\t@p add.s32 %0, %0, 1;\n\t@p add.s32 %1, %1, 1;\n\t}"
      : "+r"(a), "+r"(b)
      : "f"(d2));
}

__device__ __forceinline__ float d2f(const float4 &r, float lx, float ly, float lz) {
  const float dx = __fsub_rn(r.x, lx), dy = __fsub_rn(r.y, ly), dz = __fsub_rn(r.z, lz);
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// soft-core LJ in FP32 (src/fitness.rs:57-70): eps*(q^2 - 2q) with
// q = R6/(r^6 + R6/2), evaluated as 4 eps x (x - 1) = 4 eps (x^2 - x),
// x = q/2 = 1/(r^6 2/R6 + 1); at d2 = 0 it is exactly 0
template <bool CLAMP>
__device__ __forceinline__ float vdw_term(float d2, float2 tp) {
  const float r6 = d2 * d2 * d2;
  const float x = rcp_approx(__fmaf_rn(r6, tp.x, 1.0f));
  float v = __fmaf_rn(x, x, -x) * tp.y;
  if (CLAMP) v = v < -50.0f ? -50.0f : (v > 500.0f ? 500.0f : v);
  return v;
}

// One pair's FP32 terms.  The Coulomb sum accumulates q_r / d2 (scaled by
// the lane's ligand charge once per segment).  The vdW decision is d2 < 144
// alone: the reference's 0 < r excludes only coincident atoms, whose FP32
// d2 is then exactly 0 too (the FP32 coordinates are roundings of the same
// doubles) and whose FP32 term is exactly 0, so the sums are unchanged; the
// guard band of the vdW cutoff is the one at 144.
template <bool SERIAL, bool CLAMP>
__device__ __forceinline__ void pair32(const float4 &r, int rtrow, int rser, const float2 *tab, float lx, float ly,
                                       float lz, int lt, int lser, float gv, float ge, float gdd, float &av,
                                       float &ae, int &lc, int &rc, bool &amb) {
  const float d2 = d2f(r, lx, ly, lz);
  const float2 tp = __ldg(&tab[rtrow + lt]);
  const float tv = __fsub_rn(d2, 144.0f);  // d2 < 144  <=>  tv < 0
  if (SERIAL || CLAMP) {
    const float v = vdw_term<CLAMP>(d2, tp);
    if (SERIAL) av += (tv < 0.0f && rser != lser) ? v : 0.0f;
    else add_if_lt0(av, tv, v);
  } else {
    // the well depth multiplies into the sum: one FMA (vdw_term without the
    // product's own rounding)
    const float x = rcp_approx(__fmaf_rn(d2 * d2 * d2, tp.x, 1.0f));
    fma_if_lt0(av, tv, __fmaf_rn(x, x, -x), tp.y);
  }
  const float te = __fsub_rn(d2, 113.0f);  // 1 < d2 < 225  <=>  |te| < 112
  fma_if_abs_lt(ae, te, 112.0f, r.w, rcp_approx(d2));
  count_if_lt64(lc, rc, d2);
  amb = amb | (fabsf(__fsub_rn(fabsf(te), 112.0f)) < ge) | (fabsf(tv) < gv) | (fabsf(__fsub_rn(d2, 64.0f)) < gdd);
}

// One pair of a far row (no pair within the vdW cutoff): Coulomb only, the
// same FP32 expressions and decision as pair32().  Every FP32 d2 of a far
// row exceeds 144, where d2 - 113 and d2 - 225 are exact (Sterbenz) and
// |d2 - 113| < 112 is d2 < 225: one bound, one band.
__device__ __forceinline__ void pair32_elec(const float4 &r, float lx, float ly, float lz, float ge, float &ae,
                                            bool &amb) {
  const float d2 = d2f(r, lx, ly, lz);
  const float tf = __fsub_rn(d2, 225.0f);
  fma_if_lt0(ae, tf, r.w, rcp_approx(d2));
  amb = amb | (fabsf(tf) < ge);
}

__device__ __forceinline__ bool near_band(float d2, float gv, float ge, float gdd) {
  const float tv = __fsub_rn(d2, 144.0f), te = __fsub_rn(d2, 113.0f);
  return (fabsf(__fsub_rn(fabsf(te), 112.0f)) < ge) | (fabsf(tv) < gv) | (fabsf(__fsub_rn(d2, 64.0f)) < gdd);
}

// Corrections of one pair's FP32 contributions after its FP64 re-decision.
struct FixOut {
  float dv, de;
  int dl;
};

// FP64 re-decision of one flagged pair (exact ligand coordinates X, Y, Z):
// recomputes the FP32 d2 and decisions bit-identically to pair32() and
// returns the corrections where the exact decision differs.
template <bool SERIAL, bool CLAMP>
__device__ __forceinline__ FixOut fix_pair(const ScoreParams &p, double X, double Y, double Z, float4 r, int ridx,
                                        int rtrow, int rser, float lx, float ly, float lz, float lq, int lt, int lser) {
  FixOut o{0.0f, 0.0f, 0};
  const float d2 = d2f(r, lx, ly, lz);
  const float te = __fsub_rn(d2, 113.0f);
  bool pv32 = __fsub_rn(d2, 144.0f) < 0.0f;
  if (SERIAL) pv32 = pv32 && (rser != lser);
  const bool pe32 = fabsf(te) < 112.0f;
  const bool pd32 = d2 < 64.0f;
  const D4 r64 = p.rec_pos64[ridx];
  const double d2x = exact_d2(r64.x, r64.y, r64.z, X, Y, Z);
  bool pv64 = d2x > 0.0 && d2x < p.thr.vdw_lt;
  if (SERIAL) pv64 = pv64 && (rser != lser);
  const bool pe64 = d2x > p.thr.elec_gt && d2x < p.thr.elec_lt;
  const bool pd64 = d2x < p.thr.desolv_lt;
  if (pv64 != pv32) {
    const float v = vdw_term<CLAMP>(d2, __ldg(reinterpret_cast<const float2 *>(p.tab32) + rtrow + lt));
    o.dv = pv64 ? v : -v;
  }
  if (pe64 != pe32) {
    const float e = (r.w * rcp_approx(d2)) * lq;
    o.de = pe64 ? e : -e;
  }
  if (pd64 != pd32) o.dl = pd64 ? 1 : -1;
  return o;
}

// A segment's FP32 energy partial as a 2^-32 fixed-point integer.  Integer
// sums are exact, so the energies do not depend on how the segments are
// grouped into work items (whole poses, chunks, receptor parts) nor on the
// order the partials arrive in.  A segment's partial covers at most 256 pairs
// (64 receptor atoms x 4 lanes' slots) whose soft-core LJ terms are bounded
// by their well depths and Coulomb terms by 332 q q; a partial of 2^24
// kcal/mol or more (or not a number) is reported instead of wrapped.
__device__ __forceinline__ long long fx_energy(float x, int *err) {
  if (!(fabsf(x) < 16777216.0f)) {
    atomicCAS(err, 0, kDevRange);
    return 0;
  }
  return __float2ll_rn(x * 4294967296.0f);
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ void bump_count(uint8_t *cnt, int i, int delta) {
  const int c = static_cast<int>(cnt[i]) + delta;
  cnt[i] = static_cast<uint8_t>(c > 255 ? 255 : (c < 0 ? 0 : c));
}

// SPLIT: 0 whole poses, 1 ligand chunks, 2 ligand chunks in receptor parts
// (bp.rparts; a separate instantiation keeps the single-part kernel's loops
// free of the part arithmetic)
template <int S, int kAtoms, int MINB, bool SERIAL, bool CLAMP, int SPLIT>
__global__ void __launch_bounds__(kWarps * 32, MINB) k_score_f32w(const BatchParams bp) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const WarpSmem L = warp_layout(bp.smem_cnt);
  unsigned char *base = smem + static_cast<size_t>(wib) * L.total;
  float4 *s_pos = reinterpret_cast<float4 *>(base + L.pos);
  int4 *s_meta = reinterpret_cast<int4 *>(base + L.meta);
  uint16_t *s_list = reinterpret_cast<uint16_t *>(base + L.list);  // kept rows per slot, as stage indices
  uint16_t *s_fixq = reinterpret_cast<uint16_t *>(base + L.fixq);  // flagged steps: list position | slot << 8
  unsigned *s_cmask = reinterpret_cast<unsigned *>(base + L.cmask);  // near rows' burial ballots (this segment)
  uint16_t *s_cidx = reinterpret_cast<uint16_t *>(base + L.cidx);
  int *s_lfix = reinterpret_cast<int *>(base + L.lfix);            // ligand burial corrections per slot and lane
  uint64_t *s_bar = reinterpret_cast<uint64_t *>(base + L.bars);
  ScoreParams *s_desc = reinterpret_cast<ScoreParams *>(base + L.desc);
  gd_pose_frame *s_frame = reinterpret_cast<gd_pose_frame *>(base + L.frame);
  float4 *s_blob = reinterpret_cast<float4 *>(base + L.blob);
  float4 *s_box = reinterpret_cast<float4 *>(base + L.box);  // per slot: (centre, hx), (hy, hz, -, -)
  int *s_rc = reinterpret_cast<int *>(base + L.rc);  // receptor burial counts of the current segment
  float4 *s_ssph = reinterpret_cast<float4 *>(base + L.ssph);
  uint16_t *s_segl = reinterpret_cast<uint16_t *>(base + L.segl);
  const int gwarp = static_cast<int>(blockIdx.x) * kWarps + wib;
  uint8_t *cnt = bp.smem_cnt ? reinterpret_cast<uint8_t *>(base + L.cnt)
                             : bp.gcounts + static_cast<size_t>(gwarp) * bp.gcount_stride;

  if (lane == 0) {
    for (int s = 0; s < kWS; ++s) mbar_init(&s_bar[s], 1);
    fence_mbar_init();
    s_pos[kFar] = make_float4(1.0e9f, 1.0e9f, 1.0e9f, 0.0f);  // far from real and idle ligand lanes
    s_meta[kFar] = make_int4(0, 0, 0, 0);
  }
  if (!SPLIT)
    for (int i = lane; i < bp.max_nr; i += 32) cnt[i] = 0;
  for (int i = lane; i < kSeg; i += 32) s_rc[i] = 0;
  for (int i = lane; i < kMaxS * 32; i += 32) s_lfix[i] = 0;
  __syncwarp();

  static_assert(S >= 1 && S <= kMaxS, "one row-test round covers at most four slots");
  constexpr int kChunk = 32 * S;
  const int my_s = lane >> 3, my_a = lane & 7;
  const unsigned my_group = 0xffu << (8 * my_s), lt_mask = (1u << lane) - 1u;
  long long q = 0;  // ring uses of this warp so far
  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(bp.queue, 1ull);
    item = __shfl_sync(kFull, item, 0);
    if (static_cast<long long>(item) >= bp.total) break;
    // complex of this item: last c with item_start[c] <= item
    int lo = 0, hi = bp.ncx - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (bp.item_start[mid] <= static_cast<long long>(item)) lo = mid;
      else hi = mid - 1;
    }
    const long long kk = static_cast<long long>(item) - bp.item_start[lo];
    __syncwarp();
    {
      const uint64_t *src = reinterpret_cast<const uint64_t *>(bp.descs + lo);
      uint64_t *dst = reinterpret_cast<uint64_t *>(s_desc);
      for (int w = lane; w < static_cast<int>(sizeof(ScoreParams) / 8); w += 32) dst[w] = src[w];
    }
    __syncwarp();
    const ScoreParams &p = *s_desc;
    if (p.skip && *p.skip) continue;  // this complex is finished (e.g. a converged GA job)
    // split mode: item = (pose, chunk, receptor part), at least one chunk per
    // pose (an empty ligand's single chunk holds no atom); otherwise item =
    // pose
    const int R = SPLIT == 2 ? bp.rparts : 1;
    const int nchunks = SPLIT ? max(1, (p.nl + kChunk - 1) / kChunk) : (p.nl + kChunk - 1) / kChunk;
    const int per_pose = nchunks * R;
    const int pose = static_cast<int>(SPLIT ? kk / per_pose : kk);
    const int rem = SPLIT ? static_cast<int>(kk % per_pose) : 0;
    const int ch0 = rem / R, rpart = rem % R;
    const int ch1 = SPLIT ? ch0 + 1 : nchunks;
    const int gp = SPLIT ? static_cast<int>(bp.pose_start[lo]) + pose : 0;  // poses of a launch fit an int
    if (!p.models && lane < 16)
      reinterpret_cast<double *>(s_frame)[lane] = reinterpret_cast<const double *>(p.frames + pose)[lane];
    __syncwarp();
    const gd_pose_frame &f = *s_frame;
    const int nseg = (p.nr + kSeg - 1) / kSeg;
    long long q_issued = q;  // ring uses issued so far (lane 0 issues; read on failure)
    const float gv = p.guard_v, ge = p.guard_e, gdd = p.guard_d;
    // a row (receptor atom, ligand slot) whose atom lies farther than this
    // from the slot's bounding sphere has every FP32 d2 beyond the elec
    // cutoff and its guard band: all its terms, counts and guard tests are 0
    const float reach = sqrtf(225.01f + 2.0f * ge) + 0.01f;
    // ... and one farther than this has every FP32 d2 beyond the vdW cutoff
    // and its band (so beyond the desolvation one too): Coulomb terms only
    const float reach_v = sqrtf(144.01f + 2.0f * gv) + 0.01f;
    const float reach2 = reach * reach, reach_v2 = reach_v * reach_v;
    const float2 *tab = reinterpret_cast<const float2 *>(p.tab32);
    long long vdw_i = 0, elec_i = 0;  // 2^-32 fixed point
    double desolv_t = 0.0;
    bool failed = false;

    for (int ch = ch0; ch < ch1 && !failed; ++ch) {
      // Receptor segments within reach of the chunk: each slot's precomputed
      // sphere moves rigidly with the pose (its centre transformed exactly),
      // and a segment whose sphere lies beyond the elec reach of every slot
      // sphere holds only rows the row test would drop.  Explicit model
      // coordinates (no rigid pose) keep every segment.
      const bool cull = p.models == nullptr && p.lig_slot_sph != nullptr && p.rec_seg != nullptr;
      if (cull && lane < S) {
        const int sl = ch * S + lane;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        if (sl * 32 < p.nl) {
          const D4 sp = p.lig_slot_sph[sl];
          double X, Y, Z;
          transform_atom(f, p.cx, p.cy, p.cz, sp.x, sp.y, sp.z, X, Y, Z);
          v = make_float4(static_cast<float>(X - p.ox), static_cast<float>(Y - p.oy), static_cast<float>(Z - p.oz),
                          static_cast<float>(sp.w));
        }
        s_ssph[lane] = v;
      }
      __syncwarp();
      // this item's segments: those of its receptor part (g mod R = part),
      // culled for a rigid pose
      const int nseg_part = (nseg - rpart + R - 1) / R;
      int nk = nseg_part;
      bool listed = false;
      if (cull) {
        nk = 0;
        for (int g0 = 0; g0 < nseg; g0 += 32) {
          const int g = g0 + lane;
          bool keep = false;
          if (g < nseg && g % R == rpart) {
            const float4 sg = __ldg(&p.rec_seg[g]);
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2) {
              const float4 ss = s_ssph[s2];
              const float dx = sg.x - ss.x, dy = sg.y - ss.y, dz = sg.z - ss.z;
              const float lim = sg.w + ss.w + reach + 0.1f + 1e-3f * (sg.w + ss.w);
              keep = keep || (ss.w >= 0.0f && dx * dx + dy * dy + dz * dz < lim * lim);
            }
          }
          const unsigned m = __ballot_sync(kFull, keep);
          const int pos = nk + __popc(m & lt_mask);
          if (keep && pos < kSegListMax) s_segl[pos] = static_cast<uint16_t>(g);
          nk += __popc(m);
        }
        listed = nk <= kSegListMax;
        if (!listed) nk = nseg_part;  // too many to list: every segment of the part
        __syncwarp();
      }
      auto seg_at = [&](int k) { return listed ? static_cast<int>(s_segl[k]) : rpart + k * R; };
      if (lane == 0)
        for (int k = 0; k < nk && k < kWS; ++k)
          if (!(bp.drop_copy && item == 0 && ch == ch0 && k == 0))
            issue_seg(q + k, seg_at(k), p, s_pos, s_meta, s_bar);
      q_issued = q + min(nk, kWS);
      float lx[S], ly[S], lz[S], lq[S];
      int lt[S], lser[S], lcnt[S];
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int j = ch * kChunk + s * 32 + lane;
        lcnt[s] = 0;
        const bool on = j < p.nl;
        if (on) {
          double X, Y, Z;
          ligand_atom(p, f, pose, j, X, Y, Z);
          lx[s] = static_cast<float>(X - p.ox);
          ly[s] = static_cast<float>(Y - p.oy);
          lz[s] = static_cast<float>(Z - p.oz);
          lq[s] = static_cast<float>(p.lig_q[j]);
          lt[s] = p.lig_type[j];
          if (!GD_DCHECK(bp.err, lt[s] >= 0 && lt[s] < p.nt, 6)) lt[s] = 0;
          lser[s] = SERIAL ? p.lig_serial[j] : 0;
        } else {
          // far from every receptor atom, including the padding at +1e9
          lx[s] = ly[s] = lz[s] = -1.0e9f;
          lq[s] = 0.0f;
          lt[s] = 0;
          lser[s] = 0;
        }
        // bounding sphere of the slot's 32 atoms: with a rigid pose the
        // precomputed small enclosing sphere moved with it (s_ssph, smaller
        // than the centroid's sphere), else the centroid's of these atoms
        const unsigned on_mask = __ballot_sync(kFull, on);
        float cx = 0.0f, cy = 0.0f, cz = 0.0f, rr = 0.0f;
        if (!cull) {
          cx = on ? lx[s] : 0.f, cy = on ? ly[s] : 0.f, cz = on ? lz[s] : 0.f;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            cx += __shfl_xor_sync(kFull, cx, o);
            cy += __shfl_xor_sync(kFull, cy, o);
            cz += __shfl_xor_sync(kFull, cz, o);
          }
          const float inv = on_mask ? 1.0f / static_cast<float>(__popc(on_mask)) : 0.0f;
          cx *= inv;
          cy *= inv;
          cz *= inv;
          rr = on ? sqrtf((lx[s] - cx) * (lx[s] - cx) + (ly[s] - cy) * (ly[s] - cy) + (lz[s] - cz) * (lz[s] - cz))
                  : 0.0f;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) rr = fmaxf(rr, __shfl_xor_sync(kFull, rr, o));
        }
        // axis-aligned bounding box of the same atoms (half-widths widened
        // like the radius so that FP32 rounding never shrinks it)
        float lo_x = on ? lx[s] : 3.0e38f, lo_y = on ? ly[s] : 3.0e38f, lo_z = on ? lz[s] : 3.0e38f;
        float hi_x = on ? lx[s] : -3.0e38f, hi_y = on ? ly[s] : -3.0e38f, hi_z = on ? lz[s] : -3.0e38f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          lo_x = fminf(lo_x, __shfl_xor_sync(kFull, lo_x, o));
          lo_y = fminf(lo_y, __shfl_xor_sync(kFull, lo_y, o));
          lo_z = fminf(lo_z, __shfl_xor_sync(kFull, lo_z, o));
          hi_x = fmaxf(hi_x, __shfl_xor_sync(kFull, hi_x, o));
          hi_y = fmaxf(hi_y, __shfl_xor_sync(kFull, hi_y, o));
          hi_z = fmaxf(hi_z, __shfl_xor_sync(kFull, hi_z, o));
        }
        if (lane == 0) {
          s_blob[s] = !on_mask ? make_float4(0.0f, 0.0f, 0.0f, -1.0e30f)
                               : (cull ? s_ssph[s] : make_float4(cx, cy, cz, rr * 1.0001f + 0.01f));
          if (on_mask) {
            s_box[2 * s] = make_float4(0.5f * (lo_x + hi_x), 0.5f * (lo_y + hi_y), 0.5f * (lo_z + hi_z),
                                       0.5f * (hi_x - lo_x) * 1.0001f + 0.01f);
            s_box[2 * s + 1] = make_float4(0.5f * (hi_y - lo_y) * 1.0001f + 0.01f,
                                           0.5f * (hi_z - lo_z) * 1.0001f + 0.01f, 0.0f, 0.0f);
          } else {
            s_box[2 * s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            s_box[2 * s + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          }
        }
      }
      __syncwarp();
      // phase-1 role of this lane: row (slot my_s, atom my_a of each 8-atom round)
      const float4 myb = my_s < S ? s_blob[my_s] : make_float4(0.0f, 0.0f, 0.0f, -1.0e30f);
      const float mlim = myb.w + reach;
      const float mlim2 = (myb.w >= 0.0f) ? mlim * mlim : -1.0f;  // empty slot: no row kept
      const float mnear = myb.w + reach_v, mnear2 = mnear * mnear;
      long long fv = 0, fe = 0;  // this item's vdW and Coulomb sums, 2^-32 fixed point
      // per segment: flagged steps (high 16 bits) and recorded near rows (low 16)
      int seg_cnt = 0;
      for (int kk = 0; kk < nk; ++kk, ++q) {
        const int g = seg_at(kk);
        const int st = static_cast<int>(q % kWS);
        const bool ok = __all_sync(kFull, mbar_wait(&s_bar[st], static_cast<uint32_t>((q / kWS) & 1)));
        if (!ok) {
          failed = true;
          break;
        }
        const int gbase = g * kSeg;
        const int na = min(kSeg, p.nr - gbase);
        const int sbase = st * kSeg;

        // Phase 1: lane (slot, atom) tests one row against the slot's sphere.
        // Kept rows go to the slot's list: far rows (Coulomb only) from the
        // front, near rows from the back; each run is padded with the far
        // dummy atom to whole steps.
        int nf_mine = 0, nn_mine = 0;  // far / near rows of this lane's slot
        uint16_t *my_list = s_list + my_s * kList;
        for (int b0 = 0; b0 < na; b0 += kBlk) {
          const float4 ra = s_pos[sbase + b0 + my_a];  // atoms past nr are padding far away
          const float dx = ra.x - myb.x, dy = ra.y - myb.y, dz = ra.z - myb.z;
          const float dc2 = dx * dx + dy * dy + dz * dz;
          // distance from the atom to the slot's box: a second lower bound on
          // every pair distance of the row (either bound may drop the row or
          // make it far)
          const float4 bx0 = s_box[2 * (my_s & (kMaxS - 1))], bx1 = s_box[2 * (my_s & (kMaxS - 1)) + 1];
          const float ex = fmaxf(fabsf(ra.x - bx0.x) - bx0.w, 0.0f), ey = fmaxf(fabsf(ra.y - bx0.y) - bx1.x, 0.0f),
                      ez = fmaxf(fabsf(ra.z - bx0.z) - bx1.y, 0.0f);
          const float db2 = ex * ex + ey * ey + ez * ez;
          const bool keep = dc2 < mlim2 && db2 < reach2, nearr = dc2 < mnear2 && db2 < reach_v2;
          const unsigned Mf = __ballot_sync(kFull, keep && !nearr), Mn = __ballot_sync(kFull, keep && nearr);
          const uint16_t idx = static_cast<uint16_t>(sbase + b0 + my_a);
          // at most na <= kSeg rows per slot: far rows fill [0, nf), near rows
          // (kList - nn, kList - 1], with room for both paddings in between
          const int pf = nf_mine + __popc(Mf & my_group & lt_mask), pn = kList - 1 - nn_mine - __popc(Mn & my_group & lt_mask);
          if (keep && !nearr && GD_DCHECK(bp.err, pf >= 0 && pf < kList, 1)) my_list[pf] = idx;
          if (keep && nearr && GD_DCHECK(bp.err, pn >= 0 && pn < kList, 2)) my_list[pn] = idx;

          nf_mine += __popc(Mf & my_group);
          nn_mine += __popc(Mn & my_group);
        }
        if (my_s < S && my_a < kAtoms &&
            GD_DCHECK(bp.err, nf_mine + my_a < kList && kList - 1 - nn_mine - my_a >= 0, 3)) {
          my_list[nf_mine + my_a] = static_cast<uint16_t>(kFar);
          my_list[kList - 1 - nn_mine - my_a] = static_cast<uint16_t>(kFar);
        }
        __syncwarp();

        // Phase 2: every term of the kept rows, kAtoms rows per step
        float av = 0.0f, ae = 0.0f;  // ae: corrections from FP64 re-decisions (charge included)
#pragma unroll
        for (int s = 0; s < S; ++s) {
          float aes = 0.0f;  // sum of q_r / d2 over this slot's kept pairs
          const int nf = __shfl_sync(kFull, nf_mine, s * 8), nn = __shfl_sync(kFull, nn_mine, s * 8);
          const uint16_t *lst = s_list + s * kList;
          // far rows: Coulomb only
#pragma unroll 1
          for (int k0 = 0; k0 < nf; k0 += kAtoms) {
            int ix[kAtoms];
            float4 r[kAtoms];
#pragma unroll
            for (int i = 0; i < kAtoms; ++i) {
              ix[i] = lst[k0 + i];
              if (!GD_DCHECK(bp.err, ix[i] <= kFar, 4)) ix[i] = kFar;
              r[i] = s_pos[ix[i]];
            }
            bool amb = false;
#pragma unroll
            for (int i = 0; i < kAtoms; ++i) pair32_elec(r[i], lx[s], ly[s], lz[s], ge, aes, amb);
            if (__any_sync(kFull, amb)) {  // at most one entry per step: <= 4 * 18 per segment
              if (lane == 0 && GD_DCHECK(bp.err, (seg_cnt >> 16) < kMaxS * kList, 7))
                s_fixq[seg_cnt >> 16] = static_cast<uint16_t>(k0 | (s << 8));
              seg_cnt += 1 << 16;
            }
          }
          // near rows: every term; the first step may start in the padding
#pragma unroll 1
          for (int k0 = kList - (nn + kAtoms - 1) / kAtoms * kAtoms; k0 < kList; k0 += kAtoms) {
            int ix[kAtoms];
            float4 r[kAtoms];
            int rt[kAtoms], rs[kAtoms], rc[kAtoms];
#pragma unroll
            for (int i = 0; i < kAtoms; ++i) {
              ix[i] = lst[k0 + i];
              if (!GD_DCHECK(bp.err, ix[i] <= kFar, 4)) ix[i] = kFar;
              r[i] = s_pos[ix[i]];
              const int4 mt = s_meta[ix[i]];
              rt[i] = mt.x;
              if (!GD_DCHECK(bp.err, rt[i] >= 0 && rt[i] + lt[s] < p.nt * p.nt, 5)) rt[i] = 0;
              rs[i] = mt.y;
              rc[i] = 0;
            }
            bool amb = false;
#pragma unroll
            for (int i = 0; i < kAtoms; ++i)
              pair32<SERIAL, CLAMP>(r[i], rt[i], rs[i], tab, lx[s], ly[s], lz[s], lt[s], lser[s], gv, ge, gdd, av,
                                    aes, lcnt[s], rc[i], amb);
            if (__any_sync(kFull, amb)) {  // at most one entry per step: <= 4 * 18 per segment
              if (lane == 0 && GD_DCHECK(bp.err, (seg_cnt >> 16) < kMaxS * kList, 7))
                s_fixq[seg_cnt >> 16] = static_cast<uint16_t>(k0 | (s << 8));
              seg_cnt += 1 << 16;
            }
            // receptor burial counts of the step's rows: their ballots are
            // recorded here and added up once per segment (below); a step
            // with no pair within 8 A (about half of them) records nothing
            int any_rc = 0;
#pragma unroll
            for (int i = 0; i < kAtoms; ++i) any_rc |= rc[i];
            if (__any_sync(kFull, any_rc != 0)) {
#pragma unroll
              for (int i = 0; i < kAtoms; ++i) {
                const unsigned bm = __ballot_sync(kFull, rc[i] != 0);
                if (lane == i && GD_DCHECK(bp.err, (seg_cnt & 0xffff) + i < kMaxS * kList, 8)) {
                  s_cmask[(seg_cnt & 0xffff) + i] = bm;
                  s_cidx[(seg_cnt & 0xffff) + i] = static_cast<uint16_t>(ix[i]);
                }
              }
              seg_cnt += kAtoms;
            }
          }
          ae = __fmaf_rn(aes, lq[s], ae);
        }
        __syncwarp();
        // FP64 re-decisions of the flagged steps' pairs in the guard band
        const int nfix = seg_cnt >> 16, ncm = seg_cnt & 0xffff;
#pragma unroll 1
        for (int t = 0; t < nfix; ++t) {
          const int e = s_fixq[t], k0 = e & 255, s = e >> 8;
          const int j = ch * kChunk + s * 32 + lane;
          if (j >= p.nl) continue;
          double X, Y, Z;
          ligand_atom(p, f, pose, j, X, Y, Z);
          // the lane's FP32 coordinates, as in the chunk set-up
          const float fx = static_cast<float>(X - p.ox), fy = static_cast<float>(Y - p.oy),
                      fz = static_cast<float>(Z - p.oz);
          const float fq = static_cast<float>(p.lig_q[j]);
          const int ft = p.lig_type[j], fs = SERIAL ? p.lig_serial[j] : 0;
#pragma unroll 1
          for (int i = 0; i < kAtoms; ++i) {
            const int ixi = s_list[s * kList + k0 + i];
            if (ixi == kFar || !GD_DCHECK(bp.err, ixi < kFar, 4)) continue;
            const float4 ri = s_pos[ixi];
            if (!near_band(d2f(ri, fx, fy, fz), gv, ge, gdd)) continue;
            const int4 mt = s_meta[ixi];
            const FixOut fo = fix_pair<SERIAL, CLAMP>(p, X, Y, Z, ri, gbase + ixi - sbase, mt.x, mt.y, fx, fy, fz, fq,
                                                      ft, fs);
            av += fo.dv;
            ae += fo.de;
            if (fo.dl) {
              s_lfix[s * 32 + lane] += fo.dl;
              atomicAdd(&s_rc[ixi - sbase], fo.dl);
            }
          }
        }
        // receptor burial counts of the near rows (the far atom's ballots are 0)
        for (int t = lane; t < ncm; t += 32) {
          const unsigned bm = s_cmask[t];
          if (bm) atomicAdd(&s_rc[s_cidx[t] - sbase], __popc(bm));
        }
        seg_cnt = 0;
        fv += fx_energy(av, bp.err);
        fe += fx_energy(ae, bp.err);
        __syncwarp();
        // receptor burial counts of this segment into the per-item counters
        for (int i = lane; i < na; i += 32) {
          const int c = s_rc[i];
          if (c) {
            if (SPLIT) {
              // a count never exceeds the ligand's atoms (< 65,536 in split
              // launches), so the two halves of a word never carry into each other
              const int a = gbase + i;
              if (GD_DCHECK(bp.err, a < bp.max_nr, 10))
                atomicAdd(&bp.pcount[static_cast<size_t>(gp) * ((bp.max_nr + 1) >> 1) + (a >> 1)],
                          static_cast<unsigned>(c) << ((a & 1) * 16));
            }
            else bump_count(cnt, gbase + i, c);
            s_rc[i] = 0;
          }
        }
        __syncwarp();
        if (lane == 0 && kk + kWS < nk) {
          issue_seg(q + kWS, seg_at(kk + kWS), p, s_pos, s_meta, s_bar);
          q_issued = q + kWS + 1;
        }
      }
      if (failed) break;
      __syncwarp();
      // the chunk's per-lane partials (split and whole-pose items add them
      // alike, so both give bit-identical energies): ligand desolvation from
      // this chunk's burial counts; with receptor parts the counts are only
      // partial here and go to the pose's counters
      double dch = 0.0;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        lcnt[s] += s_lfix[s * 32 + lane];  // burial corrections of FP64 re-decisions
        s_lfix[s * 32 + lane] = 0;
        const int j = ch * kChunk + s * 32 + lane;
        if (R == 1) {
          if (j < p.nl) dch += p.lig_desolv[static_cast<size_t>(j) * 11 + min(lcnt[s], 10)];
        } else if (j < p.nl && lcnt[s] != 0 && GD_DCHECK(bp.err, j < bp.max_nl, 11)) {
          atomicAdd(&bp.lcount[static_cast<size_t>(gp) * bp.max_nl + j], static_cast<unsigned>(lcnt[s]));
        }
      }
      if (SPLIT) {
        const int slot = ch * R + rpart;
        if (!GD_DCHECK(bp.err, slot < bp.max_chunks, 9)) break;
        double *pt = bp.part + (static_cast<size_t>(gp) * bp.max_chunks + slot) * 96;
        reinterpret_cast<long long *>(pt)[lane] = fv;
        reinterpret_cast<long long *>(pt)[32 + lane] = fe;
        pt[64 + lane] = dch;
      } else {
        vdw_i += fv;
        elec_i += fe;
        desolv_t += dch;
      }
    }
    if (failed) {
      // a bulk copy did not land in time: record it, wait (bounded) for the
      // copies this warp still has in flight, and stop this warp
      if (lane == 0) {
        atomicExch(bp.err, kDevTimeout);
        for (long long u = q; u < q_issued; ++u) mbar_wait(&s_bar[u % kWS], static_cast<uint32_t>((u / kWS) & 1));
      }
      __syncwarp();
      return;
    }
    if (SPLIT) {
      // publish this chunk; the warp that completes the pose reduces it
      __threadfence();
      __syncwarp();
      int done = 0;
      if (lane == 0) done = atomicAdd(&bp.pdone[gp], 1);
      done = __shfl_sync(kFull, done, 0);
      if (done != per_pose - 1) continue;
      __threadfence();
      for (int c = 0; c < per_pose; ++c) {
        const long long *pi =
            reinterpret_cast<const long long *>(bp.part + (static_cast<size_t>(gp) * bp.max_chunks + c) * 96);
        vdw_i += __ldcg(pi + lane);
        elec_i += __ldcg(pi + 32 + lane);
      }
      // ligand desolvation chunk by chunk, in the same order and arithmetic
      // as whole-pose items
      for (int c = 0; c < nchunks; ++c) {
        if (R == 1) {
          desolv_t += __ldcg(bp.part + (static_cast<size_t>(gp) * bp.max_chunks + c) * 96 + 64 + lane);
        } else {
          double dc = 0.0;
          for (int s = 0; s < S; ++s) {
            const int j = c * kChunk + s * 32 + lane;
            if (j < p.nl) {
              const unsigned n = __ldcg(&bp.lcount[static_cast<size_t>(gp) * bp.max_nl + j]);
              dc += p.lig_desolv[static_cast<size_t>(j) * 11 + (n < 10u ? n : 10u)];
            }
          }
          desolv_t += dc;
        }
      }
      for (int i = lane; i < p.nr; i += 32) {
        const unsigned w = __ldcg(&bp.pcount[static_cast<size_t>(gp) * ((bp.max_nr + 1) >> 1) + (i >> 1)]);
        const unsigned c = (w >> ((i & 1) * 16)) & 0xffffu;
        desolv_t += p.rec_desolv[static_cast<size_t>(i) * 11 + (c < 10u ? c : 10u)];
      }
    } else {
      // receptor burial -> desolvation; reset the counters for the next item
      for (int i = lane; i < p.nr; i += 32) {
        const int c = cnt[i];
        desolv_t += p.rec_desolv[static_cast<size_t>(i) * 11 + (c < 10 ? c : 10)];
        cnt[i] = 0;
      }
    }
    const double vdw_t = static_cast<double>(warp_sum_ll(vdw_i)) * 0x1p-32;
    const double elec_t = static_cast<double>(warp_sum_ll(elec_i)) * 0x1p-32;
    desolv_t = warp_sum(desolv_t);
    // AIR: one restraint per lane, summed in restraint order
    double air = 0.0;
    int sat = 0;
    for (int r0 = 0; r0 < p.K; r0 += 32) {
      double term = 0.0;
      int ok = 0;
      const int r = r0 + lane;
      if (r < p.K) {
        const D4 a = p.restr_rec[r];
        double X, Y, Z;
        ligand_atom(p, f, pose, p.restr_lig[r], X, Y, Z);
        const double dist = sqrt(exact_d2(a.x, a.y, a.z, X, Y, Z));
        double v = 0.0;
        if (dist < 0.0) v = __dsub_rn(0.0, dist);
        else if (dist > 7.0) v = __dsub_rn(dist, 7.0);
        term = __dmul_rn(__dmul_rn(10.0, v), v);
        ok = dist <= 7.0;
      }
      for (int k = 0; k < 32 && r0 + k < p.K; ++k) {
        air = __dadd_rn(air, __shfl_sync(kFull, term, k));
        sat += __shfl_sync(kFull, ok, k);
      }
    }
    if (lane == 0) {
      const double ratio = p.K > 0 ? static_cast<double>(sat) / static_cast<double>(p.K) : 0.0;
      gd_pose_energy o;
      o.vdw = vdw_t;
      o.elec = elec_t;
      o.desolv = desolv_t;
      o.air = air;
      o.restraint_penalty = __dmul_rn(__dsub_rn(1.0, ratio), static_cast<double>(p.K));
      o.fitness = __dadd_rn(
          __dadd_rn(__dadd_rn(__dmul_rn(p.wv, vdw_t), __dmul_rn(p.we, elec_t)), __dmul_rn(p.wd, desolv_t)),
          __dmul_rn(p.wa, air));
      p.out[pose] = o;
    }
    __syncwarp();
  }
}

// Split-mode kernel (a work item is one ligand chunk of a pose): one variant,
// 4 slots and 4 rows per step, five CTAs per SM, used for launches with few
// poses per warp.
constexpr int kSplitTune = -1;
constexpr int kSplitPartsTune = -2;  // the split kernel with receptor parts

// Kernel variants.  The common case (no equal receptor/ligand serials, no
// clamp needed) has a tuning grid of slots per lane S, receptor atoms per
// inner step A and minimum CTAs per SM (register cap); the rare cases run
// one variant.  The tuning value encodes S + 16 (A = 2) or + 64 (A = 4),
// + 256 for the register cap of five resident CTAs per SM.
template <typename F>
cudaError_t with_variant(int tune, bool serial, bool clamp, F f) {
  if (tune == kSplitTune) return f(k_score_f32w<4, 4, 5, false, false, 1>);
  if (tune == kSplitPartsTune) return f(k_score_f32w<4, 4, 5, false, false, 2>);
  if (serial || clamp) {
    if (serial && clamp) return f(k_score_f32w<4, 1, 4, true, true, 0>);
    if (serial) return f(k_score_f32w<4, 1, 4, true, false, 0>);
    return f(k_score_f32w<4, 1, 4, false, true, 0>);
  }
  switch (tune) {
    case 4: return f(k_score_f32w<4, 1, 4, false, false, 0>);
    case 64 + 2: return f(k_score_f32w<2, 4, 4, false, false, 0>);
    case 64 + 4: return f(k_score_f32w<4, 4, 4, false, false, 0>);
    case 256 + 64 + 2: return f(k_score_f32w<2, 4, 5, false, false, 0>);
    case 16 + 4: return f(k_score_f32w<4, 2, 4, false, false, 0>);
    default: return f(k_score_f32w<4, 4, 5, false, false, 0>);  // 256 + 64 + 4 = kDefaultF32Tune
  }
}

// The dynamic shared memory of a CTA can exceed the 48 KB default (receptors
// near kCntSmemMax keep their burial counters there): the kernel's limit is
// raised before the occupancy query, which otherwise reports an invalid
// configuration.
cudaError_t occupancy_var(int tune, bool serial, bool clamp, size_t smem, int *per_sm) {
  return with_variant(tune, serial, clamp, [&](auto kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kern, kWarps * 32, smem);
  });
}

cudaError_t launch_var(int tune, const BatchParams &bp, bool serial, bool clamp, size_t smem, int grid,
                       cudaStream_t st) {
  return with_variant(tune, serial, clamp, [&](auto kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    kern<<<grid, kWarps * 32, smem, st>>>(bp);
    return cudaGetLastError();
  });
}

}  // namespace

// Work items are taken from the queue in descriptor order: put the complexes
// with the costliest poses first so that the last items of a launch are the
// cheap ones (longest-processing-time-first).
static std::vector<ScoreParams> lpt_order(const std::vector<ScoreParams> &descs) {
  std::vector<ScoreParams> v = descs;
  std::stable_sort(v.begin(), v.end(), [](const ScoreParams &a, const ScoreParams &b) {
    return static_cast<long long>(a.nr) * a.nl > static_cast<long long>(b.nr) * b.nl;
  });
  return v;
}

// Launch geometry of a batch: slots per lane, shared memory, grid.
struct BatchPlan {
  int tune, smem_cnt, max_nr, grid;
  size_t smem;
  std::vector<long long> start;       // work-item prefix per complex
  std::vector<long long> pose_start;  // pose prefix per complex
  int split = 0, max_chunks = 1;
  int rparts = 1, max_nl = 0;  // receptor parts per chunk (split mode), longest ligand
  size_t part_b = 0, cnt_b = 0, done_b = 0, lcnt_b = 0;  // split-mode scratch
};

constexpr size_t kSplitScratchMax = size_t(4) << 30;  // split scratch beyond this: whole poses
constexpr int kMaxRparts = 8;  // receptor parts per chunk, at most (GD_TUNE_RPARTS accepts 1..8)

static size_t al256(size_t b) { return (b + 255) / 256 * 256; }

// Work items are the ligand chunks of the poses (split mode) whenever the
// split scratch fits (4 GiB and the context's HBM budget): no warp waits on a
// long pose at the end of a launch, which matters most with few poses per
// warp (one GA generation of a few jobs, one docking run's population, a few
// thousand poses of a large complex) and was measured no slower with many.
// Whole poses per item otherwise; the energies are bit-identical either way.
static gd_status plan_batch(gd_context *ctx, const std::vector<ScoreParams> &descs, bool serial, bool clamp,
                            int slots, bool allow_split, BatchPlan *pl) {
  const int ncx = static_cast<int>(descs.size());
  const int chunk_split = 32 * 4;  // the split kernel's chunk of ligand atoms
  pl->start.assign(ncx + 1, 0);
  pl->pose_start.assign(ncx + 1, 0);
  pl->max_nr = 0;
  pl->max_nl = 0;
  pl->max_chunks = 1;
  long long chunk_items = 0;  // (pose, chunk) items of a split launch
  int max_nseg = 1;
  for (int c = 0; c < ncx; ++c) {
    pl->pose_start[c + 1] = pl->pose_start[c] + descs[c].n_poses;
    pl->max_nr = std::max(pl->max_nr, descs[c].nr);
    pl->max_nl = std::max(pl->max_nl, descs[c].nl);
    const int nch = std::max(1, (descs[c].nl + chunk_split - 1) / chunk_split);
    pl->max_chunks = std::max(pl->max_chunks, nch);
    chunk_items += static_cast<long long>(descs[c].n_poses) * nch;
    max_nseg = std::max(max_nseg, (descs[c].nr + kSeg - 1) / kSeg);
  }
  const long long poses = pl->pose_start[ncx];
  pl->tune = slots;
  auto fit = [&](int smem_cnt, int *per_sm) -> cudaError_t {
    pl->smem_cnt = smem_cnt;
    pl->smem = warp_layout(smem_cnt).total * kWarps;
    cudaError_t e = occupancy_var(pl->tune, serial, clamp, pl->smem, per_sm);
    if (e == cudaSuccess && *per_sm < 1) e = cudaErrorInvalidConfiguration;
    return e;
  };
  int per_sm = 0;
  cudaError_t e = fit(pl->max_nr <= kCntSmemMax ? ((pl->max_nr + 15) / 16) * 16 : 0, &per_sm);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched scoring occupancy");
  // receptor parts: a launch with fewer (pose, chunk) items than about two
  // rounds of the split kernel's resident warps splits each chunk's receptor
  // into R interleaved segment sets, so that the SMs fill, keeping at least
  // two segments per part.  A part's item also pays the chunk's set-up, so
  // for receptors of fewer than 16 segments the target shrinks in
  // proportion (measured on receptors of 6, 40 and 107 segments at 150 to
  // 1,200 poses).  GD_TUNE_RPARTS forces R.  The energies do not depend on R
  // (fixed-point sums).
  int split_per_sm = 0;
  {
    const int keep_tune = pl->tune;
    pl->tune = kSplitTune;
    e = fit(0, &split_per_sm);
    pl->tune = keep_tune;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batched scoring occupancy");
    e = fit(pl->max_nr <= kCntSmemMax ? ((pl->max_nr + 15) / 16) * 16 : 0, &per_sm);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batched scoring occupancy");
  }
  const long long target = static_cast<long long>(std::min(2.0, max_nseg / 8.0) * split_per_sm * kWarps *
                                                  ctx->sm_count);
  int R = ctx->tune_rparts > 0 ? ctx->tune_rparts
                               : static_cast<int>(std::min<long long>(
                                     kMaxRparts, std::max<long long>(1, (target + std::max(chunk_items, 1LL) - 1) /
                                                                            std::max(chunk_items, 1LL))));
  if (ctx->tune_rparts <= 0) R = std::max(1, std::min(R, max_nseg / 2));
  auto split_bytes = [&](int r, size_t *part_b, size_t *cnt_b, size_t *lcnt_b) {
    *part_b = static_cast<size_t>(poses) * pl->max_chunks * r * 96 * sizeof(double);
    *cnt_b = static_cast<size_t>(poses) * ((pl->max_nr + 1) / 2) * sizeof(unsigned);
    *lcnt_b = r > 1 ? static_cast<size_t>(poses) * std::max(pl->max_nl, 1) * sizeof(unsigned) : 0;
    const size_t b = al256(*part_b) + al256(*cnt_b) + al256(static_cast<size_t>(poses) * sizeof(int)) + al256(*lcnt_b);
    return b <= kSplitScratchMax && (ctx->budget == 0 || ctx->in_use + b <= ctx->budget);
  };
  size_t part_b = 0, cnt_b = 0, lcnt_b = 0;
  bool fits = split_bytes(R, &part_b, &cnt_b, &lcnt_b);
  if (!fits && R > 1 && ctx->tune_rparts <= 0) {
    R = 1;
    fits = split_bytes(R, &part_b, &cnt_b, &lcnt_b);
  }
  pl->split = 0;
  // split launches keep receptor burial counts in 16 bits: ligands up to 65,535 atoms
  if (allow_split && fits && poses > 0 && (pl->max_chunks > 1 || R > 1) && !serial && !clamp && pl->max_nl < 65536)
    pl->split = ctx->tune_split != 1;
  if (pl->split) {
    pl->rparts = R;
    pl->part_b = part_b;
    pl->cnt_b = cnt_b;
    pl->lcnt_b = lcnt_b;
    pl->done_b = static_cast<size_t>(poses) * sizeof(int);
    pl->tune = R > 1 ? kSplitPartsTune : kSplitTune;
    e = fit(0, &per_sm);  // burial counters live in the split scratch
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batched scoring occupancy");
  } else {
    pl->rparts = 1;
    pl->part_b = pl->cnt_b = pl->done_b = pl->lcnt_b = 0;
  }
  for (int c = 0; c < ncx; ++c) {
    const long long per_pose =
        pl->split ? static_cast<long long>(std::max(1, (descs[c].nl + chunk_split - 1) / chunk_split)) * pl->rparts : 1;
    pl->start[c + 1] = pl->start[c] + static_cast<long long>(descs[c].n_poses) * per_pose;
  }
  const long long items = pl->start[ncx];
  pl->grid = static_cast<int>(std::max<long long>(
      1, std::min<long long>((items + kWarps - 1) / kWarps, static_cast<long long>(per_sm) * ctx->sm_count)));
  return GD_OK;
}

// Layout of the argument block: descriptors, item prefix, work counter, pose
// prefix, per-warp global burial counters (large receptors, whole-pose
// items), split-mode partials, receptor burial counts, item counters and
// (receptor parts) ligand burial counts.
struct ArgLayout {
  size_t desc, start, queue, pstart, gcounts, part, pcount, pdone, lcount, total;
};

static ArgLayout arg_layout(int ncx, const BatchPlan &pl, size_t gcount_bytes) {
  ArgLayout L{};
  size_t o = 0;
  L.desc = o;
  o += al256(sizeof(ScoreParams) * ncx);
  L.start = o;
  o += al256(sizeof(long long) * (ncx + 1));
  L.queue = o;
  o += al256(sizeof(unsigned long long));
  L.pstart = o;
  o += al256(sizeof(long long) * (ncx + 1));
  L.gcounts = o;
  o += al256(gcount_bytes);
  L.part = o;
  o += al256(pl.part_b);
  L.pcount = o;
  o += al256(pl.cnt_b);
  L.pdone = o;
  o += al256(pl.done_b);
  L.lcount = o;
  o += al256(pl.lcnt_b);
  L.total = o;
  return L;
}

static size_t gcount_stride(const BatchPlan &pl) {
  return (pl.smem_cnt || pl.split) ? 0 : ((pl.max_nr + 127) / 128) * 128;
}

static gd_status upload_args(gd_context *ctx, const std::vector<ScoreParams> &descs, const BatchPlan &pl,
                             const ArgLayout &L, char *arg, cudaStream_t stream, bool sync) {
  const int ncx = static_cast<int>(descs.size());
  // staged from pageable memory: the copy has left the host buffer when the
  // call returns, so back-to-back launches cannot race on it
  std::vector<char> h(L.gcounts);
  std::memcpy(h.data() + L.desc, descs.data(), sizeof(ScoreParams) * ncx);
  std::memcpy(h.data() + L.start, pl.start.data(), sizeof(long long) * (ncx + 1));
  std::memcpy(h.data() + L.pstart, pl.pose_start.data(), sizeof(long long) * (ncx + 1));
  const cudaError_t e = sync ? cudaMemcpy(arg, h.data(), h.size(), cudaMemcpyHostToDevice)
                             : cudaMemcpyAsync(arg, h.data(), h.size(), cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched scoring arguments");
  return GD_OK;
}

// Reset the work counter (and the split-mode counters) and launch.
static gd_status launch_args(gd_context *ctx, int ncx, const BatchPlan &pl, const ArgLayout &L, char *arg,
                             bool serial, bool clamp, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(arg + L.queue, 0, sizeof(unsigned long long), stream);
  if (e == cudaSuccess && pl.split) e = cudaMemsetAsync(arg + L.pcount, 0, L.total - L.pcount, stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched scoring reset");
  BatchParams bp{};
  bp.descs = reinterpret_cast<const ScoreParams *>(arg + L.desc);
  bp.item_start = reinterpret_cast<const long long *>(arg + L.start);
  bp.ncx = ncx;
  bp.total = pl.start[ncx];
  bp.queue = reinterpret_cast<unsigned long long *>(arg + L.queue);
  const size_t gs = gcount_stride(pl);
  bp.gcounts = gs ? reinterpret_cast<uint8_t *>(arg + L.gcounts) : nullptr;
  bp.gcount_stride = static_cast<int>(gs);
  bp.smem_cnt = pl.smem_cnt;
  bp.max_nr = pl.max_nr;
  bp.warp_smem = static_cast<int>(warp_layout(pl.smem_cnt).total);
  bp.err = ctx->d_err;
  bp.split = pl.split;
  bp.drop_copy = ctx->tune_fault == 1;
  bp.pose_start = reinterpret_cast<const long long *>(arg + L.pstart);
  bp.max_chunks = pl.max_chunks * pl.rparts;
  bp.part = pl.split ? reinterpret_cast<double *>(arg + L.part) : nullptr;
  bp.pcount = pl.split ? reinterpret_cast<unsigned *>(arg + L.pcount) : nullptr;
  bp.pdone = pl.split ? reinterpret_cast<int *>(arg + L.pdone) : nullptr;
  bp.rparts = pl.split ? pl.rparts : 1;
  bp.lcount = pl.split && pl.rparts > 1 ? reinterpret_cast<unsigned *>(arg + L.lcount) : nullptr;
  bp.max_nl = pl.max_nl;
  e = launch_var(pl.tune, bp, serial, clamp, pl.smem, pl.grid, stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched scoring launch");
  return GD_OK;
}

// Score the poses of several complexes in one persistent launch (FP32 form).
// descs[c] describes complex c with its frames/models, outputs and pose count.
gd_status launch_score_batch_f32(gd_context *ctx, const std::vector<ScoreParams> &descs_in, bool serial, bool clamp,
                                 int slots, cudaStream_t stream) {
  const std::vector<ScoreParams> descs = lpt_order(descs_in);
  const int ncx = static_cast<int>(descs.size());
  if (ncx == 0) return GD_OK;
  BatchPlan pl;
  gd_status s = plan_batch(ctx, descs, serial, clamp, slots, true, &pl);
  if (s != GD_OK) return s;
  if (pl.start[ncx] == 0) return GD_OK;
  const ArgLayout L = arg_layout(ncx, pl, gcount_stride(pl) * static_cast<size_t>(pl.grid) * kWarps);
  s = ensure_batch_scratch(ctx, L.total);
  if (s != GD_OK) return s;
  char *arg = static_cast<char *>(ctx->d_batch);
  s = upload_args(ctx, descs, pl, L, arg, stream, false);
  if (s != GD_OK) return s;
  return launch_args(ctx, ncx, pl, L, arg, serial, clamp, stream);
}

// A batched scoring launch whose argument block is uploaded once and whose
// launch (counter resets + kernel) can be replayed, e.g. inside a captured
// CUDA graph.
struct BatchLaunch {
  BatchPlan plan;
  ArgLayout layout{};
  bool serial = false, clamp = false;
  char *d_arg = nullptr;
  int ncx = 0;
};

gd_status batch_prepare(gd_context *ctx, const std::vector<ScoreParams> &descs_in, bool serial, bool clamp, int slots,
                        BatchLaunch **out) {
  *out = nullptr;
  const std::vector<ScoreParams> descs = lpt_order(descs_in);
  BatchLaunch *b = new BatchLaunch();
  b->serial = serial;
  b->clamp = clamp;
  b->ncx = static_cast<int>(descs.size());
  gd_status s = plan_batch(ctx, descs, serial, clamp, slots, true, &b->plan);
  if (s != GD_OK) {
    delete b;
    return s;
  }
  b->layout = arg_layout(b->ncx, b->plan, gcount_stride(b->plan) * static_cast<size_t>(b->plan.grid) * kWarps);
  void *p = nullptr;
  s = dev_alloc(ctx, b->layout.total, &p);
  if (s != GD_OK) {
    delete b;
    return s;
  }
  b->d_arg = static_cast<char *>(p);
  s = upload_args(ctx, descs, b->plan, b->layout, b->d_arg, nullptr, true);
  if (s != GD_OK) {
    batch_free(ctx, b);
    return s;
  }
  *out = b;
  return GD_OK;
}

gd_status batch_launch(gd_context *ctx, BatchLaunch *b, cudaStream_t stream) {
  if (b->plan.start[b->ncx] == 0) return GD_OK;
  return launch_args(ctx, b->ncx, b->plan, b->layout, b->d_arg, b->serial, b->clamp, stream);
}

void batch_free(gd_context *ctx, BatchLaunch *b) {
  if (!b) return;
  if (b->d_arg) dev_free(ctx, b->d_arg, b->layout.total);
  delete b;
}

// ---------------------------------------------------------------------------
// Scoring without any device allocation.
//
// Some hosts of this library cannot allocate device memory once scoring
// starts: a docking service that hands the whole GPU to a pool allocator at
// start-up (a cudaMalloc from inside the scoring path would fail or fragment
// that pool), or a real-time host loop that forbids the unbounded latency of
// an allocation.  For them the FP32 scoring kernel can take its small argument
// block (complex descriptor, pose-count prefix sums, work counter) from the
// file-scope array below instead of from context scratch memory.  The array
// is kNoAllocScratchBytes bytes on every GPU that loads the library and stays
// allocated until the process exits.  In host code its name is only a
// stand-in: the device address is looked up once per device with
// cudaGetSymbolAddress while that device is current.
constexpr size_t kNoAllocScratchBytes = 4096;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up on
// the first call for that device).
gd_status noalloc_scratch(gd_context *ctx, void **out) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices) return fail(ctx, GD_ERR_INVALID_ARG, "device index too large");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[ctx->device]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) return cuda_fail(ctx, e, "cudaGetSymbolAddress(no-allocation scratch)");
    g_noalloc_addr[ctx->device] = ptr;
  }
  *out = g_noalloc_addr[ctx->device];
  return GD_OK;
}
}  // namespace

}  // namespace gd

extern "C" gd_status gd_score_frames_device_noalloc(gd_complex *cx, const gd_pose_frame *d_frames, int32_t n,
                                                    double max_displacement, gd_pose_energy *d_out, void *stream) {
  using namespace gd;
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  if (n < 0 || (n > 0 && (!d_frames || !d_out))) return fail(ctx, GD_ERR_INVALID_ARG, "bad frames/out");
  if (!(max_displacement >= 0.0)) return fail(ctx, GD_ERR_INVALID_ARG, "bad max_displacement");
  if (cx->nr > kCntSmemMax)
    return fail(ctx, GD_ERR_INVALID_ARG,
                "receptor has " + std::to_string(cx->nr) + " atoms; scoring without allocation handles at most " +
                    std::to_string(kCntSmemMax));
  static_assert(4 * 256 + 2 * 256 + sizeof(ScoreParams) <= kNoAllocScratchBytes,
                "no-allocation scratch too small for one complex");
  if (n == 0) return GD_OK;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  void *scratch = nullptr;
  gd_status s = noalloc_scratch(ctx, &scratch);
  if (s != GD_OK) return s;
  const std::vector<ScoreParams> descs{make_params(cx, d_frames, nullptr, n, d_out, max_displacement)};
  const int slots = ctx->tune_f32_slots ? ctx->tune_f32_slots : kDefaultF32Tune;
  BatchPlan pl;
  s = plan_batch(ctx, descs, cx->serial_overlap, cx->need_clamp, slots, false, &pl);
  if (s != GD_OK) return s;
  // whole-pose items with counters in shared memory (receptor <= kCntSmemMax
  // atoms): the argument block is all the scratch there is
  const ArgLayout L = arg_layout(1, pl, 0);
  if (L.total > kNoAllocScratchBytes) return fail(ctx, GD_ERR_STATE, "no-allocation scratch too small");
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  char *arg = static_cast<char *>(scratch);
  s = upload_args(ctx, descs, pl, L, arg, st, false);
  if (s != GD_OK) return s;
  return launch_args(ctx, 1, pl, L, arg, cx->serial_overlap, cx->need_clamp, st);
}

