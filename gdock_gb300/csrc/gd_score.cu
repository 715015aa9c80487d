// Population fitness kernels: pose transform + all-pairs receptor x ligand
// soft-core LJ, Coulomb (epsilon = r), desolvation burial counts and the AIR
// restraint term, one pose per CTA iteration of a persistent grid.
//
// Reference arithmetic (gdock): transform src/structure.rs:80-131 and
// src/chromosome.rs:79-83; energies src/fitness.rs:57-302; per-pose
// combination src/chromosome.rs:110-127.
//
// Layout.  Receptor atoms are streamed through shared memory in tiles of
// kTile atoms by bulk (TMA) copies into a kStages-deep ring guarded by
// mbarriers; the receptor stream is the same for every pose, so the ring runs
// continuously across the poses a CTA owns.  Each thread holds S ligand atoms
// of the current pose ("slots", atoms tid, tid+NT, ... of the chunk) in
// registers after transforming them in FP64 with the reference's operation
// order, so coordinates are bit-identical to gdock's.  Ligands longer than
// NT*S atoms are processed in chunks, each streaming the whole receptor.
//
// FP32 form: per-pair terms in FP32, partial sums per receptor tile folded
// into per-thread Kahan accumulators, FP64 per-pose reduction.  Every cutoff
// decision is made on d2 against the FP32 image of the cutoff; pairs whose
// FP32 d2 lies within a guard band of a discontinuous cutoff (1, 8, 12,
// 15 A) are re-decided in FP64 from the exact coordinates and the FP32
// contribution corrected, so that all decisions equal the FP64 ones.
//
// FP64 form: the plain method, FP64 throughout, decisions against exact
// thresholds on d2.
#include <algorithm>
#include <cmath>

#include "gd_internal.cuh"

namespace gd {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared (the TMA engine), completing on an mbarrier.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait on an mbarrier phase: false after kWaitLimitNs of wall time
// (or kSpinLimit polls), so that a copy that never lands ends the kernel
// with an error instead of a hang.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t i = 1; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 0 && global_ns() - t0 > kWaitLimitNs) return false;
  }
  return false;
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Rigid transform of one ligand atom with the reference's operation order
// (src/structure.rs:83-115, then displace :119-131); explicit _rn intrinsics
// keep the compiler from fusing multiply-adds, so the result is bit-identical
// to the host's double arithmetic.
__device__ __forceinline__ void transform_atom(const gd_pose_frame &f, double cx, double cy, double cz,
                                               double xo, double yo, double zo, double &X, double &Y,
                                               double &Z) {
  const double x = __dsub_rn(xo, cx), y = __dsub_rn(yo, cy), z = __dsub_rn(zo, cz);
  const double nx = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(x, f.ca), f.cb), __dmul_rn(y, f.m01)),
                              __dmul_rn(z, f.m02));
  const double ny = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(x, f.sa), f.cb), __dmul_rn(y, f.m11)),
                              __dmul_rn(z, f.m12));
  const double nz = __dadd_rn(__dadd_rn(__dmul_rn(-x, f.sb), __dmul_rn(__dmul_rn(y, f.cb), f.sg)),
                              __dmul_rn(__dmul_rn(z, f.cb), f.cg));
  X = __dadd_rn(__dadd_rn(nx, cx), f.dx);
  Y = __dadd_rn(__dadd_rn(ny, cy), f.dy);
  Z = __dadd_rn(__dadd_rn(nz, cz), f.dz);
}

// Exact ligand coordinates of atom j of the current pose.
__device__ __forceinline__ void ligand_atom(const ScoreParams &p, const gd_pose_frame &f, int pose, int j,
                                            double &X, double &Y, double &Z) {
  if (p.models) {
    const double *m = p.models + (static_cast<size_t>(pose) * p.nl + j) * 3;
    X = m[0];
    Y = m[1];
    Z = m[2];
  } else {
    transform_atom(f, p.cx, p.cy, p.cz, p.lig_x[j], p.lig_y[j], p.lig_z[j], X, Y, Z);
  }
}

// structure::distance squared, (dx*dx + dy*dy) + dz*dz (src/structure.rs:312-317)
__device__ __forceinline__ double exact_d2(double ax, double ay, double az, double bx, double by, double bz) {
  const double dx = __dsub_rn(ax, bx), dy = __dsub_rn(ay, by), dz = __dsub_rn(az, bz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Block-wide FP64 sum of three values; result valid in thread 0.
template <int NT>
__device__ __forceinline__ void block_sum3(double &a, double &b, double &c, double *s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  c = warp_sum(c);
  if (lane == 0) {
    s_red[warp * 3 + 0] = a;
    s_red[warp * 3 + 1] = b;
    s_red[warp * 3 + 2] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = c = 0.0;
    for (int w = 0; w < NT / 32; ++w) {
      a += s_red[w * 3 + 0];
      b += s_red[w * 3 + 1];
      c += s_red[w * 3 + 2];
    }
  }
}

// AIR energy and satisfied-restraint count in restraint order
// (src/fitness.rs:205-267, src/restraints.rs:11-40); one thread.
__device__ void air_terms(const ScoreParams &p, const gd_pose_frame &f, int pose, double &air, int &sat) {
  air = 0.0;
  sat = 0;
  for (int r = 0; r < p.K; ++r) {
    const D4 a = p.restr_rec[r];
    double X, Y, Z;
    ligand_atom(p, f, pose, p.restr_lig[r], X, Y, Z);
    const double dist = sqrt(exact_d2(a.x, a.y, a.z, X, Y, Z));
    double v = 0.0;
    if (dist < 0.0) v = __dsub_rn(0.0, dist);
    else if (dist > 7.0) v = __dsub_rn(dist, 7.0);
    air = __dadd_rn(air, __dmul_rn(__dmul_rn(10.0, v), v));
    if (dist <= 7.0) ++sat;
  }
}

// Final per-pose record (src/chromosome.rs:111-127).
__device__ void write_pose(const ScoreParams &p, int pose, double vdw, double elec, double desolv,
                           const gd_pose_frame &f) {
  double air;
  int sat;
  air_terms(p, f, pose, air, sat);
  const double ratio = p.K > 0 ? static_cast<double>(sat) / static_cast<double>(p.K) : 0.0;
  gd_pose_energy o;
  o.vdw = vdw;
  o.elec = elec;
  o.desolv = desolv;
  o.air = air;
  o.restraint_penalty = __dmul_rn(__dsub_rn(1.0, ratio), static_cast<double>(p.K));
  o.fitness = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(p.wv, vdw), __dmul_rn(p.we, elec)), __dmul_rn(p.wd, desolv)),
                        __dmul_rn(p.wa, air));
  p.out[pose] = o;
}

struct SmemLayout {
  size_t pos, meta, bars, tab, frame, red, rcnt, total;
};

template <typename PosT>
__host__ __device__ inline SmemLayout smem_layout(int nt, int nr, int nthreads, size_t tab_entry) {
  SmemLayout L;
  size_t o = 0;
  auto al = [&](size_t a) { o = (o + a - 1) / a * a; };
  L.pos = o;
  o += sizeof(PosT) * kStages * kTile;
  al(16);
  L.meta = o;
  o += sizeof(int2) * kStages * kTile;
  al(16);
  L.bars = o;
  o += 8 * 8;
  al(16);
  L.tab = o;
  o += tab_entry * nt * nt;
  al(16);
  L.frame = o;
  o += sizeof(gd_pose_frame);
  al(16);
  L.red = o;
  o += sizeof(double) * 3 * (nthreads / 32);
  al(16);
  L.rcnt = o;
  o += sizeof(uint32_t) * nr;
  al(16);
  L.total = o;
  return L;
}

// Producer side of the receptor ring: tile q of the CTA's sequence.
template <typename PosT>
__device__ __forceinline__ void issue_tile(long long q, int n_tiles, const PosT *g_pos, const int2 *g_meta,
                                           PosT *s_pos, int2 *s_meta, uint64_t *s_full) {
  const int st = static_cast<int>(q % kStages);
  const int t = static_cast<int>(q % n_tiles);
  mbar_expect_tx(&s_full[st], kTile * (sizeof(PosT) + sizeof(int2)));
  bulk_g2s(&s_pos[st * kTile], g_pos + static_cast<size_t>(t) * kTile, kTile * sizeof(PosT), &s_full[st]);
  bulk_g2s(&s_meta[st * kTile], g_meta + static_cast<size_t>(t) * kTile, kTile * sizeof(int2), &s_full[st]);
}

// After an abort: wait (bounded) for copies still in flight, then return.
__device__ void drain(uint64_t *s_full, long long q_from, long long q_to) {
  for (long long q = q_from; q < q_to; ++q) mbar_wait(&s_full[q % kStages], static_cast<uint32_t>((q / kStages) & 1));
}

// --------------------------------------------------------------- FP32 ----

// Receptor atoms per culling block: each block of kBlk consecutive receptor
// atoms carries a bounding sphere; a (block, warp slot) pair is skipped when
// the spheres are further apart than the 15 A electrostatics cutoff (every
// term and count is exactly zero there, and no pair is near a cutoff).
constexpr int kBlk = 8;

struct SmemLayout32 {
  size_t pos, meta, sph, bars, tab, frame, red, blob, rcnt, total;
};

__host__ __device__ inline SmemLayout32 smem_layout32(int nt, int nr, int nthreads) {
  SmemLayout32 L;
  size_t o = 0;
  auto al = [&](size_t a) { o = (o + a - 1) / a * a; };
  L.pos = o;
  o += sizeof(float4) * kStages * kTile;
  L.meta = o;
  o += sizeof(int2) * kStages * kTile;
  L.sph = o;
  o += sizeof(float4) * kStages * (kTile / kBlk);
  L.bars = o;
  o += 8 * 8;
  al(16);
  L.tab = o;
  o += sizeof(float2) * nt * nt;
  al(16);
  L.frame = o;
  o += sizeof(gd_pose_frame);
  al(16);
  L.red = o;
  o += sizeof(double) * 3 * (nthreads / 32);
  al(16);
  L.blob = o;
  o += sizeof(float4) * 8 * (nthreads / 32);
  al(16);
  L.rcnt = o;
  o += sizeof(uint32_t) * nr;
  al(16);
  L.total = o;
  return L;
}

__device__ __forceinline__ void issue_tile32(long long q, int n_tiles, const ScoreParams &p, float4 *s_pos,
                                             int2 *s_meta, float4 *s_sph, uint64_t *s_full) {
  const int st = static_cast<int>(q % kStages);
  const int t = static_cast<int>(q % n_tiles);
  constexpr uint32_t kBytes = kTile * (sizeof(float4) + sizeof(int2)) + (kTile / kBlk) * sizeof(float4);
  mbar_expect_tx(&s_full[st], kBytes);
  bulk_g2s(&s_pos[st * kTile], p.rec_pos32 + static_cast<size_t>(t) * kTile, kTile * sizeof(float4), &s_full[st]);
  bulk_g2s(&s_meta[st * kTile], p.rec_meta + static_cast<size_t>(t) * kTile, kTile * sizeof(int2), &s_full[st]);
  bulk_g2s(&s_sph[st * (kTile / kBlk)], p.rec_sph32 + static_cast<size_t>(t) * (kTile / kBlk),
           (kTile / kBlk) * sizeof(float4), &s_full[st]);
}

// acc += v when |t| < lim (predicated add, no select)
__device__ __forceinline__ void add_if_abs_lt(float &acc, float t, float lim, float v) {
  asm("{\n\t.reg .pred p;\n\tsetp.lt.f32 p, %1, %2;\n\t@p add.f32 %0, %0, %3;\n\t}" : "+f"(acc)
      : "f"(fabsf(t)), "f"(lim), "f"(v));
}
// both counters += 1 when d2 < 64
__device__ __forceinline__ void count_if_lt64(int &a, int &b, float d2) {
  asm("{\n\t.reg .pred p;\n\tsetp.lt.f32 p, %2, 0f42800000;\n\t@p add.s32 %0, %0, 1;\n\t@p add.s32 %1, %1, 1;\n\t}"
      : "+r"(a), "+r"(b)
      : "f"(d2));
}

template <bool SERIAL, bool CLAMP>
struct Pair32 {
  static __device__ __forceinline__ float d2f(const float4 &r, float lx, float ly, float lz) {
    const float dx = __fsub_rn(r.x, lx), dy = __fsub_rn(r.y, ly), dz = __fsub_rn(r.z, lz);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
  }
  // soft-core LJ term in FP32 (src/fitness.rs:57-70): eps*(q^2 - 2q),
  // q = R6 / (r^6 + R6/2)
  static __device__ __forceinline__ float vdw(float d2, float2 tp) {
    const float r6 = d2 * d2 * d2;
    const float q = tp.x * rcp_approx(__fmaf_rn(0.5f, tp.x, r6));
    float v = (q * (q - 2.0f)) * tp.y;
    if (CLAMP) v = v < -50.0f ? -50.0f : (v > 500.0f ? 500.0f : v);
    return v;
  }
  // One receptor x ligand pair; accumulates into the per-tile partials.
  static __device__ __forceinline__ void run(const float4 &r, int rtrow, int rser, const float2 *s_tab, float lx,
                                             float ly, float lz, float lq, int lt, int lser, const ScoreParams &p,
                                             float &av, float &ae, int &lc, int &rc, bool &amb) {
    const float d2 = d2f(r, lx, ly, lz);
    const float v = vdw(d2, s_tab[rtrow + lt]);
    const float tv = __fsub_rn(d2, 72.0f);  // 0 < d2 < 144  <=>  |tv| < 72
    if (SERIAL) {
      av += (fabsf(tv) < 72.0f && rser != lser) ? v : 0.0f;
    } else {
      add_if_abs_lt(av, tv, 72.0f, v);
    }
    const float e = (r.w * lq) * rcp_approx(d2);
    const float te = __fsub_rn(d2, 113.0f);  // 1 < d2 < 225  <=>  |te| < 112
    add_if_abs_lt(ae, te, 112.0f, e);
    count_if_lt64(lc, rc, d2);
    amb = amb | (fabsf(__fsub_rn(fabsf(te), 112.0f)) < p.guard_e) | (fabsf(__fsub_rn(fabsf(tv), 72.0f)) < p.guard_v) |
          (fabsf(__fsub_rn(d2, 64.0f)) < p.guard_d);
  }

  // FP64 re-decision of a pair flagged by the guard band.  Recomputes the FP32
  // d2 with the same intrinsic sequence as run() (bit-identical) and corrects
  // the accumulated terms where the exact decision differs.
  static __device__ __noinline__ void fix(const float4 r, const D4 r64, int rtrow, int rser, const float2 *s_tab,
                                          float lx, float ly, float lz, float lq, int lt, int lser, double X,
                                          double Y, double Z, const Thresholds thr, float *av, float *ae, int *lc,
                                          int *rfix) {
    const float d2 = d2f(r, lx, ly, lz);
    const float tv = __fsub_rn(d2, 72.0f);
    const float te = __fsub_rn(d2, 113.0f);
    bool pv32 = fabsf(tv) < 72.0f;
    if (SERIAL) pv32 = pv32 && (rser != lser);
    const bool pe32 = fabsf(te) < 112.0f;
    const bool pd32 = d2 < 64.0f;
    const double d2x = exact_d2(r64.x, r64.y, r64.z, X, Y, Z);
    bool pv64 = d2x > 0.0 && d2x < thr.vdw_lt;
    if (SERIAL) pv64 = pv64 && (rser != lser);
    const bool pe64 = d2x > thr.elec_gt && d2x < thr.elec_lt;
    const bool pd64 = d2x < thr.desolv_lt;
    if (pv64 != pv32) {
      const float v = vdw(d2, s_tab[rtrow + lt]);
      *av += pv64 ? v : -v;
    }
    if (pe64 != pe32) {
      const float e = (r.w * lq) * rcp_approx(d2);
      *ae += pe64 ? e : -e;
    }
    if (pd64 != pd32) {
      const int dlt = pd64 ? 1 : -1;
      *lc += dlt;
      *rfix += dlt;
    }
  }
};

template <int NT, int S, bool SERIAL, bool CLAMP>
__global__ void __launch_bounds__(NT, 2) k_score_f32(const ScoreParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  const SmemLayout32 L = smem_layout32(p.nt, p.nr, NT);
  float4 *s_pos = reinterpret_cast<float4 *>(smem + L.pos);
  int2 *s_meta = reinterpret_cast<int2 *>(smem + L.meta);
  float4 *s_sph = reinterpret_cast<float4 *>(smem + L.sph);
  uint64_t *s_full = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *s_tab = reinterpret_cast<float2 *>(smem + L.tab);
  gd_pose_frame *s_frame = reinterpret_cast<gd_pose_frame *>(smem + L.frame);
  double *s_red = reinterpret_cast<double *>(smem + L.red);
  float4 *s_blob = reinterpret_cast<float4 *>(smem + L.blob);
  uint32_t *s_rcnt = reinterpret_cast<uint32_t *>(smem + L.rcnt);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&s_full[s], 1);
    fence_mbar_init();
  }
  for (int i = tid; i < p.nt * p.nt; i += NT) {
    const TypePair32 t = p.tab32[i];
    s_tab[i] = make_float2(t.r6, t.eps);
  }
  for (int i = tid; i < p.nr; i += NT) s_rcnt[i] = 0;
  __syncthreads();

  constexpr int kChunk = NT * S;
  const int nchunks = (p.nl + kChunk - 1) / kChunk;
  const int my_poses =
      (static_cast<int>(blockIdx.x) < p.n_poses) ? (p.n_poses - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1 : 0;
  const long long Q = static_cast<long long>(my_poses) * nchunks * p.n_tiles;
  if (tid == 0)
    for (long long q = 0; q < Q && q < kStages; ++q) issue_tile32(q, p.n_tiles, p, s_pos, s_meta, s_sph, s_full);

  float4 *my_blob = s_blob + warp * 8;
  long long q = 0;
  for (int k = 0; k < my_poses; ++k) {
    const int pose = static_cast<int>(blockIdx.x) + k * static_cast<int>(gridDim.x);
    if (!p.models && tid < 16)
      reinterpret_cast<double *>(s_frame)[tid] = reinterpret_cast<const double *>(p.frames + pose)[tid];
    __syncthreads();
    const gd_pose_frame &f = *s_frame;
    double vdw_t = 0.0, elec_t = 0.0, desolv_t = 0.0;

    for (int ch = 0; ch < nchunks; ++ch) {
      float lx[S], ly[S], lz[S], lq[S];
      int lt[S], lser[S], lcnt[S];
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int j = ch * kChunk + s * NT + tid;
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
          lser[s] = SERIAL ? p.lig_serial[j] : 0;
        } else {
          lx[s] = ly[s] = lz[s] = 1.0e9f;  // far away: no term, no count, no guard hit
          lq[s] = 0.0f;
          lt[s] = 0;
          lser[s] = 0;
        }
        // bounding sphere of this warp's 32 atoms of slot s (warp-uniform)
        const unsigned on_mask = __ballot_sync(kFull, on);
        float cx = on ? lx[s] : 0.f, cy = on ? ly[s] : 0.f, cz = on ? lz[s] : 0.f;
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
        float rr = on ? sqrtf((lx[s] - cx) * (lx[s] - cx) + (ly[s] - cy) * (ly[s] - cy) + (lz[s] - cz) * (lz[s] - cz))
                      : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rr = fmaxf(rr, __shfl_xor_sync(kFull, rr, o));
        if (lane == 0) my_blob[s] = make_float4(cx, cy, cz, on_mask ? rr * 1.0001f + 0.01f : -1.0e30f);
      }
      __syncwarp();
      float sv = 0.0f, cv = 0.0f, se = 0.0f, ce = 0.0f;
      for (int t = 0; t < p.n_tiles; ++t, ++q) {
        const int st = static_cast<int>(q % kStages);
        const bool ok = __all_sync(kFull, mbar_wait(&s_full[st], static_cast<uint32_t>((q / kStages) & 1)));
        const int base = t * kTile;
        const int cnt = min(kTile, p.nr - base);
        float av = 0.0f, ae = 0.0f;
        if (ok) {
          for (int b0 = 0; b0 < cnt; b0 += kBlk) {
            // which slots of this warp can reach receptor block b0 / kBlk
            const float4 sp = s_sph[st * (kTile / kBlk) + b0 / kBlk];  // (centre, radius + cutoff reach)
            unsigned act = 0;
#pragma unroll
            for (int s = 0; s < S; ++s) {
              const float4 bl = my_blob[s];
              const float dx = sp.x - bl.x, dy = sp.y - bl.y, dz = sp.z - bl.z;
              const float lim = sp.w + bl.w;
              act |= (lim > 0.0f && dx * dx + dy * dy + dz * dz < lim * lim) ? (1u << s) : 0u;
            }
            if (act == 0) continue;
            const int bend = min(b0 + kBlk, cnt);
            for (int a = b0; a < bend; ++a) {
              const float4 r = s_pos[st * kTile + a];
              const int2 m = s_meta[st * kTile + a];
              int rc = 0;
              bool amb = false;
#pragma unroll
              for (int s = 0; s < S; ++s)
                if (act & (1u << s))
                  Pair32<SERIAL, CLAMP>::run(r, m.x, m.y, s_tab, lx[s], ly[s], lz[s], lq[s], lt[s], lser[s], p, av,
                                             ae, lcnt[s], rc, amb);
              const int tot = __reduce_add_sync(kFull, rc);
              if (lane == 0 && tot) atomicAdd(&s_rcnt[base + a], static_cast<uint32_t>(tot));
              if (__any_sync(kFull, amb)) {
                const D4 r64 = p.rec_pos64[base + a];
                int rfix = 0;
#pragma unroll
                for (int s = 0; s < S; ++s) {
                  const int j = ch * kChunk + s * NT + tid;
                  if (j >= p.nl || !(act & (1u << s))) continue;
                  const float d2 = Pair32<SERIAL, CLAMP>::d2f(r, lx[s], ly[s], lz[s]);
                  const float tv = __fsub_rn(d2, 72.0f), te = __fsub_rn(d2, 113.0f);
                  const bool near = (fabsf(__fsub_rn(fabsf(te), 112.0f)) < p.guard_e) |
                                    (fabsf(__fsub_rn(fabsf(tv), 72.0f)) < p.guard_v) |
                                    (fabsf(__fsub_rn(d2, 64.0f)) < p.guard_d);
                  if (!near) continue;
                  double X, Y, Z;
                  ligand_atom(p, f, pose, j, X, Y, Z);
                  Pair32<SERIAL, CLAMP>::fix(r, r64, m.x, m.y, s_tab, lx[s], ly[s], lz[s], lq[s], lt[s], lser[s], X,
                                             Y, Z, p.thr, &av, &ae, &lcnt[s], &rfix);
                }
                const int fx = __reduce_add_sync(kFull, rfix);
                if (lane == 0 && fx) atomicAdd(&s_rcnt[base + a], static_cast<uint32_t>(fx));
              }
            }
          }
        }
        kahan_add(sv, cv, av);
        kahan_add(se, ce, ae);
        // all threads are done with stage st: refill it, or give up together
        if (__syncthreads_or(!ok)) {
          if (tid == 0) {
            atomicExch(p.err, kDevTimeout);
            drain(s_full, q, q + kStages < Q ? q + kStages : Q);
          }
          return;
        }
        if (tid == 0 && q + kStages < Q) issue_tile32(q + kStages, p.n_tiles, p, s_pos, s_meta, s_sph, s_full);
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int j = ch * kChunk + s * NT + tid;
        if (j < p.nl) desolv_t += p.lig_desolv[static_cast<size_t>(j) * 11 + min(lcnt[s], 10)];
      }
      vdw_t += static_cast<double>(sv) - static_cast<double>(cv);
      elec_t += static_cast<double>(se) - static_cast<double>(ce);
    }
    // receptor burial -> desolvation; reset counters for the next pose
    for (int i = tid; i < p.nr; i += NT) {
      desolv_t += p.rec_desolv[static_cast<size_t>(i) * 11 + min(s_rcnt[i], 10u)];
      s_rcnt[i] = 0;
    }
    block_sum3<NT>(vdw_t, elec_t, desolv_t, s_red);
    if (tid == 0) write_pose(p, pose, vdw_t, elec_t, desolv_t, f);
    __syncthreads();
  }
}

// --------------------------------------------------------------- FP64 ----

template <int NT, int S, bool SERIAL, bool CLAMP>
__global__ void __launch_bounds__(NT) k_score_f64(const ScoreParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  const SmemLayout L = smem_layout<D4>(p.nt, p.nr, NT, sizeof(D4));
  D4 *s_pos = reinterpret_cast<D4 *>(smem + L.pos);
  int2 *s_meta = reinterpret_cast<int2 *>(smem + L.meta);
  uint64_t *s_full = reinterpret_cast<uint64_t *>(smem + L.bars);
  D4 *s_tab = reinterpret_cast<D4 *>(smem + L.tab);
  gd_pose_frame *s_frame = reinterpret_cast<gd_pose_frame *>(smem + L.frame);
  double *s_red = reinterpret_cast<double *>(smem + L.red);
  uint32_t *s_rcnt = reinterpret_cast<uint32_t *>(smem + L.rcnt);

  const int tid = threadIdx.x, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&s_full[s], 1);
    fence_mbar_init();
  }
  for (int i = tid; i < p.nt * p.nt; i += NT) {
    const TypePair64 t = p.tab64[i];
    s_tab[i] = D4{t.r6, t.hr6, t.eps, 0.0};
  }
  for (int i = tid; i < p.nr; i += NT) s_rcnt[i] = 0;
  __syncthreads();

  constexpr int kChunk = NT * S;
  const int nchunks = (p.nl + kChunk - 1) / kChunk;
  const int my_poses =
      (static_cast<int>(blockIdx.x) < p.n_poses) ? (p.n_poses - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1 : 0;
  const long long Q = static_cast<long long>(my_poses) * nchunks * p.n_tiles;
  if (tid == 0)
    for (long long q = 0; q < Q && q < kStages; ++q)
      issue_tile(q, p.n_tiles, p.rec_pos64, p.rec_meta, s_pos, s_meta, s_full);

  const double vdw_lt = p.thr.vdw_lt, elec_gt = p.thr.elec_gt, elec_lt = p.thr.elec_lt, des_lt = p.thr.desolv_lt;
  long long q = 0;
  for (int k = 0; k < my_poses; ++k) {
    const int pose = static_cast<int>(blockIdx.x) + k * static_cast<int>(gridDim.x);
    if (!p.models && tid < 16)
      reinterpret_cast<double *>(s_frame)[tid] = reinterpret_cast<const double *>(p.frames + pose)[tid];
    __syncthreads();
    const gd_pose_frame f = *s_frame;
    double vdw_t = 0.0, elec_t = 0.0, desolv_t = 0.0;

    for (int ch = 0; ch < nchunks; ++ch) {
      double lx[S], ly[S], lz[S], lq[S];
      int lt[S], lser[S], lcnt[S];
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int j = ch * kChunk + s * NT + tid;
        lcnt[s] = 0;
        if (j < p.nl) {
          ligand_atom(p, f, pose, j, lx[s], ly[s], lz[s]);
          lq[s] = p.lig_q[j];
          lt[s] = p.lig_type[j];
          lser[s] = SERIAL ? p.lig_serial[j] : 0;
        } else {
          lx[s] = ly[s] = lz[s] = 1.0e30;
          lq[s] = 0.0;
          lt[s] = 0;
          lser[s] = 0;
        }
      }
      for (int t = 0; t < p.n_tiles; ++t, ++q) {
        const int st = static_cast<int>(q % kStages);
        const bool ok = __all_sync(kFull, mbar_wait(&s_full[st], static_cast<uint32_t>((q / kStages) & 1)));
        const int base = t * kTile;
        const int cnt = min(kTile, p.nr - base);
        if (ok) {
          for (int a = 0; a < cnt; ++a) {
            const D4 r = s_pos[st * kTile + a];
            const int2 m = s_meta[st * kTile + a];
            int rc = 0;
#pragma unroll
            for (int s = 0; s < S; ++s) {
              const double d2 = exact_d2(r.x, r.y, r.z, lx[s], ly[s], lz[s]);
              bool pv = d2 > 0.0 && d2 < vdw_lt;
              if (SERIAL) pv = pv && (m.y != lser[s]);
              const bool pe = d2 > elec_gt && d2 < elec_lt;
              const bool pd = d2 < des_lt;
              if (__any_sync(kFull, pv)) {
                // softcore_lj_potential (src/fitness.rs:57-70) with r^6 from d2
                const D4 tp = s_tab[m.x + lt[s]];
                const double d4 = d2 * d2;
                const double r6 = d2 * d4;
                const double ratio = tp.x / (r6 + tp.y);
                double v = tp.z * (ratio * ratio - 2.0 * ratio);
                if (CLAMP) v = v < -50.0 ? -50.0 : (v > 500.0 ? 500.0 : v);
                vdw_t += pv ? v : 0.0;
              }
              if (__any_sync(kFull, pe)) {
                // elec_energy term (src/fitness.rs:296): k*(q1*q2)/r^2
                const double e = (332.0636 * (r.w * lq[s])) / d2;
                elec_t += pe ? e : 0.0;
              }
              lcnt[s] += pd;
              rc += pd;
            }
            const int tot = __reduce_add_sync(kFull, rc);
            if (lane == 0 && tot) atomicAdd(&s_rcnt[base + a], static_cast<uint32_t>(tot));
          }
        }
        if (__syncthreads_or(!ok)) {
          if (tid == 0) {
            atomicExch(p.err, kDevTimeout);
            drain(s_full, q, (q + kStages < Q ? q + kStages : Q));
          }
          return;
        }
        if (tid == 0 && q + kStages < Q) issue_tile(q + kStages, p.n_tiles, p.rec_pos64, p.rec_meta, s_pos, s_meta, s_full);
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int j = ch * kChunk + s * NT + tid;
        if (j < p.nl) desolv_t += p.lig_desolv[static_cast<size_t>(j) * 11 + min(lcnt[s], 10)];
      }
    }
    for (int i = tid; i < p.nr; i += NT) {
      desolv_t += p.rec_desolv[static_cast<size_t>(i) * 11 + min(s_rcnt[i], 10u)];
      s_rcnt[i] = 0;
    }
    block_sum3<NT>(vdw_t, elec_t, desolv_t, s_red);
    if (tid == 0) write_pose(p, pose, vdw_t, elec_t, desolv_t, f);
    __syncthreads();
  }
}

// ------------------------------------------------------------ dispatch ----

constexpr int kNT = 256;

template <typename Kern>
cudaError_t launch_kernel(Kern kern, int n, size_t smem, int sm_count, cudaStream_t stream, const ScoreParams &p,
                          int *grid_out) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kNT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int grid = std::max(1, std::min(n, per_sm * sm_count));
  if (grid_out) *grid_out = grid;
  kern<<<grid, kNT, smem, stream>>>(p);
  return cudaGetLastError();
}

template <int S>
cudaError_t launch_f32(const ScoreParams &p, bool serial, bool clamp, size_t smem, int sm, cudaStream_t st) {
  if (!serial && !clamp) return launch_kernel(k_score_f32<kNT, S, false, false>, p.n_poses, smem, sm, st, p, nullptr);
  if (serial && !clamp) return launch_kernel(k_score_f32<kNT, S, true, false>, p.n_poses, smem, sm, st, p, nullptr);
  if (!serial && clamp) return launch_kernel(k_score_f32<kNT, S, false, true>, p.n_poses, smem, sm, st, p, nullptr);
  return launch_kernel(k_score_f32<kNT, S, true, true>, p.n_poses, smem, sm, st, p, nullptr);
}

template <int S>
cudaError_t launch_f64(const ScoreParams &p, bool serial, bool clamp, size_t smem, int sm, cudaStream_t st) {
  if (!serial && !clamp) return launch_kernel(k_score_f64<kNT, S, false, false>, p.n_poses, smem, sm, st, p, nullptr);
  if (serial && !clamp) return launch_kernel(k_score_f64<kNT, S, true, false>, p.n_poses, smem, sm, st, p, nullptr);
  if (!serial && clamp) return launch_kernel(k_score_f64<kNT, S, false, true>, p.n_poses, smem, sm, st, p, nullptr);
  return launch_kernel(k_score_f64<kNT, S, true, true>, p.n_poses, smem, sm, st, p, nullptr);
}

}  // namespace

gd_status launch_score(gd_complex *cx, const gd_pose_frame *d_frames, const double *d_models, int n,
                       gd_precision prec, gd_pose_energy *d_out, cudaStream_t stream, double max_disp) {
  gd_context *ctx = cx->ctx;
  if (n <= 0) return GD_OK;
  ScoreParams p{};
  p.rec_pos32 = cx->rec_pos32;
  p.rec_pos64 = cx->rec_pos64;
  p.rec_sph32 = cx->rec_sph32;
  p.rec_meta = cx->rec_meta;
  p.rec_desolv = cx->rec_desolv;
  p.nr = cx->nr;
  p.n_tiles = cx->nr_pad / kTile;
  p.lig_x = cx->lig_x;
  p.lig_y = cx->lig_y;
  p.lig_z = cx->lig_z;
  p.lig_q = cx->lig_q;
  p.lig_type = cx->lig_type;
  p.lig_serial = cx->lig_serial;
  p.lig_desolv = cx->lig_desolv;
  p.nl = cx->nl;
  p.cx = cx->cx;
  p.cy = cx->cy;
  p.cz = cx->cz;
  p.ox = cx->ox;
  p.oy = cx->oy;
  p.oz = cx->oz;
  p.tab32 = cx->tab32;
  p.tab64 = cx->tab64;
  p.nt = cx->nt;
  p.need_clamp = cx->need_clamp;
  p.restr_rec = cx->restr_rec;
  p.restr_lig = cx->restr_lig;
  p.K = cx->K;
  p.wv = cx->w.vdw;
  p.we = cx->w.elec;
  p.wd = cx->w.desolv;
  p.wa = cx->w.air;
  p.thr = make_thresholds(5.0);
  guard_widths(cx, max_disp, &p.guard_v, &p.guard_e, &p.guard_d);
  p.frames = d_frames;
  p.models = d_models;
  p.n_poses = n;
  p.out = d_out;
  p.err = ctx->d_err;
  if (p.nr == 0 || p.nl == 0) {
    // no pairs: every energy but AIR is zero; run with one empty tile anyway
  }
  const bool serial = cx->serial_overlap, clamp = cx->need_clamp;
  cudaError_t e;
  if (prec == GD_PREC_F32) {
    const size_t smem = smem_layout32(p.nt, p.nr, kNT).total;
    const int S = std::max(1, std::min(8, (p.nl + kNT - 1) / kNT));
    switch (S) {
      case 1: e = launch_f32<1>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      case 2: e = launch_f32<2>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      case 3: e = launch_f32<3>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      case 4: e = launch_f32<4>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      case 5: e = launch_f32<5>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      case 6: e = launch_f32<6>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      default: e = launch_f32<8>(p, serial, clamp, smem, ctx->sm_count, stream); break;
    }
  } else {
    const size_t smem = smem_layout<D4>(p.nt, p.nr, kNT, sizeof(D4)).total;
    const int S = std::max(1, std::min(4, (p.nl + kNT - 1) / kNT));
    switch (S) {
      case 1: e = launch_f64<1>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      case 2: e = launch_f64<2>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      case 3: e = launch_f64<3>(p, serial, clamp, smem, ctx->sm_count, stream); break;
      default: e = launch_f64<4>(p, serial, clamp, smem, ctx->sm_count, stream); break;
    }
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "score kernel launch");
  return GD_OK;
}

}  // namespace gd
