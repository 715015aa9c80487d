// The plain FP64 scoring kernel (the correctness form) and the per-call
// scoring set-up shared with the FP32 form (gd_score_warp.cu): the
// parameter block of a complex and the dispatch by precision.
//
// Reference arithmetic (gdock): transform src/structure.rs:80-131 and
// src/chromosome.rs:79-83; energies src/fitness.rs:57-302; per-pose
// combination src/chromosome.rs:110-127.
//
// k_score_f64: one pose per CTA iteration of a persistent grid.  Receptor
// atoms are streamed through shared memory in tiles of kTile atoms by bulk
// (TMA) copies into a kStages-deep ring guarded by mbarriers with bounded
// waits; the receptor stream is the same for every pose, so the ring runs
// continuously across the poses a CTA owns.  Each thread holds S ligand atoms
// of the current pose (atoms tid, tid+NT, ... of the chunk) in registers
// after transforming them in FP64 with the reference's operation order, so
// coordinates are bit-identical to gdock's.  Every pair is evaluated in FP64
// (no culling), with decisions against exact thresholds on d2.
#include <algorithm>
#include <cmath>

#include "gd_device.cuh"

namespace gd {
namespace {

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
          if (!GD_DCHECK(p.err, lt[s] >= 0 && lt[s] < p.nt, 22)) lt[s] = 0;
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
            int2 m = s_meta[st * kTile + a];
            if (!GD_DCHECK(p.err, m.x >= 0 && m.x + p.nt <= p.nt * p.nt, 20)) m.x = 0;
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
            if (lane == 0 && tot && GD_DCHECK(p.err, base + a < p.nr, 21))
              atomicAdd(&s_rcnt[base + a], static_cast<uint32_t>(tot));
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
cudaError_t launch_f64(const ScoreParams &p, bool serial, bool clamp, size_t smem, int sm, cudaStream_t st) {
  if (!serial && !clamp) return launch_kernel(k_score_f64<kNT, S, false, false>, p.n_poses, smem, sm, st, p, nullptr);
  if (serial && !clamp) return launch_kernel(k_score_f64<kNT, S, true, false>, p.n_poses, smem, sm, st, p, nullptr);
  if (!serial && clamp) return launch_kernel(k_score_f64<kNT, S, false, true>, p.n_poses, smem, sm, st, p, nullptr);
  return launch_kernel(k_score_f64<kNT, S, true, true>, p.n_poses, smem, sm, st, p, nullptr);
}

}  // namespace

ScoreParams make_params(gd_complex *cx, const gd_pose_frame *d_frames, const double *d_models, int n,
                        gd_pose_energy *d_out, double max_disp) {
  ScoreParams p{};
  p.rec_pos32 = cx->rec_pos32;
  p.rec_pos64 = cx->rec_pos64;
  p.rec_meta = cx->rec_meta;
  p.rec_meta16 = cx->rec_meta16;
  p.rec_desolv = cx->rec_desolv;
  p.nr = cx->nr;
  p.n_tiles = cx->nr_pad / kTile;
  p.lig_perm = cx->lig_perm;
  p.lig_slot_sph = cx->lig_slot_sph;
  p.rec_seg = cx->rec_seg;
  p.nseg = cx->nseg;
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
  p.err = cx->ctx->d_err;
  return p;
}

gd_status launch_score(gd_complex *cx, const gd_pose_frame *d_frames, const double *d_models, int n,
                       gd_precision prec, gd_pose_energy *d_out, cudaStream_t stream, double max_disp) {
  gd_context *ctx = cx->ctx;
  if (n <= 0) return GD_OK;
  const ScoreParams p = make_params(cx, d_frames, d_models, n, d_out, max_disp);
  const bool serial = cx->serial_overlap, clamp = cx->need_clamp;
  if (prec == GD_PREC_F32)
    return launch_score_batch_f32(ctx, std::vector<ScoreParams>{p}, serial, clamp,
                                  ctx->tune_f32_slots ? ctx->tune_f32_slots : kDefaultF32Tune, stream);
  cudaError_t e;
  const size_t smem = smem_layout<D4>(p.nt, p.nr, kNT, sizeof(D4)).total;
  const int S = std::max(1, std::min(4, (p.nl + kNT - 1) / kNT));
  switch (S) {
    case 1: e = launch_f64<1>(p, serial, clamp, smem, ctx->sm_count, stream); break;
    case 2: e = launch_f64<2>(p, serial, clamp, smem, ctx->sm_count, stream); break;
    case 3: e = launch_f64<3>(p, serial, clamp, smem, ctx->sm_count, stream); break;
    default: e = launch_f64<4>(p, serial, clamp, smem, ctx->sm_count, stream); break;
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "score kernel launch");
  return GD_OK;
}

}  // namespace gd
