// Docking-quality metrics of poses against a reference ligand structure: the
// evaluator of gdock (src/evaluator.rs:50-186), used for the per-generation
// metrics report and as the debug fitness (src/chromosome.rs:93-106).
//
// Host (gd_evaluator_create), following src/evaluator.rs:50-66,170-186:
//   - interface residues: receptor and reference residues with an atom pair
//     at distance <= 5 A;
//   - receptor interface = receptor atoms of those residues, reference
//     interface likewise, native contacts = their atom pairs at <= 5 A,
//     identified by (chain, residue, atom name) on both sides;
//   - the per-pose work then needs, per ligand atom: its pairing in the
//     L-RMSD (zip of the ligand with the reference), its pairing in the
//     i-RMSD (zip of the ligand's interface-residue atoms with the reference
//     interface), and the receptor atoms whose contact with it has a native
//     identity (a docked contact counts once when it is native); ligand atoms
//     with none of these are left out.
// Device (k_dockq): one warp per pose; each ligand atom moved once, exactly
// (FP64, the reference's operation order); distances sqrt(d2) with d2 in the
// reference's order; contact decisions against the exact d2 threshold of 5 A.
//   rmsd  = sqrt(sum over pairs of distance / |reference|)    (src/evaluator.rs:86-103;
//   irmsd = likewise over the interface pairings               the sum is of distances)
//   fnat  = docked native contacts / |native contacts|
//   dockq = (fnat + 1/(1 + (irmsd/1.5)^2) + 1/(1 + (rmsd/8.5)^2)) / 3
#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <tuple>
#include <vector>

#include "gd_device.cuh"

struct gd_evaluator {
  gd_complex *cx = nullptr;
  gd_context *ctx = nullptr;
  int n_u = 0;                            // ligand atoms the metrics read
  int n_ref = 0, n_iref = 0, n_native = 0;  // divisors: |reference|, |reference interface|, |native contacts|
  int n_p = 0;                            // native-identity (receptor atom, ligand atom) pairs
  int64_t counts[GD_EVAL_COUNTS] = {};    // as gd_evaluator_counts reports them
  const int *u_slot = nullptr;            // [n_u] device slot of each such ligand atom (interface atoms first)
  const D4 *u_ref = nullptr, *u_iref = nullptr;  // [n_u] paired reference atom (w = 1) or none (w = 0)
  const int *u_pbeg = nullptr;            // [n_u + 1] CSR offsets into p_rec
  const D4 *p_rec = nullptr;              // [n_p] receptor atoms whose contact with the ligand atom is native
  double thr5 = 0.0;
  void *block = nullptr;
  size_t bytes = 0;
};

namespace gd {
namespace {

struct EvalParams {
  ScoreParams p;  // ligand arrays, frames and the rotation centre
  const int *u_slot, *u_pbeg;
  const D4 *u_ref, *u_iref, *p_rec;
  int n_u, n_ref, n_iref, n_native;
  double thr5;
  const int *skip;  // nonzero: no work (a finished GA job); may be null
  gd_dock_metrics *out;
};

constexpr int kEvalWarps = 4;

// One warp per pose; each lane moves its ligand atoms once and uses each for
// the L-RMSD pairing, the i-RMSD pairing and its native-identity contacts.
__global__ void __launch_bounds__(kEvalWarps * 32) k_dockq(const EvalParams e) {
  const int lane = threadIdx.x & 31;
  const int pose = blockIdx.x * kEvalWarps + (threadIdx.x >> 5);
  if (pose >= e.p.n_poses || (e.skip && *e.skip)) return;
  gd_pose_frame f;
  {
    const double *src = reinterpret_cast<const double *>(e.p.frames + pose);
    double *dst = reinterpret_cast<double *>(&f);
#pragma unroll
    for (int k = 0; k < 16; ++k) dst[k] = src[k];
  }
  double sl = 0.0, si = 0.0;
  int common = 0;
  for (int u = lane; u < e.n_u; u += 32) {
    double X, Y, Z;
    int slot = e.u_slot[u];
    if (!GD_DCHECK(e.p.err, slot >= 0 && slot < e.p.nl, 40)) slot = 0;
    ligand_atom(e.p, f, pose, slot, X, Y, Z);
    const D4 r = e.u_ref[u], q = e.u_iref[u];
    // ligand atom first, as atom1.distance_to(atom2) (src/evaluator.rs:96-100)
    if (r.w != 0.0) sl += sqrt(exact_d2(X, Y, Z, r.x, r.y, r.z));
    if (q.w != 0.0) si += sqrt(exact_d2(X, Y, Z, q.x, q.y, q.z));
    const int k1 = e.u_pbeg[u + 1];
    for (int k = e.u_pbeg[u]; k < k1; ++k) {
      const D4 a = e.p_rec[k];  // receptor atom first, as calculate_contacts (src/evaluator.rs:150-152)
      common += exact_d2(a.x, a.y, a.z, X, Y, Z) <= e.thr5;
    }
  }
  sl = warp_sum(sl);
  si = warp_sum(si);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) common += __shfl_xor_sync(kFull, common, o);
  if (lane == 0) {
    // src/evaluator.rs:68-84, without contraction into fused multiply-adds
    const double rmsd = e.n_ref ? __dsqrt_rn(__ddiv_rn(sl, static_cast<double>(e.n_ref))) : 0.0;
    const double irmsd = e.n_iref ? __dsqrt_rn(__ddiv_rn(si, static_cast<double>(e.n_iref))) : 0.0;
    const double fnat = e.n_native ? __ddiv_rn(static_cast<double>(common), static_cast<double>(e.n_native)) : 0.0;
    const double a = __ddiv_rn(irmsd, 1.5), b = __ddiv_rn(rmsd, 8.5);
    const double is = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(a, a)));
    const double ls = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(b, b)));
    const double dockq = __ddiv_rn(__dadd_rn(__dadd_rn(fnat, is), ls), 3.0);
    e.out[pose] = gd_dock_metrics{rmsd, irmsd, fnat, dockq};
  }
}

double host_dist(double ax, double ay, double az, double bx, double by, double bz) {
  const double dx = ax - bx, dy = ay - by, dz = az - bz;
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

}  // namespace

gd_complex *evaluator_complex(const gd_evaluator *ev) { return ev->cx; }

gd_status launch_dockq(gd_evaluator *ev, const gd_pose_frame *d_frames, int n, gd_dock_metrics *d_out,
                       const int *skip, cudaStream_t stream) {
  if (n == 0) return GD_OK;
  EvalParams ep{};
  ep.p = make_params(ev->cx, d_frames, nullptr, n, nullptr, 0.0);
  ep.u_slot = ev->u_slot;
  ep.u_pbeg = ev->u_pbeg;
  ep.u_ref = ev->u_ref;
  ep.u_iref = ev->u_iref;
  ep.p_rec = ev->p_rec;
  ep.n_u = ev->n_u;
  ep.n_ref = ev->n_ref;
  ep.n_iref = ev->n_iref;
  ep.n_native = ev->n_native;
  ep.thr5 = ev->thr5;
  ep.skip = skip;
  ep.out = d_out;
  k_dockq<<<(n + kEvalWarps - 1) / kEvalWarps, kEvalWarps * 32, 0, stream>>>(ep);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GD_OK : cuda_fail(ev->ctx, e, "evaluator launch");
}

}  // namespace gd

using namespace gd;

extern "C" {

gd_status gd_evaluator_create(gd_complex *cx, const gd_atoms *reference, const uint32_t *rec_names,
                              const uint32_t *lig_names, const uint32_t *ref_names, gd_evaluator **out) {
  gd::NvtxRange nvtx_range("gd_evaluator_create");
  if (!cx || !reference || !out) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  *out = nullptr;
  const int nr = static_cast<int>(cx->h_rx.size()), nl = static_cast<int>(cx->h_lx.size()), nf = reference->n;
  if (nf < 0 || (nf > 0 && (!reference->x || !reference->y || !reference->z || !reference->resseq ||
                            !reference->chain || !ref_names)) ||
      (nr > 0 && !rec_names) || (nl > 0 && !lig_names))
    return fail(ctx, GD_ERR_INVALID_ARG, "bad reference or atom names");
  cudaSetDevice(ctx->device);
  // interface residues (src/evaluator.rs:170-186)
  std::set<int16_t> rec_if, ref_if;
  for (int a = 0; a < nr; ++a)
    for (int b = 0; b < nf; ++b)
      if (host_dist(cx->h_rx[a], cx->h_ry[a], cx->h_rz[a], reference->x[b], reference->y[b], reference->z[b]) <=
          5.0) {
        rec_if.insert(cx->h_rres[a]);
        ref_if.insert(reference->resseq[b]);
      }
  std::vector<int> rec_i, ref_i, lig_i;  // interface atoms, in order
  for (int a = 0; a < nr; ++a)
    if (rec_if.count(cx->h_rres[a])) rec_i.push_back(a);
  for (int b = 0; b < nf; ++b)
    if (ref_if.count(reference->resseq[b])) ref_i.push_back(b);
  for (int j = 0; j < nl; ++j)
    if (ref_if.count(cx->h_lres[j])) lig_i.push_back(j);
  // native contacts: identities (chain, residue, name) of both atoms
  using Id = std::tuple<uint8_t, int16_t, uint32_t, uint8_t, int16_t, uint32_t>;
  std::set<Id> native_set;
  int n_native = 0;
  for (int a : rec_i)
    for (int b : ref_i)
      if (host_dist(cx->h_rx[a], cx->h_ry[a], cx->h_rz[a], reference->x[b], reference->y[b], reference->z[b]) <=
          5.0) {
        native_set.insert(Id{cx->h_rchain[a], cx->h_rres[a], rec_names[a], reference->chain[b],
                             reference->resseq[b], ref_names[b]});
        ++n_native;
      }
  // per ligand atom (in device slot order): its L-RMSD partner (the
  // reference atom of the same index: zip truncates at the shorter), its
  // i-RMSD partner (same rank among the interface atoms of both), and the
  // receptor interface atoms whose contact with it has a native identity
  std::vector<D4> l_ref(nl, D4{0, 0, 0, 0}), l_iref(nl, D4{0, 0, 0, 0});
  std::vector<std::vector<int>> l_rec(nl);
  for (int k = 0; k < std::min(nl, nf); ++k) l_ref[k] = D4{reference->x[k], reference->y[k], reference->z[k], 1.0};
  for (size_t k = 0; k < std::min(lig_i.size(), ref_i.size()); ++k) {
    const int b = ref_i[k];
    l_iref[lig_i[k]] = D4{reference->x[b], reference->y[b], reference->z[b], 1.0};
  }
  int n_p = 0;
  for (int a : rec_i)
    for (int j : lig_i)
      if (native_set.count(Id{cx->h_rchain[a], cx->h_rres[a], rec_names[a], cx->h_lchain[j], cx->h_lres[j],
                              lig_names[j]})) {
        l_rec[j].push_back(a);
        ++n_p;
      }
  // ligand atoms the metrics read: the interface ones (i-RMSD pairing or
  // contacts) first, so that the warps' branches for them stay uniform, then
  // the rest; each group by device slot
  std::vector<int> order;
  for (int j = 0; j < nl; ++j)
    if (l_ref[j].w != 0.0 || l_iref[j].w != 0.0 || !l_rec[j].empty()) order.push_back(j);
  auto group = [&](int j) { return (l_iref[j].w != 0.0 || !l_rec[j].empty()) ? 0 : 1; };
  std::sort(order.begin(), order.end(), [&](int x, int y) {
    return group(x) != group(y) ? group(x) < group(y) : cx->h_lig_slot[x] < cx->h_lig_slot[y];
  });
  const int nu = static_cast<int>(order.size());
  std::vector<int> u_slot(nu), u_pbeg(nu + 1, 0);
  std::vector<D4> u_ref(nu), u_iref(nu), p_rec;
  p_rec.reserve(n_p);
  for (int u = 0; u < nu; ++u) {
    const int j = order[u];
    u_slot[u] = cx->h_lig_slot[j];
    u_ref[u] = l_ref[j];
    u_iref[u] = l_iref[j];
    for (int a : l_rec[j]) p_rec.push_back(D4{cx->h_rx[a], cx->h_ry[a], cx->h_rz[a], 0.0});
    u_pbeg[u + 1] = static_cast<int>(p_rec.size());
  }
  gd_evaluator *ev = new gd_evaluator();
  ev->cx = cx;
  ev->ctx = ctx;
  ev->n_u = nu;
  ev->n_ref = nf;
  ev->n_iref = static_cast<int>(ref_i.size());
  ev->n_native = n_native;
  ev->n_p = n_p;
  ev->thr5 = make_thresholds(5.0).contact_le;
  const int64_t cnt[GD_EVAL_COUNTS] = {static_cast<int64_t>(rec_if.size()), static_cast<int64_t>(ref_if.size()),
                                       n_native, nu, std::min(nl, nf),
                                       static_cast<int64_t>(std::min(lig_i.size(), ref_i.size())), n_p};
  std::copy(cnt, cnt + GD_EVAL_COUNTS, ev->counts);
  auto al = [](size_t b) { return (std::max<size_t>(b, 1) + 255) / 256 * 256; };
  const size_t b_slot = al(sizeof(int) * nu), b_beg = al(sizeof(int) * (nu + 1)), b_ref = al(sizeof(D4) * nu),
               b_prec = al(sizeof(D4) * p_rec.size());
  ev->bytes = b_slot + b_beg + 2 * b_ref + b_prec;
  gd_status s = dev_alloc(ctx, ev->bytes, &ev->block);
  if (s != GD_OK) {
    delete ev;
    return s;
  }
  std::vector<char> h(ev->bytes, 0);
  size_t o = 0;
  auto put = [&](const void *src, size_t n, size_t b) {
    if (n) std::memcpy(h.data() + o, src, n);
    char *d = static_cast<char *>(ev->block) + o;
    o += b;
    return d;
  };
  ev->u_slot = reinterpret_cast<const int *>(put(u_slot.data(), sizeof(int) * nu, b_slot));
  ev->u_pbeg = reinterpret_cast<const int *>(put(u_pbeg.data(), sizeof(int) * (nu + 1), b_beg));
  ev->u_ref = reinterpret_cast<const D4 *>(put(u_ref.data(), sizeof(D4) * nu, b_ref));
  ev->u_iref = reinterpret_cast<const D4 *>(put(u_iref.data(), sizeof(D4) * nu, b_ref));
  ev->p_rec = reinterpret_cast<const D4 *>(put(p_rec.data(), sizeof(D4) * p_rec.size(), b_prec));
  const cudaError_t e = cudaMemcpy(ev->block, h.data(), ev->bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    dev_free(ctx, ev->block, ev->bytes);
    delete ev;
    return cuda_fail(ctx, e, "evaluator upload");
  }
  *out = ev;
  return GD_OK;
}

gd_status gd_evaluator_counts(const gd_evaluator *ev, int64_t *counts) {
  if (!ev || !counts) return GD_ERR_INVALID_ARG;
  std::copy(ev->counts, ev->counts + GD_EVAL_COUNTS, counts);
  return GD_OK;
}

gd_status gd_evaluator_destroy(gd_evaluator *ev) {
  if (!ev) return GD_ERR_INVALID_ARG;
  gd_context *ctx = ev->ctx;
  cudaSetDevice(ctx->device);
  if (ev->block) dev_free(ctx, ev->block, ev->bytes);
  delete ev;
  return GD_OK;
}

gd_status gd_evaluate_frames_device(gd_evaluator *ev, const gd_pose_frame *d_frames, int32_t n,
                                    gd_dock_metrics *d_out, void *stream) {
  if (!ev) return GD_ERR_INVALID_ARG;
  gd_context *ctx = ev->ctx;
  if (n < 0 || (n > 0 && (!d_frames || !d_out))) return fail(ctx, GD_ERR_INVALID_ARG, "bad frames/out");
  cudaSetDevice(ctx->device);
  return launch_dockq(ev, d_frames, n, d_out, nullptr, stream ? static_cast<cudaStream_t>(stream) : ctx->stream);
}

gd_status gd_evaluate_poses(gd_evaluator *ev, const double *genes, int32_t n, gd_dock_metrics *out) {
  gd::NvtxRange nvtx_range("gd_evaluate_poses");
  if (!ev) return GD_ERR_INVALID_ARG;
  gd_context *ctx = ev->ctx;
  if (n < 0 || (n > 0 && (!genes || !out))) return fail(ctx, GD_ERR_INVALID_ARG, "bad genes/out");
  if (n == 0) return GD_OK;
  cudaSetDevice(ctx->device);
  const size_t fb = sizeof(gd_pose_frame) * n, ob = sizeof(gd_dock_metrics) * n;
  const size_t fb_al = (fb + 255) / 256 * 256;
  gd_status s = ensure_scratch(ctx, fb_al + ob, 0);
  if (s != GD_OK) return s;
  gd_pose_frame *d_frames = static_cast<gd_pose_frame *>(ctx->d_scratch);
  gd_dock_metrics *d_out = reinterpret_cast<gd_dock_metrics *>(static_cast<char *>(ctx->d_scratch) + fb_al);
  std::vector<gd_pose_frame> frames(n);
  gd_make_frames(genes, n, frames.data());
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(d_frames, frames.data(), fb, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "evaluator frames upload");
  if ((s = gd_evaluate_frames_device(ev, d_frames, n, d_out, st)) != GD_OK) return s;
  e = cudaMemcpyAsync(out, d_out, ob, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "evaluator");
  return check_device_error(ctx);
}

}  // extern "C"
