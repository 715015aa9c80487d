// FCC clustering: residue contacts per pose, all-pairs fraction of common
// contacts by popcount, neighbour graph, greedy clustering.
//
// Reference: src/clustering.rs:62-293.  Residues are keyed by (chain,
// resseq) over non-hydrogen atoms of the receptor+ligand complex; a contact
// is a pair of residues on different chains with an atom pair at distance
// <= cutoff; FCC(i,j) = |Xi & Xj| / |Xi| (and / |Xj|), an edge i->j when
// FCC >= c and FCC_v >= c * strictness; greedy clustering picks the element
// with most unused neighbours (ties: lower index).
//
// GPU pieces:
//   k_contacts_rl  one warp per (pose, ligand residue): transforms the residue's
//                  atoms exactly (FP64, reference operation order), culls
//                  receptor residues by bounding spheres, and decides atom
//                  pairs on exact d2 against the exact threshold; each contact
//                  is appended to the pose's list.
//   k_fcc          64x64 tiles of pose pairs; contact bitsets over the
//                  compacted contact universe staged in shared memory; AND +
//                  popcount; FP64 ratios and threshold tests exactly as the
//                  reference; edges written to an adjacency bit matrix.
// Host pieces: key canonicalisation (smaller chain first), receptor-only and
// ligand-only inter-chain contacts of multi-chain molecules, the universe
// compaction, and the greedy clustering over the adjacency bit matrix.
#include <algorithm>
#include <chrono>
#include <iterator>
#include <cmath>
#include <cstring>
#include <map>
#include <functional>
#include <numeric>
#include <thread>
#include <vector>

#include "gd_internal.cuh"

namespace gd {

struct ClusterTopo {
  // receptor heavy atoms grouped by residue (canonical ids), ligand likewise
  int GR = 0, GL = 0;
  std::vector<int64_t> rg_key, lg_key;  // (chain << 16) | uint16(resseq)
  std::vector<int> rg_off, lg_off;      // atom ranges
  std::vector<int> r_atoms, l_atoms;    // original atom indices, grouped
  bool multi_chain_rec = false, multi_chain_lig = false;
  bool mixed = false;  // a (chain, resseq) residue with atoms in both molecules
  float4 *d_r32 = nullptr;  // receptor heavy atoms (x-O, y-O, z-O, 0) FP32, grouped
  std::vector<int64_t> rr_keys;         // receptor-only inter-chain contacts (pose independent)
  double rr_cutoff = -1.0;
  // ligand-only inter-chain contacts in the positioned frame: their count,
  // and whether some residue pair's closest atom pair lies so near the cutoff
  // that FP64 rounding of a pose's transform could flip it (then the count is
  // not pose independent and the per-pose host path decides)
  long long ll_count = 0;
  bool ll_unstable = false;
  double ll_cutoff = -1.0;
  // device
  double *d_rx = nullptr, *d_ry = nullptr, *d_rz = nullptr;
  double *d_lx = nullptr, *d_ly = nullptr, *d_lz = nullptr;
  int *d_rg_off = nullptr, *d_lg_off = nullptr;
  float4 *d_rg_sph = nullptr;   // (centre - O, radius) FP32
  D4 *d_lg_sph = nullptr;  // (centre in the positioned frame, radius)
  D4 *d_lb_sph = nullptr;  // per block of kLigBlock ligand residues: sphere enclosing theirs
  uint8_t *d_rg_chain = nullptr, *d_lg_chain = nullptr;
  std::vector<void *> allocs;
  uint64_t bytes = 0;
};

namespace {

constexpr int kMaxGroupAtoms = 64;

// Under GD_TRACE: wait for the stream and print the time since `t` (then
// reset it), so that device phases can be told apart.  No-op otherwise.
void trace_step(const char *name, cudaStream_t st, std::chrono::steady_clock::time_point &t) {
  if (!trace_on()) return;
  cudaStreamSynchronize(st);
  const auto now = std::chrono::steady_clock::now();
  trace(name, std::chrono::duration<double>(now - t).count());
  t = now;
}

struct PhaseTimer {
  const char *name;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit PhaseTimer(const char *n) : name(n) {}
  ~PhaseTimer() { trace(name, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count()); }
};

__device__ __forceinline__ void xform(const gd_pose_frame &f, double cx, double cy, double cz, double xo, double yo,
                                      double zo, double &X, double &Y, double &Z) {
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

// ((dx)^2 + (dy)^2) + (dz)^2 as src/clustering.rs:98 forms it
__device__ __forceinline__ double d2_exact(double ax, double ay, double az, double bx, double by, double bz) {
  const double dx = __dsub_rn(ax, bx), dy = __dsub_rn(ay, by), dz = __dsub_rn(az, bz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

struct ContactParams {
  const double *rx, *ry, *rz;
  const int *rg_off;
  const float4 *rg_sph;
  const uint8_t *rg_chain;
  const double *lx, *ly, *lz;
  const int *lg_off;
  const D4 *lg_sph;
  const uint8_t *lg_chain;
  int GR, GL;
  double cx, cy, cz, ox, oy, oz;
  const gd_pose_frame *frames;
  int n;
  double t_le;     // contact decision: d2 <= t_le
  float reach;     // cutoff + culling margin
  int *counts;     // [n]
  uint32_t *lists; // [n * cap]
  int cap;
};

constexpr int kContactWarps = 8;
constexpr int kLigBlock = 8;    // ligand residues per contact-bitmap work item
constexpr int kCandMax = 1024;  // receptor residue candidates kept per block
constexpr int kBlockAtoms = 128;  // ligand atoms of a block transformed in one pass (else residue by residue)
constexpr int kRecAtoms = 32;     // receptor residues up to this size are pre-filtered atom by atom

__global__ void __launch_bounds__(kContactWarps * 32) k_contacts_rl(const ContactParams p) {
  __shared__ double s_xyz[kContactWarps][3][kMaxGroupAtoms];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long items = static_cast<long long>(p.n) * p.GL;
  for (long long it = static_cast<long long>(blockIdx.x) * kContactWarps + wib; it < items;
       it += static_cast<long long>(gridDim.x) * kContactWarps) {
    const int pose = static_cast<int>(it / p.GL), lg = static_cast<int>(it % p.GL);
    const gd_pose_frame f = p.frames[pose];
    const int a0 = p.lg_off[lg], na = p.lg_off[lg + 1] - a0;
    const bool staged = na <= kMaxGroupAtoms;
    if (staged) {
      for (int a = lane; a < na; a += 32) {
        double X, Y, Z;
        xform(f, p.cx, p.cy, p.cz, p.lx[a0 + a], p.ly[a0 + a], p.lz[a0 + a], X, Y, Z);
        s_xyz[wib][0][a] = X;
        s_xyz[wib][1][a] = Y;
        s_xyz[wib][2][a] = Z;
      }
    }
    __syncwarp();
    // culling sphere of the ligand residue after the transform
    const D4 ls = p.lg_sph[lg];
    double CX, CY, CZ;
    xform(f, p.cx, p.cy, p.cz, ls.x, ls.y, ls.z, CX, CY, CZ);
    const float lcx = static_cast<float>(CX - p.ox), lcy = static_cast<float>(CY - p.oy),
                lcz = static_cast<float>(CZ - p.oz);
    const float lrad = static_cast<float>(ls.w);
    const uint8_t lchain = p.lg_chain[lg];
    for (int rg = lane; rg < p.GR; rg += 32) {
      if (p.rg_chain[rg] == lchain) continue;
      const float4 rs = p.rg_sph[rg];
      const float dx = rs.x - lcx, dy = rs.y - lcy, dz = rs.z - lcz;
      const float lim = rs.w + lrad + p.reach;
      if (dx * dx + dy * dy + dz * dz > lim * lim) continue;
      bool found = false;
      for (int b = p.rg_off[rg]; b < p.rg_off[rg + 1] && !found; ++b) {
        const double bx = p.rx[b], by = p.ry[b], bz = p.rz[b];
        for (int a = 0; a < na; ++a) {
          double X, Y, Z;
          if (staged) {
            X = s_xyz[wib][0][a];
            Y = s_xyz[wib][1][a];
            Z = s_xyz[wib][2][a];
          } else {
            xform(f, p.cx, p.cy, p.cz, p.lx[a0 + a], p.ly[a0 + a], p.lz[a0 + a], X, Y, Z);
          }
          if (d2_exact(bx, by, bz, X, Y, Z) <= p.t_le) {
            found = true;
            break;
          }
        }
      }
      if (found) {
        const int slot = atomicAdd(&p.counts[pose], 1);
        if (slot < p.cap) p.lists[static_cast<size_t>(pose) * p.cap + slot] = static_cast<uint32_t>(rg) * p.GL + lg;
      }
    }
    __syncwarp();
  }
}

// pose bitsets over the compacted contact universe: n rows of W 64-bit words
struct FccParams {
  const unsigned long long *bits;
  const int *sizes;
  int n, W;
  double c, cs;  // fcc_cutoff and fcc_cutoff * strictness
  uint32_t *adj; // n rows of ceil(n/32) words; bit j of row i: edge i -> j
  int adj_words;
  int c0;        // contacts every pose has (inter-chain ones within one molecule), not in the bitsets
};

constexpr int kFT = 64;   // pose tile
constexpr int kFW = 18;   // words per staged chunk (groups of 3; row stride 19 words: no bank conflicts)

// The common count of a pose pair is symmetric: only tiles on or above the
// diagonal run, and an off-diagonal tile decides both directions of each pair.
__global__ void __launch_bounds__(256) k_fcc(const FccParams p) {
  if (blockIdx.y > blockIdx.x) return;
  __shared__ unsigned long long sa[kFT][kFW + 1];
  __shared__ unsigned long long sb[kFT][kFW + 1];
  const int i0 = blockIdx.y * kFT, j0 = blockIdx.x * kFT;
  const bool diag = blockIdx.y == blockIdx.x;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads, 4 x 4 pairs each
  int cnt[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) cnt[a][b] = 0;
  for (int w0 = 0; w0 < p.W; w0 += kFW) {
    for (int e = threadIdx.x; e < kFT * kFW; e += 256) {
      const int r = e / kFW, w = e % kFW;
      const int gi = i0 + r, gj = j0 + r, gw = w0 + w;
      sa[r][w] = (gi < p.n && gw < p.W) ? p.bits[static_cast<size_t>(gi) * p.W + gw] : 0ull;
      sb[r][w] = (gj < p.n && gw < p.W) ? p.bits[static_cast<size_t>(gj) * p.W + gw] : 0ull;
    }
    __syncthreads();
    // three words at a time through a carry-save step: with l = x0^x1^x2 and
    // h = majority(x0, x1, x2), popc(x0) + popc(x1) + popc(x2) =
    // 2 popc(h) + popc(l): two popcounts (the XU pipe) instead of three
#pragma unroll 1
    for (int w = 0; w < kFW; w += 3) {
      unsigned long long av[4][3], bv[4][3];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i) av[a][i] = sa[ty + 16 * a][w + i];
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int i = 0; i < 3; ++i) bv[b][i] = sb[tx + 16 * b][w + i];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const unsigned long long x0 = av[a][0] & bv[b][0], x1 = av[a][1] & bv[b][1], x2 = av[a][2] & bv[b][2];
          const unsigned long long l = x0 ^ x1 ^ x2, h = (x0 & x1) | (x2 & (x0 ^ x1));
          cnt[a][b] += 2 * __popcll(h) + __popcll(l);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = i0 + ty + 16 * a;
    if (i >= p.n) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + tx + 16 * b;
      if (j >= p.n) continue;
      const int si = p.sizes[i] + p.c0, sj = p.sizes[j] + p.c0;
      // calculate_fcc (src/clustering.rs:122-132) and the first test of
      // create_elements (src/clustering.rs:171); the second test for the
      // pair (j, i) is the same condition, evaluated in that pair's thread.
      bool edge = false, back = false;
      if (si > 0 && sj > 0) {
        const double common = static_cast<double>(cnt[a][b] + p.c0);
        const double fcc = common / static_cast<double>(si);
        const double fcc_v = common / static_cast<double>(sj);
        edge = fcc >= p.c && fcc_v >= p.cs;  // i -> j
        back = fcc_v >= p.c && fcc >= p.cs;  // j -> i: the same ratios, roles swapped
      }
      if (edge) atomicOr(&p.adj[static_cast<size_t>(i) * p.adj_words + (j >> 5)], 1u << (j & 31));
      if (back && !diag) atomicOr(&p.adj[static_cast<size_t>(j) * p.adj_words + (i >> 5)], 1u << (i & 31));
    }
  }
}

__global__ void k_compact_lists(const uint32_t *lists, const int *counts, const long long *offs, int n, int cap,
                                uint32_t *out) {
  for (long long pose = blockIdx.x; pose < n; pose += gridDim.x) {
    const int c = min(counts[pose], cap);
    for (int k = threadIdx.x; k < c; k += blockDim.x) out[offs[pose] + k] = lists[pose * cap + k];
  }
}

// ---- contact bitmaps on the device (single-chain receptor and ligand) ----

struct BitsParams {
  const float4 *r32;
  const double *rx, *ry, *rz;
  const int *rg_off;
  const float4 *rg_sph;
  const uint8_t *rg_chain;
  const double *lx, *ly, *lz;
  const int *lg_off;
  const D4 *lg_sph;
  const D4 *lb_sph;
  const uint8_t *lg_chain;
  int GR, GL;
  double cx, cy, cz, ox, oy, oz;
  const gd_pose_frame *frames;
  int n;
  double t_le;       // exact decision d2 <= t_le
  float t32, guard;  // FP32 decision d2 <= t32 outside |d2 - t32| < guard
  float reach;
  uint32_t *bits;    // [n][words], bit rg*GL + lg
  long long words;
  int *err;          // the context's error word (index checks of the debug library)
};

// One warp per (pose, block of kLigBlock consecutive ligand residues).  The
// block's enclosing sphere first selects the receptor residues within reach
// of any of its residues (a shared-memory candidate list; all residues when
// the list would overflow).  Then, residue by residue, the atoms are
// transformed exactly and kept in FP64 and FP32, and each lane tests
// candidate receptor residues (culled by bounding spheres), first in FP32,
// re-deciding in FP64 the atom pairs whose FP32 d2 is within the guard band
// of the cutoff.
__global__ void __launch_bounds__(kContactWarps * 32) k_contact_bits(const BitsParams p) {
  // FP32 images of the exact ligand coordinates: the whole block's atoms when
  // they fit (one lane per atom, all residues at once), else one residue's
  __shared__ float4 s_f[kContactWarps][kBlockAtoms];
  __shared__ float4 s_ls[kContactWarps][kLigBlock + 1];  // residue spheres, then the block's (FP32 centre, radius)
  __shared__ uint16_t s_cand[kContactWarps][kCandMax];
  // the current receptor residue's atoms that reach the ligand residue's
  // sphere, compacted (FP32 coordinates, atom index within the residue)
  __shared__ float4 s_ra[kContactWarps][kRecAtoms];
  __shared__ uint8_t s_ri[kContactWarps][kRecAtoms];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nb = (p.GL + kLigBlock - 1) / kLigBlock;
  const long long items = static_cast<long long>(p.n) * nb;
  for (long long it = static_cast<long long>(blockIdx.x) * kContactWarps + wib; it < items;
       it += static_cast<long long>(gridDim.x) * kContactWarps) {
    const int pose = static_cast<int>(it / nb), blk = static_cast<int>(it % nb);
    // the frame is read where it is used (not held in registers across the item)
    const gd_pose_frame &f = p.frames[pose];
    const int lg0 = blk * kLigBlock, lg_end = min(p.GL, lg0 + kLigBlock);
    // the FP64 transforms of the item in lane-parallel rounds (FP64 issues at
    // a small fraction of the FP32 rate on this part): the residue spheres'
    // and the block sphere's centres in one round, the block's atoms in
    // rounds of 32
    if (lane <= kLigBlock) {
      const bool on = lane == kLigBlock || lg0 + lane < lg_end;
      const D4 sp = lane == kLigBlock ? p.lb_sph[blk] : (on ? p.lg_sph[lg0 + lane] : D4{0.0, 0.0, 0.0, 0.0});
      double X, Y, Z;
      xform(f, p.cx, p.cy, p.cz, sp.x, sp.y, sp.z, X, Y, Z);
      s_ls[wib][lane] = make_float4(static_cast<float>(X - p.ox), static_cast<float>(Y - p.oy),
                                    static_cast<float>(Z - p.oz), static_cast<float>(sp.w));
    }
    const int A0 = p.lg_off[lg0], A1 = p.lg_off[lg_end];
    const bool batched = A1 - A0 <= kBlockAtoms;
    if (batched)
      for (int a = lane; a < A1 - A0; a += 32) {
        double X, Y, Z;
        xform(f, p.cx, p.cy, p.cz, p.lx[A0 + a], p.ly[A0 + a], p.lz[A0 + a], X, Y, Z);
        s_f[wib][a] = make_float4(static_cast<float>(X - p.ox), static_cast<float>(Y - p.oy),
                                  static_cast<float>(Z - p.oz), 0.0f);
      }
    __syncwarp();
    int ncand = 0;
    {
      const float4 bs = s_ls[wib][kLigBlock];
      for (int r0 = 0; r0 < p.GR; r0 += 32) {
        const int rg = r0 + lane;
        bool near = false;
        if (rg < p.GR) {
          const float4 rs = p.rg_sph[rg];
          const float dx = rs.x - bs.x, dy = rs.y - bs.y, dz = rs.z - bs.z;
          const float lim = rs.w + bs.w + p.reach;
          near = dx * dx + dy * dy + dz * dz <= lim * lim;
        }
        const unsigned m = __ballot_sync(0xffffffffu, near);
        const int pos = ncand + __popc(m & ((1u << lane) - 1u));
        if (near && pos < kCandMax) s_cand[wib][pos] = static_cast<uint16_t>(rg);
        ncand += __popc(m);
      }
      __syncwarp();
    }
    const bool every = ncand > kCandMax;  // list overflowed: scan every receptor residue
    const int nscan = every ? p.GR : ncand;
    for (int lg = lg0; lg < lg_end; ++lg) {
    const int a0 = p.lg_off[lg], na = min(p.lg_off[lg + 1] - a0, kMaxGroupAtoms);
    const float4 *laf = s_f[wib] + (batched ? a0 - A0 : 0);
    if (!batched) {
      for (int a = lane; a < na; a += 32) {
        double X, Y, Z;
        xform(f, p.cx, p.cy, p.cz, p.lx[a0 + a], p.ly[a0 + a], p.lz[a0 + a], X, Y, Z);
        s_f[wib][a] = make_float4(static_cast<float>(X - p.ox), static_cast<float>(Y - p.oy),
                                  static_cast<float>(Z - p.oz), 0.0f);
      }
      __syncwarp();
    }
    const float4 ls = s_ls[wib][lg - lg0];
    const uint8_t lchain = p.lg_chain[lg];
    uint32_t *row = p.bits + static_cast<size_t>(pose) * p.words;
    // exact re-decision of a pair in the guard band: the ligand atom moved in
    // FP64 again (rare), the reference's distance order
    auto exact_le = [&](int b, int a) {
      double X, Y, Z;
      xform(f, p.cx, p.cy, p.cz, p.lx[a0 + a], p.ly[a0 + a], p.lz[a0 + a], X, Y, Z);
      return d2_exact(p.rx[b], p.ry[b], p.rz[b], X, Y, Z) <= p.t_le;
    };
    // lanes split a residue pair's atom pairs: lane = (receptor atom step,
    // ligand atom a); na <= 32 gives per = 32 / na receptor atoms per round
    const int per = na <= 32 ? 32 / na : 1;
    const int my_a = na <= 32 ? lane % na : 0, my_b = na <= 32 ? lane / na : 0;
    const bool lane_on = na <= 32 && lane < per * na;
    for (int k0 = 0; k0 < nscan; k0 += 32) {
      // 32 candidates at a time: the sphere test on one lane each
      const int k = k0 + lane;
      int rg = -1;
      bool near = false;
      if (k < nscan) {
        rg = every ? k : s_cand[wib][k];
        if (p.rg_chain[rg] != lchain) {
          const float4 rs = p.rg_sph[rg];
          const float dx = rs.x - ls.x, dy = rs.y - ls.y, dz = rs.z - ls.z;
          const float lim = rs.w + ls.w + p.reach;
          near = dx * dx + dy * dy + dz * dz <= lim * lim;
        }
      }
      unsigned m = __ballot_sync(0xffffffffu, near);
      while (m) {
        // each near receptor residue: the whole warp over its atom pairs,
        // stopping at the first contact
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const int r = __shfl_sync(0xffffffffu, rg, src);
        const int b0 = p.rg_off[r], b1 = p.rg_off[r + 1];
        bool found = false;
        if (na <= 32 && b1 - b0 <= kRecAtoms) {
          // one lane per receptor atom: only the atoms within reach of the
          // ligand residue's sphere can make a contact; they are compacted
          // and paired with the residue's atoms, `per` of them per round
          bool cand = false;
          float4 ra = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          if (lane < b1 - b0) {
            ra = p.r32[b0 + lane];
            const float dx = ra.x - ls.x, dy = ra.y - ls.y, dz = ra.z - ls.z;
            const float lim = ls.w + p.reach;
            cand = dx * dx + dy * dy + dz * dz <= lim * lim;
          }
          const unsigned M = __ballot_sync(0xffffffffu, cand);
          if (cand) {
            const int pos = __popc(M & ((1u << lane) - 1u));
            s_ra[wib][pos] = ra;
            s_ri[wib][pos] = static_cast<uint8_t>(lane);
          }
          __syncwarp();
          const int nc = __popc(M);
          for (int kb = 0; kb < nc && !found; kb += per) {
            const int k = kb + my_b;
            bool hit = false;
            if (lane_on && k < nc) {
              const float4 rb = s_ra[wib][k];
              const float4 la = laf[GD_DCHECK(p.err, laf + my_a < s_f[wib] + kBlockAtoms, 30) ? my_a : 0];
              const float ex = rb.x - la.x, ey = rb.y - la.y, ez = rb.z - la.z;
              const float d2 = ex * ex + ey * ey + ez * ez;
              if (d2 <= p.t32 + p.guard) hit = d2 < p.t32 - p.guard || exact_le(b0 + s_ri[wib][k], my_a);
            }
            found = __any_sync(0xffffffffu, hit);
          }
          __syncwarp();  // the compacted atoms are read before the next residue's
        } else if (na <= 32) {
          for (int bb = b0; bb < b1 && !found; bb += per) {
            const int b = bb + my_b;
            bool hit = false;
            if (lane_on && b < b1) {
              const float4 rb = p.r32[b];
              const float4 la = laf[GD_DCHECK(p.err, laf + my_a < s_f[wib] + kBlockAtoms, 30) ? my_a : 0];
              const float ex = rb.x - la.x, ey = rb.y - la.y, ez = rb.z - la.z;
              const float d2 = ex * ex + ey * ey + ez * ez;
              if (d2 <= p.t32 + p.guard) hit = d2 < p.t32 - p.guard || exact_le(b, my_a);
            }
            found = __any_sync(0xffffffffu, hit);
          }
        } else {
          // a residue with more than 32 heavy atoms: lanes over its atoms
          for (int b = b0; b < b1 && !found; ++b) {
            const float4 rb = p.r32[b];
            bool hit = false;
            for (int a = lane; a < na; a += 32) {
              const float4 la = laf[a];
              const float ex = rb.x - la.x, ey = rb.y - la.y, ez = rb.z - la.z;
              const float d2 = ex * ex + ey * ey + ez * ez;
              if (d2 <= p.t32 + p.guard) hit = hit || d2 < p.t32 - p.guard || exact_le(b, a);
            }
            found = __any_sync(0xffffffffu, hit);
          }
        }
        if (found && lane == 0) {
          const long long idx = static_cast<long long>(r) * p.GL + lg;
          if (GD_DCHECK(p.err, (idx >> 5) < p.words, 31)) atomicOr(&row[idx >> 5], 1u << (idx & 31));
        }
      }
    }
    __syncwarp();
    }
    __syncwarp();
  }
}

// Set bits of each pose's contact bitmap (one block per pose at a time).
__global__ void __launch_bounds__(256) k_bits_count(const uint32_t *bits, int n, long long words, int *counts) {
  __shared__ int s_w[8];
  for (int pose = blockIdx.x; pose < n; pose += gridDim.x) {
    const uint32_t *row = bits + static_cast<size_t>(pose) * words;
    int c = 0;
    for (long long w = threadIdx.x; w < words; w += blockDim.x) c += __popc(row[w]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int k = 0; k < 8; ++k) tot += s_w[k];
      counts[pose] = tot;
    }
    __syncthreads();
  }
}

// The set bits' indices (rg * GL + lg) of each pose's bitmap, in ascending
// order, from offs[pose] on: blocks of 256 words, a block-wide exclusive scan
// of their popcounts placing each word's bits.
__global__ void __launch_bounds__(256) k_bits_lists(const uint32_t *bits, int n, long long words,
                                                    const long long *offs, uint32_t *out) {
  __shared__ int s_w[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int pose = blockIdx.x; pose < n; pose += gridDim.x) {
    const uint32_t *row = bits + static_cast<size_t>(pose) * words;
    long long o = offs[pose];
    for (long long w0 = 0; w0 < words; w0 += blockDim.x) {
      const long long w = w0 + threadIdx.x;
      uint32_t v = w < words ? row[w] : 0u;
      const int c = __popc(v);
      int inc = c;  // inclusive scan within the warp
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += y;
      }
      if (lane == 31) s_w[wid] = inc;
      __syncthreads();
      int before = 0, tot = 0;
      for (int k = 0; k < 8; ++k) {
        before += k < wid ? s_w[k] : 0;
        tot += s_w[k];
      }
      long long pos = o + before + inc - c;
      while (v) {
        const int b = __ffs(v) - 1;
        v &= v - 1;
        out[pos++] = static_cast<uint32_t>(w * 32 + b);
      }
      o += tot;
      __syncthreads();
    }
  }
}

// Union over poses and set-bit count of each bitmap word.
__global__ void k_union(const uint32_t *bits, int n, long long words, uint32_t *ubits, int *ucount) {
  for (long long w = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; w < words;
       w += static_cast<long long>(gridDim.x) * blockDim.x) {
    uint32_t u = 0;
    for (int p = 0; p < n; ++p) u |= bits[static_cast<size_t>(p) * words + w];
    ubits[w] = u;
    ucount[w] = __popc(u);
  }
}

// Exclusive prefix sum of the per-word counts (one CTA) -> compacted offsets.
__global__ void __launch_bounds__(1024) k_scan(const int *cnt, long long words, int *base, int *total) {
  __shared__ int s[1024];
  const int t = threadIdx.x;
  const long long per = (words + 1023) / 1024;
  const long long w0 = t * per, w1 = min(words, w0 + per);
  int sum = 0;
  for (long long w = w0; w < w1; ++w) sum += cnt[w];
  s[t] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int v = t >= o ? s[t - o] : 0;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  int run = s[t] - sum;
  for (long long w = w0; w < w1; ++w) {
    base[w] = run;
    run += cnt[w];
  }
  if (t == 1023) *total = s[1023];
}

// Pose bitsets over the compacted universe: bit base[w] + rank of the bit
// within ubits[w].
__global__ void k_compact(const uint32_t *bits, const uint32_t *ubits, const int *base, int n, long long words, int W,
                          unsigned long long *out, int *sizes) {
  for (long long it = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; it < static_cast<long long>(n) * words;
       it += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int p = static_cast<int>(it / words);
    const long long w = it % words;
    const uint32_t u = ubits[w];
    if (!u) continue;
    uint32_t v = bits[static_cast<size_t>(p) * words + w] & u;
    if (!v) continue;
    atomicAdd(&sizes[p], __popc(v));
    unsigned long long *row = out + static_cast<size_t>(p) * W;
    while (v) {
      const int b = __ffs(v) - 1;
      v &= v - 1;
      const int pos = base[w] + __popc(u & ((1u << b) - 1u));
      atomicOr(&row[pos >> 6], 1ull << (pos & 63));
    }
  }
}

// ---- FCC pair counts from per-contact pose lists ("postings") ----
// For poses whose contacts are spread (few poses per contact), the common
// count of a pose pair is the number of contacts whose list holds both: the
// work is the sum over contacts of k (k - 1) / 2 for k poses per contact,
// against n^2 / 2 pose pairs x W words for the bitsets.  Counts are exact
// integers either way, so the clusters are identical.

// Per contact (compacted index): how many poses make it; per pose: its size.
__global__ void k_post_count(const uint32_t *bits, const uint32_t *ubits, const int *base, int n, long long words,
                             int *kc, int *sizes) {
  for (long long it = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; it < static_cast<long long>(n) * words;
       it += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int p = static_cast<int>(it / words);
    const long long w = it % words;
    const uint32_t u = ubits[w];
    if (!u) continue;
    uint32_t v = bits[static_cast<size_t>(p) * words + w] & u;
    if (!v) continue;
    atomicAdd(&sizes[p], __popc(v));
    while (v) {
      const int b = __ffs(v) - 1;
      v &= v - 1;
      atomicAdd(&kc[base[w] + __popc(u & ((1u << b) - 1u))], 1);
    }
  }
}

// Sum over contacts of k (k - 1) / 2: the pair increments of the posting path.
__global__ void k_post_work(const int *kc, int U, unsigned long long *sum) {
  unsigned long long acc = 0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < U; c += gridDim.x * blockDim.x) {
    const unsigned long long k = static_cast<unsigned long long>(kc[c]);
    acc += k * (k - (k > 0 ? 1 : 0)) / 2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(sum, acc);
}

// The poses of each contact, at offs[c] onwards (order within a list is
// free: the counts do not depend on it).
__global__ void k_post_fill(const uint32_t *bits, const uint32_t *ubits, const int *base, int n, long long words,
                            const int *offs, int *cursor, int *post) {
  for (long long it = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; it < static_cast<long long>(n) * words;
       it += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int p = static_cast<int>(it / words);
    const long long w = it % words;
    const uint32_t u = ubits[w];
    if (!u) continue;
    uint32_t v = bits[static_cast<size_t>(p) * words + w] & u;
    while (v) {
      const int b = __ffs(v) - 1;
      v &= v - 1;
      const int c = base[w] + __popc(u & ((1u << b) - 1u));
      post[offs[c] + atomicAdd(&cursor[c], 1)] = p;
    }
  }
}

// One warp per contact: +1 on the common count of every pose pair in its list.
__global__ void k_post_pairs(const int *offs, const int *kc, const int *post, int U, int n, uint32_t *common) {
  const int lane = threadIdx.x & 31;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < U; c += (gridDim.x * blockDim.x) >> 5) {
    const int k = kc[c], o = offs[c];
    for (int a = 0; a + 1 < k; ++a) {
      const int i = post[o + a];
      for (int b = a + 1 + lane; b < k; b += 32) {
        const int j = post[o + b];
        const int lo = min(i, j), hi = max(i, j);
        atomicAdd(&common[static_cast<size_t>(lo) * n + hi], 1u);
      }
    }
  }
}

// calculate_fcc and create_elements (src/clustering.rs:122-132,171) from the
// common counts of the pairs i <= j (the diagonal: the pose's own size), as
// k_fcc decides them.
__global__ void k_post_decide(const uint32_t *common, const int *sizes, int n, double c, double cs, uint32_t *adj,
                              int adj_words, int c0) {
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const int si = sizes[i] + c0;
    for (int j = i + threadIdx.x; j < n; j += blockDim.x) {
      const int sj = sizes[j] + c0;
      bool edge = false, back = false;
      if (si > 0 && sj > 0) {
        const double cm =
            static_cast<double>(i == j ? si : static_cast<int>(common[static_cast<size_t>(i) * n + j]) + c0);
        const double fcc = cm / static_cast<double>(si);
        const double fcc_v = cm / static_cast<double>(sj);
        edge = fcc >= c && fcc_v >= cs;
        back = fcc_v >= c && fcc >= cs;
      }
      if (edge) atomicOr(&adj[static_cast<size_t>(i) * adj_words + (j >> 5)], 1u << (j & 31));
      if (back && j != i) atomicOr(&adj[static_cast<size_t>(j) * adj_words + (i >> 5)], 1u << (i & 31));
    }
  }
}

// host mirror of the device transform (same operation order, no fused ops)
void xform_host(const gd_pose_frame &f, double cx, double cy, double cz, double xo, double yo, double zo, double &X,
                double &Y, double &Z) {
  const double x = xo - cx, y = yo - cy, z = zo - cz;
  const double nx = x * f.ca * f.cb + y * f.m01 + z * f.m02;
  const double ny = x * f.sa * f.cb + y * f.m11 + z * f.m12;
  const double nz = -x * f.sb + y * f.cb * f.sg + z * f.cb * f.cg;
  X = nx + cx + f.dx;
  Y = ny + cy + f.dy;
  Z = nz + cz + f.dz;
}

inline int64_t canon(int64_t ka, int64_t kb) {
  // "cA rA cB rB" with the smaller chain first (src/clustering.rs:100-105)
  const int64_t ca = ka >> 16, cb = kb >> 16;
  if (ca > cb) std::swap(ka, kb);
  return ((ka >> 16) << 48) | ((ka & 0xffff) << 32) | ((kb >> 16) << 16) | (kb & 0xffff);
}

// Inter-chain contacts among the residues of one molecule at coordinates x,
// y, z (host; multi-chain receptors once, multi-chain ligands per pose):
// residue pairs on different chains with an atom pair at d2 <= t_le.  Pairs
// whose enclosing spheres are beyond the cutoff are skipped.  When unstable is
// given it is set if some residue pair's closest atom pair lies within a
// relative 1e-6 of t_le: a decision that the FP64 rounding of a rigid
// transform (some 1e-12 A^2 on d2) could not flip lies far outside that.
void intra_contacts(const std::vector<int64_t> &gkey, const std::vector<int> &goff, const std::vector<int> &atoms,
                    const double *x, const double *y, const double *z, double t_le, std::vector<int64_t> &out,
                    bool *unstable = nullptr) {
  const int G = static_cast<int>(gkey.size());
  std::vector<double> c(3 * static_cast<size_t>(G)), r(G);
  for (int g = 0; g < G; ++g)
    enclosing_ball(x, y, z, atoms.data() + goff[g], goff[g + 1] - goff[g], &c[3 * static_cast<size_t>(g)], r[g]);
  // a skipped pair's closest atoms lie beyond the cutoff by more than the band
  const double band = 1e-6 * t_le, reach = std::sqrt(t_le) + 1e-4;
  for (int g = 0; g < G; ++g)
    for (int h = g + 1; h < G; ++h) {
      if ((gkey[g] >> 16) == (gkey[h] >> 16)) continue;
      const double *cg = &c[3 * static_cast<size_t>(g)], *ch = &c[3 * static_cast<size_t>(h)];
      const double ex = cg[0] - ch[0], ey = cg[1] - ch[1], ez = cg[2] - ch[2];
      const double lim = r[g] + r[h] + reach;
      if (ex * ex + ey * ey + ez * ez > lim * lim * (1.0 + 1e-9)) continue;
      double best = INFINITY;
      for (int a = goff[g]; a < goff[g + 1] && !(best < t_le - band); ++a)
        for (int b = goff[h]; b < goff[h + 1]; ++b) {
          const int ia = atoms[a], ib = atoms[b];
          const double dx = x[ia] - x[ib], dy = y[ia] - y[ib], dz = z[ia] - z[ib];
          best = std::min(best, dx * dx + dy * dy + dz * dz);
          if (best < t_le - band) break;
        }
      if (best <= t_le) out.push_back(canon(gkey[g], gkey[h]));
      if (unstable && std::fabs(best - t_le) <= band) *unstable = true;
    }
}

// The topology's device arrays, staged on the host and copied in one piece
// (each 256-byte aligned): one cudaMalloc and one cudaMemcpy per complex.
struct TopoPack {
  struct Item {
    const void *src;
    size_t bytes, off;
    std::function<void(char *)> bind;
  };
  std::vector<Item> items;
  size_t total = 0;
  template <typename T>
  void add(const std::vector<T> &h, T **d) {
    const size_t off = total;
    items.push_back(Item{h.empty() ? nullptr : h.data(), sizeof(T) * h.size(), off,
                         [d, off](char *base) { *d = reinterpret_cast<T *>(base + off); }});
    total += (sizeof(T) * std::max<size_t>(h.size(), 1) + 255) / 256 * 256;
  }
  gd_status commit(gd_context *ctx, ClusterTopo *t) {
    void *p = nullptr;
    gd_status s = dev_alloc(ctx, total, &p);
    if (s != GD_OK) return s;
    t->allocs.push_back(p);
    t->bytes += total;
    std::vector<char> h(total, 0);
    for (const Item &it : items)
      if (it.bytes) std::memcpy(h.data() + it.off, it.src, it.bytes);
    const cudaError_t e = cudaMemcpy(p, h.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpy (contact topology)");
    for (const Item &it : items) it.bind(static_cast<char *>(p));
    return GD_OK;
  }
};

void group_atoms(const std::vector<uint8_t> &chain, const std::vector<int16_t> &res, const std::vector<uint8_t> &elem,
                 std::vector<int64_t> &gkey, std::vector<int> &goff, std::vector<int> &atoms) {
  std::map<int64_t, std::vector<int>> g;
  for (size_t i = 0; i < chain.size(); ++i) {
    if (elem[i] == GD_ELEM_H) continue;  // src/clustering.rs:67-70
    g[(static_cast<int64_t>(chain[i]) << 16) | static_cast<uint16_t>(res[i])].push_back(static_cast<int>(i));
  }
  goff.assign(1, 0);
  for (auto &kv : g) {
    gkey.push_back(kv.first);
    atoms.insert(atoms.end(), kv.second.begin(), kv.second.end());
    goff.push_back(static_cast<int>(atoms.size()));
  }
}

gd_status build_topo(gd_complex *cx, ClusterTopo **out) {
  gd_context *ctx = cx->ctx;
  ClusterTopo *t = new ClusterTopo();
  group_atoms(cx->h_rchain, cx->h_rres, cx->h_relem, t->rg_key, t->rg_off, t->r_atoms);
  group_atoms(cx->h_lchain, cx->h_lres, cx->h_lelem, t->lg_key, t->lg_off, t->l_atoms);
  t->GR = static_cast<int>(t->rg_key.size());
  t->GL = static_cast<int>(t->lg_key.size());
  for (int g = 1; g < t->GR; ++g) t->multi_chain_rec |= (t->rg_key[g] >> 16) != (t->rg_key[0] >> 16);
  for (int g = 1; g < t->GL; ++g) t->multi_chain_lig |= (t->lg_key[g] >> 16) != (t->lg_key[0] >> 16);
  {
    std::vector<int64_t> a = t->rg_key, b = t->lg_key, both;
    std::set_intersection(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(both));
    t->mixed = !both.empty();
  }
  std::vector<double> rx, ry, rz, lx, ly, lz;
  for (int i : t->r_atoms) {
    rx.push_back(cx->h_rx[i]);
    ry.push_back(cx->h_ry[i]);
    rz.push_back(cx->h_rz[i]);
  }
  for (int i : t->l_atoms) {
    lx.push_back(cx->h_lx[i]);
    ly.push_back(cx->h_ly[i]);
    lz.push_back(cx->h_lz[i]);
  }
  std::vector<float4> r32(rx.size());
  for (size_t a = 0; a < rx.size(); ++a)
    r32[a] = make_float4(static_cast<float>(rx[a] - cx->ox), static_cast<float>(ry[a] - cx->oy),
                         static_cast<float>(rz[a] - cx->oz), 0.0f);
  std::vector<float4> rsph(t->GR);
  std::vector<uint8_t> rch(t->GR), lch(t->GL);
  for (int g = 0; g < t->GR; ++g) {
    double c[3], r;
    const int a0 = t->rg_off[g];
    enclosing_ball(rx.data() + a0, ry.data() + a0, rz.data() + a0, nullptr, t->rg_off[g + 1] - a0, c, r);
    rsph[g] = make_float4(static_cast<float>(c[0] - cx->ox), static_cast<float>(c[1] - cx->oy),
                          static_cast<float>(c[2] - cx->oz), static_cast<float>(r * (1 + 1e-6) + 1e-3));
    rch[g] = static_cast<uint8_t>(t->rg_key[g] >> 16);
  }
  std::vector<D4> lsph(t->GL);
  for (int g = 0; g < t->GL; ++g) {
    double c[3], r;
    const int a0 = t->lg_off[g];
    enclosing_ball(lx.data() + a0, ly.data() + a0, lz.data() + a0, nullptr, t->lg_off[g + 1] - a0, c, r);
    lsph[g] = D4{c[0], c[1], c[2], r * (1 + 1e-6) + 1e-3};
    lch[g] = static_cast<uint8_t>(t->lg_key[g] >> 16);
  }
  // blocks of kLigBlock consecutive ligand residues: a sphere enclosing all
  // their atoms (with the same small widening)
  const int nb = (t->GL + kLigBlock - 1) / kLigBlock;
  std::vector<D4> lbsph(std::max(nb, 1), D4{0, 0, 0, 0});
  for (int b = 0; b < nb; ++b) {
    const int g0 = b * kLigBlock, g1 = std::min(t->GL, g0 + kLigBlock);
    double c[3], r;
    const int a0 = t->lg_off[g0];
    enclosing_ball(lx.data() + a0, ly.data() + a0, lz.data() + a0, nullptr, t->lg_off[g1] - a0, c, r);
    lbsph[b] = D4{c[0], c[1], c[2], r * (1 + 1e-6) + 1e-3};
  }
  // one allocation and one copy for every array of the topology
  TopoPack pack;
  pack.add(lbsph, &t->d_lb_sph);
  pack.add(rx, &t->d_rx);
  pack.add(ry, &t->d_ry);
  pack.add(rz, &t->d_rz);
  pack.add(lx, &t->d_lx);
  pack.add(ly, &t->d_ly);
  pack.add(lz, &t->d_lz);
  pack.add(t->rg_off, &t->d_rg_off);
  pack.add(t->lg_off, &t->d_lg_off);
  pack.add(rsph, &t->d_rg_sph);
  pack.add(lsph, &t->d_lg_sph);
  pack.add(rch, &t->d_rg_chain);
  pack.add(lch, &t->d_lg_chain);
  pack.add(r32, &t->d_r32);
  const gd_status s = pack.commit(ctx, t);
  if (s != GD_OK) {
    for (void *q : t->allocs) cudaFree(q);
    ctx->in_use -= std::min<uint64_t>(ctx->in_use, t->bytes);
    delete t;
    return s;
  }
  *out = t;
  return GD_OK;
}

gd_status get_topo(gd_complex *cx, ClusterTopo **t) {
  if (!cx->cluster_cache) {
    ClusterTopo *nt = nullptr;
    gd_status s = build_topo(cx, &nt);
    if (s != GD_OK) return s;
    cx->cluster_cache = nt;
  }
  *t = static_cast<ClusterTopo *>(cx->cluster_cache);
  return GD_OK;
}

// Greedy clustering of cluster_elements (src/clustering.rs:183-254) over an
// adjacency bit matrix (row e, bit m: edge e -> m), then the size filter
// (src/clustering.rs:289-292).
//  - count[e] = unused neighbours of e (its self-edge included, as in the
//    reference); the centre is the unused element with the largest count,
//    lower index on ties.
//  - A cluster holds the centre and its unused neighbours, so its size is at
//    most count + 1 (+1 only without a self-edge, i.e. an empty contact set).
//    Counts never grow, so once the best count + 1 is below min_size every
//    later cluster would be dropped by the size filter: the loop stops there
//    without changing the kept clusters or their order.
//  - After a cluster M is formed, every unused e loses |N(e) & M|, taken
//    from the bit rows (per member bit for small M, popcounts for large M).
int greedy_clusters(const std::vector<uint32_t> &adj, int n, int words, int min_size, int32_t *centers, int32_t *sizes,
                    int32_t *members) {
  std::vector<int> count(n, 0);
  for (int e = 0; e < n; ++e)
    for (int w = 0; w < words; ++w) count[e] += __builtin_popcount(adj[static_cast<size_t>(e) * words + w]);
  std::vector<char> used(n, 0);
  std::vector<uint32_t> mbits(words, 0);
  struct Cl { int center, first, size; };
  std::vector<Cl> cls;
  std::vector<int> mem;
  for (;;) {
    int center = -1, best = -1;
    for (int e = 0; e < n; ++e)
      if (!used[e] && count[e] > best) {
        best = count[e];
        center = e;
      }
    if (center < 0 || best + 1 < min_size) break;
    const int first = static_cast<int>(mem.size());
    mem.push_back(center);
    const uint32_t *row = &adj[static_cast<size_t>(center) * words];
    for (int w = 0; w < words; ++w) {
      uint32_t v = row[w];
      while (v) {
        const int b = __builtin_ctz(v);
        v &= v - 1;
        const int m = w * 32 + b;
        if (m != center && !used[m]) mem.push_back(m);
      }
    }
    const int size = static_cast<int>(mem.size()) - first;
    for (int k = first; k < first + size; ++k) used[mem[k]] = 1;
    // counts of the remaining elements lose their edges into the cluster
    if (size < words) {
      for (int k = first; k < first + size; ++k) {
        const int m = mem[k], mw = m >> 5;
        const uint32_t mb = 1u << (m & 31);
        for (int e = 0; e < n; ++e)
          if (!used[e] && (adj[static_cast<size_t>(e) * words + mw] & mb)) --count[e];
      }
    } else {
      std::fill(mbits.begin(), mbits.end(), 0u);
      for (int k = first; k < first + size; ++k) mbits[mem[k] >> 5] |= 1u << (mem[k] & 31);
      for (int e = 0; e < n; ++e) {
        if (used[e]) continue;
        const uint32_t *re = &adj[static_cast<size_t>(e) * words];
        int c = 0;
        for (int w = 0; w < words; ++w) c += __builtin_popcount(re[w] & mbits[w]);
        count[e] -= c;
      }
    }
    std::sort(mem.begin() + first, mem.end());
    cls.push_back(Cl{center, first, size});
  }
  std::stable_sort(cls.begin(), cls.end(), [](const Cl &a, const Cl &b) { return a.size > b.size; });
  int k = 0, mo = 0;
  for (const Cl &c : cls) {
    if (c.size < min_size) continue;
    centers[k] = c.center;
    sizes[k] = c.size;
    std::memcpy(members + mo, mem.data() + c.first, sizeof(int32_t) * c.size);
    mo += c.size;
    ++k;
  }
  return k;
}

}  // namespace

void free_cluster_cache(gd_complex *cx) {
  if (!cx->cluster_cache) return;
  ClusterTopo *t = static_cast<ClusterTopo *>(cx->cluster_cache);
  for (void *p : t->allocs) cudaFree(p);
  cx->ctx->in_use -= std::min<uint64_t>(cx->ctx->in_use, t->bytes);
  delete t;
  cx->cluster_cache = nullptr;
}

bool bits_path_ok(const ClusterTopo *t, int n, bool multi_chain = false);
long long bits_words(const ClusterTopo *t);
gd_status launch_contact_bits(gd_complex *cx, ClusterTopo *t, const gd_pose_frame *d_frames, int n, double cutoff,
                              double maxd, uint32_t *d_bits, long long words, cudaStream_t st);
double max_displacement(const double *genes, int n);

// Contacts of n poses through the contact bitmaps: k_contact_bits, then the
// set bits of every pose as (receptor residue group * GL + ligand residue
// group) entries, flat with per-pose offsets loffs (n + 1 entries).
static gd_status contacts_via_bits(gd_complex *cx, ClusterTopo *t, const std::vector<gd_pose_frame> &frames, int n,
                                   double cutoff, double maxd, std::vector<uint32_t> &flat,
                                   std::vector<long long> &loffs) {
  gd_context *ctx = cx->ctx;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  const long long words = bits_words(t);
  const size_t fb = sizeof(gd_pose_frame) * n, bits_b = sizeof(uint32_t) * static_cast<size_t>(words) * n,
               cb = sizeof(int) * n, ob = sizeof(long long) * (n + 1);
  gd_status s = ensure_scratch(ctx, al(fb) + al(bits_b) + al(cb) + al(ob), 0);
  if (s != GD_OK) return s;
  char *base = static_cast<char *>(ctx->d_scratch);
  gd_pose_frame *d_frames = reinterpret_cast<gd_pose_frame *>(base);
  uint32_t *d_bits = reinterpret_cast<uint32_t *>(base + al(fb));
  int *d_counts = reinterpret_cast<int *>(base + al(fb) + al(bits_b));
  long long *d_offs = reinterpret_cast<long long *>(base + al(fb) + al(bits_b) + al(cb));
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(d_frames, frames.data(), fb, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "contacts setup");
  s = launch_contact_bits(cx, t, d_frames, n, cutoff, maxd, d_bits, words, st);
  if (s != GD_OK) return s;
  const int grid = std::max(1, std::min(n, ctx->sm_count * 8));
  k_bits_count<<<grid, 256, 0, st>>>(d_bits, n, words, d_counts);
  std::vector<int> counts(n);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts.data(), d_counts, cb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "contact bitmaps");
  s = check_device_error(ctx);
  if (s != GD_OK) return s;
  loffs.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) loffs[i + 1] = loffs[i] + counts[i];
  flat.resize(static_cast<size_t>(loffs[n]));
  ctx->last_contacts = 2;
  if (loffs[n] == 0) return GD_OK;
  void *d_flat = nullptr;
  const size_t flat_b = sizeof(uint32_t) * flat.size();
  s = dev_alloc(ctx, flat_b, &d_flat);
  if (s != GD_OK) return s;
  e = cudaMemcpyAsync(d_offs, loffs.data(), ob, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_bits_lists<<<grid, 256, 0, st>>>(d_bits, n, words, d_offs, static_cast<uint32_t *>(d_flat));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(flat.data(), d_flat, flat_b, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  dev_free(ctx, d_flat, flat_b);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "contact bitmap lists");
  return GD_OK;
}

// Contact keys of n poses (sorted per pose) into a host vector + offsets:
// through the contact bitmaps when the topology allows it (and
// GD_TUNE_CONTACTS does not ask for the lists), else through per-residue
// contact lists (k_contacts_rl).  Both decide every atom pair exactly.
gd_status pose_contacts_host(gd_complex *cx, const double *genes, int n, double cutoff, std::vector<int64_t> &keys,
                             std::vector<int64_t> &offs) {
  gd_context *ctx = cx->ctx;
  PhaseTimer pt_all("contacts: total");
  ClusterTopo *t = nullptr;
  gd_status s = get_topo(cx, &t);
  if (s != GD_OK) return s;
  const Thresholds thr = make_thresholds(cutoff);
  if (t->multi_chain_rec && t->rr_cutoff != cutoff) {
    t->rr_keys.clear();
    intra_contacts(t->rg_key, t->rg_off, t->r_atoms, cx->h_rx.data(), cx->h_ry.data(), cx->h_rz.data(),
                   thr.contact_le, t->rr_keys);
    t->rr_cutoff = cutoff;
  }
  std::vector<gd_pose_frame> frames(n);
  gd_make_frames(genes, n, frames.data());
  const long long pairs = static_cast<long long>(t->GR) * t->GL;
  int cap = static_cast<int>(std::min<long long>(std::max<long long>(pairs, 1), 2048));
  std::vector<int> counts(n);
  std::vector<uint32_t> flat;
  std::vector<long long> loffs(n + 1, 0);
  const bool via_bits = ctx->tune_contacts != 1 && n > 0 && bits_path_ok(t, n);
  if (via_bits) {
    s = contacts_via_bits(cx, t, frames, n, cutoff, max_displacement(genes, n), flat, loffs);
    if (s != GD_OK) return s;
  } else {
    ctx->last_contacts = 1;
  }
  for (int attempt = 0; attempt < 2 && !via_bits; ++attempt) {
    const size_t fb = sizeof(gd_pose_frame) * n, cb = sizeof(int) * n,
                 lb = sizeof(uint32_t) * static_cast<size_t>(n) * cap, ob = sizeof(long long) * (n + 1);
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    s = ensure_scratch(ctx, al(fb) + al(cb) + al(lb) + al(ob) + al(lb), 0);
    if (s != GD_OK) return s;
    char *base = static_cast<char *>(ctx->d_scratch);
    gd_pose_frame *d_frames = reinterpret_cast<gd_pose_frame *>(base);
    int *d_counts = reinterpret_cast<int *>(base + al(fb));
    uint32_t *d_lists = reinterpret_cast<uint32_t *>(base + al(fb) + al(cb));
    long long *d_offs = reinterpret_cast<long long *>(base + al(fb) + al(cb) + al(lb));
    uint32_t *d_flat = reinterpret_cast<uint32_t *>(base + al(fb) + al(cb) + al(lb) + al(ob));
    cudaError_t e = cudaMemcpyAsync(d_frames, frames.data(), fb, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_counts, 0, cb, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "contacts setup");
    if (pairs > 0) {
      ContactParams p{};
      p.rx = t->d_rx;
      p.ry = t->d_ry;
      p.rz = t->d_rz;
      p.rg_off = t->d_rg_off;
      p.rg_sph = t->d_rg_sph;
      p.rg_chain = t->d_rg_chain;
      p.lx = t->d_lx;
      p.ly = t->d_ly;
      p.lz = t->d_lz;
      p.lg_off = t->d_lg_off;
      p.lg_sph = t->d_lg_sph;
      p.lg_chain = t->d_lg_chain;
      p.GR = t->GR;
      p.GL = t->GL;
      p.cx = cx->cx;
      p.cy = cx->cy;
      p.cz = cx->cz;
      p.ox = cx->ox;
      p.oy = cx->oy;
      p.oz = cx->oz;
      p.frames = d_frames;
      p.n = n;
      p.t_le = thr.contact_le;
      p.reach = static_cast<float>(cutoff) + 0.05f;
      p.counts = d_counts;
      p.lists = d_lists;
      p.cap = cap;
      const long long items = static_cast<long long>(n) * t->GL;
      const int grid = static_cast<int>(std::min<long long>((items + kContactWarps - 1) / kContactWarps,
                                                            static_cast<long long>(ctx->sm_count) * 16));
      k_contacts_rl<<<grid, kContactWarps * 32, 0, ctx->stream>>>(p);
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, e, "contacts kernel launch");
    }
    e = cudaMemcpyAsync(counts.data(), d_counts, cb, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "contacts kernel");
    trace("contacts: kernel + counts", std::chrono::duration<double>(std::chrono::steady_clock::now() - pt_all.t0).count());
    const int maxc = n > 0 ? *std::max_element(counts.begin(), counts.end()) : 0;
    if (maxc > cap) {  // rerun once with room for the largest pose
      cap = maxc;
      continue;
    }
    for (int i = 0; i < n; ++i) loffs[i + 1] = loffs[i] + counts[i];
    flat.resize(static_cast<size_t>(loffs[n]));
    if (loffs[n] > 0) {
      e = cudaMemcpyAsync(d_offs, loffs.data(), ob, cudaMemcpyHostToDevice, ctx->stream);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "H2D offsets");
      k_compact_lists<<<std::min(n, ctx->sm_count * 8), 128, 0, ctx->stream>>>(d_lists, d_counts, d_offs, n, cap,
                                                                                 d_flat);
      e = cudaMemcpyAsync(flat.data(), d_flat, sizeof(uint32_t) * flat.size(), cudaMemcpyDeviceToHost, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "contact list gather");
    }
    break;
  }
  PhaseTimer pt_keys("contacts: host keys");
  // each pose's keys on up to 16 threads (contiguous pose ranges), then
  // concatenated in pose order
  const int nth = n >= 256 ? static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency()))) : 1;
  std::vector<std::vector<int64_t>> part(nth);
  std::vector<int64_t> cnt(n, 0);
  auto work = [&](int q) {
    const int i0 = static_cast<int>(static_cast<long long>(n) * q / nth),
              i1 = static_cast<int>(static_cast<long long>(n) * (q + 1) / nth);
    std::vector<int64_t> pk;
    std::vector<double> tx, ty, tz;
    for (int i = i0; i < i1; ++i) {
      pk.clear();
      for (long long k = loffs[i]; k < loffs[i + 1]; ++k) {
        const uint32_t v = flat[k];
        pk.push_back(canon(t->rg_key[v / t->GL], t->lg_key[v % t->GL]));
      }
      pk.insert(pk.end(), t->rr_keys.begin(), t->rr_keys.end());
      if (t->multi_chain_lig) {
        tx.resize(cx->nl);
        ty.resize(cx->nl);
        tz.resize(cx->nl);
        for (int a : t->l_atoms)
          xform_host(frames[i], cx->cx, cx->cy, cx->cz, cx->h_lx[a], cx->h_ly[a], cx->h_lz[a], tx[a], ty[a], tz[a]);
        intra_contacts(t->lg_key, t->lg_off, t->l_atoms, tx.data(), ty.data(), tz.data(), thr.contact_le, pk);
      }
      std::sort(pk.begin(), pk.end());
      pk.erase(std::unique(pk.begin(), pk.end()), pk.end());
      part[q].insert(part[q].end(), pk.begin(), pk.end());
      cnt[i] = static_cast<int64_t>(pk.size());
    }
  };
  if (nth == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int q = 0; q < nth; ++q) th.emplace_back(work, q);
    for (auto &x : th) x.join();
  }
  offs.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) offs[i + 1] = offs[i] + cnt[i];
  keys.clear();
  keys.reserve(static_cast<size_t>(offs[n]));
  for (const auto &v : part) keys.insert(keys.end(), v.begin(), v.end());
  return GD_OK;
}

gd_status cluster_sets(gd_context *ctx, const int64_t *keys, const int64_t *offs, int n, const gd_cluster_cfg &cfg,
                       int32_t *n_clusters, int32_t *centers, int32_t *sizes, int32_t *members) {
  *n_clusters = 0;
  if (n <= 0) return GD_OK;
  PhaseTimer pt_all("fcc: total");
  // compacted contact universe, each pose's contacts as universe indices
  // (distinct, ascending) and the number of poses per contact; the host work
  // runs on up to 16 threads (poses split in contiguous ranges)
  const size_t nk = static_cast<size_t>(offs[n]);
  const int nth = nk >= (1u << 16) ? static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency()))) : 1;
  auto parallel = [nth](int count, const std::function<void(int, int, int)> &f) {
    if (nth == 1) return f(0, 0, count);
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t)
      th.emplace_back(f, t, static_cast<int>(static_cast<long long>(count) * t / nth),
                      static_cast<int>(static_cast<long long>(count) * (t + 1) / nth));
    for (auto &x : th) x.join();
  };
  std::vector<int64_t> uni(keys, keys + nk);
  {
    // sorted runs per thread, then pairwise merges
    std::vector<size_t> cut(nth + 1);
    for (int t = 0; t <= nth; ++t) cut[t] = nk * t / nth;
    parallel(nth, [&](int, int t0, int t1) {
      for (int t = t0; t < t1; ++t) std::sort(uni.begin() + cut[t], uni.begin() + cut[t + 1]);
    });
    for (int w = 1; w < nth; w *= 2)
      for (int t = 0; t + w < nth; t += 2 * w)
        std::inplace_merge(uni.begin() + cut[t], uni.begin() + cut[t + w], uni.begin() + cut[std::min(nth, t + 2 * w)]);
    uni.erase(std::unique(uni.begin(), uni.end()), uni.end());
  }
  const int U = static_cast<int>(uni.size());
  std::vector<int> ui(nk);
  std::vector<int64_t> uoff(n + 1, 0);
  std::vector<int> sz(n), kc(std::max(U, 1), 0);
  parallel(n, [&](int, int i0, int i1) {
    for (int i = i0; i < i1; ++i) {
      const size_t o = static_cast<size_t>(offs[i]);
      size_t m = o;
      for (int64_t k = offs[i]; k < offs[i + 1]; ++k)
        ui[m++] = static_cast<int>(std::lower_bound(uni.begin(), uni.end(), keys[k]) - uni.begin());
      if (!std::is_sorted(ui.begin() + o, ui.begin() + m)) std::sort(ui.begin() + o, ui.begin() + m);
      sz[i] = static_cast<int>(std::unique(ui.begin() + o, ui.begin() + m) - (ui.begin() + o));
    }
  });
  // each pose's distinct indices packed to the front of its range
  for (int i = 0; i < n; ++i) {
    const size_t o = static_cast<size_t>(offs[i]), d = static_cast<size_t>(uoff[i]);
    if (d != o) std::copy(ui.begin() + o, ui.begin() + o + sz[i], ui.begin() + d);
    for (int k = 0; k < sz[i]; ++k) ++kc[ui[d + k]];
    uoff[i + 1] = uoff[i] + sz[i];
  }
  const int W = std::max(1, (U + 63) / 64);
  const int aw = (n + 31) / 32;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  // pair counts: bitsets, or the poses of each contact (postings) when the
  // contacts are spread thin (GD_TUNE_FCC; the same cost model as the device
  // clustering path)
  double work = 0.0;
  for (int u = 0; u < U; ++u) work += 0.5 * static_cast<double>(kc[u]) * (kc[u] - 1);
  const double bits_work = 0.5 * static_cast<double>(n) * (n + 1) * W;
  bool postings = n <= 16384 && (ctx->tune_fcc == 2 || (ctx->tune_fcc == 0 && bits_work > 2e10 && 80.0 * work < bits_work));
  const size_t sb = sizeof(int) * n, ab = sizeof(uint32_t) * static_cast<size_t>(n) * aw;
  std::vector<uint32_t> adj(static_cast<size_t>(n) * aw);
  cudaStream_t st = ctx->stream;
  if (postings) {
    const size_t memb = static_cast<size_t>(uoff[n]);
    std::vector<int> poff(U + 1, 0), list(std::max<size_t>(memb, 1));
    for (int u = 0; u < U; ++u) poff[u + 1] = poff[u] + kc[u];
    std::vector<int> cur(poff.begin(), poff.end() - 1);
    for (int i = 0; i < n; ++i)
      for (int64_t k = uoff[i]; k < uoff[i + 1]; ++k) list[cur[ui[k]]++] = i;
    const size_t ob = sizeof(int) * (U + 1), kb = sizeof(int) * std::max(U, 1), lb = sizeof(int) * list.size(),
                 cb = sizeof(uint32_t) * static_cast<size_t>(n) * n;
    const size_t total = al(ob) + al(kb) + al(lb) + al(cb) + al(sb) + al(ab);
    void *buf = nullptr;
    gd_status s = dev_alloc(ctx, total, &buf);
    if (s != GD_OK && ctx->tune_fcc != 2) {
      postings = false;  // no room for the n x n counts: the bitsets
      ctx->last_error.clear();
    } else if (s != GD_OK) {
      return s;
    }
    if (postings) {
      trace("fcc: universe + postings (host)",
            std::chrono::duration<double>(std::chrono::steady_clock::now() - pt_all.t0).count());
      const auto t_k = std::chrono::steady_clock::now();
      char *b = static_cast<char *>(buf);
      int *d_off = reinterpret_cast<int *>(b);
      int *d_kc = reinterpret_cast<int *>(b + al(ob));
      int *d_list = reinterpret_cast<int *>(b + al(ob) + al(kb));
      uint32_t *d_common = reinterpret_cast<uint32_t *>(b + al(ob) + al(kb) + al(lb));
      int *d_sz = reinterpret_cast<int *>(b + al(ob) + al(kb) + al(lb) + al(cb));
      uint32_t *d_adj = reinterpret_cast<uint32_t *>(b + al(ob) + al(kb) + al(lb) + al(cb) + al(sb));
      cudaError_t e = cudaMemcpyAsync(d_off, poff.data(), ob, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_kc, kc.data(), kb, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_list, list.data(), lb, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_sz, sz.data(), sb, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(d_common, 0, cb, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(d_adj, 0, ab, st);
      if (e == cudaSuccess && U > 0)
        k_post_pairs<<<std::max(1, std::min((U + 7) / 8, ctx->sm_count * 16)), 256, 0, st>>>(d_off, d_kc, d_list, U, n,
                                                                                            d_common);
      if (e == cudaSuccess) {
        k_post_decide<<<std::min(n, ctx->sm_count * 16), 256, 0, st>>>(d_common, d_sz, n, cfg.fcc_cutoff,
                                                                       cfg.fcc_cutoff * cfg.strictness, d_adj, aw, 0);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaMemcpyAsync(adj.data(), d_adj, ab, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      dev_free(ctx, buf, total);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "FCC postings");
      ctx->last_fcc = 2;
      trace("fcc: kernels + transfers", std::chrono::duration<double>(std::chrono::steady_clock::now() - t_k).count());
    }
  }
  if (!postings) {
    std::vector<unsigned long long> bits(static_cast<size_t>(n) * W, 0ull);
    parallel(n, [&](int, int i0, int i1) {
      for (int i = i0; i < i1; ++i)
        for (int64_t k = uoff[i]; k < uoff[i + 1]; ++k)
          bits[static_cast<size_t>(i) * W + ui[k] / 64] |= 1ull << (ui[k] % 64);
    });
    const size_t bb = sizeof(unsigned long long) * bits.size();
    gd_status s = ensure_scratch(ctx, al(bb) + al(sb) + al(ab), 0);
    if (s != GD_OK) return s;
    char *base = static_cast<char *>(ctx->d_scratch);
    unsigned long long *d_bits = reinterpret_cast<unsigned long long *>(base);
    int *d_sz = reinterpret_cast<int *>(base + al(bb));
    uint32_t *d_adj = reinterpret_cast<uint32_t *>(base + al(bb) + al(sb));
    trace("fcc: universe + bitsets (host)",
          std::chrono::duration<double>(std::chrono::steady_clock::now() - pt_all.t0).count());
    const auto t_k = std::chrono::steady_clock::now();
    cudaError_t e = cudaMemcpyAsync(d_bits, bits.data(), bb, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_sz, sz.data(), sb, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_adj, 0, ab, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "FCC setup");
    FccParams p{};
    p.bits = d_bits;
    p.sizes = d_sz;
    p.n = n;
    p.W = W;
    p.c = cfg.fcc_cutoff;
    p.cs = cfg.fcc_cutoff * cfg.strictness;
    p.adj = d_adj;
    p.adj_words = aw;
    dim3 grid((n + kFT - 1) / kFT, (n + kFT - 1) / kFT);
    k_fcc<<<grid, 256, 0, st>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, e, "FCC kernel launch");
    e = cudaMemcpyAsync(adj.data(), d_adj, ab, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "FCC kernel");
    ctx->last_fcc = 1;
    trace("fcc: kernel + transfers", std::chrono::duration<double>(std::chrono::steady_clock::now() - t_k).count());
  }
  PhaseTimer pt_g("fcc: greedy clustering (host)");
  *n_clusters = greedy_clusters(adj, n, aw, cfg.min_cluster_size, centers, sizes, members);
  return GD_OK;
}

// cluster_structures entirely on the device for a single-chain receptor and
// ligand that share no residue: contact bitmaps, union, compaction, FCC; the
// greedy pass runs on the host.  Returns GD_ERR_STATE when the topology or the
// bitmap size calls for the general path.
// The contact-bitmap path (k_contact_bits) serves receptors and ligands that
// share no residue, with every ligand residue staged whole, at most 8 GiB of
// bitmaps and bit indices that fit 32 bits; single-chain ones only unless
// multi_chain (clustering adds the inter-chain contacts within each molecule
// as a constant; per-pose contact lists take the host path for them).
bool bits_path_ok(const ClusterTopo *t, int n, bool multi_chain) {
  if (t->mixed || (!multi_chain && (t->multi_chain_rec || t->multi_chain_lig))) return false;
  for (int g = 0; g < t->GL; ++g)
    if (t->lg_off[g + 1] - t->lg_off[g] > kMaxGroupAtoms) return false;  // residues staged whole
  const long long pairs = static_cast<long long>(t->GR) * t->GL;
  if (pairs > static_cast<long long>(UINT32_MAX)) return false;
  const long long words = std::max<long long>(1, (pairs + 31) / 32);
  return sizeof(uint32_t) * static_cast<size_t>(words) * static_cast<size_t>(n) <= (static_cast<size_t>(8) << 30);
}

long long bits_words(const ClusterTopo *t) {
  return std::max<long long>(1, (static_cast<long long>(t->GR) * t->GL + 31) / 32);
}

// Contact bitmaps of n device-resident poses: d_bits (n rows of `words`
// words, bit rg * GL + lg) is cleared and filled by k_contact_bits on st.
// maxd bounds the poses' |displacement| components (it sizes the FP32 guard
// band, as for the scoring kernels).
gd_status launch_contact_bits(gd_complex *cx, ClusterTopo *t, const gd_pose_frame *d_frames, int n, double cutoff,
                              double maxd, uint32_t *d_bits, long long words, cudaStream_t st) {
  gd_context *ctx = cx->ctx;
  const Thresholds thr = make_thresholds(cutoff);
  cudaError_t e = cudaMemsetAsync(d_bits, 0, sizeof(uint32_t) * static_cast<size_t>(words) * n, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "contact bitmaps setup");
  BitsParams p{};
  p.r32 = t->d_r32;
  p.rx = t->d_rx;
  p.ry = t->d_ry;
  p.rz = t->d_rz;
  p.rg_off = t->d_rg_off;
  p.rg_sph = t->d_rg_sph;
  p.rg_chain = t->d_rg_chain;
  p.lx = t->d_lx;
  p.ly = t->d_ly;
  p.lz = t->d_lz;
  p.lg_off = t->d_lg_off;
  p.lg_sph = t->d_lg_sph;
  p.lb_sph = t->d_lb_sph;
  p.lg_chain = t->d_lg_chain;
  p.GR = t->GR;
  p.GL = t->GL;
  p.cx = cx->cx;
  p.cy = cx->cy;
  p.cz = cx->cz;
  p.ox = cx->ox;
  p.oy = cx->oy;
  p.oz = cx->oz;
  p.frames = d_frames;
  p.n = n;
  p.t_le = thr.contact_le;
  p.t32 = static_cast<float>(thr.contact_le);
  {
    // FP32 error bound of d2 near the cutoff (as for the scoring guard bands)
    const double u = std::ldexp(1.0, -24), c = cutoff;
    const double M = std::max(cx->rec_extent, cx->lig_radius + maxd +
                                                  std::max({std::fabs(cx->cx - cx->ox), std::fabs(cx->cy - cx->oy),
                                                            std::fabs(cx->cz - cx->oz)})) + 1.0;
    const double err = 2.0 * c * std::sqrt(3.0) * (2.0 * M * u + c * u) + 4.0 * c * c * u;
    p.guard = static_cast<float>(4.0 * err + 1e-6);
  }
  p.reach = static_cast<float>(cutoff) + 0.05f;
  p.bits = d_bits;
  p.words = words;
  p.err = ctx->d_err;
  const long long pairs = static_cast<long long>(t->GR) * t->GL;
  if (pairs > 0 && n > 0) {
    const long long items = static_cast<long long>(n) * ((t->GL + kLigBlock - 1) / kLigBlock);
    const int grid = static_cast<int>(std::min<long long>((items + kContactWarps - 1) / kContactWarps,
                                                          static_cast<long long>(ctx->sm_count) * 16));
    k_contact_bits<<<grid, kContactWarps * 32, 0, st>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, e, "contact bitmaps launch");
  }
  return GD_OK;
}

double max_displacement(const double *genes, int n) {
  double maxd = 0.0;
  for (int i = 0; i < n; ++i)
    for (int k = 3; k < 6; ++k) maxd = std::max(maxd, std::fabs(genes[6 * static_cast<size_t>(i) + k]));
  return maxd;
}

gd_status cluster_device(gd_complex *cx, const double *genes, int n, const gd_cluster_cfg &cfg, int32_t *n_clusters,
                         int32_t *centers, int32_t *sizes, int32_t *members) {
  gd_context *ctx = cx->ctx;
  PhaseTimer pt_all("cluster (device): total");
  ClusterTopo *t = nullptr;
  gd_status s = get_topo(cx, &t);
  if (s != GD_OK) return s;
  if (!bits_path_ok(t, n, true)) return GD_ERR_STATE;
  // contacts within one molecule across its chains are the same in every
  // pose (the receptor does not move; the ligand moves rigidly and its
  // decisions are checked to be far from the cutoff): a constant c0 in every
  // set size and pair count, outside the bitmaps
  const Thresholds thr = make_thresholds(cfg.contact_distance);
  long long c0 = 0;
  if (t->multi_chain_rec) {
    if (t->rr_cutoff != cfg.contact_distance) {
      t->rr_keys.clear();
      intra_contacts(t->rg_key, t->rg_off, t->r_atoms, cx->h_rx.data(), cx->h_ry.data(), cx->h_rz.data(),
                     thr.contact_le, t->rr_keys);
      t->rr_cutoff = cfg.contact_distance;
    }
    c0 += static_cast<long long>(t->rr_keys.size());
  }
  if (t->multi_chain_lig) {
    if (t->ll_cutoff != cfg.contact_distance) {
      std::vector<int64_t> ll;
      bool unstable = false;
      intra_contacts(t->lg_key, t->lg_off, t->l_atoms, cx->h_lx.data(), cx->h_ly.data(), cx->h_lz.data(),
                     thr.contact_le, ll, &unstable);
      t->ll_count = static_cast<long long>(ll.size());
      t->ll_unstable = unstable;
      t->ll_cutoff = cfg.contact_distance;
    }
    if (t->ll_unstable) return GD_ERR_STATE;
    c0 += t->ll_count;
  }
  if (c0 > (1 << 30)) return GD_ERR_STATE;
  const long long words = bits_words(t);
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t bits_b = sizeof(uint32_t) * words * static_cast<size_t>(n);
  std::vector<gd_pose_frame> frames(n);
  gd_make_frames(genes, n, frames.data());
  const double maxd = max_displacement(genes, n);
  const size_t fb = sizeof(gd_pose_frame) * n, ub = sizeof(uint32_t) * words, cb = sizeof(int) * words;
  // the compacted universe is at most min(pairs, sum of sizes); size it after the scan
  auto t_step = std::chrono::steady_clock::now();
  s = ensure_scratch(ctx, al(fb) + al(bits_b) + al(ub) + 2 * al(cb) + al(sizeof(int)), 0);
  if (s != GD_OK) return s;
  char *base = static_cast<char *>(ctx->d_scratch);
  gd_pose_frame *d_frames = reinterpret_cast<gd_pose_frame *>(base);
  uint32_t *d_bits = reinterpret_cast<uint32_t *>(base + al(fb));
  uint32_t *d_u = reinterpret_cast<uint32_t *>(base + al(fb) + al(bits_b));
  int *d_cnt = reinterpret_cast<int *>(base + al(fb) + al(bits_b) + al(ub));
  int *d_base = reinterpret_cast<int *>(base + al(fb) + al(bits_b) + al(ub) + al(cb));
  int *d_total = reinterpret_cast<int *>(base + al(fb) + al(bits_b) + al(ub) + 2 * al(cb));
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(d_frames, frames.data(), fb, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "contact bitmaps setup");
  trace_step("cluster (device):   scratch + frames", st, t_step);
  s = launch_contact_bits(cx, t, d_frames, n, cfg.contact_distance, maxd, d_bits, words, st);
  if (s != GD_OK) return s;
  ctx->last_contacts = 2;
  trace_step("cluster (device):   k_contact_bits", st, t_step);
  const int g2 = static_cast<int>(std::min<long long>((words + 255) / 256, static_cast<long long>(ctx->sm_count) * 8));
  k_union<<<std::max(g2, 1), 256, 0, st>>>(d_bits, n, words, d_u, d_cnt);
  k_scan<<<1, 1024, 0, st>>>(d_cnt, words, d_base, d_total);
  trace_step("cluster (device):   k_union + k_scan", st, t_step);
  int U = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&U, d_total, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "contact bitmaps");
  const auto t_union = std::chrono::steady_clock::now();
  trace("cluster (device): contacts + union", std::chrono::duration<double>(t_union - pt_all.t0).count());
  const int W = std::max(1, (U + 63) / 64);
  const int aw = (n + 31) / 32;
  const size_t adj_b = sizeof(uint32_t) * static_cast<size_t>(n) * aw, sz_b = sizeof(int) * n;
  const long long tot = static_cast<long long>(n) * words;
  const int g3 = static_cast<int>(std::min<long long>((tot + 255) / 256, static_cast<long long>(ctx->sm_count) * 32));
  // pair counts: contact postings or bitsets (GD_TUNE_FCC; automatic: the
  // estimated cheaper one, postings only up to 16,384 poses, and considered
  // only when the bitsets would take more than ~2e10 word pairs, some 5 ms:
  // counting the postings costs a pass and a synchronisation)
  bool postings = ctx->tune_fcc == 2 && n <= 16384;
  const double bits_work = 0.5 * static_cast<double>(n) * (n + 1) * W;
  void *pre = nullptr;  // posting counts: kc[U], sizes[n], the work sum
  const size_t kc_b = sizeof(int) * static_cast<size_t>(std::max(U, 1));
  if (ctx->tune_fcc != 1 && n <= 16384 && (ctx->tune_fcc == 2 || bits_work > 2e10)) {
    s = dev_alloc(ctx, al(kc_b) + al(sz_b) + al(8), &pre);
    if (s != GD_OK) return s;
    int *d_kc = static_cast<int *>(pre);
    int *d_psz = reinterpret_cast<int *>(static_cast<char *>(pre) + al(kc_b));
    unsigned long long *d_work = reinterpret_cast<unsigned long long *>(static_cast<char *>(pre) + al(kc_b) + al(sz_b));
    unsigned long long work = 0;
    e = cudaMemsetAsync(pre, 0, al(kc_b) + al(sz_b) + al(8), st);
    if (e == cudaSuccess) {
      k_post_count<<<std::max(g3, 1), 256, 0, st>>>(d_bits, d_u, d_base, n, words, d_kc, d_psz);
      k_post_work<<<std::max(1, std::min((U + 255) / 256, ctx->sm_count * 8)), 256, 0, st>>>(d_kc, U, d_work);
      e = cudaMemcpyAsync(&work, d_work, 8, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      dev_free(ctx, pre, al(kc_b) + al(sz_b) + al(8));
      return cuda_fail(ctx, e, "FCC posting counts");
    }
    // an atomic increment costs about as much as 80 word pairs of popcount
    if (ctx->tune_fcc == 0) postings = 80.0 * static_cast<double>(work) < bits_work;
  }
  if (!postings && pre) {
    dev_free(ctx, pre, al(kc_b) + al(sz_b) + al(8));
    pre = nullptr;
  }
  auto compact_bytes = [&]() { return sizeof(unsigned long long) * static_cast<size_t>(W) * n; };
  size_t compact_b = postings ? 0 : compact_bytes();
  // postings: offsets and cursors per contact, the lists (one entry per
  // (pose, contact)), the n x n common counts
  const size_t off_b = sizeof(int) * (static_cast<size_t>(U) + 1), cur_b = kc_b;
  size_t memberships = 0;
  if (postings) {
    // the lists hold sum(kc) = sum of the pose sizes entries
    std::vector<int> hsz(n);
    e = cudaMemcpy(hsz.data(), static_cast<char *>(pre) + al(kc_b), sz_b, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      dev_free(ctx, pre, al(kc_b) + al(sz_b) + al(8));
      return cuda_fail(ctx, e, "FCC posting sizes");
    }
    for (int v : hsz) memberships += static_cast<size_t>(v);
  }
  const size_t list_b = sizeof(int) * std::max<size_t>(memberships, 1),
               common_b = postings ? sizeof(uint32_t) * static_cast<size_t>(n) * n : 0;
  size_t extra_b = postings ? al(off_b) + al(cur_b) + al(list_b) + al(common_b) + al(sz_b) + al(adj_b)
                            : al(compact_b) + al(sz_b) + al(adj_b);
  void *extra = nullptr;
  s = dev_alloc(ctx, extra_b, &extra);
  if (s != GD_OK && postings && ctx->tune_fcc != 2) {
    // no room for the n x n counts: the bitsets after all
    dev_free(ctx, pre, al(kc_b) + al(sz_b) + al(8));
    pre = nullptr;
    postings = false;
    compact_b = compact_bytes();
    extra_b = al(compact_b) + al(sz_b) + al(adj_b);
    s = dev_alloc(ctx, extra_b, &extra);
    if (s == GD_OK) ctx->last_error.clear();  // the refused allocation is not this call's failure
  }
  if (s != GD_OK) {
    if (pre) dev_free(ctx, pre, al(kc_b) + al(sz_b) + al(8));
    return s;
  }
  ctx->last_fcc = postings ? 2 : 1;
  char *xp = static_cast<char *>(extra);
  uint32_t *d_adj = reinterpret_cast<uint32_t *>(xp + extra_b - al(adj_b));
  int *d_sizes = reinterpret_cast<int *>(xp + extra_b - al(adj_b) - al(sz_b));
  e = cudaMemsetAsync(extra, 0, extra_b, st);
  if (e == cudaSuccess && postings) {
    int *d_kc = static_cast<int *>(pre);
    int *d_psz = reinterpret_cast<int *>(static_cast<char *>(pre) + al(kc_b));
    int *d_offs = reinterpret_cast<int *>(xp);
    int *d_cur = reinterpret_cast<int *>(xp + al(off_b));
    int *d_list = reinterpret_cast<int *>(xp + al(off_b) + al(cur_b));
    uint32_t *d_common = reinterpret_cast<uint32_t *>(xp + al(off_b) + al(cur_b) + al(list_b));
    e = cudaMemcpyAsync(d_sizes, d_psz, sz_b, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) {
      k_scan<<<1, 1024, 0, st>>>(d_kc, U, d_offs, d_offs + U);
      k_post_fill<<<std::max(g3, 1), 256, 0, st>>>(d_bits, d_u, d_base, n, words, d_offs, d_cur, d_list);
      k_post_pairs<<<std::max(1, std::min((U + 7) / 8, ctx->sm_count * 16)), 256, 0, st>>>(d_offs, d_kc, d_list, U, n,
                                                                                          d_common);
      k_post_decide<<<std::min(n, ctx->sm_count * 16), 256, 0, st>>>(
          d_common, d_sizes, n, cfg.fcc_cutoff, cfg.fcc_cutoff * cfg.strictness, d_adj, aw, static_cast<int>(c0));
      e = cudaGetLastError();
    }
  } else if (e == cudaSuccess) {
    unsigned long long *d_compact = reinterpret_cast<unsigned long long *>(xp);
    k_compact<<<std::max(g3, 1), 256, 0, st>>>(d_bits, d_u, d_base, n, words, W, d_compact, d_sizes);
    FccParams fp{};
    fp.bits = d_compact;
    fp.sizes = d_sizes;
    fp.n = n;
    fp.W = W;
    fp.c = cfg.fcc_cutoff;
    fp.cs = cfg.fcc_cutoff * cfg.strictness;
    fp.adj = d_adj;
    fp.adj_words = aw;
    fp.c0 = static_cast<int>(c0);
    dim3 grid((n + kFT - 1) / kFT, (n + kFT - 1) / kFT);
    k_fcc<<<grid, 256, 0, st>>>(fp);
    e = cudaGetLastError();
  }
  std::vector<uint32_t> adj(static_cast<size_t>(n) * aw);
  if (e == cudaSuccess) e = cudaMemcpyAsync(adj.data(), d_adj, adj_b, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  dev_free(ctx, extra, extra_b);
  if (pre) dev_free(ctx, pre, al(kc_b) + al(sz_b) + al(8));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "FCC on the device");
  const auto t_fcc = std::chrono::steady_clock::now();
  trace(postings ? "cluster (device): postings + fcc" : "cluster (device): compact + fcc",
        std::chrono::duration<double>(t_fcc - t_union).count());
  *n_clusters = greedy_clusters(adj, n, aw, cfg.min_cluster_size, centers, sizes, members);
  trace("cluster (device): greedy (host)", std::chrono::duration<double>(std::chrono::steady_clock::now() - t_fcc).count());
  return GD_OK;
}

}  // namespace gd

using namespace gd;

static gd_cluster_cfg default_cfg() { return gd_cluster_cfg{5.0, 0.60, 0.75, 4}; }

extern "C" {

gd_status gd_pose_contacts(gd_complex *cx, const double *genes, int32_t n, int64_t *keys, int64_t cap,
                           int64_t *offsets) {
  gd::NvtxRange nvtx_range("gd_pose_contacts");
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  if (n < 0 || (n > 0 && (!genes || !offsets)) || cap < 0 || (cap > 0 && !keys))
    return fail(ctx, GD_ERR_INVALID_ARG, "bad genes/keys/offsets");
  cudaSetDevice(ctx->device);
  std::vector<int64_t> k, o;
  gd_status s = pose_contacts_host(cx, genes, n, 5.0, k, o);
  if (s != GD_OK) return s;
  std::memcpy(offsets, o.data(), sizeof(int64_t) * (n + 1));
  if (static_cast<int64_t>(k.size()) > cap) return fail(ctx, GD_ERR_CAPACITY, "contact key buffer too small");
  if (!k.empty()) std::memcpy(keys, k.data(), sizeof(int64_t) * k.size());
  return GD_OK;
}

gd_status gd_cluster(gd_complex *cx, const double *genes, int32_t n, const gd_cluster_cfg *cfg, int32_t *n_clusters,
                     int32_t *centers, int32_t *sizes, int32_t *members) {
  gd::NvtxRange nvtx_range("gd_cluster");
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  if (n < 0 || (n > 0 && (!genes || !centers || !sizes || !members)) || !n_clusters)
    return fail(ctx, GD_ERR_INVALID_ARG, "bad cluster arguments");
  const gd_cluster_cfg c = cfg ? *cfg : default_cfg();
  *n_clusters = 0;
  if (n == 0) return GD_OK;  // cluster_structures on no structures
  cudaSetDevice(ctx->device);
  gd_status s = cluster_device(cx, genes, n, c, n_clusters, centers, sizes, members);
  if (s == GD_OK) s = check_device_error(ctx);
  if (s != GD_ERR_STATE) return s;
  // multi-chain molecules or shared residues: contact keys on the host path
  std::vector<int64_t> k, o;
  s = pose_contacts_host(cx, genes, n, c.contact_distance, k, o);
  if (s != GD_OK) return s;
  return cluster_sets(ctx, k.data(), o.data(), n, c, n_clusters, centers, sizes, members);
}

gd_status gd_cluster_sets(gd_context *ctx, const int64_t *keys, const int64_t *offsets, int32_t n,
                          const gd_cluster_cfg *cfg, int32_t *n_clusters, int32_t *centers, int32_t *sizes,
                          int32_t *members) {
  gd::NvtxRange nvtx_range("gd_cluster_sets");
  if (!ctx) return GD_ERR_INVALID_ARG;
  if (n < 0 || (n > 0 && (!offsets || !centers || !sizes || !members)) || !n_clusters)
    return fail(ctx, GD_ERR_INVALID_ARG, "bad cluster arguments");
  if (n > 0 && offsets[n] > 0 && !keys) return fail(ctx, GD_ERR_INVALID_ARG, "null keys");
  cudaSetDevice(ctx->device);
  const gd_cluster_cfg c = cfg ? *cfg : default_cfg();
  return cluster_sets(ctx, keys, offsets, n, c, n_clusters, centers, sizes, members);
}

}  // extern "C"
