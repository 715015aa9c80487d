// Device helpers shared by the scoring kernels: bulk-copy/mbarrier
// primitives (inline PTX), the exact pose transform, exact squared distance,
// compensated and warp sums, and the per-pose AIR/record epilogue.
#pragma once

#include "gd_internal.cuh"

namespace gd {

constexpr unsigned kFull = 0xffffffffu;

static __device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
static __device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
static __device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
static __device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared (the TMA engine), completing on an mbarrier.
static __device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
static __device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
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
static __device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait on an mbarrier phase: false after kWaitLimitNs of wall time
// (or kSpinLimit polls), so that a copy that never lands ends the kernel
// with an error instead of a hang.
static __device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t i = 1; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 0 && global_ns() - t0 > kWaitLimitNs) return false;
  }
  return false;
}

static __device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Rigid transform of one ligand atom with the reference's operation order
// (src/structure.rs:83-115, then displace :119-131); explicit _rn intrinsics
// keep the compiler from fusing multiply-adds, so the result is bit-identical
// to the host's double arithmetic.
static __device__ __forceinline__ void transform_atom(const gd_pose_frame &f, double cx, double cy, double cz,
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
static __device__ __forceinline__ void ligand_atom(const ScoreParams &p, const gd_pose_frame &f, int pose, int j,
                                            double &X, double &Y, double &Z) {
  if (p.models) {
    const double *m = p.models + (static_cast<size_t>(pose) * p.nl + p.lig_perm[j]) * 3;  // models: original order
    X = m[0];
    Y = m[1];
    Z = m[2];
  } else {
    transform_atom(f, p.cx, p.cy, p.cz, p.lig_x[j], p.lig_y[j], p.lig_z[j], X, Y, Z);
  }
}

// structure::distance squared, (dx*dx + dy*dy) + dz*dz (src/structure.rs:312-317)
static __device__ __forceinline__ double exact_d2(double ax, double ay, double az, double bx, double by, double bz) {
  const double dx = __dsub_rn(ax, bx), dy = __dsub_rn(ay, by), dz = __dsub_rn(az, bz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

static __device__ __forceinline__ double warp_sum(double v) {
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
static __device__ void air_terms(const ScoreParams &p, const gd_pose_frame &f, int pose, double &air, int &sat) {
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
static __device__ void write_pose(const ScoreParams &p, int pose, double vdw, double elec, double desolv,
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

}  // namespace gd
