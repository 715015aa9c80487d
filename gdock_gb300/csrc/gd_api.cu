// C ABI of gdock_gb300: contexts, complex upload (host-side packing of the
// receptor/ligand into the device layout), pose frames, and the scoring
// entry points.  No call throws across the ABI; every failure becomes a
// gd_status with a message in gd_last_error().
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <chrono>
#include <functional>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <unistd.h>
#include <cstdint>
#include <utility>

#include "gd_internal.cuh"

namespace gd {

bool trace_on() {
  static const bool on = std::getenv("GD_TRACE") != nullptr;
  return on;
}

void trace(const char *phase, double seconds) {
  if (trace_on()) std::fprintf(stderr, "[gdock_gb300] %-32s %10.3f ms\n", phase, seconds * 1e3);
}

gd_status fail(gd_context *ctx, gd_status s, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  return s;
}

gd_status cuda_fail(gd_context *ctx, cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return fail(ctx, e == cudaErrorMemoryAllocation ? GD_ERR_OOM : GD_ERR_CUDA, m);
}

gd_status dev_alloc(gd_context *ctx, uint64_t bytes, void **p) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (ctx->budget && ctx->in_use + bytes > ctx->budget)
    return fail(ctx, GD_ERR_OOM, "HBM budget exceeded: " + std::to_string(ctx->in_use + bytes) + " > " +
                                     std::to_string(ctx->budget) + " bytes");
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    // a failed allocation is not a sticky error: clear it, so that a caller
    // that falls back to a smaller plan does not read it back from
    // cudaGetLastError() after its next launch
    (void)cudaGetLastError();
    return cuda_fail(ctx, e, "cudaMalloc");
  }
  ctx->in_use += bytes;
  return GD_OK;
}

void dev_free(gd_context *ctx, void *p, uint64_t bytes) {
  if (!p) return;
  if (bytes == 0) bytes = 16;
  cudaFree(p);
  ctx->in_use -= std::min<uint64_t>(ctx->in_use, bytes);
}

gd_status ensure_scratch(gd_context *ctx, size_t dev_bytes, size_t pinned_bytes) {
  if (dev_bytes > ctx->d_scratch_bytes) {
    if (ctx->d_scratch) dev_free(ctx, ctx->d_scratch, ctx->d_scratch_bytes);
    ctx->d_scratch = nullptr;
    ctx->d_scratch_bytes = 0;
    size_t want = std::max(dev_bytes, static_cast<size_t>(1) << 20);
    gd_status s = dev_alloc(ctx, want, &ctx->d_scratch);
    if (s != GD_OK) return s;
    ctx->d_scratch_bytes = want;
  }
  if (pinned_bytes > ctx->h_pinned_bytes) {
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    ctx->h_pinned = nullptr;
    ctx->h_pinned_bytes = 0;
    size_t want = std::max(pinned_bytes, static_cast<size_t>(1) << 20);
    cudaError_t e = cudaMallocHost(&ctx->h_pinned, want);
    if (e != cudaSuccess) {
      ctx->h_pinned = nullptr;
      return cuda_fail(ctx, e, "cudaMallocHost");
    }
    ctx->h_pinned_bytes = want;
  }
  return GD_OK;
}

gd_status ensure_batch_scratch(gd_context *ctx, size_t dev_bytes) {
  if (dev_bytes <= ctx->d_batch_bytes) return GD_OK;
  if (ctx->d_batch) {
    cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, ctx->d_batch, ctx->d_batch_bytes);
  }
  ctx->d_batch = nullptr;
  ctx->d_batch_bytes = 0;
  const size_t want = std::max(dev_bytes, static_cast<size_t>(1) << 20);
  gd_status s = dev_alloc(ctx, want, &ctx->d_batch);
  if (s != GD_OK) return s;
  ctx->d_batch_bytes = want;
  return GD_OK;
}

gd_status check_device_error(gd_context *ctx) {
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "reading the device error word");
  if (h == kDevOk) return GD_OK;
  cudaMemset(ctx->d_err, 0, sizeof(int));
  if (h == kDevTimeout) return fail(ctx, GD_ERR_TIMEOUT, "a device-side wait exceeded its spin limit");
  if (h == kDevCapacity) return fail(ctx, GD_ERR_CAPACITY, "a device-side buffer was too small");
  if (h == kDevRange)
    return fail(ctx, GD_ERR_INVALID_ARG,
                "an FP32 energy partial left the fixed-point range (2^24 kcal/mol per segment): use the FP64 form");
  if (h > kDevBoundsBase)
    return fail(ctx, GD_ERR_CUDA, "device index check failed at site " + std::to_string(h - kDevBoundsBase) +
                                      " (debug library)");
  return fail(ctx, GD_ERR_CUDA, "device error code " + std::to_string(h));
}

// Smallest double x with sqrt(x) >= c: then sqrt(d2) < c  <=>  d2 < x.
static double thr_lt(double c) {
  double x = c * c;
  while (std::sqrt(x) >= c) x = std::nextafter(x, 0.0);
  while (!(std::sqrt(x) >= c)) x = std::nextafter(x, INFINITY);
  return x;
}
// Largest double x with sqrt(x) <= c: then sqrt(d2) <= c <=> d2 <= x, and
// sqrt(d2) > c <=> d2 > x.
static double thr_le(double c) {
  double x = c * c;
  while (std::sqrt(x) <= c) x = std::nextafter(x, INFINITY);
  while (std::sqrt(x) > c) x = std::nextafter(x, 0.0);
  return x;
}

// Cutoffs of src/constants.rs:59-63 and the clustering contact distance.
Thresholds make_thresholds(double contact_cutoff) {
  Thresholds t;
  t.vdw_lt = thr_lt(12.0);
  t.elec_gt = thr_le(1.0);
  t.elec_lt = thr_lt(15.0);
  t.desolv_lt = thr_lt(8.0);
  t.contact_le = thr_le(contact_cutoff);
  return t;
}

// Frame of one pose: the cosines/sines the reference evaluates per atom, and
// the composite matrix entries in its operation order (src/structure.rs:96-103).
void make_frame(const double *g, gd_pose_frame *f) {
  const double ca = std::cos(g[0]), sa = std::sin(g[0]);
  const double cb = std::cos(g[1]), sb = std::sin(g[1]);
  const double cg = std::cos(g[2]), sg = std::sin(g[2]);
  f->ca = ca;
  f->sa = sa;
  f->cb = cb;
  f->sb = sb;
  f->cg = cg;
  f->sg = sg;
  f->m01 = -sa * cg + ca * sb * sg;
  f->m02 = sa * sg + ca * sb * cg;
  f->m11 = ca * cg + sa * sb * sg;
  f->m12 = -ca * sg + sa * sb * cg;
  f->dx = g[3];
  f->dy = g[4];
  f->dz = g[5];
  f->pad[0] = f->pad[1] = f->pad[2] = 0.0;
}

// Half-widths of the FP32 guard bands on d2.  The FP32 coordinates carry at
// most M*2^-24 rounding (M bounds |x - O|); for a pair at distance c the
// computed d2 is then off by at most ~2c*sqrt(3)*(2M*2^-24 + c*2^-24) +
// 4c^2*2^-24.  Four times that is the band.
void guard_widths(const gd_complex *cx, double max_disp, float *gv, float *ge, float *gdd) {
  const double u = std::ldexp(1.0, -24);
  const double lig = std::max({std::fabs(cx->cx - cx->ox), std::fabs(cx->cy - cx->oy), std::fabs(cx->cz - cx->oz)}) +
                     cx->lig_radius + max_disp;
  const double M = std::max(cx->rec_extent, lig) + 1.0;
  auto band = [&](double c) {
    const double err = 2.0 * c * std::sqrt(3.0) * (2.0 * M * u + c * u) + 4.0 * c * c * u;
    return static_cast<float>(4.0 * err + 1e-6);
  };
  *gv = band(12.0);
  *ge = band(15.0);
  *gdd = band(8.0);
}

static double asp_of(uint8_t e) {  // src/fitness.rs:129-138
  switch (e) {
    case GD_ELEM_C: return 0.012;
    case GD_ELEM_N: return -0.160;
    case GD_ELEM_O: return -0.160;
    case GD_ELEM_S: return 0.012;
    default: return 0.0;
  }
}

// Energy contribution of one atom at burial counts 0..10: the reference's
// `energy -= asp * burial * r * r * 4.0 * PI` (src/fitness.rs:141-181).
static void desolv_row(uint8_t elem, double r, double *row) {
  const double asp = asp_of(elem);
  for (int c = 0; c <= 10; ++c) {
    if (std::fabs(asp) < 0.001) {
      row[c] = 0.0;
      continue;
    }
    double burial = static_cast<double>(c) / 10.0;
    if (!(burial < 1.0)) burial = 1.0;
    const double term = asp * burial * r * r * 4.0 * 3.141592653589793;
    row[c] = -term;
  }
}

static double powi6(double x) {
  const double x2 = x * x;
  const double x4 = x2 * x2;
  return x2 * x4;
}

static bool atoms_ok(const gd_atoms *a) {
  if (!a || a->n < 0) return false;
  if (a->n == 0) return true;
  return a->x && a->y && a->z && a->epsilon && a->rmin2 && a->charge && a->vdw_radius && a->serial && a->resseq &&
         a->chain && a->element && a->is_ca;
}

// All device arrays of a complex in one allocation and one copy (admitting a
// docking job costs one cudaMalloc and one cudaMemcpy, not one per array).
struct UploadPack {
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
  gd_status commit(gd_complex *cx) {
    void *p = nullptr;
    gd_status s = dev_alloc(cx->ctx, total, &p);
    if (s != GD_OK) return s;
    cx->allocs.push_back(p);
    cx->bytes += total;
    std::vector<char> h(total, 0);
    for (const Item &it : items)
      if (it.bytes) std::memcpy(h.data() + it.off, it.src, it.bytes);
    const cudaError_t e = cudaMemcpy(p, h.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(cx->ctx, e, "cudaMemcpy (complex upload)");
    for (const Item &it : items) it.bind(static_cast<char *>(p));
    return GD_OK;
  }
};

// Ligand atoms grouped into spatially compact runs of 32 (one FP32 scoring
// slot each): repeatedly take the remaining atom farthest from the remaining
// atoms' centroid and its 31 nearest remaining atoms.  The ligand is rigid, so
// tight groups keep their small bounding spheres in every pose and the
// kernel's row test drops more rows.  Deterministic (ties by index).
// Returns order[k] = original index of the atom at slot position k.
static std::vector<int> slot_order(const double *x, const double *y, const double *z, int n) {
  std::vector<int> order;
  order.reserve(n);
  if (n > 65536) {  // quadratic grouping: keep chain order for very large ligands
    for (int j = 0; j < n; ++j) order.push_back(j);
    return order;
  }
  std::vector<int> rest(n);
  for (int j = 0; j < n; ++j) rest[j] = j;
  std::vector<char> taken(n, 0);
  std::vector<std::pair<double, int>> d;
  d.reserve(n);
  while (!rest.empty()) {
    double c[3] = {0, 0, 0};
    for (int j : rest) {
      c[0] += x[j];
      c[1] += y[j];
      c[2] += z[j];
    }
    for (double &v : c) v /= static_cast<double>(rest.size());
    int far = rest[0];
    double best = -1.0;
    for (int j : rest) {
      const double dx = x[j] - c[0], dy = y[j] - c[1], dz = z[j] - c[2];
      const double e = dx * dx + dy * dy + dz * dz;
      if (e > best) {
        best = e;
        far = j;
      }
    }
    d.clear();
    for (int j : rest) {
      const double dx = x[j] - x[far], dy = y[j] - y[far], dz = z[j] - z[far];
      d.emplace_back(dx * dx + dy * dy + dz * dz, j);
    }
    const size_t take = std::min<size_t>(32, d.size());
    std::nth_element(d.begin(), d.begin() + (take - 1), d.end());
    const size_t o0 = order.size();
    for (size_t k = 0; k < take; ++k) {
      order.push_back(d[k].second);
      taken[d[k].second] = 1;
    }
    std::sort(order.begin() + o0, order.end());
    size_t w = 0;
    for (int j : rest)
      if (!taken[j]) rest[w++] = j;
    rest.resize(w);
  }
  return order;
}

// Receptor atoms grouped into spatially compact segments of kRecSeg (the FP32
// kernel's ring stage): recursive bisection along the longest extent of the
// bounding box, the left part always a whole number of segments, so every
// segment but the last is full; inside a segment the bisection goes on down
// to compact runs of 8 (one row-test round).  Deterministic (a stable sort
// per level).  Returns order[k] = original index of the atom at position k.
static std::vector<int> segment_order(const double *x, const double *y, const double *z, int n) {
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  struct Span { int lo, hi, unit; };
  std::vector<Span> pending{{0, n, kRecSeg}};
  while (!pending.empty()) {
    const Span sp = pending.back();
    pending.pop_back();
    const int m = sp.hi - sp.lo;
    if (m <= sp.unit) {
      if (sp.unit > 8 && m > 8) pending.push_back({sp.lo, sp.hi, 8});
      continue;
    }
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = sp.lo; k < sp.hi; ++k) {
      const double v[3] = {x[order[k]], y[order[k]], z[order[k]]};
      for (int a = 0; a < 3; ++a) lo[a] = std::min(lo[a], v[a]), hi[a] = std::max(hi[a], v[a]);
    }
    int ax = 0;
    for (int a = 1; a < 3; ++a)
      if (hi[a] - lo[a] > hi[ax] - lo[ax]) ax = a;
    const double *c = ax == 0 ? x : (ax == 1 ? y : z);
    std::stable_sort(order.begin() + sp.lo, order.begin() + sp.hi, [c](int a, int b) { return c[a] < c[b]; });
    const int nseg = (m + sp.unit - 1) / sp.unit;
    const int mid = sp.lo + (nseg / 2) * sp.unit;
    pending.push_back({mid, sp.hi, sp.unit});
    pending.push_back({sp.lo, mid, sp.unit});
  }
  return order;
}

}  // namespace gd

// The centre starts at the centroid and moves toward the farthest point with
// steps 1/(i + 1) (Badoiu and Clarkson's iteration for the minimum enclosing
// ball); the centre with the smallest farthest-point distance seen is kept,
// with that distance as the radius, so the ball encloses every point whatever
// the iteration reached.  Sixteen steps bring clusters of protein atoms within
// about 1 % of the minimum radius, about 10 % below the centroid's sphere.
void gd::enclosing_ball(const double *x, const double *y, const double *z, const int *idx, int n, double c[3],
                        double &r) {
  c[0] = c[1] = c[2] = 0.0;
  r = 0.0;
  if (n <= 0) return;
  auto at = [&](int k) { return idx ? idx[k] : k; };
  double m[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < n; ++k) {
    m[0] += x[at(k)];
    m[1] += y[at(k)];
    m[2] += z[at(k)];
  }
  for (double &v : m) v /= n;
  double best = -1.0;
  for (int i = 1; i <= 16; ++i) {
    int f = at(0);
    double d2max = -1.0;
    for (int k = 0; k < n; ++k) {
      const int j = at(k);
      const double d2 = (x[j] - m[0]) * (x[j] - m[0]) + (y[j] - m[1]) * (y[j] - m[1]) + (z[j] - m[2]) * (z[j] - m[2]);
      if (d2 > d2max) {
        d2max = d2;
        f = j;
      }
    }
    if (best < 0.0 || d2max < best) {
      best = d2max;
      c[0] = m[0];
      c[1] = m[1];
      c[2] = m[2];
    }
    if (n == 1) break;
    const double step = 1.0 / (i + 1);
    m[0] += (x[f] - m[0]) * step;
    m[1] += (y[f] - m[1]) * step;
    m[2] += (z[f] - m[2]) * step;
  }
  r = std::sqrt(best);
}

namespace gd {

static void centroid(const double *x, const double *y, const double *z, int n, double *c) {
  double sx = -0.0, sy = -0.0, sz = -0.0;  // left folds, as Molecule::center_of_mass
  for (int i = 0; i < n; ++i) sx += x[i];
  for (int i = 0; i < n; ++i) sy += y[i];
  for (int i = 0; i < n; ++i) sz += z[i];
  c[0] = sx / n;
  c[1] = sy / n;
  c[2] = sz / n;
}

}  // namespace gd

using namespace gd;

extern "C" {

int32_t gd_abi_version(void) { return GD_ABI_VERSION; }

const char *gd_status_string(gd_status s) {
  switch (s) {
    case GD_OK: return "ok";
    case GD_ERR_INVALID_ARG: return "invalid argument";
    case GD_ERR_OOM: return "out of device memory";
    case GD_ERR_CUDA: return "CUDA error";
    case GD_ERR_TIMEOUT: return "device wait timed out";
    case GD_ERR_CAPACITY: return "output capacity too small";
    case GD_ERR_STATE: return "invalid state";
  }
  return "unknown status";
}

gd_status gd_context_create(int32_t device, uint64_t hbm_budget_bytes, gd_context **out) {
  if (!out) return GD_ERR_INVALID_ARG;
  *out = nullptr;
  gd_context *ctx = new (std::nothrow) gd_context();
  if (!ctx) return GD_ERR_OOM;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || device < 0 || device >= ndev) {
    delete ctx;
    return e != cudaSuccess ? GD_ERR_CUDA : GD_ERR_INVALID_ARG;
  }
  ctx->device = device;
  ctx->budget = hbm_budget_bytes;
  if ((e = cudaSetDevice(device)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&ctx->ev0)) != cudaSuccess || (e = cudaEventCreate(&ctx->ev1)) != cudaSuccess) {
    delete ctx;
    return GD_ERR_CUDA;
  }
  void *p = nullptr;
  if (dev_alloc(ctx, sizeof(int), &p) != GD_OK) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GD_ERR_OOM;
  }
  ctx->d_err = static_cast<int *>(p);
  cudaMemset(ctx->d_err, 0, sizeof(int));
  *out = ctx;
  return GD_OK;
}

gd_status gd_context_destroy(gd_context *ctx) {
  if (!ctx) return GD_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->d_scratch) cudaFree(ctx->d_scratch);
  if (ctx->d_batch) cudaFree(ctx->d_batch);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GD_OK;
}

const char *gd_last_error(const gd_context *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

gd_status gd_context_set_tuning(gd_context *ctx, int32_t knob, int32_t value) {
  if (!ctx) return GD_ERR_INVALID_ARG;
  if (knob == GD_TUNE_F32_SLOTS) {
    static const int kValid[] = {0, 4, 16 + 4, 64 + 2, 64 + 4, 256 + 64 + 2, 256 + 64 + 4};
    bool ok = false;
    for (int v : kValid) ok = ok || v == value;
    if (!ok)
      return fail(ctx, GD_ERR_INVALID_ARG,
                  "F32 tuning: one of 4, 20, 66, 68, 322, 324 (ligand slots per lane + 16 or 64 for two or "
                  "four receptor rows per step, + 256 for the five-CTA register cap)");
    ctx->tune_f32_slots = value;
    return GD_OK;
  }
  if (knob == GD_TUNE_SPLIT) {
    if (value < 0 || value > 2) return fail(ctx, GD_ERR_INVALID_ARG, "split tuning: 0 (automatic), 1 (never), 2 (always)");
    ctx->tune_split = value;
    return GD_OK;
  }
  if (knob == GD_TUNE_FAULT) {
    if (value < 0 || value > 1) return fail(ctx, GD_ERR_INVALID_ARG, "fault knob: 0 (off) or 1 (drop one stage copy)");
    ctx->tune_fault = value;
    return GD_OK;
  }
  if (knob == GD_TUNE_FCC) {
    if (value < 0 || value > 2)
      return fail(ctx, GD_ERR_INVALID_ARG, "FCC tuning: 0 (automatic), 1 (bitsets), 2 (contact postings)");
    ctx->tune_fcc = value;
    return GD_OK;
  }
  if (knob == GD_TUNE_CONTACTS) {
    if (value < 0 || value > 1)
      return fail(ctx, GD_ERR_INVALID_ARG, "contacts tuning: 0 (automatic), 1 (per-residue lists)");
    ctx->tune_contacts = value;
    return GD_OK;
  }
  if (knob == GD_TUNE_RPARTS) {
    if (value < 0 || value > 8)
      return fail(ctx, GD_ERR_INVALID_ARG, "receptor-parts tuning: 0 (automatic) or 1..8 parts per ligand chunk");
    ctx->tune_rparts = value;
    return GD_OK;
  }
  if (knob == GD_INFO_LAST_FCC || knob == GD_INFO_LAST_CONTACTS)
    return fail(ctx, GD_ERR_INVALID_ARG, "read-only knob");
  return fail(ctx, GD_ERR_INVALID_ARG, "unknown tuning knob");
}

int32_t gd_context_get_tuning(const gd_context *ctx, int32_t knob) {
  if (!ctx) return -1;
  if (knob == GD_TUNE_F32_SLOTS) return ctx->tune_f32_slots;
  if (knob == GD_TUNE_SPLIT) return ctx->tune_split;
  if (knob == GD_TUNE_FAULT) return ctx->tune_fault;
  if (knob == GD_TUNE_FCC) return ctx->tune_fcc;
  if (knob == GD_TUNE_CONTACTS) return ctx->tune_contacts;
  if (knob == GD_TUNE_RPARTS) return ctx->tune_rparts;
  if (knob == GD_INFO_LAST_FCC) return ctx->last_fcc;
  if (knob == GD_INFO_LAST_CONTACTS) return ctx->last_contacts;
  return -1;
}

uint64_t gd_context_bytes_in_use(const gd_context *ctx) { return ctx ? ctx->in_use : 0; }

gd_status gd_complex_create(gd_context *ctx, const gd_atoms *rec, const gd_atoms *lig, const int32_t *restraint_pairs,
                            int32_t n_pairs, const gd_weights *w, gd_complex **out) {
  gd::NvtxRange nvtx_range("gd_complex_create");
  if (!ctx || !out) return GD_ERR_INVALID_ARG;
  *out = nullptr;
  if (!atoms_ok(rec) || !atoms_ok(lig)) return fail(ctx, GD_ERR_INVALID_ARG, "receptor/ligand arrays incomplete");
  if (n_pairs < 0 || (n_pairs > 0 && !restraint_pairs)) return fail(ctx, GD_ERR_INVALID_ARG, "bad restraint pairs");
  cudaSetDevice(ctx->device);
  gd_complex *cx = new (std::nothrow) gd_complex();
  if (!cx) return fail(ctx, GD_ERR_OOM, "host allocation");
  cx->ctx = ctx;
  cx->nr = rec->n;
  cx->nl = lig->n;
  cx->w = w ? *w : gd_weights{0.4, 0.05, 3.4, 1.0};

  // atom types: distinct (epsilon, Rmin/2) pairs over both molecules
  std::map<std::pair<uint64_t, uint64_t>, int> types;
  std::vector<double> t_eps, t_rmin;
  auto type_of = [&](double e, double r) {
    uint64_t be, br;
    std::memcpy(&be, &e, 8);
    std::memcpy(&br, &r, 8);
    auto it = types.find({be, br});
    if (it != types.end()) return it->second;
    const int id = static_cast<int>(t_eps.size());
    types[{be, br}] = id;
    t_eps.push_back(e);
    t_rmin.push_back(r);
    return id;
  };
  std::vector<int> rtype(rec->n), ltype(lig->n);
  for (int i = 0; i < rec->n; ++i) rtype[i] = type_of(rec->epsilon[i], rec->rmin2[i]);
  for (int j = 0; j < lig->n; ++j) ltype[j] = type_of(lig->epsilon[j], lig->rmin2[j]);
  if (t_eps.empty()) type_of(0.0, 0.0);
  const int nt = static_cast<int>(t_eps.size());
  if (nt > kMaxTypes) {
    delete cx;
    return fail(ctx, GD_ERR_INVALID_ARG, "more than 64 distinct (epsilon, rmin2) atom types");
  }
  cx->nt = nt;
  std::vector<TypePair32> tab32(static_cast<size_t>(nt) * nt);
  std::vector<TypePair64> tab64(static_cast<size_t>(nt) * nt);
  for (int a = 0; a < nt; ++a)
    for (int b = 0; b < nt; ++b) {
      // softcore_lj_potential's per-pair constants (src/fitness.rs:58-63)
      const double eps = std::sqrt(t_eps[a] * t_eps[b]);
      const double r6 = powi6(t_rmin[a] + t_rmin[b]);
      tab64[a * nt + b] = TypePair64{r6, 0.5 * r6, eps, 0.0};
      const double inv2 = r6 > 0.0 ? 2.0 / r6 : 0.0;
      tab32[a * nt + b] = TypePair32{r6 > 0.0 && inv2 < FLT_MAX ? static_cast<float>(inv2) : FLT_MAX,
                                     static_cast<float>(4.0 * eps)};
      if (eps > 50.0) cx->need_clamp = true;
    }

  double c[3] = {0, 0, 0};
  if (lig->n > 0) centroid(lig->x, lig->y, lig->z, lig->n, c);
  cx->cx = c[0];
  cx->cy = c[1];
  cx->cz = c[2];
  double o[3] = {c[0], c[1], c[2]};
  if (rec->n > 0) centroid(rec->x, rec->y, rec->z, rec->n, o);
  cx->ox = o[0];
  cx->oy = o[1];
  cx->oz = o[2];

  // receptor, padded to whole tiles
  cx->nr_pad = ((rec->n + kTile - 1) / kTile) * kTile;
  std::vector<float4> rp32(cx->nr_pad, make_float4(1e9f, 1e9f, 1e9f, 0.f));
  std::vector<D4> rp64(cx->nr_pad, D4{1e30, 1e30, 1e30, 0.0});
  std::vector<int2> rmeta(cx->nr_pad, make_int2(0, 0));
  std::vector<int4> rmeta16(cx->nr_pad, make_int4(0, 0, 0, 0));
  std::vector<double> rdes(static_cast<size_t>(std::max(rec->n, 1)) * 11, 0.0);
  double ext = 0.0;
  // receptor in compact segments (sums are order-free; the burial tables
  // follow the same order)
  const std::vector<int> rperm = segment_order(rec->x, rec->y, rec->z, rec->n);
  for (int k = 0; k < rec->n; ++k) {
    const int i = rperm[k];
    rp32[k] = make_float4(static_cast<float>(rec->x[i] - o[0]), static_cast<float>(rec->y[i] - o[1]),
                          static_cast<float>(rec->z[i] - o[2]), static_cast<float>(332.0636 * rec->charge[i]));
    rp64[k] = D4{rec->x[i], rec->y[i], rec->z[i], rec->charge[i]};
    rmeta[k] = make_int2(rtype[i] * nt, rec->serial[i]);
    rmeta16[k] = make_int4(rtype[i] * nt, rec->serial[i], 0, 0);
    desolv_row(rec->element[i], rec->vdw_radius[i], &rdes[static_cast<size_t>(k) * 11]);
    ext = std::max({ext, std::fabs(rec->x[i] - o[0]), std::fabs(rec->y[i] - o[1]), std::fabs(rec->z[i] - o[2])});
  }
  cx->rec_extent = ext;
  // bounding sphere of each segment (FP32, relative to O)
  cx->nseg = (rec->n + kRecSeg - 1) / kRecSeg;
  std::vector<float4> rseg(std::max(cx->nseg, 1), make_float4(0.f, 0.f, 0.f, -1.f));
  for (int g = 0; g < cx->nseg; ++g) {
    // widened so that the FP32 images of the atoms and of the centre stay inside
    const int k0 = g * kRecSeg, k1 = std::min(rec->n, (g + 1) * kRecSeg);
    double cs[3], r;
    enclosing_ball(rec->x, rec->y, rec->z, rperm.data() + k0, k1 - k0, cs, r);
    rseg[g] = make_float4(static_cast<float>(cs[0] - o[0]), static_cast<float>(cs[1] - o[1]),
                          static_cast<float>(cs[2] - o[2]), static_cast<float>(r * (1.0 + 1e-6) + 0.01));
  }
  // ligand on the device in slot order (sums are order-free; restraint and
  // model indices go through the permutation)
  const std::vector<int> perm = slot_order(lig->x, lig->y, lig->z, lig->n);
  std::vector<int> inv(lig->n);
  std::vector<double> lx(lig->n), ly(lig->n), lz(lig->n), lq(lig->n);
  std::vector<int> lser(lig->n), ltp(lig->n);
  std::vector<double> ldes(static_cast<size_t>(std::max(lig->n, 1)) * 11, 0.0);
  double rad = 0.0;
  for (int k = 0; k < lig->n; ++k) {
    const int j = perm[k];
    inv[j] = k;
    lx[k] = lig->x[j];
    ly[k] = lig->y[j];
    lz[k] = lig->z[j];
    lq[k] = lig->charge[j];
    lser[k] = lig->serial[j];
    ltp[k] = ltype[j];
    desolv_row(lig->element[j], lig->vdw_radius[j], &ldes[static_cast<size_t>(k) * 11]);
    const double dx = lig->x[j] - c[0], dy = lig->y[j] - c[1], dz = lig->z[j] - c[2];
    rad = std::max(rad, std::sqrt(dx * dx + dy * dy + dz * dz));
  }
  cx->lig_radius = rad;
  // bounding sphere of each 32-atom slot in the positioned frame: a pose moves
  // it rigidly, so its transformed centre and the same radius bound the
  // slot's atoms in every pose
  std::vector<D4> lslot(std::max((lig->n + 31) / 32, 1), D4{0.0, 0.0, 0.0, -1.0});
  for (int s0 = 0; s0 < lig->n; s0 += 32) {
    const int s1 = std::min(lig->n, s0 + 32);
    double cs[3], r;
    enclosing_ball(lx.data() + s0, ly.data() + s0, lz.data() + s0, nullptr, s1 - s0, cs, r);
    lslot[s0 / 32] = D4{cs[0], cs[1], cs[2], r * (1.0 + 1e-6) + 0.01};
  }
  {
    // equal receptor/ligand serials (vdW pairs skipped): disjoint serial
    // ranges, the usual case, settle it without a search
    int32_t rlo = INT32_MAX, rhi = INT32_MIN, llo = INT32_MAX, lhi = INT32_MIN;
    for (int i = 0; i < rec->n; ++i) rlo = std::min(rlo, rec->serial[i]), rhi = std::max(rhi, rec->serial[i]);
    for (int j = 0; j < lig->n; ++j) llo = std::min(llo, lig->serial[j]), lhi = std::max(lhi, lig->serial[j]);
    if (rec->n > 0 && lig->n > 0 && rlo <= lhi && llo <= rhi) {
      std::vector<int32_t> rs(rec->serial, rec->serial + rec->n);
      std::sort(rs.begin(), rs.end());
      for (int j = 0; j < lig->n && !cx->serial_overlap; ++j)
        cx->serial_overlap = std::binary_search(rs.begin(), rs.end(), lig->serial[j]);
    }
  }

  // restraints: first CA with each residue number (src/restraints.rs:44-77)
  std::vector<D4> rr;
  std::vector<int> rl;
  auto first_ca = [](const gd_atoms *m, int32_t res) {
    for (int i = 0; i < m->n; ++i)
      if (m->is_ca[i] && static_cast<int32_t>(m->resseq[i]) == res) return i;
    return -1;
  };
  for (int k = 0; k < n_pairs; ++k) {
    const int a = first_ca(rec, restraint_pairs[2 * k]);
    const int b = first_ca(lig, restraint_pairs[2 * k + 1]);
    if (a >= 0 && b >= 0) {
      rr.push_back(D4{rec->x[a], rec->y[a], rec->z[a], 0.0});
      rl.push_back(inv[b]);
    }
  }
  cx->K = static_cast<int>(rl.size());

  gd_status s;
  UploadPack pack;
  pack.add(rp32, &cx->rec_pos32);
  pack.add(rp64, &cx->rec_pos64);
  pack.add(rmeta, &cx->rec_meta);
  pack.add(rmeta16, &cx->rec_meta16);
  pack.add(rdes, &cx->rec_desolv);
  pack.add(lx, &cx->lig_x);
  pack.add(ly, &cx->lig_y);
  pack.add(lz, &cx->lig_z);
  pack.add(lq, &cx->lig_q);
  pack.add(ltp, &cx->lig_type);
  pack.add(lser, &cx->lig_serial);
  pack.add(ldes, &cx->lig_desolv);
  pack.add(tab32, &cx->tab32);
  pack.add(tab64, &cx->tab64);
  pack.add(rr, &cx->restr_rec);
  pack.add(rl, &cx->restr_lig);
  pack.add(perm, &cx->lig_perm);
  pack.add(rseg, &cx->rec_seg);
  pack.add(lslot, &cx->lig_slot_sph);
  if ((s = pack.commit(cx)) != GD_OK) {
    gd_complex_destroy(cx);
    return s;
  }
  // host copies for clustering
  cx->h_rx.assign(rec->x, rec->x + rec->n);
  cx->h_ry.assign(rec->y, rec->y + rec->n);
  cx->h_rz.assign(rec->z, rec->z + rec->n);
  cx->h_lx.assign(lig->x, lig->x + lig->n);
  cx->h_ly.assign(lig->y, lig->y + lig->n);
  cx->h_lz.assign(lig->z, lig->z + lig->n);
  cx->h_rchain.assign(rec->chain, rec->chain + rec->n);
  cx->h_lchain.assign(lig->chain, lig->chain + lig->n);
  cx->h_relem.assign(rec->element, rec->element + rec->n);
  cx->h_lelem.assign(lig->element, lig->element + lig->n);
  cx->h_rres.assign(rec->resseq, rec->resseq + rec->n);
  cx->h_lres.assign(lig->resseq, lig->resseq + lig->n);
  cx->h_lig_slot = inv;
  *out = cx;
  return GD_OK;
}

gd_status gd_complex_destroy(gd_complex *cx) {
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_cluster_cache(cx);
  for (void *p : cx->allocs) cudaFree(p);
  ctx->in_use -= std::min<uint64_t>(ctx->in_use, cx->bytes);
  delete cx;
  return GD_OK;
}

int32_t gd_complex_num_restraints(const gd_complex *cx) { return cx ? cx->K : -1; }

gd_status gd_complex_set_weights(gd_complex *cx, const gd_weights *w) {
  if (!cx || !w) return GD_ERR_INVALID_ARG;
  cx->w = *w;
  return GD_OK;
}

// Host worker threads kept across calls: starting 16 threads costs more than
// building a large batch's frames on them, and gdock builds frames every
// generation.  run(k, f) calls f(0..k-1) on the workers and the calling
// thread and returns when all are done; callers are serialised.  The pool is
// never destroyed (its threads end with the process), and a process forked
// after it was made builds its own (a child has none of the parent's
// threads).
class HostPool {
 public:
  static HostPool &get() {
    static std::mutex mu;
    static HostPool *pool = nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (!pool || pool->pid_ != getpid()) pool = new HostPool();  // a forked child's pool replaces the parent's
    return *pool;
  }
  int size() const { return static_cast<int>(workers_.size()) + 1; }
  void run(int k, const std::function<void(int)> &f) {
    std::lock_guard<std::mutex> caller(run_mu_);
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &f;
      tasks_ = k;
      next_ = 0;
      done_ = 0;
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return done_ == tasks_; });
    fn_ = nullptr;
  }

 private:
  HostPool() : pid_(getpid()) {
    const int n = static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency()))) - 1;
    for (int i = 0; i < n; ++i)
      workers_.emplace_back([this] {
        long long seen = 0;
        for (;;) {
          {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return gen_ != seen; });
            seen = gen_;
          }
          work();
        }
      });
    for (auto &w : workers_) w.detach();
  }
  // take tasks until none is left
  void work() {
    for (;;) {
      int t;
      const std::function<void(int)> *f;
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (!fn_ || next_ >= tasks_) return;
        t = next_++;
        f = fn_;
      }
      (*f)(t);
      std::lock_guard<std::mutex> lk(mu_);
      if (++done_ == tasks_) done_cv_.notify_all();
    }
  }
  pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex mu_, run_mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)> *fn_ = nullptr;
  int tasks_ = 0, next_ = 0, done_ = 0;
  long long gen_ = 0;
};

// Frames of n poses, on the host pool from 4,096 poses, and the largest
// |displacement| component among them (sizes the FP32 guard bands).
static void frames_and_max_disp(const double *genes, int n, gd_pose_frame *frames, double *max_disp) {
  const int nt = n >= 4096 ? 64 : 1;  // contiguous ranges of poses
  std::vector<double> m(nt, 0.0);
  auto work = [&](int t) {
    const int i0 = static_cast<int>(static_cast<long long>(n) * t / nt),
              i1 = static_cast<int>(static_cast<long long>(n) * (t + 1) / nt);
    double mt = 0.0;
    for (int i = i0; i < i1; ++i) {
      const double *g = genes + 6 * static_cast<size_t>(i);
      make_frame(g, frames + i);
      mt = std::max({mt, std::fabs(g[3]), std::fabs(g[4]), std::fabs(g[5])});
    }
    m[t] = mt;
  };
  if (nt == 1) {
    work(0);
  } else {
    HostPool::get().run(nt, work);
  }
  if (max_disp) *max_disp = *std::max_element(m.begin(), m.end());
}

// memcpy on the host pool for copies of 1 MiB or more (a large scoring
// call's results out of the pinned staging buffer)
static void copy_out(void *dst, const void *src, size_t bytes) {
  if (bytes < (size_t(1) << 20)) {
    std::memcpy(dst, src, bytes);
    return;
  }
  const int nt = 16;
  HostPool::get().run(nt, [&](int t) {
    const size_t b0 = bytes * t / nt, b1 = bytes * (t + 1) / nt;
    std::memcpy(static_cast<char *>(dst) + b0, static_cast<const char *>(src) + b0, b1 - b0);
  });
}

gd_status gd_make_frames(const double *genes, int32_t n, gd_pose_frame *frames) {
  if (n < 0 || (n > 0 && (!genes || !frames))) return GD_ERR_INVALID_ARG;
  frames_and_max_disp(genes, n, frames, nullptr);
  return GD_OK;
}

gd_status gd_score_poses(gd_complex *cx, const double *genes, int32_t n, gd_precision prec, gd_pose_energy *out) {
  gd::NvtxRange nvtx_range("gd_score_poses");
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  if (n < 0 || (n > 0 && (!genes || !out))) return fail(ctx, GD_ERR_INVALID_ARG, "bad genes/out");
  if (prec != GD_PREC_F32 && prec != GD_PREC_F64) return fail(ctx, GD_ERR_INVALID_ARG, "bad precision");
  if (n == 0) return GD_OK;
  cudaSetDevice(ctx->device);
  const size_t fb = sizeof(gd_pose_frame) * n, ob = sizeof(gd_pose_energy) * n;
  gd_status s = ensure_scratch(ctx, fb + ob + 256, fb + ob + 256);
  if (s != GD_OK) return s;
  gd_pose_frame *h_frames = static_cast<gd_pose_frame *>(ctx->h_pinned);
  gd_pose_energy *h_out = reinterpret_cast<gd_pose_energy *>(static_cast<char *>(ctx->h_pinned) + ((fb + 255) / 256) * 256);
  gd_pose_frame *d_frames = static_cast<gd_pose_frame *>(ctx->d_scratch);
  gd_pose_energy *d_out = reinterpret_cast<gd_pose_energy *>(static_cast<char *>(ctx->d_scratch) + ((fb + 255) / 256) * 256);
  // phase times on stderr with GD_TRACE (host frames, launch set-up, device
  // work and copies, result copy)
  const bool tr = trace_on();
  auto t = std::chrono::steady_clock::now();
  auto lap = [&](const char *name) {
    if (!tr) return;
    const auto now = std::chrono::steady_clock::now();
    trace(name, std::chrono::duration<double>(now - t).count());
    t = now;
  };
  double maxd = 0.0;
  frames_and_max_disp(genes, n, h_frames, &maxd);
  lap("score_poses: frames (host)");
  cudaError_t e = cudaMemcpyAsync(d_frames, h_frames, fb, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "H2D frames");
  s = launch_score(cx, d_frames, nullptr, n, prec, d_out, ctx->stream, maxd);
  if (s != GD_OK) return s;
  e = cudaMemcpyAsync(h_out, d_out, ob, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "D2H energies");
  lap("score_poses: copies and launch issued");
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "score kernel");
  lap("score_poses: wait for the device");
  s = check_device_error(ctx);
  if (s != GD_OK) return s;
  copy_out(out, h_out, ob);
  lap("score_poses: error word and result copy");
  return GD_OK;
}

gd_status gd_score_frames_device(gd_complex *cx, const gd_pose_frame *d_frames, int32_t n, gd_precision prec,
                                 double max_displacement, gd_pose_energy *d_out, void *stream) {
  gd::NvtxRange nvtx_range("gd_score_frames_device");
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  if (n < 0 || (n > 0 && (!d_frames || !d_out))) return fail(ctx, GD_ERR_INVALID_ARG, "bad frames/out");
  if (prec != GD_PREC_F32 && prec != GD_PREC_F64) return fail(ctx, GD_ERR_INVALID_ARG, "bad precision");
  if (!(max_displacement >= 0.0)) return fail(ctx, GD_ERR_INVALID_ARG, "bad max_displacement");
  cudaSetDevice(ctx->device);
  return launch_score(cx, d_frames, nullptr, n, prec, d_out, stream ? static_cast<cudaStream_t>(stream) : ctx->stream,
                      max_displacement);
}

gd_status gd_autotune_f32(gd_complex *cx, const gd_pose_frame *d_frames, int32_t n, double max_displacement,
                          gd_pose_energy *d_out, void *stream, double *rates, int32_t *best) {
  gd::NvtxRange nvtx_range("gd_autotune_f32");
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  if (n <= 0 || !d_frames || !d_out) return fail(ctx, GD_ERR_INVALID_ARG, "bad frames/out");
  if (!(max_displacement >= 0.0)) return fail(ctx, GD_ERR_INVALID_ARG, "bad max_displacement");
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  // (GD_TUNE_F32_SLOTS, GD_TUNE_SPLIT): whole-pose variants, then the split kernel
  static const int kCand[GD_AUTOTUNE_CANDIDATES][2] = {{16 + 4, 1}, {64 + 2, 1}, {64 + 4, 1},
                                                       {256 + 64 + 2, 1}, {256 + 64 + 4, 1}, {kDefaultF32Tune, 2}};
  const int keep_tune = ctx->tune_f32_slots, keep_split = ctx->tune_split;
  int arg = -1;
  double top = -1.0;
  for (int c = 0; c < GD_AUTOTUNE_CANDIDATES; ++c) {
    ctx->tune_f32_slots = kCand[c][0];
    ctx->tune_split = kCand[c][1];
    gd_status s = launch_score(cx, d_frames, nullptr, n, GD_PREC_F32, d_out, st, max_displacement);
    cudaError_t e = cudaSuccess;
    if (s == GD_OK) e = cudaEventRecord(ctx->ev0, st);
    if (s == GD_OK && e == cudaSuccess) s = launch_score(cx, d_frames, nullptr, n, GD_PREC_F32, d_out, st, max_displacement);
    if (s == GD_OK && e == cudaSuccess) e = cudaEventRecord(ctx->ev1, st);
    if (s == GD_OK && e == cudaSuccess) e = cudaEventSynchronize(ctx->ev1);
    float ms = 0.0f;
    if (s == GD_OK && e == cudaSuccess) e = cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    if (s == GD_OK && e != cudaSuccess) s = cuda_fail(ctx, e, "autotune timing");
    if (s == GD_OK) s = check_device_error(ctx);
    if (s != GD_OK) {
      ctx->tune_f32_slots = keep_tune;
      ctx->tune_split = keep_split;
      return s;
    }
    const double r = ms > 0.0f ? n / (ms * 1e-3) : 0.0;
    if (rates) rates[c] = r;
    if (r > top) {
      top = r;
      arg = c;
    }
  }
  ctx->tune_f32_slots = kCand[arg][0];
  ctx->tune_split = kCand[arg][1];
  if (best) *best = arg;
  return GD_OK;
}

gd_status gd_sync(gd_context *ctx) {
  if (!ctx) return GD_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "device synchronize");
  return check_device_error(ctx);
}

gd_status gd_score_models(gd_complex *cx, const double *lig_xyz, int32_t n_models, gd_precision prec,
                          gd_pose_energy *out) {
  gd::NvtxRange nvtx_range("gd_score_models");
  if (!cx) return GD_ERR_INVALID_ARG;
  gd_context *ctx = cx->ctx;
  if (n_models < 0 || (n_models > 0 && (!lig_xyz || !out))) return fail(ctx, GD_ERR_INVALID_ARG, "bad models/out");
  if (prec != GD_PREC_F32 && prec != GD_PREC_F64) return fail(ctx, GD_ERR_INVALID_ARG, "bad precision");
  if (n_models == 0) return GD_OK;
  cudaSetDevice(ctx->device);
  const size_t mb = sizeof(double) * 3 * static_cast<size_t>(cx->nl) * n_models;
  const size_t ob = sizeof(gd_pose_energy) * n_models;
  const size_t mb_al = ((mb + 255) / 256) * 256;
  gd_status s = ensure_scratch(ctx, mb_al + ob, ob);
  if (s != GD_OK) return s;
  double *d_models = static_cast<double *>(ctx->d_scratch);
  gd_pose_energy *d_out = reinterpret_cast<gd_pose_energy *>(static_cast<char *>(ctx->d_scratch) + mb_al);
  // displacement bound: furthest model coordinate from the ligand centroid
  double m = 0.0;
  for (size_t i = 0; i < 3 * static_cast<size_t>(cx->nl) * n_models; i += 3)
    m = std::max({m, std::fabs(lig_xyz[i] - cx->cx), std::fabs(lig_xyz[i + 1] - cx->cy),
                  std::fabs(lig_xyz[i + 2] - cx->cz)});
  cudaError_t e = cudaMemcpyAsync(d_models, lig_xyz, mb, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "H2D models");
  s = launch_score(cx, nullptr, d_models, n_models, prec, d_out, ctx->stream, m);
  if (s != GD_OK) return s;
  gd_pose_energy *h_out = static_cast<gd_pose_energy *>(ctx->h_pinned);
  e = cudaMemcpyAsync(h_out, d_out, ob, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "D2H energies");
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "score kernel");
  s = check_device_error(ctx);
  if (s != GD_OK) return s;
  copy_out(out, h_out, ob);
  return GD_OK;
}

}  // extern "C"
