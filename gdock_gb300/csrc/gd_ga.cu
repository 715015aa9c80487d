// Device-resident genetic algorithm: gdock's generation loop
// (src/commands/run.rs:381-531) with Population::evolve (src/population.rs:74-121)
// on the GPU, for one or many docking jobs at once.
//
// Randomness.  The number and order of random draws of a generation do not
// depend on fitness (3n tournament indices, the shuffle, 6 uniforms per
// crossover pair, 6 uniforms per mutated individual plus one normal sample
// where a uniform triggers), so the host draws them up front in the
// reference's order from a seeded generator and uploads them; the device then
// applies them to whatever individuals fitness selects.  The generator is
// xoshiro256** seeded through SplitMix64 (Blackman & Vigna; Steele, Lea &
// Flood), uniforms are 53-bit, normals are Box-Muller; gdock's own stream
// (rand's StdRng) is not reproduced.
//
// Per generation, for all jobs: pose frames from genes (device sin/cos),
// batched scoring (the persistent FP32 kernel, or the plain FP64 kernel per
// job), optionally the DockQ metrics of every pose (gd_eval.cu), then one CTA
// per job runs the convergence bookkeeping of the reference loop, the Hall
// of Fame (src/commands/run.rs:75-215,385) and, unless the job stopped,
// evolve.  One generation is captured as a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gd_device.cuh"

namespace gd {
namespace {

// ------------------------------------------------------------ host RNG ----

struct Rng {
  uint64_t s[4];
  static uint64_t splitmix(uint64_t &x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto &v : s) v = splitmix(x);
  }
  static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }  // [0, 1)
  int range(int n) {                                                           // [0, n)
    const int v = static_cast<int>(uniform() * n);
    return v < n ? v : n - 1;
  }
  double normal() {  // Box-Muller, one value per call
    const double u1 = 1.0 - uniform(), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

// Random inputs of one generation of one job, in consumption order.
struct GenDraws {
  std::vector<int> tour, perm;
  std::vector<double> cross_u, mut_u, mut_z;
};

void draw_generation(Rng &rng, const gd_ga_cfg &c, GenDraws &d) {
  const int n = c.pop_size, m = 2 * (n / 2);
  d.tour.resize(static_cast<size_t>(c.tournament_size) * n);
  for (auto &t : d.tour) t = rng.range(n);  // tournament_selection (src/population.rs:135-142)
  d.perm.resize(n);
  for (int k = 0; k < n; ++k) d.perm[k] = k;
  for (int i = n - 1; i >= 1; --i) std::swap(d.perm[i], d.perm[rng.range(i + 1)]);  // shuffle (:88)
  d.cross_u.resize(static_cast<size_t>(6) * (n / 2));
  for (auto &u : d.cross_u) u = rng.uniform();  // ga::crossover (src/ga.rs:19-31)
  d.mut_u.resize(static_cast<size_t>(6) * m);
  d.mut_z.resize(static_cast<size_t>(6) * m);
  for (int k = 0; k < m; ++k)  // Chromosome::mutate (src/chromosome.rs:61-76)
    for (int g = 0; g < 6; ++g) {
      const double u = rng.uniform();
      d.mut_u[6 * k + g] = u;
      d.mut_z[6 * k + g] = u <= c.mutation_rate ? (g < 3 ? c.rot_sigma : c.trans_sigma) * rng.normal() : 0.0;
    }
}

// Chromosome::new (src/chromosome.rs:27-34): angles in [0, 2pi], displacement in [-M, M]
void draw_initial(Rng &rng, const gd_ga_cfg &c, double *genes) {
  for (int k = 0; k < c.pop_size; ++k) {
    for (int g = 0; g < 3; ++g) genes[6 * k + g] = 6.283185307179586 * rng.uniform();
    for (int g = 3; g < 6; ++g) genes[6 * k + g] = -c.max_displacement + 2.0 * c.max_displacement * rng.uniform();
  }
}

// ------------------------------------------------------------- kernels ----

// Pose frames from genes on the device (CUDA's sin/cos; the composite
// entries in the reference's operation order).
// slots (may be null): the k-th group of n poses belongs to slot slots[k / n]
// (the server's resident jobs); else pose k belongs to job job_of[k].
__global__ void k_frames(const double *genes, gd_pose_frame *frames, const int *job_of, const GaJobState *state,
                         int total, const int *slots, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int job = slots ? slots[t / n] : job_of[t];
  const int k = slots ? job * n + t % n : t;
  if (state[job].stop) return;
  const double *g = genes + 6 * static_cast<size_t>(k);
  double sa, ca, sb, cb, sg, cg;
  sincos(g[0], &sa, &ca);
  sincos(g[1], &sb, &cb);
  sincos(g[2], &sg, &cg);
  gd_pose_frame f;
  f.ca = ca;
  f.sa = sa;
  f.cb = cb;
  f.sb = sb;
  f.cg = cg;
  f.sg = sg;
  f.m01 = __dadd_rn(__dmul_rn(-sa, cg), __dmul_rn(__dmul_rn(ca, sb), sg));
  f.m02 = __dadd_rn(__dmul_rn(sa, sg), __dmul_rn(__dmul_rn(ca, sb), cg));
  f.m11 = __dadd_rn(__dmul_rn(ca, cg), __dmul_rn(__dmul_rn(sa, sb), sg));
  f.m12 = __dadd_rn(__dmul_rn(-ca, sg), __dmul_rn(__dmul_rn(sa, sb), cg));
  f.dx = g[3];
  f.dy = g[4];
  f.dz = g[5];
  f.pad[0] = f.pad[1] = f.pad[2] = 0.0;
  frames[k] = f;
}

struct GaStepParams {
  double *genes;              // [jobs][n][6], updated in place
  double *genes_tmp;          // scratch [jobs][m][6]
  const gd_pose_energy *energies;  // [jobs][n]
  GaJobState *state;          // [jobs]
  double *history;            // [jobs][max_gen] best fitness per generation
  const int *tour, *perm;     // [jobs][max_gen][...]
  const double *cross_u, *mut_u, *mut_z;
  gd_hof_entry *hof, *hof_tmp;  // [jobs][hof_max_size + 1]; null = no Hall of Fame
  const gd_dock_metrics *metrics;  // [jobs][n] DockQ of the evaluated population; null = none
  const int *eval_on;              // [jobs] 1 = the job has an evaluator
  gd_dock_metrics *best_metrics;   // [jobs][max_gen]
  double *mean_dockq;              // [jobs][max_gen]
  int *err;                        // the context's error word (index checks of the debug library)
  const int *slots;                // block b runs job slots[b] (the server's resident jobs); null: job b
  gd_ga_cfg cfg;
};

// NaN ranks after every number (a total order the reference's partial_cmp
// sort does not define; it never arises for finite inputs)
__device__ __forceinline__ double key_of(double f) { return f != f ? INFINITY : f; }

// HallOfFame::genes_are_similar (src/commands/run.rs:140-160) with
// angular_difference (:162-171): every angle within 0.2 rad (with the wrap
// at 2 pi) and every displacement within 2 A.
__device__ __forceinline__ bool hof_similar(const double *a, const double *b) {
  const double pi = 3.141592653589793, two_pi = 6.283185307179586;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double d = fabs(__dsub_rn(a[i], b[i]));
    if (d > pi) d = __dsub_rn(two_pi, d);
    if (d > 0.2) return false;
  }
#pragma unroll
  for (int i = 3; i < 6; ++i)
    if (fabs(__dsub_rn(a[i], b[i])) > 2.0) return false;
  return true;
}

constexpr int kHofChunk = 32;    // candidates pre-checked per round (one per lane)
constexpr int kHofNewMax = 32;   // entries a round may add before the pre-check is redone
constexpr int kHofF32Max = 512;  // entries mirrored in FP32 for the pre-filter

// FP32 pre-filter of hof_similar: true only where the exact FP64 test says
// "not similar": some angle differs by more than 0.2 and less than
// 2 pi - 0.2 (so also by more than 0.2 across the wrap), or some
// displacement by more than 2, each by a margin (1e-4 + 1e-6 (|a| + |b|))
// far above the FP32 rounding of both values and of their difference.
__device__ __forceinline__ bool hof_far32(const float *a, const float *b) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float d = fabsf(a[i] - b[i]), mg = 1e-4f + 1e-6f * (fabsf(a[i]) + fabsf(b[i]));
    if (d > 0.2f + mg && d < 6.0831853f - mg) return true;
  }
#pragma unroll
  for (int i = 3; i < 6; ++i) {
    const float d = fabsf(a[i] - b[i]), mg = 1e-4f + 1e-6f * (fabsf(a[i]) + fabsf(b[i]));
    if (d > 2.0f + mg) return true;
  }
  return false;
}

__device__ __forceinline__ bool genes_equal(const double *a, const double *b) {
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3] && a[4] == b[4] && a[5] == b[5];
}

// HallOfFame::add_from_population (src/commands/run.rs:193-213) for one job,
// by the whole CTA: the population in stable ascending fitness order (order)
// goes through try_add (:101-127) until top_k entries went in; each add over
// capacity prunes (:174-179): a stable sort by fitness, then truncation.
// Rounds of kHofChunk candidates: all threads first count, per candidate, the
// similar entries held at the start of the round (the O(candidates x entries)
// part: lane = candidate, warp = a slice of the entries, an FP32 pre-filter
// before the exact FP64 test); one warp then walks the round in order.  A candidate goes in when no
// entry of the round's start is left similar to it and it is not similar to
// an entry added in this round.  The entry a prune drops is either one added
// in this round (taken off that list) or one of the round's start (the later
// candidates similar to it lose one count).  Once a prune has sorted the
// entries, the next prune only moves the new last entry behind the entries of
// equal or lower fitness, which is what the stable sort does to a sorted list
// with one entry appended.
__device__ void hof_update(const GaStepParams &P, GaJobState &st, int job, int gen, const double *G,
                           const double *f, const int *order, int *s_csim, double *s_new, int *s_ctl, int *s_part,
                           float *s_hf) {
  const gd_ga_cfg &c = P.cfg;
  const int tid = threadIdx.x, lane = tid & 31, cap = c.hof_max_size, n = c.pop_size;
  gd_hof_entry *H = P.hof + static_cast<size_t>(job) * (cap + 1);
  gd_hof_entry *T = P.hof_tmp + static_cast<size_t>(job) * (cap + 1);
  if (tid == 0) {
    s_ctl[0] = 0;  // first candidate of the round (rank)
    s_ctl[1] = 0;  // entries added in this generation
    s_ctl[2] = st.hof_n;
    s_ctl[3] = st.hof_sorted;
  }
  __syncthreads();
  for (;;) {
    const int base = s_ctl[0], cnt0 = s_ctl[2];
    if (base >= n || s_ctl[1] >= c.hof_top_k) break;
    const int end = min(base + kHofChunk, n);
    const int nw = blockDim.x >> 5, w = tid >> 5;
    const bool f32 = cnt0 <= kHofF32Max;
    if (f32)
      for (int i = tid; i < 6 * cnt0; i += blockDim.x) s_hf[i] = __double2float_rn(H[i / 6].genes[i % 6]);
    __syncthreads();
    {
      int cs = 0;
      if (base + lane < end) {
        const double *gp = G + 6 * order[base + lane];
        double g[6];
        float g32[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          g[i] = gp[i];
          g32[i] = __double2float_rn(g[i]);
        }
        for (int e = w; e < cnt0; e += nw)
          if (!(f32 && hof_far32(g32, s_hf + 6 * e))) cs += hof_similar(g, H[e].genes);
      }
      s_part[tid] = cs;
    }
    __syncthreads();
    if (tid < 32) {
      {
        int cs = 0;
        for (int q = 0; q < nw; ++q) cs += s_part[32 * q + lane];
        s_csim[lane] = cs;
      }
      __syncwarp();
      int cnt = cnt0, sorted = s_ctl[3], added = s_ctl[1], n_new = 0, next = end;
      for (int r = base; r < end; ++r) {
        if (s_csim[r - base] > 0) continue;
        const double *gp = G + 6 * order[r];
        double g[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) g[i] = gp[i];
        const bool sim = lane < n_new && hof_similar(g, s_new + 6 * lane);
        if (__any_sync(kFull, sim)) continue;
        if (lane == 0 && GD_DCHECK(P.err, cnt <= cap, 50)) {
          gd_hof_entry &x = H[cnt];
#pragma unroll
          for (int i = 0; i < 6; ++i) {
            x.genes[i] = g[i];
            s_new[6 * n_new + i] = g[i];
          }
          x.fitness = f[order[r]];
          x.generation = gen;
          x.pad = 0;
        }
        ++cnt;
        ++n_new;
        ++added;
        __syncwarp();
        if (cnt > cap) {
          if (sorted) {
            const double fn = key_of(H[cnt - 1].fitness);
            int pos = 0;  // entries before the new one: fitness <= its fitness
            for (int e = lane; e < cnt - 1; e += 32) pos += key_of(H[e].fitness) <= fn;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) pos += __shfl_xor_sync(kFull, pos, o);
            for (int e = lane; e < cnt; e += 32) {
              const int d = e < pos ? e : (e == cnt - 1 ? pos : e + 1);
              if (GD_DCHECK(P.err, d >= 0 && d <= cap, 51)) T[d] = H[e];
            }
          } else {
            for (int e = lane; e < cnt; e += 32) {
              const double fe = key_of(H[e].fitness);
              int rk = 0;
              for (int q = 0; q < cnt; ++q) {
                const double fq = key_of(H[q].fitness);
                rk += (fq < fe) || (fq == fe && q < e);
              }
              T[rk] = H[e];
            }
          }
          __syncwarp();
          // the entry the prune drops: T[cap]
          double x[6];
#pragma unroll
          for (int i = 0; i < 6; ++i) x[i] = T[cap].genes[i];
          const unsigned mine = __ballot_sync(kFull, lane < n_new && genes_equal(x, s_new + 6 * lane));
          if (mine) {
            const int w = __ffs(mine) - 1;
            if (lane == 0 && w != n_new - 1)
              for (int i = 0; i < 6; ++i) s_new[6 * w + i] = s_new[6 * (n_new - 1) + i];
            --n_new;
          } else {
            for (int q = r + 1 + lane; q < end; q += 32) {
              const double *gq = G + 6 * order[q];
              if (s_csim[q - base] > 0 && hof_similar(gq, x)) --s_csim[q - base];
            }
          }
          cnt = cap;
          for (int e = lane; e < cnt; e += 32) H[e] = T[e];
          sorted = 1;
          __syncwarp();
        }
        if (added >= c.hof_top_k || n_new == kHofNewMax) {
          next = r + 1;
          break;
        }
      }
      if (lane == 0) {
        s_ctl[0] = next;
        s_ctl[1] = added;
        s_ctl[2] = cnt;
        s_ctl[3] = sorted;
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    st.hof_n = s_ctl[2];
    st.hof_sorted = s_ctl[3];
  }
}

// Sort keys of fitness values: unsigned order = the order of the values,
// -0 with +0, NaN after every number (an order the reference's partial_cmp
// sorts do not define; NaN never arises for finite inputs).
__device__ __forceinline__ unsigned long long asc_key(double f) {
  if (f != f) f = INFINITY;
  if (f == 0.0) f = 0.0;
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(f));
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Block-wide bitonic sort of (key, idx) pairs, ascending by key then index,
// over P (a power of two) entries; every thread of the block calls it.
__device__ void bitonic_sort(unsigned long long *key, int *idx, int P) {
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
        const int i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i | j;
        const unsigned long long a = key[i], b = key[l];
        const int ia = idx[i], ib = idx[l];
        const bool a_after_b = a > b || (a == b && ia > ib);
        if (a_after_b == ((i & k) == 0)) {
          key[i] = b;
          key[l] = a;
          idx[i] = ib;
          idx[l] = ia;
        }
      }
      __syncthreads();
    }
}

__host__ __device__ inline int pow2_at_least(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

// dynamic shared memory of k_ga_step for a population of n
inline size_t ga_step_smem(int n) {
  const size_t p2 = static_cast<size_t>(pow2_at_least(n));
  return sizeof(double) * n + sizeof(unsigned long long) * p2 + sizeof(int) * (n + p2);
}

// One CTA per job: the reference loop's bookkeeping for the fitness just
// computed (with the Hall of Fame), then evolve.  The stable orders of the
// population (elitism, Hall of Fame, best of the generation) and of the
// offspring are bitonic sorts of integer keys: FP64 comparisons run at a
// small fraction of the integer rate on this part, and the O(n^2) rank
// counts they replace took 29 ms per generation at 4,096 poses.
__global__ void __launch_bounds__(256) k_ga_step(const GaStepParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gd_ga_cfg &c = P.cfg;
  const int job = P.slots ? P.slots[blockIdx.x] : static_cast<int>(blockIdx.x), tid = threadIdx.x, nt = blockDim.x;
  const int n = c.pop_size, m = 2 * (n / 2), P2 = pow2_at_least(n);
  double *f = reinterpret_cast<double *>(smem);                            // [n] fitness of the population
  unsigned long long *kb = reinterpret_cast<unsigned long long *>(f + n);  // [P2] sort keys
  int *sel = reinterpret_cast<int *>(kb + P2);                             // [n] tournament winners
  int *order = sel + n;                                                    // [P2] sort indices
  __shared__ double s_eg[64 * 6];                  // elites' genes, staged before the population is overwritten
  __shared__ int s_evolve, s_hof, s_gen, s_final, s_nan;
  __shared__ int s_csim[kHofChunk], s_hctl[4], s_hpart[256];  // Hall of Fame rounds
  __shared__ double s_hnew[kHofNewMax * 6];
  __shared__ float s_hf[kHofF32Max * 6];
  GaJobState &st = P.state[job];
  if (st.stop) return;
  const gd_pose_energy *E = P.energies + static_cast<size_t>(job) * n;
  if (tid == 0) {
    s_final = st.gen >= c.max_generations;
    s_nan = 0;
  }
  for (int k = tid; k < n; k += nt) f[k] = E[k].fitness;
  __syncthreads();
  if (s_final) {
    // the evaluation just done was of the final population: stop here
    if (tid == 0) st.stop = 2;
    return;
  }
  // stable ascending order of the population (src/population.rs:76-82 for
  // the elites, src/commands/run.rs:195-201 for the Hall of Fame)
  for (int k = tid; k < P2; k += nt) {
    if (k < n && f[k] != f[k]) s_nan = 1;
    kb[k] = k < n ? asc_key(f[k]) : ~0ull;
    order[k] = k;
  }
  __syncthreads();
  bitonic_sort(kb, order, P2);
  if (tid == 0) {
    const int gen = st.gen;
    s_gen = gen;
    // Hall of Fame of every evaluation inside the loop (src/commands/run.rs:385)
    s_hof = P.hof != nullptr && c.hof_max_size > 0 && c.hof_top_k > 0;
    // best of this generation, first minimum (src/commands/run.rs:391-398):
    // the head of the stable order unless a NaN makes the comparisons differ
    int bi = order[0];
    if (s_nan) {
      bi = 0;
      for (int k = 1; k < n; ++k)
        if (f[bi] > f[k]) bi = k;
    }
    const double best = f[bi];
    P.history[static_cast<size_t>(job) * c.max_generations + gen] = best;
    if (P.metrics && P.eval_on[job]) {
      // the generation's metrics: the best pose's and the mean DockQ as a
      // left-to-right sum (src/commands/run.rs:388,449-451)
      const gd_dock_metrics *M = P.metrics + static_cast<size_t>(job) * n;
      const size_t jg = static_cast<size_t>(job) * c.max_generations + gen;
      P.best_metrics[jg] = M[bi];
      double sum = 0.0;
      for (int k = 0; k < n; ++k) sum += M[k].dockq;
      P.mean_dockq[jg] = sum / static_cast<double>(n);
    }
    if (gen > 0) {  // convergence window (src/commands/run.rs:400-409)
      const double imp = (st.last_best - best) / fabs(st.last_best);
      if (imp < c.convergence_threshold) st.stagnant += 1;
      else st.stagnant = 0;
    }
    st.last_best = best;
    if (c.early_stopping && st.stagnant >= c.convergence_window) {
      st.stop = 1;  // converged: this population is the final one
      s_evolve = 0;
    } else {
      st.gen = gen + 1;
      s_evolve = 1;
    }
  }
  __syncthreads();
  if (!s_evolve && !s_hof) return;
  double *G = P.genes + static_cast<size_t>(job) * n * 6;
  const int ne = c.elitism < n ? c.elitism : n;
  if (s_hof) hof_update(P, st, job, s_gen, G, f, order, s_csim, s_hnew, s_hctl, s_hpart, s_hf);
  if (!s_evolve) return;
  const int gen = st.gen - 1;  // draws of the generation being evolved
  const size_t jg = static_cast<size_t>(job) * c.max_generations + gen;
  const int *tour = P.tour + jg * c.tournament_size * n;
  const int *perm = P.perm + jg * n;
  const double *cu = P.cross_u + jg * 6 * (n / 2);
  const double *mu = P.mut_u + jg * 6 * m;
  const double *mz = P.mut_z + jg * 6 * m;
  double *T = P.genes_tmp + static_cast<size_t>(job) * m * 6;
  // tournament: first minimum of the draws (src/population.rs:136-156)
  for (int k = tid; k < n; k += nt) {
    int best = tour[c.tournament_size * k];
    for (int t = 1; t < c.tournament_size; ++t) {
      const int q = tour[c.tournament_size * k + t];
      if (f[best] > f[q]) best = q;
    }
    sel[k] = best;
  }
  // elites: the first ne of the stable order
  for (int i = tid; i < ne * 6; i += nt) s_eg[i] = G[6 * order[i / 6] + i % 6];
  __syncthreads();
  // shuffle + crossover + mutation (src/population.rs:88-107, src/ga.rs:7-39,
  // src/chromosome.rs:56-77); the offspring's carried fitness goes straight
  // into descending sort keys
  const double two_pi = 6.283185307179586;
  for (int p = tid; p < n / 2; p += nt) {
    const int a = sel[perm[2 * p]], b = sel[perm[2 * p + 1]];
    for (int g = 0; g < 6; ++g) {
      const double ga = G[6 * a + g], gb = G[6 * b + g];
      const bool sw = cu[6 * p + g] <= c.crossover_rate;
      double o[2] = {sw ? gb : ga, sw ? ga : gb};
      for (int h = 0; h < 2; ++h) {
        const int k = 2 * p + h;
        if (mu[6 * k + g] <= c.mutation_rate) {
          double v = __dadd_rn(o[h], mz[6 * k + g]);
          if (g < 3) {
            double r = fmod(v, two_pi);  // f64::rem_euclid
            if (r < 0.0) r = __dadd_rn(r, two_pi);
            v = r;
          } else {
            v = v < -c.max_displacement ? -c.max_displacement : (v > c.max_displacement ? c.max_displacement : v);
          }
          o[h] = v;
        }
        T[6 * k + g] = o[h];
      }
    }
    kb[2 * p] = ~asc_key(f[a]);
    kb[2 * p + 1] = ~asc_key(f[b]);
  }
  for (int k = m + tid; k < P2; k += nt) kb[k] = ~0ull;
  for (int k = tid; k < P2; k += nt) order[k] = k;
  __syncthreads();
  // stable descending order by the carried fitness; elites over the first
  // slots (src/population.rs:110-118)
  bitonic_sort(kb, order, P2);
  for (int r = ne + tid; r < m; r += nt) {
    const int k = order[r];
    if (!GD_DCHECK(P.err, k >= 0 && k < m, 52)) continue;
    for (int g = 0; g < 6; ++g) G[6 * r + g] = T[6 * k + g];
  }
  for (int i = tid; i < ne * 6; i += nt) G[i] = s_eg[i];
}

}  // namespace
}  // namespace gd

using namespace gd;

extern "C" {

gd_status gd_ga_default_cfg(gd_ga_cfg *cfg) {
  if (!cfg) return GD_ERR_INVALID_ARG;
  // src/constants.rs:2-16 and src/chromosome.rs:64-71
  // src/commands/run.rs:56-57 (Hall of Fame)
  *cfg = gd_ga_cfg{150, 5, 3, 0.6, 0.1, 50.0, 0.174, 1.0, 250, 1, 0.001, 10, 42, 500, 10};
  return GD_OK;
}

gd_status gd_ga_draw(const gd_ga_cfg *cfg, uint64_t seed, int32_t generations, double *init_genes, int32_t *tour,
                     int32_t *perm, double *cross_u, double *mut_u, double *mut_z) {
  if (!cfg || generations < 0 || cfg->pop_size < 2 || cfg->tournament_size < 1) return GD_ERR_INVALID_ARG;
  Rng rng(seed);
  const int n = cfg->pop_size, m = 2 * (n / 2);
  if (init_genes) draw_initial(rng, *cfg, init_genes);
  GenDraws d;
  for (int g = 0; g < generations; ++g) {
    draw_generation(rng, *cfg, d);
    if (tour) std::memcpy(tour + static_cast<size_t>(g) * cfg->tournament_size * n, d.tour.data(), sizeof(int) * d.tour.size());
    if (perm) std::memcpy(perm + static_cast<size_t>(g) * n, d.perm.data(), sizeof(int) * n);
    if (cross_u) std::memcpy(cross_u + static_cast<size_t>(g) * 6 * (n / 2), d.cross_u.data(), sizeof(double) * d.cross_u.size());
    if (mut_u) std::memcpy(mut_u + static_cast<size_t>(g) * 6 * m, d.mut_u.data(), sizeof(double) * d.mut_u.size());
    if (mut_z) std::memcpy(mut_z + static_cast<size_t>(g) * 6 * m, d.mut_z.data(), sizeof(double) * d.mut_z.size());
  }
  return GD_OK;
}

}  // extern "C"

namespace gd {

// Device buffers of a GA batch.
struct GaRun {
  int jobs = 0, n = 0, G = 0;
  double *genes = nullptr, *genes_tmp = nullptr, *history = nullptr, *cross_u = nullptr, *mut_u = nullptr,
         *mut_z = nullptr;
  int *tour = nullptr, *perm = nullptr, *job_of = nullptr;
  gd_pose_frame *frames = nullptr;
  gd_pose_energy *energies = nullptr;
  GaJobState *state = nullptr;
  gd_hof_entry *hof = nullptr, *hof_tmp = nullptr;
  gd_dock_metrics *metrics = nullptr, *best_metrics = nullptr;
  double *mean_dockq = nullptr;
  int *eval_on = nullptr;
  std::vector<std::pair<void *, size_t>> allocs;
};

static gd_status ga_alloc(gd_context *ctx, GaRun &R, size_t bytes, void **p) {
  gd_status s = dev_alloc(ctx, bytes, p);
  if (s == GD_OK) R.allocs.push_back({*p, bytes});
  return s;
}

static void ga_release(gd_context *ctx, GaRun &R) {
  for (auto &a : R.allocs) dev_free(ctx, a.first, a.second);
  R.allocs.clear();
}

}  // namespace gd

extern "C" gd_status gd_ga_run(gd_context *ctx, gd_complex *const *complexes, int32_t jobs, const gd_ga_cfg *cfg,
                               gd_precision prec, int32_t use_graph, double *out_genes, gd_pose_energy *out_energies,
                               int32_t *out_generations, double *out_history, gd_hof_entry *out_hof,
                               int32_t *out_hof_count, const gd_ga_metrics *metrics) {
  gd::NvtxRange nvtx_range("gd_ga_run");
  using namespace gd;
  if (!ctx) return GD_ERR_INVALID_ARG;
  if (!complexes || jobs <= 0 || !cfg || !out_genes || !out_energies)
    return fail(ctx, GD_ERR_INVALID_ARG, "bad GA arguments");
  const gd_ga_cfg c = *cfg;
  if (c.pop_size < 2 || c.pop_size % 2 || c.tournament_size < 1 || c.elitism < 0 || c.elitism > 64 ||
      c.elitism > c.pop_size || c.max_generations < 0 || c.pop_size > 8192)
    return fail(ctx, GD_ERR_INVALID_ARG, "GA config: even pop_size in [2, 8192], elitism <= 64");
  if (prec != GD_PREC_F32 && prec != GD_PREC_F64) return fail(ctx, GD_ERR_INVALID_ARG, "bad precision");
  const bool hof = out_hof || out_hof_count;
  if (hof && (!out_hof || !out_hof_count || c.hof_max_size < 0 || c.hof_max_size > (1 << 20) || c.hof_top_k < 0))
    return fail(ctx, GD_ERR_INVALID_ARG, "Hall of Fame: out_hof and out_hof_count together, hof_max_size in [0, 2^20]");
  const int hcap = hof ? c.hof_max_size : 0;
  const bool with_metrics = metrics && metrics->evaluators;
  if (with_metrics && (!metrics->best || !metrics->mean_dockq))
    return fail(ctx, GD_ERR_INVALID_ARG, "GA metrics: best and mean_dockq are required with evaluators");
  if (with_metrics)
    for (int j = 0; j < jobs; ++j)
      if (metrics->evaluators[j] && evaluator_complex(metrics->evaluators[j]) != complexes[j])
        return fail(ctx, GD_ERR_INVALID_ARG, "GA metrics: an evaluator of another complex");
  for (int j = 0; j < jobs; ++j)
    if (!complexes[j] || complexes[j]->ctx != ctx) return fail(ctx, GD_ERR_INVALID_ARG, "complex of another context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  const int n = c.pop_size, m = n, G = c.max_generations;
  GaRun R;
  R.jobs = jobs;
  R.n = n;
  R.G = G;
  // host draws: initial genes + every generation's randoms, per job
  const size_t gT = static_cast<size_t>(c.tournament_size) * n, gC = 6 * static_cast<size_t>(n / 2), gM = 6 * static_cast<size_t>(m);
  std::vector<double> h_genes(static_cast<size_t>(jobs) * n * 6);
  std::vector<int> h_tour(static_cast<size_t>(jobs) * std::max(G, 1) * gT), h_perm(static_cast<size_t>(jobs) * std::max(G, 1) * n);
  std::vector<double> h_cu(static_cast<size_t>(jobs) * std::max(G, 1) * gC), h_mu(static_cast<size_t>(jobs) * std::max(G, 1) * gM),
      h_mz(static_cast<size_t>(jobs) * std::max(G, 1) * gM);
  for (int j = 0; j < jobs; ++j) {
    gd_ga_draw(&c, c.seed + static_cast<uint64_t>(j), G, &h_genes[static_cast<size_t>(j) * n * 6],
               &h_tour[static_cast<size_t>(j) * G * gT], &h_perm[static_cast<size_t>(j) * G * n],
               &h_cu[static_cast<size_t>(j) * G * gC], &h_mu[static_cast<size_t>(j) * G * gM],
               &h_mz[static_cast<size_t>(j) * G * gM]);
  }
  std::vector<int> h_job(static_cast<size_t>(jobs) * n);
  for (int j = 0; j < jobs; ++j)
    for (int k = 0; k < n; ++k) h_job[static_cast<size_t>(j) * n + k] = j;
  std::vector<GaJobState> h_state(jobs);
  for (auto &s : h_state) s = GaJobState{0, 0, 0, 0, 1.7976931348623157e308, 0, 0};

  auto up = [&](const void *src, size_t bytes, void **dst) -> gd_status {
    gd_status s = ga_alloc(ctx, R, std::max<size_t>(bytes, 16), dst);
    if (s != GD_OK) return s;
    const cudaError_t ee = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    return ee == cudaSuccess ? GD_OK : cuda_fail(ctx, ee, "GA upload");
  };
  gd_status s;
  void *p;
  const size_t jn = static_cast<size_t>(jobs) * n;
  if ((s = up(h_genes.data(), sizeof(double) * h_genes.size(), &p)) != GD_OK) goto done;
  R.genes = static_cast<double *>(p);
  if ((s = up(h_tour.data(), sizeof(int) * h_tour.size(), &p)) != GD_OK) goto done;
  R.tour = static_cast<int *>(p);
  if ((s = up(h_perm.data(), sizeof(int) * h_perm.size(), &p)) != GD_OK) goto done;
  R.perm = static_cast<int *>(p);
  if ((s = up(h_cu.data(), sizeof(double) * h_cu.size(), &p)) != GD_OK) goto done;
  R.cross_u = static_cast<double *>(p);
  if ((s = up(h_mu.data(), sizeof(double) * h_mu.size(), &p)) != GD_OK) goto done;
  R.mut_u = static_cast<double *>(p);
  if ((s = up(h_mz.data(), sizeof(double) * h_mz.size(), &p)) != GD_OK) goto done;
  R.mut_z = static_cast<double *>(p);
  if ((s = up(h_job.data(), sizeof(int) * h_job.size(), &p)) != GD_OK) goto done;
  R.job_of = static_cast<int *>(p);
  if ((s = up(h_state.data(), sizeof(GaJobState) * jobs, &p)) != GD_OK) goto done;
  R.state = static_cast<GaJobState *>(p);
  if ((s = ga_alloc(ctx, R, sizeof(double) * jn * 6, &p)) != GD_OK) goto done;
  R.genes_tmp = static_cast<double *>(p);
  if ((s = ga_alloc(ctx, R, sizeof(double) * static_cast<size_t>(jobs) * std::max(G, 1), &p)) != GD_OK) goto done;
  R.history = static_cast<double *>(p);
  if ((s = ga_alloc(ctx, R, sizeof(gd_pose_frame) * jn, &p)) != GD_OK) goto done;
  R.frames = static_cast<gd_pose_frame *>(p);
  if ((s = ga_alloc(ctx, R, sizeof(gd_pose_energy) * jn, &p)) != GD_OK) goto done;
  R.energies = static_cast<gd_pose_energy *>(p);
  if (hcap > 0) {
    const size_t hb = sizeof(gd_hof_entry) * static_cast<size_t>(jobs) * (hcap + 1);
    if ((s = ga_alloc(ctx, R, hb, &p)) != GD_OK) goto done;
    R.hof = static_cast<gd_hof_entry *>(p);
    if ((s = ga_alloc(ctx, R, hb, &p)) != GD_OK) goto done;
    R.hof_tmp = static_cast<gd_hof_entry *>(p);
  }
  if (with_metrics) {
    std::vector<int> on(jobs);
    for (int j = 0; j < jobs; ++j) on[j] = metrics->evaluators[j] != nullptr;
    if ((s = up(on.data(), sizeof(int) * jobs, &p)) != GD_OK) goto done;
    R.eval_on = static_cast<int *>(p);
    if ((s = ga_alloc(ctx, R, sizeof(gd_dock_metrics) * jn, &p)) != GD_OK) goto done;
    R.metrics = static_cast<gd_dock_metrics *>(p);
    const size_t jgb = static_cast<size_t>(jobs) * std::max(G, 1);
    if ((s = ga_alloc(ctx, R, sizeof(gd_dock_metrics) * jgb, &p)) != GD_OK) goto done;
    R.best_metrics = static_cast<gd_dock_metrics *>(p);
    if ((s = ga_alloc(ctx, R, sizeof(double) * jgb, &p)) != GD_OK) goto done;
    R.mean_dockq = static_cast<double *>(p);
    // entries of generations not reached keep the caller's values
    if (G > 0) {
      e = cudaMemcpy(R.best_metrics, metrics->best, sizeof(gd_dock_metrics) * jobs * G, cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(R.mean_dockq, metrics->mean_dockq, sizeof(double) * jobs * G, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        s = cuda_fail(ctx, e, "GA metrics upload");
        goto done;
      }
    }
  }
  {
    // one scoring descriptor per job; poses outside [-M, M] never occur
    std::vector<ScoreParams> descs;
    bool serial = false, clamp = false;
    for (int j = 0; j < jobs; ++j) {
      ScoreParams d = make_params(complexes[j], R.frames + static_cast<size_t>(j) * n, nullptr, n,
                                  R.energies + static_cast<size_t>(j) * n, c.max_displacement);
      d.skip = &R.state[j].stop;
      descs.push_back(d);
      serial |= complexes[j]->serial_overlap;
      clamp |= complexes[j]->need_clamp;
    }
    BatchLaunch *bl = nullptr;
    if (prec == GD_PREC_F32) {
      s = batch_prepare(ctx, descs, serial, clamp, ctx->tune_f32_slots ? ctx->tune_f32_slots : kDefaultF32Tune, &bl);
      if (s != GD_OK) goto done;
    }
    GaStepParams P{};
    P.genes = R.genes;
    P.genes_tmp = R.genes_tmp;
    P.energies = R.energies;
    P.state = R.state;
    P.history = R.history;
    P.tour = R.tour;
    P.perm = R.perm;
    P.cross_u = R.cross_u;
    P.mut_u = R.mut_u;
    P.mut_z = R.mut_z;
    P.hof = R.hof;
    P.hof_tmp = R.hof_tmp;
    P.metrics = R.metrics;
    P.eval_on = R.eval_on;
    P.best_metrics = R.best_metrics;
    P.mean_dockq = R.mean_dockq;
    P.err = ctx->d_err;
    P.cfg = c;
    P.cfg.hof_max_size = hcap;
    const size_t ga_smem = ga_step_smem(n);
    cudaStream_t st = ctx->stream;
    auto generation = [&]() -> gd_status {
      const int total = static_cast<int>(jn);
      k_frames<<<(total + 255) / 256, 256, 0, st>>>(R.genes, R.frames, R.job_of, R.state, total, nullptr, n);
      cudaError_t ee = cudaGetLastError();
      if (ee != cudaSuccess) return cuda_fail(ctx, ee, "frames kernel");
      if (prec == GD_PREC_F32) {
        gd_status ss = batch_launch(ctx, bl, st);
        if (ss != GD_OK) return ss;
      } else {
        // plain form: one FP64 launch per job; finished jobs are skipped on
        // the device by the GA step, so their scores stay final
        for (int j = 0; j < jobs; ++j) {
          gd_status ss = launch_score(complexes[j], descs[j].frames, nullptr, n, GD_PREC_F64, descs[j].out, st,
                                      c.max_displacement);
          if (ss != GD_OK) return ss;
        }
      }
      if (with_metrics)
        for (int j = 0; j < jobs; ++j)
          if (metrics->evaluators[j]) {
            gd_status ss = launch_dockq(metrics->evaluators[j], descs[j].frames, n,
                                        R.metrics + static_cast<size_t>(j) * n, &R.state[j].stop, st);
            if (ss != GD_OK) return ss;
          }
      k_ga_step<<<jobs, 256, ga_smem, st>>>(P);
      ee = cudaGetLastError();
      return ee == cudaSuccess ? GD_OK : cuda_fail(ctx, ee, "GA step kernel");
    };
    if (ga_smem > 48 * 1024) cudaFuncSetAttribute(k_ga_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  static_cast<int>(ga_smem));
    const int iters = G + 1;  // G evolutions + the evaluation of the final population
    if (use_graph && prec == GD_PREC_F32) {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) {
        s = cuda_fail(ctx, e, "begin graph capture");
      } else {
        s = generation();
        e = cudaStreamEndCapture(st, &graph);
        if (s == GD_OK && e != cudaSuccess) s = cuda_fail(ctx, e, "end graph capture");
        if (s == GD_OK && (e = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess)
          s = cuda_fail(ctx, e, "graph instantiate");
        for (int it = 0; s == GD_OK && it < iters; ++it)
          if ((e = cudaGraphLaunch(exec, st)) != cudaSuccess) s = cuda_fail(ctx, e, "graph launch");
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
      }
    } else {
      for (int it = 0; s == GD_OK && it < iters; ++it) s = generation();
    }
    if (s == GD_OK) {
      e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) s = cuda_fail(ctx, e, "GA run");
    }
    if (s == GD_OK) s = check_device_error(ctx);
    if (bl) batch_free(ctx, bl);
    if (s != GD_OK) goto done;
  }
  {
    // results: the final population, its energies, generations and history
    e = cudaMemcpy(out_genes, R.genes, sizeof(double) * jn * 6, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_energies, R.energies, sizeof(gd_pose_energy) * jn, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_state.data(), R.state, sizeof(GaJobState) * jobs, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && out_history && G > 0)
      e = cudaMemcpy(out_history, R.history, sizeof(double) * jobs * G, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      s = cuda_fail(ctx, e, "GA results");
      goto done;
    }
    if (out_generations)
      for (int j = 0; j < jobs; ++j) out_generations[j] = h_state[j].gen;
    if (with_metrics && G > 0) {
      e = cudaMemcpy(metrics->best, R.best_metrics, sizeof(gd_dock_metrics) * jobs * G, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess)
        e = cudaMemcpy(metrics->mean_dockq, R.mean_dockq, sizeof(double) * jobs * G, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        s = cuda_fail(ctx, e, "GA metrics results");
        goto done;
      }
    }
    if (hof) {
      for (int j = 0; j < jobs; ++j) {
        out_hof_count[j] = hcap > 0 ? h_state[j].hof_n : 0;
        if (out_hof_count[j] > 0 &&
            (e = cudaMemcpy(out_hof + static_cast<size_t>(j) * hcap, R.hof + static_cast<size_t>(j) * (hcap + 1),
                            sizeof(gd_hof_entry) * out_hof_count[j], cudaMemcpyDeviceToHost)) != cudaSuccess) {
          s = cuda_fail(ctx, e, "Hall of Fame results");
          goto done;
        }
      }
    }
  }
done:
  ga_release(ctx, R);
  return s;
}

// =========================================================================
// Serving loop: docking jobs admitted into resident slots by HBM budget,
// all resident jobs advanced one generation per tick in shared launches.
// =========================================================================
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

namespace gd {
namespace {

using Clock = std::chrono::steady_clock;

struct HostMol {
  std::vector<double> x, y, z, eps, rmin2, q, r;
  std::vector<int32_t> serial;
  std::vector<int16_t> resseq;
  std::vector<uint8_t> chain, elem, ca;
  void copy(const gd_atoms *a) {
    const int n = a->n;
    x.assign(a->x, a->x + n);
    y.assign(a->y, a->y + n);
    z.assign(a->z, a->z + n);
    eps.assign(a->epsilon, a->epsilon + n);
    rmin2.assign(a->rmin2, a->rmin2 + n);
    q.assign(a->charge, a->charge + n);
    r.assign(a->vdw_radius, a->vdw_radius + n);
    serial.assign(a->serial, a->serial + n);
    resseq.assign(a->resseq, a->resseq + n);
    chain.assign(a->chain, a->chain + n);
    elem.assign(a->element, a->element + n);
    ca.assign(a->is_ca, a->is_ca + n);
  }
  gd_atoms view() const {
    return gd_atoms{static_cast<int32_t>(x.size()), x.data(), y.data(), z.data(), eps.data(), rmin2.data(),
                    q.data(), r.data(), serial.data(), resseq.data(), chain.data(), elem.data(), ca.data()};
  }
};

struct Job {
  int64_t id = 0;
  HostMol rec, lig;
  std::vector<int32_t> pairs;
  gd_weights w{};
  uint64_t seed = 0;
  int status = GD_JOB_QUEUED;
  Clock::time_point t_submit, t_admit, t_done;
  gd_complex *cx = nullptr;
  int slot = -1;
  int generations = 0;
  std::vector<double> genes, history;
  std::vector<gd_pose_energy> energies;
  std::vector<gd_hof_entry> hof;  // the job's Hall of Fame, in the reference's order
  int error = GD_OK;
  // host draws (made on the submitting thread, uploaded at admission)
  std::vector<double> d_init, d_cu, d_mu, d_mz;
  std::vector<int> d_tour, d_perm;
};

}  // namespace
}  // namespace gd

struct gd_server {
  gd_context *ctx = nullptr;
  gd_server_cfg cfg{};
  gd::GaRun arena;  // max_slots "jobs" worth of device buffers
  std::vector<gd::Job *> slot_job;
  gd::BatchLaunch *bl = nullptr;
  bool dirty = true;       // slot membership changed since bl was prepared
  uint64_t job_bytes = 0;  // device bytes held by resident complexes
  std::mutex mu;
  std::condition_variable cv;
  std::deque<gd::Job *> queue;
  std::map<int64_t, gd::Job *> jobs;
  int64_t next_id = 1;
  std::thread worker;
  bool running = false;
  gd_status failed = GD_OK;  // the worker stopped on this error: no job runs any more
  std::string fail_msg;      // the context's error message at that moment
  // statistics
  int64_t completed = 0, poses_scored = 0, generations_run = 0;
  std::vector<double> latencies;
  gd::Clock::time_point t_first;
  // host time per tick phase (GD_TRACE prints the totals when the server is destroyed)
  double t_admit = 0, t_load = 0, t_prepare = 0, t_gpu = 0, t_retire = 0;
  bool started_clock = false;
  // admission beside the running generation: uploads go to their own stream,
  // the next generation waits for them (ev_up)
  cudaStream_t up = nullptr;
  cudaEvent_t ev_up = nullptr, ev0 = nullptr, ev1 = nullptr;
  bool upload_pending = false;
  gd::GaJobState *h_states = nullptr;  // pinned: the slots' states after a generation
  int *d_slots = nullptr;              // the slots of the resident jobs (k_frames, k_ga_step)
  double gpu_busy = 0;                 // device time of the generations (CUDA events), seconds
};

namespace gd {
namespace {

constexpr int kStopFree = 3;  // slot without a job

gd_status server_alloc(gd_server *S) {
  gd_context *ctx = S->ctx;
  const gd_ga_cfg &c = S->cfg.ga;
  GaRun &R = S->arena;
  const int J = S->cfg.max_slots, n = c.pop_size, G = std::max(c.max_generations, 1);
  R.jobs = J;
  R.n = n;
  R.G = c.max_generations;
  const size_t jn = static_cast<size_t>(J) * n;
  void *p;
  gd_status s;
  auto A = [&](size_t bytes, void **out) { return ga_alloc(ctx, R, std::max<size_t>(bytes, 16), out); };
  if ((s = A(sizeof(double) * jn * 6, &p)) != GD_OK) return s;
  R.genes = static_cast<double *>(p);
  if ((s = A(sizeof(double) * jn * 6, &p)) != GD_OK) return s;
  R.genes_tmp = static_cast<double *>(p);
  if ((s = A(sizeof(double) * static_cast<size_t>(J) * G, &p)) != GD_OK) return s;
  R.history = static_cast<double *>(p);
  if ((s = A(sizeof(int) * jn * c.tournament_size * G, &p)) != GD_OK) return s;
  R.tour = static_cast<int *>(p);
  if ((s = A(sizeof(int) * jn * G, &p)) != GD_OK) return s;
  R.perm = static_cast<int *>(p);
  if ((s = A(sizeof(double) * static_cast<size_t>(J) * 6 * (n / 2) * G, &p)) != GD_OK) return s;
  R.cross_u = static_cast<double *>(p);
  if ((s = A(sizeof(double) * jn * 6 * G, &p)) != GD_OK) return s;
  R.mut_u = static_cast<double *>(p);
  if ((s = A(sizeof(double) * jn * 6 * G, &p)) != GD_OK) return s;
  R.mut_z = static_cast<double *>(p);
  if ((s = A(sizeof(gd_pose_frame) * jn, &p)) != GD_OK) return s;
  R.frames = static_cast<gd_pose_frame *>(p);
  if ((s = A(sizeof(gd_pose_energy) * jn, &p)) != GD_OK) return s;
  R.energies = static_cast<gd_pose_energy *>(p);
  if ((s = A(sizeof(GaJobState) * J, &p)) != GD_OK) return s;
  R.state = static_cast<GaJobState *>(p);
  if ((s = A(sizeof(int) * jn, &p)) != GD_OK) return s;
  R.job_of = static_cast<int *>(p);
  if (c.hof_max_size > 0 && c.hof_top_k > 0) {  // each slot's Hall of Fame
    const size_t hb = sizeof(gd_hof_entry) * static_cast<size_t>(J) * (c.hof_max_size + 1);
    if ((s = A(hb, &p)) != GD_OK) return s;
    R.hof = static_cast<gd_hof_entry *>(p);
    if ((s = A(hb, &p)) != GD_OK) return s;
    R.hof_tmp = static_cast<gd_hof_entry *>(p);
  }
  if ((s = A(sizeof(int) * J, &p)) != GD_OK) return s;
  S->d_slots = static_cast<int *>(p);
  cudaError_t ce = cudaMallocHost(reinterpret_cast<void **>(&S->h_states), sizeof(GaJobState) * J);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&S->up, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&S->ev_up, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreate(&S->ev0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&S->ev1);
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "server streams and events");
  std::vector<int> job_of(jn);
  for (size_t k = 0; k < jn; ++k) job_of[k] = static_cast<int>(k / n);
  std::vector<GaJobState> st(J, GaJobState{0, kStopFree, 0, 0, 0.0, 0, 0});
  cudaError_t e = cudaMemcpy(R.job_of, job_of.data(), sizeof(int) * jn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(R.state, st.data(), sizeof(GaJobState) * J, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "server arena");
  S->slot_job.assign(J, nullptr);
  return GD_OK;
}

void server_free_host(gd_server *S) {
  if (S->h_states) cudaFreeHost(S->h_states);
  if (S->up) cudaStreamDestroy(S->up);
  if (S->ev_up) cudaEventDestroy(S->ev_up);
  if (S->ev0) cudaEventDestroy(S->ev0);
  if (S->ev1) cudaEventDestroy(S->ev1);
  S->h_states = nullptr;
  S->up = nullptr;
  S->ev_up = S->ev0 = S->ev1 = nullptr;
}

// Upload a job's draws and initial state into slot j.
// The job's draws for all generations, in the reference's consumption order
// (src/population.rs:74-158); pure host work, done when the job is submitted.
void draw_job(const gd_ga_cfg &c, Job *job) {
  const int n = c.pop_size, m = n, G = std::max(c.max_generations, 1);
  const size_t gT = static_cast<size_t>(c.tournament_size) * n, gC = 6 * static_cast<size_t>(n / 2),
               gM = 6 * static_cast<size_t>(m);
  job->d_init.resize(static_cast<size_t>(n) * 6);
  job->d_cu.resize(gC * G);
  job->d_mu.resize(gM * G);
  job->d_mz.resize(gM * G);
  job->d_tour.resize(gT * G);
  job->d_perm.resize(static_cast<size_t>(n) * G);
  gd_ga_draw(&c, job->seed, c.max_generations, job->d_init.data(), job->d_tour.data(), job->d_perm.data(),
             job->d_cu.data(), job->d_mu.data(), job->d_mz.data());
}

gd_status server_load_slot(gd_server *S, int j, Job *job) {
  const gd_ga_cfg &c = S->cfg.ga;
  GaRun &R = S->arena;
  const int n = c.pop_size, m = n, G = c.max_generations;
  const size_t gT = static_cast<size_t>(c.tournament_size) * n, gC = 6 * static_cast<size_t>(n / 2),
               gM = 6 * static_cast<size_t>(m);
  const size_t Gs = static_cast<size_t>(G);
  // the admission stream: slot j is not part of the generation that may be
  // running on the context's stream, and the next one waits for these copies
  cudaStream_t st = S->up;
  cudaError_t e = cudaMemcpyAsync(R.genes + static_cast<size_t>(j) * n * 6, job->d_init.data(),
                                  sizeof(double) * job->d_init.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && G > 0) {
    e = cudaMemcpyAsync(R.tour + j * Gs * gT, job->d_tour.data(), sizeof(int) * gT * Gs, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R.perm + j * Gs * n, job->d_perm.data(), sizeof(int) * n * Gs, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R.cross_u + j * Gs * gC, job->d_cu.data(), sizeof(double) * gC * Gs, cudaMemcpyHostToDevice,
                          st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R.mut_u + j * Gs * gM, job->d_mu.data(), sizeof(double) * gM * Gs, cudaMemcpyHostToDevice,
                          st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R.mut_z + j * Gs * gM, job->d_mz.data(), sizeof(double) * gM * Gs, cudaMemcpyHostToDevice,
                          st);
  }
  GaJobState s0{0, 0, 0, 0, 1.7976931348623157e308, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(R.state + j, &s0, sizeof(s0), cudaMemcpyHostToDevice, st);
  // pageable sources: staged before the calls return, so the host draws can go
  if (e != cudaSuccess) return cuda_fail(S->ctx, e, "server slot upload");
  std::vector<double>().swap(job->d_cu);
  std::vector<double>().swap(job->d_mu);
  std::vector<double>().swap(job->d_mz);
  std::vector<int>().swap(job->d_tour);
  std::vector<int>().swap(job->d_perm);
  std::vector<double>().swap(job->d_init);
  return GD_OK;
}

// Admission: queued jobs, first come first served, into free slots while the
// HBM budget allows.  Each admitted job's complex is created (host packing,
// one allocation and one copy) and its draws and state are uploaded on the
// admission stream; the generation that is running meanwhile does not touch
// free slots.
gd_status server_admit(gd_server *S) {
  gd_context *ctx = S->ctx;
  const int J = S->cfg.max_slots;
  gd_status s = GD_OK;
  bool uploaded = false;
  for (;;) {
    int free_slot = -1;
    for (int j = 0; j < J; ++j)
      if (!S->slot_job[j]) {
        free_slot = j;
        break;
      }
    Job *job = nullptr;
    {
      std::lock_guard<std::mutex> lock(S->mu);
      if (free_slot < 0 || S->queue.empty()) break;
      job = S->queue.front();
    }
    const gd_atoms ra = job->rec.view(), la = job->lig.view();
    gd_complex *cx = nullptr;
    const uint64_t before = ctx->in_use;
    const auto ta = Clock::now();
    s = gd_complex_create(ctx, &ra, &la, job->pairs.empty() ? nullptr : job->pairs.data(),
                          static_cast<int32_t>(job->pairs.size() / 2), &job->w, &cx);
    S->t_admit += std::chrono::duration<double>(Clock::now() - ta).count();
    if (s == GD_ERR_OOM) {  // wait for a resident job to finish
      s = GD_OK;
      break;
    }
    const uint64_t bytes = ctx->in_use - before;
    if (s == GD_OK && S->cfg.hbm_budget && S->job_bytes + bytes > S->cfg.hbm_budget && S->job_bytes > 0) {
      gd_complex_destroy(cx);  // over the server's budget: admit later
      break;
    }
    {
      std::lock_guard<std::mutex> lock(S->mu);
      S->queue.pop_front();
      if (s != GD_OK) {
        job->status = GD_JOB_FAILED;
        job->error = s;
        job->t_done = Clock::now();
        S->cv.notify_all();
        s = GD_OK;
        continue;
      }
      job->cx = cx;
      job->slot = free_slot;
      job->status = GD_JOB_RUNNING;
      job->t_admit = Clock::now();
      S->slot_job[free_slot] = job;
    }
    S->job_bytes += bytes;
    S->dirty = true;
    const auto tl = Clock::now();
    s = server_load_slot(S, free_slot, job);
    S->t_load += std::chrono::duration<double>(Clock::now() - tl).count();
    if (s != GD_OK) return s;
    uploaded = true;
  }
  if (uploaded) {
    const cudaError_t e = cudaEventRecord(S->ev_up, S->up);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "server admission event");
    S->upload_pending = true;
  }
  return s;
}

// One tick: one generation of every resident job (continuous batching), the
// admission of queued jobs while it runs, then the retirement of the jobs it
// finished.  With no job resident the admission comes first, so that an idle
// server starts new work in the same tick.
gd_status server_tick(gd_server *S, int *active_out) {
  gd::NvtxRange nvtx_range("server_tick");
  gd_context *ctx = S->ctx;
  const gd_ga_cfg &c = S->cfg.ga;
  GaRun &R = S->arena;
  const int J = S->cfg.max_slots, n = c.pop_size;
  gd_status s = GD_OK;
  auto resident = [&]() {
    int a = 0;
    for (Job *j : S->slot_job) a += j != nullptr;
    return a;
  };
  if (resident() == 0) {
    s = server_admit(S);
    if (s != GD_OK) return s;
  }
  // 1. one generation for the resident jobs
  std::vector<int> slots;
  for (int j = 0; j < J; ++j)
    if (S->slot_job[j]) slots.push_back(j);
  const int active = static_cast<int>(slots.size());
  cudaStream_t st = ctx->stream;
  const auto tg = Clock::now();
  if (active > 0) {
    cudaError_t e = cudaSuccess;
    if (S->upload_pending) {  // the admitted jobs' uploads come first
      e = cudaStreamWaitEvent(st, S->ev_up, 0);
      S->upload_pending = false;
    }
    if (e == cudaSuccess && S->dirty)
      e = cudaMemcpyAsync(S->d_slots, slots.data(), sizeof(int) * active, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "server tick set-up");
    if (S->cfg.precision == GD_PREC_F32 && (S->dirty || !S->bl)) {
      // the argument block only changes when jobs enter or leave a slot
      std::vector<ScoreParams> descs(J);
      bool serial = false, clamp = false;
      for (int j = 0; j < J; ++j) {
        Job *job = S->slot_job[j];
        if (job) {
          descs[j] = make_params(job->cx, R.frames + static_cast<size_t>(j) * n, nullptr, n,
                                 R.energies + static_cast<size_t>(j) * n, c.max_displacement);
          descs[j].skip = &R.state[j].stop;
          serial |= job->cx->serial_overlap;
          clamp |= job->cx->need_clamp;
        } else {
          descs[j] = ScoreParams{};
          descs[j].n_poses = 0;
        }
      }
      if (S->bl) batch_free(ctx, S->bl);
      S->bl = nullptr;
      const auto tp = Clock::now();
      s = batch_prepare(ctx, descs, serial, clamp, ctx->tune_f32_slots ? ctx->tune_f32_slots : kDefaultF32Tune, &S->bl);
      S->t_prepare += std::chrono::duration<double>(Clock::now() - tp).count();
      if (s != GD_OK) return s;
    }
    S->dirty = false;
    const int total = active * n;
    cudaEventRecord(S->ev0, st);
    k_frames<<<(total + 255) / 256, 256, 0, st>>>(R.genes, R.frames, R.job_of, R.state, total, S->d_slots, n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "frames kernel");
    if (S->cfg.precision == GD_PREC_F32) {
      s = batch_launch(ctx, S->bl, st);
    } else {
      for (int j : slots) {
        if (s != GD_OK) break;
        s = launch_score(S->slot_job[j]->cx, R.frames + static_cast<size_t>(j) * n, nullptr, n, GD_PREC_F64,
                         R.energies + static_cast<size_t>(j) * n, st, c.max_displacement);
      }
    }
    if (s != GD_OK) return s;
    GaStepParams P{};
    P.genes = R.genes;
    P.genes_tmp = R.genes_tmp;
    P.energies = R.energies;
    P.state = R.state;
    P.history = R.history;
    P.tour = R.tour;
    P.perm = R.perm;
    P.cross_u = R.cross_u;
    P.mut_u = R.mut_u;
    P.mut_z = R.mut_z;
    P.hof = R.hof;
    P.hof_tmp = R.hof_tmp;
    P.err = ctx->d_err;
    P.slots = S->d_slots;
    P.cfg = c;
    const size_t ga_smem = ga_step_smem(n);
    if (ga_smem > 48 * 1024)
      cudaFuncSetAttribute(k_ga_step, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(ga_smem));
    k_ga_step<<<active, 256, ga_smem, st>>>(P);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, e, "GA step kernel");
    cudaEventRecord(S->ev1, st);
    e = cudaMemcpyAsync(S->h_states, R.state, sizeof(GaJobState) * J, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "server tick");
    // 2. admission while the generation runs
    s = server_admit(S);
    if (s != GD_OK) return s;
    // 3. the generation's end
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "server tick");
    s = check_device_error(ctx);
    if (s != GD_OK) return s;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, S->ev0, S->ev1) == cudaSuccess) S->gpu_busy += 1e-3 * ms;
    S->generations_run += 1;
    S->poses_scored += static_cast<int64_t>(active) * n;
  }
  S->t_gpu += std::chrono::duration<double>(Clock::now() - tg).count();
  const auto tr = Clock::now();
  // 4. retire the jobs this generation finished (only the slots it ran)
  for (int j : slots) {
    Job *job = S->slot_job[j];
    const GaJobState &sj = S->h_states[j];
    if (!job || sj.stop == 0) continue;
    job->generations = sj.gen;
    job->genes.resize(static_cast<size_t>(n) * 6);
    job->energies.resize(n);
    job->history.resize(std::max(c.max_generations, 0));
    cudaError_t e = cudaMemcpy(job->genes.data(), R.genes + static_cast<size_t>(j) * n * 6, sizeof(double) * n * 6,
                               cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(job->energies.data(), R.energies + static_cast<size_t>(j) * n, sizeof(gd_pose_energy) * n,
                     cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && c.max_generations > 0)
      e = cudaMemcpy(job->history.data(), R.history + static_cast<size_t>(j) * c.max_generations,
                     sizeof(double) * c.max_generations, cudaMemcpyDeviceToHost);
    job->hof.resize(R.hof ? sj.hof_n : 0);
    if (e == cudaSuccess && !job->hof.empty())
      e = cudaMemcpy(job->hof.data(), R.hof + static_cast<size_t>(j) * (c.hof_max_size + 1),
                     sizeof(gd_hof_entry) * job->hof.size(), cudaMemcpyDeviceToHost);
    GaJobState freed{0, kStopFree, 0, 0, 0.0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(R.state + j, &freed, sizeof(freed), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "server retire");
    const uint64_t before = ctx->in_use;
    gd_complex_destroy(job->cx);
    S->job_bytes -= std::min<uint64_t>(S->job_bytes, before - ctx->in_use);
    job->cx = nullptr;
    // history entries past the generations this job ran are not its own
    const int valid = std::min(c.max_generations, sj.stop == 1 ? sj.gen + 1 : sj.gen);
    for (int g = std::max(valid, 0); g < c.max_generations; ++g) job->history[g] = NAN;
    S->dirty = true;
    std::lock_guard<std::mutex> lock(S->mu);
    S->slot_job[j] = nullptr;
    job->status = GD_JOB_DONE;
    job->t_done = Clock::now();
    S->completed += 1;
    S->latencies.push_back(std::chrono::duration<double>(job->t_done - job->t_submit).count());
    S->cv.notify_all();
  }
  S->t_retire += std::chrono::duration<double>(Clock::now() - tr).count();
  if (active_out) *active_out = resident();
  return GD_OK;
}

}  // namespace
}  // namespace gd

using gd::Clock;

extern "C" {

gd_status gd_server_default_cfg(gd_server_cfg *cfg) {
  if (!cfg) return GD_ERR_INVALID_ARG;
  cfg->max_slots = 64;
  cfg->hbm_budget = 0;
  gd_ga_default_cfg(&cfg->ga);
  cfg->ga.max_generations = 200;
  cfg->precision = GD_PREC_F32;
  return GD_OK;
}

gd_status gd_server_create(gd_context *ctx, const gd_server_cfg *cfg, gd_server **out) {
  if (!ctx || !cfg || !out) return GD_ERR_INVALID_ARG;
  *out = nullptr;
  const gd_ga_cfg &c = cfg->ga;
  if (cfg->max_slots < 1 || cfg->max_slots > 4096 || c.pop_size < 2 || c.pop_size % 2 || c.elitism > 64 ||
      c.elitism > c.pop_size || c.tournament_size < 1 || c.max_generations < 0 ||
      (cfg->precision != GD_PREC_F32 && cfg->precision != GD_PREC_F64))
    return gd::fail(ctx, GD_ERR_INVALID_ARG, "bad server config");
  cudaSetDevice(ctx->device);
  gd_server *S = new gd_server();
  S->ctx = ctx;
  S->cfg = *cfg;
  gd_status s = gd::server_alloc(S);
  if (s != GD_OK) {
    gd::ga_release(ctx, S->arena);
    gd::server_free_host(S);
    delete S;
    return s;
  }
  *out = S;
  return GD_OK;
}

gd_status gd_server_submit(gd_server *S, const gd_atoms *rec, const gd_atoms *lig, const int32_t *pairs,
                           int32_t n_pairs, const gd_weights *w, uint64_t seed, int64_t *job_id) {
  if (!S || !rec || !lig || !job_id || n_pairs < 0 || (n_pairs > 0 && !pairs)) return GD_ERR_INVALID_ARG;
  gd::Job *job = new gd::Job();
  job->rec.copy(rec);
  job->lig.copy(lig);
  job->pairs.assign(pairs, pairs + 2 * static_cast<size_t>(n_pairs));
  job->w = w ? *w : gd_weights{0.4, 0.05, 3.4, 1.0};
  job->seed = seed;
  job->t_submit = Clock::now();  // latency counts the draws below
  gd::draw_job(S->cfg.ga, job);  // on the caller's thread, not the server's
  std::lock_guard<std::mutex> lock(S->mu);
  if (S->failed != GD_OK) {
    delete job;
    return gd::fail(S->ctx, GD_ERR_STATE, "the server stopped on an error: " + S->fail_msg);
  }
  job->id = S->next_id++;
  if (!S->started_clock) {
    S->t_first = job->t_submit;
    S->started_clock = true;
  }
  S->jobs[job->id] = job;
  S->queue.push_back(job);
  *job_id = job->id;
  S->cv.notify_all();
  return GD_OK;
}

gd_status gd_server_step(gd_server *S, int32_t *active) {
  if (!S) return GD_ERR_INVALID_ARG;
  if (S->running) return gd::fail(S->ctx, GD_ERR_STATE, "the server's own thread is running");
  cudaSetDevice(S->ctx->device);
  return gd::server_tick(S, active);
}

gd_status gd_server_start(gd_server *S) {
  if (!S) return GD_ERR_INVALID_ARG;
  if (S->running) return GD_OK;
  S->running = true;
  S->worker = std::thread([S]() {
    cudaSetDevice(S->ctx->device);
    while (true) {
      {
        std::unique_lock<std::mutex> lock(S->mu);
        bool idle = S->queue.empty();
        for (auto *j : S->slot_job) idle = idle && j == nullptr;
        if (!S->running && idle) break;
        if (idle) S->cv.wait_for(lock, std::chrono::milliseconds(5));
        if (!S->running && S->queue.empty()) {
          bool none = true;
          for (auto *j : S->slot_job) none = none && j == nullptr;
          if (none) break;
        }
      }
      int active = 0;
      const gd_status ts = gd::server_tick(S, &active);
      if (ts != GD_OK) {
        // every resident and queued job fails with the tick's status; later
        // submissions are refused (see gd_server_submit)
        std::lock_guard<std::mutex> lock(S->mu);
        S->failed = ts;
        S->fail_msg = gd_last_error(S->ctx);
        const auto now = gd::Clock::now();
        for (auto &kv : S->jobs)
          if (kv.second->status == GD_JOB_RUNNING || kv.second->status == GD_JOB_QUEUED) {
            kv.second->status = GD_JOB_FAILED;
            kv.second->error = ts;
            kv.second->t_done = now;
          }
        S->queue.clear();
        S->cv.notify_all();
        break;
      }
    }
  });
  return GD_OK;
}

gd_status gd_server_stop(gd_server *S) {
  if (!S) return GD_ERR_INVALID_ARG;
  if (S->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lock(S->mu);
      S->running = false;
      S->cv.notify_all();
    }
    S->worker.join();
  }
  S->running = false;
  return GD_OK;
}

gd_status gd_server_wait(gd_server *S, int64_t job_id, double timeout_s, int32_t *status) {
  if (!S) return GD_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->jobs.find(job_id);
  if (it == S->jobs.end()) return gd::fail(S->ctx, GD_ERR_INVALID_ARG, "unknown job");
  gd::Job *job = it->second;
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
  while (job->status == GD_JOB_QUEUED || job->status == GD_JOB_RUNNING) {
    if (S->cv.wait_until(lock, deadline) == std::cv_status::timeout) break;
  }
  if (status) *status = job->status;
  return (job->status == GD_JOB_DONE || job->status == GD_JOB_FAILED) ? GD_OK : GD_ERR_TIMEOUT;
}

gd_status gd_server_result(gd_server *S, int64_t job_id, gd_job_result *res, double *genes, gd_pose_energy *energies,
                           double *history) {
  if (!S || !res) return GD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->jobs.find(job_id);
  if (it == S->jobs.end()) return gd::fail(S->ctx, GD_ERR_INVALID_ARG, "unknown job");
  gd::Job *job = it->second;
  res->status = job->status;
  res->error = job->error;
  res->generations = job->generations;
  const auto now = Clock::now();
  const auto end = job->status == GD_JOB_DONE || job->status == GD_JOB_FAILED ? job->t_done : now;
  res->latency_s = std::chrono::duration<double>(end - job->t_submit).count();
  res->queue_s = job->status == GD_JOB_QUEUED
                     ? std::chrono::duration<double>(now - job->t_submit).count()
                     : std::chrono::duration<double>(job->t_admit - job->t_submit).count();
  if (job->status == GD_JOB_DONE) {
    if (genes) std::memcpy(genes, job->genes.data(), sizeof(double) * job->genes.size());
    if (energies) std::memcpy(energies, job->energies.data(), sizeof(gd_pose_energy) * job->energies.size());
    if (history) std::memcpy(history, job->history.data(), sizeof(double) * job->history.size());
  }
  return GD_OK;
}

gd_status gd_server_hall_of_fame(gd_server *S, int64_t job_id, gd_hof_entry *entries, int32_t cap, int32_t *count) {
  if (!S || !count || cap < 0 || (cap > 0 && !entries)) return GD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->jobs.find(job_id);
  if (it == S->jobs.end()) return gd::fail(S->ctx, GD_ERR_INVALID_ARG, "unknown job");
  gd::Job *job = it->second;
  if (job->status != GD_JOB_DONE) return gd::fail(S->ctx, GD_ERR_STATE, "the job has not finished");
  *count = static_cast<int32_t>(job->hof.size());
  if (job->hof.size() > static_cast<size_t>(cap)) return GD_ERR_CAPACITY;
  if (!job->hof.empty()) std::memcpy(entries, job->hof.data(), sizeof(gd_hof_entry) * job->hof.size());
  return GD_OK;
}

gd_status gd_server_release(gd_server *S, int64_t job_id) {
  if (!S) return GD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->jobs.find(job_id);
  if (it == S->jobs.end()) return gd::fail(S->ctx, GD_ERR_INVALID_ARG, "unknown job");
  if (it->second->status != GD_JOB_DONE && it->second->status != GD_JOB_FAILED)
    return gd::fail(S->ctx, GD_ERR_STATE, "job still queued or running");
  delete it->second;
  S->jobs.erase(it);
  return GD_OK;
}

gd_status gd_server_get_stats(gd_server *S, gd_server_stats *out) {
  if (!S || !out) return GD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(S->mu);
  out->completed = S->completed;
  out->queued = static_cast<int64_t>(S->queue.size());
  int act = 0;
  for (auto *j : S->slot_job) act += j != nullptr;
  out->resident = act;
  out->generations_run = S->generations_run;
  out->poses_scored = S->poses_scored;
  out->device_bytes = S->job_bytes;
  std::vector<double> l = S->latencies;
  std::sort(l.begin(), l.end());
  auto pct = [&](double p) {
    if (l.empty()) return 0.0;
    const size_t k = static_cast<size_t>(std::ceil(p * l.size())) - 1;
    return l[std::min(k, l.size() - 1)];
  };
  out->latency_p50_s = pct(0.50);
  out->latency_p99_s = pct(0.99);
  out->latency_max_s = l.empty() ? 0.0 : l.back();
  out->gpu_busy_s = S->gpu_busy;
  out->elapsed_s = S->started_clock ? std::chrono::duration<double>(Clock::now() - S->t_first).count() : 0.0;
  return GD_OK;
}

gd_status gd_server_destroy(gd_server *S) {
  if (!S) return GD_ERR_INVALID_ARG;
  gd_server_stop(S);
  gd::trace("server: admit (complex create)", S->t_admit);
  gd::trace("server: load (draws + uploads)", S->t_load);
  gd::trace("server: batch prepare", S->t_prepare);
  gd::trace("server: kernels + sync (incl. prepare)", S->t_gpu);
  gd::trace("server: retire", S->t_retire);
  cudaSetDevice(S->ctx->device);
  cudaStreamSynchronize(S->ctx->stream);
  if (S->up) cudaStreamSynchronize(S->up);
  for (auto *j : S->slot_job)
    if (j && j->cx) gd_complex_destroy(j->cx);
  if (S->bl) gd::batch_free(S->ctx, S->bl);
  gd::ga_release(S->ctx, S->arena);
  gd::server_free_host(S);
  for (auto &kv : S->jobs) delete kv.second;
  delete S;
  return GD_OK;
}

}  // extern "C"
