// Likelihood losses on the probabilistic front end's distributions and
// their gradients with respect to the distributions:
//
// - ProbabilisticLossStrategy.compute (optimize/strategies.py:338-567):
//   each target hit is matched to the simulated pixel list by a lower-bound
//   search (the list is sorted, jnp.searchsorted), its occurrence index
//   within its run of equal pixel ids (compute_occurrence_indices,
//   strategies.py:14-40) picks the hit row of the distributions, and the
//   tick's log-probability (clamped below at log(eps)) and the distribution's
//   charge at that tick enter two log-likelihood sums T (ticks, with a
//   log(eps) penalty per unmatched hit) and C (Gaussian charge term);
//   loss = sqrt(T * C).
// - llhd_loss (src/larndsim/losses_jax.py:414-441): per row, log(p[tick] +
//   eps) or log(no_hit_prob + eps) past tick T - 3, plus a Gaussian charge
//   term.
// - compute_occurrence_indices on its own (a max-scan of run starts).
//
// The work is one gather per target hit: latency-bound, tiny next to the
// front end that makes the distributions.  The gradient kernels write the
// dense cotangent arrays the front end's adjoint takes (zeroed, then one
// atomic add per hit: several hits can read the same entry).  Indices follow
// jax.numpy indexing: negative counts from the end, out of range clamps.
// Per-hit terms are float32 in the reference's operation order; the sums are
// accumulated in double per block and reduced in a fixed order.
#include "lsim_internal.cuh"

namespace lsim {
namespace {

constexpr int kHitThreads = 256;
constexpr int kRunTile = 1024;

__device__ __forceinline__ int64_t jax_index(int64_t i, int64_t n) {
  if (i < 0) i += n;
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// adc2charge (losses_jax.py:380-383) in its float32 operation order
__device__ __forceinline__ float adc_to_charge(const LsimParams &p, float dw) {
  return __fmul_rn(__fdiv_rn(__fsub_rn(__fadd_rn(__fmul_rn(__fdiv_rn(dw, p.adc_counts), p.vref_minus_cm), p.v_cm),
                                       p.v_pedestal),
                             p.gain),
                   1e-3f);
}

// block sum of up to three doubles into part[blockIdx.x * 3 + k]
__device__ void block_sum3(double a, double b, double c, double *part) {
  __shared__ double red[3][kHitThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = a;
    red[1][threadIdx.x >> 5] = b;
    red[2][threadIdx.x >> 5] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (int k = 0; k < kHitThreads / 32; ++k) {
      s0 += red[0][k];
      s1 += red[1][k];
      s2 += red[2][k];
    }
    part[3 * (int64_t)blockIdx.x + 0] = s0;
    part[3 * (int64_t)blockIdx.x + 1] = s1;
    part[3 * (int64_t)blockIdx.x + 2] = s2;
  }
}

struct ProbLoss {
  LsimParams p;
  const int32_t *sim;       // [n_pix] sorted pixel ids
  int64_t n_pix;
  int32_t n_values, n_ticks;
  const float *log_prob, *adcs;  // [n_pix][n_values][n_ticks]
  const int32_t *tgt_pix, *tgt_tick;
  const float *tgt_adc;
  int64_t n_hits;
  float s, half_log, log_eps;    // sigma/1000, 0.5 log(2 pi s^2), log(eps) as float32
};

struct HitTerm {
  int64_t pos;     // flat index of the entry read
  bool valid, miss;
  float lp, llt, llc, r;
};

__device__ HitTerm prob_hit(const ProbLoss &a, int64_t i) {
  HitTerm h;
  const int32_t id = a.tgt_pix[i];
  int64_t lo = 0, hi = a.n_pix;   // first index with sim[idx] >= id
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a.sim[mid] < id) lo = mid + 1; else hi = mid;
  }
  const int64_t safe = lo < a.n_pix ? lo : a.n_pix - 1;
  const int32_t found = a.sim[safe];
  h.miss = found != id;
  h.valid = !h.miss && id >= 0;
  // occurrence index, clamped to the hit rows the gather can read
  int32_t occ = 0;
  for (int64_t j = i; occ < a.n_values - 1 && j > 0 && a.tgt_pix[j - 1] == id; --j) ++occ;
  const int64_t tick = jax_index(a.tgt_tick[i], a.n_ticks);
  h.pos = (safe * a.n_values + occ) * (int64_t)a.n_ticks + tick;
  h.lp = a.log_prob[h.pos];
  h.llt = h.valid ? fmaxf(h.lp, a.log_eps) : 0.0f;
  const float tq = adc_to_charge(a.p, a.tgt_adc[i]);
  const float hq = h.valid ? adc_to_charge(a.p, a.adcs[h.pos]) : 0.0f;
  h.r = __fdiv_rn(__fsub_rn(tq, hq), a.s);
  h.llc = __fsub_rn(__fmul_rn(-0.5f, __fmul_rn(h.r, h.r)), a.half_log);
  return h;
}

__global__ void __launch_bounds__(kHitThreads) k_prob_llhd_hits(ProbLoss a, double *part) {
  const int64_t i = (int64_t)blockIdx.x * kHitThreads + threadIdx.x;
  double t = 0, c = 0, m = 0;
  if (i < a.n_hits) {
    const HitTerm h = prob_hit(a, i);
    t = h.llt;
    c = h.llc;
    m = h.miss ? 1.0 : 0.0;
  }
  block_sum3(t, c, m, part);
}

// out = [loss, -C, -T, -penalty]; coef = [dL/dT, dL/dC] times the cotangent
__global__ void k_prob_llhd_reduce(const double *part, int64_t n_blocks, float log_eps, const float *g_loss,
                                   float *out, float *coef) {
  __shared__ double red[3][32];
  double t = 0, c = 0, m = 0;
  for (int64_t b = threadIdx.x; b < n_blocks; b += blockDim.x) {
    t += part[3 * b];
    c += part[3 * b + 1];
    m += part[3 * b + 2];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t += __shfl_xor_sync(0xffffffffu, t, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    m += __shfl_xor_sync(0xffffffffu, m, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = t;
    red[1][threadIdx.x >> 5] = c;
    red[2][threadIdx.x >> 5] = m;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double T = 0, C = 0, M = 0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
    T += red[0][k];
    C += red[1][k];
    M += red[2][k];
  }
  const float penalty = __fmul_rn(log_eps, (float)M);
  const float Tf = (float)(T + (double)penalty), Cf = (float)C;
  const float prod = __fmul_rn(Tf, Cf);
  const float root = sqrtf(prod);
  out[0] = root;
  out[1] = -Cf;
  out[2] = -Tf;
  out[3] = -penalty;
  if (coef) {
    const float g = g_loss ? g_loss[0] : 1.0f;
    const float half = __fdiv_rn(__fmul_rn(g, 0.5f), root);   // d sqrt(x) = g * 0.5 / sqrt(x)
    coef[0] = __fmul_rn(half, Cf);
    coef[1] = __fmul_rn(half, Tf);
  }
}

__global__ void __launch_bounds__(kHitThreads) k_prob_llhd_scatter(ProbLoss a, const float *coef, float *g_lp,
                                                                    float *g_ad) {
  const int64_t i = (int64_t)blockIdx.x * kHitThreads + threadIdx.x;
  if (i >= a.n_hits) return;
  const HitTerm h = prob_hit(a, i);
  if (!h.valid) return;
  // lax.max's derivative: 1 to the larger operand, 1/2 each on a tie
  const float tie = h.lp > a.log_eps ? 1.0f : (h.lp == a.log_eps ? 0.5f : 0.0f);
  if (g_lp && tie != 0.0f) atomicAdd(g_lp + h.pos, __fmul_rn(coef[0], tie));
  if (g_ad) {
    // d llc / d hq = r / s, then adc2charge's slope in reverse order
    float d = __fdiv_rn(__fmul_rn(coef[1], h.r), a.s);
    d = __fdiv_rn(__fmul_rn(__fdiv_rn(__fmul_rn(d, 1e-3f), a.p.gain), a.p.vref_minus_cm), a.p.adc_counts);
    atomicAdd(g_ad + h.pos, d);
  }
}

// ---- llhd_loss

struct Llhd {
  const float *tpd, *nohit, *cd, *cmc;
  const int32_t *ticks;
  int64_t n_rows;
  int32_t n_ticks;
  float sigma, half_log, eps;
};

__global__ void __launch_bounds__(kHitThreads) k_llhd_rows(Llhd a, double *part) {
  const int64_t i = (int64_t)blockIdx.x * kHitThreads + threadIdx.x;
  double v = 0;
  if (i < a.n_rows) {
    const int32_t t = a.ticks[i];
    const int64_t pos = i * a.n_ticks + jax_index(t, a.n_ticks);
    const bool on = t < a.n_ticks - 3;
    const float llt = on ? logf(__fadd_rn(a.tpd[pos], a.eps)) : logf(__fadd_rn(a.nohit[i], a.eps));
    const float r = __fdiv_rn(__fsub_rn(a.cmc[i], a.cd[pos]), a.sigma);
    const float llc = on ? __fsub_rn(__fmul_rn(-0.5f, __fmul_rn(r, r)), a.half_log) : 0.0f;
    v = __fadd_rn(llt, llc);
  }
  block_sum3(v, 0.0, 0.0, part);
}

__global__ void k_llhd_reduce(const double *part, int64_t n_blocks, float *out) {
  __shared__ double red[32];
  double v = 0;
  for (int64_t b = threadIdx.x; b < n_blocks; b += blockDim.x) v += part[3 * b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x != 0) return;
  double s = 0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
  out[0] = -(float)s;
}

__global__ void __launch_bounds__(kHitThreads) k_llhd_grad(Llhd a, const float *g_loss, float *g_tpd,
                                                            float *g_nohit, float *g_cd, float *g_cmc) {
  const int64_t i = (int64_t)blockIdx.x * kHitThreads + threadIdx.x;
  if (i >= a.n_rows) return;
  const float g = g_loss ? -g_loss[0] : -1.0f;   // loss = -sum
  const int32_t t = a.ticks[i];
  const int64_t pos = i * a.n_ticks + jax_index(t, a.n_ticks);
  const bool on = t < a.n_ticks - 3;
  if (g_tpd && on) atomicAdd(g_tpd + pos, __fdiv_rn(g, __fadd_rn(a.tpd[pos], a.eps)));
  if (g_nohit) g_nohit[i] = on ? 0.0f : __fdiv_rn(g, __fadd_rn(a.nohit[i], a.eps));
  const float r = __fdiv_rn(__fsub_rn(a.cmc[i], a.cd[pos]), a.sigma);
  const float d = on ? __fdiv_rn(__fmul_rn(g, -r), a.sigma) : 0.0f;   // d llc / d cmc = -r / sigma
  if (g_cd && on) atomicAdd(g_cd + pos, -d);
  if (g_cmc) g_cmc[i] = d;
}

// ---- occurrence indices: i - (last run start at or before i)

__device__ __forceinline__ int32_t block_max_scan(int32_t v, int32_t *sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v = max(v, u);
  }
  if (lane == 31) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int32_t w = lane < (int)(blockDim.x >> 5) ? sm[lane] : -1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w = max(w, u);
    }
    sm[lane] = w;
  }
  __syncthreads();
  return warp > 0 ? max(v, sm[warp - 1]) : v;
}

__global__ void __launch_bounds__(kRunTile) k_runs_tile(const int32_t *ids, int32_t n, int32_t *start,
                                                          int32_t *tile_max) {
  __shared__ int32_t sm[32];
  const int64_t i = (int64_t)blockIdx.x * kRunTile + threadIdx.x;
  int32_t v = -1;
  if (i < n) v = (i == 0 || ids[i] != ids[i - 1]) ? (int32_t)i : -1;
  v = block_max_scan(v, sm);
  if (i < n) start[i] = v;
  if (threadIdx.x == kRunTile - 1) tile_max[blockIdx.x] = v;
}

// inclusive max-scan of the tiles' largest run starts, in place
__global__ void __launch_bounds__(kRunTile) k_runs_carry(int32_t *tile_max, int32_t n_tiles) {
  __shared__ int32_t sm[32];
  __shared__ int32_t last;
  int32_t carry = -1;
  for (int32_t base = 0; base < n_tiles; base += kRunTile) {
    const int32_t b = base + (int32_t)threadIdx.x;
    const int32_t v = b < n_tiles ? tile_max[b] : -1;
    const int32_t inc = max(block_max_scan(v, sm), carry);
    if (b < n_tiles) tile_max[b] = inc;
    if (threadIdx.x == kRunTile - 1) last = inc;
    __syncthreads();
    carry = last;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kRunTile) k_runs_apply(const int32_t *start, const int32_t *tile_incl, int32_t n,
                                                           int32_t *out) {
  const int64_t i = (int64_t)blockIdx.x * kRunTile + threadIdx.x;
  if (i >= n) return;
  const int32_t before = blockIdx.x > 0 ? tile_incl[blockIdx.x - 1] : -1;
  out[i] = (int32_t)i - max(start[i], before);
}

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

size_t prob_llhd_workspace_bytes(int64_t n_hits) {
  const int64_t nb = (n_hits + kHitThreads - 1) / kHitThreads + 1;
  return al256(sizeof(double) * 3 * (size_t)nb) + al256(2 * sizeof(float));
}

int run_prob_llhd(const LsimParams &p, const int32_t *sim, int64_t n_pix, int32_t n_values, int32_t n_ticks,
                  const float *log_prob, const float *adcs, const int32_t *tgt_pix, const int32_t *tgt_tick,
                  const float *tgt_adc, int64_t n_hits, double sigma_charge, double eps, const float *g_loss,
                  float *out, float *g_log_prob, float *g_adcs, void *ws, cudaStream_t st) {
  ProbLoss a{};
  a.p = p;
  a.sim = sim;
  a.n_pix = n_pix;
  a.n_values = n_values;
  a.n_ticks = n_ticks;
  a.log_prob = log_prob;
  a.adcs = adcs;
  a.tgt_pix = tgt_pix;
  a.tgt_tick = tgt_tick;
  a.tgt_adc = tgt_adc;
  a.n_hits = n_hits;
  const double s = sigma_charge / 1000.0;
  a.s = (float)s;
  a.half_log = 0.5f * logf((float)(2.0 * 3.14159265358979323846 * (s * s)));
  a.log_eps = logf((float)eps);
  const int64_t nb = (n_hits + kHitThreads - 1) / kHitThreads;
  char *b = static_cast<char *>(ws);
  double *part = reinterpret_cast<double *>(b);
  float *coef = reinterpret_cast<float *>(b + al256(sizeof(double) * 3 * (size_t)(nb + 1)));
  if (nb > 0) k_prob_llhd_hits<<<(unsigned)nb, kHitThreads, 0, st>>>(a, part);
  const bool grad = g_log_prob || g_adcs;
  k_prob_llhd_reduce<<<1, 1024, 0, st>>>(part, nb, a.log_eps, g_loss, out, grad ? coef : nullptr);
  if (!grad) return LSIM_OK;
  const size_t dense = sizeof(float) * (size_t)n_pix * (size_t)n_values * (size_t)n_ticks;
  if (g_log_prob && cudaMemsetAsync(g_log_prob, 0, dense, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (g_adcs && cudaMemsetAsync(g_adcs, 0, dense, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (nb > 0) k_prob_llhd_scatter<<<(unsigned)nb, kHitThreads, 0, st>>>(a, coef, g_log_prob, g_adcs);
  return LSIM_OK;
}

size_t llhd_workspace_bytes(int64_t n_rows) {
  const int64_t nb = (n_rows + kHitThreads - 1) / kHitThreads + 1;
  return al256(sizeof(double) * 3 * (size_t)nb);
}

int run_llhd(const float *tpd, const int32_t *ticks, const float *nohit, const float *cd, const float *cmc,
             int64_t n_rows, int32_t n_ticks, double sigma, const float *g_loss, float *out, float *g_tpd,
             float *g_nohit, float *g_cd, float *g_cmc, void *ws, cudaStream_t st) {
  Llhd a{tpd, nohit, cd, cmc, ticks, n_rows, n_ticks, (float)sigma,
         0.5f * logf((float)(2.0 * 3.14159265358979323846 * (sigma * sigma))), 1e-10f};
  const int64_t nb = (n_rows + kHitThreads - 1) / kHitThreads;
  double *part = static_cast<double *>(ws);
  if (nb > 0) k_llhd_rows<<<(unsigned)nb, kHitThreads, 0, st>>>(a, part);
  k_llhd_reduce<<<1, 1024, 0, st>>>(part, nb, out);
  if (!(g_tpd || g_nohit || g_cd || g_cmc)) return LSIM_OK;
  const size_t dense = sizeof(float) * (size_t)n_rows * (size_t)n_ticks;
  if (g_tpd && cudaMemsetAsync(g_tpd, 0, dense, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (g_cd && cudaMemsetAsync(g_cd, 0, dense, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (nb > 0) k_llhd_grad<<<(unsigned)nb, kHitThreads, 0, st>>>(a, g_loss, g_tpd, g_nohit, g_cd, g_cmc);
  return LSIM_OK;
}

size_t occurrence_workspace_bytes(int64_t n) {
  const int64_t tiles = (n + kRunTile - 1) / kRunTile + 1;
  return al256(sizeof(int32_t) * (size_t)(n + 1)) + al256(sizeof(int32_t) * (size_t)tiles);
}

int run_occurrence(const int32_t *ids, int32_t n, int32_t *out, void *ws, cudaStream_t st) {
  if (n == 0) return LSIM_OK;
  const int32_t tiles = (n + kRunTile - 1) / kRunTile;
  int32_t *start = static_cast<int32_t *>(ws);
  int32_t *tile_max = reinterpret_cast<int32_t *>(static_cast<char *>(ws) + al256(sizeof(int32_t) * (size_t)(n + 1)));
  k_runs_tile<<<tiles, kRunTile, 0, st>>>(ids, n, start, tile_max);
  k_runs_carry<<<1, kRunTile, 0, st>>>(tile_max, tiles);
  k_runs_apply<<<tiles, kRunTile, 0, st>>>(start, tile_max, n, out);
  return LSIM_OK;
}

}  // namespace lsim
