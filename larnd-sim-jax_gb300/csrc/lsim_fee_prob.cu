// Probabilistic self-trigger front end: the beam search of
// get_adc_values_average_noise_vmap (src/larndsim/fee_jax.py:386-461) with
// its step _find_one_hit_step (:334-384) and log_diff_ndtr (:33-53), plus
// the per-hit reductions of get_average_hit_values (:463-480).
//
// One 256-thread block per pixel (persistent over pixels).  The block keeps
// the pixel's cumulative charge q, its running maximum and its suffix
// maximum in shared memory; because max(x - c) = max(x) - c holds exactly
// in floating point, the per-path running maxima of q - c are read from the
// two shared arrays instead of being rescanned for each of the K paths.
// For each of the H hit steps the block walks the K paths; per path it
// tabulates log Phi of (q - c - thr)/sigma and of the running maximum over
// all ticks, then every thread folds its 8 ticks into three online
// log-sum-exp accumulators (hit, total, selection).  A block top-K over the
// selection values (largest first, lower tick first on ties, as lax.top_k)
// gives the next K paths.  The reference stops the whole batch once no pixel
// keeps a total path probability above stop_threshold; the step kernel
// records per step whether any pixel stayed active and a second kernel
// blanks the steps the reference would not have run.
#include "lsim_internal.cuh"
#include "lsim_fee.cuh"

namespace lsim {
namespace {

constexpr int kProbThreads = 256;
constexpr int kProbTicks = 8;   // ticks per thread: up to 2048 ticks
constexpr int kProbMaxT = kProbThreads * kProbTicks;
constexpr int kProbMaxPaths = 32;
constexpr int kProbArrays = 7;  // q, running max, suffix max, esperance, soft-where weight, log Phi(q), log Phi(max)
constexpr float kProbFloor = -1000.0f;

// ---------------------------------------------------------------- special functions
// jax.scipy.special.ndtr / log_ndtr in float32 (the published piecewise
// form: erf near zero and erfc in the tails for ndtr; -ndtr(-x) above 5,
// log(ndtr(x)) down to -10, the order-3 asymptotic series below).

__device__ __forceinline__ float ndtr_f(float x) {
  const float hs2 = 0.70710678118654752f;
  const float w = x * hs2;
  const float z = fabsf(w);
  const float y = z < hs2 ? 1.0f + erff(w) : (w > 0.0f ? 2.0f - erfcf(z) : erfcf(z));
  return 0.5f * y;
}

__device__ __forceinline__ float log_ndtr_f(float x) {
  if (x > 5.0f) return -ndtr_f(-x);
  if (x > -10.0f) return logf(ndtr_f(x));
  const float x2 = x * x;
  const float log_scale = (-(x2 / 2.0f) - logf(-x)) - 0.918938533204672742f;   // 0.5 log(2 pi)
  const float x4 = x2 * x2;
  const float x6 = x4 * x2;
  const float odd = 1.0f / x2 + 15.0f / x6;
  const float even = 3.0f / x4;
  return log_scale + logf((1.0f + even) - odd);
}

// jax.nn.softplus = logaddexp(y, 0) = max(y, 0) + log1p(exp(-|y|)).  For
// |y| > 110 exp(-|y|) is 0 in float32, so the value is exactly max(y, 0).
__device__ __forceinline__ float softplus_f(float y) {
  if (fabsf(y) > 110.0f) return fmaxf(y, 0.0f);
  return fmaxf(y, 0.0f) + log1pf(expf(-fabsf(y)));
}

__device__ __forceinline__ float sigmoid_f(float x) { return 1.0f / (1.0f + expf(-x)); }

// log(Phi(a) - Phi(b)) with the reference's smooth clamps; la, lb = log_ndtr(a), log_ndtr(b)
__device__ __forceinline__ float log_diff_ndtr_f(float a, float b, float la, float lb) {
  const float safe = a > b ? lb - la : -1.0f;
  const float neg = -expm1f(safe);
  const float neg_safe = 1e-30f + softplus_f((neg - 1e-30f) * 1e10f) / 1e10f;
  // neg_safe >= 1e-30, so lt >= -69.1 and the clamp's softplus argument
  // (lt + 100) * 10 >= 309: softplus is the identity there
  const float lt = logf(neg_safe);
  const float lts = -100.0f + ((lt + 100.0f) * 10.0f) / 10.0f;
  const float lp = la + lts;
  const float w = sigmoid_f((a - b) * 1000.0f);
  return w * lp + (1.0f - w) * kProbFloor;
}

// online log-sum-exp: m = running maximum, s = sum of exp(x - m)
__device__ __forceinline__ void lse_add(float &m, float &s, float x) {
  if (x > m) {
    s = s * expf(m - x) + 1.0f;
    m = x;
  } else {
    s += expf(x - m);
  }
}

__device__ __forceinline__ float lse_final(float m, float s) { return logf(s) + m; }

__device__ __forceinline__ bool better(float va, int ia, float vb, int ib) {
  return va > vb || (va == vb && ia < ib);
}

// ---------------------------------------------------------------- block scans over a pixel row

// in-place inclusive scan of a[0..n) with op (sum, max) or a suffix max;
// each thread scans a contiguous chunk of kProbTicks, warps and the block
// combine the chunk totals.
enum ScanOp { kScanSum = 0, kScanMax = 1, kScanSuffixMax = 2 };

template <int OP>
__device__ void block_scan_row(float *a, int n, float *red) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  float v[kProbTicks];
  const int base = OP == kScanSuffixMax ? n - (tid + 1) * kProbTicks : tid * kProbTicks;
  float run = OP == kScanSum ? 0.0f : -INFINITY;
#pragma unroll
  for (int i = 0; i < kProbTicks; ++i) {
    // suffix max walks its chunk from the right
    const int t = OP == kScanSuffixMax ? base + kProbTicks - 1 - i : base + i;
    const bool ok = t >= 0 && t < n;
    const float x = ok ? a[t] : (OP == kScanSum ? 0.0f : -INFINITY);
    run = OP == kScanSum ? run + x : fmaxf(run, x);
    v[i] = run;
  }
  // exclusive prefix of the chunk totals across the block
  float incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl = OP == kScanSum ? incl + y : fmaxf(incl, y);
  }
  if (lane == 31) red[wid] = incl;
  __syncthreads();
  float carry = OP == kScanSum ? 0.0f : -INFINITY;
  for (int w = 0; w < wid; ++w) carry = OP == kScanSum ? carry + red[w] : fmaxf(carry, red[w]);
  float ex = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) ex = OP == kScanSum ? 0.0f : -INFINITY;
  const float pre = OP == kScanSum ? carry + ex : fmaxf(carry, ex);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kProbTicks; ++i) {
    const int t = OP == kScanSuffixMax ? base + kProbTicks - 1 - i : base + i;
    if (t >= 0 && t < n) a[t] = OP == kScanSum ? pre + v[i] : fmaxf(pre, v[i]);
  }
  __syncthreads();
}

__device__ __forceinline__ float block_sum(float v, float *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  float t = 0.0f;
#pragma unroll
  for (int w = 0; w < kProbThreads / 32; ++w) t += red[w];
  return t;
}

struct ProbArgs {
  LsimParams p;
  const float *wfs;
  int64_t n_pix;
  int T, K, interval;
  float z, thr, log_stop;
  float *log_prob, *charge, *e_tick, *e_adc, *lam;
  int32_t *step_active;   // [H]: some pixel kept a total path probability above the stop level after step h
};

__global__ void __launch_bounds__(kProbThreads, 3) k_fee_prob(ProbArgs a) {
  extern __shared__ __align__(16) float sm[];
  float *qs = sm, *cm = qs + kProbMaxT, *cr = cm + kProbMaxT, *esp = cr + kProbMaxT, *sw = esp + kProbMaxT;
  float *LQ = sw + kProbMaxT, *LM = LQ + kProbMaxT;
  __shared__ float red[kProbThreads / 32];
  __shared__ float red_v[kProbThreads / 32];
  __shared__ int red_i[kProbThreads / 32];
  __shared__ float pc[kProbMaxPaths], plp[kProbMaxPaths], nc[kProbMaxPaths], nlp[kProbMaxPaths];
  __shared__ int pskip[kProbMaxPaths];
  __shared__ int top_t;

  const LsimParams &p = a.p;
  const int T = a.T, K = a.K, H = p.max_adc_values, tid = threadIdx.x;
  const float z = a.z, thr = a.thr;
  auto shifted = [&](int t) { return min(t + a.interval + 1, T - 1); };

  for (int64_t pix = blockIdx.x; pix < a.n_pix; pix += gridDim.x) {
    const float *w = a.wfs + pix * T;
    for (int t = tid; t < T; t += kProbThreads) qs[t] = w[t] * p.t_sampling;
    __syncthreads();
    block_scan_row<kScanSum>(qs, T, red);
    for (int t = tid; t < T; t += kProbThreads) cm[t] = cr[t] = qs[t];
    __syncthreads();
    block_scan_row<kScanMax>(cm, T, red);
    block_scan_row<kScanSuffixMax>(cr, T, red);
    for (int t = tid; t < T - 1; t += kProbThreads) {
      const float e = (qs[shifted(t)] + thr) - 0.5f * (qs[t + 1] + qs[t]);
      esp[t] = e;
      sw[t] = sigmoid_f((e - thr) * 10.0f);
    }
    if (tid < K) {
      pc[tid] = 0.0f;
      plp[tid] = tid == 0 ? 0.0f : kProbFloor;
    }
    __syncthreads();

    for (int h = 0; h < H; ++h) {
      // paths whose charge repeats that of a path more than 110 log units
      // likelier add exp(< -110) = 0 to every float32 log-sum-exp: skip them
      if (tid < K) {
        int s = 0;
        for (int j = 0; j < K; ++j)
          if (j != tid && pc[j] == pc[tid] && plp[j] > plp[tid] + 110.0f) s = 1;
        pskip[tid] = s;
      }
      float hm[kProbTicks], hs[kProbTicks], dm[kProbTicks], ds[kProbTicks], sm_[kProbTicks], ss[kProbTicks];
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        hm[i] = dm[i] = sm_[i] = -INFINITY;
        hs[i] = ds[i] = ss[i] = 0.0f;
      }
      __syncthreads();
      for (int k = 0; k < K; ++k) {
        if (pskip[k]) continue;
        const float c = pc[k], lp = plp[k];
        for (int t = tid; t < T; t += kProbThreads) {
          LQ[t] = log_ndtr_f(((qs[t] - c) - thr) * z);
          LM[t] = log_ndtr_f(((cm[t] - c) - thr) * z);
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kProbTicks; ++i) {
          const int t = tid + i * kProbThreads;
          if (t < T - 1) {
            const int s = shifted(t);
            const float zm0 = ((cm[t] - c) - thr) * z, zm1 = ((cm[t + 1] - c) - thr) * z;
            const float lg = log_diff_ndtr_f(zm1, zm0, LM[t + 1], LM[t]);
            const float zq0 = ((qs[t] - c) - thr) * z, zqs = ((qs[s] - c) - thr) * z;
            float le = log_diff_ndtr_f(zqs, zq0, LQ[s], LQ[t]);
            le = fminf(le, lg);
            le = kProbFloor + softplus_f(le - kProbFloor);
            le = sw[t] * le + (1.0f - sw[t]) * kProbFloor;
            lse_add(hm[i], hs[i], le + lp);
            lse_add(dm[i], ds[i], lg + lp);
            const int fe = min(s + a.interval + 1, T - 1);
            const float x = (((cr[fe] - c) - (qs[min(s + 1, T - 1)] - c)) - thr) * z;
            lse_add(sm_[i], ss[i], (lg + log_ndtr_f(x)) + lp);
          }
        }
        __syncthreads();
      }
      // step outputs and the per-hit reductions
      float l_sum = 0.0f, t_sum = 0.0f, a_sum = 0.0f;
      const int64_t row = (pix * H + h) * (int64_t)(T - 1);
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        const int t = tid + i * kProbThreads;
        if (t < T - 1) {
          const float hit = lse_final(hm[i], hs[i]);
          dm[i] = lse_final(dm[i], ds[i]);
          sm_[i] = lse_final(sm_[i], ss[i]);
          if (a.log_prob) a.log_prob[row + t] = hit;
          if (a.charge) a.charge[row + t] = esp[t];
          const float pr = expf(hit);
          l_sum += pr;
          t_sum += (float)t * pr;
          a_sum += digitize(p, esp[t]) * pr;
        }
      }
      if (a.lam) {
        const float L = block_sum(l_sum, red);
        const float Ts = block_sum(t_sum, red);
        const float As = block_sum(a_sum, red);
        if (tid == 0) {
          const float den = fmaxf(L, 1e-10f);
          a.lam[pix * H + h] = L;
          a.e_tick[pix * H + h] = Ts / den;
          a.e_adc[pix * H + h] = As / den;
        }
      }
      // top-K ticks by selection value -> next paths
      unsigned taken = 0;
      for (int r = 0; r < K; ++r) {
        float bv = -INFINITY;
        int bi = 0x7fffffff;
#pragma unroll
        for (int i = 0; i < kProbTicks; ++i) {
          const int t = tid + i * kProbThreads;
          if (t < T - 1 && !(taken >> i & 1u) && better(sm_[i], t, bv, bi)) {
            bv = sm_[i];
            bi = t;
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (better(ov, oi, bv, bi)) {
            bv = ov;
            bi = oi;
          }
        }
        if ((tid & 31) == 0) {
          red_v[tid >> 5] = bv;
          red_i[tid >> 5] = bi;
        }
        __syncthreads();
        if (tid == 0) {
          float v = red_v[0];
          int ix = red_i[0];
          for (int w2 = 1; w2 < kProbThreads / 32; ++w2)
            if (better(red_v[w2], red_i[w2], v, ix)) {
              v = red_v[w2];
              ix = red_i[w2];
            }
          top_t = ix;
        }
        __syncthreads();
        const int tt = top_t;
        if (tt >= 0 && tt < T - 1 && (tt % kProbThreads) == tid) {
          const int ii = tt / kProbThreads;
          float d = 0.0f;
#pragma unroll
          for (int i = 0; i < kProbTicks; ++i)
            if (i == ii) d = dm[i];
          taken |= 1u << ii;
          nlp[r] = d;
          nc[r] = qs[min(shifted(tt) + 1, T - 1)];
        }
        __syncthreads();
      }
      if (tid < 32) {
        const float v = tid < K ? nlp[tid] : -INFINITY;
        float m = v;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        const float mm = isfinite(m) ? m : 0.0f;
        float s = tid < K ? expf(v - mm) : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (tid < K) {
          pc[tid] = nc[tid];
          plp[tid] = nlp[tid];
        }
        if (tid == 0 && logf(s) + mm > a.log_stop && !*(volatile int32_t *)(a.step_active + h))
          atomicOr(a.step_active + h, 1);
      }
      __syncthreads();
    }
  }
}

// Steps after the first one that left no pixel active were not run by the
// reference: their log-probabilities are -1000 and their charges 0, and so
// are the reductions (exp(-1000) = 0 in float32).
__global__ void k_fee_prob_mask(ProbArgs a, int H) {
  int first = H;
  for (int h = 1; h < H; ++h)
    if (!a.step_active[h - 1]) {
      first = h;
      break;
    }
  if (first >= H) return;
  const int64_t T1 = a.T - 1;
  const int64_t rows = a.n_pix * (int64_t)(H - first);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < rows * T1; e += stride) {
    const int64_t r = e / T1, t = e - r * T1;
    const int64_t pix = r / (H - first), h = first + r % (H - first);
    const int64_t o = (pix * H + h) * T1 + t;
    if (a.log_prob) a.log_prob[o] = kProbFloor;
    if (a.charge) a.charge[o] = 0.0f;
    if (t == 0 && a.lam) {
      a.lam[pix * H + h] = 0.0f;
      a.e_tick[pix * H + h] = 0.0f;
      a.e_adc[pix * H + h] = 0.0f;
    }
  }
}

}  // namespace

size_t fee_prob_workspace_bytes(int32_t max_adc_values) {
  return ((size_t)(max_adc_values > 0 ? max_adc_values : 1) * sizeof(int32_t) + 255) & ~size_t(255);
}

int run_fee_prob(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                 float stop_threshold, float *log_prob, float *charge, float *e_tick, float *e_adc, float *lam,
                 void *ws, cudaStream_t st) {
  if (n_t < 3 || n_t > kProbMaxT) return set_error(LSIM_ERR_UNSUPPORTED, "probabilistic FEE: n_t must be in [3, 2048]");
  if (n_paths < 1 || n_paths > kProbMaxPaths || n_paths > n_t - 1)
    return set_error(LSIM_ERR_UNSUPPORTED, "probabilistic FEE: fee_paths_scaling must be in [1, min(32, n_t - 1)]");
  if (!(p.reset_noise > 0.0f)) return set_error(LSIM_ERR_INVALID, "probabilistic FEE: RESET_NOISE_CHARGE must be > 0");
  ProbArgs a;
  a.p = p;
  a.wfs = wfs;
  a.n_pix = n_pix;
  a.T = n_t;
  a.K = n_paths;
  a.interval = p.fee_interval;
  a.z = (float)(1.0 / (double)p.reset_noise);
  a.thr = p.threshold;
  a.log_stop = logf(stop_threshold);
  a.log_prob = log_prob;
  a.charge = charge;
  a.e_tick = e_tick;
  a.e_adc = e_adc;
  a.lam = lam;
  a.step_active = static_cast<int32_t *>(ws);
  if (cudaMemsetAsync(a.step_active, 0, sizeof(int32_t) * p.max_adc_values, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (n_pix == 0) return LSIM_OK;
  const size_t smem = sizeof(float) * kProbArrays * kProbMaxT;
  if (cudaFuncSetAttribute(k_fee_prob, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return LSIM_ERR_CUDA;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fee_prob, kProbThreads, smem);
  const int64_t cap = (int64_t)device_sm_count() * (per_sm > 0 ? per_sm : 1);
  const unsigned grid = (unsigned)(n_pix < cap ? n_pix : cap);
  k_fee_prob<<<grid, kProbThreads, smem, st>>>(a);
  k_fee_prob_mask<<<(unsigned)device_sm_count() * 4, 256, 0, st>>>(a, p.max_adc_values);
  return LSIM_OK;
}

}  // namespace lsim
