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
// Ticks whose inputs are bit-identical to the previous tick's are grouped
// into classes (one evaluation per class; flat stretches of a waveform
// collapse).  For each of the H hit steps the block walks the K paths and
// every thread folds its classes into three online log-sum-exp
// accumulators (hit, total, selection), with no barrier between paths.  A
// block top-K over the
// selection values (largest first, lower tick first on ties, as lax.top_k)
// gives the next K paths.  The reference stops the whole batch once no pixel
// keeps a total path probability above stop_threshold; the step kernel
// records per step whether any pixel stayed active and a second kernel
// blanks the steps the reference would not have run.
#include "lsim_internal.cuh"
#include "lsim_fee.cuh"

namespace lsim {
namespace {

constexpr int kProbThreads = 512;
constexpr int kProbTicks = 4;   // ticks per thread: up to 2048 ticks
constexpr int kProbMaxT = kProbThreads * kProbTicks;
constexpr int kProbMaxPaths = 32;
constexpr int kProbArrays = 10;  // q, running max, suffix max, esperance, soft-where weight, 3 class values, class, representative
// plus 6 partial sums per thread and the per-warp top-K candidates (value, index)
constexpr int kProbExtraFloats = 6 * kProbThreads + 2 * (kProbThreads / 32) * kProbMaxPaths + kProbMaxT;
static_assert(6 * kProbThreads >= kProbMaxT, "the path-group partials hold one tick array");
constexpr float kProbFloor = -1000.0f;

// ---------------------------------------------------------------- special functions
// jax.scipy.special.ndtr / log_ndtr in float32 (the published piecewise
// form: erf near zero and erfc in the tails for ndtr; -ndtr(-x) above 5,
// log(ndtr(x)) down to -10, the order-3 asymptotic series below).
// ndtr, log_ndtr and log_diff_ndtr's log term are called, not inlined:
// inlined at every call site of the per-path loops their erf/erfc/log
// bodies overflowed the instruction cache (the beam search ran 2.0x and
// its adjoint 2.2x slower, with identical results).

__device__ __noinline__ float ndtr_f(float x) {
  const float hs2 = 0.70710678118654752f;
  const float w = x * hs2;
  const float z = fabsf(w);
  const float y = z < hs2 ? 1.0f + erff(w) : (w > 0.0f ? 2.0f - erfcf(z) : erfcf(z));
  return 0.5f * y;
}

__device__ __noinline__ float log_ndtr_f(float x) {
  // above 15, erfc(x / sqrt 2) < 1e-50 is 0 in float32: -ndtr(-x) = -0
  if (x > 15.0f) return -0.0f;
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

// The clamped log(1 - exp(safe)) term of log_diff_ndtr.
__device__ __noinline__ float ldn_log_term(float safe) {
  const float neg = -expm1f(safe);
  const float neg_safe = 1e-30f + softplus_f((neg - 1e-30f) * 1e10f) / 1e10f;
  // neg_safe >= 1e-30, so lt >= -69.1 and the clamp's softplus argument
  // (lt + 100) * 10 >= 309: softplus is the identity there
  const float lt = logf(neg_safe);
  return -100.0f + ((lt + 100.0f) * 10.0f) / 10.0f;
}

// log(Phi(a) - Phi(b)) with the reference's smooth clamps; la, lb =
// log_ndtr(a), log_ndtr(b); term_m1 = ldn_log_term(-1), the value every
// a <= b takes (safe = -1 there), so flat stretches (a == b, w = 1/2 exactly)
// need no transcendental function at all.
__device__ __forceinline__ float log_diff_ndtr_f(float a, float b, float la, float lb, float term_m1) {
  if (a == b) return 0.5f * (la + term_m1) + 0.5f * kProbFloor;
  const float lts = a > b ? ldn_log_term(lb - la) : term_m1;
  const float lp = la + lts;
  const float w = sigmoid_f((a - b) * 1000.0f);
  return w * lp + (1.0f - w) * kProbFloor;
}

// online log-sum-exp: m = running maximum, s = sum of exp(x - m)
// (exp of arguments below -110 is 0 in float32 and is skipped)
__device__ __forceinline__ void lse_add(float &m, float &s, float x) {
  if (x > m) {
    s = m - x > -110.0f ? s * expf(m - x) + 1.0f : 1.0f;
    m = x;
  } else if (x - m > -110.0f) {
    s += expf(x - m);
  }
}

__device__ __forceinline__ float lse_final(float m, float s) { return logf(s) + m; }

// merge a partial (m2, s2) into (m, s)
__device__ __forceinline__ void lse_merge(float &m, float &s, float m2, float s2) {
  if (!(s2 > 0.0f)) return;
  if (!(s > 0.0f)) {
    m = m2;
    s = s2;
    return;
  }
  if (m2 > m) {
    s = (m - m2 > -110.0f ? s * expf(m - m2) : 0.0f) + s2;
    m = m2;
  } else if (m2 - m > -110.0f) {
    s += s2 * expf(m2 - m);
  }
}

__device__ __forceinline__ bool better(float va, int ia, float vb, int ib) {
  return va > vb || (va == vb && ia < ib);
}

// warp-wide best (value, index) under better(); every lane gets the result
__device__ __forceinline__ void warp_best(float &bv, int &bi) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (better(ov, oi, bv, bi)) {
      bv = ov;
      bi = oi;
    }
  }
}

// ---------------------------------------------------------------- block scans over a pixel row

// in-place inclusive scan of a[0..n) with op (sum, max) or a suffix max;
// each thread scans a contiguous chunk of kProbTicks, warps and the block
// combine the chunk totals.
enum ScanOp { kScanSum = 0, kScanMax = 1, kScanSuffixMax = 2, kScanSuffixSum = 3 };

template <int OP>
__device__ void block_scan_row(float *a, int n, float *red) {
  constexpr bool SUFFIX = OP == kScanSuffixMax || OP == kScanSuffixSum;
  constexpr bool SUM = OP == kScanSum || OP == kScanSuffixSum;
  const float ident = SUM ? 0.0f : -INFINITY;
  auto comb = [](float x, float y) { return SUM ? x + y : fmaxf(x, y); };
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  float v[kProbTicks];
  // suffix scans walk each thread's chunk from the right, thread 0 holding the last chunk
  const int base = SUFFIX ? n - (tid + 1) * kProbTicks : tid * kProbTicks;
  float run = ident;
#pragma unroll
  for (int i = 0; i < kProbTicks; ++i) {
    const int t = SUFFIX ? base + kProbTicks - 1 - i : base + i;
    const bool ok = t >= 0 && t < n;
    const float x = ok ? a[t] : ident;
    run = comb(run, x);
    v[i] = run;
  }
  // exclusive prefix of the chunk totals across the block
  float incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl = comb(incl, y);
  }
  if (lane == 31) red[wid] = incl;
  __syncthreads();
  float carry = ident;
  for (int w = 0; w < wid; ++w) carry = comb(carry, red[w]);
  float ex = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) ex = ident;
  const float pre = comb(carry, ex);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kProbTicks; ++i) {
    const int t = SUFFIX ? base + kProbTicks - 1 - i : base + i;
    if (t >= 0 && t < n) a[t] = comb(pre, v[i]);
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
  float *state;           // optional [n_pix][H][2][K]: each step's input path charges and log-probabilities
  int32_t *state_top;     // optional [n_pix][H][K]: each step's selected ticks (for the adjoint)
};

// The per-tick work of a step reads, for tick t, only the running maximum
// at t and t+1, q at t, t+1, s = shifted(t) and s+1, and the suffix maximum
// at the selection window end.  Ticks whose 7 values are bit-identical to
// those of the tick before give bit-identical results, so the block
// evaluates one representative per run of equal ticks (a "class") and
// expands the class values back to ticks; flat stretches of a waveform
// (no charge arriving) collapse to a handful of classes.
__global__ void __launch_bounds__(kProbThreads, 2) k_fee_prob(ProbArgs a) {
  extern __shared__ __align__(16) float sm[];
  float *qs = sm, *cm = qs + kProbMaxT, *cr = cm + kProbMaxT, *esp = cr + kProbMaxT, *sw = esp + kProbMaxT;
  float *vh = sw + kProbMaxT, *vd = vh + kProbMaxT, *vs = vd + kProbMaxT;
  int *cls = reinterpret_cast<int *>(vs + kProbMaxT), *rep = cls + kProbMaxT;
  float *part = reinterpret_cast<float *>(rep + kProbMaxT);   // [kProbThreads][6] partial sums of path groups
  float *cand_v = part + 6 * kProbThreads;                     // [warps][K] per-warp top-K candidates
  int *cand_i = reinterpret_cast<int *>(cand_v + (kProbThreads / 32) * kProbMaxPaths);
  // per-tick log_ndtr of the running maximum and of q for one path, shared by
  // neighbouring classes on dense pixels (the path-group partials, unused
  // then, hold the first)
  float *lmv = part, *lqv = reinterpret_cast<float *>(cand_i + (kProbThreads / 32) * kProbMaxPaths);
  __shared__ float red[kProbThreads / 32];
  __shared__ float pc[kProbMaxPaths], plp[kProbMaxPaths], nc[kProbMaxPaths], nlp[kProbMaxPaths];
  __shared__ int pskip[kProbMaxPaths];
  __shared__ int n_cls;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  const LsimParams &p = a.p;
  const int T = a.T, K = a.K, H = p.max_adc_values, tid = threadIdx.x;
  const float z = a.z, thr = a.thr;
  const float term_m1 = ldn_log_term(-1.0f);
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
    // esperance values, soft-where weights and the tick classes
    for (int t = tid; t < T - 1; t += kProbThreads) {
      const int s = shifted(t);
      const float e = (qs[s] + thr) - 0.5f * (qs[t + 1] + qs[t]);
      esp[t] = e;
      sw[t] = sigmoid_f((e - thr) * 10.0f);
      bool head = t == 0;
      if (!head) {
        const int sp = shifted(t - 1);
        const int s1 = min(s + 1, T - 1), sp1 = min(sp + 1, T - 1);
        const int fe = min(s + a.interval + 1, T - 1), fep = min(sp + a.interval + 1, T - 1);
        auto ne = [](float x, float y) { return __float_as_uint(x) != __float_as_uint(y); };
        head = ne(cm[t], cm[t - 1]) || ne(cm[t + 1], cm[t]) || ne(qs[t], qs[t - 1]) || ne(qs[t + 1], qs[t]) ||
               ne(qs[s], qs[sp]) || ne(qs[s1], qs[sp1]) || ne(cr[fe], cr[fep]);
      }
      vh[t] = head ? 1.0f : 0.0f;
    }
    __syncthreads();
    block_scan_row<kScanSum>(vh, T - 1, red);   // integer counts, exact in float32
    for (int t = tid; t < T - 1; t += kProbThreads) {
      const int u = (int)vh[t] - 1;
      cls[t] = u;
      if (t == 0 || (int)vh[t - 1] != u + 1) rep[u] = t;
      if (t == T - 2) n_cls = u + 1;
    }
    if (tid < K) {
      pc[tid] = 0.0f;
      plp[tid] = tid == 0 ? 0.0f : kProbFloor;
    }
    __syncthreads();
    const int U = n_cls;
    // with few classes, G groups of threads share a class and split the paths
    const int G = U <= kProbThreads / 2 ? min(8, kProbThreads / U) : 1;
    const int grp = G > 1 ? tid / U : 0;
    const int n_own = G > 1 ? (grp < G ? 1 : 0) : kProbTicks;
    const int r0 = G > 1 ? tid - grp * U : tid;
    // dense pixels: per path, log_ndtr at every tick (2 T calls) instead of
    // four per class (the running maximum at t + 1 and q at the shifted tick
    // are other ticks' values at t)
    const bool tick_mode = G == 1 && 2 * U > T;

    for (int h = 0; h < H; ++h) {
      // paths whose charge repeats that of a path more than 110 log units
      // likelier add exp(< -110) = 0 to every float32 log-sum-exp: skip them
      if (tid < K) {
        int sk = 0;
        for (int j = 0; j < K; ++j)
          if (j != tid && pc[j] == pc[tid] && plp[j] > plp[tid] + 110.0f) sk = 1;
        pskip[tid] = sk;
        if (a.state) {
          float *st = a.state + ((pix * H + h) * 2) * (int64_t)K;
          st[tid] = pc[tid];
          st[K + tid] = plp[tid];
        }
      }
      float hm[kProbTicks], hs[kProbTicks], dm[kProbTicks], ds[kProbTicks], sm_[kProbTicks], ss[kProbTicks];
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        hm[i] = dm[i] = sm_[i] = -INFINITY;
        hs[i] = ds[i] = ss[i] = 0.0f;
      }
      __syncthreads();
      for (int k = grp; n_own > 0 && k < K; k += G) {
        if (pskip[k]) continue;
        const float c = pc[k], lp = plp[k];
        if (tick_mode) {
          __syncthreads();   // the previous path's reads are done
          for (int t = tid; t < T; t += kProbThreads) {
            lmv[t] = log_ndtr_f(((cm[t] - c) - thr) * z);
            lqv[t] = log_ndtr_f(((qs[t] - c) - thr) * z);
          }
          __syncthreads();
        }
#pragma unroll
        for (int i = 0; i < kProbTicks; ++i) {
          const int r = r0 + i * kProbThreads;
          if (i < n_own && r < U) {
            const int t = rep[r];
            const int s = shifted(t);
            const float zm0 = ((cm[t] - c) - thr) * z, zm1 = ((cm[t + 1] - c) - thr) * z;
            const float LM0 = tick_mode ? lmv[t] : log_ndtr_f(zm0);
            const float LM1 = tick_mode ? lmv[t + 1] : (zm1 == zm0 ? LM0 : log_ndtr_f(zm1));
            const float lg = log_diff_ndtr_f(zm1, zm0, LM1, LM0, term_m1);
            const float zq0 = ((qs[t] - c) - thr) * z, zqs = ((qs[s] - c) - thr) * z;
            const float LQ0 = tick_mode ? lqv[t] : log_ndtr_f(zq0);
            const float LQs = tick_mode ? lqv[s] : (zqs == zq0 ? LQ0 : log_ndtr_f(zqs));
            float le = log_diff_ndtr_f(zqs, zq0, LQs, LQ0, term_m1);
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
      }
      if (G > 1) {
        // merge the path groups' partial log-sum-exps into group 0
        if (grp > 0 && grp < G) {
          float *q = part + 6 * tid;
          q[0] = hm[0], q[1] = hs[0], q[2] = dm[0], q[3] = ds[0], q[4] = sm_[0], q[5] = ss[0];
        }
        __syncthreads();
        if (grp == 0) {
          for (int g2 = 1; g2 < G; ++g2) {
            const float *q = part + 6 * (g2 * U + tid);
            lse_merge(hm[0], hs[0], q[0], q[1]);
            lse_merge(dm[0], ds[0], q[2], q[3]);
            lse_merge(sm_[0], ss[0], q[4], q[5]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        const int r = r0 + i * kProbThreads;
        if (i < n_own && grp == 0 && r < U) {
          vh[r] = lse_final(hm[i], hs[i]);
          vd[r] = lse_final(dm[i], ds[i]);
          vs[r] = lse_final(sm_[i], ss[i]);
        }
      }
      __syncthreads();
      // step outputs and the per-hit reductions
      float l_sum = 0.0f, t_sum = 0.0f, a_sum = 0.0f;
      float selv[kProbTicks];
      const int64_t row = (pix * H + h) * (int64_t)(T - 1);
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        const int t = tid + i * kProbThreads;
        selv[i] = -INFINITY;
        if (t < T - 1) {
          const int u = cls[t];
          const float hit = vh[u];
          selv[i] = vs[u];
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
      // top-K ticks by selection value -> next paths: each warp keeps the K
      // best of its ticks (largest first, lower tick first on ties), then
      // warp 0 takes the K best of those candidates
      {
        unsigned taken = 0;
        for (int r = 0; r < K; ++r) {
          float bv = -INFINITY;
          int bi = 0x7fffffff;
#pragma unroll
          for (int i = 0; i < kProbTicks; ++i) {
            const int t = tid + i * kProbThreads;
            if (t < T - 1 && !(taken >> i & 1u) && better(selv[i], t, bv, bi)) {
              bv = selv[i];
              bi = t;
            }
          }
          warp_best(bv, bi);
          if (bi != 0x7fffffff && (bi % kProbThreads) == tid) taken |= 1u << (bi / kProbThreads);
          if (lane == 0) {
            cand_v[wid * kProbMaxPaths + r] = bv;
            cand_i[wid * kProbMaxPaths + r] = bi;
          }
        }
      }
      __syncthreads();
      if (wid == 0) {
        constexpr int kCand = (kProbThreads / 32) * kProbMaxPaths / 32;   // candidates per lane
        float cv[kCand];
        int ci[kCand];
#pragma unroll
        for (int j = 0; j < kCand; ++j) {
          const int e = lane + 32 * j, w2 = e / kProbMaxPaths, r2 = e % kProbMaxPaths;
          cv[j] = r2 < K ? cand_v[w2 * kProbMaxPaths + r2] : -INFINITY;
          ci[j] = r2 < K ? cand_i[w2 * kProbMaxPaths + r2] : 0x7fffffff;
        }
        unsigned taken = 0;
        for (int r = 0; r < K; ++r) {
          float bv = -INFINITY;
          int bi = 0x7fffffff, bj = -1;
#pragma unroll
          for (int j = 0; j < kCand; ++j)
            if (!(taken >> j & 1u) && better(cv[j], ci[j], bv, bi)) {
              bv = cv[j];
              bi = ci[j];
              bj = j;
            }
          const int mine = bi;
          warp_best(bv, bi);
          if (bj >= 0 && mine == bi) taken |= 1u << bj;
          if (lane == r) {
            const int tt = bi >= 0 && bi < T - 1 ? bi : T - 2;
            nlp[r] = vd[cls[tt]];
            nc[r] = qs[min(shifted(tt) + 1, T - 1)];
            if (a.state_top) a.state_top[(pix * H + h) * (int64_t)K + r] = tt;
          }
        }
      }
      __syncthreads();
      if (tid < 32) {
        const float v = tid < K ? nlp[tid] : -INFINITY;
        float m = v;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        const float mm = isfinite(m) ? m : 0.0f;
        float sum = tid < K ? expf(v - mm) : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (tid < K) {
          pc[tid] = nc[tid];
          plp[tid] = nlp[tid];
        }
        if (tid == 0 && logf(sum) + mm > a.log_stop && !*(volatile int32_t *)(a.step_active + h))
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

// ---------------------------------------------------------------- adjoint
// Reverse mode through the beam search as jax.grad takes it: the top-K tick
// choices are held (lax.stop_gradient), jnp.where passes the cotangent to
// the selected branch, jnp.minimum to the smaller argument (half each at a
// tie), the running maximum to the tick where it was first attained, and
// softplus / sigmoid / log-sum-exp by their derivatives.

// d log_ndtr / dx as jax.scipy.special.log_ndtr defines it (a custom
// derivative, the same on every branch): exp(norm_logpdf(x) - log_ndtr(x))
__device__ __forceinline__ float dlog_ndtr_f(float x, float lx) {
  return expf((-0.5f * x * x - 0.918938533204672742f) - lx);
}

// log_diff_ndtr value and partials d/da, d/db (la = log_ndtr(a), dla its derivative)
__device__ __forceinline__ float ldn_grad(float a, float b, float la, float lb, float dla, float dlb, float term_m1,
                                          float &ga, float &gb) {
  float lts, dlts_du = 0.f;
  const bool sel = a > b;
  if (sel) {
    const float u = lb - la;
    const float neg = -expm1f(u);
    const float y = (neg - 1e-30f) * 1e10f;
    const float ns = 1e-30f + softplus_f(y) / 1e10f;
    const float lt = logf(ns);
    lts = -100.0f + ((lt + 100.0f) * 10.0f) / 10.0f;
    // softplus' = sigmoid; d neg / du = -exp(u); the second clamp is the identity there
    dlts_du = (1.0f / ns) * sigmoid_f(y) * (-expf(u));
  } else {
    lts = term_m1;
  }
  const float lp = la + lts;
  const float w = sigmoid_f((a - b) * 1000.0f);
  const float out = w * lp + (1.0f - w) * kProbFloor;
  const float gw = (lp - kProbFloor) * w * (1.0f - w) * 1000.0f;   // through the gate
  ga = w * (dla - dlts_du * dla) + gw;
  gb = w * (dlts_du * dlb) - gw;
  if (!sel) {
    ga = w * dla + gw;
    gb = -gw;
  }
  return out;
}

struct ProbVjpArgs {
  ProbArgs f;                  // the forward's arguments (state, state_top, step_active read)
  const float *g_log_prob;     // optional [n_pix][H][T-1]
  const float *g_charge;       // optional [n_pix][H][T-1]
  const float *g_e_tick, *g_e_adc, *g_lam;   // optional [n_pix][H] (all three or none)
  float *g_wfs;                // [n_pix][T]
};

// Ticks are grouped into classes as in the forward, here by the five
// values a tick's hit and dist terms read (the running maximum at t and
// t + 1, q at t, t + 1 and at the shifted tick; the selection value is not
// differentiated).  Within a class every per-path partial derivative is the
// same; the per-tick cotangents (on the hit log-probability and on the dist
// value) enter linearly, so the partials are evaluated once per class and
// path, folded into seven per-class coefficients, and spread back to the
// class's ticks with the ticks' own cotangents.  Classes are also cut at
// every kVjpSpan ticks, so the per-class loops over ticks stay short (flat
// stretches of a waveform are long).
constexpr int kVjpSpan = 16;
constexpr int kVjpArrays = 13;   // q, running max, 5 accumulators, dist and hit cotangents, class hit and
                                 // dist values (the hit values double as scratch), class, representative;
                                 // the esperance and the soft-where weight are recomputed from q, so two
                                 // blocks fit on an SM

__global__ void __launch_bounds__(kProbThreads, 2) k_fee_prob_vjp(ProbVjpArgs va) {
  extern __shared__ __align__(16) float sm[];
  const ProbArgs &a = va.f;
  float *qs = sm, *cm = qs + kProbMaxT;
  float *Aq0 = cm + kProbMaxT, *Aqs = Aq0 + kProbMaxT, *Am0 = Aqs + kProbMaxT, *Am1 = Am0 + kProbMaxT;
  float *Aesp = Am1 + kProbMaxT, *Gd = Aesp + kProbMaxT, *Gh = Gd + kProbMaxT;
  float *vh = Gh + kProbMaxT, *vd = vh + kProbMaxT;
  float *tmp = vh;   // scratch before and after the steps, when the class values are not in use
  int *cls = reinterpret_cast<int *>(vd + kProbMaxT), *rep = cls + kProbMaxT;
  float *part = reinterpret_cast<float *>(rep + kProbMaxT);   // [warps][2][kProbMaxPaths]
  __shared__ float red[kProbThreads / 32];
  __shared__ float pc[kProbMaxPaths], plp[kProbMaxPaths], glp_n[kProbMaxPaths], gc_n[kProbMaxPaths];
  __shared__ int pskip[kProbMaxPaths], ptop[kProbMaxPaths];
  __shared__ int n_exec, n_cls;

  const LsimParams &p = a.p;
  const int T = a.T, K = a.K, H = p.max_adc_values, tid = threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
  const float z = a.z, thr = a.thr;
  const float term_m1 = ldn_log_term(-1.0f);
  auto shifted = [&](int t) { return min(t + a.interval + 1, T - 1); };
  // the esperance and the soft-where weight of tick t, recomputed from q
  auto esp_at = [&](int t) { return (qs[shifted(t)] + thr) - 0.5f * (qs[t + 1] + qs[t]); };
  auto sw_at = [&](float e) { return sigmoid_f((e - thr) * 10.0f); };
  if (tid == 0) {
    int first = H;
    for (int h = 1; h < H; ++h)
      if (!a.step_active[h - 1]) {
        first = h;
        break;
      }
    n_exec = first;
  }

  for (int64_t pix = blockIdx.x; pix < a.n_pix; pix += gridDim.x) {
    const float *w = a.wfs + pix * T;
    for (int t = tid; t < T; t += kProbThreads) qs[t] = w[t] * p.t_sampling;
    __syncthreads();
    block_scan_row<kScanSum>(qs, T, red);
    for (int t = tid; t < T; t += kProbThreads) {
      cm[t] = qs[t];
      Aq0[t] = Aqs[t] = Am0[t] = Am1[t] = Aesp[t] = 0.f;
    }
    __syncthreads();
    block_scan_row<kScanMax>(cm, T, red);
    for (int t = tid; t < T - 1; t += kProbThreads) {
      const int s = shifted(t);
      bool head = t % kVjpSpan == 0;
      if (!head) {
        const int sp = shifted(t - 1);
        auto ne = [](float x, float y) { return __float_as_uint(x) != __float_as_uint(y); };
        head = ne(cm[t], cm[t - 1]) || ne(cm[t + 1], cm[t]) || ne(qs[t], qs[t - 1]) || ne(qs[t + 1], qs[t]) ||
               ne(qs[s], qs[sp]);
      }
      tmp[t] = head ? 1.0f : 0.0f;
    }
    __syncthreads();
    block_scan_row<kScanSum>(tmp, T - 1, red);   // integer counts, exact in float32
    for (int t = tid; t < T - 1; t += kProbThreads) {
      const int u = (int)tmp[t] - 1;
      cls[t] = u;
      if (t == 0 || (int)tmp[t - 1] != u + 1) rep[u] = t;
      if (t == T - 2) n_cls = u + 1;
    }
    if (tid < K) {
      glp_n[tid] = 0.f;
      gc_n[tid] = 0.f;
    }
    __syncthreads();
    const int U = n_cls;
    if (tid == 0) rep[U] = T - 1;     // end of the last class

    for (int h = n_exec - 1; h >= 0; --h) {
      // step h's input paths and selected ticks, recorded by the forward
      if (tid < K) {
        const float *st = a.state + ((pix * H + h) * 2) * (int64_t)K;
        pc[tid] = st[tid];
        plp[tid] = st[K + tid];
        ptop[tid] = a.state_top[(pix * H + h) * (int64_t)K + tid];
      }
      for (int t = tid; t < T; t += kProbThreads) Gd[t] = 0.f;
      __syncthreads();
      if (tid < K) {
        int sk = 0;
        for (int j = 0; j < K; ++j)
          if (j != tid && pc[j] == pc[tid] && plp[j] > plp[tid] + 110.0f) sk = 1;
        pskip[tid] = sk;
      }
      if (tid == 0) {
        // the next step's state cotangents: new lp_j = dist[top_j], new c_j = q[best_j]
        for (int j = 0; j < K; ++j) {
          const int tt = ptop[j];
          Gd[tt] += glp_n[j];
          Aq0[min(shifted(tt) + 1, T - 1)] += gc_n[j];
        }
      }
      __syncthreads();
      // ---- pass 1: hit and dist log-sum-exps per class
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        const int u = tid + i * kProbThreads;
        if (u < U) {
          float hm = -INFINITY, hs = 0.f, dm = -INFINITY, ds = 0.f;
          const int t = rep[u];
          const int sidx = shifted(t);
          const float swt = sw_at(esp_at(t));
          for (int k = 0; k < K; ++k) {
            if (pskip[k]) continue;
            const float c = pc[k], lp = plp[k];
            const float zm0 = ((cm[t] - c) - thr) * z, zm1 = ((cm[t + 1] - c) - thr) * z;
            const float LM0 = log_ndtr_f(zm0);
            const float LM1 = zm1 == zm0 ? LM0 : log_ndtr_f(zm1);
            const float lg = log_diff_ndtr_f(zm1, zm0, LM1, LM0, term_m1);
            const float zq0 = ((qs[t] - c) - thr) * z, zqs = ((qs[sidx] - c) - thr) * z;
            const float LQ0 = log_ndtr_f(zq0);
            const float LQs = zqs == zq0 ? LQ0 : log_ndtr_f(zqs);
            float le = log_diff_ndtr_f(zqs, zq0, LQs, LQ0, term_m1);
            le = fminf(le, lg);
            le = kProbFloor + softplus_f(le - kProbFloor);
            le = swt * le + (1.0f - swt) * kProbFloor;
            lse_add(hm, hs, le + lp);
            lse_add(dm, ds, lg + lp);
          }
          vh[u] = lse_final(hm, hs);
          vd[u] = lse_final(dm, ds);
        }
      }
      __syncthreads();
      // ---- cotangents of the step's outputs on each tick
      float l_sum = 0.f, t_sum = 0.f, a_sum = 0.f;
      float pr[kProbTicks];
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        const int t = tid + i * kProbThreads;
        pr[i] = 0.f;
        if (t < T - 1) {
          const int64_t o = (pix * H + h) * (int64_t)(T - 1) + t;
          Gh[t] = va.g_log_prob ? va.g_log_prob[o] : 0.f;
          if (va.g_charge) Aesp[t] += va.g_charge[o];
          pr[i] = expf(vh[cls[t]]);
          l_sum += pr[i];
          t_sum += (float)t * pr[i];
          a_sum += digitize(p, esp_at(t)) * pr[i];
        }
      }
      if (va.g_lam) {
        const float L = block_sum(l_sum, red);
        const float Ts = block_sum(t_sum, red);
        const float As = block_sum(a_sum, red);
        const float den = fmaxf(L, 1e-10f);
        const float on = L > 1e-10f ? 1.f : (L == 1e-10f ? 0.5f : 0.f);   // jnp.maximum's share
        const float ET = Ts / den, EA = As / den;
        const int64_t o = pix * H + h;
        const float gl = va.g_lam[o], gt = va.g_e_tick[o], ga = va.g_e_adc[o];
        // the lambda cotangent also reaches ET and EA through the denominator
        const float gden = -(gt * ET + ga * EA) / den;
#pragma unroll
        for (int i = 0; i < kProbTicks; ++i) {
          const int t = tid + i * kProbThreads;
          if (t < T - 1) {
            const float et = esp_at(t);
            const float adc = digitize(p, et);
            const float gp = gl + gt * (float)t / den + ga * adc / den + on * gden;
            Gh[t] += gp * pr[i];
            Aesp[t] += digitize_vjp(p, et, ga * pr[i] / den);
          }
        }
      }
      __syncthreads();
      // ---- per class: sums of the ticks' cotangents
      float Hs[kProbTicks], Ds[kProbTicks];
      bool anyH[kProbTicks], anyD[kProbTicks];
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        const int u = tid + i * kProbThreads;
        Hs[i] = Ds[i] = 0.f;
        anyH[i] = anyD[i] = false;
        if (u < U)
          for (int t = rep[u]; t < rep[u + 1]; ++t) {
            const float gh = Gh[t], gd = Gd[t];
            Hs[i] += gh;
            Ds[i] += gd;
            anyH[i] |= gh != 0.f;
            anyD[i] |= gd != 0.f;
          }
      }
      // ---- pass 2: the partials per class and path, folded into seven
      // per-class coefficients of the ticks' (hit, dist) cotangents
      float co[kProbTicks][7];
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i)
#pragma unroll
        for (int j = 0; j < 7; ++j) co[i][j] = 0.f;
      for (int k = 0; k < K; ++k) {
        float glp = 0.f, gc = 0.f;
        if (!pskip[k]) {
          const float c = pc[k], lp = plp[k];
#pragma unroll
          for (int i = 0; i < kProbTicks; ++i) {
            const int u = tid + i * kProbThreads;
            if (u >= U || !(anyH[i] || anyD[i])) continue;
            const int t = rep[u];
            const int sidx = shifted(t);
            const float zm0 = ((cm[t] - c) - thr) * z, zm1 = ((cm[t + 1] - c) - thr) * z;
            const float LM0 = log_ndtr_f(zm0), LM1 = log_ndtr_f(zm1);
            float g_m1, g_m0;
            const float lg = ldn_grad(zm1, zm0, LM1, LM0, dlog_ndtr_f(zm1, LM1), dlog_ndtr_f(zm0, LM0), term_m1,
                                      g_m1, g_m0);
            const float zq0 = ((qs[t] - c) - thr) * z, zqs = ((qs[sidx] - c) - thr) * z;
            const float LQ0 = log_ndtr_f(zq0), LQs = log_ndtr_f(zqs);
            float g_qs, g_q0;
            const float lep = ldn_grad(zqs, zq0, LQs, LQ0, dlog_ndtr_f(zqs, LQs), dlog_ndtr_f(zq0, LQ0), term_m1,
                                       g_qs, g_q0);
            const float le1 = fminf(lep, lg);
            const float le2 = kProbFloor + softplus_f(le1 - kProbFloor);
            const float wt = sw_at(esp_at(t));
            const float le = wt * le2 + (1.0f - wt) * kProbFloor;
            // d(hit log-sum-exp)/d(le + lp) and d(dist log-sum-exp)/d(lg + lp)
            const float al = anyH[i] ? expf((le + lp) - vh[u]) : 0.f;
            const float be = anyD[i] ? expf((lg + lp) - vd[u]) : 0.f;
            glp += al * Hs[i] + be * Ds[i];
            // per unit hit cotangent: le = w le2 + (1 - w)(-1000), w = sigmoid((esp - thr) 10)
            const float gl1 = al * wt * sigmoid_f(le1 - kProbFloor);
            const float s_lep = lep < lg ? 1.f : (lep == lg ? 0.5f : 0.f);
            const float hl = gl1 * s_lep, hg = gl1 * (1.f - s_lep);
            co[i][0] += hl * g_q0 * z;
            co[i][1] += hl * g_qs * z;
            co[i][2] += hg * g_m0 * z;
            co[i][3] += be * g_m0 * z;
            co[i][4] += hg * g_m1 * z;
            co[i][5] += be * g_m1 * z;
            co[i][6] += al * (le2 - kProbFloor) * wt * (1.0f - wt) * 10.0f;
            gc -= (Hs[i] * (hl * (g_q0 + g_qs) + hg * (g_m0 + g_m1)) + Ds[i] * be * (g_m0 + g_m1)) * z;
          }
        }
        glp = warp_sum(glp);
        gc = warp_sum(gc);
        if (lane == 0) {
          part[(wid * 2) * kProbMaxPaths + k] = glp;
          part[(wid * 2 + 1) * kProbMaxPaths + k] = gc;
        }
      }
      // spread the coefficients to the class's ticks with their cotangents
#pragma unroll
      for (int i = 0; i < kProbTicks; ++i) {
        const int u = tid + i * kProbThreads;
        if (u >= U || !(anyH[i] || anyD[i])) continue;
        for (int t = rep[u]; t < rep[u + 1]; ++t) {
          const float gh = Gh[t], gd = Gd[t];
          Aq0[t] += gh * co[i][0];
          Aqs[t] += gh * co[i][1];
          Am0[t] += gh * co[i][2] + gd * co[i][3];
          Am1[t] += gh * co[i][4] + gd * co[i][5];
          Aesp[t] += gh * co[i][6];
        }
      }
      __syncthreads();
      if (tid < K) {
        float s1 = 0.f, s2 = 0.f;
        for (int w2 = 0; w2 < kProbThreads / 32; ++w2) {
          s1 += part[(w2 * 2) * kProbMaxPaths + tid];
          s2 += part[(w2 * 2 + 1) * kProbMaxPaths + tid];
        }
        glp_n[tid] = s1;   // cotangent of this step's input state = the previous step's output state
        gc_n[tid] = s2;
      }
      __syncthreads();
    }
    // ---- assemble dL/dq from the per-tick partials
    // running maximum: cm[t] (tick t's zm0) and cm[t] as tick t-1's cm[t+1]
    for (int t = tid; t < T; t += kProbThreads) tmp[t] = (t < T - 1 ? Am0[t] : 0.f) + (t > 0 ? Am1[t - 1] : 0.f);
    __syncthreads();
    block_scan_row<kScanSum>(tmp, T, red);   // prefix sums P of dL/dcm
    // each run of a constant running maximum routes its sum to the run's first tick
    for (int t = tid; t < T; t += kProbThreads) {
      float g = Aq0[t];
      const bool start = t == 0 || cm[t] != cm[t - 1];
      if (start) {
        int e = t;
        while (e + 1 < T && cm[e + 1] == cm[t]) ++e;
        g += tmp[e] - (t > 0 ? tmp[t - 1] : 0.f);
      }
      // shifted-tick role q[s_t] (s_t = min(t + interval + 1, T - 1)), with the esperance terms
      const int t0 = t - a.interval - 1;
      if (t < T - 1) {
        if (t0 >= 0) g += Aqs[t0] + Aesp[t0];
      } else {
        for (int u = max(t0, 0); u < T - 1; ++u) g += Aqs[u] + Aesp[u];
      }
      // esperance: - 0.5 (q[t + 1] + q[t])
      if (t < T - 1) g -= 0.5f * Aesp[t];
      if (t > 0) g -= 0.5f * Aesp[t - 1];
      Gd[t] = g;
    }
    __syncthreads();
    // q = cumsum(w * ts): dL/dw[i] = ts * sum_{j >= i} dL/dq[j]
    block_scan_row<kScanSuffixSum>(Gd, T, red);
    for (int t = tid; t < T; t += kProbThreads) va.g_wfs[pix * T + t] = Gd[t] * p.t_sampling;
    __syncthreads();
  }
}

}  // namespace

size_t fee_prob_workspace_bytes(int32_t max_adc_values) {
  return ((size_t)(max_adc_values > 0 ? max_adc_values : 1) * sizeof(int32_t) + 255) & ~size_t(255);
}

static ProbArgs prob_args(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                          float stop_threshold, float *log_prob, float *charge, float *e_tick, float *e_adc,
                          float *lam, void *ws) {
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
  a.state = nullptr;
  a.state_top = nullptr;
  return a;
}

static int run_fee_prob_impl(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                             float stop_threshold, float *log_prob, float *charge, float *e_tick, float *e_adc,
                             float *lam, void *ws, float *state, int32_t *state_top, cudaStream_t st) {
  if (n_t < 3 || n_t > kProbMaxT) return set_error(LSIM_ERR_UNSUPPORTED, "probabilistic FEE: n_t must be in [3, 2048]");
  if (n_paths < 1 || n_paths > kProbMaxPaths || n_paths > n_t - 1)
    return set_error(LSIM_ERR_UNSUPPORTED, "probabilistic FEE: fee_paths_scaling must be in [1, min(32, n_t - 1)]");
  if (!(p.reset_noise > 0.0f)) return set_error(LSIM_ERR_INVALID, "probabilistic FEE: RESET_NOISE_CHARGE must be > 0");
  ProbArgs a = prob_args(p, wfs, n_pix, n_t, n_paths, stop_threshold, log_prob, charge, e_tick, e_adc, lam, ws);
  a.state = state;
  a.state_top = state_top;
  if (cudaMemsetAsync(a.step_active, 0, sizeof(int32_t) * p.max_adc_values, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (n_pix == 0) return LSIM_OK;
  const size_t smem = sizeof(float) * (kProbArrays * kProbMaxT + kProbExtraFloats);
  if (cudaFuncSetAttribute(k_fee_prob, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return LSIM_ERR_CUDA;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fee_prob, kProbThreads, smem);
  const int64_t cap = (int64_t)device_sm_count() * (per_sm > 0 ? per_sm : 1);
  const unsigned grid = (unsigned)(n_pix < cap ? n_pix : cap);
  k_fee_prob<<<grid, kProbThreads, smem, st>>>(a);
  if (log_prob || charge || lam)
    k_fee_prob_mask<<<(unsigned)device_sm_count() * 4, 256, 0, st>>>(a, p.max_adc_values);
  return LSIM_OK;
}

size_t fee_prob_vjp_workspace_bytes(int64_t n_pix, int32_t max_adc_values, int32_t n_paths) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t states = (size_t)(n_pix > 0 ? n_pix : 0) * (size_t)max_adc_values * (size_t)n_paths;
  return fee_prob_workspace_bytes(max_adc_values) + al(sizeof(float) * 2 * states) + al(sizeof(int32_t) * states);
}

int run_fee_prob_vjp(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                     float stop_threshold, const float *g_log_prob, const float *g_charge, const float *g_e_tick,
                     const float *g_e_adc, const float *g_lam, float *g_wfs, void *ws, cudaStream_t st) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t states = (size_t)n_pix * (size_t)p.max_adc_values * (size_t)n_paths;
  char *b = static_cast<char *>(ws);
  float *state = reinterpret_cast<float *>(b + fee_prob_workspace_bytes(p.max_adc_values));
  int32_t *state_top = reinterpret_cast<int32_t *>(reinterpret_cast<char *>(state) + al(sizeof(float) * 2 * states));
  // forward with the step states recorded (no outputs), then the reverse pass
  int rc = run_fee_prob_impl(p, wfs, n_pix, n_t, n_paths, stop_threshold, nullptr, nullptr, nullptr, nullptr,
                             nullptr, ws, state, state_top, st);
  if (rc != LSIM_OK || n_pix == 0) return rc;
  ProbVjpArgs va;
  va.f = prob_args(p, wfs, n_pix, n_t, n_paths, stop_threshold, nullptr, nullptr, nullptr, nullptr, nullptr, ws);
  va.f.state = state;
  va.f.state_top = state_top;
  va.g_log_prob = g_log_prob;
  va.g_charge = g_charge;
  va.g_e_tick = g_e_tick;
  va.g_e_adc = g_e_adc;
  va.g_lam = g_lam;
  va.g_wfs = g_wfs;
  const size_t smem = sizeof(float) * (kVjpArrays * kProbMaxT + 2 * (kProbThreads / 32) * kProbMaxPaths);
  if (cudaFuncSetAttribute(k_fee_prob_vjp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return LSIM_ERR_CUDA;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fee_prob_vjp, kProbThreads, smem);
  const int64_t cap = (int64_t)device_sm_count() * (per_sm > 0 ? per_sm : 1);
  k_fee_prob_vjp<<<(unsigned)(n_pix < cap ? n_pix : cap), kProbThreads, smem, st>>>(va);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

int run_fee_prob(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                 float stop_threshold, float *log_prob, float *charge, float *e_tick, float *e_adc, float *lam,
                 void *ws, cudaStream_t st) {
  return run_fee_prob_impl(p, wfs, n_pix, n_t, n_paths, stop_threshold, log_prob, charge, e_tick, e_adc, lam, ws,
                           nullptr, nullptr, st);
}

}  // namespace lsim
