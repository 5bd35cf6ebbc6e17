// Warp-cooperative self-trigger front end on a waveform held in shared
// memory: cumulative charge, threshold crossing, integration window, reset,
// digitisation, and the adjoint of all of it.
//
// Reference: get_adc_values (fee_jax.py:168-279) and digitize
// (fee_jax.py:55-71).  Per hit h the reference finds the first i with
// Q[i] <= thr <= Q[i+1] (Q = base + C, C = cumsum(w * t_sampling)),
// integrates to e = min(i + 1 + interval, T-1), accepts the hit when
// C[e] >= thr and a crossing exists, and resets
// C <- max(C - C[min(i + 2 + interval, T-1)], 0).
#pragma once

#include "lsim_common.cuh"

namespace lsim {

constexpr int kMaskWords = 64;   // bits per hit for T <= 2048

struct FeeState {
  int n_done;                  // hits evaluated before the early exit (the rest are empty)
  int e[LSIM_MAX_HITS];        // integration end index
  int e2[LSIM_MAX_HITS];       // reset index
  int cond[LSIM_MAX_HITS];     // 1 = rejected (adc forced to 0)
  float raw[LSIM_MAX_HITS];    // integrated charge before digitisation
  uint32_t *mask;              // [max_adc_values][kMaskWords]: (C - R >= 0) per tick, per hit
};

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// digitize (fee_jax.py:68-69): continuous, clamped to [0, ADC_COUNTS].
__device__ __forceinline__ float digitize(const LsimParams &p, float q) {
  float x = (q * p.gain + p.v_pedestal) - p.v_cm;
  x = x < 0.f ? 0.f : x;
  float y = (x * p.adc_counts) / p.vref_minus_cm;
  return y > p.adc_counts ? p.adc_counts : y;
}

// d digitize / d q times g, with JAX's 0.5 rule at the clamp ties.
__device__ __forceinline__ float digitize_vjp(const LsimParams &p, float q, float g) {
  float x = (q * p.gain + p.v_pedestal) - p.v_cm;
  float gx = x > 0.f ? 1.f : (x == 0.f ? 0.5f : 0.f);
  float y = ((x < 0.f ? 0.f : x) * p.adc_counts) / p.vref_minus_cm;
  float gy = y < p.adc_counts ? 1.f : (y == p.adc_counts ? 0.5f : 0.f);
  return ((g * gy) * (p.adc_counts / p.vref_minus_cm)) * gx * p.gain;
}

// In-place cumulative charge C[i] = sum_{j<=i} X[j]*ts over T ticks
// (lane-contiguous chunks + warp exclusive scan of the chunk totals).
__device__ __forceinline__ void warp_cumsum_charge(float *X, int T, float ts, int lane) {
  const int per = (T + kWarp - 1) / kWarp;
  const int b = lane * per;
  const int e = min(b + per, T);
  float s = 0.f;
  for (int i = b; i < e; ++i) {
    s = s + X[i] * ts;
    X[i] = s;
  }
  float incl = s;
  for (int o = 1; o < kWarp; o <<= 1) {
    float y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const float offset = incl - s;
  if (lane > 0)
    for (int i = b; i < e; ++i) X[i] = offset + X[i];
  __syncwarp();
}

// Forward self-trigger on C (in place).  normals: per-pixel standard
// normals [1 + 3H] or null (noise off).  Writes adc (digitized) and tick
// per hit through lane 0; fills st when non-null.
//
// early_exit (noise off, threshold > 0): once a rejected hit leaves C all
// zero, every later hit is provably empty (no crossing of a positive
// threshold, C[e] = 0, reset by 0 keeps C zero), so the remaining hits are
// written as empty without sweeping the row again.
__device__ __forceinline__ void fee_forward(const LsimParams &p, float *C, int T, const float *normals,
                                            float *adc_out, float *tick_out, FeeState *st, float *raw_out,
                                            bool early_exit, int lane) {
  const float thr = p.threshold;
  const int H = p.max_adc_values;
  float base = normals ? normals[0] * p.reset_noise : 0.f;
  const int nwords = (T + kWarp - 1) / kWarp;
  for (int h = 0; h < H; ++h) {
    int idx = T - 2;
    for (int m = 0; m * kWarp < T - 1; ++m) {
      int i = m * kWarp + lane;
      bool c = false;
      if (i < T - 1) {
        float q0 = base + C[i];
        float q1 = base + C[i + 1];
        c = (q1 >= thr) && (q0 <= thr);
      }
      unsigned bal = __ballot_sync(0xffffffffu, c);
      if (bal) { idx = m * kWarp + __ffs(bal) - 1; break; }
    }
    int e = idx + 1 + p.fee_interval;
    if (e >= T) e = T - 1;
    const float qvn = C[e];
    const float qv = base + qvn;
    const float extra = normals ? normals[1 + 3 * h] * p.uncorr_noise : 0.f;
    float adc = (qvn != 0.f) ? (qv + extra) : qvn;
    const bool cond = (adc < thr) || (idx == T - 2);
    if (cond) adc = 0.f;
    const float tick = cond ? (float)(T - 2) : (float)idx;
    if (normals) base = cond ? normals[3 + 3 * h] * p.uncorr_noise : normals[2 + 3 * h] * p.reset_noise;
    int e2 = idx + 2 + p.fee_interval;
    if (e2 >= T) e2 = T - 1;
    const float R = C[e2];
    __syncwarp();
    bool nz = false;
    for (int m = 0; m < nwords; ++m) {
      int i = m * kWarp + lane;
      bool keep = true;
      if (i < T) {
        float c = C[i] - R;
        keep = !(c < 0.f);
        C[i] = keep ? c : 0.f;
        nz |= keep && c != 0.f;
      }
      if (st) {
        unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) st->mask[h * kMaskWords + m] = bal;
      }
    }
    __syncwarp();
    if (lane == 0) {
      if (adc_out) adc_out[h] = digitize(p, adc);
      if (tick_out) tick_out[h] = tick;
      if (raw_out) raw_out[h] = adc;
      if (st) { st->e[h] = e; st->e2[h] = e2; st->cond[h] = cond ? 1 : 0; st->raw[h] = adc; }
    }
    if (early_exit && cond && !__any_sync(0xffffffffu, nz)) {
      if (lane == 0) {
        const float a0 = digitize(p, 0.f);
        for (int k = h + 1; k < H; ++k) {
          if (adc_out) adc_out[k] = a0;
          if (tick_out) tick_out[k] = (float)(T - 2);
          if (raw_out) raw_out[k] = 0.f;
          if (st) { st->e[k] = T - 1; st->e2[k] = T - 1; st->cond[k] = 1; st->raw[k] = 0.f; }
        }
        if (st) st->n_done = h + 1;
      }
      __syncwarp();
      return;
    }
  }
  if (st && lane == 0) st->n_done = H;
  __syncwarp();
}

// Adjoint of fee_forward + cumsum: from dL/d(integrated charge) per hit
// (gint, identical in all lanes) to dL/dW[i] over T ticks, written to G.
__device__ __forceinline__ void fee_backward(const LsimParams &p, float *G, int T, const FeeState *st,
                                             const float *gint, int lane) {
  const int H = p.max_adc_values;
  const int nwords = (T + kWarp - 1) / kWarp;
  for (int i = lane; i < T; i += kWarp) G[i] = 0.f;
  __syncwarp();
  // hits skipped by the early exit: all-true masks, reset index T-1, rejected
  for (int h = H - 1; h >= st->n_done; --h) {
    float S = 0.f;
    for (int i = lane; i < T; i += kWarp) S += G[i];
    S = warp_sum(S);
    __syncwarp();
    if (lane == 0) G[T - 1] -= S;
    __syncwarp();
  }
  for (int h = st->n_done - 1; h >= 0; --h) {
    float S = 0.f;
    for (int m = 0; m < nwords; ++m) {
      int i = m * kWarp + lane;
      if (i < T) {
        bool bit = (st->mask[h * kMaskWords + m] >> lane) & 1u;
        float g = G[i];
        if (bit) S += g; else G[i] = 0.f;
      }
    }
    S = warp_sum(S);
    __syncwarp();
    if (lane == 0) {
      G[st->e2[h]] -= S;
      if (!st->cond[h]) G[st->e[h]] += gint[h];
    }
    __syncwarp();
  }
  // C = cumsum(W * ts)  ->  dL/dW[i] = ts * sum_{j >= i} dL/dC[j]
  const int per = (T + kWarp - 1) / kWarp;
  const int b = lane * per;
  const int e = min(b + per, T);
  float s = 0.f;
  for (int i = e - 1; i >= b; --i) {
    s += G[i];
    G[i] = s;
  }
  float incl = s;   // suffix sums across lanes
  for (int o = 1; o < kWarp; o <<= 1) {
    float y = __shfl_down_sync(0xffffffffu, incl, o);
    if (lane + o < kWarp) incl += y;
  }
  const float offset = incl - s;
  const float ts = p.t_sampling;
  for (int i = b; i < e; ++i) G[i] = (offset + G[i]) * ts;
  __syncwarp();
}

}  // namespace lsim
