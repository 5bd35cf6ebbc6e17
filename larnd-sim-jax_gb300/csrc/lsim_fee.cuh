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

constexpr int kMaskWords = 64;   // words per hit: 2 per lane, bit 4m + q for tick 128m + 4 lane + q (T <= 2048)
static_assert(kFeeMaskWords == LSIM_MAX_HITS * kMaskWords, "reset-mask scratch per warp");
constexpr int kFeePass = 4 * kWarp;   // ticks per warp pass: lane l holds ticks 4l .. 4l + 3

struct FeeState {
  int n_done;                  // hits evaluated before the early exit (the rest are empty)
  int e[LSIM_MAX_HITS];        // integration end index
  int e2[LSIM_MAX_HITS];       // reset index
  int cond[LSIM_MAX_HITS];     // 1 = rejected (adc forced to 0)
  float raw[LSIM_MAX_HITS];    // integrated charge before digitisation
  uint32_t *mask;              // [max_adc_values][kMaskWords]: (C - R >= 0) per tick, per hit, lane-private
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

// First q in 0..3 with Q[i0+q] <= thr <= Q[i0+q+1] (Q = base + value) over
// the ticks v0..v3 and the following tick nx, counting only pairs with
// i0 + q < lim - 1; 4 if none.
__device__ __forceinline__ int first_crossing(float v0, float v1, float v2, float v3, float nx, float base, float thr,
                                              int i0, int lim) {
  const float q0 = base + v0, q1 = base + v1, q2 = base + v2, q3 = base + v3, q4 = base + nx;
  int first = 4;
  if (i0 + 3 < lim - 1 && q4 >= thr && q3 <= thr) first = 3;
  if (i0 + 2 < lim - 1 && q3 >= thr && q2 <= thr) first = 2;
  if (i0 + 1 < lim - 1 && q2 >= thr && q1 <= thr) first = 1;
  if (i0 < lim - 1 && q1 >= thr && q0 <= thr) first = 0;
  return first;
}

// Forward self-trigger on C (in place).  normals: per-pixel standard
// normals [1 + 3H] or null (noise off).  Writes adc (digitized) and tick
// per hit through lane 0; fills st when non-null.  C must be 16-byte
// aligned with room for whole 4-tick groups (T rounded up to 4).
//
// Lane l works on ticks 128m + 4l .. 128m + 4l + 3 of pass m (one float4).
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
  float4 *C4 = reinterpret_cast<float4 *>(C);
  // first i < T - 1 with Q[i] <= thr <= Q[i + 1], Q = base + C, for hit 0;
  // later hits' searches run inside the previous hit's reset sweep
  int idx = T - 2;
  for (int i0 = 4 * lane, m = 0; m * kFeePass < T - 1; ++m, i0 += kFeePass) {
    const float4 c = i0 < T ? C4[i0 / 4] : make_float4(0.f, 0.f, 0.f, 0.f);
    float nx = __shfl_down_sync(0xffffffffu, c.x, 1);
    if (lane == kWarp - 1) nx = i0 + 4 < T ? C[i0 + 4] : 0.f;
    const int first = first_crossing(c.x, c.y, c.z, c.w, nx, base, thr, i0, T);
    const unsigned bal = __ballot_sync(0xffffffffu, first < 4);
    if (bal) {
      const int ln = __ffs(bal) - 1;
      idx = m * kFeePass + 4 * ln + __shfl_sync(0xffffffffu, first, ln);
      break;
    }
  }
  for (int h = 0; h < H; ++h) {
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
    // reset: C <- where(C - R < 0, 0, C - R), keep bits per lane (bit 4m + q),
    // and the next hit's crossing search on the reset values: pairs inside a
    // lane's 4 ticks and with the next lane's first tick are tested in the
    // pass; lane 31's last pair waits for lane 0's first value of the next pass
    bool nz = false;
    uint64_t km = 0u;
    int nidx = T - 2;
    bool found = false;
    float carry = 0.f;          // lane 31's last reset value of the previous pass
    for (int i0 = 4 * lane, sh = 0, m = 0; i0 - 4 * lane < T; i0 += kFeePass, sh += 4, ++m) {
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (i0 < T) {
        const float4 c = C4[i0 / 4];
        v[0] = c.x; v[1] = c.y; v[2] = c.z; v[3] = c.w;
        uint32_t bits = 0u;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (i0 + q < T) {
            const float d = v[q] - R;
            const bool keep = !(d < 0.f);
            v[q] = keep ? d : 0.f;
            nz |= keep && d != 0.f;
            bits |= (keep ? 1u : 0u) << q;
          }
        }
        C4[i0 / 4] = make_float4(v[0], v[1], v[2], v[3]);
        km |= (uint64_t)bits << sh;
      }
      const float nx = __shfl_down_sync(0xffffffffu, v[0], 1);
      const float v0 = __shfl_sync(0xffffffffu, v[0], 0);
      if (!found) {
        // the pair (128m - 1, 128m) left over from the previous pass
        const int ip = m * kFeePass - 1;
        if (m > 0 && ip < T - 1 && base + v0 >= thr && base + carry <= thr) {
          nidx = ip;
          found = true;
        } else {
          const int first = lane < kWarp - 1 ? first_crossing(v[0], v[1], v[2], v[3], nx, base, thr, i0, T)
                                             : first_crossing(v[0], v[1], v[2], v[3], 0.f, base, thr, i0, min(T, i0 + 4));
          const unsigned bal = __ballot_sync(0xffffffffu, first < 4);
          if (bal) {
            const int ln = __ffs(bal) - 1;
            nidx = m * kFeePass + 4 * ln + __shfl_sync(0xffffffffu, first, ln);
            found = true;
          }
        }
      }
      carry = __shfl_sync(0xffffffffu, v[3], kWarp - 1);
    }
    idx = nidx;
    if (st) {
      st->mask[h * kMaskWords + 2 * lane] = (uint32_t)km;
      st->mask[h * kMaskWords + 2 * lane + 1] = (uint32_t)(km >> 32);
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
// T must be a multiple of 4 and G 16-byte aligned.
__device__ __forceinline__ void fee_backward(const LsimParams &p, float *G, int T, const FeeState *st,
                                             const float *gint, int lane) {
  float4 *G4 = reinterpret_cast<float4 *>(G);
  for (int i = 4 * lane; i < T; i += kFeePass) G4[i / 4] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncwarp();
  // Hits skipped by the early exit have all-true masks, reset index T-1 and
  // no charge: each maps G to G - e_{T-1} sum(G).  After the first of them
  // sum(G) is zero, so one application is the whole chain.
  if (st->n_done < p.max_adc_values) {
    float S = 0.f;
    for (int i = 4 * lane; i < T; i += kFeePass) {
      const float4 g = G4[i / 4];
      S += (g.x + g.y) + (g.z + g.w);
    }
    S = warp_sum(S);
    __syncwarp();
    if (lane == 0) G[T - 1] -= S;
    __syncwarp();
  }
  // this lane's 64 keep bits of hit h (the next hit's are loaded ahead)
  auto keep_bits = [&](int h) {
    const uint2 m = *reinterpret_cast<const uint2 *>(st->mask + h * kMaskWords + 2 * lane);
    return (uint64_t)m.x | ((uint64_t)m.y << 32);
  };
  uint64_t kn = st->n_done > 0 ? keep_bits(st->n_done - 1) : 0u;
  for (int h = st->n_done - 1; h >= 0; --h) {
    uint64_t km = kn;
    if (h > 0) kn = keep_bits(h - 1);
    float S = 0.f;
    for (int i0 = 4 * lane; i0 < T; i0 += kFeePass, km >>= 4) {
      const uint32_t bits = (uint32_t)km;
      float4 g = G4[i0 / 4];
      if (bits & 1u) S += g.x; else g.x = 0.f;
      if (bits & 2u) S += g.y; else g.y = 0.f;
      if (bits & 4u) S += g.z; else g.z = 0.f;
      if (bits & 8u) S += g.w; else g.w = 0.f;
      G4[i0 / 4] = g;
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
