// Pixel-major LUT accumulation: one warp owns one pixel row at a time
// (persistent warps pull rows from a work counter), holds the 2001-tick
// waveform in shared memory and adds every contribution of every segment
// whose principal pixel lies within number_pix_neighbors of it.  No global
// atomics touch waveform data; the per-pixel contribution order is fixed,
// so results are deterministic.
//
// Reference: simulate_signals (sim_jax.py:141-286).  A contribution of
// segment s to pixel p places, at window origin col0 = Nt - L - c - 1,
//   r = 0      : corr * frac
//   r = 1      : corr * (1 - frac) + V[0] * frac
//   r = 2..L   : V[r-2] * (1 - frac) + V[r-1] * frac
//   r = L + 1  : V[L-1] * (1 - frac)
// where V[k] = sum over the main bins on p of q_ij * (T_i b + T_{i-1} a +
// T_{i+1} c)[cx, cy, Nt-L+k]  plus, when p is a neighbour, T_0[cx, cy,
// Nt-L+k] * n_e; corr is the matching cumulative-sum boundary correction.
// Value parts land only in waveform columns [2, Nticks-1], correction parts
// only in [1, Nticks-2] (the index remaps of sim_jax.py:177-178, :243-244).
#include "lsim_internal.cuh"
#include "lsim_fee.cuh"

namespace lsim {

constexpr int kAccWarps = 4;
constexpr int kRowPad = 3;            // row[col] at buf[kRowPad + col]: col 1 is 16-byte aligned
constexpr int kRowFloats = 2052;      // >= kRowPad + n_ticks (2001), multiple of 4
constexpr int kMaxList = 81;          // (2 * 4 + 1)^2 neighbourhood slots

struct ListSmem {
  int off[kMaxList];
  int cnt[kMaxList];
  int dxy[kMaxList];
  int n;
};

template <bool GRAD>
struct WarpSmem;
template <>
struct WarpSmem<false> {
  float buf[kRowFloats];
  ListSmem list;
  float adc[LSIM_MAX_HITS];
};
template <>
struct WarpSmem<true> {
  float buf[kRowFloats];
  ListSmem list;
  float adc[LSIM_MAX_HITS];
  float gint[LSIM_MAX_HITS];
  FeeState fee;
};

struct Theta {
  float v[LSIM_NPARAM];
  float loss;
};

// Sub-pixel LUT index of a bin, int(|b % nb - nb//2 + 0.5 - shift|)
// (sim_jax.py:435, :443).
__device__ __forceinline__ int lut_index(int b, int nb, int shift) {
  return (int)fabsf(__fsub_rn(__fadd_rn((float)(imod(b, nb) - nb / 2), 0.5f), (float)shift));
}

// Weight (sum of 1-D bin integrals) per main LUT sub-position u in [0, 5)
// for the bins of one axis that fall on the target pixel.
__device__ __forceinline__ void axis_weights(const float e[kMaxTran], const float de[kMaxTran], int b, int nb,
                                             int d, float W[kMainSub], float dW[kMainSub], unsigned *umask) {
  const int pp = ifloordiv(b, nb);
  unsigned um = 0;
#pragma unroll
  for (int u = 0; u < kMainSub; ++u) { W[u] = 0.f; dW[u] = 0.f; }
#pragma unroll
  for (int i = 0; i < kMaxTran; ++i) {
    const int bi = b + i - kMaxTran / 2;
    if (ifloordiv(bi, nb) - pp != d) continue;
    const int u = lut_index(bi, nb, 0);
#pragma unroll
    for (int uu = 0; uu < kMainSub; ++uu)
      if (uu == u) { W[uu] += e[i]; dW[uu] += de[i]; }
    um |= 1u << u;
  }
  *umask = um;
}

struct Contribution {
  // segment quantities
  float ne, frac, qa, qb, qc;
  int cath, tidx;
  // neighbour part
  bool has_n;
  int n_off;              // (cx * ny + cy)
  // main part
  unsigned umask, vmask;
  float Xw[kMainSub], Yw[kMainSub], dXw[kMainSub], dYw[kMainSub];
  // window
  int cb;                 // window origin column (s0 - 1)
  float corr;             // boundary correction (forward)
};

__device__ __forceinline__ bool setup_contribution(const LsimParams &p, const SegFwd *__restrict__ segf,
                                                   const SegAdj *__restrict__ sega, int s, int dx, int dy,
                                                   bool need_deriv, Contribution &c) {
  const SegFwd &f = segf[s];
  c.ne = f.ne;
  if (c.ne == 0.f) return false;
  c.frac = f.frac; c.qa = f.qa; c.qb = f.qb; c.qc = f.qc;
  c.cath = f.cath; c.tidx = f.tidx;
  const int nb = p.nb_bins_per_pixel;
  c.has_n = (dx != 0 || dy != 0);
  if (c.has_n) {
    const int cx = lut_index(f.bx, nb, dx * nb);
    const int cy = lut_index(f.by, nb, dy * nb);
    c.n_off = cx * p.lut_ny + cy;
  }
  c.umask = 0; c.vmask = 0;
  if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1) {
    float ex[kMaxTran], ey[kMaxTran], dex[kMaxTran], dey[kMaxTran];
#pragma unroll
    for (int i = 0; i < kMaxTran; ++i) {
      ex[i] = f.ex[i]; ey[i] = f.ey[i];
      dex[i] = need_deriv ? sega[s].dex[i] : 0.f;
      dey[i] = need_deriv ? sega[s].dey[i] : 0.f;
    }
    axis_weights(ex, dex, f.bx, nb, dx, c.Xw, c.dXw, &c.umask);
    axis_weights(ey, dey, f.by, nb, dy, c.Yw, c.dYw, &c.vmask);
    if (!c.umask || !c.vmask) { c.umask = 0; c.vmask = 0; }
  }
  if (!c.has_n && !c.umask) return false;
  c.cb = p.lut_nt - p.signal_length - c.cath - 1;
  return true;
}

// Boundary correction of a contribution (sim_jax.py:236-261), and for the
// adjoint its per-part derivative pieces.
struct CorrParts {
  float Dn;      // neighbour: Cum0[Nt-L] - lerp
  float dCn;     // neighbour: Cum0[c] - Cum0[c+1]
};

__device__ __forceinline__ float cum_terms(const float *row, int cath, int Nt, int L, float frac, float *dlerp) {
  const float v0 = __ldg(row + cath);
  const float v1 = __ldg(row + min(cath + 1, Nt - 1));
  const float vs = __ldg(row + Nt - L);
  *dlerp = v0 - v1;
  return vs - (v0 * (1.f - frac) + v1 * frac);
}

__device__ __forceinline__ float correction(const LsimParams &p, const Tables &tab, const Contribution &c) {
  const int Nt = p.lut_nt, L = p.signal_length;
  float corr = 0.f, dl;
  if (c.has_n) corr += cum_terms(tab.c0 + (size_t)c.n_off * Nt, c.cath, Nt, L, c.frac, &dl) * c.ne;
  if (c.umask) {
    float cm = 0.f;
#pragma unroll
    for (int u = 0; u < kMainSub; ++u) {
      if (!((c.umask >> u) & 1u)) continue;
#pragma unroll
      for (int v = 0; v < kMainSub; ++v) {
        if (!((c.vmask >> v) & 1u)) continue;
        const float *row = tab.cm + ((size_t)(c.tidx * kMainSub + u) * kMainSub + v) * Nt;
        cm += (c.Xw[u] * c.Yw[v]) * cum_terms(row, c.cath, Nt, L, c.frac, &dl);
      }
    }
    corr += cm * c.ne;
  }
  return corr;
}

// V[k] of a contribution (k in [0, L)).
__device__ __forceinline__ float value_at(const LsimParams &p, const Tables &tab, const Contribution &c, int k) {
  const int L = p.signal_length;
  float V = 0.f;
  if (c.has_n) V = __ldg(tab.w0 + (size_t)c.n_off * L + k) * c.ne;
  if (c.umask) {
    float vm = 0.f;
#pragma unroll
    for (int u = 0; u < kMainSub; ++u) {
      if (!((c.umask >> u) & 1u)) continue;
#pragma unroll
      for (int v = 0; v < kMainSub; ++v) {
        if (!((c.vmask >> v) & 1u)) continue;
        const float4 t = __ldg(tab.wmp + ((size_t)(c.tidx * kMainSub + u) * kMainSub + v) * L + k);
        const float B = (t.y * c.qb + t.x * c.qa) + t.z * c.qc;
        vm += (c.Xw[u] * c.Yw[v]) * B;
      }
    }
    V += vm * c.ne;
  }
  return V;
}

// Forward: add one contribution's L+2 window into the pixel row.
__device__ __forceinline__ void add_window(const LsimParams &p, const Tables &tab, const Contribution &c, float *row,
                                           int lane) {
  const int L = p.signal_length, NT = p.n_ticks;
  const float corr = correction(p, tab, c);
  const float f = c.frac, f1 = 1.f - c.frac;
  float carry = 0.f;
  for (int r0 = 0; r0 < L + 2; r0 += kWarp) {
    const int r = r0 + lane;
    const int k = r - 1;
    const float Vk = (k >= 0 && k < L) ? value_at(p, tab, c, k) : 0.f;
    float prev = __shfl_up_sync(0xffffffffu, Vk, 1);
    if (lane == 0) prev = carry;
    carry = __shfl_sync(0xffffffffu, Vk, kWarp - 1);
    const int col = c.cb + r;
    if (r < L + 2) {
      float val = 0.f;
      if (col >= 2 && col <= NT - 1) val = prev * f1 + Vk * f;
      if (col >= 1 && col <= NT - 2) {
        if (r == 0) val += corr * f;
        else if (r == 1) val += corr * f1;
      }
      if (col >= 1 && col <= NT - 1) row[col] += val;
    }
  }
}

// Adjoint: accumulate dL/dtheta of one contribution given the waveform
// cotangent grow[col] (zero outside [1, Nticks-1]).
__device__ __forceinline__ void window_vjp(const LsimParams &p, const Tables &tab, const Contribution &c,
                                           const SegAdj &a, const float *grow, Theta &th, int lane) {
  const int L = p.signal_length, NT = p.n_ticks, Nt = p.lut_nt;
  const float f = c.frac, f1 = 1.f - c.frac;
  auto Gv = [&](int col) { return (col >= 2 && col <= NT - 1) ? grow[col] : 0.f; };
  auto Gc = [&](int col) { return (col >= 1 && col <= NT - 2) ? grow[col] : 0.f; };
  // acc_fr holds frac terms already scaled by ne; acc_frm main-part terms
  // still to be multiplied by ne (as are acc_sig, acc_a, acc_b, acc_c).
  float acc_ne = 0.f, acc_sig = 0.f, acc_a = 0.f, acc_b = 0.f, acc_c = 0.f, acc_fr = 0.f, acc_frm = 0.f;
  for (int k = lane; k < L; k += kWarp) {
    const float gA = Gv(c.cb + k + 1);   // V[k] * frac lands at col cb + k + 1
    const float gB = Gv(c.cb + k + 2);   // V[k] * (1 - frac) at col cb + k + 2
    const float dV = gA * f + gB * f1;
    const float dG = gA - gB;
    if (c.has_n) {
      const float t0 = __ldg(tab.w0 + (size_t)c.n_off * L + k);
      acc_ne += dV * t0;
      acc_fr += (t0 * c.ne) * dG;
    }
    if (c.umask) {
#pragma unroll
      for (int u = 0; u < kMainSub; ++u) {
        if (!((c.umask >> u) & 1u)) continue;
#pragma unroll
        for (int v = 0; v < kMainSub; ++v) {
          if (!((c.vmask >> v) & 1u)) continue;
          const float4 t = __ldg(tab.wmp + ((size_t)(c.tidx * kMainSub + u) * kMainSub + v) * L + k);
          const float B = (t.y * c.qb + t.x * c.qa) + t.z * c.qc;
          const float W = c.Xw[u] * c.Yw[v];
          const float dW = c.dXw[u] * c.Yw[v] + c.Xw[u] * c.dYw[v];
          const float dVB = dV * B;
          acc_ne += W * dVB;
          acc_sig += dW * dVB;
          const float dVW = dV * W;
          acc_a += dVW * t.x;
          acc_b += dVW * t.y;
          acc_c += dVW * t.z;
          acc_frm += (W * B) * dG;
        }
      }
    }
  }
  // boundary corrections (per contribution, counted once by lane 0)
  if (lane == 0) {
    const int cb = c.cb;
    const float gc0 = Gc(cb), gc1 = Gc(cb + 1);
    const float dcorr = gc0 * f + gc1 * f1;
    const float dgc = gc0 - gc1;
    float dl;
    if (c.has_n) {
      const float Dn = cum_terms(tab.c0 + (size_t)c.n_off * Nt, c.cath, Nt, L, f, &dl);
      acc_ne += dcorr * Dn;
      acc_fr += (dcorr * dl + Dn * dgc) * c.ne;
    }
    if (c.umask) {
#pragma unroll
      for (int u = 0; u < kMainSub; ++u) {
        if (!((c.umask >> u) & 1u)) continue;
#pragma unroll
        for (int v = 0; v < kMainSub; ++v) {
          if (!((c.vmask >> v) & 1u)) continue;
          const float *row = tab.cm + ((size_t)(c.tidx * kMainSub + u) * kMainSub + v) * Nt;
          const float D = cum_terms(row, c.cath, Nt, L, f, &dl);
          const float W = c.Xw[u] * c.Yw[v];
          const float dW = c.dXw[u] * c.Yw[v] + c.Xw[u] * c.dYw[v];
          acc_ne += dcorr * W * D;
          acc_sig += dcorr * dW * D;
          acc_frm += W * (dcorr * dl + D * dgc);
        }
      }
    }
  }
  const float ne = c.ne;
  const float sig = acc_sig * ne;
  const float lsum = (acc_a * a.dqa + acc_b * a.dqb + acc_c * a.dqc) * ne;
  const float dt0 = (acc_fr + acc_frm * ne) / p.t_sampling;
  th.v[0] += acc_ne * a.dne[0];
  th.v[1] += acc_ne * a.dne[1];
  th.v[2] += acc_ne * a.dne[2] + sig * a.dsig[0] + lsum * a.dld[0] + dt0 * a.dt0;
  th.v[3] += acc_ne * a.dne[3];
  th.v[5] += lsum * a.dld[1];
  th.v[6] += sig * a.dsig[1];
  th.v[7] += acc_ne * a.dne[4];
}

// Build the neighbourhood slot list of a pixel (compacted, fixed order).
__device__ __forceinline__ void build_list(const Grid &g, const int32_t *__restrict__ cnt,
                                           const int32_t *__restrict__ off, int64_t slot, ListSmem &ls, int lane) {
  const int D = 2 * g.n + 1;
  int base = 0;
  for (int i0 = 0; i0 < D * D; i0 += kWarp) {
    const int idx = i0 + lane;
    int c = 0, o = 0, dxy = 0;
    if (idx < D * D) {
      const int dx = idx / D - g.n, dy = idx % D - g.n;
      const int64_t q = slot - (int64_t)dy * g.nxe - dx;
      c = __ldg(cnt + q);
      if (c > 0) o = __ldg(off + q);
      dxy = (dx + 16) | ((dy + 16) << 8);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, c > 0);
    if (c > 0) {
      const int pos = base + __popc(bal & ((1u << lane) - 1u));
      ls.off[pos] = o; ls.cnt[pos] = c; ls.dxy[pos] = dxy;
    }
    base += __popc(bal);
  }
  if (lane == 0) ls.n = base;
  __syncwarp();
}

template <typename F>
__device__ __forceinline__ void for_each_contribution(const int32_t *__restrict__ seg_list, const ListSmem &ls,
                                                      int lane, F &&fn) {
  for (int e = 0; e < ls.n; ++e) {
    const int o = ls.off[e], c = ls.cnt[e], dxy = ls.dxy[e];
    const int dx = (dxy & 0xff) - 16, dy = ((dxy >> 8) & 0xff) - 16;
    for (int j0 = 0; j0 < c; j0 += kWarp) {
      const int mine = (j0 + lane < c) ? __ldg(seg_list + o + j0 + lane) : -1;
      const int m = min(kWarp, c - j0);
      for (int jj = 0; jj < m; ++jj) {
        const int s = __shfl_sync(0xffffffffu, mine, jj);
        fn(s, dx, dy);
      }
    }
  }
}

__device__ __forceinline__ int32_t slot_pid(const LsimParams &p, const Grid &g, int64_t slot) {
  const int64_t ev = slot / g.event_stride;
  const int64_t rem = slot - ev * g.event_stride;
  const int plane = (int)(rem / g.plane_stride);
  const int64_t inplane = rem % g.plane_stride;
  const int py = (int)(inplane / g.nxe) - g.n, px = (int)(inplane % g.nxe) - g.n;
  return pixel2id(p, px, py, plane, (int)ev - 1);
}

template <int MODE>
__global__ void __launch_bounds__(kAccWarps * kWarp) k_lut_pixels(AccumArgs a) {
  constexpr bool GRAD = (MODE == kModeGrad);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  WarpSmem<GRAD> &sm = reinterpret_cast<WarpSmem<GRAD> *>(smem_raw)[wid];
  const LsimParams &p = a.p;
  float *row = sm.buf + kRowPad;
  const int NT = p.n_ticks;
  const int T = NT - 1;
  const int H = p.max_adc_values;
  const int n_valid = a.w.counts->n_valid;
  Theta th;
#pragma unroll
  for (int i = 0; i < LSIM_NPARAM; ++i) th.v[i] = 0.f;
  th.loss = 0.f;
  for (;;) {
    int r = 0;
    if (lane == 0) r = atomicAdd(&a.w.counts->work, 1);
    r = __shfl_sync(0xffffffffu, r, 0);
    if (r >= n_valid) break;
    const int64_t slot = a.w.pix_slot[r];
    // zero the row
    float4 *b4 = reinterpret_cast<float4 *>(sm.buf);
    for (int i = lane; i < kRowFloats / 4; i += kWarp) b4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    build_list(a.g, a.w.cnt, a.w.off, slot, sm.list, lane);
    __syncwarp();
    for_each_contribution(a.w.seg_list, sm.list, lane, [&](int s, int dx, int dy) {
      Contribution c;
      if (setup_contribution(p, a.w.segf, a.w.sega, s, dx, dy, false, c)) add_window(p, a.tab, c, row, lane);
    });
    __syncwarp();
    if (MODE == kModeWfs) {
      float4 *dst = reinterpret_cast<float4 *>(a.wfs + (a.row_offset + r) * (int64_t)T);
      const float4 *src = reinterpret_cast<const float4 *>(row + 1);
      for (int i = lane; i < T / 4; i += kWarp) dst[i] = src[i];
      continue;
    }
    // ---- front end on the output ticks (row + 1)
    const float *nrm = a.normals ? a.normals + (int64_t)r * (1 + 3 * H) : nullptr;
    float *adc_dst = a.adc_out ? a.adc_out + (int64_t)r * H : nullptr;
    float *tick_dst = a.tick_out ? a.tick_out + (int64_t)r * H : nullptr;
    warp_cumsum_charge(row + 1, T, p.t_sampling, lane);
    if (MODE == kModeAdc) {
      fee_forward(p, row + 1, T, nrm, adc_dst, tick_dst, nullptr, nullptr, lane);
      continue;
    }
    if constexpr (GRAD) {
      fee_forward(p, row + 1, T, nrm, adc_dst, tick_dst, &sm.fee, nullptr, lane);
      // cotangent of the integrated charges
      if (lane == 0) {
        int32_t pid = -2;
        int64_t tr = -1;
        if (!a.g_adc) {
          pid = slot_pid(p, a.g, slot);
          int64_t lo = 0, hi = a.n_tgt;
          while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (a.tgt_pids[mid] < pid) lo = mid + 1; else hi = mid;
          }
          if (lo < a.n_tgt && a.tgt_pids[lo] == pid) tr = lo;
        }
        const float adc0 = digitize(p, 0.f);
        for (int h = 0; h < H; ++h) {
          const float raw = sm.fee.raw[h];
          const float adc = digitize(p, raw);
          float g;
          if (a.g_adc) {
            g = a.g_adc[(int64_t)r * H + h];
          } else {
            const float tgt = tr >= 0 ? a.tgt_adc[tr * H + h] : adc0;
            const float d = adc - tgt;
            th.loss += d * d;
            g = 2.f * d;
          }
          sm.gint[h] = digitize_vjp(p, raw, g);
        }
      }
      __syncwarp();
      // dL/dW over output ticks, in place (row + 1), column 0 and tail zeroed
      fee_backward(p, row + 1, T, &sm.fee, sm.gint, lane);
      if (lane == 0) row[0] = 0.f;
      __syncwarp();
      for_each_contribution(a.w.seg_list, sm.list, lane, [&](int s, int dx, int dy) {
        Contribution c;
        if (setup_contribution(p, a.w.segf, a.w.sega, s, dx, dy, true, c)) {
          const SegAdj &adj = a.w.sega[s];
          window_vjp(p, a.tab, c, adj, row, th, lane);
        }
      });
      __syncwarp();
    }
  }
  if constexpr (GRAD) {
    const int gw = blockIdx.x * kAccWarps + wid;
    for (int i = 0; i < LSIM_NPARAM; ++i) th.v[i] = warp_sum(th.v[i]);
    th.loss = warp_sum(th.loss);
    if (lane == 0) {
      float *dst = a.w.grad_partials + (size_t)gw * kGradSlots;
      dst[0] = th.loss;
      for (int i = 0; i < LSIM_NPARAM; ++i) dst[1 + i] = th.v[i];
    }
  }
}

// Loss terms of target pixels that the prediction does not have.
__global__ void k_target_only(AccumArgs a, float *partials) {
  __shared__ float sh[256 / kWarp];
  const LsimParams &p = a.p;
  const int H = p.max_adc_values;
  const float adc0 = digitize(p, 0.f);
  const int n_valid = a.w.counts->n_valid;
  float acc = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < a.n_tgt; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t pid = a.tgt_pids[t];
    int lo = 0, hi = n_valid;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (slot_pid(p, a.g, a.w.pix_slot[mid]) < pid) lo = mid + 1; else hi = mid;
    }
    const bool present = lo < n_valid && slot_pid(p, a.g, a.w.pix_slot[lo]) == pid;
    if (!present && pid >= 0)
      for (int h = 0; h < H; ++h) {
        const float d = adc0 - a.tgt_adc[t * H + h];
        acc += d * d;
      }
  }
  acc = warp_sum(acc);
  if (threadIdx.x % kWarp == 0) sh[threadIdx.x / kWarp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < 256 / kWarp; ++i) s += sh[i];
    partials[blockIdx.x] = s;
  }
}

__global__ void k_grad_finalize(const float *grad_partials, int n_warps, const float *tgt_partials, int n_tgt_blocks,
                                float *loss_out, float *grad_out) {
  const int i = threadIdx.x;   // 0: loss, 1..8: grads
  if (i > LSIM_NPARAM) return;
  float s = 0.f;
  for (int w = 0; w < n_warps; ++w) s += grad_partials[(size_t)w * kGradSlots + i];
  if (i == 0) {
    for (int b = 0; b < n_tgt_blocks; ++b) s += tgt_partials[b];
    if (loss_out) loss_out[0] = s;
  } else if (grad_out) {
    grad_out[i - 1] = s;
  }
}

// ---------------------------------------------------------------- launch

// Persistent grid: every SM filled to its occupancy limit, capped so the
// per-warp gradient partials fit their buffer.  A pure function of the
// device and the mode, so it is the same at launch and at finalisation.
template <int MODE>
static int grid_blocks(int *blocks) {
  constexpr bool GRAD = (MODE == kModeGrad);
  const size_t smem = sizeof(WarpSmem<GRAD>) * kAccWarps;
  if (cudaFuncSetAttribute(k_lut_pixels<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return LSIM_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lut_pixels<MODE>, kAccWarps * kWarp, smem) !=
      cudaSuccess)
    return LSIM_ERR_CUDA;
  if (per_sm < 1) per_sm = 1;
  int b = device_sm_count() * per_sm;
  const int max_blocks = kGradBlocks / kAccWarps;
  *blocks = b > max_blocks ? max_blocks : b;
  return LSIM_OK;
}

template <int MODE>
static int launch_mode(const AccumArgs &a, cudaStream_t st) {
  constexpr bool GRAD = (MODE == kModeGrad);
  const size_t smem = sizeof(WarpSmem<GRAD>) * kAccWarps;
  int blocks = 0;
  int rc = grid_blocks<MODE>(&blocks);
  if (rc != LSIM_OK) return rc;
  // reset the work counter
  if (cudaMemsetAsync(&a.w.counts->work, 0, sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  k_lut_pixels<MODE><<<blocks, kAccWarps * kWarp, smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

int run_accum(AccumMode mode, const AccumArgs &a, cudaStream_t st) {
  if (a.p.n_neighbors > 4 || a.p.n_tran_bins != kMaxTran || a.p.nb_bins_per_pixel != 2 * kMainSub ||
      a.p.n_ticks - 1 + kRowPad > kRowFloats || (a.p.n_ticks - 1) % 4 != 0 || a.p.max_adc_values > LSIM_MAX_HITS)
    return LSIM_ERR_UNSUPPORTED;
  switch (mode) {
    case kModeWfs: return launch_mode<kModeWfs>(a, st);
    case kModeAdc: return launch_mode<kModeAdc>(a, st);
    case kModeGrad: return launch_mode<kModeGrad>(a, st);
  }
  return LSIM_ERR_INVALID;
}

int run_grad_finalize(const AccumArgs &a, float *loss_out, float *grad_out, cudaStream_t st) {
  int blocks = 0;
  int rc = grid_blocks<kModeGrad>(&blocks);
  if (rc != LSIM_OK) return rc;
  const int n_warps = blocks * kAccWarps;
  // target-only partials reuse the tail of the grad-partials buffer
  float *tgt_partials = a.w.grad_partials + (size_t)n_warps * kGradSlots;
  int tb = 0;
  if (!a.g_adc && a.n_tgt > 0) {
    tb = 64;
    k_target_only<<<tb, 256, 0, st>>>(a, tgt_partials);
  }
  k_grad_finalize<<<1, 32, 0, st>>>(a.w.grad_partials, n_warps, tgt_partials, tb, loss_out, grad_out);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
