// Sub-pixel bin helpers shared by the pixel-major accumulation
// (lsim_accum.cu) and the segment-major main-bin kernels (lsim_main.cu),
// and the layout of the per-(segment, main pixel) records they exchange.
#pragma once

#include "lsim_common.cuh"

namespace lsim {

constexpr int kChunks = kWinSamples / kWarp;   // window chunks per lane
// Sub-pixel bins per pixel (nb_sampling_bins_per_pixel); the LUT kernels
// require it, so divisions by it compile to multiplications.
constexpr int kBinsPerPixel = 2 * kMainSub;

// Main-bin record of one (segment, pixel whose main bins it covers) pair:
//   rec[0]        boundary correction  n_e * sum_uv W_uv D_uv
//   rec[1 + k]    window value V[k] = n_e * sum_uv W_uv (qa T_{i-1} + qb T_i + qc T_{i+1})[k], k < L
//   rec[1 + k]    0 for L <= k < 159 (so a lane can read 5 chunks unguarded)
//   rec[kRecDl]   d rec[0] / d frac = n_e * sum_uv W_uv (T[c] - T[c+1]) of the cumulative sums
// The adjoint pass overwrites rec[0 .. L] with the cotangents of the same
// quantities.  A segment's bins cover at most 2 x 2 pixels, so each segment
// owns 4 consecutive records, indexed by its pixel offsets.
constexpr int kRecDl = kWinSamples;          // 160
constexpr int kRecFloats = kMainRecFloats;   // 164 floats = 656 bytes
constexpr int kRecPerSeg = kMainRecPerSeg;
static_assert(kRecFloats >= kRecDl + 1 && kRecFloats % 4 == 0, "main-bin record layout");

// Sub-pixel LUT index of a bin, int(|b % nb - nb//2 + 0.5 - shift|)
// (sim_jax.py:435, :443).
__device__ __forceinline__ int lut_index(int b, int nb, int shift) {
  return (int)fabsf(__fsub_rn(__fadd_rn((float)(imod(b, nb) - nb / 2), 0.5f), (float)shift));
}

// Pixel offsets [lo, hi] (relative to the pixel of bin b) covered by the
// kMaxTran bins b - 2 .. b + 2 of one axis; hi - lo <= 1 for nb >= kMaxTran.
__device__ __forceinline__ void axis_range(int b, int nb, int *lo, int *hi) {
  const int pp = ifloordiv(b, nb);
  *lo = ifloordiv(b - kMaxTran / 2, nb) - pp;
  *hi = ifloordiv(b + kMaxTran / 2, nb) - pp;
}

// Record slot (0..3) of the pixel at offset (dx, dy) from the segment's pixel.
__device__ __forceinline__ int rec_slot(int bx, int by, int nb, int dx, int dy) {
  int lx, hx, ly, hy;
  axis_range(bx, nb, &lx, &hx);
  axis_range(by, nb, &ly, &hy);
  return (dx - lx) * 2 + (dy - ly);
}

// Weight (sum of 1-D bin integrals) per main LUT sub-position u in [0, 5)
// for the bins of one axis that fall on the pixel at offset d, and its
// derivative with respect to sigma_T.
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

// Boundary-correction term of one LUT row from its cumulative sums
// (sim_jax.py:237-241, :251-255): cum[Nt-L] - lerp(cum[c], cum[c+1], frac), and its
// derivative with respect to frac.
__device__ __forceinline__ float cum_terms(const float *row, int cath, int Nt, int L, float frac, float *dlerp) {
  const float v0 = __ldg(row + cath);
  const float v1 = __ldg(row + min(cath + 1, Nt - 1));
  const float vs = __ldg(row + Nt - L);
  *dlerp = v0 - v1;
  return vs - (v0 * (1.f - frac) + v1 * frac);
}

}  // namespace lsim
