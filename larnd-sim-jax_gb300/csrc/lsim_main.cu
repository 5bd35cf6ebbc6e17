// Main-bin parts of LUT mode, segment-major.
//
// A segment's 5 x 5 transverse-diffusion bins cover at most 2 x 2 pixels.
// For each covered pixel the window it adds is
//   V[k] = n_e * sum over the bins (i, j) on that pixel of
//          ex_i ey_j * (a T_{t-1} + b T_t + c T_{t+1})[cx_i, cy_j, Nt - L + k]
// (main_vals_2d, sim_jax.py:186-192) with the quadratic long-diffusion
// interpolation weights (a, b, c) (sim_jax.py:162-168) and the
// cumulative-sum boundary term (sim_jax.py:237-241).  Bins of one pixel that share a LUT sub-position
// (u, v) are grouped, W_uv = sum ex_i * sum ey_j, so each window reads at
// most 25 LUT rows.
//
// k_main_records computes V and the boundary term once per (segment,
// pixel) and stores them as a record; the pixel-major accumulation adds the
// record like a neighbour part.  After the pixel-major adjoint has replaced
// the record by its cotangent, k_main_adjoint projects it back onto n_e,
// sigma_T and (a, b, c) and accumulates dL/dtheta per warp.  One warp owns
// one segment at a time; blocks own fixed contiguous segment ranges that
// their warps interleave, so the per-warp gradient records and their
// reduction order are fixed.
#include "lsim_internal.cuh"
#include "lsim_bins.cuh"
#include "lsim_fee.cuh"

namespace lsim {

constexpr int kMainBlockWarps = 8;

// Grouped LUT sub-positions of one (segment, pixel) pair: row offset
// (tidx*5 + u)*5 + v into the window tables, W, dW/dsigma_T, the
// cumulative-sum term D and dD/dfrac.
struct MainSmem {
  int off[kMainSub * kMainSub];
  float W[kMainSub * kMainSub], dW[kMainSub * kMainSub];
  float D[kMainSub * kMainSub], dl[kMainSub * kMainSub];
};

// Lane l < 25 owns sub-position (u, v) = (l / 5, l % 5); the owners of
// sub-positions with bins on the pixel are compacted in (u, v) order.
// Returns the entry count; *wd and *wdl are sum W D and sum W dD/dfrac.
template <bool GRAD>
__device__ __forceinline__ int main_entries(const LsimParams &p, const Tables &tab, const SegFwd &f,
                                            const SegAdj *a, int dx, int dy, MainSmem &ms, float *wd, float *wdl,
                                            int lane) {
  constexpr int nbp = kBinsPerPixel;
  // this lane's sub-position (u, v): summed 1-D bin integrals of the bins of
  // each axis that fall on the pixel with that LUT index (axis_weights, per lane)
  const int u = lane / kMainSub, v = lane % kMainSub;
  float xw = 0.f, yw = 0.f, dxw = 0.f, dyw = 0.f;
  unsigned um = 0u, vm = 0u;
  const int bx = f.bx, by = f.by, ppx = ifloordiv(bx, nbp), ppy = ifloordiv(by, nbp);
  // the record's bin integrals, loaded up front (one 96-byte segment record)
  float ex[kMaxTran], ey[kMaxTran], dex[kMaxTran], dey[kMaxTran];
#pragma unroll
  for (int i = 0; i < kMaxTran; ++i) {
    ex[i] = f.ex[i];
    ey[i] = f.ey[i];
    dex[i] = GRAD ? a->dex[i] : 0.f;
    dey[i] = GRAD ? a->dey[i] : 0.f;
  }
#pragma unroll
  for (int i = 0; i < kMaxTran; ++i) {
    const int bi = bx + i - kMaxTran / 2, bj = by + i - kMaxTran / 2;
    const bool onx = ifloordiv(bi, nbp) - ppx == dx, ony = ifloordiv(bj, nbp) - ppy == dy;
    const int ui = lut_index(bi, nbp, 0), vj = lut_index(bj, nbp, 0);
    um |= onx ? 1u << ui : 0u;
    vm |= ony ? 1u << vj : 0u;
    const bool tx = onx && ui == u, ty = ony && vj == v;
    xw += tx ? ex[i] : 0.f;
    dxw += tx ? dex[i] : 0.f;
    yw += ty ? ey[i] : 0.f;
    dyw += ty ? dey[i] : 0.f;
  }
  const bool mine = lane < kMainSub * kMainSub && ((um >> u) & 1u) && ((vm >> v) & 1u);
  const unsigned bal = __ballot_sync(0xffffffffu, mine);
  float s_wd = 0.f, s_wdl = 0.f;
  if (mine) {
    const int pos = __popc(bal & ((1u << lane) - 1u));
    const int off = (f.tidx * kMainSub + u) * kMainSub + v;
    float dl;
    const float D = cum_terms(tab.cm + (size_t)off * p.lut_nt, f.cath, p.lut_nt, p.signal_length, f.frac, &dl);
    const float W = xw * yw;
    ms.off[pos] = off;
    ms.W[pos] = W;
    ms.dW[pos] = dxw * yw + xw * dyw;
    ms.D[pos] = D;
    ms.dl[pos] = dl;
    s_wd = W * D;
    s_wdl = W * dl;
  }
  *wd = warp_sum(s_wd);
  *wdl = warp_sum(s_wdl);
  __syncwarp();
  return __popc(bal);
}

// Segments of this block: a contiguous range, interleaved over its warps
// (warp w takes s0 + w, s0 + w + kMainBlockWarps, ...), so the warps of a
// block work on neighbouring segments -- usually of one track, with the same
// template index -- and share their LUT rows in L1.
__device__ __forceinline__ void block_range(int64_t n_rows, int64_t *s0, int64_t *s1) {
  const int64_t chunk = (n_rows + gridDim.x - 1) / gridDim.x;
  *s0 = (int64_t)blockIdx.x * chunk + threadIdx.x / kWarp;
  *s1 = min(n_rows, (int64_t)blockIdx.x * chunk + chunk);
}

__global__ void __launch_bounds__(kMainBlockWarps * kWarp, 2) k_main_records(LsimParams p, Tables tab, Workspace w, Grid g,
                                                                           int64_t n_rows) {
  __shared__ MainSmem sms[kMainBlockWarps];
  const int lane = threadIdx.x % kWarp;
  MainSmem &ms = sms[threadIdx.x / kWarp];
  constexpr int nbp = kBinsPerPixel;
  int n_rec = 0;
  int64_t s0, s1;
  block_range(n_rows, &s0, &s1);
  for (int64_t s = s0; s < s1; s += kMainBlockWarps) {
    const SegFwd &f = w.segf[s];
    const float ne = f.ne;
    const int32_t key = w.key[s];
    if (ne == 0.f || key < 0) continue;
    const float qa = f.qa, qb = f.qb, qc = f.qc;
    int lx, hx, ly, hy;
    axis_range(f.bx, nbp, &lx, &hx);
    axis_range(f.by, nbp, &ly, &hy);
#pragma unroll 1
    for (int dx = lx; dx <= hx; ++dx)
#pragma unroll 1
      for (int dy = ly; dy <= hy; ++dy) {
        // records of pixels that are not simulated are never read (the
        // reference drops main bins outside unique_pixels, sim_jax.py:152-154)
        if (!slot_is_pixel(g, w.cnt, (int64_t)key + (int64_t)dy * g.nxe + dx)) continue;
        float wd, wdl;
        const int n = main_entries<false>(p, tab, f, nullptr, dx, dy, ms, &wd, &wdl, lane);
        float acc[kChunks];
#pragma unroll
        for (int j = 0; j < kChunks; ++j) acc[j] = 0.f;
#pragma unroll 2
        for (int e = 0; e < n; ++e) {
          // padded rows: entry idx is sample idx - 1, matching the record layout
          const float4 *src = tab.wmp + (size_t)ms.off[e] * kWinSamples + lane;
          const float W = ms.W[e];
          const float wa = W * qa, wb = W * qb, wc = W * qc;
#pragma unroll
          for (int j = 0; j < kChunks; ++j) {
            const float4 t = __ldg(src + j * kWarp);
            acc[j] = fmaf(t.z, wc, fmaf(t.x, wa, fmaf(t.y, wb, acc[j])));
          }
        }
        float *rec = w.mrec + ((size_t)s * kRecPerSeg + (dx - lx) * 2 + (dy - ly)) * kRecFloats;
#pragma unroll
        for (int j = 0; j < kChunks; ++j) {
          const int idx = lane + j * kWarp;
          rec[idx] = idx == 0 ? wd * ne : acc[j] * ne;
        }
        if (lane == 0) rec[kRecDl] = wdl * ne;
        ++n_rec;
        __syncwarp();
      }
  }
  if (lane == 0 && n_rec) atomicAdd(&w.counts->n_main_rec, n_rec);
}

__global__ void __launch_bounds__(kMainBlockWarps * kWarp, 3) k_main_adjoint(LsimParams p, Tables tab, Workspace w, Grid g,
                                                                           int64_t n_rows) {
  __shared__ MainSmem sms[kMainBlockWarps];
  const int lane = threadIdx.x % kWarp;
  MainSmem &ms = sms[threadIdx.x / kWarp];
  const int L = p.signal_length;
  constexpr int nbp = kBinsPerPixel;
  float th[LSIM_NPARAM];
#pragma unroll
  for (int i = 0; i < LSIM_NPARAM; ++i) th[i] = 0.f;
  int64_t s0, s1;
  block_range(n_rows, &s0, &s1);
  for (int64_t s = s0; s < s1; s += kMainBlockWarps) {
    const SegFwd &f = w.segf[s];
    const float ne = f.ne;
    const int32_t key = w.key[s];
    if (ne == 0.f || key < 0) continue;
    const SegAdj &a = w.sega[s];
    const float qa = f.qa, qb = f.qb, qc = f.qc;
    float acc_ne = 0.f, acc_sig = 0.f, acc_a = 0.f, acc_b = 0.f, acc_c = 0.f;
    int lx, hx, ly, hy;
    axis_range(f.bx, nbp, &lx, &hx);
    axis_range(f.by, nbp, &ly, &hy);
#pragma unroll 1
    for (int dx = lx; dx <= hx; ++dx)
#pragma unroll 1
      for (int dy = ly; dy <= hy; ++dy) {
        // records of pixels that are not simulated are never read (the
        // reference drops main bins outside unique_pixels, sim_jax.py:152-154)
        if (!slot_is_pixel(g, w.cnt, (int64_t)key + (int64_t)dy * g.nxe + dx)) continue;
        float wd, wdl;
        const int n = main_entries<true>(p, tab, f, &a, dx, dy, ms, &wd, &wdl, lane);
        const float *rec = w.mrec + ((size_t)s * kRecPerSeg + (dx - lx) * 2 + (dy - ly)) * kRecFloats;
        // cotangents of the samples (idx >= 1; the padded rows are zero at
        // idx = 0, where the record holds the boundary term's cotangent)
        float d[kChunks];
#pragma unroll
        for (int j = 0; j < kChunks; ++j) d[j] = rec[lane + j * kWarp];
        const float dcorr = rec[0];
#pragma unroll 1
        for (int e = 0; e < n; ++e) {
          const float4 *src = tab.wmp + (size_t)ms.off[e] * kWinSamples + lane;
          float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
          for (int j = 0; j < kChunks; ++j) {
            const float4 t = __ldg(src + j * kWarp);
            sx = fmaf(d[j], t.x, sx);
            sy = fmaf(d[j], t.y, sy);
            sz = fmaf(d[j], t.z, sz);
          }
          const float W = ms.W[e], dW = ms.dW[e];
          const float sB = (sy * qb + sx * qa) + sz * qc;
          acc_ne = fmaf(W, sB, acc_ne);
          acc_sig = fmaf(dW, sB, acc_sig);
          acc_a = fmaf(W, sx, acc_a);
          acc_b = fmaf(W, sy, acc_b);
          acc_c = fmaf(W, sz, acc_c);
        }
        if (lane < n) {
          acc_ne += dcorr * ms.W[lane] * ms.D[lane];
          acc_sig += dcorr * ms.dW[lane] * ms.D[lane];
        }
        __syncwarp();
      }
    // V and the boundary term carry n_e * W(sigma_T) * (a, b, c)(longdiff)
    const float sig = acc_sig * ne;
    const float lsum = (acc_a * a.dqa + acc_b * a.dqb + acc_c * a.dqc) * ne;
    th[0] += acc_ne * a.dne[0];
    th[1] += acc_ne * a.dne[1];
    th[2] += acc_ne * a.dne[2] + sig * a.dsig[0] + lsum * a.dld[0];
    th[3] += acc_ne * a.dne[3];
    th[5] += lsum * a.dld[1];
    th[6] += sig * a.dsig[1];
    th[7] += acc_ne * a.dne[4];
  }
#pragma unroll
  for (int i = 0; i < LSIM_NPARAM; ++i) th[i] = warp_sum(th[i]);
  if (lane == 0) {
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
    float *dst = w.main_out + gw * kPixRec;
    dst[0] = 0.f;
#pragma unroll
    for (int i = 0; i < LSIM_NPARAM; ++i) dst[1 + i] = th[i];
  }
}

int run_main_records(const AccumArgs &a, cudaStream_t st) {
  if (cudaMemsetAsync(&a.w.counts->n_main_rec, 0, sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (a.n_rows <= 0) return LSIM_OK;
  k_main_records<<<kMainWarps / kMainBlockWarps, kMainBlockWarps * kWarp, 0, st>>>(a.p, a.tab, a.w, a.g, a.n_rows);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

int run_main_adjoint(const AccumArgs &a, cudaStream_t st) {
  // every warp writes its record, also when it owns no segment
  k_main_adjoint<<<kMainWarps / kMainBlockWarps, kMainBlockWarps * kWarp, 0, st>>>(a.p, a.tab, a.w, a.g, a.n_rows);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
