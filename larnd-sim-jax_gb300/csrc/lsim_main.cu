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
// sigma_T and (a, b, c) and writes dL/dtheta per segment (reduced later in
// segment order, so the result does not depend on the processing order).
// Both kernels take the segments grouped by template index: one warp owns
// one segment at a time, the warps of a block interleave a contiguous range
// of that order, so a block's segments share their 25 LUT window rows in L1.
#include "lsim_internal.cuh"
#include "lsim_bins.cuh"
#include "lsim_fee.cuh"

namespace lsim {


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

// Positions [i0, i1) of the template-ordered segment list owned by this
// block, interleaved over its warps (warp w takes i0 + w, i0 + w + 8, ...).
__device__ __forceinline__ void block_range(int64_t n, int64_t *i0, int64_t *i1) {
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  *i0 = (int64_t)blockIdx.x * chunk + threadIdx.x / kWarp;
  *i1 = min(n, (int64_t)blockIdx.x * chunk + chunk);
}

// Launch shape of the main-bin kernels: tuned or the default 1024 x 8 warps.
static void main_shape(int *blocks, int *warps) {
  const LsimTuning tu = tuning();
  *warps = tu.main_block_warps == 4 ? 4 : 8;
  *blocks = tu.main_blocks > 0 ? min(tu.main_blocks, kMainWarps / *warps) : 1024;
}

// ---------------------------------------------------------------- order

// Segments with main-bin records (n_e != 0 and a grid slot), grouped by
// template index with a counting sort (the order inside a group is
// arbitrary).  Warp-aggregated atomics: one per distinct index per warp.
__device__ __forceinline__ bool main_active(const Workspace &w, int64_t s, int64_t n_rows, int *bin) {
  if (s >= n_rows) return false;
  const SegFwd &f = w.segf[s];
  *bin = f.tidx;
  return f.ne != 0.f && w.key[s] >= 0;
}

__global__ void k_main_order_count(Workspace w, int64_t n_rows) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int bin = 0;
  const bool act = main_active(w, s, n_rows, &bin);
  const unsigned am = __ballot_sync(0xffffffffu, act);
  if (act) {
    const unsigned peers = __match_any_sync(am, bin);
    if ((threadIdx.x % kWarp) == __ffs(peers) - 1) atomicAdd(&w.tidx_hist[bin], __popc(peers));
  }
}

__global__ void k_main_order_scan(Workspace w) {
  __shared__ int sh[kMaxTemplates];
  const int t = threadIdx.x;
  const int c = w.tidx_hist[t];
  sh[t] = c;
  __syncthreads();
  for (int o = 1; o < kMaxTemplates; o <<= 1) {
    const int v = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  w.tidx_hist[kMaxTemplates + t] = sh[t] - c;
  if (t == kMaxTemplates - 1) w.counts->n_main_seg = sh[t];
}

__global__ void k_main_order_scatter(Workspace w, int64_t n_rows) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x % kWarp;
  int bin = 0;
  const bool act = main_active(w, s, n_rows, &bin);
  const unsigned am = __ballot_sync(0xffffffffu, act);
  if (act) {
    const unsigned peers = __match_any_sync(am, bin);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&w.tidx_hist[kMaxTemplates + bin], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    w.seg_order[base + __popc(peers & ((1u << lane) - 1u))] = (int32_t)s;
  }
}

// ---------------------------------------------------------------- kernels

// L1 prefetch of the next segment's records (segments come in template
// order, so their records are scattered; the next one's lines are fetched
// while this one is processed).
__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

template <int kMainBlockWarps>
__global__ void __launch_bounds__(kMainBlockWarps * kWarp, 16 / kMainBlockWarps) k_main_records(LsimParams p, Tables tab, Workspace w, Grid g,
                                                                           int64_t n_rows) {
  __shared__ MainSmem sms[kMainBlockWarps];
  const int lane = threadIdx.x % kWarp;
  MainSmem &ms = sms[threadIdx.x / kWarp];
  constexpr int nbp = kBinsPerPixel;
  int n_rec = 0;
  int64_t i0, i1;
  block_range(w.counts->n_main_seg, &i0, &i1);
  for (int64_t i = i0; i < i1; i += kMainBlockWarps) {
    const int64_t s = w.seg_order[i];
    if (lane < 2 && i + kMainBlockWarps < i1)
      prefetch_l1(reinterpret_cast<const char *>(w.segf + w.seg_order[i + kMainBlockWarps]) + 64 * lane);
    const SegFwd &f = w.segf[s];
    const float ne = f.ne;
    const int32_t key = w.key[s];
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

template <int kMainBlockWarps>
__global__ void __launch_bounds__(kMainBlockWarps * kWarp, 24 / kMainBlockWarps) k_main_adjoint(LsimParams p, Tables tab, Workspace w, Grid g,
                                                                           int64_t n_rows) {
  __shared__ MainSmem sms[kMainBlockWarps];
  const int lane = threadIdx.x % kWarp;
  MainSmem &ms = sms[threadIdx.x / kWarp];
  const int L = p.signal_length;
  constexpr int nbp = kBinsPerPixel;
  int64_t i0, i1;
  block_range(w.counts->n_main_seg, &i0, &i1);
  for (int64_t i = i0; i < i1; i += kMainBlockWarps) {
    const int64_t s = w.seg_order[i];
    if (i + kMainBlockWarps < i1) {
      const int64_t sn = w.seg_order[i + kMainBlockWarps];
      if (lane < 2) prefetch_l1(reinterpret_cast<const char *>(w.segf + sn) + 64 * lane);
      else if (lane < 4) prefetch_l1(reinterpret_cast<const char *>(w.sega + sn) + 64 * (lane - 2));
      else if (lane < 4 + 21) prefetch_l1(w.mrec + (size_t)sn * kRecPerSeg * kRecFloats + 32 * (lane - 4));
    }
    const SegFwd &f = w.segf[s];
    const float ne = f.ne;
    const int32_t key = w.key[s];
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
          float2 sxy = make_float2(0.f, 0.f);
          float sz = 0.f;
#pragma unroll
          for (int j = 0; j < kChunks; ++j) {
            const float4 t = __ldg(src + j * kWarp);
            sxy = __ffma2_rn(make_float2(d[j], d[j]), make_float2(t.x, t.y), sxy);
            sz = fmaf(d[j], t.z, sz);
          }
          const float sx = sxy.x, sy = sxy.y;
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
    float th[LSIM_NPARAM];
    th[0] = acc_ne * a.dne[0];
    th[1] = acc_ne * a.dne[1];
    th[2] = acc_ne * a.dne[2] + sig * a.dsig[0] + lsum * a.dld[0];
    th[3] = acc_ne * a.dne[3];
    th[4] = 0.f;
    th[5] = lsum * a.dld[1];
    th[6] = sig * a.dsig[1];
    th[7] = acc_ne * a.dne[4];
#pragma unroll
    for (int q = 0; q < LSIM_NPARAM; ++q)
      if (q != 4) th[q] = warp_sum(th[q]);
    if (lane == 0) {
      float *dst = w.main_out + s * kPixRec;
#pragma unroll
      for (int q = 0; q < LSIM_NPARAM; ++q) dst[1 + q] = th[q];
    }
  }
}

int run_main_records(const AccumArgs &a, cudaStream_t st) {
  if (cudaMemsetAsync(&a.w.counts->n_main_rec, 0, 2 * sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (a.n_rows <= 0) return LSIM_OK;
  if (a.p.n_templates > kMaxTemplates) return LSIM_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(a.w.tidx_hist, 0, sizeof(int32_t) * kMaxTemplates, st) != cudaSuccess) return LSIM_ERR_CUDA;
  const unsigned nb = (unsigned)((a.n_rows + 255) / 256);
  k_main_order_count<<<nb, 256, 0, st>>>(a.w, a.n_rows);
  k_main_order_scan<<<1, kMaxTemplates, 0, st>>>(a.w);
  k_main_order_scatter<<<nb, 256, 0, st>>>(a.w, a.n_rows);
  int blocks, warps;
  main_shape(&blocks, &warps);
  if (warps == 4)
    k_main_records<4><<<blocks, 4 * kWarp, 0, st>>>(a.p, a.tab, a.w, a.g, a.n_rows);
  else
    k_main_records<8><<<blocks, 8 * kWarp, 0, st>>>(a.p, a.tab, a.w, a.g, a.n_rows);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

int run_main_adjoint(const AccumArgs &a, cudaStream_t st) {
  // per-segment records; segments without main-bin records contribute zeros
  if (cudaMemsetAsync(a.w.main_out, 0, sizeof(float) * kPixRec * (size_t)a.n_rows, st) != cudaSuccess)
    return LSIM_ERR_CUDA;
  if (a.n_rows <= 0) return LSIM_OK;
  int blocks, warps;
  main_shape(&blocks, &warps);
  if (warps == 4)
    k_main_adjoint<4><<<blocks, 4 * kWarp, 0, st>>>(a.p, a.tab, a.w, a.g, a.n_rows);
  else
    k_main_adjoint<8><<<blocks, 8 * kWarp, 0, st>>>(a.p, a.tab, a.w, a.g, a.n_rows);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
