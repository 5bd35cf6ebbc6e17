// Hit records of the simulate driver (optimize/simulate.py:129-176): from
// the compacted hits of simulate_stochastic / simulate_parametrized keep the
// rows whose ADC differs from the lowest ADC, digitize(threshold), and whose
// event is not -1; write the kept rows' columns, the cleaned ADC
// (adc - adc_lowest) and the charge in ke- (adc2charge, losses_jax.py:380-383),
// and list the runs of equal event id in the kept rows (start offset and
// event of each run), which is what splitting the output per event needs.
//
// Three launches over tiles of 4096 hits (a block of 256 threads walks four
// chunks of 1024 hits, 4 sub-tiles each, carrying the tile's state):
//   k_rec_tiles  reads adc and event and summarises each tile: kept rows,
//                run heads whose previous kept row is in the tile, first
//                and last kept event;
//   k_rec_scan   one CTA: exclusive row and run offsets per tile and the
//                last kept event before it (kept and run totals to counts,
//                run_start[n_runs] = n_kept);
//   k_rec_write  loads all requested columns of its tile up front, ranks the
//                kept rows and the run heads (ballots, one warp combining the
//                32 warp-parts of the tile) and stores both.
// A run head is a kept row whose previous kept row has another event (or
// the first kept row).  Traffic: 8 B per hit in the summary pass, the input
// columns once and the kept rows' outputs once in the write pass.  The
// rounding: every operation is a _rn intrinsic, so the compiler contracts
// nothing beyond the one FMA written out in adc_to_charge.
#include "lsim_internal.cuh"

namespace lsim {
namespace {

constexpr int kRecThreads = 256;                   // threads per block
constexpr int kRecSub = 4;                         // sub-tiles of kRecThreads rows per chunk
constexpr int kRecChunk = kRecThreads * kRecSub;   // 1024 rows per chunk
constexpr int kRecChunks = 4;                      // chunks per tile, in order, with a carry
constexpr int kRecTile = kRecChunk * kRecChunks;   // 4096 rows per tile
constexpr int kRecWarps = kRecThreads / kWarp;     // 8
constexpr int kRecParts = kRecSub * kRecWarps;     // 32 warp-parts of 32 rows, one lane of a warp each
constexpr int kRecScanThreads = 1024;
constexpr unsigned kFull = 0xffffffffu;
static_assert(kRecParts == kWarp, "one combining lane per warp-part");

struct TileSum {
  int32_t kept;      // kept rows
  int32_t heads;     // run heads whose previous kept row lies in the tile
  int32_t first_ev;  // event of the first / last kept row (kept > 0)
  int32_t last_ev;
};

struct TileOff {
  int64_t row;       // kept rows before the tile
  int64_t run;       // runs starting before the tile
  int32_t prev_ev;   // event of the last kept row before the tile (has_prev)
  int32_t has_prev;
};

struct Part {
  int kept, heads, first_ev, last_ev;
};

__device__ __forceinline__ bool rec_keep(float adc, int32_t event, float adc_lowest) {
  return __fsub_rn(adc, adc_lowest) != 0.f && event != -1;
}

// adc2charge, (((dw / ADC_COUNTS) * (V_REF - V_CM)) + V_CM - V_PEDESTAL) / GAIN
// * 1e-3, in the form XLA compiled it to for the reference's committed
// outputs (output/jax_ref/output_{lut,parametrized}_1.npz, whose charges it
// reproduces bit for bit): constants folded, one fused multiply-add,
//   q = fma(dw * (1 / ADC_COUNTS), V_REF - V_CM, V_CM - V_PEDESTAL) * (1e-3 / GAIN).
// With the module0 constants 1/256 and 1e-3/0.004 = 0.25 are exact.
__device__ __forceinline__ float adc_to_charge(const LsimParams &p, float dw) {
  const float inv_counts = __frcp_rn(p.adc_counts);
  const float offset = __fsub_rn(p.v_cm, p.v_pedestal);
  const float scale = __fdiv_rn(1e-3f, p.gain);
  return __fmul_rn(__fmaf_rn(__fmul_rn(dw, inv_counts), p.vref_minus_cm, offset), scale);
}

__device__ __forceinline__ unsigned lanes_below() { return (1u << (threadIdx.x & 31)) - 1u; }

// One warp's 32 rows: the ballot of kept rows, for each lane whether a kept
// row precedes it in the warp and that row's event, and the part summary.
__device__ __forceinline__ Part warp_part(bool keep, int ev, unsigned &bal, bool &has_prev, int &prev_ev) {
  bal = __ballot_sync(kFull, keep);
  const unsigned before = bal & lanes_below();
  prev_ev = __shfl_sync(kFull, ev, before ? 31 - __clz(before) : 0);
  has_prev = before != 0;
  const unsigned heads = __ballot_sync(kFull, keep && has_prev && ev != prev_ev);
  Part q;
  q.kept = __popc(bal);
  q.heads = __popc(heads);
  q.first_ev = __shfl_sync(kFull, ev, bal ? __ffs(bal) - 1 : 0);
  q.last_ev = __shfl_sync(kFull, ev, bal ? 31 - __clz(bal) : 0);
  return q;
}

__device__ __forceinline__ int warp_incl_sum(int v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, v, o);
    if ((int)(threadIdx.x & 31) >= o) v += y;
  }
  return v;
}

// Lane p of one warp holds part p of the tile (parts in row order).  Gives
// the last kept event of the parts before p within the tile.
__device__ __forceinline__ bool prior_part(const Part &q, int &prior_last) {
  const unsigned kb = __ballot_sync(kFull, q.kept > 0);
  const unsigned before = kb & lanes_below();
  prior_last = __shfl_sync(kFull, q.last_ev, before ? 31 - __clz(before) : 0);
  return before != 0;
}

__global__ void __launch_bounds__(kRecThreads) k_rec_tiles(const float *__restrict__ adc,
                                                           const int32_t *__restrict__ event, int64_t n,
                                                           float adc_lowest, TileSum *__restrict__ sums) {
  __shared__ Part parts[kRecParts];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // carried by warp 0 from chunk to chunk: the tile's summary so far
  int kept = 0, heads = 0, first = 0, last = 0;
  bool any = false;
#pragma unroll 1
  for (int c = 0; c < kRecChunks; ++c) {
    const int64_t base = (int64_t)blockIdx.x * kRecTile + (int64_t)c * kRecChunk + threadIdx.x;
    float a[kRecSub];
    int e[kRecSub];
#pragma unroll
    for (int s = 0; s < kRecSub; ++s) {
      const int64_t i = base + s * kRecThreads;
      a[s] = i < n ? adc[i] : adc_lowest;
      e[s] = i < n ? event[i] : -1;
    }
#pragma unroll
    for (int s = 0; s < kRecSub; ++s) {
      unsigned bal;
      bool hp;
      int pe;
      const Part q = warp_part(rec_keep(a[s], e[s], adc_lowest), e[s], bal, hp, pe);
      if (lane == 0) parts[s * kRecWarps + wid] = q;
    }
    __syncthreads();
    if (wid == 0) {
      const Part q = parts[lane];
      int prior_last;
      const bool has_prior = prior_part(q, prior_last);
      // the previous kept row: in this chunk, else the tile's last so far
      const bool pp_has = has_prior || any;
      const int pp_ev = has_prior ? prior_last : last;
      const int boundary = q.kept > 0 && pp_has && q.first_ev != pp_ev;
      kept += __reduce_add_sync(kFull, (unsigned)q.kept);
      heads += __reduce_add_sync(kFull, (unsigned)(q.heads + boundary));
      const unsigned kb = __ballot_sync(kFull, q.kept > 0);
      if (kb) {
        const int cf = __shfl_sync(kFull, q.first_ev, __ffs(kb) - 1);
        if (!any) first = cf;
        last = __shfl_sync(kFull, q.last_ev, 31 - __clz(kb));
        any = true;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = TileSum{kept, heads, first, last};
}

// Inclusive warp scans (max, sum) of one int64 per lane.
__device__ __forceinline__ int64_t warp_incl_max(int64_t v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(kFull, v, o);
    if ((int)(threadIdx.x & 31) >= o && y > v) v = y;
  }
  return v;
}

__device__ __forceinline__ int64_t warp_incl_sum64(int64_t v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(kFull, v, o);
    if ((int)(threadIdx.x & 31) >= o) v += y;
  }
  return v;
}

// The last kept event before each tile is found by a max-scan of
// (tile index << 32 | event) over the tiles with kept rows.
__device__ __forceinline__ int64_t pack_last(int64_t tile, int32_t ev) {
  return (int64_t)((uint64_t)tile << 32 | (uint32_t)ev);
}

// One CTA over all tiles, 1024 tiles per round: a max-scan for the last
// kept event before each tile, then sum-scans of its kept rows and runs.
// Every scan is warp shuffles plus one warp scanning the 32 warp totals;
// four barriers per round, the next round's summaries loaded ahead.
__global__ void __launch_bounds__(kRecScanThreads) k_rec_scan(const TileSum *__restrict__ sums, int64_t n_tiles,
                                                              TileOff *__restrict__ offs,
                                                              int64_t *__restrict__ counts,
                                                              int64_t *__restrict__ run_start) {
  constexpr int kW = kRecScanThreads / 32;
  static_assert(kW == 32, "one lane of warp 0 per warp");
  __shared__ int64_t w_last[kW], w_rows[kW], w_runs[kW];
  __shared__ int64_t carry_sh[3];  // rows, runs and last key before the round
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t kNone = INT64_MIN;
  if (threadIdx.x == 0) {
    carry_sh[0] = 0;
    carry_sh[1] = 0;
    carry_sh[2] = kNone;
  }
  TileSum next = threadIdx.x < n_tiles ? sums[threadIdx.x] : TileSum{0, 0, 0, 0};
  __syncthreads();
  for (int64_t base = 0; base < n_tiles; base += kRecScanThreads) {
    const int64_t t = base + threadIdx.x;
    const TileSum ts = next;
    const int64_t tn = t + kRecScanThreads;
    next = tn < n_tiles ? sums[tn] : TileSum{0, 0, 0, 0};
    const int64_t c_rows = carry_sh[0], c_runs = carry_sh[1], c_last = carry_sh[2];
    // last kept event before the tile
    const int64_t key = ts.kept > 0 ? pack_last(t, ts.last_ev) : kNone;
    const int64_t wl = warp_incl_max(key);
    if (lane == 31) w_last[wid] = wl;
    __syncthreads();
    if (wid == 0) {
      const int64_t v = warp_incl_max(w_last[lane]);
      const int64_t before = __shfl_up_sync(kFull, v, 1);
      const int64_t ex = lane == 0 ? c_last : (before > c_last ? before : c_last);
      w_last[lane] = ex;  // max over the warps before this one and the earlier rounds
    }
    __syncthreads();
    const int64_t wprev = w_last[wid];
    const int64_t lprev = __shfl_up_sync(kFull, wl, 1);
    const int64_t prev = lane == 0 ? wprev : (lprev > wprev ? lprev : wprev);
    const bool has_prev = prev != kNone;
    const int32_t prev_ev = has_prev ? (int32_t)(uint32_t)(uint64_t)prev : 0;
    const int64_t runs = ts.kept > 0 ? ts.heads + ((!has_prev || ts.first_ev != prev_ev) ? 1 : 0) : 0;
    // row and run offsets
    const int64_t ir = warp_incl_sum64(ts.kept);
    const int64_t iu = warp_incl_sum64(runs);
    if (lane == 31) {
      w_rows[wid] = ir;
      w_runs[wid] = iu;
    }
    __syncthreads();
    if (wid == 0) {
      const int64_t vr = warp_incl_sum64(w_rows[lane]);
      const int64_t vu = warp_incl_sum64(w_runs[lane]);
      const int64_t tr = __shfl_sync(kFull, vr, 31), tu = __shfl_sync(kFull, vu, 31);
      w_rows[lane] = c_rows + vr - w_rows[lane];
      w_runs[lane] = c_runs + vu - w_runs[lane];
      if (lane == 0) {
        carry_sh[0] = c_rows + tr;
        carry_sh[1] = c_runs + tu;
      }
    }
    __syncthreads();
    if (t < n_tiles) offs[t] = TileOff{w_rows[wid] + ir - ts.kept, w_runs[wid] + iu - runs, prev_ev, has_prev ? 1 : 0};
    // the round's last key: the last thread's inclusive max
    if (threadIdx.x == kRecScanThreads - 1) {
      const int64_t incl = wl > wprev ? wl : wprev;
      carry_sh[2] = incl > c_last ? incl : c_last;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    counts[0] = carry_sh[0];
    counts[1] = carry_sh[1];
    if (run_start) run_start[carry_sh[1]] = carry_sh[0];
  }
}

__global__ void __launch_bounds__(kRecThreads, 4) k_rec_write(LsimParams p, LsimHitColumns in, int64_t n,
                                                           float adc_lowest, const TileOff *__restrict__ offs,
                                                           LsimHitColumns out, float *__restrict__ out_clean,
                                                           float *__restrict__ out_q, int32_t *__restrict__ run_event,
                                                           int64_t *__restrict__ run_start) {
  __shared__ Part parts[kRecParts];
  __shared__ int part_row[kRecParts], part_run[kRecParts], part_prev_ev[kRecParts];
  __shared__ bool part_prev_has[kRecParts];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const TileOff to = offs[blockIdx.x];
  // carried by warp 0 from chunk to chunk: rows and runs of the tile so far
  // and the last kept event before the next chunk
  int c_row = 0, c_run = 0, c_ev = to.prev_ev;
  bool c_has = to.has_prev != 0;
#pragma unroll 1
  for (int c = 0; c < kRecChunks; ++c) {
    const int64_t base = (int64_t)blockIdx.x * kRecTile + (int64_t)c * kRecChunk + threadIdx.x;
    float a[kRecSub], x[kRecSub], y[kRecSub], z[kRecSub], tk[kRecSub], hp[kRecSub];
    int ev[kRecSub], px[kRecSub];
#pragma unroll
    for (int s = 0; s < kRecSub; ++s) {
      const int64_t i = base + s * kRecThreads;
      const bool in_range = i < n;
      a[s] = in_range ? in.adc[i] : adc_lowest;
      ev[s] = in_range ? in.event[i] : -1;
      x[s] = in_range && out.pixel_x ? in.pixel_x[i] : 0.f;
      y[s] = in_range && out.pixel_y ? in.pixel_y[i] : 0.f;
      z[s] = in_range && out.pixel_z ? in.pixel_z[i] : 0.f;
      tk[s] = in_range && out.ticks ? in.ticks[i] : 0.f;
      hp[s] = in_range && out.hit_prob ? in.hit_prob[i] : 0.f;
      px[s] = in_range && out.pixels ? in.pixels[i] : 0;
    }
    unsigned bal[kRecSub];
    bool has_prev[kRecSub];
    int prev_ev[kRecSub];
#pragma unroll
    for (int s = 0; s < kRecSub; ++s) {
      const Part q = warp_part(rec_keep(a[s], ev[s], adc_lowest), ev[s], bal[s], has_prev[s], prev_ev[s]);
      if (lane == 0) parts[s * kRecWarps + wid] = q;
    }
    __syncthreads();
    if (wid == 0) {
      const Part q = parts[lane];
      int prior_last;
      const bool has_prior = prior_part(q, prior_last);
      const bool pp_has = has_prior || c_has;
      const int pp_ev = has_prior ? prior_last : c_ev;
      const int heads = q.heads + (q.kept > 0 && (!pp_has || q.first_ev != pp_ev) ? 1 : 0);
      const int ir = warp_incl_sum(q.kept), iu = warp_incl_sum(heads);
      part_row[lane] = c_row + ir - q.kept;
      part_run[lane] = c_run + iu - heads;
      part_prev_has[lane] = pp_has;
      part_prev_ev[lane] = pp_ev;
      c_row += __shfl_sync(kFull, ir, 31);
      c_run += __shfl_sync(kFull, iu, 31);
      const unsigned kb = __ballot_sync(kFull, q.kept > 0);
      if (kb) {
        c_ev = __shfl_sync(kFull, q.last_ev, 31 - __clz(kb));
        c_has = true;
      }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < kRecSub; ++s) {
      const int pi = s * kRecWarps + wid;
      const bool keep = (bal[s] >> lane) & 1u;
      const bool head = keep && (has_prev[s] ? ev[s] != prev_ev[s]
                                             : (part_prev_has[pi] ? ev[s] != part_prev_ev[pi] : true));
      const unsigned hb = __ballot_sync(kFull, head);
      if (!keep) continue;
      const int64_t o = to.row + part_row[pi] + __popc(bal[s] & lanes_below());
      out.event[o] = ev[s];
      if (out.adc) out.adc[o] = a[s];
      if (out_clean) out_clean[o] = __fsub_rn(a[s], adc_lowest);
      if (out_q) out_q[o] = adc_to_charge(p, a[s]);
      if (out.pixel_x) out.pixel_x[o] = x[s];
      if (out.pixel_y) out.pixel_y[o] = y[s];
      if (out.pixel_z) out.pixel_z[o] = z[s];
      if (out.ticks) out.ticks[o] = tk[s];
      if (out.hit_prob) out.hit_prob[o] = hp[s];
      if (out.pixels) out.pixels[o] = px[s];
      if (head && run_start) {
        const int64_t k = to.run + part_run[pi] + __popc(hb & lanes_below());
        run_start[k] = o;
        if (run_event) run_event[k] = ev[s];
      }
    }
  }
}

}  // namespace

size_t records_workspace_bytes(int64_t n) {
  const int64_t tiles = (n + kRecTile - 1) / kRecTile;
  return align256((size_t)tiles * sizeof(TileSum)) + align256((size_t)tiles * sizeof(TileOff));
}

int run_records(const LsimParams &p, float adc_lowest, const LsimHitColumns &in, int64_t n, const LsimHitColumns &out,
                float *out_clean, float *out_q, int32_t *run_event, int64_t *run_start, int64_t *counts, void *ws,
                cudaStream_t st) {
  if (n == 0) {
    if (cudaMemsetAsync(counts, 0, 2 * sizeof(int64_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
    if (run_start && cudaMemsetAsync(run_start, 0, sizeof(int64_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
    return LSIM_OK;
  }
  const int64_t tiles = (n + kRecTile - 1) / kRecTile;
  TileSum *sums = (TileSum *)ws;
  TileOff *offs = (TileOff *)((char *)ws + align256((size_t)tiles * sizeof(TileSum)));
  k_rec_tiles<<<(unsigned)tiles, kRecThreads, 0, st>>>(in.adc, in.event, n, adc_lowest, sums);
  k_rec_scan<<<1, kRecScanThreads, 0, st>>>(sums, tiles, offs, counts, run_start);
  k_rec_write<<<(unsigned)tiles, kRecThreads, 0, st>>>(p, in, n, adc_lowest, offs, out, out_clean, out_q, run_event,
                                                       run_start);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
