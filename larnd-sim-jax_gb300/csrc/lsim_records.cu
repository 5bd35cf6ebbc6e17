// Hit records of the simulate driver (optimize/simulate.py:129-176): from
// the compacted hits of simulate_stochastic / simulate_parametrized keep the
// rows whose ADC differs from the lowest ADC, digitize(threshold), and whose
// event is not -1; write the kept rows' columns, the cleaned ADC
// (adc - adc_lowest) and the charge in ke- (adc2charge, losses_jax.py:380-383),
// then list the runs of equal event id in the kept rows (start offset and
// event of each run), which is what splitting the output per event needs.
//
// Six launches, all over tiles of 1024 rows: count the kept rows per tile,
// one CTA scanning the tile counts (kept total to counts[0]), a write pass
// that recomputes the keep flag and stores every requested column at its
// compacted position; then the same three steps over the compacted event
// column for the run starts (run total to counts[1], run_start[n_runs] =
// counts[0]).  The run kernels read the kept count from device memory, so
// the whole sequence runs without a host synchronisation.  All arithmetic
// uses _rn intrinsics, so the compiler contracts nothing beyond the one FMA
// written out in adc_to_charge.
#include "lsim_internal.cuh"

namespace lsim {
namespace {

constexpr int kRecTile = 1024;  // rows per block

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

// Number of flagged rows of this block's tile, summed over its warps.
__device__ __forceinline__ int64_t tile_count(bool flag) {
  __shared__ int warp_n[kRecTile / kWarp];
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = __popc(bal);
  __syncthreads();
  int64_t s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kRecTile / kWarp; ++w) s += warp_n[w];
  return s;
}

// Position of a flagged row among the flagged rows of its tile.
__device__ __forceinline__ int64_t tile_rank(bool flag) {
  __shared__ int warp_n[kRecTile / kWarp];
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_n[wid] = __popc(bal);
  __syncthreads();
  int ofs = 0;
  for (int w = 0; w < wid; ++w) ofs += warp_n[w];
  return ofs + __popc(bal & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(kRecTile) k_rec_count(const float *__restrict__ adc,
                                                        const int32_t *__restrict__ event, int64_t n,
                                                        float adc_lowest, int64_t *__restrict__ tile_n) {
  const int64_t i = (int64_t)blockIdx.x * kRecTile + threadIdx.x;
  const bool keep = i < n && rec_keep(adc[i], event[i], adc_lowest);
  const int64_t s = tile_count(keep);
  if (threadIdx.x == 0) tile_n[blockIdx.x] = s;
}

// Exclusive scan of the tile counts in place; *total gets the sum.  When
// run_start is given, run_start[sum] = *sentinel (the kept-row count).
__global__ void __launch_bounds__(kRecTile) k_rec_scan(int64_t *__restrict__ tile_n, int64_t n_tiles,
                                                       int64_t *__restrict__ total, int64_t *__restrict__ run_start,
                                                       const int64_t *__restrict__ sentinel) {
  __shared__ int64_t warp_tot[kRecTile / kWarp];
  __shared__ int64_t chunk_total;
  int64_t carry = 0;
  for (int64_t base = 0; base < n_tiles; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < n_tiles ? tile_n[i] : 0;
    const int64_t inc = block_scan_i64(v, warp_tot, &chunk_total);
    if (i < n_tiles) tile_n[i] = carry + inc - v;
    __syncthreads();
    carry += chunk_total;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *total = carry;
    if (run_start) run_start[carry] = *sentinel;
  }
}

__global__ void __launch_bounds__(kRecTile) k_rec_write(LsimParams p, LsimHitColumns in, int64_t n, float adc_lowest,
                                                        const int64_t *__restrict__ tile_off, LsimHitColumns out,
                                                        float *__restrict__ out_clean, float *__restrict__ out_q) {
  const int64_t i = (int64_t)blockIdx.x * kRecTile + threadIdx.x;
  float a = 0.f;
  int32_t ev = -1;
  if (i < n) {
    a = in.adc[i];
    ev = in.event[i];
  }
  const bool keep = i < n && rec_keep(a, ev, adc_lowest);
  const int64_t r = tile_rank(keep);
  if (!keep) return;
  const int64_t o = tile_off[blockIdx.x] + r;
  out.event[o] = ev;
  if (out.adc) out.adc[o] = a;
  if (out_clean) out_clean[o] = __fsub_rn(a, adc_lowest);
  if (out_q) out_q[o] = adc_to_charge(p, a);
  if (out.pixel_x) out.pixel_x[o] = in.pixel_x[i];
  if (out.pixel_y) out.pixel_y[o] = in.pixel_y[i];
  if (out.pixel_z) out.pixel_z[o] = in.pixel_z[i];
  if (out.ticks) out.ticks[o] = in.ticks[i];
  if (out.hit_prob) out.hit_prob[o] = in.hit_prob[i];
  if (out.pixels) out.pixels[o] = in.pixels[i];
}

// Run starts of the compacted event column: row o starts a run when it is
// the first kept row or its event differs from the row before it.
__device__ __forceinline__ bool run_head(const int32_t *__restrict__ ev, int64_t o, int64_t n_kept) {
  return o < n_kept && (o == 0 || ev[o] != ev[o - 1]);
}

__global__ void __launch_bounds__(kRecTile) k_run_count(const int32_t *__restrict__ ev,
                                                        const int64_t *__restrict__ counts,
                                                        int64_t *__restrict__ tile_n) {
  const int64_t n_kept = counts[0];
  const int64_t o = (int64_t)blockIdx.x * kRecTile + threadIdx.x;
  const int64_t s = tile_count(run_head(ev, o, n_kept));
  if (threadIdx.x == 0) tile_n[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRecTile) k_run_write(const int32_t *__restrict__ ev,
                                                        const int64_t *__restrict__ counts,
                                                        const int64_t *__restrict__ tile_off,
                                                        int32_t *__restrict__ run_event,
                                                        int64_t *__restrict__ run_start) {
  const int64_t n_kept = counts[0];
  const int64_t o = (int64_t)blockIdx.x * kRecTile + threadIdx.x;
  const bool head = run_head(ev, o, n_kept);
  const int64_t r = tile_rank(head);
  if (!head) return;
  const int64_t k = tile_off[blockIdx.x] + r;
  if (run_event) run_event[k] = ev[o];
  run_start[k] = o;
}

}  // namespace

size_t records_workspace_bytes(int64_t n) {
  const int64_t tiles = (n + kRecTile - 1) / kRecTile;
  return 2 * align256((size_t)(tiles + 1) * sizeof(int64_t));
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
  int64_t *tile_rows = (int64_t *)ws;
  int64_t *tile_runs = (int64_t *)((char *)ws + align256((size_t)(tiles + 1) * sizeof(int64_t)));
  k_rec_count<<<(unsigned)tiles, kRecTile, 0, st>>>(in.adc, in.event, n, adc_lowest, tile_rows);
  k_rec_scan<<<1, kRecTile, 0, st>>>(tile_rows, tiles, counts, nullptr, nullptr);
  k_rec_write<<<(unsigned)tiles, kRecTile, 0, st>>>(p, in, n, adc_lowest, tile_rows, out, out_clean, out_q);
  if (run_start) {
    k_run_count<<<(unsigned)tiles, kRecTile, 0, st>>>(out.event, counts, tile_runs);
    k_rec_scan<<<1, kRecTile, 0, st>>>(tile_runs, tiles, counts + 1, run_start, counts);
    k_run_write<<<(unsigned)tiles, kRecTile, 0, st>>>(out.event, counts, tile_runs, run_event, run_start);
  } else if (cudaMemsetAsync(counts + 1, 0, sizeof(int64_t), st) != cudaSuccess) {
    return LSIM_ERR_CUDA;
  }
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
