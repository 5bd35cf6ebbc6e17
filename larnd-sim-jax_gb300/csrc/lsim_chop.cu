// Track chopping on the device: every input track becomes
// max(ceil(length / precision), 1) steps of length `precision`, the last step
// taking the remainder (optimize/dataio.py:63-106, chop_tracks).
//
// Four launches: per-track step counts with per-block sums, one CTA scanning
// the block sums (total to the caller's counter), per-track output offsets,
// then a persistent fill kernel that assembles 128 output rows per tile in
// shared memory and writes them with coalesced stores.  The arithmetic is the
// reference's under NumPy 2 promotion: length, direction, step count and the
// per-step dE in float32; step positions and the last step's dE and dx in
// float64, rounded once to float32; midpoints in float32.  The explicit
// _rn intrinsics keep the compiler from contracting any of it into FMAs.
#include "lsim_internal.cuh"

namespace lsim {
namespace {

constexpr int kChopThreads = 256;   // tracks per block in the count/offset kernels
constexpr int kFillRows = 128;      // output rows per tile of the fill kernel
constexpr int kMaxChopFields = 96;  // columns: kFillRows * 96 * 4 B = 48 KiB of shared memory

struct TrackGeom {
  float s[3], e[3], d[3];
  float len, lpe;  // length and length + 1e-10 (float32, dataio.py:98-100)
};

__device__ __forceinline__ TrackGeom track_geom(const float *row, const LsimFieldMap &f) {
  TrackGeom g;
  g.s[0] = row[f.x_start];
  g.s[1] = row[f.y_start];
  g.s[2] = row[f.z_start];
  g.e[0] = row[f.x_end];
  g.e[1] = row[f.y_end];
  g.e[2] = row[f.z_end];
  float seg[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) seg[a] = __fsub_rn(g.e[a], g.s[a]);
  // np.sum over the 3 squared components: left to right in float32
  float l2 = __fadd_rn(__fadd_rn(__fmul_rn(seg[0], seg[0]), __fmul_rn(seg[1], seg[1])), __fmul_rn(seg[2], seg[2]));
  g.len = __fsqrt_rn(l2);
  g.lpe = __fadd_rn(g.len, (float)1e-10);
#pragma unroll
  for (int a = 0; a < 3; ++a) g.d[a] = __fdiv_rn(seg[a], g.lpe);
  return g;
}

// max(ceil(length / precision), 1) as an integer; -1 when the quotient is
// not finite or does not fit (the reference's int cast then fails).
__device__ __forceinline__ int64_t step_count(float len, float prec32) {
  float q = ceilf(__fdiv_rn(len, prec32));
  if (!(q <= 9.0e18f)) return -1;
  return q < 1.0f ? 1 : (int64_t)q;
}

__device__ __forceinline__ int64_t block_sum_i64(int64_t v, int64_t *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  int64_t t = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
  return t;
}

__global__ void __launch_bounds__(kChopThreads) k_chop_count(const float *__restrict__ tracks, int64_t n_rows,
                                                             LsimFieldMap f, float prec32,
                                                             int64_t *__restrict__ row_n,
                                                             int64_t *__restrict__ blk_sum, int32_t *bad) {
  __shared__ int64_t red[kChopThreads / 32];
  const int64_t r = (int64_t)blockIdx.x * kChopThreads + threadIdx.x;
  int64_t n = 0;
  if (r < n_rows) {
    TrackGeom g = track_geom(tracks + r * f.n_fields, f);
    n = step_count(g.len, prec32);
    if (n < 0) {
      *bad = 1;
      n = 0;
    }
    row_n[r] = n;
  }
  int64_t t = block_sum_i64(n, red);
  if (threadIdx.x == 0) blk_sum[blockIdx.x] = t;
}

// One CTA: exclusive scan of the block sums in place; the total (or -1 on
// a bad track) to *n_out.
__global__ void __launch_bounds__(1024) k_chop_scan_blocks(int64_t *blk, int64_t nblk, const int32_t *bad,
                                                           int64_t *n_out) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t chunk_total;
  int64_t carry = 0;
  for (int64_t base = 0; base < nblk; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < nblk ? blk[i] : 0;
    const int64_t inc = block_scan_i64(v, warp_tot, &chunk_total);
    if (i < nblk) blk[i] = carry + inc - v;
    __syncthreads();
    carry += chunk_total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *n_out = *bad ? -1 : carry;
}

__global__ void __launch_bounds__(kChopThreads) k_chop_offsets(const int64_t *__restrict__ row_n, int64_t n_rows,
                                                               const int64_t *__restrict__ blk_off,
                                                               int64_t *__restrict__ row_off) {
  __shared__ int64_t warp_tot[kChopThreads / 32];
  __shared__ int64_t total;
  const int64_t r = (int64_t)blockIdx.x * kChopThreads + threadIdx.x;
  const int64_t v = r < n_rows ? row_n[r] : 0;
  const int64_t inc = block_scan_i64(v, warp_tot, &total);
  if (r < n_rows) row_off[r] = blk_off[blockIdx.x] + inc - v;
}

// The track whose output rows contain row `o`: the last r with row_off[r] <= o
// (offsets are strictly increasing: every track has at least one step).
__device__ __forceinline__ int64_t source_track(const int64_t *__restrict__ row_off, int64_t n_rows, int64_t o) {
  int64_t lo = 0, hi = n_rows - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (__ldg(row_off + mid) <= o)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kFillRows) k_chop_fill(const float *__restrict__ tracks, int64_t n_rows,
                                                         LsimFieldMap f, double prec, float prec32,
                                                         const int64_t *__restrict__ row_n,
                                                         const int64_t *__restrict__ row_off,
                                                         const int64_t *__restrict__ n_out, float *__restrict__ out,
                                                         int64_t capacity) {
  extern __shared__ float tile[];
  const int64_t total = *n_out;
  if (total <= 0) return;
  const int64_t lim = total < capacity ? total : capacity;
  const int F = f.n_fields;
  for (int64_t t0 = (int64_t)blockIdx.x * kFillRows; t0 < lim; t0 += (int64_t)gridDim.x * kFillRows) {
    const int64_t o = t0 + threadIdx.x;
    if (o < lim) {
      const int64_t src = source_track(row_off, n_rows, o);
      const float *row = tracks + src * F;
      float *dst = tile + threadIdx.x * F;
      for (int c = 0; c < F; ++c) dst[c] = row[c];
      const TrackGeom g = track_geom(row, f);
      const int64_t k = o - row_off[src];
      const int64_t n = row_n[src];
      const bool last = k == n - 1;
      const float dE = row[f.dE];
      dst[f.dE] = __fdiv_rn(__fmul_rn(dE, prec32), g.lpe);   // dataio.py:67
      const int cs[3] = {f.x_start, f.y_start, f.z_start};
      const int ce[3] = {f.x_end, f.y_end, f.z_end};
      float st[3], en[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double s0 = (double)g.s[a], d = (double)g.d[a];
        st[a] = (float)__dadd_rn(s0, __dmul_rn(__dmul_rn((double)k, prec), d));                   // :70-72
        en[a] = last ? g.e[a] : (float)__dadd_rn(s0, __dmul_rn(__dmul_rn(prec, (double)(k + 1)), d));   // :74-76, :80-82
        dst[cs[a]] = st[a];
        dst[ce[a]] = en[a];
      }
      dst[f.dx] = prec32;   // :77
      if (last) {
        const double m = __dmul_rn(prec, (double)(n - 1));
        dst[f.dE] = (float)__dmul_rn((double)dE, __dsub_rn(1.0, __ddiv_rn(m, (double)g.lpe)));   // :83
        dst[f.dx] = (float)__dsub_rn((double)g.len, m);                                          // :84
      }
      dst[f.x] = __fmul_rn(0.5f, __fadd_rn(st[0], en[0]));   // :87-89
      dst[f.y] = __fmul_rn(0.5f, __fadd_rn(st[1], en[1]));
      dst[f.z] = __fmul_rn(0.5f, __fadd_rn(st[2], en[2]));
    }
    __syncthreads();
    const int64_t rows = (lim - t0) < kFillRows ? (lim - t0) : kFillRows;
    float *base = out + t0 * F;
    for (int64_t e = threadIdx.x; e < rows * F; e += kFillRows) base[e] = tile[e];
    __syncthreads();
  }
}

struct ChopWs {
  int64_t *row_n, *row_off, *blk;
  int32_t *bad;
};

size_t chop_layout(int64_t n_rows, ChopWs *w, char *base) {
  const int64_t nblk = (n_rows + kChopThreads - 1) / kChopThreads;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t at = off;
    off += (bytes + 255) & ~size_t(255);
    return base ? base + at : nullptr;
  };
  char *a = take(sizeof(int64_t) * (size_t)n_rows);
  char *b = take(sizeof(int64_t) * (size_t)n_rows);
  char *c = take(sizeof(int64_t) * (size_t)(nblk > 0 ? nblk : 1));
  char *d = take(sizeof(int32_t));
  if (w) {
    w->row_n = reinterpret_cast<int64_t *>(a);
    w->row_off = reinterpret_cast<int64_t *>(b);
    w->blk = reinterpret_cast<int64_t *>(c);
    w->bad = reinterpret_cast<int32_t *>(d);
  }
  return off;
}

}  // namespace

size_t chop_workspace_bytes(int64_t n_rows) { return chop_layout(n_rows, nullptr, nullptr); }

int run_chop(const LsimFieldMap &f, const float *tracks, int64_t n_rows, double precision, float *out,
             int64_t capacity, int64_t *n_out, void *ws, cudaStream_t st) {
  if (f.n_fields > kMaxChopFields) return set_error(LSIM_ERR_UNSUPPORTED, "chop: more than 96 columns");
  ChopWs w;
  chop_layout(n_rows, &w, static_cast<char *>(ws));
  const float prec32 = (float)precision;
  const int64_t nblk = (n_rows + kChopThreads - 1) / kChopThreads;
  if (cudaMemsetAsync(w.bad, 0, sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (nblk > 0)
    k_chop_count<<<(unsigned)nblk, kChopThreads, 0, st>>>(tracks, n_rows, f, prec32, w.row_n, w.blk, w.bad);
  k_chop_scan_blocks<<<1, 1024, 0, st>>>(w.blk, nblk, w.bad, n_out);
  if (nblk > 0) k_chop_offsets<<<(unsigned)nblk, kChopThreads, 0, st>>>(w.row_n, n_rows, w.blk, w.row_off);
  if (out && capacity > 0 && n_rows > 0) {
    const int64_t tiles = (capacity + kFillRows - 1) / kFillRows;
    const int64_t cap = (int64_t)device_sm_count() * 16;
    const unsigned grid = (unsigned)(tiles < cap ? tiles : cap);
    const size_t smem = sizeof(float) * kFillRows * (size_t)f.n_fields;
    k_chop_fill<<<grid, kFillRows, smem, st>>>(tracks, n_rows, f, precision, prec32, w.row_n, w.row_off, n_out,
                                               out, capacity);
  }
  return LSIM_OK;
}

}  // namespace lsim
