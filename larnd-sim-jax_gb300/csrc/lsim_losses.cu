// Hit-level fit loss mse_adc (src/larndsim/losses_jax.py:13-39 rbf_kernel and
// mmd, :60-79 mse_adc): a weighted maximum mean discrepancy between the
// predicted hits and the reference hits with a Gaussian (RBF) kernel on the
// stacked coordinates (x + event * 1e5, y, z), plus a squared relative
// difference of the total charges.  Also its gradient with respect to the
// predicted weights w = Q * hit_prob and hit z (the coordinates with a
// gradient path: z depends on the drift velocity).
//
// The pairwise sums are computed row-wise: for each row hit i of one set and
// all column hits j of another, s_i = sum_j v_j K_ij and, for the predicted
// rows, s'_i = sum_j v_j K_ij (z_i - z_j).  Columns are staged through shared
// memory in chunks of 256; chunks whose event range is disjoint from the row
// tile's are skipped: hits of different events are at least 1e5 - (detector
// size) apart in x, so their kernel value exp(-d / (2 sigma^2)) is exactly 0
// in float32 and skipping them changes nothing.  Inputs ordered by event
// (as the hit compaction emits them) make almost all chunks skippable.
#include <cmath>

#include "lsim_internal.cuh"

namespace lsim {
namespace {

constexpr int kRbfRows = 128;    // row hits per block (one per thread)
constexpr int kRbfChunk = 256;   // column hits staged per chunk
constexpr float kEventOffset = 1e5f;

struct HitSet {
  const float *x, *y, *z, *w;
  const int32_t *event;
  int64_t n;
};

// stacked coordinates, float32 as the reference forms them: x + event * 1e5
__device__ __forceinline__ float stacked_x(const HitSet &h, int64_t i) {
  return __fadd_rn(h.x[i], __fmul_rn((float)h.event[i], kEventOffset));
}

// per chunk of kRbfChunk hits: the smallest and largest event id
__global__ void k_chunk_events(const int32_t *__restrict__ event, int64_t n, int2 *__restrict__ ranges) {
  __shared__ int lo[kRbfChunk / 32], hi[kRbfChunk / 32];
  const int64_t i = (int64_t)blockIdx.x * kRbfChunk + threadIdx.x;
  int a = 0x7fffffff, b = -0x7fffffff - 1;
  if (i < n) a = b = event[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    lo[threadIdx.x >> 5] = a;
    hi[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kRbfChunk / 32; ++k) {
      a = min(a, lo[k]);
      b = max(b, hi[k]);
    }
    ranges[blockIdx.x] = make_int2(min(a, lo[0]), max(b, hi[0]));
  }
}

// s[i] = sum_j cols.w[j] K_ij; with zs, zs[i] = sum_j cols.w[j] K_ij (z_i - z_j).
// Each thread owns two row hits (a block covers 2 kRbfRows rows) and reads
// each staged column once for both (x, y, z, w in one 16-byte word).  The
// exponent is -d / (2 sigma^2) as the reference divides; when 2 sigma^2 is a
// power of two that is the exact product with its reciprocal (kMul).
constexpr int kRbfPerThread = 2;

__device__ __forceinline__ float rbf_term(float xi, float yi, float zi, const float4 &c, float two_sigma2,
                                          float inv, bool mul, float *dz_out) {
  const float dx = __fsub_rn(xi, c.x), dy = __fsub_rn(yi, c.y), dz = __fsub_rn(zi, c.z);
  const float d = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  *dz_out = dz;
  return expf(mul ? __fmul_rn(-d, inv) : __fdiv_rn(-d, two_sigma2)) * c.w;
}

template <bool kMul>
__global__ void __launch_bounds__(kRbfRows) k_rbf_rows(HitSet rows, HitSet cols, const int2 *__restrict__ col_ranges,
                                                       float two_sigma2, float inv_two_sigma2, float *__restrict__ s,
                                                       float *__restrict__ zs) {
  __shared__ float4 col[kRbfChunk];
  __shared__ int tile_lo, tile_hi;
  const int64_t i0 = (int64_t)blockIdx.x * (kRbfPerThread * kRbfRows) + threadIdx.x, i1 = i0 + kRbfRows;
  const bool ok0 = i0 < rows.n, ok1 = i1 < rows.n;
  float x0 = 0.f, y0 = 0.f, z0 = 0.f, x1 = 0.f, y1 = 0.f, z1 = 0.f;
  int a = 0x7fffffff, b = -0x7fffffff - 1;
  if (ok0) {
    x0 = stacked_x(rows, i0);
    y0 = rows.y[i0];
    z0 = rows.z[i0];
    a = min(a, rows.event[i0]);
    b = max(b, rows.event[i0]);
  }
  if (ok1) {
    x1 = stacked_x(rows, i1);
    y1 = rows.y[i1];
    z1 = rows.z[i1];
    a = min(a, rows.event[i1]);
    b = max(b, rows.event[i1]);
  }
  {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
      b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if (threadIdx.x == 0) {
      tile_lo = 0x7fffffff;
      tile_hi = -0x7fffffff - 1;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&tile_lo, a);
      atomicMax(&tile_hi, b);
    }
    __syncthreads();
  }
  const int lo = tile_lo, hi = tile_hi;
  float acc0 = 0.f, accz0 = 0.f, acc1 = 0.f, accz1 = 0.f;
  const int64_t n_chunks = (cols.n + kRbfChunk - 1) / kRbfChunk;
  for (int64_t c = 0; c < n_chunks; ++c) {
    const int2 r = col_ranges[c];
    if (r.y < lo || r.x > hi) continue;   // no common event: every K_ij is 0
    const int64_t j0 = c * kRbfChunk;
    const int cnt = cols.n - j0 < kRbfChunk ? (int)(cols.n - j0) : kRbfChunk;
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kRbfRows)
      col[k] = make_float4(stacked_x(cols, j0 + k), cols.y[j0 + k], cols.z[j0 + k], cols.w[j0 + k]);
    __syncthreads();
    if (ok0) {
      for (int k = 0; k < cnt; ++k) {
        const float4 cv = col[k];
        float dz0, dz1;
        const float kv0 = rbf_term(x0, y0, z0, cv, two_sigma2, inv_two_sigma2, kMul, &dz0);
        const float kv1 = rbf_term(x1, y1, z1, cv, two_sigma2, inv_two_sigma2, kMul, &dz1);
        acc0 += kv0;
        accz0 = fmaf(kv0, dz0, accz0);
        acc1 += kv1;
        accz1 = fmaf(kv1, dz1, accz1);
      }
    }
  }
  if (ok0) {
    s[i0] = acc0;
    if (zs) zs[i0] = accz0;
  }
  if (ok1) {
    s[i1] = acc1;
    if (zs) zs[i1] = accz1;
  }
}

// k_rbf_rows over all rows, with the exponent's form chosen for 2 sigma^2
void launch_rbf_rows(const HitSet &rows, const HitSet &cols, const int2 *col_ranges, float two_sigma2, float *s,
                     float *zs, cudaStream_t st) {
  if (rows.n <= 0) return;
  int e;
  const bool pow2 = std::frexp((double)two_sigma2, &e) == 0.5;
  const float inv = (float)(1.0 / (double)two_sigma2);
  const unsigned g = (unsigned)((rows.n + kRbfPerThread * kRbfRows - 1) / (kRbfPerThread * kRbfRows));
  if (pow2)
    k_rbf_rows<true><<<g, kRbfRows, 0, st>>>(rows, cols, col_ranges, two_sigma2, inv, s, zs);
  else
    k_rbf_rows<false><<<g, kRbfRows, 0, st>>>(rows, cols, col_ranges, two_sigma2, inv, s, zs);
}

struct MseAdcTotals {
  double sw, sv, A, B, C;
  float loss, mmd, charge;
};

// one block: the totals and the loss
__global__ void k_mse_adc_reduce(HitSet pred, HitSet ref, const float *__restrict__ a, const float *__restrict__ b,
                                 const float *__restrict__ c, float lambda_q, MseAdcTotals *tot, float *out) {
  __shared__ double red[5][32];
  double sw = 0, sv = 0, A = 0, B = 0, C = 0;
  for (int64_t i = threadIdx.x; i < pred.n; i += blockDim.x) {
    const double w = pred.w[i];
    sw += w;
    A += w * a[i];
    B += w * b[i];
  }
  for (int64_t j = threadIdx.x; j < ref.n; j += blockDim.x) {
    const double v = ref.w[j];
    sv += v;
    C += v * c[j];
  }
  double vals[5] = {sw, sv, A, B, C};
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    double v = vals[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    double t[5] = {0, 0, 0, 0, 0};
    for (int q = 0; q < 5; ++q)
      for (int k = 0; k < nw; ++k) t[q] += red[q][k];
    MseAdcTotals r;
    r.sw = t[0];
    r.sv = t[1];
    r.A = t[2];
    r.B = t[3];
    r.C = t[4];
    const double mmd = r.A / (r.sw * r.sw) + r.C / (r.sv * r.sv) - 2.0 * r.B / (r.sw * r.sv);
    const double rel = (r.sw - r.sv) / (r.sv + 1e-6);
    r.mmd = (float)mmd;
    r.charge = (float)(rel * rel);
    r.loss = (float)(mmd + (double)lambda_q * rel * rel);
    *tot = r;
    out[0] = r.loss;
    out[1] = r.mmd;
    out[2] = r.charge;
  }
}

// dL/dw_i and dL/dz_i of L = mmd + lambda_q * charge
__global__ void k_mse_adc_grad(HitSet pred, const float *__restrict__ a, const float *__restrict__ b,
                               const float *__restrict__ az, const float *__restrict__ bz,
                               const MseAdcTotals *__restrict__ tot, float lambda_q, float inv_sigma2,
                               float *__restrict__ gw, float *__restrict__ gz) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pred.n) return;
  const MseAdcTotals t = *tot;
  const double sw2 = t.sw * t.sw, swsv = t.sw * t.sv;
  if (gw) {
    const double dm = 2.0 * a[i] / sw2 - 2.0 * t.A / (sw2 * t.sw) - 2.0 * b[i] / swsv + 2.0 * t.B / (sw2 * t.sv);
    const double dc = 2.0 * (t.sw - t.sv) / ((t.sv + 1e-6) * (t.sv + 1e-6));
    gw[i] = (float)(dm + (double)lambda_q * dc);
  }
  if (gz) {
    const double w = pred.w[i];
    gz[i] = (float)(-2.0 * w * (double)inv_sigma2 * ((double)az[i] / sw2 - (double)bz[i] / swsv));
  }
}

// ---------------------------------------------------------------- nll_loss and chamfer_3d
// Both stack (x + event * 1e9, y, z[, Q / adc_norm]) (losses_jax.py:221-222,
// :337-338); hits of different events are 1e9 apart and never interact.

struct HitSet4 {
  const float *x, *y, *z, *q, *w;   // q: 4th coordinate (nll) or null
  const int32_t *event;
  int64_t n;
};

__device__ __forceinline__ float stacked_x9(const HitSet4 &h, int64_t i) {
  return __fadd_rn(h.x[i], __fmul_rn((float)h.event[i], 1e9f));
}

// block-wide event range of the row tile into (lo, hi)
__device__ __forceinline__ void tile_event_range(bool ok, int ev, int *lo_s, int *hi_s, int &lo, int &hi) {
  int a = ok ? ev : 0x7fffffff, b = ok ? ev : -0x7fffffff - 1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if (threadIdx.x == 0) {
    *lo_s = 0x7fffffff;
    *hi_s = -0x7fffffff - 1;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicMin(lo_s, a);
    atomicMax(hi_s, b);
  }
  __syncthreads();
  lo = *lo_s;
  hi = *hi_s;
}

// nll_loss sums: s[i] = sum_j w_j K_ij, sz[i] = sum_j w_j K_ij (z_i - z_j),
// sq[i] = sum_j w_j K_ij (q_i - q_j), K = exp(-|4-d difference|^2 / (2 sigma^2)).
// Two row hits per thread, as k_rbf_rows.
struct Row4 {
  float x, y, z, q;
};

__device__ __forceinline__ float gauss4_term(const Row4 &r, const float4 &c, float w, float two_sigma2, float inv,
                                             bool mul, float *dz_out, float *dq_out) {
  const float dx = __fsub_rn(r.x, c.x), dy = __fsub_rn(r.y, c.y), dz = __fsub_rn(r.z, c.z);
  const float dq = __fsub_rn(r.q, c.w);
  const float d = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)),
                            __fmul_rn(dq, dq));
  *dz_out = dz;
  *dq_out = dq;
  return expf(mul ? __fmul_rn(-d, inv) : __fdiv_rn(-d, two_sigma2)) * w;
}

template <bool kMul>
__global__ void __launch_bounds__(kRbfRows) k_gauss4_rows(HitSet4 rows, HitSet4 cols,
                                                          const int2 *__restrict__ col_ranges, float two_sigma2,
                                                          float inv_two_sigma2, float *__restrict__ s,
                                                          float *__restrict__ sz, float *__restrict__ sq) {
  __shared__ float4 col[kRbfChunk];
  __shared__ float cw[kRbfChunk];
  __shared__ int lo_s, hi_s;
  const int64_t i0 = (int64_t)blockIdx.x * (kRbfPerThread * kRbfRows) + threadIdx.x, i1 = i0 + kRbfRows;
  const bool ok0 = i0 < rows.n, ok1 = i1 < rows.n;
  Row4 r0{0.f, 0.f, 0.f, 0.f}, r1{0.f, 0.f, 0.f, 0.f};
  int ev0 = 0, ev1 = 0;
  if (ok0) {
    r0 = Row4{stacked_x9(rows, i0), rows.y[i0], rows.z[i0], rows.q[i0]};
    ev0 = rows.event[i0];
  }
  if (ok1) {
    r1 = Row4{stacked_x9(rows, i1), rows.y[i1], rows.z[i1], rows.q[i1]};
    ev1 = rows.event[i1];
  }
  int a = 0x7fffffff, b = -0x7fffffff - 1;   // the tile's event range
  if (ok0) a = b = ev0;
  if (ok1) {
    a = min(a, ev1);
    b = max(b, ev1);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if (threadIdx.x == 0) {
    lo_s = 0x7fffffff;
    hi_s = -0x7fffffff - 1;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&lo_s, a);
    atomicMax(&hi_s, b);
  }
  __syncthreads();
  const int lo = lo_s, hi = hi_s;
  float acc0 = 0.f, accz0 = 0.f, accq0 = 0.f, acc1 = 0.f, accz1 = 0.f, accq1 = 0.f;
  const int64_t n_chunks = (cols.n + kRbfChunk - 1) / kRbfChunk;
  for (int64_t c = 0; c < n_chunks; ++c) {
    const int2 r = col_ranges[c];
    if (r.y < lo || r.x > hi) continue;
    const int64_t j0 = c * kRbfChunk;
    const int cnt = cols.n - j0 < kRbfChunk ? (int)(cols.n - j0) : kRbfChunk;
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kRbfRows) {
      col[k] = make_float4(stacked_x9(cols, j0 + k), cols.y[j0 + k], cols.z[j0 + k], cols.q[j0 + k]);
      cw[k] = cols.w[j0 + k];
    }
    __syncthreads();
    if (ok0) {
      for (int k = 0; k < cnt; ++k) {
        const float4 cv = col[k];
        const float w = cw[k];
        float dz0, dq0, dz1, dq1;
        const float kv0 = gauss4_term(r0, cv, w, two_sigma2, inv_two_sigma2, kMul, &dz0, &dq0);
        const float kv1 = gauss4_term(r1, cv, w, two_sigma2, inv_two_sigma2, kMul, &dz1, &dq1);
        acc0 += kv0;
        accz0 = fmaf(kv0, dz0, accz0);
        accq0 = fmaf(kv0, dq0, accq0);
        acc1 += kv1;
        accz1 = fmaf(kv1, dz1, accz1);
        accq1 = fmaf(kv1, dq1, accq1);
      }
    }
  }
  if (ok0) {
    s[i0] = acc0;
    if (sz) sz[i0] = accz0;
    if (sq) sq[i0] = accq0;
  }
  if (ok1) {
    s[i1] = acc1;
    if (sz) sz[i1] = accz1;
    if (sq) sq[i1] = accq1;
  }
}

void launch_gauss4_rows(const HitSet4 &rows, const HitSet4 &cols, const int2 *col_ranges, float two_sigma2, float *s,
                        float *sz, float *sq, cudaStream_t st) {
  if (rows.n <= 0) return;
  int e;
  const bool pow2 = std::frexp((double)two_sigma2, &e) == 0.5;
  const float inv = (float)(1.0 / (double)two_sigma2);
  const unsigned g = (unsigned)((rows.n + kRbfPerThread * kRbfRows - 1) / (kRbfPerThread * kRbfRows));
  if (pow2)
    k_gauss4_rows<true><<<g, kRbfRows, 0, st>>>(rows, cols, col_ranges, two_sigma2, inv, s, sz, sq);
  else
    k_gauss4_rows<false><<<g, kRbfRows, 0, st>>>(rows, cols, col_ranges, two_sigma2, inv, s, sz, sq);
}

// column weights of the second nll pass: (ref_hit_prob > 0.5) / (lambda + 1e-10)
__global__ void k_nll_colw(const float *__restrict__ ref_hp, const float *__restrict__ lam, int64_t m,
                           float *__restrict__ c) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m) c[j] = ref_hp[j] > 0.5f ? 1.0f / (lam[j] + 1e-10f) : 0.0f;
}

__global__ void k_nll_reduce(const float *__restrict__ hp, int64_t n, const float *__restrict__ ref_hp,
                             const float *__restrict__ lam, int64_t m, float *out) {
  __shared__ double red[2][32];
  double t2 = 0, t1 = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) t2 += hp[i];
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x)
    if (ref_hp[j] > 0.5f) t1 += (double)logf(lam[j] + 1e-10f);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t2 += __shfl_xor_sync(0xffffffffu, t2, o);
    t1 += __shfl_xor_sync(0xffffffffu, t1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = t2;
    red[1][threadIdx.x >> 5] = t1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      a += red[0][k];
      b += red[1][k];
    }
    out[0] = (float)(a - b);
    out[1] = (float)a;
    out[2] = (float)b;
  }
}

__global__ void k_nll_grad(const float *__restrict__ hp, int64_t n, const float *__restrict__ s,
                           const float *__restrict__ sz, const float *__restrict__ sq, float inv_sigma2,
                           float *__restrict__ g_hp, float *__restrict__ g_z, float *__restrict__ g_q) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (g_hp) g_hp[i] = 1.0f - s[i];
  if (g_z) g_z[i] = hp[i] * inv_sigma2 * sz[i];
  if (g_q) g_q[i] = hp[i] * inv_sigma2 * sq[i];
}

// chamfer: nearest column of every row (first index on ties) and its
// squared distance; rows with no column in their events get (inf, -1)
__global__ void __launch_bounds__(kRbfRows) k_nn_rows(HitSet4 rows, HitSet4 cols, const int2 *__restrict__ col_ranges,
                                                      float *__restrict__ dmin, int32_t *__restrict__ amin) {
  __shared__ float cx[kRbfChunk], cy[kRbfChunk], cz[kRbfChunk];
  __shared__ int lo_s, hi_s;
  const int64_t i = (int64_t)blockIdx.x * kRbfRows + threadIdx.x;
  const bool ok = i < rows.n;
  float xi = 0.f, yi = 0.f, zi = 0.f;
  int ev = 0;
  if (ok) {
    xi = stacked_x9(rows, i);
    yi = rows.y[i];
    zi = rows.z[i];
    ev = rows.event[i];
  }
  int lo, hi;
  tile_event_range(ok, ev, &lo_s, &hi_s, lo, hi);
  float best = INFINITY;
  int64_t arg = -1;
  const int64_t n_chunks = (cols.n + kRbfChunk - 1) / kRbfChunk;
  for (int64_t c = 0; c < n_chunks; ++c) {
    const int2 r = col_ranges[c];
    if (r.y < lo || r.x > hi) continue;   // 1e9 apart: never the nearest when the row's event has columns
    const int64_t j0 = c * kRbfChunk;
    const int cnt = cols.n - j0 < kRbfChunk ? (int)(cols.n - j0) : kRbfChunk;
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kRbfRows) {
      cx[k] = stacked_x9(cols, j0 + k);
      cy[k] = cols.y[j0 + k];
      cz[k] = cols.z[j0 + k];
    }
    __syncthreads();
    if (ok) {
      for (int k = 0; k < cnt; ++k) {
        const float dx = __fsub_rn(xi, cx[k]), dy = __fsub_rn(yi, cy[k]), dz = __fsub_rn(zi, cz[k]);
        const float d = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        if (d < best) {
          best = d;
          arg = j0 + k;
        }
      }
    }
  }
  if (ok) {
    dmin[i] = best;
    amin[i] = (int32_t)arg;
  }
}

// chamfer gradient gathers for predicted row i over the reference hits j
// whose nearest predicted hit is i: sum of mb_j wb_j and of wb_j 2 (z_i - z_j)
__global__ void __launch_bounds__(kRbfRows) k_chamfer_back(HitSet4 rows, HitSet4 cols,
                                                           const int2 *__restrict__ col_ranges,
                                                           const float *__restrict__ col_dmin,
                                                           const int32_t *__restrict__ col_amin,
                                                           float *__restrict__ acc_w, float *__restrict__ acc_z) {
  __shared__ float cz[kRbfChunk], cw[kRbfChunk], cd[kRbfChunk];
  __shared__ int ca[kRbfChunk];
  __shared__ int lo_s, hi_s;
  const int64_t i = (int64_t)blockIdx.x * kRbfRows + threadIdx.x;
  const bool ok = i < rows.n;
  const int ev = ok ? rows.event[i] : 0;
  const float zi = ok ? rows.z[i] : 0.f;
  int lo, hi;
  tile_event_range(ok, ev, &lo_s, &hi_s, lo, hi);
  double aw = 0.0, az = 0.0;
  const int64_t n_chunks = (cols.n + kRbfChunk - 1) / kRbfChunk;
  for (int64_t c = 0; c < n_chunks; ++c) {
    const int2 r = col_ranges[c];
    if (r.y < lo || r.x > hi) continue;
    const int64_t j0 = c * kRbfChunk;
    const int cnt = cols.n - j0 < kRbfChunk ? (int)(cols.n - j0) : kRbfChunk;
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kRbfRows) {
      cz[k] = cols.z[j0 + k];
      cw[k] = cols.w[j0 + k];
      cd[k] = col_dmin[j0 + k];
      ca[k] = col_amin[j0 + k];
    }
    __syncthreads();
    if (ok) {
      for (int k = 0; k < cnt; ++k) {
        if (ca[k] == (int)i && cd[k] < 1e4f) {
          aw += (double)cd[k] * (double)cw[k];
          az += (double)cw[k] * 2.0 * (double)__fsub_rn(zi, cz[k]);
        }
      }
    }
  }
  if (ok) {
    acc_w[i] = (float)aw;
    acc_z[i] = (float)az;
  }
}

// loss and gradients of chamfer_distance_3d_og (losses_jax.py:181-211)
__global__ void k_chamfer_reduce(const float *__restrict__ wa, int64_t n, const float *__restrict__ wb, int64_t m,
                                 const float *__restrict__ ma, const int32_t *__restrict__ ia,
                                 const float *__restrict__ mb, const int32_t *__restrict__ ib, float *out) {
  __shared__ double red[32];
  double t = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
    if (ma[i] < 1e4f) t += (double)ma[i] * wa[i] * wb[ia[i]];
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x)
    if (mb[j] < 1e4f) t += (double)mb[j] * wb[j] * wa[ib[j]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) a += red[k];
    out[0] = (float)a;
  }
}

__global__ void k_chamfer_grad(HitSet4 pred, HitSet4 ref, const float *__restrict__ ma,
                               const int32_t *__restrict__ ia, const float *__restrict__ acc_w,
                               const float *__restrict__ acc_z, float *__restrict__ g_w, float *__restrict__ g_z) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pred.n) return;
  double gw = acc_w[i], gz = (double)pred.w[i] * acc_z[i];
  if (ma[i] < 1e4f) {
    const int j = ia[i];
    gw += (double)ma[i] * ref.w[j];
    gz += (double)pred.w[i] * ref.w[j] * 2.0 * (double)__fsub_rn(pred.z[i], ref.z[j]);
  }
  if (g_w) g_w[i] = (float)gw;
  if (g_z) g_z[i] = (float)gz;
}

struct MseAdcWs {
  float *a, *az, *b, *bz, *c;
  int2 *rng_pred, *rng_ref;
  MseAdcTotals *tot;
};

size_t mse_adc_layout(int64_t n, int64_t m, MseAdcWs *w, char *base) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t at = off;
    off += (bytes + 255) & ~size_t(255);
    return base ? base + at : nullptr;
  };
  char *pa = take(4 * (size_t)n), *paz = take(4 * (size_t)n), *pb = take(4 * (size_t)n), *pbz = take(4 * (size_t)n);
  char *pc = take(4 * (size_t)m);
  char *r1 = take(sizeof(int2) * (size_t)((n + kRbfChunk - 1) / kRbfChunk + 1));
  char *r2 = take(sizeof(int2) * (size_t)((m + kRbfChunk - 1) / kRbfChunk + 1));
  char *pt = take(sizeof(MseAdcTotals));
  if (w) {
    w->a = reinterpret_cast<float *>(pa);
    w->az = reinterpret_cast<float *>(paz);
    w->b = reinterpret_cast<float *>(pb);
    w->bz = reinterpret_cast<float *>(pbz);
    w->c = reinterpret_cast<float *>(pc);
    w->rng_pred = reinterpret_cast<int2 *>(r1);
    w->rng_ref = reinterpret_cast<int2 *>(r2);
    w->tot = reinterpret_cast<MseAdcTotals *>(pt);
  }
  return off;
}

}  // namespace

size_t mse_adc_workspace_bytes(int64_t n, int64_t m) { return mse_adc_layout(n, m, nullptr, nullptr); }

int run_mse_adc(const float *x, const float *y, const float *z, const int32_t *event, const float *w, int64_t n,
                const float *rx, const float *ry, const float *rz, const int32_t *revent, const float *rw, int64_t m,
                float sigma, float lambda_q, float *out, float *grad_w, float *grad_z, void *ws, cudaStream_t st) {
  MseAdcWs s;
  mse_adc_layout(n, m, &s, static_cast<char *>(ws));
  const HitSet pred{x, y, z, w, event, n}, ref{rx, ry, rz, rw, revent, m};
  const float two_s2 = (float)(2.0 * (double)sigma * (double)sigma);
  if (n > 0) k_chunk_events<<<(unsigned)((n + kRbfChunk - 1) / kRbfChunk), kRbfChunk, 0, st>>>(event, n, s.rng_pred);
  if (m > 0) k_chunk_events<<<(unsigned)((m + kRbfChunk - 1) / kRbfChunk), kRbfChunk, 0, st>>>(revent, m, s.rng_ref);
  launch_rbf_rows(pred, pred, s.rng_pred, two_s2, s.a, s.az, st);
  launch_rbf_rows(pred, ref, s.rng_ref, two_s2, s.b, s.bz, st);
  launch_rbf_rows(ref, ref, s.rng_ref, two_s2, s.c, nullptr, st);
  k_mse_adc_reduce<<<1, 1024, 0, st>>>(pred, ref, s.a, s.b, s.c, lambda_q, s.tot, out);
  if (n > 0 && (grad_w || grad_z))
    k_mse_adc_grad<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pred, s.a, s.b, s.az, s.bz, s.tot, lambda_q,
                                                                (float)(1.0 / ((double)sigma * (double)sigma)),
                                                                grad_w, grad_z);
  return LSIM_OK;
}


// nll_loss: out[0..2] = loss, sum of hit_prob, sum of log(lambda + 1e-10)
size_t nll_workspace_bytes(int64_t n, int64_t m) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  return 3 * al(4 * (size_t)n) + 2 * al(4 * (size_t)m) +
         al(sizeof(int2) * (size_t)((n + kRbfChunk - 1) / kRbfChunk + 1)) +
         al(sizeof(int2) * (size_t)((m + kRbfChunk - 1) / kRbfChunk + 1));
}

int run_nll(const float *x, const float *y, const float *z, const float *q, const int32_t *event, const float *hp,
            int64_t n, const float *rx, const float *ry, const float *rz, const float *rq, const int32_t *revent,
            const float *rhp, int64_t m, float sigma, float *out, float *g_q, float *g_z, float *g_hp, void *ws,
            cudaStream_t st) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  char *b = static_cast<char *>(ws);
  float *s = reinterpret_cast<float *>(b); b += al(4 * (size_t)n);
  float *sz = reinterpret_cast<float *>(b); b += al(4 * (size_t)n);
  float *sq = reinterpret_cast<float *>(b); b += al(4 * (size_t)n);
  float *lam = reinterpret_cast<float *>(b); b += al(4 * (size_t)m);
  float *cw = reinterpret_cast<float *>(b); b += al(4 * (size_t)m);
  int2 *rng_pred = reinterpret_cast<int2 *>(b); b += al(sizeof(int2) * (size_t)((n + kRbfChunk - 1) / kRbfChunk + 1));
  int2 *rng_ref = reinterpret_cast<int2 *>(b);
  const float two_s2 = (float)(2.0 * (double)sigma * (double)sigma);
  const HitSet4 pred{x, y, z, q, hp, event, n};
  if (n > 0) k_chunk_events<<<(unsigned)((n + kRbfChunk - 1) / kRbfChunk), kRbfChunk, 0, st>>>(event, n, rng_pred);
  if (m > 0) k_chunk_events<<<(unsigned)((m + kRbfChunk - 1) / kRbfChunk), kRbfChunk, 0, st>>>(revent, m, rng_ref);
  if (m > 0)   // lambda_j = sum_i hp_i K_ij
    launch_gauss4_rows(HitSet4{rx, ry, rz, rq, rhp, revent, m}, pred, rng_pred, two_s2, lam, nullptr, nullptr, st);
  if (m > 0) k_nll_colw<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(rhp, lam, m, cw);
  if (n > 0)
    launch_gauss4_rows(pred, HitSet4{rx, ry, rz, rq, cw, revent, m}, rng_ref, two_s2, s, sz, sq, st);
  k_nll_reduce<<<1, 1024, 0, st>>>(hp, n, rhp, lam, m, out);
  if (n > 0 && (g_q || g_z || g_hp))
    k_nll_grad<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(hp, n, s, sz, sq,
                                                            (float)(1.0 / ((double)sigma * (double)sigma)), g_hp,
                                                            g_z, g_q);
  return LSIM_OK;
}

size_t chamfer_workspace_bytes(int64_t n, int64_t m) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  return 4 * al(4 * (size_t)n) + 2 * al(4 * (size_t)m) +
         al(sizeof(int2) * (size_t)((n + kRbfChunk - 1) / kRbfChunk + 1)) +
         al(sizeof(int2) * (size_t)((m + kRbfChunk - 1) / kRbfChunk + 1));
}

int run_chamfer(const float *x, const float *y, const float *z, const int32_t *event, const float *w, int64_t n,
                const float *rx, const float *ry, const float *rz, const int32_t *revent, const float *rw, int64_t m,
                float *out, float *g_w, float *g_z, void *ws, cudaStream_t st) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  char *b = static_cast<char *>(ws);
  float *ma = reinterpret_cast<float *>(b); b += al(4 * (size_t)n);
  int32_t *ia = reinterpret_cast<int32_t *>(b); b += al(4 * (size_t)n);
  float *aw = reinterpret_cast<float *>(b); b += al(4 * (size_t)n);
  float *az = reinterpret_cast<float *>(b); b += al(4 * (size_t)n);
  float *mb = reinterpret_cast<float *>(b); b += al(4 * (size_t)m);
  int32_t *ib = reinterpret_cast<int32_t *>(b); b += al(4 * (size_t)m);
  int2 *rng_pred = reinterpret_cast<int2 *>(b); b += al(sizeof(int2) * (size_t)((n + kRbfChunk - 1) / kRbfChunk + 1));
  int2 *rng_ref = reinterpret_cast<int2 *>(b);
  const HitSet4 pred{x, y, z, nullptr, w, event, n}, ref{rx, ry, rz, nullptr, rw, revent, m};
  if (n > 0) k_chunk_events<<<(unsigned)((n + kRbfChunk - 1) / kRbfChunk), kRbfChunk, 0, st>>>(event, n, rng_pred);
  if (m > 0) k_chunk_events<<<(unsigned)((m + kRbfChunk - 1) / kRbfChunk), kRbfChunk, 0, st>>>(revent, m, rng_ref);
  if (n > 0) k_nn_rows<<<(unsigned)((n + kRbfRows - 1) / kRbfRows), kRbfRows, 0, st>>>(pred, ref, rng_ref, ma, ia);
  if (m > 0) k_nn_rows<<<(unsigned)((m + kRbfRows - 1) / kRbfRows), kRbfRows, 0, st>>>(ref, pred, rng_pred, mb, ib);
  k_chamfer_reduce<<<1, 1024, 0, st>>>(w, n, rw, m, ma, ia, mb, ib, out);
  if (n > 0 && (g_w || g_z)) {
    k_chamfer_back<<<(unsigned)((n + kRbfRows - 1) / kRbfRows), kRbfRows, 0, st>>>(pred, ref, rng_ref, mb, ib, aw,
                                                                                   az);
    k_chamfer_grad<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pred, ref, ma, ia, aw, az, g_w, g_z);
  }
  return LSIM_OK;
}

}  // namespace lsim
