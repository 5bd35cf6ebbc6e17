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

// s[i] = sum_j cols.w[j] K_ij; with zs, zs[i] = sum_j cols.w[j] K_ij (z_i - z_j)
__global__ void __launch_bounds__(kRbfRows) k_rbf_rows(HitSet rows, HitSet cols, const int2 *__restrict__ col_ranges,
                                                       float two_sigma2, float *__restrict__ s,
                                                       float *__restrict__ zs) {
  __shared__ float cx[kRbfChunk], cy[kRbfChunk], cz[kRbfChunk], cw[kRbfChunk];
  __shared__ int tile_lo, tile_hi;
  const int64_t i = (int64_t)blockIdx.x * kRbfRows + threadIdx.x;
  const bool ok = i < rows.n;
  float xi = 0.f, yi = 0.f, zi = 0.f;
  int ev = 0;
  if (ok) {
    xi = stacked_x(rows, i);
    yi = rows.y[i];
    zi = rows.z[i];
    ev = rows.event[i];
  }
  {
    int a = ok ? ev : 0x7fffffff, b = ok ? ev : -0x7fffffff - 1;
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
  float acc = 0.f, accz = 0.f;
  const int64_t n_chunks = (cols.n + kRbfChunk - 1) / kRbfChunk;
  for (int64_t c = 0; c < n_chunks; ++c) {
    const int2 r = col_ranges[c];
    if (r.y < lo || r.x > hi) continue;   // no common event: every K_ij is 0
    const int64_t j0 = c * kRbfChunk;
    const int cnt = cols.n - j0 < kRbfChunk ? (int)(cols.n - j0) : kRbfChunk;
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kRbfRows) {
      cx[k] = stacked_x(cols, j0 + k);
      cy[k] = cols.y[j0 + k];
      cz[k] = cols.z[j0 + k];
      cw[k] = cols.w[j0 + k];
    }
    __syncthreads();
    if (ok) {
      for (int k = 0; k < cnt; ++k) {
        const float dx = __fsub_rn(xi, cx[k]), dy = __fsub_rn(yi, cy[k]), dz = __fsub_rn(zi, cz[k]);
        const float d = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        const float kv = expf(__fdiv_rn(-d, two_sigma2)) * cw[k];
        acc += kv;
        accz = fmaf(kv, dz, accz);
      }
    }
  }
  if (ok) {
    s[i] = acc;
    if (zs) zs[i] = accz;
  }
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
  if (n > 0) {
    const unsigned g = (unsigned)((n + kRbfRows - 1) / kRbfRows);
    k_rbf_rows<<<g, kRbfRows, 0, st>>>(pred, pred, s.rng_pred, two_s2, s.a, s.az);
    k_rbf_rows<<<g, kRbfRows, 0, st>>>(pred, ref, s.rng_ref, two_s2, s.b, s.bz);
  }
  if (m > 0) k_rbf_rows<<<(unsigned)((m + kRbfRows - 1) / kRbfRows), kRbfRows, 0, st>>>(ref, ref, s.rng_ref, two_s2,
                                                                                            s.c, nullptr);
  k_mse_adc_reduce<<<1, 1024, 0, st>>>(pred, ref, s.a, s.b, s.c, lambda_q, s.tot, out);
  if (n > 0 && (grad_w || grad_z))
    k_mse_adc_grad<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pred, s.a, s.b, s.az, s.bz, s.tot, lambda_q,
                                                                (float)(1.0 / ((double)sigma * (double)sigma)),
                                                                grad_w, grad_z);
  return LSIM_OK;
}

}  // namespace lsim
