// LUT preparation.
//
// lsim_lut_build_templates: the long-diffusion template bank of load_lut
// (consts_jax.py:387-449): template k = response convolved along time
// ('same' mode) with the normalised Gaussian of width sigma_k sampled on
// integer ticks -extent..extent; template 0 is the raw response.
//
// lsim_lut_prepare: the quantities simulate_signals reads from the bank
// (sim_jax.py:184-190, :221-222, :228-255), computed once per bank instead
// of once per call:
//   wmp[i][u][v][k] = (T[i-1], T[i], T[i+1], 0)[u, v, Nt-L+k]   (u, v < 5)
//   cm[i][u][v][t]  = cumsum_t T[i][u, v, :]
//   w0[x][y][k]     = T[0][x, y, Nt-L+k]
//   c0[x][y][t]     = cumsum_t T[0][x, y, :]
// Cumulative sums run sequentially in float32, as numpy/XLA-CPU do.
#include "lsim_internal.cuh"

namespace lsim {

constexpr int kConvThreads = 256;
constexpr int kMaxTaps = 129;

// One CTA per (template k >= 1, LUT row): stage the row in shared memory,
// each thread produces output ticks.
__global__ void k_build_templates(const float *__restrict__ resp, int rows, int nt, const float *__restrict__ sigmas,
                                  int extent, float *__restrict__ out) {
  extern __shared__ float sh[];
  float *x = sh;                           // nt + 2*extent (zero padded)
  float *gk = sh + nt + 2 * extent;        // 2*extent + 1 taps
  const int k = blockIdx.y + 1;
  const int row = blockIdx.x;
  const float *src = resp + (size_t)row * nt;
  const int taps = 2 * extent + 1;
  for (int i = threadIdx.x; i < nt + 2 * extent; i += blockDim.x) {
    const int t = i - extent;
    x[i] = (t >= 0 && t < nt) ? src[t] : 0.f;
  }
  if (threadIdx.x == 0) {
    // norm.pdf(j, scale=sigma) normalised over the taps
    const float sg = sigmas[k];
    float sum = 0.f;
    for (int j = 0; j < taps; ++j) {
      const float z = (float)(j - extent) / sg;
      const float v = expf(-0.5f * z * z) / (2.50662827463100050f * sg);
      gk[j] = v;
      sum += v;
    }
    for (int j = 0; j < taps; ++j) gk[j] = gk[j] / sum;
  }
  __syncthreads();
  float *dst = out + ((size_t)k * rows + row) * nt;
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    // 'same' convolution: y[t] = sum_j g[j] * x[t + extent - j]
    float acc = 0.f;
    for (int j = 0; j < taps; ++j) acc += gk[j] * x[t + 2 * extent - j];
    dst[t] = acc;
  }
}

int run_build_templates(const float *response, int nx, int ny, int nt, const float *sigmas, int n_templates,
                        int extent, float *out, cudaStream_t st) {
  if (2 * extent + 1 > kMaxTaps || n_templates < 1) return LSIM_ERR_UNSUPPORTED;
  const int rows = nx * ny;
  if (cudaMemcpyAsync(out, response, sizeof(float) * (size_t)rows * nt, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return LSIM_ERR_CUDA;
  if (n_templates > 1) {
    const size_t smem = sizeof(float) * (size_t)(nt + 2 * extent + 2 * extent + 1);
    if (smem > 48 * 1024) {
      if (cudaFuncSetAttribute(k_build_templates, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return LSIM_ERR_CUDA;
    }
    dim3 grid(rows, n_templates - 1);
    k_build_templates<<<grid, kConvThreads, smem, st>>>(response, rows, nt, sigmas, extent, out);
  }
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

// (T[i-1], T[i], T[i+1], 0) windows of the main sub-positions, padded like
// the template-0 windows: entry idx is sample idx - 1 (zero at idx = 0 and
// past the signal length).
__global__ void k_prep_wmp(LsimParams p, const float *__restrict__ tmpl, float4 *__restrict__ wmp) {
  const int L = p.signal_length, Nt = p.lut_nt, T = p.n_templates;
  const int64_t total = (int64_t)T * kMainSub * kMainSub * kWinSamples;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int idx = (int)(i % kWinSamples), k = idx - 1;
    const int64_t q = i / kWinSamples;
    const int v = (int)(q % kMainSub), u = (int)((q / kMainSub) % kMainSub), t = (int)(q / (kMainSub * kMainSub));
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (t >= 1 && t <= T - 2 && idx >= 1 && idx <= L) {
      auto at = [&](int tt) { return tmpl[(((size_t)tt * p.lut_nx + u) * p.lut_ny + v) * Nt + (Nt - L) + k]; };
      o.x = at(t - 1); o.y = at(t); o.z = at(t + 1);
    }
    wmp[i] = o;
  }
}

// Template-0 windows padded to kWinSamples: w0[row][idx] is sample idx - 1
// of the window (0 at idx = 0 and past the signal length), so the window
// passes read whole 32-sample chunks without bounds tests.
__global__ void k_prep_w0(LsimParams p, const float *__restrict__ tmpl, float *__restrict__ w0) {
  const int L = p.signal_length, Nt = p.lut_nt;
  const int64_t total = (int64_t)p.lut_nx * p.lut_ny * kWinSamples;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int idx = (int)(i % kWinSamples);
    const int64_t row = i / kWinSamples;
    w0[i] = (idx >= 1 && idx <= L) ? tmpl[(size_t)row * Nt + (Nt - L) + idx - 1] : 0.f;
  }
}

// Sequential float32 cumulative sums, one thread per row.
__global__ void k_prep_cum(LsimParams p, const float *__restrict__ tmpl, float *__restrict__ cm, float *__restrict__ c0) {
  const int Nt = p.lut_nt;
  const int n_main = p.n_templates * kMainSub * kMainSub;
  const int n0 = p.lut_nx * p.lut_ny;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_main + n0) return;
  const float *src;
  float *dst;
  if (r < n_main) {
    const int v = r % kMainSub, u = (r / kMainSub) % kMainSub, t = r / (kMainSub * kMainSub);
    src = tmpl + (((size_t)t * p.lut_nx + u) * p.lut_ny + v) * Nt;
    dst = cm + (size_t)r * Nt;
  } else {
    src = tmpl + (size_t)(r - n_main) * Nt;
    dst = c0 + (size_t)(r - n_main) * Nt;
  }
  float s = 0.f;
  for (int t = 0; t < Nt; ++t) {
    s += src[t];
    dst[t] = s;
  }
}

int run_prepare_tables(const LsimParams &p, const float *templates, void *tables, cudaStream_t st) {
  if (p.lut_nx < kMainSub || p.lut_ny < kMainSub || p.signal_length > p.lut_nt || p.n_templates < 3 ||
      p.signal_length + 2 > kWinSamples)
    return LSIM_ERR_UNSUPPORTED;
  size_t a, b, c, d;
  tables_layout(p, &a, &b, &c, &d);
  char *base = (char *)tables;
  const int blocks = device_sm_count() * 8;
  k_prep_wmp<<<blocks, 256, 0, st>>>(p, templates, (float4 *)(base + a));
  k_prep_w0<<<blocks, 256, 0, st>>>(p, templates, (float *)(base + c));
  const int rows = p.n_templates * kMainSub * kMainSub + p.lut_nx * p.lut_ny;
  k_prep_cum<<<(rows + 127) / 128, 128, 0, st>>>(p, templates, (float *)(base + b), (float *)(base + d));
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
