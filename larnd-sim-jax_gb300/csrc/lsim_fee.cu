// Standalone front end on materialised waveforms, hit assembly + stream
// compaction, and the parametrised-current accumulation.
//
// Reference: get_adc_values / digitize (fee_jax.py:55-71, :168-279),
// simulate_stochastic (sim_jax.py:738-769), parse_output (sim_jax.py:619-647),
// current_mc / current_model_diff / integrated_expon_diff / emg_pdf
// (detsim_jax.py:440-474, :581-639) and accumulate_signals_parametrized
// (detsim_jax.py:207-228).
#include <cuda.h>

#include <cstdio>
#include <mutex>

#include "lsim_internal.cuh"
#include "lsim_fee.cuh"

namespace lsim {

constexpr int kFeeWarps = 4;
constexpr int kFeeRow = 2048;

// ---------------------------------------------------------------- FEE on wfs

__global__ void __launch_bounds__(kFeeWarps * kWarp)
    k_fee(LsimParams p, const float *__restrict__ wfs, int64_t n_pix, int32_t T, const float *__restrict__ normals,
          float *adc_out, float *tick_out, float *integral_out) {
  __shared__ __align__(16) float rows[kFeeWarps][kFeeRow];
  const int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  float *C = rows[wid];
  const int H = p.max_adc_values;
  for (int64_t r = (int64_t)blockIdx.x * kFeeWarps + wid; r < n_pix; r += (int64_t)gridDim.x * kFeeWarps) {
    const float *src = wfs + r * (int64_t)T;
    if ((T & 3) == 0) {
      const float4 *s4 = reinterpret_cast<const float4 *>(src);
      float4 *d4 = reinterpret_cast<float4 *>(C);
      for (int i = lane; i < T / 4; i += kWarp) d4[i] = __ldg(s4 + i);
    } else {
      for (int i = lane; i < T; i += kWarp) C[i] = __ldg(src + i);
    }
    __syncwarp();
    warp_cumsum_charge(C, T, p.t_sampling, lane);
    const float *nrm = normals ? normals + r * (1 + 3 * H) : nullptr;
    fee_forward(p, C, T, nrm, adc_out + r * H, tick_out + r * H, nullptr,
                integral_out ? integral_out + r * H : nullptr, normals == nullptr && p.threshold > 0.f, lane);
    __syncwarp();
  }
}

int run_fee(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals, float *adc_out,
            float *tick_out, float *integral_out, cudaStream_t st) {
  if (n_t > kFeeRow || n_t < 2 || p.max_adc_values > LSIM_MAX_HITS) return LSIM_ERR_UNSUPPORTED;
  if (n_pix <= 0) return LSIM_OK;
  int64_t blocks = (n_pix + kFeeWarps - 1) / kFeeWarps;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  k_fee<<<(unsigned)blocks, kFeeWarps * kWarp, 0, st>>>(p, wfs, n_pix, n_t, normals, adc_out, tick_out, integral_out);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

// ---------------------------------------------------------------- FEE vector-Jacobian product

// dL/dwfs of the front end + digitize for a cotangent on the ADCs: the
// forward is recomputed per row (reset masks kept per warp in the
// workspace), then the same adjoint the fused LUT gradient runs.
__global__ void __launch_bounds__(kFeeWarps * kWarp)
    k_fee_vjp(LsimParams p, const float *__restrict__ wfs, int64_t n_pix, int32_t T, const float *__restrict__ normals,
              const float *__restrict__ g_adc, float *__restrict__ g_wfs, uint32_t *masks) {
  __shared__ __align__(16) float rows[kFeeWarps][kFeeRow];
  __shared__ FeeState fs[kFeeWarps];
  __shared__ float gint[kFeeWarps][LSIM_MAX_HITS];
  const int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  float *C = rows[wid];
  FeeState &st = fs[wid];
  if (lane == 0) st.mask = masks + (size_t)(blockIdx.x * kFeeWarps + wid) * kFeeMaskWords;
  __syncwarp();
  const int H = p.max_adc_values;
  const bool early_exit = normals == nullptr && p.threshold > 0.f;
  for (int64_t r = (int64_t)blockIdx.x * kFeeWarps + wid; r < n_pix; r += (int64_t)gridDim.x * kFeeWarps) {
    const float4 *s4 = reinterpret_cast<const float4 *>(wfs + r * (int64_t)T);
    float4 *c4 = reinterpret_cast<float4 *>(C);
    for (int i = lane; i < T / 4; i += kWarp) c4[i] = __ldg(s4 + i);
    __syncwarp();
    warp_cumsum_charge(C, T, p.t_sampling, lane);
    const float *nrm = normals ? normals + r * (1 + 3 * H) : nullptr;
    fee_forward(p, C, T, nrm, nullptr, nullptr, &st, nullptr, early_exit, lane);
    __syncwarp();
    if (lane < H) gint[wid][lane] = digitize_vjp(p, st.raw[lane], g_adc[r * H + lane]);
    __syncwarp();
    fee_backward(p, C, T, &st, gint[wid], lane);
    float4 *d4 = reinterpret_cast<float4 *>(g_wfs + r * (int64_t)T);
    for (int i = lane; i < T / 4; i += kWarp) d4[i] = c4[i];
    __syncwarp();
  }
}

constexpr int64_t kFeeVjpMaxWarps = 8192;

size_t fee_vjp_workspace_bytes(int64_t n_pix) {
  const int64_t warps = n_pix < kFeeVjpMaxWarps ? n_pix : kFeeVjpMaxWarps;
  const int64_t blocks = (warps + kFeeWarps - 1) / kFeeWarps;
  return (size_t)(blocks > 0 ? blocks : 1) * kFeeWarps * kFeeMaskWords * sizeof(uint32_t);
}

int run_fee_vjp(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals,
                const float *g_adc, float *g_wfs, void *ws, cudaStream_t st) {
  if (n_t > kFeeRow || n_t < 4 || n_t % 4 != 0 || p.max_adc_values > LSIM_MAX_HITS) return LSIM_ERR_UNSUPPORTED;
  if (n_pix <= 0) return LSIM_OK;
  const int64_t warps = n_pix < kFeeVjpMaxWarps ? n_pix : kFeeVjpMaxWarps;
  const int64_t blocks = (warps + kFeeWarps - 1) / kFeeWarps;
  k_fee_vjp<<<(unsigned)blocks, kFeeWarps * kWarp, 0, st>>>(p, wfs, n_pix, n_t, normals, g_adc, g_wfs,
                                                           static_cast<uint32_t *>(ws));
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

// ---------------------------------------------------------------- hits

struct PixelGeo {
  int px, py, plane, event;
};

// id2pixel (detsim_jax.py:264-278), Python floor semantics.
__device__ __forceinline__ PixelGeo id2pixel(const LsimParams &p, int32_t pid) {
  const int nx = p.n_pixels_x, ny = p.n_pixels_y, nt = p.n_tpc;
  PixelGeo g;
  g.px = imod(pid, nx);
  g.py = imod(ifloordiv(pid, nx), ny);
  g.plane = imod(ifloordiv(pid, nx * ny), nt);
  g.event = ifloordiv(pid, nx * ny * nt);
  return g;
}

constexpr int kHitTile = 1024;

__device__ __forceinline__ bool hit_keep(const LsimParams &p, const float *ticks, const int32_t *unique_pixels,
                                         int64_t i, int H, int tick_limit) {
  const int64_t r = i / H;
  const int32_t pid = unique_pixels[r];
  const float hp = ticks[i] < (float)tick_limit ? 1.f : 0.f;
  const PixelGeo g = id2pixel(p, pid);
  return hp > p.hit_prob_threshold && g.event >= 0 && pid >= 0;
}

__global__ void k_hits_count(LsimParams p, const float *ticks, const int32_t *unique_pixels, int64_t n, int H,
                             int tick_limit, int32_t *block_counts) {
  __shared__ int sh[kHitTile / kWarp];
  const int64_t base = (int64_t)blockIdx.x * kHitTile;
  const int64_t i = base + threadIdx.x;
  const bool keep = i < n && hit_keep(p, ticks, unique_pixels, i, H, tick_limit);
  const unsigned bal = __ballot_sync(0xffffffffu, keep);
  if (threadIdx.x % kWarp == 0) sh[threadIdx.x / kWarp] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kHitTile / kWarp; ++w) s += sh[w];
    block_counts[blockIdx.x] = s;
  }
}

// Exclusive scan of the per-tile kept counts, one CTA of kHitsScanThreads:
// each thread owns a contiguous run of tiles (scanned serially in
// registers), the run totals are scanned across the block, and each thread
// writes its run's offsets.  *total gets the kept count.
constexpr int kHitsScanThreads = 1024;
__global__ void __launch_bounds__(kHitsScanThreads) k_hits_scan(int32_t *block_counts, int64_t nblocks,
                                                                 int32_t *total) {
  __shared__ int64_t warp_tot[kHitsScanThreads / kWarp];
  __shared__ int64_t all;
  const int64_t per = (nblocks + kHitsScanThreads - 1) / kHitsScanThreads;
  const int64_t lo = min(nblocks, (int64_t)threadIdx.x * per), hi = min(nblocks, lo + per);
  int64_t run = 0;
  for (int64_t b = lo; b < hi; ++b) run += block_counts[b];
  const int64_t incl = block_scan_i64(run, warp_tot, &all);
  int64_t off = incl - run;
  for (int64_t b = lo; b < hi; ++b) {
    const int32_t c = block_counts[b];
    block_counts[b] = (int32_t)off;
    off += c;
  }
  if (threadIdx.x == 0) *total = (int32_t)all;
}

// Row-major compaction (parse_output) with the coordinates of
// get_pixel_coordinates / get_hit_z.  Pixel centres and hit z use the
// fused forms XLA compiles these expressions to:
//   x = fma(px, pitch, border_x) + pitch/2,   z = z_anode - tick * (t_sampling * vdrift)
// (z_anode + tick*ts*v*sign with sign folded); both match the reference's
// committed outputs bit for bit.
__global__ void k_hits_write(LsimParams p, const float *adc, const float *ticks, const int32_t *unique_pixels,
                             int64_t n, int H, int tick_limit, const int32_t *block_offsets, float *out_adc,
                             float *out_x, float *out_y, float *out_z, float *out_ticks, float *out_hp,
                             int32_t *out_event, int32_t *out_pixels) {
  __shared__ int sh[kHitTile / kWarp];
  const int64_t base = (int64_t)blockIdx.x * kHitTile;
  const int64_t i = base + threadIdx.x;
  const bool keep = i < n && hit_keep(p, ticks, unique_pixels, i, H, tick_limit);
  const unsigned bal = __ballot_sync(0xffffffffu, keep);
  const int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  if (lane == 0) sh[wid] = __popc(bal);
  __syncthreads();
  int wofs = 0;
  for (int w = 0; w < wid; ++w) wofs += sh[w];
  if (!keep) return;
  const int64_t o = block_offsets[blockIdx.x] + wofs + __popc(bal & ((1u << lane) - 1u));
  const int64_t r = i / H;
  const int32_t pid = unique_pixels[r];
  const PixelGeo g = id2pixel(p, pid);
  const float bx0 = border(p, g.plane, 0, 0), by0 = border(p, g.plane, 1, 0);
  const float za = border(p, g.plane, 2, 0), zh = border(p, g.plane, 2, 1);
  const float tk = ticks[i];
  const float tv = __fmul_rn(p.t_sampling, p.vdrift);
  const float dz = __fmul_rn(tk, tv);
  out_adc[o] = adc[i];
  out_x[o] = __fadd_rn(__fmaf_rn((float)g.px, p.pixel_pitch, bx0), p.half_pitch);
  out_y[o] = __fadd_rn(__fmaf_rn((float)g.py, p.pixel_pitch, by0), p.half_pitch);
  out_z[o] = (zh - za) < 0.f ? __fsub_rn(za, dz) : ((zh - za) > 0.f ? __fadd_rn(za, dz) : za);
  out_ticks[o] = tk;
  out_hp[o] = tk < (float)tick_limit ? 1.f : 0.f;
  out_event[o] = g.event;
  out_pixels[o] = pid;
}

// Per-pixel id2pixel + get_pixel_coordinates (detsim_jax.py:264-306), the
// same centre arithmetic as the hit compaction above.
__global__ void k_pixel_coords(LsimParams p, const int32_t *unique_pixels, int64_t n, float *x, float *y,
                               int32_t *plane, int32_t *event) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PixelGeo g = id2pixel(p, unique_pixels[i]);
  if (x) x[i] = __fadd_rn(__fmaf_rn((float)g.px, p.pixel_pitch, border(p, g.plane, 0, 0)), p.half_pitch);
  if (y) y[i] = __fadd_rn(__fmaf_rn((float)g.py, p.pixel_pitch, border(p, g.plane, 1, 0)), p.half_pitch);
  if (plane) plane[i] = g.plane;
  if (event) event[i] = g.event;
}

int run_pixel_coords(const LsimParams &p, const int32_t *unique_pixels, int64_t n, float *x, float *y,
                     int32_t *plane, int32_t *event, cudaStream_t st) {
  if (n <= 0) return LSIM_OK;
  k_pixel_coords<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, unique_pixels, n, x, y, plane, event);
  return LSIM_OK;
}

size_t hits_ws_bytes(int64_t n) { return align256(4 * (size_t)((n + kHitTile - 1) / kHitTile + 1)); }

int run_hits(const LsimParams &p, const float *adc, const float *ticks, const int32_t *unique_pixels, int64_t n_pix,
             int32_t tick_limit, float *out_adc, float *out_x, float *out_y, float *out_z, float *out_ticks,
             float *out_hit_prob, int32_t *out_event, int32_t *out_pixels, int32_t *nb_valid_dev, void *ws,
             cudaStream_t st) {
  const int H = p.max_adc_values;
  const int64_t n = n_pix * H;
  const int64_t nb = (n + kHitTile - 1) / kHitTile;
  int32_t *blocks = (int32_t *)ws;
  if (n == 0) return cudaMemsetAsync(nb_valid_dev, 0, 4, st) == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
  k_hits_count<<<(unsigned)nb, kHitTile, 0, st>>>(p, ticks, unique_pixels, n, H, tick_limit, blocks);
  k_hits_scan<<<1, kHitsScanThreads, 0, st>>>(blocks, nb, nb_valid_dev);
  k_hits_write<<<(unsigned)nb, kHitTile, 0, st>>>(p, adc, ticks, unique_pixels, n, H, tick_limit, blocks, out_adc,
                                                  out_x, out_y, out_z, out_ticks, out_hit_prob, out_event, out_pixels);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

// ---------------------------------------------------------------- hits without allocation

// Fixed scratch for lsim_hits_noalloc: one int per 1024 hit slots (the
// per-tile counts of the two-pass compaction).  64 KiB per CUDA context that
// loads this module (with lazy module loading: on the first use of any kernel
// of this file in that context), held until the context is destroyed.
constexpr int64_t kHitsStaticTiles = 16384;
static __device__ __align__(256) int32_t g_hits_static_scratch[kHitsStaticTiles];

// The array's device address belongs to the module as loaded in one CUDA
// context, so the lookup is cached per context, keyed by the context's
// process-unique id (cuCtxGetId): a context made with cuCtxCreate, or the
// primary context re-created after cudaDeviceReset, gets its own lookup.
// The two driver calls are fetched through the runtime, so the library does
// not link libcuda itself.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
constexpr int kMaxContexts = 64;
static std::mutex g_hits_static_mu;
static unsigned long long g_hits_ctx_id[kMaxContexts] = {};
static int32_t *g_hits_ctx_ptr[kMaxContexts] = {};
static int g_hits_ctx_n = 0;

static int current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    void *f1 = nullptr, *f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return LSIM_ERR_CUDA;
    get_current = (CtxGetCurrentFn)f1;
    get_id = (CtxGetIdFn)f2;
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return LSIM_ERR_CUDA;
  if (!ctx) {
    // no context current yet on this thread: make the current device's
    // primary context current, as the runtime's first call would
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return LSIM_ERR_CUDA;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return LSIM_ERR_CUDA;
  }
  return get_id(ctx, id) == CUDA_SUCCESS ? LSIM_OK : LSIM_ERR_CUDA;
}

// Device address of g_hits_static_scratch in the current context: looked
// up once per context (cudaGetSymbolAddress with that context current).
static int hits_static_scratch(int32_t **out) {
  unsigned long long id = 0;
  std::lock_guard<std::mutex> lock(g_hits_static_mu);
  if (current_context_id(&id) != LSIM_OK) return LSIM_ERR_CUDA;
  for (int i = 0; i < g_hits_ctx_n; ++i)
    if (g_hits_ctx_id[i] == id) {
      *out = g_hits_ctx_ptr[i];
      return LSIM_OK;
    }
  void *ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_hits_static_scratch) != cudaSuccess || !ptr) return LSIM_ERR_CUDA;
  // a full table starts over (a process that made more than kMaxContexts
  // contexts); entries are only a cache of the lookup
  if (g_hits_ctx_n == kMaxContexts) g_hits_ctx_n = 0;
  g_hits_ctx_id[g_hits_ctx_n] = id;
  g_hits_ctx_ptr[g_hits_ctx_n] = (int32_t *)ptr;
  ++g_hits_ctx_n;
  *out = (int32_t *)ptr;
  return LSIM_OK;
}

// ---------------------------------------------------------------- parametrised current

// 0.5*erf((x-loc)/(sqrt2*diff)) - emg_pdf(x, loc, diff, lambd)/lambd
// (integrated_expon_diff's per-edge term, detsim_jax.py:467-468).
__device__ __forceinline__ float ied_edge(float x, float loc, float diff, float lambd) {
  const float s2 = 1.41421356237309515f;
  const float e = 0.5f * erff((x - loc) / (s2 * diff));
  const float coeff = lambd / 2.f;
  const float ls2 = lambd * (diff * diff);
  const float expo = coeff * (((2.f * loc) + ls2) - (2.f * x));
  const float pdf = (coeff * expf(expo)) * erfcf(((loc + ls2) - x) / (s2 * diff));
  return e - pdf / lambd;
}

__device__ __forceinline__ float quad(const float c[6], float x, float y) {
  return ((((c[0] + c[1] * x) + c[2] * y) + (c[3] * x) * y) + (c[4] * x) * x) + (c[5] * y) * y;
}

// current_model_diff (detsim_jax.py:581-615) at tick k of the 51-tick grid,
// times n_e (current_mc, detsim_jax.py:637).
struct ParamShape {
  float a, lam_b, lam_c, loc, diff, norm_b, norm_c;
};

__device__ __forceinline__ ParamShape param_shape(const LsimParams &p, const SegPar &s) {
  const float B[6] = {1.060f, -0.909f, -0.909f, 5.856f, 0.207f, 0.207f};
  const float C[6] = {0.679f, -1.083f, -1.083f, 8.772f, -5.521f, -5.521f};
  const float D[6] = {2.644f, -9.174f, -9.174f, 13.483f, 45.887f, 45.887f};
  const float T0[6] = {2.948f, -2.705f, -2.705f, 4.825f, 20.814f, 20.814f};
  ParamShape sh;
  const float x = s.xd, y = s.yd;
  sh.a = fminf(quad(B, x, y), 1.f);
  const float b = quad(C, x, y), c = quad(D, x, y);
  const float st0 = s.t0f + T0[0] + T0[1] * x + T0[2] * y + (T0[3] * x) * y + (T0[4] * x) * x + (T0[5] * y) * y;
  sh.loc = -st0;
  sh.diff = s.sigma;
  sh.lam_b = 1.f / b;
  sh.lam_c = 1.f / c;
  const int n = p.param_nticks;
  const float hd = p.param_dt * 0.5f;
  // normalisation: lower edge of the first tick minus upper edge of the last
  const float x0 = -p.param_ticks[0], xl = -p.param_ticks[n - 1];
  sh.norm_b = ied_edge(x0 - hd, sh.loc, sh.diff, sh.lam_b) - ied_edge(xl + hd, sh.loc, sh.diff, sh.lam_b);
  sh.norm_c = ied_edge(x0 - hd, sh.loc, sh.diff, sh.lam_c) - ied_edge(xl + hd, sh.loc, sh.diff, sh.lam_c);
  return sh;
}

__device__ __forceinline__ float param_value(const LsimParams &p, const ParamShape &sh, int k) {
  const float x = -p.param_ticks[k];
  const float hd = p.param_dt * 0.5f;
  const float ub = ied_edge(x + hd, sh.loc, sh.diff, sh.lam_b), lb = ied_edge(x - hd, sh.loc, sh.diff, sh.lam_b);
  const float uc = ied_edge(x + hd, sh.loc, sh.diff, sh.lam_c), lc = ied_edge(x - hd, sh.loc, sh.diff, sh.lam_c);
  const float vb = ((ub - lb) / sh.norm_b) / p.param_dt;
  const float vc = ((uc - lc) / sh.norm_c) / p.param_dt;
  return sh.a * vb + (1.f - sh.a) * vc;
}

constexpr int kParWarps = 4;

__global__ void __launch_bounds__(kParWarps * kWarp)
    k_param_pixels(LsimParams p, Workspace w, Grid g, int64_t row_offset, float *wfs) {
  __shared__ __align__(16) float rows[kParWarps][2052];
  const int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  float *row = rows[wid] + 3;   // col 1 16-byte aligned
  const int NT = p.n_ticks, T = NT - 1;
  const int n = p.param_nticks;
  const int n_valid = w.counts->n_valid;
  for (;;) {
    int r = 0;
    if (lane == 0) r = atomicAdd(&w.counts->work, 1);
    r = __shfl_sync(0xffffffffu, r, 0);
    if (r >= n_valid) break;
    const int64_t slot = w.pix_slot[r];
    float4 *b4 = reinterpret_cast<float4 *>(rows[wid]);
    for (int i = lane; i < 2052 / 4; i += kWarp) b4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    const int c = w.cnt[slot], o = w.off[slot];
    for (int j = 0; j < c; ++j) {
      const int s = w.seg_list[o + j];
      const SegPar sp = w.segp[s];
      if (sp.ne == 0.f) continue;
      const ParamShape sh = param_shape(p, sp);
      const int start = sp.t0_tick - n;
      for (int k = lane; k < n; k += kWarp) {
        const float v = param_value(p, sh, k) * sp.ne;
        const int tt = start + k;
        if (tt >= 0 && tt < NT - 1) row[tt + 1] += v;   // accumulate_signals_parametrized remap
      }
      __syncwarp();
    }
    float4 *dst = reinterpret_cast<float4 *>(wfs + (row_offset + r) * (int64_t)T);
    const float4 *src = reinterpret_cast<const float4 *>(row + 1);
    for (int i = lane; i < T / 4; i += kWarp) dst[i] = src[i];
    __syncwarp();
  }
}

// ---------------------------------------------------------------- parametrised adjoint
// Forward-mode derivatives of the current model with respect to its four
// continuous inputs (x_dist, y_dist, t0f, sigma), carried as dual numbers
// through the same expressions as the forward (so the window
// normalisation, which couples all 51 ticks, is differentiated exactly).

struct Dual {
  float v, d[4];
};

__device__ __forceinline__ Dual dconst(float c) { return Dual{c, {0.f, 0.f, 0.f, 0.f}}; }
__device__ __forceinline__ Dual dseed(float c, int i) {
  Dual r = dconst(c);
  r.d[i] = 1.f;
  return r;
}
__device__ __forceinline__ Dual operator+(const Dual &a, const Dual &b) {
  return Dual{a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2], a.d[3] + b.d[3]}};
}
__device__ __forceinline__ Dual operator-(const Dual &a, const Dual &b) {
  return Dual{a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2], a.d[3] - b.d[3]}};
}
__device__ __forceinline__ Dual operator*(const Dual &a, const Dual &b) {
  Dual r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
__device__ __forceinline__ Dual operator*(float c, const Dual &a) {
  return Dual{c * a.v, {c * a.d[0], c * a.d[1], c * a.d[2], c * a.d[3]}};
}
__device__ __forceinline__ Dual operator/(const Dual &a, const Dual &b) {
  Dual r;
  r.v = a.v / b.v;
  const float ib = 1.f / b.v;
#pragma unroll
  for (int i = 0; i < 4; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
__device__ __forceinline__ Dual chain(float v, float dv, const Dual &a) {
  return Dual{v, {dv * a.d[0], dv * a.d[1], dv * a.d[2], dv * a.d[3]}};
}
__device__ __forceinline__ Dual dexp(const Dual &a) {
  const float e = expf(a.v);
  return chain(e, e, a);
}
// erf' = 2/sqrt(pi) exp(-x^2), erfc' = -erf'
__device__ __forceinline__ Dual derf(const Dual &a) {
  return chain(erff(a.v), 1.12837916709551257f * expf(-a.v * a.v), a);
}
__device__ __forceinline__ Dual derfc(const Dual &a) {
  return chain(erfcf(a.v), -1.12837916709551257f * expf(-a.v * a.v), a);
}

__device__ __forceinline__ Dual ied_edge_d(float x, const Dual &loc, const Dual &diff, const Dual &lambd) {
  const float s2 = 1.41421356237309515f;
  const Dual sd = s2 * diff;
  const Dual e = 0.5f * derf((dconst(x) - loc) / sd);
  const Dual coeff = 0.5f * lambd;
  const Dual ls2 = lambd * (diff * diff);
  const Dual expo = coeff * (((2.f * loc) + ls2) - dconst(2.f * x));
  const Dual pdf = (coeff * dexp(expo)) * derfc(((loc + ls2) - dconst(x)) / sd);
  return e - pdf / lambd;
}

__device__ __forceinline__ Dual quad_d(const float c[6], const Dual &x, const Dual &y) {
  return ((((dconst(c[0]) + c[1] * x) + c[2] * y) + (c[3] * x) * y) + (c[4] * x) * x) + (c[5] * y) * y;
}

struct ParamShapeD {
  Dual a, lam_b, lam_c, loc, diff, norm_b, norm_c;
};

__device__ __forceinline__ ParamShapeD param_shape_d(const LsimParams &p, const SegPar &s) {
  const float B[6] = {1.060f, -0.909f, -0.909f, 5.856f, 0.207f, 0.207f};
  const float C[6] = {0.679f, -1.083f, -1.083f, 8.772f, -5.521f, -5.521f};
  const float D[6] = {2.644f, -9.174f, -9.174f, 13.483f, 45.887f, 45.887f};
  const float T0[6] = {2.948f, -2.705f, -2.705f, 4.825f, 20.814f, 20.814f};
  const Dual x = dseed(s.xd, 0), y = dseed(s.yd, 1), t0f = dseed(s.t0f, 2);
  ParamShapeD sh;
  Dual a = quad_d(B, x, y);
  // jnp.minimum(a, 1): the derivative passes below 1, half of it at a tie
  if (a.v > 1.f) a = dconst(1.f);
  else if (a.v == 1.f) a = Dual{1.f, {0.5f * a.d[0], 0.5f * a.d[1], 0.5f * a.d[2], 0.5f * a.d[3]}};
  sh.a = a;
  const Dual b = quad_d(C, x, y), c = quad_d(D, x, y);
  const Dual st0 = t0f + quad_d(T0, x, y);
  sh.loc = dconst(0.f) - st0;
  sh.diff = dseed(s.sigma, 3);
  sh.lam_b = dconst(1.f) / b;
  sh.lam_c = dconst(1.f) / c;
  const int n = p.param_nticks;
  const float hd = p.param_dt * 0.5f;
  const float x0 = -p.param_ticks[0], xl = -p.param_ticks[n - 1];
  sh.norm_b = ied_edge_d(x0 - hd, sh.loc, sh.diff, sh.lam_b) - ied_edge_d(xl + hd, sh.loc, sh.diff, sh.lam_b);
  sh.norm_c = ied_edge_d(x0 - hd, sh.loc, sh.diff, sh.lam_c) - ied_edge_d(xl + hd, sh.loc, sh.diff, sh.lam_c);
  return sh;
}

__device__ __forceinline__ Dual param_value_d(const LsimParams &p, const ParamShapeD &sh, int k) {
  const float x = -p.param_ticks[k];
  const float hd = p.param_dt * 0.5f;
  const float idt = 1.f / p.param_dt;
  const Dual ub = ied_edge_d(x + hd, sh.loc, sh.diff, sh.lam_b), lb = ied_edge_d(x - hd, sh.loc, sh.diff, sh.lam_b);
  const Dual uc = ied_edge_d(x + hd, sh.loc, sh.diff, sh.lam_c), lc = ied_edge_d(x - hd, sh.loc, sh.diff, sh.lam_c);
  const Dual vb = idt * ((ub - lb) / sh.norm_b);
  const Dual vc = idt * ((uc - lc) / sh.norm_c);
  return sh.a * vb + (dconst(1.f) - sh.a) * vc;
}

// dL/dtheta per pixel for a waveform cotangent g_wfs (rows as stage 2
// writes them): per segment the cotangent of its 51 current samples,
// folded into d/d(ne, x_dist, y_dist, t0f, sigma) and projected through the
// segment's SegParAdj record.
__global__ void __launch_bounds__(kParWarps * kWarp)
    k_param_vjp(LsimParams p, Workspace w, Grid g, int64_t row_offset, const float *__restrict__ g_wfs) {
  __shared__ __align__(16) float rows[kParWarps][2052];
  const int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  float *row = rows[wid] + 3;   // col 1 16-byte aligned
  const int NT = p.n_ticks, T = NT - 1;
  const int n = p.param_nticks;
  const int n_valid = w.counts->n_valid;
  for (;;) {
    int r = 0;
    if (lane == 0) r = atomicAdd(&w.counts->work, 1);
    r = __shfl_sync(0xffffffffu, r, 0);
    if (r >= n_valid) break;
    const int64_t slot = w.pix_slot[r];
    const float4 *src = reinterpret_cast<const float4 *>(g_wfs + (row_offset + r) * (int64_t)T);
    float4 *dst = reinterpret_cast<float4 *>(row + 1);
    for (int i = lane; i < T / 4; i += kWarp) dst[i] = __ldg(src + i);
    if (lane == 0) row[0] = 0.f;   // the garbage column carries no gradient
    __syncwarp();
    float th[LSIM_NPARAM];
#pragma unroll
    for (int i = 0; i < LSIM_NPARAM; ++i) th[i] = 0.f;
    const int c = w.cnt[slot], o = w.off[slot];
    for (int j = 0; j < c; ++j) {
      const int s = w.seg_list[o + j];
      const SegPar sp = w.segp[s];
      if (sp.ne == 0.f) continue;
      const ParamShapeD sh = param_shape_d(p, sp);
      const int start = sp.t0_tick - n;
      float gne = 0.f, gq[4] = {0.f, 0.f, 0.f, 0.f};
      for (int k = lane; k < n; k += kWarp) {
        const int tt = start + k;
        const float gk = (tt >= 0 && tt < NT - 1) ? row[tt + 1] : 0.f;
        if (gk != 0.f) {
          const Dual v = param_value_d(p, sh, k);
          gne += gk * v.v;
#pragma unroll
          for (int q = 0; q < 4; ++q) gq[q] += gk * sp.ne * v.d[q];
        }
      }
      gne = warp_sum(gne);
#pragma unroll
      for (int q = 0; q < 4; ++q) gq[q] = warp_sum(gq[q]);
      const SegParAdj ja = *reinterpret_cast<const SegParAdj *>(w.sega + s);
      // order: Ab kb eField lifetime vdrift long_diff tran_diff lArDensity
      th[0] += gne * ja.dne[0];
      th[1] += gne * ja.dne[1];
      th[2] += gne * ja.dne[2] + gq[0] * ja.dxd[0] + gq[1] * ja.dyd[0] + gq[2] * ja.dt0f[0] + gq[3] * ja.dsig[0];
      th[3] += gne * ja.dne[3];
      th[5] += gq[2] * ja.dt0f[1] + gq[3] * ja.dsig[1];
      th[6] += gq[0] * ja.dxd[1] + gq[1] * ja.dyd[1];
      th[7] += gne * ja.dne[4];
    }
    if (lane == 0) {
      float *out = w.pix_out + (size_t)r * kPixRec;
      out[0] = 0.f;
#pragma unroll
      for (int i = 0; i < LSIM_NPARAM; ++i) out[1 + i] = th[i];
    }
    __syncwarp();
  }
}

int run_param_vjp(const LsimParams &p, const Workspace &w, const Grid &g, int32_t n_valid, int64_t row_offset,
                  const float *g_wfs, int64_t n_rows, cudaStream_t st) {
  if (p.n_ticks - 1 > 2048 || (p.n_ticks - 1) % 4 != 0 || p.param_nticks > 64) return LSIM_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(&w.counts->work, 0, sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  // no main-bin records in this mode: their adjoint partials are zero
  if (n_rows > 0 && cudaMemsetAsync(w.main_out, 0, sizeof(float) * kPixRec * (size_t)n_rows, st) != cudaSuccess)
    return LSIM_ERR_CUDA;
  int blocks = device_sm_count() * 4;
  k_param_vjp<<<blocks, kParWarps * kWarp, 0, st>>>(p, w, g, row_offset, g_wfs);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

int run_param_accum(const LsimParams &p, const Workspace &w, const Grid &g, int32_t n_valid, int64_t row_offset,
                    float *wfs, cudaStream_t st) {
  if (p.n_ticks - 1 > 2048 || (p.n_ticks - 1) % 4 != 0 || p.param_nticks > 64) return LSIM_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(&w.counts->work, 0, sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  int blocks = device_sm_count() * 4;
  k_param_pixels<<<blocks, kParWarps * kWarp, 0, st>>>(p, w, g, row_offset, wfs);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim

extern "C" int64_t lsim_hits_noalloc_max_slots(void) { return lsim::kHitsStaticTiles * (int64_t)lsim::kHitTile; }

extern "C" int lsim_hits_noalloc(const LsimParams *p, const float *adc, const float *ticks,
                                 const int32_t *unique_pixels, int64_t n_pix, int32_t tick_limit, float *out_adc,
                                 float *out_x, float *out_y, float *out_z, float *out_ticks, float *out_hit_prob,
                                 int32_t *out_event, int32_t *out_pixels, int32_t *nb_valid_dev, void *stream) {
  using namespace lsim;
  clear_error();
  if (!p) return set_error(LSIM_ERR_INVALID, "lsim_hits_noalloc: null parameter block");
  if (!nb_valid_dev || (n_pix > 0 && (!adc || !ticks || !unique_pixels || !out_adc || !out_x || !out_y || !out_z ||
                                      !out_ticks || !out_hit_prob || !out_event || !out_pixels)))
    return set_error(LSIM_ERR_INVALID, "lsim_hits_noalloc: null pointer");
  if (n_pix < 0) return set_error(LSIM_ERR_INVALID, "lsim_hits_noalloc: negative pixel count");
  if (p->max_adc_values < 1 || p->max_adc_values > LSIM_MAX_HITS)
    return set_error(LSIM_ERR_INVALID, "lsim_hits_noalloc: max_adc_values outside 1..LSIM_MAX_HITS");
  // compare before multiplying, so a huge pixel count cannot wrap past the limit
  const int64_t max_slots = kHitsStaticTiles * (int64_t)kHitTile;
  const int64_t slots = n_pix > max_slots / p->max_adc_values ? max_slots + 1 : n_pix * (int64_t)p->max_adc_values;
  if (slots > max_slots) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "lsim_hits_noalloc: %lld hit slots (%lld pixels x %d hits) exceed the fixed scratch limit of %lld "
             "slots; use lsim_hits with a caller-allocated workspace",
             (long long)n_pix * p->max_adc_values, (long long)n_pix, p->max_adc_values, (long long)max_slots);
    return set_error(LSIM_ERR_CAPACITY, msg);
  }
  int32_t *scratch = nullptr;
  if (hits_static_scratch(&scratch) != LSIM_OK)
    return set_error(LSIM_ERR_CUDA, "lsim_hits_noalloc: cannot resolve the device address of the fixed scratch");
  int rc = run_hits(*p, adc, ticks, unique_pixels, n_pix, tick_limit, out_adc, out_x, out_y, out_z, out_ticks,
                    out_hit_prob, out_event, out_pixels, nb_valid_dev, scratch, (cudaStream_t)stream);
  if (rc != LSIM_OK) {
    cudaError_t e = cudaGetLastError();
    char msg[256];
    snprintf(msg, sizeof(msg), "lsim_hits_noalloc: CUDA error %s", cudaGetErrorString(e));
    return set_error(rc, msg);
  }
  return LSIM_OK;
}
