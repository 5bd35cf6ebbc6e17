// extern "C" entry points of liblsim (declared in include/lsim.h).  Each
// validates its arguments, launches on the caller's stream, converts CUDA
// errors into LSIM_* codes with a thread-local message, and never throws.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "lsim_internal.cuh"

namespace lsim {

static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int set_error(int code, const char *msg) {
  g_err = msg;
  return code;
}

void clear_error() { g_err.clear(); }

static int check_cuda(const char *where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(LSIM_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
  return LSIM_OK;
}

static int wrap(int rc, const char *where) {
  if (rc == LSIM_OK) return check_cuda(where);
  if (rc == LSIM_ERR_CUDA) {
    cudaError_t e = cudaGetLastError();
    return fail(rc, "%s: CUDA error %s", where, cudaGetErrorString(e));
  }
  if (g_err.empty()) fail(rc, "%s: error %d", where, rc);
  return rc;
}

int device_sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

static int check_params(const LsimParams *p) {
  if (!p) return fail(LSIM_ERR_INVALID, "null parameter block");
  if (p->n_tpc < 1 || p->n_tpc > LSIM_MAX_TPC) return fail(LSIM_ERR_UNSUPPORTED, "n_tpc %d not in [1, %d]", p->n_tpc, LSIM_MAX_TPC);
  if (p->n_templates > LSIM_MAX_TEMPLATES) return fail(LSIM_ERR_UNSUPPORTED, "%d templates > %d", p->n_templates, LSIM_MAX_TEMPLATES);
  if (p->max_adc_values < 1 || p->max_adc_values > LSIM_MAX_HITS)
    return fail(LSIM_ERR_UNSUPPORTED, "MAX_ADC_VALUES %d not in [1, %d]", p->max_adc_values, LSIM_MAX_HITS);
  if (p->n_neighbors < 0 || p->n_neighbors > 4) return fail(LSIM_ERR_UNSUPPORTED, "number_pix_neighbors %d not in [0, 4]", p->n_neighbors);
  if (p->n_pixels_x <= 0 || p->n_pixels_y <= 0 || p->nb_bins_per_pixel <= 0) return fail(LSIM_ERR_INVALID, "bad pixel geometry");
  if (p->n_ticks < 4 || p->n_ticks - 1 > 2048 || (p->n_ticks - 1) % 4 != 0)
    return fail(LSIM_ERR_UNSUPPORTED, "n_ticks %d: waveform length must be a multiple of 4 up to 2048", p->n_ticks);
  return LSIM_OK;
}

static int check_fields(const LsimFieldMap *f) {
  if (!f) return fail(LSIM_ERR_INVALID, "null field map");
  const int32_t cols[] = {f->eventID, f->x, f->y, f->z, f->x_start, f->y_start, f->z_start,
                          f->x_end, f->y_end, f->z_end, f->dx, f->dE, f->dEdx};
  for (int32_t c : cols)
    if (c < 0 || c >= f->n_fields) return fail(LSIM_ERR_INVALID, "field index %d outside [0, %d)", c, f->n_fields);
  return LSIM_OK;
}

static thread_local cudaEvent_t g_ev_start = nullptr, g_ev_stop = nullptr;
void kernel_events(cudaEvent_t *start, cudaEvent_t *stop) {
  *start = g_ev_start;
  *stop = g_ev_stop;
}

static thread_local LsimTuning g_tuning = {0, 0, 0, {0, 0, 0, 0, 0}};
LsimTuning tuning() { return g_tuning; }

}  // namespace lsim

using namespace lsim;

extern "C" {

int lsim_abi_version(void) { return LSIM_ABI_VERSION; }

void lsim_set_tuning(const LsimTuning *t) {
  if (t) {
    lsim::g_tuning = *t;
  } else {
    lsim::g_tuning = LsimTuning{0, 0, 0, {0, 0, 0, 0, 0}};
  }
}

void lsim_set_kernel_events(void *start, void *stop) {
  const bool on = start != nullptr && stop != nullptr;
  lsim::g_ev_start = on ? (cudaEvent_t)start : nullptr;
  lsim::g_ev_stop = on ? (cudaEvent_t)stop : nullptr;
}

const char *lsim_last_error(void) { return g_err.c_str(); }

void lsim_struct_sizes(size_t *params, size_t *fields, size_t *counts) {
  if (params) *params = sizeof(LsimParams);
  if (fields) *fields = sizeof(LsimFieldMap);
  if (counts) *counts = sizeof(LsimCounts);
}

int lsim_lut_build_templates(const float *response, int32_t nx, int32_t ny, int32_t nt, const float *sigmas_dev,
                             int32_t n_templates, int32_t extent, float *templates_out, void *stream) {
  g_err.clear();
  if (!response || !sigmas_dev || !templates_out || nx <= 0 || ny <= 0 || nt <= 0 || extent < 0)
    return fail(LSIM_ERR_INVALID, "lsim_lut_build_templates: bad arguments");
  return wrap(run_build_templates(response, nx, ny, nt, sigmas_dev, n_templates, extent, templates_out,
                                  (cudaStream_t)stream),
              "lsim_lut_build_templates");
}

size_t lsim_lut_tables_bytes(const LsimParams *p) {
  if (!p) return 0;
  size_t a, b, c, d;
  return tables_layout(*p, &a, &b, &c, &d);
}

int lsim_lut_prepare(const LsimParams *p, const float *templates, void *tables, size_t tables_bytes, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!templates || !tables) return fail(LSIM_ERR_INVALID, "lsim_lut_prepare: null pointer");
  if (tables_bytes < lsim_lut_tables_bytes(p))
    return fail(LSIM_ERR_CAPACITY, "lsim_lut_prepare: tables buffer %zu < %zu bytes", tables_bytes,
                lsim_lut_tables_bytes(p));
  return wrap(run_prepare_tables(*p, templates, tables, (cudaStream_t)stream), "lsim_lut_prepare");
}

size_t lsim_workspace_bytes(const LsimParams *p, int64_t n_rows, int32_t n_events) {
  if (!p || n_rows < 0 || n_events < 0) return 0;
  return carve_workspace(nullptr, *p, n_rows, n_events).bytes;
}

static int stage1(bool param_mode, const LsimParams *p, const LsimFieldMap *f, const float *tracks, int64_t n_rows,
                  int32_t n_events, const float *normals, void *ws, size_t ws_bytes, LsimCounts *counts_dev,
                  void *stream, const char *name, const float *theta_dev = nullptr) {
  g_err.clear();
  int rc = check_params(p);
  if (!rc) rc = check_fields(f);
  if (rc) return rc;
  if (param_mode && p->n_neighbors != 0)
    return fail(LSIM_ERR_UNSUPPORTED, "%s: parametrised mode requires number_pix_neighbors == 0", name);
  if (n_rows < 0 || n_rows > 0x7fffffff || n_events < 0) return fail(LSIM_ERR_INVALID, "%s: bad sizes", name);
  if ((n_rows > 0 && !tracks) || !ws) return fail(LSIM_ERR_INVALID, "%s: null pointer", name);
  Workspace w = carve_workspace(ws, *p, n_rows, n_events);
  if (ws_bytes < w.bytes) return fail(LSIM_ERR_CAPACITY, "%s: workspace %zu < %zu bytes", name, ws_bytes, w.bytes);
  Grid g = make_grid(*p, n_events);
  if (g.G > 0x7fffffff) return fail(LSIM_ERR_CAPACITY, "%s: pixel grid of %lld slots exceeds int32", name, (long long)g.G);
  cudaStream_t st = (cudaStream_t)stream;
  rc = run_stage1(param_mode, *p, *f, tracks, normals, n_rows, n_events, w, st, theta_dev);
  if (rc) return wrap(rc, name);
  if (counts_dev && cudaMemcpyAsync(counts_dev, w.counts, sizeof(LsimCounts), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return check_cuda(name);
  return check_cuda(name);
}

int lsim_lut_stage1(const LsimParams *p, const LsimFieldMap *f, const float *tracks, int64_t n_rows, int32_t n_events,
                    void *ws, size_t ws_bytes, LsimCounts *counts_dev, void *stream) {
  return stage1(false, p, f, tracks, n_rows, n_events, nullptr, ws, ws_bytes, counts_dev, stream, "lsim_lut_stage1");
}

int lsim_lut_stage1_theta(const LsimParams *p, const LsimFieldMap *f, const float *tracks, int64_t n_rows,
                          int32_t n_events, const float *theta_dev, void *ws, size_t ws_bytes,
                          LsimCounts *counts_dev, void *stream) {
  if (!theta_dev) {
    g_err.clear();
    return fail(LSIM_ERR_INVALID, "lsim_lut_stage1_theta: null theta");
  }
  return stage1(false, p, f, tracks, n_rows, n_events, nullptr, ws, ws_bytes, counts_dev, stream,
                "lsim_lut_stage1_theta", theta_dev);
}

int lsim_adam_step(float *theta_dev, const float *grad_dev, const float *scale_dev, const float *lr_dev,
                   float *state_dev, float beta1, float beta2, float eps, void *stream) {
  g_err.clear();
  if (!theta_dev || !grad_dev || !scale_dev || !lr_dev || !state_dev)
    return fail(LSIM_ERR_INVALID, "lsim_adam_step: null pointer");
  return wrap(run_adam(theta_dev, grad_dev, scale_dev, lr_dev, state_dev, beta1, beta2, eps, (cudaStream_t)stream),
              "lsim_adam_step");
}

static int check_fit_options(const LsimFitOptions *o, const char *who) {
  if (!o) return fail(LSIM_ERR_INVALID, "%s: null options", who);
  if (o->scheme < LSIM_NORM_SIGMOID || o->scheme > LSIM_NORM_DIVIDE)
    return fail(LSIM_ERR_INVALID, "%s: unknown normalization scheme %d", who, o->scheme);
  if (!(o->norm_scale > 0.f)) return fail(LSIM_ERR_INVALID, "%s: normalization scale must be > 0", who);
  for (int i = 0; i < LSIM_NPARAM; ++i) {
    if (!((o->fit_mask >> i) & 1)) continue;
    if (o->scheme == LSIM_NORM_EXP_LOG && !(o->nom[i] > 0.f))
      return fail(LSIM_ERR_INVALID, "%s: exp_log normalization requires a positive nominal value (parameter %d)",
                  who, i);
    if (o->scheme == LSIM_NORM_SIGMOID && !(o->hi[i] > o->lo[i]))
      return fail(LSIM_ERR_INVALID, "%s: sigmoid normalization requires max > min (parameter %d)", who, i);
    if (o->scheme == LSIM_NORM_DIVIDE && o->clip_from_range && o->norm[i] == 0.f)
      return fail(LSIM_ERR_INVALID, "%s: clip_from_range with a zero normalization (parameter %d)", who, i);
  }
  return LSIM_OK;
}

int lsim_fit_init(float *theta_dev, const LsimFitOptions *opt, float *state_dev, void *stream) {
  g_err.clear();
  int rc = check_fit_options(opt, "lsim_fit_init");
  if (rc) return rc;
  if (!theta_dev || !state_dev) return fail(LSIM_ERR_INVALID, "lsim_fit_init: null pointer");
  return wrap(run_fit_init(theta_dev, *opt, state_dev, (cudaStream_t)stream), "lsim_fit_init");
}

int lsim_fit_step(float *theta_dev, const float *grad_dev, const LsimFitOptions *opt, float *state_dev,
                  void *stream) {
  g_err.clear();
  int rc = check_fit_options(opt, "lsim_fit_step");
  if (rc) return rc;
  if (!theta_dev || !grad_dev || !state_dev) return fail(LSIM_ERR_INVALID, "lsim_fit_step: null pointer");
  return wrap(run_fit_step(theta_dev, grad_dev, *opt, state_dev, (cudaStream_t)stream), "lsim_fit_step");
}

int lsim_param_stage1(const LsimParams *p, const LsimFieldMap *f, const float *tracks, int64_t n_rows,
                      int32_t n_events, const float *normals, void *ws, size_t ws_bytes, LsimCounts *counts_dev,
                      void *stream) {
  g_err.clear();
  if (p && !p->diffusion_in_current_sim)
    return fail(LSIM_ERR_UNSUPPORTED, "lsim_param_stage1: diffusion_in_current_sim = false (current_model without "
                                      "longitudinal smearing) is not implemented");
  return stage1(true, p, f, tracks, n_rows, n_events, normals, ws, ws_bytes, counts_dev, stream, "lsim_param_stage1");
}

static AccumArgs make_args(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events) {
  AccumArgs a;
  memset(&a, 0, sizeof(a));
  a.p = *p;
  if (tables) a.tab = carve_tables(tables, *p);
  a.w = carve_workspace(const_cast<void *>(ws), *p, n_rows, n_events);
  a.g = make_grid(*p, n_events);
  a.n_rows = n_rows;
  return a;
}

int lsim_lut_stage2(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events,
                    int64_t p_pad, int32_t n_em1, int32_t n_valid, float *wfs, int32_t *unique_pixels, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!tables || !ws || (p_pad > 0 && (!wfs || !unique_pixels))) return fail(LSIM_ERR_INVALID, "lsim_lut_stage2: null pointer");
  if (n_em1 < 0 || n_valid < 0 || (int64_t)n_em1 + n_valid > p_pad)
    return fail(LSIM_ERR_CAPACITY, "lsim_lut_stage2: p_pad %lld < %d + %d rows", (long long)p_pad, n_em1, n_valid);
  cudaStream_t st = (cudaStream_t)stream;
  AccumArgs a = make_args(p, tables, ws, n_rows, n_events);
  rc = run_fill_unique(*p, a.w, a.g, p_pad, n_em1, n_valid, unique_pixels, wfs, p->n_ticks - 1, st);
  if (rc) return wrap(rc, "lsim_lut_stage2");
  a.n_valid = n_valid;
  a.row_offset = p_pad - n_valid;
  a.wfs = wfs;
  return wrap(run_accum(kModeWfs, a, st), "lsim_lut_stage2");
}

int lsim_valid_pixels(const LsimParams *p, const void *ws, int64_t n_rows, int32_t n_events, int32_t n_valid,
                      int32_t *pids_out, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!ws || (n_valid > 0 && !pids_out)) return fail(LSIM_ERR_INVALID, "lsim_valid_pixels: null pointer");
  AccumArgs a = make_args(p, nullptr, ws, n_rows, n_events);
  return wrap(run_fill_unique(*p, a.w, a.g, n_valid, 0, n_valid, pids_out, nullptr, 0, (cudaStream_t)stream),
              "lsim_valid_pixels");
}

int lsim_lut_adc(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events,
                 int32_t n_valid, const float *normals, float *adc_out, float *tick_out, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!tables || !ws || !adc_out || !tick_out) return fail(LSIM_ERR_INVALID, "lsim_lut_adc: null pointer");
  AccumArgs a = make_args(p, tables, ws, n_rows, n_events);
  a.n_valid = n_valid;
  a.normals = normals;
  a.adc_out = adc_out;
  a.tick_out = tick_out;
  return wrap(run_accum(kModeAdc, a, (cudaStream_t)stream), "lsim_lut_adc");
}

int lsim_lut_grad(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events,
                  int32_t n_valid, const float *normals, const float *g_adc, const int32_t *tgt_pids,
                  const float *tgt_adc, int64_t n_tgt, float *loss_out, float *grad_out, float *adc_out, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!tables || !ws || !grad_out) return fail(LSIM_ERR_INVALID, "lsim_lut_grad: null pointer");
  if (!g_adc && n_tgt > 0 && (!tgt_pids || !tgt_adc)) return fail(LSIM_ERR_INVALID, "lsim_lut_grad: null target");
  cudaStream_t st = (cudaStream_t)stream;
  AccumArgs a = make_args(p, tables, ws, n_rows, n_events);
  a.n_valid = n_valid;
  a.normals = normals;
  a.g_adc = g_adc;
  a.tgt_pids = tgt_pids;
  a.tgt_adc = tgt_adc;
  a.n_tgt = g_adc ? 0 : n_tgt;
  a.adc_out = adc_out;
  rc = run_accum(kModeGrad, a, st);
  if (rc) return wrap(rc, "lsim_lut_grad");
  return wrap(run_grad_finalize(a, loss_out, grad_out, st), "lsim_lut_grad");
}

int lsim_lut_grad_stored(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events,
                         const float *wfs, int64_t p_pad, int32_t n_valid, const float *normals, const float *g_adc,
                         const int32_t *tgt_pids, const float *tgt_adc, int64_t n_tgt, float *loss_out,
                         float *grad_out, float *adc_out, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!tables || !ws || !grad_out || !wfs) return fail(LSIM_ERR_INVALID, "lsim_lut_grad_stored: null pointer");
  if (!g_adc && n_tgt > 0 && (!tgt_pids || !tgt_adc)) return fail(LSIM_ERR_INVALID, "lsim_lut_grad_stored: null target");
  if (n_valid < 0 || p_pad < n_valid) return fail(LSIM_ERR_CAPACITY, "lsim_lut_grad_stored: p_pad < n_valid");
  cudaStream_t st = (cudaStream_t)stream;
  AccumArgs a = make_args(p, tables, ws, n_rows, n_events);
  a.n_valid = n_valid;
  a.row_offset = p_pad - n_valid;
  a.wfs = const_cast<float *>(wfs);
  a.normals = normals;
  a.g_adc = g_adc;
  a.tgt_pids = tgt_pids;
  a.tgt_adc = tgt_adc;
  a.n_tgt = g_adc ? 0 : n_tgt;
  a.adc_out = adc_out;
  rc = run_accum(kModeGradStored, a, st);
  if (rc) return wrap(rc, "lsim_lut_grad_stored");
  return wrap(run_grad_finalize(a, loss_out, grad_out, st), "lsim_lut_grad_stored");
}

int lsim_lut_wfs_vjp(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events,
                     const float *g_wfs, int64_t p_pad, int32_t n_valid, float *grad_out, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!tables || !ws || !grad_out || (n_valid > 0 && !g_wfs)) return fail(LSIM_ERR_INVALID, "lsim_lut_wfs_vjp: null pointer");
  if (n_valid < 0 || p_pad < n_valid) return fail(LSIM_ERR_CAPACITY, "lsim_lut_wfs_vjp: p_pad < n_valid");
  cudaStream_t st = (cudaStream_t)stream;
  AccumArgs a = make_args(p, tables, ws, n_rows, n_events);
  a.n_valid = n_valid;
  a.row_offset = p_pad - n_valid;
  a.wfs = const_cast<float *>(g_wfs);
  rc = run_accum(kModeVjpWfs, a, st);
  if (rc) return wrap(rc, "lsim_lut_wfs_vjp");
  return wrap(run_grad_finalize(a, nullptr, grad_out, st), "lsim_lut_wfs_vjp");
}

int lsim_fee(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals, float *adc_out,
             float *tick_out, float *integral_out, void *stream) {
  g_err.clear();
  if (!p) return fail(LSIM_ERR_INVALID, "lsim_fee: null parameter block");
  if (n_pix > 0 && (!wfs || !adc_out || !tick_out)) return fail(LSIM_ERR_INVALID, "lsim_fee: null pointer");
  if (p->max_adc_values < 1 || p->max_adc_values > LSIM_MAX_HITS) return fail(LSIM_ERR_UNSUPPORTED, "lsim_fee: bad MAX_ADC_VALUES");
  return wrap(run_fee(*p, wfs, n_pix, n_t, normals, adc_out, tick_out, integral_out, (cudaStream_t)stream), "lsim_fee");
}

size_t lsim_fee_vjp_workspace_bytes(int64_t n_pix) { return n_pix < 0 ? 0 : fee_vjp_workspace_bytes(n_pix); }

int lsim_fee_vjp(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals,
                 const float *g_adc, float *g_wfs, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  if (!p) return fail(LSIM_ERR_INVALID, "lsim_fee_vjp: null parameter block");
  if (n_pix < 0 || (n_pix > 0 && (!wfs || !g_adc || !g_wfs))) return fail(LSIM_ERR_INVALID, "lsim_fee_vjp: null pointer");
  if (p->max_adc_values < 1 || p->max_adc_values > LSIM_MAX_HITS)
    return fail(LSIM_ERR_UNSUPPORTED, "lsim_fee_vjp: bad MAX_ADC_VALUES");
  if (n_t < 4 || n_t > 2048 || n_t % 4 != 0)
    return fail(LSIM_ERR_UNSUPPORTED, "lsim_fee_vjp: n_t %d must be a multiple of 4 up to 2048", n_t);
  if (!ws || ws_bytes < fee_vjp_workspace_bytes(n_pix))
    return fail(LSIM_ERR_CAPACITY, "lsim_fee_vjp: workspace %zu < %zu bytes", ws_bytes, fee_vjp_workspace_bytes(n_pix));
  return wrap(run_fee_vjp(*p, wfs, n_pix, n_t, normals, g_adc, g_wfs, ws, (cudaStream_t)stream), "lsim_fee_vjp");
}

int lsim_pixel_coords(const LsimParams *p, const int32_t *unique_pixels, int64_t n_pix, float *x_out, float *y_out,
                      int32_t *plane_out, int32_t *event_out, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (n_pix < 0 || (n_pix > 0 && !unique_pixels)) return fail(LSIM_ERR_INVALID, "lsim_pixel_coords: bad arguments");
  return wrap(run_pixel_coords(*p, unique_pixels, n_pix, x_out, y_out, plane_out, event_out, (cudaStream_t)stream),
              "lsim_pixel_coords");
}

size_t lsim_fee_prob_workspace_bytes(const LsimParams *p) {
  return p ? fee_prob_workspace_bytes(p->max_adc_values) : 0;
}

int lsim_fee_prob(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                  float stop_threshold, float *log_prob_out, float *charge_out, float *exp_tick_out,
                  float *exp_adc_out, float *lambda_out, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (n_pix < 0 || (n_pix > 0 && !wfs)) return fail(LSIM_ERR_INVALID, "lsim_fee_prob: bad waveform arguments");
  const bool any_red = exp_tick_out || exp_adc_out || lambda_out;
  if (any_red && !(exp_tick_out && exp_adc_out && lambda_out))
    return fail(LSIM_ERR_INVALID, "lsim_fee_prob: give all three of exp_tick, exp_adc, lambda or none");
  if (!(stop_threshold > 0.0f)) return fail(LSIM_ERR_INVALID, "lsim_fee_prob: stop_threshold %g", stop_threshold);
  if (!ws || ws_bytes < fee_prob_workspace_bytes(p->max_adc_values))
    return fail(LSIM_ERR_CAPACITY, "lsim_fee_prob: workspace %zu < %zu bytes", ws_bytes,
                fee_prob_workspace_bytes(p->max_adc_values));
  return wrap(run_fee_prob(*p, wfs, n_pix, n_t, n_paths, stop_threshold, log_prob_out, charge_out, exp_tick_out,
                           exp_adc_out, lambda_out, ws, (cudaStream_t)stream),
              "lsim_fee_prob");
}

size_t lsim_fee_prob_vjp_workspace_bytes(const LsimParams *p, int64_t n_pix, int32_t n_paths) {
  return p && n_pix >= 0 && n_paths > 0 ? fee_prob_vjp_workspace_bytes(n_pix, p->max_adc_values, n_paths) : 0;
}

int lsim_fee_prob_vjp(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                      float stop_threshold, const float *g_log_prob, const float *g_charge, const float *g_e_tick,
                      const float *g_e_adc, const float *g_lambda, float *g_wfs, void *ws, size_t ws_bytes,
                      void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (n_pix < 0 || (n_pix > 0 && (!wfs || !g_wfs))) return fail(LSIM_ERR_INVALID, "lsim_fee_prob_vjp: bad arguments");
  const bool any_red = g_e_tick || g_e_adc || g_lambda;
  if (any_red && !(g_e_tick && g_e_adc && g_lambda))
    return fail(LSIM_ERR_INVALID, "lsim_fee_prob_vjp: give all three reduction cotangents or none");
  if (!(stop_threshold > 0.0f)) return fail(LSIM_ERR_INVALID, "lsim_fee_prob_vjp: stop_threshold %g", stop_threshold);
  if (n_paths < 1 || n_paths > 32) return fail(LSIM_ERR_UNSUPPORTED, "lsim_fee_prob_vjp: n_paths %d", n_paths);
  const size_t need = fee_prob_vjp_workspace_bytes(n_pix, p->max_adc_values, n_paths);
  if (!ws || ws_bytes < need) return fail(LSIM_ERR_CAPACITY, "lsim_fee_prob_vjp: workspace %zu < %zu bytes", ws_bytes, need);
  return wrap(run_fee_prob_vjp(*p, wfs, n_pix, n_t, n_paths, stop_threshold, g_log_prob, g_charge, g_e_tick, g_e_adc,
                               g_lambda, g_wfs, ws, (cudaStream_t)stream),
              "lsim_fee_prob_vjp");
}

size_t lsim_mse_adc_workspace_bytes(int64_t n_hits, int64_t n_ref) {
  return n_hits < 0 || n_ref < 0 ? 0 : mse_adc_workspace_bytes(n_hits, n_ref);
}

int lsim_mse_adc(const float *x, const float *y, const float *z, const int32_t *event, const float *w, int64_t n_hits,
                 const float *ref_x, const float *ref_y, const float *ref_z, const int32_t *ref_event,
                 const float *ref_w, int64_t n_ref, float sigma, float lambda_q, float *out, float *grad_w,
                 float *grad_z, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  if (n_hits < 0 || n_ref < 0 || !out) return fail(LSIM_ERR_INVALID, "lsim_mse_adc: bad arguments");
  if (n_hits > 0 && (!x || !y || !z || !event || !w)) return fail(LSIM_ERR_INVALID, "lsim_mse_adc: null hit array");
  if (n_ref > 0 && (!ref_x || !ref_y || !ref_z || !ref_event || !ref_w))
    return fail(LSIM_ERR_INVALID, "lsim_mse_adc: null reference array");
  if (!(sigma > 0.0f)) return fail(LSIM_ERR_INVALID, "lsim_mse_adc: sigma %g", sigma);
  if (!ws || ws_bytes < mse_adc_workspace_bytes(n_hits, n_ref))
    return fail(LSIM_ERR_CAPACITY, "lsim_mse_adc: workspace %zu < %zu bytes", ws_bytes,
                mse_adc_workspace_bytes(n_hits, n_ref));
  return wrap(run_mse_adc(x, y, z, event, w, n_hits, ref_x, ref_y, ref_z, ref_event, ref_w, n_ref, sigma, lambda_q,
                          out, grad_w, grad_z, ws, (cudaStream_t)stream),
              "lsim_mse_adc");
}

size_t lsim_nll_workspace_bytes(int64_t n_hits, int64_t n_ref) {
  return n_hits < 0 || n_ref < 0 ? 0 : nll_workspace_bytes(n_hits, n_ref);
}

int lsim_nll_loss(const float *x, const float *y, const float *z, const float *q, const int32_t *event,
                  const float *hit_prob, int64_t n_hits, const float *ref_x, const float *ref_y, const float *ref_z,
                  const float *ref_q, const int32_t *ref_event, const float *ref_hit_prob, int64_t n_ref, float sigma,
                  float *out, float *grad_q, float *grad_z, float *grad_hit_prob, void *ws, size_t ws_bytes,
                  void *stream) {
  g_err.clear();
  if (n_hits < 0 || n_ref < 0 || !out) return fail(LSIM_ERR_INVALID, "lsim_nll_loss: bad arguments");
  if (n_hits > 0 && (!x || !y || !z || !q || !event || !hit_prob))
    return fail(LSIM_ERR_INVALID, "lsim_nll_loss: null hit array");
  if (n_ref > 0 && (!ref_x || !ref_y || !ref_z || !ref_q || !ref_event || !ref_hit_prob))
    return fail(LSIM_ERR_INVALID, "lsim_nll_loss: null reference array");
  if (!(sigma > 0.0f)) return fail(LSIM_ERR_INVALID, "lsim_nll_loss: sigma %g", sigma);
  if (!ws || ws_bytes < nll_workspace_bytes(n_hits, n_ref))
    return fail(LSIM_ERR_CAPACITY, "lsim_nll_loss: workspace %zu < %zu bytes", ws_bytes,
                nll_workspace_bytes(n_hits, n_ref));
  return wrap(run_nll(x, y, z, q, event, hit_prob, n_hits, ref_x, ref_y, ref_z, ref_q, ref_event, ref_hit_prob, n_ref,
                      sigma, out, grad_q, grad_z, grad_hit_prob, ws, (cudaStream_t)stream),
              "lsim_nll_loss");
}

size_t lsim_chamfer_workspace_bytes(int64_t n_hits, int64_t n_ref) {
  return n_hits < 0 || n_ref < 0 ? 0 : chamfer_workspace_bytes(n_hits, n_ref);
}

int lsim_chamfer_3d(const float *x, const float *y, const float *z, const int32_t *event, const float *w,
                    int64_t n_hits, const float *ref_x, const float *ref_y, const float *ref_z,
                    const int32_t *ref_event, const float *ref_w, int64_t n_ref, float *out, float *grad_w,
                    float *grad_z, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  if (n_hits < 0 || n_ref < 0 || !out || n_hits > INT32_MAX || n_ref > INT32_MAX)
    return fail(LSIM_ERR_INVALID, "lsim_chamfer_3d: bad arguments");
  if (n_hits > 0 && (!x || !y || !z || !event || !w)) return fail(LSIM_ERR_INVALID, "lsim_chamfer_3d: null hit array");
  if (n_ref > 0 && (!ref_x || !ref_y || !ref_z || !ref_event || !ref_w))
    return fail(LSIM_ERR_INVALID, "lsim_chamfer_3d: null reference array");
  if (!ws || ws_bytes < chamfer_workspace_bytes(n_hits, n_ref))
    return fail(LSIM_ERR_CAPACITY, "lsim_chamfer_3d: workspace %zu < %zu bytes", ws_bytes,
                chamfer_workspace_bytes(n_hits, n_ref));
  return wrap(run_chamfer(x, y, z, event, w, n_hits, ref_x, ref_y, ref_z, ref_event, ref_w, n_ref, out, grad_w,
                          grad_z, ws, (cudaStream_t)stream),
              "lsim_chamfer_3d");
}

size_t lsim_prob_llhd_workspace_bytes(int64_t n_hits) { return n_hits < 0 ? 0 : prob_llhd_workspace_bytes(n_hits); }

int lsim_prob_llhd(const LsimParams *p, const int32_t *sim_pixels, int64_t n_pix, int32_t n_values, int32_t n_ticks,
                   const float *log_prob, const float *adcs_distrib, const int32_t *tgt_pixels,
                   const int32_t *tgt_ticks, const float *tgt_adcs, int64_t n_hits, double sigma_charge, double eps,
                   const float *g_loss, float *out, float *g_log_prob, float *g_adcs, void *ws, size_t ws_bytes,
                   void *stream) {
  g_err.clear();
  if (!p || n_pix < 0 || n_hits < 0 || n_values <= 0 || n_ticks <= 0 || !out)
    return fail(LSIM_ERR_INVALID, "lsim_prob_llhd: bad arguments");
  if (n_hits > 0 && n_pix == 0)
    return fail(LSIM_ERR_INVALID, "lsim_prob_llhd: %lld target hits but no simulated pixels", (long long)n_hits);
  if (n_pix > 0 && n_pix > INT64_MAX / n_values / n_ticks)
    return fail(LSIM_ERR_INVALID, "lsim_prob_llhd: distributions too large");
  if (n_pix > 0 && (!sim_pixels || !log_prob || !adcs_distrib))
    return fail(LSIM_ERR_INVALID, "lsim_prob_llhd: null prediction array");
  if (n_hits > 0 && (!tgt_pixels || !tgt_ticks || !tgt_adcs))
    return fail(LSIM_ERR_INVALID, "lsim_prob_llhd: null target array");
  if (!(sigma_charge > 0.0) || !(eps > 0.0))
    return fail(LSIM_ERR_INVALID, "lsim_prob_llhd: sigma_charge %g, eps %g", sigma_charge, eps);
  if (!ws || ws_bytes < prob_llhd_workspace_bytes(n_hits))
    return fail(LSIM_ERR_CAPACITY, "lsim_prob_llhd: workspace %zu < %zu bytes", ws_bytes,
                prob_llhd_workspace_bytes(n_hits));
  return wrap(run_prob_llhd(*p, sim_pixels, n_pix, n_values, n_ticks, log_prob, adcs_distrib, tgt_pixels, tgt_ticks,
                            tgt_adcs, n_hits, sigma_charge, eps, g_loss, out, g_log_prob, g_adcs, ws,
                            (cudaStream_t)stream),
              "lsim_prob_llhd");
}

size_t lsim_llhd_workspace_bytes(int64_t n_rows) { return n_rows < 0 ? 0 : llhd_workspace_bytes(n_rows); }

int lsim_llhd_loss(const float *ticks_prob, const int32_t *ticks_mc, const float *no_hit_prob,
                   const float *charge_distrib, const float *charge_mc, int64_t n_rows, int32_t n_ticks, double sigma,
                   const float *g_loss, float *out, float *g_ticks_prob, float *g_no_hit_prob, float *g_charge_distrib,
                   float *g_charge_mc, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  if (n_rows < 0 || n_ticks <= 0 || !out) return fail(LSIM_ERR_INVALID, "lsim_llhd_loss: bad arguments");
  if (n_rows > INT64_MAX / n_ticks) return fail(LSIM_ERR_INVALID, "lsim_llhd_loss: distributions too large");
  if (n_rows > 0 && (!ticks_prob || !ticks_mc || !no_hit_prob || !charge_distrib || !charge_mc))
    return fail(LSIM_ERR_INVALID, "lsim_llhd_loss: null input array");
  if (!(sigma > 0.0)) return fail(LSIM_ERR_INVALID, "lsim_llhd_loss: sigma %g", sigma);
  if (!ws || ws_bytes < llhd_workspace_bytes(n_rows))
    return fail(LSIM_ERR_CAPACITY, "lsim_llhd_loss: workspace %zu < %zu bytes", ws_bytes,
                llhd_workspace_bytes(n_rows));
  return wrap(run_llhd(ticks_prob, ticks_mc, no_hit_prob, charge_distrib, charge_mc, n_rows, n_ticks, sigma, g_loss,
                       out, g_ticks_prob, g_no_hit_prob, g_charge_distrib, g_charge_mc, ws, (cudaStream_t)stream),
              "lsim_llhd_loss");
}

size_t lsim_occurrence_workspace_bytes(int64_t n) { return n < 0 ? 0 : occurrence_workspace_bytes(n); }

int lsim_occurrence_indices(const int32_t *ids, int64_t n, int32_t *out, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  if (n < 0 || n > INT32_MAX - 1 || (n > 0 && (!ids || !out)))
    return fail(LSIM_ERR_INVALID, "lsim_occurrence_indices: bad arguments");
  if (n > 0 && (!ws || ws_bytes < occurrence_workspace_bytes(n)))
    return fail(LSIM_ERR_CAPACITY, "lsim_occurrence_indices: workspace %zu < %zu bytes", ws_bytes,
                occurrence_workspace_bytes(n));
  return wrap(run_occurrence(ids, (int32_t)n, out, ws, (cudaStream_t)stream), "lsim_occurrence_indices");
}

int lsim_gather_tracks(const float *table, int64_t n_table, int32_t n_fields, const int64_t *rows, int64_t n_rows,
                       int32_t event_col, const float *event_values, float *out, int32_t *status_dev, void *stream) {
  g_err.clear();
  if (n_table < 0 || n_rows < 0 || n_fields <= 0 || n_fields > 96 || !status_dev ||
      (n_rows > 0 && (!table || !rows || !out)))
    return fail(LSIM_ERR_INVALID, "lsim_gather_tracks: bad arguments");
  if (event_values && (event_col < 0 || event_col >= n_fields))
    return fail(LSIM_ERR_INVALID, "lsim_gather_tracks: event column %d outside [0, %d)", event_col, n_fields);
  return wrap(run_gather_tracks(table, n_table, n_fields, rows, n_rows, event_col, event_values, out, status_dev,
                                (cudaStream_t)stream),
              "lsim_gather_tracks");
}

int lsim_pad_tracks(float *batch, int64_t n_rows, int64_t target_rows, int32_t n_fields, int32_t event_col,
                    const int8_t *col_roles, int64_t n_local_events, void *stream) {
  g_err.clear();
  if (n_rows < 0 || n_fields <= 0 || n_fields > 96 || event_col < 0 || event_col >= n_fields ||
      (target_rows > 0 && !batch))
    return fail(LSIM_ERR_INVALID, "lsim_pad_tracks: bad arguments");
  if (col_roles)
    for (int c = 0; c < n_fields; ++c)
      if (col_roles[c] < 0 || col_roles[c] > 2) return fail(LSIM_ERR_INVALID, "lsim_pad_tracks: column role %d", col_roles[c]);
  const int64_t rows = target_rows > n_rows ? target_rows : n_rows;
  return wrap(run_pad_tracks(batch, n_rows, rows, n_fields, event_col, col_roles, n_local_events,
                             (cudaStream_t)stream),
              "lsim_pad_tracks");
}

size_t lsim_chop_workspace_bytes(int64_t n_rows) { return n_rows < 0 ? 0 : chop_workspace_bytes(n_rows); }

int lsim_chop_tracks(const LsimFieldMap *f, const float *tracks, int64_t n_rows, double precision, float *out,
                     int64_t out_capacity, int64_t *n_out_dev, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  int rc = check_fields(f);
  if (rc) return rc;
  if (n_rows < 0 || out_capacity < 0 || !n_out_dev || (n_rows > 0 && !tracks) || (out_capacity > 0 && !out))
    return fail(LSIM_ERR_INVALID, "lsim_chop_tracks: bad arguments");
  if (!(precision > 0) || !(precision < 1e30)) return fail(LSIM_ERR_INVALID, "lsim_chop_tracks: precision %g", precision);
  if (!ws || ws_bytes < chop_workspace_bytes(n_rows))
    return fail(LSIM_ERR_CAPACITY, "lsim_chop_tracks: workspace %zu < %zu bytes", ws_bytes,
                chop_workspace_bytes(n_rows));
  return wrap(run_chop(*f, tracks, n_rows, precision, out, out_capacity, n_out_dev, ws, (cudaStream_t)stream),
              "lsim_chop_tracks");
}

size_t lsim_hit_records_workspace_bytes(int64_t n) { return n < 0 ? 0 : records_workspace_bytes(n); }

int lsim_hit_records(const LsimParams *p, float adc_lowest, const LsimHitColumns *in, int64_t n,
                     const LsimHitColumns *out, float *out_adc_clean, float *out_q, int32_t *run_event,
                     int64_t *run_start, int64_t *counts_dev, void *ws, size_t ws_bytes, void *stream) {
  g_err.clear();
  if (!p) return fail(LSIM_ERR_INVALID, "lsim_hit_records: null parameter block");
  if (!in || !out || !counts_dev || n < 0) return fail(LSIM_ERR_INVALID, "lsim_hit_records: bad arguments");
  if (n > 0) {
    if (!in->adc || !in->event || !out->event) return fail(LSIM_ERR_INVALID, "lsim_hit_records: adc and event columns are required");
    const bool missing = (out->pixel_x && !in->pixel_x) || (out->pixel_y && !in->pixel_y) ||
                         (out->pixel_z && !in->pixel_z) || (out->ticks && !in->ticks) ||
                         (out->hit_prob && !in->hit_prob) || (out->pixels && !in->pixels);
    if (missing) return fail(LSIM_ERR_INVALID, "lsim_hit_records: an output column has no input column");
  }
  if (run_event && !run_start) return fail(LSIM_ERR_INVALID, "lsim_hit_records: run_event needs run_start");
  if (n > 0 && (!ws || ws_bytes < records_workspace_bytes(n)))
    return fail(LSIM_ERR_CAPACITY, "lsim_hit_records: workspace %zu < %zu bytes", ws_bytes, records_workspace_bytes(n));
  return wrap(run_records(*p, adc_lowest, *in, n, *out, out_adc_clean, out_q, run_event, run_start, counts_dev, ws,
                          (cudaStream_t)stream),
              "lsim_hit_records");
}

size_t lsim_hits_workspace_bytes(int64_t n_pix, int32_t max_adc_values) {
  return hits_ws_bytes(n_pix * (int64_t)max_adc_values);
}

int lsim_hits(const LsimParams *p, const float *adc, const float *ticks, const int32_t *unique_pixels, int64_t n_pix,
              int32_t tick_limit, float *out_adc, float *out_x, float *out_y, float *out_z, float *out_ticks,
              float *out_hit_prob, int32_t *out_event, int32_t *out_pixels, int32_t *nb_valid_dev, void *ws,
              size_t ws_bytes, void *stream) {
  g_err.clear();
  if (!p) return fail(LSIM_ERR_INVALID, "lsim_hits: null parameter block");
  if (!nb_valid_dev || (n_pix > 0 && (!adc || !ticks || !unique_pixels || !out_adc || !out_x || !out_y || !out_z ||
                                      !out_ticks || !out_hit_prob || !out_event || !out_pixels || !ws)))
    return fail(LSIM_ERR_INVALID, "lsim_hits: null pointer");
  if (n_pix < 0) return fail(LSIM_ERR_INVALID, "lsim_hits: negative pixel count");
  if (p->max_adc_values < 1 || p->max_adc_values > LSIM_MAX_HITS)
    return fail(LSIM_ERR_INVALID, "lsim_hits: max_adc_values outside 1..LSIM_MAX_HITS");
  // the kept count and the hit slots are indexed in int32
  if (n_pix > INT32_MAX / p->max_adc_values) return fail(LSIM_ERR_CAPACITY, "lsim_hits: more than 2^31 - 1 hit slots");
  if (ws_bytes < hits_ws_bytes(n_pix * (int64_t)p->max_adc_values))
    return fail(LSIM_ERR_CAPACITY, "lsim_hits: workspace too small");
  return wrap(run_hits(*p, adc, ticks, unique_pixels, n_pix, tick_limit, out_adc, out_x, out_y, out_z, out_ticks,
                       out_hit_prob, out_event, out_pixels, nb_valid_dev, ws, (cudaStream_t)stream),
              "lsim_hits");
}

int lsim_param_stage2(const LsimParams *p, const void *ws, int64_t n_rows, int32_t n_events, int64_t p_pad,
                      int32_t n_em1, int32_t n_valid, float *wfs, int32_t *unique_pixels, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!ws || (p_pad > 0 && (!wfs || !unique_pixels))) return fail(LSIM_ERR_INVALID, "lsim_param_stage2: null pointer");
  if (n_em1 < 0 || n_valid < 0 || (int64_t)n_em1 + n_valid > p_pad)
    return fail(LSIM_ERR_CAPACITY, "lsim_param_stage2: p_pad too small");
  cudaStream_t st = (cudaStream_t)stream;
  AccumArgs a = make_args(p, nullptr, ws, n_rows, n_events);
  rc = run_fill_unique(*p, a.w, a.g, p_pad, n_em1, n_valid, unique_pixels, wfs, p->n_ticks - 1, st);
  if (rc) return wrap(rc, "lsim_param_stage2");
  return wrap(run_param_accum(*p, a.w, a.g, n_valid, p_pad - n_valid, wfs, st), "lsim_param_stage2");
}

int lsim_param_wfs_vjp(const LsimParams *p, const void *ws, int64_t n_rows, int32_t n_events, const float *g_wfs,
                       int64_t p_pad, int32_t n_valid, float *grad_out, void *stream) {
  g_err.clear();
  int rc = check_params(p);
  if (rc) return rc;
  if (!ws || !grad_out || (n_valid > 0 && !g_wfs)) return fail(LSIM_ERR_INVALID, "lsim_param_wfs_vjp: null pointer");
  if (n_valid < 0 || p_pad < n_valid) return fail(LSIM_ERR_CAPACITY, "lsim_param_wfs_vjp: p_pad < n_valid");
  cudaStream_t st = (cudaStream_t)stream;
  AccumArgs a = make_args(p, nullptr, ws, n_rows, n_events);
  a.n_valid = n_valid;
  rc = run_param_vjp(*p, a.w, a.g, n_valid, p_pad - n_valid, g_wfs, n_rows, st);
  if (rc) return wrap(rc, "lsim_param_wfs_vjp");
  return wrap(run_grad_finalize(a, nullptr, grad_out, st), "lsim_param_wfs_vjp");
}

}  // extern "C"
