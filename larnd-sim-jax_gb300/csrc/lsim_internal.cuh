// Host-side drivers shared between the translation units of liblsim.
#pragma once

#include "lsim_common.cuh"

namespace lsim {

// lsim_segments.cu
int run_stage1(bool param_mode, const LsimParams &p, const LsimFieldMap &f, const float *tracks,
               const float *normals, int64_t n_rows, int32_t n_events, const Workspace &w, cudaStream_t st,
               const float *theta_dev = nullptr);
int run_adam(float *theta, const float *grad, const float *scale, const float *lr, float *state, float beta1,
             float beta2, float eps, cudaStream_t st);
int run_fit_init(float *theta, const LsimFitOptions &o, float *state, cudaStream_t st);
int run_fit_step(float *theta, const float *grad, const LsimFitOptions &o, float *state, cudaStream_t st);
int run_fill_unique(const LsimParams &p, const Workspace &w, const Grid &g, int64_t p_pad, int32_t n_em1,
                    int32_t n_valid, int32_t *unique_pixels, float *wfs, int32_t nt_out, cudaStream_t st);

// lsim_accum.cu
enum AccumMode { kModeWfs = 0, kModeAdc = 1, kModeGrad = 2, kModeGradStored = 3, kModeVjpWfs = 4 };
struct AccumArgs {
  LsimParams p;
  int64_t n_rows;           // segments (rows of the track table)
  Tables tab;
  Workspace w;
  Grid g;
  int32_t n_valid;
  int64_t row_offset;       // output row of valid row 0 (wfs mode)
  float *wfs;               // [rows][n_ticks-1] (wfs mode: written; stored-gradient mode: read)
  const float *normals;     // [n_valid][1+3H] or null
  float *adc_out, *tick_out;  // [n_valid][H] (adc/grad modes, optional in grad)
  const float *g_adc;       // [n_valid][H] cotangent (grad mode) or null
  const int32_t *tgt_pids;  // target pixels for the SSE loss (grad mode, when g_adc is null)
  const float *tgt_adc;
  int64_t n_tgt;
  int warp_smem;            // shared-memory bytes per warp of the pixel kernel (set at launch)
};
int run_accum(AccumMode mode, const AccumArgs &a, cudaStream_t st);
int run_grad_finalize(const AccumArgs &a, float *loss_out, float *grad_out, cudaStream_t st);

// lsim_main.cu: segment-major main-bin records and their adjoint
int run_main_records(const AccumArgs &a, cudaStream_t st);
int run_main_adjoint(const AccumArgs &a, cudaStream_t st);

int run_param_accum(const LsimParams &p, const Workspace &w, const Grid &g, int32_t n_valid, int64_t row_offset,
                    float *wfs, cudaStream_t st);

// lsim_fee.cu
int run_fee(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals, float *adc_out,
            float *tick_out, float *integral_out, cudaStream_t st);
size_t hits_ws_bytes(int64_t n);
int run_hits(const LsimParams &p, const float *adc, const float *ticks, const int32_t *unique_pixels, int64_t n_pix,
             int32_t tick_limit, float *out_adc, float *out_x, float *out_y, float *out_z, float *out_ticks,
             float *out_hit_prob, int32_t *out_event, int32_t *out_pixels, int32_t *nb_valid_dev, void *ws,
             cudaStream_t st);

// lsim_lut.cu
int run_build_templates(const float *response, int nx, int ny, int nt, const float *sigmas, int n_templates,
                        int extent, float *out, cudaStream_t st);
int run_prepare_tables(const LsimParams &p, const float *templates, void *tables, cudaStream_t st);

int run_param_vjp(const LsimParams &p, const Workspace &w, const Grid &g, int32_t n_valid, int64_t row_offset,
                  const float *g_wfs, int64_t n_rows, cudaStream_t st);
size_t fee_vjp_workspace_bytes(int64_t n_pix);
int run_fee_vjp(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals,
                const float *g_adc, float *g_wfs, void *ws, cudaStream_t st);
int run_pixel_coords(const LsimParams &p, const int32_t *unique_pixels, int64_t n, float *x, float *y,
                     int32_t *plane, int32_t *event, cudaStream_t st);

// lsim_fee_prob.cu
size_t fee_prob_workspace_bytes(int32_t max_adc_values);
int run_fee_prob(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                 float stop_threshold, float *log_prob, float *charge, float *e_tick, float *e_adc, float *lam,
                 void *ws, cudaStream_t st);

// lsim_prob_loss.cu
size_t prob_llhd_workspace_bytes(int64_t n_hits);
int run_prob_llhd(const LsimParams &p, const int32_t *sim, int64_t n_pix, int32_t n_values, int32_t n_ticks,
                  const float *log_prob, const float *adcs, const int32_t *tgt_pix, const int32_t *tgt_tick,
                  const float *tgt_adc, int64_t n_hits, double sigma_charge, double eps, const float *g_loss,
                  float *out, float *g_log_prob, float *g_adcs, void *ws, cudaStream_t st);
size_t llhd_workspace_bytes(int64_t n_rows);
int run_llhd(const float *tpd, const int32_t *ticks, const float *nohit, const float *cd, const float *cmc,
             int64_t n_rows, int32_t n_ticks, double sigma, const float *g_loss, float *out, float *g_tpd,
             float *g_nohit, float *g_cd, float *g_cmc, void *ws, cudaStream_t st);
size_t occurrence_workspace_bytes(int64_t n);
int run_occurrence(const int32_t *ids, int32_t n, int32_t *out, void *ws, cudaStream_t st);

// lsim_losses.cu
size_t mse_adc_workspace_bytes(int64_t n, int64_t m);
int run_mse_adc(const float *x, const float *y, const float *z, const int32_t *event, const float *w, int64_t n,
                const float *rx, const float *ry, const float *rz, const int32_t *revent, const float *rw, int64_t m,
                float sigma, float lambda_q, float *out, float *grad_w, float *grad_z, void *ws, cudaStream_t st);

size_t nll_workspace_bytes(int64_t n, int64_t m);
int run_nll(const float *x, const float *y, const float *z, const float *q, const int32_t *event, const float *hp,
            int64_t n, const float *rx, const float *ry, const float *rz, const float *rq, const int32_t *revent,
            const float *rhp, int64_t m, float sigma, float *out, float *g_q, float *g_z, float *g_hp, void *ws,
            cudaStream_t st);
size_t chamfer_workspace_bytes(int64_t n, int64_t m);
int run_chamfer(const float *x, const float *y, const float *z, const int32_t *event, const float *w, int64_t n,
                const float *rx, const float *ry, const float *rz, const int32_t *revent, const float *rw, int64_t m,
                float *out, float *g_w, float *g_z, void *ws, cudaStream_t st);

size_t fee_prob_vjp_workspace_bytes(int64_t n_pix, int32_t max_adc_values, int32_t n_paths);
int run_fee_prob_vjp(const LsimParams &p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                     float stop_threshold, const float *g_log_prob, const float *g_charge, const float *g_e_tick,
                     const float *g_e_adc, const float *g_lam, float *g_wfs, void *ws, cudaStream_t st);

// lsim_records.cu
size_t records_workspace_bytes(int64_t n);
int run_records(const LsimParams &p, float adc_lowest, const LsimHitColumns &in, int64_t n, const LsimHitColumns &out,
                float *out_clean, float *out_q, int32_t *run_event, int64_t *run_start, int64_t *counts, void *ws,
                cudaStream_t st);

// lsim_tracks.cu
int run_gather_tracks(const float *table, int64_t n_table, int32_t n_fields, const int64_t *rows, int64_t n_rows,
                      int32_t event_col, const float *event_values, float *out, int32_t *status, cudaStream_t st);
int run_pad_tracks(float *batch, int64_t n_rows, int64_t target_rows, int32_t n_fields, int32_t event_col,
                   const int8_t *col_roles, int64_t n_local_events, cudaStream_t st);

// lsim_chop.cu
size_t chop_workspace_bytes(int64_t n_rows);
int run_chop(const LsimFieldMap &f, const float *tracks, int64_t n_rows, double precision, float *out,
             int64_t capacity, int64_t *n_out, void *ws, cudaStream_t st);

int device_sm_count();

// profiling events around the pixel-accumulation kernel (lsim_set_kernel_events)
void kernel_events(cudaEvent_t *start, cudaEvent_t *stop);
// launch shapes set by lsim_set_tuning (zero fields: defaults)
LsimTuning tuning();

// lsim_api.cu: thread-local error message shared by all entry points
int set_error(int code, const char *msg);
void clear_error();

}  // namespace lsim
