/*
 * lsim.h -- C ABI of the GB300 (sm_103a) larnd-sim simulate path.
 *
 * Every entry point takes caller-allocated DEVICE pointers, sizes, a POD
 * parameter block and a CUDA stream (passed as void*), returns an LSIM_*
 * status and never throws.  Device memory is owned by the caller: the
 * library allocates nothing; sizes of the workspace and of the prepared LUT
 * tables are queried with the *_bytes functions.  On error,
 * lsim_last_error() returns a thread-local message.
 *
 * The reference (larnd-sim-jax) is Python/JAX with no FFI of its own; each
 * function below names the reference function(s) it replaces.  File paths
 * are relative to the reference project root.
 */
#ifndef LSIM_H
#define LSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LSIM_ABI_VERSION 2

enum {
  LSIM_OK = 0,
  LSIM_ERR_INVALID = 1,     /* bad argument or bad input value (e.g. eventID < -1) */
  LSIM_ERR_CAPACITY = 2,    /* a buffer or workspace is too small */
  LSIM_ERR_CUDA = 3,        /* a CUDA runtime error */
  LSIM_ERR_UNSUPPORTED = 4  /* configuration outside what the kernels support */
};

enum { LSIM_RECOMB_BOX = 1, LSIM_RECOMB_BIRKS = 2, LSIM_RECOMB_ELLIPSOID = 3 };

#define LSIM_MAX_TPC 2
#define LSIM_MAX_TEMPLATES 128
#define LSIM_MAX_HITS 16
#define LSIM_NPARAM 8   /* gradient order: Ab kb eField lifetime vdrift long_diff tran_diff lArDensity */

/* Column indices of the (N, F) float32 track array (the reference's
 * `fields` tuple resolved to integers, optimize/dataio.py:130-141). */
typedef struct LsimFieldMap {
  int32_t n_fields;
  int32_t eventID, x, y, z, x_start, y_start, z_start, x_end, y_end, z_end;
  int32_t dx, dE, dEdx;
} LsimFieldMap;

/* Parameter block.  Scalars hold the float32 values the reference computes
 * in float64 from its static parameters and rounds once (e.g. erho is
 * float32(eField * lArDensity), vdrift is float32(get_vdrift(params))). */
typedef struct LsimParams {
  /* quenching, src/larndsim/quenching_jax.py:18-74 */
  int32_t recombination_mode;
  float Ab, kb, alpha, beta, r_inv2, erho, mev_to_electrons;
  /* drift, src/larndsim/drifting_jax.py:18-58 */
  float vdrift, lifetime, long_diff, tran_diff, size_margin;
  float shift_x, shift_y, shift_z;
  int32_t n_tpc;
  float tpc_borders[LSIM_MAX_TPC * 3 * 2];
  /* pixels and sub-pixel bins, src/larndsim/sim_jax.py:374-453 */
  float pixel_pitch, half_pitch, bin_width;
  int32_t n_pixels_x, n_pixels_y, nb_bins_per_pixel, n_tran_bins, n_neighbors;
  float tran_edges[8];
  /* time axis and LUT, src/larndsim/sim_jax.py:141-286 */
  float t_sampling;
  int32_t n_ticks;           /* time_interval[1]/t_sampling + 1 (2001), incl. garbage tick 0 */
  int32_t signal_length;     /* L */
  int32_t lut_nx, lut_ny, lut_nt, n_templates;
  float long_diff_template[LSIM_MAX_TEMPLATES];
  /* front end, src/larndsim/fee_jax.py:55-71 and :168-279 */
  float threshold, gain, v_pedestal, v_cm, vref_minus_cm, adc_counts;
  float reset_noise, uncorr_noise, hit_prob_threshold;
  int32_t max_adc_values, fee_interval;
  /* parametrised current, src/larndsim/detsim_jax.py:618-639 */
  int32_t diffusion_in_current_sim, param_nticks;
  float param_dt;
  float param_ticks[64];
  /* adjoint: raw parameter values and d(vdrift)/d(eField) */
  float eField, lArDensity, dvdrift_deField;
  int32_t reserved[8];
  /* electron mobility parametrisation (ELECTRON_MOBILITY_PARAMS) and the
   * temperature factor (T/89)^-1.5 / 1000, for lsim_lut_stage1_theta */
  double mobility[6];
  double mobility_temp;
} LsimParams;

/* Device counters filled by the stage-1 calls (read after a sync). */
typedef struct LsimCounts {
  int32_t n_valid;      /* distinct pixel ids >= 0 with a main-pixel segment */
  int32_t n_em1;        /* distinct negative pixel ids < -1 (eventID -1 rows) */
  int32_t any_m1;       /* 1 if some main pixel id equals -1 */
  int32_t status;       /* device-detected LSIM_* error, 0 if none */
  int32_t max_slot;     /* largest number of segments sharing one pixel */
  int32_t bad_row;      /* first offending track row, or -1 */
  int32_t work;         /* internal work counter */
  int32_t n_main_rec;   /* main-bin records written by the last LUT accumulation */
  int32_t n_main_seg;   /* segments with main-bin records in the last LUT accumulation */
  int32_t n_big_slots;  /* internal: pixel slots whose segment lists are sorted by a whole block */
  int32_t n_heavy;      /* internal: pixels handed out first by the accumulation kernel */
  int32_t reserved[5];
} LsimCounts;

int lsim_abi_version(void);
const char *lsim_last_error(void);

/* sizeof(LsimParams), sizeof(LsimFieldMap), sizeof(LsimCounts), so a
 * binding can check its structure layout against the library. */
void lsim_struct_sizes(size_t *params, size_t *fields, size_t *counts);

/* Launch shapes of the LUT kernels, chosen by the Python autotuner
 * (larndsim_gb300/tune.py) per device and workload; zero fields keep the
 * defaults (pixel kernel: as many 128-thread blocks per SM as fit; main-bin
 * kernels: 1024 blocks of 8 warps).  Applies to the calling thread's later
 * calls.  Not part of the reference interface. */
typedef struct LsimTuning {
  int32_t pixel_blocks_per_sm;  /* persistent pixel-kernel blocks per SM, 1..occupancy limit */
  int32_t main_blocks;          /* blocks of the segment-major main-bin kernels */
  int32_t main_block_warps;     /* warps per main-bin block: 4 or 8 */
  int32_t reserved[5];
} LsimTuning;
void lsim_set_tuning(const LsimTuning *t);

/* Profiling hook: when both are non-null, the calling thread's subsequent
 * lsim_lut_stage2 / lsim_lut_adc / lsim_lut_grad calls record start/stop
 * (cudaEvent_t handles) on their stream around the pixel-accumulation
 * kernel, the dominant launch of the LUT path; null, null turns it off.
 * Not part of the reference interface. */
void lsim_set_kernel_events(void *start, void *stop);

/* ---------------------------------------------------------------- LUT */

/* Build the long-diffusion template bank from a raw response LUT:
 * out[k] = response convolved along time with the normalised Gaussian of
 * width sigmas[k] (taps -extent..extent, 'same' mode), out[0] = response.
 * Replaces load_lut, src/larndsim/consts_jax.py:387-449. */
int lsim_lut_build_templates(const float *response, int32_t nx, int32_t ny, int32_t nt,
                             const float *sigmas_dev, int32_t n_templates, int32_t extent,
                             float *templates_out, void *stream);

/* Bytes of the prepared tables derived from a template bank. */
size_t lsim_lut_tables_bytes(const LsimParams *p);

/* Derive the per-call LUT tables once per template bank: the L-tick
 * windows and the cumulative sums along time that the reference recomputes
 * on every call (src/larndsim/sim_jax.py:184-190, :221-222, :228). */
int lsim_lut_prepare(const LsimParams *p, const float *templates, void *tables, size_t tables_bytes,
                     void *stream);

/* ---------------------------------------------------------------- workspace */

/* Workspace bytes for n_rows track rows with event ids in [-1, n_events). */
size_t lsim_workspace_bytes(const LsimParams *p, int64_t n_rows, int32_t n_events);

/* ---------------------------------------------------------------- LUT mode */

/* Stage 1 of simulate_wfs: shift, quench, drift, sub-pixel binning and
 * 5x5 transverse weights per segment, then the pixel map (unique main
 * pixels, segments grouped by pixel).  Replaces simulate_drift_new
 * (src/larndsim/sim_jax.py:374-453) and the unique/renumbering step
 * (src/larndsim/sim_jax.py:715-725).  Writes an LsimCounts to counts_dev. */
int lsim_lut_stage1(const LsimParams *p, const LsimFieldMap *f, const float *tracks, int64_t n_rows,
                    int32_t n_events, void *ws, size_t ws_bytes, LsimCounts *counts_dev, void *stream);

/* lsim_lut_stage1 with the fit parameters read from device memory:
 * theta_dev[LSIM_NPARAM] = (Ab, kb, eField, lifetime, vdrift, long_diff,
 * tran_diff, lArDensity) replace the matching LsimParams fields, and the
 * quantities derived from them (eField*lArDensity, the drift velocity
 * get_vdrift of src/larndsim/consts_jax.py:192-217 and its derivative) are
 * recomputed on the device in float64 from p->mobility.  Every size the
 * later stages use is read from device memory, so a whole fit step
 * (this call, lsim_lut_grad, lsim_adam_step) can be captured once in a CUDA
 * graph and replayed with theta updated in place.  Not part of the
 * reference interface (the reference rebuilds its params pytree per step,
 * optimize/fit_params.py:704-731). */
int lsim_lut_stage1_theta(const LsimParams *p, const LsimFieldMap *f, const float *tracks, int64_t n_rows,
                          int32_t n_events, const float *theta_dev, void *ws, size_t ws_bytes,
                          LsimCounts *counts_dev, void *stream);

/* One Adam step on the fit parameters in place, in the reference's
 * "divide" normalisation (optimize/fit_params.py:89-95, :872-895: the
 * optimiser sees theta / scale and gradients * scale; optax.adam with
 * eps = 1e-8): m, v and the step count live in state[2 * LSIM_NPARAM + 1];
 * lr[i] = 0 freezes parameter i; a non-finite gradient skips the update
 * (fit_params.py:873-876). */
int lsim_adam_step(float *theta_dev, const float *grad_dev, const float *scale_dev, const float *lr_dev,
                   float *state_dev, float beta1, float beta2, float eps, void *stream);

/* Options of the fit step (GradientDescentFitter, optimize/fit_params.py:
 * 168-199 map_norm_to_phys / map_phys_to_norm, :781-895 the optax chain
 * and process_grads).  Arrays are indexed in LSIM_NPARAM order. */
#define LSIM_NORM_SIGMOID 0   /* phys = lo + (hi - lo) sigmoid(k u) (the reference's default) */
#define LSIM_NORM_EXP_LOG 1   /* phys = nom exp(k u) */
#define LSIM_NORM_DIVIDE 2    /* phys = u * norm */
#define LSIM_FIT_STATE 32     /* floats of fit-step state: m[8], v[8], u[8], step count, padding */
typedef struct LsimFitOptions {
  int32_t scheme;           /* LSIM_NORM_* */
  int32_t fit_mask;         /* bit i set: parameter i is fitted; the others never change */
  int32_t clip_from_range;  /* divide only: clip u to [down, up] / norm after each update */
  float norm_scale;         /* k: normalization_scale_sigmoid or _exp_log (> 0); 1 for divide */
  float max_clip_norm;      /* optax.clip_by_global_norm threshold; <= 0 or NaN: no clipping */
  float beta1, beta2, eps;  /* optax.adam (0.9, 0.999, 1e-8) */
  float lr[LSIM_NPARAM];
  float lo[LSIM_NPARAM], hi[LSIM_NPARAM];        /* sigmoid: the ranges' min and max */
  float nom[LSIM_NPARAM];                        /* exp_log: the ranges' nominal value (> 0) */
  float norm[LSIM_NPARAM];                       /* divide: params_normalization */
  float down[LSIM_NPARAM], up[LSIM_NPARAM];      /* clip_from_range: the ranges' down and up */
} LsimFitOptions;

/* Start a fit: for the fitted parameters, u = map_phys_to_norm(theta)
 * (optimize/fit_params.py:182-199; divide: u = 1 for non-zero values), and
 * theta <- map_norm_to_phys(u), the values the reference's first step
 * evaluates (its loss maps the normalised parameters back,
 * fit_params.py:713-731); Adam moments and step count cleared.
 * state_dev holds LSIM_FIT_STATE floats. */
int lsim_fit_init(float *theta_dev, const LsimFitOptions *opt, float *state_dev, void *stream);

/* One step of the reference's gradient-descent fitter on device, in place,
 * given grad_dev = dL/dtheta in physical units: the chain rule to the
 * normalised parameters (jax.value_and_grad with respect to norm_params,
 * fit_params.py:713-731), the NaN check that skips a step (:873-876), the
 * extra normalisation factor of the divide scheme (:878-882),
 * optax.clip_by_global_norm when enabled (:833-838), optax.adam per
 * parameter with its learning rate, clip_values_from_range (divide and
 * clip_from_range, :890-891) and the map back to physical values (:894).
 * Needs no host synchronisation, so it can run inside a captured fit step. */
int lsim_fit_step(float *theta_dev, const float *grad_dev, const LsimFitOptions *opt, float *state_dev,
                  void *stream);

/* Stage 2 of simulate_wfs: fill unique_pixels (p_pad rows: n_em1 negative
 * ids, n_m1 = p_pad - n_em1 - n_valid entries of -1, then the valid ids
 * ascending) and the waveforms wfs[p_pad][n_ticks-1] (garbage tick 0
 * dropped, as sim_jax.py:736 returns).  Rows with id < 0 are zero.
 * Replaces simulate_signals, src/larndsim/sim_jax.py:141-286. */
int lsim_lut_stage2(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows,
                    int32_t n_events, int64_t p_pad, int32_t n_em1, int32_t n_valid, float *wfs,
                    int32_t *unique_pixels, void *stream);

/* Pixel ids of the n_valid valid rows (ascending), as stage 2 orders them. */
int lsim_valid_pixels(const LsimParams *p, const void *ws, int64_t n_rows, int32_t n_events, int32_t n_valid,
                      int32_t *pids_out, void *stream);

/* Fused per-pixel forward: waveform accumulation + self-trigger FEE +
 * digitisation for the n_valid valid rows, without materialising the
 * waveforms.  adc_out/tick_out are [n_valid][max_adc_values]. */
int lsim_lut_adc(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows,
                 int32_t n_events, int32_t n_valid, const float *normals, float *adc_out,
                 float *tick_out, void *stream);

/* Adjoint of lsim_lut_adc: given dL/dADC (g_adc, [n_valid][H]), or an SSE
 * target (tgt_pids ascending + tgt_adc [n_tgt][H]) when g_adc is NULL,
 * recompute each pixel's waveform and FEE state, and accumulate dL/dtheta
 * for the LSIM_NPARAM parameters into grad_out[LSIM_NPARAM] (and the loss
 * into loss_out[0] when a target is given).  Gradient semantics follow
 * jax.value_and_grad through src/larndsim/sim_jax.py:141-286,
 * src/larndsim/fee_jax.py:55-71, :168-279 (fit_params.py:731). */
int lsim_lut_grad(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows,
                  int32_t n_events, int32_t n_valid, const float *normals, const float *g_adc,
                  const int32_t *tgt_pids, const float *tgt_adc, int64_t n_tgt, float *loss_out,
                  float *grad_out, float *adc_out, void *stream);

/* The store-the-waveforms variant of lsim_lut_grad: instead of recomputing
 * the waveforms, the adjoint reads the rows that lsim_lut_stage2 wrote to
 * wfs (P_pad x (n_ticks - 1), valid rows last) with the same workspace, and
 * reuses that pass's main-bin records.  Same outputs as lsim_lut_grad; it
 * trades the forward recomputation for P_pad x (n_ticks - 1) x 4 bytes of
 * stored waveforms (the reference keeps the forward's materialised arrays
 * for its backward pass, src/larndsim/sim_jax.py:141-286). */
int lsim_lut_grad_stored(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events,
                         const float *wfs, int64_t p_pad, int32_t n_valid, const float *normals, const float *g_adc,
                         const int32_t *tgt_pids, const float *tgt_adc, int64_t n_tgt, float *loss_out,
                         float *grad_out, float *adc_out, void *stream);

/* Vector-Jacobian product of simulate_wfs: for a cotangent g_wfs on the
 * waveforms lsim_lut_stage2 writes ([p_pad][n_ticks - 1], the n_valid valid
 * rows last), dL/dtheta = sum g_wfs * d wfs / d theta for the LSIM_NPARAM
 * parameters into grad_out.  ws holds the stage-1 state at the parameters
 * (lsim_lut_stage1 / lsim_lut_stage1_theta).  Rows with a negative pixel id
 * are zero in this library and carry no gradient.  Replaces jax.vjp /
 * jax.grad through simulate_wfs, src/larndsim/sim_jax.py:689-736, as the
 * reference's Taylor scans (tests/taylor/scan_utils.py:120-137) and
 * waveform-level losses use it. */
int lsim_lut_wfs_vjp(const LsimParams *p, const void *tables, const void *ws, int64_t n_rows, int32_t n_events,
                     const float *g_wfs, int64_t p_pad, int32_t n_valid, float *grad_out, void *stream);

/* ---------------------------------------------------------------- FEE + hits */

/* Self-trigger FEE + digitize on waveforms wfs[n_pix][n_t]: ADC values and
 * crossing ticks per hit ([n_pix][max_adc_values]).  normals (optional,
 * [n_pix][1 + 3*max_adc_values]) are standard-normal noise draws.
 * Replaces get_adc_values + digitize, src/larndsim/fee_jax.py:55-71, :168-279. */
int lsim_fee(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals,
             float *adc_out, float *tick_out, float *integral_out, void *stream);

/* Workspace bytes of lsim_fee_vjp for n_pix pixel rows. */
size_t lsim_fee_vjp_workspace_bytes(int64_t n_pix);

/* Vector-Jacobian product of lsim_fee's ADCs with respect to the waveforms:
 * for g_adc[n_pix][max_adc_values] = dL/dADC, writes g_wfs[n_pix][n_t] =
 * dL/dwfs (n_t a multiple of 4, at most 2048).  The gradient treatment is
 * the reference's under jax.vjp: crossing ticks, rejections and reset
 * positions carry none, the reset clamp max(C - C[e2], 0) and the digitize
 * clamps pass the cotangent where active (1/2 at exact ties).  normals
 * (optional) are the noise draws of the forward.  Replaces the backward of
 * get_adc_values + digitize, src/larndsim/fee_jax.py:55-71, :168-279. */
int lsim_fee_vjp(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, const float *normals,
                 const float *g_adc, float *g_wfs, void *ws, size_t ws_bytes, void *stream);

/* Workspace bytes of lsim_hits for n_pix pixel rows. */
size_t lsim_hits_workspace_bytes(int64_t n_pix, int32_t max_adc_values);

/* Hit assembly and compaction: hit probability (tick < tick_limit), pixel
 * centres, hit z, event ids and the row-major compaction of accepted hits.
 * Replaces simulate_stochastic's tail and parse_output,
 * src/larndsim/sim_jax.py:757-769, :619-647.  Output arrays hold up to
 * n_pix*max_adc_values entries; the count goes to nb_valid_dev. */
int lsim_hits(const LsimParams *p, const float *adc, const float *ticks, const int32_t *unique_pixels,
              int64_t n_pix, int32_t tick_limit, float *out_adc, float *out_x, float *out_y,
              float *out_z, float *out_ticks, float *out_hit_prob, int32_t *out_event,
              int32_t *out_pixels, int32_t *nb_valid_dev, void *ws, size_t ws_bytes, void *stream);

/* Hit assembly and compaction like lsim_hits, for callers that cannot
 * allocate device memory: a caller embedded in a framework that has
 * reserved the device memory for its own pool (JAX, for one, preallocates
 * most of the GPU at start-up, so a fresh cudaMalloc from a plug-in in that
 * process can fail), or code running under a fixed device-memory budget.
 * No counterpart in the reference (larnd-sim-jax allocates through XLA).
 * Instead of a workspace it uses a fixed scratch array compiled into the
 * library (64 KiB), so it accepts at most lsim_hits_noalloc_max_slots() =
 * 16384 * 1024 = 16,777,216 hit slots (n_pix * max_adc_values) and returns
 * LSIM_ERR_CAPACITY beyond that (max_adc_values outside 1..LSIM_MAX_HITS is
 * LSIM_ERR_INVALID).  It calls no cudaMalloc/cudaFree.
 * The scratch is reserved in a CUDA context when this library's module is
 * loaded there: under CUDA's default lazy module loading that is the first
 * call of lsim_fee, lsim_hits or lsim_hits_noalloc in the context, so a
 * process that will later give all free memory to another allocator should
 * make one such call first (or run with CUDA_MODULE_LOADING=EAGER).  The
 * first call in each context (the device's primary context, a context made
 * with cuCtxCreate, or a primary context re-created after cudaDeviceReset)
 * looks up the scratch's device address (cudaGetSymbolAddress) with that
 * context current and caches it by the context's id; make that first call
 * before any stream capture.  Every call in a context shares the one
 * scratch array: calls that overlap on the GPU (for example on two streams)
 * race and must be serialised by the caller.  The scratch needs no clearing
 * between calls: every entry a call reads is written by the same call
 * first. */
int64_t lsim_hits_noalloc_max_slots(void);
int lsim_hits_noalloc(const LsimParams *p, const float *adc, const float *ticks, const int32_t *unique_pixels,
                      int64_t n_pix, int32_t tick_limit, float *out_adc, float *out_x, float *out_y,
                      float *out_z, float *out_ticks, float *out_hit_prob, int32_t *out_event,
                      int32_t *out_pixels, int32_t *nb_valid_dev, void *stream);

/* ---------------------------------------------------------------- output side */

/* One set of hit columns, each of one entry per hit (the 8 outputs of
 * simulate_stochastic / simulate_parametrized, src/larndsim/sim_jax.py:738-769
 * and :339-372, in that order).  Read-only where it is an input. */
typedef struct LsimHitColumns {
  float *adc;
  float *pixel_x, *pixel_y, *pixel_z;
  float *ticks, *hit_prob;
  int32_t *event, *pixels;
} LsimHitColumns;

/* Workspace bytes of lsim_hit_records for n hits. */
size_t lsim_hit_records_workspace_bytes(int64_t n);

/* The hit records the simulate driver writes, optimize/simulate.py:129-176:
 * keep hit i when adc[i] - adc_lowest != 0 and event[i] != -1 (adc_lowest =
 * digitize(params, DISCRIMINATION_THRESHOLD), computed by the caller as the
 * reference does once per run), in input order.  For the kept rows write
 * out->event (required) and every other non-NULL column of *out (its input
 * column must then be non-NULL), the cleaned ADC adc - adc_lowest to
 * out_adc_clean and the charge adc2charge(adc) in ke-
 * (src/larndsim/losses_jax.py:380-383) to out_q (either may be NULL).
 * With run_start non-NULL, also list the runs of equal event in the kept
 * rows: run_event[r] (may be NULL) and run_start[r] for each run r, and
 * run_start[n_runs] = n_kept, which splits the records per event like the
 * reference's per-event groups (simulate.py:139-166) when, as in the
 * simulation's own output, the hits of each event are contiguous.
 * counts_dev (int64[2], device memory) receives n_kept and n_runs (the
 * runs are counted whether or not run_start is given).  Output
 * columns hold n entries, run_event n and run_start n + 1.  The cleaned ADC
 * is one float32 subtraction; the charge is computed in the form XLA gave
 * adc2charge for the reference's committed outputs (folded constants, one
 * fused multiply-add), which reproduces their charges bit for bit. */
int lsim_hit_records(const LsimParams *p, float adc_lowest, const LsimHitColumns *in, int64_t n,
                     const LsimHitColumns *out, float *out_adc_clean, float *out_q, int32_t *run_event,
                     int64_t *run_start, int64_t *counts_dev, void *ws, size_t ws_bytes, void *stream);

/* ---------------------------------------------------------------- input side */

/* Gather n_rows rows (row indices `rows`, device int64) of a (n_table,
 * n_fields <= 96) float32 track table resident in device memory into out
 * (n_rows, n_fields); with event_values non-NULL, column event_col of row r
 * becomes event_values[r] (the batch-local event id).  Replaces the row
 * selection and remap_event_ids_to_local of TracksDataset.__getitem__,
 * optimize/dataio.py:378-395 and :47-61 (the host computes the local ids
 * once per batch, as the reference does).  A row index outside the table
 * sets *status_dev (int32, device memory, zeroed by the caller) to
 * LSIM_ERR_INVALID and that row is not written. */
int lsim_gather_tracks(const float *table, int64_t n_table, int32_t n_fields, const int64_t *rows, int64_t n_rows,
                       int32_t event_col, const float *event_values, float *out, int32_t *status_dev, void *stream);

/* Pad a batch of n_rows rows in place to target_rows rows (the buffer holds
 * max(n_rows, target_rows) rows) and invalidate rows, as TracksDataset.pad_batch
 * / _invalidate_rows do (optimize/dataio.py:347-373): an invalidated row gets
 * eventID -1 in event_col, 0 in the columns whose col_roles entry is 1
 * (n_electrons, dE, dEdx, dx, long_diff, tran_diff) and -1 in those with 2
 * (trackID, pixel_plane); other columns keep their values, and are 0 in the
 * padding rows [n_rows, target_rows).  With n_local_events >= 0 the rows
 * [0, n_rows) whose eventID is >= 0 and whose integer part (truncated, like
 * numpy's astype(int64)) is not in [0, n_local_events) are invalidated too.
 * col_roles is a HOST array of n_fields entries in {0, 1, 2}, or NULL. */
int lsim_pad_tracks(float *batch, int64_t n_rows, int64_t target_rows, int32_t n_fields, int32_t event_col,
                    const int8_t *col_roles, int64_t n_local_events, void *stream);

/* Workspace bytes of lsim_chop_tracks for n_rows input tracks. */
size_t lsim_chop_workspace_bytes(int64_t n_rows);

/* Cut each of the n_rows tracks (float32 rows of f->n_fields <= 96 columns)
 * into max(ceil(length / precision), 1) steps: step k starts at
 * start + k * precision * direction, every step has dx = precision and
 * dE = dE * precision / length except the last, which ends at the track's
 * end and takes the remaining dx and dE; x, y, z become the step midpoints
 * and every other column is copied.  Output rows follow the input order.
 * Replaces chop_tracks, optimize/dataio.py:63-106, with its float32/float64
 * arithmetic (NumPy 2 promotion) reproduced bit for bit.
 * The number of output rows goes to *n_out_dev (int64, device memory), or
 * -1 when some track length is not finite (the reference's integer cast
 * fails there); the first min(n_out, out_capacity) rows are written to out.
 * A caller that does not know the count calls once with out = NULL and
 * out_capacity = 0, reads *n_out_dev, and calls again. */
int lsim_chop_tracks(const LsimFieldMap *f, const float *tracks, int64_t n_rows, double precision, float *out,
                     int64_t out_capacity, int64_t *n_out_dev, void *ws, size_t ws_bytes, void *stream);

/* ---------------------------------------------------------------- probabilistic front end */

/* Pixel centres, plane and event of each pixel id (any of the outputs may
 * be NULL).  Replaces id2pixel + get_pixel_coordinates,
 * src/larndsim/detsim_jax.py:264-306, as simulate_probabilistic uses them
 * (src/larndsim/sim_jax.py:807-811). */
int lsim_pixel_coords(const LsimParams *p, const int32_t *unique_pixels, int64_t n_pix, float *x_out, float *y_out,
                      int32_t *plane_out, int32_t *event_out, void *stream);

/* Workspace bytes of lsim_fee_prob (one flag per hit step). */
size_t lsim_fee_prob_workspace_bytes(const LsimParams *p);

/* Probabilistic self-trigger front end on waveforms wfs[n_pix][n_t]
 * (n_t <= 2048): the beam search over n_paths (fee_paths_scaling <= 32)
 * paths and p->max_adc_values hit steps of
 * get_adc_values_average_noise_vmap, src/larndsim/fee_jax.py:386-461
 * (step _find_one_hit_step :334-384, log_diff_ndtr :33-53), with noise
 * sigma p->reset_noise (> 0) and the whole batch stopped once no pixel keeps
 * a total path probability above stop_threshold.  Outputs, each optional:
 * log_prob_out and charge_out [n_pix][H][n_t - 1] (the reference's two
 * outputs after its moveaxis), and the reductions of get_average_hit_values
 * (fee_jax.py:463-480) applied to exp(log_prob) and digitize(charge):
 * exp_tick_out, exp_adc_out, lambda_out [n_pix][H] (all three or none). */
int lsim_fee_prob(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                  float stop_threshold, float *log_prob_out, float *charge_out, float *exp_tick_out,
                  float *exp_adc_out, float *lambda_out, void *ws, size_t ws_bytes, void *stream);

/* Workspace bytes of lsim_fee_prob_vjp (the forward's per-step path states). */
size_t lsim_fee_prob_vjp_workspace_bytes(const LsimParams *p, int64_t n_pix, int32_t n_paths);

/* Vector-Jacobian product of lsim_fee_prob with respect to the waveforms:
 * given cotangents on any of its outputs (g_log_prob, g_charge
 * [n_pix][H][n_t - 1]; g_e_tick, g_e_adc, g_lambda [n_pix][H], all three or
 * none), writes g_wfs[n_pix][n_t].  The forward is re-run with each step's
 * paths recorded; the reverse pass follows jax.grad of
 * get_adc_values_average_noise_vmap (src/larndsim/fee_jax.py:334-461) and
 * get_average_hit_values (:463-480): top-K choices held, the running
 * maximum's cotangent routed to the tick where it was first attained (the
 * reference splits exact ties), jax.scipy.special.log_ndtr's derivative
 * exp(norm_logpdf(x) - log_ndtr(x)). */
int lsim_fee_prob_vjp(const LsimParams *p, const float *wfs, int64_t n_pix, int32_t n_t, int32_t n_paths,
                      float stop_threshold, const float *g_log_prob, const float *g_charge, const float *g_e_tick,
                      const float *g_e_adc, const float *g_lambda, float *g_wfs, void *ws, size_t ws_bytes,
                      void *stream);

/* ---------------------------------------------------------------- fit losses */

/* Workspace bytes of lsim_mse_adc for n_hits predicted and n_ref reference hits. */
size_t lsim_mse_adc_workspace_bytes(int64_t n_hits, int64_t n_ref);

/* The hit-level loss mse_adc, src/larndsim/losses_jax.py:60-79 (with
 * rbf_kernel and mmd, :13-39): the weighted maximum mean discrepancy with a
 * Gaussian kernel of width sigma between the predicted hits (x, y, z,
 * event, weight w = Q * hit_prob) and the reference hits, on the stacked
 * coordinates (x + event * 1e5, y, z), plus lambda_q times the squared
 * relative difference of the total weights.  out[0..2] = loss, MMD term,
 * charge term (device floats).  grad_w and grad_z (optional, [n_hits]) get
 * dL/dw and dL/dz of the predicted hits; x, y and the events carry no
 * gradient.  Hits of different events never interact (their kernel value
 * is 0 in float32); inputs ordered by event run fastest. */
int lsim_mse_adc(const float *x, const float *y, const float *z, const int32_t *event, const float *w, int64_t n_hits,
                 const float *ref_x, const float *ref_y, const float *ref_z, const int32_t *ref_event,
                 const float *ref_w, int64_t n_ref, float sigma, float lambda_q, float *out, float *grad_w,
                 float *grad_z, void *ws, size_t ws_bytes, void *stream);

/* Workspace bytes of lsim_nll_loss / lsim_chamfer_3d. */
size_t lsim_nll_workspace_bytes(int64_t n_hits, int64_t n_ref);
size_t lsim_chamfer_workspace_bytes(int64_t n_hits, int64_t n_ref);

/* nll_loss, src/larndsim/losses_jax.py:329-359: the Poisson-process
 * negative log-likelihood sum(hit_prob) - sum_j [ref_hit_prob_j > 0.5]
 * log(lambda_j + 1e-10), lambda_j = sum_i hit_prob_i exp(-|p_i - r_j|^2 /
 * (2 sigma^2)) on the 4-d points (x + event * 1e9, y, z, q) with
 * q = Q / adc_norm given by the caller.  out[0..2] = loss, sum(hit_prob),
 * the log-likelihood sum; optional gradients [n_hits] with respect to q, z
 * and hit_prob.  (The reference's padding rows at -1e9 with zero
 * probabilities add nothing and are not needed.) */
int lsim_nll_loss(const float *x, const float *y, const float *z, const float *q, const int32_t *event,
                  const float *hit_prob, int64_t n_hits, const float *ref_x, const float *ref_y, const float *ref_z,
                  const float *ref_q, const int32_t *ref_event, const float *ref_hit_prob, int64_t n_ref, float sigma,
                  float *out, float *grad_q, float *grad_z, float *grad_hit_prob, void *ws, size_t ws_bytes,
                  void *stream);

/* chamfer_distance_3d_og as chamfer_3d calls it, src/larndsim/losses_jax.py:
 * 181-229: nearest neighbours both ways on (x + event * 1e9, y, z) in
 * float32 (first index on ties); loss = sum over hits closer than 1e4 of
 * min distance x own weight x neighbour weight.  The caller passes the
 * weights Q / adc_norm and the padded rows (zeros, event 0) the reference
 * appends.  out[0] = loss; optional gradients [n_hits] with respect to w
 * and z (the neighbour choices carry none).  At most 2^31 - 1 hits a side. */
int lsim_chamfer_3d(const float *x, const float *y, const float *z, const int32_t *event, const float *w,
                    int64_t n_hits, const float *ref_x, const float *ref_y, const float *ref_z,
                    const int32_t *ref_event, const float *ref_w, int64_t n_ref, float *out, float *grad_w,
                    float *grad_z, void *ws, size_t ws_bytes, void *stream);

/* ---------------------------------------------------------------- likelihood losses on distributions */

/* Workspace bytes of lsim_prob_llhd for n_hits target hits. */
size_t lsim_prob_llhd_workspace_bytes(int64_t n_hits);

/* ProbabilisticLossStrategy.compute, optimize/strategies.py:338-567: the
 * likelihood of the target hits (pixel id, tick, ADC count; n_hits) under
 * the probabilistic front end's distributions of the simulated pixels
 * (sim_pixels [n_pix], sorted ascending, -1 pads first; log_prob and
 * adcs_distrib [n_pix][n_values][n_ticks]).  Each hit is matched by a
 * lower-bound search, its occurrence index within its run of equal target
 * ids (compute_occurrence_indices, :14-40) picks the hit row, and the
 * entry at its tick (jax.numpy indexing: negative from the end, clamped)
 * gives T = sum of max(log_prob, log(eps)) over matched hits + log(eps) x
 * the number of hits whose lower bound holds another id, and C = sum of
 * -0.5 ((q_tgt - q) / s)^2 - 0.5 log(2 pi s^2), s = sigma_charge / 1000,
 * q = adc2charge of the distribution's ADC (0 for unmatched hits).
 * out[0..3] = loss sqrt(T C), -C, -T, -penalty (the reference's loss and
 * aux).  With g_log_prob or g_adcs (dense, same shape as the
 * distributions; zeroed here) the gradient of the loss times g_loss[0]
 * (device float, null = 1) is written; ties of the log(eps) clamp get 1/2,
 * as jax.lax.max's derivative gives.  n_hits > 0 needs n_pix > 0. */
int lsim_prob_llhd(const LsimParams *p, const int32_t *sim_pixels, int64_t n_pix, int32_t n_values, int32_t n_ticks,
                   const float *log_prob, const float *adcs_distrib, const int32_t *tgt_pixels,
                   const int32_t *tgt_ticks, const float *tgt_adcs, int64_t n_hits, double sigma_charge, double eps,
                   const float *g_loss, float *out, float *g_log_prob, float *g_adcs, void *ws, size_t ws_bytes,
                   void *stream);

/* Workspace bytes of lsim_llhd_loss for n_rows rows. */
size_t lsim_llhd_workspace_bytes(int64_t n_rows);

/* llhd_loss, src/larndsim/losses_jax.py:414-441: out[0] = -sum over rows i
 * of [log(p_i + 1e-10) + c_i] where tick_i < n_ticks - 3 and
 * log(no_hit_prob_i + 1e-10) otherwise, p_i = ticks_prob[i][tick_i],
 * c_i = -0.5 ((charge_mc_i - charge_distrib[i][tick_i]) / sigma)^2 -
 * 0.5 log(2 pi sigma^2).  Optional gradients (times g_loss[0], device float,
 * null = 1): dense g_ticks_prob and g_charge_distrib [n_rows][n_ticks]
 * (zeroed here), g_no_hit_prob and g_charge_mc [n_rows]. */
int lsim_llhd_loss(const float *ticks_prob, const int32_t *ticks_mc, const float *no_hit_prob,
                   const float *charge_distrib, const float *charge_mc, int64_t n_rows, int32_t n_ticks, double sigma,
                   const float *g_loss, float *out, float *g_ticks_prob, float *g_no_hit_prob, float *g_charge_distrib,
                   float *g_charge_mc, void *ws, size_t ws_bytes, void *stream);

/* Workspace bytes of lsim_occurrence_indices for n ids. */
size_t lsim_occurrence_workspace_bytes(int64_t n);

/* compute_occurrence_indices, optimize/strategies.py:14-40: out[i] = i minus
 * the start of the run of equal consecutive ids holding i (a max-scan of
 * run starts); n < 2^31 - 1. */
int lsim_occurrence_indices(const int32_t *ids, int64_t n, int32_t *out, void *ws, size_t ws_bytes, void *stream);

/* ---------------------------------------------------------------- parametrised mode */

/* Stage 1 of simulate_parametrized: shift, quench, drift, Monte-Carlo
 * diffusion offsets (normals [n_rows][3], supplied), pixel of each
 * electron, pixel map.  Replaces simulate_drift + generate_electrons +
 * get_pixels, src/larndsim/sim_jax.py:122-139, src/larndsim/detsim_jax.py:376-400, :477-491.
 * Implements the reference's default current model with longitudinal
 * smearing (diffusion_in_current_sim = true, current_model_diff); false
 * returns LSIM_ERR_UNSUPPORTED. */
int lsim_param_stage1(const LsimParams *p, const LsimFieldMap *f, const float *tracks, int64_t n_rows,
                      int32_t n_events, const float *normals, void *ws, size_t ws_bytes,
                      LsimCounts *counts_dev, void *stream);

/* Stage 2 of simulate_parametrized: unique pixels and waveforms from the
 * parametrised (EMG-smoothed) induced current.  Replaces
 * simulate_signals_parametrized + current_mc + accumulate_signals_parametrized,
 * src/larndsim/sim_jax.py:289-335, src/larndsim/detsim_jax.py:207-228, :581-639. */
int lsim_param_stage2(const LsimParams *p, const void *ws, int64_t n_rows, int32_t n_events,
                      int64_t p_pad, int32_t n_em1, int32_t n_valid, float *wfs, int32_t *unique_pixels,
                      void *stream);

/* Vector-Jacobian product of simulate_parametrized's waveforms: for a
 * cotangent g_wfs on the rows lsim_param_stage2 writes ([p_pad][n_ticks - 1],
 * the n_valid valid rows last), dL/dtheta into grad_out[LSIM_NPARAM].  ws
 * holds the lsim_param_stage1 state at the parameters (including the
 * per-segment partial derivatives it records); the Monte-Carlo offsets are
 * held fixed and pixel and tick assignments carry no gradient, as under
 * jax.grad of simulate_parametrized (src/larndsim/sim_jax.py:339-372,
 * src/larndsim/detsim_jax.py:581-639; the gradient params_loss_parametrized
 * takes in optimize/fit_params.py). */
int lsim_param_wfs_vjp(const LsimParams *p, const void *ws, int64_t n_rows, int32_t n_events, const float *g_wfs,
                       int64_t p_pad, int32_t n_valid, float *grad_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* LSIM_H */
