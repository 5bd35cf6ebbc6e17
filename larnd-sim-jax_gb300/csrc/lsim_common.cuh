// Shared definitions of the sm_103a larnd-sim kernels: per-segment records,
// workspace layout, and helpers that reproduce the reference's exact index
// arithmetic (JAX float floor_divide / remainder, Python integer division,
// int32 pixel-id packing).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "lsim.h"

namespace lsim {

constexpr int kWarp = 32;
constexpr int kMaxNeigh = 8;             // number_pix_neighbors supported: 0..8
constexpr int kMaxTran = 5;              // nb_tran_diff_bins supported: 5
constexpr int kMainSub = 5;              // main-bin LUT sub-positions (nb_bins_per_pixel / 2)
constexpr int kMaxSlotSegments = (1 << 23) - 1;   // segments sharing one principal pixel
constexpr int kWinSamples = 160;         // padded window samples k = -1 .. 158 (signal_length <= 158)
constexpr int kScanTile = 2048;          // slots per scan block
constexpr int kSortLocal = 64;           // slot lists up to this length are sorted by one thread
constexpr int kThetaDerived = 16;
constexpr int kScanThreads = 256;

// --------------------------------------------------------------- records

// Per-segment forward record of LUT mode (96 bytes).
struct __align__(16) SegFwd {
  float ne;          // electrons after recombination, lifetime and TPC mask
  float frac;        // t0/t_sampling - cathode tick (sub-tick shift)
  float qa, qb, qc;  // quadratic long-diffusion template weights (sim_jax.py:166-168)
  int cath;          // cathode tick c = clip(floor(t0/ts), 0, Nt-1)
  int tidx;          // central template index, clip(searchsorted, 1, T-2)
  int bx, by;        // sub-pixel bin indices (get_bin_shifts)
  float ex[kMaxTran], ey[kMaxTran];  // 1-D transverse bin integrals
  int plane, event;
  float sigT, t0, ld;
};

// Per-segment adjoint record (96 bytes): partial derivatives of the
// per-segment quantities with respect to the LSIM_NPARAM parameters.
struct __align__(16) SegAdj {
  float dne[5];      // d ne / d(Ab, kb, eField, lifetime, lArDensity)
  float dsig[2];     // d sigmaT / d(eField, tran_diff)
  float dld[2];      // d longdiff_ticks / d(eField, long_diff)
  float dt0;         // d t0 / d eField
  float dqa, dqb, dqc;  // d(a, b, c) / d longdiff_ticks
  float dex[kMaxTran], dey[kMaxTran];  // d ex_i / d sigmaT, d ey_j / d sigmaT
  float pad[1];
};

// Compact copy of what the neighbour passes of the pixel kernel read per
// contribution, one 16-byte load each: electrons, sub-tick fraction, cathode
// tick, and the sub-pixel bins packed as two int16 (bx in bits 0..15, by in
// 16..31; stage 1 rejects segments with charge whose bins do not fit).
struct __align__(16) SegNb {
  float ne, frac;
  int cath;
  int bxy;
};
// Compact adjoint partials of the neighbour passes: d ne / d(Ab, kb,
// eField, lifetime) in the first float4; d ne / d lArDensity and d t0 /
// d eField in the second.
struct __align__(16) SegNbAdj {
  float4 dne03;
  float4 dne4_dt0;
};

// Per-segment record of parametrised mode (64 bytes).
struct __align__(16) SegPar {
  float ne;
  float t0f;         // t0 - t0_tick * t_sampling
  int t0_tick;       // int(t0/ts + 0.5)
  float xd, yd;      // |x_e - pixel centre|, |y_e - pixel centre|
  float sigma;       // long diffusion in time units (sigma_L / vdrift)
  int plane, event;
  int px, py;
  float pad[6];
};

// Per-segment adjoint record of parametrised mode, stored in the SegAdj
// slot: the non-zero partial derivatives of the current model's inputs.
struct __align__(16) SegParAdj {
  float dne[5];      // d ne / d(Ab, kb, eField, lifetime, lArDensity)
  float dxd[2];      // d x_dist / d(eField, tran_diff)
  float dyd[2];      // d y_dist / d(eField, tran_diff)
  float dt0f[2];     // d t0f / d(eField, long_diff)
  float dsig[2];     // d sigma / d(eField, long_diff)
  float pad[11];
};
static_assert(sizeof(SegParAdj) <= sizeof(SegAdj), "parametrised adjoint record fits the SegAdj slot");

// --------------------------------------------------------------- layout

struct Grid {
  int nxe, nye, ntpc;          // extended pixel grid per (event, plane)
  int n;                       // neighbour radius (number_pix_neighbors)
  int h;                       // halo = max(n, 1): main bins reach the 3x3 pixels around a segment's pixel
  int64_t plane_stride, event_stride, G;
};

__host__ __device__ inline Grid make_grid(const LsimParams &p, int32_t n_events) {
  Grid g;
  g.n = p.n_neighbors;
  g.h = g.n > 1 ? g.n : 1;
  g.nxe = p.n_pixels_x + 2 * g.h;
  g.nye = p.n_pixels_y + 2 * g.h;
  g.ntpc = p.n_tpc;
  g.plane_stride = (int64_t)g.nxe * g.nye;
  g.event_stride = g.plane_stride * g.ntpc;
  g.G = g.event_stride * (int64_t)(n_events + 1);   // events -1 .. n_events-1
  return g;
}

// Whether grid slot t is a simulated pixel: it holds segments, lies inside
// the detector (not in the halo) and belongs to an event >= 0.
__device__ __forceinline__ bool slot_is_pixel(const Grid &g, const int32_t *cnt, int64_t t) {
  if (t < 0 || t >= g.G || cnt[t] <= 0) return false;
  const int64_t ev = t / g.event_stride;
  if (ev == 0) return false;
  const int64_t inplane = (t - ev * g.event_stride) % g.plane_stride;
  const int pye = (int)(inplane / g.nxe), pxe = (int)(inplane % g.nxe);
  return pxe >= g.h && pxe < g.nxe - g.h && pye >= g.h && pye < g.nye - g.h;
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Workspace carve-up shared by all entry points.
struct Workspace {
  LsimCounts *counts;
  SegFwd *segf;
  SegAdj *sega;
  SegPar *segp;
  int32_t *key, *pid;
  int32_t *cnt, *off, *cursor;
  int32_t *seg_list, *pix_slot, *em1_slot;
  int32_t *big_slots;       // slots with more than kSortLocal segments (sorted by a block each)
  float *theta_derived;     // fit parameters and derived quantities for lsim_lut_stage1_theta (kThetaDerived)
  int32_t *heavy;           // pixels with many contributions, handed out first (count in counts->reserved[0])
  uint8_t *heavy_flag;      // per valid pixel: 1 if it is in the heavy list
  int32_t *scan_blocks;     // 3 ints per scan block (+1 block)
  float *pix_out;           // per valid pixel: [loss, 8 gradient terms] (kPixRec floats)
  double *red_partials;     // fixed-order reduction partials (kRedSlots * 16 doubles)
  float *mrec;              // main-bin records: kMainRecPerSeg per segment, kMainRecFloats each
  uint32_t *fee_masks;      // per pixel-kernel warp: front-end reset masks (kFeeMaskWords)
  int32_t *tgt_index;       // per valid pixel: row of the loss target with the same pixel id, or -1
  float *main_out;          // per segment: main-bin adjoint [0, 8 gradient terms] (kPixRec floats)
  int32_t *seg_order;       // segments with main-bin records, grouped by template index
  int32_t *tidx_hist;       // kMaxTemplates counts, then kMaxTemplates cursors
  SegNb *segn;              // per segment: compact neighbour-pass record (LUT mode)
  SegNbAdj *segna;          // per segment: compact neighbour-pass adjoint partials (LUT mode)
  SegNb *lnb;               // segn in slot-list order (seg_list positions): a slot's run reads contiguously
  SegNbAdj *lna;            // segna in slot-list order
  size_t bytes;
};

constexpr int kPixRec = 12;      // floats per per-pixel record (loss + 8 grads, padded)
constexpr int kRedSlots = 4096;  // reduction blocks (pixels + main-bin warps + target-only)
constexpr int kMainWarps = 8192; // warps of the segment-major main-bin kernels
constexpr int kMaxTemplates = 1024;    // long-diffusion templates the main-bin ordering supports
constexpr int kMainRecPerSeg = 4;      // a segment's main bins cover at most 2 x 2 pixels
constexpr int kMainRecFloats = 164;    // window of 160 samples + d(corr)/d(frac), padded to 16 bytes
constexpr int kMaxPixelWarps = 8192;   // warps of the persistent pixel kernel
constexpr int kFeeMaskWords = LSIM_MAX_HITS * 64;   // reset masks per warp: hits x (2 words per lane)

inline Workspace carve_workspace(void *base, const LsimParams &p, int64_t n_rows, int32_t n_events) {
  Grid g = make_grid(p, n_events);
  int64_t nscan = (g.G + kScanTile - 1) / kScanTile + 1;
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
  size_t o_counts = take(sizeof(LsimCounts));
  size_t o_segf = take(sizeof(SegFwd) * (size_t)n_rows);
  size_t o_sega = take(sizeof(SegAdj) * (size_t)n_rows);
  size_t o_segp = take(sizeof(SegPar) * (size_t)n_rows);
  size_t o_key = take(4 * (size_t)n_rows);
  size_t o_pid = take(4 * (size_t)n_rows);
  size_t o_cnt = take(4 * (size_t)g.G);
  size_t o_off = take(4 * (size_t)g.G);
  size_t o_cur = take(4 * (size_t)g.G);
  size_t o_list = take(4 * (size_t)n_rows);
  size_t o_pixs = take(4 * (size_t)n_rows);
  size_t o_em1 = take(4 * (size_t)n_rows);
  size_t o_big = take(4 * ((size_t)n_rows / (kSortLocal + 1) + 1));
  size_t o_theta = take(4 * (size_t)kThetaDerived);
  size_t o_heavy = take(4 * (size_t)n_rows);
  size_t o_hflag = take((size_t)n_rows);
  size_t o_scan = take(3 * 4 * (size_t)nscan);
  size_t o_pix = take(4 * (size_t)kPixRec * (size_t)n_rows);
  size_t o_red = take(8 * (size_t)kRedSlots * 16);
  size_t o_mrec = take(4 * (size_t)kMainRecFloats * kMainRecPerSeg * (size_t)n_rows);
  size_t o_mout = take(4 * (size_t)kPixRec * (size_t)n_rows);
  size_t o_sord = take(4 * (size_t)n_rows);
  size_t o_thist = take(4 * (size_t)kMaxTemplates * 2);
  size_t o_fmask = take(4 * (size_t)kFeeMaskWords * kMaxPixelWarps);
  size_t o_tidx = take(4 * (size_t)n_rows);
  size_t o_segn = take(sizeof(SegNb) * (size_t)n_rows);
  size_t o_segna = take(sizeof(SegNbAdj) * (size_t)n_rows);
  size_t o_lnb = take(sizeof(SegNb) * (size_t)n_rows);
  size_t o_lna = take(sizeof(SegNbAdj) * (size_t)n_rows);
  Workspace w;
  char *b = (char *)base;
  w.counts = (LsimCounts *)(b + o_counts);
  w.segf = (SegFwd *)(b + o_segf);
  w.sega = (SegAdj *)(b + o_sega);
  w.segp = (SegPar *)(b + o_segp);
  w.key = (int32_t *)(b + o_key);
  w.pid = (int32_t *)(b + o_pid);
  w.cnt = (int32_t *)(b + o_cnt);
  w.off = (int32_t *)(b + o_off);
  w.cursor = (int32_t *)(b + o_cur);
  w.seg_list = (int32_t *)(b + o_list);
  w.pix_slot = (int32_t *)(b + o_pixs);
  w.em1_slot = (int32_t *)(b + o_em1);
  w.big_slots = (int32_t *)(b + o_big);
  w.theta_derived = (float *)(b + o_theta);
  w.heavy = (int32_t *)(b + o_heavy);
  w.heavy_flag = (uint8_t *)(b + o_hflag);
  w.scan_blocks = (int32_t *)(b + o_scan);
  w.pix_out = (float *)(b + o_pix);
  w.red_partials = (double *)(b + o_red);
  w.mrec = (float *)(b + o_mrec);
  w.main_out = (float *)(b + o_mout);
  w.seg_order = (int32_t *)(b + o_sord);
  w.tidx_hist = (int32_t *)(b + o_thist);
  w.fee_masks = (uint32_t *)(b + o_fmask);
  w.tgt_index = (int32_t *)(b + o_tidx);
  w.segn = (SegNb *)(b + o_segn);
  w.segna = (SegNbAdj *)(b + o_segna);
  w.lnb = (SegNb *)(b + o_lnb);
  w.lna = (SegNbAdj *)(b + o_lna);
  w.bytes = off;
  return w;
}

// Prepared LUT tables (see lsim_lut_prepare).
struct Tables {
  const float4 *wmp;   // [T][5][5][kWinSamples]: (T[i-1], T[i], T[i+1], 0) windows, i in [1, T-2], padded as w0
  const float *cm;     // [T][5][5][Nt] cumulative sums of the main sub-positions
  const float *w0;     // [nx][ny][kWinSamples] template-0 windows: 0, T0[Nt-L .. Nt-1], zeros
  const float *c0;     // [nx][ny][Nt] template-0 cumulative sums
};

inline size_t tables_layout(const LsimParams &p, size_t *o_wmp, size_t *o_cm, size_t *o_w0, size_t *o_c0) {
  const size_t T = p.n_templates, L = p.signal_length, Nt = p.lut_nt;
  const size_t nx = p.lut_nx, ny = p.lut_ny, m = kMainSub * kMainSub;
  size_t off = 0;
  *o_wmp = off; off += align256(sizeof(float4) * T * m * kWinSamples);
  *o_cm = off;  off += align256(sizeof(float) * T * m * Nt);
  *o_w0 = off;  off += align256(sizeof(float) * nx * ny * kWinSamples);
  *o_c0 = off;  off += align256(sizeof(float) * nx * ny * Nt);
  return off;
}

inline Tables carve_tables(const void *base, const LsimParams &p) {
  size_t a, b, c, d;
  tables_layout(p, &a, &b, &c, &d);
  const char *x = (const char *)base;
  Tables t;
  t.wmp = (const float4 *)(x + a);
  t.cm = (const float *)(x + b);
  t.w0 = (const float *)(x + c);
  t.c0 = (const float *)(x + d);
  return t;
}

// --------------------------------------------------------------- exact arithmetic

// jnp.floor_divide for float32 (fmod-based divmod, quotient rounded half
// away from zero), as used by get_bin_shifts (detsim_jax.py:505-507) and
// get_pixels (detsim_jax.py:482-483).
__device__ __forceinline__ float jax_floordiv_f32(float a, float b) {
  float mod = fmodf(a, b);
  float div = __fdiv_rn(__fsub_rn(a, mod), b);
  if (mod != 0.0f && ((b < 0.0f) != (mod < 0.0f))) div = __fsub_rn(div, 1.0f);
  return roundf(div);
}

// jnp.remainder for float32 (result has the sign of the divisor).
__device__ __forceinline__ float jax_rem_f32(float a, float b) {
  float mod = fmodf(a, b);
  if (mod != 0.0f && ((mod < 0.0f) != (b < 0.0f))) mod = __fadd_rn(mod, b);
  return mod;
}

// Python integer floor division / modulo.
__host__ __device__ __forceinline__ int ifloordiv(int a, int b) {
  int q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}
__host__ __device__ __forceinline__ int imod(int a, int b) {
  int r = a % b;
  if (r != 0 && ((r < 0) != (b < 0))) r += b;
  return r;
}

// pixel2id (detsim_jax.py:230-244) with the int32 wrap-around of JAX
// without x64: -1 outside the pixel plane.
__host__ __device__ __forceinline__ int32_t pixel2id(const LsimParams &p, int px, int py, int plane, int event) {
  if (px >= p.n_pixels_x || py >= p.n_pixels_y || px < 0 || py < 0) return -1;
  uint32_t pid = ((uint32_t)event * (uint32_t)p.n_tpc + (uint32_t)plane) * (uint32_t)p.n_pixels_y + (uint32_t)py;
  pid = pid * (uint32_t)p.n_pixels_x + (uint32_t)px;
  return (int32_t)pid;
}

__device__ __forceinline__ float border(const LsimParams &p, int plane, int axis, int side) {
  return p.tpc_borders[(plane * 3 + axis) * 2 + side];
}

// searchsorted(side='left') on the long-diffusion template grid.
__device__ __forceinline__ int searchsorted_left(const float *grid, int n, float v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (grid[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Inclusive block scan of one int64 per thread (blockDim.x a multiple of 32,
// at most 1024); returns the inclusive prefix, *total gets the block total.
// warp_tot holds blockDim.x / 32 entries.
__device__ __forceinline__ int64_t block_scan_i64(int64_t v, int64_t *warp_tot, int64_t *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int i = 0; i < nw; ++i) {
      int64_t t = warp_tot[i];
      warp_tot[i] = run;
      run += t;
    }
    *total = run;
  }
  __syncthreads();
  x += warp_tot[wid];
  return x;
}

__device__ __forceinline__ void set_status(LsimCounts *c, int code, int row) {
  atomicCAS(&c->status, 0, code);
  atomicMin(&c->bad_row, row);
}

}  // namespace lsim
