// Pixel-major LUT accumulation: one warp owns one pixel row at a time
// (persistent warps pull rows from a work counter), holds the 2001-tick
// waveform in shared memory and adds every contribution of every segment
// whose principal pixel lies within number_pix_neighbors of it.  No global
// atomics touch waveform data; the per-pixel contribution order is fixed,
// so results are deterministic.
//
// Reference: simulate_signals (sim_jax.py:141-286).  A contribution of
// segment s to pixel p places, at window origin col0 = Nt - L - c - 1,
//   r = 0      : corr * frac
//   r = 1      : corr * (1 - frac) + V[0] * frac
//   r = 2..L   : V[r-2] * (1 - frac) + V[r-1] * frac
//   r = L + 1  : V[L-1] * (1 - frac)
// where V[k] = sum over the main bins on p of q_ij * (T_i b + T_{i-1} a +
// T_{i+1} c)[cx, cy, Nt-L+k]  plus, when p is a neighbour, T_0[cx, cy,
// Nt-L+k] * n_e; corr is the matching cumulative-sum boundary correction.
// Value parts land only in waveform columns [2, Nticks-1], correction parts
// only in [1, Nticks-2] (the index remaps of sim_jax.py:177-178, :243-244).
//
// Work split.  Neighbour parts (every slot of the (2n+1)^2 neighbourhood but
// the centre, ~300 per pixel on dense events) go through a batched path:
// 32 contributions at a time, lane j computes contribution j's descriptor
// (LUT row, window origin, sub-tick fraction, charge, boundary correction,
// adjoint partials) so the per-contribution L2 latency overlaps across
// lanes; the window pass then streams two contributions' LUT rows with all
// loads in flight.  Main-bin parts (segments in the 3x3 slots whose bins
// fall on the pixel) take a per-contribution path over up to 5x5 grouped
// LUT sub-positions.
#include "lsim_internal.cuh"
#include "lsim_bins.cuh"
#include "lsim_fee.cuh"

namespace lsim {

constexpr int kAccWarps = 4;
constexpr int kRowPad = 3;            // row[col] at buf[kRowPad + col]: col 1 is 16-byte aligned
constexpr int kRowFloats = 2052;      // >= kRowPad + n_ticks (2001), multiple of 4
constexpr int kMaxList = 81;          // (2 * 4 + 1)^2 neighbourhood slots

// Descriptor of one contribution, written by one lane of the batch setup
// and read by the whole warp with 16-byte broadcast loads.
//   neighbour, forward:  w = (n_e (1 - f), n_e f, D, pack)
//   neighbour, adjoint:  w = (f, 1 - f, D, pack), g0 = (dD/df, n_e dt0/ts, dn_e[4], 0),
//                        g1 = dn_e[0..3]
//   main-bin record:     w = (1 - f, f, d corr/df, pack), g0 = (dt0/ts, record index, 0, 0)
// with pack = window origin + 16384 in bits 16..30, the LUT row in bits
// 0..14 (0 for records) and bit 15 set for a window that is not interior;
// pack = -1 marks an empty descriptor (valid packs are non-negative).
struct __align__(16) NDesc {
  float4 w, g0, g1;
};
struct NBatch {
  NDesc d[kWarp];
};
constexpr int kPackEdge = 1 << 15;
constexpr int kPackRowMask = kPackEdge - 1;

constexpr int kPackCbBias = 1 << 14;   // window origins in [-16384, 16383]

__device__ __forceinline__ float pack_window(int row, int cb, bool interior) {
  return __int_as_float(((cb + kPackCbBias) << 16) | row | (interior ? 0 : kPackEdge));
}
__device__ __forceinline__ int pack_cb(int pk) { return (pk >> 16) - kPackCbBias; }

// Compacted neighbourhood slot list of one pixel.  cd packs the slot's
// segment count (bits 8..31, at most kMaxSlotSegments, checked in stage 1)
// with its offset from the pixel, (dx + 4) | (dy + 4) << 4 (bits 0..7).
struct ListSmem {
  int off[kMaxList];
  int cd[kMaxList];
  int pre_n[kMaxList + 1];   // prefix of neighbour contributions (centre slot excluded)
  int n;
};

__device__ __forceinline__ int list_count(int cd) { return cd >> 8; }
__device__ __forceinline__ int list_dx(int cd) { return (cd & 15) - 4; }
__device__ __forceinline__ int list_dy(int cd) { return ((cd >> 4) & 15) - 4; }


// ---------------------------------------------------------------- neighbour batches

// Decode global neighbour-contribution index g into its slot-list position
// and the slot's offset (dx, dy) from the pixel.
__device__ __forceinline__ bool neigh_lookup(const ListSmem &ls, int g, int *pos, int *dx, int *dy) {
  int lo = 0, hi = ls.n;                 // last entry with pre_n <= g
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (ls.pre_n[mid] <= g) lo = mid; else hi = mid;
  }
  const int cd = ls.cd[lo];
  *dx = list_dx(cd);
  *dy = list_dy(cd);
  if (*dx == 0 && *dy == 0) return false;
  *pos = ls.off[lo] + (g - ls.pre_n[lo]);
  return true;
}

// Lane-parallel descriptor setup for neighbour contributions [g0, g0 + 32).
template <bool GRAD>
__device__ __forceinline__ void neigh_setup(const LsimParams &p, const Tables &tab, const Workspace &w,
                                            const ListSmem &ls, NBatch &nb, int g0, int n_total, int lane);

// Forward window update with a column-owner lane map: lane l handles the
// window positions r with (cb + r) = l (mod 32), i.e. r = rl + 32j with
// rl = (l - cb) mod 32, so each lane only ever touches its own columns.
// Contributions therefore need no warp barrier between them and their
// updates can be interleaved; the samples a block of lanes reads are still
// 32 consecutive ticks.  U[j] is the window sample k = rl + 32j - 1: the
// boundary correction at k = -1, V[k] for 0 <= k < L, 0 beyond, and
//   val[r] = U(r-2) (1 - f) + U(r-1) f,
// where U(r-2) comes from lane (l - 1) mod 32 (from the previous block for
// the lane with rl = 0).

__device__ __forceinline__ int owner_rl(int cb, int lane) { return (lane - cb) & (kWarp - 1); }

// A window is interior when all its columns are valid waveform columns and
// all kWinSamples padded positions (cb .. cb + kWinSamples) stay inside the
// row buffer; interior passes skip the per-column tests (padded positions
// past L + 1 add or meet exact zeros).
__device__ __forceinline__ bool window_interior(int cb, int L, int NT) {
  return cb >= 1 && cb + L + 1 <= NT - 2 && cb + kWinSamples + 1 <= kRowFloats - kRowPad;
}

// The window update with weights a = s (1 - frac), b = s frac (s = n_e for
// neighbour parts, whose samples are the raw template values and the
// boundary term per electron; s = 1 for main-bin records, stored scaled):
//   val[r] = U(r-2) a + U(r-1) b.

// Window that crosses the edge of the waveform: value parts are kept only
// in columns [2, Nticks-1], correction parts only in [1, Nticks-2].
__device__ __noinline__ void window_apply_edge(float U0, float U1, float U2, float U3, float U4, int cb, int rl,
                                               float a, float b, int L, int NT, float *row, int lane) {
  static_assert(kChunks == 5, "window_apply_edge takes the five chunks by value");
  const float U[kChunks] = {U0, U1, U2, U3, U4};
  float sprev = 0.f;
#pragma unroll
  for (int j = 0; j < kChunks; ++j) {
    const float sh = __shfl_sync(0xffffffffu, U[j], (lane + kWarp - 1) & (kWarp - 1));
    const float prev = rl == 0 ? sprev : sh;
    sprev = sh;
    const int r = rl + j * kWarp;
    const int col = cb + r;
    if (r >= L + 2 || col < 1 || col > NT - 1) continue;
    const bool vc = col <= NT - 2, vv = col >= 2;
    float val;
    if (r == 0) val = vc ? U[j] * b : 0.f;
    else if (r == 1) val = (vc ? prev * a : 0.f) + (vv ? U[j] * b : 0.f);
    else val = vv ? prev * a + U[j] * b : 0.f;
    row[col] += val;
  }
}

// Interior window (window_interior): all columns valid; positions past
// L + 1 add exact zeros.
__device__ __forceinline__ void window_apply_interior(const float U[kChunks], int cb, int rl, float a, float b,
                                                      float *row, int lane) {
  float P[kChunks];
  float sprev = 0.f;
#pragma unroll
  for (int j = 0; j < kChunks; ++j) {
    const float sh = __shfl_sync(0xffffffffu, U[j], (lane + kWarp - 1) & (kWarp - 1));
    P[j] = rl == 0 ? sprev : sh;
    sprev = sh;
  }
  // chunk pairs advance in packed f32x2 FMAs
  float *x = row + cb + rl;
  const float2 aa = make_float2(a, a), bb = make_float2(b, b);
#pragma unroll
  for (int j = 0; j + 1 < kChunks; j += 2) {
    float2 v = make_float2(x[j * kWarp], x[(j + 1) * kWarp]);
    v = __ffma2_rn(make_float2(U[j], U[j + 1]), bb, __ffma2_rn(make_float2(P[j], P[j + 1]), aa, v));
    x[j * kWarp] = v.x;
    x[(j + 1) * kWarp] = v.y;
  }
  if (kChunks & 1) {
    constexpr int j = kChunks - 1;
    x[j * kWarp] = fmaf(U[j], b, fmaf(P[j], a, x[j * kWarp]));
  }
}

template <bool GRAD>
__device__ __forceinline__ void neigh_setup(const LsimParams &p, const Tables &tab, const Workspace &w,
                                            const ListSmem &ls, NBatch &nb, int g0, int n_total, int lane) {
  const int g = g0 + lane;
  int pos = 0, dx = 0, dy = 0;
  NDesc d;
  d.w = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
  d.g0 = make_float4(0.f, 0.f, 0.f, 0.f);
  d.g1 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (g < n_total && neigh_lookup(ls, g, &pos, &dx, &dy)) {
    // the slot lists' compact records: consecutive contributions of a slot
    // read consecutive 16-byte records, with no segment-index indirection
    const SegNb q = w.lnb[pos];
    const float ne = q.ne;
    if (ne != 0.f) {
      constexpr int nbp = kBinsPerPixel;
      const int cx = lut_index((int)(int16_t)(q.bxy & 0xffff), nbp, dx * nbp);
      const int cy = lut_index(q.bxy >> 16, nbp, dy * nbp);
      const int row = cx * p.lut_ny + cy;
      const int cath = q.cath;
      const float frac = q.frac;
      const int cb = p.lut_nt - p.signal_length - cath - 1;
      float dl;
      const float D = cum_terms(tab.c0 + (size_t)row * p.lut_nt, cath, p.lut_nt, p.signal_length, frac, &dl);
      const float pk = pack_window(row, cb, window_interior(cb, p.signal_length, p.n_ticks));
      if (GRAD) {
        const SegNbAdj a = w.lna[pos];
        d.w = make_float4(frac, 1.f - frac, D, pk);
        d.g0 = make_float4(dl, ne * a.dne4_dt0.y / p.t_sampling, a.dne4_dt0.x, 0.f);
        d.g1 = a.dne03;
      } else {
        d.w = make_float4(ne * (1.f - frac), ne * frac, D, pk);
      }
    }
  }
  nb.d[lane] = d;
  __syncwarp();
}

// Template-0 window samples of a neighbour contribution (per electron),
// with the boundary term D as sample k = -1 (padded table: idx = k + 1).
__device__ __forceinline__ void neigh_samples(const Tables &tab, int row, int rl, float D, float U[kChunks]) {
  const float *src = tab.w0 + (size_t)row * kWinSamples + rl;
#pragma unroll
  for (int j = 0; j < kChunks; ++j) U[j] = __ldg(src + j * kWarp);
  if (rl == 0) U[0] = D;
}

// Forward: all neighbour parts of the pixel, four contributions in flight.
__device__ __forceinline__ void neigh_forward(const LsimParams &p, const Tables &tab, const Workspace &w,
                                              const ListSmem &ls, NBatch &nb, float *row, int lane) {
  const int L = p.signal_length, NT = p.n_ticks;
  const int n_total = ls.pre_n[ls.n];
  for (int g0 = 0; g0 < n_total; g0 += kWarp) {
    neigh_setup<false>(p, tab, w, ls, nb, g0, n_total, lane);
    const int m = min(kWarp, n_total - g0);
    for (int j = 0; j < m; j += 4) {
      float u[4][kChunks];
      float4 dw[4];
      int pk[4], cb[4], rl[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        dw[q] = nb.d[j + q].w;                   // stale descriptors past m are masked below
        pk[q] = j + q < m ? __float_as_int(dw[q].w) : -1;
        cb[q] = pack_cb(pk[q]);
        rl[q] = owner_rl(cb[q], lane);
        neigh_samples(tab, pk[q] < 0 ? 0 : (pk[q] & kPackRowMask), rl[q], dw[q].z, u[q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (pk[q] < 0) continue;
        if (pk[q] & kPackEdge)
          window_apply_edge(u[q][0], u[q][1], u[q][2], u[q][3], u[q][4], cb[q], rl[q], dw[q].x, dw[q].y, L, NT, row,
                            lane);
        else
          window_apply_interior(u[q], cb[q], rl[q], dw[q].x, dw[q].y, row, lane);
      }
    }
    __syncwarp();
  }
}

struct Theta {
  float v[LSIM_NPARAM];
};

// Adjoint of one neighbour contribution (descriptor d) given its padded
// template-0 samples v[c] = w0[row][32c + lane] (sample idx - 1 of the
// window, idx = 32c + lane): sample k lands on columns cb + k + 1 (x frac)
// and cb + k + 2 (x (1 - frac)); lane 0's idx = 0 is the boundary
// correction D * n_e (table value 0).  Accumulates dL/dtheta.
__device__ __forceinline__ void neigh_vjp_one(const NDesc &d, const float v[kChunks], int L, int NT,
                                              const float *grow, Theta &th, int lane) {
  const int pk = __float_as_int(d.w.w);
  const int cb = pack_cb(pk);
  const float f = d.w.x, f1 = d.w.y, D = d.w.z;
  float sA = 0.f, sB = 0.f, gA0 = 0.f, gB0 = 0.f;   // sum v gA, sum v gB
  if (!(pk & kPackEdge)) {
    // interior window: every column in range (columns past cb + L + 1 hold
    // zeros of the row padding and meet zero samples); the two sums advance
    // together in one packed FMA per chunk
    float2 sAB = make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
      const int c1 = cb + c * kWarp + lane;
      const float2 g = make_float2(grow[c1], grow[c1 + 1]);
      sAB = __ffma2_rn(make_float2(v[c], v[c]), g, sAB);
      if (c == 0) { gA0 = g.x; gB0 = g.y; }
    }
    sA = sAB.x;
    sB = sAB.y;
  } else {
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
      const int idx = c * kWarp + lane;
      if (idx <= L) {
        const int c1 = cb + idx;
        const int lo = idx == 0 ? 1 : 2, hi = idx == 0 ? NT - 2 : NT - 1;
        const float gA = (c1 >= lo && c1 <= hi) ? grow[c1] : 0.f;
        const float gB = (c1 + 1 >= lo && c1 + 1 <= hi) ? grow[c1 + 1] : 0.f;
        sA = fmaf(v[c], gA, sA);
        sB = fmaf(v[c], gB, sB);
        if (c == 0) { gA0 = gA; gB0 = gB; }
      }
    }
  }
  float acc_ne = sA * f + sB * f1, acc_fr = sA - sB;
  if (lane == 0) {
    const float dcorr = gA0 * f + gB0 * f1;
    acc_ne += dcorr * D;
    acc_fr += dcorr * d.g0.x + D * (gA0 - gB0);
  }
  th.v[0] = fmaf(acc_ne, d.g1.x, th.v[0]);
  th.v[1] = fmaf(acc_ne, d.g1.y, th.v[1]);
  th.v[2] = fmaf(acc_ne, d.g1.z, fmaf(acc_fr, d.g0.y, th.v[2]));
  th.v[3] = fmaf(acc_ne, d.g1.w, th.v[3]);
  th.v[7] = fmaf(acc_ne, d.g0.z, th.v[7]);
}

__device__ __forceinline__ void neigh_rows(const Tables &tab, int row, float v[kChunks], int lane) {
  const float *src = tab.w0 + (size_t)row * kWinSamples + lane;
#pragma unroll
  for (int c = 0; c < kChunks; ++c) v[c] = __ldg(src + c * kWarp);
}

// Adjoint: all neighbour parts, given the waveform cotangent grow[col].
__device__ __forceinline__ void neigh_backward(const LsimParams &p, const Tables &tab, const Workspace &w,
                                               const ListSmem &ls, NBatch &nb, const float *grow, Theta &th,
                                               int lane) {
  const int L = p.signal_length, NT = p.n_ticks;
  const int n_total = ls.pre_n[ls.n];
  for (int g0 = 0; g0 < n_total; g0 += kWarp) {
    neigh_setup<true>(p, tab, w, ls, nb, g0, n_total, lane);
    const int m = min(kWarp, n_total - g0);
    // software pipeline: the template row of contribution j + 1 is in
    // flight while contribution j is projected (empty descriptors read row 0)
    float vn[kChunks];
    neigh_rows(tab, max(__float_as_int(nb.d[0].w.w), 0) & kPackRowMask, vn, lane);
    for (int j = 0; j < m; ++j) {
      const NDesc d = nb.d[j];
      const int pk = __float_as_int(d.w.w);
      float v[kChunks];
#pragma unroll
      for (int c = 0; c < kChunks; ++c) v[c] = vn[c];
      if (j + 1 < m) neigh_rows(tab, max(__float_as_int(nb.d[j + 1].w.w), 0) & kPackRowMask, vn, lane);
      if (pk >= 0) neigh_vjp_one(d, v, L, NT, grow, th, lane);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- main-bin records

// The main-bin records that land on this pixel: segments of the 3x3 slots
// whose bins reach it (tested 32 candidates at a time).  Accepted records
// are packed into the batch as descriptors (NDesc) and handed to flush(m)
// 32 at a time.
template <bool GRAD, typename F>
__device__ __forceinline__ void main_batches(const LsimParams &p, const Workspace &w, const ListSmem &ls, NBatch &nb,
                                             int lane, F &&flush) {
  constexpr int nbp = kBinsPerPixel;
  int m = 0;
  for (int e = 0; e < ls.n; ++e) {
    const int cd = ls.cd[e];
    const int dx = list_dx(cd), dy = list_dy(cd);
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1) continue;
    const int o = ls.off[e], c = list_count(cd);
    for (int j0 = 0; j0 < c; j0 += kWarp) {
      int s = 0, slot = 0;
      bool hit = false;
      if (j0 + lane < c) {
        s = __ldg(w.seg_list + o + j0 + lane);
        const SegFwd &f = w.segf[s];
        int lx, hx, ly, hy;
        axis_range(__ldg(&f.bx), nbp, &lx, &hx);
        axis_range(__ldg(&f.by), nbp, &ly, &hy);
        hit = __ldg(&f.ne) != 0.f && lx <= dx && dx <= hx && ly <= dy && dy <= hy;
        slot = (dx - lx) * 2 + (dy - ly);
      }
      const unsigned bal = __ballot_sync(0xffffffffu, hit);
      const int nh = __popc(bal);
      if (m + nh > kWarp) {
        flush(m);
        m = 0;
      }
      if (hit) {
        const int pos = m + __popc(bal & ((1u << lane) - 1u));
        const SegFwd &f = w.segf[s];
        const int rec = s * kRecPerSeg + slot;
        const int cb = p.lut_nt - p.signal_length - __ldg(&f.cath) - 1;
        const float frac = __ldg(&f.frac);
        NDesc d;
        d.w = make_float4(1.f - frac, frac, GRAD ? w.mrec[(size_t)rec * kRecFloats + kRecDl] : 0.f,
                          pack_window(0, cb, window_interior(cb, p.signal_length, p.n_ticks)));
        d.g0 = make_float4(GRAD ? __ldg(&w.sega[s].dt0) / p.t_sampling : 0.f, __int_as_float(rec), 0.f, 0.f);
        d.g1 = make_float4(0.f, 0.f, 0.f, 0.f);
        nb.d[pos] = d;
      }
      m += nh;
      __syncwarp();
    }
  }
  if (m) flush(m);
}

// Forward: add m batched records (window samples k = -1 .. 158 stored at
// rec[k + 1], zero past L), four in flight.
__device__ __forceinline__ void main_rec_forward(const LsimParams &p, const float *mrec, const NBatch &nb, int m,
                                                 float *row, int lane) {
  const int L = p.signal_length, NT = p.n_ticks;
  __syncwarp();
  for (int j = 0; j < m; j += 4) {
    float u[4][kChunks];
    float4 dw[4];
    int pk[4], cb[4], rl[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool ok = j + q < m;
      dw[q] = nb.d[j + q].w;
      pk[q] = __float_as_int(dw[q].w);
      cb[q] = pack_cb(pk[q]);
      rl[q] = owner_rl(cb[q], lane);
      const int rec = ok ? __float_as_int(nb.d[j + q].g0.y) : 0;
      const float *src = mrec + (size_t)rec * kRecFloats + rl[q];
#pragma unroll
      for (int c = 0; c < kChunks; ++c) u[q][c] = ok ? src[c * kWarp] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (j + q >= m) continue;
      if (pk[q] & kPackEdge)
        window_apply_edge(u[q][0], u[q][1], u[q][2], u[q][3], u[q][4], cb[q], rl[q], dw[q].x, dw[q].y, L, NT, row,
                          lane);
      else
        window_apply_interior(u[q], cb[q], rl[q], dw[q].x, dw[q].y, row, lane);
    }
  }
  __syncwarp();
}

// Adjoint of m batched records given the waveform cotangent grow[col]:
// each record is replaced by the cotangent of its samples (rec[0]: the
// boundary correction, rec[1 + k]: V[k]); the sub-tick-fraction part goes
// straight to dL/d eField through d t0/d eField.
__device__ __forceinline__ void main_rec_backward(const LsimParams &p, float *mrec, const NBatch &nb, int m,
                                                  const float *grow, Theta &th, int lane) {
  const int L = p.signal_length, NT = p.n_ticks;
  __syncwarp();
  // samples of record j + 1 are in flight while record j is processed
  auto load = [&](int j, float u[kChunks]) {
    const float *rec = mrec + (size_t)__float_as_int(nb.d[j].g0.y) * kRecFloats + lane;
#pragma unroll
    for (int c = 0; c < kChunks; ++c) u[c] = lane + c * kWarp <= L ? rec[c * kWarp] : 0.f;
  };
  float un[kChunks];
  load(0, un);
  for (int j = 0; j < m; ++j) {
    float u[kChunks];
#pragma unroll
    for (int c = 0; c < kChunks; ++c) u[c] = un[c];
    if (j + 1 < m) load(j + 1, un);
    const NDesc d = nb.d[j];
    float *rec = mrec + (size_t)__float_as_int(d.g0.y) * kRecFloats;
    const int pk = __float_as_int(d.w.w);
    const int cb = pack_cb(pk);
    const float f1 = d.w.x, f = d.w.y;
    const bool interior = !(pk & kPackEdge);
    float dfr = 0.f, dcorr = 0.f;
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
      const int idx = lane + c * kWarp;     // sample idx - 1 lands on columns cb + idx (x frac), cb + idx + 1
      if (idx <= L) {
        const int c1 = cb + idx;
        float gA, gB;
        if (interior) {
          gA = grow[c1];
          gB = grow[c1 + 1];
        } else {
          const int lo = idx == 0 ? 1 : 2, hi = idx == 0 ? NT - 2 : NT - 1;
          gA = (c1 >= lo && c1 <= hi) ? grow[c1] : 0.f;
          gB = (c1 + 1 >= lo && c1 + 1 <= hi) ? grow[c1 + 1] : 0.f;
        }
        const float du = gA * f + gB * f1;
        rec[idx] = du;
        dfr += u[c] * (gA - gB);
        if (idx == 0) dcorr = du;
      }
    }
    if (lane == 0) dfr += dcorr * d.w.z;
    th.v[2] = fmaf(dfr, d.g0.x, th.v[2]);
  }
  __syncwarp();
}

// Per-warp shared memory.  Each warp's block starts on a 16-byte boundary
// (the row is accessed with float4), so the size stays a 16-byte multiple.
template <bool GRAD>
struct __align__(16) WarpSmem {
  float buf[kRowFloats];
  ListSmem list;
  NBatch nb;
};
template <>
struct __align__(16) WarpSmem<true> {
  float buf[kRowFloats];
  ListSmem list;
  NBatch nb;
  float gint[LSIM_MAX_HITS];
  FeeState fee;
};
static_assert(sizeof(WarpSmem<false>) % 16 == 0, "per-warp shared memory must keep 16-byte alignment");
static_assert(sizeof(WarpSmem<true>) % 16 == 0, "per-warp shared memory must keep 16-byte alignment");
static_assert(offsetof(WarpSmem<false>, buf) == 0 && offsetof(WarpSmem<true>, buf) == 0, "row first");
static_assert((kRowPad + 1) % 4 == 0 && kRowFloats % 4 == 0, "output column 1 of the row must be 16-byte aligned");

// ---------------------------------------------------------------- per pixel

// Neighbourhood slot list of a pixel (compacted, fixed order) over the
// (2h+1)^2 slots around it, with the prefix count of neighbour
// contributions (slots within the neighbour radius n, centre excluded).
__device__ __forceinline__ void build_list(const Grid &g, const int32_t *__restrict__ cnt,
                                           const int32_t *__restrict__ off, int64_t slot, ListSmem &ls, int lane) {
  const int D = 2 * g.h + 1;
  int base = 0, nbase = 0;
  for (int i0 = 0; i0 < D * D; i0 += kWarp) {
    const int idx = i0 + lane;
    int c = 0, o = 0, dxy = 0;
    bool neigh = false;
    if (idx < D * D) {
      const int dx = idx / D - g.h, dy = idx % D - g.h;
      const int64_t q = slot - (int64_t)dy * g.nxe - dx;
      c = __ldg(cnt + q);
      if (c > 0) o = __ldg(off + q);
      dxy = (dx + 4) | ((dy + 4) << 4);
      neigh = !(dx == 0 && dy == 0) && abs(dx) <= g.n && abs(dy) <= g.n;
    }
    const bool has = c > 0;
    const unsigned bal = __ballot_sync(0xffffffffu, has);
    const int nc = (has && neigh) ? c : 0;
    int incl = nc;   // inclusive scan of neighbour counts over the compacted entries
    for (int o2 = 1; o2 < kWarp; o2 <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o2);
      if (lane >= o2) incl += y;
    }
    if (has) {
      const int pos = base + __popc(bal & ((1u << lane) - 1u));
      ls.off[pos] = o;
      ls.cd[pos] = (c << 8) | dxy;
      ls.pre_n[pos] = nbase + incl - nc;
    }
    base += __popc(bal);
    nbase += __shfl_sync(0xffffffffu, incl, kWarp - 1);
  }
  if (lane == 0) {
    ls.n = base;
    ls.pre_n[base] = nbase;
  }
  __syncwarp();
}

__device__ __forceinline__ int32_t slot_pid(const LsimParams &p, const Grid &g, int64_t slot) {
  const int64_t ev = slot / g.event_stride;
  const int64_t rem = slot - ev * g.event_stride;
  const int plane = (int)(rem / g.plane_stride);
  const int64_t inplane = rem % g.plane_stride;
  const int py = (int)(inplane / g.nxe) - g.h, px = (int)(inplane % g.nxe) - g.h;
  return pixel2id(p, px, py, plane, (int)ev - 1);
}

// The persistent kernel hands out heavy pixels first (k_heavy_pixels) only
// while at most 1 in kHeavyFractionInv pixels is heavy.
constexpr int kHeavyFractionInv = 8;

template <int MODE>
__global__ void __launch_bounds__(kAccWarps * kWarp, 5) k_lut_pixels(AccumArgs a) {
  // kModeVjpWfs: the cotangent row comes from memory (no forward, no front end)
  constexpr bool VJP = MODE == kModeVjpWfs;
  constexpr bool GRAD = (MODE == kModeGrad || MODE == kModeGradStored || VJP);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  unsigned char *wbase = smem_raw + (size_t)wid * a.warp_smem;
  WarpSmem<GRAD> &sm = *reinterpret_cast<WarpSmem<GRAD> *>(wbase);
  if constexpr (GRAD) {
    if (lane == 0) sm.fee.mask = a.w.fee_masks + (size_t)(blockIdx.x * kAccWarps + wid) * kFeeMaskWords;
    __syncwarp();
  }
  const LsimParams &p = a.p;
  float *row = sm.buf + kRowPad;
  const int NT = p.n_ticks;
  const int T = NT - 1;
  const int H = p.max_adc_values;
  const int n_valid = a.w.counts->n_valid;
  // heavy pixels first only while they are few: when most pixels are heavy
  // (one dense event), grid order keeps neighbouring pixels, and their
  // shared segments and LUT rows, together in time
  const int n_heavy0 = a.w.counts->n_heavy;
  const int n_heavy = n_heavy0 * kHeavyFractionInv > n_valid ? 0 : n_heavy0;
  const bool early_exit = (a.normals == nullptr) && p.threshold > 0.f;
  for (;;) {
    int r = 0;
    if (lane == 0) r = atomicAdd(&a.w.counts->work, 1);
    r = __shfl_sync(0xffffffffu, r, 0);
    // work items: the heavy pixels first, then all pixels in grid order
    // (skipping the heavy ones), so the grid does not end on a few long rows
    if (r >= n_valid + n_heavy) break;
    if (r < n_heavy) {
      r = a.w.heavy[r];
    } else {
      r -= n_heavy;
      if (n_heavy > 0 && a.w.heavy_flag[r]) continue;
    }
    const int64_t slot = a.w.pix_slot[r];
    // adjoint mode: this lane's hit cotangent, or the target ADC of the
    // pixel (digitize(0) where the target has no such pixel), loaded early
    float cot = 0.f;
    if constexpr (GRAD && !VJP) {
      if (lane < H) {
        if (a.g_adc) {
          cot = a.g_adc[(int64_t)r * H + lane];
        } else {
          const int tr = a.n_tgt > 0 ? a.w.tgt_index[r] : -1;
          cot = tr >= 0 ? a.tgt_adc[(int64_t)tr * H + lane] : digitize(p, 0.f);
        }
      }
    }
    float4 *b4 = reinterpret_cast<float4 *>(sm.buf);
    for (int i = lane; i < kRowFloats / 4; i += kWarp) b4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    build_list(a.g, a.w.cnt, a.w.off, slot, sm.list, lane);
    if (MODE == kModeGradStored || VJP) {
      // the waveform stored by a preceding simulate_wfs pass, or (VJP) the
      // cotangent of the waveform row (columns 1..T; tick 0 stays zero)
      const float4 *src = reinterpret_cast<const float4 *>(a.wfs + (a.row_offset + r) * (int64_t)T);
      float4 *dst = reinterpret_cast<float4 *>(row + 1);
      for (int i = lane; i < T / 4; i += kWarp) dst[i] = __ldg(src + i);
      __syncwarp();
    } else {
      // ---- forward: neighbour parts, then main-bin parts
      neigh_forward(p, a.tab, a.w, sm.list, sm.nb, row, lane);
      main_batches<false>(p, a.w, sm.list, sm.nb, lane,
                          [&](int m) { main_rec_forward(p, a.w.mrec, sm.nb, m, row, lane); });
      __syncwarp();
    }
    if (MODE == kModeWfs) {
      float4 *dst = reinterpret_cast<float4 *>(a.wfs + (a.row_offset + r) * (int64_t)T);
      const float4 *src = reinterpret_cast<const float4 *>(row + 1);
      for (int i = lane; i < T / 4; i += kWarp) dst[i] = src[i];
      continue;
    }
    float loss = 0.f;
    if constexpr (!VJP) {
      // ---- front end on the output ticks (row + 1)
      const float *nrm = a.normals ? a.normals + (int64_t)r * (1 + 3 * H) : nullptr;
      float *adc_dst = a.adc_out ? a.adc_out + (int64_t)r * H : nullptr;
      float *tick_dst = a.tick_out ? a.tick_out + (int64_t)r * H : nullptr;
      warp_cumsum_charge(row + 1, T, p.t_sampling, lane);
      if (MODE == kModeAdc) {
        fee_forward(p, row + 1, T, nrm, adc_dst, tick_dst, nullptr, nullptr, early_exit, lane);
        continue;
      }
    }
    if constexpr (GRAD && !VJP) {
      const float *nrm = a.normals ? a.normals + (int64_t)r * (1 + 3 * H) : nullptr;
      float *adc_dst = a.adc_out ? a.adc_out + (int64_t)r * H : nullptr;
      float *tick_dst = a.tick_out ? a.tick_out + (int64_t)r * H : nullptr;
      fee_forward(p, row + 1, T, nrm, adc_dst, tick_dst, &sm.fee, nullptr, early_exit, lane);
      // loss terms and digitisation adjoint, lane h for hit h
      if (lane < H) {
        const float raw = sm.fee.raw[lane];
        const float adc = digitize(p, raw);
        float g;
        if (a.g_adc) {
          g = cot;
        } else {
          const float d = adc - cot;
          loss = d * d;
          g = 2.f * d;
        }
        sm.gint[lane] = digitize_vjp(p, raw, g);
      }
      loss = warp_sum(loss);
      __syncwarp();
      fee_backward(p, row + 1, T, &sm.fee, sm.gint, lane);
      if (lane == 0) row[0] = 0.f;
      __syncwarp();
    }
    if constexpr (GRAD) {
      Theta th;
#pragma unroll
      for (int i = 0; i < LSIM_NPARAM; ++i) th.v[i] = 0.f;
      neigh_backward(p, a.tab, a.w, sm.list, sm.nb, row, th, lane);
      main_batches<true>(p, a.w, sm.list, sm.nb, lane,
                         [&](int m) { main_rec_backward(p, a.w.mrec, sm.nb, m, row, th, lane); });
      // per-pixel record [loss, dL/dtheta]
#pragma unroll
      for (int i = 0; i < LSIM_NPARAM; ++i) th.v[i] = warp_sum(th.v[i]);
      if (lane == 0) {
        float *dst = a.w.pix_out + (size_t)r * kPixRec;
        dst[0] = loss;
#pragma unroll
        for (int i = 0; i < LSIM_NPARAM; ++i) dst[1 + i] = th.v[i];
      }
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------- reductions

constexpr int kRedThreads = 256;
constexpr int kPixBlocks = 1024;     // reduction blocks over pixel records
constexpr int kMainBlocks = 256;     // reduction blocks over per-segment main-bin adjoint records
constexpr int kTgtBlocks = 256;      // reduction blocks over target-only rows
static_assert(kPixBlocks + kMainBlocks + kTgtBlocks <= kRedSlots, "reduction partials");

// Fixed-order float64 sum of per-pixel (or per-warp) records [loss, 8
// gradient terms]: block b reduces a contiguous chunk; the chunking depends
// only on the record count (n_fixed, or the valid-pixel count when < 0).
__global__ void k_reduce_records(const float *__restrict__ pix, int64_t n_fixed, const LsimCounts *counts,
                                 double *partials) {
  __shared__ double sh[kRedThreads];
  const int64_t n = n_fixed >= 0 ? n_fixed : counts->n_valid;
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (int q = 0; q <= LSIM_NPARAM; ++q) {
    double s = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += kRedThreads) s += (double)pix[i * kPixRec + q];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = kRedThreads / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) partials[(size_t)blockIdx.x * 16 + q] = sh[0];
    __syncthreads();
  }
}

// Row of the loss target with the pixel id of each valid pixel (both lists
// are sorted), or -1.
__global__ void k_target_index(AccumArgs a) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= a.w.counts->n_valid) return;
  const int32_t pid = slot_pid(a.p, a.g, a.w.pix_slot[r]);
  int64_t lo = 0, hi = a.n_tgt;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a.tgt_pids[mid] < pid) lo = mid + 1; else hi = mid;
  }
  a.w.tgt_index[r] = (lo < a.n_tgt && a.tgt_pids[lo] == pid) ? (int32_t)lo : -1;
}

// Loss terms of target pixels that the prediction does not have.
__global__ void k_target_only(AccumArgs a, double *partials) {
  __shared__ double sh[kRedThreads];
  const LsimParams &p = a.p;
  const int H = p.max_adc_values;
  const float adc0 = digitize(p, 0.f);
  const int n_valid = a.w.counts->n_valid;
  const int64_t chunk = (a.n_tgt + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk, hi = min(a.n_tgt, lo + chunk);
  double acc = 0.0;
  for (int64_t t = lo + threadIdx.x; t < hi; t += kRedThreads) {
    const int32_t pid = a.tgt_pids[t];
    int l = 0, h2 = n_valid;
    while (l < h2) {
      const int mid = (l + h2) >> 1;
      if (slot_pid(p, a.g, a.w.pix_slot[mid]) < pid) l = mid + 1; else h2 = mid;
    }
    const bool present = l < n_valid && slot_pid(p, a.g, a.w.pix_slot[l]) == pid;
    if (!present && pid >= 0)
      for (int h = 0; h < H; ++h) {
        const float d = adc0 - a.tgt_adc[t * H + h];
        acc += (double)(d * d);
      }
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kRedThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[(size_t)blockIdx.x * 16] = sh[0];
}

// One block per output (0: loss, 1..8: gradient): fixed-order float64 sum
// of the reduction partials.
__global__ void k_grad_finalize(const double *partials, int n_rec_blocks, const double *tgt_partials,
                                int n_tgt_blocks, float *loss_out, float *grad_out) {
  __shared__ double sh[kRedThreads];
  const int q = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < n_rec_blocks; b += kRedThreads) acc += partials[(size_t)b * 16 + q];
  if (q == 0)
    for (int b = threadIdx.x; b < n_tgt_blocks; b += kRedThreads) acc += tgt_partials[(size_t)b * 16];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kRedThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (q == 0) {
      if (loss_out) loss_out[0] = (float)sh[0];
    } else if (grad_out) {
      grad_out[q - 1] = (float)sh[0];
    }
  }
}

// ---------------------------------------------------------------- work order

// Pixels whose (2h+1)^2 neighbourhood holds more than kHeavyPixel segments
// (contributions) are listed so that the persistent kernel starts with them.
constexpr int kHeavyPixel = 2048;

__global__ void k_heavy_pixels(Grid g, Workspace w) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= w.counts->n_valid) return;
  const int64_t slot = w.pix_slot[r];
  int cost = 0;
  for (int dy = -g.h; dy <= g.h; ++dy)
    for (int dx = -g.h; dx <= g.h; ++dx) cost += __ldg(w.cnt + slot - (int64_t)dy * g.nxe - dx);
  const bool heavy = cost > kHeavyPixel;
  w.heavy_flag[r] = heavy ? 1 : 0;
  if (heavy) w.heavy[atomicAdd(&w.counts->n_heavy, 1)] = (int32_t)r;
}

static int run_heavy_pixels(const AccumArgs &a, cudaStream_t st) {
  if (cudaMemsetAsync(&a.w.counts->n_heavy, 0, sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (a.n_rows <= 0) return LSIM_OK;
  k_heavy_pixels<<<(unsigned)((a.n_rows + 255) / 256), 256, 0, st>>>(a.g, a.w);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

// ---------------------------------------------------------------- launch

// Persistent grid: every SM filled to its occupancy limit.
// Per-warp shared memory (the front end's reset masks live in the
// workspace, one kFeeMaskWords block per warp).
template <int MODE>
static size_t warp_smem_bytes(const LsimParams &) {
  return (sizeof(WarpSmem<MODE == kModeGrad || MODE == kModeGradStored || MODE == kModeVjpWfs>) + 15) &
         ~size_t(15);
}

// Persistent grid: every SM filled to its occupancy limit.
template <int MODE>
static int grid_blocks(const LsimParams &p, int *blocks, size_t *smem_out) {
  const size_t smem = warp_smem_bytes<MODE>(p) * kAccWarps;
  if (cudaFuncSetAttribute(k_lut_pixels<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return LSIM_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lut_pixels<MODE>, kAccWarps * kWarp, smem) !=
      cudaSuccess)
    return LSIM_ERR_CUDA;
  if (per_sm < 1) per_sm = 1;
  const LsimTuning tu = tuning();
  if (tu.pixel_blocks_per_sm > 0 && tu.pixel_blocks_per_sm < per_sm) per_sm = tu.pixel_blocks_per_sm;
  *blocks = min(device_sm_count() * per_sm, kMaxPixelWarps / kAccWarps);
  *smem_out = smem;
  return LSIM_OK;
}

template <int MODE>
static int launch_mode(const AccumArgs &a0, cudaStream_t st) {
  int blocks = 0;
  size_t smem = 0;
  int rc = grid_blocks<MODE>(a0.p, &blocks, &smem);
  if (rc != LSIM_OK) return rc;
  AccumArgs a = a0;
  a.warp_smem = (int)warp_smem_bytes<MODE>(a0.p);
  if (cudaMemsetAsync(&a.w.counts->work, 0, sizeof(int32_t), st) != cudaSuccess) return LSIM_ERR_CUDA;
  cudaEvent_t ev0, ev1;
  kernel_events(&ev0, &ev1);
  if (ev0 && cudaEventRecord(ev0, st) != cudaSuccess) return LSIM_ERR_CUDA;
  k_lut_pixels<MODE><<<blocks, kAccWarps * kWarp, smem, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return LSIM_ERR_CUDA;
  if (ev1 && cudaEventRecord(ev1, st) != cudaSuccess) return LSIM_ERR_CUDA;
  return LSIM_OK;
}

int run_accum(AccumMode mode, const AccumArgs &a, cudaStream_t st) {
  if (a.p.n_neighbors > 4 || a.p.n_tran_bins != kMaxTran || a.p.nb_bins_per_pixel != kBinsPerPixel ||
      a.p.n_ticks - 1 + kRowPad > kRowFloats || (a.p.n_ticks - 1) % 4 != 0 || a.p.max_adc_values > LSIM_MAX_HITS ||
      a.p.signal_length + 2 > kChunks * kWarp || a.p.signal_length > a.p.lut_nt)
    return LSIM_ERR_UNSUPPORTED;
  // neighbour LUT indices reach nb*n + nb/2 - 1 (sim_jax.py:443)
  const int need = a.p.nb_bins_per_pixel * a.p.n_neighbors + a.p.nb_bins_per_pixel / 2;
  if (a.p.lut_nx < need || a.p.lut_ny < need || a.p.lut_nx < kMainSub || a.p.lut_ny < kMainSub)
    return LSIM_ERR_UNSUPPORTED;
  if (a.n_rows > 0x7fffffff / kRecPerSeg) return LSIM_ERR_UNSUPPORTED;   // record indices are int32
  // descriptor packing: LUT rows in 15 bits, window origins within +-16384
  if (a.p.lut_nx * a.p.lut_ny > kPackRowMask + 1 || a.p.lut_nt >= kPackCbBias || a.p.signal_length >= kPackCbBias)
    return LSIM_ERR_UNSUPPORTED;
  // the stored-waveform adjoint reuses the records (and their template
  // order) of the simulate_wfs pass that wrote the waveforms
  int rc = mode == kModeGradStored ? LSIM_OK : run_main_records(a, st);
  if (rc == LSIM_OK) rc = run_heavy_pixels(a, st);
  if (rc != LSIM_OK) return rc;
  switch (mode) {
    case kModeWfs: return launch_mode<kModeWfs>(a, st);
    case kModeAdc: return launch_mode<kModeAdc>(a, st);
    case kModeGrad:
      if (!a.g_adc && a.n_tgt > 0 && a.n_rows > 0) {
        k_target_index<<<(unsigned)((a.n_rows + 255) / 256), 256, 0, st>>>(a);
        if (cudaGetLastError() != cudaSuccess) return LSIM_ERR_CUDA;
      }
      rc = launch_mode<kModeGrad>(a, st);
      return rc != LSIM_OK ? rc : run_main_adjoint(a, st);
    case kModeVjpWfs:
      rc = launch_mode<kModeVjpWfs>(a, st);
      return rc != LSIM_OK ? rc : run_main_adjoint(a, st);
    case kModeGradStored:
      if (!a.g_adc && a.n_tgt > 0 && a.n_rows > 0) {
        k_target_index<<<(unsigned)((a.n_rows + 255) / 256), 256, 0, st>>>(a);
        if (cudaGetLastError() != cudaSuccess) return LSIM_ERR_CUDA;
      }
      rc = launch_mode<kModeGradStored>(a, st);
      return rc != LSIM_OK ? rc : run_main_adjoint(a, st);
  }
  return LSIM_ERR_INVALID;
}

int run_grad_finalize(const AccumArgs &a, float *loss_out, float *grad_out, cudaStream_t st) {
  double *rec_partials = a.w.red_partials;
  double *tgt_partials = a.w.red_partials + (size_t)(kPixBlocks + kMainBlocks) * 16;
  k_reduce_records<<<kPixBlocks, kRedThreads, 0, st>>>(a.w.pix_out, -1, a.w.counts, rec_partials);
  k_reduce_records<<<kMainBlocks, kRedThreads, 0, st>>>(a.w.main_out, a.n_rows, a.w.counts,
                                                        rec_partials + (size_t)kPixBlocks * 16);
  int tb = 0;
  if (!a.g_adc && a.n_tgt > 0) {
    tb = kTgtBlocks;
    k_target_only<<<tb, kRedThreads, 0, st>>>(a, tgt_partials);
  }
  k_grad_finalize<<<1 + LSIM_NPARAM, kRedThreads, 0, st>>>(rec_partials, kPixBlocks + kMainBlocks, tgt_partials, tb,
                                                         loss_out, grad_out);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
