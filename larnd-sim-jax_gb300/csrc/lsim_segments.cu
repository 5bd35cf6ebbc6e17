// Per-segment physics (quench + drift + sub-pixel binning) and the pixel
// map (dense-grid counting sort of segments by principal pixel).
//
// Reference: shift_tracks (sim_jax.py:108-119), quench
// (quenching_jax.py:37-74), drift (drifting_jax.py:18-58),
// simulate_drift_new (sim_jax.py:374-453), the unique/renumbering step of
// simulate_wfs (sim_jax.py:715-725), and for parametrised mode
// generate_electrons (detsim_jax.py:376-400) and get_pixels
// (detsim_jax.py:477-491).
#include "lsim_internal.cuh"

namespace lsim {

__global__ void k_reset_counts(LsimCounts *c) {
  if (threadIdx.x == 0) {
    c->n_valid = 0; c->n_em1 = 0; c->any_m1 = 0; c->status = 0; c->max_slot = 0; c->n_big_slots = 0;
    c->bad_row = 0x7fffffff; c->work = 0; c->n_main_rec = 0; c->n_main_seg = 0; c->n_heavy = 0;
    for (int i = 0; i < (int)(sizeof(c->reserved) / sizeof(c->reserved[0])); ++i) c->reserved[i] = 0;
  }
}

struct TrackRow {
  float x, y, z, zs, ze, dE, dEdx, dx;
  int event;
};

__device__ __forceinline__ TrackRow load_row(const LsimParams &p, const LsimFieldMap &f, const float *tracks,
                                             int64_t s) {
  const float *r = tracks + s * (int64_t)f.n_fields;
  TrackRow t;
  // shift_tracks: position columns minus shift (sim_jax.py:110-118)
  t.x = __fsub_rn(r[f.x], p.shift_x);
  t.y = __fsub_rn(r[f.y], p.shift_y);
  t.z = __fsub_rn(r[f.z], p.shift_z);
  t.zs = __fsub_rn(r[f.z_start], p.shift_z);
  t.ze = __fsub_rn(r[f.z_end], p.shift_z);
  t.dE = r[f.dE];
  t.dEdx = r[f.dEdx];
  t.dx = r[f.dx];
  t.event = (int)r[f.eventID];   // astype(int): truncation
  return t;
}

// The parameter-dependent values the segment kernels use: from the
// parameter block, or (lsim_lut_stage1_theta) from device memory.  Kept
// apart from LsimParams so the large kernel-parameter block is never copied.
struct Phys {
  float Ab, kb, erho, vdrift, lifetime, long_diff, tran_diff, eField, lArDensity, dvdrift;
};

__device__ __forceinline__ Phys phys_of(const LsimParams &p, const float *__restrict__ derived) {
  if (derived)
    return Phys{derived[0], derived[1], derived[2], derived[3], derived[4],
                derived[5], derived[6], derived[7], derived[8], derived[9]};
  return Phys{p.Ab, p.kb, p.erho, p.vdrift, p.lifetime, p.long_diff, p.tran_diff, p.eField, p.lArDensity,
              p.dvdrift_deField};
}

// Recombination factor and its derivatives d/d(Ab, kb, eField, lArDensity).
__device__ __forceinline__ float recombination(const LsimParams &p, const Phys &ph, const TrackRow &t, float d[4]) {
  d[0] = d[1] = d[2] = d[3] = 0.f;
  if (p.recombination_mode == LSIM_RECOMB_BIRKS) {
    // Ab / (1 + kb*dEdx/(eField*lArDensity)), quenching_jax.py:23-25
    float X = __fdiv_rn(__fmul_rn(ph.kb, t.dEdx), ph.erho);
    float den = __fadd_rn(1.0f, X);
    float R = __fdiv_rn(ph.Ab, den);
    float r_den = R / den;
    d[0] = 1.0f / den;
    d[1] = -r_den * (t.dEdx / ph.erho);
    d[2] = r_den * X / ph.eField;
    d[3] = r_den * X / ph.lArDensity;
    return R;
  }
  float csi, denom;
  if (p.recombination_mode == LSIM_RECOMB_BOX) {
    // max(0, log(alpha + csi)/csi), quenching_jax.py:18-21
    csi = __fdiv_rn(__fmul_rn(p.beta, t.dEdx), ph.erho);
    denom = csi;
  } else {
    // ellipsoid Box model, quenching_jax.py:30-35 and :55-66
    float cosphi = __fdiv_rn(fabsf(__fsub_rn(t.ze, t.zs)), __fadd_rn(t.dx, 1e-10f));
    float c2 = __fmul_rn(cosphi, cosphi);
    float b_phi = __fdiv_rn(p.beta, sqrtf(__fadd_rn(__fsub_rn(1.0f, c2), __fmul_rn(p.r_inv2, c2))));
    csi = __fdiv_rn(__fmul_rn(b_phi, t.dEdx), ph.erho);
    denom = __fadd_rn(csi, 1e-10f);
  }
  float lg = logf(__fadd_rn(p.alpha, csi));
  float f = __fdiv_rn(lg, denom);
  float R = fmaxf(0.0f, f);
  // jnp.maximum(0, f) passes 1 for f > 0, 0.5 at a tie
  float gate = f > 0.f ? 1.0f : (f == 0.f ? 0.5f : 0.0f);
  float dRdcsi = gate * (1.0f / ((p.alpha + csi) * denom) - lg / (denom * denom));
  d[2] = dRdcsi * (-csi / ph.eField);
  d[3] = dRdcsi * (-csi / ph.lArDensity);
  return R;
}

// Drift membership: mask and plane (drifting_jax.py:21-35).
__device__ __forceinline__ int tpc_plane(const LsimParams &p, float x, float y, float z, bool *mask) {
  int plane = 0;
  bool any = false;
  const float m = p.size_margin;
  for (int i = p.n_tpc - 1; i >= 0; --i) {
    float bz0 = border(p, i, 2, 0), bz1 = border(p, i, 2, 1);
    float zmin = fminf(__fsub_rn(bz1, m), __fsub_rn(bz0, m));
    float zmax = fmaxf(__fadd_rn(bz1, m), __fadd_rn(bz0, m));
    bool c = x >= __fsub_rn(border(p, i, 0, 0), m) && x <= __fadd_rn(border(p, i, 0, 1), m) &&
             y >= __fsub_rn(border(p, i, 1, 0), m) && y <= __fadd_rn(border(p, i, 1, 1), m) &&
             z >= zmin && z <= zmax;
    if (c) { plane = i; any = true; }   // argmax: first true
  }
  *mask = any;
  return plane;
}

// 1-D Gaussian bin integrals over 5 bins with open outer edges
// (gaussian_1d_integral_new, detsim_jax.py:332-341) and d/dsigma.
__device__ __forceinline__ void bin_integrals(const LsimParams &p, float x0, float sigma, float out[kMaxTran],
                                              float dout[kMaxTran]) {
  const int nb = p.n_tran_bins;
  float e[kMaxTran + 1], de[kMaxTran + 1];
  e[0] = -1.0f; de[0] = 0.f;
  e[nb] = 1.0f; de[nb] = 0.f;
  const float s2 = 1.41421356237309515f;        // float32(sqrt(2)), as jnp.sqrt(2)
  const float den = __fmul_rn(s2, sigma);
  const float two_over_sqrtpi = 1.12837916709551257f;
  for (int k = 1; k < nb; ++k) {
    float u = __fsub_rn(p.tran_edges[k], x0);
    float z = __fdiv_rn(u, den);
    e[k] = erff(z);
    // d erf(u/(sqrt2*sigma)) / d sigma = 2/sqrt(pi) * exp(-z^2) * (-z/sigma)
    de[k] = two_over_sqrtpi * expf(-z * z) * (-z / sigma);
  }
  for (int k = 0; k < nb; ++k) {
    out[k] = __fmul_rn(0.5f, __fsub_rn(e[k + 1], e[k]));
    dout[k] = 0.5f * (de[k + 1] - de[k]);
  }
}

// K1, LUT mode: one thread per track row.
// Fit parameters from device memory (lsim_lut_stage1_theta): theta in the
// gradient order, the derived quantities computed in float64 as
// _abi.make_params does on the host (get_vdrift, consts_jax.py:192-217, and
// its analytic derivative) and rounded once to float32.
// out: Ab, kb, erho, vdrift, lifetime, long_diff, tran_diff, eField,
// lArDensity, dvdrift/deField.
__global__ void k_theta_derive(LsimParams p, const float *__restrict__ theta, float *out) {
  if (threadIdx.x != 0) return;
  const double e = theta[2], rho = theta[7];
  const double *a = p.mobility;
  const double se = sqrt(e);
  const double num = a[0] + a[1] * e + a[2] * pow(e, 1.5) + a[3] * pow(e, 2.5);
  const double den = 1.0 + (a[1] / a[0]) * e + a[4] * pow(e, 2.0) + a[5] * pow(e, 3.0);
  const double mu = num / den * p.mobility_temp;
  const double dnum = a[1] + 1.5 * a[2] * se + 2.5 * a[3] * pow(e, 1.5);
  const double dden = (a[1] / a[0]) + 2.0 * a[4] * e + 3.0 * a[5] * e * e;
  const double dmu = (dnum * den - num * dden) / (den * den) * p.mobility_temp;
  out[0] = theta[0];
  out[1] = theta[1];
  out[2] = (float)(e * rho);
  out[3] = (float)(mu * e);
  out[4] = theta[3];
  out[5] = theta[5];
  out[6] = theta[6];
  out[7] = theta[2];
  out[8] = theta[7];
  out[9] = (float)(dmu * e + mu);
}

__global__ void k_segments_lut(LsimParams p, LsimFieldMap f, const float *__restrict__ tracks, int64_t n_rows,
                               int32_t n_events, Workspace w, Grid g, const float *__restrict__ derived) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n_rows) return;
  const Phys ph = phys_of(p, derived);
  TrackRow t = load_row(p, f, tracks, s);
  if (t.event < -1 || t.event >= n_events) {
    set_status(w.counts, LSIM_ERR_INVALID, (int)s);
    t.event = -1;
  }
  // quench (quenching_jax.py:73-74)
  float dR[4];
  float R = recombination(p, ph, t, dR);
  float ne0 = __fmul_rn(__fmul_rn(R, t.dE), p.mev_to_electrons);
  // drift (drifting_jax.py:34-50)
  bool mask;
  int plane = tpc_plane(p, t.x, t.y, t.z, &mask);
  float z_anode = border(p, plane, 2, 0);
  float dist = __fadd_rn(fabsf(__fsub_rn(t.z, z_anode)), 1e-6f);
  const float v = ph.vdrift;
  float tdr = __fdiv_rn(dist, v);
  float red = expf(__fdiv_rn(-tdr, ph.lifetime));
  float mf = mask ? 1.0f : 0.0f;
  float ne = __fmul_rn(__fmul_rn(ne0, red), mf);
  float sigL = sqrtf(__fmul_rn(__fmul_rn(tdr, 2.0f), ph.long_diff));
  float sigT = sqrtf(__fmul_rn(__fmul_rn(tdr, 2.0f), ph.tran_diff));
  // binning (get_bin_shifts, detsim_jax.py:505-510; sim_jax.py:405-409)
  float bx0 = border(p, plane, 0, 0), by0 = border(p, plane, 1, 0);
  float relx = __fsub_rn(t.x, bx0), rely = __fsub_rn(t.y, by0);
  int bx = (int)jax_floordiv_f32(relx, p.bin_width);
  int by = (int)jax_floordiv_f32(rely, p.bin_width);
  float x0 = jax_rem_f32(relx, p.bin_width);
  float y0 = jax_rem_f32(rely, p.bin_width);
  SegFwd r;
  SegAdj a;
  bin_integrals(p, x0, sigT, r.ex, a.dex);
  bin_integrals(p, y0, sigT, r.ey, a.dey);
  // time: cathode-referenced t0 (sim_jax.py:418-420), long diffusion in ticks (:423)
  float z_cathode = border(p, plane, 2, 1);
  float t0 = __fdiv_rn(fabsf(__fsub_rn(t.z, z_cathode)), v);
  float ld = __fdiv_rn(__fdiv_rn(sigL, v), p.t_sampling);
  float ft = __fdiv_rn(t0, p.t_sampling);
  float fl = floorf(ft);
  int cath = (fl >= (float)(p.lut_nt - 1)) ? p.lut_nt - 1 : (fl <= 0.f ? 0 : (int)fl);
  float frac = __fsub_rn(ft, (float)cath);
  // template interpolation weights (sim_jax.py:162-168)
  const int T = p.n_templates;
  int idx = searchsorted_left(p.long_diff_template, T, ld);
  idx = idx < 1 ? 1 : (idx > T - 2 ? T - 2 : idx);
  float X0 = p.long_diff_template[idx - 1], X1 = p.long_diff_template[idx], X2 = p.long_diff_template[idx + 1];
  float d01 = __fmul_rn(__fsub_rn(X0, X1), __fsub_rn(X0, X2));
  float d10 = __fmul_rn(__fsub_rn(X1, X0), __fsub_rn(X1, X2));
  float d20 = __fmul_rn(__fsub_rn(X2, X0), __fsub_rn(X2, X1));
  float l0 = __fsub_rn(ld, X0), l1 = __fsub_rn(ld, X1), l2 = __fsub_rn(ld, X2);
  r.qa = __fdiv_rn(__fmul_rn(l1, l2), d01);
  r.qb = __fdiv_rn(__fmul_rn(l0, l2), d10);
  r.qc = __fdiv_rn(__fmul_rn(l0, l1), d20);
  r.ne = ne;
  r.frac = frac;
  r.cath = cath;
  r.tidx = idx;
  r.bx = bx;
  r.by = by;
  r.plane = plane;
  r.event = t.event;
  r.sigT = sigT;
  r.t0 = t0;
  r.ld = ld;
  // ---- adjoint partials (parameter order: Ab kb eField lifetime vdrift long_diff tran_diff lArDensity)
  const float dv = ph.dvdrift;
  float dtdE = -tdr * dv / v;
  float k = t.dE * p.mev_to_electrons * red * mf;
  a.dne[0] = dR[0] * k;
  a.dne[1] = dR[1] * k;
  a.dne[2] = dR[2] * k + ne * (-1.0f / ph.lifetime) * dtdE;
  a.dne[3] = ne * tdr / (ph.lifetime * ph.lifetime);
  a.dne[4] = dR[3] * k;
  a.dsig[0] = (ph.tran_diff / sigT) * dtdE;
  a.dsig[1] = tdr / sigT;
  a.dld[0] = ((ph.long_diff / sigL) * dtdE / v - sigL * dv / (v * v)) / p.t_sampling;
  a.dld[1] = (tdr / sigL) / v / p.t_sampling;
  a.dt0 = -t0 * dv / v;
  a.dqa = (l1 + l2) / d01;
  a.dqb = (l0 + l2) / d10;
  a.dqc = (l0 + l1) / d20;
  a.pad[0] = 0.f;
  w.segf[s] = r;
  w.sega[s] = a;
  SegNb nbr;
  nbr.ne = ne;
  nbr.frac = frac;
  nbr.cath = cath;
  nbr.bxy = (int)(((unsigned)bx & 0xffffu) | ((unsigned)by << 16));
  if (ne != 0.f && (bx < -32768 || bx > 32767 || by < -32768 || by > 32767)) {
    set_status(w.counts, LSIM_ERR_UNSUPPORTED, (int)s);
    nbr.ne = 0.f;
  }
  w.segn[s] = nbr;
  SegNbAdj nba;
  nba.dne03 = make_float4(a.dne[0], a.dne[1], a.dne[2], a.dne[3]);
  nba.dne4_dt0 = make_float4(a.dne[4], a.dt0, 0.f, 0.f);
  w.segna[s] = nba;
  // ---- principal pixel, main pixel id, grid slot
  const int nb = p.nb_bins_per_pixel;
  int ppx = ifloordiv(bx, nb), ppy = ifloordiv(by, nb);
  int32_t pid = pixel2id(p, ppx, ppy, plane, t.event);
  w.pid[s] = pid;
  if (pid == -1) atomicExch(&w.counts->any_m1, 1);
  int32_t key = -1;
  const int h = g.h;
  if (t.event >= 0) {
    if (ppx >= -h && ppx < p.n_pixels_x + h && ppy >= -h && ppy < p.n_pixels_y + h)
      key = (int32_t)((t.event + 1) * g.event_stride + plane * g.plane_stride + (int64_t)(ppy + h) * g.nxe + (ppx + h));
  } else if (pid != -1) {
    key = (int32_t)(plane * g.plane_stride + (int64_t)(ppy + h) * g.nxe + (ppx + h));
  }
  w.key[s] = key;
  if (key >= 0) atomicAdd(&w.cnt[key], 1);
}

// K1, parametrised mode (number_pix_neighbors == 0): Monte-Carlo diffusion
// offsets supplied as standard normals (S, 3).
__global__ void k_segments_param(LsimParams p, LsimFieldMap f, const float *__restrict__ tracks,
                                 const float *__restrict__ normals, int64_t n_rows, int32_t n_events,
                                 Workspace w, Grid g) {
  const Phys ph = phys_of(p, nullptr);
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n_rows) return;
  TrackRow t = load_row(p, f, tracks, s);
  if (t.event < -1 || t.event >= n_events) {
    set_status(w.counts, LSIM_ERR_INVALID, (int)s);
    t.event = -1;
  }
  float dR[4];
  float R = recombination(p, ph, t, dR);
  float ne0 = __fmul_rn(__fmul_rn(R, t.dE), p.mev_to_electrons);
  bool mask;
  int plane = tpc_plane(p, t.x, t.y, t.z, &mask);
  float z_anode = border(p, plane, 2, 0);
  float dist = __fadd_rn(fabsf(__fsub_rn(t.z, z_anode)), 1e-6f);
  const float v = ph.vdrift;
  float tdr = __fdiv_rn(dist, v);
  float red = expf(__fdiv_rn(-tdr, ph.lifetime));
  float ne = __fmul_rn(__fmul_rn(ne0, red), mask ? 1.0f : 0.0f);
  float sigL = sqrtf(__fmul_rn(__fmul_rn(tdr, 2.0f), ph.long_diff));
  float sigT = sqrtf(__fmul_rn(__fmul_rn(tdr, 2.0f), ph.tran_diff));
  // generate_electrons (detsim_jax.py:390-399)
  float nx = normals ? normals[3 * s + 0] : 0.f;
  float ny = normals ? normals[3 * s + 1] : 0.f;
  float nz = normals ? normals[3 * s + 2] : 0.f;
  float xe = __fadd_rn(t.x, __fmul_rn(nx, sigT));
  float ye = __fadd_rn(t.y, __fmul_rn(ny, sigT));
  float ze = p.diffusion_in_current_sim ? t.z : __fadd_rn(t.z, __fmul_rn(nz, sigL));
  // get_pixels (detsim_jax.py:481-491)
  float bx0 = border(p, plane, 0, 0), by0 = border(p, plane, 1, 0);
  int px = (int)jax_floordiv_f32(__fsub_rn(xe, bx0), p.pixel_pitch);
  int py = (int)jax_floordiv_f32(__fsub_rn(ye, by0), p.pixel_pitch);
  int32_t pid = pixel2id(p, px, py, plane, t.event);
  // current_mc geometry (detsim_jax.py:623-633), pixel centre from the id
  float pcx = __fadd_rn(__fadd_rn(__fmul_rn((float)px, p.pixel_pitch), bx0), p.half_pitch);
  float pcy = __fadd_rn(__fadd_rn(__fmul_rn((float)py, p.pixel_pitch), by0), p.half_pitch);
  float t0 = __fdiv_rn(fabsf(__fsub_rn(ze, z_anode)), v);
  int t0_tick = (int)__fadd_rn(__fdiv_rn(t0, p.t_sampling), 0.5f);
  SegPar r;
  r.ne = ne;
  r.t0f = __fsub_rn(t0, __fmul_rn((float)t0_tick, p.t_sampling));
  r.t0_tick = t0_tick;
  r.xd = fabsf(__fsub_rn(xe, pcx));
  r.yd = fabsf(__fsub_rn(ye, pcy));
  r.sigma = __fdiv_rn(sigL, v);
  r.plane = plane;
  r.event = t.event;
  r.px = px;
  r.py = py;
  for (int i = 0; i < 6; ++i) r.pad[i] = 0.f;
  w.segp[s] = r;
  // ---- adjoint partials (the current model's inputs; parameter order as in LUT mode)
  {
    const float dv = ph.dvdrift;
    const float dtdE = -tdr * dv / v;
    const float k = t.dE * p.mev_to_electrons * red * (mask ? 1.0f : 0.0f);
    SegParAdj ja;
    ja.dne[0] = dR[0] * k;
    ja.dne[1] = dR[1] * k;
    ja.dne[2] = dR[2] * k + ne * (-1.0f / ph.lifetime) * dtdE;
    ja.dne[3] = ne * tdr / (ph.lifetime * ph.lifetime);
    ja.dne[4] = dR[3] * k;
    const float dsT_E = sigT > 0.f ? (ph.tran_diff / sigT) * dtdE : 0.f;
    const float dsT_D = sigT > 0.f ? tdr / sigT : 0.f;
    const float dsL_E = sigL > 0.f ? (ph.long_diff / sigL) * dtdE : 0.f;
    const float dsL_D = sigL > 0.f ? tdr / sigL : 0.f;
    // |u| passes sign(u) (0 at 0, as jnp.abs)
    const float ux = xe - pcx, uy = ye - pcy;
    const float sx = ux > 0.f ? 1.f : (ux < 0.f ? -1.f : 0.f);
    const float sy = uy > 0.f ? 1.f : (uy < 0.f ? -1.f : 0.f);
    ja.dxd[0] = sx * nx * dsT_E;
    ja.dxd[1] = sx * nx * dsT_D;
    ja.dyd[0] = sy * ny * dsT_E;
    ja.dyd[1] = sy * ny * dsT_D;
    // t0 = |z - z_anode| / v (z carries no offset with the smeared current model)
    ja.dt0f[0] = -t0 * dv / v;
    ja.dt0f[1] = 0.f;
    ja.dsig[0] = dsL_E / v - sigL * dv / (v * v);
    ja.dsig[1] = dsL_D / v;
    for (int i = 0; i < 11; ++i) ja.pad[i] = 0.f;
    *reinterpret_cast<SegParAdj *>(w.sega + s) = ja;
  }
  w.pid[s] = pid;
  if (pid == -1) atomicExch(&w.counts->any_m1, 1);
  int32_t key = -1;
  if (pid != -1)
    key = (int32_t)((t.event + 1) * g.event_stride + plane * g.plane_stride + (int64_t)(py + g.h) * g.nxe +
                    (px + g.h));
  w.key[s] = key;
  if (key >= 0) atomicAdd(&w.cnt[key], 1);
}

// ---------------------------------------------------------------- scan

__device__ __forceinline__ void slot_flags(const Grid &g, int64_t slot, int c, int *fv, int *fe) {
  *fv = 0; *fe = 0;
  if (c <= 0) return;
  int64_t ev = slot / g.event_stride;       // 0 means event -1
  int64_t rem = slot - ev * g.event_stride;
  int64_t inplane = rem % g.plane_stride;
  int pye = (int)(inplane / g.nxe), pxe = (int)(inplane % g.nxe);
  bool interior = pxe >= g.h && pxe < g.nxe - g.h && pye >= g.h && pye < g.nye - g.h;
  if (!interior) return;
  if (ev == 0) *fe = 1; else *fv = 1;
}

// Block-local sums of (count, valid flag, em1 flag) over kScanTile slots.
__global__ void k_scan_reduce(const int32_t *__restrict__ cnt, int64_t G, Grid g, int32_t *__restrict__ blocks) {
  __shared__ int sh[3][kScanThreads / kWarp];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int a = 0, b = 0, c = 0;
  for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
    int64_t slot = base + i;
    if (slot < G) {
      int v = cnt[slot], fv, fe;
      slot_flags(g, slot, v, &fv, &fe);
      a += v; b += fv; c += fe;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  int wid = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  if (lane == 0) { sh[0][wid] = a; sh[1][wid] = b; sh[2][wid] = c; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int ta = 0, tb = 0, tc = 0;
    for (int i = 0; i < kScanThreads / kWarp; ++i) { ta += sh[0][i]; tb += sh[1][i]; tc += sh[2][i]; }
    blocks[3 * blockIdx.x + 0] = ta;
    blocks[3 * blockIdx.x + 1] = tb;
    blocks[3 * blockIdx.x + 2] = tc;
  }
}

// Exclusive scan of the block sums (one CTA), totals into counts.
__global__ void k_scan_blocks(int32_t *blocks, int64_t nblocks, LsimCounts *counts) {
  __shared__ int carry[3];
  __shared__ int wsum[3][kScanThreads / kWarp];
  if (threadIdx.x < 3) carry[threadIdx.x] = 0;
  __syncthreads();
  int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  for (int64_t base = 0; base < nblocks; base += kScanThreads) {
    int64_t i = base + threadIdx.x;
    int v[3];
    for (int k = 0; k < 3; ++k) v[k] = (i < nblocks) ? blocks[3 * i + k] : 0;
    int incl[3];
    for (int k = 0; k < 3; ++k) {
      int x = v[k];
      for (int o = 1; o < kWarp; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      incl[k] = x;
      if (lane == kWarp - 1) wsum[k][wid] = x;
    }
    __syncthreads();
    int wofs[3] = {0, 0, 0}, tot[3] = {0, 0, 0};
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < kScanThreads / kWarp; ++j) {
        if (j < wid) wofs[k] += wsum[k][j];
        tot[k] += wsum[k][j];
      }
    if (i < nblocks)
      for (int k = 0; k < 3; ++k) blocks[3 * i + k] = carry[k] + wofs[k] + incl[k] - v[k];
    __syncthreads();
    if (threadIdx.x < 3) carry[threadIdx.x] += tot[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    counts->n_valid = carry[1];
    counts->n_em1 = carry[2];
  }
}

// Final pass: per-slot exclusive offsets, and the row lists of valid and
// negative-id pixels in ascending slot (= ascending pixel id) order.
__global__ void k_scan_final(const int32_t *__restrict__ cnt, int64_t G, Grid g, const int32_t *__restrict__ blocks,
                             int32_t *__restrict__ off, int32_t *__restrict__ pix_slot, int32_t *__restrict__ em1_slot) {
  constexpr int PER = kScanTile / kScanThreads;   // 8 consecutive slots per thread
  __shared__ int wsum[3][kScanThreads / kWarp];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * PER;
  int v[PER], fv[PER], fe[PER];
  int la = 0, lb = 0, lc = 0;
  for (int i = 0; i < PER; ++i) {
    int64_t slot = base + i;
    v[i] = slot < G ? cnt[slot] : 0;
    slot_flags(g, slot, v[i], &fv[i], &fe[i]);
    la += v[i]; lb += fv[i]; lc += fe[i];
  }
  int lane = threadIdx.x % kWarp, wid = threadIdx.x / kWarp;
  int tot[3] = {la, lb, lc}, ex[3];
  for (int k = 0; k < 3; ++k) {
    int x = tot[k];
    for (int o = 1; o < kWarp; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    ex[k] = x - tot[k];
    if (lane == kWarp - 1) wsum[k][wid] = x;
  }
  __syncthreads();
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < wid; ++j) ex[k] += wsum[k][j];
  int ra = blocks[3 * blockIdx.x + 0] + ex[0];
  int rb = blocks[3 * blockIdx.x + 1] + ex[1];
  int rc = blocks[3 * blockIdx.x + 2] + ex[2];
  for (int i = 0; i < PER; ++i) {
    int64_t slot = base + i;
    if (slot >= G) break;
    off[slot] = ra;
    if (fv[i]) pix_slot[rb] = (int32_t)slot;
    if (fe[i]) em1_slot[rc] = (int32_t)slot;
    ra += v[i]; rb += fv[i]; rc += fe[i];
  }
}

// Scatter segment indices into their slot ranges.
__global__ void k_scatter(const int32_t *__restrict__ key, int64_t n_rows, const int32_t *__restrict__ off,
                          int32_t *__restrict__ cursor, int32_t *__restrict__ seg_list) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n_rows) return;
  int32_t k = key[s];
  if (k < 0) return;
  int pos = off[k] + atomicAdd(&cursor[k], 1);
  seg_list[pos] = (int32_t)s;
}

// Sort each slot's segment list ascending so accumulation order, and hence
// every float32 result, is deterministic.  Lists of up to kSortLocal
// segments are sorted here by one thread; longer ones are queued for
// k_sort_big_slots.
// List-ordered copies of the compact neighbour-pass records (LUT mode;
// lnb null in parametrised mode): entry i of the slot lists gets the record
// of segment seg_list[i].
__device__ __forceinline__ void copy_list_records(const Workspace &w, int64_t pos, int32_t s) {
  if (!w.lnb) return;
  w.lnb[pos] = w.segn[s];
  w.lna[pos] = w.segna[s];
}

__global__ void k_sort_slots(const int32_t *__restrict__ cnt, const int32_t *__restrict__ off, int64_t G,
                             int32_t *__restrict__ seg_list, int32_t *__restrict__ big_slots, LsimCounts *counts,
                             Workspace w) {
  int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int c = slot < G ? cnt[slot] : 0;
  // one atomic per warp for the largest slot (a shared counter is hot)
  const int cmax = __reduce_max_sync(0xffffffffu, c);
  if ((threadIdx.x % kWarp) == 0 && cmax > 1) {
    atomicMax(&counts->max_slot, cmax);
    if (cmax > kMaxSlotSegments) atomicCAS(&counts->status, 0, (int)LSIM_ERR_CAPACITY);
  }
  if (c <= 0) return;
  const int64_t o = off[slot];
  int32_t *l = seg_list + o;
  if (c == 1) {
    copy_list_records(w, o, l[0]);
    return;
  }
  if (c > kSortLocal) {
    big_slots[atomicAdd(&counts->n_big_slots, 1)] = (int32_t)slot;
    return;
  }
  {
    // short lists (nearly all): insertion sort in a thread-local copy
    int32_t v[kSortLocal];
    for (int i = 0; i < c; ++i) v[i] = l[i];
    for (int i = 1; i < c; ++i) {
      const int32_t x = v[i];
      int j = i - 1;
      while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; --j; }
      v[j + 1] = x;
    }
    for (int i = 0; i < c; ++i) {
      l[i] = v[i];
      copy_list_records(w, o + i, v[i]);
    }
  }
}

// One block per queued long list: bitonic sort in shared memory for lists
// up to kSortBig entries, a block-wide odd-even transposition sort in place
// beyond (lists that long do not occur in practice).
constexpr int kSortBig = 8192;
constexpr int kSortThreads = 256;

__global__ void __launch_bounds__(kSortThreads) k_sort_big_slots(const int32_t *__restrict__ cnt,
                                                                 const int32_t *__restrict__ off,
                                                                 int32_t *__restrict__ seg_list,
                                                                 const int32_t *__restrict__ big_slots,
                                                                 const LsimCounts *counts, Workspace w) {
  __shared__ int32_t sh[kSortBig];
  const int nbig = counts->n_big_slots;
  for (int b = blockIdx.x; b < nbig; b += gridDim.x) {
    const int64_t slot = big_slots[b];
    const int c = cnt[slot];
    int32_t *l = seg_list + off[slot];
    if (c <= kSortBig) {
      int n2 = 1;
      while (n2 < c) n2 <<= 1;
      for (int i = threadIdx.x; i < n2; i += kSortThreads) sh[i] = i < c ? l[i] : INT32_MAX;
      __syncthreads();
      for (int k = 2; k <= n2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int i = threadIdx.x; i < n2; i += kSortThreads) {
            const int ij = i ^ j;
            if (ij > i) {
              const bool up = (i & k) == 0;
              const int32_t a = sh[i], d = sh[ij];
              if ((a > d) == up) { sh[i] = d; sh[ij] = a; }
            }
          }
          __syncthreads();
        }
      for (int i = threadIdx.x; i < c; i += kSortThreads) {
        l[i] = sh[i];
        copy_list_records(w, off[slot] + i, sh[i]);
      }
    } else {
      for (int phase = 0; phase < c; ++phase) {
        for (int i = 2 * threadIdx.x + (phase & 1); i + 1 < c; i += 2 * kSortThreads) {
          const int32_t a = l[i], d = l[i + 1];
          if (a > d) { l[i] = d; l[i + 1] = a; }
        }
        __syncthreads();
      }
      for (int i = threadIdx.x; i < c; i += kSortThreads) copy_list_records(w, off[slot] + i, l[i]);
    }
    __syncthreads();
  }
}

// unique_pixels rows and zeroed garbage waveform rows (stage 2 prologue).
__global__ void k_fill_unique(LsimParams p, Grid g, const int32_t *__restrict__ pix_slot,
                              const int32_t *__restrict__ em1_slot, int64_t p_pad, int32_t n_em1, int32_t n_valid,
                              int32_t *__restrict__ unique_pixels) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= p_pad) return;
  int64_t n_m1 = p_pad - n_em1 - n_valid;
  int32_t pid;
  int64_t slot = -1;
  if (r < n_em1) slot = em1_slot[r];
  else if (r >= n_em1 + n_m1) slot = pix_slot[r - n_em1 - n_m1];
  if (slot < 0) {
    pid = -1;
  } else {
    int64_t ev = slot / g.event_stride;
    int64_t rem = slot - ev * g.event_stride;
    int plane = (int)(rem / g.plane_stride);
    int64_t inplane = rem % g.plane_stride;
    int py = (int)(inplane / g.nxe) - g.h, px = (int)(inplane % g.nxe) - g.h;
    pid = pixel2id(p, px, py, plane, (int)ev - 1);
  }
  unique_pixels[r] = pid;
}

// ---------------------------------------------------------------- host drivers

int run_pixel_map(const LsimParams &p, const Workspace &w0, const Grid &g, int64_t n_rows, cudaStream_t st,
                  bool list_records) {
  Workspace w = w0;
  if (!list_records) w.lnb = nullptr, w.lna = nullptr;
  int64_t nscan = (g.G + kScanTile - 1) / kScanTile;
  if (nscan > 0) {
    k_scan_reduce<<<(unsigned)nscan, kScanThreads, 0, st>>>(w.cnt, g.G, g, w.scan_blocks);
    k_scan_blocks<<<1, kScanThreads, 0, st>>>(w.scan_blocks, nscan, w.counts);
    k_scan_final<<<(unsigned)nscan, kScanThreads, 0, st>>>(w.cnt, g.G, g, w.scan_blocks, w.off, w.pix_slot,
                                                          w.em1_slot);
  }
  if (cudaMemsetAsync(w.cursor, 0, 4 * (size_t)g.G, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (n_rows > 0) k_scatter<<<(unsigned)((n_rows + 255) / 256), 256, 0, st>>>(w.key, n_rows, w.off, w.cursor, w.seg_list);
  if (g.G > 0) {
    k_sort_slots<<<(unsigned)((g.G + 255) / 256), 256, 0, st>>>(w.cnt, w.off, g.G, w.seg_list, w.big_slots,
                                                                 w.counts, w);
    k_sort_big_slots<<<(unsigned)(device_sm_count() * 4), kSortThreads, 0, st>>>(w.cnt, w.off, w.seg_list,
                                                                                w.big_slots, w.counts, w);
  }
  return LSIM_OK;
}

int run_stage1(bool param_mode, const LsimParams &p, const LsimFieldMap &f, const float *tracks,
               const float *normals, int64_t n_rows, int32_t n_events, const Workspace &w, cudaStream_t st,
               const float *theta_dev) {
  Grid g = make_grid(p, n_events);
  k_reset_counts<<<1, 32, 0, st>>>(w.counts);
  if (theta_dev) k_theta_derive<<<1, 32, 0, st>>>(p, theta_dev, w.theta_derived);
  if (cudaMemsetAsync(w.cnt, 0, 4 * (size_t)g.G, st) != cudaSuccess) return LSIM_ERR_CUDA;
  if (n_rows > 0) {
    unsigned nb = (unsigned)((n_rows + 127) / 128);
    if (param_mode)
      k_segments_param<<<nb, 128, 0, st>>>(p, f, tracks, normals, n_rows, n_events, w, g);
    else
      k_segments_lut<<<nb, 128, 0, st>>>(p, f, tracks, n_rows, n_events, w, g,
                                         theta_dev ? w.theta_derived : nullptr);
  }
  return run_pixel_map(p, w, g, n_rows, st, !param_mode);
}

int run_fill_unique(const LsimParams &p, const Workspace &w, const Grid &g, int64_t p_pad, int32_t n_em1,
                    int32_t n_valid, int32_t *unique_pixels, float *wfs, int32_t nt_out, cudaStream_t st) {
  if (p_pad <= 0) return LSIM_OK;
  if (unique_pixels)
    k_fill_unique<<<(unsigned)((p_pad + 127) / 128), 128, 0, st>>>(p, g, w.pix_slot, w.em1_slot, p_pad, n_em1,
                                                                    n_valid, unique_pixels);
  // rows with a negative pixel id come first and are zero
  int64_t n_garbage = p_pad - n_valid;
  if (wfs && n_garbage > 0 &&
      cudaMemsetAsync(wfs, 0, sizeof(float) * (size_t)n_garbage * (size_t)nt_out, st) != cudaSuccess)
    return LSIM_ERR_CUDA;
  return LSIM_OK;
}

// ---------------------------------------------------------------- optimiser

// One Adam step over the LSIM_NPARAM fit parameters (one thread each) in
// "divide" normalisation: the optimiser works on theta / scale with
// gradients g * scale (optax.adam: bias-corrected moments, eps added to
// sqrt(v_hat)).  state = m[8], v[8], step count; skipped when any gradient is
// not finite.
__global__ void k_adam(float *theta, const float *grad, const float *scale, const float *lr, float *state,
                       float beta1, float beta2, float eps) {
  const int i = threadIdx.x;
  const float g = i < LSIM_NPARAM ? grad[i] * scale[i] : 0.f;
  const bool bad = __any_sync(0xffffffffu, i < LSIM_NPARAM && !isfinite(g));
  if (bad || i >= LSIM_NPARAM) return;
  const float t = state[2 * LSIM_NPARAM] + 1.f;
  const float m = beta1 * state[i] + (1.f - beta1) * g;
  const float v = beta2 * state[LSIM_NPARAM + i] + (1.f - beta2) * g * g;
  state[i] = m;
  state[LSIM_NPARAM + i] = v;
  const float mh = m / (1.f - powf(beta1, t)), vh = v / (1.f - powf(beta2, t));
  const float xn = theta[i] / scale[i] - lr[i] * mh / (sqrtf(vh) + eps);
  theta[i] = xn * scale[i];
  __syncwarp(0xffu);
  if (i == 0) state[2 * LSIM_NPARAM] = t;
}

int run_adam(float *theta, const float *grad, const float *scale, const float *lr, float *state, float beta1,
             float beta2, float eps, cudaStream_t st) {
  k_adam<<<1, 32, 0, st>>>(theta, grad, scale, lr, state, beta1, beta2, eps);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

// ---------------------------------------------------------------- fit step
//
// The reference's GradientDescentFitter (optimize/fit_params.py:781-895):
// the optimiser works on normalised parameters u, phys = map_norm_to_phys(u)
// (:168-179); gradients are taken with respect to u.  One warp, lane i for
// parameter i; float32 throughout, as the reference computes.

// jax.nn.sigmoid in float32: 1 / (1 + exp(-x)).
__device__ __forceinline__ float fit_sigmoid(float x) { return 1.f / (1.f + expf(-x)); }

__device__ __forceinline__ float norm_to_phys(const LsimFitOptions &o, int i, float u) {
  const float k = o.norm_scale;
  if (o.scheme == LSIM_NORM_SIGMOID) return o.lo[i] + (o.hi[i] - o.lo[i]) * fit_sigmoid(k * u);
  if (o.scheme == LSIM_NORM_EXP_LOG) return o.nom[i] * expf(k * u);
  return u * o.norm[i];
}

// d phys / d u, the chain rule JAX applies through norm_to_phys.
__device__ __forceinline__ float dphys_du(const LsimFitOptions &o, int i, float u) {
  const float k = o.norm_scale;
  if (o.scheme == LSIM_NORM_SIGMOID) {
    const float sg = fit_sigmoid(k * u);
    return (o.hi[i] - o.lo[i]) * (sg * (1.f - sg)) * k;
  }
  if (o.scheme == LSIM_NORM_EXP_LOG) return o.nom[i] * expf(k * u) * k;
  return o.norm[i];
}

// map_phys_to_norm (fit_params.py:182-199) in float32.
__device__ __forceinline__ float phys_to_norm(const LsimFitOptions &o, int i, float v) {
  const float k = o.norm_scale;
  if (o.scheme == LSIM_NORM_SIGMOID) {
    const float eps = 1.1920928955078125e-07f;   // float32 machine epsilon
    float fr = (v - o.lo[i]) / (o.hi[i] - o.lo[i]);
    fr = fminf(fmaxf(fr, eps), 1.f - eps);
    return logf(fr / (1.f - fr)) / k;
  }
  if (o.scheme == LSIM_NORM_EXP_LOG) return logf(fmaxf(v, 1.17549435e-38f) / o.nom[i]) / k;
  return v != 0.f ? 1.f : 0.f;
}

constexpr int kFitM = 0, kFitV = LSIM_NPARAM, kFitU = 2 * LSIM_NPARAM, kFitT = 3 * LSIM_NPARAM;
static_assert(kFitT < LSIM_FIT_STATE, "fit-step state layout");

__global__ void k_fit_init(float *theta, LsimFitOptions o, float *state) {
  const int i = threadIdx.x;
  if (i < LSIM_FIT_STATE) state[i] = 0.f;
  if (i >= LSIM_NPARAM || !((o.fit_mask >> i) & 1)) return;
  const float u = phys_to_norm(o, i, theta[i]);
  state[kFitU + i] = u;
  theta[i] = norm_to_phys(o, i, u);
}

__global__ void k_fit_step(float *theta, const float *grad, LsimFitOptions o, float *state) {
  const int i = threadIdx.x;
  const bool fit = i < LSIM_NPARAM && ((o.fit_mask >> i) & 1);
  const float u = fit ? state[kFitU + i] : 0.f;
  float g = fit ? grad[i] * dphys_du(o, i, u) : 0.f;
  // a NaN gradient skips the whole update (process_grads returns early)
  if (__any_sync(0xffffffffu, fit && isnan(g))) return;
  if (o.scheme == LSIM_NORM_DIVIDE) g = g * o.norm[i & (LSIM_NPARAM - 1)];
  // optax.clip_by_global_norm: scaled to the threshold when the norm reaches it
  float sq = g * g;
  for (int off = 16; off > 0; off >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, off);
  const float gnorm = sqrtf(sq);
  if (o.max_clip_norm > 0.f && !(gnorm < o.max_clip_norm)) g = (g / gnorm) * o.max_clip_norm;
  const float t = state[kFitT] + 1.f;
  __syncwarp();
  if (i == 0) state[kFitT] = t;
  if (!fit) return;
  // optax.adam: bias-corrected moments, eps outside the square root, then -lr
  const float m = o.beta1 * state[kFitM + i] + (1.f - o.beta1) * g;
  const float v = o.beta2 * state[kFitV + i] + (1.f - o.beta2) * (g * g);
  state[kFitM + i] = m;
  state[kFitV + i] = v;
  const float mh = m / (1.f - powf(o.beta1, t)), vh = v / (1.f - powf(o.beta2, t));
  float un = u + (-o.lr[i]) * (mh / (sqrtf(vh) + o.eps));
  if (o.scheme == LSIM_NORM_DIVIDE && o.clip_from_range)
    un = fmaxf(o.down[i] / o.norm[i], fminf(o.up[i] / o.norm[i], un));
  state[kFitU + i] = un;
  theta[i] = norm_to_phys(o, i, un);
}

int run_fit_init(float *theta, const LsimFitOptions &o, float *state, cudaStream_t st) {
  k_fit_init<<<1, 32, 0, st>>>(theta, o, state);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

int run_fit_step(float *theta, const float *grad, const LsimFitOptions &o, float *state, cudaStream_t st) {
  k_fit_step<<<1, 32, 0, st>>>(theta, grad, o, state);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
