// Monte-Carlo collisions of electrons with the neutral gas
// (CollisionHandler, src/collision.cpp:60-207) for both particle layouts.
//
// Built with -fmad=false: the collision arithmetic keeps the reference's
// association order (the FP64 form is compared with the reference draw for
// draw on injected uniforms).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "epic_batch.cuh"
#include "epic_device.cuh"
#include "epic_internal.cuh"

namespace epic {

// ---------------------------------------------------------------- MCC ---
// Draws come from Philox (epic_device.cuh), counter-based, so the k-th draw of
// electron p at step s is a pure function of (p, s, k, seed); or, in check
// mode, from an injected array.
struct Injected {
  const double* u;
  __device__ double next() { return *u++; }
};

// Cross-section lookup: reference linear table (nearest index,
// src/collision.cpp:194-197) or the logarithmic extension.
struct Sigma {
  double tot, ela, exc, ion;
};

__device__ __forceinline__ Sigma sigma_at(const CrossSections& cs, double energy, double velocity_unused) {
  Sigma s;
  if (cs.kind == 0) {
    int idx = (int)(energy / cs.de + 0.5);
    if (idx > (int)cs.n - 1) idx = (int)cs.n - 1;
    s.tot = __ldg(&cs.tot[idx]);
    s.ela = __ldg(&cs.ela[idx]);
    s.exc = __ldg(&cs.exc[idx]);
    s.ion = __ldg(&cs.ion[idx]);
  } else {
    double e = fmin(fmax(energy, cs.e_min), cs.e_max);
    double u = (log(e) - cs.log_emin) * cs.inv_dlog;
    int i = (int)u;
    if (i > (int)cs.n - 2) i = (int)cs.n - 2;
    if (i < 0) i = 0;
    double f = u - i;
    if (cs.stab) {  // the same interpolation from the shared-memory copy
      const double4 a = cs.stab[i], b = cs.stab[i + 1];
      s.ela = a.y * (1 - f) + b.y * f;
      s.exc = a.z * (1 - f) + b.z * f;
      s.ion = a.w * (1 - f) + b.w * f;
      s.tot = a.x * (1 - f) + b.x * f;
    } else {
      s.ela = __ldg(&cs.ela[i]) * (1 - f) + __ldg(&cs.ela[i + 1]) * f;
      s.exc = __ldg(&cs.exc[i]) * (1 - f) + __ldg(&cs.exc[i + 1]) * f;
      s.ion = __ldg(&cs.ion[i]) * (1 - f) + __ldg(&cs.ion[i + 1]) * f;
      s.tot = __ldg(&cs.tot[i]) * (1 - f) + __ldg(&cs.tot[i + 1]) * f;
    }
  }
  return s;
}

// The logarithmic table into shared memory (the whole CTA; ends with a
// barrier) when it fits: every lookup of the collision pass then reads
// shared memory instead of L2.
__device__ __forceinline__ void mcc_stage_table(CrossSections& cs, double4* s_tab) {
  if (cs.kind != 1 || cs.n > MCC_SMEM_TABLE) return;
  for (int i = threadIdx.x; i < (int)cs.n; i += blockDim.x)
    s_tab[i] = make_double4(__ldg(&cs.tot[i]), __ldg(&cs.ela[i]), __ldg(&cs.exc[i]), __ldg(&cs.ion[i]));
  __syncthreads();
  cs.stab = s_tab;
}

// Init::SampleVel (src/init.cpp:104-114).
template <class D>
__device__ __forceinline__ double sample_vel(D& src, double mass, double temp) {
  double v_th = sqrt(2 * K_B * temp * (QE / K_B) / mass);
  double u1 = src.next();
  double u2 = src.next();
  double u3 = src.next();
  return v_th * sqrt(2.0) * (u1 + u2 + u3 - 1.5);
}

struct MccParams {
  double vn, dt_phys, ion_mass, ion_temp, F1, F2, p_cut;
  unsigned long long cut53;  // ceil(p_cut * 2^53): u < p_cut  <=>  M < cut53 for u = M * 2^-53
  const unsigned long long* bin_cut;  // per speed bin (CrossSections::bin_cut), or null: cut53 for all
  int null_collision;
};

// Products of one ionisation: the secondary electron and the new ion at the
// primary's position.
struct IonEvent {
  double x, y, z, ev[3], iv[3];  // position (x, y, -) or (cell, ox, oy); velocities
};

// Particle layouts the MCC runs on: FP64 positions and velocities, or the
// mixed form's cell index + FP32 offsets and FP32 velocities.
struct Fp64Particles {
  SoA p;
  // Integer operations on the bits only (FP64 issues slowly on GB300).
  __device__ int speed_bin(long long q) const { return speed_bin_fp64(p.vx[q], p.vy[q], p.vz[q]); }
  __device__ void load_v(long long q, double& a, double& b, double& c) const { a = p.vx[q]; b = p.vy[q]; c = p.vz[q]; }
  __device__ void store_v(long long q, double a, double b, double c) const { p.vx[q] = a; p.vy[q] = b; p.vz[q] = c; }
  __device__ void load_pos(long long q, double& a, double& b, double& c) const { a = p.x[q]; b = p.y[q]; c = 0; }
  __device__ void append(long long o, double a, double b, double, const double* v) const {
    p.x[o] = a; p.y[o] = b; p.vx[o] = v[0]; p.vy[o] = v[1]; p.vz[o] = v[2];
  }
};

struct MixedParticles {
  MixedSoA p;
  __device__ int speed_bin(long long q) const { return speed_bin_fp32(p.vx[q], p.vy[q], p.vz[q]); }
  __device__ void load_v(long long q, double& a, double& b, double& c) const { a = p.vx[q]; b = p.vy[q]; c = p.vz[q]; }
  __device__ void store_v(long long q, double a, double b, double c) const {
    p.vx[q] = (float)a; p.vy[q] = (float)b; p.vz[q] = (float)c;
  }
  __device__ void load_pos(long long q, double& a, double& b, double& c) const {
    a = (double)p.cell[q]; b = p.ox[q]; c = p.oy[q];
  }
  __device__ void append(long long o, double a, double b, double c, const double* v) const {
    p.cell[o] = (int)a; p.ox[o] = (float)b; p.oy[o] = (float)c;
    p.vx[o] = (float)v[0]; p.vy[o] = (float)v[1]; p.vz[o] = (float)v[2];
  }
};

// CollisionHandler::handle_collisions for one electron plus collision_electron
// (src/collision.cpp:60-207), after its first draw u0 passed the early-out
// below; later draws come from `src` in the reference's order.  Returns 0
// (none), 1 elastic, 2 excitation, 3 ionisation (products in evt).
//
// Early-out: p_cut bounds the collision probability of every electron from
// above (1 - exp(-nu_max dt), nu_max >= tot(E)*|v| over the table, plus a
// relative margin of 1e-9 for rounding), so u0 >= p_cut means "no collision"
// in the reference's test p_coll > u0 too, and such electrons are rejected
// before their velocity is read.  With Philox the test is an integer compare
// of the draw's 53-bit mantissa.  In null-collision mode p_cut is the
// null-collision probability itself and a second draw accepts with nu/nu_max.
template <class P, class D>
__device__ int mcc_collide(const CrossSections& cs, const MccParams& m, const P& e, long long q, D& src, double u0,
                           IonEvent& evt) {
  double* pe = evt.ev;
  double* pi = evt.iv;
  double vx, vy, vz;
  e.load_v(q, vx, vy, vz);
  double v_sqr = (vx * vx + vy * vy + vz * vz) * m.vn * m.vn;
  double velocity = sqrt(v_sqr);
  double energy = (0.5 * ME * v_sqr) / EV;
  Sigma s = sigma_at(cs, energy, velocity);
  double nu = s.tot * velocity;
  if (m.null_collision) {
    if (!(src.next() * cs.nu_max < nu)) return 0;
  } else {
    double p_coll = 1 - exp(-nu * m.dt_phys);
    if (!(p_coll > u0)) return 0;
  }
  double gx = vx, gy = vy, gz = vz;
  double g = sqrt(gx * gx + gy * gy + gz * gz);
  double wx = m.F1 * vx, wy = m.F1 * vy, wz = m.F1 * vz;
  // Euler angles theta = atan2(|(gy, gz)|, gx), phi = atan2(gz, gy) enter only
  // through their sines and cosines, which are the direction cosines
  // themselves (equal to the reference's sin/cos of the rounded angles to a
  // few ulps, and far shorter dependent FP64 chains); the reference's special
  // angles (PI_REF halves, gx or gy zero) are kept as written.
  double st, ct, sp, cp;
  if (gx == 0 || gy == 0) {
    double theta, phi;
    if (gx == 0) theta = 0.5 * PI_REF;
    else theta = atan2(sqrt(gy * gy + gz * gz), gx);
    if (gy == 0) phi = gz > 0 ? 0.5 * PI_REF : -0.5 * PI_REF;
    else phi = atan2(gz, gy);
    st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
  } else {
    const double rho = sqrt(gy * gy + gz * gz);
    st = rho / g;
    ct = gx / g;
    sp = gz / rho;
    cp = gy / rho;
  }
  // chi enters through cos(chi) and sin(chi): for chi = acos(c) they are c and
  // sqrt((1 - c)(1 + c)).
  double cchi, schi, eta;
  double t0 = s.ela;
  double t1 = t0 + s.exc;
  double t2 = t1 + s.ion;
  int kind;
  if (src.next() < (t0 / t2)) {
    kind = 1;
    cchi = 1.0 - 2.0 * src.next();
    schi = sqrt((1.0 - cchi) * (1.0 + cchi));
    eta = 2 * PI_REF * src.next();
  } else if (src.next() < (t1 / t2)) {
    kind = 2;
    double en = 0.5 * ME * g * g * m.vn * m.vn;
    en = fabs(en - E_EXC_TH * EV);
    g = sqrt(2.0 * en / ME);
    g = g / m.vn;
    cchi = 1.0 - 2.0 * src.next();
    schi = sqrt((1.0 - cchi) * (1.0 + cchi));
    eta = 2 * PI_REF * src.next();
  } else {
    kind = 3;
    double en = 0.5 * ME * g * g * m.vn * m.vn;
    en = fabs(en - E_ION_TH * EV);
    double e_ej = 10.0 * tan(src.next() * atan(en / EV / 20.0)) * EV;
    double e_sc = fabs(en - e_ej);
    g = sqrt(2.0 * e_sc / ME);
    double g2 = sqrt(2.0 * e_ej / ME);
    g = g / m.vn;
    g2 = g2 / m.vn;
    // chi = acos(sqrt(e_sc/en)), chi2 = acos(sqrt(e_ej/en)) with e_sc + e_ej = en
    // (e_ej <= en/2): sin(chi) = cos(chi2) = sqrt(e_ej/en) and the reverse.
    cchi = sqrt(e_sc / en);
    schi = sqrt(e_ej / en);
    eta = 2 * PI_REF * src.next();
    double eta2 = eta + PI_REF;
    double sc = cchi, cc = schi, se = sin(eta2), ce = cos(eta2);
    double hx = g2 * (ct * cc - st * sc * ce);
    double hy = g2 * (st * cp * cc + ct * cp * sc * ce - sp * sc * se);
    double hz = g2 * (st * sp * cc + ct * sp * sc * ce + cp * sc * se);
    pe[0] = (wx + m.F2 * hx);
    pe[1] = (wy + m.F2 * hy);
    pe[2] = (wz + m.F2 * hz);
    // The reference builds Particle(x, y, SampleVel, SampleVel, SampleVel)
    // and GCC evaluates those arguments right to left: vz draws first.  The
    // ion keeps its velocity in m/s (not divided by vel_norm), as there.
    pi[2] = sample_vel(src, m.ion_mass, m.ion_temp);
    pi[1] = sample_vel(src, m.ion_mass, m.ion_temp);
    pi[0] = sample_vel(src, m.ion_mass, m.ion_temp);
    e.load_pos(q, evt.x, evt.y, evt.z);
  }
  double sc = schi, cc = cchi, se = sin(eta), ce = cos(eta);
  gx = g * (ct * cc - st * sc * ce);
  gy = g * (st * cp * cc + ct * cp * sc * ce - sp * sc * se);
  gz = g * (st * sp * cc + ct * sp * sc * ce + cp * sc * se);
  e.store_v(q, wx + m.F2 * gx, wy + m.F2 * gy, wz + m.F2 * gz);
  return kind;
}

// Pass 1a: every electron draws u0 (no ordering, fixed grid); the few below
// the cut of their speed bin are appended, in any order, to a candidate list.
// Compacting them first keeps whole warps on the FP64 collision path instead
// of one lane in 32 (divergent FP64 work costs full warp throughput).  A bin's
// cut bounds the collision probability of every speed in it and its two
// neighbours from above (mcc_bin_cuts), so an electron it rejects fails the
// reference's test p_coll > u0 as well.  One atomic per block and round
// reserves the block's candidates.
template <int MODE, class P>
__global__ void __launch_bounds__(PART_THREADS) k_mcc_select(MccParams m, P e, const long long* __restrict__ d_ne,
                                                             const double* __restrict__ uniforms, int ustride,
                                                             uint64_t seed, const unsigned long long* __restrict__ d_step,
                                                             McEvents ev) {
  __shared__ unsigned int s_cnt[PART_THREADS / 32];
  __shared__ unsigned int s_base;
  const long long ne = *d_ne;
  const unsigned long long step = *d_step;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long nround = (ne + stride - 1) / stride;
  for (long long rd = 0; rd < nround; rd++) {
    const long long q = rd * stride + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool cand = false;
    if (q < ne) {
      const unsigned long long cut = m.bin_cut ? __ldg(&m.bin_cut[e.speed_bin(q)]) : m.cut53;
      if (MODE == EPIC_MCC_INJECTED) {
        cand = __ldg(&uniforms[q * ustride]) * 9007199254740992.0 < (double)cut;
      } else {
        Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)seed, (uint32_t)(seed >> 32), 0,
                   make_uint4(0, 0, 0, 0)};
        cand = src.next53() < cut;
      }
    }
    const unsigned int mask = __ballot_sync(0xffffffffu, cand);
    if (lane == 0) s_cnt[wid] = (unsigned int)__popc(mask);
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned int tot = 0;
#pragma unroll
      for (int w = 0; w < PART_THREADS / 32; w++) {
        const unsigned int c = s_cnt[w];
        s_cnt[w] = tot;
        tot += c;
      }
      s_base = tot ? atomicAdd(ev.cand_count, tot) : 0u;
    }
    __syncthreads();
    if (cand) ev.cand[s_base + s_cnt[wid] + __popc(mask & ((1u << lane) - 1))] = (unsigned int)q;
    __syncthreads();
  }
}

// Pass 1b: the candidates, whole warps at a time.  Each redraws u0 from the
// same stream position and runs the collision; an ionisation stores its
// products in the event buffer and marks the electron (slot) and its tile of
// MCC_TILE electrons (tile_cnt).
template <int MODE, class P>
__global__ void __launch_bounds__(PART_THREADS) k_mcc_collide(CrossSections cs, MccParams m, P e,
                                                              const double* __restrict__ uniforms, int ustride,
                                                              uint64_t seed,
                                                              const unsigned long long* __restrict__ d_step,
                                                              McEvents ev, unsigned long long* pending, int* flags) {
  extern __shared__ double4 s_tab[];
  __shared__ unsigned long long s_coll;
  const unsigned int nc = *ev.cand_count;
  if ((unsigned long long)blockIdx.x * blockDim.x >= nc) return;  // no candidates for this CTA
  if (threadIdx.x == 0) s_coll = 0;
  mcc_stage_table(cs, s_tab);
  __syncthreads();
  const unsigned long long step = *d_step;
  unsigned int ncoll = 0;
  for (unsigned int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const long long q = ev.cand[c];
    IonEvent evt;
    int kind;
    if (MODE == EPIC_MCC_INJECTED) {
      Injected src{uniforms + q * ustride};
      double u0 = src.next();
      kind = mcc_collide(cs, m, e, q, src, u0, evt);
    } else {
      Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)seed, (uint32_t)(seed >> 32), 0,
                 make_uint4(0, 0, 0, 0)};
      unsigned long long M = src.next53();
      kind = mcc_collide(cs, m, e, q, src, (double)M * (1.0 / 9007199254740992.0), evt);
    }
    ncoll += kind != 0;
    if (kind == 3) {
      unsigned int slot = atomicAdd(ev.count, 1u);
      if (slot < ev.cap) {
        ev.buf[slot] = evt;
        ev.slot[q] = (int)slot;
        atomicAdd(&ev.tile_cnt[q / MCC_TILE], 1u);
      } else {
        set_flag(flags, FLAG_CAPACITY);
      }
    }
  }
  if (ncoll) atomicAdd(&s_coll, (unsigned long long)ncoll);
  __syncthreads();
  if (threadIdx.x == 0 && s_coll) atomicAdd(&pending[1], s_coll);
}

// Pass 2 (one block): exclusive scan of the per-tile event counts, 4,096
// tiles (four per thread) per round.
__global__ void __launch_bounds__(1024) k_mcc_scan(const long long* __restrict__ d_ne, McEvents ev,
                                                   unsigned long long* pending) {
  __shared__ unsigned int warp_tot[32];
  __shared__ unsigned int carry;
  const long long ne = *d_ne;
  const int tiles = (int)((ne + MCC_TILE - 1) / MCC_TILE);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < tiles; base += 4 * blockDim.x) {
    const int t0 = base + 4 * threadIdx.x;
    unsigned int v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k] = t0 + k < tiles ? ev.tile_cnt[t0 + k] : 0u;
      s += v[k];
    }
    unsigned int x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      unsigned int y = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned int z = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) y += z;
      }
      warp_tot[lane] = y;
    }
    __syncthreads();
    const unsigned int c0 = carry;
    unsigned int run = c0 + (w ? warp_tot[w - 1] : 0u) + x - s;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (t0 + k < tiles) ev.tile_off[t0 + k] = run;
      run += v[k];
    }
    __syncthreads();  // every thread has read carry and warp_tot
    if (threadIdx.x == blockDim.x - 1) carry = run;
    __syncthreads();
  }
  if (threadIdx.x == 0) pending[0] = carry;
}

// Pass 3: tiles that had events append their products in electron order at
// [n_e + tile offset + rank] / [n_i + ...] (the reference appends in loop
// order, src/collision.cpp:163-164), then clear their marks.
template <class P>
__global__ void __launch_bounds__(PART_THREADS) k_mcc_append(P e, const long long* __restrict__ d_ne,
                                                             long long e_cap, P ion,
                                                             const long long* __restrict__ d_ni, long long i_cap,
                                                             McEvents ev, int* flags) {
  constexpr int ITEMS = MCC_TILE / PART_THREADS;
  __shared__ int sm[40];
  __shared__ int s_list[PART_THREADS];
  __shared__ int s_nlist;
  const long long ne = *d_ne, ni = *d_ni;
  const int tiles = (int)((ne + MCC_TILE - 1) / MCC_TILE);
  // Each CTA takes PART_THREADS consecutive tiles at a time, finds those
  // with events in one pass (a load per thread) and appends them in turn.
  for (int t0 = blockIdx.x * PART_THREADS; t0 < tiles; t0 += gridDim.x * PART_THREADS) {
    if (threadIdx.x == 0) s_nlist = 0;
    __syncthreads();
    const int tt = t0 + threadIdx.x;
    if (tt < tiles && ev.tile_cnt[tt] != 0) s_list[atomicAdd(&s_nlist, 1)] = tt;
    __syncthreads();
    const int nlist = s_nlist;
    for (int li = 0; li < nlist; li++) {
    const int t = s_list[li];
    const long long base = (long long)t * MCC_TILE;
    int slot[ITEMS], flag[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      const long long q = base + k * PART_THREADS + threadIdx.x;
      slot[k] = q < ne ? ev.slot[q] : -1;
      flag[k] = slot[k] >= 0;
    }
    int run = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      int row_total;
      const int rank = run + block_exclusive_scan(flag[k], &row_total, sm);
      run += row_total;
      if (flag[k]) {
        const IonEvent v = ev.buf[slot[k]];
        const long long oe = ne + ev.tile_off[t] + rank, oi = ni + ev.tile_off[t] + rank;
        if (oe < e_cap && oi < i_cap) {
          e.append(oe, v.x, v.y, v.z, v.ev);
          ion.append(oi, v.x, v.y, v.z, v.iv);
        } else {
          set_flag(flags, FLAG_CAPACITY);
        }
        ev.slot[base + k * PART_THREADS + threadIdx.x] = -1;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) ev.tile_cnt[t] = 0;
    }
    __syncthreads();  // s_list and s_nlist are rewritten for the next tiles
  }
}

__global__ void k_mcc_commit(long long* d_ne, long long e_cap, long long* d_ni, long long i_cap,
                             unsigned long long* pending, unsigned long long* ncoll_out,
                             unsigned long long* d_step, McEvents ev, int* flags) {
  long long add = (long long)pending[0];
  long long ne = *d_ne + add, ni = *d_ni + add;
  if (ne > e_cap || ni > i_cap) {
    set_flag(flags, FLAG_CAPACITY);
    ne = ne > e_cap ? e_cap : ne;
    ni = ni > i_cap ? i_cap : ni;
  }
  *d_ne = ne;
  *d_ni = ni;
  *ncoll_out = pending[1];
  pending[0] = 0;
  pending[1] = 0;
  *ev.count = 0;
  *ev.cand_count = 0;
  *d_step += 1;
}

size_t ion_event_bytes() { return sizeof(IonEvent); }

// Bin b of the early-out holds the m = max |v_i| of speed_bin_of, so |v|^2
// (vel_norm units) lies in [m_lo^2, 3 m_hi^2] up to the rounding of the
// collision test's own sum (relative 1e-12 of margin).  Its cut bounds
// 1 - exp(-nu dt) there: the largest table entry the lookup of sigma_at can
// reach (one index of margin each side) times the largest speed, with a
// relative margin of 1e-9 and an absolute one of 1e-15 (1 - exp(-x) carries an
// absolute rounding error of about 1e-16).
void mcc_bin_cuts(const CrossSections& cs, const double* tot, double vn, double dt_phys, unsigned long long* out) {
  const double two53 = 9007199254740992.0;
  const long long n = (long long)cs.n;
  for (int b = 0; b < MCC_SPEED_BINS; b++) {
    const int e = MCC_BIN_EMIN + (b - 1) / 4, q = (b - 1) % 4;
    if (b == MCC_SPEED_BINS - 1 || (b > 0 && e > MCC_BIN_EMAX)) {
      out[b] = (unsigned long long)two53;
      continue;
    }
    const double m_lo = b == 0 ? 0.0 : std::ldexp(1.0 + q / 4.0, e);
    const double m_hi = b == 0 ? std::ldexp(1.0, MCC_BIN_EMIN) : std::ldexp(1.0 + (q + 1) / 4.0, e);
    const double s_lo = m_lo * m_lo * (1 - 1e-12), s_hi = 3 * m_hi * m_hi * (1 + 1e-12);
    const double e_lo = 0.5 * ME * (s_lo * vn * vn) / EV * (1 - 1e-12);
    const double e_hi = 0.5 * ME * (s_hi * vn * vn) / EV * (1 + 1e-12);
    double tmax = 0;
    if (cs.kind == 0) {
      const double x0 = e_lo / cs.de + 0.5, x1 = e_hi / cs.de + 0.5;
      long long i0 = x0 >= (double)n ? n - 1 : (long long)floor(x0) - 1;
      long long i1 = x1 >= (double)n ? n - 1 : (long long)floor(x1) + 1;
      i0 = std::max(0LL, std::min(i0, n - 1));
      i1 = std::max(0LL, std::min(i1, n - 1));
      for (long long i = i0; i <= i1; i++) tmax = std::max(tmax, tot[i]);
    } else {
      auto pos = [&](double e) { return (log(fmin(fmax(e, cs.e_min), cs.e_max)) - cs.log_emin) * cs.inv_dlog; };
      long long i0 = (long long)floor(pos(e_lo)) - 1, i1 = (long long)floor(pos(e_hi)) + 1;
      i0 = std::max(0LL, std::min(i0, n - 2));
      i1 = std::max(0LL, std::min(i1, n - 2));
      for (long long i = i0; i <= i1; i++) tmax = std::max(tmax, std::max(tot[i], tot[i + 1]));
    }
    const double v_hi = sqrt(s_hi * vn * vn) * (1 + 1e-12);
    const double p = 1 - exp(-(tmax * v_hi) * dt_phys);
    const double pc = fmin(1.0, p * (1 + 1e-9) + 1e-15);
    out[b] = (unsigned long long)ceil(pc * two53);
  }
}

template <class P>
static void launch_mcc_t(cudaStream_t st, int mode, const CrossSections& cs, const P& e, long long* d_ne,
                         long long e_cap, const P& ion, long long* d_ni, long long i_cap, const MccParams& m,
                         const double* uniforms, int ustride, uint64_t seed, unsigned long long* d_step,
                         const McEvents& ev, unsigned long long* d_ncoll, int* flags, int grid, int skip_select) {
  unsigned long long* pending = d_ncoll + 1;
  if (skip_select) {  // the push selected the candidates (mcc_candidate)
    k_mcc_collide<EPIC_MCC_PHILOX, P><<<grid, PART_THREADS, mcc_table_smem(cs), st>>>(cs, m, e, uniforms, ustride, seed, d_step, ev,
                                                                      pending, flags);
  } else if (mode == EPIC_MCC_INJECTED) {
    k_mcc_select<EPIC_MCC_INJECTED, P><<<grid, PART_THREADS, 0, st>>>(m, e, d_ne, uniforms, ustride, seed, d_step, ev);
    k_mcc_collide<EPIC_MCC_INJECTED, P><<<grid, PART_THREADS, mcc_table_smem(cs), st>>>(cs, m, e, uniforms, ustride, seed, d_step, ev,
                                                                        pending, flags);
  } else {
    k_mcc_select<EPIC_MCC_PHILOX, P><<<grid, PART_THREADS, 0, st>>>(m, e, d_ne, uniforms, ustride, seed, d_step, ev);
    k_mcc_collide<EPIC_MCC_PHILOX, P><<<grid, PART_THREADS, mcc_table_smem(cs), st>>>(cs, m, e, uniforms, ustride, seed, d_step, ev,
                                                                      pending, flags);
  }
  k_mcc_scan<<<1, 1024, 0, st>>>(d_ne, ev, pending);
  k_mcc_append<P><<<grid, PART_THREADS, 0, st>>>(e, d_ne, e_cap, ion, d_ni, i_cap, ev, flags);
  k_mcc_commit<<<1, 1, 0, st>>>(d_ne, e_cap, d_ni, i_cap, pending, d_ncoll, d_step, ev, flags);
}

void mcc_select_cut(const CrossSections& cs, int mode, double dt_phys, unsigned long long* cut53,
                    const unsigned long long** bin_cut) {
  const double p_null = 1 - exp(-cs.nu_max * dt_phys);
  const bool null_collision = mode == EPIC_MCC_NULL;
  const double p_cut = null_collision ? p_null : fmin(1.0, p_null * (1 + 1e-9) + 1e-300);
  *cut53 = (unsigned long long)ceil(p_cut * 9007199254740992.0);
  *bin_cut = null_collision ? nullptr : cs.bin_cut;
}

void launch_mcc(cudaStream_t st, int mode, const CrossSections& cs, const ParticleRef& e, long long* d_ne,
                long long e_cap, const ParticleRef& ion, long long* d_ni, long long i_cap, double vel_norm,
                double dt_phys, double ion_mass, double ion_temp, const double* uniforms, int ustride, uint64_t seed,
                unsigned long long* d_step, const McEvents& ev, unsigned long long* d_ncoll, int* flags, int grid,
                int skip_select) {
  MccParams m;
  m.vn = vel_norm;
  m.dt_phys = dt_phys;
  m.ion_mass = ion_mass;
  m.ion_temp = ion_temp;
  m.F1 = ME / (ME + ion_mass);
  m.F2 = ion_mass / (ME + ion_mass);
  m.null_collision = mode == EPIC_MCC_NULL;
  const double p_null = 1 - exp(-cs.nu_max * dt_phys);
  m.p_cut = m.null_collision ? p_null : fmin(1.0, p_null * (1 + 1e-9) + 1e-300);
  mcc_select_cut(cs, mode, dt_phys, &m.cut53, &m.bin_cut);
  if (e.mixed)
    launch_mcc_t(st, mode, cs, MixedParticles{e.m}, d_ne, e_cap, MixedParticles{ion.m}, d_ni, i_cap, m, uniforms,
                 ustride, seed, d_step, ev, d_ncoll, flags, grid, skip_select);
  else
    launch_mcc_t(st, mode, cs, Fp64Particles{e.f}, d_ne, e_cap, Fp64Particles{ion.f}, d_ni, i_cap, m, uniforms,
                 ustride, seed, d_step, ev, d_ncoll, flags, grid, skip_select);
}


// ------------------------------------------------------------ batches ---
// The select and collide passes for a batch (include/epic2d_batch.h): every
// electron finds its run from its cell and uses that run's parameters and
// seed; the scan, ordered append and commit passes above serve the batch's
// particle arrays unchanged (products carry the primary's cell, so they
// belong to its run).
__device__ __forceinline__ MccParams batch_mcc_params(const BRun& r) {
  MccParams m;
  m.vn = r.vn;
  m.dt_phys = r.dt_phys;
  m.ion_mass = r.ion_mass;
  m.ion_temp = r.ion_temp;
  m.F1 = r.F1;
  m.F2 = r.F2;
  m.p_cut = r.p_cut;
  m.cut53 = r.cut53;
  m.bin_cut = nullptr;
  m.null_collision = 0;
  return m;
}

__global__ void __launch_bounds__(PART_THREADS) k_batch_mcc_select(const BRun* __restrict__ runs,
                                                                   const int* __restrict__ node_run, MixedSoA e,
                                                                   const long long* __restrict__ d_ne,
                                                                   const unsigned long long* __restrict__ d_step,
                                                                   McEvents ev) {
  const long long ne = *d_ne;
  const unsigned long long step = *d_step;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const long long nround = (ne + stride - 1) / stride;
  for (long long rd = 0; rd < nround; rd++) {
    const long long q = rd * stride + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool cand = false;
    if (q < ne) {
      const BRun& r = runs[node_run[e.cell[q]]];
      if (r.mcc) {
        Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)r.seed, (uint32_t)(r.seed >> 32), 0,
                   make_uint4(0, 0, 0, 0)};
        cand = src.next53() < r.cut53;
      }
    }
    const unsigned int mask = __ballot_sync(0xffffffffu, cand);
    if (mask) {
      unsigned int base = 0;
      if (lane == __ffs(mask) - 1) base = atomicAdd(ev.cand_count, (unsigned int)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
      if (cand) ev.cand[base + __popc(mask & ((1u << lane) - 1))] = (unsigned int)q;
    }
  }
}

__global__ void __launch_bounds__(PART_THREADS) k_batch_mcc_collide(CrossSections cs, const BRun* __restrict__ runs,
                                                                    const int* __restrict__ node_run,
                                                                    MixedParticles e,
                                                                    const unsigned long long* __restrict__ d_step,
                                                                    McEvents ev, unsigned long long* pending,
                                                                    int* flags) {
  extern __shared__ double4 s_tab[];
  __shared__ unsigned long long s_coll;
  const unsigned int nc = *ev.cand_count;
  if ((unsigned long long)blockIdx.x * blockDim.x >= nc) return;  // no candidates for this CTA
  if (threadIdx.x == 0) s_coll = 0;
  mcc_stage_table(cs, s_tab);
  __syncthreads();
  const unsigned long long step = *d_step;
  unsigned int ncoll = 0;
  for (unsigned int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const long long q = ev.cand[c];
    const BRun& r = runs[node_run[e.p.cell[q]]];
    const MccParams m = batch_mcc_params(r);
    IonEvent evt;
    Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)r.seed, (uint32_t)(r.seed >> 32), 0,
               make_uint4(0, 0, 0, 0)};
    const unsigned long long M = src.next53();
    const int kind = mcc_collide(cs, m, e, q, src, (double)M * (1.0 / 9007199254740992.0), evt);
    ncoll += kind != 0;
    if (kind == 3) {
      unsigned int slot = atomicAdd(ev.count, 1u);
      if (slot < ev.cap) {
        ev.buf[slot] = evt;
        ev.slot[q] = (int)slot;
        atomicAdd(&ev.tile_cnt[q / MCC_TILE], 1u);
      } else {
        set_flag(flags, FLAG_CAPACITY);
      }
    }
  }
  if (ncoll) atomicAdd(&s_coll, (unsigned long long)ncoll);
  __syncthreads();
  if (threadIdx.x == 0 && s_coll) atomicAdd(&pending[1], s_coll);
}

void launch_batch_mcc(cudaStream_t st, const CrossSections& cs, const BRun* runs, const int* node_run,
                      const MixedSoA& e, long long* d_ne, long long e_cap, const MixedSoA& ion, long long* d_ni,
                      long long i_cap, unsigned long long* d_step, const McEvents& ev, unsigned long long* d_ncoll,
                      int* flags, int grid, int skip_select) {
  unsigned long long* pending = d_ncoll + 1;
  if (!skip_select)  // else the electrons' push selected the candidates (k_batch_push_dep)
    k_batch_mcc_select<<<grid, PART_THREADS, 0, st>>>(runs, node_run, e, d_ne, d_step, ev);
  k_batch_mcc_collide<<<grid, PART_THREADS, mcc_table_smem(cs), st>>>(cs, runs, node_run, MixedParticles{e}, d_step, ev, pending, flags);
  k_mcc_scan<<<1, 1024, 0, st>>>(d_ne, ev, pending);
  k_mcc_append<MixedParticles><<<grid, PART_THREADS, 0, st>>>(MixedParticles{e}, d_ne, e_cap, MixedParticles{ion}, d_ni,
                                                              i_cap, ev, flags);
  k_mcc_commit<<<1, 1, 0, st>>>(d_ne, e_cap, d_ni, i_cap, pending, d_ncoll, d_step, ev, flags);
}

}  // namespace epic
