// Device pieces of the mixed-precision Poisson solve shared by the single-run
// kernels (epic_spectral.cu) and the batched ones (epic_batch.cu), which must
// give bit-identical potentials; both files are compiled with the same flags.
//
// The residual of a lattice is reduced in fixed chunks of SPEC_CHUNK entries
// (one CTA each, fixed in-CTA order) and the chunk sums are added exactly
// (fixed point, rounded once), so the stopping norm depends only on the
// lattice, not on how the launch is shaped or who adds the chunk sums.  The GEMM tiles accumulate every output over k = 0..K-1
// in order with one fma per step, so the tile shape does not change results
// either (zero padding adds exact zeros).
#pragma once

#include "epic_internal.cuh"
#include "epic_xsum.cuh"

namespace epic {

// Exact sum of v[0..n) rounded once (epic_xsum.cuh), by one thread: the
// batched solve's per-run test.
__device__ __forceinline__ double spec_exact_sum_serial(const double* v, int n) {
  int A = 0;
  for (int b = 0; b < n; b++) A = max(A, xs_exponent(__ldcg(&v[b])));
  xs_int acc = 0;
  for (int b = 0; b < n; b++) acc += xs_from_double(__ldcg(&v[b]), A);
  return xs_to_double(acc, A);
}

// The same sum by a whole CTA of 256 threads (the same value: exact, then
// rounded once), in every thread; s_e and s_v: shared scratch of 8 entries.
__device__ __forceinline__ double spec_exact_sum_cta(const double* v, int n, int* s_e, unsigned long long (*s_v)[2],
                                                     double* s_out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int e = 0;
  for (int b = threadIdx.x; b < n; b += 256) e = max(e, xs_exponent(__ldcg(&v[b])));
  e = (int)__reduce_max_sync(0xffffffffu, (unsigned)e);
  if (lane == 0) s_e[wid] = e;
  __syncthreads();
  int A = 0;
  for (int w = 0; w < 8; w++) A = max(A, s_e[w]);
  xs_int acc = 0;
  for (int b = threadIdx.x; b < n; b += 256) acc += xs_from_double(__ldcg(&v[b]), A);
  acc = xs_warp_sum(acc);
  if (lane == 0) {
    s_v[wid][0] = (unsigned long long)(xs_uint)acc;
    s_v[wid][1] = (unsigned long long)((xs_uint)acc >> 64);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    xs_uint tot = 0;
    for (int w = 0; w < 8; w++) tot += ((xs_uint)s_v[w][1] << 64) | s_v[w][0];
    *s_out = xs_to_double((xs_int)tot, A);
  }
  __syncthreads();
  const double r = *s_out;
  __syncthreads();
  return r;
}

constexpr int SPEC_CHUNK = 1024;  // lattice entries per residual CTA (256 threads x 4)

// One solve's lattice and where its nodes live: node (i, j) of the run's
// nx x ny grid is at (I_off + i) * NY + j of the node arrays (I_off = 0,
// NY = ny for a single run).
struct SpecLattice {
  int nx, ny, I_off, NY;
  int R, C, flat, gs_norm;
  // EPIC_POISSON_* : with an extension the unknowns are rows i = r + i0
  // (i0 = 1 for DIRICHLET_X, 0 for PERIODIC) of columns j = c, neighbours
  // wrapped where periodic, and PERIODIC subtracts *bmean from b.
  int mode;
  const double* bmean;
  double dx2, K, tol;
  const double* rho;
  double* phi;
  float* t0;          // R * C residual, transform layout
  double* partials;   // per chunk
  int* state;         // [0] done, [1] stage
  SolveInfo* info;    // may be null
  unsigned long long* iter_total;  // may be null
};

__device__ __forceinline__ int spec_node(const SpecLattice& L, int i, int j) { return (L.I_off + i) * L.NY + j; }

__device__ __forceinline__ double spec_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Zero phi on the run's nodes (cold start, as both reference solvers).
__device__ __forceinline__ void spec_init_node(const SpecLattice& L, int q) {
  const int i = q / L.ny, j = q - i * L.ny;
  L.phi[spec_node(L, i, j)] = 0;
}

// r = b - A x for the entries of one chunk (FP64) into t0 (FP32); the chunk's
// sum of r^2 goes to partials[chunk].  Called by a whole CTA of 256 threads.
// x and the products' operands are read through L2 (__ldcg): inside the
// cooperative solve other CTAs wrote them since this SM last read them, and
// its L1 is not coherent.
__device__ __forceinline__ void spec_residual_chunk(const SpecLattice& L, int chunk, double* sm8) {
  const int total = L.R * L.C;
  const int nx = L.nx, ny = L.ny, R = L.R, C = L.C;
  double acc = 0;
#pragma unroll
  for (int u = 0; u < SPEC_CHUNK / 256; u++) {
    const int q = chunk * SPEC_CHUNK + u * 256 + threadIdx.x;
    if (q < total) {
      const int ri = q / C, cj = q - ri * C;
      const double* x = L.phi;
      int i, j;
      double ax;
      if (L.mode != EPIC_POISSON_DIRICHLET) {  // extension lattice: rows i = ri + i0, wrapped neighbours
        const int i0 = L.mode == EPIC_POISSON_PERIODIC ? 0 : 1;
        i = ri + i0;
        j = cj;
        const int ru = lattice_wrap(ri - 1, R, L.mode == EPIC_POISSON_PERIODIC);
        const int rd = lattice_wrap(ri + 1, R, L.mode == EPIC_POISSON_PERIODIC);
        ax = -4 * __ldcg(&x[spec_node(L, i, j)]);
        if (ru >= 0) ax += __ldcg(&x[spec_node(L, ru + i0, j)]);
        if (rd >= 0) ax += __ldcg(&x[spec_node(L, rd + i0, j)]);
        ax += __ldcg(&x[spec_node(L, i, cj > 0 ? cj - 1 : C - 1)]);
        ax += __ldcg(&x[spec_node(L, i, cj < C - 1 ? cj + 1 : 0)]);
      } else if (L.flat) {  // pcgsolver: rows of C = nx nodes of the flattened vector
        auto nd = [&](int k) { const int ii = k / ny; return spec_node(L, ii, k - ii * ny); };
        i = q / ny;
        j = q - i * ny;
        ax = -4 * __ldcg(&x[spec_node(L, i, j)]);
        if (ri > 0) ax += __ldcg(&x[nd(q - C)]);
        if (ri < R - 1) ax += __ldcg(&x[nd(q + C)]);
        if (cj > 0) ax += __ldcg(&x[nd(q - 1)]);
        if (cj < C - 1) ax += __ldcg(&x[nd(q + 1)]);
      } else {  // gssolver: interior nodes, physical neighbours
        i = ri + 1;
        j = cj + 1;
        ax = -4 * __ldcg(&x[spec_node(L, i, j)]);
        if (i > 0) ax += __ldcg(&x[spec_node(L, i - 1, j)]);
        if (i < nx - 1) ax += __ldcg(&x[spec_node(L, i + 1, j)]);
        if (j > 0) ax += __ldcg(&x[spec_node(L, i, j - 1)]);
        if (j < ny - 1) ax += __ldcg(&x[spec_node(L, i, j + 1)]);
      }
      const bool edge = L.mode == EPIC_POISSON_DIRICHLET && (i == 0 || i == nx - 1 || j == 0 || j == ny - 1);
      double b = edge ? 0.0 : -L.rho[spec_node(L, i, j)] * L.dx2 * L.K;
      if (L.mode == EPIC_POISSON_PERIODIC) b = b - *L.bmean;
      const double r = b - ax;
      L.t0[q] = (float)r;
      acc += r * r;
    }
  }
  acc = spec_warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sm8[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < 8; w++) t += sm8[w];
    L.partials[chunk] = t;
  }
}

// The reference solver's stopping test on the residual just computed (one
// thread): pcgsolver |r|_2 < tol, gssolver sqrt(sum R^2/(nx ny)) < tol with
// R = r/dx^2.  final_pass closes an unconverged solve at the stage cap.
// The stopping norm and the reported error from the sum of r^2.
__device__ __forceinline__ void spec_norm(const SpecLattice& L, double s, double& norm, double& err) {
  const double nn = (double)L.nx * L.ny;
  if (L.gs_norm) {
    norm = sqrt(s / (L.dx2 * L.dx2) / nn);
    err = norm;
  } else {
    norm = sqrt(s);
    err = sqrt(s) / nn;
  }
}

// Records the test's outcome (done: converged; final_pass: the stage cap).
__device__ __forceinline__ void spec_record(const SpecLattice& L, int done, int final_pass, double err) {
  if (L.info) {
    L.info->iterations = L.state[1];
    L.info->error = err;
    L.info->converged = done;
  }
  if (done || final_pass) {
    L.state[0] = 1;
    if (L.iter_total) atomicAdd(L.iter_total, (unsigned long long)L.state[1]);
  } else {
    L.state[1] += 1;
  }
}

__device__ __forceinline__ void spec_check(const SpecLattice& L, int final_pass) {
  if (L.state[0]) return;
  const int nchunks = (L.R * L.C + SPEC_CHUNK - 1) / SPEC_CHUNK;
  const double s = spec_exact_sum_serial(L.partials, nchunks);
  double norm, err;
  spec_norm(L, s, norm, err);
  spec_record(L, norm < L.tol, final_pass, err);
}

// The output element (r, c) of the last product goes to phi at its node.
__device__ __forceinline__ void spec_add_phi(const SpecLattice* L, int N, int r, int c, float v) {
  int i, j;
  if (L->mode != EPIC_POISSON_DIRICHLET) {
    i = r + (L->mode == EPIC_POISSON_PERIODIC ? 0 : 1);
    j = c;
  } else if (L->flat) {
    const int k = r * N + c;  // N = C: the flattened vector
    i = k / L->ny;
    j = k - i * L->ny;
  } else {
    i = r + 1;
    j = c + 1;
  }
  double* const ph = &L->phi[spec_node(*L, i, j)];
  *ph = __ldcg(ph) + (double)v;
}

// One TILE x TILE output tile of C = A B (M x K by K x N, row-major FP32) at
// tile (tr, tc), 256 threads.  EPI 0: store; 1: store C o D; 2: add to phi
// (FP64) at the node of lattice entry (r, c).
template <int EPI, int TILE>
__device__ __forceinline__ void spec_gemm_tile(int M, int N, int K, const float* __restrict__ A,
                                               const float* __restrict__ B, float* __restrict__ Cm,
                                               const float* __restrict__ D, const SpecLattice* L, int tr, int tc,
                                               float (*As)[33], float (*Bs)[33]) {
  constexpr int PT = TILE / 16;  // outputs per thread per direction (2 for 32, 1 for 16)
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row0 = tr * TILE, col0 = tc * TILE;
  float acc[PT][PT];
#pragma unroll
  for (int a = 0; a < PT; a++)
#pragma unroll
    for (int b = 0; b < PT; b++) acc[a][b] = 0.f;
  for (int k0 = 0; k0 < K; k0 += TILE) {
    for (int e = threadIdx.x; e < TILE * TILE; e += 256) {
      const int r = e / TILE, c = e % TILE;
      As[r][c] = (row0 + r < M && k0 + c < K) ? __ldcg(&A[(row0 + r) * K + k0 + c]) : 0.f;
      Bs[r][c] = (k0 + r < K && col0 + c < N) ? __ldcg(&B[(k0 + r) * N + col0 + c]) : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < TILE; kk++) {
#pragma unroll
      for (int a = 0; a < PT; a++)
#pragma unroll
        for (int b = 0; b < PT; b++) acc[a][b] = fmaf(As[PT * ty + a][kk], Bs[kk][PT * tx + b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < PT; a++)
#pragma unroll
    for (int b = 0; b < PT; b++) {
      const int r = row0 + PT * ty + a, c = col0 + PT * tx + b;
      if (r >= M || c >= N) continue;
      if (EPI == 0) Cm[r * N + c] = acc[a][b];
      else if (EPI == 1) Cm[r * N + c] = acc[a][b] * D[r * N + c];
      else spec_add_phi(L, N, r, c, acc[a][b]);
    }
}

// A 64 x 64 output tile of C = A B for large lattices, 256 threads with 4 x 4
// outputs each (register blocking: two 16-byte shared loads feed 16 fmas),
// k in steps of 16 with the next step's operands loaded into registers while
// the current one is multiplied (double-buffered shared memory, one barrier
// per step).  Every output accumulates over k = 0, 1, ... in order with one
// fma per step, as spec_gemm_tile: the same results.
constexpr int SG_BM = 64, SG_BK = 16, SG_LDA = SG_BM + 4;
struct SpecGemmSmem {
  float A[2][SG_BK][SG_LDA];  // k-major (transposed) A tile
  float B[2][SG_BK][SG_BM];
};

template <int EPI>
__device__ __forceinline__ void spec_gemm_tile64(int M, int N, int K, const float* __restrict__ A,
                                                 const float* __restrict__ B, float* __restrict__ Cm,
                                                 const float* __restrict__ D, const SpecLattice* L, int tr, int tc,
                                                 SpecGemmSmem& sm) {
  const int t = threadIdx.x;
  const int tx = t & 15, ty = t >> 4;
  const int row0 = tr * SG_BM, col0 = tc * SG_BM;
  // loader coordinates: A row t/4, k quad (t%4)*4; B k row t/16, column quad (t%16)*4
  const int la_r = t >> 2, la_k = (t & 3) * 4, lb_k = t >> 4, lb_c = (t & 15) * 4;
  const bool vec = (K & 3) == 0 && (N & 3) == 0;
  float ra[4], rb[4];
  auto load = [&](int k0) {
    const int ar = row0 + la_r, ak = k0 + la_k, bk = k0 + lb_k, bc = col0 + lb_c;
    if (vec && ar < M && ak + 3 < K) {
      const float4 v = __ldcg(reinterpret_cast<const float4*>(A + (size_t)ar * K + ak));
      ra[0] = v.x; ra[1] = v.y; ra[2] = v.z; ra[3] = v.w;
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) ra[q] = (ar < M && ak + q < K) ? __ldcg(A + (size_t)ar * K + ak + q) : 0.f;
    }
    if (vec && bk < K && bc + 3 < N) {
      const float4 v = __ldcg(reinterpret_cast<const float4*>(B + (size_t)bk * N + bc));
      rb[0] = v.x; rb[1] = v.y; rb[2] = v.z; rb[3] = v.w;
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) rb[q] = (bk < K && bc + q < N) ? __ldcg(B + (size_t)bk * N + bc + q) : 0.f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; q++) sm.A[buf][la_k + q][la_r] = ra[q];
    *reinterpret_cast<float4*>(&sm.B[buf][lb_k][lb_c]) = make_float4(rb[0], rb[1], rb[2], rb[3]);
  };
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = 0.f;
  const int nk = (K + SG_BK - 1) / SG_BK;
  load(0);
  store(0);
  __syncthreads();
  for (int s = 0; s < nk; s++) {
    const int cur = s & 1;
    if (s + 1 < nk) load((s + 1) * SG_BK);
#pragma unroll
    for (int kk = 0; kk < SG_BK; kk++) {
      const float4 a4 = *reinterpret_cast<const float4*>(&sm.A[cur][kk][ty * 4]);
      const float4 b4 = *reinterpret_cast<const float4*>(&sm.B[cur][kk][tx * 4]);
      const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
    }
    if (s + 1 < nk) store(cur ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int r = row0 + ty * 4 + a, c = col0 + tx * 4 + b;
      if (r >= M || c >= N) continue;
      if (EPI == 0) Cm[r * N + c] = acc[a][b];
      else if (EPI == 1) Cm[r * N + c] = acc[a][b] * D[r * N + c];
      else spec_add_phi(L, N, r, c, acc[a][b]);
    }
}

// ---- FFT passes (SpecFFT) ----
// Lines per unit of work: two complex FFTs, each carrying two real lines (one
// in the real part, one in the imaginary part).
constexpr int SPEC_FFT_LINES = 4;
// Shared-memory slots of one FFT sequence of length m (padded).
__host__ __device__ __forceinline__ int spec_fft_seq(int m) { return m + (m >> 5); }
__device__ __forceinline__ int spec_fft_pad(int i) { return i + (i >> 5); }

// One unit of an FFT pass: lines [l0, l0 + SPEC_FFT_LINES) of `in`, transformed
// along direction dir (0: along r, a line per column c; 1: along c, a line per
// row r), the results (r, c) through the epilogue EPI as in spec_gemm_tile:
// 0 store to out, 1 store times D, 2 add to phi.  buf: shared memory for
// SPEC_FFT_LINES / 2 sequences of the FFT length, each element i of a
// sequence at i + i / 32 (spec_fft_pad: one spare slot per 32, so that the
// bit-reversed stores and the short-span butterflies spread over the
// banks).  Decimation in time from bit-reversed loads, radix 2 taken two
// stages at a time.  Hartley: Z = FFT(x + i y), H_k = (Re X_k - Im X_k)
// with X_k = (Z_k + conj Z_(m-k)) / 2 (and Y likewise).  Sine: the odd
// extension of length m = 2 (n + 1) has FFT -2i S'(x) + 2 S'(y), with S' the
// unnormalised DST-I at index k + 1.
template <int EPI>
__device__ __forceinline__ void spec_fft_unit(const SpecLattice& L, const SpecFFT& F, int dir, int l0,
                                              const float* in, float* out, const float* __restrict__ D,
                                              float2* buf, const float2* twR, const float2* twC) {
  constexpr int NF = SPEC_FFT_LINES / 2, LN = SPEC_FFT_LINES, U = 4;
  static_assert(LN == 4, "element q of a unit is line q & 3, index q >> 2");
  const int R = L.R, C = L.C;
  const int n = dir == 0 ? R : C, nl = dir == 0 ? C : R;
  const int m = dir == 0 ? F.mR : F.mC, lg = dir == 0 ? F.lgR : F.lgC;
  const int sine = dir == 0 ? F.sineR : F.sineC;
  const float sc = dir == 0 ? F.scaleR : F.scaleC;
  const float2* tw = dir == 0 ? twR : twC;  // shared memory
  float* const bf = reinterpret_cast<float*>(buf);
  // Element q of the unit: line q & 3, index q >> 2 along it (a warp reads
  // eight 16-byte runs: adjacent columns along r, or eight adjacent values of
  // four rows along c - the same sectors as one 128-byte run).
  auto at = [&](int line, int e) { return dir == 0 ? e * C + line : line * C + e; };
  const int seq = spec_fft_seq(m);
  auto slot = [&](int f, int pos, int comp) {
    return 2 * (f * seq + spec_fft_pad((int)(__brev((unsigned)pos) >> (32 - lg)))) + comp;
  };
  if (sine && threadIdx.x < 2 * NF * 2) {  // the odd extension's zeros at 0 and n + 1
    const int f = threadIdx.x >> 2, which = (threadIdx.x >> 1) & 1, comp = threadIdx.x & 1;
    bf[slot(f, which ? n + 1 : 0, comp)] = 0.f;
  }
  // loads: U per thread in flight, then their shared-memory stores
  for (int q0 = threadIdx.x; q0 < LN * n; q0 += U * blockDim.x) {
    float v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * blockDim.x, l = q & (LN - 1), e = q >> 2;
      v[u] = q < LN * n && l0 + l < nl ? __ldcg(&in[at(l0 + l, e)]) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * blockDim.x, l = q & (LN - 1), e = q >> 2;
      if (q >= LN * n) continue;
      const int f = l >> 1, comp = l & 1;
      if (sine) {
        bf[slot(f, e + 1, comp)] = v[u];
        bf[slot(f, m - 1 - e, comp)] = -v[u];
      } else {
        bf[slot(f, e, comp)] = v[u];
      }
    }
  }
  __syncthreads();
  // Stages s = 0 .. lg-1 (half-span 2^s) two at a time: a thread takes the
  // four elements g 4h + j + {0, h, 2h, 3h} (j < h = 2^s) through stage s
  // (pairs at distance h, twiddle j) and stage s + 1 (pairs at distance 2h,
  // twiddles j and j + h) in registers - one barrier and one shared-memory
  // round trip per two stages; an odd last stage alone.
  auto bfly = [](float2& a, float2& c, float2 w) {
    const float2 t = make_float2(w.x * c.x - w.y * c.y, w.x * c.y + w.y * c.x);
    c = make_float2(a.x - t.x, a.y - t.y);
    a = make_float2(a.x + t.x, a.y + t.y);
  };
  int st = 0;
  for (; st + 1 < lg; st += 2) {
    const int h = 1 << st, quarter = m >> 2;
    for (int q = threadIdx.x; q < NF * quarter; q += blockDim.x) {
      const int f = q >> (lg - 2), b = q & (quarter - 1);
      const int j = b & (h - 1), i0 = ((b >> st) << (st + 2)) + j;
      float2* x = buf + f * seq;
      const int p0 = spec_fft_pad(i0), p1 = spec_fft_pad(i0 + h), p2 = spec_fft_pad(i0 + 2 * h),
                p3 = spec_fft_pad(i0 + 3 * h);
      float2 a0 = x[p0], a1 = x[p1], a2 = x[p2], a3 = x[p3];
      const float2 w1 = tw[j << (lg - 1 - st)];
      bfly(a0, a1, w1);
      bfly(a2, a3, w1);
      bfly(a0, a2, tw[j << (lg - 2 - st)]);
      bfly(a1, a3, tw[(j + h) << (lg - 2 - st)]);
      x[p0] = a0;
      x[p1] = a1;
      x[p2] = a2;
      x[p3] = a3;
    }
    __syncthreads();
  }
  if (st < lg) {
    const int h = 1 << st, half = m >> 1;
    for (int q = threadIdx.x; q < NF * half; q += blockDim.x) {
      const int f = q >> (lg - 1), b = q & (half - 1);
      const int j = b & (h - 1), i1 = ((b >> st) << (st + 1)) + j;
      float2* x = buf + f * seq;
      const int p1 = spec_fft_pad(i1), p2 = spec_fft_pad(i1 + h);
      float2 a = x[p1], c = x[p2];
      bfly(a, c, tw[j << (lg - 1 - st)]);
      x[p1] = a;
      x[p2] = c;
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < LN * n; q += blockDim.x) {
    const int l = q & (LN - 1), k = q >> 2, line = l0 + l;
    if (line >= nl) continue;
    const int f = l >> 1, comp = l & 1;
    const float2* Z = buf + f * seq;
    float y;
    if (sine) {
      const float2 z = Z[spec_fft_pad(k + 1)];
      y = comp ? 0.5f * z.x : -0.5f * z.y;
    } else {
      const float2 z = Z[spec_fft_pad(k)], zc = Z[spec_fft_pad((m - k) & (m - 1))];
      y = comp ? 0.5f * ((z.y + zc.y) + (z.x - zc.x)) : 0.5f * ((z.x + zc.x) - (z.y - zc.y));
    }
    y *= sc;
    const int r = dir == 0 ? k : line, c = dir == 0 ? line : k;
    if (EPI == 0) out[r * C + c] = y;
    else if (EPI == 1) out[r * C + c] = y * __ldg(&D[r * C + c]);
    else spec_add_phi(&L, C, r, c, y);
  }
  __syncthreads();  // buf is reused by the next unit
}

}  // namespace epic
