// Cell sort of a species' particles (no counterpart in the reference, which
// never reorders its particle vector).
//
// The key of a particle is the flat index of the lower-left node of its cell,
// i*ny + j with i = (int)((x - x0)/dx), j = (int)((y - y0)/dy) — the node the
// reference's deposit starts from (src/domain.cpp:207-208) — which is the
// mixed form's stored cell.  The sort is a stable LSD radix sort of
// (key, particle index) pairs with 9-bit digits (two passes up to 2^18
// nodes), then one gather of the particle records by the resulting
// permutation and a copy back in place.  Stable means particles of a cell
// keep their relative order, so the permutation is fully determined by the
// keys (the same as a stable argsort of them).
//
// Each pass: k_radix_hist counts the digits of every 4096-key tile
// (digit-major table [digit][tile]); a three-kernel exclusive scan of that
// table gives every (digit, tile) its output offset; k_radix_scatter ranks
// each key within its tile in input order (warp-synchronous match of equal
// digits, per-warp running counts) and writes it to offset + rank.  All
// launches are sized by the species capacity and read the live count on the
// device, so the sort can be captured in a CUDA graph.
#include <cuda_runtime.h>

#include <climits>

#include "epic_internal.cuh"
#include "epic_mixed.cuh"

namespace epic {

constexpr int SORT_T = 256;                 // threads per CTA
constexpr int SORT_PER_WARP = 512;          // keys per warp and tile
constexpr int SORT_TILE = SORT_T / 32 * SORT_PER_WARP;  // 4096 keys per tile
constexpr int RADIX_BITS = 9;
constexpr int RADIX = 1 << RADIX_BITS;      // 512 digits
constexpr int SCAN_BLOCK = 4096;            // scan entries per CTA (1024 threads x 4)

long long sort_tiles(long long cap) { return (cap + SORT_TILE - 1) / SORT_TILE; }

int sort_passes(int nodes) {
  int bits = 1;
  while (bits < 31 && (1ll << bits) < (long long)nodes) bits++;
  return (bits + RADIX_BITS - 1) / RADIX_BITS;
}

__global__ void k_sort_keys_fp64(Geom g, SoA p, const long long* __restrict__ d_n, unsigned* __restrict__ keys) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double lx = (p.x[q] - g.x0) / g.dx, ly = (p.y[q] - g.y0) / g.dy;
    int i = (int)lx, j = (int)ly;
    i = min(max(i, 0), g.nx - 1);
    j = min(max(j, 0), g.ny - 1);
    keys[q] = (unsigned)(i * g.ny + j);
  }
}

__global__ void k_sort_keys_mixed(MixedSoA p, const long long* __restrict__ d_n, unsigned* __restrict__ keys) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    keys[q] = (unsigned)p.cell[q];
}

// Digit counts of one tile: hist[d * T + tile].
__global__ void __launch_bounds__(SORT_T) k_radix_hist(const unsigned* __restrict__ keys,
                                                      const long long* __restrict__ d_n, int shift,
                                                      unsigned* __restrict__ hist, int T) {
  __shared__ unsigned cnt[RADIX];
  for (int d = threadIdx.x; d < RADIX; d += SORT_T) cnt[d] = 0;
  __syncthreads();
  const long long n = *d_n;
  const long long base = (long long)blockIdx.x * SORT_TILE;
  for (int m = threadIdx.x; m < SORT_TILE; m += SORT_T) {
    const long long q = base + m;
    if (q < n) atomicAdd(&cnt[(keys[q] >> shift) & (RADIX - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += SORT_T) hist[(long long)d * T + blockIdx.x] = cnt[d];
}

// Exclusive scan of E entries: per-CTA scans with the CTA totals in bsum,
// a one-CTA scan of the totals, then the totals added back.
__device__ __forceinline__ unsigned block_exscan_1024(unsigned v, unsigned* sm /* >= 32 */, unsigned* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned s = sm[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    sm[lane] = s;
  }
  __syncthreads();
  const unsigned before = (wid ? sm[wid - 1] : 0u) + x - v;
  *total = sm[31];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(1024) k_scan_local(unsigned* __restrict__ a, long long E, unsigned* __restrict__ bsum) {
  __shared__ unsigned sm[32];
  const long long base = (long long)blockIdx.x * SCAN_BLOCK + threadIdx.x * 4;
  unsigned v[4], s = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[k] = base + k < E ? a[base + k] : 0u;
    s += v[k];
  }
  unsigned total;
  unsigned run = block_exscan_1024(s, sm, &total);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (base + k < E) a[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_top(unsigned* __restrict__ bsum, int nb) {
  __shared__ unsigned sm[32];
  __shared__ unsigned carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int k = base + threadIdx.x;
    const unsigned v = k < nb ? bsum[k] : 0u;
    unsigned total;
    const unsigned ex = block_exscan_1024(v, sm, &total);
    if (k < nb) bsum[k] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
}

__global__ void k_scan_add(unsigned* __restrict__ a, long long E, const unsigned* __restrict__ bsum) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < E) a[q] += bsum[q / SCAN_BLOCK];
}

// Stable scatter of one tile.  Warp w owns keys [w*512, w*512 + 512) of the
// tile and walks them 32 at a time in order; lanes holding the same digit
// (__match_any_sync) rank themselves by lane, on top of the warp's running
// count for that digit.  Then per digit the warps' counts are turned into
// absolute bases: the tile's scanned offset plus the counts of the warps
// before.  vals_in == nullptr means the identity (first pass).
__global__ void __launch_bounds__(SORT_T) k_radix_scatter(const unsigned* __restrict__ keys_in,
                                                         const unsigned* __restrict__ vals_in,
                                                         unsigned* __restrict__ keys_out,
                                                         unsigned* __restrict__ vals_out,
                                                         const long long* __restrict__ d_n, int shift,
                                                         const unsigned* __restrict__ offs, int T) {
  __shared__ unsigned cnt[SORT_T / 32][RADIX];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int m = threadIdx.x; m < SORT_T / 32 * RADIX; m += SORT_T) (&cnt[0][0])[m] = 0;
  __syncthreads();
  const long long n = *d_n;
  const long long base = (long long)blockIdx.x * SORT_TILE + (long long)w * SORT_PER_WARP;
  const unsigned lt = (1u << lane) - 1u;
  constexpr int R = SORT_PER_WARP / 32;
  unsigned key[R], val[R], rank[R];
  // All of the warp's loads first: the ranking rounds below are ordered by
  // __syncwarp, which loads issued inside them could not cross.
#pragma unroll
  for (int r = 0; r < R; r++) {
    const long long q = base + r * 32 + lane;
    const bool valid = q < n;
    key[r] = valid ? __ldg(&keys_in[q]) : 0xFFFFFFFFu;
    val[r] = valid ? (vals_in ? __ldg(&vals_in[q]) : (unsigned)q) : 0u;
  }
#pragma unroll
  for (int r = 0; r < R; r++) {
    const long long q = base + r * 32 + lane;
    const bool valid = q < n;
    const unsigned d = valid ? (key[r] >> shift) & (RADIX - 1) : (unsigned)RADIX;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned pos = __popc(peers & lt);
    unsigned c = 0;
    if (valid) c = cnt[w][d];
    __syncwarp();
    if (valid && pos == 0) cnt[w][d] = c + __popc(peers);
    __syncwarp();
    rank[r] = c + pos;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += SORT_T) {
    unsigned run = offs[(long long)d * T + blockIdx.x];
#pragma unroll
    for (int k = 0; k < SORT_T / 32; k++) {
      const unsigned t = cnt[k][d];
      cnt[k][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < R; r++) {
    const long long q = base + r * 32 + lane;
    if (q < n) {
      const unsigned dst = cnt[w][(key[r] >> shift) & (RADIX - 1)] + rank[r];
      keys_out[dst] = key[r];
      vals_out[dst] = val[r];
    }
  }
}

__global__ void k_gather_fp64(SoA src, SoA tmp, const unsigned* __restrict__ perm, const long long* __restrict__ d_n) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const unsigned j = perm[q];
    tmp.x[q] = src.x[j];
    tmp.y[q] = src.y[j];
    tmp.vx[q] = src.vx[j];
    tmp.vy[q] = src.vy[j];
    tmp.vz[q] = src.vz[j];
  }
}

__global__ void k_copy_fp64(SoA tmp, SoA dst, const long long* __restrict__ d_n) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    dst.x[q] = tmp.x[q];
    dst.y[q] = tmp.y[q];
    dst.vx[q] = tmp.vx[q];
    dst.vy[q] = tmp.vy[q];
    dst.vz[q] = tmp.vz[q];
  }
}

__global__ void k_gather_mixed(MixedSoA src, MixedSoA tmp, const unsigned* __restrict__ perm,
                               const long long* __restrict__ d_n) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const unsigned j = perm[q];
    tmp.cell[q] = src.cell[j];
    tmp.ox[q] = src.ox[j];
    tmp.oy[q] = src.oy[j];
    tmp.vx[q] = src.vx[j];
    tmp.vy[q] = src.vy[j];
    tmp.vz[q] = src.vz[j];
  }
}

__global__ void k_copy_mixed(MixedSoA tmp, MixedSoA dst, const long long* __restrict__ d_n) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    dst.cell[q] = tmp.cell[q];
    dst.ox[q] = tmp.ox[q];
    dst.oy[q] = tmp.oy[q];
    dst.vx[q] = tmp.vx[q];
    dst.vy[q] = tmp.vy[q];
    dst.vz[q] = tmp.vz[q];
  }
}

int launch_sort(cudaStream_t st, const Geom& g, const ParticleRef& p, const long long* d_n, long long cap,
                const SortScratch& sc, int grid) {
  const int T = (int)sort_tiles(cap);
  const long long E = (long long)RADIX * T;
  const int nscan = (int)((E + SCAN_BLOCK - 1) / SCAN_BLOCK);
  int launches = 0;
  if (p.mixed) k_sort_keys_mixed<<<grid, PART_THREADS, 0, st>>>(p.m, d_n, sc.keys[0]);
  else k_sort_keys_fp64<<<grid, PART_THREADS, 0, st>>>(g, p.f, d_n, sc.keys[0]);
  launches++;
  const int passes = sort_passes(g.nx * g.ny);
  int cur = 0;
  for (int ps = 0; ps < passes; ps++) {
    const int shift = ps * RADIX_BITS;
    k_radix_hist<<<T, SORT_T, 0, st>>>(sc.keys[cur], d_n, shift, sc.hist, T);
    k_scan_local<<<nscan, 1024, 0, st>>>(sc.hist, E, sc.bsum);
    k_scan_top<<<1, 1024, 0, st>>>(sc.bsum, nscan);
    k_scan_add<<<(int)((E + 255) / 256), 256, 0, st>>>(sc.hist, E, sc.bsum);
    k_radix_scatter<<<T, SORT_T, 0, st>>>(sc.keys[cur], ps ? sc.vals[cur] : nullptr, sc.keys[cur ^ 1],
                                          sc.vals[cur ^ 1], d_n, shift, sc.hist, T);
    launches += 5;
    cur ^= 1;
  }
  if (p.mixed) {
    MixedSoA tmp;
    char* b = static_cast<char*>(sc.tmp);
    tmp.cell = reinterpret_cast<int*>(b);
    tmp.ox = reinterpret_cast<float*>(b + 4 * cap);
    tmp.oy = reinterpret_cast<float*>(b + 8 * cap);
    tmp.vx = reinterpret_cast<float*>(b + 12 * cap);
    tmp.vy = reinterpret_cast<float*>(b + 16 * cap);
    tmp.vz = reinterpret_cast<float*>(b + 20 * cap);
    k_gather_mixed<<<grid, PART_THREADS, 0, st>>>(p.m, tmp, sc.vals[cur], d_n);
    k_copy_mixed<<<grid, PART_THREADS, 0, st>>>(tmp, p.m, d_n);
  } else {
    SoA tmp;
    double* b = static_cast<double*>(sc.tmp);
    tmp.x = b;
    tmp.y = b + cap;
    tmp.vx = b + 2 * cap;
    tmp.vy = b + 3 * cap;
    tmp.vz = b + 4 * cap;
    k_gather_fp64<<<grid, PART_THREADS, 0, st>>>(p.f, tmp, sc.vals[cur], d_n);
    k_copy_fp64<<<grid, PART_THREADS, 0, st>>>(tmp, p.f, d_n);
  }
  return launches + 2;
}

// One buffer: keys x2, vals x2 (4 bytes each per slot), the digit table, the
// scan totals and the payload copy (payload bytes per slot: 24 for the mixed
// form's records, 40 for the FP64 form's), each 256-byte aligned.
static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t sort_scratch_bytes(long long cap, int payload) {
  const long long T = sort_tiles(cap);
  const long long E = (long long)RADIX * T;
  const long long nscan = (E + SCAN_BLOCK - 1) / SCAN_BLOCK;
  return 4 * al256(4 * (size_t)cap) + al256(4 * (size_t)E) + al256(4 * (size_t)nscan) +
         al256((size_t)payload * (size_t)cap);
}

SortScratch carve_sort_scratch(void* buf, long long cap) {
  const long long T = sort_tiles(cap);
  const long long E = (long long)RADIX * T;
  const long long nscan = (E + SCAN_BLOCK - 1) / SCAN_BLOCK;
  char* b = static_cast<char*>(buf);
  SortScratch s;
  for (int k = 0; k < 2; k++) {
    s.keys[k] = reinterpret_cast<unsigned*>(b);
    b += al256(4 * (size_t)cap);
    s.vals[k] = reinterpret_cast<unsigned*>(b);
    b += al256(4 * (size_t)cap);
  }
  s.hist = reinterpret_cast<unsigned*>(b);
  b += al256(4 * (size_t)E);
  s.bsum = reinterpret_cast<unsigned*>(b);
  b += al256(4 * (size_t)nscan);
  s.tmp = b;
  return s;
}

// ----------------------------------------------- deposit of sorted particles ---
// CIC deposit of the mixed form for particles sorted by cell (or nearly so,
// between sorts): each warp takes a contiguous chunk of DEP_WARP_CHUNK
// particles and deposits it with deposit_warp_sorted (epic_mixed.cuh).  The sums are
// integers, so the result is identical to k_deposit_mixed's.
__global__ void __launch_bounds__(PART_THREADS) k_deposit_mixed_sorted(Geom g, MixedSoA p,
                                                                       const long long* __restrict__ d_n,
                                                                       unsigned long long* __restrict__ acc) {
  __shared__ DepWarp tables[PART_THREADS / 32];
  DepWarp& w = tables[threadIdx.x >> 5];
  const long long n = *d_n;
  dep_init(w);
  for (long long chunk = (long long)blockIdx.x * DEP_CHUNK; chunk < n; chunk += (long long)gridDim.x * DEP_CHUNK) {
    const long long q0 = chunk + (long long)threadIdx.x * DEP_PER_THREAD;
    int c[DEP_PER_THREAD];
    float ox[DEP_PER_THREAD], oy[DEP_PER_THREAD];
    if (q0 + DEP_PER_THREAD <= n) {
      const int4* pc = reinterpret_cast<const int4*>(p.cell + q0);
      const float4* px = reinterpret_cast<const float4*>(p.ox + q0);
      const float4* py = reinterpret_cast<const float4*>(p.oy + q0);
#pragma unroll
      for (int h = 0; h < DEP_PER_THREAD / 4; h++) {
        const int4 cc = __ldg(pc + h);
        const float4 xx = __ldg(px + h), yy = __ldg(py + h);
        c[4 * h] = cc.x; c[4 * h + 1] = cc.y; c[4 * h + 2] = cc.z; c[4 * h + 3] = cc.w;
        ox[4 * h] = xx.x; ox[4 * h + 1] = xx.y; ox[4 * h + 2] = xx.z; ox[4 * h + 3] = xx.w;
        oy[4 * h] = yy.x; oy[4 * h + 1] = yy.y; oy[4 * h + 2] = yy.z; oy[4 * h + 3] = yy.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < DEP_PER_THREAD; k++) {
        const long long q = q0 + k;
        c[k] = q < n ? __ldg(&p.cell[q]) : -1;
        ox[k] = q < n ? __ldg(&p.ox[q]) : 0.f;
        oy[k] = q < n ? __ldg(&p.oy[q]) : 0.f;
      }
    }
    deposit_warp_sorted(acc, w, ConstNy{g.ny}, c, ox, oy);
  }
}

void launch_deposit_mixed_sorted(cudaStream_t st, const Geom& g, const MixedSoA& p, const long long* d_n,
                                 unsigned long long* acc, int grid) {
  k_deposit_mixed_sorted<<<grid, PART_THREADS, 0, st>>>(g, p, d_n, acc);
}

}  // namespace epic
