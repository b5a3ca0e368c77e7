// Device-side particle loading and the run digest (no counterparts in the
// reference).
//
// The loader places particles exactly as Init::Init (src/init.cpp:3-114) and
// Init::SampleVel do — uniform random, uniform lattice, or sin/cos(n)
// positions, and v = v_th*sqrt(2)*(u1 + u2 + u3 - 1.5) + drift per component
// (vz = 0, or drawn like vx and vy with load_3v), normalised by vel_norm — but
// draws its uniforms from Philox keyed
// by (seed, species, particle) on the GPU instead of the host mt19937 stream,
// so a run can be loaded without a host-side pass over its particles (the
// serving loop admits runs of ~10^7 particles while others are in flight).
// The host loader (epic_load_particles) remains the one that reproduces the
// reference's particles.  Conductor rectangles keep particles out as Init's
// loop does (src/init.cpp:71-86, Grid::IsGrid; a CircularGrid has no
// electrodes yet): a random position inside one is drawn again from the
// particle's own stream (up to LOAD_REDRAWS times, then an error), and a
// deterministic position inside one is an error (the reference would loop
// forever).
//
// The digest is an order-independent 64-bit hash of a run's state: the sum
// over elements of a mix of (bits, position, array) — integer additions, so
// the total does not depend on the order the GPU adds them in — used to show
// that a run's result is bit-identical whether it ran alone or beside others.
#include <cuda_runtime.h>

#include "epic_device.cuh"
#include "epic_internal.cuh"

namespace epic {

struct LoadSpec {
  int kind;   // 0 random, 1 uniform, 2 sin(n), 3 cos(n)
  int narg;
  long long n;
  int species;
  double x0, y0, Lx, Ly;
  double v_th, vsx, vsy, vel_norm;
  double pi;
  int load_3v;
  int nrect;
  const double4* rect;
  int* flags;
};

constexpr int LOAD_REDRAWS = 1024;

__device__ __forceinline__ bool load_in_rect(const LoadSpec& L, double x, double y) {
  for (int k = 0; k < L.nrect; k++) {
    const double4 r = L.rect[k];
    if (x >= r.x && x <= r.y && y >= r.z && y <= r.w) return true;
  }
  return false;
}

__global__ void k_load(LoadSpec L, double* __restrict__ aos, unsigned long long seed) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < L.n; p += (long long)gridDim.x * blockDim.x) {
    Philox r;
    r.c0 = (uint32_t)p;
    r.c1 = (uint32_t)((unsigned long long)p >> 32);
    r.c2 = 0x10AD0000u + (uint32_t)L.species;
    r.key0 = (uint32_t)seed;
    r.key1 = (uint32_t)(seed >> 32);
    r.k = 0;
    double x, y;
    bool bad = false;
    if (L.kind == 0) {
      x = L.x0 + L.Lx * r.next();
      y = L.y0 + L.Ly * r.next();
      for (int t = 0; L.nrect && load_in_rect(L, x, y); t++) {
        if (t == LOAD_REDRAWS) {
          bad = true;
          break;
        }
        x = L.x0 + L.Lx * r.next();
        y = L.y0 + L.Ly * r.next();
      }
    } else if (L.kind == 1) {
      const int nxp = (int)sqrt((double)L.n);
      const int px = (int)(p % nxp), py = (int)(p / nxp);
      x = L.x0 + px * (L.Lx / (nxp - 1));
      y = L.y0 + py * (L.Ly / (nxp - 1));
    } else {
      x = L.x0 + p * (L.Lx / (L.n - 1));
      y = L.y0 + p * (L.Ly / (L.n - 1));
      const double kx = 2 * L.pi * L.narg / L.Lx, ky = 2 * L.pi * L.narg / L.Ly;
      if (L.kind == 2) {
        x += sin(kx * x);
        y += sin(ky * y);
      } else {
        x += cos(kx * x);
        y += cos(ky * y);
      }
    }
    if (L.kind != 0 && L.nrect) bad = load_in_rect(L, x, y);
    if (bad) atomicOr(L.flags, FLAG_LOAD_IN_CONDUCTOR);
    const double s2 = sqrt(2.0);
    double u1 = r.next(), u2 = r.next(), u3 = r.next();
    double vx = L.v_th * s2 * (u1 + u2 + u3 - 1.5) + L.vsx * L.vel_norm;
    u1 = r.next(); u2 = r.next(); u3 = r.next();
    double vy = L.v_th * s2 * (u1 + u2 + u3 - 1.5) + L.vsy * L.vel_norm;
    double* q = aos + 5 * p;
    q[0] = x;
    q[1] = y;
    q[2] = vx / L.vel_norm;
    q[3] = vy / L.vel_norm;
    double vz = 0.0;
    if (L.load_3v) {
      u1 = r.next(); u2 = r.next(); u3 = r.next();
      vz = L.v_th * s2 * (u1 + u2 + u3 - 1.5);
    }
    q[4] = vz / L.vel_norm;
  }
}

__global__ void k_set_count(long long* d_n, long long n) { *d_n = n; }

void launch_load(cudaStream_t st, const Geom& g, const epic_species_desc& d, const epic_config& c, int species,
                 int kind, int narg, double* aos, unsigned long long seed, int grid, const double4* rect, int nrect,
                 int* flags) {
  LoadSpec L;
  L.kind = kind;
  L.narg = narg;
  L.n = d.numparticle;
  L.species = species;
  L.x0 = c.x0;
  L.y0 = c.y0;
  L.Lx = (c.nx - 1) * c.dx;
  L.Ly = (c.ny - 1) * c.dy;
  L.v_th = sqrt(2 * K_B * d.temp * (QE / K_B) / d.mass);
  L.vsx = d.vsx;
  L.vsy = d.vsy;
  L.vel_norm = c.vel_norm;
  L.pi = PI_REF;
  L.load_3v = c.load_3v;
  L.nrect = rect && flags ? nrect : 0;
  L.rect = rect;
  L.flags = flags;
  if (L.n > 0) k_load<<<grid, PART_THREADS, 0, st>>>(L, aos, seed);
  (void)g;
}

void launch_set_count(cudaStream_t st, long long* d_n, long long n) { k_set_count<<<1, 1, 0, st>>>(d_n, n); }

// ---------------------------------------------------------------- digest ---
// splitmix64's output function (Steele, Lea, Flood, OOPSLA'14) as the mixer.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Adds sum_k mix(bits(a[k]) + tag + k * golden) over k < *d_n (or n if d_n is
// null) to *out.  Elements are 4 or 8 bytes.
__global__ void k_digest(const void* __restrict__ a, int elem_bytes, const long long* __restrict__ d_n, long long n,
                         unsigned long long tag, unsigned long long* out) {
  const long long m = d_n ? *d_n : n;
  unsigned long long h = 0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
    const unsigned long long bits = elem_bytes == 8 ? static_cast<const unsigned long long*>(a)[k]
                                                    : static_cast<const unsigned int*>(a)[k];
    h += mix64(bits + tag * 0xD6E8FEB86659FD93ull + (unsigned long long)k * 0x9E3779B97F4A7C15ull);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) h += __shfl_down_sync(0xffffffffu, h, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, h);
}

void launch_digest(cudaStream_t st, const void* a, int elem_bytes, const long long* d_n, long long n,
                   unsigned long long tag, unsigned long long* out, int grid) {
  k_digest<<<grid, PART_THREADS, 0, st>>>(a, elem_bytes, d_n, n, tag, out);
}

}  // namespace epic
