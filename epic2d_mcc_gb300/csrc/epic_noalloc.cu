// epic_pcg_solve_static: the PCG Poisson solve on caller-owned device
// buffers, with all of its scratch in a fixed array compiled into this
// library, so a call never allocates device memory.
//
// Who needs this: callers that may not allocate device memory themselves —
// a host framework whose memory pool or budget owns every byte of the GPU and
// forbids private allocations, a plugin that may only touch the buffers its
// host hands it, and real-time loops that must not meet the allocator's
// latency or an out-of-memory failure in the middle of a run.  The regular
// entry points (epic_create and the epic_sim handle) allocate their workspace
// themselves and cannot serve such callers.
//
// The scratch is one static device array of PCG_STATIC_BYTES, enough for
// grids of up to PCG_STATIC_MAX_NODES nodes (257 x 257); it is held by every
// GPU that loads the library, for as long as the library stays loaded.  The
// array is shared by all calls and keeps what the last call left in it; the
// parts that must start at zero (the grid-barrier counter, the error flags)
// are cleared on the caller's stream at the start of every call.  Calls
// whose GPU work overlaps (on different streams, or from several host
// threads without ordering) race on the array: order them on one stream or
// serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "epic_internal.cuh"

namespace {

using namespace epic;

constexpr int PCG_STATIC_MAX_NODES = 257 * 257;
constexpr int PCG_STATIC_MAX_BLOCKS = 1024;
// 8 node vectors + 2 x 4 partials per block + barrier counter, solve outcome,
// iteration total and error flags, each section 256-byte aligned.
constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t PCG_VEC_BYTES = align256((size_t)PCG_STATIC_MAX_NODES * sizeof(double));
constexpr size_t PCG_PART_BYTES = align256((size_t)8 * PCG_STATIC_MAX_BLOCKS * sizeof(double));
constexpr size_t PCG_STATIC_BYTES = 8 * PCG_VEC_BYTES + PCG_PART_BYTES + 4 * 256;

static __device__ __align__(256) unsigned char g_pcg_scratch[PCG_STATIC_BYTES];

epic_status fail_na(epic_status st, const char* msg) {
  set_last_error(msg);  // reported by epic_last_error(), as for every entry point
  return st;
}

// Device address of the static array on the current device.  Looked up on
// every call (a host-side query, not a stream operation): the address belongs
// to the context that loaded this library's device code, and a caller that
// resets the device (cudaDeviceReset) gets a new context in which the array
// may sit elsewhere, so an address kept from an earlier call could be stale.
epic_status scratch_address(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_pcg_scratch);
  if (e != cudaSuccess || !p) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "cudaGetSymbolAddress(g_pcg_scratch): %s", cudaGetErrorString(e));
    return fail_na(EPIC_ERR_CUDA, buf);
  }
  *out = static_cast<unsigned char*>(p);
  return EPIC_OK;
}

}  // namespace

extern "C" {

epic_status epic_pcg_solve_static(const double* rho, double* phi, int nx, int ny, double dx, double K,
                                  double tolerance, int max_iteration, void* stream, int* iterations,
                                  double* error) {
  if (!rho || !phi || nx < 3 || ny < 3 || !(dx > 0) || max_iteration < 0)
    return fail_na(EPIC_ERR_INVALID, "epic_pcg_solve_static: bad argument");
  if ((long long)nx * ny > PCG_STATIC_MAX_NODES) {
    char buf[200];
    std::snprintf(buf, sizeof(buf),
                  "epic_pcg_solve_static: %d x %d = %lld nodes exceed the static scratch limit of %d nodes "
                  "(257 x 257); use the epic_sim entry points for larger grids",
                  nx, ny, (long long)nx * ny, PCG_STATIC_MAX_NODES);
    return fail_na(EPIC_ERR_CAPACITY, buf);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_na(EPIC_ERR_CUDA, "no usable CUDA device");
  unsigned char* base = nullptr;
  epic_status st = scratch_address(&base);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  SolverArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g.nx = nx;
  a.g.ny = ny;
  a.g.dx = dx;
  a.g.dy = dx;
  a.tol = tolerance;
  a.max_iter = max_iteration;
  a.K = K;
  a.rho = rho;
  a.phi = phi;
  for (int k = 0; k < 8; k++) a.work[k] = reinterpret_cast<double*>(base + k * PCG_VEC_BYTES);
  unsigned char* tail = base + 8 * PCG_VEC_BYTES;
  a.partials = reinterpret_cast<double*>(tail);
  tail += PCG_PART_BYTES;
  a.bar = reinterpret_cast<unsigned int*>(tail);
  a.info = reinterpret_cast<SolveInfo*>(tail + 256);
  a.iter_total = reinterpret_cast<unsigned long long*>(tail + 512);
  a.flags = reinterpret_cast<int*>(tail + 768);
  // Same CTA count as the epic_sim path, so both give identical results.
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int blocks = std::max(1, std::min(pcg_default_blocks((long long)nx * ny, sms), PCG_STATIC_MAX_BLOCKS));
  // Zero what the kernel expects zeroed (the barrier counter is also reset
  // inside launch_pcg); the rest is written before it is read.
  if ((e = cudaMemsetAsync(a.flags, 0, sizeof(int), s)) != cudaSuccess ||
      (e = cudaMemsetAsync(a.iter_total, 0, sizeof(unsigned long long), s)) != cudaSuccess)
    return fail_na(EPIC_ERR_CUDA, cudaGetErrorString(e));
  launch_pcg(s, a, blocks);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail_na(EPIC_ERR_CUDA, cudaGetErrorString(e));
  SolveInfo info;
  int flags = 0;
  if ((e = cudaMemcpyAsync(&info, a.info, sizeof(info), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&flags, a.flags, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail_na(EPIC_ERR_CUDA, cudaGetErrorString(e));
  if (flags & FLAG_TIMEOUT) return fail_na(EPIC_ERR_TIMEOUT, "epic_pcg_solve_static: a grid barrier gave up");
  if (iterations) *iterations = info.iterations;
  if (error) *error = info.error;
  if (!info.converged) return fail_na(EPIC_WARN_NOT_CONVERGED, "epic_pcg_solve_static: max_iteration reached");
  return EPIC_OK;
}

}  // extern "C"
