// Emitter::inject's draws for one point (src/emitter.cpp:5-36), shared by the
// single-run injection (k_emit) and the batched one (k_batch_emit), so that a
// batched run injects the same records as the same run alone.
#pragma once

#include "epic_device.cuh"

namespace epic {

// Point q of emitter e: uniforms 0-1 place it (std::uniform_real_distribution:
// u (b - a) + a) and 2 + 6*slot .. 7 + 6*slot give its velocity
// (Init::SampleVel, src/init.cpp:110-114: vth sqrt(2) (u1 + u2 + u3 - 1.5),
// plus the drift, over vel_norm), from the caller's rows of 14 or from Philox
// keyed by (q, emitter | 2^31, injection, seed) - distinct from the MCC's keys.
__device__ __forceinline__ void emit_point(const EmitDev& e, int q, unsigned long long seed, unsigned long long inj,
                                           const double* __restrict__ uniforms, double& x, double& y, double& vx,
                                           double& vy, double& vz) {
  double u[8];
  if (uniforms) {
    const double* r = uniforms + (long long)q * 14;
    u[0] = r[0];
    u[1] = r[1];
#pragma unroll
    for (int k = 0; k < 6; k++) u[2 + k] = r[2 + 6 * e.slot + k];
  } else {
    Philox src{(uint32_t)q, 0x80000000u | (uint32_t)e.emitter, (uint32_t)inj, (uint32_t)seed,
               (uint32_t)(seed >> 32), 0, make_uint4(0, 0, 0, 0)};
    double all[14];
#pragma unroll
    for (int k = 0; k < 14; k++) all[k] = src.next();
    u[0] = all[0];
    u[1] = all[1];
#pragma unroll
    for (int k = 0; k < 6; k++) u[2 + k] = e.slot ? all[8 + k] : all[2 + k];
  }
  // uncontracted in every file (the files including this one build with and
  // without FMA contraction): ((vth sqrt2) ((u1 + u2) + u3 - 1.5)) + drift
  const double vs = __dmul_rn(e.vth, sqrt(2.0));
  vx = __dadd_rn(__dmul_rn(vs, __dsub_rn(__dadd_rn(__dadd_rn(u[2], u[3]), u[4]), 1.5)), e.vdx);
  vy = __dadd_rn(__dmul_rn(vs, __dsub_rn(__dadd_rn(__dadd_rn(u[5], u[6]), u[7]), 1.5)), e.vdy);
  vz = 0.0;
  vx /= e.vel_norm;
  vy /= e.vel_norm;
  vz /= e.vel_norm;
  x = __dadd_rn(__dmul_rn(u[0], __dsub_rn(e.x1, e.x0)), e.x0);
  y = __dadd_rn(__dmul_rn(u[1], __dsub_rn(e.y1, e.y0)), e.y0);
}

}  // namespace epic
