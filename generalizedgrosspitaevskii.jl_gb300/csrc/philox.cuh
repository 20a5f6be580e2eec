// philox.cuh -- counter-based normal deviates for the position noise.
//
// The reference draws xi with randn! once per component per real-space half step
// (src/misc.jl:44-51, called from src/strang_splitting.jl:79).  Here xi is a pure
// function of (seed, half step, trajectory, point): Philox4x32-10 (Salmon, Moraes,
// Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11) turns the
// counter into four 32-bit words, and the Box-Muller transform turns each pair of
// words into one complex normal with E|xi|^2 = 1 (re, im ~ N(0, 1/2)), the
// distribution randn! gives for complex arrays.  Word pair (0,1) feeds component 0,
// pair (2,3) component 1.  No state is stored, so a resumed run draws the same
// numbers as an uninterrupted one.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gpe {

struct Philox4x32 {
  static constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  static constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  __host__ __device__ static inline void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
  }
  __host__ __device__ static inline uint4 gen(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      if (r > 0) { k0 += W0; k1 += W1; }
      uint32_t hi0, lo0, hi1, lo1;
      mulhilo(M0, c.x, hi0, lo0);
      mulhilo(M1, c.z, hi1, lo1);
      uint4 n;
      n.x = hi1 ^ c.y ^ k0;
      n.y = lo1;
      n.z = hi0 ^ c.w ^ k1;
      n.w = lo0;
      c = n;
    }
    return c;
  }
};

// counter for (point p, global trajectory index b, half step h): a handle holding
// trajectories b0 .. b0 + B - 1 of an ensemble (gpe_set_noise_offset) draws exactly their
// part of the whole ensemble's noise
__device__ __forceinline__ uint4 noise_counter(int64_t p, int64_t b, int64_t h) {
  return make_uint4((uint32_t)p, (uint32_t)b, (uint32_t)h, (uint32_t)((uint64_t)h >> 32));
}

// Box-Muller: (w0, w1) -> sqrt(-ln u1) * (cos 2 pi u2, sin 2 pi u2),
// u1 = (w0 + 1/2) 2^-32 in (0, 1), u2 = w1 2^-32 in [0, 1).
__device__ __forceinline__ double2 box_muller_f64(uint32_t w0, uint32_t w1) {
  const double u1 = ((double)w0 + 0.5) * 2.3283064365386963e-10;
  const double u2 = (double)w1 * 2.3283064365386963e-10;
  const double mag = sqrt(-log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  return make_double2(mag * c, mag * s);
}
// FP32 variant on the top 24 bits of each word: u1 = (w0>>8 + 1/2) 2^-24.
// FP32 fields (the truncated-Wigner bulk): the same transform with the hardware
// approximations of log and sin/cos (absolute error near 2^-21), a few instructions
// instead of the accurate routines' range reduction.  The angle is taken in [-pi, pi),
// where the approximation holds: (cos, sin)(2 pi u2) = -(cos, sin)(pi (2 u2 - 1)).  The
// draws are Gaussian to that accuracy; they are not meant to repeat the FP64 variant
// bit for bit.
__device__ __forceinline__ float2 box_muller_f32(uint32_t w0, uint32_t w1) {
  const float u1 = ((float)(w0 >> 8) + 0.5f) * 5.9604644775390625e-8f;
  const float u2 = (float)(w1 >> 8) * 5.9604644775390625e-8f;
  const float mag = sqrtf(fmaxf(-__logf(u1), 0.0f));  // the approximation may cross 0 near u1 = 1
  float s, c;
  __sincosf(3.14159265358979f * (2.0f * u2 - 1.0f), &s, &c);
  return make_float2(-mag * c, -mag * s);
}

template <typename Real> struct BoxMuller;
template <> struct BoxMuller<double> {
  __device__ static __forceinline__ double2 get(uint32_t a, uint32_t b) { return box_muller_f64(a, b); }
};
template <> struct BoxMuller<float> {
  __device__ static __forceinline__ float2 get(uint32_t a, uint32_t b) { return box_muller_f32(a, b); }
};

}  // namespace gpe
