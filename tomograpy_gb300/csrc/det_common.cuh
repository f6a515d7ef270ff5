// Pieces of the deterministic (64-bit fixed-point) backprojection shared by
// the single-job entry point (deterministic.cu) and the packed multi-job one
// (packed.cu), so that a job's cube is bitwise the same through either.
//
// Per job: the largest |y| over the traced pixels sets a power-of-two input
// scale, the ray count and the voxel diagonal bound every voxel sum so that it
// stays below 2^61 in magnitude, every segment L*y is added as an integer
// multiple of 2^-s with red.add.u64 (order-independent), and a final pass adds
// the scaled integers into the caller's cube.
#pragma once

#include "siddon_fast.cuh"

namespace tg {

// max |y| over the unmasked pixels of views [G.view0, G.view0 + n_views),
// elements first, first + stride, ... of the flattened (view, row, column)
// range; the warp's maximum is folded into dsc->ymax_bits.
__device__ __forceinline__ void det_prepass_range(const Geometry &G, const float *__restrict__ data, int n_views,
                                                  DetScale *__restrict__ dsc, long long first, long long stride) {
  const long long total = (long long)G.n1 * G.n2 * n_views;
  float m = 0.f;
  for (long long p = first; p < total; p += stride) {
    const int j = (int)(p % G.n2);
    const long long r = p / G.n2;
    const int i = (int)(r % G.n1);
    const int t = G.view0 + (int)(r / G.n1);
    if (masked(G, i, j, t)) continue;
    const float v = fabsf(data[(long long)i * G.ds[0] + (long long)j * G.ds[1] + (long long)t * G.ds[2]]);
    m = fmaxf(m, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(&dsc->ymax_bits, __float_as_uint(m));
}

// Scale factors from max |y|: yscale = 2^-e brings max |y| into [0.5, 1),
// qscale = 2^s with s = floor(61 - log2(rays * lmax)).
__device__ __forceinline__ void det_scale(DetScale *dsc, double rays, double lmax) {
  const float ymax = __uint_as_float(dsc->ymax_bits);
  int e = 0;
  if (ymax > 0.f && isfinite(ymax)) frexpf(ymax, &e);
  const double bound = fmax(rays * lmax, 1e-30);
  int s = (int)floor(61.0 - log2(bound));
  s = max(-100, min(100, s));
  dsc->yscale = ldexpf(1.f, -e);
  dsc->qscale = ldexpf(1.f, s);
  dsc->out_scale = ldexp(1.0, e - s);
}

// map += out_scale * acc over accumulator elements first, first + stride, ...
// (acc dense C order, frame-major (F, n0, n1, n2); map with G's strides).
__device__ __forceinline__ void det_finalize_range(const Geometry &G, const long long *__restrict__ acc,
                                                   const DetScale *__restrict__ dsc, float *__restrict__ map,
                                                   long long first, long long stride) {
  const long long nvox = (long long)G.n[0] * G.n[1] * G.n[2];
  const long long total = nvox * G.nframes;
  const double sc = dsc->out_scale;
  for (long long p = first; p < total; p += stride) {
    const long long q = acc[p];
    if (q == 0) continue;
    const long long f = p / nvox;
    long long r = p - f * nvox;
    const int z = (int)(r % G.n[2]);
    r /= G.n[2];
    const int y = (int)(r % G.n[1]);
    const int x = (int)(r / G.n[1]);
    const long long o = (long long)x * G.ms[0] + (long long)y * G.ms[1] + (long long)z * G.ms[2] + f * G.ms[3];
    map[o] += (float)((double)q * sc);
  }
}

// Host: the voxel diagonal (the longest segment one voxel can hold).
inline double det_lmax(const Geometry &G) {
  double l2 = 0.0;
  for (int k = 0; k < 3; ++k) l2 += G.mh.cdelt[k] * G.mh.cdelt[k];
  return sqrt(l2);
}

// Dense accumulator strides (C order within a frame, frames outermost).
inline void det_acc_strides(const Geometry &G, long long ms[4]) {
  ms[2] = 1;
  ms[1] = G.n[2];
  ms[0] = (long long)G.n[1] * G.n[2];
  ms[3] = (long long)G.n[0] * G.n[1] * G.n[2];
}

}  // namespace tg
