// Deterministic backprojection: 64-bit fixed-point accumulation.
//
// The float atomics of the fast backprojector (like the reference's OpenMP
// atomics, tomograpy/C_siddon.c.template:926,942) sum in whatever order the
// rays run, so results vary in the last bits from run to run.  Here every
// segment contribution L*y is converted to an integer multiple of a power of
// two and added with red.add.u64; integer addition is associative, so the
// cube is bitwise reproducible.  The scale is chosen on the device from
// max|y|: with yscale = 2^-e bringing max|y| into [0.5, 1) and
// qscale = 2^s, s = floor(61 - log2(R * Lmax)) (R rays, Lmax the voxel
// diagonal), no voxel sum can exceed 2^61 in magnitude.
//
// Workspace layout (256-byte aligned): [DetScale | pad to 256 B |
// int64 accumulator, dense C order (F, n0, n1, n2)].
#include "siddon_fast.cuh"

namespace tg {

__global__ void det_prepass_kernel(const Geometry G, const float *__restrict__ data, int n_views,
                                   DetScale *__restrict__ dsc) {
  const long long total = (long long)G.n1 * G.n2 * n_views;
  float m = 0.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
       p += (long long)gridDim.x * blockDim.x) {
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

__global__ void det_scale_kernel(DetScale *dsc, double rays, double lmax) {
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

__global__ void det_finalize_kernel(const Geometry G, const long long *__restrict__ acc,
                                    const DetScale *__restrict__ dsc, float *__restrict__ map) {
  const long long nvox = (long long)G.n[0] * G.n[1] * G.n[2];
  const long long total = nvox * G.nframes;
  const double sc = dsc->out_scale;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
       p += (long long)gridDim.x * blockDim.x) {
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

cudaError_t launch_deterministic_bpj(const Geometry &G, int mode, int obstacle, bool idx64, const float *data,
                                     float *map, void *workspace, int gx, int gy, int gz, cudaStream_t s) {
  const bool sun = obstacle == TG_OBSTACLE_SUN;
  DetScale *dsc = (DetScale *)workspace;
  long long *acc = (long long *)((char *)workspace + 256);
  const long long nvox = (long long)G.n[0] * G.n[1] * G.n[2];
  const size_t acc_bytes = (size_t)(nvox * G.nframes) * sizeof(long long);
  cudaError_t e = cudaMemsetAsync(workspace, 0, 256 + acc_bytes, s);
  if (e != cudaSuccess) return e;
  // max |y| over the traced pixels
  const long long total = (long long)G.n1 * G.n2 * gz;
  int pblocks = (int)((total + 255) / 256);
  if (pblocks > 152 * 16) pblocks = 152 * 16;
  if (pblocks < 1) pblocks = 1;
  det_prepass_kernel<<<pblocks, 256, 0, s>>>(G, data, gz, dsc);
  double lmax = 0.0;
  for (int k = 0; k < 3; ++k) lmax += G.mh.cdelt[k] * G.mh.cdelt[k];
  lmax = sqrt(lmax);
  det_scale_kernel<<<1, 1, 0, s>>>(dsc, (double)total, lmax);
  // walk with accumulator strides (dense C order, frame-major)
  Geometry A = G;
  A.ms[2] = 1;
  A.ms[1] = G.n[2];
  A.ms[0] = (long long)G.n[1] * G.n[2];
  A.ms[3] = nvox;
  const dim3 grid(gx, gy, gz);
  unsigned long long *a64 = (unsigned long long *)acc;
  const bool t4 = (mode == TG_BPJT);
  if (idx64) {
    if (t4) {
      if (sun) fast_kernel<TG_BPJT, true, long long, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
      else fast_kernel<TG_BPJT, false, long long, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
    } else {
      if (sun) fast_kernel<TG_BPJ, true, long long, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
      else fast_kernel<TG_BPJ, false, long long, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
    }
  } else {
    if (t4) {
      if (sun) fast_kernel<TG_BPJT, true, int, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
      else fast_kernel<TG_BPJT, false, int, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
    } else {
      if (sun) fast_kernel<TG_BPJ, true, int, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
      else fast_kernel<TG_BPJ, false, int, true><<<grid, kThreads, 0, s>>>(A, data, nullptr, a64, dsc);
    }
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int fblocks = (int)((nvox * G.nframes + 255) / 256);
  if (fblocks > 152 * 32) fblocks = 152 * 32;
  if (fblocks < 1) fblocks = 1;
  det_finalize_kernel<<<fblocks, 256, 0, s>>>(G, acc, dsc, map);
  return cudaGetLastError();
}

}  // namespace tg
