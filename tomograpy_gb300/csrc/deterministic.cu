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
#include "det_common.cuh"

namespace tg {

__global__ void det_prepass_kernel(const Geometry G, const float *__restrict__ data, int n_views,
                                   DetScale *__restrict__ dsc) {
  det_prepass_range(G, data, n_views, dsc, blockIdx.x * (long long)blockDim.x + threadIdx.x,
                    (long long)gridDim.x * blockDim.x);
}

__global__ void det_scale_kernel(DetScale *dsc, double rays, double lmax) { det_scale(dsc, rays, lmax); }

__global__ void det_finalize_kernel(const Geometry G, const long long *__restrict__ acc,
                                    const DetScale *__restrict__ dsc, float *__restrict__ map) {
  det_finalize_range(G, acc, dsc, map, blockIdx.x * (long long)blockDim.x + threadIdx.x,
                     (long long)gridDim.x * blockDim.x);
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
  det_scale_kernel<<<1, 1, 0, s>>>(dsc, (double)total, det_lmax(G));
  // walk with accumulator strides (dense C order, frame-major)
  Geometry A = G;
  det_acc_strides(G, A.ms);
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
