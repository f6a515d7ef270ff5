// Vector kernels of the CG driver: inner products of float32 vectors
// accumulated in float64 (deterministic two-pass reduction), and the fused
// CG vector updates with their scalars read from device memory, so that a CG
// iteration needs no host synchronisation and can be captured in a CUDA graph.
#include "tg_internal.cuh"

namespace tg {

constexpr int kDotBlocks = 1216;  // 152 SMs x 8
constexpr int kDotThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s[kDotThreads / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s[warp] = v;
  __syncthreads();
  v = (threadIdx.x < kDotThreads / 32) ? s[threadIdx.x] : 0.0;
  if (warp == 0) v = warp_sum(v);
  return v;
}

// partial[b] = sum over the block's grid-stride share of a[i] * b[i] (float64)
__global__ void __launch_bounds__(kDotThreads) dot_partial_kernel(const float *__restrict__ a,
                                                                   const float *__restrict__ b, long long n,
                                                                   double *__restrict__ partial) {
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n4 = n & ~3LL;
  // float4 body when both pointers are 16-byte aligned
  if ((((uintptr_t)a | (uintptr_t)b) & 15) == 0) {
    const float4 *a4 = (const float4 *)a;
    const float4 *b4 = (const float4 *)b;
    for (long long k = i; k < n4 / 4; k += stride) {
      const float4 x = __ldg(a4 + k), y = __ldg(b4 + k);
      acc += (double)x.x * y.x + (double)x.y * y.y + (double)x.z * y.z + (double)x.w * y.w;
    }
    for (long long k = n4 + i; k < n; k += stride) acc += (double)a[k] * b[k];
  } else {
    for (long long k = i; k < n; k += stride) acc += (double)a[k] * b[k];
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// out[0] = sum of partials in a fixed order (deterministic)
__global__ void __launch_bounds__(kDotThreads) dot_final_kernel(const double *__restrict__ partial, int np,
                                                                 double *__restrict__ out) {
  double acc = 0.0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) acc += partial[k];
  acc = block_sum(acc);
  if (threadIdx.x == 0) out[0] = acc;
}

cudaError_t launch_dot(const float *a, const float *b, long long n, double *partial, double *out, cudaStream_t s) {
  long long blocks = (n / 4 + kDotThreads - 1) / kDotThreads;
  if (blocks > kDotBlocks) blocks = kDotBlocks;
  if (blocks < 1) blocks = 1;
  dot_partial_kernel<<<(int)blocks, kDotThreads, 0, s>>>(a, b, n, partial);
  dot_final_kernel<<<1, kDotThreads, 0, s>>>(partial, (int)blocks, out);
  return cudaGetLastError();
}

}  // namespace tg
