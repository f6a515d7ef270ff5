// Instantiation and launch of the fast single-precision kernels
// (pj / bpj / pjt / bpjt x obstacle none / sun x 32- / 64-bit cube offsets).
#include "siddon_fast.cuh"

namespace tg {

template <int MODE, typename IDX, int BATCH = 0>
static void launch_mode(const Geometry &G, bool sun, const float *xin, float *xout, dim3 grid, cudaStream_t s) {
  if (sun) fast_kernel<MODE, true, IDX, false, BATCH><<<grid, kThreads, 0, s>>>(G, xin, xout, nullptr, nullptr);
  else fast_kernel<MODE, false, IDX, false, BATCH><<<grid, kThreads, 0, s>>>(G, xin, xout, nullptr, nullptr);
}

// projections over fine cubes take the longer batches
template <int MODE, typename IDX>
static void launch_pj(const Geometry &G, bool sun, const float *xin, float *xout, dim3 grid, cudaStream_t s) {
  if (fine_projection(G)) launch_mode<MODE, IDX, TG_PJ_FINE_BATCH>(G, sun, xin, xout, grid, s);
  else launch_mode<MODE, IDX>(G, sun, xin, xout, grid, s);
}

template <typename IDX>
static void launch_idx(const Geometry &G, int mode, bool sun, float *data, float *map, dim3 grid,
                       cudaStream_t s) {
  switch (mode) {
  case TG_PJ: launch_pj<TG_PJ, IDX>(G, sun, map, data, grid, s); break;
  case TG_BPJ: launch_mode<TG_BPJ, IDX>(G, sun, data, map, grid, s); break;
  case TG_PJT: launch_pj<TG_PJT, IDX>(G, sun, map, data, grid, s); break;
  default: launch_mode<TG_BPJT, IDX>(G, sun, data, map, grid, s); break;
  }
}

cudaError_t launch_count_f32(const Geometry &G, int obstacle, bool idx64, float *counts, int gx, int gy, int gz,
                             cudaStream_t s) {
  const dim3 grid(gx, gy, gz);
  const bool sun = obstacle == TG_OBSTACLE_SUN;
  if (idx64) {
    if (sun) fast_kernel<kModeCount, true, long long, false><<<grid, kThreads, 0, s>>>(G, nullptr, counts, nullptr, nullptr);
    else fast_kernel<kModeCount, false, long long, false><<<grid, kThreads, 0, s>>>(G, nullptr, counts, nullptr, nullptr);
  } else {
    if (sun) fast_kernel<kModeCount, true, int, false><<<grid, kThreads, 0, s>>>(G, nullptr, counts, nullptr, nullptr);
    else fast_kernel<kModeCount, false, int, false><<<grid, kThreads, 0, s>>>(G, nullptr, counts, nullptr, nullptr);
  }
  return cudaGetLastError();
}

cudaError_t launch_fast_f32(const Geometry &G, int mode, int obstacle, bool idx64, float *data, float *map,
                            int gx, int gy, int gz, cudaStream_t s) {
  const dim3 grid(gx, gy, gz);
  const bool sun = obstacle == TG_OBSTACLE_SUN;
  if (idx64) launch_idx<long long>(G, mode, sun, data, map, grid, s);
  else launch_idx<int>(G, mode, sun, data, map, grid, s);
  return cudaGetLastError();
}

}  // namespace tg
