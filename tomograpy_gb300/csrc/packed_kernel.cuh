// The packed multi-job kernel and its job record, shared by the translation
// units that instantiate it (packed.cu: the default schedule and the
// deterministic backprojection; packed_tuned.cu: the other schedules the
// autotuner may pick).
#pragma once

#include "det_common.cuh"

namespace tg {

struct PackedJob {
  Geometry G;
  float *data;
  float *cube;
  long long tile0;      // first CTA tile of this job
  int gx, gy;           // column / row tiles per view
  // deterministic backprojection: the job's part of the workspace (byte
  // offset: DetScale, then its int64 accumulator at +256), the accumulator's
  // dense strides, and the ray count and voxel diagonal behind its scale
  long long ws_off;
  long long acc_ms[4];
  double rays, lmax;
};

// LMAJ / BATCH: the tile schedule (lanes along lambda or gamma, steps per
// batch; see tile_body); the plan's tile counts gx, gy follow the same
// schedule.
#ifndef TG_PACKED_PJ_MIN_BLOCKS
#define TG_PACKED_PJ_MIN_BLOCKS TG_PJ_MIN_BLOCKS
#endif
// CTAs per SM the packed kernel's register budget allows (its job record and
// schedule state make it heavier than the single-job kernel)
__host__ __device__ constexpr int packed_min_blocks(int mode) {
  return is_backprojection(mode) ? TG_BPJ_MIN_BLOCKS : TG_PACKED_PJ_MIN_BLOCKS;
}

template <int MODE, bool SUN, typename IDX, int RPW, bool DET, bool LMAJ = true, int BATCH = 0>
__global__ void __launch_bounds__(kThreads, packed_min_blocks(MODE))
    packed_kernel(const long long *__restrict__ tile0, const PackedJob *__restrict__ jobs, int n_jobs,
                  unsigned char *__restrict__ ws) {
  static_assert(sizeof(PackedJob) % 4 == 0, "job record copied as 32-bit words");
  __shared__ int s_job;
  __shared__ __align__(16) int s_rec[sizeof(PackedJob) / 4];
  if (threadIdx.x == 0) {
    const long long b = blockIdx.x;
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {  // last job whose first tile is <= b
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(tile0 + mid) <= b) lo = mid;
      else hi = mid - 1;
    }
    s_job = lo;
  }
  __syncthreads();
  const int *src = reinterpret_cast<const int *>(jobs + s_job);
  for (int k = threadIdx.x; k < (int)(sizeof(PackedJob) / 4); k += blockDim.x) s_rec[k] = __ldg(src + k);
  __syncthreads();
  PackedJob &J = *reinterpret_cast<PackedJob *>(s_rec);
  if (DET) {  // the walk indexes the job's dense accumulator instead of its cube
    if (threadIdx.x < 4) J.G.ms[threadIdx.x] = J.acc_ms[threadIdx.x];
    __syncthreads();
  }
  long long local = (long long)blockIdx.x - J.tile0;
  const int bx = (int)(local % J.gx);
  local /= J.gx;
  const int by = (int)(local % J.gy);
  const int t = (int)(local / J.gy);
  if (t >= J.G.n_views) return;  // a tile count beyond the plan's (whole CTA)
  constexpr bool PJ = (MODE == TG_PJ || MODE == TG_PJT);
  unsigned long long *acc = DET ? reinterpret_cast<unsigned long long *>(ws + J.ws_off + 256) : nullptr;
  const DetScale *dsc = DET ? reinterpret_cast<const DetScale *>(ws + J.ws_off) : nullptr;
  const int col0 = LMAJ ? bx * 32 : bx * (RPW * kRows);
  const int row0 = LMAJ ? by * (RPW * kRows) : by * 32;
  tile_body<MODE, SUN, IDX, DET, RPW, LMAJ, BATCH>(J.G, t, col0, row0, PJ ? J.cube : J.data, PJ ? J.data : J.cube,
                                                   acc, dsc);
}

// byte offset of the job records in a plan of n_jobs jobs
inline size_t packed_records_offset_of(int n_jobs) {
  return ((size_t)n_jobs * sizeof(long long) + 255) & ~(size_t)255;
}

}  // namespace tg
