// The packed kernel under the non-default tile schedules the autotuner
// (tomograpy_gb300/batch.py) may pick: lanes along image axis 0 (gamma)
// and / or 16-step batches, for 32-bit cube offsets.  A separate
// translation unit so that the library's parallel build stays short.
#include "packed_kernel.cuh"

namespace tg {

template <int MODE, int RPW, bool LMAJ, int BATCH>
static void launch_one(const long long *tile0, const PackedJob *jobs, int n_jobs, long long tiles, bool sun,
                       cudaStream_t s) {
  if (sun)
    packed_kernel<MODE, true, int, RPW, false, LMAJ, BATCH><<<(unsigned)tiles, kThreads, 0, s>>>(tile0, jobs, n_jobs,
                                                                                                  nullptr);
  else
    packed_kernel<MODE, false, int, RPW, false, LMAJ, BATCH><<<(unsigned)tiles, kThreads, 0, s>>>(tile0, jobs, n_jobs,
                                                                                                   nullptr);
}

template <int MODE, bool LMAJ, int BATCH>
static void launch_rpw(const long long *tile0, const PackedJob *jobs, int n_jobs, long long tiles, int rpw, bool sun,
                       cudaStream_t s) {
  if (rpw == 1) launch_one<MODE, 1, LMAJ, BATCH>(tile0, jobs, n_jobs, tiles, sun, s);
  else if (rpw == 2) launch_one<MODE, 2, LMAJ, BATCH>(tile0, jobs, n_jobs, tiles, sun, s);
  else launch_one<MODE, 4, LMAJ, BATCH>(tile0, jobs, n_jobs, tiles, sun, s);
}

template <int MODE>
static void launch_sched(const long long *tile0, const PackedJob *jobs, int n_jobs, long long tiles, int rpw, bool sun,
                         int lane_axis, int batch, cudaStream_t s) {
  if (lane_axis == 1) launch_rpw<MODE, true, 16>(tile0, jobs, n_jobs, tiles, rpw, sun, s);
  else if (batch == 0) launch_rpw<MODE, false, 0>(tile0, jobs, n_jobs, tiles, rpw, sun, s);
  else launch_rpw<MODE, false, 16>(tile0, jobs, n_jobs, tiles, rpw, sun, s);
}

cudaError_t launch_packed_tuned(const long long *tile0, const PackedJob *jobs, int n_jobs, long long tiles, int rpw,
                                int mode, bool sun, int lane_axis, int batch, cudaStream_t s) {
  switch (mode) {
  case TG_PJ: launch_sched<TG_PJ>(tile0, jobs, n_jobs, tiles, rpw, sun, lane_axis, batch, s); break;
  case TG_BPJ: launch_sched<TG_BPJ>(tile0, jobs, n_jobs, tiles, rpw, sun, lane_axis, batch, s); break;
  case TG_PJT: launch_sched<TG_PJT>(tile0, jobs, n_jobs, tiles, rpw, sun, lane_axis, batch, s); break;
  default: launch_sched<TG_BPJT>(tile0, jobs, n_jobs, tiles, rpw, sun, lane_axis, batch, s); break;
  }
  return cudaGetLastError();
}

}  // namespace tg
