// Packed multi-job launches: many independent reconstructions (each with its
// own cube size, view count, image size and geometry) traced by ONE kernel
// launch, and the per-job (segmented) vector kernels of a batched CG.
//
// A plan is a device buffer holding the first CTA tile of every job (int64,
// ascending) followed by one PackedJob record per job (the job's kernel
// Geometry and its data / cube pointers), sorted by decreasing work.  A CTA
// finds its job by binary search on the compact tile array, copies the job's
// record into shared memory and runs the same tile body as the single-job
// kernel.
#include "packed_kernel.cuh"

namespace tg {

template <int MODE, typename IDX, int RPW, bool DET>
static void launch_packed_rpw(const long long *tile0, const PackedJob *jobs, int n_jobs, long long tiles, bool sun,
                              unsigned char *ws, cudaStream_t s) {
  if (sun) packed_kernel<MODE, true, IDX, RPW, DET><<<(unsigned)tiles, kThreads, 0, s>>>(tile0, jobs, n_jobs, ws);
  else packed_kernel<MODE, false, IDX, RPW, DET><<<(unsigned)tiles, kThreads, 0, s>>>(tile0, jobs, n_jobs, ws);
}

template <int MODE, typename IDX, bool DET = false>
static void launch_packed_mode(const long long *tile0, const PackedJob *jobs, int n_jobs, long long tiles, int rpw,
                               bool sun, cudaStream_t s, unsigned char *ws = nullptr) {
  if (rpw == 1) launch_packed_rpw<MODE, IDX, 1, DET>(tile0, jobs, n_jobs, tiles, sun, ws, s);
  else if (rpw == 2) launch_packed_rpw<MODE, IDX, 2, DET>(tile0, jobs, n_jobs, tiles, sun, ws, s);
  else launch_packed_rpw<MODE, IDX, 4, DET>(tile0, jobs, n_jobs, tiles, sun, ws, s);
}

// Deterministic packed backprojection, per job (blockIdx.y): max |y|, scale,
// and the final scaled add of the accumulator into the job's cube.
constexpr int kDetBlocks = 64;  // blocks per job of the prepass / finalize

__global__ void packed_det_prepass(const PackedJob *__restrict__ jobs, unsigned char *__restrict__ ws) {
  const PackedJob &J = jobs[blockIdx.y];
  det_prepass_range(J.G, J.data, J.G.n_views, reinterpret_cast<DetScale *>(ws + J.ws_off),
                    blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

__global__ void packed_det_scale(const PackedJob *__restrict__ jobs, int n_jobs, unsigned char *__restrict__ ws) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_jobs) return;
  const PackedJob &J = jobs[k];
  det_scale(reinterpret_cast<DetScale *>(ws + J.ws_off), J.rays, J.lmax);
}

__global__ void packed_det_finalize(const PackedJob *__restrict__ jobs, unsigned char *__restrict__ ws) {
  const PackedJob &J = jobs[blockIdx.y];
  det_finalize_range(J.G, reinterpret_cast<const long long *>(ws + J.ws_off + 256),
                     reinterpret_cast<const DetScale *>(ws + J.ws_off), J.cube,
                     blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

size_t packed_records_offset(int n_jobs) { return packed_records_offset_of(n_jobs); }

cudaError_t launch_packed(const void *plan, int n_jobs, long long tiles, int rpw, bool idx64, int mode, int obstacle,
                          int lane_axis, int batch, cudaStream_t s) {
  const long long *tile0 = (const long long *)plan;
  const PackedJob *jobs = (const PackedJob *)((const unsigned char *)plan + packed_records_offset(n_jobs));
  const bool sun = obstacle == TG_OBSTACLE_SUN;
  if (lane_axis != 1 || batch != 0)  // the plan builder keeps 64-bit plans on the default schedule
    return launch_packed_tuned(tile0, jobs, n_jobs, tiles, rpw, mode, sun, lane_axis, batch, s);
  if (idx64) {
    switch (mode) {
    case TG_PJ: launch_packed_mode<TG_PJ, long long>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    case TG_BPJ: launch_packed_mode<TG_BPJ, long long>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    case TG_PJT: launch_packed_mode<TG_PJT, long long>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    default: launch_packed_mode<TG_BPJT, long long>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    }
  } else {
    switch (mode) {
    case TG_PJ: launch_packed_mode<TG_PJ, int>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    case TG_BPJ: launch_packed_mode<TG_BPJ, int>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    case TG_PJT: launch_packed_mode<TG_PJT, int>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    default: launch_packed_mode<TG_BPJT, int>(tile0, jobs, n_jobs, tiles, rpw, sun, s); break;
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_packed_det(const void *plan, int n_jobs, long long tiles, int rpw, bool idx64, bool four_d,
                              int obstacle, void *workspace, size_t ws_bytes, cudaStream_t s) {
  const long long *tile0 = (const long long *)plan;
  const PackedJob *jobs = (const PackedJob *)((const unsigned char *)plan + packed_records_offset(n_jobs));
  unsigned char *ws = (unsigned char *)workspace;
  const bool sun = obstacle == TG_OBSTACLE_SUN;
  cudaError_t e = cudaMemsetAsync(workspace, 0, ws_bytes, s);
  if (e != cudaSuccess) return e;
  packed_det_prepass<<<dim3(kDetBlocks, n_jobs), 256, 0, s>>>(jobs, ws);
  packed_det_scale<<<(n_jobs + 127) / 128, 128, 0, s>>>(jobs, n_jobs, ws);
  if (idx64) {
    if (four_d) launch_packed_mode<TG_BPJT, long long, true>(tile0, jobs, n_jobs, tiles, rpw, sun, s, ws);
    else launch_packed_mode<TG_BPJ, long long, true>(tile0, jobs, n_jobs, tiles, rpw, sun, s, ws);
  } else {
    if (four_d) launch_packed_mode<TG_BPJT, int, true>(tile0, jobs, n_jobs, tiles, rpw, sun, s, ws);
    else launch_packed_mode<TG_BPJ, int, true>(tile0, jobs, n_jobs, tiles, rpw, sun, s, ws);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  packed_det_finalize<<<dim3(kDetBlocks, n_jobs), 256, 0, s>>>(jobs, ws);
  return cudaGetLastError();
}

size_t packed_job_bytes() { return sizeof(PackedJob); }

void packed_fill(void *dst, const Geometry &G, float *data, float *cube, long long tile0, int gx, int gy,
                 long long ws_off) {
  PackedJob *J = (PackedJob *)dst;
  J->G = G;
  J->data = data;
  J->cube = cube;
  J->tile0 = tile0;
  J->gx = gx;
  J->gy = gy;
  J->ws_off = ws_off;
  det_acc_strides(G, J->acc_ms);
  J->rays = (double)G.n1 * G.n2 * G.n_views;
  J->lmax = det_lmax(G);
}

// ---------------------------------------------------------------------------
// segmented vector kernels of the batched CG: segment s = [seg[2s], seg[2s+1])

constexpr int kSegBlocks = 32;  // blocks per segment
constexpr int kSegThreads = 256;

__device__ __forceinline__ double seg_block_sum(double v) {
  __shared__ double sh[kSegThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  v = (threadIdx.x < kSegThreads / 32) ? sh[threadIdx.x] : 0.0;
  if (warp == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v;
}

// partial[s * kSegBlocks + b] = block b's share of <a, b>_s (float64)
__global__ void __launch_bounds__(kSegThreads) seg_dot_partial(const float *__restrict__ a,
                                                               const float *__restrict__ b,
                                                               const long long *__restrict__ off,
                                                               double *__restrict__ partial) {
  const int s = blockIdx.y;
  const long long lo = off[2 * s], hi = off[2 * s + 1];
  double acc = 0.0;
  for (long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += (long long)gridDim.x * blockDim.x)
    acc += (double)a[i] * b[i];
  acc = seg_block_sum(acc);
  if (threadIdx.x == 0) partial[s * kSegBlocks + blockIdx.x] = acc;
}

// out[s] = sum of segment s's partials in block order (deterministic)
__global__ void seg_dot_final(const double *__restrict__ partial, int n_seg, double *__restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_seg) return;
  double acc = 0.0;
  for (int b = 0; b < kSegBlocks; ++b) acc += partial[s * kSegBlocks + b];
  out[s] = acc;
}

// x += alpha_s p, r -= alpha_s Ap with alpha_s = rr_s / pAp_s
__global__ void __launch_bounds__(kSegThreads) seg_cg_x(float *__restrict__ x, float *__restrict__ r,
                                                        const float *__restrict__ p, const float *__restrict__ Ap,
                                                        const double *__restrict__ rr,
                                                        const double *__restrict__ pAp,
                                                        const long long *__restrict__ off) {
  const int s = blockIdx.y;
  const double den = pAp[s];
  const float alpha = (den != 0.0) ? (float)(rr[s] / den) : 0.f;
  const long long lo = off[2 * s], hi = off[2 * s + 1];
  for (long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += (long long)gridDim.x * blockDim.x) {
    x[i] = fmaf(alpha, p[i], x[i]);
    r[i] = fmaf(-alpha, Ap[i], r[i]);
  }
}

// p = r + beta_s p with beta_s = rr_new_s / rr_s
__global__ void __launch_bounds__(kSegThreads) seg_cg_p(float *__restrict__ p, const float *__restrict__ r,
                                                        const double *__restrict__ rr,
                                                        const double *__restrict__ rr_new,
                                                        const long long *__restrict__ off) {
  const int s = blockIdx.y;
  const double den = rr[s];
  const float beta = (den != 0.0) ? (float)(rr_new[s] / den) : 0.f;
  const long long lo = off[2 * s], hi = off[2 * s + 1];
  for (long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = fmaf(beta, p[i], r[i]);
}

// y[i] = alpha * x[i] + beta * y[i] over the segments (beta = 0: y = alpha x)
__global__ void __launch_bounds__(kSegThreads) seg_axpby(float *__restrict__ y, const float *__restrict__ x, float alpha,
                                                         float beta, const long long *__restrict__ off) {
  const int s = blockIdx.y;
  const long long lo = off[2 * s], hi = off[2 * s + 1];
  for (long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hi;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = (beta == 0.f) ? (x ? alpha * x[i] : 0.f) : fmaf(alpha, x ? x[i] : 0.f, beta * y[i]);
}

cudaError_t launch_seg_axpby(float *y, const float *x, float alpha, float beta, const long long *off, int n_seg,
                             cudaStream_t st) {
  seg_axpby<<<dim3(kSegBlocks, n_seg), kSegThreads, 0, st>>>(y, x, alpha, beta, off);
  return cudaGetLastError();
}

__global__ void seg_copy(double *__restrict__ dst, const double *__restrict__ src, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) dst[s] = src[s];
}

cudaError_t launch_seg_dot(const float *a, const float *b, const long long *off, int n_seg, double *partial,
                           double *out, cudaStream_t st) {
  seg_dot_partial<<<dim3(kSegBlocks, n_seg), kSegThreads, 0, st>>>(a, b, off, partial);
  seg_dot_final<<<(n_seg + 127) / 128, 128, 0, st>>>(partial, n_seg, out);
  return cudaGetLastError();
}

cudaError_t launch_seg_cg_x(float *x, float *r, const float *p, const float *Ap, const double *rr, const double *pAp,
                            const long long *off, int n_seg, cudaStream_t st) {
  seg_cg_x<<<dim3(kSegBlocks, n_seg), kSegThreads, 0, st>>>(x, r, p, Ap, rr, pAp, off);
  return cudaGetLastError();
}

cudaError_t launch_seg_cg_p(float *p, const float *r, double *rr, const double *rr_new, const long long *off,
                            int n_seg, cudaStream_t st) {
  seg_cg_p<<<dim3(kSegBlocks, n_seg), kSegThreads, 0, st>>>(p, r, rr, rr_new, off);
  seg_copy<<<(n_seg + 127) / 128, 128, 0, st>>>(rr, rr_new, n_seg);
  return cudaGetLastError();
}

size_t seg_workspace_bytes(int n_seg) { return (size_t)n_seg * kSegBlocks * sizeof(double); }

}  // namespace tg
