// Double-precision projector that follows the reference's arithmetic step by
// step, and the unit-vector / intersection-parameter diagnostics.
//
// This translation unit is compiled with --fmad=false: the reference is
// built without FMA contraction, and every expression below is evaluated in
// the reference's order, so with the same ray direction the f64 GPU path
// reproduces the reference's double-precision results (differences come only
// from the last bits of CUDA's sin / cos versus the host libm).
//
//   conic_image_projector  tomograpy/C_siddon.c.template:500-528
//   ray_projector          :530-580
//   voxel (merge step)     :811-912
//   pj / bpj / pjt / bpjt  :914-944
//   in_map / sun           :947-961
#include "siddon_geom.cuh"

namespace tg {

template <int MODE, bool SUN>
__global__ void __launch_bounds__(kThreads)
ref64_kernel(const Geometry G, const double *__restrict__ xin, double *__restrict__ xout) {
  constexpr bool PJ = (MODE == TG_PJ || MODE == TG_PJT);
  constexpr bool T4 = (MODE == TG_PJT || MODE == TG_BPJT);
  __shared__ TrigTables T;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = G.view0 + blockIdx.z;
  const tg_image_header &V = G.views[t];
  const int col0 = (G.bx0 + blockIdx.x) * 32, row0 = (G.by0 + blockIdx.y) * kRows;
  fill_trig(T, V, col0, row0);
  __syncthreads();
  const int i = row0 + warp, j = col0 + lane;
  if (i >= G.n1 || j >= G.n2) return;
  if (G.ray_i >= 0 && (i != G.ray_i || j != G.ray_j)) return;
  if (masked(G, i, j, t)) return;
  long long fbase = 0;
  if (T4) {
    const int f = V.frame;
    if (f < 0 || f >= G.nframes) return;
    fbase = (long long)f * G.ms[3];
  }
  const long long po = (long long)i * G.ds[0] + (long long)j * G.ds[1] + (long long)t * G.ds[2];
  const double M[3] = {V.M[0], V.M[1], V.M[2]};
  double u[3];
  ray_direction(T.cl[lane], T.sl[lane], T.cg[warp], T.sg[warp], V.R, u);
  RefWalk w;
  if (!ref_setup(G.mh, G.n, M, u, w)) return;
  const double *cin = PJ ? xin + fbase : nullptr;
  double *cout = PJ ? nullptr : xout + fbase;
  double acc = PJ ? xout[po] : 0.0;
  const double yv = PJ ? 0.0 : xin[po];
  bool touched = false;
  double ac = w.amin;
  int guard = G.n[0] + G.n[1] + G.n[2] + 8;
  while (guard-- > 0) {
    if (!(w.iv[0] >= 0 && w.iv[0] < G.n[0] && w.iv[1] >= 0 && w.iv[1] < G.n[1] && w.iv[2] >= 0 &&
          w.iv[2] < G.n[2]))
      break;
    if (SUN && !ref_outside_sun(M, u, ac)) break;
    double dmin = w.D[0];
    if (w.D[1] < dmin) dmin = w.D[1];
    if (w.D[2] < dmin) dmin = w.D[2];
    if (dmin != dmin) break;
    ac = __dadd_rn(ac, dmin);
    const long long off =
        (long long)w.iv[0] * G.ms[0] + (long long)w.iv[1] * G.ms[1] + (long long)w.iv[2] * G.ms[2];
    if (PJ) {
      acc = __dadd_rn(acc, __dmul_rn(dmin, cin[off]));
      touched = true;
    } else {
      atomicAdd(cout + off, __dmul_rn(dmin, yv));
    }
    bool hit[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) hit[k] = (w.D[k] == dmin);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (hit[k]) {
        w.iv[k] += w.upd[k];
        w.D[k] = w.pabs[k];
      } else {
        w.D[k] = __dsub_rn(w.D[k], dmin);
      }
    }
  }
  if (PJ && touched) xout[po] = acc;
}

// Unit vectors of the pixel rays in the arithmetic of C type CT (float or
// double): angles and rotation in CT, cosines / sines in double
// (tomograpy/C_siddon.c.template:618-648,1013-1046).  NaN data pixels are left
// untouched.
template <typename CT>
__device__ __forceinline__ void ct_direction(const tg_image_header &V, int i, int j, CT u0[3]) {
  const CT s0 = (CT)V.crpix[0], p0 = (CT)V.cdelt[0], v0 = (CT)V.crval[0];
  const CT s1 = (CT)V.crpix[1], p1 = (CT)V.cdelt[1], v1 = (CT)V.crval[1];
  const CT gam = ((CT)(unsigned int)i - s0 + (CT)1) * p0 + v0;
  const CT lam = ((CT)(unsigned int)j - s1 + (CT)1) * p1 + v1;
  CT u2[3];
  u2[0] = (CT)(cos((double)lam) * cos((double)gam));
  u2[1] = (CT)(cos((double)lam) * sin((double)gam));
  u2[2] = (CT)sin((double)lam);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    u0[k] = (CT)V.R[3 * k] * u2[0] + (CT)V.R[3 * k + 1] * u2[1] + (CT)V.R[3 * k + 2] * u2[2];
}

template <typename CT>
__global__ void unit_vector_kernel(const Geometry G, const CT *__restrict__ data, double *__restrict__ u,
                                   long long us0, long long us1, long long us2, long long us3) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  const int t = G.view0 + blockIdx.z;
  if (i >= G.n1 || j >= G.n2) return;
  const CT v = data[(long long)i * G.ds[0] + (long long)j * G.ds[1] + (long long)t * G.ds[2]];
  if (v != v) return;
  CT u0[3];
  ct_direction<CT>(G.views[t], i, j, u0);
  const long long o = (long long)i * us0 + (long long)j * us1 + (long long)t * us2;
#pragma unroll
  for (int k = 0; k < 3; ++k) u[o + k * us3] = (double)u0[k];
}

template <typename CT>
__global__ void intersection_kernel(const Geometry G, const double *__restrict__ u, double *__restrict__ a1,
                                    double *__restrict__ an, long long us0, long long us1, long long us2,
                                    long long us3) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  const int t = G.view0 + blockIdx.z;
  if (i >= G.n1 || j >= G.n2) return;
  const tg_image_header &V = G.views[t];
  const long long o = (long long)i * us0 + (long long)j * us1 + (long long)t * us2;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const CT uk = (CT)u[o + k * us3];
    const CT Mk = (CT)V.M[k];
    CT b1, bn;
    if (uk != (CT)0) {
      b1 = ((CT)G.mh.mmin[k] - Mk) / uk;
      bn = ((CT)G.mh.mmax[k] - Mk) / uk;
    } else {
      b1 = -(CT)kRefInf;
      bn = (CT)kRefInf;
    }
    a1[o + k * us3] = (double)b1;
    an[o + k * us3] = (double)bn;
  }
}

cudaError_t launch_ref_f64(const Geometry &G, int mode, int obstacle, double *data, double *map, int gx, int gy,
                           int gz, cudaStream_t s) {
  dim3 grid(gx, gy, gz), block(kThreads);
  const bool sun = obstacle == TG_OBSTACLE_SUN;
  switch (mode) {
  case TG_PJ:
    if (sun) ref64_kernel<TG_PJ, true><<<grid, block, 0, s>>>(G, map, data);
    else ref64_kernel<TG_PJ, false><<<grid, block, 0, s>>>(G, map, data);
    break;
  case TG_BPJ:
    if (sun) ref64_kernel<TG_BPJ, true><<<grid, block, 0, s>>>(G, data, map);
    else ref64_kernel<TG_BPJ, false><<<grid, block, 0, s>>>(G, data, map);
    break;
  case TG_PJT:
    if (sun) ref64_kernel<TG_PJT, true><<<grid, block, 0, s>>>(G, map, data);
    else ref64_kernel<TG_PJT, false><<<grid, block, 0, s>>>(G, map, data);
    break;
  default:
    if (sun) ref64_kernel<TG_BPJT, true><<<grid, block, 0, s>>>(G, data, map);
    else ref64_kernel<TG_BPJT, false><<<grid, block, 0, s>>>(G, data, map);
    break;
  }
  return cudaGetLastError();
}

cudaError_t launch_unit_vector(const Geometry &G, int ctype_f64, const void *data, double *u,
                               const long long us[4], int gx, int gy, int gz, cudaStream_t s) {
  dim3 grid(gx, gy, gz), block(128);
  if (ctype_f64)
    unit_vector_kernel<double><<<grid, block, 0, s>>>(G, (const double *)data, u, us[0], us[1], us[2], us[3]);
  else
    unit_vector_kernel<float><<<grid, block, 0, s>>>(G, (const float *)data, u, us[0], us[1], us[2], us[3]);
  return cudaGetLastError();
}

cudaError_t launch_intersection_parameters(const Geometry &G, int ctype_f64, const double *u,
                                           const long long us[4], double *a1, double *an, int gx, int gy,
                                           int gz, cudaStream_t s) {
  dim3 grid(gx, gy, gz), block(128);
  if (ctype_f64)
    intersection_kernel<double><<<grid, block, 0, s>>>(G, u, a1, an, us[0], us[1], us[2], us[3]);
  else
    intersection_kernel<float><<<grid, block, 0, s>>>(G, u, a1, an, us[0], us[1], us[2], us[3]);
  return cudaGetLastError();
}

}  // namespace tg
