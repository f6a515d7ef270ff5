// Per-ray geometry set-up shared by the f32 and f64 projector kernels.
//
// The double-precision helpers here restate the reference's set-up stage with
// its order of operations and without FMA contraction (explicit _rn
// intrinsics), so that, given the same ray direction, they return the
// reference's own amin / amax, voxel index and plane distances:
//   pixel2physical            tomograpy/C_siddon.c.template:1043-1046
//   define_rotated_unit_vector tomograpy/C_siddon.c.template:1013-1032
//   get_intersection_parameters / intersect_map   :723-748
//   get_intersection_steps / get_pabs / get_update :750-774
//   get_voxel_index / get_next_voxel_index / get_intersection_distance :776-809
#pragma once

#include "tg_internal.cuh"

namespace tg {

// (idx - CRPIX + 1) * CDELT + CRVAL for image axis `axis` (0: gamma, 1: lambda).
__device__ __forceinline__ double pixel_angle(int idx, const tg_image_header &h, int axis) {
  return __dadd_rn(__dmul_rn(__dadd_rn(__dsub_rn((double)idx, h.crpix[axis]), 1.0), h.cdelt[axis]),
                   h.crval[axis]);
}

// u0 = R . (cos l cos g, cos l sin g, sin l), evaluated left to right.
__device__ __forceinline__ void ray_direction(double cl, double sl, double cg, double sg, const double *R,
                                              double u[3]) {
  const double u2x = __dmul_rn(cl, cg), u2y = __dmul_rn(cl, sg), u2z = sl;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    u[k] = __dadd_rn(__dadd_rn(__dmul_rn(R[3 * k], u2x), __dmul_rn(R[3 * k + 1], u2y)),
                     __dmul_rn(R[3 * k + 2], u2z));
}

// The reference stores (unsigned int)(quotient) into an int; on its x86-64
// build that is the low 32 bits of a truncating 64-bit conversion.
__device__ __forceinline__ int ref_utrunc(double x) {
  return (int)(unsigned int)(unsigned long long)__double2ll_rz(x);
}

__device__ __forceinline__ double ref_max3(double x, double y, double z) {
  if (x > y && x > z) return x;
  if (y >= x && y > z) return y;
  return z;
}

__device__ __forceinline__ double ref_min3(double x, double y, double z) {
  if (x < y && x < z) return x;
  if (y <= x && y < z) return y;
  return z;
}

struct RefWalk {
  int iv[3];      // entry voxel
  int upd[3];     // sign(u0)
  double D[3];    // distance from the entry point to the next plane of each family
  double pabs[3]; // distance between consecutive planes of each family
  double amin, amax;
};

// Full reference set-up in double precision.  Returns false when the ray
// misses the cube (amin >= amax).
__device__ __forceinline__ bool ref_setup(const tg_map_header &mh, const int n[3], const double M[3],
                                          const double u[3], RefWalk &w) {
  double a1[3], an[3], lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (u[k] != 0.0) {
      a1[k] = __ddiv_rn(__dsub_rn(mh.mmin[k], M[k]), u[k]);
      an[k] = __ddiv_rn(__dsub_rn(mh.mmax[k], M[k]), u[k]);
    } else {
      a1[k] = -kRefInf;
      an[k] = kRefInf;
    }
    if (a1[k] > an[k]) {
      lo[k] = an[k];
      hi[k] = a1[k];
    } else {
      lo[k] = a1[k];
      hi[k] = an[k];
    }
  }
  w.amin = ref_max3(lo[0], lo[1], lo[2]);
  w.amax = ref_min3(hi[0], hi[1], hi[2]);
  if (!(w.amin < w.amax)) return false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double p = (u[k] != 0.0) ? __ddiv_rn(mh.cdelt[k], u[k]) : kRefInf;
    w.pabs[k] = fabs(p);
    w.upd[k] = (u[k] > 0.0) ? 1 : ((u[k] < 0.0) ? -1 : 0);
    const double e = __dadd_rn(M[k], __dmul_rn(w.amin, u[k]));
    const double ep = __dsub_rn(e, mh.mmin[k]);
    w.iv[k] = ref_utrunc(__ddiv_rn(ep, mh.cdelt[k])) - ref_utrunc(__ddiv_rn(ep, mh.pshape[k]));
    unsigned int nx;
    if (w.upd[k] == 1) nx = (unsigned int)w.iv[k] + 1u;
    else if (w.upd[k] == -1) nx = (unsigned int)w.iv[k];
    else nx = 100000u * (unsigned int)n[k];
    w.D[k] = __dsub_rn(__dadd_rn(__dmul_rn((double)nx, p), a1[k]), w.amin);
  }
  return true;
}

// Squared distance to the cube origin at ray parameter ac, compared with 1
// (the "sun" obstacle, tomograpy/C_siddon.c.template:955-961,1034-1041).
__device__ __forceinline__ bool ref_outside_sun(const double M[3], const double u[3], double ac) {
  const double x = __dadd_rn(M[0], __dmul_rn(ac, u[0]));
  const double y = __dadd_rn(M[1], __dmul_rn(ac, u[1]));
  const double z = __dadd_rn(M[2], __dmul_rn(ac, u[2]));
  double d = __dmul_rn(x, x);
  d = __dadd_rn(d, __dmul_rn(y, y));
  d = __dadd_rn(d, __dmul_rn(z, z));
  return d > 1.0;
}

// Shared-memory tables of the CTA's angles: cos / sin of lambda for its 32
// columns and of gamma for its kRows rows.  Computed once per CTA.
struct TrigTables {
  double cl[32], sl[32], cg[kRows], sg[kRows];
};

__device__ __forceinline__ void fill_trig(TrigTables &T, const tg_image_header &V, int col0, int row0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
    double s, c;
    sincos(pixel_angle(col0 + lane, V, 1), &s, &c);
    T.sl[lane] = s;
    T.cl[lane] = c;
  } else if (warp == 1 && lane < kRows) {
    double s, c;
    sincos(pixel_angle(row0 + lane, V, 0), &s, &c);
    T.sg[lane] = s;
    T.cg[lane] = c;
  }
}

}  // namespace tg
