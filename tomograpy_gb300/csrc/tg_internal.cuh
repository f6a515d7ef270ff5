// Internal declarations shared by the CUDA translation units of
// libtomograpy_gb300.so.  Not part of the public ABI (include/tomograpy_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tomograpy_gb300.h"

namespace tg {

// Rows of pixels (one warp each) per CTA; a warp covers 32 consecutive pixels
// of one row (image axis 1, the lambda axis), so that for equatorial observers
// its 32 rays walk neighbouring voxels of the cube's fastest axis.
constexpr int kRows = 8;
constexpr int kThreads = 32 * kRows;
// The fast kernels give each warp kFastRowsPerWarp rows, so a CTA's
// per-tile trigonometry serves kFastRows x 32 rays.
constexpr int kFastRowsPerWarp = 4;
constexpr int kFastRows = kRows * kFastRowsPerWarp;

// The reference's finite "infinity" for zero direction components
// (tomograpy/C_siddon.c.template:17).
constexpr double kRefInf = 100000.0;

// Direction components below this magnitude are treated as exactly zero by
// the fast f32 kernel (a ray lying within 1e-14 rad of a voxel-plane family is
// traced as lying in it).  The f64 kernel keeps the reference's behaviour.
constexpr double kSnapZero = 1e-14;

// Launch description shared by all projector kernels.
struct Geometry {
  const tg_image_header *views;
  int n_views;
  int view0;           // first view of this launch (grid.z offset)
  int n1, n2;          // image rows (axis 0, gamma) / columns (axis 1, lambda)
  int bx0, by0;        // tile offsets (single-ray launches)
  int ray_i, ray_j;    // >= 0: trace only this pixel
  long long ds[3];     // data strides (elements)
  const void *mask;
  long long ks[3];
  int mask_dtype;      // tg_dtype
  int mask_eq1;        // 1: skip when mask == 1 (ray_projector); 0: skip when mask != 0
  int overwrite;       // projection: write every traced pixel (0 where skipped) instead of adding
  int n[3];            // cube voxels per axis
  int nframes;         // frames of a 4-D cube (1 for 3-D)
  long long ms[4];     // cube strides (elements)
  tg_map_header mh;
  float cdeltf[3], cdeltl[3], mminf[3], mmaxf[3], inv_cdeltf[3];  // cdeltl: CDELT - (float)CDELT
  double inv_cdelt[3];
};

// Read the mask of pixel (i, j, t); true when the ray must be skipped.
__device__ __forceinline__ bool masked(const Geometry &G, int i, int j, int t) {
  if (G.mask == nullptr) return false;
  long long o = (long long)i * G.ks[0] + (long long)j * G.ks[1] + (long long)t * G.ks[2];
  double v;
  if (G.mask_dtype == TG_U8) v = (double)((const unsigned char *)G.mask)[o];
  else if (G.mask_dtype == TG_F32) v = (double)((const float *)G.mask)[o];
  else v = ((const double *)G.mask)[o];
  return G.mask_eq1 ? (v == 1.0) : (v != 0.0);
}

// Host-side launchers (return a cudaError_t of the launch).
cudaError_t launch_fast_f32(const Geometry &G, int mode, int obstacle, bool idx64, float *data, float *map,
                            int grid_x, int grid_y, int grid_z, cudaStream_t s);
cudaError_t launch_count_f32(const Geometry &G, int obstacle, bool idx64, float *counts, int grid_x, int grid_y,
                             int grid_z, cudaStream_t s);
cudaError_t launch_ref_f64(const Geometry &G, int mode, int obstacle, double *data, double *map, int grid_x,
                           int grid_y, int grid_z, cudaStream_t s);
cudaError_t launch_unit_vector(const Geometry &G, int ctype_f64, const void *data, double *u,
                               const long long us[4], int grid_x, int grid_y, int grid_z, cudaStream_t s);
cudaError_t launch_intersection_parameters(const Geometry &G, int ctype_f64, const double *u,
                                           const long long us[4], double *a1, double *an, int grid_x,
                                           int grid_y, int grid_z, cudaStream_t s);
cudaError_t launch_deterministic_bpj(const Geometry &G, int mode, int obstacle, bool idx64, const float *data,
                                     float *map, void *workspace, int grid_x, int grid_y, int grid_z,
                                     cudaStream_t s);

cudaError_t launch_packed(const void *plan, int n_jobs, long long tiles, int rpw, bool idx64, int mode, int obstacle,
                          int lane_axis, int batch, cudaStream_t s);
struct PackedJob;
cudaError_t launch_packed_tuned(const long long *tile0, const PackedJob *jobs, int n_jobs, long long tiles, int rpw,
                                int mode, bool sun, int lane_axis, int batch, cudaStream_t s);
size_t packed_job_bytes();
size_t packed_records_offset(int n_jobs);
void packed_fill(void *dst, const Geometry &G, float *data, float *cube, long long tile0, int gx, int gy,
                 long long ws_off);
cudaError_t launch_packed_det(const void *plan, int n_jobs, long long tiles, int rpw, bool idx64, bool four_d,
                              int obstacle, void *workspace, size_t ws_bytes, cudaStream_t s);
cudaError_t launch_seg_dot(const float *a, const float *b, const long long *off, int n_seg, double *partial,
                           double *out, cudaStream_t st);
cudaError_t launch_seg_cg_x(float *x, float *r, const float *p, const float *Ap, const double *rr, const double *pAp,
                            const long long *off, int n_seg, cudaStream_t st);
cudaError_t launch_seg_cg_p(float *p, const float *r, double *rr, const double *rr_new, const long long *off,
                            int n_seg, cudaStream_t st);
size_t seg_workspace_bytes(int n_seg);
cudaError_t launch_seg_axpby(float *y, const float *x, float alpha, float beta, const long long *off, int n_seg,
                             cudaStream_t st);
cudaError_t noalloc_scratch(void **ptr);
size_t noalloc_scratch_bytes();
size_t noalloc_scratch_voxels();
cudaError_t launch_dot(const float *a, const float *b, long long n, double *partial, double *out, cudaStream_t s);

}  // namespace tg
