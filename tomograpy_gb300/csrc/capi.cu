// C ABI of libtomograpy_gb300.so (declared in include/tomograpy_gb300.h):
// argument validation, launch geometry and dispatch to the kernels.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "tg_internal.cuh"

namespace {

thread_local char g_err[512] = "";

tg_status fail(tg_status st, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return st;
}

tg_status launch_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return TG_OK;
  return fail(TG_ELAUNCH, "%s: %s", what, cudaGetErrorString(e));
}

bool finite3(const double *v) { return isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]); }

// Validate the shared arguments and fill the kernel geometry.
tg_status make_geometry(tg::Geometry &G, const tg_map_header *mh, const tg_image_header *views, int32_t n_views,
                        int64_t n1, int64_t n2, const int64_t ds[3], const int64_t map_shape[4],
                        const int64_t ms[4], const void *mask, tg_dtype mask_dtype, const int64_t ks[3],
                        bool four_d, bool *idx64) {
  memset(&G, 0, sizeof(G));
  if (!mh) return fail(TG_EINVAL, "map header is NULL");
  if (!finite3(mh->cdelt) || !finite3(mh->pshape) || !finite3(mh->mmin) || !finite3(mh->mmax))
    return fail(TG_EINVAL, "map header has a non-finite value");
  for (int k = 0; k < 3; ++k)
    if (!(mh->cdelt[k] > 0.0) || !(mh->pshape[k] > 0.0))
      return fail(TG_EINVAL, "map header CDELT%d / PSHAPE%d must be positive", k + 1, k + 1);
  if (n_views < 0) return fail(TG_EINVAL, "negative number of views");
  if (n_views > 0 && !views) return fail(TG_EINVAL, "view header table is NULL");
  if (n1 < 0 || n2 < 0 || n1 > (1 << 24) || n2 > (1 << 24))
    return fail(TG_EINVAL, "image shape (%lld, %lld) out of range", (long long)n1, (long long)n2);
  if (!ds || !map_shape || !ms) return fail(TG_EINVAL, "stride / shape array is NULL");
  for (int k = 0; k < 3; ++k)
    if (map_shape[k] < 1 || map_shape[k] > (1 << 20))
      return fail(TG_EINVAL, "cube axis %d has %lld voxels", k, (long long)map_shape[k]);
  if (four_d && (map_shape[3] < 1 || map_shape[3] > 2147483647LL))
    return fail(TG_EINVAL, "4-D cube has %lld frames (1 to 2^31 - 1 allowed)", (long long)map_shape[3]);
  if (mask) {
    if (!ks) return fail(TG_EINVAL, "mask strides are NULL");
    if (mask_dtype != TG_U8 && mask_dtype != TG_F32 && mask_dtype != TG_F64)
      return fail(TG_EINVAL, "mask dtype must be u8, f32 or f64");
  }
  G.views = views;
  G.n_views = n_views;
  G.n1 = (int)n1;
  G.n2 = (int)n2;
  G.ray_i = G.ray_j = -1;
  for (int k = 0; k < 3; ++k) {
    G.ds[k] = ds[k];
    G.ks[k] = mask ? ks[k] : 0;
    G.n[k] = (int)map_shape[k];
    G.ms[k] = ms[k];
    G.mh.cdelt[k] = mh->cdelt[k];
    G.mh.pshape[k] = mh->pshape[k];
    G.mh.mmin[k] = mh->mmin[k];
    G.mh.mmax[k] = mh->mmax[k];
    G.cdeltf[k] = (float)mh->cdelt[k];
    G.cdeltl[k] = (float)(mh->cdelt[k] - (double)G.cdeltf[k]);
    G.mminf[k] = (float)mh->mmin[k];
    G.mmaxf[k] = (float)mh->mmax[k];
    G.inv_cdelt[k] = 1.0 / mh->cdelt[k];
    G.inv_cdeltf[k] = (float)(1.0 / mh->cdelt[k]);
  }
  G.ms[3] = four_d ? ms[3] : 0;
  G.nframes = four_d ? (int)map_shape[3] : 1;
  G.mask = mask;
  G.mask_dtype = (int)mask_dtype;
  double span = 0.0;
  for (int k = 0; k < 3; ++k) span += (double)(map_shape[k] - 1) * fabs((double)ms[k]);
  *idx64 = span >= 2147483647.0;
  return TG_OK;
}

tg_status project_views(const tg_map_header *mh, const tg_image_header *views, int32_t n_views, int32_t view0,
                        int32_t count, int ray_i, int ray_j, tg_dtype dtype, void *data, int64_t n1, int64_t n2,
                        const int64_t ds[3], void *map, const int64_t map_shape[4], const int64_t ms[4],
                        const void *mask, tg_dtype mask_dtype, const int64_t ks[3], int32_t obstacle,
                        int32_t mode, void *stream) {
  const bool overwrite = (mode & TG_OVERWRITE) != 0;
  mode &= ~TG_OVERWRITE;
  if (mode < TG_PJ || mode > TG_BPJT) return fail(TG_EINVAL, "mode must be pj, bpj, pjt or bpjt");
  if (overwrite && (mode == TG_BPJ || mode == TG_BPJT)) return fail(TG_EINVAL, "overwrite is for projections");
  if (overwrite && dtype != TG_F32) return fail(TG_EUNSUPPORTED, "overwrite projections take f32 data");
  if (obstacle != TG_OBSTACLE_NONE && obstacle != TG_OBSTACLE_SUN)
    return fail(TG_EINVAL, "obstacle must be none or sun");
  if (dtype != TG_F32 && dtype != TG_F64) return fail(TG_EINVAL, "data dtype must be f32 or f64");
  const bool four_d = (mode == TG_PJT || mode == TG_BPJT);
  tg::Geometry G;
  bool idx64 = false;
  tg_status st = make_geometry(G, mh, views, n_views, n1, n2, ds, map_shape, ms, mask, mask_dtype, ks, four_d,
                               &idx64);
  if (st != TG_OK) return st;
  // nothing to trace: an empty stack may come with NULL data / cube pointers
  if (count <= 0 || n1 == 0 || n2 == 0) return TG_OK;
  if (!data || !map) return fail(TG_EINVAL, "data or map pointer is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  int gx, gy;
  const int rows = (dtype == TG_F32) ? tg::kFastRows : tg::kRows;
  G.overwrite = overwrite ? 1 : 0;
  if (ray_i >= 0) {
    G.ray_i = ray_i;
    G.ray_j = ray_j;
    G.mask_eq1 = 1;
    G.bx0 = ray_j / 32;
    G.by0 = ray_i / rows;
    gx = gy = 1;
  } else {
    gx = (int)((n2 + 31) / 32);
    gy = (int)((n1 + rows - 1) / rows);
    if (gy > 65535) return fail(TG_EUNSUPPORTED, "image has too many rows (%lld)", (long long)n1);
  }
  for (int32_t v = 0; v < count; v += 65535) {
    const int gz = (count - v) < 65535 ? (count - v) : 65535;
    G.view0 = view0 + v;
    cudaError_t e;
    if (dtype == TG_F32)
      e = tg::launch_fast_f32(G, mode, obstacle, idx64, (float *)data, (float *)map, gx, gy, gz, s);
    else
      e = tg::launch_ref_f64(G, mode, obstacle, (double *)data, (double *)map, gx, gy, gz, s);
    if (e != cudaSuccess) return launch_status(e, "projector launch");
  }
  return TG_OK;
}

}  // namespace

extern "C" {

tg_status tg_conic_full_projector(const tg_map_header *map_header, const tg_image_header *views, int32_t n_views,
                                  tg_dtype dtype, void *data, int64_t n1, int64_t n2, const int64_t data_strides[3],
                                  void *map, const int64_t map_shape[4], const int64_t map_strides[4],
                                  const void *mask, tg_dtype mask_dtype, const int64_t mask_strides[3],
                                  int32_t obstacle, int32_t mode, void *stream) {
  return project_views(map_header, views, n_views, 0, n_views, -1, -1, dtype, data, n1, n2, data_strides, map,
                       map_shape, map_strides, mask, mask_dtype, mask_strides, obstacle, mode, stream);
}

tg_status tg_conic_image_projector(const tg_map_header *map_header, const tg_image_header *views, int32_t n_views,
                                   int32_t t, tg_dtype dtype, void *data, int64_t n1, int64_t n2,
                                   const int64_t data_strides[3], void *map, const int64_t map_shape[4],
                                   const int64_t map_strides[4], const void *mask, tg_dtype mask_dtype,
                                   const int64_t mask_strides[3], int32_t obstacle, int32_t mode, void *stream) {
  if (t < 0 || t >= n_views) return fail(TG_EINVAL, "view index %d outside [0, %d)", t, n_views);
  return project_views(map_header, views, n_views, t, 1, -1, -1, dtype, data, n1, n2, data_strides, map,
                       map_shape, map_strides, mask, mask_dtype, mask_strides, obstacle, mode, stream);
}

tg_status tg_ray_projector(const tg_map_header *map_header, const tg_image_header *views, int32_t n_views,
                           int32_t i, int32_t j, int32_t t, tg_dtype dtype, void *data, int64_t n1, int64_t n2,
                           const int64_t data_strides[3], void *map, const int64_t map_shape[4],
                           const int64_t map_strides[4], const void *mask, tg_dtype mask_dtype,
                           const int64_t mask_strides[3], int32_t obstacle, int32_t mode, void *stream) {
  if (t < 0 || t >= n_views) return fail(TG_EINVAL, "view index %d outside [0, %d)", t, n_views);
  if (i < 0 || i >= n1 || j < 0 || j >= n2) return fail(TG_EINVAL, "pixel (%d, %d) outside the image", i, j);
  return project_views(map_header, views, n_views, t, 1, i, j, dtype, data, n1, n2, data_strides, map, map_shape,
                       map_strides, mask, mask_dtype, mask_strides, obstacle, mode, stream);
}

tg_status tg_unit_vector(const tg_image_header *views, int32_t n_views, int32_t t, tg_dtype dtype,
                         const void *data, int64_t n1, int64_t n2, const int64_t data_strides[3], double *u,
                         const int64_t u_strides[4], void *stream) {
  if (dtype != TG_F32 && dtype != TG_F64) return fail(TG_EINVAL, "data dtype must be f32 or f64");
  if (!views || !data || !u || !data_strides || !u_strides) return fail(TG_EINVAL, "NULL argument");
  if (n1 < 0 || n2 < 0 || n1 > 65535 || n2 > (1 << 24)) return fail(TG_EINVAL, "image shape out of range");
  if (t < -1 || t >= n_views) return fail(TG_EINVAL, "view index %d outside [-1, %d)", t, n_views);
  if (n1 == 0 || n2 == 0 || n_views == 0) return TG_OK;
  tg::Geometry G;
  memset(&G, 0, sizeof(G));
  G.views = views;
  G.n_views = n_views;
  G.n1 = (int)n1;
  G.n2 = (int)n2;
  for (int k = 0; k < 3; ++k) G.ds[k] = data_strides[k];
  const long long us[4] = {u_strides[0], u_strides[1], u_strides[2], u_strides[3]};
  const int count = (t < 0) ? n_views : 1;
  for (int v = 0; v < count; v += 65535) {
    G.view0 = (t < 0 ? 0 : t) + v;
    const int gz = (count - v) < 65535 ? (count - v) : 65535;
    cudaError_t e = tg::launch_unit_vector(G, dtype == TG_F64, data, u, us, (int)((n2 + 127) / 128), (int)n1, gz,
                                           (cudaStream_t)stream);
    if (e != cudaSuccess) return launch_status(e, "unit vector launch");
  }
  return TG_OK;
}

tg_status tg_intersection_parameters(const tg_map_header *map_header, const tg_image_header *views,
                                     int32_t n_views, int32_t t, tg_dtype dtype, int64_t n1, int64_t n2,
                                     const double *u, const int64_t u_strides[4], double *a1, double *an,
                                     void *stream) {
  if (dtype != TG_F32 && dtype != TG_F64) return fail(TG_EINVAL, "dtype must be f32 or f64");
  if (!map_header || !views || !u || !u_strides || !a1 || !an) return fail(TG_EINVAL, "NULL argument");
  if (n1 < 0 || n2 < 0 || n1 > 65535 || n2 > (1 << 24)) return fail(TG_EINVAL, "image shape out of range");
  if (t < -1 || t >= n_views) return fail(TG_EINVAL, "view index %d outside [-1, %d)", t, n_views);
  if (n1 == 0 || n2 == 0 || n_views == 0) return TG_OK;
  tg::Geometry G;
  memset(&G, 0, sizeof(G));
  G.views = views;
  G.n_views = n_views;
  G.n1 = (int)n1;
  G.n2 = (int)n2;
  G.mh = *map_header;
  const long long us[4] = {u_strides[0], u_strides[1], u_strides[2], u_strides[3]};
  const int count = (t < 0) ? n_views : 1;
  for (int v = 0; v < count; v += 65535) {
    G.view0 = (t < 0 ? 0 : t) + v;
    const int gz = (count - v) < 65535 ? (count - v) : 65535;
    cudaError_t e = tg::launch_intersection_parameters(G, dtype == TG_F64, u, us, a1, an, (int)((n2 + 127) / 128),
                                                       (int)n1, gz, (cudaStream_t)stream);
    if (e != cudaSuccess) return launch_status(e, "intersection parameters launch");
  }
  return TG_OK;
}

size_t tg_deterministic_workspace_bytes(const int64_t map_shape[4]) {
  if (!map_shape) return 0;
  // checked arithmetic: a shape whose accumulator does not fit in size_t
  // needs SIZE_MAX bytes, which no workspace (or the built-in scratch) holds
  size_t vox = 1;
  for (int k = 0; k < 4; ++k)
    if (__builtin_mul_overflow(vox, (size_t)(map_shape[k] > 0 ? map_shape[k] : 1), &vox)) return SIZE_MAX;
  size_t bytes;
  if (__builtin_mul_overflow(vox, (size_t)8, &bytes) || __builtin_add_overflow(bytes, (size_t)(256 + 255), &bytes))
    return SIZE_MAX;
  return bytes & ~(size_t)255;
}

tg_status tg_conic_full_backprojector_deterministic(
    const tg_map_header *map_header, const tg_image_header *views, int32_t n_views, float *data, int64_t n1,
    int64_t n2, const int64_t data_strides[3], float *map, const int64_t map_shape[4], const int64_t map_strides[4],
    const void *mask, tg_dtype mask_dtype, const int64_t mask_strides[3], int32_t obstacle, int32_t mode,
    void *workspace, size_t workspace_bytes, void *stream) {
  if (mode != TG_BPJ && mode != TG_BPJT) return fail(TG_EINVAL, "deterministic mode is for bpj / bpjt");
  if (obstacle != TG_OBSTACLE_NONE && obstacle != TG_OBSTACLE_SUN)
    return fail(TG_EINVAL, "obstacle must be none or sun");
  if (!data || !map) return fail(TG_EINVAL, "data or map pointer is NULL");
  if (!workspace || ((uintptr_t)workspace & 255u)) return fail(TG_EINVAL, "workspace must be 256-byte aligned");
  const bool four_d = (mode == TG_BPJT);
  int64_t shape4[4] = {map_shape ? map_shape[0] : 0, map_shape ? map_shape[1] : 0, map_shape ? map_shape[2] : 0,
                       four_d && map_shape ? map_shape[3] : 1};
  const size_t need = tg_deterministic_workspace_bytes(shape4);
  if (need == SIZE_MAX) return fail(TG_EINVAL, "cube too large for a 64-bit accumulator");
  if (workspace_bytes < need) return fail(TG_ENOMEM, "workspace has %zu bytes, needs %zu", workspace_bytes, need);
  tg::Geometry G;
  bool idx64 = false;
  tg_status st = make_geometry(G, map_header, views, n_views, n1, n2, data_strides, map_shape, map_strides, mask,
                               mask_dtype, mask_strides, four_d, &idx64);
  if (st != TG_OK) return st;
  if (n_views == 0 || n1 == 0 || n2 == 0) return TG_OK;
  // accumulator offsets are dense C order (n0, n1, n2) within a frame
  const double span = (double)G.n[0] * G.n[1] * G.n[2];
  idx64 = span >= 2147483647.0;
  const int gx = (int)((n2 + 31) / 32), gy = (int)((n1 + tg::kFastRows - 1) / tg::kFastRows);
  if (gy > 65535) return fail(TG_EUNSUPPORTED, "image has too many rows");
  if (n_views > 65535) return fail(TG_EUNSUPPORTED, "deterministic mode takes at most 65535 views per call");
  G.view0 = 0;
  cudaError_t e = tg::launch_deterministic_bpj(G, mode, obstacle, idx64, data, map, workspace, gx, gy, n_views,
                                               (cudaStream_t)stream);
  return launch_status(e, "deterministic backprojection launch");
}

tg_status tg_segment_counts(const tg_map_header *map_header, const tg_image_header *views, int32_t n_views,
                            float *counts, int64_t n1, int64_t n2, const int64_t count_strides[3],
                            const int64_t map_shape[3], const void *mask, tg_dtype mask_dtype,
                            const int64_t mask_strides[3], int32_t obstacle, void *stream) {
  if (obstacle != TG_OBSTACLE_NONE && obstacle != TG_OBSTACLE_SUN)
    return fail(TG_EINVAL, "obstacle must be none or sun");
  if (!counts || !map_shape) return fail(TG_EINVAL, "NULL argument");
  const int64_t shape4[4] = {map_shape[0], map_shape[1], map_shape[2], 1};
  const int64_t strides4[4] = {map_shape[1] * map_shape[2], map_shape[2], 1, 0};
  tg::Geometry G;
  bool idx64 = false;
  tg_status st = make_geometry(G, map_header, views, n_views, n1, n2, count_strides, shape4, strides4, mask,
                               mask_dtype, mask_strides, false, &idx64);
  if (st != TG_OK) return st;
  if (n_views == 0 || n1 == 0 || n2 == 0) return TG_OK;
  const int gx = (int)((n2 + 31) / 32), gy = (int)((n1 + tg::kFastRows - 1) / tg::kFastRows);
  if (gy > 65535) return fail(TG_EUNSUPPORTED, "image has too many rows");
  for (int32_t v = 0; v < n_views; v += 65535) {
    G.view0 = v;
    const int gz = (n_views - v) < 65535 ? (n_views - v) : 65535;
    cudaError_t e = tg::launch_count_f32(G, obstacle, idx64, counts, gx, gy, gz, (cudaStream_t)stream);
    if (e != cudaSuccess) return launch_status(e, "segment count launch");
  }
  return TG_OK;
}

size_t tg_packed_plan_bytes(int32_t n_jobs) {
  if (n_jobs < 0) return 0;
  return tg::packed_records_offset(n_jobs) + (((size_t)n_jobs * tg::packed_job_bytes() + 255) & ~(size_t)255);
}

static tg_status build_packed_plan(const tg_job *jobs, int32_t n_jobs, const tg_schedule &sched, int32_t four_d,
                                   unsigned char *host, tg_packed_info *info);

tg_status tg_packed_plan_scheduled(const tg_job *jobs, int32_t n_jobs, const tg_schedule *schedule, int32_t four_d,
                                   void *plan, size_t plan_bytes, tg_packed_info *info) {
  if (!info || !schedule) return fail(TG_EINVAL, "info or schedule is NULL");
  if (n_jobs <= 0 || !jobs) return fail(TG_EINVAL, "no jobs");
  if (!plan || plan_bytes < tg_packed_plan_bytes(n_jobs)) return fail(TG_ENOMEM, "plan buffer too small");
  std::vector<unsigned char> host(tg_packed_plan_bytes(n_jobs), 0);
  tg_status st = build_packed_plan(jobs, n_jobs, *schedule, four_d, host.data(), info);
  if (st != TG_OK) return st;
  cudaError_t e = cudaMemcpy(plan, host.data(), host.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return launch_status(e, "plan upload");
  return TG_OK;
}

tg_status tg_packed_plan_scheduled_host(const tg_job *jobs, int32_t n_jobs, const tg_schedule *schedule,
                                        int32_t four_d, void *host_plan, size_t plan_bytes, tg_packed_info *info) {
  if (!info || !schedule) return fail(TG_EINVAL, "info or schedule is NULL");
  if (n_jobs <= 0 || !jobs) return fail(TG_EINVAL, "no jobs");
  if (!host_plan || plan_bytes < tg_packed_plan_bytes(n_jobs)) return fail(TG_ENOMEM, "plan buffer too small");
  std::memset(host_plan, 0, tg_packed_plan_bytes(n_jobs));
  return build_packed_plan(jobs, n_jobs, *schedule, four_d, (unsigned char *)host_plan, info);
}

tg_status tg_packed_plan(const tg_job *jobs, int32_t n_jobs, int32_t rows_per_warp, int32_t four_d, void *plan,
                         size_t plan_bytes, tg_packed_info *info) {
  const tg_schedule sched = {rows_per_warp, 1, 0, 0};
  return tg_packed_plan_scheduled(jobs, n_jobs, &sched, four_d, plan, plan_bytes, info);
}

tg_status tg_packed_plan_host(const tg_job *jobs, int32_t n_jobs, int32_t rows_per_warp, int32_t four_d,
                              void *host_plan, size_t plan_bytes, tg_packed_info *info) {
  const tg_schedule sched = {rows_per_warp, 1, 0, 0};
  return tg_packed_plan_scheduled_host(jobs, n_jobs, &sched, four_d, host_plan, plan_bytes, info);
}

static tg_status build_packed_plan(const tg_job *jobs, int32_t n_jobs, const tg_schedule &sched, int32_t four_d,
                                   unsigned char *host, tg_packed_info *info) {
  const int rows_per_warp = sched.rows_per_warp;
  if (rows_per_warp != 1 && rows_per_warp != 2 && rows_per_warp != 4)
    return fail(TG_EINVAL, "rows_per_warp must be 1, 2 or 4");
  if (sched.lane_axis != 0 && sched.lane_axis != 1) return fail(TG_EINVAL, "lane_axis must be 0 or 1");
  if (sched.batch_steps != 0 && sched.batch_steps != 16) return fail(TG_EINVAL, "batch_steps must be 0 or 16");
  const int rows = rows_per_warp * tg::kRows;
  struct Item {
    double work;
    int idx;
  };
  std::vector<Item> order((size_t)n_jobs);
  std::vector<tg::Geometry> geoms((size_t)n_jobs);
  bool idx64 = false;
  for (int j = 0; j < n_jobs; ++j) {
    const tg_job &J = jobs[j];
    bool i64 = false;
    tg_status st = make_geometry(geoms[j], &J.map_header, J.views, J.n_views, J.n1, J.n2, J.data_strides,
                                 J.map_shape, J.map_strides, J.mask, (tg_dtype)J.mask_dtype, J.mask_strides,
                                 four_d != 0, &i64);
    if (st != TG_OK) {
      char why[sizeof(g_err)];
      std::memcpy(why, g_err, sizeof(why));  // fail() writes g_err: format from a copy
      return fail(st, "job %d: %s", j, why);
    }
    if (J.n_views > 0 && J.n1 > 0 && J.n2 > 0 && (!J.data || !J.map))
      return fail(TG_EINVAL, "job %d: data or map pointer is NULL", j);
    idx64 = idx64 || i64;
    order[j] = {(double)J.n_views * J.n1 * J.n2 * (double)(J.map_shape[0] + J.map_shape[1] + J.map_shape[2]), j};
  }
  std::stable_sort(order.begin(), order.end(), [](const Item &a, const Item &b) { return a.work > b.work; });
  // the other schedules are built for 32-bit cube offsets only
  const bool lmaj = idx64 || sched.lane_axis == 1;
  const int batch = idx64 ? 0 : sched.batch_steps;
  const int tile_cols = lmaj ? 32 : rows, tile_rows = lmaj ? rows : 32;
  const size_t rec0 = tg::packed_records_offset(n_jobs);
  long long tiles = 0;
  size_t ws = 0;             // deterministic workspace: one 256-byte aligned part per job
  bool det_idx64 = false;
  for (int k = 0; k < n_jobs; ++k) {
    const int j = order[k].idx;
    const tg_job &J = jobs[j];
    const int gx = (int)((J.n2 + tile_cols - 1) / tile_cols), gy = (int)((J.n1 + tile_rows - 1) / tile_rows);
    const int64_t shape4[4] = {J.map_shape[0], J.map_shape[1], J.map_shape[2], four_d ? J.map_shape[3] : 1};
    const size_t part = tg_deterministic_workspace_bytes(shape4);
    if (part == SIZE_MAX || ws > SIZE_MAX - part) return fail(TG_EINVAL, "job %d: cube too large", j);
    det_idx64 = det_idx64 || (double)J.map_shape[0] * J.map_shape[1] * J.map_shape[2] >= 2147483647.0;
    std::memcpy(host + (size_t)k * sizeof(long long), &tiles, sizeof(long long));
    tg::packed_fill(host + rec0 + (size_t)k * tg::packed_job_bytes(), geoms[j], J.data, J.map, tiles, gx, gy,
                    (long long)ws);
    tiles += (long long)gx * gy * J.n_views;
    ws += part;
  }
  if (tiles > 2147483647LL) return fail(TG_EUNSUPPORTED, "packed launch of %lld CTAs is too large", tiles);
  info->n_jobs = n_jobs;
  info->rows_per_warp = rows_per_warp;
  info->four_d = four_d != 0;
  info->idx64 = idx64 ? 1 : 0;
  info->tiles = tiles;
  info->det_workspace_bytes = (int64_t)ws;
  info->det_idx64 = det_idx64 ? 1 : 0;
  info->lane_axis = lmaj ? 1 : 0;
  info->batch_steps = batch;
  info->reserved = 0;
  return TG_OK;
}

tg_status tg_packed_projector(const void *plan, const tg_packed_info *info, int32_t mode, int32_t obstacle,
                              void *stream) {
  if (!plan || !info) return fail(TG_EINVAL, "NULL plan");
  if (obstacle != TG_OBSTACLE_NONE && obstacle != TG_OBSTACLE_SUN)
    return fail(TG_EINVAL, "obstacle must be none or sun");
  const bool four_d = (mode == TG_PJT || mode == TG_BPJT);
  if (mode < TG_PJ || mode > TG_BPJT || four_d != (info->four_d != 0))
    return fail(TG_EINVAL, "mode does not match the plan (3-D / 4-D)");
  if (info->n_jobs <= 0) return fail(TG_EINVAL, "plan has %d jobs", info->n_jobs);
  if (info->tiles <= 0) return TG_OK;
  if (info->tiles > 2147483647LL) return fail(TG_EUNSUPPORTED, "packed launch of %lld CTAs is too large",
                                              (long long)info->tiles);
  if (info->idx64 && (info->lane_axis != 1 || info->batch_steps != 0))
    return fail(TG_EINVAL, "a plan with 64-bit cube offsets takes the default schedule");
  return launch_status(tg::launch_packed(plan, info->n_jobs, info->tiles, info->rows_per_warp, info->idx64 != 0,
                                         mode, obstacle, info->lane_axis, info->batch_steps, (cudaStream_t)stream),
                       "packed projector launch");
}

tg_status tg_packed_backprojector_deterministic(const void *plan, const tg_packed_info *info, int32_t obstacle,
                                               void *workspace, size_t workspace_bytes, void *stream) {
  if (!plan || !info) return fail(TG_EINVAL, "NULL plan");
  if (obstacle != TG_OBSTACLE_NONE && obstacle != TG_OBSTACLE_SUN)
    return fail(TG_EINVAL, "obstacle must be none or sun");
  if (info->n_jobs <= 0 || info->n_jobs > 65535) return fail(TG_EINVAL, "plan has %d jobs (1 to 65535)", info->n_jobs);
  if (info->tiles <= 0) return TG_OK;
  if (info->lane_axis != 1)
    return fail(TG_EINVAL, "deterministic packed backprojection takes plans with lane_axis 1");
  if (!workspace || ((uintptr_t)workspace & 255u)) return fail(TG_EINVAL, "workspace must be 256-byte aligned");
  if (info->det_workspace_bytes <= 0 || workspace_bytes < (size_t)info->det_workspace_bytes)
    return fail(TG_ENOMEM, "workspace has %zu bytes, the plan needs %lld", workspace_bytes,
                (long long)info->det_workspace_bytes);
  return launch_status(tg::launch_packed_det(plan, info->n_jobs, info->tiles, info->rows_per_warp,
                                             info->idx64 != 0 || info->det_idx64 != 0, info->four_d != 0, obstacle,
                                             workspace, (size_t)info->det_workspace_bytes, (cudaStream_t)stream),
                       "deterministic packed backprojection launch");
}

size_t tg_segmented_workspace_bytes(int32_t n_seg) { return n_seg > 0 ? tg::seg_workspace_bytes(n_seg) : 0; }

tg_status tg_segmented_dot_f32(const float *a, const float *b, const int64_t *off, int32_t n_seg, double *out,
                               void *workspace, size_t workspace_bytes, void *stream) {
  if (!a || !b || !off || !out || n_seg <= 0 || n_seg > 65535) return fail(TG_EINVAL, "bad segmented dot arguments");
  if (!workspace || workspace_bytes < tg::seg_workspace_bytes(n_seg))
    return fail(TG_ENOMEM, "segmented dot workspace needs %zu bytes", tg::seg_workspace_bytes(n_seg));
  return launch_status(tg::launch_seg_dot(a, b, (const long long *)off, n_seg, (double *)workspace, out,
                                          (cudaStream_t)stream),
                       "segmented dot launch");
}

tg_status tg_cg_update_x(float *x, float *r, const float *p, const float *Ap, const double *rr, const double *pAp,
                         const int64_t *off, int32_t n_seg, void *stream) {
  if (!x || !r || !p || !Ap || !rr || !pAp || !off || n_seg <= 0 || n_seg > 65535)
    return fail(TG_EINVAL, "bad CG update arguments");
  return launch_status(
      tg::launch_seg_cg_x(x, r, p, Ap, rr, pAp, (const long long *)off, n_seg, (cudaStream_t)stream), "CG update");
}

tg_status tg_cg_update_p(float *p, const float *r, double *rr, const double *rr_new, const int64_t *off,
                         int32_t n_seg, void *stream) {
  if (!p || !r || !rr || !rr_new || !off || n_seg <= 0 || n_seg > 65535) return fail(TG_EINVAL, "bad CG update arguments");
  return launch_status(tg::launch_seg_cg_p(p, r, rr, rr_new, (const long long *)off, n_seg, (cudaStream_t)stream),
                       "CG update");
}

tg_status tg_segmented_axpby(float *y, const float *x, float alpha, float beta, const int64_t *seg, int32_t n_seg,
                             void *stream) {
  if (!y || !seg || n_seg <= 0 || n_seg > 65535) return fail(TG_EINVAL, "bad segmented axpby arguments");
  return launch_status(tg::launch_seg_axpby(y, x, alpha, beta, (const long long *)seg, n_seg, (cudaStream_t)stream),
                       "segmented axpby");
}

size_t tg_noalloc_scratch_bytes(void) { return tg::noalloc_scratch_bytes(); }

tg_status tg_conic_full_backprojector_deterministic_noalloc(
    const tg_map_header *map_header, const tg_image_header *views, int32_t n_views, float *data, int64_t n1,
    int64_t n2, const int64_t data_strides[3], float *map, const int64_t map_shape[4], const int64_t map_strides[4],
    const void *mask, tg_dtype mask_dtype, const int64_t mask_strides[3], int32_t obstacle, int32_t mode,
    void *stream) {
  if (mode != TG_BPJ && mode != TG_BPJT) return fail(TG_EINVAL, "deterministic mode is for bpj / bpjt");
  if (!map_shape) return fail(TG_EINVAL, "map shape is NULL");
  const bool four_d = (mode == TG_BPJT);
  const int64_t shape4[4] = {map_shape[0], map_shape[1], map_shape[2], four_d ? map_shape[3] : 1};
  const size_t need = tg_deterministic_workspace_bytes(shape4);
  if (need > tg::noalloc_scratch_bytes())
    return fail(TG_ENOMEM,
                "cube of %lld x %lld x %lld x %lld voxels needs %zu bytes of scratch; the built-in scratch holds "
                "%zu bytes (%zu voxels): use tg_conic_full_backprojector_deterministic with a workspace",
                (long long)shape4[0], (long long)shape4[1], (long long)shape4[2], (long long)shape4[3], need,
                tg::noalloc_scratch_bytes(), tg::noalloc_scratch_voxels());
  void *scratch = nullptr;
  cudaError_t e = tg::noalloc_scratch(&scratch);
  if (e != cudaSuccess) return launch_status(e, "scratch address lookup");
  return tg_conic_full_backprojector_deterministic(map_header, views, n_views, data, n1, n2, data_strides, map,
                                                   map_shape, map_strides, mask, mask_dtype, mask_strides, obstacle,
                                                   mode, scratch, tg::noalloc_scratch_bytes(), stream);
}

size_t tg_dot_workspace_bytes(void) { return 1216 * sizeof(double); }

tg_status tg_dot_f32(const float *a, const float *b, int64_t n, double *out, void *workspace, size_t workspace_bytes,
                     void *stream) {
  if (!a || !b || !out || n < 0) return fail(TG_EINVAL, "bad dot arguments");
  if (!workspace || workspace_bytes < tg_dot_workspace_bytes() || ((uintptr_t)workspace & 7u))
    return fail(TG_ENOMEM, "dot workspace needs %zu bytes, 8-byte aligned", tg_dot_workspace_bytes());
  return launch_status(tg::launch_dot(a, b, n, (double *)workspace, out, (cudaStream_t)stream), "dot launch");
}

tg_status tg_host_alias(const void *host, void **device) {
  if (!host || !device) return fail(TG_EINVAL, "NULL argument");
  *device = nullptr;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, host);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return launch_status(e, "pointer attributes");
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr)
    return fail(TG_EINVAL, "not page-locked host memory mapped into the device's address space");
  *device = a.devicePointer;
  return TG_OK;
}

const char *tg_last_error(void) { return g_err; }

int32_t tg_abi_version(void) { return 2; }

}  // extern "C"
