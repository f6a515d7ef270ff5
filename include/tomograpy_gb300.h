/*
 * tomograpy_gb300 -- C ABI of the GB300 (sm_103a) Siddon conic projector.
 *
 * One shared library, libtomograpy_gb300.so, replaces the 16 CPython modules
 * _C_siddon_{float,double}_{none,sun}_{pj,bpj,pjt,bpjt} that TomograPy builds
 * from tomograpy/C_siddon.c.template (method table at
 * tomograpy/C_siddon.c.template:163-172).  The variant that the reference
 * selects by module name (data type x obstacle x accumulate kind) is selected
 * here by arguments.
 *
 * Conventions
 *  - Every array argument is a DEVICE pointer, except the cube header, which
 *    is a host struct passed by pointer.  The per-view header table is a
 *    device array of tg_image_header.
 *  - Arrays are given as base pointer + per-axis strides counted in ELEMENTS
 *    (not bytes); any signed strides are accepted, so the reference's C-order
 *    layouts (data (N1, N2, T) with T fastest; cube (n0, n1, n2[, F])) and
 *    view-major / frame-major layouts work without copies.
 *  - Calls are asynchronous on `stream` (a cudaStream_t; NULL = legacy default
 *    stream).  The data / cube outputs ACCUMULATE, as in the reference
 *    (tomograpy/C_siddon.c.template:914-944): zero them first for a plain
 *    projection.
 *  - The mask skips a pixel when its element is non-zero, element by element,
 *    for u8 / f32 / f64 masks.  (The reference reads its mask with the data's
 *    C type whatever the mask's own dtype, tomograpy/C_siddon.c.template:29-31,520;
 *    interpreting each element by its own dtype is a deliberate fix.)
 *  - Status codes instead of Python exceptions; tg_last_error() returns a
 *    thread-local message for the last non-OK status.
 *
 * Arithmetic: f64 data runs a reference-faithful double-precision trace (the
 * reference's order of operations, no FMA contraction).  f32 data runs the
 * fast kernel: per-ray set-up in double precision, the voxel walk in single
 * precision relative to the cube entry point, and the obstacle test confirmed
 * in double precision whenever single precision cannot decide it.
 */
#ifndef TOMOGRAPY_GB300_H
#define TOMOGRAPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TG_OK = 0,
  TG_EINVAL = 1,       /* bad argument (reference: ValueError, C_siddon.c.template:42,188-201) */
  TG_ENOMEM = 2,       /* workspace too small */
  TG_ELAUNCH = 3,      /* CUDA launch / runtime error */
  TG_EUNSUPPORTED = 4  /* valid but not supported by this build */
} tg_status;

typedef enum { TG_PJ = 0, TG_BPJ = 1, TG_PJT = 2, TG_BPJT = 3 } tg_mode;
/* Flag ORed into TG_PJ / TG_PJT (f32 data) of the projector entry points:
 * every pixel of the traced views is written -- the projection, or 0 where
 * the ray is masked or misses the cube -- instead of added, so the stack
 * needs no zeroing first (e.g. a stack in page-locked host memory written
 * directly by the kernel, see tg_host_alias).  The reference always adds. */
#define TG_OVERWRITE 16
typedef enum { TG_OBSTACLE_NONE = 0, TG_OBSTACLE_SUN = 1 } tg_obstacle;
typedef enum { TG_F32 = 0, TG_F64 = 1, TG_U8 = 2 } tg_dtype;

/* Cube ("map") header: CDELT1-3, PSHAPE1-3, MMIN1-3, MMAX1-3 in solar radii
   (reference map_header, tomograpy/C_siddon.c.template:50-56,1058-1075). */
typedef struct {
  double cdelt[3];
  double pshape[3];
  double mmin[3];
  double mmax[3];
} tg_map_header;

/* Per-view header: CRPIX1-2, CDELT1-2 and CRVAL1-2 (radians), observer
   position M1-3 and rotation R1_1..R3_3 row-major (reference image_header,
   tomograpy/C_siddon.c.template:58-65,1077-1101), plus the cube frame this view
   reads / writes in the 4-D modes (the reference uses the view index,
   tomograpy/C_siddon.c.template:931-944).  152 bytes. */
typedef struct {
  double crpix[2];
  double cdelt[2];
  double crval[2];
  double M[3];
  double R[9];
  int32_t frame;
  int32_t reserved;
} tg_image_header;

/* Project (TG_PJ / TG_PJT) or backproject (TG_BPJ / TG_BPJT) all n_views views.
 * Replaces conic_full_projector (tomograpy/C_siddon.c.template:182-205,460-498),
 * i.e. tomograpy.projector / backprojector / projector4d / backprojector4d
 * (tomograpy/siddon.py:85-219).
 *   data      (n1, n2, n_views) image stack, strides data_strides[3]
 *   map       cube (map_shape[0..2] voxels, map_shape[3] frames; 1 for 3-D),
 *             strides map_strides[4] (map_strides[3] ignored for 3-D modes)
 *   mask      NULL or (n1, n2, n_views) with mask_strides[3], type mask_dtype
 *   dtype     TG_F32 or TG_F64, shared by data and map
 * In the 4-D modes a view whose frame is outside [0, map_shape[3]) is skipped
 * (the reference does not check, tomograpy/C_siddon.c.template:935,943). */
tg_status tg_conic_full_projector(const tg_map_header *map_header, const tg_image_header *views,
                                  int32_t n_views, tg_dtype dtype, void *data, int64_t n1, int64_t n2,
                                  const int64_t data_strides[3], void *map, const int64_t map_shape[4],
                                  const int64_t map_strides[4], const void *mask, tg_dtype mask_dtype,
                                  const int64_t mask_strides[3], int32_t obstacle, int32_t mode,
                                  void *stream);

/* Same for a single view t of the stack.  Replaces conic_image_projector
   (tomograpy/C_siddon.c.template:207-248,500-528; tomograpy/siddon.py:221-243). */
tg_status tg_conic_image_projector(const tg_map_header *map_header, const tg_image_header *views,
                                   int32_t n_views, int32_t t, tg_dtype dtype, void *data, int64_t n1,
                                   int64_t n2, const int64_t data_strides[3], void *map,
                                   const int64_t map_shape[4], const int64_t map_strides[4],
                                   const void *mask, tg_dtype mask_dtype, const int64_t mask_strides[3],
                                   int32_t obstacle, int32_t mode, void *stream);

/* One ray (pixel i, j of view t).  Replaces ray_projector
   (tomograpy/C_siddon.c.template:250-307): the ray is skipped when its mask
   element equals exactly 1, as there. */
tg_status tg_ray_projector(const tg_map_header *map_header, const tg_image_header *views, int32_t n_views,
                           int32_t i, int32_t j, int32_t t, tg_dtype dtype, void *data, int64_t n1,
                           int64_t n2, const int64_t data_strides[3], void *map, const int64_t map_shape[4],
                           const int64_t map_strides[4], const void *mask, tg_dtype mask_dtype,
                           const int64_t mask_strides[3], int32_t obstacle, int32_t mode, void *stream);

/* Unit vector of every pixel ray whose data value is not NaN, written as f64
   into u[i, j, t, k] (strides u_strides[4]).  Replaces full_unit_vector /
   image_unit_vector (tomograpy/C_siddon.c.template:310-365,582-648). Pass
   t = -1 for all views, else one view. */
tg_status tg_unit_vector(const tg_image_header *views, int32_t n_views, int32_t t, tg_dtype dtype,
                         const void *data, int64_t n1, int64_t n2, const int64_t data_strides[3], double *u,
                         const int64_t u_strides[4], void *stream);

/* Ray parameters a1 / an of the MMIN / MMAX planes of every pixel for given
   unit vectors (f64, layout as u).  Replaces full_intersection_parameters /
   image_intersection_parameters (tomograpy/C_siddon.c.template:368-455,650-735).
   dtype selects the arithmetic precision (the reference casts to its C type).
   t = -1 for all views. */
tg_status tg_intersection_parameters(const tg_map_header *map_header, const tg_image_header *views,
                                     int32_t n_views, int32_t t, tg_dtype dtype, int64_t n1, int64_t n2,
                                     const double *u, const int64_t u_strides[4], double *a1, double *an,
                                     void *stream);

/* Deterministic backprojection (TG_BPJ / TG_BPJT, f32 only): every segment is
 * accumulated as a 64-bit fixed-point integer, so the result is bitwise the
 * same whatever the order in which rays run.  No counterpart in the reference,
 * whose OpenMP atomics (tomograpy/C_siddon.c.template:926,942) sum in thread
 * order.  Needs a device workspace of tg_deterministic_workspace_bytes()
 * bytes, 256-byte aligned; its contents need not be initialised. */
size_t tg_deterministic_workspace_bytes(const int64_t map_shape[4]);
tg_status tg_conic_full_backprojector_deterministic(
    const tg_map_header *map_header, const tg_image_header *views, int32_t n_views, float *data, int64_t n1,
    int64_t n2, const int64_t data_strides[3], float *map, const int64_t map_shape[4],
    const int64_t map_strides[4], const void *mask, tg_dtype mask_dtype, const int64_t mask_strides[3],
    int32_t obstacle, int32_t mode, void *workspace, size_t workspace_bytes, void *stream);

/* Deterministic backprojection without any device allocation, for callers
 * that cannot allocate device memory: hosts that own all device memory through
 * their own allocator or budget and do not let a plug-in call cudaMalloc
 * (which also synchronises the device), and FFI callers that reach only this C
 * ABI.  No counterpart in the reference.  Same arguments and result as
 * tg_conic_full_backprojector_deterministic, but the scratch is a fixed array
 * inside the library of tg_noalloc_scratch_bytes() bytes (32 MiB, held on
 * every GPU that loads the library until the process exits), which limits the
 * cube to (32 MiB - 256 B) / 8 = 4,194,272 voxels (n0*n1*n2, times the frame
 * count for TG_BPJT); larger cubes are rejected with TG_ENOMEM.  The first
 * call on a device looks up the scratch address (cudaGetSymbolAddress) with
 * that device current and keeps it for the life of the process, so make that
 * first call before any stream capture, and do not call this entry point on a
 * device after a cudaDeviceReset() of it (the kept address would then name
 * freed memory).  Every call
 * shares the scratch and clears it first: calls that overlap on the GPU
 * (different streams or host threads) race. */
size_t tg_noalloc_scratch_bytes(void);
tg_status tg_conic_full_backprojector_deterministic_noalloc(
    const tg_map_header *map_header, const tg_image_header *views, int32_t n_views, float *data, int64_t n1,
    int64_t n2, const int64_t data_strides[3], float *map, const int64_t map_shape[4],
    const int64_t map_strides[4], const void *mask, tg_dtype mask_dtype, const int64_t mask_strides[3],
    int32_t obstacle, int32_t mode, void *stream);

/* Number of voxel segments the f32 kernel accumulates along each ray, added
 * as float into counts (n1, n2, n_views) with strides count_strides[3].  A
 * diagnostic with no counterpart in the reference: it gives the exact
 * intersection count behind the throughput and roofline figures.  The cube is
 * described by its shape only (no cube data is read). */
tg_status tg_segment_counts(const tg_map_header *map_header, const tg_image_header *views, int32_t n_views,
                            float *counts, int64_t n1, int64_t n2, const int64_t count_strides[3],
                            const int64_t map_shape[3], const void *mask, tg_dtype mask_dtype,
                            const int64_t mask_strides[3], int32_t obstacle, void *stream);

/* out[0] = sum_i a[i] * b[i] over n float32 elements, accumulated in float64
 * with a fixed reduction order (bitwise reproducible).  The inner product of
 * the CG driver (TomograPy delegates CG to the external lo package,
 * tomograpy/srt.py:225); workspace of tg_dot_workspace_bytes() bytes. */
size_t tg_dot_workspace_bytes(void);
tg_status tg_dot_f32(const float *a, const float *b, int64_t n, double *out, void *workspace,
                     size_t workspace_bytes, void *stream);

/* ---- Packed multi-job launches --------------------------------------------
 * Many independent reconstructions traced by ONE kernel launch (no
 * counterpart in the reference, which runs one projector call per stack).
 * Describe each job with a tg_job, build a device plan once with
 * tg_packed_plan (jobs are ordered by decreasing work; the plan keeps the
 * device pointers, so reuse it while the buffers stay where they are), then
 * launch tg_packed_projector(plan, info, mode, ...) -- e.g. once per CG
 * iteration for every job.  rows_per_warp (1, 2 or 4) sets the CTA tile
 * height (8 * rows_per_warp rows x 32 columns); pick it by timing (see
 * tomograpy_gb300/batch.py). */
typedef struct {
  tg_map_header map_header;      /* cube header (host values) */
  const tg_image_header *views;  /* device view table */
  int32_t n_views;
  int32_t reserved;
  int64_t n1, n2;                /* image rows / columns */
  int64_t data_strides[3];
  int64_t map_shape[4];          /* map_shape[3] = frames (1 for 3-D) */
  int64_t map_strides[4];
  const void *mask;              /* NULL or device mask, type mask_dtype */
  int64_t mask_strides[3];
  int32_t mask_dtype;
  int32_t reserved2;
  float *data;                   /* device data stack (n1, n2, n_views) */
  float *map;                    /* device cube */
} tg_job;

typedef struct {
  int32_t n_jobs;
  int32_t rows_per_warp;
  int32_t four_d;
  int32_t idx64;
  int64_t tiles;                 /* CTAs of one packed launch */
  int64_t det_workspace_bytes;   /* workspace of tg_packed_backprojector_deterministic */
  int32_t det_idx64;             /* a job's accumulator needs 64-bit offsets */
  int32_t lane_axis;             /* schedule of the plan (see tg_schedule) */
  int32_t batch_steps;
  int32_t reserved;
} tg_packed_info;

/* Tile schedule of a packed plan (picked by timing, see
 * tomograpy_gb300/batch.py): rows_per_warp 1, 2 or 4; lane_axis 1 = a warp's
 * 32 lanes trace neighbouring pixels along image axis 1 (lambda; tiles of
 * 8*rows_per_warp rows x 32 columns), 0 = along image axis 0 (gamma; tiles of
 * 32 rows x 8*rows_per_warp columns), the better mapping when image axis 0
 * follows the cube's fastest axis; batch_steps 0 = the default walk batches,
 * 16 = 16-step batches.  Plans whose cube offsets need 64 bits always use
 * lane_axis 1, batch_steps 0 (info reports the schedule used). */
typedef struct {
  int32_t rows_per_warp;
  int32_t lane_axis;
  int32_t batch_steps;
  int32_t reserved;
} tg_schedule;

size_t tg_packed_plan_bytes(int32_t n_jobs);
tg_status tg_packed_plan(const tg_job *jobs, int32_t n_jobs, int32_t rows_per_warp, int32_t four_d, void *plan,
                         size_t plan_bytes, tg_packed_info *info);
/* Same plan written to host memory (no device work, no synchronisation): the
 * caller uploads it, e.g. with cudaMemcpyAsync from pinned memory on its
 * stream, so re-planning does not stall a stream that is busy. */
tg_status tg_packed_plan_host(const tg_job *jobs, int32_t n_jobs, int32_t rows_per_warp, int32_t four_d,
                              void *host_plan, size_t plan_bytes, tg_packed_info *info);
/* Plans with an explicit tile schedule (tg_packed_plan(rows_per_warp) is the
 * schedule {rows_per_warp, 1, 0}). */
tg_status tg_packed_plan_scheduled(const tg_job *jobs, int32_t n_jobs, const tg_schedule *schedule, int32_t four_d,
                                   void *plan, size_t plan_bytes, tg_packed_info *info);
tg_status tg_packed_plan_scheduled_host(const tg_job *jobs, int32_t n_jobs, const tg_schedule *schedule,
                                        int32_t four_d, void *host_plan, size_t plan_bytes, tg_packed_info *info);
tg_status tg_packed_projector(const void *plan, const tg_packed_info *info, int32_t mode, int32_t obstacle,
                              void *stream);
/* Deterministic packed backprojection (TG_BPJ, or TG_BPJT for a 4-D plan):
 * every job's cube gets, added in place, exactly the result of
 * tg_conic_full_backprojector_deterministic on that job alone (per-job
 * fixed-point scale, order-independent integer sums), so a job's result does
 * not depend on the other jobs of the plan.  Workspace:
 * info->det_workspace_bytes bytes, 256-byte aligned, cleared by the call.
 * No counterpart in the reference. */
tg_status tg_packed_backprojector_deterministic(const void *plan, const tg_packed_info *info, int32_t obstacle,
                                               void *workspace, size_t workspace_bytes, void *stream);

/* Segmented float64-accumulated inner products over float32 buffers:
 * out[s] = sum_{i in [seg[2s], seg[2s+1])} a[i] b[i] for s < n_seg (seg:
 * device int64[2 n_seg], element ranges that need not be contiguous or
 * ordered); fixed reduction order.  Workspace of
 * tg_segmented_workspace_bytes(n_seg) bytes. */
size_t tg_segmented_workspace_bytes(int32_t n_seg);
tg_status tg_segmented_dot_f32(const float *a, const float *b, const int64_t *seg, int32_t n_seg, double *out,
                               void *workspace, size_t workspace_bytes, void *stream);
/* Batched CG updates over the same segments, per segment s: alpha_s = rr[s] / pAp[s],
 * x += alpha_s p, r -= alpha_s Ap (tg_cg_update_x); beta_s = rr_new[s] / rr[s],
 * p = r + beta_s p, then rr[s] = rr_new[s] (tg_cg_update_p). */
tg_status tg_cg_update_x(float *x, float *r, const float *p, const float *Ap, const double *rr, const double *pAp,
                         const int64_t *seg, int32_t n_seg, void *stream);
tg_status tg_cg_update_p(float *p, const float *r, double *rr, const double *rr_new, const int64_t *seg,
                         int32_t n_seg, void *stream);

/* y = alpha x + beta y over the segments (x may be NULL: y = beta y; with
 * beta = 0, y = alpha x -- e.g. clearing a job's vectors or adding lam x). */
tg_status tg_segmented_axpby(float *y, const float *x, float alpha, float beta, const int64_t *seg, int32_t n_seg,
                             void *stream);

/* Device address of page-locked host memory (e.g. cudaHostAlloc'd, or a
 * pinned torch tensor) that the GPU can read and write directly over the
 * host link: a data stack there can be passed to the projectors without a
 * staging copy.  TG_EINVAL when the pointer is not such memory.  No
 * counterpart in the reference. */
tg_status tg_host_alias(const void *host, void **device);

/* Message for the last non-OK status returned on this thread. */
const char *tg_last_error(void);

/* ABI version (incremented on incompatible changes). */
int32_t tg_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* TOMOGRAPY_GB300_H */
