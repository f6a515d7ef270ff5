/*
 * ORACLE -- test infrastructure only.  Body of the CPU restatement of
 * TomograPy's Siddon conic projector, instantiated twice by siddon_oracle.c
 * (CT = double and CT = float, suffix SFX), the way the reference expands
 * tomograpy/C_siddon.c.template for ctype in {float, double}
 * (tomograpy/parse_templates.py:11,19-26).
 *
 * Every arithmetic step follows the reference's order of operations so that
 * the double instantiation reproduces the reference's double path bit for bit
 * (compile with -ffp-contract=off: the reference is compiled without FMA
 * contraction on x86-64).
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* Scalar-typed copies of the two headers (the reference casts every header
   value to CTYPE when it marshals them: tomograpy/C_siddon.c.template:1051-1101). */
typedef struct { CT p[3], d[3], min[3], max[3]; } FN(mapc_);
typedef struct { CT s[2], p[2], v[2], M[3], R[3][3]; } FN(imgc_);

static void FN(cast_map_)(const oracle_map_header *h, FN(mapc_) *m)
{
  for (int k = 0; k < 3; k++) {
    m->p[k] = (CT)h->cdelt[k];
    m->d[k] = (CT)h->pshape[k];
    m->min[k] = (CT)h->mmin[k];
    m->max[k] = (CT)h->mmax[k];
  }
}

static void FN(cast_img_)(const oracle_image_header *h, FN(imgc_) *g)
{
  for (int k = 0; k < 2; k++) {
    g->s[k] = (CT)h->crpix[k];
    g->p[k] = (CT)h->cdelt[k];
    g->v[k] = (CT)h->crval[k];
  }
  for (int k = 0; k < 3; k++) {
    g->M[k] = (CT)h->M[k];
    for (int l = 0; l < 3; l++) g->R[k][l] = (CT)h->R[3 * k + l];
  }
}

/* Pixel index -> angle: (i - CRPIX + 1) * CDELT + CRVAL
   (tomograpy/C_siddon.c.template:1043-1046). */
static CT FN(pixel_angle_)(unsigned int idx, int axis, const FN(imgc_) *g)
{
  return (idx - g->s[axis] + 1) * g->p[axis] + g->v[axis];
}

/* Ray direction u0 = R . (cos l cos g, cos l sin g, sin l), trig in double
   (libm), products in CT (tomograpy/C_siddon.c.template:1013-1032). */
static void FN(ray_direction_)(CT lam, CT gam, const FN(imgc_) *g, CT u0[3])
{
  CT u2[3];
  u2[0] = cos(lam) * cos(gam);
  u2[1] = cos(lam) * sin(gam);
  u2[2] = sin(lam);
  for (int k = 0; k < 3; k++)
    u0[k] = g->R[k][0] * u2[0] + g->R[k][1] * u2[1] + g->R[k][2] * u2[2];
}

/* Ray parameters of the MMIN / MMAX planes; +-INF stand-ins when the direction
   component is exactly zero (tomograpy/C_siddon.c.template:723-735). */
static void FN(face_params_)(const FN(mapc_) *m, const CT M[3], const CT u0[3], CT a1[3], CT an[3])
{
  for (int k = 0; k < 3; k++) {
    if (u0[k] != 0) {
      a1[k] = (m->min[k] - M[k]) / u0[k];
      an[k] = (m->max[k] - M[k]) / u0[k];
    } else {
      a1[k] = -ORACLE_INF;
      an[k] = ORACLE_INF;
    }
  }
}

/* Entry / exit parameters: max of per-axis minima, min of per-axis maxima, with
   the reference's tie rules (tomograpy/C_siddon.c.template:737-748,969-1011). */
static CT FN(max3_)(CT x, CT y, CT z)
{
  if (x > y && x > z) return x;
  if (y >= x && y > z) return y;
  return z;
}

static CT FN(min3_)(CT x, CT y, CT z)
{
  if (x < y && x < z) return x;
  if (y <= x && y < z) return y;
  return z;
}

static void FN(chord_)(const CT a1[3], const CT an[3], CT *amin, CT *amax)
{
  CT lo[3], hi[3];
  for (int k = 0; k < 3; k++) {
    if (a1[k] > an[k]) { lo[k] = an[k]; hi[k] = a1[k]; }
    else { lo[k] = a1[k]; hi[k] = an[k]; }
  }
  *amin = FN(max3_)(lo[0], lo[1], lo[2]);
  *amax = FN(min3_)(hi[0], hi[1], hi[2]);
}

/* Conversion used by the reference for voxel indices: (unsigned int)(x) of a
   truncated quotient, stored in an int.  Done through a 64-bit integer so the
   result is the same on every host (x86-64 semantics). */
static int FN(utrunc_)(CT x)
{
  return (int)(unsigned int)(long long)x;
}

typedef struct {
  int iv[3];      /* current voxel */
  int upd[3];     /* index step per axis: sign(u0) */
  CT D[3];        /* distance to the next plane of each family */
  CT pabs[3];     /* |CDELT / u0| : distance between planes of a family */
} FN(walk_);

/* Loop initialisation (tomograpy/C_siddon.c.template:564-573,750-809). */
static void FN(walk_init_)(const FN(mapc_) *m, const unsigned int n[3], const CT M[3],
                           const CT u0[3], const CT a1[3], CT amin, FN(walk_) *w)
{
  for (int k = 0; k < 3; k++) {
    CT p = (u0[k] != 0) ? m->p[k] / u0[k] : (CT)ORACLE_INF;
    w->pabs[k] = (CT)fabs(p);
    w->upd[k] = (u0[k] > 0) ? 1 : ((u0[k] < 0) ? -1 : 0);
    CT e = M[k] + amin * u0[k];
    CT ep = e - m->min[k];
    w->iv[k] = FN(utrunc_)(ep / m->p[k]);
    w->iv[k] -= FN(utrunc_)(ep / m->d[k]);
    unsigned int nx;
    if (w->upd[k] == 1) nx = (unsigned int)w->iv[k] + 1u;
    else if (w->upd[k] == -1) nx = (unsigned int)w->iv[k];
    else nx = (unsigned int)ORACLE_INF * n[k];
    w->D[k] = ((CT)nx) * p + a1[k] - amin;
  }
}

/* Strided element access of the caller's arrays. */
#define DATA_AT(i, j, t) (A->data[(long long)(i) * A->ds[0] + (long long)(j) * A->ds[1] + (long long)(t) * A->ds[2]])
#define MAP_AT(iv, f) (A->map[(long long)(iv)[0] * A->ms[0] + (long long)(iv)[1] * A->ms[1] + \
                              (long long)(iv)[2] * A->ms[2] + (long long)(f) * A->ms[3]])

typedef struct {
  CT *data; long long ds[3];
  CT *map; long long ms[4]; unsigned int n[3];
  const CT *mask; long long ks[3];
  int mode, obstacle;
} FN(args_);

/* One segment of length d through voxel iv of ray (i, j, t): the four
   accumulate kernels pj / bpj / pjt / bpjt (tomograpy/C_siddon.c.template:914-944).
   The 4-D variants index the cube's 4th axis with the view index t. */
static void FN(segment_)(const FN(args_) *A, unsigned int i, unsigned int j, unsigned int t,
                         const int iv[3], CT d)
{
  switch (A->mode) {
  case ORACLE_PJ:
    DATA_AT(i, j, t) += d * MAP_AT(iv, 0);
    break;
  case ORACLE_BPJ: {
    CT v = d * DATA_AT(i, j, t);
#pragma omp atomic
    MAP_AT(iv, 0) += v;
    break;
  }
  case ORACLE_PJT:
    DATA_AT(i, j, t) += d * MAP_AT(iv, t);
    break;
  default: { /* ORACLE_BPJT */
    CT v = d * DATA_AT(i, j, t);
#pragma omp atomic
    MAP_AT(iv, t) += v;
    break;
  }
  }
}

/* Squared distance of the point at ray parameter ac to the cube origin, and the
   "sun" obstacle test d > 1 (tomograpy/C_siddon.c.template:955-961,1034-1041). */
static int FN(outside_sun_)(const CT M[3], const CT u0[3], CT ac)
{
  CT d = (M[0] + ac * u0[0]) * (M[0] + ac * u0[0]);
  d += (M[1] + ac * u0[1]) * (M[1] + ac * u0[1]);
  d += (M[2] + ac * u0[2]) * (M[2] + ac * u0[2]);
  return d > 1;
}

/* Trace one ray (tomograpy/C_siddon.c.template:530-580 and the merge step
   voxel(), :811-912).  The merge takes the smallest of the three plane
   distances; every family that ties with it advances in the same step, which
   is exactly the reference's seven-way case analysis for non-NaN distances.
   The step count is capped at the number of planes the ray can cross so that a
   NaN header cannot make the loop spin. */
static void FN(trace_ray_)(const FN(args_) *A, const FN(mapc_) *m, const CT M[3], const CT u0[3],
                           unsigned int i, unsigned int j, unsigned int t)
{
  CT a1[3], an[3], amin = 0, amax = 0;
  FN(face_params_)(m, M, u0, a1, an);
  FN(chord_)(a1, an, &amin, &amax);
  if (!(amin < amax)) return;
  FN(walk_) w;
  FN(walk_init_)(m, A->n, M, u0, a1, amin, &w);
  CT ac = amin;
  long long cap = (long long)A->n[0] + A->n[1] + A->n[2] + 8;
  while (cap-- > 0) {
    if (!(w.iv[0] >= 0 && (unsigned int)w.iv[0] < A->n[0] &&
          w.iv[1] >= 0 && (unsigned int)w.iv[1] < A->n[1] &&
          w.iv[2] >= 0 && (unsigned int)w.iv[2] < A->n[2]))
      break;
    if (A->obstacle == ORACLE_SUN && !FN(outside_sun_)(M, u0, ac)) break;
    CT dmin = w.D[0];
    if (w.D[1] < dmin) dmin = w.D[1];
    if (w.D[2] < dmin) dmin = w.D[2];
    if (dmin != dmin) break; /* NaN */
    ac += dmin;
    FN(segment_)(A, i, j, t, w.iv, dmin);
    int hit[3];
    for (int k = 0; k < 3; k++) hit[k] = (w.D[k] == dmin);
    for (int k = 0; k < 3; k++) {
      if (hit[k]) {
        w.iv[k] += w.upd[k];
      } else {
        w.D[k] -= dmin;
      }
    }
    for (int k = 0; k < 3; k++)
      if (hit[k]) w.D[k] = w.pabs[k];
  }
}

/* All pixels of one view (tomograpy/C_siddon.c.template:500-528): a pixel is
   traced when its mask value is exactly zero. */
static void FN(trace_view_)(const FN(args_) *A, const FN(mapc_) *m, const FN(imgc_) *g,
                            unsigned int n1, unsigned int n2, unsigned int t)
{
  for (unsigned int i = 0; i < n1; i++) {
    CT gam = FN(pixel_angle_)(i, 0, g);
    for (unsigned int j = 0; j < n2; j++) {
      if (A->mask && A->mask[(long long)i * A->ks[0] + (long long)j * A->ks[1] + (long long)t * A->ks[2]] != 0)
        continue;
      CT lam = FN(pixel_angle_)(j, 1, g);
      CT u0[3];
      FN(ray_direction_)(lam, gam, g, u0);
      FN(trace_ray_)(A, m, g->M, u0, i, j, t);
    }
  }
}

/* Full projector over T views, OpenMP over views with num_threads(nthread)
   (0 = runtime default), as conic_full_projector
   (tomograpy/C_siddon.c.template:460-498). */
int FN(oracle_conic_full_projector_)(const oracle_map_header *mh, const oracle_image_header *views,
                                     int T, CT *data, long long n1, long long n2, const long long ds[3],
                                     CT *map, const long long mshape[3], const long long ms[4],
                                     const CT *mask, const long long ks[3],
                                     int obstacle, int mode, int nthread)
{
  if (!mh || !views || !data || !map || T < 0 || n1 < 0 || n2 < 0) return ORACLE_EINVAL;
  if (mode < ORACLE_PJ || mode > ORACLE_BPJT) return ORACLE_EINVAL;
  FN(args_) A;
  A.data = data; A.map = map; A.mask = mask;
  for (int k = 0; k < 3; k++) {
    A.ds[k] = ds[k];
    A.ms[k] = ms[k];
    A.n[k] = (unsigned int)mshape[k];
    A.ks[k] = mask ? ks[k] : 0;
  }
  A.ms[3] = ms[3];
  A.mode = mode;
  A.obstacle = obstacle;
  FN(mapc_) m;
  FN(cast_map_)(mh, &m);
  int t;
#pragma omp parallel for num_threads(nthread > 0 ? nthread : omp_get_max_threads()) schedule(static)
  for (t = 0; t < T; t++) {
    FN(imgc_) g;
    FN(cast_img_)(&views[t], &g);
    FN(trace_view_)(&A, &m, &g, (unsigned int)n1, (unsigned int)n2, (unsigned int)t);
  }
  return ORACLE_OK;
}

/* Diagnostic twins: per-pixel unit vectors, skipping NaN data pixels
   (tomograpy/C_siddon.c.template:582-648), written into u[i,j,t,k]. */
int FN(oracle_full_unit_vector_)(const oracle_image_header *views, int T, const CT *data,
                                 long long n1, long long n2, const long long ds[3],
                                 double *u, const long long us[4])
{
  for (int t = 0; t < T; t++) {
    FN(imgc_) g;
    FN(cast_img_)(&views[t], &g);
    for (unsigned int i = 0; i < (unsigned int)n1; i++) {
      CT gam = FN(pixel_angle_)(i, 0, &g);
      for (unsigned int j = 0; j < (unsigned int)n2; j++) {
        CT v = data[(long long)i * ds[0] + (long long)j * ds[1] + (long long)t * ds[2]];
        if (v != v) continue;
        CT lam = FN(pixel_angle_)(j, 1, &g);
        CT u0[3];
        FN(ray_direction_)(lam, gam, &g, u0);
        for (int k = 0; k < 3; k++)
          u[(long long)i * us[0] + (long long)j * us[1] + (long long)t * us[2] + k * us[3]] = u0[k];
      }
    }
  }
  return ORACLE_OK;
}

/* a1 / an of every pixel from given unit vectors
   (tomograpy/C_siddon.c.template:650-720). */
int FN(oracle_full_intersection_parameters_)(const oracle_map_header *mh, const oracle_image_header *views,
                                             int T, long long n1, long long n2, const double *u,
                                             const long long us[4], double *a1, double *an)
{
  FN(mapc_) m;
  FN(cast_map_)(mh, &m);
  for (int t = 0; t < T; t++) {
    FN(imgc_) g;
    FN(cast_img_)(&views[t], &g);
    for (long long i = 0; i < n1; i++)
      for (long long j = 0; j < n2; j++) {
        CT u0[3], b1[3], bn[3];
        long long o = i * us[0] + j * us[1] + t * us[2];
        for (int k = 0; k < 3; k++) u0[k] = (CT)u[o + k * us[3]];
        FN(face_params_)(&m, g.M, u0, b1, bn);
        for (int k = 0; k < 3; k++) {
          a1[o + k * us[3]] = b1[k];
          an[o + k * us[3]] = bn[k];
        }
      }
  }
  return ORACLE_OK;
}

#undef DATA_AT
#undef MAP_AT
#undef FN
#undef CAT
#undef CAT_
