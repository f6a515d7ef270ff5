// Fast single-precision Siddon projector / backprojector for sm_103a.
//
// Work mapping: one thread per detector ray.  A CTA is kFastRows rows x 32
// columns of one view; a warp traces 32 consecutive pixels of a row at a time,
// i.e. 32 rays that are neighbours along image axis 1 (lambda).  For observers near the
// solar equator that axis maps to the cube's fastest axis, so at a given step
// the warp's lanes read / update neighbouring voxels of one cube row and the
// whole warp walks the same (x, y) voxel sequence in lock step.  (The packed
// kernel can also run lanes along image axis 0, see tile_body.)
//
// Arithmetic (the reference does everything in its C type,
// tomograpy/C_siddon.c.template:530-580,811-912):
//  * per-ray set-up in double-float (pairs of floats, FMA-based error-free
//    products) from per-CTA tables computed in double precision: direction
//    cos l * (A_row + tan l * R[:, 2]) with A_row = R . (cos g, sin g, 0),
//    entry parameter, entry point (the two ~d-sized terms cancel to ~1e-11),
//    entry voxel by a floor division against the exact plane positions, the
//    remainder and the first crossing of each family (a float remainder
//    divided by a small |w| would misplace a nearly parallel family's
//    crossings), and the crossing spacing CDELT / |w|.  Single precision only
//    classifies the
//    ray (miss / clear entry face); the full double-precision reference
//    set-up (siddon_geom.cuh) runs when that classification is within its
//    error bound;
//  * the voxel walk in single precision, measured from the chord's midpoint:
//    the k-th plane crossing of family a is t = d_a + k * |p_a| (one FMA)
//    with k counted from the crossing nearest the midpoint, so crossing
//    positions carry no accumulated drift, their rounding scales with the
//    distance from the midpoint, and the catastrophic cancellation of the
//    reference's float path (D[k] = next*p + a1 - amin with a1, amin ~ 215)
//    never occurs.  Steps run in batches that are proven, by one bound, to
//    start before the stop parameter, so a batch needs no per-step test and
//    its gathers / atomics are issued together; inside a batch the crossings
//    advance by running sums (one add) in a frame local to the batch and are
//    recomputed exactly after it (24-step batches; 32 for projections over
//    cubes of at least 256 voxels per axis);
//  * the "sun" obstacle: the reference tests |M + ac u|^2 > 1 at every voxel
//    entry (:575).  Here the walk runs unchecked up to the sphere-entry
//    parameter minus an error bound; from there on every voxel entry is tested
//    in single precision relative to the entry point, and in double precision
//    (the reference's formula) when the single-precision value is within its
//    error bound of the sphere.
//  * exit: the reference stops when the voxel index leaves the cube (in_map,
//    :948-953).  Equivalently the walk stops at the first crossing that takes an
//    index out of range; its parameter is computed with the same FMA as the
//    walk, so the comparison is exact.
#pragma once

#include "siddon_geom.cuh"

namespace tg {

// Compile-time tuning per direction (measured on GB300 at 256^3 x 360 x 512^2).
// Both walk in drift batches (running-sum crossings, exact resynchronisation
// per batch) at 4 CTAs per SM (64 registers); the projection issues each
// step's gather as the step is known and adds it to the batch's sum
// TG_PJ_LAG steps later, so only that window of values is live, the
// backprojection issues each atomic at once.
#ifndef TG_PJ_BATCH
#define TG_PJ_BATCH 24
#endif
#ifndef TG_PJ_MIN_BLOCKS
#define TG_PJ_MIN_BLOCKS 4
#endif
// projection: a batch's gathered values are summed TG_PJ_LAG steps behind the
// walk (the gather of step s is consumed at step s + TG_PJ_LAG)
#ifndef TG_PJ_LAG
#define TG_PJ_LAG 8
#endif
// projection over fine cubes (every axis at least TG_PJ_FINE_MIN_N voxels):
// longer batches.  A batch's running sums drift by ~B ulps of its extent
// (~B voxel widths), so a pixel's relative error grows like B^2 / n for n
// voxels along the ray: 32-step batches measured 1.3e-5 per-pixel at 64^3
// x 128^2 (24-step: 6.5e-6) and 6.7e-6 at 256^3 x 512^2 (24-step: 4.8e-6).
// They pay off on long rays only: 15.75 -> 15.37 ms at 256^3 x 360 x 512^2,
// but 5.50 -> 5.58 ms for 128^3 x 28 frames x 784 x 256^2.
#ifndef TG_PJ_FINE_BATCH
#define TG_PJ_FINE_BATCH 32
#endif
#ifndef TG_PJ_FINE_MIN_N
#define TG_PJ_FINE_MIN_N 256
#endif
#ifndef TG_BPJ_BATCH
#define TG_BPJ_BATCH 24
#endif
#ifndef TG_BPJ_MIN_BLOCKS
#define TG_BPJ_MIN_BLOCKS 4
#endif
#ifndef TG_PJ_SHORT_BATCH
#define TG_PJ_SHORT_BATCH 4
#endif
#ifndef TG_BPJ_SHORT_BATCH
#define TG_BPJ_SHORT_BATCH 1
#endif
#ifndef TG_PJ_DRIFT
#define TG_PJ_DRIFT 1
#endif
#ifndef TG_BPJ_DRIFT
#define TG_BPJ_DRIFT 1
#endif
__host__ __device__ constexpr bool is_backprojection(int mode) { return mode == TG_BPJ || mode == TG_BPJT; }
// running-sum crossings inside batches (drift_step), per direction
__host__ __device__ constexpr bool drift_batches(int mode) {
  return is_backprojection(mode) ? TG_BPJ_DRIFT : TG_PJ_DRIFT;
}
// steps per batch of independent gathers / atomics
__host__ __device__ constexpr int batch_steps(int mode) { return is_backprojection(mode) ? TG_BPJ_BATCH : TG_PJ_BATCH; }
// CTAs per SM the register budget must allow
__host__ __device__ constexpr int min_blocks(int mode) {
  return is_backprojection(mode) ? TG_BPJ_MIN_BLOCKS : TG_PJ_MIN_BLOCKS;
}
constexpr float kSunTh = 1e-5f;            // single-precision |d - 1| decision threshold

struct DetScale {                          // deterministic-mode scale factors (device)
  float yscale;                            // power of two bringing max|y| into [0.5, 1)
  float qscale;                            // power of two: fixed-point unit
  double out_scale;                        // 1 / (yscale * qscale)
  unsigned int ymax_bits;
  unsigned int pad;
};

// Per-CTA tables.  A ray's direction R . (cos l cos g, cos l sin g, sin l) is
// cos l * w with w = A_row + tan(l) R[:, 2], A_row = R . (cos g, sin g, 0);
// the fast walk runs in the scaled parameter beta = alpha cos l along w and
// rescales lengths by 1 / cos l.  A (per row) and tan l (per column) are
// computed once per CTA in double precision and kept as hi + lo float pairs,
// so the per-ray set-up is double-float arithmetic on the FP32 pipes.
struct FastTables {
  double cl[32], sl[32];               // cos / sin lambda per column
  float th[32], tl[32];                // tan(lambda), hi + lo
  float icl[32];                       // 1 / cos(lambda)
  double A[kFastRows][3];              // R . (cos g, sin g, 0) per row
  float ah[kFastRows][3], al[kFastRows][3];    // A, hi + lo
  float B[3], Bl[3];                   // R[:, 2], hi + lo
  float mh[3], ml[3];                  // M - MMIN, hi + lo
  float fh[3][2], fl[3][2];            // F - M for the MMIN (0) / MMAX (1) face, hi + lo
};

// Double-float helpers (pairs hi + lo of floats; error-free products by FMA).
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_from(float a, float b) {  // renormalise a + b
  const float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_from(p, e);
}

__device__ __forceinline__ df df_add(df a, df b) {
  const float s = a.hi + b.hi;
  const float v = s - a.hi;
  const float e = (a.hi - (s - v)) + (b.hi - v);  // two-sum error
  return df_from(s, e + a.lo + b.lo);
}

__device__ __forceinline__ df df_rcp(df a) {  // 1 / a to ~2^-46
  const float r = __frcp_rn(a.hi);
  const float e = fmaf(-a.lo, r, fmaf(-a.hi, r, 1.f));
  return df_from(r, r * e);
}

__device__ __forceinline__ double split_lo(double v, float hi) { return v - (double)hi; }

__device__ __forceinline__ void fill_fast_tables(FastTables &T, const Geometry &G, const tg_image_header &V,
                                                 int col0, int row0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
    double s, c;
    sincos(pixel_angle(col0 + lane, V, 1), &s, &c);
    T.sl[lane] = s;
    T.cl[lane] = c;
    const double tau = s / c;
    T.th[lane] = (float)tau;
    T.tl[lane] = (float)split_lo(tau, T.th[lane]);
    T.icl[lane] = __frcp_rn((float)c);
    if (lane < 3) {
      const double B = V.R[3 * lane + 2];
      T.B[lane] = (float)B;
      T.Bl[lane] = (float)split_lo(B, T.B[lane]);
      const double mm = V.M[lane] - G.mh.mmin[lane];
      T.mh[lane] = (float)mm;
      T.ml[lane] = (float)split_lo(mm, T.mh[lane]);
      const double f0 = G.mh.mmin[lane] - V.M[lane], f1 = G.mh.mmax[lane] - V.M[lane];
      T.fh[lane][0] = (float)f0;
      T.fl[lane][0] = (float)split_lo(f0, T.fh[lane][0]);
      T.fh[lane][1] = (float)f1;
      T.fl[lane][1] = (float)split_lo(f1, T.fh[lane][1]);
    }
  } else if (warp == 1 && lane < kFastRows) {
    double sg, cg;
    sincos(pixel_angle(row0 + lane, V, 0), &sg, &cg);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double A = __dadd_rn(__dmul_rn(V.R[3 * k], cg), __dmul_rn(V.R[3 * k + 1], sg));
      T.A[lane][k] = A;
      T.ah[lane][k] = (float)A;
      T.al[lane][k] = (float)split_lo(A, T.ah[lane][k]);
    }
  }
}

// State of one ray's walk in the single-precision relative frame.
template <typename IDX>
struct Walk {
  float t[3];   // next crossing of each plane family (walk parameter)
  float d[3];   // crossing m = 0 of each family (the one nearest the chord midpoint)
  float pa[3];  // spacing of crossings
  float m[3];   // index of the next crossing, counted from that one (exact integers)
  int iv0[3];   // voxel index that goes with m = 0
  int upd[3];
  IDX st[3];    // offset change when crossing a plane of each family
  IDX off;      // current voxel offset
  float texit;  // parameter of the first crossing that leaves the cube
  float E[3];   // entry point (absolute)
  float uf[3];  // direction of the walk parameter (w, or u on the exact path)
  float lscale; // walk-parameter length -> path length (1 / cos l, or 1)
  float t0;     // walk origin: parameters are measured from the chord midpoint
};

// The ray direction u in double precision (exact path and obstacle
// confirmation): u = cos l A_row + sin l R[:, 2], components below 1e-14
// taken as zero.
__device__ __forceinline__ void ray_u(const FastTables &T, const tg_image_header &V, int lane, int slot,
                                      double u[3]) {
  const double cl = T.cl[lane], sl = T.sl[lane];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    u[k] = fma(cl, T.A[slot][k], sl * V.R[3 * k + 2]);
    if (fabs(u[k]) < kSnapZero) u[k] = 0.0;
  }
}

// Result of the exact (double-precision reference) set-up.
struct ExactSetup {
  int iv[3], upd[3];
  float d[3], pa[3], uf[3], ef[3];
  float dl[3], pl[3];  // low parts: D = d + dl, |p| = pa + pl
};

// Full double-precision reference set-up (ambiguous rays): walk in alpha.
// Kept out of line and writing to its own struct, so the walk state of the
// common path stays in registers.
static __device__ __noinline__ bool exact_setup(const Geometry &G, const tg_image_header &V, const FastTables &T,
                                                int lane, int slot, ExactSetup &X) {
  const float kInf = __int_as_float(0x7f800000);
  double u[3];
  ray_u(T, V, lane, slot, u);
  const double M[3] = {V.M[0], V.M[1], V.M[2]};
  RefWalk rw;
  if (!ref_setup(G.mh, G.n, M, u, rw)) return false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    X.iv[k] = rw.iv[k];
    X.upd[k] = rw.upd[k];
    X.d[k] = X.upd[k] ? (float)rw.D[k] : kInf;
    X.pa[k] = X.upd[k] ? (float)rw.pabs[k] : kInf;
    X.dl[k] = X.upd[k] ? (float)(rw.D[k] - (double)X.d[k]) : 0.f;
    X.pl[k] = X.upd[k] ? (float)(rw.pabs[k] - (double)X.pa[k]) : 0.f;
    X.uf[k] = (float)u[k];
    X.ef[k] = (float)__dsub_rn(__dadd_rn(M[k], __dmul_rn(rw.amin, u[k])), G.mh.mmin[k]);
  }
  return true;
}

// Per-ray set-up.  Returns false when the ray does not enter the cube (the
// reference's loop would not run).  `sun_lo` receives the parameter up to which
// no obstacle test is needed (+inf when the ray cannot reach the sphere).
template <bool SUN, typename IDX>
__device__ __forceinline__ bool setup_ray(const Geometry &G, const tg_image_header &V, const FastTables &T,
                                          int lane, int slot, Walk<IDX> &w, float &sun_lo) {
  const float kInf = __int_as_float(0x7f800000);
  const df tau = {T.th[lane], T.tl[lane]};
  df wd[3];  // w in double-float
  float lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    wd[k] = df_add({T.ah[slot][k], T.al[slot][k]}, df_mul(tau, {T.B[k], T.Bl[k]}));
    float wk = wd[k].hi;
    if (fabsf(wk) < 1e-14f) {  // in-plane (or within 1e-14 rad of it)
      wk = 0.f;
      wd[k] = {0.f, 0.f};
    }
    w.uf[k] = wk;
    if (wk != 0.f) {
      const float inv = __frcp_rn(wk);
      const float a = T.fh[k][0] * inv;
      const float b = T.fh[k][1] * inv;
      lo[k] = fminf(a, b);
      hi[k] = fmaxf(a, b);
    } else {
      lo[k] = -1e5f;
      hi[k] = 1e5f;
    }
  }
  int kin = 0;
  float aminf = lo[0];
  if (lo[1] > aminf) {
    kin = 1;
    aminf = lo[1];
  }
  if (lo[2] > aminf) {
    kin = 2;
    aminf = lo[2];
  }
  const float second = fmaxf(kin == 0 ? lo[1] : lo[0], kin == 2 ? lo[1] : lo[2]);
  const float amaxf = fminf(hi[0], fminf(hi[1], hi[2]));
  const float tol = 4e-6f * (fabsf(aminf) + fabsf(amaxf)) + 1e-6f;
  if (amaxf - aminf < -tol) return false;  // clear miss
  int iv[3];
  float ef[3];  // entry point relative to MMIN
  float pl[3], dl[3];  // low parts of the crossing spacing and of the first crossing
  const float ukin = (kin == 0) ? w.uf[0] : ((kin == 1) ? w.uf[1] : w.uf[2]);
  if (amaxf - aminf < tol || aminf - second < tol || ukin == 0.f) {
    ExactSetup X;
    if (!exact_setup(G, V, T, lane, slot, X)) return false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      iv[k] = X.iv[k];
      w.upd[k] = X.upd[k];
      w.d[k] = X.d[k];
      w.pa[k] = X.pa[k];
      pl[k] = X.pl[k];
      dl[k] = X.dl[k];
      w.uf[k] = X.uf[k];
      ef[k] = X.ef[k];
    }
    w.lscale = 1.f;
  } else {
    // All arrays below are indexed with compile-time indices only (unrolled
    // loops with k == kin tests): a run-time index would move the walk state
    // to local memory.
    w.lscale = T.icl[lane];
    float wk = 0.f, fh = 0.f, fl = 0.f;
    df wkd = {0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (k == kin) {
        wk = w.uf[k];
        wkd = wd[k];
        fh = (wk > 0.f) ? T.fh[k][0] : T.fh[k][1];
        fl = (wk > 0.f) ? T.fl[k][0] : T.fl[k][1];
      }
    }
    // beta_in = (F - M_kin) / w_kin in double-float (F = MMIN if w > 0 else MMAX)
    const df bin = df_mul({fh, fl}, df_rcp(wkd));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      w.upd[k] = (w.uf[k] > 0.f) ? 1 : ((w.uf[k] < 0.f) ? -1 : 0);
      // |p| = CDELT / |w| in double-float: its rounding would otherwise shift
      // every crossing of the family by a fraction 2^-24 of its distance
      // from the entry point
      w.pa[k] = kInf;
      pl[k] = 0.f;
      dl[k] = 0.f;
      df iaw = {0.f, 0.f};  // 1 / |w_k|, double-float
      if (w.upd[k]) {
        const df aw = (wd[k].hi > 0.f) ? wd[k] : df{-wd[k].hi, -wd[k].lo};
        iaw = df_rcp(aw);
        const df pd = df_mul({G.cdeltf[k], G.cdeltl[k]}, iaw);
        w.pa[k] = pd.hi;
        pl[k] = pd.lo;
      }
      if (k == kin) {
        iv[k] = (wk > 0.f) ? 0 : G.n[k] - 1;
        w.d[k] = w.pa[k];
        dl[k] = pl[k];
        ef[k] = (wk > 0.f) ? 0.f : (float)G.mh.pshape[k];
      } else if (w.upd[k] == 0) {
        // In-plane ray: the index holds for the whole chord, so it is taken
        // exactly as the reference computes it (:783-786).
        const double ep = __dsub_rn(V.M[k], G.mh.mmin[k]);
        iv[k] = ref_utrunc(__ddiv_rn(ep, G.mh.cdelt[k])) - ref_utrunc(__ddiv_rn(ep, G.mh.pshape[k]));
        w.d[k] = kInf;
        ef[k] = (float)ep;
      } else {
        // E_k - MMIN_k = (M_k - MMIN_k) + beta_in w_k in double-float (the
        // cancellation of the two ~d-sized terms leaves ~1e-11 radii), then
        // the remainder against the exact plane position q * CDELT.
        const df e = df_add({T.mh[k], T.ml[k]}, df_mul(bin, wd[k]));
        const df C = {G.cdeltf[k], G.cdeltl[k]};
        const df mC = {-C.hi, -C.lo};
        const float q = floorf((e.hi + e.lo) * G.inv_cdeltf[k]);
        // remainder r = e - q CDELT, kept in double-float: the distance to
        // the next plane is r / |w|, and for a ray nearly parallel to the
        // family (|w| ~ 1e-4 .. 1e-5) a float remainder (one ulp of CDELT,
        // ~1e-9 radii) would shift that crossing by ~1e-5, which showed as
        // per-voxel errors of 3e-4 on sparse backprojections
        const df qc = df_mul({q, 0.f}, C);
        df r = df_add(e, {-qc.hi, -qc.lo});
        int qi = (int)q;
        if (r.hi < 0.f || (r.hi == 0.f && r.lo < 0.f)) {
          qi -= 1;
          r = df_add(r, C);
        } else {
          const df rc = df_add(r, mC);
          if (rc.hi > 0.f || (rc.hi == 0.f && rc.lo >= 0.f)) {
            qi += 1;
            r = rc;
          }
        }
        // the reference truncates: a point just outside the first / last
        // voxel still maps to it (:785-786)
        if (qi == -1) {
          qi = 0;
          r = df_add(r, mC);
        } else if (qi == G.n[k]) {
          qi = G.n[k] - 1;
          r = df_add(r, C);
        }
        iv[k] = qi;
        // parameter of the first crossing: (CDELT - r) / w or r / -w
        const df dd = df_mul((w.upd[k] > 0) ? df_add(C, {-r.hi, -r.lo}) : r, iaw);
        w.d[k] = dd.hi;
        dl[k] = dd.lo;
        ef[k] = e.hi + e.lo;
      }
    }
  }
  float texit0 = kInf;
  float ce[3];  // crossings of each family until its index leaves the cube
  IDX off = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (iv[k] < 0 || iv[k] >= G.n[k]) return false;  // reference: in_map fails at once
    w.iv0[k] = iv[k];
    w.m[k] = 0.f;
    w.st[k] = (IDX)w.upd[k] * (IDX)G.ms[k];
    off += (IDX)iv[k] * (IDX)G.ms[k];
    ce[k] = (float)((w.upd[k] > 0) ? G.n[k] - iv[k] : iv[k] + 1);
    if (w.upd[k] != 0) texit0 = fminf(texit0, fmaf(ce[k] - 1.f, w.pa[k], w.d[k]));
    w.E[k] = G.mminf[k] + ef[k];
  }
  w.off = off;
  // Re-origin the walk at the chord's midpoint h, and count each family's
  // crossings from the one nearest to it (m0): crossing m of family a is
  // then t = fma(m - m0, p, d'') with d'' = D + m0 (p + pl) - h evaluated
  // with an exact product (|d''| <= |p|), so a crossing's rounding error
  // scales with its distance from the midpoint instead of from the entry
  // point.  The exit parameter is computed from the same values with the
  // walk's own FMA, so the stop stays exact.
  const float h = 0.5f * texit0;
  w.t0 = -h;
  float texit = kInf;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    w.t[k] = kInf;
    if (w.upd[k] != 0) {
      const float m0 = fminf(fmaxf(rintf(__fdividef(h - w.d[k], w.pa[k])), 0.f), ce[k] - 1.f);
      const float p = m0 * w.pa[k];
      const float e = fmaf(m0, w.pa[k], -p) + fmaf(m0, pl[k], dl[k]);
      w.d[k] = ((p - h) + e) + w.d[k];
      w.m[k] = -m0;
      w.iv0[k] += w.upd[k] * (int)m0;
      w.t[k] = fmaf(-m0, w.pa[k], w.d[k]);
      texit = fminf(texit, fmaf(ce[k] - 1.f - m0, w.pa[k], w.d[k]));
    }
  }
  w.texit = texit;
  sun_lo = kInf;
  if (SUN) {
    // |E + s dir|^2 = 1:  s^2 |dir|^2 + 2 s (E.dir) + |E|^2 - 1 = 0
    const float ww = fmaf(w.uf[0], w.uf[0], fmaf(w.uf[1], w.uf[1], w.uf[2] * w.uf[2]));
    const float b = fmaf(w.E[0], w.uf[0], fmaf(w.E[1], w.uf[1], w.E[2] * w.uf[2]));
    const float c = fmaf(w.E[0], w.E[0], fmaf(w.E[1], w.E[1], w.E[2] * w.E[2])) - 1.f;
    const float disc = fmaf(b, b, -ww * c);
    if (c < 1e-4f) {
      sun_lo = -kInf;  // entry at / inside the sphere: test from the start
    } else if (b < 0.f && disc > -2e-5f * ww) {
      const float sq = sqrtf(fmaxf(disc, 0.f));
      const float s1 = __fdividef(-b - sq, ww);
      const float g = 1e-5f + __fdividef(1e-5f, sq);
      sun_lo = (sq > 0.f) ? s1 - g - h : -kInf;
    }
  }
  return true;
}

// Double-precision decision of the obstacle test at the entry of voxel iv
// (the reference's |M + ac u0|^2 > 1 with ac the entry parameter of the
// voxel): the entry parameter is the largest of the crossing parameters of the
// voxel's lower planes along the ray.
static __device__ __noinline__ bool exact_outside(const Geometry &G, const tg_image_header &V, const FastTables &T,
                                                  int lane, int slot, const int iv[3]) {
  double u[3];
  ray_u(T, V, lane, slot, u);
  const double M[3] = {V.M[0], V.M[1], V.M[2]};
  double ac = -1e300;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (u[k] == 0.0) continue;
    const int plane = (u[k] > 0.0) ? iv[k] : iv[k] + 1;
    const double P = __dadd_rn(G.mh.mmin[k], __dmul_rn((double)plane, G.mh.cdelt[k]));
    ac = fmax(ac, __ddiv_rn(__dsub_rn(P, M[k]), u[k]));
  }
  return ref_outside_sun(M, u, ac);
}

// One step of the walk: returns the segment length and the voxel offset it
// belongs to, and advances the state.  Every plane family whose next crossing
// equals the smallest advances (the reference's 2- and 3-way tie cases).
// Smallest of three floats in one instruction (PTX three-input min, sm_100+);
// a NaN operand is ignored like fminf does.
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Family advances are written as predicated PTX: per family one compare and
// predicated updates that share its predicate (the three compares read the
// crossings before any update, as in the reference's tie cases).
//
// Exact advance: every family whose next crossing equals tm takes its next
// crossing fma(m + 1, p, d), and the voxel offset moves by its stride.
template <typename IDX>
__device__ __forceinline__ void advance_exact(Walk<IDX> &w, float tm) {
  if constexpr (sizeof(IDX) == 4) {
    asm("{\n\t.reg .pred p0, p1, p2;\n\t"
        "setp.eq.f32 p0, %0, %7;\n\t"
        "setp.eq.f32 p1, %1, %7;\n\t"
        "setp.eq.f32 p2, %2, %7;\n\t"
        "@p0 add.f32 %3, %3, 0f3F800000;\n\t"
        "@p1 add.f32 %4, %4, 0f3F800000;\n\t"
        "@p2 add.f32 %5, %5, 0f3F800000;\n\t"
        "@p0 fma.rn.f32 %0, %3, %8, %11;\n\t"
        "@p1 fma.rn.f32 %1, %4, %9, %12;\n\t"
        "@p2 fma.rn.f32 %2, %5, %10, %13;\n\t"
        "@p0 add.s32 %6, %6, %14;\n\t"
        "@p1 add.s32 %6, %6, %15;\n\t"
        "@p2 add.s32 %6, %6, %16;\n\t}"
        : "+f"(w.t[0]), "+f"(w.t[1]), "+f"(w.t[2]), "+f"(w.m[0]), "+f"(w.m[1]), "+f"(w.m[2]), "+r"(w.off)
        : "f"(tm), "f"(w.pa[0]), "f"(w.pa[1]), "f"(w.pa[2]), "f"(w.d[0]), "f"(w.d[1]), "f"(w.d[2]), "r"(w.st[0]),
          "r"(w.st[1]), "r"(w.st[2]));
  } else {
    asm("{\n\t.reg .pred p0, p1, p2;\n\t"
        "setp.eq.f32 p0, %0, %7;\n\t"
        "setp.eq.f32 p1, %1, %7;\n\t"
        "setp.eq.f32 p2, %2, %7;\n\t"
        "@p0 add.f32 %3, %3, 0f3F800000;\n\t"
        "@p1 add.f32 %4, %4, 0f3F800000;\n\t"
        "@p2 add.f32 %5, %5, 0f3F800000;\n\t"
        "@p0 fma.rn.f32 %0, %3, %8, %11;\n\t"
        "@p1 fma.rn.f32 %1, %4, %9, %12;\n\t"
        "@p2 fma.rn.f32 %2, %5, %10, %13;\n\t"
        "@p0 add.s64 %6, %6, %14;\n\t"
        "@p1 add.s64 %6, %6, %15;\n\t"
        "@p2 add.s64 %6, %6, %16;\n\t}"
        : "+f"(w.t[0]), "+f"(w.t[1]), "+f"(w.t[2]), "+f"(w.m[0]), "+f"(w.m[1]), "+f"(w.m[2]), "+l"(w.off)
        : "f"(tm), "f"(w.pa[0]), "f"(w.pa[1]), "f"(w.pa[2]), "f"(w.d[0]), "f"(w.d[1]), "f"(w.d[2]), "l"(w.st[0]),
          "l"(w.st[1]), "l"(w.st[2]));
  }
}

// Running-sum advance (drift batches): an advancing family's local crossing
// becomes tl + |p|.
template <typename IDX>
__device__ __forceinline__ void advance_drift(Walk<IDX> &w, float tl[3], float tm) {
  if constexpr (sizeof(IDX) == 4) {
    asm("{\n\t.reg .pred p0, p1, p2;\n\t"
        "setp.eq.f32 p0, %0, %4;\n\t"
        "setp.eq.f32 p1, %1, %4;\n\t"
        "setp.eq.f32 p2, %2, %4;\n\t"
        "@p0 add.f32 %0, %0, %5;\n\t"
        "@p1 add.f32 %1, %1, %6;\n\t"
        "@p2 add.f32 %2, %2, %7;\n\t"
        "@p0 add.s32 %3, %3, %8;\n\t"
        "@p1 add.s32 %3, %3, %9;\n\t"
        "@p2 add.s32 %3, %3, %10;\n\t}"
        : "+f"(tl[0]), "+f"(tl[1]), "+f"(tl[2]), "+r"(w.off)
        : "f"(tm), "f"(w.pa[0]), "f"(w.pa[1]), "f"(w.pa[2]), "r"(w.st[0]), "r"(w.st[1]), "r"(w.st[2]));
  } else {
    asm("{\n\t.reg .pred p0, p1, p2;\n\t"
        "setp.eq.f32 p0, %0, %4;\n\t"
        "setp.eq.f32 p1, %1, %4;\n\t"
        "setp.eq.f32 p2, %2, %4;\n\t"
        "@p0 add.f32 %0, %0, %5;\n\t"
        "@p1 add.f32 %1, %1, %6;\n\t"
        "@p2 add.f32 %2, %2, %7;\n\t"
        "@p0 add.s64 %3, %3, %8;\n\t"
        "@p1 add.s64 %3, %3, %9;\n\t"
        "@p2 add.s64 %3, %3, %10;\n\t}"
        : "+f"(tl[0]), "+f"(tl[1]), "+f"(tl[2]), "+l"(w.off)
        : "f"(tm), "f"(w.pa[0]), "f"(w.pa[1]), "f"(w.pa[2]), "l"(w.st[0]), "l"(w.st[1]), "l"(w.st[2]));
  }
}

template <typename IDX>
__device__ __forceinline__ float walk_step(Walk<IDX> &w, float &cur, IDX &seg_off) {
  const float tm = min3f(w.t[0], w.t[1], w.t[2]);
  const float L = tm - cur;
  seg_off = w.off;
  advance_exact(w, tm);
  cur = tm;
  return L;
}

// Step of a drift batch: like walk_step, but in a frame local to the batch
// (tl = t - o with o the exact position where the batch starts), an advanced
// family's next crossing becomes tl + |p| (one add instead of the count
// update and the FMA) and the counts are not kept; resync() recovers them and
// recomputes every crossing exactly after the batch.  The running sums stay
// within the batch's extent of the origin, so their rounding (at most half an
// ulp of that extent per add) does not grow with the distance from the chord
// midpoint: measured at 256^3 x 512^2 (7 views), running sums in the
// midpoint frame gave per-voxel backprojection errors up to 1.3e-4 and
// per-pixel projection errors up to 7.2e-6, against 7.8e-5 / 3.0e-6 without
// running sums.
template <typename IDX>
__device__ __forceinline__ float drift_step(Walk<IDX> &w, float tl[3], float &cl, IDX &seg_off) {
  const float tm = min3f(tl[0], tl[1], tl[2]);
  const float L = tm - cl;
  seg_off = w.off;
  advance_drift(w, tl, tm);
  cl = tm;
  return L;
}

// Local frame of a drift batch starting at the exact position o.
template <typename IDX>
__device__ __forceinline__ void to_local(const Walk<IDX> &w, float o, float tl[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) tl[k] = w.t[k] - o;  // +inf stays +inf
}

// Exact counts and crossings after a drift batch: the drifted crossing
// o + tl is within a few ulp of fma(m, p, d), so m = rint((o + tl - d) / p).
template <typename IDX>
__device__ __forceinline__ void resync(Walk<IDX> &w, const float tl[3], float o) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (w.pa[k] != __int_as_float(0x7f800000)) {
      w.m[k] = rintf(__fdividef((tl[k] + o) - w.d[k], w.pa[k]));
      w.t[k] = fmaf(w.m[k], w.pa[k], w.d[k]);
    }
  }
}

// The exact step that closes a drift batch: its crossing comes from the exact
// (resynchronised) parameters, its start from the batch's local frame, so the
// segment length is (tm - o) - cl; `cur` leaves it exact.
template <typename IDX>
__device__ __forceinline__ float close_step(Walk<IDX> &w, float o, float cl, float &cur, IDX &seg_off) {
  const float tm = min3f(w.t[0], w.t[1], w.t[2]);
  const float L = (tm - o) - cl;
  seg_off = w.off;
  advance_exact(w, tm);
  cur = tm;
  return L;
}

// Internal mode: count the steps each ray takes (written to xout as float;
// the cube is not read).
constexpr int kModeCount = 4;

// Fire-and-forget float add to global memory.  Written out because a pointer
// that the compiler cannot prove global (e.g. one read from shared memory in
// the packed kernel) turns atomicAdd into a generic atomic that returns its
// old value and stalls the warp until it does.
__device__ __forceinline__ void red_add_f32(float *p, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "f"(v) : "memory");
}

__device__ __forceinline__ void red_add_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("red.global.add.u64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "l"(v) : "memory");
}

// Accumulate one segment (length L, voxel offset o) in the mode's way.
template <int MODE, bool DET, typename IDX>
__device__ __forceinline__ void accumulate(float L, IDX o, const float *cin, float *cout, unsigned long long *aout,
                                           float yv, float yq, float qs, float &acc) {
  if (MODE == kModeCount) {
    acc += 1.f;
  } else if (MODE == TG_PJ || MODE == TG_PJT) {
    acc = fmaf(L, __ldg(cin + o), acc);
  } else if (DET) {
    red_add_u64(aout + o, (unsigned long long)__float2ll_rn((L * yq) * qs));
  } else {
    red_add_f32(cout + o, L * yv);
  }
}

// Trace ray (i, j) of view t; cidx / ridx index its column (lambda) and row
// (gamma) in the CTA tables.  BATCH: steps per batch (0: the mode's default).
// See the file header for the arithmetic.
template <int MODE, bool SUN, typename IDX, bool DET, int BATCH = 0>
__device__ __forceinline__ void trace_fast(const Geometry &G, const tg_image_header &V, const FastTables &T, int i,
                                           int j, int t, int cidx, int ridx, const float *__restrict__ xin,
                                           float *__restrict__ xout, unsigned long long *__restrict__ acc64,
                                           const DetScale *__restrict__ dsc) {
  constexpr bool CNT = (MODE == kModeCount);
  constexpr bool PJ = (MODE == TG_PJ || MODE == TG_PJT || CNT);
  constexpr bool T4 = (MODE == TG_PJT || MODE == TG_BPJT);
  if (i >= G.n1 || j >= G.n2) return;
  if (G.ray_i >= 0 && (i != G.ray_i || j != G.ray_j)) return;
  const long long po = (long long)i * G.ds[0] + (long long)j * G.ds[1] + (long long)t * G.ds[2];
  // overwrite mode (projection): every pixel is written, 0 where the ray is
  // skipped, so the stack needs no zeroing pass first
  const bool ovw = PJ && !CNT && G.overwrite;
  if (masked(G, i, j, t)) {
    if (ovw) xout[po] = 0.f;
    return;
  }
  long long fbase = 0;
  if (T4) {
    const int f = V.frame;
    if (f < 0 || f >= G.nframes) {
      if (ovw) xout[po] = 0.f;
      return;
    }
    fbase = (long long)f * G.ms[3];
  }
  float yv = 0.f;
  if (!PJ) {
    yv = xin[po];
    if (yv == 0.f) return;  // adds exact zeros only
  }
  Walk<IDX> w;
  float sun_lo;
  if (!setup_ray<SUN, IDX>(G, V, T, cidx, ridx, w, sun_lo)) {
    if (ovw) xout[po] = 0.f;
    return;
  }
  yv *= w.lscale;  // lengths of the walk parameter -> path lengths

  const float *cin = PJ ? xin + fbase : nullptr;
  float *cout = PJ ? nullptr : xout + fbase;
  unsigned long long *aout = DET ? acc64 + fbase : nullptr;
  const float yq = DET ? yv * dsc->yscale : 0.f;  // yv already carries lscale
  const float qs = DET ? dsc->qscale : 0.f;
  // Projection sums are blocked: each batch (and the tail) sums its segments
  // into `part`, which is then added to `acc`, so the float32 rounding grows
  // with kBatch + steps / kBatch rather than with the step count.
  float acc = 0.f;
  float cur = w.t0;
  const float tstop = fminf(w.texit, sun_lo);
  int guard = G.n[0] + G.n[1] + G.n[2] + 2;

  // Why no step reads outside the cube: a step that starts at cur < texit
  // reads a valid voxel.  The families advanced by the step before it had
  // their crossing fma(m, p, d) = cur < texit <= fma(ce - 1, p, d) (texit is
  // computed with the same FMA, see setup_ray), and fma(., p, d) is monotone
  // in its first argument, so m < ce - 1 and the new index is still inside.
  //
  // Batches of kBatch steps: after j steps of a batch every family has
  // advanced at most j times, so the start of step kBatch-1 (the crossing of
  // step kBatch-2) is at most min_a fma(m_a + kBatch - 2, p_a, d_a).  When
  // that bound is below tstop every step of the batch starts before tstop:
  // the batch is exactly kBatch iterations of the single-step loop below, with
  // no per-step test, and its kBatch cube gathers are issued together.
  //
  // Drift batches (drift_step): their first kBatch - 1 crossings are running
  // sums in the batch's local frame tl = t - o.  Every crossing that matters
  // lies in [-h, h] (h = half chord), so |tl| <= 2h: the conversion to the
  // local frame and each add are off by at most 2^-24 (2h), and a drifted
  // crossing by at most kBatch 2^-23 h; the bound gets a margin of
  // (kBatch + 3) 2^-23 h, so a drifted step still advances only families
  // whose exact crossing is below the stop.  The counts are then recovered
  // (resync) and the batch's last step is an exact one.
  constexpr int kBatch = BATCH ? BATCH : batch_steps(MODE);
  constexpr bool kDrift = drift_batches(MODE);
  const float margin = kDrift ? (float)(kBatch + 3) * 1.1920929e-7f * (-w.t0) : 0.f;
  while (guard >= kBatch) {
    const float bnd = min3f(fmaf(w.m[0] + (float)(kBatch - 2), w.pa[0], w.d[0]),
                            fmaf(w.m[1] + (float)(kBatch - 2), w.pa[1], w.d[1]),
                            fmaf(w.m[2] + (float)(kBatch - 2), w.pa[2], w.d[2]));
    if (!(bnd + margin < tstop)) break;
    guard -= kBatch;
    if (!PJ) {
      // backprojection: each segment's atomic is issued as soon as the step
      // is known (fire-and-forget, so nothing is kept per step)
      if (kDrift) {
        const float org = cur;
        float tl[3], cl = 0.f;
        to_local(w, org, tl);
#pragma unroll
        for (int s = 0; s < kBatch - 1; ++s) {
          IDX o;
          const float L = drift_step(w, tl, cl, o);
          accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, acc);
        }
        resync(w, tl, org);
        IDX o;
        const float L = close_step(w, org, cl, cur, o);
        accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, acc);
      } else {
#pragma unroll
        for (int s = 0; s < kBatch; ++s) {
          IDX o;
          const float L = walk_step(w, cur, o);
          accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, acc);
        }
      }
      continue;
    }
    // The batch's segments are summed in step order into `part`, each one
    // kLag steps after its gather was issued: the gather's latency is hidden
    // behind the walk and only kLag values are live at a time (which is what
    // lets the projection run at 4 CTAs per SM: 16.60 -> 15.75 ms against
    // summing the whole batch after it at 24 steps, 15.36 ms at the 32 steps
    // of fine cubes).  The summation order is unchanged.
    constexpr int kLag = TG_PJ_LAG < kBatch - 1 ? TG_PJ_LAG : kBatch - 2;
    float L[kBatch];
    float v[kBatch];
    float part = 0.f;
    if (kDrift) {
      const float org = cur;
      float tl[3], cl = 0.f;
      to_local(w, org, tl);
#pragma unroll
      for (int s = 0; s < kBatch - 1; ++s) {
        IDX os;
        L[s] = drift_step(w, tl, cl, os);
        v[s] = CNT ? 1.f : __ldg(cin + os);
        if (!CNT && s >= kLag) part = fmaf(L[s - kLag], v[s - kLag], part);
      }
      resync(w, tl, org);
      IDX os;
      L[kBatch - 1] = close_step(w, org, cl, cur, os);
      v[kBatch - 1] = CNT ? 1.f : __ldg(cin + os);
    } else {
#pragma unroll
      for (int s = 0; s < kBatch - 1; ++s) {
        IDX os;
        L[s] = walk_step(w, cur, os);
        v[s] = CNT ? 1.f : __ldg(cin + os);
        if (!CNT && s >= kLag) part = fmaf(L[s - kLag], v[s - kLag], part);
      }
      IDX os;
      L[kBatch - 1] = walk_step(w, cur, os);
      v[kBatch - 1] = CNT ? 1.f : __ldg(cin + os);
    }
    if (CNT) {
      acc += (float)kBatch;
    } else {
#pragma unroll
      for (int s = kBatch - 1 - kLag; s < kBatch; ++s) part = fmaf(L[s], v[s], part);
      acc += part;
    }
  }
  // Remaining steps before tstop: short exact batches (same bound, no
  // drift; the projection's gathers of a short batch are in flight
  // together), then one at a time.
  float part = 0.f;
  constexpr int kShort = is_backprojection(MODE) ? TG_BPJ_SHORT_BATCH : TG_PJ_SHORT_BATCH;
  while (kShort > 1 && guard >= kShort) {
    const float bnd = min3f(fmaf(w.m[0] + (float)(kShort - 2), w.pa[0], w.d[0]),
                            fmaf(w.m[1] + (float)(kShort - 2), w.pa[1], w.d[1]),
                            fmaf(w.m[2] + (float)(kShort - 2), w.pa[2], w.d[2]));
    if (!(bnd < tstop)) break;
    guard -= kShort;
    if (!PJ) {
#pragma unroll
      for (int s = 0; s < kShort; ++s) {
        IDX o;
        const float L = walk_step(w, cur, o);
        accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, part);
      }
    } else {
      float L[kShort > 1 ? kShort : 1], v[kShort > 1 ? kShort : 1];
#pragma unroll
      for (int s = 0; s < kShort; ++s) {
        IDX o;
        L[s] = walk_step(w, cur, o);
        v[s] = CNT ? 1.f : __ldg(cin + o);
      }
      if (CNT) {
        part += (float)kShort;
      } else {
#pragma unroll
        for (int s = 0; s < kShort; ++s) part = fmaf(L[s], v[s], part);
      }
    }
  }
  while (cur < tstop && guard > 0) {
    --guard;
    IDX o;
    const float L = walk_step(w, cur, o);
    accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, part);
  }
  // Obstacle zone: test each voxel entry before accumulating it.
  if (SUN && cur < w.texit) {
    while (cur < w.texit && guard > 0) {
      --guard;
      const float se = cur - w.t0;  // distance from the entry point
      const float px = fmaf(se, w.uf[0], w.E[0]);
      const float py = fmaf(se, w.uf[1], w.E[1]);
      const float pz = fmaf(se, w.uf[2], w.E[2]);
      const float dd = fmaf(px, px, fmaf(py, py, pz * pz)) - 1.f;
      bool outside;
      if (dd > kSunTh) {
        outside = true;
      } else if (dd < -kSunTh) {
        outside = false;
      } else {
        int ivn[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) ivn[k] = w.iv0[k] + w.upd[k] * (int)w.m[k];
        outside = exact_outside(G, V, T, cidx, ridx, ivn);
      }
      if (!outside) break;
      IDX o;
      const float L = walk_step(w, cur, o);
      accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, part);
    }
  }
  acc += part;
  if (ovw) xout[po] = acc * w.lscale;
  else if (PJ && !CNT && acc != 0.f) xout[po] += acc * w.lscale;
  if (CNT && acc != 0.f) xout[po] += acc;
}

// One CTA tile of view t.  LMAJ (lanes along lambda, image axis 1): rows
// [row0, row0 + 8 * RPW) x columns [col0, col0 + 32), warp w traces rows
// w, w + 8, ... (RPW rows per warp), its lanes 32 neighbouring columns.
// Otherwise lanes run along gamma (image axis 0): rows [row0, row0 + 32) x
// columns [col0, col0 + 8 * RPW), warp w traces columns w, w + 8, ... --
// the better mapping when image axis 0 follows the cube's fastest axis (a
// view rolled by 90 degrees).  The CTA tables cover 32 rows and 32 columns
// either way.
template <int MODE, bool SUN, typename IDX, bool DET, int RPW, bool LMAJ = true, int BATCH = 0>
__device__ __forceinline__ void tile_body(const Geometry &G, int t, int col0, int row0,
                                          const float *__restrict__ xin, float *__restrict__ xout,
                                          unsigned long long *__restrict__ acc64,
                                          const DetScale *__restrict__ dsc) {
  static_assert(RPW * kRows <= kFastRows && kFastRows == 32, "tile larger than the CTA tables");
  __shared__ FastTables T;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const tg_image_header &V = G.views[t];
  fill_fast_tables(T, G, V, col0, row0);
  __syncthreads();
#pragma unroll 1
  for (int r = 0; r < RPW; ++r) {
    const int slot = warp + r * kRows;
    if (LMAJ)
      trace_fast<MODE, SUN, IDX, DET, BATCH>(G, V, T, row0 + slot, col0 + lane, t, lane, slot, xin, xout, acc64,
                                             dsc);
    else
      trace_fast<MODE, SUN, IDX, DET, BATCH>(G, V, T, row0 + lane, col0 + slot, t, slot, lane, xin, xout, acc64,
                                             dsc);
  }
}

// Modes: 0 = PJ, 1 = BPJ, 2 = PJT, 3 = BPJT, kModeCount; DET: backprojection
// into the 64-bit fixed-point accumulator `acc64` instead of red.add.f32.
// Grid (N2 / 32, N1 / kFastRows, views).
// BATCH: steps per drift batch, 0 for the direction's default.
template <int MODE, bool SUN, typename IDX, bool DET, int BATCH = 0>
__global__ void __launch_bounds__(kThreads, min_blocks(MODE))
fast_kernel(const Geometry G, const float *__restrict__ xin, float *__restrict__ xout,
            unsigned long long *__restrict__ acc64, const DetScale *__restrict__ dsc) {
  tile_body<MODE, SUN, IDX, DET, kFastRowsPerWarp, true, BATCH>(G, G.view0 + blockIdx.z, (G.bx0 + blockIdx.x) * 32,
                                                                (G.by0 + blockIdx.y) * kFastRows, xin, xout,
                                                                acc64, dsc);
}

// Whether a projection over this cube takes the fine-cube batch length.
inline bool fine_projection(const Geometry &G) {
  return G.n[0] >= TG_PJ_FINE_MIN_N && G.n[1] >= TG_PJ_FINE_MIN_N && G.n[2] >= TG_PJ_FINE_MIN_N;
}

}  // namespace tg
