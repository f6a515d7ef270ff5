// Fast single-precision Siddon projector / backprojector for sm_103a.
//
// Work mapping: one thread per detector ray.  A CTA is kFastRows rows x 32
// columns of one view; a warp traces 32 consecutive pixels of a row at a time,
// i.e. 32 rays that are neighbours along image axis 1 (lambda).  For observers near the
// solar equator that axis maps to the cube's fastest axis, so at a given step
// the warp's lanes read / update neighbouring voxels of one cube row and the
// whole warp walks the same (x, y) voxel sequence in lock step.
//
// Arithmetic (the reference does everything in its C type,
// tomograpy/C_siddon.c.template:530-580,811-912):
//  * per-ray set-up in double precision: direction (cos l * A_row + sin l *
//    R[:, 2] with per-row A_row = R . (cos g, sin g, 0) tabulated per CTA),
//    entry parameter amin exactly as the reference computes it, entry voxel by
//    a floor division; single precision only classifies the ray (miss / clear
//    entry face) and the full double-precision reference set-up
//    (siddon_geom.cuh) runs when that classification is within its error
//    bound;
//  * the voxel walk in single precision RELATIVE TO THE ENTRY POINT: the k-th
//    plane crossing of family a is t = D_a + k * |p_a| (one FMA, no running
//    sum), so crossing positions carry no accumulated drift and the
//    catastrophic cancellation of the reference's float path
//    (D[k] = next*p + a1 - amin with a1, amin ~ 215) never occurs.  Steps run
//    in batches of kBatch that are proven, by one bound, to start before the
//    stop parameter, so a batch needs no per-step test and its kBatch cube
//    gathers are issued together;
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

constexpr int kBatch = 8;                  // steps per batch of independent gathers
constexpr float kSunTh = 1e-5f;            // single-precision |d - 1| decision threshold

struct DetScale {                          // deterministic-mode scale factors (device)
  float yscale;                            // power of two bringing max|y| into [0.5, 1)
  float qscale;                            // power of two: fixed-point unit
  double out_scale;                        // 1 / (yscale * qscale)
  unsigned int ymax_bits;
  unsigned int pad;
};

// Per-CTA tables: cos / sin of lambda for the 32 columns, and for each of the
// kFastRows rows A = R . (cos gamma, sin gamma, 0), so that a ray's direction
// R . (cos l cos g, cos l sin g, sin l) is cos l * A + sin l * R[:, 2].
struct FastTables {
  double cl[32], sl[32];
  double A[kFastRows][3];
};

__device__ __forceinline__ void fill_fast_tables(FastTables &T, const tg_image_header &V, int col0, int row0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
    double s, c;
    sincos(pixel_angle(col0 + lane, V, 1), &s, &c);
    T.sl[lane] = s;
    T.cl[lane] = c;
  } else if (warp == 1 && lane < kFastRows) {
    double s, c;
    sincos(pixel_angle(row0 + lane, V, 0), &s, &c);
#pragma unroll
    for (int k = 0; k < 3; ++k) T.A[lane][k] = __dadd_rn(__dmul_rn(V.R[3 * k], c), __dmul_rn(V.R[3 * k + 1], s));
  }
}

// State of one ray's walk in the single-precision relative frame.
template <typename IDX>
struct Walk {
  float t[3];   // next crossing of each plane family (relative to entry)
  float d[3];   // first crossing
  float pa[3];  // spacing of crossings
  float m[3];   // crossings done (exact small integers)
  int iv0[3];   // entry voxel
  int upd[3];
  IDX st[3];    // offset change when crossing a plane of each family
  IDX off;      // current voxel offset
  float texit;  // parameter of the first crossing that leaves the cube
  float E[3];   // entry point (absolute)
  float uf[3];  // direction (single precision)
};

// Per-ray set-up.  Returns false when the ray does not enter the cube (the
// reference's loop would not run).  `sun_lo` receives the parameter up to which
// no obstacle test is needed (+inf when the ray cannot reach the sphere).
template <bool SUN, typename IDX>
__device__ __forceinline__ bool setup_ray(const Geometry &G, const double M[3], const double u[3], Walk<IDX> &w,
                                          float &sun_lo) {
  const float kInf = __int_as_float(0x7f800000);
  float lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    w.uf[k] = (float)u[k];
    if (u[k] != 0.0) {
      const float Mf = (float)M[k];
      const float inv = __frcp_rn(w.uf[k]);
      const float a = (G.mminf[k] - Mf) * inv;
      const float b = (G.mmaxf[k] - Mf) * inv;
      lo[k] = fminf(a, b);
      hi[k] = fmaxf(a, b);
    } else {
      lo[k] = -1e5f;
      hi[k] = 1e5f;
    }
  }
  int kin = 0;
  if (lo[1] > lo[kin]) kin = 1;
  if (lo[2] > lo[kin]) kin = 2;
  const float aminf = lo[kin];
  const float second = fmaxf(kin == 0 ? lo[1] : lo[0], kin == 2 ? lo[1] : lo[2]);
  const float amaxf = fminf(hi[0], fminf(hi[1], hi[2]));
  const float tol = 4e-6f * (fabsf(aminf) + fabsf(amaxf)) + 1e-6f;
  if (amaxf - aminf < -tol) return false;  // clear miss
  int iv[3];
  float ef[3];  // entry point relative to MMIN (single precision)
  if (amaxf - aminf < tol || aminf - second < tol) {
    // Ambiguous in single precision: grazing ray or edge / corner entry.
    RefWalk rw;
    if (!ref_setup(G.mh, G.n, M, u, rw)) return false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      iv[k] = rw.iv[k];
      w.upd[k] = rw.upd[k];
      w.d[k] = w.upd[k] ? (float)rw.D[k] : kInf;
      w.pa[k] = w.upd[k] ? (float)rw.pabs[k] : kInf;
      ef[k] = (float)__dsub_rn(__dadd_rn(M[k], __dmul_rn(rw.amin, u[k])), G.mh.mmin[k]);
    }
  } else {
    const double F = (u[kin] > 0.0) ? G.mh.mmin[kin] : G.mh.mmax[kin];
    const double amin = __ddiv_rn(__dsub_rn(F, M[kin]), u[kin]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      w.upd[k] = (u[k] > 0.0) ? 1 : ((u[k] < 0.0) ? -1 : 0);
      w.pa[k] = w.upd[k] ? __fdiv_rn(G.cdeltf[k], fabsf(w.uf[k])) : kInf;
      if (k == kin) {
        iv[k] = (w.upd[k] > 0) ? 0 : G.n[k] - 1;
        w.d[k] = w.pa[k];
        ef[k] = (w.upd[k] > 0) ? 0.f : (float)G.mh.pshape[k];
      } else if (w.upd[k] == 0) {
        // In-plane ray: the index holds for the whole chord, so it is taken
        // exactly as the reference computes it (:783-786).
        const double ep = __dsub_rn(M[k], G.mh.mmin[k]);
        iv[k] = ref_utrunc(__ddiv_rn(ep, G.mh.cdelt[k])) - ref_utrunc(__ddiv_rn(ep, G.mh.pshape[k]));
        w.d[k] = kInf;
        ef[k] = (float)ep;
      } else {
        // Entry point on this axis, then floor division by CDELT; an index
        // off by one at a plane only adds a zero-length first segment.
        const double ep = fma(amin, u[k], __dsub_rn(M[k], G.mh.mmin[k]));
        const double q = floor(ep * G.inv_cdelt[k]);
        float r = (float)fma(-q, G.mh.cdelt[k], ep);
        int qi = (int)q;
        if (r < 0.f) {
          qi -= 1;
          r += G.cdeltf[k];
        } else if (r >= G.cdeltf[k]) {
          qi += 1;
          r -= G.cdeltf[k];
        }
        // the reference truncates: a point just outside the first / last
        // voxel still maps to it (:785-786)
        if (qi == -1) {
          qi = 0;
          r -= G.cdeltf[k];
        } else if (qi == G.n[k]) {
          qi = G.n[k] - 1;
          r += G.cdeltf[k];
        }
        iv[k] = qi;
        w.d[k] = (w.upd[k] > 0) ? __fdiv_rn(G.cdeltf[k] - r, w.uf[k]) : __fdiv_rn(r, -w.uf[k]);
        ef[k] = (float)ep;
      }
    }
  }
  float texit = kInf;
  IDX off = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (iv[k] < 0 || iv[k] >= G.n[k]) return false;  // reference: in_map fails at once
    w.iv0[k] = iv[k];
    w.t[k] = w.d[k];
    w.m[k] = 0.f;
    w.st[k] = (IDX)w.upd[k] * (IDX)G.ms[k];
    off += (IDX)iv[k] * (IDX)G.ms[k];
    if (w.upd[k] != 0) {
      const int cexit = (w.upd[k] > 0) ? G.n[k] - iv[k] : iv[k] + 1;
      texit = fminf(texit, fmaf((float)(cexit - 1), w.pa[k], w.d[k]));
    }
    w.E[k] = G.mminf[k] + ef[k];
  }
  w.off = off;
  w.texit = texit;
  sun_lo = kInf;
  if (SUN) {
    const float b = fmaf(w.E[0], w.uf[0], fmaf(w.E[1], w.uf[1], w.E[2] * w.uf[2]));
    const float c = fmaf(w.E[0], w.E[0], fmaf(w.E[1], w.E[1], w.E[2] * w.E[2])) - 1.f;
    const float disc = fmaf(b, b, -c);
    if (c < 1e-4f) {
      sun_lo = -kInf;  // entry at / inside the sphere: test from the start
    } else if (b < 0.f && disc > -2e-5f) {
      const float sq = sqrtf(fmaxf(disc, 0.f));
      const float s1 = -b - sq;
      const float g = 1e-5f + __fdividef(1e-5f, sq);
      sun_lo = (sq > 0.f) ? s1 - g : -kInf;
    }
  }
  return true;
}

// Double-precision decision of the obstacle test at the entry of voxel iv
// (the reference's |M + ac u0|^2 > 1 with ac the entry parameter of the
// voxel): the entry parameter is the largest of the crossing parameters of the
// voxel's lower planes along the ray.
static __device__ __noinline__ bool exact_outside(const Geometry &G, const double M[3], const double u[3],
                                                  const int iv[3]) {
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
template <typename IDX>
__device__ __forceinline__ float walk_step(Walk<IDX> &w, float &cur, IDX &seg_off) {
  const float tm = fminf(w.t[0], fminf(w.t[1], w.t[2]));
  const float L = tm - cur;
  seg_off = w.off;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (w.t[k] == tm) {
      w.m[k] += 1.f;
      w.t[k] = fmaf(w.m[k], w.pa[k], w.d[k]);
      w.off += w.st[k];
    }
  }
  cur = tm;
  return L;
}

// Internal mode: count the steps each ray takes (written to xout as float;
// the cube is not read).
constexpr int kModeCount = 4;

// Accumulate one segment (length L, voxel offset o) in the mode's way.
template <int MODE, bool DET, typename IDX>
__device__ __forceinline__ void accumulate(float L, IDX o, const float *cin, float *cout, unsigned long long *aout,
                                           float yv, float yq, float qs, float &acc) {
  if (MODE == kModeCount) {
    acc += 1.f;
  } else if (MODE == TG_PJ || MODE == TG_PJT) {
    acc = fmaf(L, __ldg(cin + o), acc);
  } else if (DET) {
    atomicAdd(aout + o, (unsigned long long)__float2ll_rn((L * yq) * qs));
  } else {
    atomicAdd(cout + o, L * yv);
  }
}

// Trace ray (i, j) of view t.  See the file header for the arithmetic.
template <int MODE, bool SUN, typename IDX, bool DET>
__device__ __forceinline__ void trace_fast(const Geometry &G, const tg_image_header &V, const FastTables &T, int i,
                                           int j, int t, int row_slot, const float *__restrict__ xin,
                                           float *__restrict__ xout, unsigned long long *__restrict__ acc64,
                                           const DetScale *__restrict__ dsc) {
  constexpr bool CNT = (MODE == kModeCount);
  constexpr bool PJ = (MODE == TG_PJ || MODE == TG_PJT || CNT);
  constexpr bool T4 = (MODE == TG_PJT || MODE == TG_BPJT);
  const int lane = threadIdx.x & 31;
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
  float yv = 0.f;
  if (!PJ) {
    yv = xin[po];
    if (yv == 0.f) return;  // adds exact zeros only
  }
  const double M[3] = {V.M[0], V.M[1], V.M[2]};
  double u[3];
  const double cl = T.cl[lane], sl = T.sl[lane];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    u[k] = fma(cl, T.A[row_slot][k], sl * V.R[3 * k + 2]);
    if (fabs(u[k]) < kSnapZero) u[k] = 0.0;
  }
  Walk<IDX> w;
  float sun_lo;
  if (!setup_ray<SUN, IDX>(G, M, u, w, sun_lo)) return;

  const float *cin = PJ ? xin + fbase : nullptr;
  float *cout = PJ ? nullptr : xout + fbase;
  unsigned long long *aout = DET ? acc64 + fbase : nullptr;
  const float yq = DET ? yv * dsc->yscale : 0.f;
  const float qs = DET ? dsc->qscale : 0.f;
  float acc = 0.f;
  float cur = 0.f;
  const float tstop = fminf(w.texit, sun_lo);
  int guard = G.n[0] + G.n[1] + G.n[2] + 2;

  // Batches of kBatch steps that are all known to start before tstop: the
  // (kBatch-1)-th upcoming crossing is at most min_a(t_a + (kBatch-2) |p_a|).
  while (guard >= kBatch) {
    const float bnd = fminf(fmaf((float)(kBatch - 2), w.pa[0], w.t[0]),
                            fminf(fmaf((float)(kBatch - 2), w.pa[1], w.t[1]),
                                  fmaf((float)(kBatch - 2), w.pa[2], w.t[2])));
    if (!(bnd + fabsf(bnd) * 5e-7f < tstop)) break;
    guard -= kBatch;
    float L[kBatch];
    IDX o[kBatch];
#pragma unroll
    for (int s = 0; s < kBatch; ++s) L[s] = walk_step(w, cur, o[s]);
    if (CNT) {
      acc += (float)kBatch;
    } else if (PJ) {
      float v[kBatch];
#pragma unroll
      for (int s = 0; s < kBatch; ++s) v[s] = __ldg(cin + o[s]);
#pragma unroll
      for (int s = 0; s < kBatch; ++s) acc = fmaf(L[s], v[s], acc);
    } else {
#pragma unroll
      for (int s = 0; s < kBatch; ++s) accumulate<MODE, DET, IDX>(L[s], o[s], cin, cout, aout, yv, yq, qs, acc);
    }
  }
  // Remaining steps before tstop, one at a time.
  while (cur < tstop && guard > 0) {
    --guard;
    IDX o;
    const float L = walk_step(w, cur, o);
    accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, acc);
  }
  // Obstacle zone: test each voxel entry before accumulating it.
  if (SUN && cur < w.texit) {
    while (cur < w.texit && guard > 0) {
      --guard;
      const float px = fmaf(cur, w.uf[0], w.E[0]);
      const float py = fmaf(cur, w.uf[1], w.E[1]);
      const float pz = fmaf(cur, w.uf[2], w.E[2]);
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
        outside = exact_outside(G, M, u, ivn);
      }
      if (!outside) break;
      IDX o;
      const float L = walk_step(w, cur, o);
      accumulate<MODE, DET, IDX>(L, o, cin, cout, aout, yv, yq, qs, acc);
    }
  }
  if (PJ && acc != 0.f) xout[po] += acc;
}

// Modes: 0 = PJ, 1 = BPJ, 2 = PJT, 3 = BPJT, kModeCount; DET: backprojection
// into the 64-bit fixed-point accumulator `acc64` instead of red.add.f32.
// CTA: kFastRows rows x 32 columns of one view; warp w traces rows w and
// w + kRows of the tile.
template <int MODE, bool SUN, typename IDX, bool DET>
__global__ void __launch_bounds__(kThreads)
fast_kernel(const Geometry G, const float *__restrict__ xin, float *__restrict__ xout,
            unsigned long long *__restrict__ acc64, const DetScale *__restrict__ dsc) {
  __shared__ FastTables T;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = G.view0 + blockIdx.z;
  const tg_image_header &V = G.views[t];
  const int col0 = (G.bx0 + blockIdx.x) * 32, row0 = (G.by0 + blockIdx.y) * kFastRows;
  fill_fast_tables(T, V, col0, row0);
  __syncthreads();
#pragma unroll 1
  for (int r = 0; r < kFastRowsPerWarp; ++r) {
    const int slot = warp + r * kRows;
    trace_fast<MODE, SUN, IDX, DET>(G, V, T, row0 + slot, col0 + lane, t, slot, xin, xout, acc64, dsc);
  }
}

}  // namespace tg
