// Fast single-precision Siddon projector / backprojector for sm_103a.
//
// Work mapping: one thread per detector ray.  A CTA is kRows rows x 32
// columns of one view; a warp is 32 consecutive pixels of one row, i.e. 32
// rays that are neighbours along image axis 1 (lambda).  For observers near the
// solar equator that axis maps to the cube's fastest axis, so at a given step
// the warp's lanes read / update neighbouring voxels of one cube row and the
// whole warp walks the same (x, y) voxel sequence in lock step.
//
// Arithmetic (the reference does everything in its C type,
// tomograpy/C_siddon.c.template:530-580,811-912):
//  * per-ray set-up in double precision: direction, entry parameter amin and
//    entry voxel exactly as the reference computes them (siddon_geom.cuh);
//    single precision only classifies the ray (miss / clear entry face) and
//    falls back to the full double-precision reference set-up when the
//    classification is within its error bound;
//  * the voxel walk in single precision RELATIVE TO THE ENTRY POINT: the k-th
//    plane crossing of family a is t = D_a + k * |p_a| (one FMA, no running
//    sum), so crossing positions carry no accumulated drift and the
//    catastrophic cancellation of the reference's float path
//    (D[k] = next*p + a1 - amin with a1, amin ~ 215) never occurs;
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

constexpr int kUnroll = 4;                 // steps per batch of independent gathers
constexpr float kSunTh = 1e-5f;            // single-precision |d - 1| decision threshold

struct DetScale {                          // deterministic-mode scale factors (device)
  float yscale;                            // power of two bringing max|y| into [0.5, 1)
  float qscale;                            // power of two: fixed-point unit
  double out_scale;                        // 1 / (yscale * qscale)
  unsigned int ymax_bits;
  unsigned int pad;
};

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

// Reference-exact voxel index and in-voxel remainder for one non-entry axis.
// iv = trunc(ep / CDELT) - trunc(ep / PSHAPE) with correctly rounded
// quotients (:785-786); computed without division unless a quotient lies
// within rounding distance of an integer, or ep is outside [0, PSHAPE).
__device__ __forceinline__ int entry_index(double ep, double C, double invC, double PS, double &r) {
  if (ep >= 0.0 && ep < PS * (1.0 - 4e-16)) {
    double q = floor(ep * invC);
    double rr = fma(-q, C, ep);
    if (rr < 0.0) {
      q -= 1.0;
      rr += C;
    } else if (rr >= C) {
      q += 1.0;
      rr -= C;
    }
    if (C - rr > C * (q + 1.0) * 2.3e-16) {
      r = rr;
      return (int)q;
    }
  }
  const int iv = ref_utrunc(__ddiv_rn(ep, C)) - ref_utrunc(__ddiv_rn(ep, PS));
  r = fma(-(double)iv, C, ep);
  return iv;
}

// Per-ray set-up.  Returns false when the ray does not enter the cube (the
// reference's loop would not run).  `sun_lo` receives the parameter up to which
// no obstacle test is needed (+inf when the ray cannot reach the sphere).
template <bool SUN, typename IDX>
__device__ __forceinline__ bool setup_ray(const Geometry &G, const double M[3], const double u[3], Walk<IDX> &w,
                                          float &sun_lo) {
  float lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    w.uf[k] = (float)u[k];
    if (u[k] != 0.0) {
      const float Mf = (float)M[k];
      const float a = __fdiv_rn(G.mminf[k] - Mf, w.uf[k]);
      const float b = __fdiv_rn(G.mmaxf[k] - Mf, w.uf[k]);
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
  double ep[3];
  int iv[3];
  if (amaxf - aminf < tol || aminf - second < tol) {
    // Ambiguous in single precision: grazing ray or edge / corner entry.
    RefWalk rw;
    if (!ref_setup(G.mh, G.n, M, u, rw)) return false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      iv[k] = rw.iv[k];
      w.upd[k] = rw.upd[k];
      w.d[k] = w.upd[k] ? (float)rw.D[k] : __int_as_float(0x7f800000);
      w.pa[k] = w.upd[k] ? (float)rw.pabs[k] : __int_as_float(0x7f800000);
      ep[k] = __dsub_rn(__dadd_rn(M[k], __dmul_rn(rw.amin, u[k])), G.mh.mmin[k]);
    }
  } else {
    const double F = (u[kin] > 0.0) ? G.mh.mmin[kin] : G.mh.mmax[kin];
    const double amin = __ddiv_rn(__dsub_rn(F, M[kin]), u[kin]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      w.upd[k] = (u[k] > 0.0) ? 1 : ((u[k] < 0.0) ? -1 : 0);
      w.pa[k] = w.upd[k] ? __fdiv_rn(G.cdeltf[k], fabsf(w.uf[k])) : __int_as_float(0x7f800000);
      if (k == kin) {
        iv[k] = (w.upd[k] > 0) ? 0 : G.n[k] - 1;
        w.d[k] = w.pa[k];
        ep[k] = (w.upd[k] > 0) ? 0.0 : G.mh.pshape[k];
      } else {
        ep[k] = __dsub_rn(__dadd_rn(M[k], __dmul_rn(amin, u[k])), G.mh.mmin[k]);
        double r;
        iv[k] = entry_index(ep[k], G.mh.cdelt[k], G.inv_cdelt[k], G.mh.pshape[k], r);
        if (w.upd[k] > 0) w.d[k] = __fdiv_rn((float)(G.mh.cdelt[k] - r), w.uf[k]);
        else if (w.upd[k] < 0) w.d[k] = __fdiv_rn((float)r, -w.uf[k]);
        else w.d[k] = __int_as_float(0x7f800000);
      }
    }
  }
  float texit = __int_as_float(0x7f800000);
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
    w.E[k] = (float)__dadd_rn(G.mh.mmin[k], ep[k]);
  }
  w.off = off;
  w.texit = texit;
  sun_lo = __int_as_float(0x7f800000);
  if (SUN) {
    const float b = fmaf(w.E[0], w.uf[0], fmaf(w.E[1], w.uf[1], w.E[2] * w.uf[2]));
    const float c = fmaf(w.E[0], w.E[0], fmaf(w.E[1], w.E[1], w.E[2] * w.E[2])) - 1.f;
    const float disc = fmaf(b, b, -c);
    if (c < 1e-4f) {
      sun_lo = -__int_as_float(0x7f800000);  // entry at / inside the sphere: test from the start
    } else if (b < 0.f && disc > -2e-5f) {
      const float sq = sqrtf(fmaxf(disc, 0.f));
      const float s1 = -b - sq;
      const float g = 1e-5f + __fdividef(1e-5f, sq);
      sun_lo = (sq > 0.f) ? s1 - g : -__int_as_float(0x7f800000);
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
// belongs to, and advances the state.
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

// Internal mode: count the segments each ray accumulates (written to xout as
// float; the cube is not read).
constexpr int kModeCount = 4;

// Modes: 0 = PJ, 1 = BPJ, 2 = PJT, 3 = BPJT, kModeCount; DET: backprojection
// into the 64-bit fixed-point accumulator `acc64` instead of red.add.f32.
template <int MODE, bool SUN, typename IDX, bool DET>
__global__ void __launch_bounds__(kThreads)
fast_kernel(const Geometry G, const float *__restrict__ xin, float *__restrict__ xout,
            unsigned long long *__restrict__ acc64, const DetScale *__restrict__ dsc) {
  constexpr bool CNT = (MODE == kModeCount);
  constexpr bool PJ = (MODE == TG_PJ || MODE == TG_PJT || CNT);
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
  float yv = 0.f;
  if (!PJ) {
    yv = xin[po];
    if (yv == 0.f) return;  // adds exact zeros only
  }
  double M[3], u[3];
  M[0] = V.M[0];
  M[1] = V.M[1];
  M[2] = V.M[2];
  ray_direction(T.cl[lane], T.sl[lane], T.cg[warp], T.sg[warp], V.R, u);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (fabs(u[k]) < kSnapZero) u[k] = 0.0;
  Walk<IDX> w;
  float sun_lo;
  if (!setup_ray<SUN, IDX>(G, M, u, w, sun_lo)) return;

  const float *cin = PJ ? xin + fbase : nullptr;
  float *cout = PJ ? nullptr : xout + fbase;
  unsigned long long *aout = DET ? acc64 + fbase : nullptr;
  float yq = 0.f;
  if (DET) yq = (yv * dsc->yscale) ;
  float acc = 0.f;
  float cur = 0.f;
  const float tstop = fminf(w.texit, sun_lo);
  int guard = G.n[0] + G.n[1] + G.n[2] + 2;

  // Fast segment: no obstacle test needed before tstop.
  while (cur < tstop && guard > 0) {
    guard -= kUnroll;
    float Ls[kUnroll];
    IDX offs[kUnroll];
#pragma unroll
    for (int s = 0; s < kUnroll; ++s) {
      if (cur < tstop) {
        Ls[s] = walk_step(w, cur, offs[s]);
      } else {
        Ls[s] = 0.f;
        offs[s] = 0;
      }
    }
    if (CNT) {
#pragma unroll
      for (int s = 0; s < kUnroll; ++s) acc += (Ls[s] != 0.f) ? 1.f : 0.f;
    } else if (PJ) {
      float v[kUnroll];
#pragma unroll
      for (int s = 0; s < kUnroll; ++s) v[s] = (Ls[s] != 0.f) ? __ldg(cin + offs[s]) : 0.f;
#pragma unroll
      for (int s = 0; s < kUnroll; ++s) acc = fmaf(Ls[s], v[s], acc);
    } else {
#pragma unroll
      for (int s = 0; s < kUnroll; ++s) {
        if (Ls[s] != 0.f) {
          if (DET) {
            const long long q = __float2ll_rn((Ls[s] * yq) * dsc->qscale);
            atomicAdd(aout + offs[s], (unsigned long long)q);
          } else {
            atomicAdd(cout + offs[s], Ls[s] * yv);
          }
        }
      }
    }
  }

  // Obstacle zone: test each voxel entry before accumulating it.
  if (SUN && cur < w.texit) {
    bool have_u = false;
    while (cur < w.texit && guard > 0) {
      --guard;
      const float px = fmaf(cur, w.uf[0], w.E[0]);
      const float py = fmaf(cur, w.uf[1], w.E[1]);
      const float pz = fmaf(cur, w.uf[2], w.E[2]);
      const float dd = fmaf(px, px, fmaf(py, py, pz * pz)) - 1.f;
      bool outside;
      if (dd > kSunTh) outside = true;
      else if (dd < -kSunTh) outside = false;
      else {
        (void)have_u;
        int ivn[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) ivn[k] = w.iv0[k] + w.upd[k] * (int)w.m[k];
        outside = exact_outside(G, M, u, ivn);
      }
      if (!outside) break;
      IDX so;
      const float L = walk_step(w, cur, so);
      if (L != 0.f) {
        if (CNT) {
          acc += 1.f;
        } else if (PJ) {
          acc = fmaf(L, __ldg(cin + so), acc);
        } else if (DET) {
          const long long q = __float2ll_rn((L * yq) * dsc->qscale);
          atomicAdd(aout + so, (unsigned long long)q);
        } else {
          atomicAdd(cout + so, L * yv);
        }
      }
    }
  }
  if (PJ && acc != 0.f) xout[po] += acc;
}

}  // namespace tg
