// gbsph_fluid.cuh -- the fluid-row Interaction_Forces kernels and their
// launchers, as templates, with the pair terms and the staging helpers they
// share with the mDBC kernels.  Each of gbsph_fluid_art.cu, gbsph_fluid_lam.cu
// and gbsph_fluid_sps.cu instantiates the kernels of one viscosity model, so
// that the three compile in parallel; gbsph_forces.cu holds the bound rows,
// mDBC, PIPS and the dispatch.
//
// Fluid rows restate JSphCpu::InteractionForcesFluid (JSphCpu.cpp:736-1141;
// GPU twin KerInteractionForcesFluidBox, JSphGpu_ker.cu:542-990): Wendland C2
// kernel gradient, Tait pressure (precomputed per particle), Monaghan
// artificial viscosity or Laminar+SPS, Molteni (DDT) or Fourtakas (DDT2)
// density diffusion with the veto for particles with boundary neighbours.
// The maxima the dt needs (|ace|^2 over fluid, visc, |v|^2) are reduced in
// the same kernels (JSphGpuSingle.cpp:719-729, JSphGpu.cpp:846-900).
//
// Pair distance: every particle carries its position relative to the origin of
// its own cell (pscell.xyz, rounded once from double); a neighbour in cell cj
// is at (lp_i - lp_j) + (ci - cj)*Scell, which needs no FP64 in the pair loop.
#pragma once
#include <cuda_runtime.h>
#include <float.h>

#include "gbsph_common.cuh"

namespace {

struct CellGrid {
  int cx, cy, cz;           // particle cell relative to the trimmed domain
  int xini, xfin, yini, yfin, zini, zfin;
};

// nsearch::Init (JCellSearch_inline.h:33-52)
__device__ __forceinline__ CellGrid gb_grid(int cx, int cy, int cz, int sd, const DivState& d) {
  CellGrid g;
  g.cx = cx; g.cy = cy; g.cz = cz;
  const int ncx = (int)d.ncx, ncy = (int)d.ncy, ncz = (int)d.ncz;
  g.xini = cx - (cx < sd ? cx : sd);
  g.xfin = cx + (ncx - cx - 1 < sd ? ncx - cx - 1 : sd) + 1;
  g.yini = cy - (cy < sd ? cy : sd);
  g.yfin = cy + (ncy - cy - 1 < sd ? ncy - cy - 1 : sd) + 1;
  g.zini = cz - (cz < sd ? cz : sd);
  g.zfin = cz + (ncz - cz - 1 < sd ? ncz - cz - 1 : sd) + 1;
  return g;
}

struct FluidAcc {
  float ax, ay, az, ar, delta, visc;
  float s0, s1, s2, s3, s4, s5;  // 2*strain (SPS)
};

// One pass of a fluid row over the fluid (boundp2=false) or boundary
// (boundp2=true) boxes.
template <int tvisco, int tdensity, bool boundp2, bool tshift>
__device__ __forceinline__ void fluid_pass(const gbsph_consts& c, const DevArrays& a, const DivState& d,
                                           const CellGrid& g, float4 ps1, float4 vr1, float4 ta1, float2 tb1,
                                           float visco, FluidAcc& r, float4& sh) {
  const unsigned cellinit = boundp2 ? 0u : d.boxfluid;
  const float scell = c.scell;
  const float ks2 = c.kernelsize2, eta2 = c.eta2, h = c.kernelh, bwenh = c.bwenh;
  const float massp2 = boundp2 ? c.massbound : c.massfluid;
  const float cbar = (float)c.cs0;
  float ax = 0, ay = 0, az = 0, arp1 = 0, deltap1 = 0, visc = 0;
  float s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0;
  for (int z = g.zini; z < g.zfin; z++) {
    for (int y = g.yini; y < g.yfin; y++) {
      const unsigned rowbase = cellinit + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
      const float offy = (float)(g.cy - y) * scell, offz = (float)(g.cz - z) * scell;
      for (int x = g.xini; x < g.xfin; x++) {
        const unsigned box = rowbase + (unsigned)x;
        const unsigned pini = a.begincell[box], pfin = a.begincell[box + 1];
        const float bx = ps1.x + (float)(g.cx - x) * scell;
        const float by = ps1.y + offy;
        const float bz = ps1.z + offz;
        for (unsigned p2 = pini; p2 < pfin; p2++) {
          const float4 ps2 = a.pscell[p2];
          const float drx = bx - ps2.x, dry = by - ps2.y, drz = bz - ps2.z;
          const float rr2 = drx * drx + dry * dry + drz * drz;
          if (rr2 <= ks2 && rr2 >= GB_ALMOSTZERO) {
            // Wendland C2 gradient factor (FunSphKernel.h:225-231)
            const float rad = sqrtf(rr2);
            const float qq = rad / h;
            const float wqq1 = 1.f - 0.5f * qq;
            const float fac = bwenh * wqq1 * wqq1 * wqq1;
            const float frx = fac * drx, fry = fac * dry, frz = fac * drz;
            const float4 vr2 = a.velrho[p2];
            // momentum (JSphCpu.cpp:846-852)
            const float prs = (ps1.w + ps2.w) / (vr1.w * vr2.w);
            const float p_vpm = -prs * massp2;
            ax += p_vpm * frx; ay += p_vpm * fry; az += p_vpm * frz;
            // continuity (JSphCpu.cpp:865-875)
            const float dvx = vr1.x - vr2.x, dvy = vr1.y - vr2.y, dvz = vr1.z - vr2.z;
            arp1 += massp2 * (dvx * frx + dvy * fry + dvz * frz) * (vr1.w / vr2.w);
            // density diffusion (JSphCpu.cpp:915-940)
            if (tdensity == GBSPH_DDT_DDT && deltap1 != FLT_MAX) {
              const float visc_densi = c.ddtkh * cbar * (vr1.w / vr2.w - 1.f) / (rr2 + eta2);
              const float dot3 = drx * frx + dry * fry + drz * frz;
              const float delta = visc_densi * dot3 * massp2;
              deltap1 = (boundp2 && c.tboundary == GBSPH_BC_DBC) ? FLT_MAX : deltap1 + delta;
            }
            if ((tdensity == GBSPH_DDT_DDT2 || (tdensity == GBSPH_DDT_DDT2FULL && !boundp2)) && deltap1 != FLT_MAX) {
              if (boundp2) {
                deltap1 = FLT_MAX;
              } else {
                const float rh = 1.f + c.ddtgz * drz;
                const float drho = c.rhopzero * powf(rh, 1.f / c.gamma) - c.rhopzero;
                const float visc_densi = c.ddtkh * cbar * ((vr2.w - vr1.w) - drho) / (rr2 + eta2);
                const float dot3 = drx * frx + dry * fry + drz * frz;
                const float delta = visc_densi * dot3 * massp2 / vr2.w;
                deltap1 = deltap1 - delta;
              }
            }
            // shifting sums (JSphCpu.cpp:942-950); a boundary neighbour cancels
            // them in NoBound mode, a fixed one in NoFixed mode
            if (tshift && sh.x != FLT_MAX) {
              const float massrho = massp2 / vr2.w;
              const bool noshift = boundp2 && (c.tshift == 1 || (c.tshift == 2 && (a.code[p2] & GB_CODE_MASKTYPE) == 0u));
              sh.x = noshift ? FLT_MAX : sh.x + massrho * frx;
              sh.y += massrho * fry;
              sh.z += massrho * frz;
              sh.w -= massrho * (drx * frx + dry * fry + drz * frz);
            }
            // viscosity (JSphCpu.cpp:990-1037)
            const float dot = drx * dvx + dry * dvy + drz * dvz;
            const float dot_rr2 = dot / (rr2 + eta2);
            visc = fmaxf(dot_rr2, visc);
            if (tvisco == GBSPH_VISCO_ARTIFICIAL) {
              if (dot < 0) {
                const float amubar = h * dot_rr2;
                const float robar = (vr1.w + vr2.w) * 0.5f;
                const float pi_visc = (-visco * cbar * amubar / robar) * massp2;
                ax -= pi_visc * frx; ay -= pi_visc * fry; az -= pi_visc * frz;
              }
            } else {
              const float robar2 = vr1.w + vr2.w;
              const float temp = 4.f * visco / ((rr2 + eta2) * robar2);
              const float vtemp = massp2 * temp * (drx * frx + dry * fry + drz * frz);
              ax += vtemp * dvx; ay += vtemp * dvy; az += vtemp * dvz;
              if (tvisco == GBSPH_VISCO_LAMINARSPS) {
                float t0 = ta1.x, t1 = ta1.y, t2 = ta1.z, t3 = ta1.w, t4 = tb1.x, t5 = tb1.y;
                if (!boundp2) {
                  const float4 ta2 = a.taua[p2];
                  const float2 tb2 = a.taub[p2];
                  t0 += ta2.x; t1 += ta2.y; t2 += ta2.z; t3 += ta2.w; t4 += tb2.x; t5 += tb2.y;
                }
                ax += massp2 * (t0 * frx + t1 * fry + t2 * frz);
                ay += massp2 * (t1 * frx + t3 * fry + t4 * frz);
                az += massp2 * (t2 * frx + t4 * fry + t5 * frz);
                const float volp2 = -massp2 / vr2.w;
                float dv = dvx * volp2; s0 += dv * frx; s1 += dv * fry; s2 += dv * frz;
                dv = dvy * volp2; s1 += dv * frx; s3 += dv * fry; s4 += dv * frz;
                dv = dvz * volp2; s2 += dv * frx; s4 += dv * fry; s5 += dv * frz;
              }
            }
          }
        }
      }
    }
  }
  r.ax = ax; r.ay = ay; r.az = az; r.ar = arp1; r.delta = deltap1; r.visc = visc;
  r.s0 = s0; r.s1 = s1; r.s2 = s2; r.s3 = s3; r.s4 = s4; r.s5 = s5;
}

template <int tvisco, int tdensity, bool tshift>
__global__ void __launch_bounds__(256) k_forces_fluid(gbsph_consts c, DevArrays a) {
  const DivState& d = *a.div;
  const unsigned np = d.np, npb = d.npb;
  const unsigned p1 = npb + blockIdx.x * blockDim.x + threadIdx.x;
  float acemax2 = 0, visc = 0, vel2 = 0;
  if (p1 < np) {
    const float4 ps1 = a.pscell[p1];
    const float4 vr1 = a.velrho[p1];
    float4 ta1 = make_float4(0, 0, 0, 0);
    float2 tb1 = make_float2(0, 0);
    if (tvisco == GBSPH_VISCO_LAMINARSPS) { ta1 = a.taua[p1]; tb1 = a.taub[p1]; }
    const unsigned dcc = c.domcellcode, cel = a.dcell[p1];
    const CellGrid g = gb_grid((int)gb_cx(dcc, cel) - (int)d.cellmin[0], (int)gb_cy(dcc, cel) - (int)d.cellmin[1],
                               (int)gb_cz(dcc, cel) - (int)d.cellmin[2], c.cellmode_div, d);
    FluidAcc ff, fb;
    float4 sh = make_float4(0.f, 0.f, 0.f, 0.f);  // InitCpu without zones: zero
    fluid_pass<tvisco, tdensity, false, tshift>(c, a, d, g, ps1, vr1, ta1, tb1, c.visco, ff, sh);
    fluid_pass<tvisco, tdensity, true, tshift>(c, a, d, g, ps1, vr1, ta1, tb1, c.visco * c.viscoboundfactor, fb, sh);
    if (tshift) a.shiftpos[p1] = sh;
    // JSphCpu.cpp:1093-1113 and JSphCpuSingle.cpp:727-735
    float ar = ff.ar + fb.ar;
    if (tdensity != GBSPH_DDT_NONE) {
      const float dl = (ff.delta == FLT_MAX || fb.delta == FLT_MAX) ? FLT_MAX : ff.delta + fb.delta;
      if (dl != FLT_MAX) ar += dl;
    }
    const float ax = ff.ax + fb.ax, ay = ff.ay + fb.ay, az = ff.az + fb.az;
    a.acear[p1] = make_float4(ax, ay, az, ar);
    if (tvisco == GBSPH_VISCO_LAMINARSPS) {
      a.straina[p1] = make_float4(ff.s0 + fb.s0, ff.s1 + fb.s1, ff.s2 + fb.s2, ff.s3 + fb.s3);
      a.strainb[p1] = make_float2(ff.s4 + fb.s4, ff.s5 + fb.s5);
    }
    // a NaN density rate makes the maximum NaN (x + 0 * ar is x otherwise)
    acemax2 = ax * ax + ay * ay + az * az + 0.f * ar;
    visc = fmaxf(ff.visc, fb.visc);
    vel2 = vr1.x * vr1.x + vr1.y * vr1.y + vr1.z * vr1.z;
  }
  // block reduction of the maxima, one atomic per block
  gb_warp_maxes(a.st, acemax2, visc, vel2);
}

// ---- fluid rows, production kernel ----------------------------------------
// Lanes are target particles.  The neighbour test (the cheap part, ~1870
// candidates per particle in 27 cells of size 2h) runs in lock step over the
// 27 cells; the ~290 candidates per particle that pass it are queued per lane
// in shared memory (relative position + index), a ring of kQCap entries.  The
// pair terms (the expensive part) run in rounds: one round evaluates up to
// kRoundEntries of the oldest entries of every lane, and rounds are taken when
// kRoundLanes lanes hold that many (or when a queue could not take another
// unrolled group of checks), so the pair body runs with the lanes active.
// The checks and the viscosity term are written without branches: a warp
// nearly always has lanes on both sides of those tests.
// Summation order per particle is the candidate order.
constexpr int kQCap = 16;
constexpr int kQBlock = 128;
constexpr int kQUnroll = 4;
constexpr int kRoundEntries = 2;  // entries a lane evaluates per round
constexpr int kRoundLanes = 32;   // lanes that must hold kRoundEntries entries for a round

struct PairAcc {
  float ax, ay, az, ar, delta, visc;
  float s0, s1, s2, s3, s4, s5;
  float sh0, sh1, sh2, sh3;  // shifting sums (sh0 = FLT_MAX: cancelled)
};

// Float constants of the pair terms, derived on the host once per launch with
// the float operations the pair body would otherwise repeat per pair (the
// products keep the left-to-right association of the expressions they come
// from, so the results are bit-identical).  As a kernel argument the struct
// lives in the constant bank.
struct PairK {
  float hinv;            // 1/h
  float ddt_kc;          // ddtkh * cs0
  // artificial: -visco*cs0*2h (the h of mu_ij and the 1/2 of rhobar folded in);
  // laminar: 4*visco (fluid / boundary neighbours)
  float vfac_f, vfac_b;
  // rho0*((1+t)^a - 1) = t*(c1 + t*(c2 + t*(c3 + t*(c4 + t*c5)))) + O(t^6), a = 1/gamma:
  // the binomial series (times rho0) of the hydrostatic DDT2 term
  // rho0*((1+ddtgz*drz)^(1/gamma)-1), which avoids the cancellation of
  // pow()-1 (truncation below 1e-8 relative for |t| < 0.05)
  float c1, c2, c3, c4, c5;
  // staged kernel: log2 of the warps that share one group of 32 rows (each
  // takes every 2^lsplit-th chunk of the rows' candidate stream)
  unsigned lsplit;
};

PairK make_pairk(const gbsph_consts& c, int split = 1) {
  PairK k;
  k.lsplit = split >= 4 ? 2u : split >= 2 ? 1u : 0u;
  const float cbar = (float)c.cs0;
  k.hinv = 1.f / c.kernelh;
  k.ddt_kc = c.ddtkh * cbar;
  const float vb = c.visco * c.viscoboundfactor;
  if (c.tvisco == GBSPH_VISCO_ARTIFICIAL) {
    k.vfac_f = -c.visco * cbar * c.kernelh * 2.f;
    k.vfac_b = -vb * cbar * c.kernelh * 2.f;
  } else {
    k.vfac_f = 4.f * c.visco;
    k.vfac_b = 4.f * vb;
  }
  const float ga = 1.f / c.gamma;
  const float b1 = ga, b2 = b1 * (ga - 1.f) * 0.5f, b3 = b2 * (ga - 2.f) * (1.f / 3.f);
  const float b4 = b3 * (ga - 3.f) * 0.25f, b5 = b4 * (ga - 4.f) * 0.2f;
  k.c1 = c.rhopzero * b1; k.c2 = c.rhopzero * b2; k.c3 = c.rhopzero * b3;
  k.c4 = c.rhopzero * b4; k.c5 = c.rhopzero * b5;
  return k;
}


// Reciprocal with a relative error of at most 2 ulp (__fdividef), used for the
// 1/rho, 1/(r^2+eta^2) and 1/rhobar factors of the pair terms.
__device__ __forceinline__ float gb_rcp(float x) { return __fdividef(1.f, x); }

// Reciprocal and reciprocal square root, one MUFU instruction each, flushing
// subnormal inputs and results to zero (rcp.approx / rsqrt.approx .ftz: the
// inputs of the staged kernel's pair terms -- densities, r^2 + eta^2, r^2 of
// a real pair -- are normal floats, where they equal the forms above).
__device__ __forceinline__ float gb_rcp_ftz(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float gb_rsqrt_ftz(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}


// The pair terms of fluid row i and neighbour j, given dr = r_i - r_j, the
// neighbour's velrho and pressure, its SPS tau/rho^2 (read only for Laminar+SPS
// fluid neighbours) and whether it is a fixed boundary particle (read only by
// the NoFixed shifting mode).  With guard0 a pair closer than ALMOSTZERO
// (r^2 < 1e-18, a particle and itself) adds nothing, as the reference's
// neighbour test leaves it out (JSphCpu.cpp:826).
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift, bool guard0 = false>
__device__ __forceinline__ void pair_core(const gbsph_consts& c, const PairK& k, float drx, float dry, float drz,
                                          float4 vr2, float p2press, float4 ta2, float2 tb2, bool nbfixed,
                                          float4 vr1, float p1press, float inv_rho1, float4 ta1, float2 tb1,
                                          float vfac, float massp2, PairAcc& r) {
  // fluid neighbours (boundp2=false) are summed without their mass, which the
  // caller applies once to the pass's sums; the continuity sum leaves out rho1
  const float m2 = boundp2 ? massp2 : 1.f;
  const float rr2 = drx * drx + dry * dry + drz * drz;
  const bool real = !guard0 || rr2 >= GB_ALMOSTZERO;
  const float rinv = rsqrtf(rr2);
  const float qq = rr2 * rinv * k.hinv;
  const float wqq1 = 1.f - 0.5f * qq;
  const float fac0 = c.bwenh * wqq1 * wqq1 * wqq1;
  const float fac = real ? fac0 : 0.f;  // every term carries fac (or fr)
  const float frx = fac * drx, fry = fac * dry, frz = fac * drz;
  const float inv_rho2 = gb_rcp(vr2.w);
  // momentum
  const float p_vpm = -(p1press + p2press) * inv_rho1 * inv_rho2 * m2;
  r.ax += p_vpm * frx; r.ay += p_vpm * fry; r.az += p_vpm * frz;
  // continuity
  const float dvx = vr1.x - vr2.x, dvy = vr1.y - vr2.y, dvz = vr1.z - vr2.z;
  r.ar += m2 * (dvx * frx + dvy * fry + dvz * frz) * inv_rho2;
  const float inv_r2eta = gb_rcp(rr2 + c.eta2);
  if (tdensity == GBSPH_DDT_DDT && r.delta != FLT_MAX) {
    const float visc_densi = k.ddt_kc * (vr1.w * inv_rho2 - 1.f) * inv_r2eta;
    const float dot3 = drx * frx + dry * fry + drz * frz;
    r.delta = (boundp2 && c.tboundary == GBSPH_BC_DBC && real) ? FLT_MAX : r.delta + visc_densi * dot3 * m2;
  }
  if (tdensity == GBSPH_DDT_DDT2 || (tdensity == GBSPH_DDT_DDT2FULL && !boundp2)) {
    // the fluid neighbours are visited first, so only the boundary pass can
    // meet the veto (and it sets it: DDT2 leaves particles next to the boundary out)
    if (boundp2) {
      if (real) r.delta = FLT_MAX;
    } else {
      const float t = c.ddtgz * drz;
      float drho;
      if (ddtgen && !(fabsf(t) < 0.05f)) drho = c.rhopzero * powf(1.f + t, 1.f / c.gamma) - c.rhopzero;
      else drho = t * (k.c1 + t * (k.c2 + t * (k.c3 + t * (k.c4 + t * k.c5))));
      // the fluid pass sums the term without delta*2h*cs0, applied with the mass
      const float visc_densi = ((vr2.w - vr1.w) - drho) * inv_r2eta;
      const float dot3 = fac * rr2;  // r . gradW
      r.delta -= visc_densi * dot3 * inv_rho2;
    }
  }
  // shifting sums (JSphCpu.cpp:942-950), fluid ones without the mass
  if (tshift && r.sh0 != FLT_MAX) {
    const float massrho = m2 * inv_rho2;
    const bool noshift = boundp2 && real && (c.tshift == 1 || (c.tshift == 2 && nbfixed));
    r.sh0 = noshift ? FLT_MAX : r.sh0 + massrho * frx;
    r.sh1 += massrho * fry;
    r.sh2 += massrho * frz;
    r.sh3 -= massrho * (fac * rr2);  // r . gradW
  }
  // viscosity
  const float dot = drx * dvx + dry * dvy + drz * dvz;
  const float dot_rr2 = dot * inv_r2eta;
  r.visc = fmaxf(real ? dot_rr2 : 0.f, r.visc);
  if (tvisco == GBSPH_VISCO_ARTIFICIAL) {
    // applied for approaching pairs (dot < 0); evaluated for every pair and
    // selected, since nearly every warp has lanes on both sides of the test
    // -alpha*cs0*h*dot_rr2 / rhobar with rhobar = (rho1+rho2)/2 (h and 2 in vfac)
    const float pi_visc = dot < 0 ? (vfac * dot_rr2 * gb_rcp(vr1.w + vr2.w)) * m2 : 0.f;
    r.ax -= pi_visc * frx; r.ay -= pi_visc * fry; r.az -= pi_visc * frz;
  } else {
    const float robar2 = vr1.w + vr2.w;
    const float temp = vfac * inv_r2eta * gb_rcp(robar2);
    const float vtemp = m2 * temp * (drx * frx + dry * fry + drz * frz);
    r.ax += vtemp * dvx; r.ay += vtemp * dvy; r.az += vtemp * dvz;
    if (tvisco == GBSPH_VISCO_LAMINARSPS) {
      float t0 = ta1.x, t1 = ta1.y, t2 = ta1.z, t3 = ta1.w, t4 = tb1.x, t5 = tb1.y;
      if (!boundp2) {
        t0 += ta2.x; t1 += ta2.y; t2 += ta2.z; t3 += ta2.w; t4 += tb2.x; t5 += tb2.y;
      }
      r.ax += m2 * (t0 * frx + t1 * fry + t2 * frz);
      r.ay += m2 * (t1 * frx + t3 * fry + t4 * frz);
      r.az += m2 * (t2 * frx + t4 * fry + t5 * frz);
      const float volp2 = -m2 * inv_rho2;
      float dv = dvx * volp2; r.s0 += dv * frx; r.s1 += dv * fry; r.s2 += dv * frz;
      dv = dvy * volp2; r.s1 += dv * frx; r.s3 += dv * fry; r.s4 += dv * frz;
      dv = dvz * volp2; r.s2 += dv * frx; r.s4 += dv * fry; r.s5 += dv * frz;
    }
  }
}

// The pair terms of pair_core arranged for the staged kernel, with fewer
// operations per pair: every term is linear in the kernel gradient factor, so
// fac leaves out the constant bwenh, which the caller applies once per row
// (with the mass of the fluid neighbours; the boundary pass passes
// massp2 = massbound * bwenh); the pressure and viscosity terms of the
// momentum share one coefficient of dr, and the continuity term takes
// v_ij . gradW from the dr . v_ij of the viscosity.  A pair closer than
// ALMOSTZERO (a particle and itself) adds nothing.
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift>
__device__ __forceinline__ void pair_tile(const gbsph_consts& c, const PairK& k, float drx, float dry, float drz,
                                          float dvx, float dvy, float dvz, float rho2, float p2press, float4 ta2,
                                          float2 tb2, bool nbfixed, float4 vr1, float p1press, float inv_rho1,
                                          float4 ta1, float2 tb1, float vfac, float massp2, PairAcc& r) {
  const float m2 = boundp2 ? massp2 : 1.f;
  const float rr2 = drx * drx + dry * dry + drz * drz;
  const bool real = rr2 >= GB_ALMOSTZERO;
  const float rinv = gb_rsqrt_ftz(rr2);
  const float qq = rr2 * rinv * k.hinv;
  const float wqq1 = 1.f - 0.5f * qq;
  const float fac = real ? wqq1 * wqq1 * wqq1 : 0.f;  // gradW / (bwenh r)
  const float inv_rho2 = gb_rcp_ftz(rho2);
  const float inv_r2eta = gb_rcp_ftz(rr2 + c.eta2);
  const float dot = drx * dvx + dry * dvy + drz * dvz;  // r_ij . v_ij
  const float dot_rr2 = dot * inv_r2eta;
  r.visc = fmaxf(real ? dot_rr2 : 0.f, r.visc);
  const float dot3 = fac * rr2;  // r . gradW
  // momentum: pressure (and artificial viscosity) along dr
  float coef = -(p1press + p2press) * inv_rho1 * inv_rho2 * m2;
  if (tvisco == GBSPH_VISCO_ARTIFICIAL) {
    // applied for approaching pairs (dot < 0); -alpha*cs0*h*dot_rr2 / rhobar
    // with rhobar = (rho1+rho2)/2 (h and 2 in vfac)
    coef -= dot < 0 ? (vfac * dot_rr2 * gb_rcp_ftz(vr1.w + rho2)) * m2 : 0.f;
  }
  const float cf = coef * fac;
  r.ax += cf * drx; r.ay += cf * dry; r.az += cf * drz;
  // continuity: v_ij . gradW = fac * dot
  r.ar += (fac * dot) * inv_rho2 * m2;
  if (tdensity == GBSPH_DDT_DDT && r.delta != FLT_MAX) {
    const float visc_densi = k.ddt_kc * (vr1.w * inv_rho2 - 1.f) * inv_r2eta;
    r.delta = (boundp2 && c.tboundary == GBSPH_BC_DBC && real) ? FLT_MAX : r.delta + visc_densi * dot3 * m2;
  }
  if (tdensity == GBSPH_DDT_DDT2 || (tdensity == GBSPH_DDT_DDT2FULL && !boundp2)) {
    if (boundp2) {
      if (real) r.delta = FLT_MAX;
    } else {
      const float t = c.ddtgz * drz;
      float drho;
      if (ddtgen && !(fabsf(t) < 0.05f)) drho = c.rhopzero * powf(1.f + t, 1.f / c.gamma) - c.rhopzero;
      else drho = t * (k.c1 + t * (k.c2 + t * (k.c3 + t * (k.c4 + t * k.c5))));
      r.delta -= ((rho2 - vr1.w) - drho) * inv_r2eta * dot3 * inv_rho2;
    }
  }
  if (tshift && r.sh0 != FLT_MAX) {
    const float massrho = m2 * inv_rho2;
    const float mf = massrho * fac;
    const bool noshift = boundp2 && real && (c.tshift == 1 || (c.tshift == 2 && nbfixed));
    r.sh0 = noshift ? FLT_MAX : r.sh0 + mf * drx;
    r.sh1 += mf * dry;
    r.sh2 += mf * drz;
    r.sh3 -= massrho * dot3;
  }
  if (tvisco != GBSPH_VISCO_ARTIFICIAL) {
    const float temp = vfac * inv_r2eta * gb_rcp_ftz(vr1.w + rho2);
    const float vtemp = m2 * temp * dot3;
    r.ax += vtemp * dvx; r.ay += vtemp * dvy; r.az += vtemp * dvz;
    if (tvisco == GBSPH_VISCO_LAMINARSPS) {
      float t0 = ta1.x, t1 = ta1.y, t2 = ta1.z, t3 = ta1.w, t4 = tb1.x, t5 = tb1.y;
      if (!boundp2) {
        t0 += ta2.x; t1 += ta2.y; t2 += ta2.z; t3 += ta2.w; t4 += tb2.x; t5 += tb2.y;
      }
      const float mfac = m2 * fac;
      r.ax += mfac * (t0 * drx + t1 * dry + t2 * drz);
      r.ay += mfac * (t1 * drx + t3 * dry + t4 * drz);
      r.az += mfac * (t2 * drx + t4 * dry + t5 * drz);
      const float volp2 = -m2 * inv_rho2 * fac;
      float dv = dvx * volp2; r.s0 += dv * drx; r.s1 += dv * dry; r.s2 += dv * drz;
      dv = dvy * volp2; r.s1 += dv * drx; r.s3 += dv * dry; r.s4 += dv * drz;
      dv = dvz * volp2; r.s2 += dv * drx; r.s4 += dv * dry; r.s5 += dv * drz;
    }
  }
}

// Packed sums of the fluid pass of pair_tile2: component x sums the pairs a
// lane evaluates first in a round, y the second ones (added together after
// the pass); dsum is the DDT2 sum, subtracted from delta.
struct PairAcc2 {
  float2 ax, ay, az, ar, dsum;
};

// Two pairs of one fluid row against fluid neighbours (A in the x components,
// B in the y components), the terms of pair_tile for artificial viscosity and
// no or Fourtakas density diffusion, in packed f32x2 arithmetic: one
// instruction evaluates an operation for both pairs.  B is a copy of A (and
// adds nothing) when the lane has one pair only.
template <int tdensity, bool ddtgen>
__device__ __forceinline__ void pair_tile2(const gbsph_consts& c, const PairK& k, float2 dx, float2 dy, float2 dz,
                                           float2 dvx, float2 dvy, float2 dvz, float2 rho2, float2 p2, bool validb,
                                           float p1press, float rho1, float ninv_rho1, float vfac, PairAcc2& q,
                                           float& visc) {
  const float2 rr2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
  const bool reala = rr2.x >= GB_ALMOSTZERO, realb = validb && rr2.y >= GB_ALMOSTZERO;
  const float2 rinv = make_float2(gb_rsqrt_ftz(rr2.x), gb_rsqrt_ftz(rr2.y));
  const float2 qq = __fmul2_rn(__fmul2_rn(rr2, rinv), make_float2(k.hinv, k.hinv));
  const float2 w = __ffma2_rn(qq, make_float2(-0.5f, -0.5f), make_float2(1.f, 1.f));
  float2 fac = __fmul2_rn(__fmul2_rn(w, w), w);  // gradW / (bwenh r)
  fac.x = reala ? fac.x : 0.f;
  fac.y = realb ? fac.y : 0.f;
  const float2 inv_rho2 = make_float2(gb_rcp_ftz(rho2.x), gb_rcp_ftz(rho2.y));
  const float2 r2e = __fadd2_rn(rr2, make_float2(c.eta2, c.eta2));
  const float2 inv_r2eta = make_float2(gb_rcp_ftz(r2e.x), gb_rcp_ftz(r2e.y));
  const float2 dot = __ffma2_rn(dz, dvz, __ffma2_rn(dy, dvy, __fmul2_rn(dx, dvx)));  // r_ij . v_ij
  const float2 dot_rr2 = __fmul2_rn(dot, inv_r2eta);
  visc = fmaxf(reala ? dot_rr2.x : 0.f, visc);
  visc = fmaxf(realb ? dot_rr2.y : 0.f, visc);
  // momentum: -(p1+p2)/(rho1 rho2), minus the artificial viscosity of approaching pairs
  float2 coef = __fmul2_rn(__fmul2_rn(__fadd2_rn(make_float2(p1press, p1press), p2),
                                      make_float2(ninv_rho1, ninv_rho1)), inv_rho2);
  const float2 rs = __fadd2_rn(make_float2(rho1, rho1), rho2);
  float2 pv = __fmul2_rn(__fmul2_rn(make_float2(vfac, vfac), dot_rr2), make_float2(gb_rcp_ftz(rs.x), gb_rcp_ftz(rs.y)));
  pv.x = dot.x < 0.f ? pv.x : 0.f;
  pv.y = dot.y < 0.f ? pv.y : 0.f;
  coef = __ffma2_rn(pv, make_float2(-1.f, -1.f), coef);
  const float2 cf = __fmul2_rn(coef, fac);
  q.ax = __ffma2_rn(cf, dx, q.ax);
  q.ay = __ffma2_rn(cf, dy, q.ay);
  q.az = __ffma2_rn(cf, dz, q.az);
  // continuity: v_ij . gradW = fac * dot
  q.ar = __ffma2_rn(__fmul2_rn(fac, dot), inv_rho2, q.ar);
  if (tdensity == GBSPH_DDT_DDT2 || tdensity == GBSPH_DDT_DDT2FULL) {
    const float2 t = __fmul2_rn(make_float2(c.ddtgz, c.ddtgz), dz);
    float2 drho;
    if (ddtgen) {
      drho.x = !(fabsf(t.x) < 0.05f) ? c.rhopzero * powf(1.f + t.x, 1.f / c.gamma) - c.rhopzero
                                     : t.x * (k.c1 + t.x * (k.c2 + t.x * (k.c3 + t.x * (k.c4 + t.x * k.c5))));
      drho.y = !(fabsf(t.y) < 0.05f) ? c.rhopzero * powf(1.f + t.y, 1.f / c.gamma) - c.rhopzero
                                     : t.y * (k.c1 + t.y * (k.c2 + t.y * (k.c3 + t.y * (k.c4 + t.y * k.c5))));
    } else {
      float2 u = __ffma2_rn(t, make_float2(k.c5, k.c5), make_float2(k.c4, k.c4));
      u = __ffma2_rn(t, u, make_float2(k.c3, k.c3));
      u = __ffma2_rn(t, u, make_float2(k.c2, k.c2));
      u = __ffma2_rn(t, u, make_float2(k.c1, k.c1));
      drho = __fmul2_rn(t, u);
    }
    // ((rho2 - rho1) - drho) / (r^2 + eta^2) * (r . gradW) / rho2
    const float2 vd = __ffma2_rn(drho, make_float2(-1.f, -1.f), __fadd2_rn(rho2, make_float2(-rho1, -rho1)));
    q.dsum = __ffma2_rn(__fmul2_rn(__fmul2_rn(vd, inv_r2eta), __fmul2_rn(fac, rr2)), inv_rho2, q.dsum);
  }
}

// A queued entry e = (dr, neighbour index): the neighbour's SPS tau and code
// are read from global memory where the pair terms need them.
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift>
__device__ __forceinline__ void pair_fluid(const gbsph_consts& c, const PairK& k, const DevArrays& a,
                                           float4 e, float4 vr2, float p2press, float4 vr1,
                                           float p1press, float inv_rho1, float4 ta1, float2 tb1, float vfac,
                                           float massp2, PairAcc& r) {
  const unsigned p2 = __float_as_uint(e.w);
  float4 ta2 = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 tb2 = make_float2(0.f, 0.f);
  if (tvisco == GBSPH_VISCO_LAMINARSPS && !boundp2) { ta2 = a.taua[p2]; tb2 = a.taub[p2]; }
  bool nbfixed = false;
  if (tshift && boundp2) nbfixed = (a.code[p2] & GB_CODE_MASKTYPE) == 0u;
  pair_core<tvisco, tdensity, boundp2, ddtgen, tshift>(c, k, e.x, e.y, e.z, vr2, p2press, ta2, tb2, nbfixed, vr1,
                                                        p1press, inv_rho1, ta1, tb1, vfac, massp2, r);
}

// One round: every lane evaluates up to two of its oldest queued pairs, with
// the loads of both neighbours issued before either pair's arithmetic.
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift, int E>
__device__ __forceinline__ void pair_round(const gbsph_consts& c, const PairK& k, const DevArrays& a,
                                           float4 (*q)[32], unsigned& qh, int& n, float4 vr1,
                                           float p1press, float inv_rho1, float4 ta1, float2 tb1, float vfac,
                                           float massp2, PairAcc& r) {
  const int lane = threadIdx.x & 31;
  const bool va = n > 0, vb = E > 1 && n > 1;
  float4 ea = make_float4(0, 0, 0, 0), eb = ea, wa = make_float4(0, 0, 0, 1), wb = wa;
  float pa = 0, pb = 0;
  if (va) {
    ea = q[qh][lane];
    const unsigned p2 = __float_as_uint(ea.w);
    wa = a.velrho[p2];
    pa = a.pscell[p2].w;
  }
  if (E > 1 && vb) {
    eb = q[(qh + 1) & (kQCap - 1)][lane];
    const unsigned p2 = __float_as_uint(eb.w);
    wb = a.velrho[p2];
    pb = a.pscell[p2].w;
  }
  if (va)
    pair_fluid<tvisco, tdensity, boundp2, ddtgen, tshift>(c, k, a, ea, wa, pa, vr1, p1press, inv_rho1, ta1, tb1, vfac,
                                                  massp2, r);
  if (E > 1 && vb)
    pair_fluid<tvisco, tdensity, boundp2, ddtgen, tshift>(c, k, a, eb, wb, pb, vr1, p1press, inv_rho1, ta1, tb1, vfac,
                                                  massp2, r);
  const int used = (int)va + (int)vb;
  qh = (qh + used) & (kQCap - 1);
  n -= used;
}

// Candidate range of neighbour cell `ci` for this lane (empty outside the
// trimmed domain).
__device__ __forceinline__ void cell_range(const DevArrays& a, const DivState& d, const CellGrid& g, bool active,
                                           unsigned cellinit, int ci, int sd, int side, unsigned& pini,
                                           unsigned& len) {
  const int dz = ci / (side * side) - sd, dy = (ci / side) % side - sd, dx = ci % side - sd;
  const int x = g.cx + dx, y = g.cy + dy, z = g.cz + dz;
  pini = 0;
  len = 0;
  if (active && x >= g.xini && x < g.xfin && y >= g.yini && y < g.yfin && z >= g.zini && z < g.zfin) {
    const unsigned box = cellinit + (unsigned)x + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
    pini = a.begincell[box];
    len = a.begincell[box + 1] - pini;
  }
}

// One pass of the fluid rows over the fluid (boundp2=false) or boundary
// (boundp2=true) boxes of the 27 neighbour cells.
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift, int E, int F>
__device__ __forceinline__ void round_pass(const gbsph_consts& c, const PairK& k, const DevArrays& a,
                                           const DivState& d, const CellGrid& g, bool active, float4 ps1,
                                           float4 vr1, float inv_rho1, float4 ta1, float2 tb1,
                                           float4 (*q)[32], PairAcc& r) {
  const int lane = threadIdx.x & 31;
  const unsigned cellinit = boundp2 ? 0u : d.boxfluid;
  const float scell = c.scell, ks2 = c.kernelsize2;
  const float vfac = boundp2 ? k.vfac_b : k.vfac_f;
  const float massp2 = boundp2 ? c.massbound : c.massfluid;
  const int sd = c.cellmode_div, side = 2 * sd + 1, ncell = side * side * side, centre = ncell / 2;
  int n = 0;
  unsigned qh = 0;
  // The neighbour cells are taken two ranges at a time -- the centre cell split
  // in halves, then each cell with its mirror image through the centre -- and
  // half of every unrolled group of checks is drawn from either range.  A
  // particle near one face of its cell finds many neighbours in the cells on
  // that side and few on the opposite one; drawing from both sides at once
  // keeps the lanes' queues filling at similar rates, so rounds find more
  // lanes with work.
  for (int step = 0; step <= centre; step++) {
    const int cia = step == 0 ? centre : step - 1, cib = ncell - 1 - cia;
    unsigned pa, la, pb, lb;
    cell_range(a, d, g, active, cellinit, cia, sd, side, pa, la);
    if (step == 0) {
      const unsigned half = (la + 1) / 2;
      pb = pa + half;
      lb = la - half;
      la = half;
    } else {
      cell_range(a, d, g, active, cellinit, cib, sd, side, pb, lb);
    }
    const unsigned maxlen = __reduce_max_sync(0xffffffffu, la > lb ? la : lb);
    const int dza = cia / (side * side) - sd, dya = (cia / side) % side - sd, dxa = cia % side - sd;
    const int dzb = cib / (side * side) - sd, dyb = (cib / side) % side - sd, dxb = cib % side - sd;
    const float bax = ps1.x - (float)dxa * scell, bay = ps1.y - (float)dya * scell, baz = ps1.z - (float)dza * scell;
    const float bbx = ps1.x - (float)dxb * scell, bby = ps1.y - (float)dyb * scell, bbz = ps1.z - (float)dzb * scell;
    for (unsigned t0 = 0; t0 < maxlen; t0 += kQUnroll / 2) {
      // slots past a range's end read particle 0 (always valid) and are masked
      float4 ps2[kQUnroll];
      unsigned idx[kQUnroll];
      bool in[kQUnroll];
#pragma unroll
      for (int j = 0; j < kQUnroll; j++) {
        const bool fromb = j >= kQUnroll / 2;
        const unsigned t = t0 + (unsigned)(fromb ? j - kQUnroll / 2 : j);
        in[j] = t < (fromb ? lb : la);
        idx[j] = in[j] ? (fromb ? pb : pa) + t : 0u;
        ps2[j] = a.pscell[idx[j]];
      }
#pragma unroll
      for (int j = 0; j < kQUnroll; j++) {
        const bool fromb = j >= kQUnroll / 2;
        const float drx = (fromb ? bbx : bax) - ps2[j].x;
        const float dry = (fromb ? bby : bay) - ps2[j].y;
        const float drz = (fromb ? bbz : baz) - ps2[j].z;
        const float rr2 = drx * drx + dry * dry + drz * drz;
        if (in[j] && rr2 <= ks2 && rr2 >= GB_ALMOSTZERO) {
          q[(qh + n) & (kQCap - 1)][lane] = make_float4(drx, dry, drz, __uint_as_float(idx[j]));
          n++;
        }
      }
      // rounds while enough lanes have work, or while some queue has no room
      // for another unrolled group of checks
      for (;;) {
        const bool forced = __any_sync(0xffffffffu, n > kQCap - kQUnroll);
        if (!forced && __popc(__ballot_sync(0xffffffffu, n >= E)) < F) break;
        pair_round<tvisco, tdensity, boundp2, ddtgen, tshift, E>(c, k, a, q, qh, n, vr1, ps1.w, inv_rho1, ta1, tb1, vfac,
                                                      massp2, r);
      }
    }
  }
  while (__any_sync(0xffffffffu, n > 0))
    pair_round<tvisco, tdensity, boundp2, ddtgen, tshift, E>(c, k, a, q, qh, n, vr1, ps1.w, inv_rho1, ta1, tb1, vfac,
                                                  massp2, r);
}

template <int tvisco, int tdensity, bool ddtgen, bool tshift, int E = kRoundEntries, int F = kRoundLanes>
__global__ void __launch_bounds__(kQBlock) k_forces_fluid_q(gbsph_consts c, PairK k, DevArrays a) {
  __shared__ float4 qbuf[kQBlock / 32][kQCap][32];
  const DivState& d = *a.div;
  const unsigned np = d.np, npb = d.npb;
  const unsigned p1 = npb + blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = p1 < np;
  if (__all_sync(0xffffffffu, !active)) return;
  float4 ps1 = make_float4(0, 0, 0, 0), vr1 = make_float4(0, 0, 0, 1);
  float4 ta1 = make_float4(0, 0, 0, 0);
  float2 tb1 = make_float2(0, 0);
  CellGrid g;
  g.cx = g.cy = g.cz = 0; g.xini = g.xfin = g.yini = g.yfin = g.zini = g.zfin = 0;
  if (active) {
    ps1 = a.pscell[p1];
    vr1 = a.velrho[p1];
    if (tvisco == GBSPH_VISCO_LAMINARSPS) { ta1 = a.taua[p1]; tb1 = a.taub[p1]; }
    const unsigned dcc = c.domcellcode, cel = a.dcell[p1];
    g = gb_grid((int)gb_cx(dcc, cel) - (int)d.cellmin[0], (int)gb_cy(dcc, cel) - (int)d.cellmin[1],
                (int)gb_cz(dcc, cel) - (int)d.cellmin[2], c.cellmode_div, d);
  }
  const float inv_rho1 = gb_rcp(vr1.w);
  float4 (*q)[32] = qbuf[threadIdx.x >> 5];
  PairAcc ff = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  // one accumulator for both passes: the boundary pass adds to the fluid sums
  // (and sets the DDT veto, FLT_MAX in delta, where it applies)
  round_pass<tvisco, tdensity, false, ddtgen, tshift, E, F>(c, k, a, d, g, active, ps1, vr1, inv_rho1, ta1, tb1, q, ff);
  {  // the fluid-neighbour sums carry no mass yet
    const float mf = c.massfluid;
    ff.ax *= mf; ff.ay *= mf; ff.az *= mf; ff.ar *= mf; ff.delta *= mf;
    if (tdensity == GBSPH_DDT_DDT2 || tdensity == GBSPH_DDT_DDT2FULL) ff.delta *= k.ddt_kc;
    ff.s0 *= mf; ff.s1 *= mf; ff.s2 *= mf; ff.s3 *= mf; ff.s4 *= mf; ff.s5 *= mf;
    if (tshift) { ff.sh0 *= mf; ff.sh1 *= mf; ff.sh2 *= mf; ff.sh3 *= mf; }
  }
  round_pass<tvisco, tdensity, true, ddtgen, tshift, E, F>(c, k, a, d, g, active, ps1, vr1, inv_rho1, ta1, tb1, q, ff);
  ff.ar *= vr1.w;  // the rho1 factor of every continuity term
  float acemax2 = 0, visc = 0, vel2 = 0;
  if (active) {
    float ar = ff.ar;
    if (tdensity != GBSPH_DDT_NONE && ff.delta != FLT_MAX) ar += ff.delta;
    const float ax = ff.ax, ay = ff.ay, az = ff.az;
    a.acear[p1] = make_float4(ax, ay, az, ar);
    if (tvisco == GBSPH_VISCO_LAMINARSPS) {
      a.straina[p1] = make_float4(ff.s0, ff.s1, ff.s2, ff.s3);
      a.strainb[p1] = make_float2(ff.s4, ff.s5);
    }
    if (tshift) a.shiftpos[p1] = make_float4(ff.sh0, ff.sh1, ff.sh2, ff.sh3);
    // a NaN density rate makes the maximum NaN (x + 0 * ar is x otherwise)
    acemax2 = ax * ax + ay * ay + az * az + 0.f * ar;
    visc = ff.visc;
    vel2 = vr1.x * vr1.x + vr1.y * vr1.y + vr1.z * vr1.z;
  }
  gb_warp_maxes(a.st, acemax2, visc, vel2);
}

// ---- fluid rows, cell-tiled staged kernel ----------------------------------
// A warp takes 32 consecutive fluid rows (targets).  The candidate neighbours
// of its targets are the particles of the neighbour boxes, which in the sorted
// order form one contiguous range per row of boxes (JCellSearch_inline.h:33-84):
// for the targets of one row of cells (y, z) the candidates are the
// (2sd+1)^2 box rows around it, each over the x range of the targets' cells
// widened by sd.  These ranges, taken as one stream, are staged 32 candidates
// (a chunk) at a time through a per-warp ring of R chunks in shared memory.
// A chunk draws kTSeg consecutive candidates from each of 32/kTSeg equal
// parts of the stream, and the chunks are taken in a strided order, so that
// every few chunks sample the whole neighbourhood and the targets' hits
// arrive at similar rates (a lane whose hits come faster than the others'
// forces rounds in which the others idle); each lane stages one candidate
// with coalesced float4 loads (pscell, velrho), its position moved into the
// frame of one cell of the group.  The distance checks read the staged
// positions as broadcasts (structure of arrays, four candidates a load) and
// evaluate two candidates per packed f32x2 instruction; each lane's hits in a
// chunk form a 32-bit mask.  The pair terms then run in rounds in which every
// lane evaluates its next hit, reading the neighbour from shared memory; a
// round is taken when every target of the row group has a hit pending, or
// when the ring slot about to be refilled still holds one.  A candidate of the
// widened ranges that lies outside a target's own 27 (or 125) boxes is more
// than 2h away from it and fails the check, so the pairs are those of the
// per-target walk; the summation order per target is the order in which the
// chunks are taken.
constexpr int kTBlock = 128;
constexpr int kTSeg = 4;             // consecutive candidates a chunk takes from each part of the stream
constexpr float kFarAway = 1.0e18f;  // position of an empty ring slot: fails every check

template <int tvisco, bool tshift, int R>
struct TileLayout {
  static constexpr bool sps = tvisco == GBSPH_VISCO_LAMINARSPS;
  // per slot, as arrays: the negated frame position (12), pressure (4), the
  // negated velocity (12), density (4), the hit mask (4) [, tau a, tau b (24)]
  // [, fixed flag (4)]
  static constexpr size_t per_warp = (size_t)R * 32 * (36 + (sps ? 24 : 0) + (tshift ? 4 : 0));
  static constexpr size_t bytes = per_warp * (kTBlock / 32);
};

struct TileRing {
  float* f;       // the arrays below, R*32 entries each, from f
  float4* st;     // SPS tau a
  float2* stb;    // SPS tau b
  unsigned* sc;   // 1: fixed boundary particle (NoFixed shifting)
};
// arrays of the ring: -x, -y, -z of the frame position, pressure, -vx, -vy,
// -vz, density, hit masks (unsigned, [R][32])
enum { TR_NX = 0, TR_NY, TR_NZ, TR_PP, TR_NVX, TR_NVY, TR_NVZ, TR_RHO, TR_SM, TR_N };
template <int R>
__device__ __forceinline__ float* tr(const TileRing& r, int k) { return r.f + k * (R * 32); }
template <int R>
__device__ __forceinline__ unsigned* tr_sm(const TileRing& r) { return (unsigned*)(r.f + TR_SM * (R * 32)); }

// Pending hits of a lane: `cur` holds the unconsumed hits of chunk `cc`;
// chunks cc+1 .. cnext-1 have their masks in the ring.  With nothing pending,
// cc = cnext (the lane waits for the next chunk).
template <int R>
__device__ __forceinline__ void tile_refill(const TileRing& ring, unsigned& cur, unsigned& cc, unsigned cnext,
                                            int lane) {
  while (cur == 0u && cc + 1u < cnext) {
    cc++;
    cur = tr_sm<R>(ring)[(cc & (R - 1)) * 32 + lane];
  }
  if (cur == 0u) cc = cnext;
}

template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift, int R>
__device__ __forceinline__ void tile_round(const gbsph_consts& c, const PairK& k, const TileRing& ring,
                                           unsigned& cur, unsigned& cc, unsigned cnext, float fx, float fy,
                                           float fz, float4 vr1, float p1press, float inv_rho1, float4 ta1,
                                           float2 tb1, float vfac, float massp2, PairAcc& r, int lane) {
  if (cur != 0u) {
    const unsigned slot = ((cc & (R - 1)) << 5) | (unsigned)(__ffs(cur) - 1);
    cur &= cur - 1u;
    float4 ta2 = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 tb2 = make_float2(0.f, 0.f);
    if (tvisco == GBSPH_VISCO_LAMINARSPS && !boundp2) { ta2 = ring.st[slot]; tb2 = ring.stb[slot]; }
    const bool nbfixed = (tshift && boundp2) ? ring.sc[slot] != 0u : false;
    const float* e = ring.f + slot;
    pair_tile<tvisco, tdensity, boundp2, ddtgen, tshift>(
        c, k, fx + e[TR_NX * R * 32], fy + e[TR_NY * R * 32], fz + e[TR_NZ * R * 32], vr1.x + e[TR_NVX * R * 32],
        vr1.y + e[TR_NVY * R * 32], vr1.z + e[TR_NVZ * R * 32], e[TR_RHO * R * 32], e[TR_PP * R * 32], ta2, tb2,
        nbfixed, vr1, p1press, inv_rho1, ta1, tb1, vfac, massp2, r);
    tile_refill<R>(ring, cur, cc, cnext, lane);
  }
}

// A round of the packed fluid pass: every lane with a pending hit evaluates
// its next two (the second only when it has one) with pair_tile2.
template <int tdensity, bool ddtgen, int R>
__device__ __forceinline__ void tile_round2(const gbsph_consts& c, const PairK& k, const TileRing& ring,
                                            unsigned& cur, unsigned& cc, unsigned cnext, float fx, float fy,
                                            float fz, float4 vr1, float p1press, float ninv_rho1, float vfac,
                                            PairAcc2& q, float& visc, int lane) {
  if (cur != 0u) {
    const unsigned sa = ((cc & (R - 1)) << 5) | (unsigned)(__ffs(cur) - 1);
    cur &= cur - 1u;
    tile_refill<R>(ring, cur, cc, cnext, lane);
    const bool hb = cur != 0u;
    unsigned sb = sa;
    if (hb) {
      sb = ((cc & (R - 1)) << 5) | (unsigned)(__ffs(cur) - 1);
      cur &= cur - 1u;
      tile_refill<R>(ring, cur, cc, cnext, lane);
    }
    const float* ea = ring.f + sa;
    const float* eb = ring.f + sb;
    constexpr int S = R * 32;
    pair_tile2<tdensity, ddtgen>(
        c, k, __fadd2_rn(make_float2(fx, fx), make_float2(ea[TR_NX * S], eb[TR_NX * S])),
        __fadd2_rn(make_float2(fy, fy), make_float2(ea[TR_NY * S], eb[TR_NY * S])),
        __fadd2_rn(make_float2(fz, fz), make_float2(ea[TR_NZ * S], eb[TR_NZ * S])),
        __fadd2_rn(make_float2(vr1.x, vr1.x), make_float2(ea[TR_NVX * S], eb[TR_NVX * S])),
        __fadd2_rn(make_float2(vr1.y, vr1.y), make_float2(ea[TR_NVY * S], eb[TR_NVY * S])),
        __fadd2_rn(make_float2(vr1.z, vr1.z), make_float2(ea[TR_NVZ * S], eb[TR_NVZ * S])),
        make_float2(ea[TR_RHO * S], eb[TR_RHO * S]), make_float2(ea[TR_PP * S], eb[TR_PP * S]), hb, p1press, vr1.w,
        ninv_rho1, vfac, q, visc);
  }
}

// The fluid pass of these cases evaluates two pairs per lane and round in
// packed arithmetic (pair_tile2); the other cases one (pair_tile).
template <int tvisco, int tdensity, bool boundp2, bool tshift>
struct TilePacked {
  static constexpr bool value = !boundp2 && !tshift && tvisco == GBSPH_VISCO_ARTIFICIAL &&
                                (tdensity == GBSPH_DDT_NONE || tdensity == GBSPH_DDT_DDT2 ||
                                 tdensity == GBSPH_DDT_DDT2FULL);
};

// One round of whichever kind the case takes.
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift, int R>
__device__ __forceinline__ void tile_step(const gbsph_consts& c, const PairK& k, const TileRing& ring,
                                          unsigned& cur, unsigned& cc, unsigned cnext, float fx, float fy, float fz,
                                          float4 vr1, float p1press, float inv_rho1, float4 ta1, float2 tb1,
                                          float vfac, float massp2, PairAcc& r, PairAcc2& q, int lane) {
  if constexpr (TilePacked<tvisco, tdensity, boundp2, tshift>::value)
    tile_round2<tdensity, ddtgen, R>(c, k, ring, cur, cc, cnext, fx, fy, fz, vr1, p1press, -inv_rho1, vfac, q,
                                     r.visc, lane);
  else
    tile_round<tvisco, tdensity, boundp2, ddtgen, tshift, R>(c, k, ring, cur, cc, cnext, fx, fy, fz, vr1, p1press,
                                                             inv_rho1, ta1, tb1, vfac, massp2, r, lane);
}

// Hit bits of four staged candidates (positions negated, structure of arrays)
// for the lane at (fx, fy, fz): two candidates per packed instruction.
__device__ __forceinline__ unsigned tile_check4(float2 fxx, float2 fyy, float2 fzz, float4 x, float4 y, float4 z,
                                                float ks2, int q) {
  const float2 dx0 = __fadd2_rn(fxx, make_float2(x.x, x.y)), dx1 = __fadd2_rn(fxx, make_float2(x.z, x.w));
  const float2 dy0 = __fadd2_rn(fyy, make_float2(y.x, y.y)), dy1 = __fadd2_rn(fyy, make_float2(y.z, y.w));
  const float2 dz0 = __fadd2_rn(fzz, make_float2(z.x, z.y)), dz1 = __fadd2_rn(fzz, make_float2(z.z, z.w));
  float2 r0 = __fmul2_rn(dx0, dx0), r1 = __fmul2_rn(dx1, dx1);
  r0 = __ffma2_rn(dy0, dy0, r0);
  r1 = __ffma2_rn(dy1, dy1, r1);
  r0 = __ffma2_rn(dz0, dz0, r0);
  r1 = __ffma2_rn(dz1, dz1, r1);
  return ((r0.x <= ks2 ? 1u : 0u) | (r0.y <= ks2 ? 2u : 0u) | (r1.x <= ks2 ? 4u : 0u) | (r1.y <= ks2 ? 8u : 0u)) << q;
}

// Minimum / maximum of v over the lanes where `in` holds (an order-preserving
// integer image of the float, reduced by the warp).
__device__ __forceinline__ int tile_fkey(float v) {
  const int i = __float_as_int(v);
  return i ^ ((i >> 31) & 0x7fffffff);
}
__device__ __forceinline__ float tile_fmin(bool in, float v) {
  const int m = __reduce_min_sync(0xffffffffu, in ? tile_fkey(v) : 0x7fffffff);
  return __int_as_float(m ^ ((m >> 31) & 0x7fffffff));
}
__device__ __forceinline__ float tile_fmax(bool in, float v) {
  const int m = __reduce_max_sync(0xffffffffu, in ? tile_fkey(v) : (int)0x80000000);
  return __int_as_float(m ^ ((m >> 31) & 0x7fffffff));
}

// Checks the full chunk cnext of the ring (four staged candidates per
// broadcast load), stores every lane's hit mask, then runs rounds while every
// target of the row group has a hit pending.
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift, int R>
__device__ __forceinline__ void tile_check(const gbsph_consts& c, const PairK& k, const TileRing& ring,
                                           unsigned& cur, unsigned& cc, unsigned& cnext, float fx, float fy,
                                           float fz, float2 fxx, float2 fyy, float2 fzz, float ks2, unsigned gmask,
                                           bool ing, unsigned grp, float4 vr1, float p1press, float inv_rho1,
                                           float4 ta1, float2 tb1, float vfac, float massp2, PairAcc& r,
                                           PairAcc2& q2, int lane) {
  const unsigned base = (cnext & (R - 1)) << 5;
  unsigned m = 0u;
#pragma unroll
  for (int q = 0; q < 32; q += 4) {
    const float4 xq = *(const float4*)(tr<R>(ring, TR_NX) + base + q);
    const float4 yq = *(const float4*)(tr<R>(ring, TR_NY) + base + q);
    const float4 zq = *(const float4*)(tr<R>(ring, TR_NZ) + base + q);
    m |= tile_check4(fxx, fyy, fzz, xq, yq, zq, ks2, q);
  }
  m &= gmask;
  tr_sm<R>(ring)[base + lane] = m;
  if (cc == cnext) cur = m;
  cnext++;
  if (cur == 0u) cc = cnext;
  while (__ballot_sync(0xffffffffu, ing && cur != 0u) == grp)
    tile_step<tvisco, tdensity, boundp2, ddtgen, tshift, R>(c, k, ring, cur, cc, cnext, fx, fy, fz, vr1, p1press,
                                                            inv_rho1, ta1, tb1, vfac, massp2, r, q2, lane);
}

// One pass of the warp's fluid rows over the fluid (boundp2=false) or boundary
// (boundp2=true) boxes.  cx, cy, cz: the lane's cell in the trimmed domain.
template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift, int R, bool tsplit>
__device__ __forceinline__ void tile_pass(const gbsph_consts& c, const PairK& k, const DevArrays& a,
                                          const DivState& d, const TileRing& ring, bool active, int cx, int cy,
                                          int cz, float4 ps1, float4 vr1, float inv_rho1, float4 ta1, float2 tb1,
                                          PairAcc& r) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned cellinit = boundp2 ? 0u : d.boxfluid;
  const float scell = c.scell, ks2 = c.kernelsize2;
  const float vfac = boundp2 ? k.vfac_b : k.vfac_f;
  // the boundary pass's terms carry their mass and the constant of gradW (pair_tile)
  const float massp2 = boundp2 ? c.massbound * c.bwenh : c.massfluid;
  const int sd = c.cellmode_div;
  const int ncx = (int)d.ncx, ncy = (int)d.ncy, ncz = (int)d.ncz;
  const unsigned dcc = c.domcellcode, cmin0 = d.cellmin[0];
  unsigned cnext = 0u, cc = 0u, cur = 0u;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  PairAcc2 q2 = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f),
                 make_float2(0.f, 0.f)};
  unsigned remaining = __ballot_sync(FULL, active);
  while (remaining) {
    // the targets in the row of cells of the lowest remaining lane
    const int leader = __ffs(remaining) - 1;
    const int rx = __shfl_sync(FULL, cx, leader), ry = __shfl_sync(FULL, cy, leader),
              rz = __shfl_sync(FULL, cz, leader);
    const bool ing = active && cy == ry && cz == rz;
    const unsigned grp = __ballot_sync(FULL, ing);
    remaining &= ~grp;
    const int xmin = __reduce_min_sync(FULL, ing ? cx : 0x7fffffff);
    const int xmax = __reduce_max_sync(FULL, ing ? cx : -1);
    const int x0 = max(xmin - sd, 0), x1 = min(xmax + sd, ncx - 1);
    const int y0 = max(ry - sd, 0), y1 = min(ry + sd, ncy - 1);
    const int z0 = max(rz - sd, 0), z1 = min(rz + sd, ncz - 1);
    const int nyr = y1 - y0 + 1, nrows = nyr * (z1 - z0 + 1);  // at most 25
    // lane w < nrows holds box row w: first candidate, count, end in the stream
    unsigned rb = 0u, rlen = 0u;
    int rdy = 0, rdz = 0;
    if (lane < nrows) {
      const int y = y0 + lane % nyr, z = z0 + lane / nyr;
      const unsigned rowbase = cellinit + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
      rb = a.begincell[rowbase + (unsigned)x0];
      rlen = a.begincell[rowbase + (unsigned)x1 + 1u] - rb;
      rdy = y - ry;
      rdz = z - rz;
    }
    unsigned incl = rlen;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    const unsigned total = __shfl_sync(FULL, incl, 31);
    if (total == 0u) continue;
    const unsigned rbase = rb - (incl - rlen);  // candidate index = rbase + stream position
    if (ing) {  // the lane's position in the frame of cell (rx, ry, rz)
      fx = ps1.x + (float)(cx - rx) * scell;
      fy = ps1.y;
      fz = ps1.z;
    }
    const float2 fxx = make_float2(fx, fx), fyy = make_float2(fy, fy), fzz = make_float2(fz, fz);
    const unsigned gmask = ing ? FULL : 0u;
    // the box of the group's targets: a candidate farther than 2h from it is
    // no target's neighbour and is not staged (the margin keeps every
    // candidate the check would accept, whatever the rounding)
    const float blox = tile_fmin(ing, fx), bloy = tile_fmin(ing, fy), bloz = tile_fmin(ing, fz);
    const float bhix = tile_fmax(ing, fx), bhiy = tile_fmax(ing, fy), bhiz = tile_fmax(ing, fz);
    const float ks2m = ks2 * 1.0001f;
    unsigned fill = 0u;  // entries staged in the open chunk (chunk cnext)
    // Chunk ch (taken in the order ch = i * stride mod nch, a stride near
    // 0.618 nch and coprime with it, so that consecutive chunks lie far apart
    // in every part of the stream) has this lane stage stream position
    // s = part * plen + ch * kTSeg + lane % kTSeg.
    const unsigned nch = (total + 31u) >> 5, plen = nch * kTSeg;
    unsigned stride = max(1u, (unsigned)__float2uint_rn(0.6180339887f * (float)nch));
    for (;;) {  // the smallest stride from there that is coprime with nch
      unsigned u = stride, v = nch;
      while (v) { const unsigned t = u % v; u = v; v = t; }
      if (u == 1u) break;
      stride++;
    }
    const unsigned pbase = (unsigned)(lane / kTSeg) * plen + (unsigned)(lane % kTSeg);
    const unsigned send = min((unsigned)(lane / kTSeg + 1) * plen, total);  // end of this lane's part
    unsigned ch = 0u, mine = nch;
    if constexpr (tsplit) {
      // a warp of a split row group takes every 2^lsplit-th chunk of that
      // order, from its index in the group on (sub * stride and
      // stride * 2^lsplit mod nch by additions: sub < 4)
      const unsigned sub = ((unsigned)threadIdx.x >> 5) & ((1u << k.lsplit) - 1u);
      for (unsigned j = 0; j < sub; j++) ch = (ch + stride >= nch) ? ch + stride - nch : ch + stride;
      for (unsigned j = 0; j < k.lsplit; j++) stride = (2u * stride >= nch) ? 2u * stride - nch : 2u * stride;
      mine = nch > sub ? (nch - sub + (1u << k.lsplit) - 1u) >> k.lsplit : 0u;
    }
    for (unsigned i = 0; i < mine; i++, ch = (ch + stride >= nch) ? ch + stride - nch : ch + stride) {
      const unsigned s = pbase + ch * kTSeg;
      // the box row holding s: the number of rows whose end is <= s
      int lo = 0, hi = nrows;
#pragma unroll
      for (int it = 0; it < 5; it++) {
        const int mid = (lo + hi) >> 1;
        const bool le = __shfl_sync(FULL, incl, mid & 31) <= s;
        if (lo < hi) {
          if (le) lo = mid + 1;
          else hi = mid;
        }
      }
      const bool has = s < send;
      const int rowc = min(lo, 31);
      const unsigned jb = __shfl_sync(FULL, rbase, rowc);
      const int dyj = __shfl_sync(FULL, rdy, rowc), dzj = __shfl_sync(FULL, rdz, rowc);
      float4 ps2 = make_float4(kFarAway, kFarAway, kFarAway, 0.f), vr2 = make_float4(0.f, 0.f, 0.f, 1.f);
      float4 ta2 = make_float4(0.f, 0.f, 0.f, 0.f);
      float2 tb2 = make_float2(0.f, 0.f);
      unsigned fixed = 0u;
      if (has) {
        const unsigned j = jb + s;
        ps2 = a.pscell[j];
        vr2 = a.velrho[j];
        const int dxj = (int)(gb_cx(dcc, a.dcell[j]) - cmin0) - rx;
        if (tvisco == GBSPH_VISCO_LAMINARSPS && !boundp2) { ta2 = a.taua[j]; tb2 = a.taub[j]; }
        if (tshift && boundp2) fixed = (a.code[j] & GB_CODE_MASKTYPE) == 0u ? 1u : 0u;
        ps2.x += (float)dxj * scell;
        ps2.y += (float)dyj * scell;
        ps2.z += (float)dzj * scell;
      }
      // keep the candidates near the targets' box; they fill the open chunk
      // in stream order and run over into the next one
      bool keep = false;
      if (has) {
        const float ex = fmaxf(fmaxf(blox - ps2.x, ps2.x - bhix), 0.f);
        const float ey = fmaxf(fmaxf(bloy - ps2.y, ps2.y - bhiy), 0.f);
        const float ez = fmaxf(fmaxf(bloz - ps2.z, ps2.z - bhiz), 0.f);
        keep = ex * ex + ey * ey + ez * ez <= ks2m;
      }
      const unsigned kb = __ballot_sync(FULL, keep);
      if (kb == 0u) continue;
      const unsigned nk = (unsigned)__popc(kb);
      // the ring slots written must hold no pending hit (of chunk cnext - R,
      // and of cnext + 1 - R when the entries run over)
      const unsigned need = fill + nk > 32u ? cnext + 1u : cnext;
      while (__any_sync(FULL, cur != 0u && cc + (unsigned)R <= need))
        tile_step<tvisco, tdensity, boundp2, ddtgen, tshift, R>(c, k, ring, cur, cc, cnext, fx, fy, fz, vr1, ps1.w,
                                                                inv_rho1, ta1, tb1, vfac, massp2, r, q2, lane);
      if (keep) {
        const unsigned pos = fill + (unsigned)__popc(kb & ((1u << lane) - 1u));
        const unsigned slot = (((pos < 32u ? cnext : cnext + 1u) & (R - 1)) << 5) | (pos & 31u);
        float* e = ring.f + slot;
        constexpr int S = R * 32;
        e[TR_NX * S] = -ps2.x;
        e[TR_NY * S] = -ps2.y;
        e[TR_NZ * S] = -ps2.z;
        e[TR_PP * S] = ps2.w;
        e[TR_NVX * S] = -vr2.x;
        e[TR_NVY * S] = -vr2.y;
        e[TR_NVZ * S] = -vr2.z;
        e[TR_RHO * S] = vr2.w;
        if (tvisco == GBSPH_VISCO_LAMINARSPS && !boundp2) { ring.st[slot] = ta2; ring.stb[slot] = tb2; }
        if (tshift && boundp2) ring.sc[slot] = fixed;
      }
      fill += nk;
      if (fill >= 32u) {
        __syncwarp();
        tile_check<tvisco, tdensity, boundp2, ddtgen, tshift, R>(c, k, ring, cur, cc, cnext, fx, fy, fz, fxx, fyy,
                                                                 fzz, ks2, gmask, ing, grp, vr1, ps1.w, inv_rho1,
                                                                 ta1, tb1, vfac, massp2, r, q2, lane);
        fill -= 32u;
      }
    }
    if (fill) {  // the last chunk of the group: empty slots fail every check
      const unsigned base = (cnext & (R - 1)) << 5;
      if ((unsigned)lane >= fill) {
        tr<R>(ring, TR_NX)[base + lane] = -kFarAway;
        tr<R>(ring, TR_NY)[base + lane] = -kFarAway;
        tr<R>(ring, TR_NZ)[base + lane] = -kFarAway;
      }
      __syncwarp();
      tile_check<tvisco, tdensity, boundp2, ddtgen, tshift, R>(c, k, ring, cur, cc, cnext, fx, fy, fz, fxx, fyy, fzz,
                                                               ks2, gmask, ing, grp, vr1, ps1.w, inv_rho1, ta1, tb1,
                                                               vfac, massp2, r, q2, lane);
      fill = 0u;
    }
  }
  while (__any_sync(FULL, cur != 0u))
    tile_step<tvisco, tdensity, boundp2, ddtgen, tshift, R>(c, k, ring, cur, cc, cnext, fx, fy, fz, vr1, ps1.w,
                                                            inv_rho1, ta1, tb1, vfac, massp2, r, q2, lane);
  if constexpr (TilePacked<tvisco, tdensity, boundp2, tshift>::value) {
    r.ax += q2.ax.x + q2.ax.y;
    r.ay += q2.ay.x + q2.ay.y;
    r.az += q2.az.x + q2.az.y;
    r.ar += q2.ar.x + q2.ar.y;
    if (tdensity == GBSPH_DDT_DDT2 || tdensity == GBSPH_DDT_DDT2FULL) r.delta -= q2.dsum.x + q2.dsum.y;
  }
  __syncwarp();  // the next pass reuses the ring
}

// Adds the partial sums of the other warps of a row group (PairAcc fields
// in shared memory, field-major) to warp 0's: sums, visc a maximum, and the
// cancellation markers (delta, sh0 = FLT_MAX) kept if any warp set them.
template <int tdensity, bool tshift>
__device__ __forceinline__ void tile_combine(PairAcc& r, const float* part, int lane) {
  constexpr int S = 32;
  r.ax += part[0 * S + lane]; r.ay += part[1 * S + lane]; r.az += part[2 * S + lane]; r.ar += part[3 * S + lane];
  if (tdensity != GBSPH_DDT_NONE) {
    const float dl = part[4 * S + lane];
    r.delta = (r.delta == FLT_MAX || dl == FLT_MAX) ? FLT_MAX : r.delta + dl;
  }
  r.visc = fmaxf(r.visc, part[5 * S + lane]);
  r.s0 += part[6 * S + lane]; r.s1 += part[7 * S + lane]; r.s2 += part[8 * S + lane];
  r.s3 += part[9 * S + lane]; r.s4 += part[10 * S + lane]; r.s5 += part[11 * S + lane];
  if (tshift) {
    const float h0 = part[12 * S + lane];
    r.sh0 = (r.sh0 == FLT_MAX || h0 == FLT_MAX) ? FLT_MAX : r.sh0 + h0;
    r.sh1 += part[13 * S + lane]; r.sh2 += part[14 * S + lane]; r.sh3 += part[15 * S + lane];
  }
}

template <int tvisco, int tdensity, bool ddtgen, bool tshift, int R, bool tsplit>
// Six blocks of 128 threads per SM leave up to 80 registers a thread; the
// Laminar+SPS and shifting cases, with more sums per row, take four.
// tsplit: 2^k.lsplit consecutive warps (2 or 4) take the same 32 rows, each
// every 2^lsplit-th chunk of their candidate streams (more warps in flight
// for cases too small to fill the device), and the first of them adds the
// others' partial sums (named barrier per row group) and writes the rows.
// A separate instantiation, so that the one-warp kernel keeps its registers;
// it runs small cases, far below a full wave, so it takes four blocks a SM
// (up to 128 registers a thread, no spills).
__global__ void __launch_bounds__(kTBlock, (tvisco == GBSPH_VISCO_LAMINARSPS || tshift || tsplit) ? 4 : 6)
    k_forces_fluid_t(gbsph_consts c, PairK k, DevArrays a) {
  extern __shared__ float4 tile_smem[];
  using L = TileLayout<tvisco, tshift, R>;
  const DivState& d = *a.div;
  const unsigned np = d.np, npb = d.npb;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned p1 = tsplit ? npb + blockIdx.x * (kTBlock >> k.lsplit) + (((unsigned)warp >> k.lsplit) << 5) + (unsigned)lane
                             : npb + blockIdx.x * kTBlock + threadIdx.x;
  const bool active = p1 < np;
  // the same for every warp of a row group, so a group leaves together
  if (__all_sync(0xffffffffu, !active)) return;
  char* wbase = (char*)tile_smem + (size_t)warp * L::per_warp;
  TileRing ring;
  ring.f = (float*)wbase;
  float* const fend = ring.f + TR_N * (R * 32);  // after the hit masks
  ring.st = L::sps ? (float4*)fend : nullptr;
  ring.stb = L::sps ? (float2*)(ring.st + R * 32) : nullptr;
  ring.sc = tshift ? (unsigned*)(L::sps ? (void*)(ring.stb + R * 32) : (void*)fend) : nullptr;
  float4 ps1 = make_float4(0, 0, 0, 0), vr1 = make_float4(0, 0, 0, 1);
  float4 ta1 = make_float4(0, 0, 0, 0);
  float2 tb1 = make_float2(0, 0);
  int cx = 0, cy = 0, cz = 0;
  if (active) {
    ps1 = a.pscell[p1];
    vr1 = a.velrho[p1];
    if (tvisco == GBSPH_VISCO_LAMINARSPS) { ta1 = a.taua[p1]; tb1 = a.taub[p1]; }
    const unsigned dcc = c.domcellcode, cel = a.dcell[p1];
    cx = (int)gb_cx(dcc, cel) - (int)d.cellmin[0];
    cy = (int)gb_cy(dcc, cel) - (int)d.cellmin[1];
    cz = (int)gb_cz(dcc, cel) - (int)d.cellmin[2];
  }
  const float inv_rho1 = gb_rcp(vr1.w);
  PairAcc ff = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  tile_pass<tvisco, tdensity, false, ddtgen, tshift, R, tsplit>(c, k, a, d, ring, active, cx, cy, cz, ps1, vr1, inv_rho1, ta1,
                                                         tb1, ff);
  {  // the fluid-neighbour sums carry neither the mass nor the constant of gradW yet
    const float mf = c.massfluid * c.bwenh;
    ff.ax *= mf; ff.ay *= mf; ff.az *= mf; ff.ar *= mf; ff.delta *= mf;
    if (tdensity == GBSPH_DDT_DDT2 || tdensity == GBSPH_DDT_DDT2FULL) ff.delta *= k.ddt_kc;
    ff.s0 *= mf; ff.s1 *= mf; ff.s2 *= mf; ff.s3 *= mf; ff.s4 *= mf; ff.s5 *= mf;
    if (tshift) { ff.sh0 *= mf; ff.sh1 *= mf; ff.sh2 *= mf; ff.sh3 *= mf; }
  }
  tile_pass<tvisco, tdensity, true, ddtgen, tshift, R, tsplit>(c, k, a, d, ring, active, cx, cy, cz, ps1, vr1, inv_rho1, ta1,
                                                        tb1, ff);
  if constexpr (tsplit) {
    // partial sums through the warps' own rings (free after the passes; 2 KB
    // of the at least 4.6 KB of a ring); the thread index is read anew, which
    // keeps the warp index out of registers during the passes
    unsigned tid;
    asm volatile("mov.u32 %0, %%tid.x;" : "=r"(tid));
    const unsigned lsplit = k.lsplit, wl = tid >> 5, ln = tid & 31u;
    const unsigned nthreads = 32u << lsplit, barid = 1u + (wl >> lsplit), sub = wl & ((1u << lsplit) - 1u);
    if (sub) {
      float* part = (float*)((char*)tile_smem + (size_t)wl * L::per_warp);
      const float v[16] = {ff.ax, ff.ay, ff.az, ff.ar, ff.delta, ff.visc, ff.s0, ff.s1,
                           ff.s2, ff.s3, ff.s4, ff.s5, ff.sh0, ff.sh1, ff.sh2, ff.sh3};
#pragma unroll
      for (int f = 0; f < 16; f++) part[f * 32 + ln] = v[f];
    }
    asm volatile("bar.sync %0, %1;" ::"r"(barid), "r"(nthreads) : "memory");
    if (sub) return;
    for (unsigned w = 1; w < (1u << lsplit); w++)
      tile_combine<tdensity, tshift>(ff, (const float*)((const char*)tile_smem + (size_t)(wl + w) * L::per_warp),
                                     (int)ln);
  }
  ff.ar *= vr1.w;  // the rho1 factor of every continuity term
  float acemax2 = 0, visc = 0, vel2 = 0;
  if (active) {
    float ar = ff.ar;
    if (tdensity != GBSPH_DDT_NONE && ff.delta != FLT_MAX) ar += ff.delta;
    const float ax = ff.ax, ay = ff.ay, az = ff.az;
    a.acear[p1] = make_float4(ax, ay, az, ar);
    if (tvisco == GBSPH_VISCO_LAMINARSPS) {
      a.straina[p1] = make_float4(ff.s0, ff.s1, ff.s2, ff.s3);
      a.strainb[p1] = make_float2(ff.s4, ff.s5);
    }
    if (tshift) a.shiftpos[p1] = make_float4(ff.sh0, ff.sh1, ff.sh2, ff.sh3);
    // a NaN density rate makes the maximum NaN (x + 0 * ar is x otherwise)
    acemax2 = ax * ax + ay * ay + az * az + 0.f * ar;
    visc = ff.visc;
    vel2 = vr1.x * vr1.x + vr1.y * vr1.y + vr1.z * vr1.z;
  }
  gb_warp_maxes(a.st, acemax2, visc, vel2);
}

// The staged kernel with a ring of R chunks; with prepare set, only raises its
// dynamic shared-memory limit (done once per context, outside any capture).
template <int tvisco, int tdensity, bool ddtgen, bool tshift, int R, bool tsplit>
cudaError_t launch_tiled(const gbsph_consts& c, const PairK& k, const DevArrays& a, unsigned cap, bool prepare,
                         cudaStream_t s) {
  using L = TileLayout<tvisco, tshift, R>;
  static_assert(L::per_warp >= 16 * 32 * sizeof(float), "a ring holds the partial sums of a split row group");
  if (prepare)
    return cudaFuncSetAttribute(k_forces_fluid_t<tvisco, tdensity, ddtgen, tshift, R, tsplit>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::bytes);
  const unsigned rows_per_block = (unsigned)kTBlock >> (tsplit ? k.lsplit : 0u);
  k_forces_fluid_t<tvisco, tdensity, ddtgen, tshift, R, tsplit>
      <<<gb_div_up(cap, rows_per_block), kTBlock, L::bytes, s>>>(c, k, a);
  return cudaSuccess;
}

template <int tvisco, int tdensity, bool ddtgen, bool tshift>
cudaError_t launch_fluid_g(const gbsph_consts& c, const PairK& k, const DevArrays& a, unsigned cap, int variant,
                           bool prepare, cudaStream_t s) {
  // the split row groups (k.lsplit > 0) are instantiated for the ring of 8
  // chunks and the series form of the hydrostatic term; otherwise one warp
  // takes a row group
  if (prepare) {
    cudaError_t e = launch_tiled<tvisco, tdensity, ddtgen, tshift, 8, false>(c, k, a, cap, true, s);
    if (e == cudaSuccess && !ddtgen) e = launch_tiled<tvisco, tdensity, ddtgen, tshift, 8, true>(c, k, a, cap, true, s);
    if (e == cudaSuccess) e = launch_tiled<tvisco, tdensity, ddtgen, tshift, 4, false>(c, k, a, cap, true, s);
    return e;
  }
  if (variant == 2) {
    if constexpr (!ddtgen) {
      if (k.lsplit) return launch_tiled<tvisco, tdensity, ddtgen, tshift, 8, true>(c, k, a, cap, false, s);
    }
    return launch_tiled<tvisco, tdensity, ddtgen, tshift, 8, false>(c, k, a, cap, false, s);
  }
  if (variant == 3) return launch_tiled<tvisco, tdensity, ddtgen, tshift, 4, false>(c, k, a, cap, false, s);
  k_forces_fluid_q<tvisco, tdensity, ddtgen, tshift><<<gb_div_up(cap, kQBlock), kQBlock, 0, s>>>(c, k, a);
  return cudaSuccess;
}

template <int tvisco, int tdensity, bool tshift>
cudaError_t launch_fluid(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, int split,
                         bool prepare, cudaStream_t s) {
  if (variant == 1 && !prepare) {  // one thread per row: any block size of 64, 128 or 256
    const unsigned bs = (bsize == 64 || bsize == 256) ? (unsigned)bsize : 128u;
    k_forces_fluid<tvisco, tdensity, tshift><<<gb_div_up(cap, bs), bs, 0, s>>>(c, a);
    return cudaSuccess;
  }
  // split row groups: the staged kernel with a ring of 8 chunks (variant 2)
  const PairK k = make_pairk(c, variant == 2 ? split : 1);
  if constexpr (tdensity == GBSPH_DDT_DDT2 || tdensity == GBSPH_DDT_DDT2FULL) {
    // the series form of the hydrostatic term holds for |ddtgz*drz| < 0.05 and
    // |drz| <= 2h for every pair; otherwise the general power form is compiled in
    if (!(fabsf(c.ddtgz) * c.kernelsize < 0.049f))
      return launch_fluid_g<tvisco, tdensity, true, tshift>(c, k, a, cap, variant, prepare, s);
  }
  return launch_fluid_g<tvisco, tdensity, false, tshift>(c, k, a, cap, variant, prepare, s);
}

template <int tvisco, int tdensity>
cudaError_t launch_fluid_s(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, int split,
                           bool prepare, cudaStream_t s) {
  if (c.tshift) return launch_fluid<tvisco, tdensity, true>(c, a, cap, variant, bsize, split, prepare, s);
  return launch_fluid<tvisco, tdensity, false>(c, a, cap, variant, bsize, split, prepare, s);
}

template <int tvisco>
cudaError_t launch_fluid_t(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, int split,
                           bool prepare, cudaStream_t s) {
  switch (c.tdensity) {
    case GBSPH_DDT_NONE: return launch_fluid_s<tvisco, GBSPH_DDT_NONE>(c, a, cap, variant, bsize, split, prepare, s);
    case GBSPH_DDT_DDT: return launch_fluid_s<tvisco, GBSPH_DDT_DDT>(c, a, cap, variant, bsize, split, prepare, s);
    case GBSPH_DDT_DDT2: return launch_fluid_s<tvisco, GBSPH_DDT_DDT2>(c, a, cap, variant, bsize, split, prepare, s);
    default: return launch_fluid_s<tvisco, GBSPH_DDT_DDT2FULL>(c, a, cap, variant, bsize, split, prepare, s);
  }
}

}  // namespace

namespace gbk {
// The fluid-row pass of one viscosity model (variant, block size and split as
// in gbk::forces; with prepare set, only raises the staged kernels' dynamic
// shared-memory limits): gbsph_fluid_art.cu, gbsph_fluid_lam.cu,
// gbsph_fluid_sps.cu.
cudaError_t fluid_artificial(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize,
                             int split, bool prepare, cudaStream_t s);
cudaError_t fluid_laminar(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, int split,
                          bool prepare, cudaStream_t s);
cudaError_t fluid_laminarsps(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize,
                             int split, bool prepare, cudaStream_t s);
}  // namespace gbk
