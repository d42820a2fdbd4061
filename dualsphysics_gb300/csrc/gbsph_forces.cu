// gbsph_forces.cu -- Interaction_Forces and the mDBC ghost-node correction.
//
// Fluid rows restate JSphCpu::InteractionForcesFluid (JSphCpu.cpp:736-1141;
// GPU twin KerInteractionForcesFluidBox, JSphGpu_ker.cu:542-990): Wendland C2
// kernel gradient, Tait pressure (precomputed per particle), Monaghan
// artificial viscosity or Laminar+SPS, Molteni (DDT) or Fourtakas (DDT2)
// density diffusion with the veto for particles with boundary neighbours.
// Bound rows restate JSphCpu::InteractionForcesBound (JSphCpu.cpp:633-703).
// The maxima the dt needs (|ace|^2 over fluid, visc, |v|^2) are reduced in
// the same kernels (JSphGpuSingle.cpp:719-729, JSphGpu.cpp:846-900).
//
// Pair distance: every particle carries its position relative to the origin of
// its own cell (pscell.xyz, rounded once from double); a neighbour in cell cj
// is at (lp_i - lp_j) + (ci - cj)*Scell, which needs no FP64 in the pair loop.
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
    acemax2 = ax * ax + ay * ay + az * az;
    visc = fmaxf(ff.visc, fb.visc);
    vel2 = vr1.x * vr1.x + vr1.y * vr1.y + vr1.z * vr1.z;
  }
  // block reduction of the maxima, one atomic per block
  for (int o = 16; o; o >>= 1) {
    acemax2 = fmaxf(acemax2, __shfl_xor_sync(0xffffffffu, acemax2, o));
    visc = fmaxf(visc, __shfl_xor_sync(0xffffffffu, visc, o));
    vel2 = fmaxf(vel2, __shfl_xor_sync(0xffffffffu, vel2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (acemax2 > 0) gb_atomic_max_nonneg(&a.st->acemax2, acemax2);
    if (visc > 0) gb_atomic_max_nonneg(&a.st->viscdt, visc);
    if (vel2 > 0) gb_atomic_max_nonneg(&a.st->velmax2, vel2);
  }
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
};

PairK make_pairk(const gbsph_consts& c) {
  PairK k;
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


template <int tvisco, int tdensity, bool boundp2, bool ddtgen, bool tshift>
__device__ __forceinline__ void pair_fluid(const gbsph_consts& c, const PairK& k, const DevArrays& a,
                                           float4 e, float4 vr2, float p2press, float4 vr1,
                                           float p1press, float inv_rho1, float4 ta1, float2 tb1, float vfac,
                                           float massp2, PairAcc& r) {
  // fluid neighbours (boundp2=false) are summed without their mass, which the
  // caller applies once to the pass's sums; the continuity sum leaves out rho1
  const float m2 = boundp2 ? massp2 : 1.f;
  const unsigned p2 = __float_as_uint(e.w);
  const float drx = e.x, dry = e.y, drz = e.z;
  const float rr2 = drx * drx + dry * dry + drz * drz;
  const float rinv = rsqrtf(rr2);
  const float qq = rr2 * rinv * k.hinv;
  const float wqq1 = 1.f - 0.5f * qq;
  const float fac = c.bwenh * wqq1 * wqq1 * wqq1;
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
    r.delta = (boundp2 && c.tboundary == GBSPH_BC_DBC) ? FLT_MAX : r.delta + visc_densi * dot3 * m2;
  }
  if (tdensity == GBSPH_DDT_DDT2 || (tdensity == GBSPH_DDT_DDT2FULL && !boundp2)) {
    // the fluid neighbours are visited first, so only the boundary pass can
    // meet the veto (and it sets it: DDT2 leaves particles next to the boundary out)
    if (boundp2) {
      r.delta = FLT_MAX;
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
    const bool noshift = boundp2 && (c.tshift == 1 || (c.tshift == 2 && (a.code[p2] & GB_CODE_MASKTYPE) == 0u));
    r.sh0 = noshift ? FLT_MAX : r.sh0 + massrho * frx;
    r.sh1 += massrho * fry;
    r.sh2 += massrho * frz;
    r.sh3 -= massrho * (fac * rr2);  // r . gradW
  }
  // viscosity
  const float dot = drx * dvx + dry * dvy + drz * dvz;
  const float dot_rr2 = dot * inv_r2eta;
  r.visc = fmaxf(dot_rr2, r.visc);
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
        const float4 ta2 = a.taua[p2];
        const float2 tb2 = a.taub[p2];
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
    acemax2 = ax * ax + ay * ay + az * az;
    visc = ff.visc;
    vel2 = vr1.x * vr1.x + vr1.y * vr1.y + vr1.z * vr1.z;
  }
  for (int o = 16; o; o >>= 1) {
    acemax2 = fmaxf(acemax2, __shfl_xor_sync(0xffffffffu, acemax2, o));
    visc = fmaxf(visc, __shfl_xor_sync(0xffffffffu, visc, o));
    vel2 = fmaxf(vel2, __shfl_xor_sync(0xffffffffu, vel2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (acemax2 > 0) gb_atomic_max_nonneg(&a.st->acemax2, acemax2);
    if (visc > 0) gb_atomic_max_nonneg(&a.st->viscdt, visc);
    if (vel2 > 0) gb_atomic_max_nonneg(&a.st->velmax2, vel2);
  }
}

// Bound rows (JSphCpu.cpp:633-703): continuity and visc from fluid neighbours.
__global__ void __launch_bounds__(128) k_forces_bound(gbsph_consts c, DevArrays a) {
  const DivState& d = *a.div;
  const unsigned npb = d.npb, npbok = d.npbok;
  const unsigned p1 = blockIdx.x * blockDim.x + threadIdx.x;
  float visc = 0, vel2 = 0;
  if (p1 < npb) {
    float arp1 = 0;
    if (p1 < npbok) {
      const float4 ps1 = a.pscell[p1];
      const float4 vr1 = a.velrho[p1];
      const unsigned dcc = c.domcellcode, cel = a.dcell[p1];
      const CellGrid g = gb_grid((int)gb_cx(dcc, cel) - (int)d.cellmin[0], (int)gb_cy(dcc, cel) - (int)d.cellmin[1],
                                 (int)gb_cz(dcc, cel) - (int)d.cellmin[2], c.cellmode_div, d);
      const float scell = c.scell, ks2 = c.kernelsize2, h = c.kernelh, bwenh = c.bwenh, eta2 = c.eta2;
      const float massp2 = c.massfluid;
      for (int z = g.zini; z < g.zfin; z++) {
        for (int y = g.yini; y < g.yfin; y++) {
          const unsigned rowbase = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
          const float by = ps1.y + (float)(g.cy - y) * scell, bz = ps1.z + (float)(g.cz - z) * scell;
          for (int x = g.xini; x < g.xfin; x++) {
            const unsigned box = rowbase + (unsigned)x;
            const unsigned pini = a.begincell[box], pfin = a.begincell[box + 1];
            const float bx = ps1.x + (float)(g.cx - x) * scell;
            for (unsigned p2 = pini; p2 < pfin; p2++) {
              const float4 ps2 = a.pscell[p2];
              const float drx = bx - ps2.x, dry = by - ps2.y, drz = bz - ps2.z;
              const float rr2 = drx * drx + dry * dry + drz * drz;
              if (rr2 <= ks2 && rr2 >= GB_ALMOSTZERO) {
                const float rad = sqrtf(rr2);
                const float qq = rad / h;
                const float wqq1 = 1.f - 0.5f * qq;
                const float fac = bwenh * wqq1 * wqq1 * wqq1;
                const float frx = fac * drx, fry = fac * dry, frz = fac * drz;
                const float4 vr2 = a.velrho[p2];
                const float dvx = vr1.x - vr2.x, dvy = vr1.y - vr2.y, dvz = vr1.z - vr2.z;
                arp1 += massp2 * (dvx * frx + dvy * fry + dvz * frz) * (vr1.w / vr2.w);
                const float dot = drx * dvx + dry * dvy + drz * dvz;
                visc = fmaxf(dot / (rr2 + eta2), visc);
              }
            }
          }
        }
      }
      if (c.dtallparticles) vel2 = vr1.x * vr1.x + vr1.y * vr1.y + vr1.z * vr1.z;
    }
    a.acear[p1] = make_float4(0.f, 0.f, 0.f, arp1);
  }
  for (int o = 16; o; o >>= 1) {
    visc = fmaxf(visc, __shfl_xor_sync(0xffffffffu, visc, o));
    vel2 = fmaxf(vel2, __shfl_xor_sync(0xffffffffu, vel2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (visc > 0) gb_atomic_max_nonneg(&a.st->viscdt, visc);
    if (vel2 > 0) gb_atomic_max_nonneg(&a.st->velmax2, vel2);
  }
}

// JSphCpu::ComputeSpsTau (JSphCpu.cpp:1279-1309) for fluid particles.
__global__ void k_sps_tau(gbsph_consts c, DevArrays a) {
  const DivState& d = *a.div;
  const unsigned p = d.npb + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.np) return;
  const float4 sa = a.straina[p];
  const float2 sb = a.strainb[p];
  const float xx = sa.x, xy = sa.y, xz = sa.z, yy = sa.w, yz = sb.x, zz = sb.y;
  const float pow1 = xx * xx + yy * yy + zz * zz;
  const float prr = xy * xy + xz * xz + yz * yz + pow1 + pow1;
  const float visc_sps = c.spssmag * sqrtf(prr);
  const float div_u = xx + yy + zz;
  const float sps_k = visc_sps * div_u;
  const float sps_blin = c.spsblin * prr;
  const float sumsps = -(sps_k + sps_blin);
  const float twovisc_sps = visc_sps + visc_sps;
  const float one_rho = 1.0f / a.velrho[p].w;
  a.taua[p] = make_float4(one_rho * (twovisc_sps * xx + sumsps), one_rho * (visc_sps * xy), one_rho * (visc_sps * xz),
                          one_rho * (twovisc_sps * yy + sumsps));
  a.taub[p] = make_float2(one_rho * (visc_sps * yz), one_rho * (twovisc_sps * zz + sumsps));
}

// ---- mDBC ghost-node correction, SlipMode=vel0, 3-D -------------------------
// JSphCpu_mdbc.cpp:36-160 (GPU twin KerInteractionMdbcCorrection_Fast,
// JSphGpu_mdbc_iker.cu:34-151).  The CPU path accumulates the 4x4 moment
// matrix in double; here each entry is a compensated FP32 sum (TwoSum: the
// rounding error of every addition is carried in a second float), which keeps
// about 48 significant bits without FP64 adds.  The first-order system is
// solved in double by Gaussian elimination with partial pivoting (one
// reciprocal per pivot; the determinant for the 1e-3 test is the signed
// product of the pivots), where the reference forms the inverse from
// cofactors: the solutions agree to ~1e-15 relative, and the FP64 work, slow
// on this part, drops about fourfold.  A ghost node with no fluid neighbour
// takes rho0 without a solve, as the reference's zero matrix leads it to.
__device__ __forceinline__ void gb_kadd(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
  hi = s;
  lo = __fadd_rn(lo, e);
}

__global__ void __launch_bounds__(128) k_mdbc(gbsph_consts c, DevArrays a) {
  const DivState& d = *a.div;
  const unsigned p1 = blockIdx.x * blockDim.x + threadIdx.x;
  if (p1 >= d.npbok) return;
  const float4 bn = a.boundnor[p1];
  if (bn.x == 0.f && bn.y == 0.f && bn.z == 0.f) return;
  double gx = a.px[p1] + (double)bn.x, gy = a.py[p1] + (double)bn.y, gz = a.pz[p1] + (double)bn.z;
  // the ghost node taken back into the domain across periodic faces
  // (UpdatePeriodicPos, JSphCpu_mdbc.cpp:50, JSph.cpp:2079-2101)
  if (c.peri[0] || c.peri[1] || c.peri[2]) {
    double dx = __dsub_rn(gx, c.maprealposmin[0]), dy = __dsub_rn(gy, c.maprealposmin[1]),
           dz = __dsub_rn(gz, c.maprealposmin[2]);
    const bool out = dx != dx || dy != dy || dz != dz || dx < 0 || dy < 0 || dz < 0 || dx >= c.maprealsize[0] ||
                     dy >= c.maprealsize[1] || dz >= c.maprealsize[2];
    if (out) {
      for (int k = 0; k < 3; k++) {
        if (!c.peri[k]) continue;
        const double* inc = c.periinc + 3 * k;
        if ((k == 0 ? dx : k == 1 ? dy : dz) < 0) {
          dx = __dsub_rn(dx, inc[0]); dy = __dsub_rn(dy, inc[1]); dz = __dsub_rn(dz, inc[2]);
        }
        if ((k == 0 ? dx : k == 1 ? dy : dz) >= c.maprealsize[k]) {
          dx = __dadd_rn(dx, inc[0]); dy = __dadd_rn(dy, inc[1]); dz = __dadd_rn(dz, inc[2]);
        }
      }
      gx = __dadd_rn(dx, c.maprealposmin[0]); gy = __dadd_rn(dy, c.maprealposmin[1]); gz = __dadd_rn(dz, c.maprealposmin[2]);
    }
  }
  const double sc = (double)c.scell;
  // cell of the ghost node, truncated toward zero as int() does (JCellSearch_inline.h:59-61)
  const int gcx = (int)((gx - c.domposmin[0]) / sc), gcy = (int)((gy - c.domposmin[1]) / sc),
            gcz = (int)((gz - c.domposmin[2]) / sc);
  const float glx = (float)(gx - c.domposmin[0] - (double)gcx * sc);
  const float gly = (float)(gy - c.domposmin[1] - (double)gcy * sc);
  const float glz = (float)(gz - c.domposmin[2] - (double)gcz * sc);
  const CellGrid g = gb_grid(gcx - (int)d.cellmin[0], gcy - (int)d.cellmin[1], gcz - (int)d.cellmin[2],
                             c.cellmode_div, d);
  const float scell = c.scell, ks2 = c.kernelsize2, h = c.kernelh;
  float rhop1 = 0, grx = 0, gry = 0, grz = 0;
  unsigned nfound = 0;
  float Ah[4][4], Al[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) Ah[i][j] = Al[i][j] = 0.f;
  for (int z = g.zini; z < g.zfin; z++) {
    for (int y = g.yini; y < g.yfin; y++) {
      const unsigned rowbase = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
      const float by = gly + (float)(g.cy - y) * scell, bz = glz + (float)(g.cz - z) * scell;
      for (int x = g.xini; x < g.xfin; x++) {
        const unsigned box = rowbase + (unsigned)x;
        const unsigned pini = a.begincell[box], pfin = a.begincell[box + 1];
        const float bx = glx + (float)(g.cx - x) * scell;
        for (unsigned p2 = pini; p2 < pfin; p2++) {
          const float4 ps2 = a.pscell[p2];
          const float drx = bx - ps2.x, dry = by - ps2.y, drz = bz - ps2.z;
          const float rr2 = drx * drx + dry * dry + drz * drz;
          if (rr2 <= ks2 && (a.code[p2] & GB_CODE_MASKTYPE) == GB_CODE_TYPE_FLUID) {
            nfound++;
            // Wendland WabFac (FunSphKernel.h:235-246)
            const float rad = sqrtf(rr2);
            const float qq = rad / h;
            const float wqq1 = 1.f - 0.5f * qq;
            const float wqq2 = wqq1 * wqq1;
            const float fac = c.bwenh * wqq2 * wqq1;
            const float wqq = qq + qq + 1.f;
            const float wab = c.awen * wqq * wqq2 * wqq2;
            const float frx = fac * drx, fry = fac * dry, frz = fac * drz;
            const float rhop2 = a.velrho[p2].w;
            const float massp2 = c.massfluid;
            const float volp2 = massp2 / rhop2;
            rhop1 += massp2 * wab;
            grx += massp2 * frx; gry += massp2 * fry; grz += massp2 * frz;
            const float vwab = wab * volp2, vfrx = frx * volp2, vfry = fry * volp2, vfrz = frz * volp2;
            const float rowv[4] = {vwab, vfrx, vfry, vfrz};
#pragma unroll
            for (int i = 0; i < 4; i++) {
              gb_kadd(Ah[i][0], Al[i][0], rowv[i]);
              gb_kadd(Ah[i][1], Al[i][1], __fmul_rn(drx, rowv[i]));
              gb_kadd(Ah[i][2], Al[i][2], __fmul_rn(dry, rowv[i]));
              gb_kadd(Ah[i][3], Al[i][3], __fmul_rn(drz, rowv[i]));
            }
          }
        }
      }
    }
  }
  float rhofinal = FLT_MAX;
  if (nfound) {
    // [A | b] with A the moment matrix and b = (rho, grad rho)
    double M[4][5];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) M[i][j] = (double)Ah[i][j] + (double)Al[i][j];
    M[0][4] = rhop1; M[1][4] = grx; M[2][4] = gry; M[3][4] = grz;
    const double a00 = M[0][0];
    double det = 1.0, rinv[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
#pragma unroll
      for (int r = k + 1; r < 4; r++) {  // bring the largest |M[r][k]| (r >= k) to row k
        if (fabs(M[r][k]) > fabs(M[k][k])) {
#pragma unroll
          for (int q = k; q < 5; q++) {
            const double t = M[k][q];
            M[k][q] = M[r][q];
            M[r][q] = t;
          }
          det = -det;
        }
      }
      const double piv = M[k][k];
      det *= piv;
      const double inv = piv != 0.0 ? 1.0 / piv : 0.0;
      rinv[k] = inv;
#pragma unroll
      for (int r = k + 1; r < 4; r++) {
        const double f = M[r][k] * inv;
#pragma unroll
        for (int q = k + 1; q < 5; q++) M[r][q] = fma(-f, M[k][q], M[r][q]);
      }
    }
    if (fabs(det) >= 1e-3f) {
      double xs[4];
#pragma unroll
      for (int k = 3; k >= 0; k--) {
        double t = M[k][4];
#pragma unroll
        for (int q = k + 1; q < 4; q++) t = fma(-M[k][q], xs[q], t);
        xs[k] = t * rinv[k];
      }
      const float rhoghost = (float)xs[0];
      const float ggx = -(float)xs[1], ggy = -(float)xs[2], ggz = -(float)xs[3];
      rhofinal = rhoghost + ggx * (-bn.x) + ggy * (-bn.y) + ggz * (-bn.z);
    } else if (a00 > 0) {
      rhofinal = (float)(rhop1 / a00);
    }
  }
  rhofinal = (rhofinal != FLT_MAX) ? rhofinal : c.rhopzero;
  float4 vr = a.velrho[p1];
  vr.w = rhofinal;
  a.velrho[p1] = vr;
  float4 ps = a.pscell[p1];
  ps.w = gb_press(rhofinal, c.rhopzero, c.cteb, c.gamma);
  a.pscell[p1] = ps;
}

// Particle-interaction count (JDsPips::ComputeGpu / KerInteractionNg,
// JDsPips.cpp:268, JDsPips_ker.cu:66): checked and real (r^2 <= (2h)^2,
// r^2 >= ALMOSTZERO) pairs of bound rows (fluid neighbours) and of fluid rows
// (fluid and bound neighbours).  out = {checked bound, real bound, checked fluid,
// real fluid}.
__global__ void k_pips(gbsph_consts c, DevArrays a) {
  const DivState& d = *a.div;
  const unsigned p1 = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long cnt[4] = {0, 0, 0, 0};
  const bool bound = p1 < d.npbok;
  const bool fluid = p1 >= d.npb && p1 < d.np;
  if (bound || fluid) {
    const float4 ps1 = a.pscell[p1];
    const unsigned dcc = c.domcellcode, cel = a.dcell[p1];
    const CellGrid g = gb_grid((int)gb_cx(dcc, cel) - (int)d.cellmin[0], (int)gb_cy(dcc, cel) - (int)d.cellmin[1],
                               (int)gb_cz(dcc, cel) - (int)d.cellmin[2], c.cellmode_div, d);
    for (int pass = 0; pass < (fluid ? 2 : 1); pass++) {
      const unsigned cellinit = (pass == 0) ? d.boxfluid : 0u;
      for (int z = g.zini; z < g.zfin; z++)
        for (int y = g.yini; y < g.yfin; y++)
          for (int x = g.xini; x < g.xfin; x++) {
            const unsigned box = cellinit + (unsigned)x + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
            const unsigned pini = a.begincell[box], pfin = a.begincell[box + 1];
            const float bx = ps1.x + (float)(g.cx - x) * c.scell;
            const float by = ps1.y + (float)(g.cy - y) * c.scell;
            const float bz = ps1.z + (float)(g.cz - z) * c.scell;
            for (unsigned p2 = pini; p2 < pfin; p2++) {
              const float4 ps2 = a.pscell[p2];
              const float drx = bx - ps2.x, dry = by - ps2.y, drz = bz - ps2.z;
              const float rr2 = drx * drx + dry * dry + drz * drz;
              const int k = fluid ? 2 : 0;
              cnt[k]++;
              if (rr2 <= c.kernelsize2 && rr2 >= GB_ALMOSTZERO) cnt[k + 1]++;
            }
          }
    }
  }
  for (int k = 0; k < 4; k++) {
    unsigned long long v = cnt[k];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&a.pips[k], v);
  }
}

template <int tvisco, int tdensity, bool tshift>
void launch_fluid(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, cudaStream_t s) {
  if (variant == 1) {  // one thread per row: any block size of 64, 128 or 256
    const unsigned bs = (bsize == 64 || bsize == 256) ? (unsigned)bsize : 128u;
    k_forces_fluid<tvisco, tdensity, tshift><<<gb_div_up(cap, bs), bs, 0, s>>>(c, a);
    return;
  }
  const PairK k = make_pairk(c);
  const unsigned grid = gb_div_up(cap, kQBlock);
  if constexpr (tdensity == GBSPH_DDT_DDT2 || tdensity == GBSPH_DDT_DDT2FULL) {
    // the series form of the hydrostatic term holds for |ddtgz*drz| < 0.05 and
    // |drz| <= 2h for every pair; otherwise the general power form is compiled in
    if (!(fabsf(c.ddtgz) * c.kernelsize < 0.049f)) {
      k_forces_fluid_q<tvisco, tdensity, true, tshift><<<grid, kQBlock, 0, s>>>(c, k, a);
      return;
    }
  }
  k_forces_fluid_q<tvisco, tdensity, false, tshift><<<grid, kQBlock, 0, s>>>(c, k, a);
}

template <int tvisco, int tdensity>
void launch_fluid_s(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, cudaStream_t s) {
  if (c.tshift) launch_fluid<tvisco, tdensity, true>(c, a, cap, variant, bsize, s);
  else launch_fluid<tvisco, tdensity, false>(c, a, cap, variant, bsize, s);
}

template <int tvisco>
void launch_fluid_t(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, cudaStream_t s) {
  switch (c.tdensity) {
    case GBSPH_DDT_NONE: launch_fluid_s<tvisco, GBSPH_DDT_NONE>(c, a, cap, variant, bsize, s); break;
    case GBSPH_DDT_DDT: launch_fluid_s<tvisco, GBSPH_DDT_DDT>(c, a, cap, variant, bsize, s); break;
    case GBSPH_DDT_DDT2: launch_fluid_s<tvisco, GBSPH_DDT_DDT2>(c, a, cap, variant, bsize, s); break;
    default: launch_fluid_s<tvisco, GBSPH_DDT_DDT2FULL>(c, a, cap, variant, bsize, s); break;
  }
}

}  // namespace

namespace gbk {

void forces(const gbsph_consts& c, const DevArrays& a, unsigned cap, int bsize, int variant, cudaStream_t s,
            unsigned long long* nlaunch, cudaEvent_t ev_fluid_begin, cudaEvent_t ev_fluid_end) {
  cudaMemsetAsync(&a.st->acemax2, 0, 3 * sizeof(unsigned), s);
  k_forces_bound<<<gb_div_up(cap, 128), 128, 0, s>>>(c, a);
  // inside a stream capture the records must be external nodes so that every
  // replay of the graph records them; outside a capture they are plain records
  cudaStreamCaptureStatus cap_st = cudaStreamCaptureStatusNone;
  if (ev_fluid_begin || ev_fluid_end) cudaStreamIsCapturing(s, &cap_st);
  const unsigned ev_flags = cap_st == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
  if (ev_fluid_begin) cudaEventRecordWithFlags(ev_fluid_begin, s, ev_flags);
  switch (c.tvisco) {
    case GBSPH_VISCO_ARTIFICIAL: launch_fluid_t<GBSPH_VISCO_ARTIFICIAL>(c, a, cap, variant, bsize, s); break;
    case GBSPH_VISCO_LAMINAR: launch_fluid_t<GBSPH_VISCO_LAMINAR>(c, a, cap, variant, bsize, s); break;
    default: launch_fluid_t<GBSPH_VISCO_LAMINARSPS>(c, a, cap, variant, bsize, s); break;
  }
  if (ev_fluid_end) cudaEventRecordWithFlags(ev_fluid_end, s, ev_flags);
  if (nlaunch) *nlaunch += 2;
}

void sps_tau(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s, unsigned long long* nlaunch) {
  k_sps_tau<<<gb_div_up(cap, 256), 256, 0, s>>>(c, a);
  if (nlaunch) *nlaunch += 1;
}

void pips(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s) {
  cudaMemsetAsync(a.pips, 0, 4 * sizeof(unsigned long long), s);
  k_pips<<<gb_div_up(cap, 128), 128, 0, s>>>(c, a);
}

void mdbc(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s, unsigned long long* nlaunch) {
  k_mdbc<<<gb_div_up(cap, 128), 128, 0, s>>>(c, a);
  if (nlaunch) *nlaunch += 1;
}

}  // namespace gbk
