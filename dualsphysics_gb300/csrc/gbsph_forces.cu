// gbsph_forces.cu -- Interaction_Forces of the bound rows, the mDBC ghost-node
// correction, the PIPS count and the dispatch of the fluid-row kernels
// (gbsph_fluid.cuh).
//
// Bound rows restate JSphCpu::InteractionForcesBound (JSphCpu.cpp:633-703).
#include <cuda_runtime.h>
#include <float.h>

#include "gbsph_common.cuh"
// the helpers this file shares with the fluid-row kernels; the kernels
// themselves are instantiated in gbsph_fluid_*.cu
#pragma nv_diag_suppress 177
#include "gbsph_fluid.cuh"
#pragma nv_diag_default 177

namespace {

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
  gb_warp_maxes(a.st, 0.f, visc, vel2);
}

// The same bound rows with G lanes a row (G = 4 or 32), for cases too small
// to fill the device with one thread a row: the lanes of a row take the
// candidates of each (y, z) box row in turn (a contiguous range of the sorted
// order, each candidate's x cell from its dcell) and their sums are added
// across the G lanes (the order of the sum changes, within the FP32
// criterion).
template <int G>
__global__ void __launch_bounds__(128) k_forces_bound_g(gbsph_consts c, DevArrays a) {
  static_assert(G == 4 || G == 8 || G == 16 || G == 32, "lanes a row");
  const DivState& d = *a.div;
  const unsigned npb = d.npb, npbok = d.npbok;
  const unsigned p1 = (unsigned)(((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) / G);
  const unsigned sl = threadIdx.x & (G - 1);
  float visc = 0, vel2 = 0, arp1 = 0;
  float4 vr1 = make_float4(0.f, 0.f, 0.f, 1.f);
  if (p1 < npbok) {
    const float4 ps1 = a.pscell[p1];
    vr1 = a.velrho[p1];
    const unsigned dcc = c.domcellcode, cel = a.dcell[p1], cmin0 = d.cellmin[0];
    const CellGrid g = gb_grid((int)gb_cx(dcc, cel) - (int)cmin0, (int)gb_cy(dcc, cel) - (int)d.cellmin[1],
                               (int)gb_cz(dcc, cel) - (int)d.cellmin[2], c.cellmode_div, d);
    const float scell = c.scell, ks2 = c.kernelsize2, h = c.kernelh, bwenh = c.bwenh, eta2 = c.eta2;
    const float massp2 = c.massfluid;
    for (int z = g.zini; z < g.zfin; z++) {
      for (int y = g.yini; y < g.yfin; y++) {
        const unsigned rowbase = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
        const float by = ps1.y + (float)(g.cy - y) * scell, bz = ps1.z + (float)(g.cz - z) * scell;
        const unsigned pini = a.begincell[rowbase + (unsigned)g.xini], pfin = a.begincell[rowbase + (unsigned)g.xfin];
        for (unsigned p2 = pini + sl; p2 < pfin; p2 += G) {
          const float4 ps2 = a.pscell[p2];
          const int x = (int)gb_cx(dcc, a.dcell[p2]) - (int)cmin0;
          const float drx = (ps1.x + (float)(g.cx - x) * scell) - ps2.x, dry = by - ps2.y, drz = bz - ps2.z;
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
    if (c.dtallparticles && sl == 0) vel2 = vr1.x * vr1.x + vr1.y * vr1.y + vr1.z * vr1.z;
  }
#pragma unroll
  for (int o = G / 2; o; o >>= 1) {
    arp1 += __shfl_xor_sync(0xffffffffu, arp1, o);
    visc = fmaxf(visc, __shfl_xor_sync(0xffffffffu, visc, o));
  }
  if (p1 < npb && sl == 0) a.acear[p1] = make_float4(0.f, 0.f, 0.f, arp1);
  gb_warp_maxes(a.st, 0.f, visc, vel2);
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

// The ghost node of boundary row p1 (position + doubled normal, taken back
// into the domain across periodic faces: UpdatePeriodicPos,
// JSphCpu_mdbc.cpp:50, JSph.cpp:2079-2101): its cell relative to the trimmed
// domain (truncated toward zero as int() does, JCellSearch_inline.h:59-61;
// it may lie outside the domain) and its position relative to that cell.
struct Ghost {
  int cx, cy, cz;
  float lx, ly, lz;
};
__device__ __forceinline__ Ghost mdbc_ghost(const gbsph_consts& c, const DevArrays& a, const DivState& d,
                                            unsigned p1, float4 bn) {
  double gx = a.px[p1] + (double)bn.x, gy = a.py[p1] + (double)bn.y, gz = a.pz[p1] + (double)bn.z;
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
  const int gcx = (int)((gx - c.domposmin[0]) / sc), gcy = (int)((gy - c.domposmin[1]) / sc),
            gcz = (int)((gz - c.domposmin[2]) / sc);
  Ghost g;
  g.lx = (float)(gx - c.domposmin[0] - (double)gcx * sc);
  g.ly = (float)(gy - c.domposmin[1] - (double)gcy * sc);
  g.lz = (float)(gz - c.domposmin[2] - (double)gcz * sc);
  g.cx = gcx - (int)d.cellmin[0];
  g.cy = gcy - (int)d.cellmin[1];
  g.cz = gcz - (int)d.cellmin[2];
  return g;
}

// Compensated sums of two entries at once (TwoSum in packed arithmetic:
// a - b is fma(b, -1, a), rounded once as a subtraction is, so every entry
// gets the bits the scalar gb_kadd gives it).
__device__ __forceinline__ void gb_kadd2(float2& hi, float2& lo, float2 x) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 s = __fadd2_rn(hi, x);
  const float2 bp = __ffma2_rn(hi, m1, s);
  const float2 e = __fadd2_rn(__ffma2_rn(__ffma2_rn(bp, m1, s), m1, hi), __ffma2_rn(bp, m1, x));
  hi = s;
  lo = __fadd2_rn(lo, e);
}

// One fluid neighbour of a ghost node at dr = ghost - neighbour: kernel
// sums and the moment matrix (Wendland WabFac, FunSphKernel.h:235-246).
// Entries (0,1) and (2,3) of every matrix row, and of b, are summed as pairs.
struct MdbcAcc {
  float2 Ah[4][2], Al[4][2];  // the moment matrix A, compensated
  float2 bh[2], bl[2];        // b = (sum m W, sum m gradW), compensated
  unsigned nfound;
};
__device__ __forceinline__ void mdbc_pair(const gbsph_consts& c, float hinv, float drx, float dry, float drz,
                                          float rr2, float rhop2, MdbcAcc& m) {
  m.nfound++;
  const float rad = sqrtf(rr2);
  const float qq = rad * hinv;
  const float wqq1 = 1.f - 0.5f * qq;
  const float wqq2 = wqq1 * wqq1;
  const float fac = c.bwenh * wqq2 * wqq1;
  const float wqq = qq + qq + 1.f;
  const float wab = c.awen * wqq * wqq2 * wqq2;
  const float frx = fac * drx, fry = fac * dry, frz = fac * drz;
  const float massp2 = c.massfluid;
  const float volp2 = massp2 / rhop2;
  const float2 mm = make_float2(massp2, massp2);
  gb_kadd2(m.bh[0], m.bl[0], __fmul2_rn(mm, make_float2(wab, frx)));
  gb_kadd2(m.bh[1], m.bl[1], __fmul2_rn(mm, make_float2(fry, frz)));
  const float rowv[4] = {wab * volp2, frx * volp2, fry * volp2, frz * volp2};
  const float2 d01 = make_float2(1.f, drx), d23 = make_float2(dry, drz);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float2 v = make_float2(rowv[i], rowv[i]);
    gb_kadd2(m.Ah[i][0], m.Al[i][0], __fmul2_rn(v, d01));
    gb_kadd2(m.Ah[i][1], m.Al[i][1], __fmul2_rn(v, d23));
  }
}

// The corrected density of boundary row p1 from its sums, written to velrho.w
// and its pressure to pscell.w.
__device__ __forceinline__ void mdbc_final(const gbsph_consts& c, const DevArrays& a, unsigned p1, float4 bn,
                                           const MdbcAcc& m) {
  float rhofinal = FLT_MAX;
  if (m.nfound) {
    // [A | b] with A the moment matrix and b = (rho, grad rho)
    double M[4][5];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      M[i][0] = (double)m.Ah[i][0].x + (double)m.Al[i][0].x;
      M[i][1] = (double)m.Ah[i][0].y + (double)m.Al[i][0].y;
      M[i][2] = (double)m.Ah[i][1].x + (double)m.Al[i][1].x;
      M[i][3] = (double)m.Ah[i][1].y + (double)m.Al[i][1].y;
    }
    M[0][4] = (double)m.bh[0].x + (double)m.bl[0].x;
    M[1][4] = (double)m.bh[0].y + (double)m.bl[0].y;
    M[2][4] = (double)m.bh[1].x + (double)m.bl[1].x;
    M[3][4] = (double)m.bh[1].y + (double)m.bl[1].y;
    const double a00 = M[0][0], b0 = M[0][4];
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
      rhofinal = (float)(b0 / a00);
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

__device__ __forceinline__ void mdbc_zero(MdbcAcc& m) {
  const float2 z = make_float2(0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 4; i++) m.Ah[i][0] = m.Ah[i][1] = m.Al[i][0] = m.Al[i][1] = z;
  m.bh[0] = m.bh[1] = m.bl[0] = m.bl[1] = z;
  m.nfound = 0u;
}

// One thread per boundary row, walking the 27 (or 125) boxes around its ghost
// node in the reference's order.
__global__ void __launch_bounds__(128) k_mdbc(gbsph_consts c, DevArrays a) {
  const DivState& d = *a.div;
  const unsigned p1 = blockIdx.x * blockDim.x + threadIdx.x;
  if (p1 >= d.npbok) return;
  const float4 bn = a.boundnor[p1];
  if (bn.x == 0.f && bn.y == 0.f && bn.z == 0.f) return;
  const Ghost gh = mdbc_ghost(c, a, d, p1, bn);
  const CellGrid g = gb_grid(gh.cx, gh.cy, gh.cz, c.cellmode_div, d);
  const float scell = c.scell, ks2 = c.kernelsize2, hinv = 1.f / c.kernelh;
  MdbcAcc m;
  mdbc_zero(m);
  for (int z = g.zini; z < g.zfin; z++) {
    for (int y = g.yini; y < g.yfin; y++) {
      const unsigned rowbase = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
      const float by = gh.ly + (float)(g.cy - y) * scell, bz = gh.lz + (float)(g.cz - z) * scell;
      for (int x = g.xini; x < g.xfin; x++) {
        const unsigned box = rowbase + (unsigned)x;
        const unsigned pini = a.begincell[box], pfin = a.begincell[box + 1];
        const float bx = gh.lx + (float)(g.cx - x) * scell;
        for (unsigned p2 = pini; p2 < pfin; p2++) {
          const float4 ps2 = a.pscell[p2];
          const float drx = bx - ps2.x, dry = by - ps2.y, drz = bz - ps2.z;
          const float rr2 = drx * drx + dry * dry + drz * drz;
          if (rr2 <= ks2 && (a.code[p2] & GB_CODE_MASKTYPE) == GB_CODE_TYPE_FLUID)
            mdbc_pair(c, hinv, drx, dry, drz, rr2, a.velrho[p2].w, m);
        }
      }
    }
  }
  mdbc_final(c, a, p1, bn, m);
}

// ---- mDBC, cell-tiled staged kernel -----------------------------------------
// The fluid-row kernel's scheme with ghost nodes as targets: a warp takes 32
// consecutive boundary rows; the ghost nodes of one row of cells (y, z) are a
// group, whose candidates -- the fluid boxes' particles around it, one range
// per row of boxes -- are staged through a ring of kMdbcR chunks (the negated
// position in the group's frame and the density), filtered by the box of the
// group's ghosts widened by 2h and by the fluid type, checked four at a time
// with packed arithmetic, and consumed in rounds in which every ghost of the
// group with a pending hit adds one neighbour to its sums.  A ghost whose cell
// lies outside the domain sees the boxes inside it only, as the per-ghost walk
// does (gb_grid).  The summation order per ghost is the order of the staged
// chunks; the moment matrix is summed compensated, as in k_mdbc.
constexpr int kMdbcR = 8;
// per slot: -x, -y, -z in the group's frame (the checks), the position
// relative to the candidate's own cell, its cell offset from the group's
// reference cell (x as a float, an integer exactly; y and z, within +-sd,
// as two 8-bit fields), the density, the hit mask
constexpr int kMdbcArrays = 10;
constexpr size_t kMdbcWarpBytes = (size_t)kMdbcR * 32 * kMdbcArrays * 4;

__device__ __forceinline__ void mdbc_refill(const float* ring, unsigned& cur, unsigned& cc, unsigned cnext,
                                            int lane) {
  const unsigned* sm = (const unsigned*)(ring + 9 * kMdbcR * 32);
  while (cur == 0u && cc + 1u < cnext) {
    cc++;
    cur = sm[(cc & (kMdbcR - 1)) * 32 + lane];
  }
  if (cur == 0u) cc = cnext;
}

// dr = ghost - neighbour formed as the per-row walk forms it, from the
// ghost's and the neighbour's positions relative to their own cells and the
// difference of their cells (fox: the ghost's cell offset from the group's
// reference cell along x; along y and z it is 0 within a group), so that the
// ill-conditioned solves of ghosts near corners see the same sums.
__device__ __forceinline__ void mdbc_round(const gbsph_consts& c, float hinv, const float* ring, unsigned& cur,
                                           unsigned& cc, unsigned cnext, const Ghost& gh, int fox, int foy, int foz,
                                           MdbcAcc& m, int lane) {
  if (cur != 0u) {
    constexpr int S = kMdbcR * 32;
    const unsigned slot = ((cc & (kMdbcR - 1)) << 5) | (unsigned)(__ffs(cur) - 1);
    cur &= cur - 1u;
    const float* e = ring + slot;
    const int o = __float_as_int(e[7 * S]);
    const int dyj = (o << 24) >> 24, dzj = (o << 16) >> 24;
    const float scell = c.scell;
    const float drx = (gh.lx + ((float)fox - e[6 * S]) * scell) - e[3 * S];
    const float dry = (gh.ly + (float)(foy - dyj) * scell) - e[4 * S];
    const float drz = (gh.lz + (float)(foz - dzj) * scell) - e[5 * S];
    mdbc_pair(c, hinv, drx, dry, drz, drx * drx + dry * dry + drz * drz, e[8 * S], m);
    mdbc_refill(ring, cur, cc, cnext, lane);
  }
}

// tsplit: 2^lsplit consecutive warps (2 or 4) take the same 32 boundary rows,
// each every 2^lsplit-th chunk of the candidate stream, for cases whose
// boundary rows make too few warps to fill the device; the first adds the
// others' compensated sums (through their rings, after a named barrier per
// row group) and solves.  A separate instantiation, so that the one-warp
// kernel keeps its registers.  Both take four blocks a SM: the split kernel
// at 128 registers (a few spilled) ran C2 0.9 % faster than at three blocks
// and 159, and the one-warp kernel was slower at five blocks and 96.
template <bool tsplit>
__global__ void __launch_bounds__(128, 4) k_mdbc_t(gbsph_consts c, DevArrays a, unsigned lsplit) {
  extern __shared__ float4 mdbc_smem[];
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int S = kMdbcR * 32;
  const DivState& d = *a.div;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned p1 = tsplit ? blockIdx.x * (128u >> lsplit) + (((unsigned)warp >> lsplit) << 5) + (unsigned)lane
                             : blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned npbok = d.npbok;
  float4 bn = make_float4(0.f, 0.f, 0.f, 0.f);
  if (p1 < npbok) bn = a.boundnor[p1];
  const bool active = p1 < npbok && !(bn.x == 0.f && bn.y == 0.f && bn.z == 0.f);
  if (__all_sync(FULL, !active)) return;
  float* ring = (float*)((char*)mdbc_smem + (size_t)warp * kMdbcWarpBytes);
  unsigned* sm = (unsigned*)(ring + 9 * S);
  Ghost gh = {0, 0, 0, 0.f, 0.f, 0.f};
  if (active) gh = mdbc_ghost(c, a, d, p1, bn);
  const int cx = gh.cx, cy = gh.cy, cz = gh.cz;
  const float scell = c.scell, ks2 = c.kernelsize2, hinv = 1.f / c.kernelh;
  const int sd = c.cellmode_div;
  const int ncx = (int)d.ncx, ncy = (int)d.ncy, ncz = (int)d.ncz;
  const unsigned dcc = c.domcellcode, cmin0 = d.cellmin[0];
  MdbcAcc m;
  mdbc_zero(m);
  unsigned cnext = 0u, cc = 0u, cur = 0u;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  int fox = 0, foy = 0, foz = 0;
  // A group takes the remaining ghosts whose rows of cells (y, z) lie within
  // `reach` rows of the leader's: the ghosts of the wall layers of a warp
  // fall in neighbouring rows, and one stream over the union of their box
  // rows (at most (2 sd + 1 + 2 reach)^2 <= 25) keeps the warp's lanes in
  // one set of rounds.
  const int reach = sd == 1 ? 1 : 0;
  unsigned remaining = __ballot_sync(FULL, active);
  while (remaining) {
    const int leader = __ffs(remaining) - 1;
    const int rx = __shfl_sync(FULL, cx, leader), ry = __shfl_sync(FULL, cy, leader),
              rz = __shfl_sync(FULL, cz, leader);
    const bool ing = ((remaining >> lane) & 1u) && abs(cy - ry) <= reach && abs(cz - rz) <= reach;
    const unsigned grp = __ballot_sync(FULL, ing);
    remaining &= ~grp;
    const int xmin = __reduce_min_sync(FULL, ing ? cx : 0x7fffffff);
    const int xmax = __reduce_max_sync(FULL, ing ? cx : (int)0x80000000);
    const int gy0 = __reduce_min_sync(FULL, ing ? cy : 0x7fffffff), gy1 = __reduce_max_sync(FULL, ing ? cy : (int)0x80000000);
    const int gz0 = __reduce_min_sync(FULL, ing ? cz : 0x7fffffff), gz1 = __reduce_max_sync(FULL, ing ? cz : (int)0x80000000);
    const int x0 = max(xmin - sd, 0), x1 = min(xmax + sd, ncx - 1);
    const int y0 = max(gy0 - sd, 0), y1 = min(gy1 + sd, ncy - 1);
    const int z0 = max(gz0 - sd, 0), z1 = min(gz1 + sd, ncz - 1);
    if (x0 > x1 || y0 > y1 || z0 > z1) continue;  // the ghosts' boxes are all outside the domain
    const int nyr = y1 - y0 + 1, nrows = nyr * (z1 - z0 + 1);
    unsigned rb = 0u, rlen = 0u;
    int rdy = 0, rdz = 0;
    if (lane < nrows) {
      const int y = y0 + lane % nyr, z = z0 + lane / nyr;
      const unsigned rowbase = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
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
    const unsigned rbase = rb - (incl - rlen);
    if (ing) {
      fox = cx - rx;
      foy = cy - ry;
      foz = cz - rz;
      fx = gh.lx + (float)fox * scell;
      fy = gh.ly + (float)foy * scell;
      fz = gh.lz + (float)foz * scell;
    }
    const float2 fxx = make_float2(fx, fx), fyy = make_float2(fy, fy), fzz = make_float2(fz, fz);
    const unsigned gmask = ing ? FULL : 0u;
    const float blox = tile_fmin(ing, fx), bloy = tile_fmin(ing, fy), bloz = tile_fmin(ing, fz);
    const float bhix = tile_fmax(ing, fx), bhiy = tile_fmax(ing, fy), bhiz = tile_fmax(ing, fz);
    const float ks2m = ks2 * 1.0001f;
    unsigned fill = 0u;
    const unsigned nch = (total + 31u) >> 5, plen = nch * kTSeg;
    unsigned stride = max(1u, (unsigned)__float2uint_rn(0.6180339887f * (float)nch));
    for (;;) {
      unsigned u = stride, v = nch;
      while (v) { const unsigned t = u % v; u = v; v = t; }
      if (u == 1u) break;
      stride++;
    }
    const unsigned pbase = (unsigned)(lane / kTSeg) * plen + (unsigned)(lane % kTSeg);
    const unsigned send = min((unsigned)(lane / kTSeg + 1) * plen, total);
    unsigned ch = 0u, mine = nch;
    if constexpr (tsplit) {  // every 2^lsplit-th chunk of the order, from the warp's index in the group on
      const unsigned sub = (unsigned)warp & ((1u << lsplit) - 1u);
      for (unsigned j = 0; j < sub; j++) ch = (ch + stride >= nch) ? ch + stride - nch : ch + stride;
      for (unsigned j = 0; j < lsplit; j++) stride = (2u * stride >= nch) ? 2u * stride - nch : 2u * stride;
      mine = nch > sub ? (nch - sub + (1u << lsplit) - 1u) >> lsplit : 0u;
    }
    // checks the full chunk cnext and runs rounds while every ghost of the
    // group has a hit pending
    auto check = [&]() {
      const unsigned base = (cnext & (kMdbcR - 1)) << 5;
      unsigned hm = 0u;
#pragma unroll
      for (int q = 0; q < 32; q += 4) {
        const float4 xq = *(const float4*)(ring + base + q);
        const float4 yq = *(const float4*)(ring + S + base + q);
        const float4 zq = *(const float4*)(ring + 2 * S + base + q);
        hm |= tile_check4(fxx, fyy, fzz, xq, yq, zq, ks2, q);
      }
      hm &= gmask;
      sm[base + lane] = hm;
      if (cc == cnext) cur = hm;
      cnext++;
      if (cur == 0u) cc = cnext;
      while (__ballot_sync(FULL, ing && cur != 0u) == grp) mdbc_round(c, hinv, ring, cur, cc, cnext, gh, fox, foy, foz, m, lane);
    };
    for (unsigned i = 0; i < mine; i++, ch = (ch + stride >= nch) ? ch + stride - nch : ch + stride) {
      const unsigned s = pbase + ch * kTSeg;
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
      bool keep = false;
      float qx = 0.f, qy = 0.f, qz = 0.f, qrho = 1.f;
      float4 ps2 = make_float4(0.f, 0.f, 0.f, 0.f);
      int dxj = 0;
      if (has) {
        const unsigned j = jb + s;
        if ((a.code[j] & GB_CODE_MASKTYPE) == GB_CODE_TYPE_FLUID) {
          ps2 = a.pscell[j];
          qrho = a.velrho[j].w;
          dxj = (int)(gb_cx(dcc, a.dcell[j]) - cmin0) - rx;
          qx = ps2.x + (float)dxj * scell;
          qy = ps2.y + (float)dyj * scell;
          qz = ps2.z + (float)dzj * scell;
          const float ex = fmaxf(fmaxf(blox - qx, qx - bhix), 0.f);
          const float ey = fmaxf(fmaxf(bloy - qy, qy - bhiy), 0.f);
          const float ez = fmaxf(fmaxf(bloz - qz, qz - bhiz), 0.f);
          keep = ex * ex + ey * ey + ez * ez <= ks2m;
        }
      }
      const unsigned kb = __ballot_sync(FULL, keep);
      if (kb == 0u) continue;
      const unsigned nk = (unsigned)__popc(kb);
      const unsigned need = fill + nk > 32u ? cnext + 1u : cnext;
      while (__any_sync(FULL, cur != 0u && cc + (unsigned)kMdbcR <= need))
        mdbc_round(c, hinv, ring, cur, cc, cnext, gh, fox, foy, foz, m, lane);
      if (keep) {
        const unsigned pos = fill + (unsigned)__popc(kb & ((1u << lane) - 1u));
        const unsigned slot = (((pos < 32u ? cnext : cnext + 1u) & (kMdbcR - 1)) << 5) | (pos & 31u);
        ring[slot] = -qx;
        ring[S + slot] = -qy;
        ring[2 * S + slot] = -qz;
        ring[3 * S + slot] = ps2.x;
        ring[4 * S + slot] = ps2.y;
        ring[5 * S + slot] = ps2.z;
        ring[6 * S + slot] = (float)dxj;
        ring[7 * S + slot] = __int_as_float((dyj & 255) | ((dzj & 255) << 8));
        ring[8 * S + slot] = qrho;
      }
      fill += nk;
      if (fill >= 32u) {
        __syncwarp();
        check();
        fill -= 32u;
      }
    }
    if (fill) {
      const unsigned base = (cnext & (kMdbcR - 1)) << 5;
      if ((unsigned)lane >= fill) {
        ring[base + lane] = -kFarAway;
        ring[S + base + lane] = -kFarAway;
        ring[2 * S + base + lane] = -kFarAway;
      }
      __syncwarp();
      check();
      fill = 0u;
    }
  }
  while (__any_sync(FULL, cur != 0u)) mdbc_round(c, hinv, ring, cur, cc, cnext, gh, fox, foy, foz, m, lane);
  if constexpr (tsplit) {
    // partial sums through the warps' own rings (41 x 32 floats of the 80 x 32)
    const unsigned sub = (unsigned)warp & ((1u << lsplit) - 1u);
    const unsigned nthreads = 32u << lsplit, barid = 1u + ((unsigned)warp >> lsplit);
    __syncwarp();
    if (sub) {
      float* part = ring;
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
          const int f = 4 * (2 * i + j);
          part[(f + 0) * 32 + lane] = m.Ah[i][j].x; part[(f + 1) * 32 + lane] = m.Ah[i][j].y;
          part[(f + 2) * 32 + lane] = m.Al[i][j].x; part[(f + 3) * 32 + lane] = m.Al[i][j].y;
        }
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int f = 32 + 4 * j;
        part[(f + 0) * 32 + lane] = m.bh[j].x; part[(f + 1) * 32 + lane] = m.bh[j].y;
        part[(f + 2) * 32 + lane] = m.bl[j].x; part[(f + 3) * 32 + lane] = m.bl[j].y;
      }
      part[40 * 32 + lane] = __uint_as_float(m.nfound);
    }
    asm volatile("bar.sync %0, %1;" ::"r"(barid), "r"(nthreads) : "memory");
    if (sub) return;
    for (unsigned w = 1; w < (1u << lsplit); w++) {
      const float* part = (const float*)((const char*)mdbc_smem + (size_t)(warp + (int)w) * kMdbcWarpBytes);
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
          const int f = 4 * (2 * i + j);
          gb_kadd2(m.Ah[i][j], m.Al[i][j], make_float2(part[(f + 0) * 32 + lane], part[(f + 1) * 32 + lane]));
          m.Al[i][j] = __fadd2_rn(m.Al[i][j], make_float2(part[(f + 2) * 32 + lane], part[(f + 3) * 32 + lane]));
        }
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int f = 32 + 4 * j;
        gb_kadd2(m.bh[j], m.bl[j], make_float2(part[(f + 0) * 32 + lane], part[(f + 1) * 32 + lane]));
        m.bl[j] = __fadd2_rn(m.bl[j], make_float2(part[(f + 2) * 32 + lane], part[(f + 3) * 32 + lane]));
      }
      m.nfound += __float_as_uint(part[40 * 32 + lane]);
    }
  }
  if (active) mdbc_final(c, a, p1, bn, m);
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

cudaError_t launch_fluid_v(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, int split,
                           bool prepare, cudaStream_t s) {
  switch (c.tvisco) {
    case GBSPH_VISCO_ARTIFICIAL: return gbk::fluid_artificial(c, a, cap, variant, bsize, split, prepare, s);
    case GBSPH_VISCO_LAMINAR: return gbk::fluid_laminar(c, a, cap, variant, bsize, split, prepare, s);
    default: return gbk::fluid_laminarsps(c, a, cap, variant, bsize, split, prepare, s);
  }
}

}  // namespace

namespace gbk {

void forces(const gbsph_consts& c, const DevArrays& a, unsigned cap, int bsize, int variant, int split,
            int bound_lanes, cudaStream_t s, unsigned long long* nlaunch, cudaEvent_t ev_fluid_begin,
            cudaEvent_t ev_fluid_end, const StreamFork* fork) {
  cudaMemsetAsync(&a.st->acemax2, 0, 3 * sizeof(unsigned), s);
  // the bound rows (p < npb) and the fluid rows write disjoint rows of acear
  // and meet only in the atomic maxima, so the bound-row pass can run beside
  // the fluid-row pass and use the issue slots the latter leaves
  cudaStream_t sb = s;
  if (fork && fork->side) {
    cudaEventRecord(fork->fork, s);
    cudaStreamWaitEvent(fork->side, fork->fork, 0);
    sb = fork->side;
  }
  if (bound_lanes == 32) k_forces_bound_g<32><<<gb_div_up(cap, 4), 128, 0, sb>>>(c, a);
  else if (bound_lanes == 4) k_forces_bound_g<4><<<gb_div_up(cap, 32), 128, 0, sb>>>(c, a);
  else k_forces_bound<<<gb_div_up(cap, 128), 128, 0, sb>>>(c, a);
  if (sb != s) cudaEventRecord(fork->join, sb);
  // inside a stream capture the records must be external nodes so that every
  // replay of the graph records them; outside a capture they are plain records
  cudaStreamCaptureStatus cap_st = cudaStreamCaptureStatusNone;
  if (ev_fluid_begin || ev_fluid_end) cudaStreamIsCapturing(s, &cap_st);
  const unsigned ev_flags = cap_st == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
  if (ev_fluid_begin) cudaEventRecordWithFlags(ev_fluid_begin, s, ev_flags);
  launch_fluid_v(c, a, cap, variant, bsize, split, false, s);
  if (ev_fluid_end) cudaEventRecordWithFlags(ev_fluid_end, s, ev_flags);
  if (sb != s) cudaStreamWaitEvent(s, fork->join, 0);
  if (nlaunch) *nlaunch += 2;
}

int forces_split_effective(const gbsph_consts& c, int variant, int split) {
  if (variant != 2 || split < 2) return 1;
  const bool series = !(c.tdensity == GBSPH_DDT_DDT2 || c.tdensity == GBSPH_DDT_DDT2FULL) ||
                      fabsf(c.ddtgz) * c.kernelsize < 0.049f;
  return series ? (split >= 4 ? 4 : 2) : 1;
}

cudaError_t forces_init(const gbsph_consts& c) {
  DevArrays a{};
  const cudaError_t e = launch_fluid_v(c, a, 0, 2, 128, 1, true, nullptr);
  if (e != cudaSuccess) return e;
  const cudaError_t e2 =
      cudaFuncSetAttribute(k_mdbc_t<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(4 * kMdbcWarpBytes));
  if (e2 != cudaSuccess) return e2;
  return cudaFuncSetAttribute(k_mdbc_t<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(4 * kMdbcWarpBytes));
}

void sps_tau(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s, unsigned long long* nlaunch) {
  k_sps_tau<<<gb_div_up(cap, 256), 256, 0, s>>>(c, a);
  if (nlaunch) *nlaunch += 1;
}

void pips(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s) {
  cudaMemsetAsync(a.pips, 0, 4 * sizeof(unsigned long long), s);
  k_pips<<<gb_div_up(cap, 128), 128, 0, s>>>(c, a);
}

void mdbc(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int split, cudaStream_t s,
          unsigned long long* nlaunch) {
  static_assert(kMdbcArrays * kMdbcR >= 41, "a ring holds the partial sums of a split row group");
  if (variant == 1) k_mdbc<<<gb_div_up(cap, 128), 128, 0, s>>>(c, a);
  else if (split >= 2) {
    const unsigned ls = split >= 4 ? 2u : 1u;
    k_mdbc_t<true><<<gb_div_up(cap, 128u >> ls), 128, 4 * kMdbcWarpBytes, s>>>(c, a, ls);
  } else {
    k_mdbc_t<false><<<gb_div_up(cap, 128), 128, 4 * kMdbcWarpBytes, s>>>(c, a, 0u);
  }
  if (nlaunch) *nlaunch += 1;
}

}  // namespace gbk
