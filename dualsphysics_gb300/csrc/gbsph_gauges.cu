// gbsph_gauges.cu -- measurement gauges on the divided particle state:
// velocity (JGaugeVelocity), surface water level (JGaugeSwl) and maximum fluid
// height (JGaugeMaxZ), JDsGaugeItem.cpp:427-478, 728-790, 1023-1087.
//
// The reference walks the neighbour cells of a point with one thread (its GPU
// kernels run a single thread per gauge, JDsGauge_ker.cu:50-110, 252-292);
// here one warp takes one measurement point: the lanes split each row of
// cells' particle range, keep double partial sums (the reference accumulates
// in double) and combine them with shuffles.  The cell walk, the kernel and
// the per-particle float arithmetic are the reference's; only the order of the
// double additions differs, below the final rounding to float.
#include <cfloat>
#include <climits>

#include "gbsph_common.cuh"

namespace {

constexpr int kGaugeWarps = 8;       // warps per block (one point each)
constexpr int kSwlChunk = 64;        // SWL sample points per block pass

// Neighbour-cell ranges of a point, nsearch::Init(pos,...) (JCellSearch_inline.h:43-57):
// the cell of the point relative to the divided domain, widened by ScellDiv
// cells and clipped to it.  `ok` is false for an empty range.
struct GaugeCells {
  int xini, xfin, yini, yfin, zini, zfin;
  bool ok;
};

__device__ __forceinline__ int gauge_cell(double p, double posmin, float scell, unsigned cellzero, bool& valid) {
  const double q = (p - posmin) / (double)scell;
  // points far outside the map would overflow int(); their range is empty anyway
  if (!(q > -1.0e9 && q < 1.0e9)) {
    valid = false;
    return 0;
  }
  return (int)q - (int)cellzero;
}

__device__ __forceinline__ GaugeCells gauge_cells(const gbsph_consts& c, const DivState& d, double px, double py,
                                                  double pz) {
  GaugeCells g;
  bool valid = true;
  const int cx = gauge_cell(px, c.domposmin[0], c.scell, d.cellmin[0], valid);
  const int cy = gauge_cell(py, c.domposmin[1], c.scell, d.cellmin[1], valid);
  const int cz = gauge_cell(pz, c.domposmin[2], c.scell, d.cellmin[2], valid);
  const int sd = c.cellmode_div;
  const int ncx = (int)d.ncx, ncy = (int)d.ncy, ncz = (int)d.ncz;
  g.xini = cx - (cx < sd ? cx : sd);
  g.xfin = cx + (ncx - cx - 1 < sd ? ncx - cx - 1 : sd) + 1;
  g.yini = cy - (cy < sd ? cy : sd);
  g.yfin = cy + (ncy - cy - 1 < sd ? ncy - cy - 1 : sd) + 1;
  g.zini = cz - (cz < sd ? cz : sd);
  g.zfin = cz + (ncz - cz - 1 < sd ? ncz - cz - 1 : sd) + 1;
  g.ok = valid && g.xini < g.xfin && g.yini < g.yfin && g.zini < g.zfin;
  return g;
}

// GetKernelWendland_Wab (FunSphKernel.h:213-220), rounded step by step as the
// reference's float expression.
__device__ __forceinline__ float gauge_wab(float rr2, float h, float awen) {
  const float rad = __fsqrt_rn(rr2);
  const float qq = __fdiv_rn(rad, h);
  const float wqq = __fadd_rn(__fadd_rn(qq, qq), 1.0f);
  const float wqq1 = __fsub_rn(1.0f, __fmul_rn(0.5f, qq));
  const float wqq2 = __fmul_rn(wqq1, wqq1);
  return __fmul_rn(__fmul_rn(__fmul_rn(awen, wqq), wqq2), wqq2);
}

// nsearch::Distance2 (JCellSearch_inline.h:99-104): float of the double differences.
__device__ __forceinline__ float gauge_rr2(double px, double py, double pz, const DevArrays& a, unsigned p) {
  const float drx = (float)(px - a.px[p]), dry = (float)(py - a.py[p]), drz = (float)(pz - a.pz[p]);
  return __fadd_rn(__fadd_rn(__fmul_rn(drx, drx), __fmul_rn(dry, dry)), __fmul_rn(drz, drz));
}

__device__ __forceinline__ bool gauge_fluid(uint16_t code) {
  return (code & GB_CODE_MASKTYPE) == GB_CODE_TYPE_FLUID;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the fluid particles within the kernel of point p of W*m/rho times
// (vx, vy, vz, m): the velocity gauge's and the SWL mass's sums
// (JGaugeVelocity::CalculeCpuT, JGaugeSwl::CalculeMassCpu).  Lane partials.
template <bool tvel>
__device__ __forceinline__ void gauge_sums(const gbsph_consts& c, const DivState& d, const DevArrays& a, double px,
                                           double py, double pz, double (&s)[3]) {
  const int lane = threadIdx.x & 31;
  s[0] = s[1] = s[2] = 0.0;
  const GaugeCells g = gauge_cells(c, d, px, py, pz);
  if (!g.ok) return;
  const float ks2 = c.kernelsize2, h = c.kernelh, awen = c.awen, massf = c.massfluid;
  for (int z = g.zini; z < g.zfin; z++) {
    for (int y = g.yini; y < g.yfin; y++) {
      const unsigned row = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
      const unsigned pini = a.begincell[row + (unsigned)g.xini], pfin = a.begincell[row + (unsigned)g.xfin];
      for (unsigned p = pini + lane; p < pfin; p += 32) {
        const float rr2 = gauge_rr2(px, py, pz, a, p);
        if (rr2 <= ks2 && rr2 >= GB_ALMOSTZERO && gauge_fluid(a.code[p])) {
          const float4 vr = a.velrho[p];
          const float wab = __fmul_rn(gauge_wab(rr2, h, awen), __fdiv_rn(massf, vr.w));
          if (tvel) {
            s[0] += (double)__fmul_rn(wab, vr.x);
            s[1] += (double)__fmul_rn(wab, vr.y);
            s[2] += (double)__fmul_rn(wab, vr.z);
          } else {
            s[0] += (double)__fmul_rn(wab, massf);
          }
        }
      }
    }
  }
}

// JGaugeItem::PointIsOut (JDsGaugeItem.h:223-227) against the map limits the
// gauge system is configured with.
__device__ __forceinline__ bool gauge_point_out(const gbsph_consts& c, double px, double py, double pz) {
  return px != px || py != py || pz != pz || px < c.maprealposmin[0] || py < c.maprealposmin[1] ||
         pz < c.maprealposmin[2] || px >= c.maprealposmax[0] || py >= c.maprealposmax[1] || pz >= c.maprealposmax[2];
}

// One warp per point: velocity = sum of W*m/rho*v (no kernel normalisation;
// zero for a point outside the domain).
__global__ void k_gauge_vel(gbsph_consts c, DevArrays a, unsigned n, const double* __restrict__ pts,
                            float* __restrict__ vel) {
  const unsigned w = blockIdx.x * kGaugeWarps + (threadIdx.x >> 5);
  if (w >= n) return;
  const DivState& d = *a.div;
  const double px = pts[3 * w], py = pts[3 * w + 1], pz = pts[3 * w + 2];
  double s[3] = {0.0, 0.0, 0.0};
  if (!gauge_point_out(c, px, py, pz)) gauge_sums<true>(c, d, a, px, py, pz, s);
  s[0] = warp_sum(s[0]);
  s[1] = warp_sum(s[1]);
  s[2] = warp_sum(s[2]);
  if ((threadIdx.x & 31) == 0) {
    vel[3 * w] = (float)s[0];
    vel[3 * w + 1] = (float)s[1];
    vel[3 * w + 2] = (float)s[2];
  }
}

// SWL: one block per gauge.  The sample points are p0 + k*dir accumulated one
// addition at a time as the reference does; each pass computes the mass of
// kSwlChunk points (one warp per point) and thread 0 scans them in order for
// the first crossing of the mass limit (JGaugeSwl::CalculeCpuT).
// par: per gauge p0 (3), dir (3) as doubles; np: PointNp; ml: mass limit.
__global__ void __launch_bounds__(kGaugeWarps * 32) k_gauge_swl(gbsph_consts c, DevArrays a, unsigned n,
                                                                  const double* __restrict__ par,
                                                                  const unsigned* __restrict__ npts,
                                                                  const float* __restrict__ mlim,
                                                                  float* __restrict__ surf) {
  __shared__ double spt[kSwlChunk][3];
  __shared__ float smass[kSwlChunk];
  __shared__ double srun[3];
  __shared__ int sdone;
  const unsigned gi = blockIdx.x;
  if (gi >= n) return;
  const DivState& d = *a.div;
  const double p0x = par[6 * gi], p0y = par[6 * gi + 1], p0z = par[6 * gi + 2];
  const double dx = par[6 * gi + 3], dy = par[6 * gi + 4], dz = par[6 * gi + 5];
  const unsigned np = npts[gi];
  const float ml = mlim[gi];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float mpre = 0.0f;  // used by thread 0 only
  double sx = 0.0, sy = 0.0, sz = 0.0;
  if (threadIdx.x == 0) {
    srun[0] = p0x;
    srun[1] = p0y;
    srun[2] = p0z;
    sdone = 0;
  }
  __syncthreads();
  // points cp = 0..np, kSwlChunk at a time
  for (unsigned long long base = 0; base <= (unsigned long long)np; base += kSwlChunk) {
    const unsigned cnt = (unsigned)min((unsigned long long)kSwlChunk, (unsigned long long)np + 1ull - base);
    if (threadIdx.x == 0) {
      double x = srun[0], y = srun[1], z = srun[2];
      for (unsigned k = 0; k < cnt; k++) {
        spt[k][0] = x;
        spt[k][1] = y;
        spt[k][2] = z;
        x += dx;
        y += dy;
        z += dz;
      }
      srun[0] = x;
      srun[1] = y;
      srun[2] = z;
    }
    __syncthreads();
    for (unsigned k = warp; k < cnt; k += kGaugeWarps) {
      double s[3];
      gauge_sums<false>(c, d, a, spt[k][0], spt[k][1], spt[k][2], s);
      const double m = warp_sum(s[0]);
      if (lane == 0) smass[k] = (float)m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (unsigned k = 0; k < cnt; k++) {
        const float mass = smass[k];
        if (mass > ml) mpre = mass;
        if (mass < ml && mpre != 0.0f) {
          const float fxm1 = __fsub_rn(__fdiv_rn(__fsub_rn(ml, mpre), __fsub_rn(mass, mpre)), 1.0f);
          sx = __dadd_rn(spt[k][0], __dmul_rn(dx, (double)fxm1));
          sy = __dadd_rn(spt[k][1], __dmul_rn(dy, (double)fxm1));
          sz = __dadd_rn(spt[k][2], __dmul_rn(dz, (double)fxm1));
          sdone = 1;
          break;
        }
      }
    }
    __syncthreads();
    if (sdone) break;
  }
  if (threadIdx.x == 0) {
    if (!sdone) {
      const double f = (double)(mpre != 0.0f ? np : 0u);
      sx = __dadd_rn(p0x, __dmul_rn(dx, f));
      sy = __dadd_rn(p0y, __dmul_rn(dy, f));
      sz = __dadd_rn(p0z, __dmul_rn(dz, f));
    }
    surf[3 * gi] = (float)sx;
    surf[3 * gi + 1] = (float)sy;
    surf[3 * gi + 2] = (float)sz;
  }
}

// MaxZ: one warp per gauge.  The cell box of the vertical segment widened by
// the distance limit (GetInteractionCellsMaxZ, JDsGaugeItem.cpp:1023-1040) is
// scanned from its top cell layer down; the first layer holding a fluid
// particle within the distance of the line gives the result, floored at the
// domain's lower z (JGaugeMaxZ::CalculeCpu).
// par: per gauge x, y, z, height (doubles); dist: distance limit.
__global__ void k_gauge_maxz(gbsph_consts c, DevArrays a, unsigned n, const double* __restrict__ par,
                             const float* __restrict__ dist, float* __restrict__ zmax_out) {
  const unsigned w = blockIdx.x * kGaugeWarps + (threadIdx.x >> 5);
  if (w >= n) return;
  const int lane = threadIdx.x & 31;
  const DivState& d = *a.div;
  const double p0x = par[4 * w], p0y = par[4 * w + 1], p0z = par[4 * w + 2], hgt = par[4 * w + 3];
  const float dl = dist[w];
  const float maxdist2 = __fmul_rn(dl, dl);
  bool valid = true;
  const int cx = gauge_cell(p0x, c.domposmin[0], c.scell, d.cellmin[0], valid);
  const int cy = gauge_cell(p0y, c.domposmin[1], c.scell, d.cellmin[1], valid);
  const int cz = gauge_cell(p0z, c.domposmin[2], c.scell, d.cellmin[2], valid);
  const int cz2 = gauge_cell(p0z + hgt, c.domposmin[2], c.scell, d.cellmin[2], valid);
  const float ncf = ceilf(__fdiv_rn(dl, c.scell));
  const int ncel = (ncf >= 0.0f && ncf < 1.0e6f) ? (int)ncf : 1000000;
  const int xini = max(cx - ncel, 0), xfin = min(cx + ncel + 1, (int)d.ncx);
  const int yini = max(cy - ncel, 0), yfin = min(cy + ncel + 1, (int)d.ncy);
  const int zini = max(cz - ncel, 0), zfin = min(cz2 + ncel + 1, (int)d.ncz);
  float zmax = -FLT_MAX;
  bool found = false;
  if (valid && xini < xfin) {
    for (int z = zfin - 1; z >= zini && !found; z--) {
      float zl = -FLT_MAX;
      bool fl = false;
      for (int y = yini; y < yfin; y++) {
        const unsigned row = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
        const unsigned pini = a.begincell[row + (unsigned)xini], pfin = a.begincell[row + (unsigned)xfin];
        for (unsigned p = pini + lane; p < pfin; p += 32) {
          const double pz2 = a.pz[p];
          if (pz2 > (double)zl) {
            const float drx = (float)(p0x - a.px[p]), dry = (float)(p0y - a.py[p]);
            const float rr2 = __fadd_rn(__fmul_rn(drx, drx), __fmul_rn(dry, dry));
            if (rr2 <= maxdist2 && gauge_fluid(a.code[p])) {
              zl = (float)pz2;
              fl = true;
            }
          }
        }
      }
      found = __any_sync(0xffffffffu, fl);
      if (found) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) zl = fmaxf(zl, __shfl_xor_sync(0xffffffffu, zl, o));
        zmax = zl;
      }
    }
  }
  if (lane == 0) zmax_out[w] = fmaxf(zmax, (float)c.maprealposmin[2]);
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Mesh gauge: one warp per grid point.  Kernel sums W*m/rho of (1, m, rho,
// vx, vy, vz) over the fluid particles within the kernel (no minimum
// distance), in float as the reference, then the kernel correction: divided
// by sum W*m/rho when that reaches kclimit, else kcdummy (FLT_MAX disables
// either) (JGaugeMesh::CalculeCpuT, JDsGaugeItem.cpp:1513-1571).  The point is
// ptref + vdp1*cp1 + vdp2*cp2 + vdp3*cp3, summed in that order.
__global__ void k_gauge_mesh(gbsph_consts c, DevArrays a, GaugeMeshPts m, float kclimit, float kcdummy,
                             float* __restrict__ vel, float* __restrict__ vdir, float* __restrict__ rhop,
                             float* __restrict__ mass) {
  const unsigned cp = blockIdx.x * kGaugeWarps + (threadIdx.x >> 5);
  if (cp >= m.npt) return;
  const int lane = threadIdx.x & 31;
  const DivState& d = *a.div;
  const unsigned npt12 = m.npt1 * m.npt2;
  const unsigned cp3 = cp / npt12, cp3r = cp - cp3 * npt12;
  const unsigned cp2 = cp3r / m.npt1, cp1 = cp3r - cp2 * m.npt1;
  double pt[3];
#pragma unroll
  for (int k = 0; k < 3; k++)
    pt[k] = __dadd_rn(__dadd_rn(__dadd_rn(m.ptref[k], __dmul_rn(m.vdp1[k], (double)cp1)),
                                __dmul_rn(m.vdp2[k], (double)cp2)),
                      __dmul_rn(m.vdp3[k], (double)cp3));
  float sw = 0.f, sm = 0.f, sr = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
  const GaugeCells g = gauge_cells(c, d, pt[0], pt[1], pt[2]);
  if (g.ok) {
    const float ks2 = c.kernelsize2, h = c.kernelh, awen = c.awen, massf = c.massfluid;
    for (int z = g.zini; z < g.zfin; z++) {
      for (int y = g.yini; y < g.yfin; y++) {
        const unsigned row = d.boxfluid + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
        const unsigned pini = a.begincell[row + (unsigned)g.xini], pfin = a.begincell[row + (unsigned)g.xfin];
        for (unsigned p = pini + lane; p < pfin; p += 32) {
          const float rr2 = gauge_rr2(pt[0], pt[1], pt[2], a, p);
          if (rr2 <= ks2 && gauge_fluid(a.code[p])) {
            const float4 vr = a.velrho[p];
            const float wab = __fmul_rn(gauge_wab(rr2, h, awen), __fdiv_rn(massf, vr.w));
            sw = __fadd_rn(sw, wab);
            sm = __fadd_rn(sm, __fmul_rn(wab, massf));
            sr = __fadd_rn(sr, __fmul_rn(wab, vr.w));
            sx = __fadd_rn(sx, __fmul_rn(wab, vr.x));
            sy = __fadd_rn(sy, __fmul_rn(wab, vr.y));
            sz = __fadd_rn(sz, __fmul_rn(wab, vr.z));
          }
        }
      }
    }
  }
  sw = warp_sumf(sw);
  sm = warp_sumf(sm);
  sr = warp_sumf(sr);
  sx = warp_sumf(sx);
  sy = warp_sumf(sy);
  sz = warp_sumf(sz);
  if (lane) return;
  if (kclimit != FLT_MAX) {
    if (sw >= kclimit) {
      sx = __fdiv_rn(sx, sw);
      sy = __fdiv_rn(sy, sw);
      sz = __fdiv_rn(sz, sw);
      sr = __fdiv_rn(sr, sw);
    } else if (kcdummy != FLT_MAX) {
      sx = sy = sz = sr = kcdummy;
    }
  }
  if (vel) {
    vel[3 * cp] = sx;
    vel[3 * cp + 1] = sy;
    vel[3 * cp + 2] = sz;
  }
  if (vdir)
    vdir[cp] = __fadd_rn(__fadd_rn(__fmul_rn(sx, m.dirdat[0]), __fmul_rn(sy, m.dirdat[1])), __fmul_rn(sz, m.dirdat[2]));
  if (rhop) rhop[cp] = sr;
  mass[cp] = sm;
}

// Surface z of each column of the mesh along its third axis: the first
// point where the mass drops below the limit, interpolated from the last
// point above it (JDsGaugeItem.cpp:1573-1596).  One thread per column.
__global__ void k_gauge_mesh_zsurf(GaugeMeshPts m, float masslimit, const float* __restrict__ mass,
                                   float* __restrict__ zsurf) {
  const unsigned col = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned npt12 = m.npt1 * m.npt2;
  if (col >= npt12) return;
  const unsigned cp2 = col / m.npt1, cp1 = col - cp2 * m.npt1;
  float masspre = 0.f, fsurf = 0.f;
  unsigned cpsurf = 0, cp = col;
  for (unsigned cp3 = 0; cp3 < m.npt3 && !cpsurf; cp3++) {
    const float ms = mass[cp];
    if (ms > masslimit) masspre = ms;
    if (ms < masslimit && masspre != 0.f) {
      fsurf = __fdiv_rn(__fsub_rn(masslimit, masspre), __fsub_rn(ms, masspre));
      cpsurf = cp3;
    }
    cp += npt12;
  }
  float z = (float)__dadd_rn(__dadd_rn(m.ptref[2], __dmul_rn(m.vdp1[2], (double)cp1)), __dmul_rn(m.vdp2[2], (double)cp2));
  if (cpsurf == 0 && masspre != 0.f) z = __fadd_rn(z, (float)__dmul_rn(m.vdp3[2], (double)(m.npt3 - 1)));
  if (cpsurf)
    z = __fadd_rn(z, (float)__dadd_rn(__dmul_rn(m.vdp3[2], (double)(cpsurf - 1)), __dmul_rn(m.vdp3[2], (double)fsurf)));
  zsurf[col] = z;
}

// Order-preserving map of a double onto unsigned 64-bit keys (for atomicMax).
__device__ __forceinline__ unsigned long long gauge_dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Surge front: the largest pos.dir over the fluid particles inside the box
// [bmin, bmax] (a flow front's position along dir, e.g. the dam-break tip for
// dir = +x), and how many fluid particles the box holds.  Grid-stride over the
// np particles of the divided state; warp max, then one atomic per warp.
__global__ void k_fluid_front(DevArrays a, double3 dir, double3 bmin, double3 bmax,
                              unsigned long long* __restrict__ key, unsigned* __restrict__ count) {
  const unsigned np = a.div->np;
  unsigned long long best = 0ull;
  unsigned cnt = 0;
  for (unsigned p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const double x = a.px[p], y = a.py[p], z = a.pz[p];
    if (gauge_fluid(a.code[p]) && x >= bmin.x && y >= bmin.y && z >= bmin.z && x <= bmax.x && y <= bmax.y &&
        z <= bmax.z) {
      const double v = __dadd_rn(__dadd_rn(__dmul_rn(x, dir.x), __dmul_rn(y, dir.y)), __dmul_rn(z, dir.z));
      const unsigned long long k = gauge_dkey(v);
      best = k > best ? k : best;
      cnt++;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
    best = ob > best ? ob : best;
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0 && cnt) {
    atomicMax(key, best);
    atomicAdd(count, cnt);
  }
}

}  // namespace

namespace gbk {

void fluid_front(const DevArrays& a, const double* dir, const double* bmin, const double* bmax,
                 unsigned long long* key, unsigned* count, int nsm, cudaStream_t s) {
  k_fluid_front<<<nsm * 4, 256, 0, s>>>(a, make_double3(dir[0], dir[1], dir[2]), make_double3(bmin[0], bmin[1], bmin[2]),
                                        make_double3(bmax[0], bmax[1], bmax[2]), key, count);
}

void gauge_mesh(const gbsph_consts& c, const DevArrays& a, const GaugeMeshPts& m, float kclimit, float kcdummy,
                float masslimit, float* vel, float* vdir, float* rhop, float* mass, float* zsurf, cudaStream_t s) {
  if (!m.npt) return;
  k_gauge_mesh<<<gb_div_up(m.npt, kGaugeWarps), kGaugeWarps * 32, 0, s>>>(c, a, m, kclimit, kcdummy, vel, vdir,
                                                                         rhop, mass);
  if (zsurf) k_gauge_mesh_zsurf<<<gb_div_up(m.npt1 * m.npt2, 128), 128, 0, s>>>(m, masslimit, mass, zsurf);
}

void gauge_velocity(const gbsph_consts& c, const DevArrays& a, unsigned n, const double* pts, float* vel,
                    cudaStream_t s) {
  if (!n) return;
  k_gauge_vel<<<gb_div_up(n, kGaugeWarps), kGaugeWarps * 32, 0, s>>>(c, a, n, pts, vel);
}

void gauge_swl(const gbsph_consts& c, const DevArrays& a, unsigned n, const double* par, const unsigned* npts,
               const float* mlim, float* surf, cudaStream_t s) {
  if (!n) return;
  k_gauge_swl<<<n, kGaugeWarps * 32, 0, s>>>(c, a, n, par, npts, mlim, surf);
}

void gauge_maxz(const gbsph_consts& c, const DevArrays& a, unsigned n, const double* par, const float* dist,
                float* zmax, cudaStream_t s) {
  if (!n) return;
  k_gauge_maxz<<<gb_div_up(n, kGaugeWarps), kGaugeWarps * 32, 0, s>>>(c, a, n, par, dist, zmax);
}

}  // namespace gbk
