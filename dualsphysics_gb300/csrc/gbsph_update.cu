// gbsph_update.cu -- time integration, position update and adaptive dt.
//
// Symplectic predictor/corrector (JSphCpu.cpp:1687-2029; GPU twin
// KerComputeStepSymplecticPre/Cor, JSphGpuSimple_ker.cu:265-516, plus
// KerComputeStepPos2, JSphGpu_ker.cu:1523-1580), Verlet (JSphCpu.cpp:1523-1680),
// UpdatePos with the out-of-domain / MovLimit / rho-out exclusions
// (JSphCpu.cpp:1464-1516) and DtVariable (JSphCpu.cpp:2035-2078).
//
// The integrators evaluate their double-precision expressions with explicit
// round-to-nearest intrinsics (no FMA contraction), so given the same ace/ar
// they reproduce the reference CPU results bit for bit.  Each integrator is one
// fused kernel: density, velocity, displacement, new position and new cell.
#include <cuda_runtime.h>
#include <float.h>

#include "gbsph_common.cuh"

namespace {

constexpr int kUpdBlock = 256;

__device__ __forceinline__ double dadd(double x, double y) { return __dadd_rn(x, y); }
__device__ __forceinline__ double dmul(double x, double y) { return __dmul_rn(x, y); }

// UpdatePos (JSphCpu.cpp:1464-1516).  With periodic conditions a particle
// that left the real domain across a periodic face comes back by the axis
// increment, and cells are taken from DomPosMin.
__device__ __forceinline__ void update_pos(const gbsph_consts& c, const DevArrays& a, unsigned p, double rx, double ry,
                                           double rz, double movx, double movy, double movz, bool outrho,
                                           double rsc) {
  const bool outmov = (fabsf(gb_d2f(movx)) > c.movlimit || fabsf(gb_d2f(movy)) > c.movlimit ||
                       fabsf(gb_d2f(movz)) > c.movlimit);
  rx = dadd(rx, movx); ry = dadd(ry, movy); rz = dadd(rz, movz);
  double dx = __dsub_rn(rx, c.maprealposmin[0]);
  double dy = __dsub_rn(ry, c.maprealposmin[1]);
  double dz = __dsub_rn(rz, c.maprealposmin[2]);
  bool out = gb_outside(dx, c.maprealsize[0]) || gb_outside(dy, c.maprealsize[1]) ||
             gb_outside(dz, c.maprealsize[2]);
  const bool periactive = c.peri[0] || c.peri[1] || c.peri[2];
  if (periactive && out) {
    for (int k = 0; k < 3; k++) {
      if (!c.peri[k]) continue;
      const double* inc = c.periinc + 3 * k;
      const double dk = k == 0 ? dx : (k == 1 ? dy : dz);
      if (dk < 0) { dx = __dsub_rn(dx, inc[0]); dy = __dsub_rn(dy, inc[1]); dz = __dsub_rn(dz, inc[2]); }
      const double dk2 = k == 0 ? dx : (k == 1 ? dy : dz);
      if (dk2 >= c.maprealsize[k]) { dx = dadd(dx, inc[0]); dy = dadd(dy, inc[1]); dz = dadd(dz, inc[2]); }
    }
    const bool outx = !c.peri[0] && (dx < 0 || dx >= c.maprealsize[0]);
    const bool outy = !c.peri[1] && (dy < 0 || dy >= c.maprealsize[1]);
    const bool outz = !c.peri[2] && (dz < 0 || dz >= c.maprealsize[2]);
    out = outx || outy || outz;
    rx = dadd(dx, c.maprealposmin[0]); ry = dadd(dy, c.maprealposmin[1]); rz = dadd(dz, c.maprealposmin[2]);
  }
  a.px[p] = rx; a.py[p] = ry; a.pz[p] = rz;
  if (outrho || outmov || out) {
    const unsigned rcode = a.code[p];
    const unsigned base = rcode & ~GB_CODE_MASKSPECIAL;
    a.code[p] = (uint16_t)(base | (out ? GB_CODE_OUTPOS : (outrho ? GB_CODE_OUTRHO : GB_CODE_OUTMOV)));
    a.dcell[p] = 0xffffffffu;
  } else {
    if (periactive) {
      dx = __dsub_rn(rx, c.domposmin[0]); dy = __dsub_rn(ry, c.domposmin[1]); dz = __dsub_rn(rz, c.domposmin[2]);
    }
    const double sc = (double)c.scell;
    const unsigned cx = gb_cellidx(dx, sc, rsc), cy = gb_cellidx(dy, sc, rsc), cz = gb_cellidx(dz, sc, rsc);
    a.dcell[p] = gb_cell(c.domcellcode, cx, cy, cz);
  }
}

__device__ __forceinline__ double read_dt(const double* dtp, double dth) { return dtp ? *dtp : dth; }

// ComputeSymplecticPre: the current state becomes the PRE state (qx/velrhopre)
// and the predicted state is written to the current arrays.
__global__ void k_sym_pre(gbsph_consts c, DevArrays a, const double* dtp, double dth, double rsc) {
  const DivState& d = *a.div;
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.np) return;
  const double dt05 = dmul(read_dt(dtp, dth), 0.5);
  const double x = a.px[p], y = a.py[p], z = a.pz[p];
  const float4 vp = a.velrho[p];
  a.qx[p] = x; a.qy[p] = y; a.qz[p] = z;
  a.velrhopre[p] = vp;
  const float ar = a.acear[p].w;
  if (p < d.npb) {
    float w = gb_d2f(dadd(gb_f2d(vp.w), dmul(dt05, gb_f2d(ar))));
    w = (w < c.rhopzero ? c.rhopzero : w);
    a.velrho[p] = make_float4(vp.x, vp.y, vp.z, w);
    return;
  }
  const float4 ace = a.acear[p];
  const unsigned rcode = a.code[p];
  const float rhonew = gb_d2f(dadd(gb_f2d(vp.w), dmul(dt05, gb_f2d(ar))));
  const double dx = dmul(gb_f2d(vp.x), dt05), dy = dmul(gb_f2d(vp.y), dt05), dz = dmul(gb_f2d(vp.z), dt05);
  const bool outrho = (rhonew < c.rhopoutmin || rhonew > c.rhopoutmax);
  const float vx = gb_d2f(dadd(gb_f2d(vp.x), dmul(dadd(gb_f2d(ace.x), gb_f2d(c.gravity[0])), dt05)));
  const float vy = gb_d2f(dadd(gb_f2d(vp.y), dmul(dadd(gb_f2d(ace.y), gb_f2d(c.gravity[1])), dt05)));
  const float vz = gb_d2f(dadd(gb_f2d(vp.z), dmul(dadd(gb_f2d(ace.z), gb_f2d(c.gravity[2])), dt05)));
  a.velrho[p] = make_float4(vx, vy, vz, rhonew);
  unsigned code = rcode;
  if (outrho && (rcode & GB_CODE_MASKSPECIAL) == GB_CODE_NORMAL) {
    code = (rcode & ~GB_CODE_MASKSPECIAL) | GB_CODE_OUTRHO;
    a.code[p] = (uint16_t)code;
  }
  // periodic copies are not moved (JSphCpu.cpp:1816): the next divide replaces them
  if ((code & GB_CODE_MASKTYPE) == GB_CODE_TYPE_FLUID && (code & GB_CODE_MASKSPECIAL) != GB_CODE_PERIODIC)
    update_pos(c, a, p, x, y, z, dx, dy, dz, (code & GB_CODE_MASKSPECIAL) == GB_CODE_OUTRHO, rsc);
}

// ComputeSymplecticCorr: PRE state + forces of the predicted state.
__global__ void k_sym_cor(gbsph_consts c, DevArrays a, const double* dtp, double dth, double rsc) {
  const DivState& d = *a.div;
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.np) return;
  const double dt = read_dt(dtp, dth);
  const double dt05 = dmul(dt, 0.5);
  const float4 ace = a.acear[p];
  const float4 vc = a.velrho[p];   // predicted
  const float4 vp = a.velrhopre[p];
  const double eps = dmul(-gb_f2d(ace.w) / gb_f2d(vc.w), dt);
  const float rhonew = gb_d2f((dmul(gb_f2d(vp.w), __dsub_rn(2., eps)) / dadd(2., eps)));
  if (p < d.npb) {
    a.velrho[p] = make_float4(0.f, 0.f, 0.f, (rhonew < c.rhopzero ? c.rhopzero : rhonew));
    return;
  }
  const unsigned rcode = a.code[p];
  const float vx = gb_d2f(dadd(gb_f2d(vp.x), dmul(dadd(gb_f2d(ace.x), gb_f2d(c.gravity[0])), dt)));
  const float vy = gb_d2f(dadd(gb_f2d(vp.y), dmul(dadd(gb_f2d(ace.y), gb_f2d(c.gravity[1])), dt)));
  const float vz = gb_d2f(dadd(gb_f2d(vp.z), dmul(dadd(gb_f2d(ace.z), gb_f2d(c.gravity[2])), dt)));
  double dx = dmul(dadd(gb_f2d(vp.x), gb_f2d(vx)), dt05);
  double dy = dmul(dadd(gb_f2d(vp.y), gb_f2d(vy)), dt05);
  double dz = dmul(dadd(gb_f2d(vp.z), gb_f2d(vz)), dt05);
  if (c.tshift) {  // the shifting displacement (JSphCpu.cpp:1940-1944)
    const float4 sh = a.shiftpos[p];
    dx = dadd(dx, gb_f2d(sh.x)); dy = dadd(dy, gb_f2d(sh.y)); dz = dadd(dz, gb_f2d(sh.z));
  }
  const bool outrho = (rhonew < c.rhopoutmin || rhonew > c.rhopoutmax);
  unsigned code = rcode;
  if (outrho && (rcode & GB_CODE_MASKSPECIAL) == GB_CODE_NORMAL) {
    code = (rcode & ~GB_CODE_MASKSPECIAL) | GB_CODE_OUTRHO;
    a.code[p] = (uint16_t)code;
  }
  a.velrho[p] = make_float4(vx, vy, vz, rhonew);
  if ((code & GB_CODE_MASKSPECIAL) == GB_CODE_PERIODIC) return;  // JSphCpu.cpp:2000
  if ((code & GB_CODE_MASKTYPE) == GB_CODE_TYPE_FLUID)
    update_pos(c, a, p, a.qx[p], a.qy[p], a.qz[p], dx, dy, dz, (code & GB_CODE_MASKSPECIAL) == GB_CODE_OUTRHO, rsc);
  else {
    a.px[p] = a.qx[p]; a.py[p] = a.qy[p]; a.pz[p] = a.qz[p];
  }
}

// ComputeVerlet (JSphCpu.cpp:1523-1680): velrhopre holds VelrhoM1.  The new
// state is written to velrho and the old velrho moves to velrhopre.
__global__ void k_verlet(gbsph_consts c, DevArrays a, const double* dtp, double dth, int euler, double rsc) {
  const DivState& d = *a.div;
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.np) return;
  const double dt = read_dt(dtp, dth);
  const double dt2 = euler ? dt : dadd(dt, dt);
  const float4 v1 = a.velrho[p];
  const float4 vm1 = a.velrhopre[p];
  const float4 v2 = euler ? v1 : vm1;
  const float ar = a.acear[p].w;
  const float rhonew = gb_d2f(dadd(gb_f2d(v2.w), dmul(dt2, gb_f2d(ar))));
  a.velrhopre[p] = v1;
  if (p < d.npb) {
    a.velrho[p] = make_float4(0.f, 0.f, 0.f, (rhonew < c.rhopzero ? c.rhopzero : rhonew));
    return;
  }
  const double dt205 = dmul(dmul(0.5, dt), dt);
  const float4 ace = a.acear[p];
  const double ax = dadd(gb_f2d(ace.x), gb_f2d(c.gravity[0]));
  const double ay = dadd(gb_f2d(ace.y), gb_f2d(c.gravity[1]));
  const double az = dadd(gb_f2d(ace.z), gb_f2d(c.gravity[2]));
  double dx = dadd(dmul(gb_f2d(v1.x), dt), dmul(ax, dt205));
  double dy = dadd(dmul(gb_f2d(v1.y), dt), dmul(ay, dt205));
  double dz = dadd(dmul(gb_f2d(v1.z), dt), dmul(az, dt205));
  if (c.tshift) {  // the shifting displacement (JSphCpu.cpp:1543-1547)
    const float4 sh = a.shiftpos[p];
    dx = dadd(dx, gb_f2d(sh.x)); dy = dadd(dy, gb_f2d(sh.y)); dz = dadd(dz, gb_f2d(sh.z));
  }
  const bool outrho = (rhonew < c.rhopoutmin || rhonew > c.rhopoutmax);
  const float nvx = gb_d2f(dadd(gb_f2d(v2.x), dmul(ax, dt2)));
  const float nvy = gb_d2f(dadd(gb_f2d(v2.y), dmul(ay, dt2)));
  const float nvz = gb_d2f(dadd(gb_f2d(v2.z), dmul(az, dt2)));
  a.velrho[p] = make_float4(nvx, nvy, nvz, rhonew);
  update_pos(c, a, p, a.px[p], a.py[p], a.pz[p], dx, dy, dz, outrho, rsc);
}

// DtVariable (JSphCpu.cpp:2035-2078): which = 0 predictor (dt_p), 1 corrector
// (dt_c), 2 Verlet (dt_var).
__global__ void k_dtvar(gbsph_consts c, StepState* st, int which) {
  const float acemax2 = __uint_as_float(st->acemax2);
  const double acemax = sqrt((double)acemax2);
  const float velmax = sqrtf(__uint_as_float(st->velmax2));
  const float viscdt = __uint_as_float(st->viscdt);
  const double h = (double)c.kernelh;
  const double dt1 = (acemax ? sqrt(h / acemax) : DBL_MAX);
  const double vm = (double)velmax * 10.;
  // std::max(Cs0, vm) and std::min(dt1, dt2) as the reference writes them: the
  // same values for numbers, and a NaN dt1 (from a NaN AceMax) is kept
  const double dt2 = h / ((c.cs0 < vm ? vm : c.cs0) + h * (double)viscdt);
  double dt = c.cflnumber * (dt2 < dt1 ? dt2 : dt1);
  if (isnan(dt) || isinf(dt)) {
    st->error |= GB_ERR_NANDT;
    dt = c.dtmin;
  }
  if (dt < c.dtmin) dt = c.dtmin;
  st->dt_var = dt;
  if (which == 0) st->dt_p = dt;
  else if (which == 1) st->dt_c = dt;
}

// End of a step: TimeStep+=dt, SymplecticDtPre=min(dt_p,dt_c) (JSphCpuSingle.cpp:930-935, 1184-1190).
__global__ void k_step_end(StepState* st, int symplectic) {
  if (symplectic) {
    st->dt_last = st->dtpre;
    st->time += st->dtpre;
    st->dtpre = (st->dt_p < st->dt_c ? st->dt_p : st->dt_c);
  } else {
    st->dt_last = st->dt_var;
    st->time += st->dt_var;
  }
  st->nstep++;
}

// Interleaved positions -> px/py/pz, and the doubled boundary normals
// (JSph::ConfigBoundNormals, JSph.cpp:1411-1418: boundary particles by id).
__global__ void k_stage_upload(DevArrays a, const double* __restrict__ stage, const float* __restrict__ nor3,
                               unsigned n, unsigned npb) {
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  a.px[p] = stage[3 * (size_t)p];
  a.py[p] = stage[3 * (size_t)p + 1];
  a.pz[p] = stage[3 * (size_t)p + 2];
  if (a.boundnor) {
    float4 bn = make_float4(0.f, 0.f, 0.f, 0.f);
    if (nor3 && a.idp[p] < npb)
      bn = make_float4(nor3[3 * (size_t)p] * 2.f, nor3[3 * (size_t)p + 1] * 2.f, nor3[3 * (size_t)p + 2] * 2.f, 0.f);
    a.boundnor[p] = bn;
  }
}

__global__ void k_stage_download(DevArrays a, double* __restrict__ stage, unsigned n) {
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  stage[3 * (size_t)p] = a.px[p];
  stage[3 * (size_t)p + 1] = a.py[p];
  stage[3 * (size_t)p + 2] = a.pz[p];
}

// JSphShifting::RunCpu (JSphShifting.cpp:390-418): the shifting sums of each
// fluid row become its displacement, dt*coef*h*|v| along the sums, cut below
// the free-surface threshold and limited to dp/10; rows cancelled next to the
// boundary get none.  dt = dtfactor * *dtp (the step's dt, or half of it).
__global__ void k_run_shifting(gbsph_consts c, DevArrays a, const double* __restrict__ dtp, double dtfactor) {
  const DivState& d = *a.div;
  const unsigned p = d.npb + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.np) return;
  const float4 rs = a.shiftpos[p];
  if (rs.x == FLT_MAX) {
    a.shiftpos[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const double dt = dmul(*dtp, dtfactor);
  const double coefumagn = dmul(dmul(dt, gb_f2d(c.shiftcoef)), gb_f2d(c.kernelh));
  const double coeftfs = __dsub_rn(c.simulate2d ? 2.0 : 3.0, gb_f2d(c.shifttfs));
  const float maxdist = gb_d2f(dmul(c.dp, 0.1));
  const float4 v = a.velrho[p];
  const double vx = gb_f2d(v.x), vy = gb_f2d(v.y), vz = gb_f2d(v.z);
  double umagn = dmul(coefumagn, __dsqrt_rn(dadd(dadd(dmul(vx, vx), dmul(vy, vy)), dmul(vz, vz))));
  if (c.shifttfs != 0.f) {
    if (rs.w < c.shifttfs) umagn = 0;
    else umagn = dmul(umagn, __ddiv_rn(__dsub_rn(gb_f2d(rs.w), gb_f2d(c.shifttfs)), coeftfs));
  }
  const float sx = gb_d2f(dmul(gb_f2d(rs.x), umagn));
  const float sy = gb_d2f(dmul(gb_f2d(rs.y), umagn));
  const float sz = gb_d2f(dmul(gb_f2d(rs.z), umagn));
  a.shiftpos[p] = make_float4(fabsf(sx) < maxdist ? sx : (sx >= 0 ? maxdist : -maxdist),
                              fabsf(sy) < maxdist ? sy : (sy >= 0 ? maxdist : -maxdist),
                              fabsf(sz) < maxdist ? sz : (sz >= 0 ? maxdist : -maxdist), rs.w);
}

// CalcRidp (JSphCpu.cpp:2099-2127) over the npb boundary particles: the
// current index of each moving particle by id (ridp preset to UINT_MAX);
// periodic copies share their source's id and are left out.
// Thread 0 also marks the boundary changed when some object is active
// (JSphCpu::RunMotion sets BoundChanged, JSphCpu.cpp:2196).
__global__ void k_motion_ridp(DevArrays a, const MotionStep* __restrict__ hdr, unsigned idmin, unsigned nmoving,
                              unsigned* __restrict__ ridp) {
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0 && hdr->active) a.div->boundchanged = 1;
  if (p >= a.div->npb) return;
  const unsigned rel = a.idp[p] - idmin;
  if (rel < nmoving && (a.code[p] & GB_CODE_MASKSPECIAL) == GB_CODE_NORMAL) ridp[rel] = p;
}

// MatrixMulPoint: rows 1..3 of a 4x4 matrix times (x, y, z, 1).
__device__ __forceinline__ double mat_row(const double* m, double x, double y, double z) {
  return dadd(dadd(dadd(dmul(x, m[0]), dmul(y, m[1])), dmul(z, m[2])), m[3]);
}

// MoveLinBound / MoveMatBound (JSphCpu.cpp:2133-2173): one thread per moving
// particle; the position goes through UpdatePos (cell, out flags), the
// velocity becomes the object's (linear) or displacement/dt (matrix), and a
// matrix movement also turns the mDBC normal.
__global__ void k_motion_move(gbsph_consts c, DevArrays a, const MotionStep* __restrict__ hdr,
                              const MotionObjDev* __restrict__ objs, unsigned nobj, const unsigned* __restrict__ ridp,
                              unsigned idmin, unsigned nmoving, double rsc) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nmoving) return;
  const unsigned id = idmin + i;
  unsigned k = 0;
  while (k < nobj && !(id >= objs[k].idbegin && id - objs[k].idbegin < objs[k].count)) k++;
  if (k == nobj || objs[k].type == 0) return;
  const unsigned p = ridp[i];
  if (p == 0xffffffffu) return;
  const MotionObjDev& o = objs[k];
  const double x = a.px[p], y = a.py[p], z = a.pz[p];
  const float4 v = a.velrho[p];
  if (o.type == 1) {
    update_pos(c, a, p, x, y, z, o.linmov[0], o.linmov[1], o.linmov[2], false, rsc);
    a.velrho[p] = make_float4(o.linvel[0], o.linvel[1], o.linvel[2], v.w);
    return;
  }
  const double* m = o.mat;
  const double x2 = mat_row(m, x, y, z), z2 = mat_row(m + 8, x, y, z);
  const double y2 = c.simulate2d ? y : mat_row(m + 4, x, y, z);
  const double dx = __dsub_rn(x2, x), dy = __dsub_rn(y2, y), dz = __dsub_rn(z2, z);
  update_pos(c, a, p, x, y, z, dx, dy, dz, false, rsc);
  const double dt = hdr->dt;
  a.velrho[p] = make_float4(gb_d2f(__ddiv_rn(dx, dt)), gb_d2f(__ddiv_rn(dy, dt)), gb_d2f(__ddiv_rn(dz, dt)), v.w);
  if (a.boundnor) {
    const float4 bn = a.boundnor[p];
    const double gx = dadd(x, gb_f2d(bn.x)), gy = dadd(y, gb_f2d(bn.y)), gz = dadd(z, gb_f2d(bn.z));
    a.boundnor[p] = make_float4(gb_d2f(__dsub_rn(mat_row(m, gx, gy, gz), x2)),
                                gb_d2f(__dsub_rn(mat_row(m + 4, gx, gy, gz), y2)),
                                gb_d2f(__dsub_rn(mat_row(m + 8, gx, gy, gz), z2)), bn.w);
  }
}

}  // namespace

namespace gbk {

void run_shifting(const gbsph_consts& c, const DevArrays& a, unsigned cap, const double* dtp, double dtfactor,
                  cudaStream_t s, unsigned long long* nlaunch) {
  k_run_shifting<<<gb_div_up(cap, kUpdBlock), kUpdBlock, 0, s>>>(c, a, dtp, dtfactor);
  if (nlaunch) *nlaunch += 1;
}

void motion_move(const gbsph_consts& c, const DevArrays& a, const MotionStep* hdr, const MotionObjDev* objs,
                 unsigned nobj, unsigned* ridp, unsigned idmin, unsigned nmoving, unsigned cap, cudaStream_t s,
                 unsigned long long* nlaunch) {
  cudaMemsetAsync(ridp, 0xff, sizeof(unsigned) * nmoving, s);
  k_motion_ridp<<<gb_div_up(cap, kUpdBlock), kUpdBlock, 0, s>>>(a, hdr, idmin, nmoving, ridp);
  k_motion_move<<<gb_div_up(nmoving, kUpdBlock), kUpdBlock, 0, s>>>(c, a, hdr, objs, nobj, ridp, idmin, nmoving,
                                                                    1.0 / (double)c.scell);
  if (nlaunch) *nlaunch += 2;
}

void stage_upload(const DevArrays& a, const double* stage, const float* nor3, unsigned n, unsigned npb, cudaStream_t s) {
  if (n) k_stage_upload<<<gb_div_up(n, kUpdBlock), kUpdBlock, 0, s>>>(a, stage, nor3, n, npb);
}

void stage_download(const DevArrays& a, double* stage, unsigned n, cudaStream_t s) {
  if (n) k_stage_download<<<gb_div_up(n, kUpdBlock), kUpdBlock, 0, s>>>(a, stage, n);
}


void symplectic_pre(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, cudaStream_t s,
                    unsigned long long* nlaunch) {
  k_sym_pre<<<gb_div_up(cap, kUpdBlock), kUpdBlock, 0, s>>>(c, a, dtp, 0.0, 1.0 / (double)c.scell);
  if (nlaunch) *nlaunch += 1;
}

void symplectic_cor(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, cudaStream_t s,
                    unsigned long long* nlaunch) {
  k_sym_cor<<<gb_div_up(cap, kUpdBlock), kUpdBlock, 0, s>>>(c, a, dtp, 0.0, 1.0 / (double)c.scell);
  if (nlaunch) *nlaunch += 1;
}

void dtvariable(const gbsph_consts& c, const DevArrays& a, int which, cudaStream_t s, unsigned long long* nlaunch) {
  k_dtvar<<<1, 1, 0, s>>>(c, a.st, which);
  if (nlaunch) *nlaunch += 1;
}

void step_end(const DevArrays& a, int symplectic, cudaStream_t s, unsigned long long* nlaunch) {
  k_step_end<<<1, 1, 0, s>>>(a.st, symplectic);
  if (nlaunch) *nlaunch += 1;
}

void verlet_step(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, int euler, cudaStream_t s,
                 unsigned long long* nlaunch) {
  k_verlet<<<gb_div_up(cap, kUpdBlock), kUpdBlock, 0, s>>>(c, a, dtp, 0.0, euler, 1.0 / (double)c.scell);
  if (nlaunch) *nlaunch += 1;
}

}  // namespace gbk
