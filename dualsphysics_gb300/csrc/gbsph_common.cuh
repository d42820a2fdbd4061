// gbsph_common.cuh -- shared definitions of the GB300 WCSPH step kernels.
//
// Device-resident state of one context and the small device helpers (cell
// codification, particle codes, Wendland kernel) used by the divide, forces
// and update kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbsph.h"

// Particle code bits: 16-bit typecode, DualSphDef.h:150-200.
#define GB_CODE_MASKSPECIAL 0xe000u
#define GB_CODE_NORMAL 0x0000u
#define GB_CODE_OUTIGNORE 0x4000u
#define GB_CODE_OUTMOV 0x6000u
#define GB_CODE_OUTPOS 0x8000u
#define GB_CODE_OUTRHO 0xA000u
#define GB_CODE_MASKTYPE 0x1800u
#define GB_CODE_TYPE_FLOATING 0x1000u
#define GB_CODE_TYPE_FLUID 0x1800u

#define GB_ALMOSTZERO 1e-18f  // DualSphDef.h:114

// error bits written by kernels into DivState::error / StepState::error
#define GB_ERR_BOUNDOUT 1u
#define GB_ERR_CELLCAP 2u
#define GB_ERR_NANDT 4u
#define GB_ERR_PARTOUT 8u   // a particle of the initial state lies outside the domain

// Device-resident cell-division state (JCellDivGpuSingle members).
struct DivState {
  unsigned np, npb, npbok;            // counts after the last divide
  unsigned nptot, npb1;               // inputs of the current divide
  unsigned cellmin[3], cellmax[3];
  unsigned ncx, ncy, ncz, nsheet, nct, nctt;
  unsigned boxboundignore, boxfluid, boxboundout, boxfluidout, boxboundoutignore, boxfluidoutignore;
  unsigned dividefull, ini;           // sorted segment is [ini, nptot)
  unsigned boundlimitok, bounddivideok;
  unsigned blmin[3], blmax[3];        // cached boundary cell limits
  unsigned bdmin[3], bdmax[3];        // cell domain of the last full divide
  unsigned fmin[3], fmax[3];          // reduction targets (fluid)
  unsigned bmin[3], bmax[3];          // reduction targets (boundary)
  unsigned npbignore, npbout, npfout, npboutignore, npfoutignore, npfinal, npbfinal;
  unsigned nout_total;
  unsigned boundchanged;
  unsigned error;
  unsigned nctt_cap;
};

// Device-resident step scalars (JSph members Symplectic*, Dt*, AceMax ...).
struct StepState {
  double dt_p, dt_c, dtpre, dt_last, time, dt_var;
  unsigned nstep, verletstep;
  unsigned acemax2, velmax2, viscdt;  // bit patterns of non-negative floats (atomicMax)
  unsigned error;
};

// Device arrays of one context.  Sorted arrays come in pairs (cur/alt) and are
// swapped after each reorder.
struct DevArrays {
  double *px, *py, *pz, *px2, *py2, *pz2;       // positions (SoA, f64)
  double *qx, *qy, *qz, *qx2, *qy2, *qz2;       // positions at the start of the step (Symplectic pre)
  float4 *velrho, *velrho2;                      // (vx,vy,vz,rho)
  float4 *velrhopre, *velrhopre2;                // Symplectic pre / Verlet m1
  unsigned *idp, *idp2, *dcell, *dcell2;
  uint16_t *code, *code2;
  float4 *boundnor, *boundnor2;                  // mDBC normal (already doubled), w unused
  float4 *taua, *taua2;                          // SPS tau/rho^2 xx,xy,xz,yy
  float2 *taub, *taub2;                          // SPS tau/rho^2 yz,zz
  float4 *straina;                               // SPS 2*strain xx,xy,xz,yy
  float2 *strainb;                               // SPS 2*strain yz,zz
  float4 *pscell;                                // (x,y,z) relative to the particle's cell origin, w=pressure
  float4 *acear;                                 // (ace.x,ace.y,ace.z,ar)
  unsigned *keys, *keys2, *vals, *vals2;         // radix sort buffers
  unsigned *hist;                                // radix sort tile histograms
  unsigned *begincell;                           // BeginCell (nctt entries, JCellDivCpu.h:150)
  DivState* div;
  StepState* st;
  unsigned long long* pips;                      // 4 counters of the particle-interaction count
};

// --- cell codification (JDsDcellDef.h:27-43) ---------------------------------
__device__ __forceinline__ unsigned gb_cx(unsigned dcc, unsigned cel) { return cel >> ((dcc >> 10) & 31); }
__device__ __forceinline__ unsigned gb_cy(unsigned dcc, unsigned cel) { return (cel << (dcc >> 25)) >> ((dcc >> 5) & 31); }
__device__ __forceinline__ unsigned gb_cz(unsigned dcc, unsigned cel) { return (cel << (dcc & 31)) >> (dcc & 31); }
__device__ __forceinline__ unsigned gb_cell(unsigned dcc, unsigned cx, unsigned cy, unsigned cz) {
  return (cx << ((dcc >> 10) & 31)) | (cy << ((dcc >> 15) & 31)) | cz;
}

// float max via the bit pattern of a non-negative float
__device__ __forceinline__ void gb_atomic_max_nonneg(unsigned* addr, float v) {
  atomicMax(addr, __float_as_uint(v));
}

// Pressure from density: Tait/Monaghan EOS B*((rho/rho0)^gamma-1)
// (FunSphEos.h:37-39).  (rho/rho0)^gamma is evaluated in double and rounded
// once to float so it matches a correctly rounded powf.
__device__ __forceinline__ float gb_press(float rho, float rhopzero, float cteb, float gamma) {
  const float x = rho / rhopzero;
  double xg;
  if (gamma == 7.0f) {
    const double xd = (double)x;
    const double x2 = __dmul_rn(xd, xd);
    const double x3 = __dmul_rn(x2, xd);
    const double x4 = __dmul_rn(x2, x2);
    xg = __dmul_rn(x4, x3);
  } else {
    xg = pow((double)x, (double)gamma);
  }
  return cteb * ((float)xg - 1.0f);
}

__host__ __device__ __forceinline__ unsigned gb_div_up(unsigned a, unsigned b) { return (a + b - 1) / b; }

// Launchers implemented in the .cu files (host side).
namespace gbk {
void load_dcell(const gbsph_consts& c, const DevArrays& a, unsigned n, cudaStream_t s);  // sets GB_ERR_PARTOUT in DivState::error
void divide(const gbsph_consts& c, DevArrays& a, unsigned cap, unsigned npasses, cudaStream_t s, unsigned long long* nlaunch);
// Stable sort of n <= sort_noalloc_max_keys() keys of nbits bits on the static
// work area (work = its device address, from sort_noalloc_address on the
// current device).
unsigned sort_noalloc_max_keys();
cudaError_t sort_noalloc_address(void** p);
void sort_noalloc(unsigned char* work, const unsigned* keys, unsigned n, unsigned nbits, unsigned* perm,
                  unsigned* sorted_keys, cudaStream_t s);
void forces(const gbsph_consts& c, const DevArrays& a, unsigned cap, int bsize, int variant, cudaStream_t s, unsigned long long* nlaunch,
            cudaEvent_t ev_fluid_begin = nullptr, cudaEvent_t ev_fluid_end = nullptr);
void mdbc(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s, unsigned long long* nlaunch);
void dtvariable(const gbsph_consts& c, const DevArrays& a, int which, cudaStream_t s, unsigned long long* nlaunch);
void symplectic_pre(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, cudaStream_t s, unsigned long long* nlaunch);
void symplectic_cor(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, cudaStream_t s, unsigned long long* nlaunch);
void verlet_step(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, int euler, cudaStream_t s, unsigned long long* nlaunch);
void sps_tau(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s, unsigned long long* nlaunch);
void pips(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s);
void step_end(const DevArrays& a, int symplectic, cudaStream_t s, unsigned long long* nlaunch);
}  // namespace gbk
