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
#define GB_ERR_PERICAP 16u  // the periodic copies do not fit the capacity
#define GB_CODE_PERIODIC 0x2000u

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
  // periodic conditions (RunPeriodic): copies of boundary (npb2) and fluid
  // (npf2) particles appended after the npb1+npf1 particles, the counts the
  // copying started from, and the group being copied (source range, first
  // new index, number of copies)
  unsigned npb2, npf2, peri_npb0, peri_npf0, peri_pini, peri_num, peri_base, peri_count;
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
  float4 *shiftpos;                              // shifting sums, then displacements (fluid rows; tshift)
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

// float max via the bit pattern of a non-negative float; a NaN (positive or
// negative) has a larger bit pattern than every finite float and stays
__device__ __forceinline__ void gb_atomic_max_nonneg(unsigned* addr, float v) {
  atomicMax(addr, __float_as_uint(v));
}

// max of the dt maxima that keeps a NaN (fmaxf drops it): a NaN in a fluid
// row's sums reaches the dt, which then reports GB_ERR_NANDT
__device__ __forceinline__ float gb_fmax_nan(float a, float b) { return (a != a || a > b) ? a : b; }

// Warp maxima of the dt quantities (NaN kept), one atomic per warp; values
// that are not above zero are not written (the maxima start at zero).
__device__ __forceinline__ void gb_warp_maxes(StepState* st, float acemax2, float visc, float vel2) {
  for (int o = 16; o; o >>= 1) {
    acemax2 = gb_fmax_nan(acemax2, __shfl_xor_sync(0xffffffffu, acemax2, o));
    visc = gb_fmax_nan(visc, __shfl_xor_sync(0xffffffffu, visc, o));
    vel2 = gb_fmax_nan(vel2, __shfl_xor_sync(0xffffffffu, vel2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (!(acemax2 <= 0.f)) gb_atomic_max_nonneg(&st->acemax2, acemax2);
    if (!(visc <= 0.f)) gb_atomic_max_nonneg(&st->viscdt, visc);
    if (!(vel2 <= 0.f)) gb_atomic_max_nonneg(&st->velmax2, vel2);
  }
}

__device__ __forceinline__ double gb_f2d(float f);
__device__ __forceinline__ float gb_d2f(double x);

// Pressure from density: Tait/Monaghan EOS B*((rho/rho0)^gamma-1)
// (FunSphEos.h:37-39).  (rho/rho0)^gamma is evaluated in double and rounded
// once to float so it matches a correctly rounded powf.
__device__ __forceinline__ float gb_press(float rho, float rhopzero, float cteb, float gamma) {
  const float x = rho / rhopzero;
  double xg;
  if (gamma == 7.0f) {
    const double xd = gb_f2d(x);
    const double x2 = __dmul_rn(xd, xd);
    const double x3 = __dmul_rn(x2, xd);
    const double x4 = __dmul_rn(x2, x2);
    xg = __dmul_rn(x4, x3);
  } else {
    xg = pow((double)x, (double)gamma);
  }
  return cteb * (gb_d2f(xg) - 1.0f);
}

__host__ __device__ __forceinline__ unsigned gb_div_up(unsigned a, unsigned b) { return (a + b - 1) / b; }

// ---- exact FP64 helpers on the integer pipe ----------------------------------
// This part executes FP64 instructions (conversions and compares included) at
// a small fraction of its FP32 / integer rate, so the integrators do the exact
// operations that need no rounding decisions -- float->double conversion,
// double->float rounding, sign/order tests -- on the bit patterns, and keep the
// FP64 pipe for the additions, products and divisions.

// (double)f, exactly: a normal float's exponent is re-biased and its
// significand widened; zeros, subnormals, infinities and NaNs take the
// hardware conversion.
__device__ __forceinline__ double gb_f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned mag = u & 0x7fffffffu;
  if (mag == 0u) return __longlong_as_double((long long)((unsigned long long)(u >> 31) << 63));
  if (mag - 0x00800000u >= 0x7f000000u) return (double)f;
  const unsigned long long b = ((unsigned long long)(u >> 31) << 63) |
                               ((unsigned long long)((mag >> 23) + 896u) << 52) |
                               ((unsigned long long)(mag & 0x7fffffu) << 29);
  return __longlong_as_double((long long)b);
}

// (float)x with round-to-nearest-even, for results that are normal floats
// (the 29 dropped significand bits decide the rounding; a carry into the
// exponent is the correct result, up to infinity); zeros, subnormal results,
// overflow, infinities and NaNs take the hardware conversion.
__device__ __forceinline__ float gb_d2f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - 897u > 253u) return (float)x;
  const unsigned long long m = b & 0xfffffffffffffull;
  unsigned r = (unsigned)(m >> 29) | ((e - 896u) << 23);
  const unsigned rem = (unsigned)(m & 0x1fffffffu);
  if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) r += 1u;
  return __uint_as_float(r | ((unsigned)(b >> 63) << 31));
}

// (double)u, exactly, for u below 2^31 (cell indices): the bits of 2^52 + u
// less 2^52 would take an FP64 subtraction, so the exponent and significand
// are placed directly.
__device__ __forceinline__ double gb_u2d(unsigned u) {
  if (u == 0u) return 0.0;
  const int lz = __clz(u);                 // u = 1.f * 2^(31 - lz)
  const unsigned long long m = (unsigned long long)u << (lz + 21);  // the leading 1 at bit 52
  const unsigned long long b = ((unsigned long long)(1023 + 31 - lz) << 52) | (m & 0xfffffffffffffull);
  return __longlong_as_double((long long)b);
}

// x < 0 || x >= size || x is NaN, for a finite size > 0 (-0 is not below 0).
__device__ __forceinline__ bool gb_outside(double x, double size) {
  const long long b = __double_as_longlong(x);
  const unsigned long long mag = (unsigned long long)b & 0x7fffffffffffffffull;
  if (mag > 0x7ff0000000000000ull) return true;
  if (b < 0) return mag != 0ull;
  return b >= __double_as_longlong(size);
}

// Cell index unsigned(d / sc) for 0 <= d, bit for bit as the correctly rounded
// double division gives it, with the division done only when needed: q =
// d * rsc (rsc = RN(1/sc)) is within 4 ulp of d / sc, below 1.5e-9 for every
// quotient under 2^22, so when the fraction of q lies more than 2^-26 from an
// integer (and q < 2^22), floor(q) is floor(RN(d / sc)); q < 0.5 gives 0.  The
// integer and fraction parts are read from q's bits.
__device__ __forceinline__ unsigned gb_cellidx(double d, double sc, double rsc) {
  const double q = __dmul_rn(d, rsc);
  const unsigned long long b = (unsigned long long)__double_as_longlong(q);
  const int ef = (int)(b >> 52);  // q >= 0: no sign bit
  if (ef < 1022) return 0u;
  if (ef < 1023 + 22) {
    const int sh = 1075 - ef;  // fraction bits of q, 31..53
    const unsigned long long m = (b & 0xfffffffffffffull) | 0x10000000000000ull;
    const unsigned long long ip = m >> sh, fr = m & ((1ull << sh) - 1ull), lim = 1ull << (sh - 26);
    if ((ip == 0ull || fr > lim) && fr < (1ull << sh) - lim) return (unsigned)ip;
  }
  return (unsigned)__ddiv_rn(d, sc);
}

// A mesh gauge's grid (jmsh::StMeshPts, JMeshDataDef.h:87-96): npt1 x npt2 x
// npt3 points ptref + vdp1*i + vdp2*j + vdp3*k, and the direction of the
// projected velocity.
struct GaugeMeshPts {
  double ptref[3], vdp1[3], vdp2[3], vdp3[3];
  unsigned npt1, npt2, npt3, npt;
  float dirdat[3];
};

// Motion of the moving objects over one step, written by the host before the
// step and read by the move kernels (JDsMotion's StMotionData,
// JDsMotionDef.h:33-44).
struct MotionObjDev {
  int type;               // 0 none, 1 linear, 2 matrix
  unsigned idbegin, count;
  double linmov[3];
  float linvel[3];
  double mat[12];         // rows 1..3 of the 4x4 matrix, row-major
};
struct MotionStep {
  int active;             // some object is active: the boundary changes
  unsigned nobj;
  double dt;
};

// Launchers implemented in the .cu files (host side).
namespace gbk {
void load_dcell(const gbsph_consts& c, const DevArrays& a, unsigned n, cudaStream_t s);  // sets GB_ERR_PARTOUT in DivState::error
// RunPeriodic (JSphCpuSingle.cpp:416-504): marks the last copies to be ignored
// and appends new periodic copies; divide() runs it first when an axis is
// periodic.  blockcounts holds gb_div_up(cap, 256) + 1 entries.
void run_periodic(const gbsph_consts& c, DevArrays& a, unsigned cap, unsigned* blockcounts, cudaStream_t s,
                  unsigned long long* nlaunch);
// learned closure (gbsph_closure.cu)
cudaError_t closure_init();
void closure_features(const gbsph_consts& c, const DevArrays& a, unsigned cap, float* feat, cudaStream_t s,
                      unsigned long long* nlaunch);
void closure_apply(const gbsph_consts& c, const DevArrays& a, unsigned cap, const void* w_bf16, const float* feat,
                   float limit, unsigned* nfallback, cudaStream_t s, unsigned long long* nlaunch);
void mlp_infer(const void* w_bf16, const float* x, unsigned n, float* y, cudaStream_t s);
void mlp_grad(const void* w_bf16, const float* x, const float* t, unsigned n, float* grad, float* loss, cudaStream_t s);
void mlp_adam(float* master, void* w_bf16, float* grad, float* m, float* v, float lr, float b1, float b2, float eps,
              float bc1, float bc2, cudaStream_t s);
void to_bf16(const float* src, void* dst, int n, cudaStream_t s);
// keybits: bits of the largest box key; radixbits: digit width of the sort
// passes, 8 or 11 (11 needs sort_init first: its scatter takes 80 KB of
// shared memory)
void divide(const gbsph_consts& c, DevArrays& a, unsigned cap, unsigned keybits, int radixbits, cudaStream_t s,
            unsigned long long* nlaunch);
cudaError_t sort_init();
// Stable sort of n <= sort_noalloc_max_keys() keys of nbits bits on the static
// work area (work = its device address, from sort_noalloc_address on the
// current device).
unsigned sort_noalloc_max_keys();
cudaError_t sort_noalloc_address(void** p);
// Upload/download reshaping on the device: interleaved (x,y,z) doubles <->
// the px/py/pz arrays, and the boundary normals (3 floats, doubled as
// JSph::ConfigBoundNormals does, zero for non-boundary particles; nor3 may be
// null) into boundnor.  `stage` holds 3*n doubles.
void stage_upload(const DevArrays& a, const double* stage, const float* nor3, unsigned n, unsigned npb, cudaStream_t s);
void stage_download(const DevArrays& a, double* stage, unsigned n, cudaStream_t s);
void sort_noalloc(unsigned char* work, const unsigned* keys, unsigned n, unsigned nbits, unsigned* perm,
                  unsigned* sorted_keys, cudaStream_t s);
// Raises the shared-memory limit of the staged fluid-row kernels that the
// constants `c` select (call once per context, before any stream capture).
cudaError_t forces_init(const gbsph_consts& c);
// variant: 0 warp-queued rounds, 1 one thread per row (block size bsize),
// 2 cell-tiled staged (ring of 8 chunks), 3 cell-tiled staged (ring of 4)
// split (variant 2): 1, 2 or 4 warps share each group of 32 fluid rows
// the split a launch of gbk::forces uses: 1 unless the variant is 2 and the
// case takes the series form of the DDT2 hydrostatic term
int forces_split_effective(const gbsph_consts& c, int variant, int split);
// A second stream for work that runs beside the main one within a step, with
// the events that fork it from and join it to the main stream.
struct StreamFork {
  cudaStream_t side;
  cudaEvent_t fork, join;
};
// bound_lanes: lanes a boundary row in the bound-row pass (1, 4 or 32); with
// fork, the bound-row pass runs on fork->side beside the fluid-row pass (they
// write disjoint rows) and is joined before the call's work ends
void forces(const gbsph_consts& c, const DevArrays& a, unsigned cap, int bsize, int variant, int split,
            int bound_lanes, cudaStream_t s, unsigned long long* nlaunch, cudaEvent_t ev_fluid_begin = nullptr,
            cudaEvent_t ev_fluid_end = nullptr, const StreamFork* fork = nullptr);
// variant 1: one thread per boundary row (k_mdbc); otherwise the cell-tiled
// staged kernel (k_mdbc_t) with split (1, 2 or 4) warps per 32 boundary rows
void mdbc(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int split, cudaStream_t s,
          unsigned long long* nlaunch);
void dtvariable(const gbsph_consts& c, const DevArrays& a, int which, cudaStream_t s, unsigned long long* nlaunch);
void symplectic_pre(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, cudaStream_t s, unsigned long long* nlaunch);
void symplectic_cor(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, cudaStream_t s, unsigned long long* nlaunch);
void verlet_step(const gbsph_consts& c, DevArrays& a, unsigned cap, const double* dtp, int euler, cudaStream_t s, unsigned long long* nlaunch);
void sps_tau(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s, unsigned long long* nlaunch);
void pips(const gbsph_consts& c, const DevArrays& a, unsigned cap, cudaStream_t s);
void step_end(const DevArrays& a, int symplectic, cudaStream_t s, unsigned long long* nlaunch);
// RunShifting (JSphCpu.cpp:2084-2088) over the fluid rows, dt = dtfactor * *dtp.
void run_shifting(const gbsph_consts& c, const DevArrays& a, unsigned cap, const double* dtp, double dtfactor,
                  cudaStream_t s, unsigned long long* nlaunch);
// RunMotion (JSphCpu.cpp:2189-2245): index of each moving particle by id, then
// the linear or matrix movement of its object; marks the boundary changed.
// ridp holds nmoving entries for the ids idmin..idmin+nmoving-1.
void motion_move(const gbsph_consts& c, const DevArrays& a, const MotionStep* hdr, const MotionObjDev* objs,
                 unsigned nobj, unsigned* ridp, unsigned idmin, unsigned nmoving, unsigned cap, cudaStream_t s,
                 unsigned long long* nlaunch);
// Gauges (gbsph_gauges.cu): device arrays in and out, n gauges per launch.
// swl par: p0 (3) and step vector (3) per gauge; npts: PointNp; mlim: mass limit.
// maxz par: p0 (3) and height per gauge.
void gauge_velocity(const gbsph_consts& c, const DevArrays& a, unsigned n, const double* pts, float* vel, cudaStream_t s);
void gauge_swl(const gbsph_consts& c, const DevArrays& a, unsigned n, const double* par, const unsigned* npts,
               const float* mlim, float* surf, cudaStream_t s);
void gauge_maxz(const gbsph_consts& c, const DevArrays& a, unsigned n, const double* par, const float* dist,
                float* zmax, cudaStream_t s);
// Largest pos.dir over the fluid particles in [bmin, bmax] as an ordered key
// (zero-initialised by the caller) and their count; nsm = the device's SMs.
void fluid_front(const DevArrays& a, const double* dir, const double* bmin, const double* bmax,
                 unsigned long long* key, unsigned* count, int nsm, cudaStream_t s);
// mass (npt floats) is required; vel, vdir, rhop and zsurf may be null.
void gauge_mesh(const gbsph_consts& c, const DevArrays& a, const GaugeMeshPts& m, float kclimit, float kcdummy,
                float masslimit, float* vel, float* vdir, float* rhop, float* mass, float* zsurf, cudaStream_t s);
}  // namespace gbk
