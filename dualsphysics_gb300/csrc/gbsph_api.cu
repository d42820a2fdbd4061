// gbsph_api.cu -- C ABI of the GB300 WCSPH step (include/gbsph.h).
//
// A context owns one CUDA stream and one device arena (a single allocation
// carved into every array the step needs), so the step functions allocate
// nothing.  The step sequence mirrors JSphGpuSingle::ComputeStep_Sym /
// ComputeStep_Ver and the Run loop (JSphGpuSingle.cpp:785-826, 950-1010), but
// the dt, the particle counts and the cell-division limits stay on the device:
// no host round trip happens inside a step, and a whole step can be captured
// into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gbsph_common.cuh"
#include "gbsph_motion_internal.h"

struct gbsph_ctx {
  gbsph_consts c;
  unsigned cap = 0;    // allocated particles (the capacity rounded up to 256, so that
                       // consecutive arrays of 4-, 8- and 16-byte elements are contiguous)
  unsigned limit = 0;  // the capacity the caller asked for
  int device = 0;
  cudaStream_t stream = nullptr;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  DevArrays a;
  unsigned keybits = 8;   // bits of the largest box key (2 Nct + 6)
  int sort_bits = 8;      // digit width of the radix sort passes (8 or 11)
  unsigned nctt_cap = 0;
  bool uploaded = false;
  int verletstep = 0;
  unsigned long long launches = 0;
  int forces_bsize = 128, forces_variant = 2;
  int forces_split = 0;   // warps per group of 32 fluid rows in the staged kernel (0: from nfluid)
  int bound_lanes = 0;    // lanes a boundary row in the bound-row pass (0: from nbound)
  int mdbc_split = 0;     // warps per 32 boundary rows in the staged mDBC kernel (0: from nbound)
  // the bound-row pass on a side stream beside the fluid-row pass: 0.2 % on
  // C2 and 1.3 % on a 38 k-particle case, but the fluid pass's timing events
  // then include it, so it is off unless asked for
  bool bound_beside = false;
  gbk::StreamFork fork = {nullptr, nullptr, nullptr};
  unsigned nfluid = 0;    // fluid rows at the last upload (chooses the automatic split)
  unsigned nbound = 0;    // boundary rows at the last upload
  int nsm = 0;            // SMs of the device
  int mdbc_variant = 0;   // 0 staged kernel, 1 one thread per boundary row
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_parity = -1;  // pointer-swap parity the graph was captured with
  unsigned long long graph_launches = 0;  // kernel launches recorded in the step graph
  unsigned swaps = 0;     // number of reorders (each swaps the cur/alt pairs)
  // multi-step graph (one graph holding `multi_steps` steps)
  cudaGraphExec_t multi_exec = nullptr;
  unsigned multi_steps = 0;
  int multi_parity = -1;
  unsigned long long multi_launches = 0;
  // profiling: event pairs bracketing the fluid Interaction_Forces launches
  std::vector<cudaEvent_t> prof_ev;
  unsigned prof_cap = 0, prof_n = 0;
  cudaEvent_t marks[16] = {};
  // moving boundaries: the attached motion, its per-step table on the device
  // (MotionStep, nobj MotionObjDev, the ridp of nmoving ids) and a host copy
  gbsph_motion* motion = nullptr;
  unsigned mot_nobj = 0, mot_idmin = 0, mot_nmoving = 0;
  void* mot_buf = nullptr;
  std::vector<char> mot_host;
  void* gauge_buf = nullptr;  // gauge inputs and results (grown on demand)
  // learned closure: BF16 weights, the feature rows (cap x 16), the fallback counter
  void* clos_w = nullptr;
  float* clos_feat = nullptr;
  unsigned* clos_nfb = nullptr;
  float clos_limit = 0.2f;
  bool clos_on = false;
  size_t gauge_bytes = 0;
  std::string err;
};

namespace {

// Warps per group of 32 fluid rows in the staged kernel: the option, or with
// 0 the largest of 4, 2, 1 that keeps the launch within about three waves of
// resident warps (24 a SM), so that a small case runs more warps, each with a
// shorter chain of chunks, and a large one keeps one warp per group.  On a
// GB300 (152 SMs) that is 4 up to 87.5 k fluid rows and 2 up to 175 k; one
// warp a group was 14 % faster at 667 k rows, four 2.9x faster at 11 k.
int forces_split(const gbsph_ctx* ctx) {
  int s = ctx->forces_split;
  if (!s) {
    const unsigned long long warps = (ctx->nfluid + 31u) / 32u,
                             resident = 24ull * (unsigned)(ctx->nsm > 0 ? ctx->nsm : 1);
    s = warps * 4ull <= 3ull * resident ? 4 : warps * 2ull <= 3ull * resident ? 2 : 1;
  }
  return gbk::forces_split_effective(ctx->c, ctx->forces_variant, s);
}

// Lanes a boundary row in the bound-row pass: the option, or with 0 from the
// boundary rows of the last upload, against the SMs' resident threads (2,048
// a SM): 32 lanes while they make at most 12 waves, 4 while they make at
// most 6, else one thread a row.  Most boundary rows of a tank are dry and
// end after a few empty ranges, so many short rows of lanes cost little; on
// a GB300 that is 32 up to 117 k rows and 4 up to 467 k (measured steps:
// 0.475 ms with 32 against 0.788 with 1 at 27 k rows, 3.79 with 4 against
// 3.84 with 1 at 420 k, and one thread a row 2 % faster at 1.85 M).
int bound_lanes(const gbsph_ctx* ctx) {
  if (ctx->bound_lanes) return ctx->bound_lanes;
  const unsigned long long rows = ctx->nbound, resident = 2048ull * (unsigned)(ctx->nsm > 0 ? ctx->nsm : 1);
  return rows * 32ull <= 12ull * resident ? 32 : rows * 4ull <= 6ull * resident ? 4 : 1;
}

// Warps per group of 32 boundary rows in the staged mDBC kernel: the option,
// or with 0 four.  Only the boundary rows whose ghosts lie in the fluid's
// domain have work, a fraction of the walls, so the kernel is a latency
// chain at every size measured: four warps a group gave the shortest steps
// from 38 k particles (0.364 ms against 0.478 with one) to C2's 7.1 M
// (21.54 ms against 21.62).
int mdbc_split(const gbsph_ctx* ctx) {
  if (ctx->mdbc_variant == 1) return 1;
  return ctx->mdbc_split ? ctx->mdbc_split : 4;
}

int set_err(gbsph_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

int cuda_check(gbsph_ctx* ctx, cudaError_t e, const char* what) {
  if (e != cudaSuccess) return set_err(ctx, GBSPH_ECUDA, "%s: %s", what, cudaGetErrorString(e));
  return GBSPH_OK;
}

#define CK(call, what)                                  \
  do {                                                  \
    int rc_ = cuda_check(ctx, (call), what);            \
    if (rc_) return rc_;                                \
  } while (0)

// Reads the device error words; returns a status for the first error found.
int check_device_errors(gbsph_ctx* ctx) {
  unsigned derr = 0, serr = 0;
  CK(cudaMemcpyAsync(&derr, &ctx->a.div->error, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream), "read error");
  CK(cudaMemcpyAsync(&serr, &ctx->a.st->error, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream), "read error");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  if (derr & GB_ERR_BOUNDOUT) return set_err(ctx, GBSPH_EBOUND_OUT, "boundary particles left the domain");
  if (derr & GB_ERR_CELLCAP) return set_err(ctx, GBSPH_ECAPACITY, "cell domain exceeds the allocated cells");
  if (derr & GB_ERR_PERICAP) return set_err(ctx, GBSPH_ECAPACITY, "the periodic copies exceed the particle capacity");
  if (serr & GB_ERR_NANDT) return set_err(ctx, GBSPH_ENAN_DT, "the computed dt is NaN or infinity");
  return GBSPH_OK;
}

struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base((char*)b) {}
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~(size_t)255;
    T* p = base ? (T*)(base + off) : nullptr;
    off += n * sizeof(T);
    return p;
  }
};

// Lays out every array of the context; with base==nullptr only measures.
size_t layout(gbsph_ctx* ctx, void* base) {
  Carver k(base);
  DevArrays& a = ctx->a;
  const size_t n = ctx->cap;
  const bool sps = ctx->c.tvisco == GBSPH_VISCO_LAMINARSPS;
  const bool nor = ctx->c.tboundary == GBSPH_BC_MDBC;
  a.px = k.take<double>(n); a.py = k.take<double>(n); a.pz = k.take<double>(n);
  a.px2 = k.take<double>(n); a.py2 = k.take<double>(n); a.pz2 = k.take<double>(n);
  a.qx = k.take<double>(n); a.qy = k.take<double>(n); a.qz = k.take<double>(n);
  a.qx2 = k.take<double>(n); a.qy2 = k.take<double>(n); a.qz2 = k.take<double>(n);
  a.velrho = k.take<float4>(n); a.velrho2 = k.take<float4>(n);
  a.velrhopre = k.take<float4>(n); a.velrhopre2 = k.take<float4>(n);
  a.idp = k.take<unsigned>(n); a.idp2 = k.take<unsigned>(n);
  a.dcell = k.take<unsigned>(n); a.dcell2 = k.take<unsigned>(n);
  a.code = k.take<uint16_t>(n); a.code2 = k.take<uint16_t>(n);
  a.boundnor = nor ? k.take<float4>(n) : nullptr;
  a.boundnor2 = nor ? k.take<float4>(n) : nullptr;
  a.taua = sps ? k.take<float4>(n) : nullptr; a.taua2 = sps ? k.take<float4>(n) : nullptr;
  a.taub = sps ? k.take<float2>(n) : nullptr; a.taub2 = sps ? k.take<float2>(n) : nullptr;
  a.straina = sps ? k.take<float4>(n) : nullptr;
  a.strainb = sps ? k.take<float2>(n) : nullptr;
  a.pscell = k.take<float4>(n);
  a.acear = k.take<float4>(n);
  a.shiftpos = ctx->c.tshift ? k.take<float4>(n) : nullptr;
  a.keys = k.take<unsigned>(n); a.keys2 = k.take<unsigned>(n);
  a.vals = k.take<unsigned>(n); a.vals2 = k.take<unsigned>(n);
  const size_t ntiles = (n + 2047) / 2048;
  a.hist = k.take<unsigned>(ntiles * 2048 + 2048 + 1);  // tile counts + digit totals, digits of up to 11 bits
  a.begincell = k.take<unsigned>(ctx->nctt_cap + 1);
  a.div = k.take<DivState>(1);
  a.st = k.take<StepState>(1);
  a.pips = k.take<unsigned long long>(4);
  return k.off + 256;
}

void reset_graph(gbsph_ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
  ctx->graph_parity = -1;
  if (ctx->multi_exec) cudaGraphExecDestroy(ctx->multi_exec);
  ctx->multi_exec = nullptr;
  ctx->multi_steps = 0;
  ctx->multi_parity = -1;
}

int do_divide(gbsph_ctx* ctx) {
  gbk::divide(ctx->c, ctx->a, ctx->cap, ctx->keybits, ctx->sort_bits, ctx->stream, &ctx->launches);
  ctx->swaps++;
  return cuda_check(ctx, cudaGetLastError(), "divide");
}

int do_forces(gbsph_ctx* ctx) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ctx->prof_n < ctx->prof_cap) {
    e0 = ctx->prof_ev[2 * ctx->prof_n];
    e1 = ctx->prof_ev[2 * ctx->prof_n + 1];
    ctx->prof_n++;
  }
  gbk::forces(ctx->c, ctx->a, ctx->cap, ctx->forces_bsize, ctx->forces_variant, forces_split(ctx), bound_lanes(ctx),
              ctx->stream, &ctx->launches, e0, e1, ctx->bound_beside ? &ctx->fork : nullptr);
  if (ctx->c.tvisco == GBSPH_VISCO_LAMINARSPS) gbk::sps_tau(ctx->c, ctx->a, ctx->cap, ctx->stream, &ctx->launches);
  if (ctx->clos_on) {  // the learned correction of the fluid accelerations
    gbk::closure_features(ctx->c, ctx->a, ctx->cap, ctx->clos_feat, ctx->stream, &ctx->launches);
    gbk::closure_apply(ctx->c, ctx->a, ctx->cap, ctx->clos_w, ctx->clos_feat, ctx->clos_limit, ctx->clos_nfb,
                       ctx->stream, &ctx->launches);
  }
  return cuda_check(ctx, cudaGetLastError(), "forces");
}

}  // namespace
extern "C" {
static int motion_table(gbsph_ctx* ctx, const StepState& st, cudaStream_t s);  // defined with the motion entries
}
namespace {

// Bytes of the device motion table before the ridp array.
size_t motion_table_bytes(unsigned nobj) { return 256 + 256 * ((sizeof(MotionObjDev) * nobj + 255) / 256); }

// One step, enqueued: ComputeStep_Sym/_Ver + RunCellDivide.
int enqueue_step(gbsph_ctx* ctx) {
  const gbsph_consts& c = ctx->c;
  double* dtpre = &ctx->a.st->dtpre;
  if (c.tstep == GBSPH_STEP_SYMPLECTIC) {
    if (c.tboundary == GBSPH_BC_MDBC) gbk::mdbc(c, ctx->a, ctx->cap, ctx->mdbc_variant, mdbc_split(ctx), ctx->stream, &ctx->launches);
    if (int rc = do_forces(ctx)) return rc;
    gbk::dtvariable(c, ctx->a, 0, ctx->stream, &ctx->launches);
    gbk::symplectic_pre(c, ctx->a, ctx->cap, dtpre, ctx->stream, &ctx->launches);
    if (int rc = do_divide(ctx)) return rc;
    if (int rc = do_forces(ctx)) return rc;
    gbk::dtvariable(c, ctx->a, 1, ctx->stream, &ctx->launches);
    // RunShifting(dt) before the corrector; the predictor's RunShifting(dt/2)
    // is not enqueued: the reference's predictor does not apply it and the
    // corrector's interaction recomputes the sums
    if (c.tshift) gbk::run_shifting(c, ctx->a, ctx->cap, dtpre, 1.0, ctx->stream, &ctx->launches);
    gbk::symplectic_cor(c, ctx->a, ctx->cap, dtpre, ctx->stream, &ctx->launches);
    gbk::step_end(ctx->a, 1, ctx->stream, &ctx->launches);
    if (ctx->motion) {  // RunMotion, before the divide that ends the step
      char* mb = (char*)ctx->mot_buf;
      gbk::motion_move(c, ctx->a, (const MotionStep*)mb, (const MotionObjDev*)(mb + 256), ctx->mot_nobj,
                       (unsigned*)(mb + motion_table_bytes(ctx->mot_nobj)), ctx->mot_idmin, ctx->mot_nmoving,
                       ctx->cap, ctx->stream, &ctx->launches);
    }
  } else {
    if (c.tboundary == GBSPH_BC_MDBC) gbk::mdbc(c, ctx->a, ctx->cap, ctx->mdbc_variant, mdbc_split(ctx), ctx->stream, &ctx->launches);
    if (int rc = do_forces(ctx)) return rc;
    gbk::dtvariable(c, ctx->a, 2, ctx->stream, &ctx->launches);
    if (ctx->motion) {
      // CalcMotion(dt) with the dt this step just computed (JSphCpuSingle.cpp:
      // 879): read back, advance the motion on the host, upload its table
      StepState st;
      CK(cudaMemcpyAsync(&st, ctx->a.st, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream), "motion dt");
      CK(cudaStreamSynchronize(ctx->stream), "motion sync");
      st.dtpre = st.dt_var;
      if (int rc = motion_table(ctx, st, ctx->stream)) return rc;
    }
    if (c.tshift) gbk::run_shifting(c, ctx->a, ctx->cap, &ctx->a.st->dt_var, 1.0, ctx->stream, &ctx->launches);
    ctx->verletstep++;
    const int euler = !(ctx->verletstep < c.verletsteps);
    if (euler) ctx->verletstep = 0;
    gbk::verlet_step(c, ctx->a, ctx->cap, &ctx->a.st->dt_var, euler, ctx->stream, &ctx->launches);
    gbk::step_end(ctx->a, 0, ctx->stream, &ctx->launches);
    if (ctx->motion) {  // RunMotion(dt), before the divide that ends the step
      char* mb = (char*)ctx->mot_buf;
      gbk::motion_move(c, ctx->a, (const MotionStep*)mb, (const MotionObjDev*)(mb + 256), ctx->mot_nobj,
                       (unsigned*)(mb + motion_table_bytes(ctx->mot_nobj)), ctx->mot_idmin, ctx->mot_nmoving,
                       ctx->cap, ctx->stream, &ctx->launches);
    }
  }
  return do_divide(ctx);
}

double* device_scalar(gbsph_ctx* ctx) { return &ctx->a.st->dt_var; }

}  // namespace

extern "C" {

int gbsph_create(const gbsph_consts* c, unsigned capacity, int device, gbsph_ctx** out) {
  // particle indices carry a tag in bit 31 inside the fluid-row kernel
  if (!c || !out || capacity == 0 || capacity > 0x7fffffffu) return GBSPH_EINVAL;
  if (c->cellmode_div != 1 && c->cellmode_div != 2) return GBSPH_EINVAL;
  *out = nullptr;
  if (c->domcellcode == 0) return GBSPH_EINVAL;
  if (c->tstep != GBSPH_STEP_SYMPLECTIC && c->tstep != GBSPH_STEP_VERLET) return GBSPH_EINVAL;
  gbsph_ctx* ctx = new gbsph_ctx();
  ctx->c = *c;
  ctx->limit = capacity;
  ctx->cap = (capacity + 255u) & ~255u;
  ctx->device = device;
  const unsigned long long maxnct = (unsigned long long)c->domcells[0] * c->domcells[1] * c->domcells[2];
  if (2ull * maxnct + 6 >= 0xffffffffull) {
    delete ctx;
    return GBSPH_ECAPACITY;
  }
  ctx->nctt_cap = (unsigned)(2ull * maxnct + 6);
  unsigned bits = 1;
  while ((1ull << bits) < ctx->nctt_cap) bits++;
  ctx->keybits = bits;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    delete ctx;
    return GBSPH_ECUDA;
  }
  if (gbk::sort_init() != cudaSuccess || gbk::forces_init(*c) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return GBSPH_ECUDA;
  }
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->fork.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->fork.fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->fork.join, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    if (ctx->fork.fork) cudaEventDestroy(ctx->fork.fork);
    if (ctx->fork.side) cudaStreamDestroy(ctx->fork.side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GBSPH_ECUDA;
  }
  ctx->arena_bytes = layout(ctx, nullptr);
  if (cudaMalloc(&ctx->arena, ctx->arena_bytes) != cudaSuccess) {
    cudaGetLastError();
    cudaEventDestroy(ctx->fork.fork);
    cudaEventDestroy(ctx->fork.join);
    cudaStreamDestroy(ctx->fork.side);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GBSPH_ENOMEM;
  }
  layout(ctx, ctx->arena);
  *out = ctx;
  return GBSPH_OK;
}

void gbsph_destroy(gbsph_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  reset_graph(ctx);
  for (auto ev : ctx->prof_ev) cudaEventDestroy(ev);
  for (auto ev : ctx->marks) if (ev) cudaEventDestroy(ev);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->arena) cudaFree(ctx->arena);
  if (ctx->gauge_buf) cudaFree(ctx->gauge_buf);
  if (ctx->mot_buf) cudaFree(ctx->mot_buf);
  if (ctx->clos_w) cudaFree(ctx->clos_w);
  if (ctx->clos_feat) cudaFree(ctx->clos_feat);
  if (ctx->clos_nfb) cudaFree(ctx->clos_nfb);
  if (ctx->fork.side) cudaStreamSynchronize(ctx->fork.side);
  if (ctx->fork.fork) cudaEventDestroy(ctx->fork.fork);
  if (ctx->fork.join) cudaEventDestroy(ctx->fork.join);
  if (ctx->fork.side) cudaStreamDestroy(ctx->fork.side);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* gbsph_last_error(const gbsph_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

static int upload_common(gbsph_ctx* ctx, unsigned np, unsigned npb) {
  const gbsph_consts& c = ctx->c;
  ctx->nfluid = np - npb;
  ctx->nbound = npb;
  DivState ds;
  memset(&ds, 0, sizeof(ds));
  ds.np = np;
  ds.npb = npb;
  ds.npbok = npb;
  ds.boundchanged = 1;
  ds.nctt_cap = ctx->nctt_cap;
  StepState st;
  memset(&st, 0, sizeof(st));
  st.dtpre = c.dtini;
  CK(cudaMemcpyAsync(ctx->a.div, &ds, sizeof(ds), cudaMemcpyHostToDevice, ctx->stream), "upload div");
  CK(cudaMemcpyAsync(ctx->a.st, &st, sizeof(st), cudaMemcpyHostToDevice, ctx->stream), "upload st");
  // InitRunCpu: VelrhoM1 = Velrho; SPS tau = 0 (JSphCpu.cpp:472-482)
  CK(cudaMemcpyAsync(ctx->a.velrhopre, ctx->a.velrho, sizeof(float4) * np, cudaMemcpyDeviceToDevice, ctx->stream), "m1");
  if (ctx->a.taua) {
    CK(cudaMemsetAsync(ctx->a.taua, 0, sizeof(float4) * ctx->cap, ctx->stream), "tau");
    CK(cudaMemsetAsync(ctx->a.taub, 0, sizeof(float2) * ctx->cap, ctx->stream), "tau");
  }
  CK(cudaMemsetAsync(ctx->a.acear, 0, sizeof(float4) * ctx->cap, ctx->stream), "acear");
  gbk::load_dcell(c, ctx->a, np, ctx->stream);
  ctx->launches++;
  ctx->verletstep = 0;
  reset_graph(ctx);
  {
    unsigned derr = 0;
    CK(cudaMemcpyAsync(&derr, &ctx->a.div->error, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream), "upload");
    CK(cudaStreamSynchronize(ctx->stream), "upload");
    if (derr & GB_ERR_PARTOUT) return set_err(ctx, GBSPH_EINVAL, "found particles outside the domain in the initial state");
  }
  if (int rc = do_divide(ctx)) return rc;
  ctx->uploaded = true;
  return check_device_errors(ctx);
}

int gbsph_upload(gbsph_ctx* ctx, unsigned np, unsigned npb, const double* pos, const float* velrho,
                 const unsigned* idp, const uint16_t* code, const float* boundnor) {
  if (!ctx || !pos || !velrho || !idp || !code) return set_err(ctx, GBSPH_EINVAL, "null argument");
  if (np > ctx->limit || npb > np) return set_err(ctx, GBSPH_ECAPACITY, "np=%u exceeds capacity %u", np, ctx->limit);
  CK(cudaSetDevice(ctx->device), "set device");
  // the caller's arrays are copied as they are; positions are split into x, y,
  // z and the normals doubled on the device, from the alternate position arrays
  // and the sort buffers as staging (both unused until the first divide)
  double* stage = ctx->a.px2;  // px2, py2, pz2: 3*cap contiguous doubles
  CK(cudaMemcpyAsync(stage, pos, sizeof(double) * 3 * (size_t)np, cudaMemcpyHostToDevice, ctx->stream), "upload pos");
  CK(cudaMemcpyAsync(ctx->a.velrho, velrho, sizeof(float4) * np, cudaMemcpyHostToDevice, ctx->stream), "upload velrho");
  CK(cudaMemcpyAsync(ctx->a.idp, idp, sizeof(unsigned) * np, cudaMemcpyHostToDevice, ctx->stream), "upload idp");
  CK(cudaMemcpyAsync(ctx->a.code, code, sizeof(uint16_t) * np, cudaMemcpyHostToDevice, ctx->stream), "upload code");
  float* nstage = nullptr;
  if (ctx->a.boundnor && boundnor) {
    nstage = (float*)ctx->a.keys;  // keys, keys2, vals, vals2: 16*cap contiguous bytes
    CK(cudaMemcpyAsync(nstage, boundnor, sizeof(float) * 3 * (size_t)np, cudaMemcpyHostToDevice, ctx->stream),
       "upload nor");
  }
  gbk::stage_upload(ctx->a, stage, nstage, np, npb, ctx->stream);
  CK(cudaGetLastError(), "upload");
  CK(cudaStreamSynchronize(ctx->stream), "upload sync");
  return upload_common(ctx, np, npb);
}

int gbsph_upload_device(gbsph_ctx* ctx, unsigned np, unsigned npb, const double* d_pos, const float* d_velrho,
                        const unsigned* d_idp, const uint16_t* d_code, const float* d_boundnor) {
  if (!ctx || !d_pos || !d_velrho || !d_idp || !d_code) return set_err(ctx, GBSPH_EINVAL, "null argument");
  if (np > ctx->limit || npb > np) return set_err(ctx, GBSPH_ECAPACITY, "np=%u exceeds capacity %u", np, ctx->limit);
  CK(cudaSetDevice(ctx->device), "set device");
  // de-interleave xyz with strided 2-D copies
  CK(cudaMemcpy2DAsync(ctx->a.px, sizeof(double), d_pos, 3 * sizeof(double), sizeof(double), np, cudaMemcpyDeviceToDevice, ctx->stream), "pos");
  CK(cudaMemcpy2DAsync(ctx->a.py, sizeof(double), d_pos + 1, 3 * sizeof(double), sizeof(double), np, cudaMemcpyDeviceToDevice, ctx->stream), "pos");
  CK(cudaMemcpy2DAsync(ctx->a.pz, sizeof(double), d_pos + 2, 3 * sizeof(double), sizeof(double), np, cudaMemcpyDeviceToDevice, ctx->stream), "pos");
  CK(cudaMemcpyAsync(ctx->a.velrho, d_velrho, sizeof(float4) * np, cudaMemcpyDeviceToDevice, ctx->stream), "velrho");
  CK(cudaMemcpyAsync(ctx->a.idp, d_idp, sizeof(unsigned) * np, cudaMemcpyDeviceToDevice, ctx->stream), "idp");
  CK(cudaMemcpyAsync(ctx->a.code, d_code, sizeof(uint16_t) * np, cudaMemcpyDeviceToDevice, ctx->stream), "code");
  if (ctx->a.boundnor) {
    CK(cudaMemsetAsync(ctx->a.boundnor, 0, sizeof(float4) * ctx->cap, ctx->stream), "nor");
    if (d_boundnor) {
      // boundary particles come first in case order; doubled as in gbsph_upload
      std::vector<float> h(3 * (size_t)npb);
      CK(cudaMemcpyAsync(h.data(), d_boundnor, sizeof(float) * 3 * npb, cudaMemcpyDeviceToHost, ctx->stream), "nor");
      CK(cudaStreamSynchronize(ctx->stream), "nor");
      std::vector<float4> bn(npb);
      for (unsigned p = 0; p < npb; p++) bn[p] = make_float4(h[3 * p] * 2.f, h[3 * p + 1] * 2.f, h[3 * p + 2] * 2.f, 0.f);
      CK(cudaMemcpyAsync(ctx->a.boundnor, bn.data(), sizeof(float4) * npb, cudaMemcpyHostToDevice, ctx->stream), "nor");
      CK(cudaStreamSynchronize(ctx->stream), "nor");
    }
  }
  return upload_common(ctx, np, npb);
}

int gbsph_divide(gbsph_ctx* ctx) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  return do_divide(ctx);
}

int gbsph_mdbc(gbsph_ctx* ctx, int interstep) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  // MdbcCorrector is false for SlipMode=vel0: only the predictor (and Verlet) correct.
  if (ctx->c.tboundary != GBSPH_BC_MDBC || interstep == GBSPH_INTERSTEP_SYMCORRECTOR) return GBSPH_OK;
  gbk::mdbc(ctx->c, ctx->a, ctx->cap, ctx->mdbc_variant, mdbc_split(ctx), ctx->stream, &ctx->launches);
  return cuda_check(ctx, cudaGetLastError(), "mdbc");
}

int gbsph_forces(gbsph_ctx* ctx, int interstep, gbsph_maxes* maxes) {
  (void)interstep;
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (int rc = do_forces(ctx)) return rc;
  if (maxes) return gbsph_get_maxes(ctx, maxes);
  return GBSPH_OK;
}

int gbsph_get_maxes(gbsph_ctx* ctx, gbsph_maxes* m) {
  if (!ctx || !m) return GBSPH_EINVAL;
  unsigned v[3];
  CK(cudaMemcpyAsync(v, &ctx->a.st->acemax2, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream), "maxes");
  CK(cudaStreamSynchronize(ctx->stream), "maxes");
  float f[3];
  memcpy(f, v, sizeof(f));
  m->acemax = sqrt((double)f[0]);
  m->velmax = sqrtf(f[1]);
  m->viscdtmax = f[2];
  return GBSPH_OK;
}

int gbsph_dtvariable(gbsph_ctx* ctx, int final, double* dt) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  const int which = (ctx->c.tstep == GBSPH_STEP_VERLET) ? 2 : (final ? 1 : 0);
  gbk::dtvariable(ctx->c, ctx->a, which, ctx->stream, &ctx->launches);
  if (dt) {
    CK(cudaMemcpyAsync(dt, &ctx->a.st->dt_var, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "dt");
    CK(cudaStreamSynchronize(ctx->stream), "dt");
    return check_device_errors(ctx);
  }
  return GBSPH_OK;
}

static int set_device_dt(gbsph_ctx* ctx, double dt) {
  CK(cudaMemcpyAsync(device_scalar(ctx), &dt, sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "dt");
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "dt");
}

int gbsph_symplectic_pre(gbsph_ctx* ctx, double dt) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (int rc = set_device_dt(ctx, dt)) return rc;
  gbk::symplectic_pre(ctx->c, ctx->a, ctx->cap, device_scalar(ctx), ctx->stream, &ctx->launches);
  return cuda_check(ctx, cudaGetLastError(), "symplectic_pre");
}

int gbsph_symplectic_cor(gbsph_ctx* ctx, double dt) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (int rc = set_device_dt(ctx, dt)) return rc;
  gbk::symplectic_cor(ctx->c, ctx->a, ctx->cap, device_scalar(ctx), ctx->stream, &ctx->launches);
  return cuda_check(ctx, cudaGetLastError(), "symplectic_cor");
}

int gbsph_run_shifting(gbsph_ctx* ctx, double dt) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (!ctx->c.tshift) return GBSPH_OK;
  if (int rc = set_device_dt(ctx, dt)) return rc;
  gbk::run_shifting(ctx->c, ctx->a, ctx->cap, device_scalar(ctx), 1.0, ctx->stream, &ctx->launches);
  return cuda_check(ctx, cudaGetLastError(), "run_shifting");
}

static int read_div(gbsph_ctx* ctx, DivState* ds);

int gbsph_get_shiftpos(gbsph_ctx* ctx, float* shiftpos) {
  if (!ctx || !ctx->uploaded || !shiftpos) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (!ctx->a.shiftpos) return set_err(ctx, GBSPH_EINVAL, "the case has no shifting");
  DivState ds;
  if (int rc = read_div(ctx, &ds)) return rc;
  CK(cudaMemcpyAsync(shiftpos, ctx->a.shiftpos, sizeof(float4) * ds.np, cudaMemcpyDeviceToHost, ctx->stream), "shiftpos");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return GBSPH_OK;
}

int gbsph_verlet(gbsph_ctx* ctx, double dt) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (int rc = set_device_dt(ctx, dt)) return rc;
  ctx->verletstep++;
  const int euler = !(ctx->verletstep < ctx->c.verletsteps);
  if (euler) ctx->verletstep = 0;
  gbk::verlet_step(ctx->c, ctx->a, ctx->cap, device_scalar(ctx), euler, ctx->stream, &ctx->launches);
  return cuda_check(ctx, cudaGetLastError(), "verlet");
}

// JSph::CalcMotion at the start of a Symplectic step (JSphGpuSingle.cpp:787):
// the host advances the motion over [time, time+SymplecticDtPre] and copies
// the step's motion table to the device.
// Advances the motion over the step that starts at st.time with st.dtpre and
// copies its table to the device on stream s.
static int motion_table(gbsph_ctx* ctx, const StepState& st, cudaStream_t s) {
  const unsigned n = ctx->mot_nobj;
  std::vector<gbsph_motion_data> md(n);
  const int rc = gbsph_motion_process(ctx->motion, st.time, st.dtpre, md.data());
  if (rc < 0) return set_err(ctx, GBSPH_EINVAL, "motion: time %.17g is before the motion's last interval", st.time);
  std::vector<char>& h = ctx->mot_host;
  h.assign(motion_table_bytes(n), 0);
  MotionStep* hdr = (MotionStep*)h.data();
  hdr->active = rc;
  hdr->nobj = n;
  hdr->dt = st.dtpre;
  MotionObjDev* o = (MotionObjDev*)(h.data() + 256);
  const gbsph_motion_object* info = gbmotion::objects(ctx->motion);
  for (unsigned k = 0; k < n; k++) {
    o[k].type = md[k].type;
    o[k].idbegin = info[k].idbegin;
    o[k].count = info[k].count;
    for (int c = 0; c < 3; c++) {
      o[k].linmov[c] = md[k].linmov[c];
      o[k].linvel[c] = (float)md[k].linvel[c];  // ToTFloat3(m.linvel)
    }
    for (int c = 0; c < 12; c++) o[k].mat[c] = md[k].mat[c];
  }
  // pageable source: the copy has read it when the call returns
  CK(cudaMemcpyAsync(ctx->mot_buf, h.data(), h.size(), cudaMemcpyHostToDevice, s), "motion table");
  return GBSPH_OK;
}

static int motion_prepare(gbsph_ctx* ctx) {
  StepState st;
  CK(cudaMemcpyAsync(&st, ctx->a.st, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream), "motion dt");
  CK(cudaStreamSynchronize(ctx->stream), "motion sync");
  return motion_table(ctx, st, ctx->stream);
}

int gbsph_set_motion(gbsph_ctx* ctx, gbsph_motion* m) {
  if (!ctx) return GBSPH_EINVAL;
  CK(cudaSetDevice(ctx->device), "set device");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  reset_graph(ctx);
  if (ctx->mot_buf) cudaFree(ctx->mot_buf);
  ctx->mot_buf = nullptr;
  ctx->motion = nullptr;
  ctx->mot_nobj = ctx->mot_idmin = ctx->mot_nmoving = 0;
  if (!m) return GBSPH_OK;
  const unsigned n = gbmotion::object_count(m);
  const gbsph_motion_object* info = gbmotion::objects(m);
  unsigned long long lo = ~0ull, hi = 0;
  for (unsigned k = 0; k < n; k++) {
    lo = info[k].idbegin < lo ? info[k].idbegin : lo;
    const unsigned long long e = (unsigned long long)info[k].idbegin + info[k].count;
    hi = e > hi ? e : hi;
  }
  if (!n || hi <= lo || hi - lo > ctx->limit) return set_err(ctx, GBSPH_EINVAL, "motion objects do not fit the particles");
  const size_t bytes = motion_table_bytes(n) + sizeof(unsigned) * (size_t)(hi - lo);
  if (cudaMalloc(&ctx->mot_buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    ctx->mot_buf = nullptr;
    return set_err(ctx, GBSPH_ENOMEM, "motion table");
  }
  CK(cudaMemset(ctx->mot_buf, 0, bytes), "motion table");
  ctx->motion = m;
  ctx->mot_nobj = n;
  ctx->mot_idmin = (unsigned)lo;
  ctx->mot_nmoving = (unsigned)(hi - lo);
  return GBSPH_OK;
}

int gbsph_step(gbsph_ctx* ctx) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (ctx->motion && ctx->c.tstep == GBSPH_STEP_SYMPLECTIC)  // Verlet advances it inside the step
    if (int rc = motion_prepare(ctx)) return rc;
  return enqueue_step(ctx);
}

int gbsph_run(gbsph_ctx* ctx, unsigned nsteps, int use_graph) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  // A step swaps the cur/alt array pairs once per divide: graphs are replayed
  // only with the pointer parity they were captured with.  Verlet steps (one
  // divide and a host-side Euler counter) run eagerly.
  if (!use_graph || ctx->c.tstep != GBSPH_STEP_SYMPLECTIC) {
    for (unsigned i = 0; i < nsteps; i++) {
      if (ctx->motion && ctx->c.tstep == GBSPH_STEP_SYMPLECTIC)
        if (int rc = motion_prepare(ctx)) return rc;
      if (int rc = enqueue_step(ctx)) return rc;
    }
    return cuda_check(ctx, cudaGetLastError(), "run");
  }
  const int parity = (int)(ctx->swaps & 1u);
  if (use_graph == 2 && !ctx->motion) {
    if (int rc = gbsph_graph_prepare(ctx, nsteps)) return rc;
    CK(cudaGraphLaunch(ctx->multi_exec, ctx->stream), "graph launch");
    ctx->swaps += 2 * nsteps;
    ctx->launches += ctx->multi_launches;
    return cuda_check(ctx, cudaGetLastError(), "run");
  }
  if (!ctx->graph_exec || ctx->graph_parity != parity) {
    reset_graph(ctx);
    const unsigned long long l0 = ctx->launches;
    const unsigned s0 = ctx->swaps;
    const DevArrays a0 = ctx->a;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "capture");
    int rc = enqueue_step(ctx);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    // capture records the work; it did not run: restore the host-side pointer state
    ctx->graph_launches = ctx->launches - l0;
    ctx->a = a0;
    ctx->swaps = s0;
    ctx->launches = l0;
    if (rc) return rc;
    CK(e, "end capture");
    ctx->graph = g;
    CK(cudaGraphInstantiate(&ctx->graph_exec, g, 0), "instantiate");
    ctx->graph_parity = parity;
  }
  for (unsigned i = 0; i < nsteps; i++) {
    // a motion is advanced on the host before each replay; its table lives in
    // device memory, which the captured step reads
    if (ctx->motion)
      if (int rc = motion_prepare(ctx)) return rc;
    CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream), "graph launch");
    // the captured step swapped every cur/alt pair twice: parity unchanged
    ctx->swaps += 2;
    ctx->launches += ctx->graph_launches;
  }
  return cuda_check(ctx, cudaGetLastError(), "run");
}

int gbsph_graph_prepare(gbsph_ctx* ctx, unsigned nsteps) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (ctx->c.tstep != GBSPH_STEP_SYMPLECTIC) return set_err(ctx, GBSPH_EINVAL, "multi-step graphs need Symplectic");
  if (ctx->motion) return set_err(ctx, GBSPH_EINVAL, "multi-step graphs cannot hold a motion advanced on the host");
  const int parity = (int)(ctx->swaps & 1u);
  if (ctx->multi_exec && ctx->multi_steps == nsteps && ctx->multi_parity == parity) return GBSPH_OK;
  if (ctx->multi_exec) cudaGraphExecDestroy(ctx->multi_exec);
  ctx->multi_exec = nullptr;
  // profiling events captured into the graph: slots 0..prof_n-1 are recorded on every replay
  ctx->prof_n = 0;
  const unsigned long long l0 = ctx->launches;
  const unsigned s0 = ctx->swaps;
  const DevArrays a0 = ctx->a;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "capture");
  int rc = GBSPH_OK;
  for (unsigned i = 0; i < nsteps && !rc; i++) rc = enqueue_step(ctx);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  ctx->multi_launches = ctx->launches - l0;
  ctx->a = a0;
  ctx->swaps = s0;
  ctx->launches = l0;
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  CK(e, "end capture");
  cudaError_t ei = cudaGraphInstantiate(&ctx->multi_exec, g, 0);
  cudaGraphDestroy(g);
  CK(ei, "instantiate");
  ctx->multi_steps = nsteps;
  ctx->multi_parity = parity;
  return GBSPH_OK;
}

int gbsph_profile(gbsph_ctx* ctx, unsigned max_launches) {
  if (!ctx) return GBSPH_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  for (auto ev : ctx->prof_ev) cudaEventDestroy(ev);
  ctx->prof_ev.clear();
  ctx->prof_cap = 0;
  ctx->prof_n = 0;
  reset_graph(ctx);
  if (!max_launches) return GBSPH_OK;
  ctx->prof_ev.resize(2 * (size_t)max_launches);
  for (auto& ev : ctx->prof_ev) CK(cudaEventCreate(&ev), "event");
  ctx->prof_cap = max_launches;
  return GBSPH_OK;
}

int gbsph_profile_read(gbsph_ctx* ctx, float* ms, unsigned cap, unsigned* n) {
  if (!ctx || !n) return GBSPH_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  const unsigned cnt = ctx->prof_n < cap ? ctx->prof_n : cap;
  for (unsigned i = 0; i < cnt; i++)
    CK(cudaEventElapsedTime(&ms[i], ctx->prof_ev[2 * i], ctx->prof_ev[2 * i + 1]), "elapsed");
  *n = cnt;
  ctx->prof_n = 0;
  return GBSPH_OK;
}

// Work area of gbsph_sort_keys_noalloc: its device address per device, looked
// up by the first call made for that device (with that device current).
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
void* g_na_work[kMaxDevices] = {};
}  // namespace

int gbsph_sort_keys_noalloc(gbsph_ctx* ctx, const unsigned* d_keys, unsigned n, unsigned nbits, unsigned* d_perm,
                            unsigned* d_sorted_keys) {
  if (!ctx) return GBSPH_EINVAL;
  if (!d_keys || !d_perm) return set_err(ctx, GBSPH_EINVAL, "gbsph_sort_keys_noalloc: null key or permutation pointer");
  if (nbits < 1 || nbits > 32) return set_err(ctx, GBSPH_EINVAL, "gbsph_sort_keys_noalloc: nbits=%u is not in 1..32", nbits);
  const unsigned maxkeys = gbk::sort_noalloc_max_keys();
  if (n > maxkeys)
    return set_err(ctx, GBSPH_ECAPACITY, "gbsph_sort_keys_noalloc: n=%u keys exceed the fixed work area of %u keys", n,
                   maxkeys);
  if (ctx->device < 0 || ctx->device >= kMaxDevices)
    return set_err(ctx, GBSPH_EINVAL, "gbsph_sort_keys_noalloc: device %d out of range", ctx->device);
  CK(cudaSetDevice(ctx->device), "set device");
  void* work = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_work[ctx->device]) CK(gbk::sort_noalloc_address(&g_na_work[ctx->device]), "work-area address");
    work = g_na_work[ctx->device];
  }
  if (n == 0) return GBSPH_OK;
  gbk::sort_noalloc((unsigned char*)work, d_keys, n, nbits, d_perm, d_sorted_keys, ctx->stream);
  return cuda_check(ctx, cudaGetLastError(), "gbsph_sort_keys_noalloc");
}

int gbsph_pips(gbsph_ctx* ctx, unsigned long long* out4) {
  if (!ctx || !ctx->uploaded || !out4) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  gbk::pips(ctx->c, ctx->a, ctx->cap, ctx->stream);
  CK(cudaGetLastError(), "pips");
  CK(cudaMemcpyAsync(out4, ctx->a.pips, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream), "pips");
  CK(cudaStreamSynchronize(ctx->stream), "pips");
  return GBSPH_OK;
}

int gbsph_mark(gbsph_ctx* ctx, unsigned slot) {
  if (!ctx || slot >= 16) return GBSPH_EINVAL;
  if (!ctx->marks[slot]) CK(cudaEventCreate(&ctx->marks[slot]), "event");
  CK(cudaEventRecord(ctx->marks[slot], ctx->stream), "record");
  return GBSPH_OK;
}

int gbsph_elapsed(gbsph_ctx* ctx, unsigned a, unsigned b, float* ms) {
  if (!ctx || a >= 16 || b >= 16 || !ctx->marks[a] || !ctx->marks[b] || !ms) return GBSPH_EINVAL;
  CK(cudaEventSynchronize(ctx->marks[b]), "sync");
  CK(cudaEventElapsedTime(ms, ctx->marks[a], ctx->marks[b]), "elapsed");
  return GBSPH_OK;
}

int gbsph_set_step_state(gbsph_ctx* ctx, double time, double dtpre) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (!(time >= 0) || !(dtpre >= 0) || std::isinf(time) || std::isinf(dtpre))
    return set_err(ctx, GBSPH_EINVAL, "invalid restart time %g or dt %g", time, dtpre);
  CK(cudaSetDevice(ctx->device), "set device");
  StepState st;
  CK(cudaMemcpyAsync(&st, ctx->a.st, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream), "step state");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  st.time = time;
  if (dtpre > 0) st.dtpre = dtpre;
  CK(cudaMemcpyAsync(ctx->a.st, &st, sizeof(st), cudaMemcpyHostToDevice, ctx->stream), "step state");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return GBSPH_OK;
}

int gbsph_step_dt(gbsph_ctx* ctx, double* dt_last, double* dt_next, double* time) {
  if (!ctx) return GBSPH_EINVAL;
  StepState st;
  CK(cudaMemcpyAsync(&st, ctx->a.st, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream), "step state");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  if (dt_last) *dt_last = st.dt_last;
  if (dt_next) *dt_next = st.dtpre;
  if (time) *time = st.time;
  return check_device_errors(ctx);
}

int gbsph_sync(gbsph_ctx* ctx) {
  if (!ctx) return GBSPH_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return check_device_errors(ctx);
}

static int read_div(gbsph_ctx* ctx, DivState* ds) {
  CK(cudaMemcpyAsync(ds, ctx->a.div, sizeof(DivState), cudaMemcpyDeviceToHost, ctx->stream), "div");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return GBSPH_OK;
}

int gbsph_download(gbsph_ctx* ctx, double* pos, float* velrho, unsigned* idp, uint16_t* code, unsigned* dcell) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  DivState ds;
  if (int rc = read_div(ctx, &ds)) return rc;
  const unsigned np = ds.np;
  if (pos) {
    // interleave on the device into the alternate position arrays (free between divides)
    double* stage = ctx->a.px2;
    gbk::stage_download(ctx->a, stage, np, ctx->stream);
    CK(cudaGetLastError(), "download");
    CK(cudaMemcpyAsync(pos, stage, sizeof(double) * 3 * (size_t)np, cudaMemcpyDeviceToHost, ctx->stream), "pos");
  }
  if (velrho) CK(cudaMemcpyAsync(velrho, ctx->a.velrho, sizeof(float4) * np, cudaMemcpyDeviceToHost, ctx->stream), "velrho");
  if (idp) CK(cudaMemcpyAsync(idp, ctx->a.idp, sizeof(unsigned) * np, cudaMemcpyDeviceToHost, ctx->stream), "idp");
  if (code) CK(cudaMemcpyAsync(code, ctx->a.code, sizeof(uint16_t) * np, cudaMemcpyDeviceToHost, ctx->stream), "code");
  if (dcell) CK(cudaMemcpyAsync(dcell, ctx->a.dcell, sizeof(unsigned) * np, cudaMemcpyDeviceToHost, ctx->stream), "dcell");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return check_device_errors(ctx);
}

int gbsph_get_forces(gbsph_ctx* ctx, float* ace, float* ar) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  DivState ds;
  if (int rc = read_div(ctx, &ds)) return rc;
  std::vector<float4> h(ds.np);
  CK(cudaMemcpyAsync(h.data(), ctx->a.acear, sizeof(float4) * ds.np, cudaMemcpyDeviceToHost, ctx->stream), "acear");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  for (unsigned p = 0; p < ds.np; p++) {
    if (ace) { ace[3 * (size_t)p] = h[p].x; ace[3 * (size_t)p + 1] = h[p].y; ace[3 * (size_t)p + 2] = h[p].z; }
    if (ar) ar[p] = h[p].w;
  }
  return GBSPH_OK;
}

int gbsph_get_divinfo(gbsph_ctx* ctx, gbsph_divinfo* info, unsigned* begincell, unsigned begincell_cap,
                      unsigned* sortpart, unsigned* cellpart) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  DivState ds;
  if (int rc = read_div(ctx, &ds)) return rc;
  if (info) {
    info->np = ds.np; info->npb = ds.npb; info->npbok = ds.npbok; info->nout_total = ds.nout_total;
    for (int k = 0; k < 3; k++) info->cellmin[k] = ds.cellmin[k];
    info->ncells[0] = ds.ncx; info->ncells[1] = ds.ncy; info->ncells[2] = ds.ncz;
    info->nct = ds.nct; info->nctt = ds.nctt; info->dividefull = ds.dividefull;
    info->npfout = ds.npfout; info->npbout = ds.npbout;
  }
  if (begincell) {
    const unsigned n = begincell_cap < ds.nctt ? begincell_cap : ds.nctt;
    CK(cudaMemcpyAsync(begincell, ctx->a.begincell, sizeof(unsigned) * n, cudaMemcpyDeviceToHost, ctx->stream), "bc");
  }
  if (sortpart) CK(cudaMemcpyAsync(sortpart, ctx->a.vals, sizeof(unsigned) * ds.nptot, cudaMemcpyDeviceToHost, ctx->stream), "sp");
  if (cellpart) CK(cudaMemcpyAsync(cellpart, ctx->a.keys, sizeof(unsigned) * ds.nptot, cudaMemcpyDeviceToHost, ctx->stream), "cp");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return GBSPH_OK;
}

// ---- gauges -------------------------------------------------------------------
// The inputs are packed on the host into one staging block, copied in one
// transfer, measured by one launch and the results copied back.
static int gauge_begin(gbsph_ctx* ctx, unsigned n, size_t bytes, bool args_ok) {
  if (!ctx) return GBSPH_EINVAL;
  if (!args_ok) return set_err(ctx, GBSPH_EINVAL, "null gauge argument");
  if (!ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (n > (1u << 26)) return set_err(ctx, GBSPH_EINVAL, "too many gauges (%u)", n);
  CK(cudaSetDevice(ctx->device), "set device");
  if (bytes > ctx->gauge_bytes) {
    CK(cudaStreamSynchronize(ctx->stream), "gauge sync");
    if (ctx->gauge_buf) cudaFree(ctx->gauge_buf);
    ctx->gauge_buf = nullptr;
    ctx->gauge_bytes = 0;
    const size_t want = bytes < 4096 ? 4096 : bytes;
    if (cudaMalloc(&ctx->gauge_buf, want) != cudaSuccess) {
      cudaGetLastError();
      return set_err(ctx, GBSPH_ENOMEM, "gauge scratch of %zu bytes", want);
    }
    ctx->gauge_bytes = want;
  }
  return GBSPH_OK;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int gbsph_gauge_velocity(gbsph_ctx* ctx, unsigned n, const double* points, float* vel) {
  const size_t ob = align256(sizeof(double) * 3 * (size_t)n);
  if (int rc = gauge_begin(ctx, n, ob + sizeof(float) * 3 * (size_t)n, n == 0 || (points && vel))) return rc;
  if (!n) return GBSPH_OK;
  char* buf = (char*)ctx->gauge_buf;
  CK(cudaMemcpyAsync(buf, points, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream), "gauge in");
  gbk::gauge_velocity(ctx->c, ctx->a, n, (const double*)buf, (float*)(buf + ob), ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "gauge velocity");
  CK(cudaMemcpyAsync(vel, buf + ob, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  CK(cudaStreamSynchronize(ctx->stream), "gauge sync");
  return GBSPH_OK;
}

int gbsph_gauge_swl(gbsph_ctx* ctx, unsigned n, const double* p0p2, const double* pointdp, const float* masslimit,
                    float* surf) {
  const size_t o1 = align256(sizeof(double) * 6 * (size_t)n);
  const size_t o2 = o1 + align256(sizeof(unsigned) * (size_t)n);
  const size_t o3 = o2 + align256(sizeof(float) * (size_t)n);
  if (int rc = gauge_begin(ctx, n, o3 + sizeof(float) * 3 * (size_t)n,
                           n == 0 || (p0p2 && pointdp && masslimit && surf)))
    return rc;
  if (!n) return GBSPH_OK;
  std::vector<char> host(o3);
  double* par = (double*)host.data();
  unsigned* npts = (unsigned*)(host.data() + o1);
  float* mlim = (float*)(host.data() + o2);
  for (unsigned i = 0; i < n; i++) {
    // JGaugeSwl::SetPoints (JDsGaugeItem.cpp:614-641): PointNp steps of PointDir
    const double* q = p0p2 + 6 * (size_t)i;
    const double vx = q[0] - q[3], vy = q[1] - q[4], vz = q[2] - q[5];
    const double dis = std::sqrt(vx * vx + vy * vy + vz * vz);
    const double pdp = pointdp[i];
    unsigned np = 0;
    double dx = 0, dy = 0, dz = 0;
    if (dis > 0 && pdp > 0) {
      if (!(dis / pdp < 1048576.0)) return set_err(ctx, GBSPH_EINVAL, "SWL gauge %u: too many points", i);
      np = (unsigned)(dis / pdp);
      if (dis - (pdp * np) >= pdp * 0.1) np++;
      if (np < 1) np++;
      const double dp = dis / np;
      double ux = q[3] - q[0], uy = q[4] - q[1], uz = q[5] - q[2];
      const double m = std::sqrt(ux * ux + uy * uy + uz * uz);
      if (m) {
        ux = ux / m;
        uy = uy / m;
        uz = uz / m;
      }
      dx = ux * dp;
      dy = uy * dp;
      dz = uz * dp;
    }
    double* pr = par + 6 * (size_t)i;
    pr[0] = q[0]; pr[1] = q[1]; pr[2] = q[2];
    pr[3] = dx; pr[4] = dy; pr[5] = dz;
    npts[i] = np;
    // JGaugeSystem::AddGaugeSwl (JDsGaugeSystem.cpp:408): the default limit
    mlim[i] = masslimit[i] > 0 ? masslimit[i] : ctx->c.massfluid * (ctx->c.simulate2d ? 0.4f : 0.5f);
  }
  char* buf = (char*)ctx->gauge_buf;
  CK(cudaMemcpyAsync(buf, host.data(), o3, cudaMemcpyHostToDevice, ctx->stream), "gauge in");
  gbk::gauge_swl(ctx->c, ctx->a, n, (const double*)buf, (const unsigned*)(buf + o1), (const float*)(buf + o2),
                 (float*)(buf + o3), ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "gauge swl");
  CK(cudaMemcpyAsync(surf, buf + o3, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  // the staging vector is read by the copy above before it goes out of scope
  CK(cudaStreamSynchronize(ctx->stream), "gauge sync");
  return GBSPH_OK;
}

int gbsph_gauge_maxz(gbsph_ctx* ctx, unsigned n, const double* p0h, const float* distlimit, float* zmax) {
  const size_t o1 = align256(sizeof(double) * 4 * (size_t)n);
  const size_t o2 = o1 + align256(sizeof(float) * (size_t)n);
  if (int rc = gauge_begin(ctx, n, o2 + sizeof(float) * (size_t)n, n == 0 || (p0h && distlimit && zmax))) return rc;
  if (!n) return GBSPH_OK;
  char* buf = (char*)ctx->gauge_buf;
  CK(cudaMemcpyAsync(buf, p0h, sizeof(double) * 4 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream), "gauge in");
  CK(cudaMemcpyAsync(buf + o1, distlimit, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream), "gauge in");
  gbk::gauge_maxz(ctx->c, ctx->a, n, (const double*)buf, (const float*)(buf + o1), (float*)(buf + o2), ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "gauge maxz");
  CK(cudaMemcpyAsync(zmax, buf + o2, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  CK(cudaStreamSynchronize(ctx->stream), "gauge sync");
  return GBSPH_OK;
}

// JMeshData::MakeMeshPt (JMeshData.cpp:474-503) with fgeo::VecUnitary.
static bool make_mesh_pts(const gbsph_mesh* mb, GaugeMeshPts* m) {
  memset(m, 0, sizeof(*m));
  unsigned npt[3] = {1, 1, 1};
  const double* vecs[3] = {mb->vec1, mb->vec2, mb->vec3};
  double* vdps[3] = {m->vdp1, m->vdp2, m->vdp3};
  for (int a = 0; a < 3; a++) {
    const double* v = vecs[a];
    const double dis = mb->dis[a], dispt = mb->dispt[a];
    if ((v[0] != 0 || v[1] != 0 || v[2] != 0) && dispt > 0 && dis >= dispt) {
      const double q = (dis + dispt * 0.01) / dispt;
      if (!(q < 67108864.0)) return false;
      const double mod = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      for (int k = 0; k < 3; k++) vdps[a][k] = (v[k] / mod) * dispt;
      npt[a] = (unsigned)q + 1;
    }
  }
  const unsigned long long n = (unsigned long long)npt[0] * npt[1] * npt[2];
  if (n > (1ull << 26)) return false;
  for (int k = 0; k < 3; k++) m->ptref[k] = mb->ptref[k];
  m->npt1 = npt[0];
  m->npt2 = npt[1];
  m->npt3 = npt[2];
  m->npt = (unsigned)n;
  const float* d = mb->dirdat;
  const float mod = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  for (int k = 0; k < 3; k++) m->dirdat[k] = mod ? d[k] / mod : d[k];
  return true;
}

int gbsph_mesh_points(const gbsph_mesh* mesh, unsigned* npt3) {
  GaugeMeshPts m;
  if (!mesh || !npt3 || !make_mesh_pts(mesh, &m)) return GBSPH_EINVAL;
  npt3[0] = m.npt1;
  npt3[1] = m.npt2;
  npt3[2] = m.npt3;
  return GBSPH_OK;
}

int gbsph_gauge_mesh(gbsph_ctx* ctx, const gbsph_mesh* mesh, float kclimit, float kcdummy, float masslimit,
                     float* vel, float* veldir, float* rhop, float* mass, float* zsurf) {
  GaugeMeshPts m;
  if (!ctx) return GBSPH_EINVAL;
  if (!mesh || !make_mesh_pts(mesh, &m)) return set_err(ctx, GBSPH_EINVAL, "invalid mesh (more than 2^26 points?)");
  const size_t n = m.npt, n12 = (size_t)m.npt1 * m.npt2;
  const size_t ov = 0, od = align256(12 * n), orh = od + align256(4 * n), om = orh + align256(4 * n),
               oz = om + align256(4 * n), total = oz + 4 * n12;
  if (int rc = gauge_begin(ctx, 0, total, true)) return rc;
  char* buf = (char*)ctx->gauge_buf;
  const float ml = masslimit > 0 ? masslimit : ctx->c.massfluid * (ctx->c.simulate2d ? 0.4f : 0.5f);
  gbk::gauge_mesh(ctx->c, ctx->a, m, kclimit, kcdummy, ml, vel ? (float*)(buf + ov) : nullptr,
                  veldir ? (float*)(buf + od) : nullptr, rhop ? (float*)(buf + orh) : nullptr, (float*)(buf + om),
                  zsurf ? (float*)(buf + oz) : nullptr, ctx->stream);
  ctx->launches += zsurf ? 2 : 1;
  CK(cudaGetLastError(), "gauge mesh");
  if (vel) CK(cudaMemcpyAsync(vel, buf + ov, 12 * n, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  if (veldir) CK(cudaMemcpyAsync(veldir, buf + od, 4 * n, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  if (rhop) CK(cudaMemcpyAsync(rhop, buf + orh, 4 * n, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  if (mass) CK(cudaMemcpyAsync(mass, buf + om, 4 * n, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  if (zsurf) CK(cudaMemcpyAsync(zsurf, buf + oz, 4 * n12, cudaMemcpyDeviceToHost, ctx->stream), "gauge out");
  CK(cudaStreamSynchronize(ctx->stream), "gauge sync");
  return GBSPH_OK;
}

int gbsph_fluid_front(gbsph_ctx* ctx, const double* dir, const double* bmin, const double* bmax, double* front,
                      unsigned* count) {
  if (int rc = gauge_begin(ctx, 0, 16, dir && bmin && bmax && front)) return rc;
  unsigned long long* key = (unsigned long long*)ctx->gauge_buf;
  unsigned* cnt = (unsigned*)(key + 1);
  CK(cudaMemsetAsync(ctx->gauge_buf, 0, 16, ctx->stream), "front init");
  int nsm = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device), "attribute");
  gbk::fluid_front(ctx->a, dir, bmin, bmax, key, cnt, nsm, ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "fluid front");
  unsigned long long hk[2];
  CK(cudaMemcpyAsync(hk, ctx->gauge_buf, 16, cudaMemcpyDeviceToHost, ctx->stream), "front out");
  CK(cudaStreamSynchronize(ctx->stream), "front sync");
  const unsigned n = (unsigned)(hk[1] & 0xffffffffu);
  if (count) *count = n;
  if (!n) {
    *front = -HUGE_VAL;
  } else {
    const unsigned long long b = (hk[0] >> 63) ? (hk[0] & 0x7fffffffffffffffull) : ~hk[0];
    memcpy(front, &b, sizeof(double));
  }
  return GBSPH_OK;
}

unsigned long long gbsph_launch_count(const gbsph_ctx* ctx) { return ctx ? ctx->launches : 0; }

void* gbsph_stream(gbsph_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int gbsph_set_option(gbsph_ctx* ctx, int key, int value) {
  if (!ctx) return GBSPH_EINVAL;
  if (key == 0) ctx->forces_bsize = value;
  else if (key == 1) {
    if (value < 0 || value > 3) return set_err(ctx, GBSPH_EINVAL, "fluid-row kernel variant %d is not 0..3", value);
    ctx->forces_variant = value;
  }
  else if (key == 2) {
    if (value != 8 && value != 11) return set_err(ctx, GBSPH_EINVAL, "sort digits of 8 or 11 bits");
    ctx->sort_bits = value;
  }
  else if (key == 3) {
    if (value != 0 && value != 1) return set_err(ctx, GBSPH_EINVAL, "mDBC kernel variant %d is not 0 or 1", value);
    ctx->mdbc_variant = value;
  }
  else if (key == 4) {
    if (value != 0 && value != 1 && value != 2 && value != 4)
      return set_err(ctx, GBSPH_EINVAL, "warps per row group %d is not 0 (automatic), 1, 2 or 4", value);
    ctx->forces_split = value;
  }
  else if (key == 6) {
    if (value != 0 && value != 1 && value != 4 && value != 32)
      return set_err(ctx, GBSPH_EINVAL, "lanes per boundary row %d is not 0 (automatic), 1, 4 or 32", value);
    ctx->bound_lanes = value;
  }
  else if (key == 8) {
    if (value != 0 && value != 1 && value != 2 && value != 4)
      return set_err(ctx, GBSPH_EINVAL, "warps per mDBC row group %d is not 0 (automatic), 1, 2 or 4", value);
    ctx->mdbc_split = value;
  }
  else if (key == 10) {
    if (value != 0 && value != 1) return set_err(ctx, GBSPH_EINVAL, "bound rows beside the fluid rows: 0 or 1");
    ctx->bound_beside = value != 0;
  }
  else return set_err(ctx, GBSPH_EINVAL, "unknown option %d", key);
  reset_graph(ctx);
  return GBSPH_OK;
}

int gbsph_get_option(const gbsph_ctx* ctx, int key, int* value) {
  if (!ctx || !value) return GBSPH_EINVAL;
  if (key == 0) *value = ctx->forces_bsize;
  else if (key == 1) *value = ctx->forces_variant;
  else if (key == 2) *value = ctx->sort_bits;
  else if (key == 3) *value = ctx->mdbc_variant;
  else if (key == 4) *value = ctx->forces_split;
  else if (key == 5) *value = forces_split(ctx);
  else if (key == 6) *value = ctx->bound_lanes;
  else if (key == 7) *value = bound_lanes(ctx);
  else if (key == 8) *value = ctx->mdbc_split;
  else if (key == 9) *value = mdbc_split(ctx);
  else if (key == 10) *value = ctx->bound_beside ? 1 : 0;
  else return GBSPH_EINVAL;
  return GBSPH_OK;
}

// Times `reps` cell divisions of the current state with each digit width of
// the radix sort (8 and 11 bits: 11 takes fewer passes for keys of 12 to 22
// bits, with 8x larger histograms) and keeps the faster.  A division of a
// divided state gives the same particle order, except for periodic copies,
// which are made anew.
int gbsph_tune_sort(gbsph_ctx* ctx, int reps, int* best_bits, float* ms) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (reps < 1) reps = 1;
  CK(cudaSetDevice(ctx->device), "set device");
  reset_graph(ctx);
  const int cand[2] = {8, 11};
  float t[2] = {0, 0};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  int rc = GBSPH_OK;
  for (int k = 0; k < 2 && !rc; k++) {
    ctx->sort_bits = cand[k];
    rc = do_divide(ctx);  // warm-up
    cudaEventRecord(e0, ctx->stream);
    for (int i = 0; i < reps && !rc; i++) rc = do_divide(ctx);
    cudaEventRecord(e1, ctx->stream);
    if (!rc) {
      cudaError_t e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t[k], e0, e1);
      if (e != cudaSuccess) rc = cuda_check(ctx, e, "tune sort");
    }
    t[k] /= (float)reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  ctx->sort_bits = t[1] < t[0] ? 11 : 8;
  if (best_bits) *best_bits = ctx->sort_bits;
  if (ms) { ms[0] = t[0]; ms[1] = t[1]; }
  return check_device_errors(ctx);
}

// ---- autotuner ------------------------------------------------------------
// Times the fluid-row kernel configurations on the context's current state
// (between steps) and keeps the fastest: the cell-tiled staged kernel with a
// ring of 8 chunks at 1, 2 and 4 warps per row group and with a ring of 4
// chunks, the warp-queued rounds kernel, and the one-thread-per-row kernel at
// 64, 128 and 256 threads per block.  Then, with that configuration, the
// lanes a boundary row of the bound-row pass (1, 4, 32) and, for mDBC, the
// warps per row group of the staged mDBC kernel (1, 2, 4).  The
// launches only rewrite the interaction outputs, which the next step
// recomputes.
int gbsph_tune_forces(gbsph_ctx* ctx, int reps, gbsph_tune_result* out) {
  if (!ctx || !ctx->uploaded) return set_err(ctx, GBSPH_ESTATE, "no particles uploaded");
  if (reps < 1) reps = 1;
  CK(cudaSetDevice(ctx->device), "set device");
  // variant, block size, warps per row group
  static const int cand[GBSPH_TUNE_CANDIDATES][3] = {{2, 128, 1}, {2, 128, 2}, {2, 128, 4}, {3, 128, 1},
                                                     {0, 128, 1}, {1, 64, 1},  {1, 128, 1}, {1, 256, 1}};
  static const int lanes[3] = {1, 4, 32}, msplits[3] = {1, 2, 4};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  // mean time of `reps` calls of f after one warm-up call
  auto timed = [&](auto&& f, float* ms) -> int {
    f();
    cudaEventRecord(e0, ctx->stream);
    for (int i = 0; i < reps; i++) f();
    cudaEventRecord(e1, ctx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    *ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    if (e != cudaSuccess) return cuda_check(ctx, e, "tune");
    *ms /= (float)reps;
    return GBSPH_OK;
  };
  int rc = GBSPH_OK;
  gbsph_tune_result r{};
  // the fluid-row configuration, with the bound-row lanes of the current choice
  int best = 0;
  const int bl0 = bound_lanes(ctx);
  for (int k = 0; k < GBSPH_TUNE_CANDIDATES && !rc; k++) {
    const int var = cand[k][0], bs = cand[k][1], sp = cand[k][2];
    rc = timed([&] { gbk::forces(ctx->c, ctx->a, ctx->cap, bs, var, sp, bl0, ctx->stream, nullptr, nullptr, nullptr); },
               &r.ms[k]);
    r.variant[k] = var;
    r.bsize[k] = bs;
    r.split[k] = sp;
    if (r.ms[k] < r.ms[best]) best = k;
  }
  // then the lanes a boundary row, with that fluid-row configuration
  int bbest = 0;
  for (int k = 0; k < 3 && !rc; k++) {
    rc = timed([&] {
      gbk::forces(ctx->c, ctx->a, ctx->cap, cand[best][1], cand[best][0], cand[best][2], lanes[k], ctx->stream, nullptr,
                  nullptr, nullptr);
    }, &r.bound_ms[k]);
    r.bound_lanes[k] = lanes[k];
    if (r.bound_ms[k] < r.bound_ms[bbest]) bbest = k;
  }
  // and the warps per mDBC row group (the correction rewrites the boundary
  // densities from the fluid's, the same values every time)
  int mbest = 0;
  const bool mdbc = ctx->c.tboundary == GBSPH_BC_MDBC && ctx->mdbc_variant == 0;
  for (int k = 0; k < 3 && !rc; k++) {
    r.mdbc_split[k] = msplits[k];
    if (!mdbc) continue;
    rc = timed([&] { gbk::mdbc(ctx->c, ctx->a, ctx->cap, 0, msplits[k], ctx->stream, nullptr); }, &r.mdbc_ms[k]);
    if (r.mdbc_ms[k] < r.mdbc_ms[mbest]) mbest = k;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  r.best = best;
  r.bound_best = bbest;
  r.mdbc_best = mdbc ? mbest : -1;
  ctx->forces_variant = cand[best][0];
  ctx->forces_bsize = cand[best][1];
  ctx->forces_split = cand[best][2];
  ctx->bound_lanes = lanes[bbest];
  if (mdbc) ctx->mdbc_split = msplits[mbest];
  reset_graph(ctx);
  if (out) *out = r;
  return check_device_errors(ctx);
}

}  // extern "C"

// ---- ensembles --------------------------------------------------------------
// Independent cases on one device advanced together: every case keeps its own
// arrays, stream and adaptive dt; one step of all of them is captured as one
// CUDA graph whose branches (one per case) run concurrently, and the graph is
// replayed.  Moving cases have their motions advanced on the host between
// replays (one read-back of all their step states, one upload each).
struct gbsph_ensemble {
  std::vector<gbsph_ctx*> cases;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<cudaEvent_t> ev;        // [0] fork/done, [1+i] case i
  cudaGraphExec_t exec = nullptr;
  std::vector<unsigned> parity;       // each case's pointer parity at capture
  std::vector<unsigned long long> nl; // each case's launches per captured step
  std::string err;
};

namespace {

int ens_err(gbsph_ensemble* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  return code;
}

int ens_cuda(gbsph_ensemble* e, cudaError_t c, const char* what) {
  if (c != cudaSuccess) return ens_err(e, GBSPH_ECUDA, std::string(what) + ": " + cudaGetErrorString(c));
  return GBSPH_OK;
}

// prior work on every case stream before the ensemble stream's next work
int ens_order_in(gbsph_ensemble* e) {
  for (size_t i = 0; i < e->cases.size(); i++) {
    if (int rc = ens_cuda(e, cudaEventRecord(e->ev[1 + i], e->cases[i]->stream), "order")) return rc;
    if (int rc = ens_cuda(e, cudaStreamWaitEvent(e->stream, e->ev[1 + i], 0), "order")) return rc;
  }
  return GBSPH_OK;
}

// the ensemble's work before later work on every case stream
int ens_order_out(gbsph_ensemble* e) {
  if (int rc = ens_cuda(e, cudaEventRecord(e->ev[0], e->stream), "order")) return rc;
  for (gbsph_ctx* c : e->cases)
    if (int rc = ens_cuda(e, cudaStreamWaitEvent(c->stream, e->ev[0], 0), "order")) return rc;
  return GBSPH_OK;
}

// RunMotion input of every moving case for the coming step
int ens_motion(gbsph_ensemble* e) {
  std::vector<StepState> st(e->cases.size());
  bool any = false;
  for (size_t i = 0; i < e->cases.size(); i++) {
    gbsph_ctx* c = e->cases[i];
    if (!c->motion) continue;
    any = true;
    if (int rc = ens_cuda(e, cudaMemcpyAsync(&st[i], c->a.st, sizeof(StepState), cudaMemcpyDeviceToHost, e->stream),
                          "motion dt"))
      return rc;
  }
  if (!any) return GBSPH_OK;
  if (int rc = ens_cuda(e, cudaStreamSynchronize(e->stream), "motion sync")) return rc;
  for (size_t i = 0; i < e->cases.size(); i++) {
    gbsph_ctx* c = e->cases[i];
    if (!c->motion) continue;
    if (int rc = motion_table(c, st[i], e->stream)) return ens_err(e, rc, "case " + std::to_string(i) + ": " + c->err);
  }
  return GBSPH_OK;
}

int ens_capture(gbsph_ensemble* e) {
  if (e->exec) cudaGraphExecDestroy(e->exec);
  e->exec = nullptr;
  const size_t n = e->cases.size();
  std::vector<DevArrays> a0(n);
  std::vector<unsigned> s0(n);
  std::vector<unsigned long long> l0(n);
  e->parity.assign(n, 0);
  e->nl.assign(n, 0);
  if (int rc = ens_cuda(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal), "capture")) return rc;
  cudaEventRecord(e->ev[0], e->stream);
  int rc = GBSPH_OK;
  size_t ncap = 0;  // cases whose host state was saved
  for (size_t i = 0; i < n && !rc; i++) {
    gbsph_ctx* c = e->cases[i];
    a0[i] = c->a; s0[i] = c->swaps; l0[i] = c->launches;
    ncap = i + 1;
    e->parity[i] = c->swaps & 1u;
    cudaStreamWaitEvent(c->stream, e->ev[0], 0);
    rc = enqueue_step(c);
    if (rc) rc = ens_err(e, rc, "case " + std::to_string(i) + ": " + c->err);
    cudaEventRecord(e->ev[1 + i], c->stream);
    cudaStreamWaitEvent(e->stream, e->ev[1 + i], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
  // the capture recorded the work without running it: restore the pointer state
  for (size_t i = 0; i < ncap; i++) {
    gbsph_ctx* c = e->cases[i];
    e->nl[i] = c->launches - l0[i];
    c->a = a0[i]; c->swaps = s0[i]; c->launches = l0[i];
  }
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  if (int r2 = ens_cuda(e, ce, "end capture")) return r2;
  const cudaError_t ie = cudaGraphInstantiate(&e->exec, g, 0);
  cudaGraphDestroy(g);
  return ens_cuda(e, ie, "instantiate");
}

}  // namespace

extern "C" {

int gbsph_ensemble_create(unsigned n, gbsph_ctx* const* ctxs, gbsph_ensemble** out) {
  if (!out || !ctxs || n == 0) return GBSPH_EINVAL;
  *out = nullptr;
  for (unsigned i = 0; i < n; i++) {
    if (!ctxs[i] || !ctxs[i]->uploaded) return GBSPH_ESTATE;
    if (ctxs[i]->device != ctxs[0]->device) return GBSPH_EINVAL;
    for (unsigned j = 0; j < i; j++) if (ctxs[j] == ctxs[i]) return GBSPH_EINVAL;
  }
  gbsph_ensemble* e = new gbsph_ensemble();
  e->cases.assign(ctxs, ctxs + n);
  e->device = ctxs[0]->device;
  e->ev.assign(n + 1, nullptr);
  bool ok = cudaSetDevice(e->device) == cudaSuccess &&
            cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) == cudaSuccess;
  for (unsigned i = 0; ok && i <= n; i++) ok = cudaEventCreateWithFlags(&e->ev[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    gbsph_ensemble_destroy(e);
    return GBSPH_ECUDA;
  }
  *out = e;
  return GBSPH_OK;
}

void gbsph_ensemble_destroy(gbsph_ensemble* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->exec) cudaGraphExecDestroy(e->exec);
  for (cudaEvent_t v : e->ev) if (v) cudaEventDestroy(v);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

const char* gbsph_ensemble_last_error(const gbsph_ensemble* e) { return e ? e->err.c_str() : "null ensemble"; }

int gbsph_ensemble_run(gbsph_ensemble* e, unsigned nsteps, int use_graph) {
  if (!e) return GBSPH_EINVAL;
  if (int rc = ens_cuda(e, cudaSetDevice(e->device), "set device")) return rc;
  bool sym = true;
  for (gbsph_ctx* c : e->cases) sym = sym && c->c.tstep == GBSPH_STEP_SYMPLECTIC;
  if (!use_graph || !sym) {
    // every case on its own stream: the streams run concurrently
    for (unsigned k = 0; k < nsteps; k++)
      for (size_t i = 0; i < e->cases.size(); i++) {
        gbsph_ctx* c = e->cases[i];
        int rc = (c->motion && c->c.tstep == GBSPH_STEP_SYMPLECTIC) ? motion_prepare(c) : GBSPH_OK;
        if (!rc) rc = enqueue_step(c);
        if (rc) return ens_err(e, rc, "case " + std::to_string(i) + ": " + c->err);
      }
    for (size_t i = 0; i < e->cases.size(); i++)
      if (int rc = ens_cuda(e, cudaGetLastError(), "run")) return rc;
    return GBSPH_OK;
  }
  bool valid = e->exec != nullptr;
  for (size_t i = 0; valid && i < e->cases.size(); i++) valid = (e->cases[i]->swaps & 1u) == e->parity[i];
  if (!valid)
    if (int rc = ens_capture(e)) return rc;
  if (int rc = ens_order_in(e)) return rc;
  for (unsigned k = 0; k < nsteps; k++) {
    if (int rc = ens_motion(e)) return rc;
    if (int rc = ens_cuda(e, cudaGraphLaunch(e->exec, e->stream), "graph launch")) return rc;
    for (size_t i = 0; i < e->cases.size(); i++) {
      e->cases[i]->swaps += 2;  // two divides per Symplectic step: parity unchanged
      e->cases[i]->launches += e->nl[i];
    }
  }
  return ens_order_out(e);
}

int gbsph_ensemble_sync(gbsph_ensemble* e) {
  if (!e) return GBSPH_EINVAL;
  if (int rc = ens_cuda(e, cudaStreamSynchronize(e->stream), "sync")) return rc;
  for (size_t i = 0; i < e->cases.size(); i++) {
    gbsph_ctx* c = e->cases[i];
    if (int rc = ens_cuda(e, cudaStreamSynchronize(c->stream), "sync")) return rc;
    if (int rc = check_device_errors(c)) return ens_err(e, rc, "case " + std::to_string(i) + ": " + c->err);
  }
  return GBSPH_OK;
}

unsigned long long gbsph_ensemble_launches_per_step(const gbsph_ensemble* e) {
  unsigned long long n = 0;
  if (e) for (unsigned long long v : e->nl) n += v;
  return n;
}

// ---- learned closure ----------------------------------------------------------
static int closure_alloc(gbsph_ctx* ctx) {
  if (ctx->clos_feat) return GBSPH_OK;
  CK(gbk::closure_init(), "closure init");
  if (cudaMalloc(&ctx->clos_feat, sizeof(float) * GBSPH_CLOSURE_FEATURES * (size_t)ctx->cap) != cudaSuccess ||
      cudaMalloc(&ctx->clos_w, sizeof(uint16_t) * GBSPH_CLOSURE_PARAMS) != cudaSuccess ||
      cudaMalloc(&ctx->clos_nfb, sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, GBSPH_ENOMEM, "closure buffers");
  }
  CK(cudaMemsetAsync(ctx->clos_nfb, 0, sizeof(unsigned), ctx->stream), "closure");
  return GBSPH_OK;
}

int gbsph_closure_set(gbsph_ctx* ctx, const uint16_t* w_bf16, float limit) {
  if (!ctx) return GBSPH_EINVAL;
  CK(cudaSetDevice(ctx->device), "set device");
  reset_graph(ctx);
  if (!w_bf16) {
    ctx->clos_on = false;
    return GBSPH_OK;
  }
  if (!(limit >= 0)) return set_err(ctx, GBSPH_EINVAL, "closure limit must be >= 0");
  if (int rc = closure_alloc(ctx)) return rc;
  CK(cudaMemcpyAsync(ctx->clos_w, w_bf16, sizeof(uint16_t) * GBSPH_CLOSURE_PARAMS, cudaMemcpyHostToDevice,
                     ctx->stream), "closure weights");
  CK(cudaStreamSynchronize(ctx->stream), "closure weights");
  ctx->clos_limit = limit;
  ctx->clos_on = true;
  return GBSPH_OK;
}

int gbsph_closure_features(gbsph_ctx* ctx, float* out) {
  if (!ctx || !ctx->uploaded || !out) return set_err(ctx, GBSPH_EINVAL, "closure_features");
  CK(cudaSetDevice(ctx->device), "set device");
  if (int rc = closure_alloc(ctx)) return rc;
  DivState ds;
  CK(cudaMemcpyAsync(&ds, ctx->a.div, sizeof(ds), cudaMemcpyDeviceToHost, ctx->stream), "div");
  gbk::closure_features(ctx->c, ctx->a, ctx->cap, ctx->clos_feat, ctx->stream, &ctx->launches);
  CK(cudaStreamSynchronize(ctx->stream), "features");
  CK(cudaMemcpy(out, ctx->clos_feat, sizeof(float) * GBSPH_CLOSURE_FEATURES * (size_t)(ds.np - ds.npb),
                cudaMemcpyDeviceToHost), "features");
  return check_device_errors(ctx);
}

int gbsph_closure_fallbacks(gbsph_ctx* ctx, unsigned long long* n) {
  if (!ctx || !n) return GBSPH_EINVAL;
  unsigned v = 0;
  if (ctx->clos_nfb) {
    CK(cudaMemcpyAsync(&v, ctx->clos_nfb, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream), "fallbacks");
    CK(cudaStreamSynchronize(ctx->stream), "fallbacks");
  }
  *n = v;
  return GBSPH_OK;
}

}  // extern "C"

// Trainer: device copies of the data, FP32 master weights with their BF16
// copy, Adam moments, the gradient and per-epoch losses.
struct gbsph_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float* master = nullptr;   // GBSPH_CLOSURE_PARAMS
  void* w = nullptr;         // BF16 copy
  float *grad = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
  unsigned nloss = 0;
  float *x = nullptr, *t = nullptr;
  unsigned n = 0;
  unsigned long long adam_t = 0;
};

extern "C" {

int gbsph_mlp_create(int device, const float* params, gbsph_mlp** out) {
  if (!params || !out) return GBSPH_EINVAL;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return GBSPH_ECUDA;
  if (gbk::closure_init() != cudaSuccess) return GBSPH_ECUDA;
  gbsph_mlp* m = new gbsph_mlp();
  m->device = device;
  const size_t P = GBSPH_CLOSURE_PARAMS;
  bool ok = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&m->master, 4 * P) == cudaSuccess && cudaMalloc(&m->w, 2 * P) == cudaSuccess &&
            cudaMalloc(&m->grad, 4 * P) == cudaSuccess && cudaMalloc(&m->m, 4 * P) == cudaSuccess &&
            cudaMalloc(&m->v, 4 * P) == cudaSuccess;
  if (ok) {
    ok = cudaMemcpy(m->master, params, 4 * P, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(m->grad, 0, 4 * P) == cudaSuccess && cudaMemset(m->m, 0, 4 * P) == cudaSuccess &&
         cudaMemset(m->v, 0, 4 * P) == cudaSuccess;
    if (ok) gbk::to_bf16(m->master, m->w, (int)P, m->stream);
    ok = ok && cudaStreamSynchronize(m->stream) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    gbsph_mlp_destroy(m);
    return GBSPH_ENOMEM;
  }
  *out = m;
  return GBSPH_OK;
}

void gbsph_mlp_destroy(gbsph_mlp* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  void* bufs[] = {m->master, m->w, m->grad, m->m, m->v, m->loss, m->x, m->t};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

int gbsph_mlp_set_data(gbsph_mlp* m, const float* x, const float* t, unsigned n) {
  if (!m || !x || !t || !n) return GBSPH_EINVAL;
  if (cudaSetDevice(m->device) != cudaSuccess) return GBSPH_ECUDA;
  cudaStreamSynchronize(m->stream);
  if (m->x) cudaFree(m->x);
  if (m->t) cudaFree(m->t);
  m->x = m->t = nullptr;
  m->n = 0;
  if (cudaMalloc(&m->x, sizeof(float) * GBSPH_CLOSURE_FEATURES * (size_t)n) != cudaSuccess ||
      cudaMalloc(&m->t, sizeof(float) * 3 * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    return GBSPH_ENOMEM;
  }
  if (cudaMemcpy(m->x, x, sizeof(float) * GBSPH_CLOSURE_FEATURES * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(m->t, t, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess)
    return GBSPH_ECUDA;
  m->n = n;
  return GBSPH_OK;
}

static int mlp_loss_buf(gbsph_mlp* m, unsigned n) {
  if (m->nloss >= n) return GBSPH_OK;
  if (m->loss) cudaFree(m->loss);
  m->loss = nullptr;
  m->nloss = 0;
  if (cudaMalloc(&m->loss, sizeof(float) * n) != cudaSuccess) {
    cudaGetLastError();
    return GBSPH_ENOMEM;
  }
  m->nloss = n;
  return GBSPH_OK;
}

int gbsph_mlp_grad(gbsph_mlp* m, unsigned first, unsigned n, float* grad, float* loss) {
  if (!m || !grad || !n || (unsigned long long)first + n > m->n) return GBSPH_EINVAL;
  if (cudaSetDevice(m->device) != cudaSuccess) return GBSPH_ECUDA;
  if (int rc = mlp_loss_buf(m, 1)) return rc;
  cudaMemsetAsync(m->grad, 0, sizeof(float) * GBSPH_CLOSURE_PARAMS, m->stream);
  cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
  gbk::mlp_grad(m->w, m->x + (size_t)first * GBSPH_CLOSURE_FEATURES, m->t + (size_t)first * 3, n, m->grad, m->loss,
                m->stream);
  if (cudaStreamSynchronize(m->stream) != cudaSuccess) return GBSPH_ECUDA;
  if (cudaMemcpy(grad, m->grad, sizeof(float) * GBSPH_CLOSURE_PARAMS, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GBSPH_ECUDA;
  if (loss && cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return GBSPH_ECUDA;
  cudaMemsetAsync(m->grad, 0, sizeof(float) * GBSPH_CLOSURE_PARAMS, m->stream);
  return cudaStreamSynchronize(m->stream) == cudaSuccess ? GBSPH_OK : GBSPH_ECUDA;
}

int gbsph_mlp_train(gbsph_mlp* m, unsigned epochs, unsigned batch, float lr, float* loss_per_epoch) {
  if (!m || !m->n || !batch || !epochs) return GBSPH_EINVAL;
  if (cudaSetDevice(m->device) != cudaSuccess) return GBSPH_ECUDA;
  if (int rc = mlp_loss_buf(m, epochs)) return rc;
  cudaMemsetAsync(m->loss, 0, sizeof(float) * epochs, m->stream);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const unsigned nb = (m->n + batch - 1) / batch;
  for (unsigned e = 0; e < epochs; e++) {
    for (unsigned b = 0; b < nb; b++) {
      const unsigned first = b * batch, n = std::min(batch, m->n - first);
      gbk::mlp_grad(m->w, m->x + (size_t)first * GBSPH_CLOSURE_FEATURES, m->t + (size_t)first * 3, n, m->grad,
                    m->loss + e, m->stream);
      m->adam_t++;
      const float bc1 = (float)(1.0 - std::pow((double)b1, (double)m->adam_t));
      const float bc2 = (float)(1.0 - std::pow((double)b2, (double)m->adam_t));
      gbk::mlp_adam(m->master, m->w, m->grad, m->m, m->v, lr, b1, b2, eps, bc1, bc2, m->stream);
    }
  }
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(m->stream) != cudaSuccess) return GBSPH_ECUDA;
  if (loss_per_epoch) {
    std::vector<float> l(epochs);
    if (cudaMemcpy(l.data(), m->loss, sizeof(float) * epochs, cudaMemcpyDeviceToHost) != cudaSuccess) return GBSPH_ECUDA;
    for (unsigned e = 0; e < epochs; e++) loss_per_epoch[e] = l[e] / (float)nb;  // mean of the batch losses
  }
  return GBSPH_OK;
}

int gbsph_mlp_infer(gbsph_mlp* m, const float* x, unsigned n, float* y) {
  if (!m || !x || !y) return GBSPH_EINVAL;
  if (!n) return GBSPH_OK;
  if (cudaSetDevice(m->device) != cudaSuccess) return GBSPH_ECUDA;
  float *dx = nullptr, *dy = nullptr;
  if (cudaMalloc(&dx, sizeof(float) * GBSPH_CLOSURE_FEATURES * (size_t)n) != cudaSuccess ||
      cudaMalloc(&dy, sizeof(float) * 3 * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    if (dx) cudaFree(dx);
    return GBSPH_ENOMEM;
  }
  int rc = GBSPH_OK;
  if (cudaMemcpyAsync(dx, x, sizeof(float) * GBSPH_CLOSURE_FEATURES * (size_t)n, cudaMemcpyHostToDevice, m->stream) !=
      cudaSuccess)
    rc = GBSPH_ECUDA;
  if (!rc) {
    gbk::mlp_infer(m->w, dx, n, dy, m->stream);
    if (cudaStreamSynchronize(m->stream) != cudaSuccess ||
        cudaMemcpy(y, dy, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = GBSPH_ECUDA;
  }
  cudaFree(dx);
  cudaFree(dy);
  return rc;
}

int gbsph_mlp_params(gbsph_mlp* m, float* master, uint16_t* w_bf16) {
  if (!m) return GBSPH_EINVAL;
  if (cudaSetDevice(m->device) != cudaSuccess || cudaStreamSynchronize(m->stream) != cudaSuccess) return GBSPH_ECUDA;
  if (master && cudaMemcpy(master, m->master, 4 * GBSPH_CLOSURE_PARAMS, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GBSPH_ECUDA;
  if (w_bf16 && cudaMemcpy(w_bf16, m->w, 2 * GBSPH_CLOSURE_PARAMS, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GBSPH_ECUDA;
  return GBSPH_OK;
}

}  // extern "C"

// ---- FP32 peak ------------------------------------------------------------------
// FFMA microbenchmark for the FP32 roofline denominator: every thread runs 8
// independent fused multiply-add chains; the best of a few timed launches
// gives the issue-limited FP32 rate of the device at its current clock.
namespace {
__global__ void k_ffma_peak(float* out, int iters, float a, float b) {
  float x[8];
  for (int k = 0; k < 8; k++) x[k] = (float)(threadIdx.x + k) * 1e-3f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int r = 0; r < 16; r++) {
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = fmaf(x[k], a, b);
    }
  }
  float s = 0;
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == -1.f) out[blockIdx.x] = s;  // keeps the chains live
}
}  // namespace

extern "C" int gbsph_ffma_peak(int device, float* tflops) {
  if (!tflops) return GBSPH_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return GBSPH_ECUDA;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return GBSPH_ECUDA;
  const int threads = 256, blocks = nsm * 8, iters = 2048;
  float* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks) != cudaSuccess) return GBSPH_ENOMEM;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  k_ffma_peak<<<blocks, threads>>>(out, iters, 0.999999f, 1e-6f);  // warm-up
  for (int rep = 0; rep < 5; rep++) {
    cudaEventRecord(e0);
    k_ffma_peak<<<blocks, threads>>>(out, iters, 0.999999f, 1e-6f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms > 0 && ms < best) best = ms;
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return GBSPH_ECUDA;
  const double flop = 2.0 * 8 * 16 * (double)iters * threads * blocks;
  *tflops = (float)(flop / (best * 1e-3) / 1e12);
  return GBSPH_OK;
}
