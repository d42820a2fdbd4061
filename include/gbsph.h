/*
 * gbsph.h -- C ABI of the GB300-native WCSPH step (libgbsph.so).
 *
 * Drop-in boundary for DualSPHysics' per-step GPU hot path.  Each entry point
 * names the reference interface it replaces (paths relative to the DualSPHysics
 * source tree src/source/).  All functions return a status code (GBSPH_OK=0 or
 * a negative GBSPH_E* value) and never throw across the ABI; the message of the
 * last failure of a context is returned by gbsph_last_error().
 *
 * Threading: one context per host thread; every context owns one CUDA stream.
 * Calls enqueue work on that stream and return without synchronising, except
 * gbsph_download*, gbsph_get_*, gbsph_gauge_*, gbsph_sync and gbsph_step_dt
 * (they read results back).  Host pointers passed in are only used for the duration of the call.
 * All device memory of a context is allocated by gbsph_create/gbsph_upload
 * (and the gauges' scratch by the first gauge call); nothing is allocated by
 * the step functions.
 */
#ifndef GBSPH_H
#define GBSPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (JException/Run_Exceptioon equivalents, JSphGpu.cpp:84-126) */
#define GBSPH_OK 0
#define GBSPH_EINVAL -1      /* invalid argument or configuration                         */
#define GBSPH_ECUDA -2       /* CUDA runtime error                                        */
#define GBSPH_ENAN_DT -3     /* computed dt is NaN or infinite (JSphGpu.cpp:1122-1131)    */
#define GBSPH_EBOUND_OUT -4  /* a boundary particle left the domain (JSph.cpp:2837)       */
#define GBSPH_ECAPACITY -5   /* particles or cells beyond the allocated capacity          */
#define GBSPH_ENOMEM -6      /* device allocation failed                                  */
#define GBSPH_ESTATE -7      /* call out of order (e.g. step before upload)               */

/* options (XML <parameters> keys of the reference, JSph.cpp:663-857) */
#define GBSPH_STEP_VERLET 1
#define GBSPH_STEP_SYMPLECTIC 2
#define GBSPH_VISCO_ARTIFICIAL 1
#define GBSPH_VISCO_LAMINARSPS 2
#define GBSPH_VISCO_LAMINAR 3
#define GBSPH_DDT_NONE 0
#define GBSPH_DDT_DDT 1
#define GBSPH_DDT_DDT2 2
#define GBSPH_DDT_DDT2FULL 3
#define GBSPH_BC_DBC 1
#define GBSPH_BC_MDBC 2

/* interaction step (TpInterStep, DualSphDef.h) */
#define GBSPH_INTERSTEP_VERLET 1
#define GBSPH_INTERSTEP_SYMPREDICTOR 2
#define GBSPH_INTERSTEP_SYMCORRECTOR 3

/* Raw case parameters as carried by the run XML (case.execution.constants and
 * .parameters) plus the resolved real map limits.  Replaces the inputs of
 * JSph::LoadConfigCtes/LoadConfigParameters (JSph.cpp:642-857). */
typedef struct {
  int tstep, tvisco, tdensity, tboundary, verletsteps, dtallparticles, simulate2d, cellmode_div;
  double dp, h, b, rhop0, gamma, massbound, massfluid, cflnumber;
  double gravity[3];
  float visco, viscoboundfactor, ddtvalue, coefdtmin, rhopoutmin, rhopoutmax;
  double dtini, dtmin;
  double maprealposmin[3], maprealposmax[3];
  int tshift;                 /* Shifting: 0 none, 1 NoBound, 2 NoFixed, 3 Full */
  float shiftcoef, shifttfs;  /* ShiftCoef (default -2), ShiftTFS (0: no free-surface threshold) */
  int peri[3];                /* periodic axes x, y, z (JSph.cpp:815-826) */
  double periinc[9];          /* per axis k, its increment (XPeriodicIncY ...); the own component is set by config */
} gbsph_params;

/* Derived constants of a case: the members of JSph / StCteSph the hot path
 * uses (JSph.h:178-365, DualSphDef.h:503-530), same types as the reference. */
typedef struct {
  int tstep, tvisco, tdensity, tboundary, verletsteps, dtallparticles, simulate2d, cellmode_div;
  float kernelh, kernelsize, kernelsize2, cteb, gamma, rhopzero, massfluid, massbound;
  float eta2, ddtkh, ddtgz, visco, viscoboundfactor, awen, bwenh, spssmag, spsblin;
  float scell, movlimit, rhopoutmin, rhopoutmax, gravity[3];
  double dp, cs0, cflnumber, dtmin, dtini;
  double mapposmin[3], maprealposmin[3], maprealsize[3], maprealposmax[3];
  double domposmin[3], domrealposmin[3], domrealposmax[3];
  unsigned mapcells[3], domcells[3], domcellcode;
  int tshift;
  float shiftcoef, shifttfs;
  int peri[3];                /* periodic axes */
  double periinc[9];          /* PeriXinc, PeriYinc, PeriZinc (JSph.cpp:2186-2188) */
  double mapposmax[3];        /* Map_PosMax: MapRealPosMax + KernelSize on periodic axes */
} gbsph_consts;

/* Cell-division summary (JCellDivGpuSingle members, JCellDivGpu.h). */
typedef struct {
  unsigned np, npb, npbok, nout_total;
  unsigned cellmin[3], ncells[3], nct, nctt;
  unsigned dividefull, npfout, npbout;
} gbsph_divinfo;

/* Maxima of the last interaction pass (AceMax, VelMax, ViscDtMax of JSph). */
typedef struct {
  double acemax;
  float velmax, viscdtmax;
} gbsph_maxes;

typedef struct gbsph_ctx gbsph_ctx;

/* Derives the constants: JSph::ConfigConstants1/2 (JSph.cpp:1481-1546),
 * ConfigCellDivision (:1877-1895) and SelecDomain(0,Map_Cells) (:1901-1944). */
int gbsph_config(const gbsph_params* prm, gbsph_consts* out);

/* Creates a context on CUDA device `device` sized for `capacity` particles.
 * Replaces JSphGpuSingle::LoadConfig/ConfigDomain memory setup
 * (JSphGpuSingle.cpp:151-240, JSphGpu.cpp:692-757). */
int gbsph_create(const gbsph_consts* c, unsigned capacity, int device, gbsph_ctx** out);
void gbsph_destroy(gbsph_ctx* ctx);
const char* gbsph_last_error(const gbsph_ctx* ctx);

/* Uploads the initial particle state (ordered as in the case file: boundary
 * first) and performs the first cell division, as JSphGpuSingle::ConfigDomain
 * does (ParticlesDataUp + LoadDcellParticles + RunCellDivide,
 * JSphGpuSingle.cpp:151-240).  pos: 3 doubles per particle; velrho: 4 floats;
 * boundnor: 3 floats per boundary particle (NULL without mDBC), doubled here as
 * JSph::ConfigBoundNormals does (JSph.cpp:1411-1418). */
int gbsph_upload(gbsph_ctx* ctx, unsigned np, unsigned npb, const double* pos, const float* velrho,
                 const unsigned* idp, const uint16_t* code, const float* boundnor);

/* Neighbour-list build: JSphGpuSingle::RunCellDivide (JSphGpuSingle.cpp:372-480)
 * = cudiv::PreSort/Sort/CalcBeginEndCell (JCellDivGpu_ker.cu:120-570,
 * JCellDivGpuSingle_ker.cu:41-165) + SortDataParticles + UpdatePosCell. */
int gbsph_divide(gbsph_ctx* ctx);

/* mDBC ghost-node correction, SlipMode=vel0:
 * cusph::Interaction_MdbcCorrection (JSphGpu_mdbc_iker.cu:194). Runs only for
 * mDBC cases, and only in the predictor (JSphGpuSingle.cpp:686-700). */
int gbsph_mdbc(gbsph_ctx* ctx, int interstep);

/* PreInteraction_Forces + Interaction_Forces: cusph::Interaction_Forces
 * (JSphGpu_ker.h:293, JSphGpu_ker.cu:1169) with the fused max reductions of
 * JSphGpu::PreInteraction_Forces/ComputeAceMax (JSphGpu.cpp:846-900,
 * JSphGpuSingle.cpp:719-729).  `maxes` may be NULL (no read-back). */
int gbsph_forces(gbsph_ctx* ctx, int interstep, gbsph_maxes* maxes);

/* JSphGpu::DtVariable (JSphGpu.cpp:1103-1150). Computes dt on the device from
 * the maxima of the last gbsph_forces call; reads it back into *dt if dt!=NULL. */
int gbsph_dtvariable(gbsph_ctx* ctx, int final, double* dt);

/* Integrators: JSphGpu::ComputeSymplecticPre/Corr (JSphGpu.cpp:996/1054,
 * cusphs::ComputeStepSymplecticPre/Cor JSphGpuSimple_ker.cu:358/518,
 * cusph::ComputeStepPos2 JSphGpu_ker.cu:1553) and JSphGpu::ComputeVerlet. */
int gbsph_symplectic_pre(gbsph_ctx* ctx, double dt);
int gbsph_symplectic_cor(gbsph_ctx* ctx, double dt);
int gbsph_verlet(gbsph_ctx* ctx, double dt);

/* One whole step: JSphGpuSingle::ComputeStep (ComputeStep_Sym/_Ver,
 * JSphGpuSingle.cpp:785-826) followed by RunCellDivide, as one iteration of
 * the Run loop (JSphGpuSingle.cpp:998-1005).  dt stays on the device; nothing
 * is read back. */
int gbsph_step(gbsph_ctx* ctx);
/* Runs `nsteps` steps; use_graph=1 captures one step into a CUDA graph once and
 * replays it nsteps times, use_graph=2 replays a graph holding all nsteps steps
 * (see gbsph_graph_prepare); no host round trips inside the loop. */
int gbsph_run(gbsph_ctx* ctx, unsigned nsteps, int use_graph);
/* Captures `nsteps` Symplectic steps into one CUDA graph (replayed by
 * gbsph_run(ctx, nsteps, 2)); capture records work without running it. */
int gbsph_graph_prepare(gbsph_ctx* ctx, unsigned nsteps);
/* Restart: sets the simulated time (TimeStep) and, for Symplectic, the next
 * SymplecticDtPre (if dtpre > 0) of an uploaded state, as JSph::InitRun does
 * when a run begins from a Part file (JSph.cpp:2214-2225, 2363-2364). */
int gbsph_set_step_state(gbsph_ctx* ctx, double time, double dtpre);
/* Reads back the dt used by the last step and the next SymplecticDtPre. */
int gbsph_step_dt(gbsph_ctx* ctx, double* dt_last, double* dt_next, double* time);

/* Standard shifting (JSphShifting, JSphShifting.cpp:390-418; modes 1-3 in
 * gbsph_consts.tshift): each fluid-row interaction writes the shifting sums
 * (m/rho grad W, and -m/rho r.grad W in w; x = FLT_MAX where a boundary
 * neighbour cancels them); gbsph_run_shifting(dt) turns them into the
 * displacements the next corrector (Symplectic) or Verlet update adds, as
 * RunShifting does.  gbsph_step / gbsph_run do this by themselves.  The
 * reference's predictor computes RunShifting(dt/2) but never applies it
 * (JSphCpu.cpp:1689), so the device step leaves it out.
 * gbsph_get_shiftpos reads the np float4 values (GBSPH_EINVAL without shifting). */
int gbsph_run_shifting(gbsph_ctx* ctx, double dt);
int gbsph_get_shiftpos(gbsph_ctx* ctx, float* shiftpos);

/* Read-back (JSphGpu::ParticlesDataDown, JSphGpu.cpp:630).  Any pointer may be
 * NULL.  Arrays hold the current np particles in the current (cell) order. */
int gbsph_download(gbsph_ctx* ctx, double* pos, float* velrho, unsigned* idp, uint16_t* code, unsigned* dcell);
int gbsph_get_forces(gbsph_ctx* ctx, float* ace, float* ar);
int gbsph_get_divinfo(gbsph_ctx* ctx, gbsph_divinfo* info, unsigned* begincell, unsigned begincell_cap,
                      unsigned* sortpart, unsigned* cellpart);
int gbsph_get_maxes(gbsph_ctx* ctx, gbsph_maxes* maxes);
int gbsph_sync(gbsph_ctx* ctx);

/* Device-pointer variant of gbsph_upload for callers whose particle state is
 * already in device memory (same layout as gbsph_upload's host arrays). */
int gbsph_upload_device(gbsph_ctx* ctx, unsigned np, unsigned npb, const double* d_pos, const float* d_velrho,
                        const unsigned* d_idp, const uint16_t* d_code, const float* d_boundnor);

/* Profiling (JDsTimersGpu counterpart, JDsTimersGpu.h:29-71): with
 * max_launches>0, the next max_launches fluid Interaction_Forces launches are
 * bracketed by CUDA events on the context stream; gbsph_profile_read returns
 * their durations in ms and resets the counter.  0 disables profiling.  The
 * events of a launch captured into a graph are recorded on every replay, so
 * after gbsph_run(ctx, n, 1) (one step captured, replayed n times) the read
 * returns the launches of the last replay; gbsph_run(ctx, n, 2) holds all n
 * steps and returns every launch. */
int gbsph_profile(gbsph_ctx* ctx, unsigned max_launches);
int gbsph_profile_read(gbsph_ctx* ctx, float* ms, unsigned cap, unsigned* n);
/* Caller timing on the context stream: records event `slot` (0..15); elapsed
 * time in ms between two recorded slots (waits for the second). */
int gbsph_mark(gbsph_ctx* ctx, unsigned slot);
int gbsph_elapsed(gbsph_ctx* ctx, unsigned a, unsigned b, float* ms);

/* No-alloc key sort.  This entry has no counterpart in the reference: it
 * offers the stable radix sort of the cell division (the sort behind
 * gbsph_divide) on a fixed work area that the library holds from load time
 * (a static device array), for callers that must not see a device allocation
 * or free during the call -- a host application that owns a pre-sized device
 * pool, or a latency-bound caller that cannot absorb the device
 * synchronisation of cudaFree.
 *   d_keys: n keys in device memory, nbits significant bits (1..32); bits
 *           above nbits are not looked at, so keys that have some leave the
 *           order undefined;
 *   d_perm: receives, for each sorted slot, the index of its key (ties keep
 *           the input order); d_sorted_keys (may be NULL) the sorted keys.
 * n is limited to GBSPH_SORT_NOALLOC_MAX_KEYS; larger n returns
 * GBSPH_ECAPACITY with a message in gbsph_last_error.  The work runs on the
 * context stream; the results are ready when that stream reaches them.  The
 * first call for a device (any n, 0 included) looks the work area up
 * (cudaGetSymbolAddress with that device current) and loads the sort's
 * kernels, so it may itself take memory for code; make it once, as a warm-up,
 * before relying on the no-allocation property and before any stream capture.
 * The address is kept for the life of the process: after cudaDeviceReset (or
 * any teardown of the device's primary context) it is stale, and this entry
 * must not be called again in that process.  There is one work area per
 * process and device: calls that overlap in time (from two threads or two
 * streams) race on it and must be serialised by the caller. */
#define GBSPH_SORT_NOALLOC_MAX_KEYS 262144u
int gbsph_sort_keys_noalloc(gbsph_ctx* ctx, const unsigned* d_keys, unsigned n, unsigned nbits, unsigned* d_perm,
                            unsigned* d_sorted_keys);

/* Particle-interaction count of the current state with the reference's PIPS
 * definition (JDsPips.cpp:187-260): out4 = {checked bound-row pairs, real
 * bound-row pairs, checked fluid-row pairs, real fluid-row pairs}. */
int gbsph_pips(gbsph_ctx* ctx, unsigned long long* out4);

/* Measurement gauges on the current divided state (after gbsph_upload,
 * gbsph_divide, gbsph_step or gbsph_run): the velocity, surface-water-level and
 * maximum-height gauges of the reference's gauge system (JGaugeSystem::
 * AddGaugeVel/AddGaugeSwl/AddGaugeMaxZ + CalculeGpu + GetResult,
 * JDsGaugeSystem.cpp:383-441, JDsGaugeItem.cpp:427-478, 614-641, 728-790,
 * 1023-1087), n gauges per call.  Host arrays in and out; the call waits for
 * the result.  The results follow the reference's CPU gauges: unnormalised
 * kernel sums W*m/rho accumulated in double, the domain of the gauges being the
 * map (maprealposmin..maprealposmax).  A small device scratch is allocated on
 * the first gauge call of a context (and grown for larger n).
 *   velocity: points 3n doubles (x,y,z) -> vel 3n floats, zero for a point
 *             outside the map;
 *   swl:      p0p2 6n doubles (point0 x,y,z, point2 x,y,z), pointdp n doubles,
 *             masslimit n floats (<= 0 takes massfluid*0.5, 0.4 in 2-D)
 *             -> surf 3n floats, the first point going from point0 to point2
 *             where the kernel mass drops below the limit (at most 2^20
 *             points per line, GBSPH_EINVAL beyond);
 *   maxz:     p0h 4n doubles (point0 x,y,z, height), distlimit n floats
 *             -> zmax n floats, the highest fluid particle within distlimit of
 *             the vertical segment, at least the map's lower z. */
int gbsph_gauge_velocity(gbsph_ctx* ctx, unsigned n, const double* points, float* vel);
int gbsph_gauge_swl(gbsph_ctx* ctx, unsigned n, const double* p0p2, const double* pointdp, const float* masslimit,
                    float* surf);
int gbsph_gauge_maxz(gbsph_ctx* ctx, unsigned n, const double* p0h, const float* distlimit, float* zmax);

/* Mesh gauge (JGaugeMesh, JDsGaugeItem.cpp:1484-1596; the grid of
 * JMeshData::MakeMeshPt, JMeshData.cpp:474-503): kernel-corrected velocity,
 * velocity along dirdat, density and kernel mass at the npt1 x npt2 x npt3
 * points ptref + i*dispt1*vec1/|vec1| + j*... + k*..., and the surface z of each
 * (i,j) column along the third axis.  An axis with a zero vector, dispt <= 0
 * or dis < dispt has one point; otherwise unsigned((dis+dispt/100)/dispt)+1.
 * Sums are float, as the reference's.  The kernel correction divides by sum
 * W*m/rho when that is >= kclimit, else sets kcdummy (FLT_MAX disables
 * either; the reference's defaults are 0.5 and 0); masslimit <= 0 takes
 * massfluid*0.5 (0.4 in 2-D).  Outputs (host arrays) may be NULL: vel 3*npt,
 * veldir/rhop/mass npt, zsurf npt1*npt2 floats, point index i + j*npt1 +
 * k*npt1*npt2.  At most 2^26 points. */
typedef struct {
  double ptref[3], vec1[3], vec2[3], vec3[3];
  double dis[3], dispt[3];
  float dirdat[3];
} gbsph_mesh;
int gbsph_mesh_points(const gbsph_mesh* mesh, unsigned* npt3);
int gbsph_gauge_mesh(gbsph_ctx* ctx, const gbsph_mesh* mesh, float kclimit, float kcdummy, float masslimit,
                     float* vel, float* veldir, float* rhop, float* mass, float* zsurf);

/* Surge front: the largest pos.dir over the fluid particles inside the box
 * [bmin, bmax] (bounds included), e.g. the dam-break tip position for
 * dir = (1,0,0), and the number of fluid particles in the box (*count may be
 * NULL).  With no fluid particle in the box, *front is -infinity.  This is the
 * surge-front extraction that the reference does in post-processing from Part
 * files (its experimental comparison X-DamTipPosition), done on the device
 * state. */
int gbsph_fluid_front(gbsph_ctx* ctx, const double* dir, const double* bmin, const double* bmax, double* front,
                      unsigned* count);

/* ---- Moving boundaries (JDsMotion / JMotion: JDsMotion.cpp:66-136,
 * JMotion.cpp:427-590, JMotionObj.cpp:416-690; applied as JSphGpu::RunMotion,
 * JSphGpu.cpp:1173-1228).
 * A motion holds the moving objects (the moving particle blocks, in block
 * order: object k is motion reference k), their movements and the events that
 * start them.  gbsph_motion_process advances it by one interval, as the
 * reference does once per step with that step's dt, and returns each object's
 * displacement: linear (linmov, with velocity linvel = linmov/dt) or a 4x4
 * matrix (rotations); an object with no active movement returns type 0.  The
 * motion is stateful (phases, velocities, chained movements), so it must be
 * advanced once per step in order.  Host-only: no device is touched. */
#define GBSPH_MOV_WAIT 1
#define GBSPH_MOV_RECT 2        /* vel (v) */
#define GBSPH_MOV_RECTACE 3     /* ace (a), velini (v) unless prev */
#define GBSPH_MOV_ROT 4         /* axisp1, axisp2, angular vel (s[0]) */
#define GBSPH_MOV_ROTACE 5      /* axisp1, axisp2, angular ace (s[1]), velini (s[0]) unless prev */
#define GBSPH_MOV_RECTSINU 6    /* freq (v), ampl (a), phase (p) unless prev */
#define GBSPH_MOV_ROTSINU 7     /* axisp1, axisp2, freq (s[0]), ampl (s[1]), phase (s[2]) unless prev */
#define GBSPH_MOV_NULL 8
typedef struct {
  int type;            /* GBSPH_MOV_* */
  unsigned obj;        /* moving object (reference) the movement belongs to */
  unsigned id, nextid; /* movement id within its object; the next movement's id (0: none) */
  double duration;     /* seconds; < 0 is an instantaneous movement */
  int angdegrees;      /* anglesunits: 1 degrees, 0 radians */
  int prev;            /* velini/phase taken from the previous movement */
  double v[3], a[3], p[3], axisp1[3], axisp2[3], s[3];  /* parameters, as the XML gives them */
} gbsph_movement;
typedef struct {
  unsigned obj, mov;   /* object and movement id */
  double start, finish;  /* finish < 0: none */
} gbsph_motion_event;
typedef struct {
  unsigned idbegin, count;  /* ids of the object's particles */
} gbsph_motion_object;
typedef struct {
  int type;              /* 0 none, 1 linear, 2 matrix */
  double linmov[3], linvel[3];
  double mat[16];        /* row-major a11..a44 */
} gbsph_motion_data;
typedef struct gbsph_motion gbsph_motion;
int gbsph_motion_create(unsigned nobj, const gbsph_motion_object* objs, unsigned nmov, const gbsph_movement* movs,
                        unsigned nevt, const gbsph_motion_event* evts, int simulate2d, gbsph_motion** out);
void gbsph_motion_destroy(gbsph_motion* m);
/* Advances the motion over [timestep, timestep+dt]; out: one entry per object.
 * Returns 1 when some object moves in the interval, 0 when none, < 0 on error. */
int gbsph_motion_process(gbsph_motion* m, double timestep, double dt, gbsph_motion_data* out);
/* Attaches a motion to a context (NULL detaches).  Each following step (and
 * every step of gbsph_run) reads back its dt and time, advances the motion on
 * the host, and after the step's update moves the objects' particles
 * (position by UpdatePos, velocity set to the motion's, normals rotated by a
 * matrix motion) and marks the boundary changed, so the next divide is full.
 * gbsph_run's multi-step graph (mode 2) is not used with a motion.  A Verlet
 * step advances the motion inside the step, with the dt it has just computed
 * (one read-back of the step state), so Verlet steps with a motion are not
 * captured in graphs.  The motion stays
 * owned by the caller and must outlive the attachment. */
int gbsph_set_motion(gbsph_ctx* ctx, gbsph_motion* m);

/* Kernel-launch counter of the context (launches issued since creation). */
unsigned long long gbsph_launch_count(const gbsph_ctx* ctx);
/* CUDA stream of the context (as void*), for callers that order their own work. */
void* gbsph_stream(gbsph_ctx* ctx);
/* Kernel options (autotuner hook).  key 1 = fluid-row kernel of
 * gbsph_forces: 2 (default) cell-tiled: the neighbour cells' particles staged
 * through a shared-memory ring of 8 chunks of 32, distance checks on the
 * staged copies, pair terms in rounds; 3 the same with a ring of 4 chunks;
 * 0 per-lane neighbour queues evaluated in rounds; 1 one thread per particle
 * with no queue.  key 0 = threads per block of the one-thread-per-particle
 * kernel (64, 128 or 256; the other kernels use 128).  The reference fixes
 * 128 threads per block (JSphGpu.cpp, BlockSizes).  key 2 = digit width of
 * the divide's radix sort, 8 (default) or 11 bits.  key 3 = mDBC kernel of
 * gbsph_mdbc: 0 (default) cell-tiled, the ghost nodes' fluid neighbours
 * staged through shared memory; 1 one thread per boundary row.  key 4 =
 * warps that share each group of 32 fluid rows in the cell-tiled kernel
 * with a ring of 8 chunks (each takes every 1st, 2nd or 4th chunk of the
 * rows' candidates and the first adds the others' sums): 1, 2, 4, or 0
 * (default) chosen from the fluid rows of the last upload, so that a case
 * too small to fill the device runs more, shorter warps.  The other kernels,
 * and cases that need the power form of the DDT2 hydrostatic term, keep one
 * warp.  The sums' order changes with it, within the FP32 criterion.
 * key 6 = lanes a boundary row in the bound-row pass of gbsph_forces: 1
 * (one thread a row, the reference's layout), 4, 32, or 0 (default) chosen
 * from the boundary rows of the last upload (32 up to 117 k rows and 4 up
 * to 467 k on 152 SMs); the lanes take a row's candidates in turn.
 * key 8 = warps that share each group of 32 boundary rows in the cell-tiled
 * mDBC kernel (each takes every 1st, 2nd or 4th chunk of the ghosts'
 * candidates, and the first adds the others' compensated sums): 1, 2, 4, or
 * 0 (default: 4, the fastest at every size measured).  key 10 = the
 * bound-row pass of gbsph_forces on a second stream beside the fluid-row
 * pass (1) or before it on the context's stream (0, the default); the two
 * write different rows, so the results are the same. */
int gbsph_set_option(gbsph_ctx* ctx, int key, int value);
/* The current value of an option of gbsph_set_option (no reference
 * counterpart); key 5 reads the warps per row group in effect (key 4
 * resolved), key 7 the lanes a boundary row in effect (key 6 resolved),
 * key 9 the warps per mDBC row group in effect (key 8 resolved). */
int gbsph_get_option(const gbsph_ctx* ctx, int key, int* value);

/* Autotuner (no reference counterpart).  Times each fluid-row kernel
 * configuration -- the cell-tiled kernel with rings of 8 chunks at 1, 2 and
 * 4 warps per row group and with a ring of 4 chunks, the queued kernel, and
 * the one-thread-per-particle kernel at 64, 128 and 256 threads per block --
 * over `reps` launches on the context's current state, then with the
 * fastest the lanes a boundary row of the bound-row pass and (for mDBC) the
 * warps per row group of the staged mDBC kernel,
 * between steps, and keeps the fastest.  The launches rewrite only the
 * interaction outputs, which the next step recomputes.  The kernels sum a
 * row's neighbours in different orders: results stay within the FP32
 * criterion of each other, not bit-identical. */
#define GBSPH_TUNE_CANDIDATES 8
typedef struct {
  int best;                              /* index of the configuration kept */
  int variant[GBSPH_TUNE_CANDIDATES];    /* gbsph_set_option key 1 */
  int bsize[GBSPH_TUNE_CANDIDATES];      /* gbsph_set_option key 0 */
  int split[GBSPH_TUNE_CANDIDATES];      /* gbsph_set_option key 4 */
  float ms[GBSPH_TUNE_CANDIDATES];       /* mean time of one interaction pass */
  int bound_best;                        /* index of the lanes a boundary row kept */
  int bound_lanes[3];                    /* gbsph_set_option key 6: 1, 4, 32 */
  float bound_ms[3];                     /* mean time of one interaction pass with each */
  int mdbc_best;                         /* index of the mDBC split kept (-1: no mDBC) */
  int mdbc_split[3];                     /* gbsph_set_option key 8: 1, 2, 4 */
  float mdbc_ms[3];                      /* mean time of one mDBC pass with each */
} gbsph_tune_result;
int gbsph_tune_forces(gbsph_ctx* ctx, int reps, gbsph_tune_result* out);
/* Autotuner of the cell division: times `reps` divisions of the current state
 * (between steps) with radix-sort digits of 8 and of 11 bits and keeps the
 * faster (gbsph_set_option key 2).  Both give the same sort order; the
 * periodic copies of the state are made anew.  ms receives the two mean
 * times (may be NULL). */
int gbsph_tune_sort(gbsph_ctx* ctx, int reps, int* best_bits, float* ms);

/* Ensembles (no reference counterpart: the reference runs one case per
 * process, JSphGpuSingle::Run, JSphGpuSingle.cpp:950-1010).  Independent,
 * uploaded contexts of one device advanced together: each keeps its own
 * arrays, dt and motion; one Symplectic step of every case is captured as one
 * CUDA graph with a concurrent branch per case and replayed.  Cases with a
 * motion have it advanced on the host between replays.  If any case uses
 * Verlet, or use_graph is 0, the steps are issued on the cases' own streams,
 * which run concurrently.  The contexts stay owned by the caller and must
 * outlive the ensemble; work the caller issues on a case after
 * gbsph_ensemble_run is ordered after the ensemble's. */
typedef struct gbsph_ensemble gbsph_ensemble;
int gbsph_ensemble_create(unsigned n, gbsph_ctx* const* ctxs, gbsph_ensemble** out);
void gbsph_ensemble_destroy(gbsph_ensemble* e);
const char* gbsph_ensemble_last_error(const gbsph_ensemble* e);
int gbsph_ensemble_run(gbsph_ensemble* e, unsigned nsteps, int use_graph);
/* Waits for the ensemble and checks every case's device error word. */
int gbsph_ensemble_sync(gbsph_ensemble* e);
/* Kernel launches one replay of the ensemble graph holds (0 before the first). */
unsigned long long gbsph_ensemble_launches_per_step(const gbsph_ensemble* e);

/* FP32 roofline denominator (no reference counterpart): an FFMA
 * microbenchmark, 8 independent chains per thread on 8 blocks of 256 threads
 * per SM, best of 5 launches; TFLOP/s at the device's current clock. */
int gbsph_ffma_peak(int device, float* tflops);

/* ---- learned closure (no reference counterpart) -------------------------
 * A 16-64-64-64-3 tanh MLP with BF16 weights and FP32 accumulation that adds
 * a per-particle correction g*y to the fluid accelerations of a coarse run.
 * Its inputs are the GBSPH_CLOSURE_FEATURES features of a fluid row over its
 * kernel neighbourhood (density, kernel-weighted velocity differences,
 * pressure-gradient moment, Shepard sum, position divergence, the plain
 * acceleration, boundary proximity).  Parameters, flat and row-major:
 * W0[64][16] b0[64] W1[64][64] b1[64] W2[64][64] b2[64] W3[3][64] b3[3]. */
#define GBSPH_CLOSURE_FEATURES 16
#define GBSPH_CLOSURE_PARAMS 9603
/* Attaches the closure to a context (w_bf16 NULL detaches): after every
 * interaction pass of every later step the correction is added to each fluid
 * row whose correction norm is at most `limit` x its plain |ace| (the others
 * keep the plain acceleration, counted by gbsph_closure_fallbacks), and AceMax
 * is taken over the corrected rows. */
int gbsph_closure_set(gbsph_ctx* ctx, const uint16_t* w_bf16, float limit);
/* Features of the fluid rows of the current state ((np-npb) x 16 floats, in the
 * order gbsph_download returns rows npb..np-1); call after gbsph_forces. */
int gbsph_closure_features(gbsph_ctx* ctx, float* out);
int gbsph_closure_fallbacks(gbsph_ctx* ctx, unsigned long long* n);

/* Trainer: the MLP's own forward/backward kernels and Adam on one device.
 * Data (features x, targets t = 3 per sample) are copied to the device once;
 * gbsph_mlp_train runs `epochs` passes of mini-batches of `batch` samples in
 * data order (the caller shuffles), the loss being the mean of (y - t)^2. */
typedef struct gbsph_mlp gbsph_mlp;
int gbsph_mlp_create(int device, const float* params, gbsph_mlp** out);
void gbsph_mlp_destroy(gbsph_mlp* m);
int gbsph_mlp_set_data(gbsph_mlp* m, const float* x, const float* t, unsigned n);
/* Gradient (GBSPH_CLOSURE_PARAMS floats) and loss of samples [first, first+n)
 * at the current weights. */
int gbsph_mlp_grad(gbsph_mlp* m, unsigned first, unsigned n, float* grad, float* loss);
int gbsph_mlp_train(gbsph_mlp* m, unsigned epochs, unsigned batch, float lr, float* loss_per_epoch);
int gbsph_mlp_infer(gbsph_mlp* m, const float* x, unsigned n, float* y);
/* FP32 master weights and their BF16 copy (either may be NULL). */
int gbsph_mlp_params(gbsph_mlp* m, float* master, uint16_t* w_bf16);

#ifdef __cplusplus
}
#endif
#endif
