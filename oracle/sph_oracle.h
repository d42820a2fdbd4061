/*
 * sph_oracle.h -- CPU restatement of the DualSPHysics v5.4 WCSPH step (test
 * infrastructure only).
 *
 * This is the ORACLE: a plain C restatement of the reference CPU solver
 * (JSphCpuSingle) for the per-step hot path, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / --impl reference
 * legs as the checker and the timed CPU baseline.  It is never linked into the
 * product library and the product path never calls it.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the DualSPHysics source tree src/source/).  Parity of this restatement is
 * pinned against golden fixtures produced by the reference solver itself
 * (oracle/ref_harness.cpp, tests/golden/).
 *
 * Floating point: the FP32 functions evaluate every expression in the order the
 * reference writes it, in float, and are compiled with -ffp-contract=off so the
 * result does not depend on FMA contraction of the host compiler.  The _f64
 * variants evaluate the same formulas in double and serve as the FP64 oracle
 * against which FP32 errors are stated.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* particle code bits (typecode = 16-bit word), DualSphDef.h:150-200 */
#define ORC_CODE_MASKSPECIAL 0xe000u
#define ORC_CODE_NORMAL      0x0000u
#define ORC_CODE_PERIODIC    0x2000u
#define ORC_CODE_OUTIGNORE   0x4000u
#define ORC_CODE_OUTMOV      0x6000u
#define ORC_CODE_OUTPOS      0x8000u
#define ORC_CODE_OUTRHO      0xA000u
#define ORC_CODE_MASKTYPE    0x1800u
#define ORC_CODE_TYPE_FIXED  0x0000u
#define ORC_CODE_TYPE_MOVING 0x0800u
#define ORC_CODE_TYPE_FLOATING 0x1000u
#define ORC_CODE_TYPE_FLUID  0x1800u

/* options (values follow the XML <parameters> keys of the reference) */
#define ORC_STEP_VERLET 1
#define ORC_STEP_SYMPLECTIC 2
#define ORC_VISCO_ARTIFICIAL 1
#define ORC_VISCO_LAMINARSPS 2
#define ORC_VISCO_LAMINAR 3
#define ORC_DDT_NONE 0
#define ORC_DDT_DDT 1
#define ORC_DDT_DDT2 2
#define ORC_DDT_DDT2FULL 3
#define ORC_BC_DBC 1
#define ORC_BC_MDBC 2

/* Constants of one case.  Field types follow the reference members
 * (JSph.h:178-365): float where the reference stores float, double where it
 * stores double. */
typedef struct {
  /* options */
  int tstep, tvisco, tdensity, tboundary, verletsteps, dtallparticles, simulate2d, cellmode_div;
  /* SPH constants */
  float kernelh, kernelsize, kernelsize2, cteb, gamma, rhopzero, massfluid, massbound;
  float eta2, ddtkh, ddtgz, visco, viscoboundfactor, awen, bwenh, spssmag, spsblin;
  float scell, movlimit, rhopoutmin, rhopoutmax, gravity[3];
  double dp, cs0, cflnumber, dtmin, dtini;
  /* domain */
  double mapposmin[3], maprealposmin[3], maprealsize[3], maprealposmax[3];
  double domposmin[3], domrealposmin[3], domrealposmax[3];
  unsigned mapcells[3], domcells[3], domcellcode;
  int tshift;
  float shiftcoef, shifttfs;
  int peri[3];
  double periinc[9];
  double mapposmax[3];
} orc_ctes;

/* Raw case parameters (what the run XML carries) from which orc_config derives
 * orc_ctes the way JSph::ConfigConstants1/2, ConfigCellDivision and
 * SelecDomain do (JSph.cpp:1481-1546,1877-1944). */
typedef struct {
  int tstep, tvisco, tdensity, tboundary, verletsteps, dtallparticles, simulate2d, cellmode_div;
  double dp, h, b, rhop0, gamma, massbound, massfluid, cflnumber;
  double gravity[3];
  float visco, viscoboundfactor, ddtvalue, coefdtmin, rhopoutmin, rhopoutmax;
  double dtini, dtmin;               /* 0 = automatic */
  double maprealposmin[3], maprealposmax[3];
  int tshift;
  float shiftcoef, shifttfs;
  int peri[3];
  double periinc[9];
} orc_params;

/* Cell-division state: JCellDivCpu/JCellDivCpuSingle members. */
typedef struct {
  unsigned npb1, npf1, nptot;
  int dividefull;
  unsigned cellmin[3], cellmax[3];
  unsigned ncx, ncy, ncz, nsheet, nct, nctt;
  unsigned boxboundignore, boxfluid, boxboundout, boxfluidout, boxboundoutignore, boxfluidoutignore;
  int boundlimitok, bounddivideok;
  unsigned boundlimitcellmin[3], boundlimitcellmax[3];
  unsigned bounddividecellmin[3], bounddividecellmax[3];
  unsigned npbignore, npbout, npfout, npboutignore, npfoutignore, npfinal, npbfinal;
  unsigned npb2, npf2; /* periodic copies of boundary and fluid particles after npb1+npf1 */
} orc_div;

/* Host-side simulation state held by the oracle (JSphCpuSingle arrays). */
typedef struct orc_sim orc_sim;

/* ---- setup ---- */
int orc_config(const orc_params* prm, orc_ctes* out);
unsigned orc_calc_cellcode(unsigned ncx, unsigned ncy, unsigned ncz);
void orc_cell_decode(unsigned dcc, unsigned cel, unsigned* cx, unsigned* cy, unsigned* cz);
void orc_load_dcell(const orc_ctes* c, unsigned n, const uint16_t* code, const double* pos, unsigned* dcell);
float orc_compute_press(const orc_ctes* c, float rho);

/* ---- neighbour list (cell division) ---- */
int orc_divide(const orc_ctes* c, orc_div* d, unsigned npb, unsigned npf, unsigned npbper, unsigned npfper,
               int boundchanged,
               const unsigned* dcell, const uint16_t* code,
               unsigned* cellpart, unsigned* sortpart, unsigned* begincell, unsigned begincell_cap);

/* ---- interaction ---- */
void orc_interaction_forces(const orc_ctes* c, const orc_div* d, const unsigned* begincell,
                            unsigned np, unsigned npb, unsigned npbok,
                            const unsigned* dcell, const double* pos, const float* velrho,
                            const uint16_t* code, const float* tau,
                            float* ace, float* ar, float* two_strain, float* viscdt_out, int nthreads,
                            float* shiftpos);  /* 4 per particle or NULL: shifting sums (tshift) */
void orc_interaction_forces_f64(const orc_ctes* c, const orc_div* d, const unsigned* begincell,
                                unsigned np, unsigned npb, unsigned npbok,
                                const unsigned* dcell, const double* pos, const float* velrho,
                                const uint16_t* code, const double* tau,
                                double* ace, double* ar, double* two_strain, double* viscdt_out, int nthreads,
                                double* absace, double* absar, double* shiftpos, double* absshift);
void orc_sps_tau(const orc_ctes* c, unsigned n, unsigned pini, const float* velrho,
                 const float* two_strain, float* tau);
void orc_mdbc_correction(const orc_ctes* c, const orc_div* d, const unsigned* begincell,
                         unsigned n, const double* pos, const uint16_t* code,
                         const float* boundnor, float* velrho, int nthreads);
void orc_pips(const orc_ctes* c, const orc_div* d, const unsigned* begincell, unsigned np,
              unsigned npb, unsigned npbok, const unsigned* dcell, const double* pos,
              unsigned long long out[4], int nthreads);

/* ---- integration and dt ---- */
float orc_velmax(unsigned n, const float* velrho);
double orc_acemax(unsigned n, const float* ace);
double orc_dtvariable(const orc_ctes* c, double acemax, float velmax, float viscdtmax, int* err);

/* ---- whole-solver state ---- */
orc_sim* orc_sim_create(const orc_ctes* c, unsigned np, unsigned npb, const double* pos,
                        const float* velrho, const unsigned* idp, const uint16_t* code,
                        const float* boundnor, int nthreads);
void orc_sim_destroy(orc_sim* s);
int orc_sim_run_cell_divide(orc_sim* s);
int orc_sim_mdbc(orc_sim* s, int corrector);
int orc_sim_interaction(orc_sim* s);
double orc_sim_dtvariable(orc_sim* s, int* err);
int orc_sim_symplectic_pre(orc_sim* s, double dt);
int orc_sim_symplectic_cor(orc_sim* s, double dt);
int orc_sim_verlet(orc_sim* s, double dt);
int orc_sim_run_shifting(orc_sim* s, double dt);   /* JSphShifting::RunCpu */
void orc_sim_get_shiftpos(const orc_sim* s, float* out);
void orc_sim_set_shiftpos(orc_sim* s, const float* in);
int orc_sim_step(orc_sim* s, double* dtused);
unsigned orc_sim_np(const orc_sim* s);
unsigned orc_sim_npb(const orc_sim* s);
unsigned orc_sim_npbok(const orc_sim* s);
const orc_div* orc_sim_div(const orc_sim* s);
void orc_sim_get(const orc_sim* s, double* pos, float* velrho, unsigned* idp, uint16_t* code, unsigned* dcell);
void orc_sim_get_forces(const orc_sim* s, float* ace, float* ar);
void orc_sim_get_begincell(const orc_sim* s, unsigned* begincell, unsigned n);
void orc_sim_get_sortpart(const orc_sim* s, unsigned* sortpart, unsigned* cellpart);
void orc_sim_maxes(const orc_sim* s, double* acemax, float* velmax, float* viscdtmax, double* dtpre);
void orc_sim_set_dtpre(orc_sim* s, double dt);
void orc_sim_set_forces(orc_sim* s, const float* ace, const float* ar);
void orc_sim_set_state(orc_sim* s, const double* pos, const float* velrho);
unsigned orc_sim_nout(const orc_sim* s);
double orc_sim_time(const orc_sim* s);
void orc_sim_times(const orc_sim* s, double* t_inter, double* t_step);
void orc_set_sampling(int stride, int phase);
void orc_sim_mdbc_f64(orc_sim* s, double* rho64);
void orc_mdbc_correction_f64(const orc_ctes* c, const orc_div* d, const unsigned* begincell, unsigned n,
                             const double* pos, const uint16_t* code, const float* boundnor, const float* velrho,
                             double* rho64, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
