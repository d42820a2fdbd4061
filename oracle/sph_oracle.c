/*
 * sph_oracle.c -- CPU restatement of the DualSPHysics v5.4 WCSPH step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline legs load this code; the product library never
 * links it.  Parity of this restatement is pinned against fixtures produced by
 * the reference solver itself (see oracle/ref_harness.cpp and tests/golden/).
 *
 * Citations are to the DualSPHysics source tree, src/source/.
 * Compile with -ffp-contract=off: float expressions are evaluated in the order
 * the reference writes them.
 */
#include "sph_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ALMOSTZERO 1e-18f /* DualSphDef.h:114 */

/* Row sampling for timing the CPU baseline on a bounded sample of a large
 * workload: with stride>1 only interaction rows p with p%stride==phase are
 * evaluated (the others keep zero forces).  Off (stride 1) for every parity use. */
static int g_sample_stride = 1, g_sample_phase = 0;
void orc_set_sampling(int stride, int phase) {
  g_sample_stride = stride > 1 ? stride : 1;
  g_sample_phase = phase;
}

static double orc_now(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

static inline unsigned codespecial(uint16_t c) { return c & ORC_CODE_MASKSPECIAL; }
static inline unsigned codetype(uint16_t c) { return c & ORC_CODE_MASKTYPE; }

/* ------------------------------------------------------------------------ */
/* Cell codification (JDsDcellDef.h:27-43, JDsDcell.cpp:34-72).              */
/* ------------------------------------------------------------------------ */
static unsigned bits_for(unsigned v, unsigned minbits) {
  /* JDsDcell::CalcBitsValue (JDsDcell.cpp:34-38) */
  unsigned n = (minbits < 1 || minbits > 30) ? 1 : minbits;
  while (v >> n) n++;
  return n;
}

unsigned orc_calc_cellcode(unsigned ncx, unsigned ncy, unsigned ncz) {
  /* JDsDcell::CalcCellDistribution + CalcCellCode (JDsDcell.cpp:44-72) with
   * 31 bits (1 extra bit goes to x). */
  const unsigned maxbits = 31;
  unsigned sx = bits_for(ncx, 2), sy = bits_for(ncy, 2), sz = bits_for(ncz, 2);
  const unsigned smin = sx + sy + sz;
  if (smin > maxbits) return 0;
  unsigned rest = maxbits - smin;
  while (rest) {
    if (rest) { sx++; rest--; }
    if (rest) { sy++; rest--; }
    if (rest) { sz++; rest--; }
  }
  return ((sx + 1) << 25) | (sy << 20) | (sz << 15) | ((sy + sz) << 10) | ((sx + 1 + sz) << 5) | (sx + 1 + sy);
}

static inline unsigned dcel_cx(unsigned dcc, unsigned cel) { return cel >> ((dcc >> 10) & 31); }
static inline unsigned dcel_cy(unsigned dcc, unsigned cel) { return (cel << (dcc >> 25)) >> ((dcc >> 5) & 31); }
static inline unsigned dcel_cz(unsigned dcc, unsigned cel) { return (cel << (dcc & 31)) >> (dcc & 31); }
static inline unsigned dcel_cell(unsigned dcc, unsigned cx, unsigned cy, unsigned cz) {
  return (cx << ((dcc >> 10) & 31)) | (cy << ((dcc >> 15) & 31)) | cz;
}

void orc_cell_decode(unsigned dcc, unsigned cel, unsigned* cx, unsigned* cy, unsigned* cz) {
  *cx = dcel_cx(dcc, cel);
  *cy = dcel_cy(dcc, cel);
  *cz = dcel_cz(dcc, cel);
}

/* ------------------------------------------------------------------------ */
/* Constants (JSph.cpp:1481-1546 ConfigConstants1/2, :1877-1944 cell       */
/* division and SelecDomain).                                                */
/* ------------------------------------------------------------------------ */
int orc_config(const orc_params* p, orc_ctes* c) {
  memset(c, 0, sizeof(*c));
  c->tstep = p->tstep; c->tvisco = p->tvisco; c->tdensity = p->tdensity; c->tboundary = p->tboundary;
  c->tshift = p->tshift; c->shiftcoef = p->tshift ? p->shiftcoef : 0.f; c->shifttfs = p->tshift ? p->shifttfs : 0.f;
  c->verletsteps = p->verletsteps; c->dtallparticles = p->dtallparticles; c->simulate2d = p->simulate2d;
  c->cellmode_div = p->cellmode_div ? p->cellmode_div : 1;
  /* JSph::LoadConfigCtes (JSph.cpp:642-658): float members */
  c->kernelh = (float)p->h;
  c->cteb = (float)p->b;
  c->gamma = (float)p->gamma;
  c->rhopzero = (float)p->rhop0;
  c->cflnumber = p->cflnumber;
  c->dp = p->dp;
  c->massfluid = (float)p->massfluid;
  c->massbound = (float)p->massbound;
  c->gravity[0] = (float)p->gravity[0]; c->gravity[1] = (float)p->gravity[1]; c->gravity[2] = (float)p->gravity[2];
  c->visco = p->visco;
  c->viscoboundfactor = p->viscoboundfactor;
  c->rhopoutmin = p->rhopoutmin; c->rhopoutmax = p->rhopoutmax;
  /* ConfigConstants1 (JSph.cpp:1481-1524); Wendland factor 2 (FunSphKernel.h:194) */
  {
    const float kernelk = 2.0f;
    const double h = c->kernelh;
    const double kh = h * kernelk;
    c->kernelsize = (float)kh;
    c->kernelsize2 = c->kernelsize * c->kernelsize;
    if (c->simulate2d) {
      c->awen = (float)(0.557 / (h * h));
      c->bwenh = (float)(-2.7852 / (h * h * h * h));
    } else {
      /* FunSphKernel.h:198-211 */
      c->awen = (float)(0.41778 / (h * h * h));
      c->bwenh = (float)(-2.08891 / (h * h * h * h * h));
    }
    c->cs0 = sqrt((double)c->gamma * (double)c->cteb / (double)c->rhopzero);
    c->eta2 = (float)((h * 0.1) * (h * 0.1));
  }
  /* ConfigConstants2 (JSph.cpp:1526-1546) */
  if (c->tvisco == ORC_VISCO_LAMINARSPS) {
    const double dp_sps = (c->simulate2d ? sqrt(c->dp * c->dp * 2.) / 2. : sqrt(c->dp * c->dp * 3.) / 3.);
    c->spssmag = (float)((2. / 3.) * pow((0.12 * dp_sps), 2));
    c->spsblin = (float)((2. / 3.) * 0.0066 * dp_sps * dp_sps);
  }
  /* DDTValue is 0 without density diffusion (JSph.cpp:923) */
  c->ddtkh = c->kernelsize * (p->tdensity == 0 ? 0.f : p->ddtvalue);
  c->ddtgz = (float)((double)c->rhopzero * (double)fabsf(c->gravity[2]) / (double)c->cteb);
  c->dtini = p->dtini;
  c->dtmin = p->dtmin;
  if (!c->dtini) c->dtini = c->kernelh / c->cs0;
  if (!c->dtmin) c->dtmin = (c->kernelh / c->cs0) * p->coefdtmin;
  /* ConfigCellDivision (JSph.cpp:1877-1886) */
  c->scell = c->kernelsize / (float)c->cellmode_div;
  c->movlimit = c->scell * 0.9f;
  for (int k = 0; k < 3; k++) {
    c->maprealposmin[k] = p->maprealposmin[k];
    c->maprealposmax[k] = p->maprealposmax[k];
    c->maprealsize[k] = p->maprealposmax[k] - p->maprealposmin[k];
    c->peri[k] = p->peri[k] != 0;
  }
  /* periodic increments: the own component is -MapRealSize (JSph.cpp:2186-2188) */
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      c->periinc[3 * k + j] = c->peri[k] ? (j == k ? -c->maprealsize[k] : p->periinc[3 * k + j]) : 0.0;
  /* Map_PosMin/Max: a KernelSize halo on periodic axes (JSph.cpp:2190-2194);
     ConfigCellDivision (JSph.cpp:1877-1886) */
  for (int k = 0; k < 3; k++) {
    c->mapposmin[k] = c->peri[k] ? c->maprealposmin[k] - (double)c->kernelsize : c->maprealposmin[k];
    c->mapposmax[k] = c->peri[k] ? c->maprealposmax[k] + (double)c->kernelsize : c->maprealposmax[k];
    const double mapsize = c->mapposmax[k] - c->mapposmin[k];
    c->mapcells[k] = (unsigned)ceil(mapsize / c->scell);
  }
  /* SelecDomain(0,Map_Cells) (JSph.cpp:1901-1944) */
  for (int k = 0; k < 3; k++) {
    c->domcells[k] = c->mapcells[k];
    c->domposmin[k] = c->mapposmin[k] + (0 * c->scell);
    double dmax = c->mapposmin[k] + (c->mapcells[k] * c->scell);
    if (dmax > c->mapposmax[k]) dmax = c->mapposmax[k];
    c->domrealposmin[k] = c->domposmin[k];
    c->domrealposmax[k] = dmax;
    if (c->domrealposmax[k] > c->maprealposmax[k]) c->domrealposmax[k] = c->maprealposmax[k];
    if (c->domrealposmin[k] < c->maprealposmin[k]) c->domrealposmin[k] = c->maprealposmin[k];
  }
  c->domcellcode = orc_calc_cellcode(c->domcells[0] + 1, c->domcells[1] + 1, c->domcells[2] + 1);
  return c->domcellcode ? 0 : -1;
}

/* JSph::LoadDcellParticles (JSph.cpp:1794-1817). Returns nothing; particles
 * out of the domain get DCEL_CodeMapOut. */
void orc_load_dcell(const orc_ctes* c, unsigned n, const uint16_t* code, const double* pos, unsigned* dcell) {
  for (unsigned p = 0; p < n; p++) {
    if (codespecial(code[p]) < ORC_CODE_OUTIGNORE) {
      const double* ps = pos + 3 * (size_t)p;
      if (ps[0] >= c->domrealposmin[0] && ps[1] >= c->domrealposmin[1] && ps[2] >= c->domrealposmin[2] &&
          ps[0] < c->domrealposmax[0] && ps[1] < c->domrealposmax[1] && ps[2] < c->domrealposmax[2]) {
        const double dx = ps[0] - c->domposmin[0], dy = ps[1] - c->domposmin[1], dz = ps[2] - c->domposmin[2];
        const unsigned cx = (unsigned)(dx / c->scell), cy = (unsigned)(dy / c->scell), cz = (unsigned)(dz / c->scell);
        dcell[p] = dcel_cell(c->domcellcode, cx, cy, cz);
      } else dcell[p] = 0xffffffffu;
    } else dcell[p] = 0xffffffffu;
  }
}

/* FunSphEos.h:37-39 (Monaghan 1994 / Tait): B*((rho/rho0)^gamma-1) */
float orc_compute_press(const orc_ctes* c, float rho) {
  return c->cteb * (powf(rho / c->rhopzero, c->gamma) - 1.0f);
}

/* ------------------------------------------------------------------------ */
/* Cell division (JCellDivCpuSingle.cpp:45-350, JCellDivCpu.cpp:256-345).    */
/* ------------------------------------------------------------------------ */
static void limits_cell(const orc_ctes* c, unsigned n, unsigned pini, const unsigned* dcell, const uint16_t* code,
                        unsigned cmin[3], unsigned cmax[3]) {
  /* JCellDivCpu::LimitsCellBound / LimitsCellFluid (JCellDivCpu.cpp:256-345) */
  cmin[0] = cmin[1] = cmin[2] = UINT_MAX;
  cmax[0] = cmax[1] = cmax[2] = 0;
  const unsigned dcc = c->domcellcode;
  for (unsigned p = pini; p < pini + n; p++) {
    if (codespecial(code[p]) < ORC_CODE_OUTIGNORE) {
      const unsigned cx = dcel_cx(dcc, dcell[p]), cy = dcel_cy(dcc, dcell[p]), cz = dcel_cz(dcc, dcell[p]);
      if (cmin[0] > cx) cmin[0] = cx;
      if (cmin[1] > cy) cmin[1] = cy;
      if (cmin[2] > cz) cmin[2] = cz;
      if (cmax[0] < cx) cmax[0] = cx;
      if (cmax[1] < cy) cmax[1] = cy;
      if (cmax[2] < cz) cmax[2] = cz;
    }
  }
}

static void calc_domain_part(const orc_ctes* c, unsigned n, unsigned pini, unsigned n2, unsigned pini2,
                             const unsigned* dcell, const uint16_t* code, unsigned cellmin[3], unsigned cellmax[3]) {
  /* CalcCellDomainBound / CalcCellDomainFluid (JCellDivCpu.cpp:295-345): the
     second range holds the periodic copies */
  unsigned cmin[3], cmax[3];
  limits_cell(c, n, pini, dcell, code, cmin, cmax);
  for (int k = 0; k < 3; k++) {
    cellmin[k] = (cmin[0] > cmax[0] ? c->domcells[k] : cmin[k]);
    cellmax[k] = (cmin[0] > cmax[0] ? 0 : cmax[k]);
  }
  if (n2) {
    limits_cell(c, n2, pini2, dcell, code, cmin, cmax);
    const int empty = cmin[0] > cmax[0];
    for (int k = 0; k < 3; k++) {
      const unsigned a = empty ? c->domcells[k] : cmin[k], b = empty ? 0 : cmax[k];
      if (a < cellmin[k]) cellmin[k] = a;
      if (b > cellmax[k]) cellmax[k] = b;
    }
  }
}

int orc_divide(const orc_ctes* c, orc_div* d, unsigned npb, unsigned npf, unsigned npbper, unsigned npfper,
               int boundchanged, const unsigned* dcell, const uint16_t* code,
               unsigned* cellpart, unsigned* sortpart, unsigned* begincell, unsigned begincell_cap) {
  /* JCellDivCpuSingle::Divide (JCellDivCpuSingle.cpp:280-350); npbper/npfper
     periodic copies follow the npb+npf particles */
  d->dividefull = 0;
  d->npb1 = npb; d->npf1 = npf; d->npb2 = npbper; d->npf2 = npfper;
  d->nptot = npb + npf + npbper + npfper;
  if (c->peri[0] || c->peri[1] || c->peri[2]) boundchanged = 1;
  d->npbout = d->npfout = d->npboutignore = d->npfoutignore = 0;
  d->npfinal = d->npbfinal = 0;
  d->npbignore = 0;
  if (boundchanged) {
    d->boundlimitok = d->bounddivideok = 0;
    memset(d->boundlimitcellmin, 0, sizeof(d->boundlimitcellmin));
    memset(d->boundlimitcellmax, 0, sizeof(d->boundlimitcellmax));
    memset(d->bounddividecellmin, 0, sizeof(d->bounddividecellmin));
    memset(d->bounddividecellmax, 0, sizeof(d->bounddividecellmax));
  }
  /* CalcCellDomain (JCellDivCpuSingle.cpp:45-71) */
  unsigned celbmin[3], celbmax[3], celfmin[3], celfmax[3];
  if (!d->boundlimitok) {
    calc_domain_part(c, d->npb1, 0, d->npb2, d->npb1 + d->npf1, dcell, code, celbmin, celbmax);
    d->boundlimitok = 1;
    memcpy(d->boundlimitcellmin, celbmin, sizeof(celbmin));
    memcpy(d->boundlimitcellmax, celbmax, sizeof(celbmax));
  } else {
    memcpy(celbmin, d->boundlimitcellmin, sizeof(celbmin));
    memcpy(celbmax, d->boundlimitcellmax, sizeof(celbmax));
  }
  calc_domain_part(c, d->npf1, d->npb1, d->npf2, d->npb1 + d->npf1 + d->npb2, dcell, code, celfmin, celfmax);
  /* MergeMapCellBoundFluid (JCellDivCpuSingle.cpp:85-101) */
  {
    const unsigned sd = (unsigned)c->cellmode_div;
    unsigned* cmn = d->cellmin; unsigned* cmx = d->cellmax;
    for (int k = 0; k < 3; k++) {
      const unsigned a = (celbmin[k] < celfmin[k] ? celbmin[k] : celfmin[k]);
      const unsigned b = (celfmin[k] >= sd ? celfmin[k] - sd : 0);
      cmn[k] = (a > b ? a : b);
      const unsigned e = (celbmax[k] > celfmax[k] ? celbmax[k] : celfmax[k]);
      const unsigned f = celfmax[k] + sd;
      cmx[k] = (e < f ? e : f);
      if (cmx[k] >= c->domcells[k]) cmx[k] = c->domcells[k] - 1;
    }
    if (cmn[0] > cmx[0] || cmn[1] > cmx[1] || cmn[2] > cmx[2]) {
      cmn[0] = cmn[1] = cmn[2] = cmx[0] = cmx[1] = cmx[2] = 0;
    }
  }
  /* PrepareNct (JCellDivCpuSingle.cpp:109-126) */
  d->ncx = d->cellmax[0] - d->cellmin[0] + 1;
  d->ncy = d->cellmax[1] - d->cellmin[1] + 1;
  d->ncz = d->cellmax[2] - d->cellmin[2] + 1;
  d->nsheet = d->ncx * d->ncy;
  d->nct = d->nsheet * d->ncz;
  d->nctt = d->nct * 2 + 5 + 1;
  d->boxboundignore = d->nct;
  d->boxfluid = d->boxboundignore + 1;
  d->boxboundout = d->boxfluid + d->nct;
  d->boxfluidout = d->boxboundout + 1;
  d->boxboundoutignore = d->boxfluidout + 1;
  d->boxfluidoutignore = d->boxboundoutignore + 1;
  if (d->nctt > begincell_cap) return -2;
  /* DivideFull decision (JCellDivCpuSingle.cpp:319-324) */
  if (!d->bounddivideok || memcmp(d->bounddividecellmin, d->cellmin, sizeof(d->cellmin)) ||
      memcmp(d->bounddividecellmax, d->cellmax, sizeof(d->cellmax))) {
    d->dividefull = 1;
    d->bounddivideok = 1;
    memcpy(d->bounddividecellmin, d->cellmin, sizeof(d->cellmin));
    memcpy(d->bounddividecellmax, d->cellmax, sizeof(d->cellmax));
  } else d->dividefull = 0;
  /* PreSortFull / PreSortFluid + MakeSortFull / MakeSortFluid
   * (JCellDivCpuSingle.cpp:137-247): counting sort stable by array index. */
  const unsigned dcc = c->domcellcode;
  const unsigned nboxes = d->nctt - 1;
  unsigned* count = (unsigned*)calloc(nboxes, sizeof(unsigned));
  const unsigned pini = d->dividefull ? 0 : d->npb1;
  const unsigned pfin = d->dividefull ? d->nptot : d->npb1 + d->npf1;
  for (unsigned p = pini; p < pfin; p++) {
    const unsigned rcell = dcell[p];
    const unsigned cx = dcel_cx(dcc, rcell) - d->cellmin[0];
    const unsigned cy = dcel_cy(dcc, rcell) - d->cellmin[1];
    const unsigned cz = dcel_cz(dcc, rcell) - d->cellmin[2];
    const unsigned cellsort = cx + cy * d->ncx + cz * d->nsheet;
    const unsigned rcode = code[p];
    const unsigned ctype = codetype(rcode);
    const unsigned cout = codespecial(rcode);
    unsigned box;
    if (d->dividefull && ctype < ORC_CODE_TYPE_FLOATING) {
      box = (cout < ORC_CODE_OUTIGNORE ? ((cx < d->ncx && cy < d->ncy && cz < d->ncz) ? cellsort : d->boxboundignore)
                                       : (cout == ORC_CODE_OUTIGNORE ? d->boxboundoutignore : d->boxboundout));
    } else {
      box = (cout <= ORC_CODE_OUTIGNORE ? (cout < ORC_CODE_OUTIGNORE ? d->boxfluid + cellsort : d->boxfluidoutignore)
                                        : (ctype == ORC_CODE_TYPE_FLOATING ? d->boxboundout : d->boxfluidout));
    }
    cellpart[p] = box;
    count[box]++;
  }
  if (d->dividefull) {
    begincell[0] = 0;
    for (unsigned box = 0; box < nboxes; box++) begincell[box + 1] = begincell[box] + count[box];
  } else {
    for (unsigned box = d->boxfluid; box < nboxes; box++) begincell[box + 1] = begincell[box] + count[box];
  }
  memset(count, 0, sizeof(unsigned) * nboxes);
  for (unsigned p = pini; p < pfin; p++) {
    const unsigned box = cellpart[p];
    sortpart[begincell[box] + count[box]] = p;
    count[box]++;
  }
  free(count);
  if (!d->dividefull) for (unsigned p = 0; p < d->npb1; p++) sortpart[p] = p;
  /* SortArray(CellPart): cellpart becomes the sorted key list. */
  {
    unsigned* tmp = (unsigned*)malloc(sizeof(unsigned) * (d->nptot ? d->nptot : 1));
    for (unsigned p = pini; p < pfin; p++) tmp[p] = cellpart[sortpart[p]];
    for (unsigned p = pini; p < pfin; p++) cellpart[p] = tmp[p];
    free(tmp);
  }
  /* counts (JCellDivCpuSingle.cpp:330-340) */
  d->npbignore = begincell[d->boxboundignore + 1] - begincell[d->boxboundignore];
  d->npbout = begincell[d->boxboundout + 1] - begincell[d->boxboundout];
  d->npfout = begincell[d->boxfluidout + 1] - begincell[d->boxfluidout];
  d->npboutignore = begincell[d->boxboundoutignore + 1] - begincell[d->boxboundoutignore];
  d->npfoutignore = begincell[d->boxfluidoutignore + 1] - begincell[d->boxfluidoutignore];
  d->npfinal = d->nptot - d->npbout - d->npfout - d->npboutignore - d->npfoutignore;
  d->npbfinal = d->npb1 + d->npb2 - d->npboutignore;
  if (d->npbout != 0 && d->dividefull) d->npbfinal = UINT_MAX;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Neighbour search ranges (JCellSearch_inline.h:33-84).                     */
/* ------------------------------------------------------------------------ */
typedef struct { int cellinit, cxini, cxfin, yini, yfin, zini, zfin; } ngsearch;

static inline ngsearch ngs_from_cell(const orc_ctes* c, const orc_div* d, int cx, int cy, int cz, int boundp2) {
  const int sd = c->cellmode_div;
  const int ncx = (int)d->ncx, ncy = (int)d->ncy, ncz = (int)d->ncz;
  ngsearch r;
  r.cellinit = boundp2 ? 0 : (int)(d->nsheet * d->ncz + 1);
  r.cxini = cx - (cx < sd ? cx : sd);
  r.cxfin = cx + (ncx - cx - 1 < sd ? ncx - cx - 1 : sd) + 1;
  r.yini = cy - (cy < sd ? cy : sd);
  r.yfin = cy + (ncy - cy - 1 < sd ? ncy - cy - 1 : sd) + 1;
  r.zini = cz - (cz < sd ? cz : sd);
  r.zfin = cz + (ncz - cz - 1 < sd ? ncz - cz - 1 : sd) + 1;
  return r;
}

static inline ngsearch ngs_init_dcell(const orc_ctes* c, const orc_div* d, unsigned rcell, int boundp2) {
  const unsigned dcc = c->domcellcode;
  const int cx = (int)dcel_cx(dcc, rcell) - (int)d->cellmin[0];
  const int cy = (int)dcel_cy(dcc, rcell) - (int)d->cellmin[1];
  const int cz = (int)dcel_cz(dcc, rcell) - (int)d->cellmin[2];
  return ngs_from_cell(c, d, cx, cy, cz, boundp2);
}

static inline ngsearch ngs_init_pos(const orc_ctes* c, const orc_div* d, const double* pos, int boundp2) {
  const int cx = (int)((pos[0] - c->domposmin[0]) / c->scell) - (int)d->cellmin[0];
  const int cy = (int)((pos[1] - c->domposmin[1]) / c->scell) - (int)d->cellmin[1];
  const int cz = (int)((pos[2] - c->domposmin[2]) / c->scell) - (int)d->cellmin[2];
  return ngs_from_cell(c, d, cx, cy, cz, boundp2);
}

static inline void particle_range(const orc_div* d, const unsigned* begincell, int y, int z, const ngsearch* g,
                                  unsigned* pini, unsigned* pfin) {
  const int v = (int)d->nsheet * z + (int)d->ncx * y + g->cellinit;
  *pini = begincell[v + g->cxini];
  *pfin = begincell[v + g->cxfin];
}

/* ------------------------------------------------------------------------ */
/* Interaction_Forces: FP32 and FP64 variants generated from one body.       */
/* ------------------------------------------------------------------------ */
#define REAL float
#define RSUF _f32
#define RSQRT sqrtf
#define RPOW powf
#define RBIG FLT_MAX
#include "sph_oracle_forces.inc"
#undef REAL
#undef RSUF
#undef RSQRT
#undef RPOW
#undef RBIG

#define REAL double
#define RSUF _f64
#define RSQRT sqrt
#define RPOW pow
#define RBIG DBL_MAX
#include "sph_oracle_forces.inc"
#undef REAL
#undef RSUF
#undef RSQRT
#undef RPOW
#undef RBIG

void orc_interaction_forces(const orc_ctes* c, const orc_div* d, const unsigned* begincell,
                            unsigned np, unsigned npb, unsigned npbok,
                            const unsigned* dcell, const double* pos, const float* velrho,
                            const uint16_t* code, const float* tau,
                            float* ace, float* ar, float* two_strain, float* viscdt_out, int nthreads,
                            float* shiftpos) {
  interaction_forces_f32(c, d, begincell, np, npb, npbok, dcell, pos, velrho, code, tau, ace, ar, two_strain,
                         viscdt_out, nthreads, NULL, NULL, shiftpos, NULL);
}

void orc_interaction_forces_f64(const orc_ctes* c, const orc_div* d, const unsigned* begincell,
                                unsigned np, unsigned npb, unsigned npbok,
                                const unsigned* dcell, const double* pos, const float* velrho,
                                const uint16_t* code, const double* tau,
                                double* ace, double* ar, double* two_strain, double* viscdt_out, int nthreads,
                                double* absace, double* absar, double* shiftpos, double* absshift) {
  interaction_forces_f64(c, d, begincell, np, npb, npbok, dcell, pos, velrho, code, tau, ace, ar, two_strain,
                         viscdt_out, nthreads, absace, absar, shiftpos, absshift);
}

/* JSphCpu::ComputeSpsTau (JSphCpu.cpp:1279-1309) */
void orc_sps_tau(const orc_ctes* c, unsigned n, unsigned pini, const float* velrho, const float* ts, float* tau) {
  for (unsigned p = pini; p < pini + n; p++) {
    const float* s = ts + 6 * (size_t)p; /* xx,xy,xz,yy,yz,zz */
    const float pow1 = s[0] * s[0] + s[3] * s[3] + s[5] * s[5];
    const float prr = s[1] * s[1] + s[2] * s[2] + s[4] * s[4] + pow1 + pow1;
    const float visc_sps = c->spssmag * sqrtf(prr);
    const float div_u = s[0] + s[3] + s[5];
    const float sps_k = visc_sps * div_u;
    const float sps_blin = c->spsblin * prr;
    const float sumsps = -(sps_k + sps_blin);
    const float twovisc_sps = (visc_sps + visc_sps);
    const float one_rho = 1.0f / velrho[4 * (size_t)p + 3];
    float* t = tau + 6 * (size_t)p;
    t[0] = one_rho * (twovisc_sps * s[0] + sumsps);
    t[1] = one_rho * (visc_sps * s[1]);
    t[2] = one_rho * (visc_sps * s[2]);
    t[3] = one_rho * (twovisc_sps * s[3] + sumsps);
    t[4] = one_rho * (visc_sps * s[4]);
    t[5] = one_rho * (twovisc_sps * s[5] + sumsps);
  }
}

/* ------------------------------------------------------------------------ */
/* mDBC ghost-node correction, SlipMode=vel0, 3-D                            */
/* (JSphCpu_mdbc.cpp:36-160).  The 4x4 moment matrix is accumulated in      */
/* double as the reference CPU does; determinant and the needed entries of   */
/* the inverse are computed by cofactor expansion in double.                 */
/* ------------------------------------------------------------------------ */
static double det3(double a, double b, double c, double d, double e, double f, double g, double h, double i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

/* Solves the first-order extrapolation: returns rho at the boundary particle. */
static float mdbc_solve(const double A[4][4], float rhop1, const float grad[3], const float dpos[3], float rhopzero,
                        int* used) {
  /* cofactor C[i][j] of A; inverse = adj(A)/det with adj = C^T */
  double C[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      double m[9];
      int k = 0;
      for (int r = 0; r < 4; r++) {
        if (r == i) continue;
        for (int s = 0; s < 4; s++) {
          if (s == j) continue;
          m[k++] = A[r][s];
        }
      }
      const double mdet = det3(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]);
      C[i][j] = ((i + j) & 1) ? -mdet : mdet;
    }
  const double det = A[0][0] * C[0][0] + A[0][1] * C[0][1] + A[0][2] * C[0][2] + A[0][3] * C[0][3];
  float rhofinal = FLT_MAX;
  if (fabs(det) >= 1e-3f) {
    /* inv[r][c] = C[c][r]/det */
    const double b[4] = {rhop1, grad[0], grad[1], grad[2]};
    double x[4];
    for (int r = 0; r < 4; r++) x[r] = (C[0][r] * b[0] + C[1][r] * b[1] + C[2][r] * b[2] + C[3][r] * b[3]) / det;
    const float rhoghost = (float)x[0];
    const float grx = -(float)x[1];
    const float gry = -(float)x[2];
    const float grz = -(float)x[3];
    rhofinal = (rhoghost + grx * dpos[0] + gry * dpos[1] + grz * dpos[2]);
    *used = 2;
  } else if (A[0][0] > 0) {
    rhofinal = (float)(rhop1 / A[0][0]);
    *used = 1;
  } else *used = 0;
  return (rhofinal != FLT_MAX ? rhofinal : rhopzero);
}

/* JSph::UpdatePeriodicPos (JSph.cpp:2079-2101): a position outside the real
 * domain comes back across the periodic faces by the axis increments. */
static void update_periodic_pos(const orc_ctes* c, double p[3]) {
  double dx = p[0] - c->maprealposmin[0], dy = p[1] - c->maprealposmin[1], dz = p[2] - c->maprealposmin[2];
  const int out = (dx != dx || dy != dy || dz != dz || dx < 0 || dy < 0 || dz < 0 || dx >= c->maprealsize[0] ||
                   dy >= c->maprealsize[1] || dz >= c->maprealsize[2]);
  if (!out) return;
  for (int k = 0; k < 3; k++) {
    if (!c->peri[k]) continue;
    const double* inc = c->periinc + 3 * k;
    if ((k == 0 ? dx : k == 1 ? dy : dz) < 0) { dx -= inc[0]; dy -= inc[1]; dz -= inc[2]; }
    if ((k == 0 ? dx : k == 1 ? dy : dz) >= c->maprealsize[k]) { dx += inc[0]; dy += inc[1]; dz += inc[2]; }
  }
  p[0] = dx + c->maprealposmin[0];
  p[1] = dy + c->maprealposmin[1];
  p[2] = dz + c->maprealposmin[2];
}

void orc_mdbc_correction(const orc_ctes* c, const orc_div* d, const unsigned* begincell, unsigned n,
                         const double* pos, const uint16_t* code, const float* boundnor, float* velrho,
                         int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(guided)
#endif
  for (int p1 = 0; p1 < (int)n; p1++) {
    if (g_sample_stride > 1 && (p1 % g_sample_stride) != g_sample_phase) continue;  /* rows not sampled keep rho */
    const float* bn = boundnor + 3 * (size_t)p1;
    if (bn[0] == 0 && bn[1] == 0 && bn[2] == 0) continue;
    const double* ps = pos + 3 * (size_t)p1;
    double gp[3] = {ps[0] + (double)bn[0], ps[1] + (double)bn[1], ps[2] + (double)bn[2]};
    /* the ghost node taken back into the domain (JSphCpu_mdbc.cpp:50) */
    if (c->peri[0] || c->peri[1] || c->peri[2]) update_periodic_pos(c, gp);
    float rhop1 = 0;
    float grad[3] = {0, 0, 0};
    double A[4][4];
    memset(A, 0, sizeof(A));
    const ngsearch g = ngs_init_pos(c, d, gp, 0);
    for (int z = g.zini; z < g.zfin; z++)
      for (int y = g.yini; y < g.yfin; y++) {
        unsigned pini, pfin;
        particle_range(d, begincell, y, z, &g, &pini, &pfin);
        for (unsigned p2 = pini; p2 < pfin; p2++) {
          const double* q = pos + 3 * (size_t)p2;
          const float drx = (float)(gp[0] - q[0]);
          const float dry = (float)(gp[1] - q[1]);
          const float drz = (float)(gp[2] - q[2]);
          const float rr2 = (drx * drx + dry * dry + drz * drz);
          if (rr2 <= c->kernelsize2 && codetype(code[p2]) == ORC_CODE_TYPE_FLUID) {
            /* Wendland WabFac (FunSphKernel.h:235-246) */
            const float rad = sqrtf(rr2);
            const float qq = rad / c->kernelh;
            const float wqq1 = 1.f - 0.5f * qq;
            const float wqq2 = wqq1 * wqq1;
            const float fac = c->bwenh * wqq2 * wqq1;
            const float wqq = qq + qq + 1.f;
            const float wab = c->awen * wqq * wqq2 * wqq2;
            const float frx = fac * drx, fry = fac * dry, frz = fac * drz;
            const float rhop2 = velrho[4 * (size_t)p2 + 3];
            const float massp2 = c->massfluid;
            const float volp2 = massp2 / rhop2;
            rhop1 += massp2 * wab;
            grad[0] += massp2 * frx;
            grad[1] += massp2 * fry;
            grad[2] += massp2 * frz;
            const float vwab = wab * volp2;
            const float vfrx = frx * volp2;
            const float vfry = fry * volp2;
            const float vfrz = frz * volp2;
            A[0][0] += vwab; A[0][1] += drx * vwab; A[0][2] += dry * vwab; A[0][3] += drz * vwab;
            A[1][0] += vfrx; A[1][1] += drx * vfrx; A[1][2] += dry * vfrx; A[1][3] += drz * vfrx;
            A[2][0] += vfry; A[2][1] += drx * vfry; A[2][2] += dry * vfry; A[2][3] += drz * vfry;
            A[3][0] += vfrz; A[3][1] += drx * vfrz; A[3][2] += dry * vfrz; A[3][3] += drz * vfrz;
          }
        }
      }
    const float dpos[3] = {bn[0] * (-1.f), bn[1] * (-1.f), bn[2] * (-1.f)};
    int used;
    velrho[4 * (size_t)p1 + 3] = mdbc_solve(A, rhop1, grad, dpos, c->rhopzero, &used);
  }
}

/* The same correction evaluated in double throughout: dr, the kernel and its
 * gradient, the sums (rho, grad rho) and the moment matrix, the solve.  Writes
 * the corrected density of every row p1 < n with a normal to rho64[p1] (the
 * other rows get the state's density); velrho is not changed.  It is the
 * FP64 reference of the mDBC density criterion. */
void orc_mdbc_correction_f64(const orc_ctes* c, const orc_div* d, const unsigned* begincell, unsigned n,
                             const double* pos, const uint16_t* code, const float* boundnor, const float* velrho,
                             double* rho64, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(guided)
#endif
  for (int p1 = 0; p1 < (int)n; p1++) {
    rho64[p1] = velrho[4 * (size_t)p1 + 3];
    if (g_sample_stride > 1 && (p1 % g_sample_stride) != g_sample_phase) continue;
    const float* bn = boundnor + 3 * (size_t)p1;
    if (bn[0] == 0 && bn[1] == 0 && bn[2] == 0) continue;
    const double* ps = pos + 3 * (size_t)p1;
    double gp[3] = {ps[0] + (double)bn[0], ps[1] + (double)bn[1], ps[2] + (double)bn[2]};
    if (c->peri[0] || c->peri[1] || c->peri[2]) update_periodic_pos(c, gp);
    double b[4] = {0, 0, 0, 0};
    double A[4][4];
    memset(A, 0, sizeof(A));
    const double h = c->kernelh, bwenh = c->bwenh, awen = c->awen, ks2 = c->kernelsize2;
    const ngsearch g = ngs_init_pos(c, d, gp, 0);
    for (int z = g.zini; z < g.zfin; z++)
      for (int y = g.yini; y < g.yfin; y++) {
        unsigned pini, pfin;
        particle_range(d, begincell, y, z, &g, &pini, &pfin);
        for (unsigned p2 = pini; p2 < pfin; p2++) {
          const double* q = pos + 3 * (size_t)p2;
          const double drx = gp[0] - q[0], dry = gp[1] - q[1], drz = gp[2] - q[2];
          const double rr2 = drx * drx + dry * dry + drz * drz;
          if (rr2 <= ks2 && codetype(code[p2]) == ORC_CODE_TYPE_FLUID) {
            const double qq = sqrt(rr2) / h;
            const double wqq1 = 1. - 0.5 * qq;
            const double wqq2 = wqq1 * wqq1;
            const double fac = bwenh * wqq2 * wqq1;
            const double wab = awen * (qq + qq + 1.) * wqq2 * wqq2;
            const double fr[3] = {fac * drx, fac * dry, fac * drz};
            const double massp2 = c->massfluid;
            const double volp2 = massp2 / (double)velrho[4 * (size_t)p2 + 3];
            b[0] += massp2 * wab;
            for (int k = 0; k < 3; k++) b[1 + k] += massp2 * fr[k];
            const double row[4] = {wab * volp2, fr[0] * volp2, fr[1] * volp2, fr[2] * volp2};
            for (int r = 0; r < 4; r++) {
              A[r][0] += row[r];
              A[r][1] += drx * row[r];
              A[r][2] += dry * row[r];
              A[r][3] += drz * row[r];
            }
          }
        }
      }
    /* cofactor solve, as mdbc_solve, in double */
    double C[4][4];
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) {
        double m[9];
        int k = 0;
        for (int r = 0; r < 4; r++) {
          if (r == i) continue;
          for (int s = 0; s < 4; s++) {
            if (s == j) continue;
            m[k++] = A[r][s];
          }
        }
        const double mdet = det3(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]);
        C[i][j] = ((i + j) & 1) ? -mdet : mdet;
      }
    const double det = A[0][0] * C[0][0] + A[0][1] * C[0][1] + A[0][2] * C[0][2] + A[0][3] * C[0][3];
    double rho = c->rhopzero;
    if (fabs(det) >= 1e-3) {
      double x[4];
      for (int r = 0; r < 4; r++) x[r] = (C[0][r] * b[0] + C[1][r] * b[1] + C[2][r] * b[2] + C[3][r] * b[3]) / det;
      rho = x[0] - x[1] * -(double)bn[0] - x[2] * -(double)bn[1] - x[3] * -(double)bn[2];
    } else if (A[0][0] > 0) {
      rho = b[0] / A[0][0];
    }
    rho64[p1] = rho;
  }
}

/* Particle-interaction counts (JDsPips.cpp:187-260): out = {checked bound
 * rows, real bound rows, checked fluid rows, real fluid rows}. */
void orc_pips(const orc_ctes* c, const orc_div* d, const unsigned* begincell, unsigned np, unsigned npb,
              unsigned npbok, const unsigned* dcell, const double* pos, unsigned long long out[4], int nthreads) {
  unsigned long long picb = 0, pirb = 0, picf = 0, pirf = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(guided) reduction(+ : picb, pirb)
#endif
  for (int p1 = 0; p1 < (int)npbok; p1++) {
    const double* ps = pos + 3 * (size_t)p1;
    const ngsearch g = ngs_init_dcell(c, d, dcell[p1], 0);
    for (int z = g.zini; z < g.zfin; z++)
      for (int y = g.yini; y < g.yfin; y++) {
        unsigned pini, pfin;
        particle_range(d, begincell, y, z, &g, &pini, &pfin);
        for (unsigned p2 = pini; p2 < pfin; p2++) {
          const double* q = pos + 3 * (size_t)p2;
          const float dx = (float)(ps[0] - q[0]), dy = (float)(ps[1] - q[1]), dz = (float)(ps[2] - q[2]);
          const float rr2 = dx * dx + dy * dy + dz * dz;
          if (rr2 <= c->kernelsize2 && rr2 >= ALMOSTZERO) pirb++;
          picb++;
        }
      }
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(guided) reduction(+ : picf, pirf)
#endif
  for (int p1 = (int)npb; p1 < (int)np; p1++) {
    const double* ps = pos + 3 * (size_t)p1;
    for (int tpfluid = 0; tpfluid <= 1; tpfluid++) {
      const ngsearch g = ngs_init_dcell(c, d, dcell[p1], !tpfluid);
      for (int z = g.zini; z < g.zfin; z++)
        for (int y = g.yini; y < g.yfin; y++) {
          unsigned pini, pfin;
          particle_range(d, begincell, y, z, &g, &pini, &pfin);
          for (unsigned p2 = pini; p2 < pfin; p2++) {
            const double* q = pos + 3 * (size_t)p2;
            const float dx = (float)(ps[0] - q[0]), dy = (float)(ps[1] - q[1]), dz = (float)(ps[2] - q[2]);
            const float rr2 = dx * dx + dy * dy + dz * dz;
            if (rr2 <= c->kernelsize2 && rr2 >= ALMOSTZERO) pirf++;
            picf++;
          }
        }
    }
  }
  out[0] = picb; out[1] = pirb; out[2] = picf; out[3] = pirf;
}

/* ------------------------------------------------------------------------ */
/* dt (JSphCpu.cpp:562-605 VelMax, JSphCpuSingle.cpp:782-843 AceMax,         */
/* JSphCpu.cpp:2035-2078 DtVariable).                                        */
/* ------------------------------------------------------------------------ */
float orc_velmax(unsigned n, const float* velrho) {
  float vmax = 0;
  for (unsigned p = 0; p < n; p++) {
    const float* v = velrho + 4 * (size_t)p;
    const float v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (vmax < v2) vmax = v2;
  }
  return sqrtf(vmax);
}

double orc_acemax(unsigned n, const float* ace) {
  float amax = 0;
  for (unsigned p = 0; p < n; p++) {
    const float* a = ace + 3 * (size_t)p;
    const float a2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (amax < a2) amax = a2;
  }
  return sqrt((double)amax);
}

double orc_dtvariable(const orc_ctes* c, double acemax, float velmax, float viscdtmax, int* err) {
  const double h = (double)c->kernelh;
  const double dt1 = (acemax ? (sqrt(h / acemax)) : DBL_MAX);
  const double vm = velmax * 10.;
  const double dt2 = h / ((c->cs0 > vm ? c->cs0 : vm) + h * viscdtmax);
  const double dt3 = DBL_MAX;
  double dt = c->cflnumber * (dt1 < (dt2 < dt3 ? dt2 : dt3) ? dt1 : (dt2 < dt3 ? dt2 : dt3));
  if (err) *err = 0;
  if (isnan(dt) || isinf(dt)) {
    if (err) *err = 1;
    return dt;
  }
  if (dt < c->dtmin) dt = c->dtmin;
  return dt;
}

/* ------------------------------------------------------------------------ */
/* Whole-solver state: JSphCpuSingle arrays and step driver.                 */
/* ------------------------------------------------------------------------ */
struct orc_sim {
  orc_ctes c;
  orc_div d;
  int nthreads;
  unsigned cap, np, npb, npbok, casenbound;
  unsigned npbper, npfper; /* periodic copies made by the last RunPeriodic */
  double *pos, *pospre;
  float *velrho, *velrhopre, *velrhom1;
  unsigned *idp, *dcell;
  uint16_t* code;
  float *boundnor, *tau, *strain, *ace, *ar;
  float* shiftpos; /* 4 per particle: shifting sums, then displacements (ShiftPosfs_c) */
  unsigned *cellpart, *sortpart, *begincell;
  unsigned begincell_cap;
  void* scratch;
  int pre_active, boundchanged, verletstep;
  double symplecticdtpre, acemax, timestep;
  float velmax, viscdtmax;
  unsigned nout, nstep;
  double t_inter, t_step; /* wall time of the interactions and of the last whole step */
};

static void* xmalloc(size_t n) {
  void* p = malloc(n ? n : 1);
  return p;
}

orc_sim* orc_sim_create(const orc_ctes* c, unsigned np, unsigned npb, const double* pos, const float* velrho,
                        const unsigned* idp, const uint16_t* code, const float* boundnor, int nthreads) {
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  s->c = *c;
  s->nthreads = nthreads;
  s->cap = np;
  s->np = np;
  s->npb = npb;
  s->npbok = npb;
  s->casenbound = npb;
  s->pos = (double*)xmalloc(sizeof(double) * 3 * np);
  s->pospre = (double*)xmalloc(sizeof(double) * 3 * np);
  s->velrho = (float*)xmalloc(sizeof(float) * 4 * np);
  s->velrhopre = (float*)xmalloc(sizeof(float) * 4 * np);
  s->velrhom1 = (float*)xmalloc(sizeof(float) * 4 * np);
  s->idp = (unsigned*)xmalloc(sizeof(unsigned) * np);
  s->dcell = (unsigned*)xmalloc(sizeof(unsigned) * np);
  s->code = (uint16_t*)xmalloc(sizeof(uint16_t) * np);
  s->boundnor = (float*)calloc((size_t)3 * np + 1, sizeof(float));
  s->tau = (float*)calloc((size_t)6 * np + 1, sizeof(float));
  s->strain = (float*)calloc((size_t)6 * np + 1, sizeof(float));
  s->ace = (float*)calloc((size_t)3 * np + 1, sizeof(float));
  s->ar = (float*)calloc((size_t)np + 1, sizeof(float));
  s->shiftpos = (float*)calloc((size_t)4 * np + 1, sizeof(float));
  s->cellpart = (unsigned*)xmalloc(sizeof(unsigned) * np);
  s->sortpart = (unsigned*)xmalloc(sizeof(unsigned) * np);
  const unsigned long long maxnct =
      (unsigned long long)c->domcells[0] * c->domcells[1] * c->domcells[2];
  s->begincell_cap = (unsigned)(maxnct * 2 + 6);
  s->begincell = (unsigned*)calloc(s->begincell_cap, sizeof(unsigned));
  s->scratch = xmalloc(sizeof(double) * 6 * np);
  memcpy(s->pos, pos, sizeof(double) * 3 * np);
  memcpy(s->velrho, velrho, sizeof(float) * 4 * np);
  memcpy(s->idp, idp, sizeof(unsigned) * np);
  memcpy(s->code, code, sizeof(uint16_t) * np);
  if (boundnor) {
    /* JSph::ConfigBoundNormals (JSph.cpp:1411-1418): normals are doubled */
    for (unsigned p = 0; p < np; p++)
      for (int k = 0; k < 3; k++) s->boundnor[3 * p + k] = (idp[p] < npb ? boundnor[3 * p + k] * 2.f : 0.f);
  }
  orc_load_dcell(c, np, s->code, s->pos, s->dcell);
  /* InitRun (JSph.cpp:2206-2210, JSphCpu.cpp:472-482) */
  s->symplecticdtpre = c->dtini;
  if (c->tstep == ORC_STEP_VERLET) memcpy(s->velrhom1, s->velrho, sizeof(float) * 4 * np);
  s->boundchanged = 1;
  if (orc_sim_run_cell_divide(s)) {
    orc_sim_destroy(s);
    return NULL;
  }
  return s;
}

void orc_sim_destroy(orc_sim* s) {
  if (!s) return;
  free(s->pos); free(s->pospre); free(s->velrho); free(s->velrhopre); free(s->velrhom1);
  free(s->idp); free(s->dcell); free(s->code); free(s->boundnor); free(s->tau); free(s->strain);
  free(s->ace); free(s->ar); free(s->shiftpos); free(s->cellpart); free(s->sortpart); free(s->begincell); free(s->scratch);
  free(s);
}

/* Grows every per-particle array to hold n particles (ResizeParticlesSizeData). */
static void ensure_cap(orc_sim* s, unsigned n) {
  if (n <= s->cap) return;
  const unsigned cap = n + n / 4 + 64;
#define GROW(T, ARR, W) do { T* q_ = (T*)calloc((size_t)(W) * cap + 1, sizeof(T)); \
    memcpy(q_, (ARR), sizeof(T) * (W) * (size_t)s->cap); free(ARR); (ARR) = q_; } while (0)
  GROW(double, s->pos, 3); GROW(double, s->pospre, 3);
  GROW(float, s->velrho, 4); GROW(float, s->velrhopre, 4); GROW(float, s->velrhom1, 4);
  GROW(unsigned, s->idp, 1); GROW(unsigned, s->dcell, 1); GROW(uint16_t, s->code, 1);
  GROW(float, s->boundnor, 3); GROW(float, s->tau, 6); GROW(float, s->strain, 6);
  GROW(float, s->ace, 3); GROW(float, s->ar, 1); GROW(float, s->shiftpos, 4);
  GROW(unsigned, s->cellpart, 1); GROW(unsigned, s->sortpart, 1);
#undef GROW
  free(s->scratch);
  s->scratch = xmalloc(sizeof(double) * 6 * cap);
  s->cap = cap;
}

/* JSphCpuSingle::RunPeriodic (JSphCpuSingle.cpp:416-504) with PeriodicMakeList
 * and PeriodicDuplicate* (JSphCpuSingle.cpp:210-356): the periodic copies of
 * the last divide are marked to be ignored; every particle within reach of a
 * periodic face gets a copy moved by the increment, appended after the np
 * particles, boundary copies then fluid ones, axis by axis (copies made for
 * one axis are themselves copied for the next). */
static void run_periodic(orc_sim* s) {
  const orc_ctes* c = &s->c;
  for (unsigned p = 0; p < s->np; p++)
    if (codespecial(s->code[p]) == ORC_CODE_PERIODIC)
      s->code[p] = (uint16_t)((s->code[p] & ~ORC_CODE_MASKSPECIAL) | ORC_CODE_OUTIGNORE);
  const unsigned npb0 = s->npb, npf0 = s->np - s->npb;
  s->npbper = s->npfper = 0;
  s->boundchanged = 1;
  unsigned* list = NULL;
  for (int ctype = 0; ctype < 2; ctype++) {
    const unsigned pini = ctype ? npb0 : 0, num = ctype ? npf0 : npb0;
    for (int cper = 0; cper < 3; cper++) {
      if (!c->peri[cper]) continue;
      const double* inc = c->periinc + 3 * cper;
      for (int cblock = 0; cblock < 2; cblock++) {
        const unsigned nper = ctype ? s->npfper : s->npbper;
        const unsigned pini2 = cblock ? pini : s->np - nper, num2 = cblock ? num : nper;
        if (!num2) continue;
        /* PeriodicMakeList */
        list = (unsigned*)realloc(list, sizeof(unsigned) * 2 * (size_t)num2 + 1);
        unsigned count = 0;
        for (unsigned p2 = pini2; p2 < pini2 + num2; p2++) {
          if (codespecial(s->code[p2]) > ORC_CODE_PERIODIC) continue;
          const double* ps = s->pos + 3 * (size_t)p2;
          for (int sgn = 0; sgn < 2; sgn++) {
            double q[3];
            for (int k = 0; k < 3; k++) q[k] = sgn ? ps[k] - inc[k] : ps[k] + inc[k];
            if (c->mapposmin[0] <= q[0] && c->mapposmin[1] <= q[1] && c->mapposmin[2] <= q[2] &&
                q[0] < c->mapposmax[0] && q[1] < c->mapposmax[1] && q[2] < c->mapposmax[2])
              list[count++] = sgn ? (p2 | 0x80000000u) : p2;
          }
        }
        /* PeriodicDuplicateSymplectic / PeriodicDuplicateVerlet / Normals */
        ensure_cap(s, s->np + count);
        for (unsigned i = 0; i < count; i++) {
          const unsigned pnew = s->np + i, rp = list[i], pcopy = rp & 0x7fffffffu;
          const int inverse = rp >= 0x80000000u;
          double ps[3];
          for (int k = 0; k < 3; k++) ps[k] = s->pos[3 * (size_t)pcopy + k];
          ps[0] += (inverse ? -inc[0] : inc[0]);
          ps[1] += (inverse ? -inc[1] : inc[1]);
          ps[2] += (inverse ? -inc[2] : inc[2]);
          unsigned cx = (unsigned)((ps[0] - c->domposmin[0]) / c->scell);
          unsigned cy = (unsigned)((ps[1] - c->domposmin[1]) / c->scell);
          unsigned cz = (unsigned)((ps[2] - c->domposmin[2]) / c->scell);
          cx = (cx <= c->domcells[0] ? cx : c->domcells[0]);
          cy = (cy <= c->domcells[1] ? cy : c->domcells[1]);
          cz = (cz <= c->domcells[2] ? cz : c->domcells[2]);
          for (int k = 0; k < 3; k++) s->pos[3 * (size_t)pnew + k] = ps[k];
          s->dcell[pnew] = dcel_cell(c->domcellcode, cx, cy, cz);
          s->idp[pnew] = s->idp[pcopy];
          s->code[pnew] = (uint16_t)((s->code[pcopy] & ~ORC_CODE_MASKSPECIAL) | ORC_CODE_PERIODIC);
          memcpy(s->velrho + 4 * (size_t)pnew, s->velrho + 4 * (size_t)pcopy, sizeof(float) * 4);
          if (c->tstep == ORC_STEP_VERLET) memcpy(s->velrhom1 + 4 * (size_t)pnew, s->velrhom1 + 4 * (size_t)pcopy, sizeof(float) * 4);
          else if (s->pre_active) {
            memcpy(s->pospre + 3 * (size_t)pnew, s->pospre + 3 * (size_t)pcopy, sizeof(double) * 3);
            memcpy(s->velrhopre + 4 * (size_t)pnew, s->velrhopre + 4 * (size_t)pcopy, sizeof(float) * 4);
          }
          if (c->tvisco == ORC_VISCO_LAMINARSPS) memcpy(s->tau + 6 * (size_t)pnew, s->tau + 6 * (size_t)pcopy, sizeof(float) * 6);
          if (c->tboundary == ORC_BC_MDBC) memcpy(s->boundnor + 3 * (size_t)pnew, s->boundnor + 3 * (size_t)pcopy, sizeof(float) * 3);
        }
        s->np += count;
        if (!ctype) s->npbper += count; else s->npfper += count;
      }
    }
  }
  free(list);
}

#define SORT_ARRAY(T, ARR, W)                                                            \
  do {                                                                                   \
    T* tmp_ = (T*)s->scratch;                                                            \
    for (unsigned p_ = ini; p_ < n; p_++)                                                \
      for (int k_ = 0; k_ < (W); k_++) tmp_[(size_t)(W)*p_ + k_] = (ARR)[(size_t)(W)*sp[p_] + k_]; \
    memcpy((ARR) + (size_t)(W)*ini, tmp_ + (size_t)(W)*ini, sizeof(T) * (W) * (n - ini)); \
  } while (0)

/* JSphCpuSingle::RunCellDivide (JSphCpuSingle.cpp:510-590), no periodicity. */
int orc_sim_run_cell_divide(orc_sim* s) {
  s->npbper = s->npfper = 0;
  if (s->c.peri[0] || s->c.peri[1] || s->c.peri[2]) run_periodic(s);
  const unsigned npf = s->np - s->npb - s->npbper - s->npfper;
  int r = orc_divide(&s->c, &s->d, s->npb, npf, s->npbper, s->npfper, s->boundchanged, s->dcell, s->code, s->cellpart, s->sortpart,
                     s->begincell, s->begincell_cap);
  if (r) return r;
  const unsigned n = s->d.nptot;
  const unsigned ini = s->d.dividefull ? 0 : s->d.npbfinal;
  const unsigned* sp = s->sortpart;
  SORT_ARRAY(unsigned, s->idp, 1);
  SORT_ARRAY(uint16_t, s->code, 1);
  SORT_ARRAY(unsigned, s->dcell, 1);
  SORT_ARRAY(double, s->pos, 3);
  SORT_ARRAY(float, s->velrho, 4);
  if (s->c.tstep == ORC_STEP_VERLET) SORT_ARRAY(float, s->velrhom1, 4);
  else if (s->pre_active) {
    SORT_ARRAY(double, s->pospre, 3);
    SORT_ARRAY(float, s->velrhopre, 4);
  }
  if (s->c.tvisco == ORC_VISCO_LAMINARSPS) SORT_ARRAY(float, s->tau, 6);
  if (s->c.tboundary == ORC_BC_MDBC) SORT_ARRAY(float, s->boundnor, 3);
  s->np = s->d.npfinal;
  s->npb = s->d.npbfinal;
  if (s->d.npbout) return -3; /* AbortBoundOut (JSphCpuSingle.cpp:593) */
  s->npbok = s->npb - s->d.npbignore;
  s->nout += s->d.npfout;
  s->boundchanged = 0;
  return 0;
}

/* JSphCpuSingle::MdbcBoundCorrection (JSphCpuSingle.cpp:754-780), vel0. */
void orc_sim_mdbc_f64(orc_sim* s, double* rho64) {
  orc_mdbc_correction_f64(&s->c, &s->d, s->begincell, s->npbok, s->pos, s->code, s->boundnor, s->velrho, rho64,
                          s->nthreads);
}

int orc_sim_mdbc(orc_sim* s, int corrector) {
  if (s->c.tboundary != ORC_BC_MDBC || corrector) return 0;
  orc_mdbc_correction(&s->c, &s->d, s->begincell, s->npbok, s->pos, s->code, s->boundnor, s->velrho, s->nthreads);
  return 0;
}

/* PreInteraction_Forces + Interaction_Forces (JSphCpu.cpp:488-547,
 * JSphCpuSingle.cpp:685-748). */
int orc_sim_interaction(orc_sim* s) {
  const double t0 = orc_now();
  const unsigned pini = (s->c.dtallparticles ? 0 : s->npb);
  s->velmax = orc_velmax(s->np - pini, s->velrho + 4 * (size_t)pini);
  float viscdt = 0;
  orc_interaction_forces(&s->c, &s->d, s->begincell, s->np, s->npb, s->npbok, s->dcell, s->pos, s->velrho, s->code,
                         s->tau, s->ace, s->ar, s->strain, &viscdt, s->nthreads, s->c.tshift ? s->shiftpos : NULL);
  s->viscdtmax = viscdt;
  /* ComputeSpsTau runs inside the interaction (JSphCpu.cpp:1366-1367) */
  if (s->c.tvisco == ORC_VISCO_LAMINARSPS) orc_sps_tau(&s->c, s->np - s->npb, s->npb, s->velrho, s->strain, s->tau);
  s->acemax = orc_acemax(s->np - s->npb, s->ace + 3 * (size_t)s->npb);
  s->t_inter += orc_now() - t0;
  return 0;
}

double orc_sim_dtvariable(orc_sim* s, int* err) {
  return orc_dtvariable(&s->c, s->acemax, s->velmax, s->viscdtmax, err);
}

/* JSphCpu::UpdatePos (JSphCpu.cpp:1464-1516), no periodicity. */
static void update_pos(const orc_ctes* c, const double* rpos0, double movx, double movy, double movz, int outrho,
                       unsigned p, double* pos, unsigned* cell, uint16_t* code) {
  const int outmov = (fabsf((float)movx) > c->movlimit || fabsf((float)movy) > c->movlimit ||
                      fabsf((float)movz) > c->movlimit);
  double rx = rpos0[0] + movx, ry = rpos0[1] + movy, rz = rpos0[2] + movz;
  double dx = rx - c->maprealposmin[0];
  double dy = ry - c->maprealposmin[1];
  double dz = rz - c->maprealposmin[2];
  int out = (dx != dx || dy != dy || dz != dz || dx < 0 || dy < 0 || dz < 0 || dx >= c->maprealsize[0] ||
             dy >= c->maprealsize[1] || dz >= c->maprealsize[2]);
  const int periactive = c->peri[0] || c->peri[1] || c->peri[2];
  if (periactive && out) {
    /* back into the domain across a periodic face (JSphCpu.cpp:1477-1494) */
    const double* inc = c->periinc;
    if (c->peri[0]) {
      if (dx < 0) { dx -= inc[0]; dy -= inc[1]; dz -= inc[2]; }
      if (dx >= c->maprealsize[0]) { dx += inc[0]; dy += inc[1]; dz += inc[2]; }
    }
    if (c->peri[1]) {
      if (dy < 0) { dx -= inc[3]; dy -= inc[4]; dz -= inc[5]; }
      if (dy >= c->maprealsize[1]) { dx += inc[3]; dy += inc[4]; dz += inc[5]; }
    }
    if (c->peri[2]) {
      if (dz < 0) { dx -= inc[6]; dy -= inc[7]; dz -= inc[8]; }
      if (dz >= c->maprealsize[2]) { dx += inc[6]; dy += inc[7]; dz += inc[8]; }
    }
    const int outx = !c->peri[0] && (dx < 0 || dx >= c->maprealsize[0]);
    const int outy = !c->peri[1] && (dy < 0 || dy >= c->maprealsize[1]);
    const int outz = !c->peri[2] && (dz < 0 || dz >= c->maprealsize[2]);
    out = outx || outy || outz;
    rx = dx + c->maprealposmin[0]; ry = dy + c->maprealposmin[1]; rz = dz + c->maprealposmin[2];
  }
  pos[3 * (size_t)p] = rx; pos[3 * (size_t)p + 1] = ry; pos[3 * (size_t)p + 2] = rz;
  if (periactive && !(outrho || outmov || out)) {
    dx = rx - c->domposmin[0];
    dy = ry - c->domposmin[1];
    dz = rz - c->domposmin[2];
  }
  if (outrho || outmov || out) {
    uint16_t rcode = code[p];
    const uint16_t base = (uint16_t)(rcode & ~ORC_CODE_MASKSPECIAL);
    if (out) rcode = (uint16_t)(base | ORC_CODE_OUTPOS);
    else if (outrho) rcode = (uint16_t)(base | ORC_CODE_OUTRHO);
    else rcode = (uint16_t)(base | ORC_CODE_OUTMOV);
    code[p] = rcode;
    cell[p] = 0xffffffffu;
  } else {
    const unsigned cx = (unsigned)(dx / c->scell), cy = (unsigned)(dy / c->scell), cz = (unsigned)(dz / c->scell);
    cell[p] = dcel_cell(c->domcellcode, cx, cy, cz);
  }
}

/* JSphCpu::ComputeSymplecticPre (JSphCpu.cpp:1687-1844). */
int orc_sim_symplectic_pre(orc_sim* s, double dt) {
  const orc_ctes* c = &s->c;
  const int periactive = c->peri[0] || c->peri[1] || c->peri[2];
  const double dt05 = dt * .5;
  const int np = (int)s->np, npb = (int)s->npb;
  memcpy(s->pospre, s->pos, sizeof(double) * 3 * (size_t)np);
  memcpy(s->velrhopre, s->velrho, sizeof(float) * 4 * (size_t)np);
  s->pre_active = 1;
  for (int p = 0; p < npb; p++) {
    float* vr = s->velrho + 4 * (size_t)p;
    const float* vp = s->velrhopre + 4 * (size_t)p;
    vr[0] = vp[0]; vr[1] = vp[1]; vr[2] = vp[2];
    float w = (float)((double)vp[3] + dt05 * s->ar[p]);
    vr[3] = (w < c->rhopzero ? c->rhopzero : w);
  }
  double* mov = (double*)s->scratch;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int p = npb; p < np; p++) {
    const uint16_t rcode = s->code[p];
    const float* vp = s->velrhopre + 4 * (size_t)p;
    const float* a = s->ace + 3 * (size_t)p;
    const float rhonew = (float)((double)vp[3] + dt05 * s->ar[p]);
    /* no shifting in the predictor: the reference applies it in the corrector
       only (shift=false in ComputeSymplecticPre, JSphCpu.cpp:1689) */
    const double dx = (double)vp[0] * dt05;
    const double dy = (double)vp[1] * dt05;
    const double dz = (double)vp[2] * dt05;
    const int outrho = (rhonew < c->rhopoutmin || rhonew > c->rhopoutmax);
    float* vr = s->velrho + 4 * (size_t)p;
    vr[0] = (float)((double)vp[0] + ((double)a[0] + c->gravity[0]) * dt05);
    vr[1] = (float)((double)vp[1] + ((double)a[1] + c->gravity[1]) * dt05);
    vr[2] = (float)((double)vp[2] + ((double)a[2] + c->gravity[2]) * dt05);
    vr[3] = rhonew;
    mov[3 * (size_t)p] = dx; mov[3 * (size_t)p + 1] = dy; mov[3 * (size_t)p + 2] = dz;
    if (outrho && codespecial(rcode) == ORC_CODE_NORMAL) s->code[p] = (uint16_t)((rcode & ~ORC_CODE_MASKSPECIAL) | ORC_CODE_OUTRHO);
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int p = npb; p < np; p++) {
    const uint16_t rcode = s->code[p];
    const int outrho = (codespecial(rcode) == ORC_CODE_OUTRHO);
    /* periodic copies are not moved (JSphCpu.cpp:1816-1817, 2000-2001) */
    if (periactive && !outrho && codespecial(rcode) != ORC_CODE_NORMAL) continue;
    if (codetype(rcode) == ORC_CODE_TYPE_FLUID)
      update_pos(c, s->pospre + 3 * (size_t)p, mov[3 * (size_t)p], mov[3 * (size_t)p + 1], mov[3 * (size_t)p + 2],
                 outrho, (unsigned)p, s->pos, s->dcell, s->code);
    else memcpy(s->pos + 3 * (size_t)p, s->pospre + 3 * (size_t)p, sizeof(double) * 3);
  }
  memcpy(s->pos, s->pospre, sizeof(double) * 3 * (size_t)npb);
  return 0;
}

/* JSphShifting::RunCpu (JSphShifting.cpp:390-418): the shifting sums of each
 * fluid particle become its displacement, proportional to dt*coef*h*|v|, cut
 * below the free-surface threshold and limited to dp/10; a particle whose
 * sums were cancelled near the boundary gets none. */
int orc_sim_run_shifting(orc_sim* s, double dt) {
  const orc_ctes* c = &s->c;
  if (!c->tshift) return 0;
  const double coefumagn = dt * c->shiftcoef * c->kernelh;
  const double coeftfs = (c->simulate2d ? 2.0 : 3.0) - c->shifttfs;
  const float maxdist = (float)(c->dp * 0.1);
  for (unsigned p = s->npb; p < s->np; p++) {
    float* rs = s->shiftpos + 4 * (size_t)p;
    if (rs[0] != FLT_MAX) {
      const float* v = s->velrho + 4 * (size_t)p;
      const double vx = (double)v[0], vy = (double)v[1], vz = (double)v[2];
      double umagn = coefumagn * sqrt(vx * vx + vy * vy + vz * vz);
      if (c->shifttfs) {
        if (rs[3] < c->shifttfs) umagn = 0;
        else umagn *= ((double)rs[3] - c->shifttfs) / coeftfs;
      }
      for (int k = 0; k < 3; k++) {
        const float d = (float)((double)rs[k] * umagn);
        rs[k] = (fabsf(d) < maxdist ? d : (d >= 0 ? maxdist : -maxdist));
      }
    } else {
      rs[0] = rs[1] = rs[2] = rs[3] = 0;
    }
  }
  return 0;
}

void orc_sim_get_shiftpos(const orc_sim* s, float* out) {
  memcpy(out, s->shiftpos, sizeof(float) * 4 * (size_t)s->np);
}

void orc_sim_set_shiftpos(orc_sim* s, const float* in) {
  memcpy(s->shiftpos, in, sizeof(float) * 4 * (size_t)s->np);
}

/* JSphCpu::ComputeSymplecticCorr (JSphCpu.cpp:1850-2029). */
int orc_sim_symplectic_cor(orc_sim* s, double dt) {
  const orc_ctes* c = &s->c;
  const int periactive = c->peri[0] || c->peri[1] || c->peri[2];
  const double dt05 = dt * .5;
  const int np = (int)s->np, npb = (int)s->npb;
  for (int p = 0; p < npb; p++) {
    float* vr = s->velrho + 4 * (size_t)p;
    const float* vp = s->velrhopre + 4 * (size_t)p;
    const double epsilon_rdot = (-(double)s->ar[p] / (double)vr[3]) * dt;
    const float rhonew = (float)((double)vp[3] * (2. - epsilon_rdot) / (2. + epsilon_rdot));
    vr[0] = 0; vr[1] = 0; vr[2] = 0;
    vr[3] = (rhonew < c->rhopzero ? c->rhopzero : rhonew);
  }
  double* mov = (double*)s->scratch;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int p = npb; p < np; p++) {
    const uint16_t rcode = s->code[p];
    float* vr = s->velrho + 4 * (size_t)p;
    const float* vp = s->velrhopre + 4 * (size_t)p;
    const float* a = s->ace + 3 * (size_t)p;
    const double epsilon_rdot = (-(double)s->ar[p] / (double)vr[3]) * dt;
    const float rhonew = (float)((double)vp[3] * (2. - epsilon_rdot) / (2. + epsilon_rdot));
    const float nx = (float)((double)vp[0] + ((double)a[0] + c->gravity[0]) * dt);
    const float ny = (float)((double)vp[1] + ((double)a[1] + c->gravity[1]) * dt);
    const float nz = (float)((double)vp[2] + ((double)a[2] + c->gravity[2]) * dt);
    double dx = ((double)vp[0] + (double)nx) * dt05;
    double dy = ((double)vp[1] + (double)ny) * dt05;
    double dz = ((double)vp[2] + (double)nz) * dt05;
    if (c->tshift) {
      const float* sh = s->shiftpos + 4 * (size_t)p;
      dx += (double)sh[0]; dy += (double)sh[1]; dz += (double)sh[2];
    }
    const int outrho = (rhonew < c->rhopoutmin || rhonew > c->rhopoutmax);
    mov[3 * (size_t)p] = dx; mov[3 * (size_t)p + 1] = dy; mov[3 * (size_t)p + 2] = dz;
    if (outrho && codespecial(rcode) == ORC_CODE_NORMAL) s->code[p] = (uint16_t)((rcode & ~ORC_CODE_MASKSPECIAL) | ORC_CODE_OUTRHO);
    vr[0] = nx; vr[1] = ny; vr[2] = nz; vr[3] = rhonew;
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int p = npb; p < np; p++) {
    const uint16_t rcode = s->code[p];
    const int outrho = (codespecial(rcode) == ORC_CODE_OUTRHO);
    /* periodic copies are not moved (JSphCpu.cpp:1816-1817, 2000-2001) */
    if (periactive && !outrho && codespecial(rcode) != ORC_CODE_NORMAL) continue;
    if (codetype(rcode) == ORC_CODE_TYPE_FLUID)
      update_pos(c, s->pospre + 3 * (size_t)p, mov[3 * (size_t)p], mov[3 * (size_t)p + 1], mov[3 * (size_t)p + 2],
                 outrho, (unsigned)p, s->pos, s->dcell, s->code);
    else memcpy(s->pos + 3 * (size_t)p, s->pospre + 3 * (size_t)p, sizeof(double) * 3);
  }
  s->pre_active = 0;
  return 0;
}

/* JSphCpu::ComputeVerlet + ComputeVerletVarsFluid + ComputeVelrhoBound
 * (JSphCpu.cpp:1523-1680). */
int orc_sim_verlet(orc_sim* s, double dt) {
  const orc_ctes* c = &s->c;
  const int np = (int)s->np, npb = (int)s->npb;
  s->verletstep++;
  const int euler = !(s->verletstep < c->verletsteps);
  const double dt2 = euler ? dt : dt + dt;
  const float* velrho2 = euler ? s->velrho : s->velrhom1; /* density/velocity base */
  const double dt205 = 0.5 * dt * dt;
  const double g[3] = {(double)c->gravity[0], (double)c->gravity[1], (double)c->gravity[2]};
  float* newv = (float*)s->scratch; /* new velrho into scratch, then swap into velrhom1 */
  for (int p = npb; p < np; p++) {
    const float* v1 = s->velrho + 4 * (size_t)p;
    const float* v2 = velrho2 + 4 * (size_t)p;
    const float* a = s->ace + 3 * (size_t)p;
    const float rhonew = (float)((double)v2[3] + dt2 * s->ar[p]);
    const double ax = (double)a[0] + g[0], ay = (double)a[1] + g[1], az = (double)a[2] + g[2];
    double dx = (double)v1[0] * dt + ax * dt205;
    double dy = (double)v1[1] * dt + ay * dt205;
    double dz = (double)v1[2] * dt + az * dt205;
    if (c->tshift) {
      const float* sh = s->shiftpos + 4 * (size_t)p;
      dx += (double)sh[0]; dy += (double)sh[1]; dz += (double)sh[2];
    }
    const int outrho = (rhonew < c->rhopoutmin || rhonew > c->rhopoutmax);
    float* nv = newv + 4 * (size_t)p;
    nv[0] = (float)((double)v2[0] + ax * dt2);
    nv[1] = (float)((double)v2[1] + ay * dt2);
    nv[2] = (float)((double)v2[2] + az * dt2);
    nv[3] = rhonew;
    double rp[3] = {s->pos[3 * (size_t)p], s->pos[3 * (size_t)p + 1], s->pos[3 * (size_t)p + 2]};
    update_pos(c, rp, dx, dy, dz, outrho, (unsigned)p, s->pos, s->dcell, s->code);
  }
  for (int p = 0; p < npb; p++) {
    const float* vo = (euler ? s->velrho : s->velrhom1) + 4 * (size_t)p;
    const float rhonew = (float)((double)vo[3] + dt2 * s->ar[p]);
    float* nv = newv + 4 * (size_t)p;
    nv[0] = 0; nv[1] = 0; nv[2] = 0;
    nv[3] = (rhonew < c->rhopzero ? c->rhopzero : rhonew);
  }
  if (euler) s->verletstep = 0;
  /* VelrhoM1 <- old Velrho, Velrho <- new */
  memcpy(s->velrhom1, s->velrho, sizeof(float) * 4 * (size_t)np);
  memcpy(s->velrho, newv, sizeof(float) * 4 * (size_t)np);
  return 0;
}

/* One JSphCpuSingle::Run iteration: ComputeStep + RunCellDivide
 * (JSphCpuSingle.cpp:873-936, 1184-1190). */
int orc_sim_step(orc_sim* s, double* dtused) {
  int err = 0, r;
  const double t0 = orc_now();
  s->t_inter = 0;
  if (s->c.tstep == ORC_STEP_SYMPLECTIC) {
    const double dt = s->symplecticdtpre;
    orc_sim_mdbc(s, 0);
    orc_sim_interaction(s);
    const double dt_p = orc_sim_dtvariable(s, &err);
    if (err) return -4;
    orc_sim_run_shifting(s, dt * .5);
    orc_sim_symplectic_pre(s, dt);
    if ((r = orc_sim_run_cell_divide(s))) return r;
    orc_sim_mdbc(s, 1);
    orc_sim_interaction(s);
    const double dt_c = orc_sim_dtvariable(s, &err);
    if (err) return -4;
    orc_sim_run_shifting(s, dt);
    orc_sim_symplectic_cor(s, dt);
    s->symplecticdtpre = (dt_p < dt_c ? dt_p : dt_c);
    if (dtused) *dtused = dt;
    s->timestep += dt;
  } else {
    orc_sim_mdbc(s, 0);
    orc_sim_interaction(s);
    const double dt = orc_sim_dtvariable(s, &err);
    if (err) return -4;
    orc_sim_run_shifting(s, dt);
    orc_sim_verlet(s, dt);
    if (dtused) *dtused = dt;
    s->timestep += dt;
  }
  s->nstep++;
  r = orc_sim_run_cell_divide(s);
  s->t_step = orc_now() - t0;
  return r;
}

void orc_sim_times(const orc_sim* s, double* t_inter, double* t_step) {
  if (t_inter) *t_inter = s->t_inter;
  if (t_step) *t_step = s->t_step;
}

unsigned orc_sim_np(const orc_sim* s) { return s->np; }
unsigned orc_sim_npb(const orc_sim* s) { return s->npb; }
unsigned orc_sim_npbok(const orc_sim* s) { return s->npbok; }
const orc_div* orc_sim_div(const orc_sim* s) { return &s->d; }
unsigned orc_sim_nout(const orc_sim* s) { return s->nout; }
double orc_sim_time(const orc_sim* s) { return s->timestep; }

void orc_sim_get(const orc_sim* s, double* pos, float* velrho, unsigned* idp, uint16_t* code, unsigned* dcell) {
  const size_t n = s->np;
  if (pos) memcpy(pos, s->pos, sizeof(double) * 3 * n);
  if (velrho) memcpy(velrho, s->velrho, sizeof(float) * 4 * n);
  if (idp) memcpy(idp, s->idp, sizeof(unsigned) * n);
  if (code) memcpy(code, s->code, sizeof(uint16_t) * n);
  if (dcell) memcpy(dcell, s->dcell, sizeof(unsigned) * n);
}

void orc_sim_get_forces(const orc_sim* s, float* ace, float* ar) {
  if (ace) memcpy(ace, s->ace, sizeof(float) * 3 * (size_t)s->np);
  if (ar) memcpy(ar, s->ar, sizeof(float) * (size_t)s->np);
}

void orc_sim_get_begincell(const orc_sim* s, unsigned* begincell, unsigned n) {
  memcpy(begincell, s->begincell, sizeof(unsigned) * n);
}

void orc_sim_get_sortpart(const orc_sim* s, unsigned* sortpart, unsigned* cellpart) {
  if (sortpart) memcpy(sortpart, s->sortpart, sizeof(unsigned) * s->d.nptot);
  if (cellpart) memcpy(cellpart, s->cellpart, sizeof(unsigned) * s->d.nptot);
}

void orc_sim_maxes(const orc_sim* s, double* acemax, float* velmax, float* viscdtmax, double* dtpre) {
  if (acemax) *acemax = s->acemax;
  if (velmax) *velmax = s->velmax;
  if (viscdtmax) *viscdtmax = s->viscdtmax;
  if (dtpre) *dtpre = s->symplecticdtpre;
}

void orc_sim_set_dtpre(orc_sim* s, double dt) { s->symplecticdtpre = dt; }

void orc_sim_set_forces(orc_sim* s, const float* ace, const float* ar) {
  if (ace) memcpy(s->ace, ace, sizeof(float) * 3 * (size_t)s->np);
  if (ar) memcpy(s->ar, ar, sizeof(float) * (size_t)s->np);
}

void orc_sim_set_state(orc_sim* s, const double* pos, const float* velrho) {
  if (pos) memcpy(s->pos, pos, sizeof(double) * 3 * (size_t)s->np);
  if (velrho) memcpy(s->velrho, velrho, sizeof(float) * 4 * (size_t)s->np);
}
