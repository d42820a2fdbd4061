// gbsph_config.cpp -- derivation of the case constants (host side).
//
// gbsph_config() computes what JSph::LoadConfigCtes (JSph.cpp:642-658),
// ConfigConstants1/2 (JSph.cpp:1481-1546), ConfigCellDivision
// (JSph.cpp:1877-1895) and SelecDomain(0,Map_Cells) (JSph.cpp:1901-1944)
// compute, with the reference's member types (float/double), so the kernels see
// the same constants as the reference solver.
#include <cmath>
#include <cstring>

#include "gbsph.h"

namespace {

// JDsDcell::CalcBitsValue / CalcCellDistribution / CalcCellCode
// (JDsDcell.cpp:34-72): bits per axis for a 31-bit cell code (+1 bit in x).
unsigned cell_bits(unsigned v) {
  unsigned n = 2;
  while (v >> n) n++;
  return n;
}

unsigned cell_code(unsigned nx, unsigned ny, unsigned nz) {
  unsigned sx = cell_bits(nx), sy = cell_bits(ny), sz = cell_bits(nz);
  if (sx + sy + sz > 31) return 0;
  unsigned rest = 31 - (sx + sy + sz);
  while (rest) {
    if (rest) { sx++; rest--; }
    if (rest) { sy++; rest--; }
    if (rest) { sz++; rest--; }
  }
  return ((sx + 1) << 25) | (sy << 20) | (sz << 15) | ((sy + sz) << 10) | ((sx + 1 + sz) << 5) | (sx + 1 + sy);
}

}  // namespace

extern "C" int gbsph_config(const gbsph_params* p, gbsph_consts* c) {
  if (!p || !c) return GBSPH_EINVAL;
  if (p->simulate2d) return GBSPH_EINVAL;  // the 3-D path only
  if (p->dp <= 0 || p->h <= 0 || p->b <= 0 || p->rhop0 <= 0) return GBSPH_EINVAL;
  std::memset(c, 0, sizeof(*c));
  c->tstep = p->tstep;
  c->tvisco = p->tvisco;
  c->tdensity = p->tdensity;
  c->tboundary = p->tboundary;
  // standard shifting (JSph.cpp:744-759); advanced shifting (4) is not built
  if (p->tshift < 0 || p->tshift > 3) return GBSPH_EINVAL;
  c->tshift = p->tshift;
  c->shiftcoef = p->tshift ? p->shiftcoef : 0.f;
  c->shifttfs = p->tshift ? p->shifttfs : 0.f;
  c->verletsteps = p->verletsteps > 0 ? p->verletsteps : 40;
  c->dtallparticles = p->dtallparticles;
  c->simulate2d = 0;
  c->cellmode_div = p->cellmode_div == 2 ? 2 : 1;
  c->kernelh = (float)p->h;
  c->cteb = (float)p->b;
  c->gamma = (float)p->gamma;
  c->rhopzero = (float)p->rhop0;
  c->cflnumber = p->cflnumber;
  c->dp = p->dp;
  c->massfluid = (float)p->massfluid;
  c->massbound = (float)p->massbound;
  for (int k = 0; k < 3; k++) c->gravity[k] = (float)p->gravity[k];
  c->visco = p->visco;
  c->viscoboundfactor = p->viscoboundfactor;
  c->rhopoutmin = p->rhopoutmin;
  c->rhopoutmax = p->rhopoutmax;
  // Wendland C2: kernel size factor 2 and constants (FunSphKernel.h:194-211)
  const double h = c->kernelh;
  c->kernelsize = (float)(h * 2.0f);
  c->kernelsize2 = c->kernelsize * c->kernelsize;
  c->awen = (float)(0.41778 / (h * h * h));
  c->bwenh = (float)(-2.08891 / (h * h * h * h * h));
  c->cs0 = std::sqrt((double)c->gamma * (double)c->cteb / (double)c->rhopzero);
  c->eta2 = (float)((h * 0.1) * (h * 0.1));
  if (c->tvisco == GBSPH_VISCO_LAMINARSPS) {
    const double dp_sps = std::sqrt(c->dp * c->dp * 3.) / 3.;
    c->spssmag = (float)((2. / 3.) * std::pow((0.12 * dp_sps), 2));
    c->spsblin = (float)((2. / 3.) * 0.0066 * dp_sps * dp_sps);
  }
  // DDTValue is 0 without density diffusion (JSph.cpp:923); DDTkh = KernelSize*DDTValue (JSph.cpp:1534)
  c->ddtkh = c->kernelsize * (p->tdensity == GBSPH_DDT_NONE ? 0.f : p->ddtvalue);
  c->ddtgz = (float)((double)c->rhopzero * (double)std::fabs(c->gravity[2]) / (double)c->cteb);
  c->dtini = p->dtini > 0 ? p->dtini : c->kernelh / c->cs0;
  c->dtmin = p->dtmin > 0 ? p->dtmin : (c->kernelh / c->cs0) * p->coefdtmin;
  c->scell = c->kernelsize / (float)c->cellmode_div;
  c->movlimit = c->scell * 0.9f;
  for (int k = 0; k < 3; k++) {
    if (!(p->maprealposmax[k] - p->maprealposmin[k] > 0)) return GBSPH_EINVAL;
    c->maprealposmin[k] = p->maprealposmin[k];
    c->maprealposmax[k] = p->maprealposmax[k];
    c->maprealsize[k] = p->maprealposmax[k] - p->maprealposmin[k];
    c->peri[k] = p->peri[k] != 0;
  }
  // periodic increments: the own component is -MapRealSize (JSph.cpp:2186-2188)
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      c->periinc[3 * k + j] = c->peri[k] ? (j == k ? -c->maprealsize[k] : p->periinc[3 * k + j]) : 0.0;
  // Map_PosMin/Max with a KernelSize halo on periodic axes (JSph.cpp:2190-2194),
  // the map cells (JSph.cpp:1883-1885) and SelecDomain(0,Map_Cells) (JSph.cpp:1901-1931)
  for (int k = 0; k < 3; k++) {
    const double ks = (double)c->kernelsize;
    c->mapposmin[k] = c->peri[k] ? c->maprealposmin[k] - ks : c->maprealposmin[k];
    c->mapposmax[k] = c->peri[k] ? c->maprealposmax[k] + ks : c->maprealposmax[k];
    const double mapsize = c->mapposmax[k] - c->mapposmin[k];
    c->mapcells[k] = (unsigned)std::ceil(mapsize / c->scell);
    c->domcells[k] = c->mapcells[k];
    c->domposmin[k] = c->mapposmin[k];
    double dmax = c->mapposmin[k] + (c->mapcells[k] * c->scell);
    if (dmax > c->mapposmax[k]) dmax = c->mapposmax[k];
    c->domrealposmin[k] = c->domposmin[k] < c->maprealposmin[k] ? c->maprealposmin[k] : c->domposmin[k];
    c->domrealposmax[k] = dmax > c->maprealposmax[k] ? c->maprealposmax[k] : dmax;
  }
  c->domcellcode = cell_code(c->domcells[0] + 1, c->domcells[1] + 1, c->domcells[2] + 1);
  return c->domcellcode ? GBSPH_OK : GBSPH_ECAPACITY;
}
