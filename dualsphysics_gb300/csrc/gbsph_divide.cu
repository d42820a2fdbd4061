// gbsph_divide.cu -- cell-linked neighbour list on the device: domain fit,
// box keys, stable LSD radix sort by box with the previous array index as
// tie-break, BeginCell, and the reorder of the particle arrays.
//
// Restates JCellDivCpuSingle::Divide (JCellDivCpuSingle.cpp:45-350; GPU twin
// JCellDivGpuSingle.cpp:152-230 with kernels in JCellDivGpuSingle_ker.cu:41-165
// and JCellDivGpu_ker.cu:120-760) bit-exactly: the CPU's counting sort is
// stable by array index, and an LSD radix sort whose values start as the array
// indices is stable in the same way.  Everything stays on the device: counts
// and limits are read by later kernels from DivState, so the whole divide can
// be captured in a CUDA graph.
#include <cuda_runtime.h>

#include "gbsph_common.cuh"

namespace {

constexpr int kDivBlock = 256;
constexpr int kSortBlock = 256;
constexpr int kSortItems = 8;                       // items per thread per tile
constexpr int kSortTile = kSortBlock * kSortItems;  // 2048 keys per tile
constexpr int kRadixBits = 8;        // digit width of the no-alloc sort and the default
constexpr int kRadix = 1 << kRadixBits;
constexpr int kRadixBitsWide = 11;   // the other digit width the divide can use

// LoadDcellParticles (JSph.cpp:1794-1817): cell of every particle.
__global__ void k_load_dcell(gbsph_consts c, DevArrays a, unsigned n) {
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const unsigned code = a.code[p];
  unsigned cell = 0xffffffffu;
  if ((code & GB_CODE_MASKSPECIAL) < GB_CODE_OUTIGNORE) {
    const double x = a.px[p], y = a.py[p], z = a.pz[p];
    if (x >= c.domrealposmin[0] && y >= c.domrealposmin[1] && z >= c.domrealposmin[2] &&
        x < c.domrealposmax[0] && y < c.domrealposmax[1] && z < c.domrealposmax[2]) {
      const double sc = (double)c.scell;
      const unsigned cx = (unsigned)(__ddiv_rn(__dsub_rn(x, c.domposmin[0]), sc));
      const unsigned cy = (unsigned)(__ddiv_rn(__dsub_rn(y, c.domposmin[1]), sc));
      const unsigned cz = (unsigned)(__ddiv_rn(__dsub_rn(z, c.domposmin[2]), sc));
      cell = gb_cell(c.domcellcode, cx, cy, cz);
    } else {
      // JSph::LoadDcellParticles raises "Found new particles out." (JSph.cpp:1811)
      atomicOr(&a.div->error, GB_ERR_PARTOUT);
    }
  }
  a.dcell[p] = cell;
}

// Start of a divide: reset the limit reductions (JCellDivCpuSingle.cpp:284-305).
// With periodic conditions the boundary always counts as changed
// (RunPeriodic sets BoundChanged, JSphCpuSingle.cpp:433): its copies are made
// anew before every divide.
__global__ void k_div_begin(DivState* d, int periactive) {
  d->nptot = d->np;
  d->npb1 = d->npb;
  d->npbout = d->npfout = d->npboutignore = d->npfoutignore = 0;
  if (d->boundchanged || periactive) {
    d->boundlimitok = d->bounddivideok = 0;
    for (int k = 0; k < 3; k++) d->blmin[k] = d->blmax[k] = d->bdmin[k] = d->bdmax[k] = 0;
  }
  for (int k = 0; k < 3; k++) {
    d->fmin[k] = 0xffffffffu; d->fmax[k] = 0;
    d->bmin[k] = 0xffffffffu; d->bmax[k] = 0;
  }
}

// LimitsCellBound/LimitsCellFluid (JCellDivCpu.cpp:256-345) as a block
// reduction followed by one atomic per block and axis.
// The arrays hold up to four segments: npb1 boundary, npf1 fluid, then the
// npb2 boundary and npf2 fluid periodic copies.
__global__ void k_limits(unsigned dcc, DevArrays a) {
  DivState* d = a.div;
  const unsigned np = d->nptot, npb = d->npb1;
  const unsigned e1 = np - d->npb2 - d->npf2, e2 = e1 + d->npb2;  // [e1, e2): boundary copies
  const bool dobound = !d->boundlimitok;
  unsigned fmn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, fmx[3] = {0, 0, 0};
  unsigned bmn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, bmx[3] = {0, 0, 0};
  const unsigned pbeg = dobound ? 0 : npb;
  for (unsigned p = pbeg + blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    if ((a.code[p] & GB_CODE_MASKSPECIAL) < GB_CODE_OUTIGNORE) {
      const unsigned cel = a.dcell[p];
      const unsigned v[3] = {gb_cx(dcc, cel), gb_cy(dcc, cel), gb_cz(dcc, cel)};
      if (p >= npb && (p < e1 || p >= e2)) {
        for (int k = 0; k < 3; k++) { fmn[k] = min(fmn[k], v[k]); fmx[k] = max(fmx[k], v[k]); }
      } else {
        for (int k = 0; k < 3; k++) { bmn[k] = min(bmn[k], v[k]); bmx[k] = max(bmx[k], v[k]); }
      }
    }
  }
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o; o >>= 1) {
      fmn[k] = min(fmn[k], __shfl_xor_sync(0xffffffffu, fmn[k], o));
      fmx[k] = max(fmx[k], __shfl_xor_sync(0xffffffffu, fmx[k], o));
      bmn[k] = min(bmn[k], __shfl_xor_sync(0xffffffffu, bmn[k], o));
      bmx[k] = max(bmx[k], __shfl_xor_sync(0xffffffffu, bmx[k], o));
    }
  }
  __shared__ unsigned s[32][12];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int k = 0; k < 3; k++) { s[w][k] = fmn[k]; s[w][3 + k] = fmx[k]; s[w][6 + k] = bmn[k]; s[w][9 + k] = bmx[k]; }
  __syncthreads();
  if (threadIdx.x < 12) {
    const int nw = blockDim.x >> 5;
    const int k = threadIdx.x;
    unsigned r = s[0][k];
    for (int i = 1; i < nw; i++) r = ((k % 6) < 3) ? min(r, s[i][k]) : max(r, s[i][k]);
    if (k < 3) { if (r != 0xffffffffu) atomicMin(&d->fmin[k], r); }
    else if (k < 6) atomicMax(&d->fmax[k - 3], r);
    else if (k < 9) { if (r != 0xffffffffu) atomicMin(&d->bmin[k - 6], r); }
    else atomicMax(&d->bmax[k - 9], r);
  }
}

// CalcCellDomain + MergeMapCellBoundFluid + PrepareNct + DivideFull decision
// (JCellDivCpuSingle.cpp:45-126, 319-324).
__global__ void k_div_setup(gbsph_consts c, DivState* d) {
  unsigned cb0[3], cb1[3], cf0[3], cf1[3];
  if (!d->boundlimitok) {
    // CalcCellDomainBound: an empty set gives (DomCells,0) (JCellDivCpu.cpp:295-305)
    const bool empty = d->bmin[0] > d->bmax[0];
    for (int k = 0; k < 3; k++) {
      cb0[k] = empty ? c.domcells[k] : d->bmin[k];
      cb1[k] = empty ? 0 : d->bmax[k];
      d->blmin[k] = cb0[k]; d->blmax[k] = cb1[k];
    }
    d->boundlimitok = 1;
  } else {
    for (int k = 0; k < 3; k++) { cb0[k] = d->blmin[k]; cb1[k] = d->blmax[k]; }
  }
  {
    const bool empty = d->fmin[0] > d->fmax[0];
    for (int k = 0; k < 3; k++) { cf0[k] = empty ? c.domcells[k] : d->fmin[k]; cf1[k] = empty ? 0 : d->fmax[k]; }
  }
  const unsigned sd = (unsigned)c.cellmode_div;
  unsigned cmn[3], cmx[3];
  for (int k = 0; k < 3; k++) {
    const unsigned a0 = min(cb0[k], cf0[k]);
    const unsigned b0 = cf0[k] >= sd ? cf0[k] - sd : 0;
    cmn[k] = max(a0, b0);
    cmx[k] = min(max(cb1[k], cf1[k]), cf1[k] + sd);
    if (cmx[k] >= c.domcells[k]) cmx[k] = c.domcells[k] - 1;
  }
  if (cmn[0] > cmx[0] || cmn[1] > cmx[1] || cmn[2] > cmx[2])
    for (int k = 0; k < 3; k++) cmn[k] = cmx[k] = 0;
  for (int k = 0; k < 3; k++) { d->cellmin[k] = cmn[k]; d->cellmax[k] = cmx[k]; }
  d->ncx = cmx[0] - cmn[0] + 1;
  d->ncy = cmx[1] - cmn[1] + 1;
  d->ncz = cmx[2] - cmn[2] + 1;
  d->nsheet = d->ncx * d->ncy;
  d->nct = d->nsheet * d->ncz;
  d->nctt = d->nct * 2 + 6;
  d->boxboundignore = d->nct;
  d->boxfluid = d->nct + 1;
  d->boxboundout = d->boxfluid + d->nct;
  d->boxfluidout = d->boxboundout + 1;
  d->boxboundoutignore = d->boxfluidout + 1;
  d->boxfluidoutignore = d->boxboundoutignore + 1;
  if (d->nctt > d->nctt_cap) d->error |= GB_ERR_CELLCAP;
  bool same = d->bounddivideok;
  for (int k = 0; k < 3; k++) same = same && d->bdmin[k] == cmn[k] && d->bdmax[k] == cmx[k];
  if (!same) {
    d->dividefull = 1;
    d->bounddivideok = 1;
    for (int k = 0; k < 3; k++) { d->bdmin[k] = cmn[k]; d->bdmax[k] = cmx[k]; }
  } else d->dividefull = 0;
  d->ini = d->dividefull ? 0 : d->npb1;
}

// PreSortFull / PreSortFluid (JCellDivCpuSingle.cpp:137-205): box key per
// particle; the value is the current array index.
__global__ void k_presort(unsigned dcc, DevArrays a) {
  const DivState* d = a.div;
  if (d->error & GB_ERR_CELLCAP) return;
  const unsigned p = d->ini + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d->nptot) return;
  const unsigned rcell = a.dcell[p];
  const unsigned cx = gb_cx(dcc, rcell) - d->cellmin[0];
  const unsigned cy = gb_cy(dcc, rcell) - d->cellmin[1];
  const unsigned cz = gb_cz(dcc, rcell) - d->cellmin[2];
  const unsigned cellsort = cx + cy * d->ncx + cz * d->nsheet;
  const unsigned rcode = a.code[p];
  const unsigned ctype = rcode & GB_CODE_MASKTYPE;
  const unsigned cout = rcode & GB_CODE_MASKSPECIAL;
  unsigned box;
  if (d->dividefull && ctype < GB_CODE_TYPE_FLOATING) {
    box = (cout < GB_CODE_OUTIGNORE ? ((cx < d->ncx && cy < d->ncy && cz < d->ncz) ? cellsort : d->boxboundignore)
                                    : (cout == GB_CODE_OUTIGNORE ? d->boxboundoutignore : d->boxboundout));
  } else {
    box = (cout <= GB_CODE_OUTIGNORE ? (cout < GB_CODE_OUTIGNORE ? d->boxfluid + cellsort : d->boxfluidoutignore)
                                     : (ctype == GB_CODE_TYPE_FLOATING ? d->boxboundout : d->boxfluidout));
  }
  a.keys[p] = box;
  a.vals[p] = p;
}

// ---- stable LSD radix sort of (key,value) over [ini, nptot) ------------------
// Tile histograms, stored digit-major: hist[digit*ntiles + tile].
template <int RB>
__global__ void k_rs_hist(const unsigned* __restrict__ keys, unsigned* __restrict__ hist, const DivState* d,
                          unsigned ntiles_cap, int shift) {
  constexpr int kRadix = 1 << RB;
  __shared__ unsigned sh[kRadix];
  const unsigned ini = d->ini, n = d->nptot - d->ini;
  const unsigned ntiles = gb_div_up(n, kSortTile);
  for (int i = threadIdx.x; i < kRadix; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const unsigned tile = blockIdx.x;
  if (tile < ntiles) {
    const unsigned base = tile * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
      const unsigned q = base + i;
      if (q < n) atomicAdd(&sh[(keys[ini + q] >> shift) & (kRadix - 1)], 1u);
    }
  }
  __syncthreads();
  for (int dgt = threadIdx.x; dgt < kRadix; dgt += blockDim.x)
    hist[dgt * ntiles_cap + tile] = (tile < ntiles) ? sh[dgt] : 0;
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024).
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* total) {
  __shared__ unsigned wsum[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  unsigned x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned ws = lane < nw ? wsum[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += y;
    }
    if (lane < nw) wsum[lane] = ws;
  }
  __syncthreads();
  const unsigned excl = x - v + (w ? wsum[w - 1] : 0);
  if (total) *total = wsum[nw - 1];
  __syncthreads();
  return excl;
}

// Exclusive scan of one digit's column of tile counts (one block per digit);
// the column total goes to tot[digit].
__global__ void k_rs_scan_cols(unsigned* __restrict__ hist, unsigned* __restrict__ tot, unsigned ntiles) {
  unsigned* col = hist + (size_t)blockIdx.x * ntiles;
  const unsigned chunk = gb_div_up(ntiles, blockDim.x);
  const unsigned b = threadIdx.x * chunk, e = min(ntiles, b + chunk);
  unsigned sum = 0;
  for (unsigned i = b; i < e; i++) sum += col[i];
  unsigned total;
  unsigned run = block_exclusive_scan(sum, &total);
  for (unsigned i = b; i < e; i++) {
    const unsigned v = col[i];
    col[i] = run;
    run += v;
  }
  if (threadIdx.x == 0) tot[blockIdx.x] = total;
}

// Exclusive scan of the 2^RB digit totals (one block; each thread owns
// 2^RB / blockDim.x consecutive digits).
template <int RB>
__global__ void k_rs_scan_digits(unsigned* __restrict__ tot) {
  constexpr int kRadix = 1 << RB;
  const int chunk = kRadix / (int)blockDim.x;
  const int b = threadIdx.x * chunk;
  unsigned sum = 0;
  for (int i = 0; i < chunk; i++) sum += tot[b + i];
  unsigned run = block_exclusive_scan(sum, nullptr);
  for (int i = 0; i < chunk; i++) {
    const unsigned v = tot[b + i];
    tot[b + i] = run;
    run += v;
  }
}

// Stable scatter: within a tile, items keep their index order per digit.
// The tile is processed in rounds of blockDim.x consecutive items; in a round
// each warp ranks its 32 items with __match_any_sync, per-digit warp counts are
// prefixed across warps in warp order, and a running per-digit offset carries
// the order from one round to the next.
// Shared memory (dynamic): s_off, s_tot and s_wc below.
template <int RB>
constexpr size_t scatter_smem() { return sizeof(unsigned) * ((size_t)(2 + kSortBlock / 32) << RB); }

template <int RB>
__global__ void __launch_bounds__(kSortBlock) k_rs_scatter(const unsigned* __restrict__ kin, const unsigned* __restrict__ vin,
                                                           unsigned* __restrict__ kout, unsigned* __restrict__ vout,
                                                           const unsigned* __restrict__ hist, const DivState* d,
                                                           unsigned ntiles_cap, int shift) {
  constexpr int kRadix = 1 << RB;
  constexpr int kWarps = kSortBlock / 32;
  extern __shared__ unsigned s_rs[];
  unsigned* s_off = s_rs;                                        // running output offset of each digit for this tile
  unsigned* s_tot = s_off + kRadix;                              // per-digit count of the current round
  unsigned(*s_wc)[kRadix] = (unsigned(*)[kRadix])(s_tot + kRadix);  // per-warp counts, then prefix across warps
  const unsigned ini = d->ini, n = d->nptot - d->ini;
  const unsigned ntiles = gb_div_up(n, kSortTile);
  const unsigned tile = blockIdx.x;
  if (tile >= ntiles) return;
  const unsigned* tot = hist + (size_t)kRadix * ntiles_cap;
  for (int i = threadIdx.x; i < kRadix; i += blockDim.x) s_off[i] = hist[i * ntiles_cap + tile] + tot[i];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lanemask_lt = (1u << lane) - 1u;
  const unsigned base = tile * kSortTile;
  for (int r = 0; r < kSortItems; r++) {
    for (int i = threadIdx.x; i < kWarps * kRadix; i += blockDim.x) (&s_wc[0][0])[i] = 0;
    __syncthreads();
    const unsigned q = base + r * kSortBlock + threadIdx.x;
    const bool valid = q < n;
    unsigned key = 0, val = 0, dgt = kRadix;  // kRadix marks an invalid item
    if (valid) {
      key = kin[ini + q];
      val = vin[ini + q];
      dgt = (key >> shift) & (kRadix - 1);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, dgt);
    const unsigned rank = __popc(peers & lanemask_lt);
    if (valid && rank == 0) s_wc[w][dgt] = __popc(peers);
    __syncthreads();
    for (int dg = threadIdx.x; dg < kRadix; dg += blockDim.x) {
      unsigned run = 0;
      for (int ww = 0; ww < kWarps; ww++) {
        const unsigned v = s_wc[ww][dg];
        s_wc[ww][dg] = run;
        run += v;
      }
      s_tot[dg] = run;
    }
    __syncthreads();
    if (valid) {
      const unsigned dst = s_off[dgt] + s_wc[w][dgt] + rank;
      kout[ini + dst] = key;
      vout[ini + dst] = val;
    }
    __syncthreads();
    for (int dg = threadIdx.x; dg < kRadix; dg += blockDim.x) s_off[dg] += s_tot[dg];
    __syncthreads();
  }
}

// BeginCell (JCellDivCpuSingle.cpp:207-247): begincell[b] = first sorted index
// with key >= b, found by binary search; b ranges over every box in a full
// divide and over the fluid boxes above BoxFluid in a fluid-only divide (the
// boundary part of the previous full divide is kept, as the reference does).
__global__ void k_begincell(const unsigned* __restrict__ keys, DevArrays a) {
  const DivState* d = a.div;
  if (d->error & GB_ERR_CELLCAP) return;
  const unsigned nctt = d->nctt;
  const unsigned b0 = d->dividefull ? 0 : d->boxfluid + 1;
  const unsigned b = b0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nctt) return;
  unsigned lo = d->ini, hi = d->nptot;
  while (lo < hi) {
    const unsigned mid = (lo + hi) >> 1;
    if (keys[mid] < b) lo = mid + 1;
    else hi = mid;
  }
  a.begincell[b] = lo;
}

// Counts and new particle numbers (JCellDivCpuSingle.cpp:327-345,
// JSphCpuSingle.cpp:566-572).
__global__ void k_div_counts(DevArrays a) {
  DivState* d = a.div;
  if (d->error & GB_ERR_CELLCAP) return;
  const unsigned* bc = a.begincell;
  d->npbignore = bc[d->boxboundignore + 1] - bc[d->boxboundignore];
  d->npbout = bc[d->boxboundout + 1] - bc[d->boxboundout];
  d->npfout = bc[d->boxfluidout + 1] - bc[d->boxfluidout];
  d->npboutignore = bc[d->boxboundoutignore + 1] - bc[d->boxboundoutignore];
  d->npfoutignore = bc[d->boxfluidoutignore + 1] - bc[d->boxfluidoutignore];
  d->npfinal = d->nptot - d->npbout - d->npfout - d->npboutignore - d->npfoutignore;
  d->npbfinal = d->npb1 + d->npb2 - d->npboutignore;
  if (d->npbout) d->error |= GB_ERR_BOUNDOUT;
  d->np = d->npfinal;
  d->npb = d->npbfinal;
  d->npbok = d->npbfinal - d->npbignore;
  d->nout_total += d->npfout;
  d->boundchanged = 0;
}

// SortDataParticles + UpdatePosCell (JCellDivGpu_ker.cu:577-760,
// JSphGpuSimple_ker.cu:41-62): gather every particle array in the new order and
// rebuild the cell-relative float position and the pressure.
template <bool withpre, bool withsps, bool withnor>
__global__ void k_reorder(gbsph_consts c, DevArrays a) {
  const DivState* d = a.div;
  if (d->error & GB_ERR_CELLCAP) return;
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d->nptot) return;
  const unsigned src = (p < d->ini) ? p : a.vals[p];
  const double x = a.px[src], y = a.py[src], z = a.pz[src];
  a.px2[p] = x; a.py2[p] = y; a.pz2[p] = z;
  const float4 vr = a.velrho[src];
  a.velrho2[p] = vr;
  a.idp2[p] = a.idp[src];
  a.code2[p] = a.code[src];
  const unsigned cel = a.dcell[src];
  a.dcell2[p] = cel;
  if (withpre) {
    a.qx2[p] = a.qx[src]; a.qy2[p] = a.qy[src]; a.qz2[p] = a.qz[src];
    a.velrhopre2[p] = a.velrhopre[src];
  }
  if (withsps) {
    a.taua2[p] = a.taua[src];
    a.taub2[p] = a.taub[src];
  }
  if (withnor) a.boundnor2[p] = a.boundnor[src];
  // position relative to the origin of the particle's cell,
  // float((pos - DomPosMin) - cell * Scell): cell * Scell (an integer below
  // 2^24 times a float) is exact in double, so one fused multiply-add rounds
  // the difference exactly as the subtraction of the rounded product does;
  // the conversions run on the integer pipe (this part's FP64 rate is low)
  const unsigned dcc = c.domcellcode;
  const double sc = gb_f2d(c.scell);
  float4 ps;
  if (cel != 0xffffffffu) {
    ps.x = gb_d2f(__fma_rn(-gb_u2d(gb_cx(dcc, cel)), sc, __dsub_rn(x, c.domposmin[0])));
    ps.y = gb_d2f(__fma_rn(-gb_u2d(gb_cy(dcc, cel)), sc, __dsub_rn(y, c.domposmin[1])));
    ps.z = gb_d2f(__fma_rn(-gb_u2d(gb_cz(dcc, cel)), sc, __dsub_rn(z, c.domposmin[2])));
  } else {
    ps.x = ps.y = ps.z = 0.f;
  }
  ps.w = gb_press(vr.w, c.rhopzero, c.cteb, c.gamma);
  a.pscell[p] = ps;
}


// ---- periodic conditions (JSphCpuSingle::RunPeriodic, JSphCpuSingle.cpp:416-504) ----
// Every particle within reach of a periodic face gets a copy moved by the
// axis increment, appended after the np particles in the order the reference's
// PeriodicMakeList gives (JSphCpuSingle.cpp:210-252): by source index, the
// copy by +inc before the one by -inc.  For each (type, axis, block) group a
// count kernel sums the copies of 256-particle tiles, one block scans the tile
// sums and reserves the room, and the duplicate kernel re-derives its tile's
// copies and writes them at the scanned offsets.  All counts stay on the
// device.

// PeriodicIgnore (JSphCpuSingle.cpp:186-203): the copies of the last divide
// are ignored from now on; the counts the copying starts from.
__global__ void k_peri_begin(DevArrays a) {
  DivState* d = a.div;
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0) {
    d->peri_npb0 = d->npb;
    d->peri_npf0 = d->np - d->npb;
    d->npb2 = d->npf2 = 0;
  }
  if (p < d->np) {
    const unsigned code = a.code[p];
    if ((code & GB_CODE_MASKSPECIAL) == GB_CODE_PERIODIC)
      a.code[p] = (uint16_t)((code & ~GB_CODE_MASKSPECIAL) | GB_CODE_OUTIGNORE);
  }
}

// Range of a group: the copies made so far of this type (cblock 0), or the
// particles of this type present before the copying (cblock 1).
__device__ __forceinline__ void peri_range(const DivState* d, int ctype, int cblock, unsigned& pini, unsigned& num) {
  if (cblock) {
    pini = ctype ? d->peri_npb0 : 0;
    num = ctype ? d->peri_npf0 : d->peri_npb0;
  } else {
    num = ctype ? d->npf2 : d->npb2;
    pini = d->np - num;
  }
}

// Copies of particle p: bit 0 for +inc, bit 1 for -inc, each kept when it
// falls inside [Map_PosMin, Map_PosMax); particles already excluded get none.
__device__ __forceinline__ unsigned peri_flags(const gbsph_consts& c, const DevArrays& a, unsigned p, int axis) {
  if ((a.code[p] & GB_CODE_MASKSPECIAL) > GB_CODE_PERIODIC) return 0u;
  const double* inc = c.periinc + 3 * axis;
  const double x = a.px[p], y = a.py[p], z = a.pz[p];
  unsigned f = 0;
  {
    const double qx = __dadd_rn(x, inc[0]), qy = __dadd_rn(y, inc[1]), qz = __dadd_rn(z, inc[2]);
    if (c.mapposmin[0] <= qx && c.mapposmin[1] <= qy && c.mapposmin[2] <= qz && qx < c.mapposmax[0] &&
        qy < c.mapposmax[1] && qz < c.mapposmax[2])
      f |= 1u;
  }
  {
    const double qx = __dsub_rn(x, inc[0]), qy = __dsub_rn(y, inc[1]), qz = __dsub_rn(z, inc[2]);
    if (c.mapposmin[0] <= qx && c.mapposmin[1] <= qy && c.mapposmin[2] <= qz && qx < c.mapposmax[0] &&
        qy < c.mapposmax[1] && qz < c.mapposmax[2])
      f |= 2u;
  }
  return f;
}

// Copies per 256-particle tile of the group's range.
__global__ void k_peri_count(gbsph_consts c, DevArrays a, int ctype, int cblock, int axis, unsigned* __restrict__ tiles) {
  unsigned pini, num;
  peri_range(a.div, ctype, cblock, pini, num);
  const unsigned i = blockIdx.x * kDivBlock + threadIdx.x;
  const unsigned n = i < num ? __popc(peri_flags(c, a, pini + i, axis)) : 0u;
  unsigned tot;
  block_exclusive_scan(n, &tot);
  if (threadIdx.x == 0) tiles[blockIdx.x] = tot;
}

// Exclusive scan of the tile counts (one block); reserves the room for the
// group's copies after np, or flags GB_ERR_PERICAP and makes none.
__global__ void k_peri_scan(DevArrays a, int ctype, int cblock, unsigned* __restrict__ tiles, unsigned ntiles,
                            unsigned cap) {
  const unsigned chunk = gb_div_up(ntiles, blockDim.x);
  const unsigned b = threadIdx.x * chunk, e = min(ntiles, b + chunk);
  unsigned sum = 0;
  for (unsigned i = b; i < e; i++) sum += tiles[i];
  unsigned total;
  unsigned run = block_exclusive_scan(sum, &total);
  for (unsigned i = b; i < e; i++) {
    const unsigned v = tiles[i];
    tiles[i] = run;
    run += v;
  }
  if (threadIdx.x == 0) {
    DivState* d = a.div;
    unsigned pini, num;
    peri_range(d, ctype, cblock, pini, num);
    d->peri_pini = pini;
    d->peri_num = num;
    d->peri_base = d->np;
    if ((unsigned long long)d->np + total > cap) {
      d->error |= GB_ERR_PERICAP;
      d->peri_count = 0;
    } else {
      d->peri_count = total;
      d->np += total;
      if (ctype) d->npf2 += total;
      else d->npb2 += total;
    }
  }
}

// PeriodicDuplicatePos / PeriodicDuplicateSymplectic / PeriodicDuplicateVerlet /
// PeriodicDuplicateNormals (JSphCpuSingle.cpp:258-380): the copy takes every
// array of its source (the PRE arrays and VelrhoM1 included, which the
// reference copies only while they are live), its position moved by the
// increment, the cell of that position clamped to the domain, and the code
// marked periodic.
template <bool withsps, bool withnor>
__global__ void k_peri_dup(gbsph_consts c, DevArrays a, int axis, const unsigned* __restrict__ tiles) {
  const DivState* d = a.div;
  const unsigned num = d->peri_num;
  const unsigned i = blockIdx.x * kDivBlock + threadIdx.x;
  const unsigned pcopy = d->peri_pini + i;
  const unsigned f = (i < num && d->peri_count) ? peri_flags(c, a, pcopy, axis) : 0u;
  const unsigned off = block_exclusive_scan(__popc(f), nullptr);
  if (!f) return;
  unsigned pnew = d->peri_base + tiles[blockIdx.x] + off;
  const double* inc = c.periinc + 3 * axis;
  const double x = a.px[pcopy], y = a.py[pcopy], z = a.pz[pcopy];
  const unsigned code = (a.code[pcopy] & ~GB_CODE_MASKSPECIAL) | GB_CODE_PERIODIC;
  const double sc = (double)c.scell;
  for (int sgn = 0; sgn < 2; sgn++) {
    if (!(f & (1u << sgn))) continue;
    const double qx = sgn ? __dadd_rn(x, -inc[0]) : __dadd_rn(x, inc[0]);
    const double qy = sgn ? __dadd_rn(y, -inc[1]) : __dadd_rn(y, inc[1]);
    const double qz = sgn ? __dadd_rn(z, -inc[2]) : __dadd_rn(z, inc[2]);
    const unsigned cx = min((unsigned)__ddiv_rn(__dsub_rn(qx, c.domposmin[0]), sc), c.domcells[0]);
    const unsigned cy = min((unsigned)__ddiv_rn(__dsub_rn(qy, c.domposmin[1]), sc), c.domcells[1]);
    const unsigned cz = min((unsigned)__ddiv_rn(__dsub_rn(qz, c.domposmin[2]), sc), c.domcells[2]);
    a.px[pnew] = qx; a.py[pnew] = qy; a.pz[pnew] = qz;
    a.dcell[pnew] = gb_cell(c.domcellcode, cx, cy, cz);
    a.idp[pnew] = a.idp[pcopy];
    a.code[pnew] = (uint16_t)code;
    a.velrho[pnew] = a.velrho[pcopy];
    a.qx[pnew] = a.qx[pcopy]; a.qy[pnew] = a.qy[pcopy]; a.qz[pnew] = a.qz[pcopy];
    a.velrhopre[pnew] = a.velrhopre[pcopy];
    if (withsps) { a.taua[pnew] = a.taua[pcopy]; a.taub[pnew] = a.taub[pcopy]; }
    if (withnor) a.boundnor[pnew] = a.boundnor[pcopy];
    pnew++;
  }
}

// One LSD pass of RB-bit digits: tile histograms, their scan per digit, the
// digit totals' scan, the stable scatter.
template <int RB>
void sort_pass(const unsigned* kin, const unsigned* vin, unsigned* kout, unsigned* vout, unsigned* hist,
               const DivState* d, unsigned ntiles_cap, int shift, cudaStream_t s) {
  constexpr int R = 1 << RB;
  k_rs_hist<RB><<<ntiles_cap, kSortBlock, 0, s>>>(kin, hist, d, ntiles_cap, shift);
  k_rs_scan_cols<<<R, 256, 0, s>>>(hist, hist + (size_t)R * ntiles_cap, ntiles_cap);
  k_rs_scan_digits<RB><<<1, R < 1024 ? R : 1024, 0, s>>>(hist + (size_t)R * ntiles_cap);
  k_rs_scatter<RB><<<ntiles_cap, kSortBlock, scatter_smem<RB>(), s>>>(kin, vin, kout, vout, hist, d, ntiles_cap, shift);
}

template <typename T>
inline void swp(T*& x, T*& y) {
  T* t = x;
  x = y;
  y = t;
}

}  // namespace

namespace gbk {

cudaError_t sort_init() {
  return cudaFuncSetAttribute(k_rs_scatter<kRadixBitsWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)scatter_smem<kRadixBitsWide>());
}

void load_dcell(const gbsph_consts& c, const DevArrays& a, unsigned n, cudaStream_t s) {
  if (!n) return;
  k_load_dcell<<<gb_div_up(n, kDivBlock), kDivBlock, 0, s>>>(c, a, n);
}

void run_periodic(const gbsph_consts& c, DevArrays& a, unsigned cap, unsigned* tiles, cudaStream_t s,
                  unsigned long long* nlaunch) {
  const unsigned ntiles = gb_div_up(cap, kDivBlock);
  const bool withsps = (c.tvisco == GBSPH_VISCO_LAMINARSPS);
  const bool withnor = (c.tboundary == GBSPH_BC_MDBC);
  unsigned long long n = 1;
  k_peri_begin<<<ntiles, kDivBlock, 0, s>>>(a);
  for (int ctype = 0; ctype < 2; ctype++) {
    bool first = true;
    for (int axis = 0; axis < 3; axis++) {
      if (!c.peri[axis]) continue;
      // before the first axis there are no copies of this type to copy again
      for (int cblock = first ? 1 : 0; cblock < 2; cblock++) {
        k_peri_count<<<ntiles, kDivBlock, 0, s>>>(c, a, ctype, cblock, axis, tiles);
        k_peri_scan<<<1, 1024, 0, s>>>(a, ctype, cblock, tiles, ntiles, cap);
        if (withsps) {
          if (withnor) k_peri_dup<true, true><<<ntiles, kDivBlock, 0, s>>>(c, a, axis, tiles);
          else k_peri_dup<true, false><<<ntiles, kDivBlock, 0, s>>>(c, a, axis, tiles);
        } else {
          if (withnor) k_peri_dup<false, true><<<ntiles, kDivBlock, 0, s>>>(c, a, axis, tiles);
          else k_peri_dup<false, false><<<ntiles, kDivBlock, 0, s>>>(c, a, axis, tiles);
        }
        n += 3;
      }
      first = false;
    }
  }
  if (nlaunch) *nlaunch += n;
}

// JSphGpuSingle::RunCellDivide: RunPeriodic first when an axis is periodic.  `cap` is the
// particle capacity (grids are sized by it; kernels read the live counts from
// DivState).  The reorder swaps the cur/alt array pairs in `a`.
void divide(const gbsph_consts& c, DevArrays& a, unsigned cap, unsigned keybits, int radixbits, cudaStream_t s,
            unsigned long long* nlaunch) {
  const unsigned dcc = c.domcellcode;
  const unsigned grid_p = gb_div_up(cap, kDivBlock);
  const bool periactive = c.peri[0] || c.peri[1] || c.peri[2];
  if (periactive) run_periodic(c, a, cap, a.hist, s, nlaunch);
  k_div_begin<<<1, 1, 0, s>>>(a.div, periactive ? 1 : 0);
  k_limits<<<min(grid_p, 152u * 8u), kDivBlock, 0, s>>>(dcc, a);
  k_div_setup<<<1, 1, 0, s>>>(c, a.div);
  k_presort<<<grid_p, kDivBlock, 0, s>>>(dcc, a);
  const unsigned ntiles_cap = gb_div_up(cap, kSortTile);
  unsigned* kin = a.keys;
  unsigned* vin = a.vals;
  unsigned* kout = a.keys2;
  unsigned* vout = a.vals2;
  const int rb = radixbits == kRadixBitsWide ? kRadixBitsWide : kRadixBits;
  const unsigned npasses = gb_div_up(keybits, (unsigned)rb);
  for (unsigned pass = 0; pass < npasses; pass++) {
    const int shift = (int)(pass * rb);
    if (rb == kRadixBitsWide) sort_pass<kRadixBitsWide>(kin, vin, kout, vout, a.hist, a.div, ntiles_cap, shift, s);
    else sort_pass<kRadixBits>(kin, vin, kout, vout, a.hist, a.div, ntiles_cap, shift, s);
    swp(kin, kout);
    swp(vin, vout);
  }
  // sorted keys/vals are in kin/vin
  a.keys = kin; a.keys2 = kout; a.vals = vin; a.vals2 = vout;
  const unsigned long long maxboxes = 2ull * c.domcells[0] * c.domcells[1] * c.domcells[2] + 6;
  k_begincell<<<(unsigned)((maxboxes + kDivBlock - 1) / kDivBlock), kDivBlock, 0, s>>>(kin, a);
  k_div_counts<<<1, 1, 0, s>>>(a);
  const bool withpre = (c.tstep == GBSPH_STEP_SYMPLECTIC) || (c.tstep == GBSPH_STEP_VERLET);
  const bool withsps = (c.tvisco == GBSPH_VISCO_LAMINARSPS);
  const bool withnor = (c.tboundary == GBSPH_BC_MDBC);
  if (withpre) {
    if (withsps) {
      if (withnor) k_reorder<true, true, true><<<grid_p, kDivBlock, 0, s>>>(c, a);
      else k_reorder<true, true, false><<<grid_p, kDivBlock, 0, s>>>(c, a);
    } else {
      if (withnor) k_reorder<true, false, true><<<grid_p, kDivBlock, 0, s>>>(c, a);
      else k_reorder<true, false, false><<<grid_p, kDivBlock, 0, s>>>(c, a);
    }
  } else {
    if (withsps) {
      if (withnor) k_reorder<false, true, true><<<grid_p, kDivBlock, 0, s>>>(c, a);
      else k_reorder<false, true, false><<<grid_p, kDivBlock, 0, s>>>(c, a);
    } else {
      if (withnor) k_reorder<false, false, true><<<grid_p, kDivBlock, 0, s>>>(c, a);
      else k_reorder<false, false, false><<<grid_p, kDivBlock, 0, s>>>(c, a);
    }
  }
  swp(a.px, a.px2); swp(a.py, a.py2); swp(a.pz, a.pz2);
  swp(a.velrho, a.velrho2);
  swp(a.idp, a.idp2); swp(a.code, a.code2); swp(a.dcell, a.dcell2);
  if (withpre) { swp(a.qx, a.qx2); swp(a.qy, a.qy2); swp(a.qz, a.qz2); swp(a.velrhopre, a.velrhopre2); }
  if (withsps) { swp(a.taua, a.taua2); swp(a.taub, a.taub2); }
  if (withnor) swp(a.boundnor, a.boundnor2);
  if (nlaunch) *nlaunch += 7 + 4ull * npasses;
}

}  // namespace gbk

// ---- no-alloc sort: the radix sort of the cell division on a fixed work area
// Some callers cannot let a library call cudaMalloc/cudaFree: a host
// application that sized its own device pool at start-up and treats any other
// device allocation as an error, or a caller on a latency-bound path where an
// allocation (and the device synchronisation cudaFree implies) would stall its
// other streams.  For them the stable key sort of the cell division is also
// offered on a work area that exists from module load on: a file-scope
// __device__ array sized for kNoAllocMaxKeys keys.  Its device address is
// looked up once per device; nothing is allocated afterwards.  There is one
// work area per process and device, so two calls that overlap in time (two
// host threads, or two streams) race on it: callers must serialise them.
namespace {

constexpr unsigned kNoAllocMaxKeys = 1u << 18;  // 262,144 keys (4.3 MB of work area)
constexpr unsigned kNoAllocTiles = kNoAllocMaxKeys / kSortTile;
constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kNaDiv = 0;                                           // DivState: ini / nptot of the sort
constexpr size_t kNaKeysA = na_align(sizeof(DivState));
constexpr size_t kNaKeysB = kNaKeysA + na_align(sizeof(unsigned) * kNoAllocMaxKeys);
constexpr size_t kNaValsA = kNaKeysB + na_align(sizeof(unsigned) * kNoAllocMaxKeys);
constexpr size_t kNaValsB = kNaValsA + na_align(sizeof(unsigned) * kNoAllocMaxKeys);
constexpr size_t kNaHist = kNaValsB + na_align(sizeof(unsigned) * kNoAllocMaxKeys);
constexpr size_t kNaBytes = kNaHist + na_align(sizeof(unsigned) * ((size_t)kNoAllocTiles * kRadix + kRadix + 1));

static __device__ __align__(256) unsigned char g_sort_work[kNaBytes];

// Puts the work area in its starting state: the sort record cleared and set
// to the range [0, n), and the values set to the identity permutation (the
// values the first pass reads).  The histogram needs no clearing: every pass
// writes all of it before reading it.
__global__ void k_na_init(DivState* d, unsigned* vals, unsigned n) {
  const unsigned i0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (i0 == 0) {
    *d = DivState{};
    d->ini = 0;
    d->nptot = n;
  }
  for (unsigned i = i0; i < n; i += gridDim.x * blockDim.x) vals[i] = i;
}

}  // namespace

namespace gbk {

unsigned sort_noalloc_max_keys() { return kNoAllocMaxKeys; }

// Device address of the work area on the current device.  The kernels of the
// no-alloc sort are loaded here as well (cudaFuncGetAttributes loads a
// function under lazy module loading), so that no later call loads code.
cudaError_t sort_noalloc_address(void** p) {
  cudaError_t e = cudaGetSymbolAddress(p, g_sort_work);
  cudaFuncAttributes fa;
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_na_init);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_rs_hist<kRadixBits>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_rs_scan_cols);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_rs_scan_digits<kRadixBits>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_rs_scatter<kRadixBits>);
  return e;
}

void sort_noalloc(unsigned char* work, const unsigned* keys, unsigned n, unsigned nbits, unsigned* perm,
                  unsigned* sorted_keys, cudaStream_t s) {
  DivState* d = (DivState*)(work + kNaDiv);
  unsigned* keys_a = (unsigned*)(work + kNaKeysA);
  unsigned* keys_b = (unsigned*)(work + kNaKeysB);
  unsigned* vals_a = (unsigned*)(work + kNaValsA);
  unsigned* vals_b = (unsigned*)(work + kNaValsB);
  unsigned* hist = (unsigned*)(work + kNaHist);
  const unsigned ntiles = gb_div_up(n, kSortTile);
  k_na_init<<<gb_div_up(n, kDivBlock), kDivBlock, 0, s>>>(d, vals_a, n);
  const unsigned npasses = gb_div_up(nbits, kRadixBits);
  const unsigned* kin = keys;
  const unsigned* vin = vals_a;
  for (unsigned pass = 0; pass < npasses; pass++) {
    const int shift = (int)(pass * kRadixBits);
    unsigned* kout = (pass & 1) ? keys_b : keys_a;
    unsigned* vout = (pass & 1) ? vals_a : vals_b;
    sort_pass<kRadixBits>(kin, vin, kout, vout, hist, d, ntiles, shift, s);
    kin = kout;
    vin = vout;
  }
  cudaMemcpyAsync(perm, vin, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s);
  if (sorted_keys) cudaMemcpyAsync(sorted_keys, kin, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s);
}

}  // namespace gbk
