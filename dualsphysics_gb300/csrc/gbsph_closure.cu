// gbsph_closure.cu -- learned acceleration closure for coarse resolutions (no
// reference counterpart): per-particle features over the kernel
// neighbourhood, a 16-64-64-64-3 tanh MLP with BF16 weights and FP32
// accumulation, its application inside the step (with a per-particle fallback
// to the plain acceleration), and the kernels that train it (forward,
// backward, Adam).
//
// Parameter vector (flat, row-major, the layout every API and the oracle
// use): W0[64][16] b0[64] W1[64][64] b1[64] W2[64][64] b2[64] W3[3][64] b3[3].
// In shared memory each layer is held transposed with a row stride of 65
// floats, so that both the forward (lanes over outputs) and the backward
// (lanes over inputs) read it without bank conflicts.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <float.h>

#include "gbsph_common.cuh"

namespace {

constexpr int kIn = GBSPH_CLOSURE_FEATURES;  // 16
constexpr int kHid = 64;
constexpr int kOut = 3;
constexpr int kStride = kHid + 1;
// offsets in the flat parameter vector
constexpr int kW0 = 0, kB0 = kW0 + kHid * kIn, kW1 = kB0 + kHid, kB1 = kW1 + kHid * kHid, kW2 = kB1 + kHid,
              kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid, kB3 = kW3 + kOut * kHid, kNParams = kB3 + kOut;
static_assert(kNParams == GBSPH_CLOSURE_PARAMS, "parameter count");
// offsets in the shared-memory layout (floats)
constexpr int sW0 = 0, sW1 = sW0 + kIn * kStride, sW2 = sW1 + kHid * kStride, sW3 = sW2 + kHid * kStride,
              sB0 = sW3 + kHid * 4, sB1 = sB0 + kHid, sB2 = sB1 + kHid, sB3 = sB2 + kHid, sNW = sB3 + 4;
constexpr int kWarpAct = kIn + 4 * kHid;  // x, h1, h2, h3, delta per warp
constexpr int kMlpBlock = 256;
constexpr int kMlpWarps = kMlpBlock / 32;

// flat parameter index -> shared-memory index
__device__ __forceinline__ int smem_index(int i) {
  if (i < kB0) { const int j = i / kIn, k = i % kIn; return sW0 + k * kStride + j; }
  if (i < kW1) return sB0 + (i - kB0);
  if (i < kB1) { const int r = i - kW1, j = r / kHid, k = r % kHid; return sW1 + k * kStride + j; }
  if (i < kW2) return sB1 + (i - kB1);
  if (i < kB2) { const int r = i - kW2, j = r / kHid, k = r % kHid; return sW2 + k * kStride + j; }
  if (i < kW3) return sB2 + (i - kB2);
  if (i < kB3) { const int r = i - kW3, o = r / kHid, k = r % kHid; return sW3 + k * 4 + o; }
  return sB3 + (i - kB3);
}

__device__ void load_weights(float* sw, const __nv_bfloat16* __restrict__ w) {
  for (int i = threadIdx.x; i < sNW; i += blockDim.x) sw[i] = 0.f;
  __syncthreads();
  for (int i = threadIdx.x; i < kNParams; i += blockDim.x) sw[smem_index(i)] = __bfloat162float(w[i]);
  __syncthreads();
}

// One dense tanh layer for one warp: lanes own outputs j = lane, lane + 32.
__device__ __forceinline__ void dense_tanh(const float* wt, const float* b, const float* in, int nin, float* out,
                                           int lane) {
  float a0 = b[lane], a1 = b[lane + 32];
  for (int k = 0; k < nin; k++) {
    const float v = in[k];
    a0 = fmaf(wt[k * kStride + lane], v, a0);
    a1 = fmaf(wt[k * kStride + lane + 32], v, a1);
  }
  out[lane] = tanhf(a0);
  out[lane + 32] = tanhf(a1);
  __syncwarp();
}

// Forward pass of one sample by one warp; act = [x(16) h1 h2 h3 delta].
// Returns the three outputs on every lane.
__device__ __forceinline__ void mlp_forward(const float* sw, float* act, int lane, float y[kOut]) {
  float* x = act;
  float* h1 = act + kIn;
  float* h2 = h1 + kHid;
  float* h3 = h2 + kHid;
  dense_tanh(sw + sW0, sw + sB0, x, kIn, h1, lane);
  dense_tanh(sw + sW1, sw + sB1, h1, kHid, h2, lane);
  dense_tanh(sw + sW2, sw + sB2, h2, kHid, h3, lane);
  for (int o = 0; o < kOut; o++) {
    float p = sw[sW3 + lane * 4 + o] * h3[lane] + sw[sW3 + (lane + 32) * 4 + o] * h3[lane + 32];
    for (int s = 16; s; s >>= 1) p += __shfl_xor_sync(0xffffffffu, p, s);
    y[o] = p + sw[sB3 + o];
  }
}

// ---- features ----------------------------------------------------------------
// Per fluid row, over its fluid and boundary neighbours (V_j = m_j/rho_j,
// Wendland W and grad W of the case, grad taken at i):
//   0      rho_i/rho0 - 1, x50
//   1-3    sum_j V_j (v_j - v_i) W_ij / S, / (0.1 cs0)
//   4-6    sum_j V_j (p_j - p_i) grad W_ij, / (rho0 |g|)
//   7      S - 1, S = V_i W(0) + sum_j V_j W_ij (Shepard sum; < 0 near the surface)
//   8      -sum_j V_j r_ij . grad W_ij - 3 (position divergence; < 0 near the surface)
//   9-11   the plain acceleration, / |g|
//   12     sum over boundary neighbours of V_j W_ij
//   13-15  0
//
// One warp per fluid row: the lanes take the candidates of each of the (2sd+1)^2
// box rows (contiguous in the sorted order) in turn, and the sums are added
// across the warp at the end.
__global__ void __launch_bounds__(128) k_closure_features(gbsph_consts c, DevArrays a, float* __restrict__ feat) {
  constexpr unsigned FULL = 0xffffffffu;
  const DivState& d = *a.div;
  const unsigned np = d.np, npb = d.npb;
  const unsigned p1 = npb + (unsigned)(((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (p1 >= np) return;  // the same for the whole warp
  const float4 ps1 = a.pscell[p1];
  const float4 vr1 = a.velrho[p1];
  const unsigned dcc = c.domcellcode, cel = a.dcell[p1], cmin0 = d.cellmin[0];
  const int cx = (int)gb_cx(dcc, cel) - (int)cmin0, cy = (int)gb_cy(dcc, cel) - (int)d.cellmin[1],
            cz = (int)gb_cz(dcc, cel) - (int)d.cellmin[2];
  const int sd = c.cellmode_div, ncx = (int)d.ncx, ncy = (int)d.ncy, ncz = (int)d.ncz;
  const int xini = cx - min(cx, sd), xfin = cx + min(ncx - cx - 1, sd);
  const int yini = cy - min(cy, sd), yfin = cy + min(ncy - cy - 1, sd) + 1;
  const int zini = cz - min(cz, sd), zfin = cz + min(ncz - cz - 1, sd) + 1;
  const float h = c.kernelh, ks2 = c.kernelsize2, scell = c.scell;
  float shep = 0, sb = 0, dv[3] = {0, 0, 0}, gp[3] = {0, 0, 0}, divr = 0;
  for (int pass = 0; pass < 2; pass++) {
    const unsigned cellinit = pass == 0 ? d.boxfluid : 0u;
    const float mass = pass == 0 ? c.massfluid : c.massbound;
    for (int z = zini; z < zfin; z++)
      for (int y = yini; y < yfin; y++) {
        const unsigned row = cellinit + (unsigned)y * d.ncx + (unsigned)z * d.nsheet;
        const unsigned pini = a.begincell[row + (unsigned)xini], pfin = a.begincell[row + (unsigned)xfin + 1u];
        const float by = ps1.y + (float)(cy - y) * scell;
        const float bz = ps1.z + (float)(cz - z) * scell;
        for (unsigned p2 = pini + (unsigned)lane; p2 < pfin; p2 += 32u) {
          const float4 ps2 = a.pscell[p2];
          const int x = (int)gb_cx(dcc, a.dcell[p2]) - (int)cmin0;
          const float drx = (ps1.x + (float)(cx - x) * scell) - ps2.x, dry = by - ps2.y, drz = bz - ps2.z;
          const float rr2 = drx * drx + dry * dry + drz * drz;
          if (rr2 > ks2 || rr2 < GB_ALMOSTZERO) continue;
          const float q = sqrtf(rr2) / h;
          const float w1 = 1.f - 0.5f * q;
          const float w = c.awen * (2.f * q + 1.f) * (w1 * w1) * (w1 * w1);
          const float fac = c.bwenh * w1 * w1 * w1;
          const float4 vr2 = a.velrho[p2];
          const float vj = mass / vr2.w;
          const float vw = vj * w;
          shep += vw;
          if (pass == 1) sb += vw;
          dv[0] += vw * (vr2.x - vr1.x); dv[1] += vw * (vr2.y - vr1.y); dv[2] += vw * (vr2.z - vr1.z);
          const float dp = vj * (ps2.w - ps1.w) * fac;
          gp[0] += dp * drx; gp[1] += dp * dry; gp[2] += dp * drz;
          divr -= vj * fac * rr2;
        }
      }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    shep += __shfl_xor_sync(FULL, shep, o);
    sb += __shfl_xor_sync(FULL, sb, o);
    dv[0] += __shfl_xor_sync(FULL, dv[0], o);
    dv[1] += __shfl_xor_sync(FULL, dv[1], o);
    dv[2] += __shfl_xor_sync(FULL, dv[2], o);
    gp[0] += __shfl_xor_sync(FULL, gp[0], o);
    gp[1] += __shfl_xor_sync(FULL, gp[1], o);
    gp[2] += __shfl_xor_sync(FULL, gp[2], o);
    divr += __shfl_xor_sync(FULL, divr, o);
  }
  shep += c.massfluid / vr1.w * c.awen;  // the particle's own term
  const float g = sqrtf(c.gravity[0] * c.gravity[0] + c.gravity[1] * c.gravity[1] + c.gravity[2] * c.gravity[2]);
  const float ig = g > 0 ? 1.f / g : 1.f;
  const float iv = 1.f / (0.1f * (float)c.cs0);
  const float ip = ig / c.rhopzero;
  const float4 ac = a.acear[p1];
  // lanes 0..15 write one feature each (a coalesced 64-byte row)
  float f;
  switch (lane) {
    case 0: f = (vr1.w / c.rhopzero - 1.f) * 50.f; break;
    case 1: f = dv[0] / shep * iv; break;
    case 2: f = dv[1] / shep * iv; break;
    case 3: f = dv[2] / shep * iv; break;
    case 4: f = gp[0] * ip; break;
    case 5: f = gp[1] * ip; break;
    case 6: f = gp[2] * ip; break;
    case 7: f = shep - 1.f; break;
    case 8: f = divr - 3.f; break;
    case 9: f = ac.x * ig; break;
    case 10: f = ac.y * ig; break;
    case 11: f = ac.z * ig; break;
    case 12: f = sb; break;
    default: f = 0.f;
  }
  if (lane < kIn) feat[(size_t)(p1 - npb) * kIn + lane] = f;
}

// The correction inside the step: one warp per fluid row; the correction
// g*y is applied unless its norm exceeds `limit` times the plain |ace| (the
// row keeps the plain acceleration).  AceMax is taken again over the rows.
__global__ void __launch_bounds__(kMlpBlock) k_closure_apply(gbsph_consts c, DevArrays a,
                                                             const __nv_bfloat16* __restrict__ w,
                                                             const float* __restrict__ feat, float limit,
                                                             unsigned* __restrict__ nfallback) {
  extern __shared__ float smem[];
  float* sw = smem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* act = smem + sNW + warp * kWarpAct;
  load_weights(sw, w);
  const DivState& d = *a.div;
  const unsigned np = d.np, npb = d.npb;
  const float g = sqrtf(c.gravity[0] * c.gravity[0] + c.gravity[1] * c.gravity[1] + c.gravity[2] * c.gravity[2]);
  float amax2 = 0;
  unsigned nfb = 0;
  for (unsigned p1 = npb + blockIdx.x * kMlpWarps + warp; p1 < np; p1 += gridDim.x * kMlpWarps) {
    if (lane < kIn) act[lane] = feat[(size_t)(p1 - npb) * kIn + lane];
    __syncwarp();
    float y[kOut];
    mlp_forward(sw, act, lane, y);
    float4 ac = a.acear[p1];
    const float cx = g * y[0], cy = g * y[1], cz = g * y[2];
    const float cn2 = cx * cx + cy * cy + cz * cz, an2 = ac.x * ac.x + ac.y * ac.y + ac.z * ac.z;
    if (cn2 <= limit * limit * an2) {
      ac.x += cx; ac.y += cy; ac.z += cz;
    } else {
      nfb++;
    }
    if (lane == 0) a.acear[p1] = ac;
    amax2 = gb_fmax_nan(amax2, ac.x * ac.x + ac.y * ac.y + ac.z * ac.z + 0.f * ac.w);
    __syncwarp();
  }
  if (lane == 0) {
    if (!(amax2 <= 0.f)) gb_atomic_max_nonneg(&a.st->acemax2, amax2);
    if (nfb && nfallback) atomicAdd(nfallback, nfb);
  }
}

// Training: forward and backward of n samples (warp per sample), loss =
// mean over samples and outputs of (y - t)^2.  Gradients are summed per block
// in shared memory and added to grad (flat layout); the loss sum to *loss.
__global__ void __launch_bounds__(kMlpBlock) k_mlp_grad(const __nv_bfloat16* __restrict__ w,
                                                        const float* __restrict__ x, const float* __restrict__ t,
                                                        unsigned n, float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ float smem[];
  float* sw = smem;
  float* sg = smem + sNW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* act = smem + 2 * sNW + warp * kWarpAct;
  for (int i = threadIdx.x; i < sNW; i += blockDim.x) sg[i] = 0.f;
  load_weights(sw, w);
  const float inv = 2.f / (3.f * (float)n);
  float lsum = 0;
  for (unsigned s = blockIdx.x * kMlpWarps + warp; s < n; s += gridDim.x * kMlpWarps) {
    if (lane < kIn) act[lane] = x[(size_t)s * kIn + lane];
    __syncwarp();
    float y[kOut];
    mlp_forward(sw, act, lane, y);
    float* h1 = act + kIn;
    float* h2 = h1 + kHid;
    float* h3 = h2 + kHid;
    float* dl = h3 + kHid;
    float g3[kOut];
    for (int o = 0; o < kOut; o++) {
      const float e = y[o] - t[(size_t)s * kOut + o];
      if (lane == 0) lsum += e * e;
      g3[o] = inv * e;
    }
    // output layer
    float d0 = 0, d1 = 0;
    for (int o = 0; o < kOut; o++) {
      atomicAdd(&sg[sW3 + lane * 4 + o], g3[o] * h3[lane]);
      atomicAdd(&sg[sW3 + (lane + 32) * 4 + o], g3[o] * h3[lane + 32]);
      d0 += sw[sW3 + lane * 4 + o] * g3[o];
      d1 += sw[sW3 + (lane + 32) * 4 + o] * g3[o];
    }
    if (lane < kOut) atomicAdd(&sg[sB3 + lane], g3[lane]);
    // hidden layers, last to first: delta of layer l, then its weights
    float* hs[3] = {h1, h2, h3};
    const int wof[3] = {sW0, sW1, sW2}, bof[3] = {sB0, sB1, sB2};
    d0 *= 1.f - h3[lane] * h3[lane];
    d1 *= 1.f - h3[lane + 32] * h3[lane + 32];
    for (int l = 2; l >= 0; l--) {
      dl[lane] = d0;
      dl[lane + 32] = d1;
      __syncwarp();
      const float* in = l == 0 ? act : hs[l - 1];
      const int nin = l == 0 ? kIn : kHid;
      atomicAdd(&sg[bof[l] + lane], d0);
      atomicAdd(&sg[bof[l] + lane + 32], d1);
      for (int k = 0; k < nin; k++) {
        const float v = in[k];
        atomicAdd(&sg[wof[l] + k * kStride + lane], d0 * v);
        atomicAdd(&sg[wof[l] + k * kStride + lane + 32], d1 * v);
      }
      if (l > 0) {
        // delta of the layer below: lanes over its units k = lane, lane + 32
        float e0 = 0, e1 = 0;
        for (int j = 0; j < kHid; j++) {
          const float dj = dl[j];
          e0 = fmaf(sw[wof[l] + lane * kStride + j], dj, e0);
          e1 = fmaf(sw[wof[l] + (lane + 32) * kStride + j], dj, e1);
        }
        const float* hb = hs[l - 1];
        d0 = e0 * (1.f - hb[lane] * hb[lane]);
        d1 = e1 * (1.f - hb[lane + 32] * hb[lane + 32]);
      }
      __syncwarp();
    }
  }
  for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0 && lsum != 0.f) atomicAdd(loss, lsum / (3.f * (float)n));
  __syncthreads();
  for (int i = threadIdx.x; i < kNParams; i += blockDim.x) {
    const float v = sg[smem_index(i)];
    if (v != 0.f) atomicAdd(&grad[i], v);
  }
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; writes the BF16 copy
// the kernels use and clears the gradient.
__global__ void k_adam(float* __restrict__ master, __nv_bfloat16* __restrict__ w, float* __restrict__ grad,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kNParams) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float p = master[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  master[i] = p;
  w[i] = __float2bfloat16_rn(p);
  grad[i] = 0.f;
}

__global__ void k_to_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

// Inference on given features (tests, evaluation): y for n samples.
__global__ void __launch_bounds__(kMlpBlock) k_mlp_infer(const __nv_bfloat16* __restrict__ w,
                                                         const float* __restrict__ x, unsigned n,
                                                         float* __restrict__ y) {
  extern __shared__ float smem[];
  float* sw = smem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* act = smem + sNW + warp * kWarpAct;
  load_weights(sw, w);
  for (unsigned s = blockIdx.x * kMlpWarps + warp; s < n; s += gridDim.x * kMlpWarps) {
    if (lane < kIn) act[lane] = x[(size_t)s * kIn + lane];
    __syncwarp();
    float out[kOut];
    mlp_forward(sw, act, lane, out);
    if (lane < kOut) y[(size_t)s * kOut + lane] = out[lane];
    __syncwarp();
  }
}

constexpr size_t kSmemInfer = sizeof(float) * (sNW + kMlpWarps * kWarpAct);
constexpr size_t kSmemGrad = sizeof(float) * (2 * sNW + kMlpWarps * kWarpAct);

unsigned mlp_grid(unsigned n) {
  const unsigned g = gb_div_up(n, kMlpWarps);
  return g < 152u * 4u ? (g ? g : 1u) : 152u * 4u;
}

}  // namespace

namespace gbk {

cudaError_t closure_init() {
  cudaError_t e = cudaFuncSetAttribute(k_closure_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemInfer);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemInfer);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemGrad);
  return e;
}

void closure_features(const gbsph_consts& c, const DevArrays& a, unsigned cap, float* feat, cudaStream_t s,
                      unsigned long long* nlaunch) {
  k_closure_features<<<gb_div_up(cap, 4), 128, 0, s>>>(c, a, feat);  // a warp per row
  if (nlaunch) *nlaunch += 1;
}

void closure_apply(const gbsph_consts& c, const DevArrays& a, unsigned cap, const void* w_bf16, const float* feat,
                   float limit, unsigned* nfallback, cudaStream_t s, unsigned long long* nlaunch) {
  cudaMemsetAsync(&a.st->acemax2, 0, sizeof(unsigned), s);
  k_closure_apply<<<mlp_grid(cap), kMlpBlock, kSmemInfer, s>>>(c, a, (const __nv_bfloat16*)w_bf16, feat, limit,
                                                               nfallback);
  if (nlaunch) *nlaunch += 1;
}

void mlp_infer(const void* w_bf16, const float* x, unsigned n, float* y, cudaStream_t s) {
  if (n) k_mlp_infer<<<mlp_grid(n), kMlpBlock, kSmemInfer, s>>>((const __nv_bfloat16*)w_bf16, x, n, y);
}

void mlp_grad(const void* w_bf16, const float* x, const float* t, unsigned n, float* grad, float* loss,
              cudaStream_t s) {
  if (n) k_mlp_grad<<<mlp_grid(n), kMlpBlock, kSmemGrad, s>>>((const __nv_bfloat16*)w_bf16, x, t, n, grad, loss);
}

void mlp_adam(float* master, void* w_bf16, float* grad, float* m, float* v, float lr, float b1, float b2, float eps,
              float bc1, float bc2, cudaStream_t s) {
  k_adam<<<gb_div_up(kNParams, 256), 256, 0, s>>>(master, (__nv_bfloat16*)w_bf16, grad, m, v, lr, b1, b2, eps, bc1,
                                                  bc2);
}

void to_bf16(const float* src, void* dst, int n, cudaStream_t s) {
  k_to_bf16<<<gb_div_up((unsigned)n, 256), 256, 0, s>>>(src, (__nv_bfloat16*)dst, n);
}

}  // namespace gbk
