// gbsph_fluid_lam.cu -- the fluid-row kernels of one viscosity model
// (GBSPH_VISCO_LAMINAR), instantiated apart from the others so that they compile in
// parallel (gbsph_fluid.cuh).
#pragma nv_diag_suppress 177
#include "gbsph_fluid.cuh"
#pragma nv_diag_default 177

namespace gbk {

cudaError_t fluid_laminar(const gbsph_consts& c, const DevArrays& a, unsigned cap, int variant, int bsize, int split,
                 bool prepare, cudaStream_t s) {
  return launch_fluid_t<GBSPH_VISCO_LAMINAR>(c, a, cap, variant, bsize, split, prepare, s);
}

}  // namespace gbk
