// The matrix-free FP32 fine-level operator of uniform hex grids: FP32-FMA
// node tiles (k_mf_tile, the default) or the tcgen05 kernel of mf_tc.cu,
// followed, when the caller asks for a Chebyshev step on the residual it
// produced, by the separate pass k_cheb_stored.
#include "fem_state.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace topt {

template <int TY, int MODE, bool DOT, bool COLMASK>
static int launch_mf_tile(topt_fem* h, const float* x, const float* b, float* y, int slot) {
  static bool attr_set = false;   // per instantiation, process-wide
  if (!attr_set) {
    TOPT_CUDA(cudaFuncSetAttribute(k_mf_tile<TY, MODE, DOT, COLMASK>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   MfTile<TY>::SMEM));
    attr_set = true;
  }
  k_mf_tile<TY, MODE, DOT, COLMASK><<<h->sm * kMfCtasPerSm, kMfThreads, MfTile<TY>::SMEM,
                                      h->stream>>>(
      h->mfg, h->k0, h->coef32.as<float>(), h->nmask32.as<uint32_t>(), x, b, y,
      h->red.partials.as<double>(), h->red.ctr(slot), h->red.res(slot));
  TOPT_CHECK_LAUNCH("k_mf_tile");
  return TOPT_OK;
}


template <int MODE, bool DOT, bool COLMASK>
static int launch_mf_ty(topt_fem* h, const float* x, const float* b, float* y, int slot) {
  if (h->mf_ty == 27) return launch_mf_tile<27, MODE, DOT, COLMASK>(h, x, b, y, slot);
  if (h->mf_ty == 16) return launch_mf_tile<16, MODE, DOT, COLMASK>(h, x, b, y, slot);
  return launch_mf_tile<32, MODE, DOT, COLMASK>(h, x, b, y, slot);
}

template <int L, int MODE, bool DOT>
static int launch_mf(topt_fem* h, const float* x, const float* b, float* y, int slot,
                     const ChebEp<float>& ep, bool zero_fixed) {
  if (L == 1) {
    int rc;
    if (h->mf_kernel == 1)
      rc = mf_tc_apply(h, MODE, DOT, !zero_fixed, x, b, y, slot);
    else
      rc = zero_fixed ? launch_mf_ty<MODE, DOT, false>(h, x, b, y, slot)
                      : launch_mf_ty<MODE, DOT, true>(h, x, b, y, slot);
    if (rc) return rc;
    if (ep.kind) {
      k_cheb_stored<<<gridsize(h, h->n_nodes), kBlock, 0, h->stream>>>(h->n_nodes, ep, y);
      TOPT_CHECK_LAUNCH("k_cheb_stored");
    }
    return TOPT_OK;
  }
  k_mf_apply<float, L, MODE, DOT><<<gridsize(h, h->n_nodes), kBlock, 0, h->stream>>>(
      h->mfg, h->ke32.as<float>(), h->coef32.as<float>(), h->mask.as<uint8_t>(), x, b, y,
      h->red.partials.as<double>(), h->red.ctr(slot), h->red.res(slot), ep);
  TOPT_CHECK_LAUNCH("k_mf_apply");
  return TOPT_OK;
}

int mf_spmv(topt_fem* h, int L, int mode, bool dot, const float* x, const float* b, float* y,
            int slot, const ChebEp<float>& ep, bool zf) {
#define TOPT_MF_CASE(L_)                                                            \
  if (L == L_) {                                                                    \
    if (mode == 0 && !dot) return launch_mf<L_, 0, false>(h, x, b, y, slot, ep, zf); \
    if (mode == 0 && dot) return launch_mf<L_, 0, true>(h, x, b, y, slot, ep, zf);   \
    if (mode == 1) return launch_mf<L_, 1, false>(h, x, b, y, slot, ep, zf);         \
    if (mode == 2) return launch_mf<L_, 2, false>(h, x, b, y, slot, ep, zf);         \
  }
  TOPT_MF_CASE(1) TOPT_MF_CASE(2) TOPT_MF_CASE(3) TOPT_MF_CASE(4)
#undef TOPT_MF_CASE
  return fail(TOPT_BAD_INPUT, "mf_spmv: unsupported nrhs");
}

int launches_mf(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}

}  // namespace topt
