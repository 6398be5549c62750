// The tcgen05 form of the matrix-free FP32 fine-level operator (k_mf_tc,
// mf_tc.cuh): launches and the set-up (K0 split into TF32 hi / lo parts in
// the MMA operand layout; column / z-segment work decomposition).
#include "fem_state.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace topt {

// Tensor-core variant: persistent, two CTAs per SM over (column, z segment)
// work items; node planes and the drainers' per-layer data in rings of
// kMfTcNpl and kMfTcNel, suspending mbarrier waits.
constexpr int kMfTcNpl = 6, kMfTcNel = 4, kMfTcWait = 1;

template <int MODE, bool DOT, bool COLMASK>
static int launch_mf_tc(topt_fem* h, const float* x, const float* b, float* y, int slot) {
  constexpr uint32_t smem = mftc::smem_bytes(kMfTcNpl, kMfTcNel);
  auto kern = k_mf_tc<MODE, DOT, COLMASK, kMfTcNpl, kMfTcNel, kMfTcWait>;
  static bool attr_set = false;   // per instantiation, process-wide
  if (!attr_set) {
    TOPT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    attr_set = true;
  }
  const MfTcGrid& G = h->mftc;
  const int64_t items = (int64_t)G.ncy * G.ncx * G.nseg;
  const int grid = (int)std::min<int64_t>(items, (int64_t)h->sm * 2);
  kern<<<grid, mftc::THREADS, smem, h->stream>>>(
      G, h->k0img.as<float>(), h->coef32.as<float>(), h->nmask32.as<uint32_t>(), x, b, y,
      h->red.partials.as<double>(), h->red.ctr(slot), h->red.res(slot),
      h->mf_err.as<int>());
  TOPT_CHECK_LAUNCH("k_mf_tc");
  return TOPT_OK;
}

// Round to TF32 (10-bit mantissa), nearest with ties away from zero: the
// rounding of cvt.rna.tf32.f32, for the host-built K0 image.
static float tf32_rna_host(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

// K0 split into TF32 hi and lo parts, rows padded to N = 32, in the K-major
// operand layout of k_mf_tc; and the column / z-segment decomposition that
// balances the work items over two CTAs per SM.
int setup_mf_tc(topt_fem* h, cudaStream_t s) {
  std::vector<float> img(mftc::K0_IMAGE_FLOATS, 0.0f);
  for (int n = 0; n < 32; ++n)
    for (int k = 0; k < 24; ++k) {
      const float v = n < 24 ? h->k0.v[n * 24 + k] : 0.0f;
      const float hi = tf32_rna_host(v);
      const float lo = tf32_rna_host(v - hi);
      const uint32_t o = tc::kmaj_off(n, k, mftc::SBO_B) / 4;
      img[o] = hi;
      img[32 * 24 + o] = lo;
    }
  int rc = upload(h->k0img, img.data(), img.size(), s);
  if (rc) return rc;
  if ((rc = h->mf_err.alloc(sizeof(int)))) return rc;
  TOPT_CUDA(cudaMemsetAsync(h->mf_err.p, 0, sizeof(int), s));
  MfTcGrid& G = h->mftc;
  G.g = h->mfg;
  const int ny1 = h->mfg.ny + 1, nx1 = h->mfg.nx + 1, nz1 = h->mfg.nz + 1;
  G.ncy = (ny1 + mftc::NY - 1) / mftc::NY;
  G.ncx = (nx1 + mftc::NX - 1) / mftc::NX;
  const int64_t cols = (int64_t)G.ncy * G.ncx, slots = (int64_t)h->sm * 2;
  int64_t best = -1;
  for (int nseg = 1; nseg <= nz1; ++nseg) {
    const int zs = (nz1 + nseg - 1) / nseg;
    const int used = (nz1 + zs - 1) / zs;
    const int64_t items = cols * used;
    const int64_t waves = (items + slots - 1) / slots;
    const int64_t cost = waves * (zs + 2);
    if (best < 0 || cost < best) {
      best = cost;
      G.nseg = used;
      G.zs = zs;
    }
  }
  TOPT_CUDA(cudaStreamSynchronize(s));
  return TOPT_OK;
}

int mf_tc_apply(topt_fem* h, int mode, bool dot, bool colmask, const float* x, const float* b,
                float* y, int slot) {
  if (mode == 0 && !dot)
    return colmask ? launch_mf_tc<0, false, true>(h, x, b, y, slot)
                   : launch_mf_tc<0, false, false>(h, x, b, y, slot);
  if (mode == 0)
    return colmask ? launch_mf_tc<0, true, true>(h, x, b, y, slot)
                   : launch_mf_tc<0, true, false>(h, x, b, y, slot);
  if (mode == 1)
    return colmask ? launch_mf_tc<1, false, true>(h, x, b, y, slot)
                   : launch_mf_tc<1, false, false>(h, x, b, y, slot);
  if (mode == 2)
    return colmask ? launch_mf_tc<2, false, true>(h, x, b, y, slot)
                   : launch_mf_tc<2, false, false>(h, x, b, y, slot);
  return fail(TOPT_BAD_INPUT, "mf_tc_apply: unsupported mode");
}

int launches_mf_tc(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}

}  // namespace topt
