// Operator applications of the FEM handle: the SELL-32 block products of
// every level (warp per row, three threads per row or one thread per row by
// level size); level 0 of a matrix-free FP32 handle goes to mf.cu.
#include "fem_state.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace topt {

// Coarse-level product shapes by level size: one warp per block row up to
// kWarpRowsMax rows, three threads per row (3x3 blocks) up to kRow3Max, one
// thread per row above; a level's row_map overrides the rule.
static const int64_t kWarpRowsMax = 16384;
static const int64_t kRow3Max = 131072;

int row_mapping(const LevelStruct& Ls, int bs) {
  if (Ls.row_map == 1 || Ls.row_map == 3 || (Ls.row_map == 2 && bs == 3)) return Ls.row_map;
  if (bs == 3 && Ls.n_nodes > kWarpRowsMax && Ls.n_nodes <= kRow3Max) return 2;
  if (Ls.n_nodes <= kWarpRowsMax) return 1;
  return 3;
}

template <typename T, int BS, int L, int MODE, bool DOT>
static int launch_spmv(topt_fem* h, const LevelStruct& Ls, const T* vals, const T* x,
                       const T* b, T* y, int red_slot, const ChebEp<T>& ep) {
  const int map = row_mapping(Ls, BS);
  if (map == 2) {
    const int g = grid_for((Ls.n_nodes + 63) / 64, 1, h->sm * 16);
    k_sell_spmv3<T, L, MODE, DOT><<<g, 192, 0, h->stream>>>(
        Ls.sell, vals, x, b, y, h->red.partials.as<double>(), h->red.ctr(red_slot),
        h->red.res(red_slot), ep);
    TOPT_CHECK_LAUNCH("k_sell_spmv3");
    return TOPT_OK;
  }
  if (map == 1) {
    const int g = gridsize(h, Ls.n_nodes * 32);
    k_sell_spmv_warp<T, BS, L, MODE, DOT><<<g, kBlock, 0, h->stream>>>(
        Ls.sell, vals, x, b, y, h->red.partials.as<double>(), h->red.ctr(red_slot),
        h->red.res(red_slot), ep);
    TOPT_CHECK_LAUNCH("k_sell_spmv_warp");
    return TOPT_OK;
  }
  const int g = gridsize(h, Ls.n_nodes);
  k_sell_spmv<T, BS, L, MODE, DOT><<<g, kBlock, 0, h->stream>>>(
      Ls.sell, vals, x, b, y, h->red.partials.as<double>(), h->red.ctr(red_slot),
      h->red.res(red_slot), ep);
  TOPT_CHECK_LAUNCH("k_sell_spmv");
  return TOPT_OK;
}

// MODE 0 y=Ax, 1 y=b-Ax, 2 y-=Ax; dot -> red slot
// zero_fixed: x is known to vanish on the fixed DOFs (every operand inside the
// solvers), so the matrix-free operator may skip zeroing them.
template <typename T>
int spmv(topt_fem* h, const LevelStruct& Ls, int bs, int L, int mode, bool dot, const T* vals,
         const T* x, const T* b, T* y, int slot, const ChebEp<T>& ep, bool zero_fixed) {
  if (std::is_same<T, float>::value && h->mf && &Ls == &h->ls[0])
    return mf_spmv(h, L, mode, dot, (const float*)x, (const float*)b, (float*)y, slot,
                   reinterpret_cast<const ChebEp<float>&>(ep), zero_fixed);
#define TOPT_SPMV_CASE(BS_, L_)                                                        \
  if (bs == BS_ && L == L_) {                                                          \
    if (mode == 0 && !dot)                                                             \
      return launch_spmv<T, BS_, L_, 0, false>(h, Ls, vals, x, b, y, slot, ep);        \
    if (mode == 0 && dot)                                                              \
      return launch_spmv<T, BS_, L_, 0, true>(h, Ls, vals, x, b, y, slot, ep);         \
    if (mode == 1) return launch_spmv<T, BS_, L_, 1, false>(h, Ls, vals, x, b, y, slot, ep); \
    if (mode == 2) return launch_spmv<T, BS_, L_, 2, false>(h, Ls, vals, x, b, y, slot, ep); \
  }
  TOPT_SPMV_CASE(3, 1) TOPT_SPMV_CASE(3, 2) TOPT_SPMV_CASE(3, 3) TOPT_SPMV_CASE(3, 4)
  TOPT_SPMV_CASE(1, 1) TOPT_SPMV_CASE(1, 2) TOPT_SPMV_CASE(1, 3) TOPT_SPMV_CASE(1, 4)
#undef TOPT_SPMV_CASE
  return fail(TOPT_BAD_INPUT, "spmv: unsupported bs/nrhs");
}

template int spmv<float>(topt_fem*, const LevelStruct&, int, int, int, bool, const float*,
                         const float*, const float*, float*, int, const ChebEp<float>&, bool);
template int spmv<double>(topt_fem*, const LevelStruct&, int, int, int, bool, const double*,
                          const double*, const double*, double*, int, const ChebEp<double>&,
                          bool);

int launches_spmv(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}

}  // namespace topt
