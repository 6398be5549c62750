// State of the FEM handle shared by the engine's translation units:
// fem.cu (creation, patterns, refresh of the hierarchy, V-cycle, PCG drivers
// and the C-ABI), spmv.cu (SELL block products of every level), mf.cu and
// mf_tc.cu (the matrix-free FP32 fine-level operator: FP32-FMA and tcgen05
// kernels) and amg.cu (the smoothed-aggregation hierarchy of meshes without
// a logical grid).
#pragma once

#include "fem_kernels.cuh"
#include "mf_tc.cuh"

#include <vector>

namespace topt {

constexpr int kBlock = 256;

struct LevelStruct {
  int64_t n_nodes = 0, n_elem = 0, nnzb = 0, npos = 0;
  int nloc = 8;
  int nx = 0, ny = 0, nz = 0;     // cells (grid levels)
  // SELL-32 block pattern (see SellT) + element contributions per position
  DevBuf grp_of_slice, slice_of_grp, col, rowlen, diagpos, cptr, contrib, csr2sell, t;
  SellT sell{};
  // cell -> element lists (level 0 only, when elements are not the cells)
  DevBuf cell_ptr, cell_elems;
  // transfer tables to the next coarser level (per axis)
  DevBuf cmx, cmy, cmz, c0x, c0y, c0z, w1x, w1y, w1z, r0x, r0y, r0z, rwx, rwy, rwz;
  GridT grid{};
  // shared-matrix Galerkin fast path (level 0 -> 1 of uniform hex meshes)
  DevBuf gal_M64, gal_M32, gal_masked, gal_list;
  int64_t n_gal_list = 0;
  bool gal_shared = false;
  bool dense = false;             // coarsest level solved densely
  int ndense = 0;
  // SELL product row mapping: 0 by level size (warp per row up to
  // kWarpRowsMax rows, three threads per row up to kRow3Max, then one
  // thread per row), 1 warp per row, 2 three threads per row (bs 3), 3 one
  // thread per row (set by topt_fem_set_row_mapping, e.g. by an autotuner)
  int row_map = 0;
  // smoothed-aggregation transfer to the next level (meshes without a grid;
  // amg_kernels.cuh): np blocks of P, nap of A P, nc_ent of the next level's
  // operator, each with the list of products summed into it
  bool amg = false;
  int64_t np = 0, nap = 0, nc_ent = 0;
  DevBuf cnt;                     // free finest-level DOFs below each DOF (every AMG level)
  DevBuf agg;                     // node -> aggregate (next level's node)
  DevBuf p_ptr, p_col, p_row, p_first, p_pos;
  DevBuf r_ptr, r_fine, r_pent;
  DevBuf ap_ptr, ap_col, ap_first, ap_pos, ap_pent;
  DevBuf c_first, c_pent, c_apent, c_pos;
  // mixed handles: the transfer values are formed in FP64 (P = T - s Dinv A T
  // and P^T A P cancel to small entries that FP32 products would swamp) and
  // rounded for the FP32 hierarchy; this level's FP64 operator (coarse
  // levels), block inverse, P and A P
  DevBuf a64_vals, a64_dinv, a64_pv, a64_apv;
};

template <typename T>
struct LevelNum {
  DevBuf ke;        // coarse levels: Galerkin cell matrices
  DevBuf vals, dinv;
  DevBuf b, x, r, d, q;
  DevBuf dense_inv;
  DevBuf pw;              // power-iteration vector (unit norm once pw_ready)
  bool pw_ready = false;
  double lmax = 0.0;
  DevBuf pv, apv;         // smoothed-aggregation transfer: P and A P blocks
};

template <typename T>
struct Hier {
  std::vector<LevelNum<T>> lv;
  bool built = false;
  DevBuf dense_scratch;   // FP64 copy of the coarsest operator for its inverse
};

// One preconditioner application (a whole V-cycle) recorded as a CUDA graph
// and replayed while the hierarchy, the operands and the smoother stay the
// same; a hierarchy refresh marks it stale, and the second application after
// it re-records it (cudaGraphExecUpdate when the kernel list is unchanged).
struct VcycleGraph {
  cudaGraphExec_t exec = nullptr;
  const void* r = nullptr;
  void* z = nullptr;
  int L = 0, degree = 0;
  bool fp32 = false;
  double cheb_ratio = 0.0;
  bool direct_done = false;      // applied once directly since the last refresh
  bool valid = false;            // exec holds the current hierarchy's V-cycle
  unsigned long long used = 0;   // last use (eviction order)
};
constexpr int kVcycleGraphs = 4;

struct Reducer {
  DevBuf partials, counter, out;
  int max_blocks = 0;
  int init(int blocks) {
    max_blocks = blocks;
    int rc = partials.alloc((size_t)blocks * 8 * sizeof(double));
    if (rc) return rc;
    rc = counter.alloc(64 * sizeof(unsigned));
    if (rc) return rc;
    TOPT_CUDA(cudaMemset(counter.p, 0, 64 * sizeof(unsigned)));
    rc = out.alloc(128 * sizeof(double));
    return rc;
  }
  unsigned* ctr(int i) const { return counter.as<unsigned>() + i; }
  double* res(int i) const { return out.as<double>() + 8 * i; }
};

}  // namespace topt

struct topt_fem {
  int bs = 3, nloc = 8;
  int64_t n_nodes = 0, n_elem = 0, n_dof = 0, n_ke = 1;
  bool mixed = false, has_grid = false;
  int mg_levels = 1, mg_coarse_max = 192;
  cudaStream_t stream = nullptr;
  // side stream of the coarsest dense inverse (overlapped with the
  // Chebyshev bounds of the other levels), created on first use
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int sm = 152;
  std::vector<topt::LevelStruct> ls;   // level 0 = fine mesh
  topt::DevBuf mask;                   // level-0 Dirichlet flags (uint8 per DOF)
  topt::DevBuf ke64, ke32;             // level-0 unit element matrices
  topt::DevBuf coef64, coef32;
  topt::DevBuf vals64_0;               // level-0 FP64 operator (always kept)
  topt::Hier<double> h64;
  topt::Hier<float> h32;
  topt::Reducer red;
  // PCG / refinement work vectors (n_dof x 8 max loads)
  topt::DevBuf fe, R, U0;
  topt::DevBuf Ubest;                  // best iterate of a stagnating refinement
  topt::DevBuf active;                 // per-load "still iterating" flags (4 ints)
  int lmax_alloc = 0;
  double E0 = 1.0, Emin = 0.0, p = 3.0;
  int interp = 0;                      // 0 SIMP, 1 RAMP, 2 RAMP / SIMP-form sensitivity
  // element energies and sensitivities in FP32 arithmetic (opt-in: measured
  // 1.2e-6 relative L2 on the sensitivities of the 240x80x80 loop, above the
  // 1e-6 gate, so the default stays FP64)
  bool energy32 = false;
  // per-element matrices added to coef_e Ke at level 0 (caller's device
  // buffer, n_elem x (bs nloc)^2 FP64; the heat plugin's Robin terms)
  const double* extra64 = nullptr;
  topt::DevBuf extra32;                // FP32 copy for the mixed hierarchy
  topt::DevBuf full64;                 // level-0 FP64 operator without enforcement
  bool full_ok = false;                // full64 holds the current operator
  double cheb_ratio = 30.0;            // smoother interval [lmax/ratio, lmax]
  bool x0 = false;                     // this solve starts from the caller's U
  bool assembled = false;
  // matrix-free FP32 level-0 operator (uniform hex grid, shared unit matrix)
  bool mf = false;
  topt::MfGrid mfg{};
  int mf_ty = 32;                      // y extent of the operator's node tiles
  topt::K0f k0{};                      // FP32 unit matrix (by-value kernel parameter)
  // fine-level operator kernel: 0 = FP32-FMA tiles (k_mf_tile, the default:
  // measured faster), 1 = tensor cores (k_mf_tc)
  int mf_kernel = 0;
  topt::MfTcGrid mftc{};
  topt::DevBuf k0img;                  // K0 hi / lo in the MMA operand layout
  topt::DevBuf mf_err;                 // set by k_mf_tc if an mbarrier wait times out
  topt::DevBuf nmask32;                // nmask widened to 32 bits (cp.async granule)
  topt::DevBuf nmask;                  // fixed flags of a node's 3 DOFs, bits 0-2
  // V-cycles replayed as CUDA graphs (recorded on a private non-blocking
  // stream, thread-local capture mode, so handles stepped from several host
  // threads record concurrently)
  bool vc_graphs = true;
  cudaStream_t cap = nullptr;
  topt::VcycleGraph vcg[topt::kVcycleGraphs];
  unsigned long long vc_clock = 0;
};

namespace topt {

inline int gridsize(const topt_fem* h, int64_t n, int block = kBlock) {
  return grid_for(n, block, h->sm * 16);
}

}  // namespace topt

namespace topt {

#define TOPT_BSL_DISPATCH(bs, L, CALL)                         \
  do {                                                         \
    if (bs == 3) {                                             \
      if (L == 1) { constexpr int BS_ = 3, L_ = 1; CALL; }     \
      else if (L == 2) { constexpr int BS_ = 3, L_ = 2; CALL; } \
      else if (L == 3) { constexpr int BS_ = 3, L_ = 3; CALL; } \
      else { constexpr int BS_ = 3, L_ = 4; CALL; }            \
    } else {                                                   \
      if (L == 1) { constexpr int BS_ = 1, L_ = 1; CALL; }     \
      else if (L == 2) { constexpr int BS_ = 1, L_ = 2; CALL; } \
      else if (L == 3) { constexpr int BS_ = 1, L_ = 3; CALL; } \
      else { constexpr int BS_ = 1, L_ = 4; CALL; }            \
    }                                                          \
  } while (0)

#define TOPT_L_DISPATCH(L, CALL)                                \
  do {                                                          \
    if (L == 1) { constexpr int L_ = 1; CALL; }                 \
    else if (L == 2) { constexpr int L_ = 2; CALL; }            \
    else if (L == 3) { constexpr int L_ = 3; CALL; }            \
    else { constexpr int L_ = 4; CALL; }                        \
  } while (0)

// ---------------------------------------------------------------- across units
// spmv.cu: y = A x (mode 0), y = b - A x (1), y -= A x (2) on level Ls, with
// the dot product x.y into reducer slot `slot` (dot) and the Chebyshev step
// of `ep` fused into the epilogue; zero_fixed: x is known to vanish on the
// fixed DOFs.  Level 0 of a matrix-free FP32 handle uses the matrix-free
// operator.
template <typename T>
int spmv(topt_fem* h, const LevelStruct& Ls, int bs, int L, int mode, bool dot, const T* vals,
         const T* x, const T* b, T* y, int slot = 0, const ChebEp<T>& ep = ChebEp<T>(),
         bool zero_fixed = false);
extern template int spmv<float>(topt_fem*, const LevelStruct&, int, int, int, bool, const float*,
                                const float*, const float*, float*, int, const ChebEp<float>&,
                                bool);
extern template int spmv<double>(topt_fem*, const LevelStruct&, int, int, int, bool,
                                 const double*, const double*, const double*, double*, int,
                                 const ChebEp<double>&, bool);
// spmv.cu: the SELL row mapping a level's products use (1 warp per row, 2
// three threads per row, 3 one thread per row)
int row_mapping(const LevelStruct& Ls, int bs);
// mf.cu: the matrix-free FP32 level-0 operator (same modes as spmv)
int mf_spmv(topt_fem* h, int L, int mode, bool dot, const float* x, const float* b, float* y,
            int slot, const ChebEp<float>& ep, bool zf);
// mf_tc.cu: the tcgen05 kernel (mode / dot as spmv; colmask: zero the fixed
// DOFs of x on the fly) and its set-up
int mf_tc_apply(topt_fem* h, int mode, bool dot, bool colmask, const float* x, const float* b,
                float* y, int slot);
int setup_mf_tc(topt_fem* h, cudaStream_t s);
// amg.cu: the smoothed-aggregation hierarchy (patterns, once per mesh), the
// values of the transfer from level li (every refresh) and its application
// in the V-cycle (restriction with the coarse level's first Chebyshev step,
// prolongation)
int setup_amg(topt_fem* h);
template <typename T>
int amg_galerkin(topt_fem* h, int li, Hier<T>& H);
template <typename T>
int amg_restrict(topt_fem* h, int li, Hier<T>& H, int L, const uint8_t* mask, const T* dinv_c,
                 T c2c);
template <typename T>
int amg_prolong(topt_fem* h, int li, Hier<T>& H, int L, const uint8_t* mask, T* x);
#define TOPT_AMG_EXTERN(T)                                                                \
  extern template int amg_galerkin<T>(topt_fem*, int, Hier<T>&);                          \
  extern template int amg_restrict<T>(topt_fem*, int, Hier<T>&, int, const uint8_t*,      \
                                      const T*, T);                                       \
  extern template int amg_prolong<T>(topt_fem*, int, Hier<T>&, int, const uint8_t*, T*);
TOPT_AMG_EXTERN(float)
TOPT_AMG_EXTERN(double)
#undef TOPT_AMG_EXTERN

}  // namespace topt
