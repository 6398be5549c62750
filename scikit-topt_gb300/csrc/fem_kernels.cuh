// Device kernels of the FEM engine: SIMP coefficients, fixed-pattern BSR
// assembly with Dirichlet enforcement, BSR SpMV/SpMM, PCG vector updates,
// block-Jacobi, Chebyshev smoothing, structured-grid transfer operators,
// element-level Galerkin coarsening, dense coarsest solve and element
// energies.  Vectors with several load cases are stored n_dof x L row-major
// (value of DOF i, load j at i*L + j), the layout of the reference's u_dofs.
#pragma once

#include "cuda_common.cuh"

namespace topt {

// --------------------------------------------------------------------------
// Material interpolation E(rho): interp 0 SIMP, Emin + (E0 - Emin) rho^p
// (composer.py:19-22); 1 RAMP, Emin + (E0 - Emin) rho / (1 + p (1 - rho))
// (composer.py:25-39); 2 RAMP operator whose sensitivity keeps the SIMP form
// (the heat plugin, solver_heat.py:928-950, calls dC_drho_simp whatever the
// interpolation).
__device__ __forceinline__ double interp_E(int interp, double r, double E0, double Emin,
                                           double p) {
  if (interp == 1 || interp == 2) return Emin + (E0 - Emin) * (r / (1.0 + p * (1.0 - r)));
  return Emin + (E0 - Emin) * (p == 3.0 ? r * r * r : pow(r, p));
}

static __global__ void k_d2f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

static __global__ void k_simp_coef(int64_t n, const double* __restrict__ rho, double E0,
                            double Emin, double p, double* __restrict__ c64,
                            float* __restrict__ c32, int interp) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double r = rho[i];
    const double v = interp_E(interp, r, E0, Emin, p);
    if (c64) c64[i] = v;
    if (c32) c32[i] = (float)v;
  }
}

// --------------------------------------------------------------------------
// Sliced-ELL block storage (SELL-32, bs x bs blocks).  Block rows (nodes) are
// grouped in slices of 32; every slice is padded to its longest row and
// stored column by column, so block j of the 32 rows of a slice occupies one
// "group" of 32 consecutive positions.  Block values are stored plane by
// plane inside a group: value v of the block at position p lives at
// ((p >> 5) * bs*bs + v) * 32 + (p & 31), so a warp reads each plane with
// one coalesced 32-wide access.  Padding blocks point at their own row and
// hold zeros.
struct SellT {
  int64_t nrows;
  const int32_t* grp_of_slice;  // nslices + 1
  const int32_t* slice_of_grp;  // ngroups
  const int32_t* col;           // npos
  const int32_t* rowlen;        // nrows
  const int32_t* diag;          // nrows, position of the diagonal block
};

// local node offsets of a hex cell (MeshHex order)
static __constant__ int c_hex_off[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 0, 0}, {0, 0, 1},
                                    {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 1}};

template <int BS>
__device__ __forceinline__ int64_t vidx(int64_t p, int v) {
  return ((p >> 5) * (BS * BS) + v) * 32 + (p & 31);
}

// Fixed-pattern assembly: one thread per block position sums its element
// contributions in ascending element order (deterministic, no atomics).
// ke_stride == 0 means one matrix shared by all elements (kept in shared
// memory).  extra (optional, one (BS NLOC)^2 matrix per element) is added
// unscaled: the heat plugin's Robin terms.  mask (per DOF) applies
// skfem.enforce: rows and columns of fixed DOFs are zeroed and their
// diagonal set to 1.
template <typename T, int BS, int NLOC>
__global__ void k_assemble(int64_t npos, SellT sp, const int64_t* __restrict__ cptr,
                           const int32_t* __restrict__ contrib,
                           const T* __restrict__ ke, int64_t ke_stride,
                           const T* __restrict__ coef, const T* __restrict__ extra,
                           const uint8_t* __restrict__ mask, T* __restrict__ vals) {
  TOPT_KERNEL_COUNT();
  constexpr int ND = BS * NLOC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* kes = reinterpret_cast<T*>(smem_raw);
  if (ke_stride == 0) {
    for (int i = threadIdx.x; i < ND * ND; i += blockDim.x) kes[i] = ke[i];
    __syncthreads();
  }
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npos;
       k += (int64_t)gridDim.x * blockDim.x) {
    T acc[BS * BS];
#pragma unroll
    for (int i = 0; i < BS * BS; ++i) acc[i] = T(0);
    const int64_t c1 = cptr[k + 1];
    for (int64_t c = cptr[k]; c < c1; ++c) {
      const int32_t code = contrib[c];
      const int32_t e = code / (NLOC * NLOC);
      const int r = code - e * (NLOC * NLOC);
      const int la = r / NLOC, lb = r - la * NLOC;
      const T* K = ke_stride ? ke + (int64_t)e * ke_stride : kes;
      const T s = coef ? coef[e] : T(1);
#pragma unroll
      for (int c0 = 0; c0 < BS; ++c0)
#pragma unroll
        for (int d0 = 0; d0 < BS; ++d0)
          acc[c0 * BS + d0] += s * K[(BS * la + c0) * ND + BS * lb + d0];
      if (extra) {
        const T* X = extra + (int64_t)e * (ND * ND);
#pragma unroll
        for (int c0 = 0; c0 < BS; ++c0)
#pragma unroll
          for (int d0 = 0; d0 < BS; ++d0)
            acc[c0 * BS + d0] += X[(BS * la + c0) * ND + BS * lb + d0];
      }
    }
    if (mask) {
      const int64_t a = (int64_t)sp.slice_of_grp[k >> 5] * 32 + (k & 31);
      if (a < sp.nrows) {
        const int64_t b = sp.col[k];
        const bool is_diag = (sp.diag[a] == k);
#pragma unroll
        for (int c0 = 0; c0 < BS; ++c0)
#pragma unroll
          for (int d0 = 0; d0 < BS; ++d0) {
            const bool ma = mask[BS * a + c0], mb = mask[BS * b + d0];
            if (ma || mb) acc[c0 * BS + d0] = (is_diag && c0 == d0 && ma) ? T(1) : T(0);
          }
      }
    }
#pragma unroll
    for (int i = 0; i < BS * BS; ++i) vals[vidx<BS>(k, i)] = acc[i];
  }
}

// Coarse levels: a DOF whose prolongation column is empty has an all-zero
// row and column; give it a unit diagonal so the level stays nonsingular.
template <typename T, int BS>
__global__ void k_fix_zero_diag(SellT sp, T* __restrict__ vals) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < sp.nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pd = sp.diag[i];
#pragma unroll
    for (int c = 0; c < BS; ++c)
      if (vals[vidx<BS>(pd, c * BS + c)] == T(0)) vals[vidx<BS>(pd, c * BS + c)] = T(1);
  }
}

// Inverse of every diagonal block (block Jacobi), in the precision of the
// level (the FP32 smoother needs no FP64 arithmetic).
template <typename T, int BS>
__global__ void k_block_diag_inv(SellT sp, const T* __restrict__ vals, T* __restrict__ dinv) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < sp.nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pd = sp.diag[i];
    T* O = dinv + i * BS * BS;
    if (BS == 1) {
      const T d = vals[vidx<BS>(pd, 0)];
      O[0] = d != T(0) ? T(1) / d : T(0);
    } else {
      T D[9];
#pragma unroll
      for (int v = 0; v < 9; ++v) D[v] = vals[vidx<BS>(pd, v)];
      const T a = D[0], b = D[1], c = D[2], d = D[3], e = D[4], f = D[5],
              g = D[6], h = D[7], k = D[8];
      const T A = e * k - f * h, B = -(d * k - f * g), C = d * h - e * g;
      const T det = a * A + b * B + c * C;
      const T s = det != T(0) ? T(1) / det : T(0);
      O[0] = (T)(A * s);
      O[1] = (T)(-(b * k - c * h) * s);
      O[2] = (T)((b * f - c * e) * s);
      O[3] = (T)(B * s);
      O[4] = (T)((a * k - c * g) * s);
      O[5] = (T)(-(a * f - c * d) * s);
      O[6] = (T)(C * s);
      O[7] = (T)(-(a * h - b * g) * s);
      O[8] = (T)((a * e - b * d) * s);
    }
  }
}

// Elements of a thread's grid-stride sequence handled per pass by the
// streaming vector kernels (loads of the pass issued together).
constexpr int kStreamUnroll = 4;

// --------------------------------------------------------------------------
// Chebyshev smoothing step fused into the operator that produced the
// residual r (= the operator kernel's output y, held in registers):
//   kind 1:  dn = c2 Dinv r                         (first step; x untouched)
//   kind 2:  dn = c1 do + c2 Dinv r,  x += dn (+ do when add_old)
// dn and do are distinct buffers (neighbouring rows still read do).
template <typename T>
struct ChebEp {
  const T* dinv = nullptr;
  const T* dold = nullptr;
  T* dnew = nullptr;
  T* x = nullptr;
  T c1 = T(0), c2 = T(0);
  int kind = 0, add_old = 0;
};

// The update of one block row given its inverted diagonal block Dv.  kind 3
// (first step from a zero guess): dn = c2 Dinv r, x = dn.  The old
// direction and x of the row are loaded before anything is stored: the
// buffers are not restrict-qualified, so loads placed after a store would be
// issued one memory round trip at a time.
template <typename T, int BS, int L>
__device__ __forceinline__ void cheb_update(const ChebEp<T>& ep, int64_t row, const T* r,
                                            const T* Dv) {
  const int64_t base = row * BS * L;
  T dold[BS * L], xo[BS * L];
  if (ep.kind == 2) {
#pragma unroll
    for (int q = 0; q < BS * L; ++q) {
      dold[q] = ep.dold[base + q];
      xo[q] = ep.x[base + q];
    }
  }
#pragma unroll
  for (int c = 0; c < BS; ++c)
#pragma unroll
    for (int j = 0; j < L; ++j) {
      T s = T(0);
#pragma unroll
      for (int d = 0; d < BS; ++d) s += Dv[c * BS + d] * r[d * L + j];
      const int q = c * L + j;
      const int64_t idx = base + q;
      if (ep.kind == 1) {
        ep.dnew[idx] = ep.c2 * s;
      } else if (ep.kind == 3) {
        const T dn = ep.c2 * s;
        ep.dnew[idx] = dn;
        ep.x[idx] = dn;
      } else {
        const T dn = ep.c1 * dold[q] + ep.c2 * s;
        ep.dnew[idx] = dn;
        ep.x[idx] = xo[q] + (ep.add_old ? dn + dold[q] : dn);
      }
    }
}

template <typename T, int BS, int L>
__device__ __forceinline__ void cheb_epilogue(const ChebEp<T>& ep, int64_t row, const T* r) {
  const T* D = ep.dinv + row * BS * BS;
  T Dv[BS * BS];
#pragma unroll
  for (int q = 0; q < BS * BS; ++q) Dv[q] = D[q];
  cheb_update<T, BS, L>(ep, row, r, Dv);
}

// --------------------------------------------------------------------------
// SELL-32 BSR SpMV / SpMM: one thread per block row, no cross-lane
// reduction; every plane load of a warp is one coalesced 32-wide access.
// MODE 0: y = A x;  MODE 1: y = b - A x;  MODE 2: y = y - A x.
// DOT: also reduce sum_j (x_row . y_row) per load into dot_out (fused p.Ap).
// ep: optional Chebyshev step on the output (ep.kind 0 = none).
template <typename T, int BS, int L, int MODE, bool DOT>
__global__ void __launch_bounds__(256)
k_sell_spmv(SellT sp, const T* __restrict__ vals, const T* __restrict__ x,
            const T* __restrict__ b, T* __restrict__ y, double* partials, unsigned* counter,
            double* dot_out, ChebEp<T> ep) {
  TOPT_KERNEL_COUNT();
  T tacc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) tacc[j] = T(0);
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       row < ((sp.nrows + 31) & ~(int64_t)31); row += nthreads) {
    const int64_t slice = row >> 5;
    const int lane = (int)(row & 31);
    const int64_t g0 = sp.grp_of_slice[slice], g1 = sp.grp_of_slice[slice + 1];
    T acc[BS * L];
#pragma unroll
    for (int i = 0; i < BS * L; ++i) acc[i] = T(0);
#pragma unroll 3
    for (int64_t g = g0; g < g1; ++g) {
      const int64_t col = sp.col[g * 32 + lane];
      const T* V = vals + g * (BS * BS * 32) + lane;
      T xv[BS * L];
#pragma unroll
      for (int i = 0; i < BS * L; ++i) xv[i] = x[col * BS * L + i];
#pragma unroll
      for (int c = 0; c < BS; ++c)
#pragma unroll
        for (int d = 0; d < BS; ++d) {
          const T a = V[(c * BS + d) * 32];
#pragma unroll
          for (int j = 0; j < L; ++j) acc[c * L + j] += a * xv[d * L + j];
        }
    }
    if (row < sp.nrows) {
#pragma unroll
      for (int i = 0; i < BS * L; ++i) {
        const int64_t idx = row * BS * L + i;
        T out;
        if (MODE == 0) out = acc[i];
        else if (MODE == 1) out = b[idx] - acc[i];
        else out = y[idx] - acc[i];
        y[idx] = out;
        acc[i] = out;
        if (DOT) tacc[i % L] += x[idx] * out;
      }
      if (ep.kind) cheb_epilogue<T, BS, L>(ep, row, acc);
    }
  }
  if (DOT) {
    double dacc[L];
#pragma unroll
    for (int j = 0; j < L; ++j) dacc[j] = (double)tacc[j];
    __shared__ double sh[32 * L];
    block_sum<double, L>(dacc, sh);
    grid_finish<double, L>(dacc, partials, counter, dot_out);
  }
}

// --------------------------------------------------------------------------
// Matrix-free operator of a uniform hex grid (one shared unit matrix K0):
// y_a = sum over the <= 8 cells c around node a of coef_c * K0[la, :] x_c,
// with la the node's local index in c.  One thread per node, K0 in shared
// memory (every lane of a warp reads the same K0 row: broadcast), the x of
// the 27 neighbouring nodes from L1.  Fixed DOFs act as identity rows and
// zero columns (skfem.enforce).  Compute-bound FP32 instead of streaming the
// assembled blocks.  MODE and DOT as k_sell_spmv.
struct MfGrid {
  int nx, ny, nz;  // cells
};

template <typename T, int L, int MODE, bool DOT>
__global__ void __launch_bounds__(256)
k_mf_apply(MfGrid g, const T* __restrict__ K0, const T* __restrict__ coef,
           const uint8_t* __restrict__ mask, const T* __restrict__ x,
           const T* __restrict__ b, T* __restrict__ y, double* partials, unsigned* counter,
           double* dot_out, ChebEp<T> ep) {
  TOPT_KERNEL_COUNT();
  __shared__ T Ks[24 * 24];
  for (int i = threadIdx.x; i < 576; i += blockDim.x) Ks[i] = K0[i];
  __syncthreads();
  const int ny1 = g.ny + 1, nx1 = g.nx + 1;
  const int64_t nn = (int64_t)nx1 * ny1 * (g.nz + 1);
  double dacc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) dacc[j] = 0.0;
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nn;
       a += (int64_t)gridDim.x * blockDim.x) {
    const int ai = (int)a;  // node counts fit 32 bits: cheap index math
    const int iy = ai % ny1;
    const int ix = (ai / ny1) % nx1;
    const int iz = ai / (ny1 * nx1);
    T acc[3 * L];
#pragma unroll
    for (int q = 0; q < 3 * L; ++q) acc[q] = T(0);
#pragma unroll
    for (int la = 0; la < 8; ++la) {
      // cell whose local node la is this node
      const int cx = ix - c_hex_off[la][0], cy = iy - c_hex_off[la][1],
                cz = iz - c_hex_off[la][2];
      if (cx < 0 || cy < 0 || cz < 0 || cx >= g.nx || cy >= g.ny || cz >= g.nz) continue;
      const T s = coef[cy + (int64_t)g.ny * (cx + (int64_t)g.nx * cz)];
      T part[3 * L];
#pragma unroll
      for (int q = 0; q < 3 * L; ++q) part[q] = T(0);
#pragma unroll
      for (int lb = 0; lb < 8; ++lb) {
        const int64_t nb = (cy + c_hex_off[lb][1]) +
                           (int64_t)ny1 * ((cx + c_hex_off[lb][0]) +
                                           (int64_t)nx1 * (cz + c_hex_off[lb][2]));
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const bool fixed = mask && mask[nb * 3 + d];
#pragma unroll
          for (int j = 0; j < L; ++j) {
            const T xv = fixed ? T(0) : x[(nb * 3 + d) * L + j];
#pragma unroll
            for (int c = 0; c < 3; ++c)
              part[c * L + j] += Ks[(3 * la + c) * 24 + 3 * lb + d] * xv;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 3 * L; ++q) acc[q] += s * part[q];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const bool fixed = mask && mask[a * 3 + c];
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const int64_t idx = (a * 3 + c) * L + j;
        const T ax = fixed ? x[idx] : acc[c * L + j];
        T out;
        if (MODE == 0) out = ax;
        else if (MODE == 1) out = b[idx] - ax;
        else out = y[idx] - ax;
        y[idx] = out;
        acc[c * L + j] = out;
        if (DOT) dacc[j] += (double)x[idx] * (double)out;
      }
    }
    if (ep.kind) cheb_epilogue<T, 3, L>(ep, a, acc);
  }
  if (DOT) {
    __shared__ double sh[32 * L];
    block_sum<double, L>(dacc, sh);
    grid_finish<double, L>(dacc, partials, counter, dot_out);
  }
}

// Single-load operator: the unit matrix is passed by value as a kernel
// parameter (2,304 B, parameter space of the launch, so concurrent handles
// with different matrices never share it) and every loop index is a
// compile-time constant, so each of the 576 FMAs per node reads its K0
// operand straight from the constant bank.  nmask packs the fixed flags of a
// node's three DOFs in bits 0-2; hoff(a, d) is the offset of local node a
// along axis d (MeshHex order).
struct K0f {
  float v[576];
  __host__ __device__ float operator[](int i) const { return v[i]; }
};

__host__ __device__ constexpr int hoff(int a, int d) {
  return d == 0 ? (0xD4 >> a) & 1 : (d == 1 ? (0xB2 >> a) & 1 : (0xE8 >> a) & 1);
}

// Tiled variant: the grid is persistent (two CTAs of 256 threads per SM) and
// walks tiles of TY x 8 x 4 nodes (y fastest; TY picked per grid to waste the
// fewest threads); each thread computes TY/8 nodes of a tile.  A CTA stages
// the next tile with cp.async while it computes the current one (two
// buffers): the node halo (x in .xyz, the node's fixed flags in .w; zeros
// outside the grid), the coefficients of every cell touching the tile (0
// outside the grid) and, for MODE 1/2, the tile's b or y.  The per-node work
// is branch-free: per cell, 8 LDS.128 of its nodes and 72 FFMA with
// constant-bank K0 operands.  COLMASK zeroes the fixed DOFs of x on use
// (skfem.enforce's zero columns); callers whose x is zero on the fixed DOFs
// already -- every operand inside the solvers -- skip it.  Fixed rows are
// identity rows.  (A Chebyshev step fused here measured slower than a
// separate pass: its loads stall this compute-bound kernel.)
__device__ __forceinline__ void cp_async4(void* smem, const void* g, bool in) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(g),
               "r"(in ? 4 : 0));
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::);
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

constexpr int kMfTX = 8, kMfTZ = 4, kMfThreads = 256, kMfCtasPerSm = 2;

template <int TY>
struct MfTile {
  static constexpr int HY = TY + 2, HX = kMfTX + 2, HZ = kMfTZ + 2;
  static constexpr int CY = TY + 1, CX = kMfTX + 1, CZ = kMfTZ + 1;
  static constexpr int NN = TY * kMfTX * kMfTZ;
  static constexpr int NPT = (NN + kMfThreads - 1) / kMfThreads;
  static constexpr int XSF = HZ * HX * HY * 4;        // floats of one buffer's parts
  static constexpr int CSF = (CZ * CX * CY + 3) & ~3;
  static constexpr int SBF = (NN * 3 + 3) & ~3;
  static constexpr int BUF = XSF + CSF + SBF;
  static constexpr int SMEM = 2 * BUF * 4;            // bytes, two buffers
};

inline int mf_pick_ty(int ny1) {
  int best = 32;
  int64_t waste = -1;
  for (int ty : {32, 27, 16}) {
    const int64_t w = (int64_t)((ny1 + ty - 1) / ty) * ty - ny1;
    if (waste < 0 || w < waste) { waste = w; best = ty; }
  }
  return best;
}

template <int TY, int MODE>
__device__ __forceinline__ void mf_stage(float* buf, int t, const MfGrid& g, int ny1, int nx1,
                                         int nz1, int nty, int ntx, const float* __restrict__ x,
                                         const uint32_t* __restrict__ m32,
                                         const float* __restrict__ coef,
                                         const float* __restrict__ bsrc) {
  using G = MfTile<TY>;
  const int ty = (t % nty) * TY, tx = ((t / nty) % ntx) * kMfTX, tz = (t / (nty * ntx)) * kMfTZ;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* xs = buf;
  float* cs = buf + G::XSF;
  float* sb = cs + G::CSF;
  for (int row = warp; row < G::HZ * G::HX; row += kMfThreads / 32) {
    const int hz = row / G::HX, hx = row % G::HX;
    const int jz = tz - 1 + hz, jx = tx - 1 + hx;
    const bool rin = jz >= 0 && jz < nz1 && jx >= 0 && jx < nx1;
    const int base = ny1 * (jx + nx1 * jz);
    for (int hy = lane; hy < G::HY; hy += 32) {
      const int jy = ty - 1 + hy;
      const bool in = rin && jy >= 0 && jy < ny1;
      const int nb = in ? base + jy : 0;
      float* d = xs + ((hz * G::HX + hx) * G::HY + hy) * 4;
      cp_async4(d + 0, x + nb * 3 + 0, in);
      cp_async4(d + 1, x + nb * 3 + 1, in);
      cp_async4(d + 2, x + nb * 3 + 2, in);
      cp_async4(d + 3, m32 + nb, in);
    }
  }
  for (int row = warp; row < G::CZ * G::CX; row += kMfThreads / 32) {
    const int cz = row / G::CX, cx = row % G::CX;
    const int ez = tz - 1 + cz, ex = tx - 1 + cx;
    const bool rin = ez >= 0 && ez < g.nz && ex >= 0 && ex < g.nx;
    const int base = g.ny * (ex + g.nx * ez);
    for (int cy = lane; cy < G::CY; cy += 32) {
      const int ey = ty - 1 + cy;
      const bool in = rin && ey >= 0 && ey < g.ny;
      cp_async4(cs + (cz * G::CX + cx) * G::CY + cy, coef + (in ? base + ey : 0), in);
    }
  }
  if (MODE != 0) {
    for (int row = warp; row < kMfTZ * kMfTX; row += kMfThreads / 32) {
      const int lz = row / kMfTX, lx = row % kMfTX;
      const int iz = tz + lz, ix = tx + lx;
      const bool rin = iz < nz1 && ix < nx1;
      const int n = min(TY, ny1 - ty) * 3;
      const int64_t a0 = (int64_t)ty + (int64_t)ny1 * (ix + (int64_t)nx1 * iz);
      for (int i = lane; i < TY * 3; i += 32) {
        const bool in = rin && i < n;
        cp_async4(sb + row * TY * 3 + i, bsrc + (in ? a0 * 3 + i : 0), in);
      }
    }
  }
}

template <int TY, int MODE, bool DOT, bool COLMASK>
__global__ void __launch_bounds__(kMfThreads, kMfCtasPerSm)
k_mf_tile(MfGrid g, const K0f k0, const float* __restrict__ coef,
          const uint32_t* __restrict__ m32, const float* __restrict__ x,
          const float* __restrict__ b, float* __restrict__ y, double* partials,
          unsigned* counter, double* dot_out) {
  TOPT_KERNEL_COUNT();
  using G = MfTile<TY>;
  constexpr int TX = kMfTX, TZ = kMfTZ, NT = kMfThreads, HY = G::HY, HX = G::HX;
  constexpr int CY = G::CY, CX = G::CX;
  extern __shared__ __align__(16) float smem[];
  const int ny1 = g.ny + 1, nx1 = g.nx + 1, nz1 = g.nz + 1;
  const int nty = (ny1 + TY - 1) / TY, ntx = (nx1 + TX - 1) / TX;
  const int ntiles = nty * ntx * ((nz1 + TZ - 1) / TZ);
  const float* bsrc = MODE == 1 ? b : y;
  float tacc = 0.0f;
  int cur = 0;
  if ((int)blockIdx.x < ntiles)
    mf_stage<TY, MODE>(smem, blockIdx.x, g, ny1, nx1, nz1, nty, ntx, x, m32, coef, bsrc);
  cp_async_commit();
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int tn = t + gridDim.x;
    if (tn < ntiles)
      mf_stage<TY, MODE>(smem + (cur ^ 1) * G::BUF, tn, g, ny1, nx1, nz1, nty, ntx, x, m32,
                         coef, bsrc);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const float4* xs = reinterpret_cast<const float4*>(smem + cur * G::BUF);
    const float* cs = smem + cur * G::BUF + G::XSF;
    const float* sb = cs + G::CSF;
    const int ty = (t % nty) * TY, tx = ((t / nty) % ntx) * TX, tz = (t / (nty * ntx)) * TZ;
#pragma unroll 1
    for (int k = 0; k < G::NPT; ++k) {
      const int li = threadIdx.x + k * NT;
      if (li >= G::NN) break;
      const int ly = li % TY, lx = (li / TY) % TX, lz = li / (TY * TX);
      const int iy = ty + ly, ix = tx + lx, iz = tz + lz;
      if (iy >= ny1 || ix >= nx1 || iz >= nz1) continue;
      float acc[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int la = 0; la < 8; ++la) {
        float part[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int lb = 0; lb < 8; ++lb) {
          const float4 v = xs[((lz + 1 - hoff(la, 2) + hoff(lb, 2)) * HX +
                               (lx + 1 - hoff(la, 0) + hoff(lb, 0))) * HY +
                              (ly + 1 - hoff(la, 1) + hoff(lb, 1))];
          float xv[3] = {v.x, v.y, v.z};
          if (COLMASK) {
            const int m = __float_as_int(v.w);
            xv[0] = (m & 1) ? 0.f : xv[0];
            xv[1] = (m & 2) ? 0.f : xv[1];
            xv[2] = (m & 4) ? 0.f : xv[2];
          }
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d)
              part[c] = fmaf(k0.v[(3 * la + c) * 24 + 3 * lb + d], xv[d], part[c]);
        }
        const float s = cs[((lz + 1 - hoff(la, 2)) * CX + (lx + 1 - hoff(la, 0))) * CY +
                           (ly + 1 - hoff(la, 1))];
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[c] = fmaf(s, part[c], acc[c]);
      }
      const float4 self = xs[((lz + 1) * HX + (lx + 1)) * HY + (ly + 1)];
      const int ma = __float_as_int(self.w);
      const int a = iy + ny1 * (ix + nx1 * iz);
      const float xself[3] = {self.x, self.y, self.z};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float ax = ((ma >> c) & 1) ? xself[c] : acc[c];
        const float out = MODE == 0 ? ax : sb[li * 3 + c] - ax;
        y[(int64_t)a * 3 + c] = out;
        if (DOT) tacc += xself[c] * out;
      }
    }
    __syncthreads();
    cur ^= 1;
  }
  cp_async_wait<0>();
  if (DOT) {
    double dacc[1] = {(double)tacc};
    __shared__ double sh[32];
    block_sum<double, 1>(dacc, sh);
    grid_finish<double, 1>(dacc, partials, counter, dot_out);
  }
}

// Inverted 3x3 diagonal block of node (ix, iy, iz) of the matrix-free
// operator (block Jacobi): D = sum_c coef_c K0[la, la] over the <= 8 cells
// around the node, fixed DOFs (bits of m) as identity rows / columns; FP32.
// K0 is the by-value parameter (K0f) or a pointer to memory.
template <class KS>
__device__ __forceinline__ void mf_node_dinv(const MfGrid& g, const KS& K0,
                                             const float* __restrict__ coef, int m, int ix,
                                             int iy, int iz, float* O) {
  float D[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int la = 0; la < 8; ++la) {
    const int cx = ix - hoff(la, 0), cy = iy - hoff(la, 1), cz = iz - hoff(la, 2);
    if (cx < 0 || cy < 0 || cz < 0 || cx >= g.nx || cy >= g.ny || cz >= g.nz) continue;
    const float s = coef[cy + (int64_t)g.ny * (cx + (int64_t)g.nx * cz)];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int k = (3 * la + c) * 24 + 3 * la + d;
        D[c * 3 + d] += s * K0[k];
      }
  }
  if (m) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (((m >> c) & 1) || ((m >> d) & 1)) D[c * 3 + d] = (c == d) ? 1.0f : 0.0f;
  }
  const float A = D[4] * D[8] - D[5] * D[7], B = -(D[3] * D[8] - D[5] * D[6]),
              C = D[3] * D[7] - D[4] * D[6];
  const float det = D[0] * A + D[1] * B + D[2] * C;
  const float si = det != 0.0f ? 1.0f / det : 0.0f;
  O[0] = A * si;
  O[1] = -(D[1] * D[8] - D[2] * D[7]) * si;
  O[2] = (D[1] * D[5] - D[2] * D[4]) * si;
  O[3] = B * si;
  O[4] = (D[0] * D[8] - D[2] * D[6]) * si;
  O[5] = -(D[0] * D[5] - D[2] * D[3]) * si;
  O[6] = C * si;
  O[7] = -(D[0] * D[7] - D[1] * D[6]) * si;
  O[8] = (D[0] * D[4] - D[1] * D[3]) * si;
}

// All blocks (stored for the power iteration and the generic smoother).
static __global__ void k_mf_diag_inv(MfGrid g, const float* __restrict__ K0,
                              const float* __restrict__ coef, const uint8_t* __restrict__ mask,
                              float* __restrict__ dinv) {
  TOPT_KERNEL_COUNT();
  const int ny1 = g.ny + 1, nx1 = g.nx + 1;
  const int64_t nn = (int64_t)nx1 * ny1 * (g.nz + 1);
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nn;
       a += (int64_t)gridDim.x * blockDim.x) {
    const int ai = (int)a;  // node counts fit 32 bits: cheap index math
    const int iy = ai % ny1, ix = (ai / ny1) % nx1, iz = ai / (ny1 * nx1);
    const int m = mask ? (mask[a * 3] | (mask[a * 3 + 1] << 1) | (mask[a * 3 + 2] << 2)) : 0;
    mf_node_dinv(g, K0, coef, m, ix, iy, iz, dinv + a * 9);
  }
}

// Chebyshev step of the matrix-free fine level as a separate pass (ChebEp
// kinds 1-3 on r), with the inverted diagonal blocks read from the level's
// stored copy (ep.dinv, written by k_mf_diag_inv at every refresh).
// Recomputing them per node from the cell coefficients instead measured
// issue-bound on GB300 (about 470 instructions per node, 58-75 % issue
// activity, 20.7 / 27.1 us on 1.05M nodes); reading them costs 36 B per
// node.  Same blocks, same update: the same bits either way.
static __global__ void k_cheb_stored(int64_t n, ChebEp<float> ep, const float* __restrict__ r) {
  TOPT_KERNEL_COUNT();
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n;
       a += (int64_t)gridDim.x * blockDim.x) {
    const float rv[3] = {r[a * 3], r[a * 3 + 1], r[a * 3 + 2]};
    cheb_epilogue<float, 3, 1>(ep, a, rv);
  }
}

// Same product for small (coarse) levels, where one thread walking a row's
// ~27 blocks is latency-bound: one warp per row, one lane per block, then a
// warp reduction (fixed order, deterministic).
template <typename T, int BS, int L, int MODE, bool DOT>
__global__ void __launch_bounds__(256)
k_sell_spmv_warp(SellT sp, const T* __restrict__ vals, const T* __restrict__ x,
                 const T* __restrict__ b, T* __restrict__ y, double* partials,
                 unsigned* counter, double* dot_out, ChebEp<T> ep) {
  TOPT_KERNEL_COUNT();
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double dacc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) dacc[j] = 0.0;
  for (int64_t row = w0; row < sp.nrows; row += nw) {
    const int64_t slice = row >> 5;
    const int r = (int)(row & 31);
    const int64_t g0 = sp.grp_of_slice[slice];
    const int len = sp.rowlen[row];
    T acc[BS * L];
#pragma unroll
    for (int q = 0; q < BS * L; ++q) acc[q] = T(0);
    for (int j = lane; j < len; j += 32) {
      const int64_t g = g0 + j;
      const int64_t col = sp.col[g * 32 + r];
      const T* V = vals + g * (BS * BS * 32) + r;
#pragma unroll
      for (int c = 0; c < BS; ++c)
#pragma unroll
        for (int d = 0; d < BS; ++d) {
          const T a = V[(c * BS + d) * 32];
#pragma unroll
          for (int jj = 0; jj < L; ++jj) acc[c * L + jj] += a * x[(col * BS + d) * L + jj];
        }
    }
#pragma unroll
    for (int q = 0; q < BS * L; ++q) acc[q] = warp_sum(acc[q]);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < BS * L; ++q) {
        const int64_t idx = row * BS * L + q;
        T out;
        if (MODE == 0) out = acc[q];
        else if (MODE == 1) out = b[idx] - acc[q];
        else out = y[idx] - acc[q];
        y[idx] = out;
        acc[q] = out;
        if (DOT) dacc[q % L] += (double)x[idx] * (double)out;
      }
      if (ep.kind) cheb_epilogue<T, BS, L>(ep, row, acc);
    }
  }
  if (DOT) {
    __shared__ double sh[32 * L];
    block_sum<double, L>(dacc, sh);
    grid_finish<double, L>(dacc, partials, counter, dot_out);
  }
}

// Mid-size levels (3x3 blocks): three threads per block row, one per output
// component, so a level of a few ten thousand rows still fills the GPU.  A
// CTA of 192 threads covers two slices; warp (slice, c) reads plane row c of
// every block with 32-wide coalesced loads.  The Chebyshev epilogue needs the
// three residual components of a row: they meet in shared memory.
template <typename T, int L, int MODE, bool DOT>
__global__ void __launch_bounds__(192)
k_sell_spmv3(SellT sp, const T* __restrict__ vals, const T* __restrict__ x,
             const T* __restrict__ b, T* __restrict__ y, double* partials, unsigned* counter,
             double* dot_out, ChebEp<T> ep) {
  TOPT_KERNEL_COUNT();
  __shared__ T rs[2][3][32 * L];
  const int sl = threadIdx.x / 96, c = (threadIdx.x % 96) >> 5, lane = threadIdx.x & 31;
  const int64_t nsl = (sp.nrows + 31) >> 5;
  T tacc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) tacc[j] = T(0);
  for (int64_t s0 = 2 * (int64_t)blockIdx.x; s0 < nsl; s0 += 2 * (int64_t)gridDim.x) {
    const int64_t slice = s0 + sl;
    const int64_t row = slice * 32 + lane;
    const bool valid = slice < nsl && row < sp.nrows;
    T acc[L];
#pragma unroll
    for (int j = 0; j < L; ++j) acc[j] = T(0);
    if (slice < nsl) {
      const int64_t g0 = sp.grp_of_slice[slice], g1 = sp.grp_of_slice[slice + 1];
#pragma unroll 3
      for (int64_t g = g0; g < g1; ++g) {
        const int64_t col = sp.col[g * 32 + lane];
        const T* V = vals + g * (9 * 32) + lane;
        const T a0 = V[(c * 3 + 0) * 32], a1 = V[(c * 3 + 1) * 32], a2 = V[(c * 3 + 2) * 32];
#pragma unroll
        for (int j = 0; j < L; ++j)
          acc[j] += a0 * x[(col * 3 + 0) * L + j] + a1 * x[(col * 3 + 1) * L + j] +
                    a2 * x[(col * 3 + 2) * L + j];
      }
    }
    T out[L];
#pragma unroll
    for (int j = 0; j < L; ++j) out[j] = T(0);
    if (valid) {
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const int64_t idx = (row * 3 + c) * L + j;
        if (MODE == 0) out[j] = acc[j];
        else if (MODE == 1) out[j] = b[idx] - acc[j];
        else out[j] = y[idx] - acc[j];
        y[idx] = out[j];
        if (DOT) tacc[j] += x[idx] * out[j];
      }
    }
    if (ep.kind) {   // uniform over the grid: the barriers below are safe
#pragma unroll
      for (int j = 0; j < L; ++j) rs[sl][c][lane * L + j] = out[j];
      __syncthreads();
      if (valid) {
        const T* D = ep.dinv + row * 9 + c * 3;
        const T D0 = D[0], D1 = D[1], D2 = D[2];
#pragma unroll
        for (int j = 0; j < L; ++j) {
          T s = T(0);
          s += D0 * rs[sl][0][lane * L + j];
          s += D1 * rs[sl][1][lane * L + j];
          s += D2 * rs[sl][2][lane * L + j];
          const int64_t idx = (row * 3 + c) * L + j;
          if (ep.kind == 1) {
            ep.dnew[idx] = ep.c2 * s;
          } else {
            const T dold = ep.dold[idx];
            const T dn = ep.c1 * dold + ep.c2 * s;
            ep.dnew[idx] = dn;
            ep.x[idx] += ep.add_old ? dn + dold : dn;
          }
        }
      }
      __syncthreads();
    }
  }
  if (DOT) {
    double dacc[L];
#pragma unroll
    for (int j = 0; j < L; ++j) dacc[j] = (double)tacc[j];
    __shared__ double sh[32 * L];
    block_sum<double, L>(dacc, sh);
    grid_finish<double, L>(dacc, partials, counter, dot_out);
  }
}

// CSR-order copy of the SELL values (the CSR stays the interface object).
template <int BS>
__global__ void k_sell_to_csr(int64_t nnzb, const int32_t* __restrict__ csr2sell,
                              const double* __restrict__ vals, double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnzb;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = csr2sell[k];
#pragma unroll
    for (int v = 0; v < BS * BS; ++v) out[k * BS * BS + v] = vals[vidx<BS>(p, v)];
  }
}

// --------------------------------------------------------------------------
// Vector kernels (n = number of DOFs; vectors n x L).

// z = Dinv r  and, optionally, partial sums of r.z per load.
template <typename T, int BS, int L, bool DOT>
__global__ void k_block_jacobi(int64_t n_nodes, const T* __restrict__ dinv,
                               const T* __restrict__ r, T* __restrict__ z,
                               double* partials, unsigned* counter, double* dot_out) {
  TOPT_KERNEL_COUNT();
  T tacc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) tacc[j] = T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T* D = dinv + i * BS * BS;
    T rv[BS * L];
#pragma unroll
    for (int q = 0; q < BS * L; ++q) rv[q] = r[i * BS * L + q];
#pragma unroll
    for (int c = 0; c < BS; ++c)
#pragma unroll
      for (int j = 0; j < L; ++j) {
        T s = T(0);
#pragma unroll
        for (int d = 0; d < BS; ++d) s += D[c * BS + d] * rv[d * L + j];
        z[i * BS * L + c * L + j] = s;
        if (DOT) tacc[j] += s * rv[c * L + j];
      }
  }
  if (DOT) {
    double dacc[L];
#pragma unroll
    for (int j = 0; j < L; ++j) dacc[j] = (double)tacc[j];
    __shared__ double sh[32 * L];
    block_sum<double, L>(dacc, sh);
    grid_finish<double, L>(dacc, partials, counter, dot_out);
  }
}

// Deterministic dot products per load: out[j] = sum_i x[i,j] y[i,j].
template <typename T, int L>
__global__ void k_dot(int64_t n, const T* __restrict__ x, const T* __restrict__ y,
                      double* partials, unsigned* counter, double* out) {
  TOPT_KERNEL_COUNT();
  // per-thread sums in T (FP64 arithmetic is scarce on this part), then FP64
  T tacc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) tacc[j] = T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int j = 0; j < L; ++j) tacc[j] += x[i * L + j] * y[i * L + j];
  }
  double acc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) acc[j] = (double)tacc[j];
  __shared__ double sh[32 * L];
  block_sum<double, L>(acc, sh);
  grid_finish<double, L>(acc, partials, counter, out);
}

// PCG update: alpha_j = rz_j / pq_j (0 when frozen or pq <= 0);
// x += alpha p; r -= alpha q; partial sums of r.r; r32 (optional) = float(r).
template <typename T, typename TQ, int L>
__global__ void k_pcg_update(int64_t n, const double* __restrict__ rz,
                             const double* __restrict__ pq, const int* __restrict__ active,
                             const T* __restrict__ p, const TQ* __restrict__ q,
                             T* __restrict__ x, T* __restrict__ r, double* partials,
                             unsigned* counter, double* rr_out, float* __restrict__ r32) {
  TOPT_KERNEL_COUNT();
  T alpha[L];
#pragma unroll
  for (int j = 0; j < L; ++j) {
    const double d = pq[j];
    alpha[j] = (active[j] && d > 0.0) ? (T)(rz[j] / d) : T(0);
  }
  double acc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) acc[j] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const int64_t q_ = i * L + j;
      x[q_] += alpha[j] * p[q_];
      const T rv = r[q_] - alpha[j] * (T)q[q_];
      r[q_] = rv;
      if (r32) r32[q_] = (float)rv;
      acc[j] += (double)rv * (double)rv;
    }
  }
  __shared__ double sh[32 * L];
  block_sum<double, L>(acc, sh);
  grid_finish<double, L>(acc, partials, counter, rr_out);
}

// Flexible CG update with FP32 recurrences and an FP64 solution:
// alpha_j = rz_j / pq_j (0 when frozen or pq <= 0); U += alpha p (FP64);
// r -= alpha q (FP32); partial sums of r.r.
template <int L>
__global__ void k_fcg_update32(int64_t n, const double* __restrict__ rz,
                               const double* __restrict__ pq, const int* __restrict__ active,
                               const float* __restrict__ p, const float* __restrict__ q,
                               double* __restrict__ U, float* __restrict__ r, double* partials,
                               unsigned* counter, double* rr_out) {
  TOPT_KERNEL_COUNT();
  double alpha[L];
  float alpha32[L];
#pragma unroll
  for (int j = 0; j < L; ++j) {
    const double d = pq[j];
    alpha[j] = (active[j] && d > 0.0) ? rz[j] / d : 0.0;
    alpha32[j] = (float)alpha[j];
  }
  float tacc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) tacc[j] = 0.0f;
  const int64_t S = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // kStreamUnroll elements of the thread's sequence per pass, all loads
  // first (memory-level parallelism); the sums keep the sequence's order
  for (; i + (kStreamUnroll - 1) * S < n; i += kStreamUnroll * S) {
    double uv[kStreamUnroll][L];
    float pv[kStreamUnroll][L], qv[kStreamUnroll][L], rv[kStreamUnroll][L];
#pragma unroll
    for (int u = 0; u < kStreamUnroll; ++u)
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const int64_t q_ = (i + u * S) * L + j;
        uv[u][j] = U[q_];
        pv[u][j] = p[q_];
        qv[u][j] = q[q_];
        rv[u][j] = r[q_];
      }
#pragma unroll
    for (int u = 0; u < kStreamUnroll; ++u)
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const int64_t q_ = (i + u * S) * L + j;
        U[q_] = uv[u][j] + alpha[j] * (double)pv[u][j];
        const float rn = rv[u][j] - alpha32[j] * qv[u][j];
        r[q_] = rn;
        tacc[j] += rn * rn;
      }
  }
  for (; i < n; i += S) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const int64_t q_ = i * L + j;
      U[q_] += alpha[j] * (double)p[q_];
      const float rv1 = r[q_] - alpha32[j] * q[q_];
      r[q_] = rv1;
      tacc[j] += rv1 * rv1;
    }
  }
  double acc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) acc[j] = (double)tacc[j];
  __shared__ double sh[32 * L];
  block_sum<double, L>(acc, sh);
  grid_finish<double, L>(acc, partials, counter, rr_out);
}

// Two dots sharing z: out[0..L) = r.z, out[L..2L) = q.z (flexible CG).
template <typename T, typename TQ, typename TZ, int L>
__global__ void k_dot2(int64_t n, const T* __restrict__ r, const TQ* __restrict__ q,
                       const TZ* __restrict__ z, double* partials, unsigned* counter,
                       double* out) {
  TOPT_KERNEL_COUNT();
  // per-thread sums in T (FP32 inputs need no FP64 arithmetic), then FP64
  T tacc[2 * L];
#pragma unroll
  for (int j = 0; j < 2 * L; ++j) tacc[j] = T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const T zv = (T)z[i * L + j];
      tacc[j] += (T)r[i * L + j] * zv;
      tacc[L + j] += (T)q[i * L + j] * zv;
    }
  }
  double acc[2 * L];
#pragma unroll
  for (int j = 0; j < 2 * L; ++j) acc[j] = (double)tacc[j];
  __shared__ double sh[32 * 2 * L];
  block_sum<double, 2 * L>(acc, sh);
  grid_finish<double, 2 * L>(acc, partials, counter, out);
}

// Flexible (Polak-Ribiere) direction: beta_j = -alpha_j (q.z_new)_j / rz_old_j
// with alpha_j = rz_old_j / pq_j, i.e. beta = -(q.z_new) / pq; p = z + beta p.
template <typename T, typename TZ, int L>
__global__ void k_fcg_direction(int64_t n, const double* __restrict__ qz,
                                const double* __restrict__ pq, const int* __restrict__ active,
                                const TZ* __restrict__ z, T* __restrict__ p,
                                float* __restrict__ p32) {
  TOPT_KERNEL_COUNT();
  T beta[L];
#pragma unroll
  for (int j = 0; j < L; ++j)
    beta[j] = (active[j] && pq[j] > 0.0) ? (T)(-qz[j] / pq[j]) : T(0);
  const int64_t S = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + (kStreamUnroll - 1) * S < n; i += kStreamUnroll * S) {
    T zv[kStreamUnroll][L], pv[kStreamUnroll][L];
#pragma unroll
    for (int u = 0; u < kStreamUnroll; ++u)
#pragma unroll
      for (int j = 0; j < L; ++j) {
        zv[u][j] = (T)z[(i + u * S) * L + j];
        pv[u][j] = p[(i + u * S) * L + j];
      }
#pragma unroll
    for (int u = 0; u < kStreamUnroll; ++u)
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const int64_t q_ = (i + u * S) * L + j;
        const T v = zv[u][j] + beta[j] * pv[u][j];
        p[q_] = v;
        if (p32) p32[q_] = (float)v;
      }
  }
  for (; i < n; i += S) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const T v = (T)z[i * L + j] + beta[j] * p[i * L + j];
      p[i * L + j] = v;
      if (p32) p32[i * L + j] = (float)v;
    }
  }
}

// p = z + beta p with beta_j = rz_new_j / rz_old_j (p = z on the first step).
template <typename T, typename TZ, int L>
__global__ void k_pcg_direction(int64_t n, const double* __restrict__ rz_new,
                                const double* __restrict__ rz_old, int first,
                                const TZ* __restrict__ z, T* __restrict__ p,
                                float* __restrict__ p32) {
  TOPT_KERNEL_COUNT();
  T beta[L];
#pragma unroll
  for (int j = 0; j < L; ++j)
    beta[j] = (first || rz_old[j] == 0.0) ? T(0) : (T)(rz_new[j] / rz_old[j]);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int j = 0; j < L; ++j) {   // p = z exactly on the first step (p may hold garbage)
      const T v = first ? (T)z[i * L + j] : (T)z[i * L + j] + beta[j] * p[i * L + j];
      p[i * L + j] = v;
      if (p32) p32[i * L + j] = (float)v;
    }
  }
}

// Chebyshev smoothing steps (Saad, Iterative Methods, Alg. 12.1):
// first: d = c2 Dinv r; x = d (x_zero) or x += d.
// next:  d = c1 d + c2 Dinv r; x += d.
template <typename T, int BS, int L>
__global__ void k_cheb(int64_t n_nodes, const T* __restrict__ dinv,
                       const T* __restrict__ r, T* __restrict__ d, T* __restrict__ x,
                       T c1, T c2, int first, int x_zero) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T* D = dinv + i * BS * BS;
    T rv[BS * L];
#pragma unroll
    for (int q = 0; q < BS * L; ++q) rv[q] = r[i * BS * L + q];
#pragma unroll
    for (int c = 0; c < BS; ++c)
#pragma unroll
      for (int j = 0; j < L; ++j) {
        T s = T(0);
#pragma unroll
        for (int dd = 0; dd < BS; ++dd) s += D[c * BS + dd] * rv[dd * L + j];
        const int64_t q_ = i * BS * L + c * L + j;
        const T dv = first ? c2 * s : c1 * d[q_] + c2 * s;
        d[q_] = dv;
        x[q_] = (first && x_zero) ? dv : x[q_] + dv;
      }
  }
}

// Elementwise helpers.
template <typename TO, typename TI>
__global__ void k_convert(int64_t n, const TI* __restrict__ a, TO* __restrict__ b) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (TO)a[i];
}
template <typename T>
__global__ void k_fill(int64_t n, T v, T* __restrict__ a) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = v;
}
// y += a x
template <typename T>
__global__ void k_axpy(int64_t n, T a, const T* __restrict__ x, T* __restrict__ y) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
// y = a x
template <typename T>
__global__ void k_scale(int64_t n, T a, const T* __restrict__ x, T* __restrict__ y) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}
// U += double(d)
static __global__ void k_add_f32_to_f64(int64_t n, const float* __restrict__ d,
                                 double* __restrict__ u) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    u[i] += (double)d[i];
}
// U[fixed DOFs] = 0 (an initial guess of the enforced system).
static __global__ void k_zero_fixed(int64_t n_dof, int L, const uint8_t* __restrict__ mask,
                             double* __restrict__ u) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof * L;
       i += (int64_t)gridDim.x * blockDim.x)
    if (mask[i / L]) u[i] = 0.0;
}
// F_e: copy of F with fixed DOFs zeroed (enforce's RHS with x = 0).
static __global__ void k_enforce_rhs(int64_t n_dof, int L, const uint8_t* __restrict__ mask,
                              const double* __restrict__ f, double* __restrict__ fe) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_dof * L;
       i += (int64_t)gridDim.x * blockDim.x)
    fe[i] = mask[i / L] ? 0.0 : f[i];
}
// Deterministic pseudo-random start vector for the power iteration.
template <typename T>
__global__ void k_hash_fill(int64_t n, T* __restrict__ a) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t h = (uint64_t)i * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    a[i] = (T)(0.5 + (double)(h >> 11) * (1.0 / 9007199254740992.0));
  }
}

// --------------------------------------------------------------------------
// Structured-grid transfers.  Level grids number nodes iy + (ny+1)(ix +
// (nx+1) iz).  Per axis, cm[i] is the fine node index of coarse node i,
// c0[f] the coarse interval holding fine node f and w1[f] the weight of its
// right end.  mask (fine DOFs, level 0 only) removes fixed DOFs from P.
struct GridT {
  int nfx, nfy, nfz;  // fine cells
  int ncx, ncy, ncz;  // coarse cells
  const int32_t *cmx, *cmy, *cmz;
  const int32_t *c0x, *c0y, *c0z;
  const float *w1x, *w1y, *w1z;   // 0, 1/2 or 1: exact in FP32
  // restriction: per coarse index, first fine index and 3 weights
  const int32_t *r0x, *r0y, *r0z;
  const float *rwx, *rwy, *rwz;
};

// bc = P^T r  (coarse node gathers its <= 3x3x3 fine support, fixed order).
// With dinv_c set, also the first Chebyshev step of the coarse level from a
// zero guess: d_c = x_c = c2 Dinv_c bc.
template <typename T, int BS, int L>
__global__ void k_restrict(GridT g, const uint8_t* __restrict__ mask,
                           const T* __restrict__ rf, T* __restrict__ bc,
                           const T* __restrict__ dinv_c, T* __restrict__ d_c,
                           T* __restrict__ x_c, T c2) {
  TOPT_KERNEL_COUNT();
  const int nnx = g.ncx + 1, nny = g.ncy + 1;
  const int nc = nnx * nny * (g.ncz + 1);
  const int fnx = g.nfx + 1, fny = g.nfy + 1;
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nc; I += gridDim.x * blockDim.x) {
    const int iy = I % nny;
    const int ix = (I / nny) % nnx;
    const int iz = I / (nny * nnx);
    const int fx0 = g.r0x[ix], fy0 = g.r0y[iy], fz0 = g.r0z[iz];
    T acc[BS * L];
#pragma unroll
    for (int q = 0; q < BS * L; ++q) acc[q] = T(0);
#pragma unroll
    for (int kz = 0; kz < 3; ++kz) {
      const float wz = g.rwz[iz * 3 + kz];
      if (wz == 0.0f) continue;
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const float wx = g.rwx[ix * 3 + kx] * wz;
        if (wx == 0.0f) continue;
#pragma unroll
        for (int ky = 0; ky < 3; ++ky) {
          const float wy = g.rwy[iy * 3 + ky];
          if (wy == 0.0f) continue;
          const T w = (T)(wy * wx);
          const int64_t fn = (fy0 + ky) + (int64_t)fny * ((fx0 + kx) + (int64_t)fnx * (fz0 + kz));
#pragma unroll
          for (int c = 0; c < BS; ++c) {
            if (mask && mask[fn * BS + c]) continue;
#pragma unroll
            for (int j = 0; j < L; ++j) acc[c * L + j] += w * rf[(fn * BS + c) * L + j];
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < BS * L; ++q) bc[(int64_t)I * BS * L + q] = acc[q];
    if (dinv_c) {
      const T* D = dinv_c + (int64_t)I * BS * BS;
#pragma unroll
      for (int c = 0; c < BS; ++c)
#pragma unroll
        for (int j = 0; j < L; ++j) {
          T s = T(0);
#pragma unroll
          for (int d = 0; d < BS; ++d) s += D[c * BS + d] * acc[d * L + j];
          const int64_t idx = (int64_t)I * BS * L + c * L + j;
          d_c[idx] = c2 * s;
          x_c[idx] = c2 * s;
        }
    }
  }
}

// xf += P xc
template <typename T, int BS, int L>
__global__ void k_prolong_add(GridT g, const uint8_t* __restrict__ mask,
                              const T* __restrict__ xc, T* __restrict__ xf) {
  TOPT_KERNEL_COUNT();
  const int fnx = g.nfx + 1, fny = g.nfy + 1, fnz = g.nfz + 1;
  const int nf = fnx * fny * fnz;
  const int64_t cnx = g.ncx + 1, cny = g.ncy + 1;
  for (int F32 = blockIdx.x * blockDim.x + threadIdx.x; F32 < nf;
       F32 += gridDim.x * blockDim.x) {
    const int64_t F = F32;
    const int fy = F32 % fny;
    const int fx = (F32 / fny) % fnx;
    const int fz = F32 / (fny * fnx);
    const int cx = g.c0x[fx], cy = g.c0y[fy], cz = g.c0z[fz];
    const float ax = g.w1x[fx], ay = g.w1y[fy], az = g.w1z[fz];
    T acc[BS * L];
#pragma unroll
    for (int q = 0; q < BS * L; ++q) acc[q] = T(0);
#pragma unroll
    for (int oz = 0; oz < 2; ++oz) {
      const float wz = oz ? az : 1.0f - az;
      if (wz == 0.0f) continue;
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const float wx = (ox ? ax : 1.0f - ax) * wz;
        if (wx == 0.0f) continue;
#pragma unroll
        for (int oy = 0; oy < 2; ++oy) {
          const float wd = (oy ? ay : 1.0f - ay) * wx;
          if (wd == 0.0f) continue;
          const T w = (T)wd;
          const int64_t cn = (cy + oy) + cny * ((cx + ox) + cnx * (int64_t)(cz + oz));
#pragma unroll
          for (int q = 0; q < BS * L; ++q) acc[q] += w * xc[cn * BS * L + q];
        }
      }
    }
#pragma unroll
    for (int c = 0; c < BS; ++c) {
      if (mask && mask[F * BS + c]) continue;
#pragma unroll
      for (int j = 0; j < L; ++j) xf[(F * BS + c) * L + j] += acc[c * L + j];
    }
  }
}

// --------------------------------------------------------------------------
// Element-level Galerkin coarsening: for every coarse cell C,
//   Kc = sum_{fine elements e in C} coef_e P_e^T Ke P_e,
// with P_e the masked trilinear interpolation from C's 8 corners (MeshHex
// local order) to e's nodes.  One CTA per coarse cell; fine elements are the
// hex cells of the finer grid (cell_ptr == nullptr) or the elements listed
// per fine cell.

template <typename T, int BS, int NLOC>
__global__ void __launch_bounds__(256)
k_galerkin(GridT g, const int32_t* __restrict__ cell_list,
           const int32_t* __restrict__ cell_ptr,
           const int32_t* __restrict__ cell_elems, const int32_t* __restrict__ t,
           int64_t n_elem_f, const T* __restrict__ ke, int64_t ke_stride,
           const T* __restrict__ coef, const T* __restrict__ extra,
           const uint8_t* __restrict__ mask, T* __restrict__ kc) {
  TOPT_KERNEL_COUNT();
  constexpr int NF = BS * NLOC;   // fine element DOFs
  constexpr int NC = BS * 8;      // coarse cell DOFs
  __shared__ T Ks[NF * NF];
  __shared__ T Wm[NLOC * 8];
  __shared__ T Mk[NF];
  __shared__ T Tm[NF * NC];
  __shared__ T sc;
  const int64_t C = cell_list ? (int64_t)cell_list[blockIdx.x] : (int64_t)blockIdx.x;
  const int Cy = (int)(C % g.ncy);
  const int Cx = (int)((C / g.ncy) % g.ncx);
  const int Cz = (int)(C / ((int64_t)g.ncy * g.ncx));
  const int ax0 = g.cmx[Cx], ax1 = g.cmx[Cx + 1];
  const int ay0 = g.cmy[Cy], ay1 = g.cmy[Cy + 1];
  const int az0 = g.cmz[Cz], az1 = g.cmz[Cz + 1];
  const int64_t fny = g.nfy + 1, fnx = g.nfx + 1;
  constexpr int PER = (NC * NC + 255) / 256;
  T acc[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) acc[q] = T(0);
  if (ke_stride == 0 && !extra) {
    for (int i = threadIdx.x; i < NF * NF; i += blockDim.x) Ks[i] = ke[i];
  }
  for (int fz = az0; fz < az1; ++fz)
    for (int fx = ax0; fx < ax1; ++fx)
      for (int fy = ay0; fy < ay1; ++fy) {
        const int64_t fc = fy + (int64_t)g.nfy * (fx + (int64_t)g.nfx * fz);
        const int64_t e0 = cell_ptr ? cell_ptr[fc] : fc;
        const int64_t e1 = cell_ptr ? cell_ptr[fc + 1] : fc + 1;
        for (int64_t ei = e0; ei < e1; ++ei) {
          const int64_t e = cell_ptr ? cell_elems[ei] : ei;
          __syncthreads();
          if (extra) {
            // coef_e Ke + X_e, folded here (the scale below is then 1)
            const T ce = coef ? coef[e] : T(1);
            for (int i = threadIdx.x; i < NF * NF; i += blockDim.x)
              Ks[i] = ce * ke[e * ke_stride + i] + extra[e * (NF * NF) + i];
          } else if (ke_stride != 0) {
            for (int i = threadIdx.x; i < NF * NF; i += blockDim.x)
              Ks[i] = ke[e * ke_stride + i];
          }
          if (threadIdx.x < NLOC * 8) {
            const int a = threadIdx.x / 8, k = threadIdx.x % 8;
            const int64_t n = t[(int64_t)a * n_elem_f + e];
            const int iy = (int)(n % fny), ix = (int)((n / fny) % fnx),
                      iz = (int)(n / (fny * fnx));
            // 0, 1/2 or 1 per axis: exact in FP32 (FP64 arithmetic is scarce)
            const float xi = (float)(ix - ax0) / (float)(ax1 - ax0);
            const float yi = (float)(iy - ay0) / (float)(ay1 - ay0);
            const float zi = (float)(iz - az0) / (float)(az1 - az0);
            const float w = (c_hex_off[k][0] ? xi : 1.0f - xi) *
                            (c_hex_off[k][1] ? yi : 1.0f - yi) *
                            (c_hex_off[k][2] ? zi : 1.0f - zi);
            Wm[a * 8 + k] = (T)w;
          }
          if (threadIdx.x < NF) {
            const int a = threadIdx.x / BS, c = threadIdx.x % BS;
            const int64_t n = t[(int64_t)a * n_elem_f + e];
            Mk[threadIdx.x] = (mask && mask[n * BS + c]) ? T(0) : T(1);
          }
          if (threadIdx.x == 0) sc = (coef && !extra) ? coef[e] : T(1);
          __syncthreads();
          // Tm[(a,c),(l,d)] = sum_b Ks[(a,c),(b,d)] Mk[(b,d)] W[b][l]
          for (int i = threadIdx.x; i < NF * NC; i += blockDim.x) {
            const int row = i / NC, col = i % NC;
            const int l = col / BS, d = col % BS;
            T s = T(0);
#pragma unroll
            for (int b = 0; b < NLOC; ++b)
              s += Ks[row * NF + b * BS + d] * Mk[b * BS + d] * Wm[b * 8 + l];
            Tm[i] = s;
          }
          __syncthreads();
          const T scale = sc;
#pragma unroll
          for (int q = 0; q < PER; ++q) {
            const int i = threadIdx.x + q * 256;
            if (i < NC * NC) {
              const int row = i / NC, col = i % NC;
              const int k = row / BS, c = row % BS;
              T s = T(0);
#pragma unroll
              for (int a = 0; a < NLOC; ++a)
                s += Wm[a * 8 + k] * Mk[a * BS + c] * Tm[(a * BS + c) * NC + col];
              acc[q] += scale * s;
            }
          }
        }
      }
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int i = threadIdx.x + q * 256;
    if (i < NC * NC) kc[C * NC * NC + i] = acc[q];
  }
}

// Galerkin coarsening when every fine element is a hex cell sharing one unit
// matrix K0: P_c^T (coef K0) P_c = coef M[pattern][child] with M precomputed
// for the 8 coarse-cell extent patterns (1 or 2 fine cells per axis) and the
// 8 child positions, so Kc = sum_children coef_child M.  Cells touching fixed
// DOFs (masked interpolation) are skipped here and done by k_galerkin.
template <typename T, int BS>
__global__ void __launch_bounds__(192)
k_galerkin_shared(GridT g, const uint8_t* __restrict__ cell_masked, const T* __restrict__ M,
                  const T* __restrict__ coef, T* __restrict__ kc) {
  TOPT_KERNEL_COUNT();
  constexpr int NC = BS * 8;
  constexpr int NN = NC * NC;
  const int64_t ncells = (int64_t)g.ncx * g.ncy * g.ncz;
  for (int64_t C = blockIdx.x; C < ncells; C += gridDim.x) {
    if (cell_masked[C]) continue;
    const int Cy = (int)(C % g.ncy);
    const int Cx = (int)((C / g.ncy) % g.ncx);
    const int Cz = (int)(C / ((int64_t)g.ncy * g.ncx));
    const int x0 = g.cmx[Cx], ex = g.cmx[Cx + 1] - x0;
    const int y0 = g.cmy[Cy], ey = g.cmy[Cy + 1] - y0;
    const int z0 = g.cmz[Cz], ez = g.cmz[Cz + 1] - z0;
    const int pat = (ex - 1) + 2 * (ey - 1) + 4 * (ez - 1);
    T cf[8];
    int nchild = 0;
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
      const int ox = ch & 1, oy = (ch >> 1) & 1, oz = ch >> 2;
      const bool ok = ox < ex && oy < ey && oz < ez;
      const int64_t fc = (y0 + oy) + (int64_t)g.nfy * ((x0 + ox) + (int64_t)g.nfx * (z0 + oz));
      cf[ch] = ok ? coef[fc] : T(0);
      nchild += ok;
    }
    (void)nchild;
    const T* Mp = M + (int64_t)pat * 8 * NN;
    for (int i = threadIdx.x; i < NN; i += blockDim.x) {
      T acc = T(0);
#pragma unroll
      for (int ch = 0; ch < 8; ++ch) acc += cf[ch] * Mp[ch * NN + i];
      kc[C * NN + i] = acc;
    }
  }
}

// --------------------------------------------------------------------------
// Dense coarsest level: BSR -> dense, in-place Gauss-Jordan inverse (one CTA,
// SPD so no pivoting), dense mat-vec.
template <typename T, int BS>
__global__ void k_sell_to_dense(int64_t npos, SellT sp, const T* __restrict__ vals, int n,
                                double* __restrict__ A) {
  TOPT_KERNEL_COUNT();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npos;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t slice = sp.slice_of_grp[k >> 5];
    const int64_t a = slice * 32 + (k & 31);
    if (a >= sp.nrows) continue;
    const int64_t j = (k >> 5) - sp.grp_of_slice[slice];
    if (j >= sp.rowlen[a]) continue;
    const int64_t b = sp.col[k];
#pragma unroll
    for (int c = 0; c < BS; ++c)
#pragma unroll
      for (int d = 0; d < BS; ++d)
        A[(a * BS + c) * n + b * BS + d] = (double)vals[vidx<BS>(k, c * BS + d)];
  }
}

static __global__ void __launch_bounds__(1024) k_gauss_jordan_inverse(int n, double* __restrict__ A) {
  TOPT_KERNEL_COUNT();
  __shared__ double pivinv;
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const double pv = A[(int64_t)k * n + k];
      pivinv = pv != 0.0 ? 1.0 / pv : 0.0;
      A[(int64_t)k * n + k] = 1.0;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) A[(int64_t)k * n + j] *= pivinv;
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
      const int i = idx / n, j = idx % n;
      if (i == k || j == k) continue;
      A[(int64_t)i * n + j] -= A[(int64_t)i * n + k] * A[(int64_t)k * n + j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (i != k) A[(int64_t)i * n + k] = -A[(int64_t)i * n + k] * A[(int64_t)k * n + k];
    __syncthreads();
  }
}

template <typename T>
__global__ void k_dense_copy(int64_t nn, const double* __restrict__ A, T* __restrict__ B) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
       i += (int64_t)gridDim.x * blockDim.x)
    B[i] = (T)A[i];
}

// x = Ainv b for L loads; one warp per output row.
template <typename T, int L>
__global__ void k_dense_matvec(int n, const T* __restrict__ Ainv, const T* __restrict__ b,
                               T* __restrict__ x) {
  TOPT_KERNEL_COUNT();
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n) return;
  T acc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) acc[j] = T(0);
  for (int c = lane; c < n; c += 32) {
    const T a = Ainv[(int64_t)w * n + c];
#pragma unroll
    for (int j = 0; j < L; ++j) acc[j] += a * b[(int64_t)c * L + j];
  }
#pragma unroll
  for (int j = 0; j < L; ++j) acc[j] = warp_sum(acc[j]);
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < L; ++j) x[(int64_t)w * L + j] = acc[j];
  }
}

// --------------------------------------------------------------------------
// Element energies and compliance sensitivities (one thread per element):
// q = u_e^T Ke u_e, energy = 1/2 coef q (solver_elastic.py:470-537),
// dc = dC_drho_simp(rho, energy) (derivatives.py:25-52) times dh.
template <int BS, int NLOC, typename TC>
__global__ void k_energy(int64_t ne, int L, const int32_t* __restrict__ t,
                         const TC* __restrict__ ke, int64_t ke_stride,
                         const double* __restrict__ U, const double* __restrict__ rho,
                         double E0, double Emin, double p, const double* __restrict__ dh,
                         double* __restrict__ energy, double* __restrict__ dc, int interp) {
  TOPT_KERNEL_COUNT();
  constexpr int ND = BS * NLOC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TC* kes = reinterpret_cast<TC*>(smem_raw);
  if (ke_stride == 0) {
    for (int i = threadIdx.x; i < ND * ND; i += blockDim.x) kes[i] = ke[i];
    __syncthreads();
  }
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    const TC* K = ke_stride ? ke + e * ke_stride : kes;
    int64_t node[NLOC];
#pragma unroll
    for (int a = 0; a < NLOC; ++a) node[a] = t[(int64_t)a * ne + e];
    const double r = rho[e];
    const double coef = interp_E(interp, r, E0, Emin, p);
    double dE, Ec;
    if (interp == 1) {   // dC_drho_ramp (derivatives.py:56-72)
      const double den = 1.0 + p * (1.0 - r);
      dE = (E0 - Emin) * (den - p * r) / (den * den);
      Ec = fmax(coef, 1e-12);
    } else {             // dC_drho_simp (derivatives.py:25-52), rho clamped at 1e-6
      const double rc = fmax(r, 1e-6);
      const double rp1 = (p == 3.0) ? rc * rc : pow(rc, p - 1.0);
      dE = p * (E0 - Emin) * rp1;
      Ec = fmax(Emin + (E0 - Emin) * rp1 * rc, 1e-12);
    }
    const double h = dh ? dh[e] : 1.0;
    for (int j = 0; j < L; ++j) {
      // u - u(node 0) per component: a translation lies in the null space of
      // every element matrix, and the shift keeps u^T K u from cancelling
      // when the field carries a large offset (a prescribed temperature)
      TC u[ND];
      double u0[BS];
#pragma unroll
      for (int c = 0; c < BS; ++c) u0[c] = U[(node[0] * BS + c) * L + j];
#pragma unroll
      for (int a = 0; a < NLOC; ++a)
#pragma unroll
        for (int c = 0; c < BS; ++c)
          u[a * BS + c] = (TC)(U[(node[a] * BS + c) * L + j] - u0[c]);
      TC q = TC(0);
#pragma unroll
      for (int i = 0; i < ND; ++i) {
        TC s = TC(0.5) * K[i * ND + i] * u[i];
#pragma unroll
        for (int k = i + 1; k < ND; ++k) s += K[i * ND + k] * u[k];
        q += u[i] * s;
      }
      const double en = coef * (double)q;
      if (energy) energy[e * L + j] = en;
      if (dc) dc[e * L + j] = (-2.0 * en * dE / Ec) * h;
    }
  }
}

}  // namespace topt
