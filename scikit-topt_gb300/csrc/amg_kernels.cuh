// Smoothed-aggregation multigrid for meshes without a logical grid: the
// device kernels.  It replaces pyamg.smoothed_aggregation_solver of the
// reference's cg_pyamg solve (solver_elastic.py:94-103) with a hierarchy
// built on the GPU from the assembled block operator (SELL storage, see
// fem_kernels.cuh):
//
//  * aggregation: a distance-2 maximal independent set of the block graph
//    (every stored block connects, the strength threshold 0 of PyAMG's SA
//    default) found with hashed priorities; each set node is the root of an
//    aggregate with its neighbours, the remaining nodes (at distance 2 of a
//    root) join an aggregated neighbour.  The graph is the sparsity pattern
//    only, so the aggregates are fixed for a mesh and built once;
//  * candidates: the bs per-component translations, zero on fixed DOFs.  The
//    tentative prolongator is then diagonal per block, with
//    T(i, a)_cc = sqrt(cnt_i,c / cnt_a,c), cnt being the number of free
//    finest-level DOFs of component c below a node (integers: exact sums);
//  * smoothed prolongator P = T - omega / lambda_max(Dinv A) Dinv A T with
//    the block-diagonal inverse Dinv and omega = 4/3 (PyAMG's Jacobi
//    smoothing);
//  * Galerkin coarse operator P^T (A P).
//
// Patterns of P, A P and P^T A P are computed once (symbolic kernels: one
// CTA per output row expands the candidate products, sorts them in shared
// memory by (column, expansion order) and keeps, per output block, the list
// of products that sum into it).  Every refresh then recomputes the values
// by summing those lists in their fixed order: deterministic, no atomics
// on values.
#pragma once

#include "fem_kernels.cuh"

namespace topt {

// ---------------------------------------------------------------- scans
// Exclusive prefix sums of n int32 counts into int64 offsets (out[n] = the
// total): per-CTA sums, one CTA scanning those, per-CTA application.
constexpr int kScanThreads = 256, kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t block_excl_scan64(int64_t v, int64_t* sh, int64_t* total) {
  // sh: kScanThreads / 32 + 1 entries
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t s = 0;
    const int nw = blockDim.x >> 5;
    for (int i = 0; i < nw; ++i) {
      const int64_t t = sh[i];
      sh[i] = s;
      s += t;
    }
    sh[nw] = s;
  }
  __syncthreads();
  const int64_t r = x - v + sh[w];
  if (total) *total = sh[blockDim.x >> 5];
  __syncthreads();
  return r;
}

static __global__ void __launch_bounds__(kScanThreads) k_scan_tiles(int64_t n, const int32_t* in,
                                                             int64_t* tile_sum) {
  TOPT_KERNEL_COUNT();
  __shared__ int64_t sh[kScanThreads / 32 + 1];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) s += in[base + k];
  int64_t tot;
  block_excl_scan64(s, sh, &tot);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

static __global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(int64_t ntiles,
                                                                 int64_t* tile_sum,
                                                                 int64_t* total) {
  TOPT_KERNEL_COUNT();
  __shared__ int64_t sh[kScanThreads / 32 + 1];
  int64_t carry = 0;
  for (int64_t b0 = 0; b0 < ntiles; b0 += kScanThreads) {
    const int64_t i = b0 + threadIdx.x;
    const int64_t v = i < ntiles ? tile_sum[i] : 0;
    int64_t tot;
    const int64_t e = block_excl_scan64(v, sh, &tot);
    if (i < ntiles) tile_sum[i] = carry + e;
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

static __global__ void __launch_bounds__(kScanThreads) k_scan_apply(int64_t n, const int32_t* in,
                                                             const int64_t* tile_sum,
                                                             int64_t* out) {
  TOPT_KERNEL_COUNT();
  __shared__ int64_t sh[kScanThreads / 32 + 1];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) s += in[base + k];
  int64_t run = block_excl_scan64(s, sh, nullptr) + tile_sum[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) {
      out[base + k] = run;
      run += in[base + k];
    }
}

// ---------------------------------------------------------------- aggregation
__device__ __forceinline__ uint32_t amg_hash(uint32_t x) {
  // integer mixer (xorshift-multiply rounds) for node priorities
  x ^= x >> 16;
  x *= 0x45d9f3bu;
  x ^= x >> 16;
  x *= 0x45d9f3bu;
  x ^= x >> 16;
  return x;
}

constexpr uint8_t kMisOut = 0, kMisUndecided = 1, kMisIn = 2;

// (state, priority, node) packed so that IN > UNDECIDED > OUT, then by
// priority, then by node index: a total order.
__device__ __forceinline__ uint64_t mis_key(uint32_t state, uint32_t i) {
  return ((uint64_t)state << 62) | ((uint64_t)(amg_hash(i) >> 2) << 32) | (uint64_t)i;
}

// Position of entry k of block row i in SELL storage.
__device__ __forceinline__ int64_t sell_pos(const SellT& sp, int64_t i, int k) {
  return ((int64_t)sp.grp_of_slice[i >> 5] + k) * 32 + (i & 31);
}

static __global__ void k_mis_keys(int64_t n, const uint8_t* __restrict__ state,
                           uint64_t* __restrict__ keys) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    keys[i] = mis_key(state[i], (uint32_t)i);
}

// out[i] = max of in[j] over the stored blocks (i, j) of row i (self included).
static __global__ void k_mis_max(SellT sp, const uint64_t* __restrict__ in, uint64_t* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < sp.nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t m = in[i];
    const int len = sp.rowlen[i];
    for (int k = 0; k < len; ++k) {
      const uint64_t v = in[sp.col[sell_pos(sp, i, k)]];
      m = v > m ? v : m;
    }
    out[i] = m;
  }
}

// An undecided node enters the set when the maximum over its distance-2
// neighbourhood is itself, and leaves it when that maximum is a set node;
// *left is set while any node stays undecided.
static __global__ void k_mis_update(int64_t n, uint8_t* __restrict__ state,
                             const uint64_t* __restrict__ m2, int* __restrict__ left) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (state[i] != kMisUndecided) continue;
    const uint64_t m = m2[i];
    if ((uint32_t)(m >> 62) == kMisIn)
      state[i] = kMisOut;
    else if ((uint32_t)m == (uint32_t)i)
      state[i] = kMisIn;
    else
      *left = 1;
  }
}

static __global__ void k_mis_roots(int64_t n, const uint8_t* __restrict__ state,
                            int32_t* __restrict__ is_root) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    is_root[i] = state[i] == kMisIn ? 1 : 0;
}

// Roots take their own aggregate; every other node the aggregate of its
// root neighbour (set nodes are >= 3 apart: at most one), else -1.
static __global__ void k_agg_first(SellT sp, const uint8_t* __restrict__ state,
                            const int64_t* __restrict__ root_id, int32_t* __restrict__ agg) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < sp.nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (state[i] == kMisIn) {
      agg[i] = (int32_t)root_id[i];
      continue;
    }
    int32_t a = -1;
    const int len = sp.rowlen[i];
    for (int k = 0; k < len; ++k) {
      const int32_t j = sp.col[sell_pos(sp, i, k)];
      if (state[j] == kMisIn) {
        a = (int32_t)root_id[j];
        break;
      }
    }
    agg[i] = a;
  }
}

// The remaining nodes join the aggregate of their aggregated neighbour of
// highest priority (reads the first pass only: order-independent).
static __global__ void k_agg_second(SellT sp, const int32_t* __restrict__ agg1,
                             int32_t* __restrict__ agg2, int* __restrict__ err) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < sp.nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t a = agg1[i];
    if (a < 0) {
      uint64_t best = 0;
      const int len = sp.rowlen[i];
      for (int k = 0; k < len; ++k) {
        const int32_t j = sp.col[sell_pos(sp, i, k)];
        if (agg1[j] < 0) continue;
        const uint64_t key = mis_key(1, (uint32_t)j);
        if (key > best) {
          best = key;
          a = agg1[j];
        }
      }
      if (a < 0) *err = 1;
    }
    agg2[i] = a;
  }
}

// cnt_c[a, c] = sum over the members i of aggregate a of cnt_f[i, c].
template <int BS>
__global__ void k_agg_counts(int64_t n, const int32_t* __restrict__ agg,
                             const int32_t* __restrict__ cnt_f, int32_t* __restrict__ cnt_c) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = agg[i];
    if (a < 0) continue;
#pragma unroll
    for (int c = 0; c < BS; ++c) {
      const int32_t v = cnt_f[i * BS + c];
      if (v) atomicAdd(cnt_c + (int64_t)a * BS + c, v);
    }
  }
}

// Level-0 counts: 1 per free DOF.
static __global__ void k_free_counts(int64_t n, const uint8_t* __restrict__ mask,
                              int32_t* __restrict__ cnt) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    cnt[i] = mask[i] ? 0 : 1;
}

// ---------------------------------------------------------------- symbolic
// One CTA per output row: the candidate products of the row are expanded
// into shared memory as (key = column << 32 | expansion index, payload),
// sorted, and reduced to the distinct columns.  Phase 0 counts (distinct
// columns, candidates); phase 1 writes, at the offsets given by the scans
// of those counts: the column of every output block, the first candidate of
// every output block, and the payloads in sorted order.
constexpr int kSymThreads = 256;
constexpr int kSymCap = 8192;        // candidates per output row (err beyond)
constexpr int kSymSegCap = 2048;     // expansion segments per row (err beyond)
constexpr size_t kSymSmem = (size_t)kSymCap * 16 + (size_t)kSymSegCap * 4 * 2 + 64 * 8;

enum SymKind : int { kSymP = 0, kSymAP = 1, kSymRAP = 2 };

struct SymArgs {
  int64_t nrows;
  // kSymP: rows of the fine level (A pattern), columns agg[col]
  SellT a;
  const int32_t* agg;
  // kSymAP: fine rows; for block (i, j) of A, the P row of j
  const int64_t* p_ptr;     // fine node -> first P entry
  const int32_t* p_col;
  // kSymRAP: coarse rows; R entries (fine node, P entry), then the AP row
  const int64_t* r_ptr;
  const int32_t* r_fine;
  const int32_t* r_pent;
  const int64_t* ap_ptr;
  const int32_t* ap_col;
  // phase 0 outputs
  int32_t* nuniq;
  int32_t* ncand;
  // phase 1 inputs (scans) and outputs
  const int64_t* u_off;     // row -> first output block
  const int64_t* c_off;     // row -> first candidate
  int32_t* out_col;         // per output block
  int32_t* out_row;         // per output block (optional)
  int64_t* out_first;       // per output block: first candidate (global index)
  int32_t* pay_a;           // per candidate
  int32_t* pay_b;           // per candidate (unused by kSymP)
  int* err;
};

__device__ __forceinline__ void sym_sort(uint64_t* key, uint64_t* val, int n2) {
  for (int k = 2; k <= n2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < n2; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const bool up = (t & k) == 0;
          const uint64_t a = key[t], b = key[u];
          if ((a > b) == up) {
            key[t] = b;
            key[u] = a;
            const uint64_t va = val[t];
            val[t] = val[u];
            val[u] = va;
          }
        }
      }
      __syncthreads();
    }
}

template <int KIND, int PHASE>
__global__ void __launch_bounds__(kSymThreads) k_sym(SymArgs g) {
  TOPT_KERNEL_COUNT();
  extern __shared__ __align__(16) unsigned char sym_smem[];
  uint64_t* key = reinterpret_cast<uint64_t*>(sym_smem);
  uint64_t* val = key + kSymCap;
  int32_t* seg_n = reinterpret_cast<int32_t*>(val + kSymCap);   // per segment: candidates
  int32_t* seg_o = seg_n + kSymSegCap;                           // per segment: offset
  int64_t* sh = reinterpret_cast<int64_t*>(seg_o + kSymSegCap);  // scan scratch
  __shared__ int s_bad;
  for (int64_t row = blockIdx.x; row < g.nrows; row += gridDim.x) {
    // 1. segments of the expansion and their candidate counts
    int nseg;
    if (KIND == kSymRAP)
      nseg = (int)(g.r_ptr[row + 1] - g.r_ptr[row]);
    else
      nseg = g.a.rowlen[row];
    if (threadIdx.x == 0) s_bad = nseg > kSymSegCap;
    __syncthreads();
    if (s_bad) {
      if (threadIdx.x == 0) *g.err = 1;
      __syncthreads();
      continue;
    }
    for (int s = threadIdx.x; s < nseg; s += blockDim.x) {
      int cnt;
      if (KIND == kSymP) {
        cnt = 1;
      } else if (KIND == kSymAP) {
        const int32_t j = g.a.col[sell_pos(g.a, row, s)];
        cnt = (int)(g.p_ptr[j + 1] - g.p_ptr[j]);
      } else {
        const int32_t i = g.r_fine[g.r_ptr[row] + s];
        cnt = (int)(g.ap_ptr[i + 1] - g.ap_ptr[i]);
      }
      seg_n[s] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t o = 0;
      for (int s = 0; s < nseg; ++s) {
        seg_o[s] = (int32_t)(o < (int64_t)INT32_MAX ? o : (int64_t)INT32_MAX);
        o += seg_n[s];
      }
      s_bad = o > kSymCap ? 1 : 0;
      sh[0] = o;
    }
    __syncthreads();
    const int n = (int)(sh[0] < (int64_t)kSymCap ? sh[0] : (int64_t)kSymCap);
    if (s_bad) {
      if (threadIdx.x == 0) *g.err = 2;
      __syncthreads();
      continue;
    }
    // 2. expansion: one thread per segment writes its candidates
    for (int s = threadIdx.x; s < nseg; s += blockDim.x) {
      const int o = seg_o[s];
      if (KIND == kSymP) {
        const int64_t pos = sell_pos(g.a, row, s);
        const uint32_t col = (uint32_t)g.agg[g.a.col[pos]];
        key[o] = ((uint64_t)col << 32) | (uint32_t)o;
        val[o] = (uint64_t)pos;
      } else if (KIND == kSymAP) {
        const int64_t pos = sell_pos(g.a, row, s);
        const int32_t j = g.a.col[pos];
        const int64_t m0 = g.p_ptr[j];
        for (int q = 0; q < seg_n[s]; ++q) {
          const uint32_t col = (uint32_t)g.p_col[m0 + q];
          key[o + q] = ((uint64_t)col << 32) | (uint32_t)(o + q);
          val[o + q] = ((uint64_t)(uint32_t)pos << 32) | (uint32_t)(m0 + q);
        }
      } else {
        const int64_t t = g.r_ptr[row] + s;
        const int32_t i = g.r_fine[t];
        const int32_t m = g.r_pent[t];
        const int64_t e0 = g.ap_ptr[i];
        for (int q = 0; q < seg_n[s]; ++q) {
          const uint32_t col = (uint32_t)g.ap_col[e0 + q];
          key[o + q] = ((uint64_t)col << 32) | (uint32_t)(o + q);
          val[o + q] = ((uint64_t)(uint32_t)m << 32) | (uint32_t)(e0 + q);
        }
      }
    }
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int t = n + threadIdx.x; t < n2; t += blockDim.x) {
      key[t] = ~0ull;
      val[t] = 0;
    }
    __syncthreads();
    // 3. sort by (column, expansion index)
    sym_sort(key, val, n2);
    // 4. distinct columns: heads of runs, counted per contiguous chunk
    const int chunk = (n + blockDim.x - 1) / blockDim.x;
    const int t0 = threadIdx.x * chunk, t1 = min(n, t0 + chunk);
    int heads = 0;
    for (int t = t0; t < t1; ++t)
      if (t == 0 || (key[t] >> 32) != (key[t - 1] >> 32)) ++heads;
    int64_t nu;
    const int64_t hb = block_excl_scan64(heads, sh, &nu);
    if (PHASE == 0) {
      if (threadIdx.x == 0) {
        g.nuniq[row] = (int32_t)nu;
        g.ncand[row] = n;
      }
    } else {
      const int64_t ub = g.u_off[row], cb = g.c_off[row];
      int64_t u = ub + hb;
      for (int t = t0; t < t1; ++t) {
        if (t == 0 || (key[t] >> 32) != (key[t - 1] >> 32)) {
          g.out_col[u] = (int32_t)(key[t] >> 32);
          if (g.out_row) g.out_row[u] = (int32_t)row;
          g.out_first[u] = cb + t;
          ++u;
        }
        if (KIND == kSymP) {
          g.pay_a[cb + t] = (int32_t)val[t];
        } else {
          g.pay_a[cb + t] = (int32_t)(val[t] >> 32);
          g.pay_b[cb + t] = (int32_t)(uint32_t)val[t];
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- transpose
// R = P^T pattern: count per coarse node, then fill in fine-row order by
// a per-coarse-row sort of the (fine node, P entry) pairs.
static __global__ void k_rt_count(int64_t np, const int32_t* __restrict__ p_col,
                           int32_t* __restrict__ cnt) {
  TOPT_KERNEL_COUNT();
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < np;
       m += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + p_col[m], 1);
}

static __global__ void k_rt_fill(int64_t np, const int32_t* __restrict__ p_col,
                          const int32_t* __restrict__ p_row, const int64_t* __restrict__ r_ptr,
                          int32_t* __restrict__ cursor, int32_t* __restrict__ r_fine,
                          int32_t* __restrict__ r_pent) {
  TOPT_KERNEL_COUNT();
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < np;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = p_col[m];
    const int64_t t = r_ptr[a] + atomicAdd(cursor + a, 1);
    r_fine[t] = p_row[m];
    r_pent[t] = (int32_t)m;
  }
}

// Insertion sort of each coarse row by fine node (a node appears once).
static __global__ void k_rt_sort(int64_t nc, const int64_t* __restrict__ r_ptr,
                          int32_t* __restrict__ r_fine, int32_t* __restrict__ r_pent) {
  TOPT_KERNEL_COUNT();
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nc;
       a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = r_ptr[a], e = r_ptr[a + 1];
    for (int64_t t = b + 1; t < e; ++t) {
      const int32_t f = r_fine[t], m = r_pent[t];
      int64_t u = t - 1;
      while (u >= b && r_fine[u] > f) {
        r_fine[u + 1] = r_fine[u];
        r_pent[u + 1] = r_pent[u];
        --u;
      }
      r_fine[u + 1] = f;
      r_pent[u + 1] = m;
    }
  }
}

// ---------------------------------------------------------------- numeric
// P(i, a) = [agg(i) == a] T_i - s Dinv_i sum_{k in list} A(pos_k) T_{col(pos_k)}
// with T_j = diag(sqrt(cnt_f[j, c] / cnt_c[agg(j), c])) and s = omega /
// lambda_max.  One thread per P block.
template <typename T, int BS>
__device__ __forceinline__ T amg_tw(const int32_t* cnt_f, const int32_t* cnt_c,
                                    const int32_t* agg, int64_t j, int c) {
  const int32_t f = cnt_f[j * BS + c];
  if (!f) return T(0);
  return (T)sqrt((double)f / (double)cnt_c[(int64_t)agg[j] * BS + c]);
}

template <typename T, int BS>
__global__ void k_amg_p(int64_t np, SellT sp, const T* __restrict__ vals,
                        const T* __restrict__ dinv, const int32_t* __restrict__ agg,
                        const int32_t* __restrict__ cnt_f, const int32_t* __restrict__ cnt_c,
                        const int32_t* __restrict__ p_row, const int32_t* __restrict__ p_col,
                        const int64_t* __restrict__ p_first, const int32_t* __restrict__ pos,
                        T s, T* __restrict__ pv) {
  TOPT_KERNEL_COUNT();
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < np;
       m += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p_row[m];
    const int32_t a = p_col[m];
    T acc[BS * BS];
#pragma unroll
    for (int v = 0; v < BS * BS; ++v) acc[v] = T(0);
    for (int64_t q = p_first[m]; q < p_first[m + 1]; ++q) {
      const int64_t ps = pos[q];
      const int64_t j = sp.col[ps];
      T w[BS];
#pragma unroll
      for (int c = 0; c < BS; ++c) w[c] = amg_tw<T, BS>(cnt_f, cnt_c, agg, j, c);
#pragma unroll
      for (int r = 0; r < BS; ++r)
#pragma unroll
        for (int c = 0; c < BS; ++c) acc[r * BS + c] += vals[vidx<BS>(ps, r * BS + c)] * w[c];
    }
    const T* D = dinv + i * BS * BS;
    T out[BS * BS];
#pragma unroll
    for (int r = 0; r < BS; ++r)
#pragma unroll
      for (int c = 0; c < BS; ++c) {
        T t = T(0);
#pragma unroll
        for (int d = 0; d < BS; ++d) t += D[r * BS + d] * acc[d * BS + c];
        out[r * BS + c] = -s * t;
      }
    if (agg[i] == a) {
#pragma unroll
      for (int c = 0; c < BS; ++c) out[c * BS + c] += amg_tw<T, BS>(cnt_f, cnt_c, agg, i, c);
    }
#pragma unroll
    for (int v = 0; v < BS * BS; ++v) pv[m * BS * BS + v] = out[v];
  }
}

// AP(e) = sum over its list of A(pos) P(m).  One thread per AP block.
template <typename T, int BS>
__global__ void k_amg_ap(int64_t nap, const T* __restrict__ vals, const T* __restrict__ pv,
                         const int64_t* __restrict__ first, const int32_t* __restrict__ pos,
                         const int32_t* __restrict__ pent, T* __restrict__ apv) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nap;
       e += (int64_t)gridDim.x * blockDim.x) {
    T acc[BS * BS];
#pragma unroll
    for (int v = 0; v < BS * BS; ++v) acc[v] = T(0);
    for (int64_t q = first[e]; q < first[e + 1]; ++q) {
      const int64_t ps = pos[q];
      const T* P = pv + (int64_t)pent[q] * BS * BS;
      T A[BS * BS], B[BS * BS];
#pragma unroll
      for (int v = 0; v < BS * BS; ++v) {
        A[v] = vals[vidx<BS>(ps, v)];
        B[v] = P[v];
      }
#pragma unroll
      for (int r = 0; r < BS; ++r)
#pragma unroll
        for (int c = 0; c < BS; ++c)
#pragma unroll
          for (int d = 0; d < BS; ++d) acc[r * BS + c] += A[r * BS + d] * B[d * BS + c];
    }
#pragma unroll
    for (int v = 0; v < BS * BS; ++v) apv[e * BS * BS + v] = acc[v];
  }
}

// A_c(e) = sum over its list of P(m)^T AP(f), written at the coarse SELL
// position of the block.  One thread per coarse block.
template <typename T, int BS>
__global__ void k_amg_rap(int64_t nc_ent, const T* __restrict__ pv, const T* __restrict__ apv,
                          const int64_t* __restrict__ first, const int32_t* __restrict__ pent,
                          const int32_t* __restrict__ apent, const int32_t* __restrict__ cpos,
                          T* __restrict__ vals_c) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nc_ent;
       e += (int64_t)gridDim.x * blockDim.x) {
    T acc[BS * BS];
#pragma unroll
    for (int v = 0; v < BS * BS; ++v) acc[v] = T(0);
    for (int64_t q = first[e]; q < first[e + 1]; ++q) {
      const T* P = pv + (int64_t)pent[q] * BS * BS;
      const T* Q = apv + (int64_t)apent[q] * BS * BS;
      T A[BS * BS], B[BS * BS];
#pragma unroll
      for (int v = 0; v < BS * BS; ++v) {
        A[v] = P[v];
        B[v] = Q[v];
      }
#pragma unroll
      for (int r = 0; r < BS; ++r)
#pragma unroll
        for (int c = 0; c < BS; ++c)
#pragma unroll
          for (int d = 0; d < BS; ++d) acc[r * BS + c] += A[d * BS + r] * B[d * BS + c];
    }
    const int64_t ps = cpos[e];
#pragma unroll
    for (int v = 0; v < BS * BS; ++v) vals_c[vidx<BS>(ps, v)] = acc[v];
  }
}

// ---------------------------------------------------------------- transfers
// bc = P^T r (coarse node gathers its R row in fine-node order); with
// dinv_c set, also the first Chebyshev step of the coarse level from a zero
// guess: d_c = x_c = c2 Dinv_c bc.  Fixed fine DOFs (mask) contribute 0.
template <typename T, int BS, int L>
__global__ void k_amg_restrict(int64_t nc, const int64_t* __restrict__ r_ptr,
                               const int32_t* __restrict__ r_fine,
                               const int32_t* __restrict__ r_pent, const T* __restrict__ pv,
                               const uint8_t* __restrict__ mask, const T* __restrict__ rf,
                               T* __restrict__ bc, const T* __restrict__ dinv_c,
                               T* __restrict__ d_c, T* __restrict__ x_c, T c2) {
  TOPT_KERNEL_COUNT();
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nc;
       a += (int64_t)gridDim.x * blockDim.x) {
    T acc[BS * L];
#pragma unroll
    for (int q = 0; q < BS * L; ++q) acc[q] = T(0);
    for (int64_t t = r_ptr[a]; t < r_ptr[a + 1]; ++t) {
      const int64_t i = r_fine[t];
      const T* P = pv + (int64_t)r_pent[t] * BS * BS;
      T ri[BS * L];
#pragma unroll
      for (int d = 0; d < BS; ++d) {
        const bool fixed = mask && mask[i * BS + d];
#pragma unroll
        for (int j = 0; j < L; ++j) ri[d * L + j] = fixed ? T(0) : rf[(i * BS + d) * L + j];
      }
#pragma unroll
      for (int c = 0; c < BS; ++c)
#pragma unroll
        for (int d = 0; d < BS; ++d) {
          const T p = P[d * BS + c];
#pragma unroll
          for (int j = 0; j < L; ++j) acc[c * L + j] += p * ri[d * L + j];
        }
    }
#pragma unroll
    for (int q = 0; q < BS * L; ++q) bc[a * BS * L + q] = acc[q];
    if (dinv_c) {
      const T* D = dinv_c + a * BS * BS;
#pragma unroll
      for (int c = 0; c < BS; ++c)
#pragma unroll
        for (int j = 0; j < L; ++j) {
          T s = T(0);
#pragma unroll
          for (int d = 0; d < BS; ++d) s += D[c * BS + d] * acc[d * L + j];
          const int64_t idx = a * BS * L + c * L + j;
          d_c[idx] = c2 * s;
          x_c[idx] = c2 * s;
        }
    }
  }
}

// xf += P xc (fixed fine DOFs untouched).
template <typename T, int BS, int L>
__global__ void k_amg_prolong_add(int64_t nf, const int64_t* __restrict__ p_ptr,
                                  const int32_t* __restrict__ p_col, const T* __restrict__ pv,
                                  const uint8_t* __restrict__ mask, const T* __restrict__ xc,
                                  T* __restrict__ xf) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    T acc[BS * L];
#pragma unroll
    for (int q = 0; q < BS * L; ++q) acc[q] = T(0);
    for (int64_t m = p_ptr[i]; m < p_ptr[i + 1]; ++m) {
      const T* P = pv + m * BS * BS;
      const int64_t a = p_col[m];
#pragma unroll
      for (int r = 0; r < BS; ++r)
#pragma unroll
        for (int c = 0; c < BS; ++c) {
          const T p = P[r * BS + c];
#pragma unroll
          for (int j = 0; j < L; ++j) acc[r * L + j] += p * xc[(a * BS + c) * L + j];
        }
    }
#pragma unroll
    for (int r = 0; r < BS; ++r) {
      if (mask && mask[i * BS + r]) continue;
#pragma unroll
      for (int j = 0; j < L; ++j) xf[(i * BS + r) * L + j] += acc[r * L + j];
    }
  }
}

}  // namespace topt
