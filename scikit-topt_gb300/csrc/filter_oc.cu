// Gaussian density filter, Heaviside projection, OC bisection, LogMOC update
// and deterministic reductions.
//
// Replaces SpacialFilter (sktopt/filters/spacial.py:19-166), the projection
// functions (sktopt/core/projection.py:27-118), bisection_with_physical_volume
// (sktopt/core/optimizers/oc.py:16-95) and lagrangian_log_update
// (sktopt/core/optimizers/logmoc.py:36-66).
#include "filter_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <unordered_map>
#include <vector>

namespace topt {

// --------------------------------------------------------------------------
// host: W = D^-1 K_gauss over design element centres (spacial.py:37-103)
static int build_gauss(topt_filter* f, const double* c, const uint8_t* mask, double radius) {
  const int64_t n = f->n_elem;
  std::vector<int32_t> design;
  design.reserve(n);
  for (int64_t i = 0; i < n; ++i)
    if (!mask || mask[i]) design.push_back((int32_t)i);
  const int64_t nd = (int64_t)design.size();
  if (nd == 0) return fail(TOPT_BAD_INPUT, "filter: empty design set");
  const double s = radius / 3.0;
  const double support = 3.0 * s;
  const double sup2 = support * support;
  // uniform grid hash of the design centres with cell size = support
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t k = 0; k < nd; ++k)
    for (int d = 0; d < 3; ++d) {
      const double v = c[d * n + design[k]];
      lo[d] = std::min(lo[d], v);
      hi[d] = std::max(hi[d], v);
    }
  const double h = support > 0 ? support : 1.0;
  int64_t dim[3];
  for (int d = 0; d < 3; ++d) dim[d] = std::max<int64_t>(1, (int64_t)std::floor((hi[d] - lo[d]) / h) + 1);
  auto cell_of = [&](const double* p, int64_t out[3]) {
    for (int d = 0; d < 3; ++d) {
      int64_t q = (int64_t)std::floor((p[d] - lo[d]) / h);
      out[d] = std::min<int64_t>(std::max<int64_t>(q, 0), dim[d] - 1);
    }
  };
  const int64_t ncell = dim[0] * dim[1] * dim[2];
  std::vector<int64_t> cptr(ncell + 1, 0);
  std::vector<int64_t> ccell(nd);
  for (int64_t k = 0; k < nd; ++k) {
    double p[3] = {c[design[k]], c[n + design[k]], c[2 * n + design[k]]};
    int64_t q[3];
    cell_of(p, q);
    ccell[k] = (q[2] * dim[1] + q[1]) * dim[0] + q[0];
    cptr[ccell[k] + 1]++;
  }
  for (int64_t i = 0; i < ncell; ++i) cptr[i + 1] += cptr[i];
  std::vector<int32_t> cidx(nd);
  {
    std::vector<int64_t> pos(cptr.begin(), cptr.end() - 1);
    for (int64_t k = 0; k < nd; ++k) cidx[pos[ccell[k]]++] = (int32_t)k;
  }
  f->h_rowptr.assign(nd + 1, 0);
  f->h_colind.clear();
  f->h_vals.clear();
  f->h_colind.reserve(nd * 20);
  f->h_vals.reserve(nd * 20);
  std::vector<std::pair<int32_t, double>> row;
  for (int64_t k = 0; k < nd; ++k) {
    const int64_t i = design[k];
    const double pi[3] = {c[i], c[n + i], c[2 * n + i]};
    int64_t q[3];
    cell_of(pi, q);
    row.clear();
    for (int64_t z = std::max<int64_t>(q[2] - 1, 0); z <= std::min(q[2] + 1, dim[2] - 1); ++z)
      for (int64_t y = std::max<int64_t>(q[1] - 1, 0); y <= std::min(q[1] + 1, dim[1] - 1); ++y)
        for (int64_t x = std::max<int64_t>(q[0] - 1, 0); x <= std::min(q[0] + 1, dim[0] - 1); ++x) {
          const int64_t cc = (z * dim[1] + y) * dim[0] + x;
          for (int64_t m = cptr[cc]; m < cptr[cc + 1]; ++m) {
            const int32_t kk = cidx[m];
            const int64_t j = design[kk];
            const double dx = c[j] - pi[0], dy = c[n + j] - pi[1], dz = c[2 * n + j] - pi[2];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 <= sup2) {
              const double dij = std::sqrt(d2);
              const double u = dij / s;
              row.push_back({kk, std::exp(-0.5 * (u * u))});
            }
          }
        }
    std::sort(row.begin(), row.end(),
              [](const std::pair<int32_t, double>& a, const std::pair<int32_t, double>& b) {
                return a.first < b.first;
              });
    double rs = 0.0;
    for (auto& pr : row) rs += pr.second;
    if (rs == 0.0) rs = 1.0;
    const double inv = 1.0 / rs;
    for (auto& pr : row) {
      f->h_colind.push_back(pr.first);
      f->h_vals.push_back(pr.second * inv);
    }
    f->h_rowptr[k + 1] = (int32_t)f->h_colind.size();
  }
  f->n_design = nd;
  f->nnz = (int64_t)f->h_colind.size();
  // device copies with full-element columns, and the transpose
  std::vector<int32_t> colfull(f->nnz);
  for (int64_t k = 0; k < f->nnz; ++k) colfull[k] = design[f->h_colind[k]];
  std::vector<int32_t> trp(nd + 1, 0), tcol(f->nnz);
  std::vector<double> tval(f->nnz);
  for (int64_t k = 0; k < f->nnz; ++k) trp[f->h_colind[k] + 1]++;
  for (int64_t i = 0; i < nd; ++i) trp[i + 1] += trp[i];
  {
    std::vector<int32_t> pos(trp.begin(), trp.end() - 1);
    for (int64_t r = 0; r < nd; ++r)
      for (int32_t k = f->h_rowptr[r]; k < f->h_rowptr[r + 1]; ++k) {
        const int32_t col = f->h_colind[k];
        tcol[pos[col]] = design[r];
        tval[pos[col]] = f->h_vals[k];
        pos[col]++;
      }
  }
  std::vector<int32_t> nondesign;
  for (int64_t i = 0; i < n; ++i)
    if (mask && !mask[i]) nondesign.push_back((int32_t)i);
  f->n_nondesign = (int64_t)nondesign.size();
  cudaStream_t st = nullptr;
  int rc;
  if ((rc = upload(f->design, design.data(), design.size(), st))) return rc;
  if ((rc = upload(f->nondesign, nondesign.data(), nondesign.size(), st))) return rc;
  if ((rc = upload(f->rowptr, f->h_rowptr.data(), f->h_rowptr.size(), st))) return rc;
  if ((rc = upload(f->colfull, colfull.data(), colfull.size(), st))) return rc;
  if ((rc = upload(f->vals, f->h_vals.data(), f->h_vals.size(), st))) return rc;
  if ((rc = upload(f->t_rowptr, trp.data(), trp.size(), st))) return rc;
  if ((rc = upload(f->t_colfull, tcol.data(), tcol.size(), st))) return rc;
  if ((rc = upload(f->t_vals, tval.data(), tval.size(), st))) return rc;
  if ((rc = f->cand.alloc(sizeof(double) * n))) return rc;
  if ((rc = f->state.alloc(sizeof(OcState)))) return rc;
  if ((rc = f->partials.alloc(sizeof(double) * f->sm * 16 * 2))) return rc;
  if ((rc = f->counter.alloc(16 * sizeof(unsigned)))) return rc;
  TOPT_CUDA(cudaMemset(f->counter.p, 0, 16 * sizeof(unsigned)));
  TOPT_CUDA(cudaDeviceSynchronize());
  return TOPT_OK;
}

// --------------------------------------------------------------------------
// y[rows[i]] = sum_k V[k] x[col[k]]  (CSR rows indexed by design position)
__global__ void k_csr_rows(int64_t nrows, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ col, const double* __restrict__ v,
                           const int32_t* __restrict__ rows, const double* __restrict__ x,
                           double* __restrict__ y) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrows;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) s += v[k] * x[col[k]];
    y[rows[i]] = s;
  }
}

__global__ void k_scatter_copy(int64_t n, const int32_t* __restrict__ idx,
                               const double* __restrict__ x, double* __restrict__ y,
                               int zero) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = idx[i];
    y[e] = zero ? 0.0 : x[e];
  }
}

// --------------------------------------------------------------------------
// Heaviside projection (projection.py:27-118)
__global__ void k_projection(int64_t n, const double* __restrict__ x, double beta, double eta,
                             double tbe, double den, double* __restrict__ h,
                             double* __restrict__ dh) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double a = (x[i] - eta) * beta;
    if (h) h[i] = (tbe + tanh(a)) / den;
    if (dh) {
      const double c = cosh(a);
      dh[i] = (1.0 / (c * c)) * beta / den;
    }
  }
}

// --------------------------------------------------------------------------
// OC bisection (oc.py:16-95).  Step 1: candidate densities for the current
// lmid; step 2: filter + projection + volume, then the bisection bookkeeping
// in the last block (deterministic reduction order).
__device__ __forceinline__ double clip_nan(double a, double lo, double hi) {
  a = (a < lo) ? lo : a;   // NaN propagates like numpy.clip
  return (a > hi) ? hi : a;
}

__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// Bisection step gates: 0 = every step until done, 1 = only steps whose FP32
// volume was ambiguous (need64), 2 = unconditionally (final pass).
__device__ __forceinline__ bool oc_gate(const OcState* st, int mode) {
  if (mode == 2) return true;
  if (st->done) return false;
  return mode == 0 || st->need64;
}

// One decision of the bisection (oc.py:16-95): stop when the volume error is
// within vol_tol, the iteration cap is reached or the bracket is narrower
// than tolerance; otherwise halve the bracket towards the error's sign.
__device__ __forceinline__ void oc_decide(OcState* st, const topt_oc_params& prm, double ve) {
  st->steps = st->it + 1;
  st->need64 = 0;
  if (fabs(ve) < prm.vol_tol || st->it >= prm.max_iter ||
      fabs(st->l2 - st->l1) <= prm.tolerance) {
    st->done = 1;
  } else {
    if (ve > 0) st->l1 = st->lmid;
    else st->l2 = st->lmid;
    st->it += 1;
    st->lmid = 0.5 * (st->l1 + st->l2);
  }
}

__global__ void k_oc_candidate(int64_t nd, const int32_t* __restrict__ design,
                               const double* __restrict__ dc, double dc_scale,
                               const double* __restrict__ rho_e,
                               const OcState* __restrict__ st, topt_oc_params prm,
                               double* __restrict__ cand, double* __restrict__ rho_new,
                               double* __restrict__ scaling, int mode) {
  TOPT_KERNEL_COUNT();
  if (!oc_gate(st, mode)) return;
  const double lm = st->lmid;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = design[i];
    double sr = (-(dc[e] / dc_scale)) / (lm + prm.eps);
    sr = (prm.eta == 0.5) ? sqrt(sr) : pow(sr, prm.eta);
    sr = clip_nan(sr, prm.scaling_min, prm.scaling_max);
    const double r = rho_e[i];
    const double lo = fmax(r - prm.move_limit, prm.rho_min);
    const double hi = fmin(r + prm.move_limit, prm.rho_max);
    const double v = clip_nan(r * sr, lo, hi);
    cand[e] = v;
    rho_new[i] = v;
    if (scaling) scaling[i] = sr;
  }
}

__global__ void k_gather(int64_t n, const int32_t* __restrict__ idx, const double* __restrict__ x,
                         double* __restrict__ y) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[idx[i]];
}

__global__ void k_scatter(int64_t n, const int32_t* __restrict__ idx, const double* __restrict__ x,
                          double* __restrict__ y) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[idx[i]] = x[i];
}

// Design-indexed reductions: OP 0 max |x[d]|, 1 max |x[d] - y[d]|,
// 2 KKT: max over interior d of |x[d] + c * w[i]| (oc.py:230-240).
template <int OP>
__global__ void k_design_reduce(int64_t nd, const int32_t* __restrict__ design,
                                const double* __restrict__ x, const double* __restrict__ y,
                                const double* __restrict__ w, double c, double rho_min,
                                double rho_max, double* partials, unsigned* counter,
                                double* out) {
  TOPT_KERNEL_COUNT();
  double m = 0.0;
  int nan = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = design[i];
    double a;
    if (OP == 0) a = fabs(x[e]);
    else if (OP == 1) a = fabs(x[e] - y[e]);
    else {
      const double r = y[e];
      if (!(r > rho_min + 1e-6 && r < rho_max - 1e-6)) continue;
      a = fabs(x[e] + c * w[i]);
    }
    if (a != a) nan = 1;
    m = a > m ? a : m;
  }
  grid_max_finish(m, nan != 0, partials, counter, out);
}

__global__ void k_oc_volume(int64_t nd, const int32_t* __restrict__ rowptr,
                            const int32_t* __restrict__ col, const double* __restrict__ w,
                            const double* __restrict__ cand, const double* __restrict__ vol,
                            double vol_sum, topt_oc_params prm, double tbe, double den,
                            OcState* st, double* partials, unsigned* counter, int mode) {
  TOPT_KERNEL_COUNT();
  if (!oc_gate(st, mode)) return;
  double acc[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) s += w[k] * cand[col[k]];
    const double a = (s - prm.beta_eta) * prm.beta;
    const double hp = (tbe + tanh(a)) / den;
    acc[0] += hp * vol[i];
  }
  __shared__ double sh[32];
  __shared__ double total;
  block_sum<double, 1>(acc, sh);
  if (grid_finish<double, 1>(acc, partials, counter, &total)) {
    if (threadIdx.x == 0) {
      const double ve = total / vol_sum - prm.vol_frac;
      st->vol_error = ve;
      if (mode != 2) oc_decide(st, prm, ve);
    }
  }
}

// FP32 bracketing of the bisection.  Per call: the sensitivity part of the
// scaling rate (-dc/scale)^eta, rho and the move-limit box in FP32.  Per
// step: the candidate and the filtered, projected volume in FP32, and the
// decision taken from it only when it is unambiguous: the FP32 volume error
// lies within err of the FP64 one (err bounds the FP32 rounding through the
// filter and the projection slope), so the decision of the FP64 bisection --
// the sign of the error and |error| < vol_tol -- is the same whenever
// |ve32| > err and ||ve32| - vol_tol| > err.  Otherwise need64 is set and
// the FP64 kernels evaluate that step exactly.  The path of lmid values, and
// hence the result, is that of the FP64 bisection.
struct Oc32 {
  float sq, r, lo, hi;
};

__global__ void k_oc_prep32(int64_t nd, const int32_t* __restrict__ design,
                            const double* __restrict__ dc, double dc_scale,
                            const double* __restrict__ rho_e, topt_oc_params prm,
                            Oc32* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double q = -(dc[design[i]] / dc_scale);
    const double sq = (prm.eta == 0.5) ? sqrt(q) : pow(q, prm.eta);
    const double r = rho_e[i];
    Oc32 o;
    o.sq = (float)sq;
    o.r = (float)r;
    o.lo = (float)fmax(r - prm.move_limit, prm.rho_min);
    o.hi = (float)fmin(r + prm.move_limit, prm.rho_max);
    out[i] = o;
  }
}

__device__ __forceinline__ float clipf_nan(float a, float lo, float hi) {
  a = (a < lo) ? lo : a;
  return (a > hi) ? hi : a;
}

__global__ void k_oc_cand32(int64_t nd, const int32_t* __restrict__ design,
                            const Oc32* __restrict__ in, const OcState* __restrict__ st,
                            topt_oc_params prm, float* __restrict__ cand) {
  TOPT_KERNEL_COUNT();
  if (st->done) return;
  __shared__ float s_lam;
  if (threadIdx.x == 0) s_lam = (float)pow(st->lmid + prm.eps, -prm.eta);
  __syncthreads();
  const float lam = s_lam, smin = (float)prm.scaling_min, smax = (float)prm.scaling_max;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Oc32 o = in[i];
    const float sr = clipf_nan(o.sq * lam, smin, smax);
    cand[design[i]] = clipf_nan(o.r * sr, o.lo, o.hi);
  }
}

__global__ void k_oc_vol32(int64_t nd, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ col, const float* __restrict__ w,
                           const float* __restrict__ cand, const double* __restrict__ vol,
                           double vol_sum, topt_oc_params prm, float tbe, float den,
                           double err, OcState* st, double* partials, unsigned* counter) {
  TOPT_KERNEL_COUNT();
  if (st->done) return;
  const float beta = (float)prm.beta, beta_eta = (float)prm.beta_eta;
  float tacc = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) s += w[k] * cand[col[k]];
    const float hp = (tbe + tanhf((s - beta_eta) * beta)) / den;
    tacc += hp * (float)vol[i];
  }
  double acc[1] = {(double)tacc};
  __shared__ double sh[32];
  __shared__ double total;
  block_sum<double, 1>(acc, sh);
  if (grid_finish<double, 1>(acc, partials, counter, &total)) {
    if (threadIdx.x == 0) {
      const double ve = total / vol_sum - prm.vol_frac;
      const double a = fabs(ve);
      if (!(a > err) || fabs(a - prm.vol_tol) <= err) {
        st->need64 = 1;
      } else {
        st->need64 = 0;
        st->vol_error = ve;
        oc_decide(st, prm, ve);
      }
    }
  }
}

// k_oc_vol32 with W applied as a stencil on a structured grid: s_k = W_kk
// sum_o g_o cand[e + lin_o] over the offsets whose bit is set in the row's
// neighbour mask (inside the grid and a design element), in the CSR column
// order.  The candidate array (4 bytes per element) stays in L2 across the
// steps of a bisection; the offsets sit in shared memory.
__global__ void k_oc_vol32s(int64_t nd, const int32_t* __restrict__ design,
                            const int32_t* __restrict__ lin, const float* __restrict__ gw,
                            int no, const unsigned long long* __restrict__ nb,
                            const float* __restrict__ invd, const float* __restrict__ cand,
                            const double* __restrict__ vol, double vol_sum, topt_oc_params prm,
                            float tbe, float den, double err, OcState* st, double* partials,
                            unsigned* counter) {
  TOPT_KERNEL_COUNT();
  if (st->done) return;
  __shared__ int s_lin[64];
  __shared__ float s_g[64];
  for (int k = threadIdx.x; k < no; k += blockDim.x) {
    s_lin[k] = lin[k];
    s_g[k] = gw[k];
  }
  __syncthreads();
  const float beta = (float)prm.beta, beta_eta = (float)prm.beta_eta;
  float tacc = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = design[i];
    unsigned long long m = nb[i];
    float s = 0.0f;
    while (m) {
      const int k = __ffsll((long long)m) - 1;
      m &= m - 1;
      s += s_g[k] * cand[e + s_lin[k]];
    }
    s *= invd[i];
    const float hp = (tbe + tanhf((s - beta_eta) * beta)) / den;
    tacc += hp * (float)vol[i];
  }
  double acc[1] = {(double)tacc};
  __shared__ double sh[32];
  __shared__ double total;
  block_sum<double, 1>(acc, sh);
  if (grid_finish<double, 1>(acc, partials, counter, &total)) {
    if (threadIdx.x == 0) {
      const double ve = total / vol_sum - prm.vol_frac;
      const double a = fabs(ve);
      if (!(a > err) || fabs(a - prm.vol_tol) <= err) {
        st->need64 = 1;
      } else {
        st->need64 = 0;
        st->vol_error = ve;
        oc_decide(st, prm, ve);
      }
    }
  }
}

// Derive the stencil form of W on an nx x ny x nz cell grid, or leave st_n
// = 0 when some row does not have it (then the CSR kernel runs).  Offsets
// are checked against every row: the same neighbour set (design cells of
// the grid within the offset set) and W_kj = g_o W_kk to 1e-12.
static int derive_stencil(topt_filter* f) {
  f->st_n = 0;
  const int nx = f->grid[0], ny = f->grid[1], nz = f->grid[2];
  const int64_t n = f->n_elem, nd = f->n_design;
  if (nx <= 0 || (int64_t)nx * ny * nz != n || nd == 0) return TOPT_OK;
  std::vector<int32_t> design(nd);
  TOPT_CUDA(cudaMemcpy(design.data(), f->design.p, sizeof(int32_t) * nd,
                       cudaMemcpyDeviceToHost));
  std::vector<uint8_t> dmask(n, 0);
  for (int64_t k = 0; k < nd; ++k) dmask[design[k]] = 1;
  auto coords = [&](int64_t e, int& x, int& y, int& z) {
    y = (int)(e % ny);
    x = (int)((e / ny) % nx);
    z = (int)(e / ((int64_t)ny * nx));
  };
  // offsets and weights from the row with the most entries
  int64_t best = 0;
  for (int64_t k = 0; k < nd; ++k)
    if (f->h_rowptr[k + 1] - f->h_rowptr[k] > f->h_rowptr[best + 1] - f->h_rowptr[best]) best = k;
  struct Off { int dx, dy, dz; double g; };
  std::vector<Off> offs;
  {
    int x0, y0, z0;
    coords(design[best], x0, y0, z0);
    double wkk = 0.0;
    for (int32_t q = f->h_rowptr[best]; q < f->h_rowptr[best + 1]; ++q)
      if (design[f->h_colind[q]] == design[best]) wkk = f->h_vals[q];
    if (!(wkk > 0.0)) return TOPT_OK;
    for (int32_t q = f->h_rowptr[best]; q < f->h_rowptr[best + 1]; ++q) {
      int x, y, z;
      coords(design[f->h_colind[q]], x, y, z);
      offs.push_back({x - x0, y - y0, z - z0, f->h_vals[q] / wkk});
    }
  }
  if (offs.empty() || offs.size() > 64) return TOPT_OK;
  for (const Off& o : offs)
    if (std::abs(o.dx) > 8 || std::abs(o.dy) > 8 || std::abs(o.dz) > 8) return TOPT_OK;
  // CSR column order = ascending element index = ascending linear offset
  std::sort(offs.begin(), offs.end(), [&](const Off& a, const Off& b) {
    return (int64_t)a.dy + (int64_t)ny * (a.dx + (int64_t)nx * a.dz) <
           (int64_t)b.dy + (int64_t)ny * (b.dx + (int64_t)nx * b.dz);
  });
  std::vector<float> invd(nd);
  std::vector<unsigned long long> nbm(nd, 0ull);
  for (int64_t k = 0; k < nd; ++k) {
    int x0, y0, z0;
    const int64_t e = design[k];
    coords(e, x0, y0, z0);
    double wkk = 0.0;
    for (int32_t q = f->h_rowptr[k]; q < f->h_rowptr[k + 1]; ++q)
      if (design[f->h_colind[q]] == e) wkk = f->h_vals[q];
    if (!(wkk > 0.0)) return TOPT_OK;
    int32_t q = f->h_rowptr[k];
    for (size_t oi = 0; oi < offs.size(); ++oi) {
      const Off& o = offs[oi];
      const int x = x0 + o.dx, y = y0 + o.dy, z = z0 + o.dz;
      if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
      const int64_t j = y + (int64_t)ny * (x + (int64_t)nx * z);
      if (!dmask[j]) continue;
      if (q >= f->h_rowptr[k + 1] || design[f->h_colind[q]] != j) return TOPT_OK;
      if (std::fabs(f->h_vals[q] - o.g * wkk) > 1e-12 * wkk) return TOPT_OK;
      nbm[k] |= 1ull << oi;
      ++q;
    }
    if (q != f->h_rowptr[k + 1]) return TOPT_OK;
    invd[k] = (float)wkk;
  }
  std::vector<int32_t> lin(offs.size());
  std::vector<float> gw(offs.size());
  for (size_t k = 0; k < offs.size(); ++k) {
    lin[k] = (int32_t)(offs[k].dy + (int64_t)ny * (offs[k].dx + (int64_t)nx * offs[k].dz));
    gw[k] = (float)offs[k].g;
  }
  int rc;
  if ((rc = upload(f->st_lin, lin.data(), lin.size(), nullptr))) return rc;
  if ((rc = upload(f->st_g, gw.data(), gw.size(), nullptr))) return rc;
  if ((rc = upload(f->st_invd, invd.data(), invd.size(), nullptr))) return rc;
  if ((rc = upload(f->st_nb, nbm.data(), nbm.size(), nullptr))) return rc;
  TOPT_CUDA(cudaDeviceSynchronize());
  f->st_n = (int)offs.size();
  return TOPT_OK;
}

// --------------------------------------------------------------------------
// Reductions with host results.
template <int OP>  // 0: max |x| (NaN-propagating), 1: dot
__global__ void k_reduce(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                         double* partials, unsigned* counter, double* out) {
  TOPT_KERNEL_COUNT();
  double acc[1] = {0.0};
  bool nan = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (OP == 0) {
      const double a = fabs(x[i]);
      if (a != a) nan = true;
      acc[0] = a > acc[0] ? a : acc[0];
    } else {
      acc[0] += x[i] * y[i];
    }
  }
  if (OP == 0) {
    grid_max_finish(acc[0], nan, partials, counter, out);
  } else {
    __shared__ double sh[32];
    block_sum<double, 1>(acc, sh);
    grid_finish<double, 1>(acc, partials, counter, out);
  }
}

// scratch of the stand-alone reductions (one set per host thread and device)
struct ReduceScratch {
  DevBuf partials, counter, out;
  int dev = -1;
};
// per host thread: calls from different threads (on different streams) never
// share it
static thread_local ReduceScratch g_red;

static int reduce_scratch(int blocks) {
  int dev = 0;
  TOPT_CUDA(cudaGetDevice(&dev));
  if (g_red.partials.p && g_red.dev == dev) return TOPT_OK;
  int rc;
  if ((rc = g_red.partials.alloc(sizeof(double) * blocks))) return rc;
  if ((rc = g_red.counter.alloc(16 * sizeof(unsigned)))) return rc;
  if ((rc = g_red.out.alloc(16 * sizeof(double)))) return rc;
  TOPT_CUDA(cudaMemset(g_red.counter.p, 0, 16 * sizeof(unsigned)));
  g_red.dev = dev;
  return TOPT_OK;
}

}  // namespace topt

using namespace topt;

extern "C" {

int topt_filter_gauss_create(int64_t n_elem, const double* centers, const uint8_t* design_mask,
                             double radius, topt_filter** out) {
  if (!out || !centers || n_elem <= 0 || !(radius > 0.0))
    return fail(TOPT_BAD_INPUT, "filter_create: bad argument");
  *out = nullptr;
  std::unique_ptr<topt_filter> f(new (std::nothrow) topt_filter());
  if (!f) return fail(TOPT_NO_MEMORY, "filter_create: host allocation");
  f->n_elem = n_elem;
  f->sm = device_sm_count();
  int rc;
  try {
    rc = build_gauss(f.get(), centers, design_mask, radius);
  } catch (const std::bad_alloc&) {
    rc = fail(TOPT_NO_MEMORY, "filter_create: host allocation");
  }
  if (rc) return rc;
  *out = f.release();
  return TOPT_OK;
}

void topt_filter_destroy(topt_filter* f) {
  if (!f) return;
  cudaDeviceSynchronize();
  delete f;
}

int topt_filter_set_grid(topt_filter* f, int32_t nx, int32_t ny, int32_t nz) {
  if (!f || nx < 0 || ny < 0 || nz < 0) return fail(TOPT_BAD_INPUT, "filter_set_grid: bad argument");
  f->grid[0] = nx;
  f->grid[1] = ny;
  f->grid[2] = nz;
  return derive_stencil(f);
}

int topt_filter_stencil_size(const topt_filter* f, int32_t* n_offsets) {
  if (!f || !n_offsets) return fail(TOPT_BAD_INPUT, "filter_stencil_size: null argument");
  *n_offsets = f->st_n;
  return TOPT_OK;
}

int topt_filter_set_stream(topt_filter* f, void* s) {
  if (!f) return fail(TOPT_BAD_INPUT, "filter: null handle");
  f->stream = (cudaStream_t)s;
  return TOPT_OK;
}

int topt_filter_sizes(const topt_filter* f, int64_t* n_design, int64_t* nnz) {
  if (!f) return fail(TOPT_BAD_INPUT, "filter: null handle");
  if (n_design) *n_design = f->n_design;
  if (nnz) *nnz = f->nnz;
  return TOPT_OK;
}

int topt_filter_export(const topt_filter* f, int32_t* rowptr, int32_t* colind, double* vals) {
  if (!f) return fail(TOPT_BAD_INPUT, "filter: null handle");
  if (rowptr) std::copy(f->h_rowptr.begin(), f->h_rowptr.end(), rowptr);
  if (colind) std::copy(f->h_colind.begin(), f->h_colind.end(), colind);
  if (vals) std::copy(f->h_vals.begin(), f->h_vals.end(), vals);
  return TOPT_OK;
}

int topt_filter_forward(topt_filter* f, const double* x, double* y) {
  if (!f || !x || !y) return fail(TOPT_BAD_INPUT, "filter_forward: null argument");
  if (x == y) return fail(TOPT_BAD_INPUT, "filter_forward: in-place call not supported");
  const int g = grid_for(f->n_design, kFB, f->sm * 16);
  k_csr_rows<<<g, kFB, 0, f->stream>>>(f->n_design, f->rowptr.as<int32_t>(),
                                       f->colfull.as<int32_t>(), f->vals.as<double>(),
                                       f->design.as<int32_t>(), x, y);
  if (f->n_nondesign)
    k_scatter_copy<<<grid_for(f->n_nondesign, kFB, f->sm * 16), kFB, 0, f->stream>>>(
        f->n_nondesign, f->nondesign.as<int32_t>(), x, y, 0);
  TOPT_CHECK_LAUNCH("filter_forward");
  return TOPT_OK;
}

int topt_filter_gradient(topt_filter* f, const double* v, double* y) {
  if (!f || !v || !y) return fail(TOPT_BAD_INPUT, "filter_gradient: null argument");
  if (v == y) return fail(TOPT_BAD_INPUT, "filter_gradient: in-place call not supported");
  const int g = grid_for(f->n_design, kFB, f->sm * 16);
  k_csr_rows<<<g, kFB, 0, f->stream>>>(f->n_design, f->t_rowptr.as<int32_t>(),
                                       f->t_colfull.as<int32_t>(), f->t_vals.as<double>(),
                                       f->design.as<int32_t>(), v, y);
  if (f->n_nondesign)
    k_scatter_copy<<<grid_for(f->n_nondesign, kFB, f->sm * 16), kFB, 0, f->stream>>>(
        f->n_nondesign, f->nondesign.as<int32_t>(), v, y, 1);
  TOPT_CHECK_LAUNCH("filter_gradient");
  return TOPT_OK;
}

int topt_projection(int64_t n, const double* x, double beta, double eta, double* h,
                    double* dh, void* stream) {
  if (n < 0 || (n > 0 && !x)) return fail(TOPT_BAD_INPUT, "projection: bad argument");
  if (n == 0) return TOPT_OK;
  const double tbe = std::tanh(beta * eta);
  const double den = tbe + std::tanh(beta * (1.0 - eta)) + 1e-12;
  k_projection<<<grid_for(n, kFB, device_sm_count() * 16), kFB, 0, (cudaStream_t)stream>>>(
      n, x, beta, eta, tbe, den, h, dh);
  TOPT_CHECK_LAUNCH("k_projection");
  return TOPT_OK;
}

int topt_oc_bisect(topt_filter* f, const double* dc, double dc_scale, double* rho,
                   const double* vol, double vol_sum, const topt_oc_params* prm,
                   double* scaling, double* lmid, double* vol_error, int32_t* steps) {
  if (!f || !dc || !rho || !vol || !prm) return fail(TOPT_BAD_INPUT, "oc_bisect: null argument");
  if (!(prm->l1 < prm->l2)) return fail(TOPT_BAD_INPUT, "oc_bisect: need l1 < l2");
  if (!(dc_scale > 0.0)) return fail(TOPT_BAD_INPUT, "oc_bisect: dc_scale must be > 0");
  const int64_t nd = f->n_design;
  int rc;
  if (!f->rho_e.p && (rc = f->rho_e.alloc(sizeof(double) * nd))) return rc;
  if (!f->rho_new.p && (rc = f->rho_new.alloc(sizeof(double) * nd))) return rc;
  OcState s0{};
  s0.l1 = prm->l1;
  s0.l2 = prm->l2;
  s0.lmid = 0.5 * (prm->l1 + prm->l2);
  TOPT_CUDA(cudaMemcpyAsync(f->state.p, &s0, sizeof(s0), cudaMemcpyHostToDevice, f->stream));
  const double tbe = std::tanh(prm->beta * prm->beta_eta);
  const double den = tbe + std::tanh(prm->beta * (1.0 - prm->beta_eta)) + 1e-12;
  // every step halves |l2 - l1|; the loop ends once it is <= tolerance
  int max_steps = 1;
  {
    double w = prm->l2 - prm->l1;
    while (w > prm->tolerance && max_steps < 4096) { w *= 0.5; ++max_steps; }
    max_steps = std::min(max_steps + 1, prm->max_iter + 1);
  }
  const int g = grid_for(nd, kFB, f->sm * 8);
  const int32_t* design = f->design.as<int32_t>();
  k_gather<<<g, kFB, 0, f->stream>>>(nd, design, rho, f->rho_e.as<double>());
  OcState* st = f->state.as<OcState>();
  const bool bracket = !(prm->flags & TOPT_OC_EXACT);
  auto fp64_step = [&](int mode) {
    k_oc_candidate<<<g, kFB, 0, f->stream>>>(nd, design, dc, dc_scale, f->rho_e.as<double>(),
                                             st, *prm, f->cand.as<double>(),
                                             f->rho_new.as<double>(), scaling, mode);
    k_oc_volume<<<g, kFB, 0, f->stream>>>(nd, f->rowptr.as<int32_t>(), f->colfull.as<int32_t>(),
                                          f->vals.as<double>(), f->cand.as<double>(), vol,
                                          vol_sum, *prm, tbe, den, st,
                                          f->partials.as<double>(), f->counter.as<unsigned>(),
                                          mode);
  };
  if (bracket) {
    if (!f->vals32.p) {
      if ((rc = f->vals32.alloc(sizeof(float) * std::max<int64_t>(f->nnz, 1)))) return rc;
      if ((rc = f->cand32.alloc(sizeof(float) * f->n_elem))) return rc;
      if ((rc = f->oc32.alloc(sizeof(Oc32) * nd))) return rc;
      k_to_f32<<<grid_for(f->nnz, kFB, f->sm * 8), kFB, 0, f->stream>>>(
          f->nnz, f->vals.as<double>(), f->vals32.as<float>());
    }
    k_oc_prep32<<<g, kFB, 0, f->stream>>>(nd, design, dc, dc_scale, f->rho_e.as<double>(), *prm,
                                          f->oc32.as<Oc32>());
    // bound on |ve32 - ve64|: FP32 rounding of the candidate and the filtered
    // density (<= 1.5e-6 absolute for weights summing to 1) amplified by the
    // projection slope beta/den, plus the FP32 tanh and partial sums; doubled
    const double err = 2.0 * (2.0e-6 * (1.0 + prm->beta / den) + 1.0e-6);
    for (int k = 0; k < max_steps; ++k) {
      k_oc_cand32<<<g, kFB, 0, f->stream>>>(nd, design, f->oc32.as<Oc32>(), st, *prm,
                                            f->cand32.as<float>());
      if (f->st_n > 0)
        k_oc_vol32s<<<g, kFB, 0, f->stream>>>(
            nd, f->design.as<int32_t>(), f->st_lin.as<int32_t>(), f->st_g.as<float>(), f->st_n,
            f->st_nb.as<unsigned long long>(), f->st_invd.as<float>(), f->cand32.as<float>(),
            vol, vol_sum, *prm, (float)tbe, (float)den, err, st, f->partials.as<double>(),
            f->counter.as<unsigned>());
      else
        k_oc_vol32<<<g, kFB, 0, f->stream>>>(nd, f->rowptr.as<int32_t>(),
                                             f->colfull.as<int32_t>(), f->vals32.as<float>(),
                                             f->cand32.as<float>(), vol, vol_sum, *prm,
                                             (float)tbe, (float)den, err, st,
                                             f->partials.as<double>(), f->counter.as<unsigned>());
      fp64_step(1);
    }
    fp64_step(2);   // exact candidate and volume error at the final lmid
  } else {
    for (int k = 0; k < max_steps; ++k) fp64_step(0);
  }
  k_scatter<<<g, kFB, 0, f->stream>>>(nd, design, f->rho_new.as<double>(), rho);
  TOPT_CHECK_LAUNCH("oc_bisect");
  OcState out{};
  TOPT_CUDA(cudaMemcpyAsync(&out, f->state.p, sizeof(out), cudaMemcpyDeviceToHost, f->stream));
  TOPT_CUDA(cudaStreamSynchronize(f->stream));
  if (lmid) *lmid = out.lmid;
  if (vol_error) *vol_error = out.vol_error;
  if (steps) *steps = out.steps;
  if (!out.done) return fail(TOPT_MAXITER, "oc_bisect: bisection did not terminate");
  return TOPT_OK;
}

int topt_design_reduce(topt_filter* f, int32_t op, const double* x, const double* y,
                       const double* w, double c, double rho_min, double rho_max,
                       double* out) {
  if (!f || !x || !out || op < 0 || op > 2 || (op > 0 && !y) || (op == 2 && !w))
    return fail(TOPT_BAD_INPUT, "design_reduce: bad argument");
  const int64_t nd = f->n_design;
  const int g = grid_for(nd, kFB, f->sm * 8);
  double* part = f->partials.as<double>();
  unsigned* ctr = f->counter.as<unsigned>() + 1;
  double* res = f->partials.as<double>() + f->sm * 16 * 2 - 1;
  const int32_t* design = f->design.as<int32_t>();
  if (op == 0)
    k_design_reduce<0><<<g, kFB, 0, f->stream>>>(nd, design, x, y, w, c, rho_min, rho_max, part,
                                                 ctr, res);
  else if (op == 1)
    k_design_reduce<1><<<g, kFB, 0, f->stream>>>(nd, design, x, y, w, c, rho_min, rho_max, part,
                                                 ctr, res);
  else
    k_design_reduce<2><<<g, kFB, 0, f->stream>>>(nd, design, x, y, w, c, rho_min, rho_max, part,
                                                 ctr, res);
  TOPT_CHECK_LAUNCH("k_design_reduce");
  TOPT_CUDA(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, f->stream));
  TOPT_CUDA(cudaStreamSynchronize(f->stream));
  return TOPT_OK;
}

int topt_reduce_max_abs(int64_t n, const double* x, double* out, void* stream) {
  if (!out || n < 0 || (n > 0 && !x)) return fail(TOPT_BAD_INPUT, "reduce_max_abs: bad argument");
  if (n == 0) { *out = 0.0; return TOPT_OK; }
  const int blocks = grid_for(n, kFB, device_sm_count() * 8);
  int rc = reduce_scratch(device_sm_count() * 8);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  k_reduce<0><<<blocks, kFB, 0, s>>>(n, x, nullptr, g_red.partials.as<double>(),
                                     g_red.counter.as<unsigned>(), g_red.out.as<double>());
  TOPT_CHECK_LAUNCH("k_reduce<max>");
  TOPT_CUDA(cudaMemcpyAsync(out, g_red.out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  TOPT_CUDA(cudaStreamSynchronize(s));
  return TOPT_OK;
}

int topt_reduce_dot(int64_t n, const double* x, const double* y, double* out, void* stream) {
  if (!out || n < 0 || (n > 0 && (!x || !y))) return fail(TOPT_BAD_INPUT, "reduce_dot: bad argument");
  if (n == 0) { *out = 0.0; return TOPT_OK; }
  const int blocks = grid_for(n, kFB, device_sm_count() * 8);
  int rc = reduce_scratch(device_sm_count() * 8);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  k_reduce<1><<<blocks, kFB, 0, s>>>(n, x, y, g_red.partials.as<double>(),
                                     g_red.counter.as<unsigned>() + 1, g_red.out.as<double>() + 1);
  TOPT_CHECK_LAUNCH("k_reduce<dot>");
  TOPT_CUDA(cudaMemcpyAsync(out, g_red.out.as<double>() + 1, sizeof(double),
                            cudaMemcpyDeviceToHost, s));
  TOPT_CUDA(cudaStreamSynchronize(s));
  return TOPT_OK;
}

}  // extern "C"

// --------------------------------------------------------------------------
// Dot product that allocates nothing.  Some callers cannot call cudaMalloc:
// a host that gives all device memory to its own pool and forbids stray
// allocations, or a loop that must not stall on the implicit device
// synchronisation of cudaMalloc/cudaFree.  For them the reduction scratch
// (one partial sum per chunk of the input, the last-block arrival counter and
// the result slot) is a file-scope device array of fixed size, ~32 KB, that
// every GPU loading the library keeps until the process exits.
namespace topt {

constexpr int64_t kNoAllocChunk = 65536;   // elements summed by one block
constexpr int kNoAllocMaxBlocks = 4096;    // partial sums the scratch can hold
constexpr int64_t kNoAllocMaxN = kNoAllocChunk * kNoAllocMaxBlocks;  // 268,435,456

struct NoAllocScratch {
  double partials[kNoAllocMaxBlocks];
  double result;
  unsigned counter;
};
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Block b sums x[i] * y[i] over its chunk [b*chunk, (b+1)*chunk); the last
// block to finish adds the partials in block order (deterministic).
__global__ void k_dot_chunked(int64_t n, const double* __restrict__ x,
                              const double* __restrict__ y, NoAllocScratch* s) {
  TOPT_KERNEL_COUNT();
  const int64_t b0 = (int64_t)blockIdx.x * kNoAllocChunk;
  const int64_t b1 = b0 + kNoAllocChunk < n ? b0 + kNoAllocChunk : n;
  double acc[1] = {0.0};
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) acc[0] += x[i] * y[i];
  __shared__ double sh[32];
  block_sum<double, 1>(acc, sh);
  grid_finish<double, 1>(acc, s->partials, &s->counter, &s->result);
}

// Device address of the scratch array, looked up once per device (host code
// only holds a host-side stand-in for the symbol; kernels need this address).
static int noalloc_scratch_address(NoAllocScratch** out) {
  static std::mutex mu;
  static NoAllocScratch* addr[64] = {};
  int dev = 0;
  TOPT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(TOPT_BAD_INPUT, "reduce_dot_noalloc: device id >= 64");
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    TOPT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[dev] = static_cast<NoAllocScratch*>(p);
  }
  *out = addr[dev];
  return TOPT_OK;
}

}  // namespace topt

extern "C" int topt_reduce_dot_noalloc(int64_t n, const double* x, const double* y,
                                       double* out, void* stream) {
  using namespace topt;
  if (!out || n < 0 || (n > 0 && (!x || !y)))
    return fail(TOPT_BAD_INPUT, "reduce_dot_noalloc: bad argument");
  if (n > kNoAllocMaxN)
    return fail(TOPT_BAD_INPUT, "reduce_dot_noalloc: n exceeds the maximum of 268435456 "
                                "elements that the fixed scratch supports");
  if (n == 0) {
    *out = 0.0;
    return TOPT_OK;
  }
  NoAllocScratch* s = nullptr;
  int rc = noalloc_scratch_address(&s);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // the arrival counter must start at zero whatever the previous call left
  TOPT_CUDA(cudaMemsetAsync(&s->counter, 0, sizeof(unsigned), st));
  const int blocks = (int)((n + kNoAllocChunk - 1) / kNoAllocChunk);
  k_dot_chunked<<<blocks, kFB, 0, st>>>(n, x, y, s);
  TOPT_CHECK_LAUNCH("k_dot_chunked");
  TOPT_CUDA(cudaMemcpyAsync(out, &s->result, sizeof(double), cudaMemcpyDeviceToHost, st));
  TOPT_CUDA(cudaStreamSynchronize(st));
  return TOPT_OK;
}

namespace topt {
int launches_filter(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}
}  // namespace topt
