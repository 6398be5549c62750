// Design-set operations shared by every filter: the identity design handle,
// the stepwise OC bisection (for filters whose forward is not a fixed matrix),
// design reductions, the numpy-compatible percentile, the LogMOC log-space
// update and the Helmholtz element<->node transfers.
//
// Replaces bisection_with_physical_volume (sktopt/core/optimizers/oc.py:16-95)
// when driven one step at a time, LogMOC_Optimizer.rho_update
// (sktopt/core/optimizers/logmoc.py:90-258) with lagrangian_log_update
// (logmoc.py:36-66), and element_to_node_density_averaging /
// node_to_element_density (sktopt/filters/helmholtz_filter_nodal.py:26-56).
#include "filter_internal.cuh"

#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <vector>

namespace topt {

__device__ __forceinline__ double clip_nan2(double a, double lo, double hi) {
  a = (a < lo) ? lo : a;
  return (a > hi) ? hi : a;
}

__global__ void k_oc_cand_step(int64_t nd, const int32_t* __restrict__ design,
                               const double* __restrict__ dc, double dc_scale,
                               const double* __restrict__ rho_e, const OcState* __restrict__ st,
                               topt_oc_params prm, double* __restrict__ cand,
                               double* __restrict__ rho_new, double* __restrict__ scaling) {
  TOPT_KERNEL_COUNT();
  if (st->done) return;
  const double lm = st->lmid;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = design[i];
    double sr = (-(dc[e] / dc_scale)) / (lm + prm.eps);
    sr = (prm.eta == 0.5) ? sqrt(sr) : pow(sr, prm.eta);
    sr = clip_nan2(sr, prm.scaling_min, prm.scaling_max);
    const double r = rho_e[i];
    const double v = clip_nan2(r * sr, fmax(r - prm.move_limit, prm.rho_min),
                               fmin(r + prm.move_limit, prm.rho_max));
    cand[e] = v;
    rho_new[i] = v;
    if (scaling) scaling[i] = sr;
  }
}

// projection of the filtered candidate, weighted volume over the design, and
// the bisection bookkeeping in the last block (oc.py:69-93)
__global__ void k_oc_vol_step(int64_t nd, const int32_t* __restrict__ design,
                              const double* __restrict__ filtered,
                              const double* __restrict__ vol, double vol_sum,
                              topt_oc_params prm, double tbe, double den, OcState* st,
                              double* partials, unsigned* counter) {
  TOPT_KERNEL_COUNT();
  if (st->done) return;
  double acc[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double a = (filtered[design[i]] - prm.beta_eta) * prm.beta;
    acc[0] += ((tbe + tanh(a)) / den) * vol[i];
  }
  __shared__ double sh[32];
  __shared__ double total;
  block_sum<double, 1>(acc, sh);
  if (grid_finish<double, 1>(acc, partials, counter, &total)) {
    if (threadIdx.x == 0) {
      const double ve = total / vol_sum - prm.vol_frac;
      st->vol_error = ve;
      st->steps = st->it + 1;
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
  }
}

__global__ void k_gather_d(int64_t n, const int32_t* __restrict__ idx,
                           const double* __restrict__ x, double* __restrict__ y) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[idx[i]];
}

__global__ void k_scatter_d(int64_t n, const int32_t* __restrict__ idx,
                            const double* __restrict__ x, double* __restrict__ y) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[idx[i]] = x[i];
}

// out[i] = x[design[i]] + c * y[design[i]]  (y may be null)
__global__ void k_gather_axpy(int64_t nd, const int32_t* __restrict__ design,
                              const double* __restrict__ x, const double* __restrict__ y,
                              double c, double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = design[i];
    out[i] = y ? x[e] + c * y[e] : x[e];
  }
}

// sum_i x[design[i]] * w[i]  (deterministic)
__global__ void k_design_wsum(int64_t nd, const int32_t* __restrict__ design,
                              const double* __restrict__ x, const double* __restrict__ w,
                              double* partials, unsigned* counter, double* out) {
  TOPT_KERNEL_COUNT();
  double acc[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x)
    acc[0] += x[design[i]] * w[i];
  __shared__ double sh[32];
  block_sum<double, 1>(acc, sh);
  grid_finish<double, 1>(acc, partials, counter, out);
}

// max over interior design elements (rho_min+1e-6 < rho[d] < rho_max-1e-6)
// of c*|w[i]| (logmoc.py:227-236 KKT of the scaled Lagrangian gradient)
__global__ void k_design_kkt_w(int64_t nd, const int32_t* __restrict__ design,
                               const double* __restrict__ rho, const double* __restrict__ w,
                               double c, double rho_min, double rho_max, double* partials,
                               unsigned* counter, double* out) {
  TOPT_KERNEL_COUNT();
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double r = rho[design[i]];
    if (!(r > rho_min + 1e-6 && r < rho_max - 1e-6)) continue;
    const double a = fabs(w[i] * c);
    m = a > m ? a : m;
  }
  // NaN entries never win a comparison here (kept as in the serial maximum)
  grid_max_finish(m, false, partials, counter, out);
}

// lagrangian_log_update (logmoc.py:36-66) on the design elements:
// s = clip(dl*inv_scale, -clip, clip); x = log(clip(rho)); du = log(1 + m/exp(x));
// rho = clip(exp(clip(x - eta s, x - du, x + du)), rho_min, rho_max)
__global__ void k_logmoc_update(int64_t nd, const int32_t* __restrict__ design,
                                const double* __restrict__ dl, double inv_scale,
                                double* __restrict__ rho, double eta, double move,
                                double rho_min, double rho_max, double lclip,
                                double* __restrict__ scaling) {
  TOPT_KERNEL_COUNT();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = design[i];
    const double s = clip_nan2(dl[i] * inv_scale, -lclip, lclip);
    const double r = clip_nan2(rho[e], rho_min, rho_max);
    const double lr = log(r);
    const double du = log(1.0 + move / exp(lr));
    const double lo = lr - du;
    const double hi = lo + 2.0 * du;
    const double x = clip_nan2(log(r) - eta * s, lo, hi);
    rho[e] = clip_nan2(exp(x), rho_min, rho_max);
    if (scaling) scaling[i] = s;
  }
}

// --------------------------------------------------------------------------
// Radix select on |x| (non-negative doubles order like their bit patterns):
// histogram of one 11-bit digit among the entries matching the prefix.
__global__ void k_radix_hist(int64_t n, const int32_t* __restrict__ idx,
                             const double* __restrict__ x, unsigned long long prefix,
                             unsigned long long pmask, int shift, unsigned* __restrict__ hist) {
  TOPT_KERNEL_COUNT();
  __shared__ unsigned sh[2048];
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = fabs(idx ? x[idx[i]] : x[i]);
    const unsigned long long key = (unsigned long long)__double_as_longlong(v);
    if ((key & pmask) == prefix) atomicAdd(&sh[(key >> shift) & 2047ull], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2048; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// --------------------------------------------------------------------------
// Helmholtz transfers (helmholtz_filter_nodal.py:26-56):
// node value = sum_e vol_e val_e / sum_e vol_e over the incident elements,
// val_e = x_e for design elements and `fixed` for the others.
__global__ void k_elem_to_node(int64_t nn, const int32_t* __restrict__ nptr,
                               const int32_t* __restrict__ nel, const double* __restrict__ vol,
                               const double* __restrict__ x, const uint8_t* __restrict__ design,
                               double fixed, double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn;
       n += (int64_t)gridDim.x * blockDim.x) {
    double num = 0.0, den = 0.0;
    for (int32_t k = nptr[n]; k < nptr[n + 1]; ++k) {
      const int32_t e = nel[k];
      const double v = (!design || design[e]) ? x[e] : fixed;
      num += vol[e] * v;
      den += vol[e];
    }
    out[n] = num / (den == 0.0 ? 1.0 : den);
  }
}

// element value = mean of its node values; optionally min(., 0)
__global__ void k_node_to_elem(int64_t ne, int nloc, const int32_t* __restrict__ t,
                               const double* __restrict__ xn, int clamp_nonpos,
                               double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int a = 0; a < nloc; ++a) s += xn[t[(int64_t)a * ne + e]];
    const double v = s / (double)nloc;
    out[e] = clamp_nonpos ? fmin(v, 0.0) : v;
  }
}

static int design_grid(const topt_filter* f) { return grid_for(f->n_design, kFB, f->sm * 8); }

// percentile scratch (one per process, per device)
struct PctScratch {
  DevBuf hist;
  int dev = -1;
};
static PctScratch g_pct;
static std::mutex g_pct_mu;

static int select_kth_abs(int64_t n, const int32_t* idx, const double* x, int64_t k,
                          cudaStream_t s, double* out) {
  int dev = 0;
  TOPT_CUDA(cudaGetDevice(&dev));
  if (!g_pct.hist.p || g_pct.dev != dev) {
    int rc = g_pct.hist.alloc(2048 * sizeof(unsigned));
    if (rc) return rc;
    g_pct.dev = dev;
  }
  unsigned long long prefix = 0ull, pmask = 0ull;
  std::vector<unsigned> h(2048);
  const int shifts[6] = {53, 42, 31, 20, 9, 0};
  const int g = grid_for(n, kFB, device_sm_count() * 8);
  for (int pass = 0; pass < 6; ++pass) {
    // 11-bit digits at bits [sh, sh+11); the last one overlaps bits 9-10,
    // which the prefix already fixes, so its scan simply finds them set
    const int sh = shifts[pass];
    const unsigned long long digit_mask = 0x7FFull;
    TOPT_CUDA(cudaMemsetAsync(g_pct.hist.p, 0, 2048 * sizeof(unsigned), s));
    k_radix_hist<<<g, kFB, 0, s>>>(n, idx, x, prefix, pmask, sh, g_pct.hist.as<unsigned>());
    TOPT_CHECK_LAUNCH("k_radix_hist");
    TOPT_CUDA(cudaMemcpyAsync(h.data(), g_pct.hist.p, 2048 * sizeof(unsigned),
                              cudaMemcpyDeviceToHost, s));
    TOPT_CUDA(cudaStreamSynchronize(s));
    int64_t cum = 0;
    int d = 0;
    for (; d <= (int)digit_mask; ++d) {
      if (cum + h[d] > (uint64_t)k) break;
      cum += h[d];
    }
    if (d > (int)digit_mask) return fail(TOPT_NONFINITE, "percentile: selection failed");
    k -= cum;
    prefix |= ((unsigned long long)d) << sh;
    pmask |= digit_mask << sh;
  }
  double v;
  std::memcpy(&v, &prefix, sizeof(v));
  *out = v;
  return TOPT_OK;
}

}  // namespace topt

using namespace topt;

extern "C" {

int topt_filter_identity_create(int64_t n_elem, const uint8_t* design_mask, topt_filter** out) {
  if (!out || n_elem <= 0) return fail(TOPT_BAD_INPUT, "identity_create: bad argument");
  *out = nullptr;
  std::unique_ptr<topt_filter> f(new (std::nothrow) topt_filter());
  if (!f) return fail(TOPT_NO_MEMORY, "identity_create: host allocation");
  f->n_elem = n_elem;
  f->sm = device_sm_count();
  std::vector<int32_t> design, nondesign;
  for (int64_t i = 0; i < n_elem; ++i) {
    if (!design_mask || design_mask[i]) design.push_back((int32_t)i);
    else nondesign.push_back((int32_t)i);
  }
  if (design.empty()) return fail(TOPT_BAD_INPUT, "identity_create: empty design set");
  const int64_t nd = (int64_t)design.size();
  f->n_design = nd;
  f->nnz = nd;
  f->n_nondesign = (int64_t)nondesign.size();
  f->h_rowptr.resize(nd + 1);
  f->h_colind.resize(nd);
  f->h_vals.assign(nd, 1.0);
  for (int64_t i = 0; i <= nd; ++i) f->h_rowptr[i] = (int32_t)i;
  for (int64_t i = 0; i < nd; ++i) f->h_colind[i] = (int32_t)i;
  int rc;
  cudaStream_t s = nullptr;
  if ((rc = upload(f->design, design.data(), design.size(), s))) return rc;
  if ((rc = upload(f->nondesign, nondesign.data(), nondesign.size(), s))) return rc;
  if ((rc = upload(f->rowptr, f->h_rowptr.data(), f->h_rowptr.size(), s))) return rc;
  if ((rc = upload(f->colfull, design.data(), design.size(), s))) return rc;
  if ((rc = upload(f->vals, f->h_vals.data(), f->h_vals.size(), s))) return rc;
  if ((rc = upload(f->t_rowptr, f->h_rowptr.data(), f->h_rowptr.size(), s))) return rc;
  if ((rc = upload(f->t_colfull, design.data(), design.size(), s))) return rc;
  if ((rc = upload(f->t_vals, f->h_vals.data(), f->h_vals.size(), s))) return rc;
  if ((rc = f->cand.alloc(sizeof(double) * n_elem))) return rc;
  if ((rc = f->state.alloc(sizeof(OcState)))) return rc;
  if ((rc = f->partials.alloc(sizeof(double) * f->sm * 16 * 2))) return rc;
  if ((rc = f->counter.alloc(16 * sizeof(unsigned)))) return rc;
  TOPT_CUDA(cudaMemset(f->counter.p, 0, 16 * sizeof(unsigned)));
  TOPT_CUDA(cudaDeviceSynchronize());
  *out = f.release();
  return TOPT_OK;
}

int topt_oc_begin(topt_filter* f, const double* rho, const topt_oc_params* prm) {
  if (!f || !rho || !prm) return fail(TOPT_BAD_INPUT, "oc_begin: null argument");
  if (!(prm->l1 < prm->l2)) return fail(TOPT_BAD_INPUT, "oc_begin: need l1 < l2");
  int rc;
  if (!f->rho_e.p && (rc = f->rho_e.alloc(sizeof(double) * f->n_design))) return rc;
  if (!f->rho_new.p && (rc = f->rho_new.alloc(sizeof(double) * f->n_design))) return rc;
  OcState s0{};
  s0.l1 = prm->l1;
  s0.l2 = prm->l2;
  s0.lmid = 0.5 * (prm->l1 + prm->l2);
  TOPT_CUDA(cudaMemcpyAsync(f->state.p, &s0, sizeof(s0), cudaMemcpyHostToDevice, f->stream));
  k_gather_d<<<design_grid(f), kFB, 0, f->stream>>>(f->n_design, f->design.as<int32_t>(), rho,
                                                    f->rho_e.as<double>());
  TOPT_CHECK_LAUNCH("oc_begin");
  return TOPT_OK;
}

int topt_oc_candidate(topt_filter* f, const double* dc, double dc_scale,
                      const topt_oc_params* prm, double* cand, double* scaling) {
  if (!f || !dc || !prm || !cand) return fail(TOPT_BAD_INPUT, "oc_candidate: null argument");
  if (!(dc_scale > 0.0)) return fail(TOPT_BAD_INPUT, "oc_candidate: dc_scale must be > 0");
  k_oc_cand_step<<<design_grid(f), kFB, 0, f->stream>>>(
      f->n_design, f->design.as<int32_t>(), dc, dc_scale, f->rho_e.as<double>(),
      f->state.as<OcState>(), *prm, cand, f->rho_new.as<double>(), scaling);
  TOPT_CHECK_LAUNCH("oc_candidate");
  return TOPT_OK;
}

int topt_oc_volume(topt_filter* f, const double* filtered, const double* vol, double vol_sum,
                   const topt_oc_params* prm, int32_t* done, double* lmid, double* vol_error,
                   int32_t* steps) {
  if (!f || !filtered || !vol || !prm) return fail(TOPT_BAD_INPUT, "oc_volume: null argument");
  const double tbe = std::tanh(prm->beta * prm->beta_eta);
  const double den = tbe + std::tanh(prm->beta * (1.0 - prm->beta_eta)) + 1e-12;
  k_oc_vol_step<<<design_grid(f), kFB, 0, f->stream>>>(
      f->n_design, f->design.as<int32_t>(), filtered, vol, vol_sum, *prm, tbe, den,
      f->state.as<OcState>(), f->partials.as<double>(), f->counter.as<unsigned>() + 2);
  TOPT_CHECK_LAUNCH("oc_volume");
  OcState st{};
  TOPT_CUDA(cudaMemcpyAsync(&st, f->state.p, sizeof(st), cudaMemcpyDeviceToHost, f->stream));
  TOPT_CUDA(cudaStreamSynchronize(f->stream));
  if (done) *done = st.done;
  if (lmid) *lmid = st.lmid;
  if (vol_error) *vol_error = st.vol_error;
  if (steps) *steps = st.steps;
  return TOPT_OK;
}

int topt_oc_finish(topt_filter* f, double* rho) {
  if (!f || !rho) return fail(TOPT_BAD_INPUT, "oc_finish: null argument");
  k_scatter_d<<<design_grid(f), kFB, 0, f->stream>>>(f->n_design, f->design.as<int32_t>(),
                                                     f->rho_new.as<double>(), rho);
  TOPT_CHECK_LAUNCH("oc_finish");
  return TOPT_OK;
}

int topt_design_gather_axpy(topt_filter* f, const double* x, const double* y, double c,
                            double* out) {
  if (!f || !x || !out) return fail(TOPT_BAD_INPUT, "design_gather_axpy: null argument");
  k_gather_axpy<<<design_grid(f), kFB, 0, f->stream>>>(f->n_design, f->design.as<int32_t>(), x,
                                                       y, c, out);
  TOPT_CHECK_LAUNCH("k_gather_axpy");
  return TOPT_OK;
}

int topt_design_wsum(topt_filter* f, const double* x, const double* w, double* out) {
  if (!f || !x || !w || !out) return fail(TOPT_BAD_INPUT, "design_wsum: null argument");
  double* res = f->partials.as<double>() + f->sm * 16 * 2 - 2;
  k_design_wsum<<<design_grid(f), kFB, 0, f->stream>>>(f->n_design, f->design.as<int32_t>(), x,
                                                       w, f->partials.as<double>(),
                                                       f->counter.as<unsigned>() + 3, res);
  TOPT_CHECK_LAUNCH("k_design_wsum");
  TOPT_CUDA(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, f->stream));
  TOPT_CUDA(cudaStreamSynchronize(f->stream));
  return TOPT_OK;
}

int topt_design_kkt(topt_filter* f, const double* rho, const double* w, double c,
                    double rho_min, double rho_max, double* out) {
  if (!f || !rho || !w || !out) return fail(TOPT_BAD_INPUT, "design_kkt: null argument");
  double* res = f->partials.as<double>() + f->sm * 16 * 2 - 3;
  k_design_kkt_w<<<design_grid(f), kFB, 0, f->stream>>>(
      f->n_design, f->design.as<int32_t>(), rho, w, c, rho_min, rho_max,
      f->partials.as<double>(), f->counter.as<unsigned>() + 4, res);
  TOPT_CHECK_LAUNCH("k_design_kkt_w");
  TOPT_CUDA(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, f->stream));
  TOPT_CUDA(cudaStreamSynchronize(f->stream));
  return TOPT_OK;
}

int topt_logmoc_update(topt_filter* f, const double* dl, double inv_scale, double* rho,
                       double eta, double move_limit, double rho_min, double rho_max,
                       double lagrangian_clip, double* scaling) {
  if (!f || !dl || !rho) return fail(TOPT_BAD_INPUT, "logmoc_update: null argument");
  k_logmoc_update<<<design_grid(f), kFB, 0, f->stream>>>(
      f->n_design, f->design.as<int32_t>(), dl, inv_scale, rho, eta, move_limit, rho_min,
      rho_max, lagrangian_clip, scaling);
  TOPT_CHECK_LAUNCH("k_logmoc_update");
  return TOPT_OK;
}

int topt_percentile_abs(int64_t n, const int32_t* idx, const double* x, double q,
                        double* out, void* stream) {
  if (!out || n <= 0 || !x || !(q >= 0.0 && q <= 100.0))
    return fail(TOPT_BAD_INPUT, "percentile_abs: bad argument");
  std::lock_guard<std::mutex> lk(g_pct_mu);
  cudaStream_t s = (cudaStream_t)stream;
  // numpy 'linear' method: virtual index (n-1) q/100, lerp of the neighbours
  const double vi = (double)(n - 1) * (q / 100.0);
  const int64_t k0 = (int64_t)std::floor(vi);
  const int64_t k1 = std::min<int64_t>(k0 + 1, n - 1);
  const double t = vi - (double)k0;
  double a = 0.0, b = 0.0;
  int rc = select_kth_abs(n, idx, x, k0, s, &a);
  if (rc) return rc;
  if (k1 != k0) {
    if ((rc = select_kth_abs(n, idx, x, k1, s, &b))) return rc;
  } else {
    b = a;
  }
  const double diff = b - a;
  *out = (t >= 0.5) ? b - diff * (1.0 - t) : a + diff * t;
  return TOPT_OK;
}

int topt_elem_to_node(int64_t n_nodes, const int32_t* node_ptr, const int32_t* node_elems,
                      const double* vol, const double* x, const uint8_t* design,
                      double fixed_value, double* out, void* stream) {
  if (n_nodes <= 0 || !node_ptr || !node_elems || !vol || !x || !out)
    return fail(TOPT_BAD_INPUT, "elem_to_node: bad argument");
  k_elem_to_node<<<grid_for(n_nodes, kFB, device_sm_count() * 16), kFB, 0,
                   (cudaStream_t)stream>>>(n_nodes, node_ptr, node_elems, vol, x, design,
                                           fixed_value, out);
  TOPT_CHECK_LAUNCH("k_elem_to_node");
  return TOPT_OK;
}

int topt_node_to_elem(int64_t n_elem, int32_t nloc, const int32_t* t, const double* x_node,
                      int32_t clamp_nonpositive, double* out, void* stream) {
  if (n_elem <= 0 || nloc <= 0 || !t || !x_node || !out)
    return fail(TOPT_BAD_INPUT, "node_to_elem: bad argument");
  k_node_to_elem<<<grid_for(n_elem, kFB, device_sm_count() * 16), kFB, 0,
                   (cudaStream_t)stream>>>(n_elem, nloc, t, x_node, clamp_nonpositive, out);
  TOPT_CHECK_LAUNCH("k_node_to_elem");
  return TOPT_OK;
}

}  // extern "C"

namespace topt {
int launches_design(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}
}  // namespace topt
