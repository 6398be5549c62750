// Smoothed-aggregation multigrid of meshes without a logical grid: the
// hierarchy set-up (aggregates and the patterns of P, A P and P^T A P, built
// once per mesh by the kernels of amg_kernels.cuh), the values of every
// refresh, the transfers of the V-cycle, and the inspection entry points.
#include "amg_kernels.cuh"
#include "fem_state.cuh"

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

namespace topt {

// ---------------------------------------------------------------- smoothed aggregation
// Exclusive prefix sums of n int32 counts into out[0..n] (out[n] = total);
// the total is also returned on the host.
static int scan_counts(topt_fem* h, int64_t n, const int32_t* in, int64_t* out,
                       int64_t* total) {
  const int64_t ntiles = std::max<int64_t>(1, (n + kScanTile - 1) / kScanTile);
  DevBuf tiles;
  int rc = tiles.alloc(sizeof(int64_t) * ntiles);
  if (rc) return rc;
  cudaStream_t s = h->stream;
  k_scan_tiles<<<(int)ntiles, kScanThreads, 0, s>>>(n, in, tiles.as<int64_t>());
  k_scan_tile_sums<<<1, kScanThreads, 0, s>>>(ntiles, tiles.as<int64_t>(), out + n);
  k_scan_apply<<<(int)ntiles, kScanThreads, 0, s>>>(n, in, tiles.as<int64_t>(), out);
  TOPT_CHECK_LAUNCH("scan");
  TOPT_CUDA(cudaMemcpyAsync(total, out + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  TOPT_CUDA(cudaStreamSynchronize(s));
  return TOPT_OK;
}

// SELL storage of a block pattern given as CSR (sorted columns, diagonal
// present in every row); c2s[k] = SELL position of CSR entry k.
static int sell_from_csr(LevelStruct& L, int64_t n, const std::vector<int64_t>& rp,
                         const std::vector<int32_t>& cols, std::vector<int32_t>& c2s,
                         cudaStream_t s) {
  L.n_nodes = n;
  L.n_elem = 0;
  L.nnzb = rp[n];
  const int64_t nsl = (n + 31) / 32;
  std::vector<int32_t> gos(nsl + 1, 0), rowlen(n);
  for (int64_t sl = 0; sl < nsl; ++sl) {
    int32_t mx = 0;
    for (int64_t r = sl * 32; r < std::min<int64_t>(n, sl * 32 + 32); ++r) {
      rowlen[r] = (int32_t)(rp[r + 1] - rp[r]);
      mx = std::max(mx, rowlen[r]);
    }
    if ((int64_t)gos[sl] + mx >= (int64_t)INT32_MAX / 32)
      return fail(TOPT_BAD_INPUT, "amg: too many blocks for SELL storage");
    gos[sl + 1] = gos[sl] + mx;
  }
  const int64_t ngrp = gos[nsl];
  L.npos = ngrp * 32;
  std::vector<int32_t> sog(ngrp), col(L.npos), diag(n, -1);
  c2s.assign(rp[n], 0);
  for (int64_t sl = 0; sl < nsl; ++sl)
    for (int32_t g = gos[sl]; g < gos[sl + 1]; ++g) sog[g] = (int32_t)sl;
  for (int64_t sl = 0; sl < nsl; ++sl)
    for (int lane = 0; lane < 32; ++lane) {
      const int64_t r = sl * 32 + lane;
      for (int32_t g = gos[sl]; g < gos[sl + 1]; ++g) {
        const int64_t pos = (int64_t)g * 32 + lane;
        const int32_t j = g - gos[sl];
        if (r < n && j < rowlen[r]) {
          const int64_t k = rp[r] + j;
          col[pos] = cols[k];
          c2s[k] = (int32_t)pos;
          if (cols[k] == r) diag[r] = (int32_t)pos;
        } else {
          col[pos] = r < n ? (int32_t)r : 0;
        }
      }
    }
  for (int64_t i = 0; i < n; ++i)
    if (diag[i] < 0) return fail(TOPT_BAD_INPUT, "amg: coarse row without a diagonal block");
  int rc;
  if ((rc = upload(L.grp_of_slice, gos.data(), gos.size(), s))) return rc;
  if ((rc = upload(L.slice_of_grp, sog.data(), sog.size(), s))) return rc;
  if ((rc = upload(L.col, col.data(), col.size(), s))) return rc;
  if ((rc = upload(L.rowlen, rowlen.data(), rowlen.size(), s))) return rc;
  if ((rc = upload(L.diagpos, diag.data(), diag.size(), s))) return rc;
  TOPT_CUDA(cudaStreamSynchronize(s));
  L.sell.nrows = n;
  L.sell.grp_of_slice = L.grp_of_slice.as<int32_t>();
  L.sell.slice_of_grp = L.slice_of_grp.as<int32_t>();
  L.sell.col = L.col.as<int32_t>();
  L.sell.rowlen = L.rowlen.as<int32_t>();
  L.sell.diag = L.diagpos.as<int32_t>();
  return TOPT_OK;
}

// One symbolic product kind: counts, scans, then the fill pass.  Returns
// the output blocks' row pointer (rows + 1) in u_off and the number of
// output blocks / candidates.
template <int KIND>
static int symbolic(topt_fem* h, SymArgs a, DevBuf& u_off, DevBuf& col, DevBuf* row,
                    DevBuf& first, DevBuf& pay_a, DevBuf* pay_b, DevBuf& err, int64_t* nu,
                    int64_t* nc) {
  const int64_t n = a.nrows;
  DevBuf nuniq, ncand, c_off;
  int rc;
  if ((rc = nuniq.alloc(sizeof(int32_t) * n)) || (rc = ncand.alloc(sizeof(int32_t) * n)) ||
      (rc = u_off.alloc(sizeof(int64_t) * (n + 1))) ||
      (rc = c_off.alloc(sizeof(int64_t) * (n + 1))))
    return rc;
  a.nuniq = nuniq.as<int32_t>();
  a.ncand = ncand.as<int32_t>();
  a.err = err.as<int>();
  const int grid = (int)std::min<int64_t>(std::max<int64_t>(n, 1), (int64_t)h->sm * 2);
  TOPT_CUDA(cudaFuncSetAttribute(k_sym<KIND, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kSymSmem));
  TOPT_CUDA(cudaFuncSetAttribute(k_sym<KIND, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kSymSmem));
  k_sym<KIND, 0><<<grid, kSymThreads, kSymSmem, h->stream>>>(a);
  TOPT_CHECK_LAUNCH("k_sym count");
  int e = 0;
  TOPT_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  if (e) return fail(TOPT_BAD_INPUT, "amg: a row of a Galerkin product has more candidate "
                                     "blocks than the symbolic kernel holds");
  if ((rc = scan_counts(h, n, a.nuniq, u_off.as<int64_t>(), nu))) return rc;
  if ((rc = scan_counts(h, n, a.ncand, c_off.as<int64_t>(), nc))) return rc;
  if ((rc = col.alloc(sizeof(int32_t) * *nu)) || (rc = first.alloc(sizeof(int64_t) * (*nu + 1))) ||
      (rc = pay_a.alloc(sizeof(int32_t) * *nc)))
    return rc;
  if (row && (rc = row->alloc(sizeof(int32_t) * *nu))) return rc;
  if (pay_b && (rc = pay_b->alloc(sizeof(int32_t) * *nc))) return rc;
  a.u_off = u_off.as<int64_t>();
  a.c_off = c_off.as<int64_t>();
  a.out_col = col.as<int32_t>();
  a.out_row = row ? row->as<int32_t>() : nullptr;
  a.out_first = first.as<int64_t>();
  a.pay_a = pay_a.as<int32_t>();
  a.pay_b = pay_b ? pay_b->as<int32_t>() : nullptr;
  k_sym<KIND, 1><<<grid, kSymThreads, kSymSmem, h->stream>>>(a);
  TOPT_CHECK_LAUNCH("k_sym fill");
  // first[nu] = number of candidates
  TOPT_CUDA(cudaMemcpyAsync(first.as<int64_t>() + *nu, c_off.as<int64_t>() + n, sizeof(int64_t),
                            cudaMemcpyDeviceToDevice, h->stream));
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

// The smoothed-aggregation hierarchy of a mesh without a logical grid: all
// patterns (aggregates, P, R = P^T, A P, the coarse operators), built once
// on the GPU from the level-0 block pattern; values come with every refresh.
int setup_amg(topt_fem* h) {
  const int bs = h->bs;
  cudaStream_t s = h->stream;
  int rc;
  DevBuf err;
  if ((rc = err.alloc(sizeof(int)))) return rc;
  TOPT_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  {
    LevelStruct& L0 = h->ls[0];
    if ((rc = L0.cnt.alloc(sizeof(int32_t) * h->n_dof))) return rc;
    k_free_counts<<<gridsize(h, h->n_dof), kBlock, 0, s>>>(h->n_dof, h->mask.as<uint8_t>(),
                                                         L0.cnt.as<int32_t>());
    TOPT_CHECK_LAUNCH("k_free_counts");
  }
  while ((int)h->ls.size() < h->mg_levels) {
    const int li = (int)h->ls.size() - 1;
    const int64_t n = h->ls[li].n_nodes;
    if (n * bs <= h->mg_coarse_max) break;
    SellT sp = h->ls[li].sell;
    // 1. distance-2 maximal independent set (hashed priorities)
    DevBuf state, keys, m1, m2, left;
    if ((rc = state.alloc(n)) || (rc = keys.alloc(8 * n)) || (rc = m1.alloc(8 * n)) ||
        (rc = m2.alloc(8 * n)) || (rc = left.alloc(sizeof(int))))
      return rc;
    TOPT_CUDA(cudaMemsetAsync(state.p, kMisUndecided, n, s));
    int rounds = 0, left_h = 1;
    for (; rounds < 200 && left_h; ++rounds) {
      TOPT_CUDA(cudaMemsetAsync(left.p, 0, sizeof(int), s));
      k_mis_keys<<<gridsize(h, n), kBlock, 0, s>>>(n, state.as<uint8_t>(), keys.as<uint64_t>());
      k_mis_max<<<gridsize(h, n), kBlock, 0, s>>>(sp, keys.as<uint64_t>(), m1.as<uint64_t>());
      k_mis_max<<<gridsize(h, n), kBlock, 0, s>>>(sp, m1.as<uint64_t>(), m2.as<uint64_t>());
      k_mis_update<<<gridsize(h, n), kBlock, 0, s>>>(n, state.as<uint8_t>(), m2.as<uint64_t>(),
                                                    left.as<int>());
      TOPT_CHECK_LAUNCH("k_mis");
      TOPT_CUDA(cudaMemcpyAsync(&left_h, left.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      TOPT_CUDA(cudaStreamSynchronize(s));
    }
    if (left_h) return fail(TOPT_BAD_INPUT, "amg: independent set did not converge");
    // 2. aggregates: roots numbered in node order
    DevBuf is_root, root_id, agg1;
    if ((rc = is_root.alloc(sizeof(int32_t) * n)) || (rc = root_id.alloc(8 * (n + 1))) ||
        (rc = agg1.alloc(sizeof(int32_t) * n)))
      return rc;
    k_mis_roots<<<gridsize(h, n), kBlock, 0, s>>>(n, state.as<uint8_t>(), is_root.as<int32_t>());
    int64_t nagg = 0;
    if ((rc = scan_counts(h, n, is_root.as<int32_t>(), root_id.as<int64_t>(), &nagg))) return rc;
    if (nagg <= 0 || (double)nagg > 0.85 * (double)n) break;   // coarsening stalled
    LevelStruct& F = h->ls[li];
    if ((rc = F.agg.alloc(sizeof(int32_t) * n))) return rc;
    k_agg_first<<<gridsize(h, n), kBlock, 0, s>>>(sp, state.as<uint8_t>(),
                                                  root_id.as<int64_t>(), agg1.as<int32_t>());
    k_agg_second<<<gridsize(h, n), kBlock, 0, s>>>(sp, agg1.as<int32_t>(), F.agg.as<int32_t>(),
                                                   err.as<int>());
    TOPT_CHECK_LAUNCH("k_agg");
    {
      int e = 0;
      TOPT_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      TOPT_CUDA(cudaStreamSynchronize(s));
      if (e) return fail(TOPT_BAD_INPUT, "amg: aggregation left a node without an aggregate");
    }
    LevelStruct C;
    if ((rc = C.cnt.alloc(sizeof(int32_t) * nagg * bs))) return rc;
    TOPT_CUDA(cudaMemsetAsync(C.cnt.p, 0, sizeof(int32_t) * nagg * bs, s));
    if (bs == 3)
      k_agg_counts<3><<<gridsize(h, n), kBlock, 0, s>>>(n, F.agg.as<int32_t>(),
                                                        F.cnt.as<int32_t>(), C.cnt.as<int32_t>());
    else
      k_agg_counts<1><<<gridsize(h, n), kBlock, 0, s>>>(n, F.agg.as<int32_t>(),
                                                        F.cnt.as<int32_t>(), C.cnt.as<int32_t>());
    TOPT_CHECK_LAUNCH("k_agg_counts");
    // 3. P pattern (one block per distinct neighbouring aggregate)
    SymArgs a{};
    a.nrows = n;
    a.a = sp;
    a.agg = F.agg.as<int32_t>();
    int64_t ncp = 0;
    if ((rc = symbolic<kSymP>(h, a, F.p_ptr, F.p_col, &F.p_row, F.p_first, F.p_pos, nullptr, err,
                              &F.np, &ncp)))
      return rc;
    // 4. R = P^T pattern, fine nodes in order
    {
      DevBuf rc_cnt, cursor;
      if ((rc = rc_cnt.alloc(sizeof(int32_t) * nagg)) || (rc = cursor.alloc(sizeof(int32_t) * nagg)) ||
          (rc = F.r_ptr.alloc(8 * (nagg + 1))) || (rc = F.r_fine.alloc(sizeof(int32_t) * F.np)) ||
          (rc = F.r_pent.alloc(sizeof(int32_t) * F.np)))
        return rc;
      TOPT_CUDA(cudaMemsetAsync(rc_cnt.p, 0, sizeof(int32_t) * nagg, s));
      TOPT_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * nagg, s));
      k_rt_count<<<gridsize(h, F.np), kBlock, 0, s>>>(F.np, F.p_col.as<int32_t>(),
                                                      rc_cnt.as<int32_t>());
      int64_t nr = 0;
      if ((rc = scan_counts(h, nagg, rc_cnt.as<int32_t>(), F.r_ptr.as<int64_t>(), &nr))) return rc;
      k_rt_fill<<<gridsize(h, F.np), kBlock, 0, s>>>(F.np, F.p_col.as<int32_t>(),
                                                     F.p_row.as<int32_t>(), F.r_ptr.as<int64_t>(),
                                                     cursor.as<int32_t>(), F.r_fine.as<int32_t>(),
                                                     F.r_pent.as<int32_t>());
      k_rt_sort<<<gridsize(h, nagg), kBlock, 0, s>>>(nagg, F.r_ptr.as<int64_t>(),
                                                     F.r_fine.as<int32_t>(), F.r_pent.as<int32_t>());
      TOPT_CHECK_LAUNCH("k_rt");
    }
    // 5. A P pattern
    a.p_ptr = F.p_ptr.as<int64_t>();
    a.p_col = F.p_col.as<int32_t>();
    int64_t napq = 0;
    if ((rc = symbolic<kSymAP>(h, a, F.ap_ptr, F.ap_col, nullptr, F.ap_first, F.ap_pos,
                               &F.ap_pent, err, &F.nap, &napq)))
      return rc;
    // 6. coarse operator pattern P^T (A P)
    SymArgs c{};
    c.nrows = nagg;
    c.r_ptr = F.r_ptr.as<int64_t>();
    c.r_fine = F.r_fine.as<int32_t>();
    c.r_pent = F.r_pent.as<int32_t>();
    c.ap_ptr = F.ap_ptr.as<int64_t>();
    c.ap_col = F.ap_col.as<int32_t>();
    DevBuf c_rp, c_col;
    int64_t ncq = 0;
    if ((rc = symbolic<kSymRAP>(h, c, c_rp, c_col, nullptr, F.c_first, F.c_pent, &F.c_apent, err,
                                &F.nc_ent, &ncq)))
      return rc;
    // 7. the coarse level in SELL storage
    std::vector<int64_t> rp(nagg + 1);
    std::vector<int32_t> cols(F.nc_ent), c2s;
    TOPT_CUDA(cudaMemcpyAsync(rp.data(), c_rp.p, 8 * (nagg + 1), cudaMemcpyDeviceToHost, s));
    TOPT_CUDA(cudaMemcpyAsync(cols.data(), c_col.p, sizeof(int32_t) * F.nc_ent,
                              cudaMemcpyDeviceToHost, s));
    TOPT_CUDA(cudaStreamSynchronize(s));
    try {
      if ((rc = sell_from_csr(C, nagg, rp, cols, c2s, s))) return rc;
    } catch (const std::bad_alloc&) {
      return fail(TOPT_NO_MEMORY, "amg: host allocation");
    }
    if ((rc = upload(F.c_pos, c2s.data(), c2s.size(), s))) return rc;
    F.amg = true;
    h->ls.push_back(std::move(C));
  }
  if (h->ls.size() > 1) {
    LevelStruct& B = h->ls.back();
    const int64_t nd_b = B.n_nodes * bs;
    if (nd_b > 4096)
      return fail(TOPT_BAD_INPUT, "amg: coarsest level too large for a dense solve; raise "
                                  "mg_levels");
    B.dense = true;
    B.ndense = (int)nd_b;
  }
  TOPT_CUDA(cudaStreamSynchronize(s));
  return TOPT_OK;
}

template <typename T, int BS>
static void amg_products(topt_fem* h, LevelStruct& F, LevelStruct& C, const T* vals,
                         const T* dinv, T sc, T* pv, T* apv, T* vals_c) {
  cudaStream_t s = h->stream;
  k_amg_p<T, BS><<<gridsize(h, F.np), kBlock, 0, s>>>(
      F.np, F.sell, vals, dinv, F.agg.as<int32_t>(), F.cnt.as<int32_t>(), C.cnt.as<int32_t>(),
      F.p_row.as<int32_t>(), F.p_col.as<int32_t>(), F.p_first.as<int64_t>(),
      F.p_pos.as<int32_t>(), sc, pv);
  k_amg_ap<T, BS><<<gridsize(h, F.nap), kBlock, 0, s>>>(F.nap, vals, pv,
                                                        F.ap_first.as<int64_t>(),
                                                        F.ap_pos.as<int32_t>(),
                                                        F.ap_pent.as<int32_t>(), apv);
  k_amg_rap<T, BS><<<gridsize(h, F.nc_ent), kBlock, 0, s>>>(
      F.nc_ent, pv, apv, F.c_first.as<int64_t>(), F.c_pent.as<int32_t>(),
      F.c_apent.as<int32_t>(), F.c_pos.as<int32_t>(), vals_c);
}

// FP32 hierarchy of a mixed handle: the products in FP64 from the level's
// FP64 operator (level 0: the refinement operator), rounded to FP32.
static int amg_galerkin_mixed(topt_fem* h, int li, Hier<float>& H) {
  LevelStruct& F = h->ls[li];
  LevelStruct& C = h->ls[li + 1];
  const int bs = h->bs;
  cudaStream_t s = h->stream;
  const double* A = li == 0 ? h->vals64_0.as<double>() : F.a64_vals.as<double>();
  const double sc = (4.0 / 3.0) / H.lv[li].lmax;
  if (bs == 3) {
    k_block_diag_inv<double, 3><<<gridsize(h, F.n_nodes), kBlock, 0, s>>>(
        F.sell, A, F.a64_dinv.as<double>());
    amg_products<double, 3>(h, F, C, A, F.a64_dinv.as<double>(), sc, F.a64_pv.as<double>(),
                            F.a64_apv.as<double>(), C.a64_vals.as<double>());
    k_fix_zero_diag<double, 3><<<gridsize(h, C.n_nodes), kBlock, 0, s>>>(
        C.sell, C.a64_vals.as<double>());
  } else {
    k_block_diag_inv<double, 1><<<gridsize(h, F.n_nodes), kBlock, 0, s>>>(
        F.sell, A, F.a64_dinv.as<double>());
    amg_products<double, 1>(h, F, C, A, F.a64_dinv.as<double>(), sc, F.a64_pv.as<double>(),
                            F.a64_apv.as<double>(), C.a64_vals.as<double>());
    k_fix_zero_diag<double, 1><<<gridsize(h, C.n_nodes), kBlock, 0, s>>>(
        C.sell, C.a64_vals.as<double>());
  }
  const int64_t nv = C.npos * bs * bs, np = F.np * bs * bs;
  k_convert<float, double><<<gridsize(h, nv), kBlock, 0, s>>>(nv, C.a64_vals.as<double>(),
                                                             H.lv[li + 1].vals.as<float>());
  k_convert<float, double><<<gridsize(h, np), kBlock, 0, s>>>(np, F.a64_pv.as<double>(),
                                                             H.lv[li].pv.as<float>());
  TOPT_CHECK_LAUNCH("amg galerkin (FP64 products)");
  return TOPT_OK;
}

// Values of the smoothed-aggregation transfer of level li and of level
// li + 1: P (needs Dinv and lambda_max of level li), A P, P^T A P.
template <typename T>
int amg_galerkin(topt_fem* h, int li, Hier<T>& H) {
  if constexpr (std::is_same<T, float>::value) {
    if (h->mixed) return amg_galerkin_mixed(h, li, H);
  }
  LevelStruct& F = h->ls[li];
  LevelStruct& C = h->ls[li + 1];
  LevelNum<T>& N = H.lv[li];
  const T sc = (T)((4.0 / 3.0) / N.lmax);
  if (h->bs == 3)
    amg_products<T, 3>(h, F, C, N.vals.template as<T>(), N.dinv.template as<T>(), sc,
                       N.pv.template as<T>(), N.apv.template as<T>(),
                       H.lv[li + 1].vals.template as<T>());
  else
    amg_products<T, 1>(h, F, C, N.vals.template as<T>(), N.dinv.template as<T>(), sc,
                       N.pv.template as<T>(), N.apv.template as<T>(),
                       H.lv[li + 1].vals.template as<T>());
  TOPT_CHECK_LAUNCH("amg galerkin");
  return TOPT_OK;
}

template <typename T>
static int amg_export_t(topt_fem* h, Hier<T>& H, int level, int32_t* agg, double* lmax,
                        int64_t* p_ptr, int32_t* p_col, double* p_vals, double* coarse) {
  const LevelStruct& F = h->ls[level];
  const LevelStruct& C = h->ls[level + 1];
  const int bs = h->bs;
  cudaStream_t s = h->stream;
  if (!H.built) return fail(TOPT_BAD_INPUT, "amg_export: hierarchy of this precision not built");
  *lmax = H.lv[level].lmax;
  TOPT_CUDA(cudaMemcpyAsync(agg, F.agg.p, sizeof(int32_t) * F.n_nodes, cudaMemcpyDeviceToHost, s));
  TOPT_CUDA(cudaMemcpyAsync(p_ptr, F.p_ptr.p, sizeof(int64_t) * (F.n_nodes + 1),
                            cudaMemcpyDeviceToHost, s));
  TOPT_CUDA(cudaMemcpyAsync(p_col, F.p_col.p, sizeof(int32_t) * F.np, cudaMemcpyDeviceToHost, s));
  const size_t npv = (size_t)F.np * bs * bs;
  std::vector<T> pv(npv);
  TOPT_CUDA(cudaMemcpyAsync(pv.data(), H.lv[level].pv.p, sizeof(T) * npv, cudaMemcpyDeviceToHost,
                            s));
  const int64_t nd = C.n_nodes * bs;
  DevBuf dense;
  int rc;
  if ((rc = dense.alloc(sizeof(double) * nd * nd))) return rc;
  TOPT_CUDA(cudaMemsetAsync(dense.p, 0, sizeof(double) * nd * nd, s));
  if (bs == 3)
    k_sell_to_dense<T, 3><<<gridsize(h, C.npos), kBlock, 0, s>>>(
        C.npos, C.sell, H.lv[level + 1].vals.template as<T>(), (int)nd, dense.as<double>());
  else
    k_sell_to_dense<T, 1><<<gridsize(h, C.npos), kBlock, 0, s>>>(
        C.npos, C.sell, H.lv[level + 1].vals.template as<T>(), (int)nd, dense.as<double>());
  TOPT_CHECK_LAUNCH("k_sell_to_dense");
  TOPT_CUDA(cudaMemcpyAsync(coarse, dense.p, sizeof(double) * nd * nd, cudaMemcpyDeviceToHost, s));
  TOPT_CUDA(cudaStreamSynchronize(s));
  for (size_t i = 0; i < npv; ++i) p_vals[i] = (double)pv[i];
  return TOPT_OK;
}

// bc = P^T r of level li's residual (fine DOFs flagged in mask excluded),
// with the coarse level's first Chebyshev step when dinv_c is given.
template <typename T>
int amg_restrict(topt_fem* h, int li, Hier<T>& H, int L, const uint8_t* mask, const T* dinv_c,
                 T c2c) {
  const LevelStruct& Ls = h->ls[li];
  const LevelStruct& Cs = h->ls[li + 1];
  LevelNum<T>& N = H.lv[li];
  LevelNum<T>& C = H.lv[li + 1];
  const int bs = h->bs;
  TOPT_BSL_DISPATCH(bs, L, (k_amg_restrict<T, BS_, L_><<<gridsize(h, Cs.n_nodes), kBlock, 0,
                                                         h->stream>>>(
                               Cs.n_nodes, Ls.r_ptr.as<int64_t>(), Ls.r_fine.as<int32_t>(),
                               Ls.r_pent.as<int32_t>(), N.pv.template as<T>(), mask,
                               N.r.template as<T>(), C.b.template as<T>(), dinv_c,
                               C.d.template as<T>(), C.x.template as<T>(), c2c)));
  TOPT_CHECK_LAUNCH("k_amg_restrict");
  return TOPT_OK;
}

// x += P x_c of level li (fine DOFs flagged in mask untouched).
template <typename T>
int amg_prolong(topt_fem* h, int li, Hier<T>& H, int L, const uint8_t* mask, T* x) {
  const LevelStruct& Ls = h->ls[li];
  LevelNum<T>& N = H.lv[li];
  LevelNum<T>& C = H.lv[li + 1];
  const int bs = h->bs;
  TOPT_BSL_DISPATCH(bs, L, (k_amg_prolong_add<T, BS_, L_><<<gridsize(h, Ls.n_nodes), kBlock, 0,
                                                            h->stream>>>(
                               Ls.n_nodes, Ls.p_ptr.as<int64_t>(), Ls.p_col.as<int32_t>(),
                               N.pv.template as<T>(), mask, C.x.template as<T>(), x)));
  TOPT_CHECK_LAUNCH("k_amg_prolong_add");
  return TOPT_OK;
}

#define TOPT_AMG_INST(T)                                                                  \
  template int amg_galerkin<T>(topt_fem*, int, Hier<T>&);                                 \
  template int amg_restrict<T>(topt_fem*, int, Hier<T>&, int, const uint8_t*, const T*, T); \
  template int amg_prolong<T>(topt_fem*, int, Hier<T>&, int, const uint8_t*, T*);
TOPT_AMG_INST(float)
TOPT_AMG_INST(double)
#undef TOPT_AMG_INST

int launches_amg(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}

}  // namespace topt

using namespace topt;

extern "C" {

int topt_fem_amg_sizes(const topt_fem* h, int32_t level, int64_t* n_fine, int64_t* n_coarse,
                       int64_t* n_p) {
  if (!h || !n_fine || !n_coarse || !n_p) return fail(TOPT_BAD_INPUT, "amg_sizes: null argument");
  if (level < 0 || level + 1 >= (int)h->ls.size() || !h->ls[level].amg)
    return fail(TOPT_BAD_INPUT, "amg_sizes: no smoothed-aggregation transfer at this level");
  *n_fine = h->ls[level].n_nodes;
  *n_coarse = h->ls[level + 1].n_nodes;
  *n_p = h->ls[level].np;
  return TOPT_OK;
}

int topt_fem_amg_export(topt_fem* h, int32_t dtype, int32_t level, int32_t* agg, double* lmax,
                        int64_t* p_ptr, int32_t* p_col, double* p_vals, double* coarse) {
  int64_t nf, nc, np;
  int rc = topt_fem_amg_sizes(h, level, &nf, &nc, &np);
  if (rc) return rc;
  if (!agg || !lmax || !p_ptr || !p_col || !p_vals || !coarse)
    return fail(TOPT_BAD_INPUT, "amg_export: null argument");
  if (nc * h->bs > 8192) return fail(TOPT_BAD_INPUT, "amg_export: coarse level too large");
  if (dtype == 1) return amg_export_t<double>(h, h->h64, level, agg, lmax, p_ptr, p_col, p_vals,
                                              coarse);
  if (dtype == 0 && h->mixed)
    return amg_export_t<float>(h, h->h32, level, agg, lmax, p_ptr, p_col, p_vals, coarse);
  return fail(TOPT_BAD_INPUT, "amg_export: dtype must be 1 (FP64) or 0 (FP32, mixed handles)");
}

}  // extern "C"
