// FEM handle: pattern, assembly, multigrid hierarchy and the PCG drivers.
//
// Replaces the state solve of FEM_SimpLinearElasticity /
// FEM_SimpLinearHeatConduction (sktopt/fea/solver_elastic.py:61-467,
// sktopt/fea/solver_heat.py:136-253): K(rho) is assembled into a pattern
// built once, Dirichlet DOFs are enforced symmetrically (skfem.enforce), and
// the system is solved by preconditioned CG, either in FP64 throughout or in
// FP32 inside an FP64 iterative-refinement loop.  The preconditioner is block
// Jacobi or a multigrid V-cycle (Chebyshev smoothing, dense coarsest solve):
// geometric on the logical cell grid (Galerkin coarse operators built element
// by element), or smoothed aggregation built on the GPU for meshes without a
// grid (amg_kernels.cuh).
#include "fem_state.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <type_traits>
#include <vector>

namespace topt {

// ---------------------------------------------------------------- patterns
static int upload_pattern(LevelStruct& L, int64_t n_nodes, int64_t n_elem, int nloc,
                          const int32_t* t, cudaStream_t s) {
  topt_pattern* P = nullptr;
  int rc = topt_pattern_build(n_nodes, n_elem, nloc, t, &P);
  if (rc) return rc;
  std::unique_ptr<topt_pattern, void (*)(topt_pattern*)> guard(P, topt_pattern_free);
  topt_pattern_view v = view_of(P);
  L.n_nodes = n_nodes;
  L.n_elem = n_elem;
  L.nloc = nloc;
  L.nnzb = v.nnzb;
  // slices of 32 block rows, padded to the longest row of the slice
  const int64_t nsl = (n_nodes + 31) / 32;
  std::vector<int32_t> gos(nsl + 1, 0), rowlen(n_nodes);
  for (int64_t sl = 0; sl < nsl; ++sl) {
    int32_t mx = 0;
    for (int64_t r = sl * 32; r < std::min<int64_t>(n_nodes, sl * 32 + 32); ++r) {
      rowlen[r] = v.rowptr[r + 1] - v.rowptr[r];
      mx = std::max(mx, rowlen[r]);
    }
    if ((int64_t)gos[sl] + mx >= (int64_t)INT32_MAX / 32)
      return fail(TOPT_BAD_INPUT, "pattern: too many blocks for SELL storage");
    gos[sl + 1] = gos[sl] + mx;
  }
  const int64_t ngrp = gos[nsl];
  const int64_t npos = ngrp * 32;
  L.npos = npos;
  std::vector<int32_t> sog(ngrp), col(npos), diag(n_nodes, -1), c2s(v.nnzb);
  std::vector<int64_t> cnt(npos + 1, 0);
  for (int64_t sl = 0; sl < nsl; ++sl)
    for (int32_t g = gos[sl]; g < gos[sl + 1]; ++g) sog[g] = (int32_t)sl;
  for (int64_t sl = 0; sl < nsl; ++sl)
    for (int lane = 0; lane < 32; ++lane) {
      const int64_t r = sl * 32 + lane;
      for (int32_t g = gos[sl]; g < gos[sl + 1]; ++g) {
        const int64_t pos = (int64_t)g * 32 + lane;
        const int32_t j = g - gos[sl];
        if (r < n_nodes && j < rowlen[r]) {
          const int64_t k = v.rowptr[r] + j;
          col[pos] = v.colind[k];
          c2s[k] = (int32_t)pos;
          cnt[pos + 1] = v.cptr[k + 1] - v.cptr[k];
          if (v.colind[k] == r) diag[r] = (int32_t)pos;
        } else {
          col[pos] = r < n_nodes ? (int32_t)r : 0;
        }
      }
    }
  for (int64_t i = 0; i < n_nodes; ++i)
    if (diag[i] < 0) return fail(TOPT_BAD_INPUT, "pattern: node without element");
  for (int64_t q = 0; q < npos; ++q) cnt[q + 1] += cnt[q];
  std::vector<int32_t> contrib(v.ncontrib);
  for (int64_t k = 0; k < v.nnzb; ++k) {
    const int64_t dst = cnt[c2s[k]];
    std::copy(v.contrib + v.cptr[k], v.contrib + v.cptr[k + 1], contrib.begin() + dst);
  }
  if ((rc = upload(L.grp_of_slice, gos.data(), gos.size(), s))) return rc;
  if ((rc = upload(L.slice_of_grp, sog.data(), sog.size(), s))) return rc;
  if ((rc = upload(L.col, col.data(), col.size(), s))) return rc;
  if ((rc = upload(L.rowlen, rowlen.data(), rowlen.size(), s))) return rc;
  if ((rc = upload(L.diagpos, diag.data(), diag.size(), s))) return rc;
  if ((rc = upload(L.cptr, cnt.data(), cnt.size(), s))) return rc;
  if ((rc = upload(L.contrib, contrib.data(), contrib.size(), s))) return rc;
  if ((rc = upload(L.csr2sell, c2s.data(), c2s.size(), s))) return rc;
  if ((rc = upload(L.t, t, (size_t)nloc * n_elem, s))) return rc;
  TOPT_CUDA(cudaStreamSynchronize(s));
  L.sell.nrows = n_nodes;
  L.sell.grp_of_slice = L.grp_of_slice.as<int32_t>();
  L.sell.slice_of_grp = L.slice_of_grp.as<int32_t>();
  L.sell.col = L.col.as<int32_t>();
  L.sell.rowlen = L.rowlen.as<int32_t>();
  L.sell.diag = L.diagpos.as<int32_t>();
  return TOPT_OK;
}

// connectivity of a structured hex grid (MeshHex local order)
static std::vector<int32_t> hex_grid_t(int nx, int ny, int nz) {
  static const int off[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 0, 0}, {0, 0, 1},
                                {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 1}};
  const int64_t ne = (int64_t)nx * ny * nz;
  std::vector<int32_t> t(8 * ne);
  for (int ez = 0; ez < nz; ++ez)
    for (int ex = 0; ex < nx; ++ex)
      for (int ey = 0; ey < ny; ++ey) {
        const int64_t e = ey + (int64_t)ny * (ex + (int64_t)nx * ez);
        for (int a = 0; a < 8; ++a) {
          const int64_t n = (ey + off[a][1]) + (int64_t)(ny + 1) *
                            ((ex + off[a][0]) + (int64_t)(nx + 1) * (ez + off[a][2]));
          t[a * ne + e] = (int32_t)n;
        }
      }
  return t;
}

static std::vector<int32_t> coarse_map(int n) {
  const int nc = (n + 1) / 2;  // coarse cells
  std::vector<int32_t> cm(nc + 1);
  for (int i = 0; i <= nc; ++i) cm[i] = std::min(2 * i, n);
  return cm;
}

static int make_transfer(LevelStruct& F, const LevelStruct& Cs, cudaStream_t s) {
  std::vector<int32_t> cm[3] = {coarse_map(F.nx), coarse_map(F.ny), coarse_map(F.nz)};
  int nf[3] = {F.nx, F.ny, F.nz};
  std::vector<int32_t> c0[3];
  std::vector<float> w1[3];
  for (int d = 0; d < 3; ++d) {
    const int nc = (int)cm[d].size() - 1;
    c0[d].resize(nf[d] + 1);
    w1[d].resize(nf[d] + 1);
    int i = 0;
    for (int f = 0; f <= nf[d]; ++f) {
      while (i + 1 < nc && cm[d][i + 1] <= f) ++i;
      c0[d][f] = i;
      w1[d][f] = (float)(f - cm[d][i]) / (float)(cm[d][i + 1] - cm[d][i]);
    }
  }
  int rc;
  if ((rc = upload(F.cmx, cm[0].data(), cm[0].size(), s))) return rc;
  if ((rc = upload(F.cmy, cm[1].data(), cm[1].size(), s))) return rc;
  if ((rc = upload(F.cmz, cm[2].data(), cm[2].size(), s))) return rc;
  if ((rc = upload(F.c0x, c0[0].data(), c0[0].size(), s))) return rc;
  if ((rc = upload(F.c0y, c0[1].data(), c0[1].size(), s))) return rc;
  if ((rc = upload(F.c0z, c0[2].data(), c0[2].size(), s))) return rc;
  if ((rc = upload(F.w1x, w1[0].data(), w1[0].size(), s))) return rc;
  if ((rc = upload(F.w1y, w1[1].data(), w1[1].size(), s))) return rc;
  if ((rc = upload(F.w1z, w1[2].data(), w1[2].size(), s))) return rc;
  TOPT_CUDA(cudaStreamSynchronize(s));
  GridT& g = F.grid;
  g.nfx = F.nx; g.nfy = F.ny; g.nfz = F.nz;
  g.ncx = Cs.nx; g.ncy = Cs.ny; g.ncz = Cs.nz;
  g.cmx = F.cmx.as<int32_t>(); g.cmy = F.cmy.as<int32_t>(); g.cmz = F.cmz.as<int32_t>();
  g.c0x = F.c0x.as<int32_t>(); g.c0y = F.c0y.as<int32_t>(); g.c0z = F.c0z.as<int32_t>();
  g.w1x = F.w1x.as<float>(); g.w1y = F.w1y.as<float>(); g.w1z = F.w1z.as<float>();
  // restriction tables: coarse node i gathers fine nodes r0[i] + k, k < 3,
  // with the hat weights of its interpolation (P^T row)
  std::vector<int32_t> r0[3];
  std::vector<float> rw[3];
  for (int d = 0; d < 3; ++d) {
    const std::vector<int32_t>& c = cm[d];
    const int nc = (int)c.size() - 1;
    r0[d].resize(nc + 1);
    rw[d].assign(3 * (nc + 1), 0.0f);
    for (int i = 0; i <= nc; ++i) {
      const int f0 = i > 0 ? c[i - 1] + 1 : 0;
      const int f1 = i < nc ? c[i + 1] - 1 : nf[d];
      r0[d][i] = f0;
      for (int f = f0; f <= f1 && f - f0 < 3; ++f) {
        double w;
        if (f == c[i]) w = 1.0;
        else if (f < c[i]) w = (double)(f - c[i - 1]) / (double)(c[i] - c[i - 1]);
        else w = (double)(c[i + 1] - f) / (double)(c[i + 1] - c[i]);
        rw[d][3 * i + (f - f0)] = (float)w;
      }
    }
  }
  if ((rc = upload(F.r0x, r0[0].data(), r0[0].size(), s))) return rc;
  if ((rc = upload(F.r0y, r0[1].data(), r0[1].size(), s))) return rc;
  if ((rc = upload(F.r0z, r0[2].data(), r0[2].size(), s))) return rc;
  if ((rc = upload(F.rwx, rw[0].data(), rw[0].size(), s))) return rc;
  if ((rc = upload(F.rwy, rw[1].data(), rw[1].size(), s))) return rc;
  if ((rc = upload(F.rwz, rw[2].data(), rw[2].size(), s))) return rc;
  TOPT_CUDA(cudaStreamSynchronize(s));
  g.r0x = F.r0x.as<int32_t>(); g.r0y = F.r0y.as<int32_t>(); g.r0z = F.r0z.as<int32_t>();
  g.rwx = F.rwx.as<float>(); g.rwy = F.rwy.as<float>(); g.rwz = F.rwz.as<float>();
  return TOPT_OK;
}

// ---------------------------------------------------------------- dispatch helpers
template <typename T, int BS, int NLOC>
static int launch_assemble(topt_fem* h, const LevelStruct& L, const T* ke, int64_t ke_stride,
                           const T* coef, const T* extra, const uint8_t* mask, T* vals) {
  const size_t sh = ke_stride == 0 ? sizeof(T) * BS * NLOC * BS * NLOC : 0;
  k_assemble<T, BS, NLOC><<<gridsize(h, L.npos), kBlock, sh, h->stream>>>(
      L.npos, L.sell, L.cptr.as<int64_t>(), L.contrib.as<int32_t>(), ke, ke_stride, coef, extra,
      mask, vals);
  TOPT_CHECK_LAUNCH("k_assemble");
  return TOPT_OK;
}

template <typename T>
static int assemble(topt_fem* h, const LevelStruct& L, int bs, int nloc, const T* ke,
                    int64_t ke_stride, const T* coef, const T* extra, const uint8_t* mask,
                    T* vals) {
  if (bs == 3 && nloc == 8)
    return launch_assemble<T, 3, 8>(h, L, ke, ke_stride, coef, extra, mask, vals);
  if (bs == 3 && nloc == 4)
    return launch_assemble<T, 3, 4>(h, L, ke, ke_stride, coef, extra, mask, vals);
  if (bs == 1 && nloc == 8)
    return launch_assemble<T, 1, 8>(h, L, ke, ke_stride, coef, extra, mask, vals);
  if (bs == 1 && nloc == 4)
    return launch_assemble<T, 1, 4>(h, L, ke, ke_stride, coef, extra, mask, vals);
  return fail(TOPT_BAD_INPUT, "assemble: unsupported bs/nloc");
}

template <typename T>
static int dot(topt_fem* h, int64_t n, int L, const T* x, const T* y, int slot) {
  TOPT_L_DISPATCH(L, (k_dot<T, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                          n, x, y, h->red.partials.as<double>(), h->red.ctr(slot),
                          h->red.res(slot))));
  TOPT_CHECK_LAUNCH("k_dot");
  return TOPT_OK;
}

static int read_slot(topt_fem* h, int slot, int L, double* out) {
  TOPT_CUDA(cudaMemcpyAsync(out, h->red.res(slot), L * sizeof(double),
                            cudaMemcpyDeviceToHost, h->stream));
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

// ---------------------------------------------------------------- hierarchy
template <typename T>
static const T* level0_ke(topt_fem* h) {
  return std::is_same<T, double>::value ? (const T*)h->ke64.p : (const T*)h->ke32.p;
}
template <typename T>
static const T* level0_coef(topt_fem* h) {
  return std::is_same<T, double>::value ? (const T*)h->coef64.p : (const T*)h->coef32.p;
}
template <typename T>
static const T* level0_extra(topt_fem* h) {
  if (!h->extra64) return nullptr;
  return std::is_same<T, double>::value ? (const T*)h->extra64 : (const T*)h->extra32.p;
}

template <typename T>
static int alloc_level_num(topt_fem* h, LevelNum<T>& N, const LevelStruct& L, int li) {
  const int bs = h->bs;
  int rc;
  const int64_t nd = L.n_nodes * bs;
  if (li > 0 && (rc = N.ke.alloc(sizeof(T) * L.n_elem * 64 * bs * bs))) return rc;
  const bool mf0 = std::is_same<T, float>::value && h->mf && li == 0;
  if (!mf0 && (rc = N.vals.alloc(sizeof(T) * L.npos * bs * bs))) return rc;
  if ((rc = N.dinv.alloc(sizeof(T) * L.n_nodes * bs * bs))) return rc;
  for (DevBuf* b : {&N.b, &N.x, &N.r, &N.d, &N.q})
    if ((rc = b->alloc(sizeof(T) * nd * 4))) return rc;
  if (!L.dense && (rc = N.pw.alloc(sizeof(T) * nd))) return rc;
  if (L.dense) {
    if ((rc = N.dense_inv.alloc(sizeof(T) * (size_t)L.ndense * L.ndense))) return rc;
  }
  const bool amg64 = std::is_same<T, float>::value && h->mixed;
  if (L.amg) {
    if ((rc = N.pv.alloc(sizeof(T) * L.np * bs * bs))) return rc;
    if (!amg64 && (rc = N.apv.alloc(sizeof(T) * L.nap * bs * bs))) return rc;
  }
  if (amg64 && L.amg) {
    LevelStruct& W = h->ls[li];
    if ((rc = W.a64_dinv.alloc(sizeof(double) * L.n_nodes * bs * bs))) return rc;
    if ((rc = W.a64_pv.alloc(sizeof(double) * L.np * bs * bs))) return rc;
    if ((rc = W.a64_apv.alloc(sizeof(double) * L.nap * bs * bs))) return rc;
  }
  if (li > 0 && h->ls[li - 1].amg) {   // SELL padding blocks stay zero
    TOPT_CUDA(cudaMemsetAsync(N.vals.p, 0, N.vals.bytes, h->stream));
    if (amg64) {
      LevelStruct& W = h->ls[li];
      if ((rc = W.a64_vals.alloc(sizeof(double) * L.npos * bs * bs))) return rc;
      TOPT_CUDA(cudaMemsetAsync(W.a64_vals.p, 0, W.a64_vals.bytes, h->stream));
    }
  }
  return TOPT_OK;
}

template <typename T>
static int galerkin(topt_fem* h, int li, Hier<T>& H) {
  LevelStruct& F = h->ls[li];
  const bool lvl0 = (li == 0);
  const int bs = h->bs;
  const T* ke = lvl0 ? level0_ke<T>(h) : H.lv[li].ke.template as<T>();
  const int64_t stride = lvl0 ? (h->n_ke == 1 ? 0 : (int64_t)(bs * h->nloc) * (bs * h->nloc))
                              : (int64_t)(bs * 8) * (bs * 8);
  const T* coef = lvl0 ? level0_coef<T>(h) : nullptr;
  const T* extra = lvl0 ? level0_extra<T>(h) : nullptr;
  const uint8_t* mask = lvl0 ? h->mask.as<uint8_t>() : nullptr;
  const int32_t* cptr = (lvl0 && F.cell_ptr.p) ? F.cell_ptr.as<int32_t>() : nullptr;
  const int32_t* cel = (lvl0 && F.cell_ptr.p) ? F.cell_elems.as<int32_t>() : nullptr;
  const int nloc = lvl0 ? h->nloc : 8;
  int64_t ncells = (int64_t)F.grid.ncx * F.grid.ncy * F.grid.ncz;
  T* out = H.lv[li + 1].ke.template as<T>();
  const int32_t* list = nullptr;
  if (lvl0 && F.gal_shared && !extra) {
    const T* M = std::is_same<T, double>::value ? (const T*)F.gal_M64.p : (const T*)F.gal_M32.p;
    const int g = (int)std::min<int64_t>(ncells, (int64_t)h->sm * 32);
    if (bs == 3)
      k_galerkin_shared<T, 3><<<g, 192, 0, h->stream>>>(F.grid, F.gal_masked.as<uint8_t>(), M,
                                                        coef, out);
    else
      k_galerkin_shared<T, 1><<<g, 192, 0, h->stream>>>(F.grid, F.gal_masked.as<uint8_t>(), M,
                                                        coef, out);
    TOPT_CHECK_LAUNCH("k_galerkin_shared");
    ncells = F.n_gal_list;
    list = F.gal_list.as<int32_t>();
    if (ncells == 0) return TOPT_OK;
  }
  if (bs == 3 && nloc == 8)
    k_galerkin<T, 3, 8><<<ncells, 256, 0, h->stream>>>(F.grid, list, cptr, cel,
                                                       F.t.as<int32_t>(), F.n_elem, ke, stride,
                                                       coef, extra, mask, out);
  else if (bs == 3 && nloc == 4)
    k_galerkin<T, 3, 4><<<ncells, 256, 0, h->stream>>>(F.grid, list, cptr, cel,
                                                       F.t.as<int32_t>(), F.n_elem, ke, stride,
                                                       coef, extra, mask, out);
  else if (bs == 1 && nloc == 8)
    k_galerkin<T, 1, 8><<<ncells, 256, 0, h->stream>>>(F.grid, list, cptr, cel,
                                                       F.t.as<int32_t>(), F.n_elem, ke, stride,
                                                       coef, extra, mask, out);
  else
    k_galerkin<T, 1, 4><<<ncells, 256, 0, h->stream>>>(F.grid, list, cptr, cel,
                                                       F.t.as<int32_t>(), F.n_elem, ke, stride,
                                                       coef, extra, mask, out);
  TOPT_CHECK_LAUNCH("k_galerkin");
  return TOPT_OK;
}

// Precompute M[pattern][child] = P^T K0 P for the shared-matrix fast path and
// the list of coarse cells whose interpolation is masked by fixed DOFs.
static int setup_shared_galerkin(topt_fem* h, const double* ke, const uint8_t* mask_h) {
  LevelStruct& F = h->ls[0];
  const int bs = h->bs, NC = bs * 8, NN = NC * NC;
  static const int off[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 0, 0}, {0, 0, 1},
                                {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 1}};
  std::vector<double> M((size_t)64 * NN, 0.0);
  for (int pat = 0; pat < 8; ++pat) {
    const int e[3] = {1 + (pat & 1), 1 + ((pat >> 1) & 1), 1 + (pat >> 2)};
    for (int ch = 0; ch < 8; ++ch) {
      const int o[3] = {ch & 1, (ch >> 1) & 1, ch >> 2};
      if (o[0] >= e[0] || o[1] >= e[1] || o[2] >= e[2]) continue;
      double W[8][8];
      for (int a = 0; a < 8; ++a)
        for (int k = 0; k < 8; ++k) {
          double w = 1.0;
          for (int d = 0; d < 3; ++d) {
            const double xi = (double)(o[d] + off[a][d]) / (double)e[d];
            w *= off[k][d] ? xi : 1.0 - xi;
          }
          W[a][k] = w;
        }
      // M = P^T K0 P, P[(a,c),(k,c)] = W[a][k]
      double* out = M.data() + ((size_t)pat * 8 + ch) * NN;
      const int ND = bs * 8;
      std::vector<double> T((size_t)ND * NC, 0.0);
      for (int row = 0; row < ND; ++row)
        for (int l = 0; l < 8; ++l)
          for (int d = 0; d < bs; ++d) {
            double sacc = 0.0;
            for (int b = 0; b < 8; ++b) sacc += ke[row * ND + b * bs + d] * W[b][l];
            T[(size_t)row * NC + l * bs + d] = sacc;
          }
      for (int k = 0; k < 8; ++k)
        for (int c = 0; c < bs; ++c)
          for (int col = 0; col < NC; ++col) {
            double sacc = 0.0;
            for (int a = 0; a < 8; ++a) sacc += W[a][k] * T[(size_t)(a * bs + c) * NC + col];
            out[(size_t)(k * bs + c) * NC + col] = sacc;
          }
    }
  }
  // masked coarse cells: any fixed DOF on the closure of their fine cells
  const GridT& g = F.grid;
  std::vector<int32_t> cmx(g.ncx + 1), cmy(g.ncy + 1), cmz(g.ncz + 1);
  for (int i = 0; i <= g.ncx; ++i) cmx[i] = std::min(2 * i, g.nfx);
  for (int i = 0; i <= g.ncy; ++i) cmy[i] = std::min(2 * i, g.nfy);
  for (int i = 0; i <= g.ncz; ++i) cmz[i] = std::min(2 * i, g.nfz);
  const int64_t ncells = (int64_t)g.ncx * g.ncy * g.ncz;
  std::vector<uint8_t> masked(ncells, 0);
  std::vector<int32_t> list;
  const int64_t fny = g.nfy + 1, fnx = g.nfx + 1;
  for (int cz = 0; cz < g.ncz; ++cz)
    for (int cx = 0; cx < g.ncx; ++cx)
      for (int cy = 0; cy < g.ncy; ++cy) {
        bool m = false;
        for (int fz = cmz[cz]; fz <= cmz[cz + 1] && !m; ++fz)
          for (int fx = cmx[cx]; fx <= cmx[cx + 1] && !m; ++fx)
            for (int fy = cmy[cy]; fy <= cmy[cy + 1] && !m; ++fy) {
              const int64_t n = fy + fny * (fx + fnx * (int64_t)fz);
              for (int c = 0; c < bs; ++c) m = m || mask_h[n * bs + c];
            }
        const int64_t C = cy + (int64_t)g.ncy * (cx + (int64_t)g.ncx * cz);
        if (m) {
          masked[C] = 1;
          list.push_back((int32_t)C);
        }
      }
  int rc;
  cudaStream_t s = nullptr;
  if ((rc = upload(F.gal_M64, M.data(), M.size(), s))) return rc;
  std::vector<float> M32(M.begin(), M.end());
  if ((rc = upload(F.gal_M32, M32.data(), M32.size(), s))) return rc;
  if ((rc = upload(F.gal_masked, masked.data(), masked.size(), s))) return rc;
  if ((rc = upload(F.gal_list, list.data(), list.size(), s))) return rc;
  TOPT_CUDA(cudaStreamSynchronize(s));
  F.n_gal_list = (int64_t)list.size();
  F.gal_shared = true;
  return TOPT_OK;
}

template <typename T>
static int block_inv(topt_fem* h, const LevelStruct& L, const T* vals, T* dinv, bool fix) {
  if (h->bs == 3) {
    if (fix) k_fix_zero_diag<T, 3><<<gridsize(h, L.n_nodes), kBlock, 0, h->stream>>>(
        L.sell, (T*)vals);
    k_block_diag_inv<T, 3><<<gridsize(h, L.n_nodes), kBlock, 0, h->stream>>>(L.sell, vals, dinv);
  } else {
    if (fix) k_fix_zero_diag<T, 1><<<gridsize(h, L.n_nodes), kBlock, 0, h->stream>>>(
        L.sell, (T*)vals);
    k_block_diag_inv<T, 1><<<gridsize(h, L.n_nodes), kBlock, 0, h->stream>>>(L.sell, vals, dinv);
  }
  TOPT_CHECK_LAUNCH("k_block_diag_inv");
  return TOPT_OK;
}

// lambda_max(D^-1 A) by power iteration with a 1.1 safety factor.  The unit
// iterate is kept per level and warm-starts the next refresh of the same
// handle (the operator changes little between design updates): 10 steps on
// the first refresh, 4 afterwards.  No host round trip until the end.
template <typename T>
static int estimate_lmax(topt_fem* h, const LevelStruct& L, LevelNum<T>& N, double* out) {
  const int bs = h->bs;
  const int64_t nd = L.n_nodes * bs;
  T* v = N.pw.template as<T>();
  T* w = N.q.template as<T>();
  T* tmp = N.r.template as<T>();
  const int iters = N.pw_ready ? 4 : 10;
  if (!N.pw_ready) k_hash_fill<T><<<gridsize(h, nd), kBlock, 0, h->stream>>>(nd, v);
  int rc;
  for (int it = 0; it < iters; ++it) {
    if (it == iters - 1 && (rc = dot<T>(h, nd, 1, v, v, 1))) return rc;
    if ((rc = spmv<T>(h, L, bs, 1, 0, false, N.vals.template as<T>(), v, nullptr, tmp))) return rc;
    if (bs == 3)
      k_block_jacobi<T, 3, 1, false><<<gridsize(h, L.n_nodes), kBlock, 0, h->stream>>>(
          L.n_nodes, N.dinv.template as<T>(), tmp, w, nullptr, nullptr, nullptr);
    else
      k_block_jacobi<T, 1, 1, false><<<gridsize(h, L.n_nodes), kBlock, 0, h->stream>>>(
          L.n_nodes, N.dinv.template as<T>(), tmp, w, nullptr, nullptr, nullptr);
    if (it < iters - 1) k_convert<T, T><<<gridsize(h, nd), kBlock, 0, h->stream>>>(nd, w, v);
  }
  if ((rc = dot<T>(h, nd, 1, w, w, 11))) return rc;
  double nv = 0.0, nw = 0.0;
  if ((rc = read_slot(h, 1, 1, &nv))) return rc;
  if ((rc = read_slot(h, 11, 1, &nw))) return rc;
  const bool ok = nw > 0.0 && nv > 0.0 && std::isfinite(nw) && std::isfinite(nv);
  const double lam = ok ? std::sqrt(nw / nv) : 0.0;
  if (ok) {
    k_scale<T><<<gridsize(h, nd), kBlock, 0, h->stream>>>(nd, (T)(1.0 / std::sqrt(nw)), w, v);
    TOPT_CHECK_LAUNCH("k_scale");
  }
  N.pw_ready = ok;
  *out = lam > 0.0 ? 1.1 * lam : 2.0;
  return TOPT_OK;
}

// Dense inverse of the coarsest level, queued on stream s (no wait).
template <typename T>
static int build_dense(topt_fem* h, const LevelStruct& L, LevelNum<T>& N, DevBuf& scratch,
                       cudaStream_t s) {
  const int n = L.ndense;
  int rc;
  if (scratch.bytes < sizeof(double) * (size_t)n * n &&
      (rc = scratch.alloc(sizeof(double) * (size_t)n * n)))
    return rc;
  TOPT_CUDA(cudaMemsetAsync(scratch.p, 0, sizeof(double) * (size_t)n * n, s));
  if (h->bs == 3)
    k_sell_to_dense<T, 3><<<gridsize(h, L.npos), kBlock, 0, s>>>(
        L.npos, L.sell, N.vals.template as<T>(), n, scratch.as<double>());
  else
    k_sell_to_dense<T, 1><<<gridsize(h, L.npos), kBlock, 0, s>>>(
        L.npos, L.sell, N.vals.template as<T>(), n, scratch.as<double>());
  k_gauss_jordan_inverse<<<1, 1024, 0, s>>>(n, scratch.as<double>());
  k_dense_copy<T><<<gridsize(h, (int64_t)n * n), kBlock, 0, s>>>(
      (int64_t)n * n, scratch.as<double>(), N.dense_inv.template as<T>());
  TOPT_CHECK_LAUNCH("dense coarse");
  return TOPT_OK;
}

// Chebyshev smoothing (Saad, Iterative Methods, Alg. 12.1) on the interval
// [lmax/ratio, lmax] of Dinv A (ratio 30 by default).
struct ChebParams {
  double theta, delta, sigma;
  ChebParams(double lmax, double ratio) {
    const double lmin = lmax / ratio;
    theta = 0.5 * (lmax + lmin);
    delta = 0.5 * (lmax - lmin);
    sigma = theta / delta;
  }
};

// Rebuild level values (level 0 from coef) and the hierarchy of precision T.
// The recorded V-cycles hold the operator values, Chebyshev bounds and
// launch shapes of the hierarchy they were recorded on.
static void vcycle_graphs_stale(topt_fem* h) {
  for (VcycleGraph& g : h->vcg) {
    g.valid = false;
    g.direct_done = false;
  }
}

static void vcycle_graphs_free(topt_fem* h) {
  for (VcycleGraph& g : h->vcg) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = VcycleGraph();
  }
}

template <typename T>
static int refresh(topt_fem* h, Hier<T>& H) {
  int rc;
  const int nlev = (int)h->ls.size();
  vcycle_graphs_stale(h);
  if (!H.built) {
    H.lv.resize(nlev);
    for (int li = 0; li < nlev; ++li)
      if ((rc = alloc_level_num<T>(h, H.lv[li], h->ls[li], li))) return rc;
    H.built = true;
  }
  const int bs = h->bs;
  const int64_t stride0 = h->n_ke == 1 ? 0 : (int64_t)(bs * h->nloc) * (bs * h->nloc);
  // level 0 operator (FP32 of a uniform hex grid: matrix-free, diagonal only)
  if (std::is_same<T, float>::value && h->mf) {
    k_mf_diag_inv<<<gridsize(h, h->n_nodes), kBlock, 0, h->stream>>>(
        h->mfg, h->ke32.as<float>(), h->coef32.as<float>(), h->mask.as<uint8_t>(),
        (float*)H.lv[0].dinv.p);
    TOPT_CHECK_LAUNCH("k_mf_diag_inv");
  } else {
    if ((rc = assemble<T>(h, h->ls[0], bs, h->nloc, level0_ke<T>(h), stride0,
                          level0_coef<T>(h), level0_extra<T>(h), h->mask.as<uint8_t>(),
                          H.lv[0].vals.template as<T>())))
      return rc;
    if ((rc = block_inv<T>(h, h->ls[0], H.lv[0].vals.template as<T>(),
                           H.lv[0].dinv.template as<T>(), false)))
      return rc;
  }
  DevBuf& scratch = H.dense_scratch;
  // every level's operator (each from the finer one) ...
  int dense_li = -1;
  for (int li = 0; li < nlev; ++li) {
    LevelStruct& L = h->ls[li];
    LevelNum<T>& N = H.lv[li];
    if (li > 0) {
      if (h->ls[li - 1].amg) {
        if ((rc = amg_galerkin<T>(h, li - 1, H))) return rc;
      } else {
        if ((rc = galerkin<T>(h, li - 1, H))) return rc;
        if ((rc = assemble<T>(h, L, bs, 8, N.ke.template as<T>(), (int64_t)(bs * 8) * (bs * 8),
                              nullptr, nullptr, nullptr, N.vals.template as<T>())))
          return rc;
      }
      if ((rc = block_inv<T>(h, L, N.vals.template as<T>(), N.dinv.template as<T>(), true)))
        return rc;
    }
    // the smoothed prolongator of this level needs its lambda_max first
    if (L.amg && (rc = estimate_lmax<T>(h, L, N, &N.lmax))) return rc;
    if (L.dense) dense_li = li;
  }
  // ... then the coarsest dense inverse (one CTA) on the side stream while
  // the power iterations of the other levels run on the handle's stream
  if (dense_li >= 0) {
    if (!h->aux) {
      TOPT_CUDA(cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking));
      TOPT_CUDA(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
      TOPT_CUDA(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    }
    TOPT_CUDA(cudaEventRecord(h->ev_fork, h->stream));
    TOPT_CUDA(cudaStreamWaitEvent(h->aux, h->ev_fork, 0));
    if ((rc = build_dense<T>(h, h->ls[dense_li], H.lv[dense_li], scratch, h->aux))) return rc;
    TOPT_CUDA(cudaEventRecord(h->ev_join, h->aux));
  }
  for (int li = 0; li < nlev; ++li) {
    if (li == dense_li || h->ls[li].amg) continue;
    LevelNum<T>& N = H.lv[li];
    if (nlev > 1) {
      if ((rc = estimate_lmax<T>(h, h->ls[li], N, &N.lmax))) return rc;
    } else {
      N.lmax = 0.0;
    }
  }
  if (dense_li >= 0) TOPT_CUDA(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
  return TOPT_OK;
}

// ---------------------------------------------------------------- V-cycle
// Chebyshev smoothing (ChebParams): every step after the first runs fused
// into the operator application that produces its residual (ChebEp); the
// search directions d ping-pong between N.d and N.q.

// Pre-smoothing from a zero guess.  On entry the first step is applied
// (N.d = x = Dinv b / theta, by the restriction or the V-cycle start); on
// exit N.r = b - A x.
template <typename T>
static int smooth_pre(topt_fem* h, int li, Hier<T>& H, int L, int degree, const T* b, T* x) {
  LevelStruct& Ls = h->ls[li];
  LevelNum<T>& N = H.lv[li];
  const ChebParams cp(N.lmax, h->cheb_ratio);
  double rho0 = 1.0 / cp.sigma;
  T* r = N.r.template as<T>();
  T* dA = N.d.template as<T>();
  T* dB = N.q.template as<T>();
  const T* vals = N.vals.template as<T>();
  int rc;
  ChebEp<T> ep;
  ep.dinv = N.dinv.template as<T>();
  ep.x = x;
  ep.kind = 2;
  for (int k = 1; k < degree; ++k) {
    const double rho1 = 1.0 / (2.0 * cp.sigma - rho0);
    ep.c1 = (T)(rho1 * rho0);
    ep.c2 = (T)(2.0 * rho1 / cp.delta);
    ep.dold = dA;
    ep.dnew = dB;
    // step 1: r = b - A d (x == d); later steps: r -= A d
    if ((rc = spmv<T>(h, Ls, h->bs, L, k == 1 ? 1 : 2, false, vals, dA, b, r, 0, ep, true)))
      return rc;
    std::swap(dA, dB);
    rho0 = rho1;
  }
  return spmv<T>(h, Ls, h->bs, L, degree == 1 ? 1 : 2, false, vals, dA, b, r, 0, ChebEp<T>(),
                 true);
}

// Post-smoothing of x (nonzero guess): r = b - A x fused with the first
// step d = Dinv r / theta, then degree-1 fused steps that update x.
template <typename T>
static int smooth_post(topt_fem* h, int li, Hier<T>& H, int L, int degree, const T* b, T* x) {
  LevelStruct& Ls = h->ls[li];
  LevelNum<T>& N = H.lv[li];
  const ChebParams cp(N.lmax, h->cheb_ratio);
  double rho0 = 1.0 / cp.sigma;
  T* r = N.r.template as<T>();
  T* dA = N.d.template as<T>();
  T* dB = N.q.template as<T>();
  const T* vals = N.vals.template as<T>();
  const int64_t nl = Ls.n_nodes * h->bs * L;
  int rc;
  ChebEp<T> ep;
  ep.dinv = N.dinv.template as<T>();
  ep.kind = 1;
  ep.c2 = (T)(1.0 / cp.theta);
  ep.dnew = dA;
  if ((rc = spmv<T>(h, Ls, h->bs, L, 1, false, vals, x, b, r, 0, ep, true))) return rc;
  if (degree == 1) {
    k_axpy<T><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, T(1), dA, x);
    TOPT_CHECK_LAUNCH("k_axpy");
    return TOPT_OK;
  }
  ep.kind = 2;
  ep.x = x;
  for (int k = 1; k < degree; ++k) {
    const double rho1 = 1.0 / (2.0 * cp.sigma - rho0);
    ep.c1 = (T)(rho1 * rho0);
    ep.c2 = (T)(2.0 * rho1 / cp.delta);
    ep.dold = dA;
    ep.dnew = dB;
    ep.add_old = (k == 1);
    if ((rc = spmv<T>(h, Ls, h->bs, L, 2, false, vals, dA, nullptr, r, 0, ep, true)))
      return rc;
    std::swap(dA, dB);
    rho0 = rho1;
  }
  return TOPT_OK;
}

// x ~= A_li^-1 b.  started: the first smoothing step is already applied
// (coarse levels: by the restriction that produced b).
template <typename T>
static int vcycle(topt_fem* h, int li, Hier<T>& H, int L, int degree, const T* b, T* x,
                  bool started) {
  LevelStruct& Ls = h->ls[li];
  LevelNum<T>& N = H.lv[li];
  const int bs = h->bs;
  int rc;
  if (Ls.dense) {
    const int n = Ls.ndense;
    TOPT_L_DISPATCH(L, (k_dense_matvec<T, L_><<<grid_for((int64_t)n * 32, 256), 256, 0,
                                                  h->stream>>>(n, N.dense_inv.template as<T>(),
                                                               b, x)));
    TOPT_CHECK_LAUNCH("k_dense_matvec");
    return TOPT_OK;
  }
  if (!started) {
    const ChebParams cp(N.lmax, h->cheb_ratio);
    if (std::is_same<T, float>::value && h->mf && li == 0 && L == 1) {
      // first step d = x = Dinv b / theta (the matrix-free level's kernel)
      ChebEp<float> ep;
      ep.kind = 3;
      ep.dinv = (const float*)N.dinv.p;
      ep.c2 = (float)(1.0 / cp.theta);
      ep.dnew = (float*)N.d.p;
      ep.x = (float*)x;
      k_cheb_stored<<<gridsize(h, Ls.n_nodes), kBlock, 0, h->stream>>>(Ls.n_nodes, ep,
                                                                      (const float*)b);
      TOPT_CHECK_LAUNCH("k_cheb_stored");
    } else {
      TOPT_BSL_DISPATCH(bs, L, (k_cheb<T, BS_, L_><<<gridsize(h, Ls.n_nodes), kBlock, 0,
                                                    h->stream>>>(
                                   Ls.n_nodes, N.dinv.template as<T>(), b, N.d.template as<T>(),
                                   x, T(0), (T)(1.0 / cp.theta), 1, 1)));
      TOPT_CHECK_LAUNCH("k_cheb");
    }
  }
  if ((rc = smooth_pre<T>(h, li, H, L, degree, b, x))) return rc;
  LevelNum<T>& C = H.lv[li + 1];
  const LevelStruct& Cs = h->ls[li + 1];
  const uint8_t* mask = li == 0 ? h->mask.as<uint8_t>() : nullptr;
  const T c2c = Cs.dense ? T(0) : (T)(1.0 / ChebParams(C.lmax, h->cheb_ratio).theta);
  const T* dinv_c = Cs.dense ? nullptr : C.dinv.template as<T>();
  if (Ls.amg) {
    if ((rc = amg_restrict<T>(h, li, H, L, mask, dinv_c, c2c))) return rc;
  } else {
    TOPT_BSL_DISPATCH(bs, L, (k_restrict<T, BS_, L_><<<gridsize(h, Cs.n_nodes), kBlock, 0,
                                                       h->stream>>>(
                                 Ls.grid, mask, N.r.template as<T>(), C.b.template as<T>(),
                                 dinv_c, C.d.template as<T>(), C.x.template as<T>(), c2c)));
    TOPT_CHECK_LAUNCH("k_restrict");
  }
  if ((rc = vcycle<T>(h, li + 1, H, L, degree, C.b.template as<T>(), C.x.template as<T>(), true)))
    return rc;
  if (Ls.amg) {
    if ((rc = amg_prolong<T>(h, li, H, L, mask, x))) return rc;
  } else {
    TOPT_BSL_DISPATCH(bs, L, (k_prolong_add<T, BS_, L_><<<gridsize(h, Ls.n_nodes), kBlock, 0,
                                                           h->stream>>>(
                                 Ls.grid, mask, C.x.template as<T>(), x)));
    TOPT_CHECK_LAUNCH("k_prolong_add");
  }
  return smooth_post<T>(h, li, H, L, degree, b, x);
}

// z = V-cycle(r).  After each refresh the first application for a given
// (precision, r, z, load cases, degree, interval) runs directly (it also sets
// the kernels' shared-memory attributes); the next one records the V-cycle
// on the private stream, and later ones replay the graph on the handle's
// stream: one launch instead of the 5 to 10 kernels per level.  Should a
// recording or an instantiation be refused, the handle stops recording and
// launches directly from then on (same kernels, same results).
template <typename T>
static int vcycle_apply(topt_fem* h, Hier<T>& H, int L, const T* r, T* z, int degree) {
  constexpr bool f32 = std::is_same<T, float>::value;
  if (!h->vc_graphs) return vcycle<T>(h, 0, H, L, degree, r, z, false);
  VcycleGraph* g = nullptr;
  for (VcycleGraph& c : h->vcg)
    if (c.r && c.fp32 == f32 && c.r == r && c.z == z && c.L == L && c.degree == degree &&
        c.cheb_ratio == h->cheb_ratio) {
      g = &c;
      break;
    }
  if (!g) {   // a free slot, else the least recently used one
    g = &h->vcg[0];
    for (VcycleGraph& c : h->vcg) {
      if (!c.r) { g = &c; break; }
      if (c.used < g->used) g = &c;
    }
    if (g->exec) cudaGraphExecDestroy(g->exec);
    *g = VcycleGraph();
    g->fp32 = f32; g->r = r; g->z = z; g->L = L; g->degree = degree;
    g->cheb_ratio = h->cheb_ratio;
  }
  g->used = ++h->vc_clock;
  if (!g->valid && !g->direct_done) {
    g->direct_done = true;
    return vcycle<T>(h, 0, H, L, degree, r, z, false);
  }
  if (!g->valid) {
    if (!h->cap) TOPT_CUDA(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking));
    TOPT_CUDA(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal));
    cudaStream_t user = h->stream;
    h->stream = h->cap;
    const int rc = vcycle<T>(h, 0, H, L, degree, r, z, false);
    h->stream = user;
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(h->cap, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    cudaError_t ei = ec;
    if (ec == cudaSuccess && g->exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(g->exec, graph, &info) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaGraphExecDestroy(g->exec);
        g->exec = nullptr;
      }
    }
    if (ec == cudaSuccess && !g->exec) ei = cudaGraphInstantiate(&g->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {   // recording refused: launch directly from now on
      (void)cudaGetLastError();
      g->exec = nullptr;
      vcycle_graphs_free(h);
      h->vc_graphs = false;
      return vcycle<T>(h, 0, H, L, degree, r, z, false);
    }
    g->valid = true;
  }
  TOPT_CUDA(cudaGraphLaunch(g->exec, h->stream));
  return TOPT_OK;
}

// ---------------------------------------------------------------- PCG
// z = M^-1 r (V-cycle or block Jacobi); r.z into reducer slot `slot` unless
// slot < 0.
template <typename T>
static int precond_apply(topt_fem* h, Hier<T>& H, int L, const T* r, T* z, int precond,
                         int degree, int slot) {
  LevelStruct& L0 = h->ls[0];
  LevelNum<T>& N0 = H.lv[0];
  const int bs = h->bs;
  if (precond == 1 && h->ls.size() > 1) {
    int rc2 = vcycle_apply<T>(h, H, L, r, z, degree);
    if (rc2) return rc2;
    return slot < 0 ? TOPT_OK : dot<T>(h, h->n_dof, L, r, z, slot);
  }
  if (slot < 0) {
    TOPT_BSL_DISPATCH(bs, L, (k_block_jacobi<T, BS_, L_, false><<<gridsize(h, L0.n_nodes),
                                                                   kBlock, 0, h->stream>>>(
                                 L0.n_nodes, N0.dinv.template as<T>(), r, z, nullptr, nullptr,
                                 nullptr)));
  } else {
    TOPT_BSL_DISPATCH(bs, L, (k_block_jacobi<T, BS_, L_, true><<<gridsize(h, L0.n_nodes),
                                                                  kBlock, 0, h->stream>>>(
                                 L0.n_nodes, N0.dinv.template as<T>(), r, z,
                                 h->red.partials.as<double>(), h->red.ctr(slot),
                                 h->red.res(slot))));
  }
  TOPT_CHECK_LAUNCH("k_block_jacobi");
  return TOPT_OK;
}

// Columns j with bit j of `cols` set are zeroed (n x L row-major).
template <typename T>
__global__ void k_zero_cols(int64_t n, int L, unsigned cols, T* __restrict__ x) {
  TOPT_KERNEL_COUNT();
  const int64_t nl = n * L;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl;
       i += (int64_t)gridDim.x * blockDim.x)
    if ((cols >> (int)(i % L)) & 1u) x[i] = T(0);
}

// Zero the fixed DOFs of an initial guess (FP64 solution vectors; the FP32
// hierarchy is never started from a guess), and the whole column of every
// load case whose right-hand side vanishes (active_h[j] == 0): such a column
// takes no iteration, so its solution is the zero vector, not the guess.
template <typename T>
static int start_from(topt_fem* h, int L, T* x, const int* active_h) {
  if (std::is_same<T, double>::value) {
    k_zero_fixed<<<gridsize(h, h->n_dof * L), kBlock, 0, h->stream>>>(
        h->n_dof, L, h->mask.as<uint8_t>(), (double*)x);
    TOPT_CHECK_LAUNCH("k_zero_fixed");
  }
  unsigned cols = 0;
  for (int j = 0; j < L; ++j)
    if (!active_h[j]) cols |= 1u << j;
  if (cols) {
    k_zero_cols<T><<<gridsize(h, h->n_dof * L), kBlock, 0, h->stream>>>(h->n_dof, L, cols, x);
    TOPT_CHECK_LAUNCH("k_zero_cols");
  }
  return TOPT_OK;
}

// Mixed precision PCG with reliable updates: CG recurrences, operator and
// preconditioner in FP32; whenever the FP32 residual has dropped by `delta`
// since the last update (or looks converged) the FP32 iterate is added to the
// FP64 solution, the FP64 residual Fe - K64 U is recomputed and replaces the
// FP32 one.  The search direction is kept across updates, so the method
// converges at the FP64 rate while FP64 is used only for the residual, the
// solution update and the norms (iterative refinement without restart).
static int pcg_reliable(topt_fem* h, int L, double* U, float* p32, float* q32, float* z32,
                        float* r32, float* x32, double rtol, int maxiter, double delta,
                        int max_updates, int precond, int degree, topt_solve_info* inf) {
  Hier<float>& H = h->h32;
  LevelStruct& L0 = h->ls[0];
  const int bs = h->bs;
  const int64_t n = h->n_dof, nl = n * L;
  const double* fe = h->fe.as<double>();
  double* R = h->R.as<double>();
  int rc;
  double bn2[4] = {0, 0, 0, 0}, rr[4], rn2[4], rmax[4];
  if ((rc = dot<double>(h, n, L, fe, fe, 2))) return rc;
  if ((rc = read_slot(h, 2, L, bn2))) return rc;
  int active_h[4] = {1, 1, 1, 1};
  for (int j = 0; j < L; ++j) {
    rmax[j] = std::sqrt(bn2[j]);
    if (!(bn2[j] > 0.0)) active_h[j] = 0;
  }
  DevBuf& active = h->active;
  TOPT_CUDA(cudaMemcpyAsync(active.p, active_h, 4 * sizeof(int), cudaMemcpyHostToDevice,
                            h->stream));
  TOPT_CUDA(cudaMemsetAsync(U, 0, sizeof(double) * nl, h->stream));
  TOPT_CUDA(cudaMemsetAsync(x32, 0, sizeof(float) * nl, h->stream));
  k_convert<float, double><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, fe, r32);
  int slot_old = 3, slot_new = 4;
  if ((rc = precond_apply<float>(h, H, L, r32, z32, precond, degree, slot_new))) return rc;
  TOPT_L_DISPATCH(L, (k_pcg_direction<float, float, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                         n, h->red.res(slot_new), h->red.res(slot_old), 1, z32, p32, nullptr)));
  std::swap(slot_old, slot_new);
  inf->status = TOPT_MAXITER;
  inf->iters = 0;
  inf->outer = 0;
  const float* A32 = H.lv[0].vals.as<float>();
  for (int it = 1; it <= maxiter; ++it) {
    if ((rc = spmv<float>(h, L0, bs, L, 0, true, A32, p32, nullptr, q32, 5, ChebEp<float>(),
                          true)))
      return rc;
    TOPT_L_DISPATCH(L, (k_pcg_update<float, float, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                           n, h->red.res(slot_old), h->red.res(5), active.as<int>(), p32, q32,
                           x32, r32, h->red.partials.as<double>(), h->red.ctr(6),
                           h->red.res(6), nullptr)));
    TOPT_CHECK_LAUNCH("k_pcg_update");
    inf->iters = it;
    if ((rc = read_slot(h, 6, L, rr))) return rc;
    bool update = (it == maxiter), all_small = true;
    for (int j = 0; j < L; ++j) {
      if (!active_h[j]) continue;
      if (!std::isfinite(rr[j])) { inf->status = TOPT_NONFINITE; return TOPT_OK; }
      const double rj = std::sqrt(rr[j]);
      if (rj < delta * rmax[j]) update = true;
      if (rj > rtol * std::sqrt(bn2[j])) all_small = false;
    }
    if (all_small) update = true;
    if (update) {
      // reliable update: U += x32; R = Fe - K64 U; r32 = R
      k_add_f32_to_f64<<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, x32, U);
      TOPT_CUDA(cudaMemsetAsync(x32, 0, sizeof(float) * nl, h->stream));
      if ((rc = spmv<double>(h, L0, bs, L, 1, false, h->vals64_0.as<double>(), U, fe, R)))
        return rc;
      if ((rc = dot<double>(h, n, L, R, R, 7))) return rc;
      if ((rc = read_slot(h, 7, L, rn2))) return rc;
      inf->outer += 1;
      bool done = true;
      double rel = 0.0;
      for (int j = 0; j < L; ++j) {
        if (!active_h[j]) continue;
        if (!std::isfinite(rn2[j])) { inf->status = TOPT_NONFINITE; return TOPT_OK; }
        rmax[j] = std::sqrt(rn2[j]);
        const double rj = std::sqrt(rn2[j] / bn2[j]);
        rel = std::max(rel, rj);
        if (rj > rtol) done = false;
      }
      inf->relres = rel;
      if (done) { inf->status = TOPT_OK; break; }
      if (inf->outer >= max_updates) break;
      k_convert<float, double><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, R, r32);
    }
    if ((rc = precond_apply<float>(h, H, L, r32, z32, precond, degree, slot_new))) return rc;
    TOPT_L_DISPATCH(L, (k_pcg_direction<float, float, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                           n, h->red.res(slot_new), h->red.res(slot_old), 0, z32, p32, nullptr)));
    std::swap(slot_old, slot_new);
  }
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

// Solves A x = b on level 0 of hierarchy H (precision T); x starts at 0.
// b, x: n_dof x L.  Uses H.lv[0] work vectors r (residual), d/q scratch and
// external p, q, z buffers.
template <typename T>
static int pcg(topt_fem* h, Hier<T>& H, int L, const T* b, T* x, T* p, T* q, T* z, T* r,
               double rtol, int maxiter, int precond, int degree, int check_every,
               int* iters_out, double* relres_out, int* status, bool x0 = false) {
  LevelStruct& L0 = h->ls[0];
  LevelNum<T>& N0 = H.lv[0];
  const int bs = h->bs;
  const int64_t n = h->n_dof;
  const int64_t nl = n * L;
  int rc;
  const T* vals = N0.vals.template as<T>();
  double bnorm2[4] = {0, 0, 0, 0};
  if ((rc = dot<T>(h, n, L, b, b, 2))) return rc;
  if ((rc = read_slot(h, 2, L, bnorm2))) return rc;
  // device scalars: slots 3 (rz A), 4 (rz B), 5 (pq), 6 (rr); active flags
  int active_h[4] = {1, 1, 1, 1};
  for (int j = 0; j < L; ++j)
    if (!(bnorm2[j] > 0.0)) active_h[j] = 0;
  if (x0) {   // r = b - A x from the caller's x (fixed DOFs zeroed first)
    if ((rc = start_from(h, L, x, active_h))) return rc;
    if ((rc = spmv<T>(h, L0, bs, L, 1, false, vals, x, b, r))) return rc;
  } else {
    TOPT_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * nl, h->stream));
    TOPT_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * nl, cudaMemcpyDeviceToDevice, h->stream));
  }
  DevBuf& active = h->active;
  TOPT_CUDA(cudaMemcpyAsync(active.p, active_h, 4 * sizeof(int), cudaMemcpyHostToDevice,
                            h->stream));
  int slot_old = 3, slot_new = 4;
  auto apply_prec = [&](int slot) -> int {
    return precond_apply<T>(h, H, L, r, z, precond, degree, slot);
  };
  if ((rc = apply_prec(slot_new))) return rc;
  TOPT_L_DISPATCH(L, (k_pcg_direction<T, T, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                         n, h->red.res(slot_new), h->red.res(slot_old), 1, z, p, nullptr)));
  std::swap(slot_old, slot_new);
  int it = 0;
  double rr[4] = {0, 0, 0, 0};
  double rel = 1.0;
  *status = TOPT_MAXITER;
  for (it = 1; it <= maxiter; ++it) {
    // q = A p, pq = p.q
    if ((rc = spmv<T>(h, L0, bs, L, 0, true, vals, p, nullptr, q, 5, ChebEp<T>(), true)))
      return rc;
    TOPT_L_DISPATCH(L, (k_pcg_update<T, T, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                           n, h->red.res(slot_old), h->red.res(5), active.as<int>(), p, q, x, r,
                           h->red.partials.as<double>(), h->red.ctr(6), h->red.res(6), nullptr)));
    TOPT_CHECK_LAUNCH("k_pcg_update");
    if (it % check_every == 0 || it == maxiter) {
      if ((rc = read_slot(h, 6, L, rr))) return rc;
      bool done = true, bad = false;
      rel = 0.0;
      for (int j = 0; j < L; ++j) {
        if (!std::isfinite(rr[j])) bad = true;
        if (!active_h[j]) continue;
        const double rj = std::sqrt(rr[j] / bnorm2[j]);
        rel = std::max(rel, rj);
        if (rj > rtol) done = false;
      }
      if (bad) { *status = TOPT_NONFINITE; break; }
      if (done) { *status = TOPT_OK; break; }
    }
    if ((rc = apply_prec(slot_new))) return rc;
    TOPT_L_DISPATCH(L, (k_pcg_direction<T, T, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                           n, h->red.res(slot_new), h->red.res(slot_old), 0, z, p, nullptr)));
    std::swap(slot_old, slot_new);
  }
  *iters_out = std::min(it, maxiter);
  *relres_out = rel;
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

// Krylov-accelerated iterative refinement: flexible CG in FP64 (operator,
// residual, solution update, dots) whose preconditioner -- the inner solve --
// is one FP32 multigrid V-cycle (or FP32 block Jacobi) applied to the
// rounded FP64 residual.  The Polak-Ribiere direction update keeps CG
// convergence although the FP32 inner solve is not exactly linear.  The FP32
// copy of r is written by the residual update itself and z stays FP32 (the
// direction and dot kernels widen it on load).
static int pcg_fcg_mixed(topt_fem* h, int L, double* U, double* p, double* q, double* r,
                         float* r32, float* z32, double rtol, int maxiter, int precond,
                         int degree, int check_every, topt_solve_info* inf) {
  Hier<float>& H = h->h32;
  LevelStruct& L0 = h->ls[0];
  const int bs = h->bs;
  const int64_t n = h->n_dof, nl = n * L;
  const double* fe = h->fe.as<double>();
  const double* A64 = h->vals64_0.as<double>();
  int rc;
  double bn2[4] = {0, 0, 0, 0}, rr[4];
  if ((rc = dot<double>(h, n, L, fe, fe, 2))) return rc;
  if ((rc = read_slot(h, 2, L, bn2))) return rc;
  int active_h[4] = {1, 1, 1, 1};
  for (int j = 0; j < L; ++j)
    if (!(bn2[j] > 0.0)) active_h[j] = 0;
  DevBuf& active = h->active;
  TOPT_CUDA(cudaMemcpyAsync(active.p, active_h, 4 * sizeof(int), cudaMemcpyHostToDevice,
                            h->stream));
  if (h->x0) {   // r = Fe - K U from the caller's U (fixed DOFs zeroed first)
    if ((rc = start_from<double>(h, L, U, active_h))) return rc;
    if ((rc = spmv<double>(h, L0, bs, L, 1, false, A64, U, fe, r))) return rc;
  } else {
    TOPT_CUDA(cudaMemsetAsync(U, 0, sizeof(double) * nl, h->stream));
    TOPT_CUDA(cudaMemcpyAsync(r, fe, sizeof(double) * nl, cudaMemcpyDeviceToDevice,
                              h->stream));
  }
  k_convert<float, double><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, r, r32);
  TOPT_CHECK_LAUNCH("k_convert");
  // z = M32(r); slot 3 <- r.z (FP64 r, FP32 z)
  if ((rc = precond_apply<float>(h, H, L, r32, z32, precond, degree, -1))) return rc;
  TOPT_L_DISPATCH(L, (k_dot2<double, double, float, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                         n, r, r, z32, h->red.partials.as<double>(), h->red.ctr(8),
                         h->red.res(8))));
  TOPT_CUDA(cudaMemcpyAsync(h->red.res(3), h->red.res(8), sizeof(double) * L,
                            cudaMemcpyDeviceToDevice, h->stream));
  TOPT_L_DISPATCH(L, (k_pcg_direction<double, float, L_><<<gridsize(h, n), kBlock, 0,
                                                           h->stream>>>(
                         n, h->red.res(3), h->red.res(3), 1, z32, p, nullptr)));
  inf->status = TOPT_MAXITER;
  double rel = 1.0;
  int it;
  for (it = 1; it <= maxiter; ++it) {
    // q = A p, pq = p.q (slot 5); x += a p, r -= a q, r32 = float(r), rr (slot 6)
    if ((rc = spmv<double>(h, L0, bs, L, 0, true, A64, p, nullptr, q, 5))) return rc;
    TOPT_L_DISPATCH(L, (k_pcg_update<double, double, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                           n, h->red.res(3), h->red.res(5), active.as<int>(), p, q, U, r,
                           h->red.partials.as<double>(), h->red.ctr(6), h->red.res(6), r32)));
    TOPT_CHECK_LAUNCH("k_pcg_update");
    if (it % check_every == 0 || it == maxiter) {
      if ((rc = read_slot(h, 6, L, rr))) return rc;
      bool done = true, bad = false;
      rel = 0.0;
      for (int j = 0; j < L; ++j) {
        if (!std::isfinite(rr[j])) bad = true;
        if (!active_h[j]) continue;
        const double rj = std::sqrt(rr[j] / bn2[j]);
        rel = std::max(rel, rj);
        if (rj > rtol) done = false;
      }
      if (bad) { inf->status = TOPT_NONFINITE; break; }
      if (done) { inf->status = TOPT_OK; break; }
    }
    if ((rc = precond_apply<float>(h, H, L, r32, z32, precond, degree, -1))) return rc;
    // slot 8 <- (r.z_new, q.z_new); slot 3 <- r.z_new
    TOPT_L_DISPATCH(L, (k_dot2<double, double, float, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                           n, r, q, z32, h->red.partials.as<double>(), h->red.ctr(8),
                           h->red.res(8))));
    TOPT_L_DISPATCH(L, (k_fcg_direction<double, float, L_><<<gridsize(h, n), kBlock, 0,
                                                             h->stream>>>(
                           n, h->red.res(8) + L, h->red.res(5), active.as<int>(), z32, p, nullptr)));
    TOPT_CUDA(cudaMemcpyAsync(h->red.res(3), h->red.res(8), sizeof(double) * L,
                              cudaMemcpyDeviceToDevice, h->stream));
    TOPT_CHECK_LAUNCH("k_fcg_direction");
  }
  inf->iters = std::min(it, maxiter);
  inf->outer = inf->iters;
  inf->relres = rel;
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

// Flexible CG with FP32 recurrences (residual, directions, products with the
// FP32 level-0 operator, dots accumulated in FP64 across threads) and the
// solution accumulated in FP64, preconditioned by the FP32 V-cycle (or block
// Jacobi).  The recursive FP32 residual drifts from Fe - A64 U by the FP32
// operator and rounding errors, so it is replaced by the FP64 residual (one
// FP64 product, rounded to FP32) whenever it has dropped by `delta` since the
// last replacement, after `max_between` iterations, and whenever it looks
// converged; convergence is declared on the FP64 residual only (residual
// replacement, van der Vorst & Ye, SIAM J. Sci. Comput. 22, 2000).  The
// Polak-Ribiere direction update beta = -(q.z_new)/(p.q) tolerates both the
// replacements and the FP32 inner solve.  Buffers: r64 FP64 (replacement
// only); p32, q32, r32, z32 FP32.
static int pcg_fcg_rr(topt_fem* h, int L, double* U, double* r64, float* p32, float* q32,
                      float* r32, float* z32, double rtol, int maxiter, int precond,
                      int degree, double delta, int max_between, topt_solve_info* inf) {
  Hier<float>& H = h->h32;
  LevelStruct& L0 = h->ls[0];
  const int bs = h->bs;
  const int64_t n = h->n_dof, nl = n * L;
  const double* fe = h->fe.as<double>();
  const double* A64 = h->vals64_0.as<double>();
  const float* A32 = H.lv[0].vals.as<float>();
  int rc;
  double bn2[4] = {0, 0, 0, 0}, rr[4], rlast2[4];
  if ((rc = dot<double>(h, n, L, fe, fe, 2))) return rc;
  if ((rc = read_slot(h, 2, L, bn2))) return rc;
  int active_h[4] = {1, 1, 1, 1};
  for (int j = 0; j < L; ++j) {
    if (!(bn2[j] > 0.0)) active_h[j] = 0;
    rlast2[j] = bn2[j];
  }
  DevBuf& active = h->active;
  TOPT_CUDA(cudaMemcpyAsync(active.p, active_h, 4 * sizeof(int), cudaMemcpyHostToDevice,
                            h->stream));
  if (h->x0) {   // r = Fe - K U from the caller's U (fixed DOFs zeroed first)
    if ((rc = start_from<double>(h, L, U, active_h))) return rc;
    if ((rc = spmv<double>(h, L0, bs, L, 1, false, A64, U, fe, r64))) return rc;
    if ((rc = dot<double>(h, n, L, r64, r64, 7))) return rc;
    if ((rc = read_slot(h, 7, L, rlast2))) return rc;
    k_convert<float, double><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, r64, r32);
  } else {
    TOPT_CUDA(cudaMemsetAsync(U, 0, sizeof(double) * nl, h->stream));
    k_convert<float, double><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, fe, r32);
  }
  TOPT_CHECK_LAUNCH("k_convert");
  if ((rc = precond_apply<float>(h, H, L, r32, z32, precond, degree, -1))) return rc;
  TOPT_L_DISPATCH(L, (k_dot2<float, float, float, L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                         n, r32, r32, z32, h->red.partials.as<double>(), h->red.ctr(8),
                         h->red.res(8))));
  TOPT_CUDA(cudaMemcpyAsync(h->red.res(3), h->red.res(8), sizeof(double) * L,
                            cudaMemcpyDeviceToDevice, h->stream));
  TOPT_L_DISPATCH(L, (k_pcg_direction<float, float, L_><<<gridsize(h, n), kBlock, 0,
                                                          h->stream>>>(
                         n, h->red.res(3), h->red.res(3), 1, z32, p32, nullptr)));
  inf->status = TOPT_MAXITER;
  inf->outer = 0;
  double rel = 1.0;
  // Stagnation: the FP32 recursion can reach the attainable accuracy of the
  // refinement before rtol (a tolerance near the FP64 rounding level, a
  // poorly conditioned preconditioned system).  After kStall replacements
  // without a new smallest true residual the solve ends with TOPT_MAXITER
  // and the iterate of the smallest one (kept in Ubest).
  const int kStall = 6;
  double best = INFINITY;
  int stall = 0;
  bool have_best = false;
  int it, since = 0;
  for (it = 1; it <= maxiter; ++it) {
    // q32 = A32 p32 and p.q (slot 5); U += a p (FP64), r32 -= a q32, r.r (slot 6)
    if ((rc = spmv<float>(h, L0, bs, L, 0, true, A32, p32, nullptr, q32, 5, ChebEp<float>(),
                          true)))
      return rc;
    TOPT_L_DISPATCH(L, (k_fcg_update32<L_><<<gridsize(h, n), kBlock, 0, h->stream>>>(
                           n, h->red.res(3), h->red.res(5), active.as<int>(), p32, q32, U, r32,
                           h->red.partials.as<double>(), h->red.ctr(6), h->red.res(6))));
    TOPT_CHECK_LAUNCH("k_fcg_update32");
    ++since;
    if ((rc = read_slot(h, 6, L, rr))) return rc;
    bool small = true, dropped = false, bad = false;
    for (int j = 0; j < L; ++j) {
      if (!std::isfinite(rr[j])) bad = true;
      if (!active_h[j]) continue;
      if (rr[j] > rtol * rtol * bn2[j]) small = false;
      if (rr[j] <= delta * delta * rlast2[j]) dropped = true;
    }
    if (bad) { inf->status = TOPT_NONFINITE; break; }
    if (small || dropped || since >= max_between || it == maxiter) {
      // residual replacement: r = Fe - A64 U in FP64, rounded to FP32
      if ((rc = spmv<double>(h, L0, bs, L, 1, false, A64, U, fe, r64))) return rc;
      k_convert<float, double><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, r64, r32);
      TOPT_CHECK_LAUNCH("k_convert");
      if ((rc = dot<double>(h, n, L, r64, r64, 7))) return rc;
      if ((rc = read_slot(h, 7, L, rr))) return rc;
      inf->outer += 1;
      since = 0;
      bool done = true;
      rel = 0.0;
      for (int j = 0; j < L; ++j) {
        if (!std::isfinite(rr[j])) bad = true;
        rlast2[j] = rr[j];
        if (!active_h[j]) continue;
        const double rj = std::sqrt(rr[j] / bn2[j]);
        rel = std::max(rel, rj);
        if (rj > rtol) done = false;
      }
      if (bad) { inf->status = TOPT_NONFINITE; break; }
      if (done) { inf->status = TOPT_OK; break; }
      if (rel < best) {
        best = rel;
        stall = 0;
        if (!h->Ubest.p && (rc = h->Ubest.alloc(sizeof(double) * h->n_dof * 4))) return rc;
        TOPT_CUDA(cudaMemcpyAsync(h->Ubest.p, U, sizeof(double) * nl, cudaMemcpyDeviceToDevice,
                                  h->stream));
        have_best = true;
      } else if (++stall >= kStall) {
        TOPT_CUDA(cudaMemcpyAsync(U, h->Ubest.p, sizeof(double) * nl, cudaMemcpyDeviceToDevice,
                                  h->stream));
        rel = best;
        break;
      }
    }
    if ((rc = precond_apply<float>(h, H, L, r32, z32, precond, degree, -1))) return rc;
    // slot 8 <- (r.z_new, q.z_new); slot 3 <- r.z_new
    TOPT_L_DISPATCH(L, (k_dot2<float, float, float, L_><<<gridsize(h, n), kBlock, 0,
                                                         h->stream>>>(
                           n, r32, q32, z32, h->red.partials.as<double>(), h->red.ctr(8),
                           h->red.res(8))));
    TOPT_L_DISPATCH(L, (k_fcg_direction<float, float, L_><<<gridsize(h, n), kBlock, 0,
                                                            h->stream>>>(
                           n, h->red.res(8) + L, h->red.res(5), active.as<int>(), z32, p32,
                           nullptr)));
    TOPT_CUDA(cudaMemcpyAsync(h->red.res(3), h->red.res(8), sizeof(double) * L,
                              cudaMemcpyDeviceToDevice, h->stream));
    TOPT_CHECK_LAUNCH("k_fcg_direction");
  }
  if (inf->status == TOPT_MAXITER && it > maxiter && have_best && best < rel) {
    // the cap came first: hand back the best iterate as well
    TOPT_CUDA(cudaMemcpyAsync(U, h->Ubest.p, sizeof(double) * nl, cudaMemcpyDeviceToDevice,
                              h->stream));
    rel = best;
  }
  inf->iters = std::min(it, maxiter);
  inf->relres = rel;
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

}  // namespace topt

using namespace topt;

extern "C" {

int topt_fem_create(const topt_fem_desc* d, topt_fem** out) {
  if (!d || !out) return fail(TOPT_BAD_INPUT, "fem_create: null argument");
  *out = nullptr;
  if (!(d->bs == 1 || d->bs == 3) || !(d->nloc == 4 || d->nloc == 8))
    return fail(TOPT_BAD_INPUT, "fem_create: bs must be 1 or 3 and nloc 4 or 8");
  if (d->n_nodes <= 0 || d->n_elem <= 0 || !d->t || !d->ke || !d->dirichlet)
    return fail(TOPT_BAD_INPUT, "fem_create: missing mesh data");
  if (!(d->n_ke == 1 || d->n_ke == d->n_elem))
    return fail(TOPT_BAD_INPUT, "fem_create: n_ke must be 1 or n_elem");
  std::unique_ptr<topt_fem> h(new (std::nothrow) topt_fem());
  if (!h) return fail(TOPT_NO_MEMORY, "fem_create: host allocation");
  h->bs = d->bs;
  h->nloc = d->nloc;
  h->n_nodes = d->n_nodes;
  h->n_elem = d->n_elem;
  h->n_dof = d->n_nodes * d->bs;
  h->n_ke = d->n_ke;
  h->mixed = d->mixed != 0;
  h->sm = device_sm_count();
  h->mg_levels = std::max(1, d->mg_levels);
  h->mg_coarse_max = d->mg_coarse_max > 0 ? d->mg_coarse_max : 192;
  cudaStream_t s = nullptr;
  int rc;
  h->ls.emplace_back();
  LevelStruct& L0 = h->ls[0];
  try {
    if ((rc = upload_pattern(L0, d->n_nodes, d->n_elem, d->nloc, d->t, s))) return rc;
  } catch (const std::bad_alloc&) {
    return fail(TOPT_NO_MEMORY, "fem_create: host allocation");
  }
  const int nd = d->bs * d->nloc;
  const size_t nke = (size_t)d->n_ke * nd * nd;
  if ((rc = upload(h->ke64, d->ke, nke, s))) return rc;
  {
    std::vector<float> k32(d->ke, d->ke + nke);
    if ((rc = upload(h->ke32, k32.data(), nke, s))) return rc;
    TOPT_CUDA(cudaStreamSynchronize(s));
    if (nke == 576) std::copy(k32.begin(), k32.end(), h->k0.v);
  }
  if ((rc = upload(h->mask, d->dirichlet, (size_t)h->n_dof, s))) return rc;
  if ((rc = h->coef64.alloc(sizeof(double) * d->n_elem))) return rc;
  if ((rc = h->coef32.alloc(sizeof(float) * d->n_elem))) return rc;
  if ((rc = h->red.init(h->sm * 16))) return rc;
  // multigrid levels on the logical grid
  h->has_grid = d->grid[0] > 0 && d->grid[1] > 0 && d->grid[2] > 0;
  if (h->has_grid) {
    const int nx = d->grid[0], ny = d->grid[1], nz = d->grid[2];
    if ((int64_t)(nx + 1) * (ny + 1) * (nz + 1) != d->n_nodes)
      return fail(TOPT_BAD_INPUT, "fem_create: grid does not match the node count");
    if (d->node_ijk) {
      for (int64_t n = 0; n < d->n_nodes; ++n) {
        const int64_t ix = d->node_ijk[n], iy = d->node_ijk[d->n_nodes + n],
                      iz = d->node_ijk[2 * d->n_nodes + n];
        if (iy + (int64_t)(ny + 1) * (ix + (int64_t)(nx + 1) * iz) != n)
          return fail(TOPT_BAD_INPUT, "fem_create: nodes are not in grid order");
      }
    }
    L0.nx = nx; L0.ny = ny; L0.nz = nz;
    const int64_t ncell = (int64_t)nx * ny * nz;
    if (d->cell_of_elem) {
      std::vector<int32_t> cptr(ncell + 1, 0), cel(d->n_elem);
      for (int64_t e = 0; e < d->n_elem; ++e) {
        const int32_t c = d->cell_of_elem[e];
        if (c < 0 || c >= ncell) return fail(TOPT_BAD_INPUT, "fem_create: bad cell id");
        cptr[c + 1]++;
      }
      for (int64_t c = 0; c < ncell; ++c) cptr[c + 1] += cptr[c];
      std::vector<int32_t> pos(cptr.begin(), cptr.end() - 1);
      for (int64_t e = 0; e < d->n_elem; ++e) cel[pos[d->cell_of_elem[e]]++] = (int32_t)e;
      if ((rc = upload(L0.cell_ptr, cptr.data(), cptr.size(), s))) return rc;
      if ((rc = upload(L0.cell_elems, cel.data(), cel.size(), s))) return rc;
    } else if (d->n_elem != ncell) {
      return fail(TOPT_BAD_INPUT, "fem_create: cell_of_elem needed when elements != cells");
    }
    while ((int)h->ls.size() < h->mg_levels) {
      LevelStruct& F = h->ls.back();
      const int64_t ndof_f = F.n_nodes * d->bs;
      if (ndof_f <= h->mg_coarse_max) break;
      if (F.nx <= 1 && F.ny <= 1 && F.nz <= 1) break;
      const int cx = (F.nx + 1) / 2, cy = (F.ny + 1) / 2, cz = (F.nz + 1) / 2;
      LevelStruct C;
      C.nx = cx; C.ny = cy; C.nz = cz;
      std::vector<int32_t> tc = hex_grid_t(cx, cy, cz);
      const int64_t cn = (int64_t)(cx + 1) * (cy + 1) * (cz + 1);
      if ((rc = upload_pattern(C, cn, (int64_t)cx * cy * cz, 8, tc.data(), s))) return rc;
      if ((rc = make_transfer(h->ls.back(), C, s))) return rc;
      h->ls.push_back(std::move(C));
    }
    if (h->ls.size() > 1 && d->n_ke == 1 && d->nloc == 8 && !d->cell_of_elem) {
      if ((rc = setup_shared_galerkin(h.get(), d->ke, d->dirichlet))) return rc;
    }
    // matrix-free FP32 level 0 on uniform hex grids (elasticity)
    if (d->n_ke == 1 && d->nloc == 8 && d->bs == 3 && !d->cell_of_elem && d->mixed &&
        d->mf_level0) {
      h->mf = true;
      h->mfg.nx = nx; h->mfg.ny = ny; h->mfg.nz = nz;
      std::vector<uint8_t> nm(d->n_nodes);
      for (int64_t n = 0; n < d->n_nodes; ++n)
        nm[n] = (uint8_t)((d->dirichlet[3 * n] ? 1 : 0) | (d->dirichlet[3 * n + 1] ? 2 : 0) |
                          (d->dirichlet[3 * n + 2] ? 4 : 0));
      if ((rc = upload(h->nmask, nm.data(), nm.size(), s))) return rc;
      {
        std::vector<uint32_t> nm32(nm.begin(), nm.end());
        if ((rc = upload(h->nmask32, nm32.data(), nm32.size(), s))) return rc;
      }
      TOPT_CUDA(cudaStreamSynchronize(s));
      h->mf_ty = mf_pick_ty(ny + 1);
      if ((rc = setup_mf_tc(h.get(), s))) return rc;
    }
    if (h->ls.size() > 1) {
      LevelStruct& B = h->ls.back();
      const int64_t nd_b = B.n_nodes * d->bs;
      if (nd_b <= 4096) {
        B.dense = true;
        B.ndense = (int)nd_b;
      } else {
        return fail(TOPT_BAD_INPUT, "fem_create: coarsest level too large for a dense solve; "
                                    "raise mg_levels");
      }
    }
  }
  if (!h->has_grid && d->amg && h->mg_levels > 1) {
    if ((rc = setup_amg(h.get()))) return rc;
  }
  if ((rc = h->active.alloc(4 * sizeof(int)))) return rc;
  if ((rc = h->fe.alloc(sizeof(double) * h->n_dof * 4))) return rc;
  if ((rc = h->R.alloc(sizeof(double) * h->n_dof * 4))) return rc;
  if ((rc = h->U0.alloc(sizeof(double) * h->n_dof * 4 * 4))) return rc;
  TOPT_CUDA(cudaDeviceSynchronize());
  *out = h.release();
  return TOPT_OK;
}

void topt_fem_destroy(topt_fem* h) {
  if (!h) return;
  cudaDeviceSynchronize();
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->aux) cudaStreamDestroy(h->aux);
  vcycle_graphs_free(h);
  if (h->cap) cudaStreamDestroy(h->cap);
  delete h;
}

int topt_fem_set_stream(topt_fem* h, void* stream) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem: null handle");
  h->stream = (cudaStream_t)stream;
  return TOPT_OK;
}

int topt_fem_sizes(const topt_fem* h, int64_t* n_dof, int64_t* nnzb, int32_t* n_levels) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem: null handle");
  if (n_dof) *n_dof = h->n_dof;
  if (nnzb) *nnzb = h->ls[0].nnzb;
  if (n_levels) *n_levels = (int32_t)h->ls.size();
  return TOPT_OK;
}

int topt_fem_set_mf_kernel(topt_fem* h, int32_t kind) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem_set_mf_kernel: null handle");
  if (kind < 0 || kind > 1)
    return fail(TOPT_BAD_INPUT, "fem_set_mf_kernel: kind must be 0 (FMA) or 1 (tensor cores)");
  h->mf_kernel = kind;
  vcycle_graphs_stale(h);
  return TOPT_OK;
}

int topt_fem_set_vcycle_graphs(topt_fem* h, int32_t on) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem_set_vcycle_graphs: null handle");
  h->vc_graphs = on != 0;
  vcycle_graphs_free(h);
  return TOPT_OK;
}

int topt_fem_mf_error(topt_fem* h, int32_t* mf_error) {
  if (!h || !mf_error) return fail(TOPT_BAD_INPUT, "fem_mf_error: null argument");
  *mf_error = 0;
  if (h->mf_err.p) {
    TOPT_CUDA(cudaStreamSynchronize(h->stream));
    TOPT_CUDA(cudaMemcpy(mf_error, h->mf_err.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  return TOPT_OK;
}

int topt_fem_set_interpolation(topt_fem* h, int32_t kind) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem_set_interpolation: null handle");
  if (kind < 0 || kind > 2)
    return fail(TOPT_BAD_INPUT, "fem_set_interpolation: kind must be 0 (SIMP), 1 (RAMP) or 2 (RAMP, SIMP-form sensitivity)");
  h->interp = kind;
  return TOPT_OK;
}

int topt_fem_update(topt_fem* h, const double* rho, double E0, double Emin, double p) {
  if (!h || !rho) return fail(TOPT_BAD_INPUT, "fem_update: null argument");
  h->E0 = E0; h->Emin = Emin; h->p = p;
  k_simp_coef<<<gridsize(h, h->n_elem), kBlock, 0, h->stream>>>(
      h->n_elem, rho, E0, Emin, p, h->coef64.as<double>(),
      h->mixed ? h->coef32.as<float>() : nullptr, h->interp);
  TOPT_CHECK_LAUNCH("k_simp_coef");
  int rc;
  h->full_ok = false;
  if (h->extra64 && h->mixed) {
    const int64_t nx = h->n_elem * (int64_t)(h->bs * h->nloc) * (h->bs * h->nloc);
    if (h->extra32.bytes < sizeof(float) * (size_t)nx &&
        (rc = h->extra32.alloc(sizeof(float) * (size_t)nx)))
      return rc;
    k_d2f<<<gridsize(h, nx), kBlock, 0, h->stream>>>(nx, h->extra64, h->extra32.as<float>());
    TOPT_CHECK_LAUNCH("k_d2f");
  }
  if (h->mixed) {
    // FP64 operator for the refinement residual, FP32 operator + hierarchy
    if (!h->vals64_0.p &&
        (rc = h->vals64_0.alloc(sizeof(double) * h->ls[0].npos * h->bs * h->bs)))
      return rc;
    const int64_t stride0 = h->n_ke == 1 ? 0 : (int64_t)(h->bs * h->nloc) * (h->bs * h->nloc);
    if ((rc = assemble<double>(h, h->ls[0], h->bs, h->nloc, h->ke64.as<double>(), stride0,
                               h->coef64.as<double>(), h->extra64, h->mask.as<uint8_t>(),
                               h->vals64_0.as<double>())))
      return rc;
    if ((rc = refresh<float>(h, h->h32))) return rc;
  } else {
    if ((rc = refresh<double>(h, h->h64))) return rc;
  }
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  h->assembled = true;
  return TOPT_OK;
}

static const double* op64(topt_fem* h) {
  return h->mixed ? h->vals64_0.as<double>() : h->h64.lv[0].vals.as<double>();
}

int topt_fem_set_element_extra(topt_fem* h, const double* extra) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem_set_element_extra: null handle");
  if (extra && h->mf)
    return fail(TOPT_BAD_INPUT,
                "fem_set_element_extra: the matrix-free level-0 operator takes no extra terms");
  h->extra64 = extra;
  h->assembled = false;
  return TOPT_OK;
}

int topt_fem_spmv(topt_fem* h, int32_t dtype, const void* x, void* y, int32_t nrhs) {
  if (!h || !x || !y) return fail(TOPT_BAD_INPUT, "fem_spmv: null argument");
  if (!h->assembled) return fail(TOPT_BAD_INPUT, "fem_spmv: call topt_fem_update first");
  if (nrhs < 1 || nrhs > 4) return fail(TOPT_BAD_INPUT, "fem_spmv: nrhs must be 1..4");
  if (dtype == TOPT_F64_FULL) {
    int rc;
    if (!h->full_ok) {
      if (!h->full64.p &&
          (rc = h->full64.alloc(sizeof(double) * h->ls[0].npos * h->bs * h->bs)))
        return rc;
      const int64_t stride0 = h->n_ke == 1 ? 0 : (int64_t)(h->bs * h->nloc) * (h->bs * h->nloc);
      if ((rc = assemble<double>(h, h->ls[0], h->bs, h->nloc, h->ke64.as<double>(), stride0,
                                 h->coef64.as<double>(), h->extra64, nullptr,
                                 h->full64.as<double>())))
        return rc;
      h->full_ok = true;
    }
    return spmv<double>(h, h->ls[0], h->bs, nrhs, 0, false, h->full64.as<double>(),
                        (const double*)x, nullptr, (double*)y);
  }
  if (dtype == TOPT_F64)
    return spmv<double>(h, h->ls[0], h->bs, nrhs, 0, false, op64(h), (const double*)x, nullptr,
                        (double*)y);
  if (dtype == TOPT_F32 && h->mixed)
    return spmv<float>(h, h->ls[0], h->bs, nrhs, 0, false, h->h32.lv[0].vals.as<float>(),
                       (const float*)x, nullptr, (float*)y);
  return fail(TOPT_BAD_INPUT, "fem_spmv: FP32 operator needs a mixed handle");
}

int topt_fem_set_mf_tile(topt_fem* h, int32_t ty) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem_set_mf_tile: null handle");
  if (!(ty == 0 || ty == 16 || ty == 27 || ty == 32))
    return fail(TOPT_BAD_INPUT, "fem_set_mf_tile: ty must be 0 (automatic), 16, 27 or 32");
  if (!h->mf) return fail(TOPT_BAD_INPUT, "fem_set_mf_tile: no matrix-free operator");
  h->mf_ty = ty ? ty : mf_pick_ty(h->mfg.ny + 1);
  vcycle_graphs_stale(h);
  return TOPT_OK;
}

int topt_fem_set_row_mapping(topt_fem* h, int32_t level, int32_t mapping) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem_set_row_mapping: null handle");
  if (level < 0 || level >= (int)h->ls.size())
    return fail(TOPT_BAD_INPUT, "fem_set_row_mapping: no such level");
  if (mapping < 0 || mapping > 3 || (mapping == 2 && h->bs != 3))
    return fail(TOPT_BAD_INPUT, "fem_set_row_mapping: mapping must be 0..3 (2 needs bs 3)");
  h->ls[level].row_map = mapping;
  vcycle_graphs_stale(h);
  return TOPT_OK;
}

int topt_fem_get_tuning(const topt_fem* h, int32_t* mf_tile, int32_t* mappings,
                        int32_t n_levels) {
  if (!h || !mf_tile || (n_levels > 0 && !mappings))
    return fail(TOPT_BAD_INPUT, "fem_get_tuning: null argument");
  *mf_tile = h->mf ? h->mf_ty : 0;
  for (int li = 0; li < n_levels && li < (int)h->ls.size(); ++li)
    mappings[li] = h->ls[li].dense ? 0 : row_mapping(h->ls[li], h->bs);
  return TOPT_OK;
}

int topt_fem_level_sizes(const topt_fem* h, int64_t* n_nodes, int32_t* dense, int32_t n_levels) {
  if (!h || (n_levels > 0 && (!n_nodes || !dense)))
    return fail(TOPT_BAD_INPUT, "fem_level_sizes: null argument");
  for (int li = 0; li < n_levels && li < (int)h->ls.size(); ++li) {
    n_nodes[li] = h->ls[li].n_nodes;
    dense[li] = h->ls[li].dense ? 1 : 0;
  }
  return TOPT_OK;
}

int topt_fem_spmv_level(topt_fem* h, int32_t level, int32_t dtype, const void* x, void* y) {
  if (!h || !x || !y) return fail(TOPT_BAD_INPUT, "fem_spmv_level: null argument");
  if (!h->assembled) return fail(TOPT_BAD_INPUT, "fem_spmv_level: call topt_fem_update first");
  if (level < 0 || level >= (int)h->ls.size() || h->ls[level].dense)
    return fail(TOPT_BAD_INPUT, "fem_spmv_level: no such (non-dense) level");
  const LevelStruct& L = h->ls[level];
  if (dtype == TOPT_F32 && h->mixed)
    return spmv<float>(h, L, h->bs, 1, 0, false,
                       level == 0 && h->mf ? nullptr : h->h32.lv[level].vals.as<float>(),
                       (const float*)x, nullptr, (float*)y);
  if (dtype == TOPT_F64 && !h->mixed)
    return spmv<double>(h, L, h->bs, 1, 0, false, h->h64.lv[level].vals.as<double>(),
                        (const double*)x, nullptr, (double*)y);
  return fail(TOPT_BAD_INPUT, "fem_spmv_level: dtype must be the handle's hierarchy precision "
                              "(FP32 for mixed handles, FP64 otherwise)");
}

// Device time of one level product, for the launch-shape autotuner: `reps`
// back-to-back products recorded as a CUDA graph on the private stream and
// timed with events around one replay (after a warm-up replay), so that host
// launch overhead, which exceeds the kernel time on small levels, does not
// enter the figure.
int topt_fem_time_spmv_level(topt_fem* h, int32_t level, int32_t dtype, const void* x, void* y,
                             int32_t reps, double* us) {
  if (!h || !x || !y || !us) return fail(TOPT_BAD_INPUT, "fem_time_spmv_level: null argument");
  if (reps < 1 || reps > 1000)
    return fail(TOPT_BAD_INPUT, "fem_time_spmv_level: reps must be in 1..1000");
  int rc = topt_fem_spmv_level(h, level, dtype, x, y);   // checks; sets kernel attributes
  if (rc) return rc;
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  if (!h->cap) TOPT_CUDA(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking));
  TOPT_CUDA(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal));
  cudaStream_t user = h->stream;
  h->stream = h->cap;
  for (int r = 0; r < reps && !rc; ++r) rc = topt_fem_spmv_level(h, level, dtype, x, y);
  h->stream = user;
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(h->cap, &graph);
  if (rc || ec != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return rc ? rc : fail_cuda((int)ec, "fem_time_spmv_level capture");
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return fail_cuda((int)ei, "fem_time_spmv_level instantiate");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, h->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e0, h->stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, h->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e1, h->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaGraphExecDestroy(exec);
  if (e != cudaSuccess) return fail_cuda((int)e, "fem_time_spmv_level");
  *us = 1e3 * (double)ms / reps;
  return TOPT_OK;
}

int topt_fem_export_values(topt_fem* h, double* vals) {
  if (!h || !vals) return fail(TOPT_BAD_INPUT, "fem_export_values: null argument");
  if (!h->assembled) return fail(TOPT_BAD_INPUT, "fem_export_values: not assembled");
  const LevelStruct& L0 = h->ls[0];
  if (h->bs == 3)
    k_sell_to_csr<3><<<gridsize(h, L0.nnzb), kBlock, 0, h->stream>>>(
        L0.nnzb, L0.csr2sell.as<int32_t>(), op64(h), vals);
  else
    k_sell_to_csr<1><<<gridsize(h, L0.nnzb), kBlock, 0, h->stream>>>(
        L0.nnzb, L0.csr2sell.as<int32_t>(), op64(h), vals);
  TOPT_CHECK_LAUNCH("k_sell_to_csr");
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

int topt_fem_solve(topt_fem* h, const double* F, double* U, int32_t nrhs,
                   const topt_solve_opts* o, topt_solve_info* info, double* compliance) {
  if (!h || !F || !U || !o) return fail(TOPT_BAD_INPUT, "fem_solve: null argument");
  if (!h->assembled) return fail(TOPT_BAD_INPUT, "fem_solve: call topt_fem_update first");
  if (nrhs < 1 || nrhs > 4) return fail(TOPT_BAD_INPUT, "fem_solve: nrhs must be 1..4");
  if (o->method < 0 || o->method > 4)
    return fail(TOPT_BAD_INPUT, "fem_solve: method must be 0..4");
  if (o->method >= 1 && !h->mixed)
    return fail(TOPT_BAD_INPUT, "fem_solve: mixed methods need a handle created with mixed=1");
  if (o->method == 0 && h->mixed)
    return fail(TOPT_BAD_INPUT, "fem_solve: FP64 method needs a handle created with mixed=0");
  if (o->precond == 1 && h->ls.size() < 2)
    return fail(TOPT_BAD_INPUT, "fem_solve: multigrid needs a logical grid");
  const int L = nrhs;
  const int64_t n = h->n_dof, nl = n * L;
  const int check = o->check_every > 0 ? o->check_every : 1;
  const int degree = o->cheb_degree > 0 ? o->cheb_degree : 2;
  h->cheb_ratio = o->cheb_ratio > 1.0 ? o->cheb_ratio : 30.0;
  h->x0 = o->x0 != 0 && (o->method == 0 || o->method == 3 || o->method == 4);
  int rc;
  topt_solve_info inf{};
  k_enforce_rhs<<<gridsize(h, nl), kBlock, 0, h->stream>>>(n, L, h->mask.as<uint8_t>(), F,
                                                            h->fe.as<double>());
  TOPT_CHECK_LAUNCH("k_enforce_rhs");
  double* p = h->U0.as<double>();
  double* q = p + nl;
  double* z = q + nl;
  double* r = z + nl;
  if (o->method == 0) {
    if ((rc = pcg<double>(h, h->h64, L, h->fe.as<double>(), U, p, q, z, r, o->rtol, o->maxiter,
                          o->precond, degree, check, &inf.iters, &inf.relres, &inf.status,
                          h->x0)))
      return rc;
  } else if (o->method == 3) {
    // FP64 flexible CG, FP32 multigrid inner solve; U0 holds p, q, r (FP64)
    // and R holds the FP32 r and z.
    float* r32 = (float*)h->R.p;
    if ((rc = pcg_fcg_mixed(h, L, U, p, q, r, r32, r32 + nl, o->rtol, o->maxiter, o->precond,
                            degree, check, &inf)))
      return rc;
  } else if (o->method == 4) {
    // flexible CG with FP32 recurrences, FP64 solution and FP64 residual
    // replacement; U0 holds the FP64 replacement residual and p32, q32 (in
    // the q slot); R holds the FP32 r and z.
    float* r32 = (float*)h->R.p;
    const double delta = (o->inner_rtol > 0.0 && o->inner_rtol < 1.0) ? o->inner_rtol : 0.1;
    const int max_between = o->max_outer > 0 ? o->max_outer : 50;
    if ((rc = pcg_fcg_rr(h, L, U, r, (float*)q, (float*)q + nl, r32, r32 + nl, o->rtol,
                         o->maxiter, o->precond, degree, delta, max_between, &inf)))
      return rc;
  } else if (o->method == 1) {
    float* p32 = (float*)p;
    const double delta = (o->inner_rtol > 0.0 && o->inner_rtol < 1.0) ? o->inner_rtol : 0.1;
    const int max_updates = o->max_outer > 0 ? o->max_outer : 50;
    if ((rc = pcg_reliable(h, L, U, p32, p32 + nl, p32 + 2 * nl, p32 + 3 * nl, p32 + 4 * nl,
                           o->rtol, o->maxiter, delta, max_updates, o->precond, degree, &inf)))
      return rc;
  } else {
    // FP32 PCG restarted inside an FP64 iterative-refinement loop
    float* p32 = (float*)p;
    float* q32 = p32 + nl;
    float* z32 = q32 + nl;
    float* r32 = z32 + nl;
    float* b32 = r32 + nl;
    float* x32 = b32 + nl;
    double bn2[4], rn2[4];
    if ((rc = dot<double>(h, n, L, h->fe.as<double>(), h->fe.as<double>(), 2))) return rc;
    if ((rc = read_slot(h, 2, L, bn2))) return rc;
    TOPT_CUDA(cudaMemsetAsync(U, 0, sizeof(double) * nl, h->stream));
    TOPT_CUDA(cudaMemcpyAsync(h->R.p, h->fe.p, sizeof(double) * nl, cudaMemcpyDeviceToDevice,
                              h->stream));
    inf.status = TOPT_MAXITER;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 20;
    for (int outer = 1; outer <= max_outer; ++outer) {
      k_convert<float, double><<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, h->R.as<double>(),
                                                                          b32);
      int it = 0, st = 0;
      double rel = 0.0;
      if ((rc = pcg<float>(h, h->h32, L, b32, x32, p32, q32, z32, r32, o->inner_rtol,
                           o->maxiter, o->precond, degree, check, &it, &rel, &st)))
        return rc;
      inf.iters += it;
      inf.outer = outer;
      k_add_f32_to_f64<<<gridsize(h, nl), kBlock, 0, h->stream>>>(nl, x32, U);
      // R = Fe - K64 U
      if ((rc = spmv<double>(h, h->ls[0], h->bs, L, 1, false, h->vals64_0.as<double>(), U,
                             h->fe.as<double>(), h->R.as<double>())))
        return rc;
      if ((rc = dot<double>(h, n, L, h->R.as<double>(), h->R.as<double>(), 7))) return rc;
      if ((rc = read_slot(h, 7, L, rn2))) return rc;
      double rel_out = 0.0;
      bool bad = false;
      for (int j = 0; j < L; ++j) {
        if (!std::isfinite(rn2[j])) bad = true;
        if (bn2[j] > 0.0) rel_out = std::max(rel_out, std::sqrt(rn2[j] / bn2[j]));
      }
      inf.relres = rel_out;
      if (bad || st == TOPT_NONFINITE) { inf.status = TOPT_NONFINITE; break; }
      if (rel_out <= o->rtol) { inf.status = TOPT_OK; break; }
    }
  }
  if (compliance) {
    if ((rc = dot<double>(h, n, L, h->fe.as<double>(), U, 7))) return rc;
    if ((rc = read_slot(h, 7, L, compliance))) return rc;
  }
  if (info) *info = inf;
  return TOPT_OK;
}

int topt_fem_energy(topt_fem* h, const double* U, int32_t nrhs, const double* rho, double E0,
                    double Emin, double p, const double* dh, double* energy, double* dc) {
  if (!h || !U || !rho) return fail(TOPT_BAD_INPUT, "fem_energy: null argument");
  if (nrhs < 1 || nrhs > 8) return fail(TOPT_BAD_INPUT, "fem_energy: nrhs must be 1..8");
  const int nd = h->bs * h->nloc;
  const int64_t stride = h->n_ke == 1 ? 0 : (int64_t)nd * nd;
  const int g = gridsize(h, h->n_elem, 128);
  const int32_t* t = h->ls[0].t.as<int32_t>();
#define TOPT_ENERGY(TC, KE)                                                                    \
  do {                                                                                         \
    const size_t sh = stride == 0 ? sizeof(TC) * nd * nd : 0;                                  \
    const TC* ke = KE;                                                                         \
    if (h->bs == 3 && h->nloc == 8)                                                            \
      k_energy<3, 8, TC><<<g, 128, sh, h->stream>>>(h->n_elem, nrhs, t, ke, stride, U, rho, E0, \
                                                    Emin, p, dh, energy, dc, h->interp);       \
    else if (h->bs == 3)                                                                       \
      k_energy<3, 4, TC><<<g, 128, sh, h->stream>>>(h->n_elem, nrhs, t, ke, stride, U, rho, E0, \
                                                    Emin, p, dh, energy, dc, h->interp);       \
    else if (h->nloc == 8)                                                                     \
      k_energy<1, 8, TC><<<g, 128, sh, h->stream>>>(h->n_elem, nrhs, t, ke, stride, U, rho, E0, \
                                                    Emin, p, dh, energy, dc, h->interp);       \
    else                                                                                       \
      k_energy<1, 4, TC><<<g, 128, sh, h->stream>>>(h->n_elem, nrhs, t, ke, stride, U, rho, E0, \
                                                    Emin, p, dh, energy, dc, h->interp);       \
  } while (0)
  if (h->energy32)
    TOPT_ENERGY(float, h->ke32.as<float>());
  else
    TOPT_ENERGY(double, h->ke64.as<double>());
#undef TOPT_ENERGY
  TOPT_CHECK_LAUNCH("k_energy");
  return TOPT_OK;
}

int topt_fem_set_energy_precision(topt_fem* h, int32_t fp32) {
  if (!h) return fail(TOPT_BAD_INPUT, "fem_set_energy_precision: null handle");
  if (fp32 != 0 && fp32 != 1)
    return fail(TOPT_BAD_INPUT, "fem_set_energy_precision: fp32 must be 0 or 1");
  h->energy32 = fp32 != 0;
  return TOPT_OK;
}

}  // extern "C"

namespace topt {
int launches_fem(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}
}  // namespace topt
