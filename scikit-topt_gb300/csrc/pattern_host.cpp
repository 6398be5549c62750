// Host-side sparsity pattern of an element mesh (no GPU).
//
// Replaces the COO -> CSR step of scikit-fem ``asm`` + ``.tocsr()`` used by
// sktopt/fea/composer.py:80-100 and sktopt/fea/solver_elastic.py:205: two
// nodes are coupled when they share an element, column indices are sorted,
// and every (element, local row node, local column node) triple is mapped
// once to the block it is summed into.  The contribution list of a block is
// in ascending element order, which fixes the summation order of assembly
// and makes it deterministic.
#include "topt_internal.h"

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

struct topt_pattern {
  int64_t n_nodes = 0, n_elem = 0;
  int32_t nloc = 0;
  std::vector<int32_t> rowptr, colind;
  std::vector<int64_t> cptr;
  std::vector<int32_t> contrib;
};

namespace topt {

int build_pattern(int64_t n_nodes, int64_t n_elem, int32_t nloc,
                  const int32_t* t, topt_pattern* P) {
  if (n_nodes <= 0 || n_elem <= 0 || nloc <= 0 || nloc > 32 || !t)
    return fail(TOPT_BAD_INPUT, "pattern: bad sizes");
  if (n_elem * (int64_t)nloc * nloc >= (int64_t)INT32_MAX)
    return fail(TOPT_BAD_INPUT, "pattern: too many element contributions");
  for (int64_t i = 0; i < n_elem * nloc; ++i)
    if (t[i] < 0 || t[i] >= n_nodes)
      return fail(TOPT_BAD_INPUT, "pattern: node index out of range");
  P->n_nodes = n_nodes;
  P->n_elem = n_elem;
  P->nloc = nloc;
  // node -> element incidence (elements ascending)
  std::vector<int64_t> inc_ptr(n_nodes + 1, 0);
  for (int32_t a = 0; a < nloc; ++a)
    for (int64_t e = 0; e < n_elem; ++e) inc_ptr[t[a * n_elem + e] + 1]++;
  for (int64_t i = 0; i < n_nodes; ++i) inc_ptr[i + 1] += inc_ptr[i];
  std::vector<int32_t> inc(inc_ptr[n_nodes]);
  {
    std::vector<int64_t> pos(inc_ptr.begin(), inc_ptr.end() - 1);
    for (int64_t e = 0; e < n_elem; ++e)
      for (int32_t a = 0; a < nloc; ++a) inc[pos[t[a * n_elem + e]]++] = (int32_t)e;
  }
  // neighbours of every node
  P->rowptr.assign(n_nodes + 1, 0);
  std::vector<int32_t> stamp(n_nodes, -1);
  std::vector<int32_t> row;
  row.reserve(256);
  std::vector<int32_t> cols;
  cols.reserve((size_t)n_nodes * 27);
  for (int64_t i = 0; i < n_nodes; ++i) {
    row.clear();
    for (int64_t k = inc_ptr[i]; k < inc_ptr[i + 1]; ++k) {
      int64_t e = inc[k];
      for (int32_t a = 0; a < nloc; ++a) {
        int32_t j = t[a * n_elem + e];
        if (stamp[j] != (int32_t)i) {
          stamp[j] = (int32_t)i;
          row.push_back(j);
        }
      }
    }
    std::sort(row.begin(), row.end());
    cols.insert(cols.end(), row.begin(), row.end());
    P->rowptr[i + 1] = (int32_t)cols.size();
    if (cols.size() >= (size_t)INT32_MAX)
      return fail(TOPT_BAD_INPUT, "pattern: too many blocks");
  }
  P->colind.swap(cols);
  const int64_t nnzb = (int64_t)P->colind.size();
  // block index of every contribution
  const int64_t nc = n_elem * nloc * nloc;
  std::vector<int32_t> kidx(nc);
  P->cptr.assign(nnzb + 1, 0);
  for (int64_t e = 0; e < n_elem; ++e) {
    for (int32_t la = 0; la < nloc; ++la) {
      const int32_t a = t[la * n_elem + e];
      const int32_t* b0 = P->colind.data() + P->rowptr[a];
      const int32_t* b1 = P->colind.data() + P->rowptr[a + 1];
      for (int32_t lb = 0; lb < nloc; ++lb) {
        const int32_t b = t[lb * n_elem + e];
        const int32_t* it = std::lower_bound(b0, b1, b);
        int64_t k = P->rowptr[a] + (it - b0);
        kidx[(e * nloc + la) * nloc + lb] = (int32_t)k;
        P->cptr[k + 1]++;
      }
    }
  }
  for (int64_t k = 0; k < nnzb; ++k) P->cptr[k + 1] += P->cptr[k];
  P->contrib.resize(nc);
  {
    std::vector<int64_t> pos(P->cptr.begin(), P->cptr.end() - 1);
    for (int64_t c = 0; c < nc; ++c) P->contrib[pos[kidx[c]]++] = (int32_t)c;
  }
  return TOPT_OK;
}

}  // namespace topt

extern "C" {

int topt_pattern_build(int64_t n_nodes, int64_t n_elem, int32_t nloc,
                       const int32_t* t, topt_pattern** out) {
  if (!out) return topt::fail(TOPT_BAD_INPUT, "pattern: null out");
  *out = nullptr;
  topt_pattern* P = new (std::nothrow) topt_pattern();
  if (!P) return topt::fail(TOPT_NO_MEMORY, "pattern: out of host memory");
  int rc;
  try {
    rc = topt::build_pattern(n_nodes, n_elem, nloc, t, P);
  } catch (const std::bad_alloc&) {
    rc = topt::fail(TOPT_NO_MEMORY, "pattern: out of host memory");
  }
  if (rc != TOPT_OK) {
    delete P;
    return rc;
  }
  *out = P;
  return TOPT_OK;
}

int topt_pattern_sizes(const topt_pattern* p, int64_t* nnzb, int64_t* ncontrib) {
  if (!p) return topt::fail(TOPT_BAD_INPUT, "pattern: null handle");
  if (nnzb) *nnzb = (int64_t)p->colind.size();
  if (ncontrib) *ncontrib = (int64_t)p->contrib.size();
  return TOPT_OK;
}

int topt_pattern_export(const topt_pattern* p, int32_t* rowptr, int32_t* colind,
                        int64_t* cptr, int32_t* contrib) {
  if (!p) return topt::fail(TOPT_BAD_INPUT, "pattern: null handle");
  if (rowptr) std::memcpy(rowptr, p->rowptr.data(), p->rowptr.size() * 4);
  if (colind) std::memcpy(colind, p->colind.data(), p->colind.size() * 4);
  if (cptr) std::memcpy(cptr, p->cptr.data(), p->cptr.size() * 8);
  if (contrib) std::memcpy(contrib, p->contrib.data(), p->contrib.size() * 4);
  return TOPT_OK;
}

void topt_pattern_free(topt_pattern* p) { delete p; }

}  // extern "C"

namespace topt {
const topt_pattern_view view_of(const topt_pattern* p) {
  topt_pattern_view v;
  v.n_nodes = p->n_nodes;
  v.nnzb = (int64_t)p->colind.size();
  v.ncontrib = (int64_t)p->contrib.size();
  v.rowptr = p->rowptr.data();
  v.colind = p->colind.data();
  v.cptr = p->cptr.data();
  v.contrib = p->contrib.data();
  return v;
}
}  // namespace topt
