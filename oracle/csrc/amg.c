/* Serial kernels of the oracle's smoothed-aggregation AMG (TEST
 * INFRASTRUCTURE; see oracle/amg.py).  Restated from the published
 * algorithms of PyAMG 5.x (a dependency of the reference, pyproject.toml:23,
 * absent from the reference tree), whose own kernels are compiled C++:
 *
 *   oracle_standard_aggregation  greedy three-pass aggregation of a strength
 *                                graph (Vanek, Mandel, Brezina 1996, the
 *                                "standard" scheme of PyAMG's SA solver)
 *   oracle_gauss_seidel          one Gauss-Seidel sweep over rows
 *                                start, start+step, ... (stop excluded)
 *
 * Plain C99 on CSR arrays (int64 indices, double values); no allocation. */
#include <stdint.h>

/* Aggregate the nodes of the graph (Ap, Aj) (self loops ignored).
 *   pass 1: a node whose neighbours are all unaggregated becomes a root and
 *           takes all of them into a new aggregate;
 *   pass 2: each node still free joins the aggregate of its first
 *           neighbour that is in a pass-1 aggregate;
 *   pass 3: each node still free becomes a root of a new aggregate with its
 *           free neighbours.
 * A node without neighbours stays unaggregated (agg = -1).
 * agg[i] = aggregate of node i, roots[a] = root node of aggregate a.
 * Returns the number of aggregates. */
int64_t oracle_standard_aggregation(int64_t n, const int64_t* Ap, const int64_t* Aj,
                                    int64_t* agg, int64_t* roots) {
  /* passes 1-2: 0 free, k > 0 in pass-1 aggregate k-1, -k joined aggregate
     k-1 in pass 2, -(n+1) isolated */
  int64_t next = 1;
  for (int64_t i = 0; i < n; ++i) agg[i] = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (agg[i] != 0) continue;
    int neighbours = 0, taken = 0;
    for (int64_t jj = Ap[i]; jj < Ap[i + 1]; ++jj) {
      const int64_t j = Aj[jj];
      if (j == i) continue;
      neighbours = 1;
      if (agg[j] != 0) { taken = 1; break; }
    }
    if (!neighbours) {
      agg[i] = -(n + 1);
    } else if (!taken) {
      agg[i] = next;
      roots[next - 1] = i;
      for (int64_t jj = Ap[i]; jj < Ap[i + 1]; ++jj) agg[Aj[jj]] = next;
      ++next;
    }
  }
  for (int64_t i = 0; i < n; ++i) {
    if (agg[i] != 0) continue;
    for (int64_t jj = Ap[i]; jj < Ap[i + 1]; ++jj) {
      const int64_t a = agg[Aj[jj]];
      if (a > 0) { agg[i] = -a; break; }
    }
  }
  --next;   /* aggregates so far: 0 .. next-1 */
  for (int64_t i = 0; i < n; ++i) {   /* final numbering; -2 marks free */
    const int64_t a = agg[i];
    if (a == 0) agg[i] = -2;
    else if (a == -(n + 1)) agg[i] = -1;
    else if (a > 0) agg[i] = a - 1;
    else agg[i] = -a - 1;
  }
  for (int64_t i = 0; i < n; ++i) {
    if (agg[i] != -2) continue;
    agg[i] = next;
    roots[next] = i;
    for (int64_t jj = Ap[i]; jj < Ap[i + 1]; ++jj) {
      const int64_t j = Aj[jj];
      if (agg[j] == -2) agg[j] = next;
    }
    ++next;
  }
  return next;
}

/* x[i] = (b[i] - sum_{j != i} a_ij x[j]) / a_ii for i = start, start+step,
 * ..., stop excluded (rows with a zero diagonal are left alone). */
void oracle_gauss_seidel(const int64_t* Ap, const int64_t* Aj, const double* Ax, double* x,
                         const double* b, int64_t start, int64_t stop, int64_t step) {
  for (int64_t i = start; i != stop; i += step) {
    double s = 0.0, d = 0.0;
    for (int64_t jj = Ap[i]; jj < Ap[i + 1]; ++jj) {
      const int64_t j = Aj[jj];
      if (j == i) d = Ax[jj];
      else s += Ax[jj] * x[j];
    }
    if (d != 0.0) x[i] = (b[i] - s) / d;
  }
}
