// Filter / design-set handle shared by the filter and design-operation units.
#pragma once

#include <vector>

#include "cuda_common.cuh"

namespace topt {

static const int kFB = 256;

// Device-resident state of an OC bisection (oc.py:16-95).
struct OcState {
  double l1, l2, lmid, vol_error;
  int it, done, steps;
  int need64;   // the FP32 volume of this step was too close to a decision edge
};

}  // namespace topt

// A design set (design / non-design element ids) with, for the Gaussian
// filter, the row-normalised matrix W over the design elements and its
// transpose; the identity filter has W = I.  Also owns the scratch of the OC
// bisection and of the design-indexed reductions.
struct topt_filter {
  int64_t n_elem = 0, n_design = 0, nnz = 0;
  cudaStream_t stream = nullptr;
  int sm = 152;
  std::vector<int32_t> h_rowptr, h_colind;   // design-local columns
  std::vector<double> h_vals;
  topt::DevBuf design, nondesign;            // element ids
  topt::DevBuf rowptr, colfull, vals;        // W with full-element columns
  topt::DevBuf t_rowptr, t_colfull, t_vals;  // W^T
  int64_t n_nondesign = 0;
  // OC work
  topt::DevBuf cand, state, partials, counter, rho_e, rho_new;
  // FP32 bracketing of the bisection: W in FP32 and per-step inputs
  topt::DevBuf vals32, cand32, oc32;
  // the same W as a stencil when the elements are the cells of an nx x ny x nz
  // grid (e = ey + ny (ex + nx ez)) and every row has the translation-invariant
  // form W_kj = g(j - i) W_kk: offsets with unnormalised weights g (int4:
  // dx, dy, dz, float bits of g), W_kk per design row, the design mask
  int grid[3] = {0, 0, 0};
  int st_n = 0;                              // 0: no stencil
  topt::DevBuf st_invd;                      // W_kk per design row (float)
  topt::DevBuf st_lin, st_g;                 // linear offset and weight per offset
  topt::DevBuf st_nb;                        // per design row: bit o = neighbour o present
};
