/*
 * topt.h -- C ABI of libtopt_gb300, the GB300 (sm_103a) engine behind the
 * scikit-topt density-method hot path.
 *
 * Every entry point takes plain pointers and sizes.  Device pointers are
 * marked "dev"; everything else is host memory.  Functions return a status
 * code (TOPT_OK on success); topt_last_error() gives the message of the most
 * recent failure on the calling thread.  Work is issued on the stream set on
 * the handle (default stream when none was set) and is stream-ordered; a
 * handle is not thread-safe.
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the scikit-topt project root).  The reference is a Python library whose
 * plugin objects (FEM, filter, rho_update) are duck-typed; these functions are
 * what those objects call through ctypes.
 */
#ifndef TOPT_GB300_H
#define TOPT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define TOPT_OK 0
#define TOPT_MAXITER 1      /* an iterative method stopped at its cap      */
#define TOPT_NONFINITE 2    /* NaN/Inf met in a residual or reduction      */
#define TOPT_BREAKDOWN 3    /* CG breakdown (p.Ap <= 0)                     */
#define TOPT_BAD_INPUT 4    /* invalid argument, size or index             */
#define TOPT_CUDA_ERROR 5   /* a CUDA runtime call failed                   */
#define TOPT_NO_MEMORY 6    /* device or host allocation failed            */

/* value types */
#define TOPT_F64 0
#define TOPT_F32 1
#define TOPT_F64_FULL 2   /* topt_fem_spmv: FP64 operator before enforcement */

const char* topt_version(void);
const char* topt_last_error(void);
/* Number of kernels this library has launched in the process (counted on the
 * device by every launch; synchronises with the device). */
int topt_launch_count(uint64_t* out);

/* ------------------------------------------------------------------------
 * Sparsity pattern (host only, no GPU).
 * Replaces the COO->CSR conversion of scikit-fem ``asm`` + ``.tocsr()``
 * (sktopt/fea/composer.py:80-100, sktopt/fea/solver_elastic.py:205).
 * Nodes i, j are coupled when they share an element; columns are sorted.
 * The scalar CSR with interleaved DOFs bs*node+comp is the bs x bs block
 * expansion of this node pattern.  contrib lists, per block, the element
 * contributions e*nloc*nloc + la*nloc + lb in ascending element order.
 * ---------------------------------------------------------------------- */
typedef struct topt_pattern topt_pattern;
int topt_pattern_build(int64_t n_nodes, int64_t n_elem, int32_t nloc,
                       const int32_t* t /* (nloc, n_elem) row-major */,
                       topt_pattern** out);
int topt_pattern_sizes(const topt_pattern* p, int64_t* nnzb, int64_t* ncontrib);
int topt_pattern_export(const topt_pattern* p, int32_t* rowptr /* n_nodes+1 */,
                        int32_t* colind /* nnzb */, int64_t* cptr /* nnzb+1 */,
                        int32_t* contrib /* ncontrib */);
void topt_pattern_free(topt_pattern* p);

/* ------------------------------------------------------------------------
 * FEM handle: SIMP-scaled stiffness / conductivity, Dirichlet enforcement,
 * preconditioned CG (FP64, or FP32-inner with FP64 iterative refinement),
 * element energies and compliance sensitivities.
 * Replaces FEM_SimpLinearElasticity (sktopt/fea/solver_elastic.py:540-676)
 * and FEM_SimpLinearHeatConduction (sktopt/fea/solver_heat.py:628-980).
 * ---------------------------------------------------------------------- */
typedef struct topt_fem topt_fem;

typedef struct topt_fem_desc {
  int32_t bs;                 /* DOFs per node: 3 elasticity, 1 conduction   */
  int32_t nloc;               /* nodes per element: 8 hex, 4 tet             */
  int64_t n_nodes;
  int64_t n_elem;
  const int32_t* t;           /* (nloc, n_elem) row-major connectivity       */
  const double* ke;           /* unit element matrices, n_ke x (bs*nloc)^2   */
  int64_t n_ke;               /* 1 (shared by all elements) or n_elem        */
  const uint8_t* dirichlet;   /* per-DOF flag (bs*n_nodes), 1 = fixed        */
  int32_t grid[3];            /* logical cell grid for multigrid; 0 = none   */
  const int32_t* node_ijk;    /* (3, n_nodes) logical node coords, or NULL   */
  const int32_t* cell_of_elem;/* logical cell of each element, or NULL (id)  */
  int32_t mixed;              /* keep an FP32 operator + hierarchy as well   */
  int32_t mg_levels;          /* max multigrid levels (1 = no coarsening)    */
  int32_t mg_coarse_max;      /* dense direct solve at <= this many DOFs     */
  int32_t mf_level0;          /* mixed, uniform hex elasticity: apply the FP32
                                 fine-level operator matrix-free from the
                                 shared element matrix (no FP32 assembly)    */
  int32_t amg;                /* no logical grid: 1 = smoothed-aggregation
                                 multigrid built on the GPU (replaces
                                 pyamg.smoothed_aggregation_solver of the
                                 cg_pyamg solve, solver_elastic.py:94-103),
                                 up to mg_levels levels; 0 = block Jacobi    */
} topt_fem_desc;

int topt_fem_create(const topt_fem_desc* d, topt_fem** out);
void topt_fem_destroy(topt_fem* h);
int topt_fem_set_stream(topt_fem* h, void* cuda_stream);
int topt_fem_sizes(const topt_fem* h, int64_t* n_dof, int64_t* nnzb,
                   int32_t* n_levels);

/* coef_e = Emin + (E0-Emin) rho_e^p (composer.py:19-22), K = sum coef_e Ke
 * assembled into the fixed pattern (composer.py:53-145), Dirichlet rows and
 * columns zeroed with unit diagonal (skfem.enforce, solver_elastic.py:211),
 * then the preconditioner refreshed.  rho: dev, n_elem doubles. */
int topt_fem_update(topt_fem* h, const double* rho, double E0, double Emin,
                    double p);
/* Material interpolation of the later topt_fem_update / topt_fem_energy calls:
 * kind 0 SIMP (default; composer.py:19-22, dC_drho_simp derivatives.py:25-52),
 * 1 RAMP E = Emin + (E0 - Emin) rho / (1 + p (1 - rho)) (composer.py:25-39,
 * dC_drho_ramp derivatives.py:56-72), p being the RAMP parameter; 2 the RAMP
 * operator and energy with the dC_drho_simp sensitivity (the heat plugin's
 * compliance_sensitivity_multi_load, solver_heat.py:928-950). */
int topt_fem_set_interpolation(topt_fem* h, int32_t kind);

/* Per-element matrices added, unscaled, to coef_e Ke in the level-0 operator,
 * its Galerkin coarse levels and the TOPT_F64_FULL product from the next
 * topt_fem_update on (the Robin terms of solve_multi_load,
 * solver_heat.py:198-253).  extra: dev, n_elem x (bs nloc)^2 FP64, row-major
 * per element, kept by pointer (the caller keeps it alive and refreshes it
 * before each update); NULL removes the terms.  Element energies and
 * sensitivities (topt_fem_energy) keep the conduction part only.  Not
 * available on handles with the matrix-free FP32 operator. */
int topt_fem_set_element_extra(topt_fem* h, const double* extra);

/* Kernel of the matrix-free FP32 level-0 operator (handles created with
 * mf_level0 on a uniform hex grid): 0 = FP32 FMA tiles (the default),
 * 1 = tensor cores (tcgen05, TF32 with the 3xTF32 split, FP32-accurate).  Both compute
 * the same operator (the element products of composer.py:53-101 on one unit
 * matrix, enforce as identity rows); they differ by rounding only.
 * mf_error (may be NULL) receives 1 if a tensor-core launch gave up on one
 * of its bounded waits (the operator then also wrote a NaN into its output,
 * so the solve ends with TOPT_NONFINITE).  No reference counterpart: the
 * reference assembles with scikit-fem and multiplies with SciPy. */
int topt_fem_set_mf_kernel(topt_fem* h, int32_t kind);
/* V-cycle replay: on = 1 (the default) records one multigrid
 * preconditioner application as a CUDA graph after the first application of
 * each operator update and replays it (one graph launch per application
 * instead of one launch per kernel); on = 0 launches every kernel.  Same
 * kernels, same arguments, same results.  No reference counterpart (PyAMG's
 * V-cycle is host code, solver_elastic.py:84-103). */
int topt_fem_set_vcycle_graphs(topt_fem* h, int32_t on);
int topt_fem_mf_error(topt_fem* h, int32_t* mf_error);

/* Launch shapes, for an autotuner (no reference counterpart; none of them
 * changes what is computed, only the tiling, so results differ by rounding
 * at most):
 * - set_mf_tile: node rows per tile of the FP32-FMA fine-level operator,
 *   16, 27 or 32, 0 = the rule (least padding of ny + 1);
 * - set_row_mapping: threads per block row of a level's SELL products,
 *   1 = a warp, 2 = three threads (bs 3), 3 = one thread, 0 = the rule by
 *   level size;
 * - get_tuning: the tile in use (0 without the matrix-free operator) and the
 *   mapping of each of the first n_levels levels (0 for the dense level);
 * - spmv_level: y = A_level x (one column) with the level's operator of the
 *   handle's hierarchy precision (FP32 for mixed handles, FP64 otherwise),
 *   dev pointers; the timing target. */
int topt_fem_set_mf_tile(topt_fem* h, int32_t ty);
int topt_fem_set_row_mapping(topt_fem* h, int32_t level, int32_t mapping);
int topt_fem_get_tuning(const topt_fem* h, int32_t* mf_tile, int32_t* mappings,
                        int32_t n_levels);
int topt_fem_spmv_level(topt_fem* h, int32_t level, int32_t dtype, const void* x,
                        void* y);
/* Average device time in microseconds of one topt_fem_spmv_level product
 * (same arguments), measured over `reps` (1..1000) back-to-back products
 * replayed as a CUDA graph, without host launch overhead: the launch-shape
 * autotuner's measurement.  Synchronises the handle's stream. */
int topt_fem_time_spmv_level(topt_fem* h, int32_t level, int32_t dtype, const void* x,
                             void* y, int32_t reps, double* us);
/* Nodes (block rows) of each of the first n_levels levels and whether the
 * level is the dense coarsest one. */
int topt_fem_level_sizes(const topt_fem* h, int64_t* n_nodes, int32_t* dense,
                         int32_t n_levels);

typedef struct topt_solve_opts {
  int32_t method;         /* 0: FP64 PCG.  Mixed (FP32 operator, hierarchy and
                             inner work; FP64 residual, update and dots):
                             1: FP32 PCG with FP64 reliable updates;
                             2: FP32 PCG restarted inside FP64 refinement;
                             3: FP64 flexible CG around an FP32 V-cycle;
                             4: flexible CG with FP32 recurrences and
                                operator, FP64 solution and FP64 residual
                                replacement, around the FP32 V-cycle      */
  int32_t precond;        /* 0: block Jacobi; 1: multigrid V-cycle           */
  double rtol;            /* relative residual target (solver_elastic.py:37) */
  int32_t maxiter;        /* iteration cap (per inner solve for method 2)    */
  double inner_rtol;      /* 1, 4: residual drop between updates; 2: inner
                             tolerance                                       */
  int32_t max_outer;      /* 1, 2: cap on FP64 refinement steps; 4: most
                             iterations between residual replacements       */
  int32_t cheb_degree;    /* Chebyshev smoother degree                       */
  int32_t check_every;    /* residual check period (iterations)              */
  double cheb_ratio;      /* Chebyshev interval [lmax/ratio, lmax] (0: 30)   */
  int32_t x0;             /* methods 0, 3, 4: start from U (its fixed DOFs are
                             zeroed) instead of 0; same stopping rule          */
  int32_t pad;
} topt_solve_opts;

typedef struct topt_solve_info {
  int32_t status;
  int32_t iters;          /* FP64 PCG iterations, or inner iterations total  */
  int32_t outer;          /* refinement steps (mixed)                        */
  int32_t pad;
  double relres;          /* final max over columns of ||f-Ku|| / ||f||      */
} topt_solve_info;

/* Solve K_e U = F_e for nrhs load cases (solve_u solver_elastic.py:61-143,
 * solve_multi_load 240-395).  F, U: dev, n_dof x nrhs row-major (the layout
 * of the reference's u_dofs); F is enforced (Dirichlet entries zeroed) in a
 * copy; U is overwritten.  compliance (host, nrhs) receives F_e . U
 * (solver_elastic.py:236, 465), or may be NULL. */
int topt_fem_solve(topt_fem* h, const double* F, double* U, int32_t nrhs,
                   const topt_solve_opts* o, topt_solve_info* info,
                   double* compliance);

/* y = K x with the enforced operator (dtype TOPT_F64 or TOPT_F32; F32 needs
 * mixed), or with the FP64 operator before enforcement (TOPT_F64_FULL: the
 * K_csr of solve_multi_load, solver_heat.py:220-237, used for T^T K T and for
 * nonzero Dirichlet values; assembled on first use after each update).
 * x, y: dev, n_dof x nrhs row-major. */
int topt_fem_spmv(topt_fem* h, int32_t dtype, const void* x, void* y,
                  int32_t nrhs);

/* Copy the enforced FP64 block values (nnzb x bs x bs) to dev memory. */
int topt_fem_export_values(topt_fem* h, double* vals);

/* Smoothed-aggregation hierarchy (desc.amg = 1), for inspection and tests:
 * sizes of the transfer from `level` to level + 1 (fine nodes, coarse nodes,
 * blocks of P), and a HOST copy of it after an update: the aggregate of
 * every fine node, lambda_max(Dinv A) used for the smoothing, P in CSR
 * (p_ptr: n_fine + 1, p_col: n_p, p_vals: n_p x bs x bs) and the coarse
 * operator as a dense (bs n_coarse)^2 row-major matrix (at most 8192 rows).
 * dtype 1: the FP64 hierarchy; 0: the FP32 one (mixed handles).  The
 * reference's PyAMG hierarchy (solver_elastic.py:95) has no such export. */
int topt_fem_amg_sizes(const topt_fem* h, int32_t level, int64_t* n_fine,
                       int64_t* n_coarse, int64_t* n_p);
int topt_fem_amg_export(topt_fem* h, int32_t dtype, int32_t level,
                        int32_t* agg, double* lmax, int64_t* p_ptr,
                        int32_t* p_col, double* p_vals, double* coarse);

/* Element energies 1/2 coef_e u_e^T Ke u_e (solver_elastic.py:507-537,
 * solver_heat.py:282-303) for every load case and, when dc != NULL, the
 * compliance sensitivity dC_drho_simp (derivatives.py:42-52) times dh
 * (dh may be NULL = 1).  rho: the density the operator was built from.
 * U: dev n_dof x nrhs; energy, dc: dev n_elem x nrhs row-major. */
int topt_fem_energy(topt_fem* h, const double* U, int32_t nrhs,
                    const double* rho, double E0, double Emin, double p,
                    const double* dh, double* energy, double* dc);
/* Arithmetic of topt_fem_energy: fp32 = 1 computes u_e^T Ke u_e in FP32 from
 * the FP64 displacements (shifted by node 0) and returns FP64 energies and
 * sensitivities (1.2e-6 relative L2 on the sensitivities of the 240x80x80
 * loop); fp32 = 0: FP64 throughout (the default). */
int topt_fem_set_energy_precision(topt_fem* h, int32_t fp32);

/* ------------------------------------------------------------------------
 * Gaussian density filter (SpacialFilter, sktopt/filters/spacial.py:106-166;
 * kernel spacial.py:37-45, matrix spacial.py:51-103).  W is built once per
 * radius over the design elements and row-normalised.
 * ---------------------------------------------------------------------- */
typedef struct topt_filter topt_filter;
int topt_filter_gauss_create(int64_t n_elem, const double* centers /* 3 x n */,
                             const uint8_t* design_mask, double radius,
                             topt_filter** out);
void topt_filter_destroy(topt_filter* f);
int topt_filter_set_stream(topt_filter* f, void* cuda_stream);
/* Declare the elements to be the cells of an nx x ny x nz grid (element
 * e = ey + ny (ex + nx ez), the structured hex meshes).  When every row of W
 * has the translation-invariant form W_kj = g(j - i) W_kk (checked against
 * the whole matrix), the FP32 bracketing steps of topt_oc_bisect apply W as
 * a stencil instead of the CSR; results and the FP64 steps are unchanged.
 * n_offsets (topt_filter_stencil_size) is 0 when the check failed. */
int topt_filter_set_grid(topt_filter* f, int32_t nx, int32_t ny, int32_t nz);
int topt_filter_stencil_size(const topt_filter* f, int32_t* n_offsets);
int topt_filter_sizes(const topt_filter* f, int64_t* n_design, int64_t* nnz);
/* host export of W (design x design CSR) for checks */
int topt_filter_export(const topt_filter* f, int32_t* rowptr, int32_t* colind,
                       double* vals);
/* forward: y[design] = W x[design], y = x elsewhere (spacial.py:135-157) */
int topt_filter_forward(topt_filter* f, const double* x, double* y);
/* gradient: y[design] = W^T v[design], 0 elsewhere (spacial.py:159-166) */
int topt_filter_gradient(topt_filter* f, const double* v, double* y);

/* ------------------------------------------------------------------------
 * Element-wise kernels, reductions and the density updates.
 * ---------------------------------------------------------------------- */
/* Heaviside projection and derivative (projection.py:27-118); either output
 * may be NULL. */
int topt_projection(int64_t n, const double* x, double beta, double eta,
                    double* h, double* dh, void* stream);

/* OC bisection on the volume multiplier (oc.py:16-95) with the filter and
 * projection applied to every candidate.  The design set is the filter's.
 * dc: full-length sensitivities, divided by dc_scale on the fly (the
 * running-scale normalisation of oc.py:186-196); rho: full-length density,
 * its design entries replaced by the accepted candidate; vol: design-element
 * volumes (design order).  scaling (design order, may be NULL) receives the
 * clipped multiplicative factor; lmid, vol_error, steps (host) the
 * bisection result.  Unless flags has TOPT_OC_EXACT, each step first
 * evaluates the volume in FP32 and re-evaluates it in FP64 only when the
 * FP32 error is within its rounding bound of a decision edge (0 or vol_tol),
 * so the sequence of brackets, the result and vol_error are those of the
 * all-FP64 bisection. */
typedef struct topt_oc_params {
  double rho_min, rho_max, move_limit, eta, eps, vol_frac, beta, beta_eta;
  double scaling_min, scaling_max, vol_tol, l1, l2, tolerance;
  int32_t max_iter;
  int32_t flags;   /* TOPT_OC_EXACT: evaluate every bisection step in FP64 */
} topt_oc_params;
#define TOPT_OC_EXACT 1
int topt_oc_bisect(topt_filter* f, const double* dc, double dc_scale, double* rho,
                   const double* vol, double vol_sum, const topt_oc_params* prm,
                   double* scaling, double* lmid, double* vol_error, int32_t* steps);

/* Reductions over the filter's design elements (host result):
 * op 0: max |x[d]|            (oc.py:186-191 sensitivity scale)
 * op 1: max |x[d] - y[d]|     (common_density.py:1137-1141 rho_change_max)
 * op 2: max |x[d] + c w[i]| over interior y[d] in (rho_min+1e-6, rho_max-1e-6)
 *       (oc.py:230-240 KKT residual; w in design order). */
int topt_design_reduce(topt_filter* f, int32_t op, const double* x, const double* y,
                       const double* w, double c, double rho_min, double rho_max,
                       double* out);

/* Identity filter (W = I on the design elements): a design-set handle for the
 * stepwise bisection and the design operations below when the density filter
 * is not a fixed matrix (HelmholtzFilterNodal, helmholtz_filter_nodal.py). */
int topt_filter_identity_create(int64_t n_elem, const uint8_t* design_mask,
                                topt_filter** out);

/* The OC bisection one step at a time (oc.py:16-95) for any filter:
 * topt_oc_begin gathers the current design densities and resets the
 * multiplier bracket; each step, topt_oc_candidate writes the candidate's
 * design entries into `cand` (full length; the caller keeps the non-design
 * entries), the caller filters cand, and topt_oc_volume projects the
 * filtered field, sums the design volume and advances the bracket (host
 * outputs; done = 1 once a stopping rule of oc.py:81-86 fired);
 * topt_oc_finish writes the accepted candidate into rho. */
int topt_oc_begin(topt_filter* f, const double* rho, const topt_oc_params* prm);
int topt_oc_candidate(topt_filter* f, const double* dc, double dc_scale,
                      const topt_oc_params* prm, double* cand, double* scaling);
int topt_oc_volume(topt_filter* f, const double* filtered, const double* vol,
                   double vol_sum, const topt_oc_params* prm, int32_t* done,
                   double* lmid, double* vol_error, int32_t* steps);
int topt_oc_finish(topt_filter* f, double* rho);

/* out[i] = x[d_i] + c y[d_i] over the design elements d_i (y may be NULL);
 * the LogMOC Lagrangian gradient dL = dC + coeff dV_chain (logmoc.py:
 * 204-215). */
int topt_design_gather_axpy(topt_filter* f, const double* x, const double* y,
                            double c, double* out);
/* sum_i x[d_i] w[i] (host result; the design volume of logmoc.py:160-163). */
int topt_design_wsum(topt_filter* f, const double* x, const double* w,
                     double* out);
/* max |c w[i]| over interior design elements (logmoc.py:227-236). */
int topt_design_kkt(topt_filter* f, const double* rho, const double* w, double c,
                    double rho_min, double rho_max, double* out);
/* lagrangian_log_update (logmoc.py:36-66) with dL = dl * inv_scale on the
 * design elements of rho (in place); scaling (design order) may be NULL. */
int topt_logmoc_update(topt_filter* f, const double* dl, double inv_scale, double* rho,
                       double eta, double move_limit, double rho_min, double rho_max,
                       double lagrangian_clip, double* scaling);
/* numpy.percentile(|x[idx]|, q) with the default 'linear' method (radix
 * select, deterministic); idx may be NULL (all of x).  Used for the OC
 * percentile scaling (oc.py:186-189) and the LogMOC scale (logmoc.py:217-225). */
int topt_percentile_abs(int64_t n, const int32_t* idx, const double* x, double q,
                        double* out, void* stream);

/* Helmholtz nodal filter transfers (helmholtz_filter_nodal.py:26-56):
 * volume-weighted element -> node average over the node's elements (CSR
 * node_ptr/node_elems), non-design elements contributing fixed_value
 * (design may be NULL = all design); and node -> element mean, optionally
 * clamped to <= 0 (the gradient's clamp, helmholtz_filter_nodal.py:232). */
int topt_elem_to_node(int64_t n_nodes, const int32_t* node_ptr, const int32_t* node_elems,
                      const double* vol, const double* x, const uint8_t* design,
                      double fixed_value, double* out, void* stream);
int topt_node_to_elem(int64_t n_elem, int32_t nloc, const int32_t* t, const double* x_node,
                      int32_t clamp_nonpositive, double* out, void* stream);

/* ------------------------------------------------------------------------
 * Heat plugin on hexahedral and P1 tetrahedral meshes
 * (FEM_SimpLinearHeatConduction, sktopt/fea/solver_heat.py:306-625,
 * 705-980): Robin terms, heat-exchange objective and adjoint load, explicit
 * Robin gradient, grad T . grad lam.  Hexahedra take the 2x2x2 Gauss rule
 * (axis-aligned boxes from their extents; any other hexahedron switches the
 * handle to the trilinear map of the 8 nodes with the Jacobian at every
 * Gauss point, which must be positive: TOPT_BAD_INPUT otherwise);
 * tetrahedra take the 4-point degree-2 rule.  Vectors are dev, n_nodes (x L row-major for several
 * columns).
 * ---------------------------------------------------------------------- */
typedef struct topt_heat topt_heat;
/* t: host, 8 x n_elem (row a = local node a, MeshHex order); p: host,
 * 3 x n_nodes.  pairing 0 gives the nodal density average the reference's
 * pairing of t.ravel() with np.repeat(rho, 8) (solver_heat.py:600-613,
 * 730-737: node t[a][e] receives rho[(a n_elem + e) / 8]); 1 gives node
 * t[a][e] the density of element e. */
int topt_heat_create(int64_t n_nodes, int64_t n_elem, const int32_t* t, const double* p,
                     int32_t pairing, topt_heat** out);
/* The same for nloc = 8 (hexahedra, as above) or nloc = 4 (P1 tetrahedra:
 * volume forms with the 4-point degree-2 rule of a basis with intorder 2;
 * pairing 0 then gives node t[a][e] rho[(a n_elem + e) / 4]). */
int topt_heat_create_mesh(int64_t n_nodes, int64_t n_elem, int32_t nloc,
                          const int32_t* t, const double* p, int32_t pairing,
                          topt_heat** out);
void topt_heat_destroy(topt_heat* h);
int topt_heat_set_stream(topt_heat* h, void* cuda_stream);
/* Surface Robin matrices h int N_a N_b over the Robin facets
 * (assemble_surface_robin task_heat.py:60-139), one nloc x nloc per facet
 * in the owning element's local numbering.  elems, mats: host. */
int topt_heat_set_surface(topt_heat* h, int64_t n_faces, const int32_t* elems,
                          const double* mats);
/* rho_node = the nodal average of the element densities rho. */
int topt_heat_nodal_average(topt_heat* h, const double* rho, double* rho_node);
/* extra (dev, n_elem x 64) = virtual Robin element matrices
 * (get_robin_virtual solver_heat.py:552-572; when virtual_on) + surface
 * matrices; load (dev, may be NULL) = the virtual Robin load. */
int topt_heat_robin(topt_heat* h, const double* rho_node, double h_coef, double t_env,
                    double p, double q, int32_t virtual_on, double* extra, double* load);
/* den = int |grad rho| and num[j] = int -T_env h (T_j - T_env) |grad rho|
 * (solver_heat.py:306-321, 382-390, 411-440) for L <= 4 columns of T
 * (L = 0: den only).  den, num: host. */
int topt_heat_exchange(topt_heat* h, const double* rho_node, const double* T, int32_t L,
                       double h_coef, double t_env, double* den, double* num);
/* rhs = (int -T_env h_eff |grad rho| v) / den, h_eff the interpolated nodal
 * h rho^p (1 - rho)^q (solver_heat.py:392-408, 825-832); den > 0. */
int topt_heat_exchange_adjoint(topt_heat* h, const double* rho_node, double h_coef,
                               double t_env, double p, double q, double den, double* rhs);
/* grad (dev, n_elem x L) += the explicit Robin gradient of the compliance
 * objective (solver_heat.py:575-597 mapped by 616-625, 952-979). */
int topt_heat_robin_grad(topt_heat* h, const double* rho_node, const double* T, int32_t L,
                         double h_coef, double t_env, double p, double q, double* grad);
/* out (dev, n_elem x L) = int_e grad X_j . grad Y_j (solver_heat.py:324-379,
 * 529-550). */
int topt_heat_grad_dot(topt_heat* h, const double* X, const double* Y, int32_t L, double* out);

/* Dot product that allocates no device memory, for callers that cannot call
 * cudaMalloc (a host whose device memory is owned by its own pool, or a loop
 * that must not stall on the device synchronisation cudaMalloc/cudaFree
 * imply).  No counterpart in the reference: it is an addition of this
 * library.  Scratch is a fixed ~32 KB device array per GPU, kept until the
 * process exits; n is limited to 268,435,456 elements (larger n returns
 * TOPT_BAD_INPUT).  The first call on a device looks up the array's device
 * address, so make it before any stream capture.  All calls share the
 * array: calls that overlap on the GPU (different streams) race.
 * x, y: dev; out: host. */
int topt_reduce_dot_noalloc(int64_t n, const double* x, const double* y,
                            double* out, void* stream);

/* Deterministic reductions (host result). */
int topt_reduce_max_abs(int64_t n, const double* x, double* out, void* stream);
int topt_reduce_dot(int64_t n, const double* x, const double* y, double* out,
                    void* stream);

#ifdef __cplusplus
}
#endif
#endif
