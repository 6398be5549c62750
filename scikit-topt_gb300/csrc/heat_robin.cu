// Heat plugin on hexahedral and P1 tetrahedral meshes: the density-dependent
// ("virtual") and surface Robin terms, the heat-exchange objective and its
// adjoint load, the explicit Robin gradient of the compliance objective and
// the per-element grad T . grad lam products of FEM_SimpLinearHeatConduction
// (sktopt/fea/solver_heat.py:306-625, 705-980).
//
// Every volume integral uses the quadrature of a basis with intorder 2: the
// 2x2x2 Gauss rule on hexahedra (MeshHex local node order; axis-aligned
// boxes from their extents, other hexahedra from the trilinear map of their
// 8 nodes, Jacobian per Gauss point), the 4-point degree-2 rule on
// tetrahedra (barycentric points (a, b, b, b), a = (5 + 3 sqrt 5) / 20,
// b = (5 - sqrt 5) / 20, weights V / 4; the P1 gradients are constant per
// element and precomputed).  Nodal sums run over
// a node -> (a, e) list kept in t.ravel() order (t is nloc x n_elem), so
// they are deterministic, and the nodal density average adds in exactly the
// order of the reference's np.add.at.

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "cuda_common.cuh"

using topt::DevBuf;
using topt::fail;

namespace topt {
namespace {

constexpr int kHB = 256;

// Offset along axis d of local node a (scikit-fem MeshHex order (0,0,0)
// (0,1,0) (1,0,0) (0,0,1) (1,1,0) (0,1,1) (1,0,1) (1,1,1)), packed 3 bits
// per node.
__host__ __device__ constexpr int hex_off(int a, int d) { return (0xF73850 >> (3 * a + d)) & 1; }

// Shape values and physical gradients of the trilinear hexahedron with
// extents (hx, hy, hz) at Gauss point q (bits: x, y, z coordinate index).
template <int NL>
struct QpT {
  double N[NL], gx[NL], gy[NL], gz[NL];
  double w;   // quadrature weight times detJ
};
using Qp = QpT<8>;
__device__ __forceinline__ void qpoint(int q, double G, double hx, double hy, double hz,
                                       Qp& o) {
  const double x = (q >> 2) & 1 ? 0.5 + G : 0.5 - G;
  const double y = (q >> 1) & 1 ? 0.5 + G : 0.5 - G;
  const double z = q & 1 ? 0.5 + G : 0.5 - G;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double fx = hex_off(a, 0) ? x : 1.0 - x;
    const double fy = hex_off(a, 1) ? y : 1.0 - y;
    const double fz = hex_off(a, 2) ? z : 1.0 - z;
    const double sx = hex_off(a, 0) ? 1.0 : -1.0;
    const double sy = hex_off(a, 1) ? 1.0 : -1.0;
    const double sz = hex_off(a, 2) ? 1.0 : -1.0;
    o.N[a] = fx * fy * fz;
    o.gx[a] = sx * fy * fz / hx;
    o.gy[a] = fx * sy * fz / hy;
    o.gz[a] = fx * fy * sz / hz;
  }
}

// The same at Gauss point q of a general hexahedron with nodes X (MeshHex
// order): x(xi) = sum_a X_a N_a(xi) on the reference cube [0, 1]^3,
// J = dx/dxi, physical gradients J^-T dN/dxi, weight detJ / 8.
__device__ __forceinline__ void qpoint_general(int q, double G, const double (&X)[8][3],
                                               Qp& o) {
  const double x = (q >> 2) & 1 ? 0.5 + G : 0.5 - G;
  const double y = (q >> 1) & 1 ? 0.5 + G : 0.5 - G;
  const double z = q & 1 ? 0.5 + G : 0.5 - G;
  double dr[8][3];
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double fx = hex_off(a, 0) ? x : 1.0 - x;
    const double fy = hex_off(a, 1) ? y : 1.0 - y;
    const double fz = hex_off(a, 2) ? z : 1.0 - z;
    const double sx = hex_off(a, 0) ? 1.0 : -1.0;
    const double sy = hex_off(a, 1) ? 1.0 : -1.0;
    const double sz = hex_off(a, 2) ? 1.0 : -1.0;
    o.N[a] = fx * fy * fz;
    dr[a][0] = sx * fy * fz;
    dr[a][1] = fx * sy * fz;
    dr[a][2] = fx * fy * sz;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int k = 0; k < 3; ++k) J[d][k] += X[a][d] * dr[a][k];
  }
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double id = 1.0 / det;
  // Ji[k][d] = d xi_k / d x_d
  const double Ji[3][3] = {
      {c00 * id, (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id,
       (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id},
      {c01 * id, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id,
       (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id},
      {c02 * id, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id,
       (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id}};
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    o.gx[a] = dr[a][0] * Ji[0][0] + dr[a][1] * Ji[1][0] + dr[a][2] * Ji[2][0];
    o.gy[a] = dr[a][0] * Ji[0][1] + dr[a][1] * Ji[1][1] + dr[a][2] * Ji[2][1];
    o.gz[a] = dr[a][0] * Ji[0][2] + dr[a][1] * Ji[1][2] + dr[a][2] * Ji[2][2];
  }
  o.w = 0.125 * det;
}

__device__ __forceinline__ double gauss_offset() { return 0.5 / sqrt(3.0); }

struct Geo {
  const int32_t* t;     // nloc x ne
  const double* hsz;    // axis-aligned hexahedra: 3 x ne extents
  const double* tg;     // tetrahedra: ne x 4 x 3 shape-function gradients
  const double* tv;     // tetrahedra: ne volumes
  int64_t ne;
  const double* xyz;    // other hexahedra: node coordinates, 3 x nn (else null)
  int64_t nn;
};

// Geometry of one element: box extents, the 8 node coordinates of a general
// hexahedron, or the tetrahedron gradients; and the quadrature weight w
// (times detJ) of a box or tetrahedron, shared by its points.
template <int NL>
struct ElemG {
  double hx, hy, hz, w;
  double g[NL][3];
  double X[8][3];
  bool general;
};

template <int NL>
__device__ __forceinline__ void load_elem(const Geo& g, int64_t e, const double* x,
                                          double (&v)[NL], int64_t (&node)[NL], ElemG<NL>& E) {
#pragma unroll
  for (int a = 0; a < NL; ++a) {
    node[a] = g.t[(int64_t)a * g.ne + e];
    v[a] = x ? x[node[a]] : 0.0;
  }
  if constexpr (NL == 8) {
    E.general = g.xyz != nullptr;
    if (E.general) {
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) E.X[a][d] = g.xyz[d * g.nn + node[a]];
      E.w = 0.0;
    } else {
      E.hx = g.hsz[e];
      E.hy = g.hsz[g.ne + e];
      E.hz = g.hsz[2 * g.ne + e];
      E.w = 0.125 * (E.hx * E.hy * E.hz);
    }
  } else {
    E.general = false;
#pragma unroll
    for (int a = 0; a < NL; ++a)
#pragma unroll
      for (int d = 0; d < 3; ++d) E.g[a][d] = g.tg[e * 12 + a * 3 + d];
    E.w = 0.25 * g.tv[e];
  }
}

// Quadrature points of an element: 8 Gauss points of the hexahedron, 4
// points of the tetrahedron rule.
template <int NL>
__host__ __device__ constexpr int n_qp() { return NL == 8 ? 8 : 4; }

template <int NL>
__device__ __forceinline__ void elem_qp(int qi, const ElemG<NL>& E, QpT<NL>& Q) {
  if constexpr (NL == 8) {
    if (E.general) {
      qpoint_general(qi, gauss_offset(), E.X, Q);
    } else {
      qpoint(qi, gauss_offset(), E.hx, E.hy, E.hz, Q);
      Q.w = E.w;
    }
  } else {
    Q.w = E.w;
    const double ta = 0.58541019662496845446, tb = 0.13819660112501051518;
#pragma unroll
    for (int a = 0; a < NL; ++a) {
      Q.N[a] = a == qi ? ta : tb;
      Q.gx[a] = E.g[a][0];
      Q.gy[a] = E.g[a][1];
      Q.gz[a] = E.g[a][2];
    }
  }
}

// rho_node[n] = sum over the (a, e) of node n, in t.ravel() order, of
// rho[src] / max(count, 1), src = (a ne + e) / nloc (pairing 0:
// np.repeat(rho, nloc) against t.ravel(), solver_heat.py:600-613) or e
// (pairing 1).
__global__ void k_nodal_average(int64_t nn, const int32_t* __restrict__ ptr,
                                const int32_t* __restrict__ adj, int64_t ne, int nloc,
                                int pairing, const double* __restrict__ rho,
                                double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k0 = ptr[n], k1 = ptr[n + 1];
    double s = 0.0;
    for (int32_t k = k0; k < k1; ++k) {
      const int64_t idx = adj[k];
      s += rho[pairing == 0 ? idx / nloc : idx % ne];
    }
    const double c = (double)(k1 - k0);
    out[n] = s / (c > 1.0 ? c : 1.0);
  }
}

// Virtual Robin element matrices and loads (get_robin_virtual,
// solver_heat.py:552-572): c = w detJ h rho^p (1 - rho)^q |grad rho| at every
// quadrature point, M_ab += c N_a N_b, f_a += c T_env N_a; plus the element's
// surface Robin matrix (task_heat.py:60-139) when it has Robin facets.
template <int NL>
__global__ void k_robin_elem(Geo g, const double* __restrict__ rho_n, double h, double t_env,
                             double p, double q, int virt, const int32_t* __restrict__ surf_idx,
                             const double* __restrict__ surf, double* __restrict__ extra,
                             double* __restrict__ fe) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    double M[NL][NL], f[NL];
#pragma unroll
    for (int a = 0; a < NL; ++a) {
      f[a] = 0.0;
#pragma unroll
      for (int b = 0; b < NL; ++b) M[a][b] = 0.0;
    }
    if (virt) {
      double r[NL];
      int64_t node[NL];
      ElemG<NL> E;
      load_elem<NL>(g, e, rho_n, r, node, E);
#pragma unroll 1
      for (int qi = 0; qi < n_qp<NL>(); ++qi) {
        QpT<NL> Q;
        elem_qp<NL>(qi, E, Q);
        double rq = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
        for (int a = 0; a < NL; ++a) {
          rq += Q.N[a] * r[a];
          gx += Q.gx[a] * r[a];
          gy += Q.gy[a] * r[a];
          gz += Q.gz[a] * r[a];
        }
        const double iface = sqrt(gx * gx + gy * gy + gz * gz);
        const double heff = h * pow(rq, p) * pow(1.0 - rq, q);
        const double c = Q.w * heff * iface;
        const double ct = c * t_env;
#pragma unroll
        for (int a = 0; a < NL; ++a) {
          f[a] += ct * Q.N[a];
          const double ca = c * Q.N[a];
#pragma unroll
          for (int b = a; b < NL; ++b) M[a][b] += ca * Q.N[b];
        }
      }
    }
    const int32_t si = surf_idx ? surf_idx[e] : -1;
    double* X = extra + e * NL * NL;
#pragma unroll
    for (int a = 0; a < NL; ++a)
#pragma unroll
      for (int b = 0; b < NL; ++b) {
        double v = a <= b ? M[a][b] : M[b][a];
        if (si >= 0) v += surf[(int64_t)si * NL * NL + a * NL + b];
        X[a * NL + b] = v;
      }
    if (fe) {
#pragma unroll
      for (int a = 0; a < NL; ++a) fe[e * NL + a] = f[a];
    }
  }
}

// out[n] = (sum over the (a, e) of node n of fe[e][a]) / div.
__global__ void k_node_gather(int64_t nn, const int32_t* __restrict__ ptr,
                              const int32_t* __restrict__ adj, int64_t ne, int nloc,
                              const double* __restrict__ fe, double div,
                              double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nn;
       n += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int32_t k = ptr[n]; k < ptr[n + 1]; ++k) {
      const int64_t idx = adj[k];
      const int64_t a = idx / ne, e = idx - a * ne;
      s += fe[e * nloc + a];
    }
    out[n] = div == 1.0 ? s : s / div;
  }
}

// Heat-exchange integrals (solver_heat.py:306-321, 382-390): den = sum of
// w detJ |grad rho|, num_j = sum of w detJ (-T_env h (T_j - T_env) |grad rho|)
// for L <= 4 temperature columns (T: n_nodes x L row-major).
template <int NL>
__global__ void __launch_bounds__(kHB)
k_hx_reduce(Geo g, const double* __restrict__ rho_n, const double* __restrict__ T, int L,
            double h, double t_env, double* __restrict__ partials, unsigned* __restrict__ counter,
            double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    double r[NL];
    int64_t node[NL];
    ElemG<NL> E;
    load_elem<NL>(g, e, rho_n, r, node, E);
    double te[4][NL];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int a = 0; a < NL; ++a) te[j][a] = j < L ? T[node[a] * L + j] : 0.0;
    double den = 0.0, num[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 1
    for (int qi = 0; qi < n_qp<NL>(); ++qi) {
      QpT<NL> Q;
      elem_qp<NL>(qi, E, Q);
      double gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
      for (int a = 0; a < NL; ++a) {
        gx += Q.gx[a] * r[a];
        gy += Q.gy[a] * r[a];
        gz += Q.gz[a] * r[a];
      }
      const double iface = sqrt(gx * gx + gy * gy + gz * gz);
      den += Q.w * iface;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (j < L) {
          double tq = 0.0;
#pragma unroll
          for (int a = 0; a < NL; ++a) tq += Q.N[a] * te[j][a];
          num[j] += Q.w * (-t_env * h * (tq - t_env) * iface);
        }
      }
    }
    v[0] += den;
#pragma unroll
    for (int j = 0; j < 4; ++j) v[1 + j] += num[j];
  }
  __shared__ double sh[32 * 5];
  block_sum<double, 5>(v, sh);
  grid_finish<double, 5>(v, partials, counter, out);
}

// Element loads of the heat-exchange adjoint (_hx_adj_rhs_,
// solver_heat.py:392-408): h_eff the interpolated nodal h rho^p (1 - rho)^q
// (825-830), f_a += w detJ (-T_env h_eff |grad rho|) N_a.
template <int NL>
__global__ void k_hx_adj_elem(Geo g, const double* __restrict__ rho_n, double h, double t_env,
                              double p, double q, double* __restrict__ fe) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    double r[NL], hn[NL];
    int64_t node[NL];
    ElemG<NL> E;
    load_elem<NL>(g, e, rho_n, r, node, E);
#pragma unroll
    for (int a = 0; a < NL; ++a) hn[a] = h * pow(r[a], p) * pow(1.0 - r[a], q);
    double f[NL];
#pragma unroll
    for (int a = 0; a < NL; ++a) f[a] = 0.0;
#pragma unroll 1
    for (int qi = 0; qi < n_qp<NL>(); ++qi) {
      QpT<NL> Q;
      elem_qp<NL>(qi, E, Q);
      double hq = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
      for (int a = 0; a < NL; ++a) {
        hq += Q.N[a] * hn[a];
        gx += Q.gx[a] * r[a];
        gy += Q.gy[a] * r[a];
        gz += Q.gz[a] * r[a];
      }
      const double c = Q.w * (-t_env * hq * sqrt(gx * gx + gy * gy + gz * gz));
#pragma unroll
      for (int a = 0; a < NL; ++a) f[a] += c * Q.N[a];
    }
#pragma unroll
    for (int a = 0; a < NL; ++a) fe[e * NL + a] = f[a];
  }
}

// Element vectors of _robin_compliance_explicit_grad_ (solver_heat.py:
// 575-597) for temperature column j: a = rho^p (1 - rho)^q, its derivative
// da, phi = 2 T_env T - T^2,
//   f_a += w detJ h (da |grad rho| phi N_a + a phi (grad rho / max(|grad rho|,
//   1e-12)) . grad N_a).
template <int NL>
__global__ void k_robin_grad_elem(Geo g, const double* __restrict__ rho_n,
                                  const double* __restrict__ T, int L, int j, double h,
                                  double t_env, double p, double q, double* __restrict__ fe) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    double r[NL], te[NL];
    int64_t node[NL];
    ElemG<NL> E;
    load_elem<NL>(g, e, rho_n, r, node, E);
#pragma unroll
    for (int a = 0; a < NL; ++a) te[a] = T[node[a] * L + j];
    double f[NL];
#pragma unroll
    for (int a = 0; a < NL; ++a) f[a] = 0.0;
#pragma unroll 1
    for (int qi = 0; qi < n_qp<NL>(); ++qi) {
      QpT<NL> Q;
      elem_qp<NL>(qi, E, Q);
      double rq = 0.0, tq = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
      for (int a = 0; a < NL; ++a) {
        rq += Q.N[a] * r[a];
        tq += Q.N[a] * te[a];
        gx += Q.gx[a] * r[a];
        gy += Q.gy[a] * r[a];
        gz += Q.gz[a] * r[a];
      }
      const double iface = sqrt(gx * gx + gy * gy + gz * gz);
      const double safe = iface > 1e-12 ? iface : 1e-12;
      const double rp = pow(rq, p), sq = pow(1.0 - rq, q);
      const double av = rp * sq;
      const double da = p * pow(rq, p - 1.0) * sq - q * rp * pow(1.0 - rq, q - 1.0);
      const double phi = 2.0 * t_env * tq - tq * tq;
      const double c1 = Q.w * h * da * iface * phi;
      const double c2 = Q.w * h * av * phi;
      const double nx = gx / safe, ny = gy / safe, nz = gz / safe;
#pragma unroll
      for (int a = 0; a < NL; ++a)
        f[a] += c1 * Q.N[a] + c2 * (nx * Q.gx[a] + ny * Q.gy[a] + nz * Q.gz[a]);
    }
#pragma unroll
    for (int a = 0; a < NL; ++a) fe[e * NL + a] = f[a];
  }
}

// _nodal_gradient_to_element_gradient (solver_heat.py:616-625), added to
// column j: grad[e][j] += sum_a nodal[t[a][e]] / max(count, 1).
template <int NL>
__global__ void k_nodal_to_elem(Geo g, const int32_t* __restrict__ ptr,
                                const double* __restrict__ nodal, int L, int j,
                                double* __restrict__ grad) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < NL; ++a) {
      const int64_t n = g.t[(int64_t)a * g.ne + e];
      const double c = (double)(ptr[n + 1] - ptr[n]);
      s += nodal[n] / (c > 1.0 ? c : 1.0);
    }
    grad[e * L + j] += s;
  }
}

// out[e][j] = integral over e of grad X_j . grad Y_j (solver_heat.py:324-379,
// 529-550).  X, Y: n_nodes x L row-major.
template <int NL>
__global__ void k_grad_dot(Geo g, const double* __restrict__ X, const double* __restrict__ Y,
                           int L, double* __restrict__ out) {
  TOPT_KERNEL_COUNT();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    double dummy[NL];
    int64_t node[NL];
    ElemG<NL> E;
    load_elem<NL>(g, e, nullptr, dummy, node, E);
    for (int j = 0; j < L; ++j) {
      // shifted by the node-0 values: gradients of large offset fields
      // (prescribed temperatures) without cancellation
      double xe[NL], ye[NL];
      const double x0 = X[node[0] * L + j], y0 = Y[node[0] * L + j];
#pragma unroll
      for (int a = 0; a < NL; ++a) {
        xe[a] = X[node[a] * L + j] - x0;
        ye[a] = Y[node[a] * L + j] - y0;
      }
      double s = 0.0;
#pragma unroll 1
      for (int qi = 0; qi < n_qp<NL>(); ++qi) {
        QpT<NL> Q;
        elem_qp<NL>(qi, E, Q);
        double ax = 0.0, ay = 0.0, az = 0.0, bx = 0.0, by = 0.0, bz = 0.0;
#pragma unroll
        for (int a = 0; a < NL; ++a) {
          ax += Q.gx[a] * xe[a]; ay += Q.gy[a] * xe[a]; az += Q.gz[a] * xe[a];
          bx += Q.gx[a] * ye[a]; by += Q.gy[a] * ye[a]; bz += Q.gz[a] * ye[a];
        }
        s += Q.w * (ax * bx + ay * by + az * bz);
      }
      out[e * L + j] = s;
    }
  }
}

}  // namespace

int launches_heat(unsigned long long* out) {
  TOPT_CUDA(cudaMemcpyFromSymbol(out, g_kernel_launches, sizeof(unsigned long long)));
  return TOPT_OK;
}

}  // namespace topt

struct topt_heat {
  int64_t n_nodes = 0, n_elem = 0;
  int nloc = 8;
  int pairing = 0;
  int sm = 152;
  cudaStream_t stream = nullptr;
  DevBuf t, hsz, tg, tv, node_ptr, adj;
  DevBuf xyz;                         // node coordinates of general hexahedra
  DevBuf surf_idx, surf;
  DevBuf fe, nodal;                   // element-vector and nodal scratch
  DevBuf partials, counter, out;      // k_hx_reduce
  int red_blocks = 0;
  topt::Geo geo() const {
    return {t.as<int32_t>(), hsz.as<double>(), tg.as<double>(), tv.as<double>(), n_elem,
            xyz.p ? xyz.as<double>() : nullptr, n_nodes};
  }
  int grid(int64_t n) const { return topt::grid_for(n, topt::kHB, sm * 16); }
};

#define TOPT_HEAT_NL(h, CALL)                      \
  do {                                             \
    if ((h)->nloc == 8) { constexpr int NL_ = 8; CALL; } \
    else { constexpr int NL_ = 4; CALL; }          \
  } while (0)

extern "C" {

int topt_heat_create_mesh(int64_t n_nodes, int64_t n_elem, int32_t nloc, const int32_t* t,
                          const double* p, int32_t pairing, topt_heat** out) {
  using namespace topt;
  if (!out || !t || !p || n_nodes <= 0 || n_elem <= 0 || (pairing != 0 && pairing != 1) ||
      (nloc != 8 && nloc != 4))
    return fail(TOPT_BAD_INPUT, "heat_create: bad argument");
  if (n_elem * nloc >= (int64_t)INT32_MAX || n_nodes >= (int64_t)INT32_MAX)
    return fail(TOPT_BAD_INPUT, "heat_create: mesh too large for 32-bit indices");
  *out = nullptr;
  for (int64_t i = 0; i < (int64_t)nloc * n_elem; ++i)
    if (t[i] < 0 || t[i] >= n_nodes) return fail(TOPT_BAD_INPUT, "heat_create: bad node index");
  std::vector<double> hs, tg, tv;
  bool general = false;
  if (nloc == 8) {
    // extents of every cell when all cells are axis-aligned boxes; any other
    // hexahedron switches the handle to the general trilinear map (node
    // coordinates on the device, Jacobian per Gauss point), whose Jacobian
    // must be positive at every Gauss point
    hs.resize(3 * (size_t)n_elem);
    for (int64_t e = 0; e < n_elem && !general; ++e) {
      int64_t nd[8];
      for (int a = 0; a < 8; ++a) nd[a] = t[(int64_t)a * n_elem + e];
      double lo[3], ext[3];
      for (int d = 0; d < 3; ++d) {
        lo[d] = p[d * n_nodes + nd[0]];
        ext[d] = p[d * n_nodes + nd[7]] - lo[d];
        if (!(ext[d] > 0.0)) general = true;
        hs[(size_t)d * n_elem + e] = ext[d];
      }
      for (int a = 0; a < 8 && !general; ++a)
        for (int d = 0; d < 3; ++d) {
          const double want = lo[d] + (hex_off(a, d) ? ext[d] : 0.0);
          if (std::fabs(p[d * n_nodes + nd[a]] - want) > 1e-9 * ext[d]) general = true;
        }
    }
    if (general) {
      hs.clear();
      const double G = 0.5 / std::sqrt(3.0);
      for (int64_t e = 0; e < n_elem; ++e) {
        double X[8][3];
        for (int a = 0; a < 8; ++a)
          for (int d = 0; d < 3; ++d) X[a][d] = p[d * n_nodes + t[(int64_t)a * n_elem + e]];
        for (int q = 0; q < 8; ++q) {
          const double xq[3] = {(q >> 2) & 1 ? 0.5 + G : 0.5 - G,
                                (q >> 1) & 1 ? 0.5 + G : 0.5 - G, q & 1 ? 0.5 + G : 0.5 - G};
          double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
          for (int a = 0; a < 8; ++a) {
            double f[3], s3[3];
            for (int k = 0; k < 3; ++k) {
              f[k] = hex_off(a, k) ? xq[k] : 1.0 - xq[k];
              s3[k] = hex_off(a, k) ? 1.0 : -1.0;
            }
            const double dr[3] = {s3[0] * f[1] * f[2], f[0] * s3[1] * f[2], f[0] * f[1] * s3[2]};
            for (int d = 0; d < 3; ++d)
              for (int k = 0; k < 3; ++k) J[d][k] += X[a][d] * dr[k];
          }
          const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) +
                             J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
                             J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
          if (!(det > 0.0))
            return fail(TOPT_BAD_INPUT,
                        "heat_create: hexahedron with a non-positive Jacobian at a Gauss point");
        }
      }
    }
  } else {
    // P1 gradients: with J the columns x1 - x0, x2 - x0, x3 - x0, the
    // reference gradients (-1,-1,-1), e1, e2, e3 map by J^-T; volume |det J|/6
    tg.resize(12 * (size_t)n_elem);
    tv.resize((size_t)n_elem);
    for (int64_t e = 0; e < n_elem; ++e) {
      double x[4][3];
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) x[a][d] = p[d * n_nodes + t[(int64_t)a * n_elem + e]];
      double J[3][3];
      for (int d = 0; d < 3; ++d)
        for (int k = 0; k < 3; ++k) J[d][k] = x[k + 1][d] - x[0][d];
      const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
      const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
      const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
      const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
      if (!(std::fabs(det) > 0.0)) return fail(TOPT_BAD_INPUT, "heat_create: degenerate tetrahedron");
      // inverse of J (rows: d xi_k / d x_d transposed as Jinv[k][d])
      double Ji[3][3];
      Ji[0][0] = c00 / det;
      Ji[1][0] = c01 / det;
      Ji[2][0] = c02 / det;
      Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
      Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
      // dN_a/dx_d = sum_k dN_a/dxi_k Jinv[k][d]
      const double gr[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) {
          double v = 0.0;
          for (int k = 0; k < 3; ++k) v += gr[a][k] * Ji[k][d];
          tg[(size_t)e * 12 + a * 3 + d] = v;
        }
      tv[e] = std::fabs(det) / 6.0;
    }
  }
  // node -> raveled (a, e) list in t.ravel() order
  const int64_t nt = (int64_t)nloc * n_elem;
  std::vector<int32_t> ptr(n_nodes + 1, 0), adj((size_t)nt);
  for (int64_t i = 0; i < nt; ++i) ptr[t[i] + 1]++;
  for (int64_t n = 0; n < n_nodes; ++n) ptr[n + 1] += ptr[n];
  {
    std::vector<int32_t> pos(ptr.begin(), ptr.end() - 1);
    for (int64_t i = 0; i < nt; ++i) adj[pos[t[i]]++] = (int32_t)i;
  }
  std::unique_ptr<topt_heat> h(new topt_heat());
  h->n_nodes = n_nodes;
  h->n_elem = n_elem;
  h->nloc = nloc;
  h->pairing = pairing;
  h->sm = device_sm_count();
  int rc;
  cudaStream_t s = nullptr;
  if ((rc = upload(h->t, t, (size_t)nt, s))) return rc;
  if (nloc == 8 && general) {
    if ((rc = upload(h->xyz, p, 3 * (size_t)n_nodes, s))) return rc;
  } else if (nloc == 8) {
    if ((rc = upload(h->hsz, hs.data(), hs.size(), s))) return rc;
  } else {
    if ((rc = upload(h->tg, tg.data(), tg.size(), s))) return rc;
    if ((rc = upload(h->tv, tv.data(), tv.size(), s))) return rc;
  }
  if ((rc = upload(h->node_ptr, ptr.data(), ptr.size(), s))) return rc;
  if ((rc = upload(h->adj, adj.data(), adj.size(), s))) return rc;
  if ((rc = h->fe.alloc(sizeof(double) * (size_t)nt))) return rc;
  if ((rc = h->nodal.alloc(sizeof(double) * (size_t)n_nodes))) return rc;
  h->red_blocks = h->grid(n_elem);
  if ((rc = h->partials.alloc(sizeof(double) * 5 * (size_t)h->red_blocks))) return rc;
  if ((rc = h->counter.alloc(sizeof(unsigned)))) return rc;
  if ((rc = h->out.alloc(sizeof(double) * 8))) return rc;
  TOPT_CUDA(cudaMemset(h->counter.p, 0, sizeof(unsigned)));
  TOPT_CUDA(cudaDeviceSynchronize());
  *out = h.release();
  return TOPT_OK;
}

int topt_heat_create(int64_t n_nodes, int64_t n_elem, const int32_t* t, const double* p,
                     int32_t pairing, topt_heat** out) {
  return topt_heat_create_mesh(n_nodes, n_elem, 8, t, p, pairing, out);
}

void topt_heat_destroy(topt_heat* h) { delete h; }

int topt_heat_set_stream(topt_heat* h, void* stream) {
  if (!h) return fail(TOPT_BAD_INPUT, "heat_set_stream: null handle");
  h->stream = (cudaStream_t)stream;
  return TOPT_OK;
}

int topt_heat_set_surface(topt_heat* h, int64_t n_faces, const int32_t* elems,
                          const double* mats) {
  using namespace topt;
  if (!h || n_faces < 0 || (n_faces > 0 && (!elems || !mats)))
    return fail(TOPT_BAD_INPUT, "heat_set_surface: bad argument");
  const int nn = h->nloc * h->nloc;
  std::vector<int32_t> idx(h->n_elem, -1);
  std::vector<double> m;
  for (int64_t k = 0; k < n_faces; ++k) {
    const int32_t e = elems[k];
    if (e < 0 || e >= h->n_elem) return fail(TOPT_BAD_INPUT, "heat_set_surface: bad element");
    if (idx[e] < 0) {
      idx[e] = (int32_t)(m.size() / nn);
      m.resize(m.size() + nn, 0.0);
    }
    double* dst = m.data() + (size_t)idx[e] * nn;
    for (int i = 0; i < nn; ++i) dst[i] += mats[k * nn + i];
  }
  int rc;
  if (m.empty()) {
    h->surf_idx.release();
    h->surf.release();
    return TOPT_OK;
  }
  if ((rc = upload(h->surf_idx, idx.data(), idx.size(), h->stream))) return rc;
  if ((rc = upload(h->surf, m.data(), m.size(), h->stream))) return rc;
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  return TOPT_OK;
}

int topt_heat_nodal_average(topt_heat* h, const double* rho, double* rho_node) {
  using namespace topt;
  if (!h || !rho || !rho_node) return fail(TOPT_BAD_INPUT, "heat_nodal_average: null argument");
  k_nodal_average<<<h->grid(h->n_nodes), kHB, 0, h->stream>>>(
      h->n_nodes, h->node_ptr.as<int32_t>(), h->adj.as<int32_t>(), h->n_elem, h->nloc,
      h->pairing, rho, rho_node);
  TOPT_CHECK_LAUNCH("k_nodal_average");
  return TOPT_OK;
}

int topt_heat_robin(topt_heat* h, const double* rho_node, double h_coef, double t_env, double p,
                    double q, int32_t virtual_on, double* extra, double* load) {
  using namespace topt;
  if (!h || !extra || (virtual_on && !rho_node))
    return fail(TOPT_BAD_INPUT, "heat_robin: null argument");
  TOPT_HEAT_NL(h, (k_robin_elem<NL_><<<h->grid(h->n_elem), kHB, 0, h->stream>>>(
                      h->geo(), rho_node, h_coef, t_env, p, q, virtual_on ? 1 : 0,
                      h->surf_idx.as<int32_t>(), h->surf.as<double>(), extra,
                      load ? h->fe.as<double>() : nullptr)));
  TOPT_CHECK_LAUNCH("k_robin_elem");
  if (load) {
    k_node_gather<<<h->grid(h->n_nodes), kHB, 0, h->stream>>>(
        h->n_nodes, h->node_ptr.as<int32_t>(), h->adj.as<int32_t>(), h->n_elem, h->nloc,
        h->fe.as<double>(), 1.0, load);
    TOPT_CHECK_LAUNCH("k_node_gather");
  }
  return TOPT_OK;
}

int topt_heat_exchange(topt_heat* h, const double* rho_node, const double* T, int32_t L,
                       double h_coef, double t_env, double* den, double* num) {
  using namespace topt;
  if (!h || !rho_node || !den || L < 0 || L > 4 || (L > 0 && (!T || !num)))
    return fail(TOPT_BAD_INPUT, "heat_exchange: bad argument");
  TOPT_HEAT_NL(h, (k_hx_reduce<NL_><<<h->red_blocks, kHB, 0, h->stream>>>(
                      h->geo(), rho_node, T, L, h_coef, t_env, h->partials.as<double>(),
                      h->counter.as<unsigned>(), h->out.as<double>())));
  TOPT_CHECK_LAUNCH("k_hx_reduce");
  double r[5];
  TOPT_CUDA(cudaMemcpyAsync(r, h->out.p, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
  TOPT_CUDA(cudaStreamSynchronize(h->stream));
  *den = r[0];
  for (int j = 0; j < L; ++j) num[j] = r[1 + j];
  return TOPT_OK;
}

int topt_heat_exchange_adjoint(topt_heat* h, const double* rho_node, double h_coef,
                               double t_env, double p, double q, double den, double* rhs) {
  using namespace topt;
  if (!h || !rho_node || !rhs || !(den > 0.0))
    return fail(TOPT_BAD_INPUT, "heat_exchange_adjoint: bad argument");
  TOPT_HEAT_NL(h, (k_hx_adj_elem<NL_><<<h->grid(h->n_elem), kHB, 0, h->stream>>>(
                      h->geo(), rho_node, h_coef, t_env, p, q, h->fe.as<double>())));
  TOPT_CHECK_LAUNCH("k_hx_adj_elem");
  k_node_gather<<<h->grid(h->n_nodes), kHB, 0, h->stream>>>(
      h->n_nodes, h->node_ptr.as<int32_t>(), h->adj.as<int32_t>(), h->n_elem, h->nloc,
      h->fe.as<double>(), den, rhs);
  TOPT_CHECK_LAUNCH("k_node_gather");
  return TOPT_OK;
}

int topt_heat_robin_grad(topt_heat* h, const double* rho_node, const double* T, int32_t L,
                         double h_coef, double t_env, double p, double q, double* grad) {
  using namespace topt;
  if (!h || !rho_node || !T || !grad || L < 1 || L > 64)
    return fail(TOPT_BAD_INPUT, "heat_robin_grad: bad argument");
  for (int j = 0; j < L; ++j) {
    TOPT_HEAT_NL(h, (k_robin_grad_elem<NL_><<<h->grid(h->n_elem), kHB, 0, h->stream>>>(
                        h->geo(), rho_node, T, L, j, h_coef, t_env, p, q, h->fe.as<double>())));
    TOPT_CHECK_LAUNCH("k_robin_grad_elem");
    k_node_gather<<<h->grid(h->n_nodes), kHB, 0, h->stream>>>(
        h->n_nodes, h->node_ptr.as<int32_t>(), h->adj.as<int32_t>(), h->n_elem, h->nloc,
        h->fe.as<double>(), 1.0, h->nodal.as<double>());
    TOPT_CHECK_LAUNCH("k_node_gather");
    TOPT_HEAT_NL(h, (k_nodal_to_elem<NL_><<<h->grid(h->n_elem), kHB, 0, h->stream>>>(
                        h->geo(), h->node_ptr.as<int32_t>(), h->nodal.as<double>(), L, j,
                        grad)));
    TOPT_CHECK_LAUNCH("k_nodal_to_elem");
  }
  return TOPT_OK;
}

int topt_heat_grad_dot(topt_heat* h, const double* X, const double* Y, int32_t L, double* out) {
  using namespace topt;
  if (!h || !X || !Y || !out || L < 1 || L > 64)
    return fail(TOPT_BAD_INPUT, "heat_grad_dot: bad argument");
  TOPT_HEAT_NL(h, (k_grad_dot<NL_><<<h->grid(h->n_elem), kHB, 0, h->stream>>>(
                      h->geo(), X, Y, L, out)));
  TOPT_CHECK_LAUNCH("k_grad_dot");
  return TOPT_OK;
}

}  // extern "C"
