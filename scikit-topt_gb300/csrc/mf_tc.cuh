// Matrix-free fine-level operator of a uniform hex grid on the tensor cores
// (tcgen05, kind::tf32 with the 3xTF32 split: FP32-accurate products).
//
// y_a = sum over the <= 8 cells c around node a of coef_c * (K0 x_c)[la],
// la the node's local index in c (MeshHex order), fixed DOFs as identity
// rows (and, with COLMASK, zero columns).  Same contract as k_mf_tile.
//
// Work decomposition.  A CTA owns a column of 15 x 7 nodes (y x) over a z
// segment and walks it layer by layer.  The 16 x 8 = 128 cells that touch a
// node plane of the column form one MMA tile (M = 128 cells): row m holds the
// cell's 24 DOF values, split into TF32 hi and lo parts, and
//     Y = [x_hi | x_lo] [K0_hi ; K0_hi] + x_hi K0_lo        (N = 24 -> 32)
// accumulates in tensor memory (9 MMAs of 128 x 32 x 8).  Row m is then
// scaled by coef_m and stored to shared memory; each node sums the rows of
// its 8 cells (two consecutive cell layers) in a fixed order, so the result
// is deterministic.  Cells on the column's border are computed by both
// neighbouring columns (16 x 8 cells for 15 x 7 nodes).
//
// Warp roles (256 threads), so that consecutive layers overlap:
//   builders (warps 0-3): stage node planes (cp.async), build the A tile of
//     layer L into A[L % 2] once the MMAs of layer L-2 have released it, and
//     (thread 0) issue layer L's MMAs into TMEM buffer L % 2 once the
//     drainers have emptied it, committing them to mbarrier full[L % 2];
//   drainers (warps 4-7, lanes 0-127 of tensor memory): wait full[L % 2],
//     load the accumulators, release the TMEM buffer (mbarrier empty[L % 2]),
//     scale by the cell coefficients, store Y[L % 2] and produce the node
//     plane of layer L from Y[L % 2] and Y[(L-1) % 2].
// Each role synchronises internally with its own named barrier.
//
// Every wait is bounded: on a timeout the CTA sets an abort flag that both
// roles poll, stops, lets in-flight MMAs drain, writes a NaN into y (the
// solvers then stop with a non-finite status), records the error and frees
// its tensor memory.
#pragma once

#include "tc_sm100.cuh"

namespace topt {

namespace mftc {
constexpr int CY = 16, CX = 8;              // cells per layer tile
constexpr int NY = CY - 1, NX = CX - 1;     // output nodes per plane
constexpr int HY = CY + 1, HX = CX + 1;     // halo nodes per plane
constexpr int M = CY * CX;                  // 128 = MMA rows
constexpr int NPN = NY * NX;                // 105 output nodes per plane
constexpr int GROUP = 128;                  // threads per role
constexpr int THREADS = 2 * GROUP;
constexpr uint32_t SBO_A = 12 * 128;        // 48 K columns = 12 core matrices
constexpr uint32_t SBO_B = 6 * 128;         // 24 K columns
constexpr int YS = 36;                      // floats per Y row (8 x float4 + pad)
constexpr int NPLANE = 3;                   // builders' node-plane ring
constexpr uint32_t A_BYTES = M * 48 * 4;    // 24576
constexpr uint32_t B_BYTES = 32 * 24 * 4;   // 3072 per split part
constexpr uint32_t Y_BYTES = M * YS * 4;    // 18432
constexpr uint32_t P_BYTES = HY * HX * 16;  // 2448 (float4 per halo node)
// drainers' per-layer slot: coefficients (128), own node x + flags (105 x
// float4), b or y of the own node (105 x 3)
constexpr uint32_t E_COEF = 0, E_SELF = M * 4, E_SRC = E_SELF + NPN * 16;
constexpr uint32_t E_BYTES = (E_SRC + NPN * 12 + 15) & ~15u;
constexpr uint32_t OFF_A = 0;
constexpr uint32_t OFF_B = OFF_A + 2 * A_BYTES;
constexpr uint32_t OFF_Y = OFF_B + 2 * B_BYTES;
constexpr uint32_t OFF_P = OFF_Y + 2 * Y_BYTES;
constexpr uint32_t OFF_E = OFF_P + NPLANE * P_BYTES;
constexpr uint32_t OFF_BAR = OFF_E + 2 * E_BYTES;   // full[2], empty[2], tmem slot, abort
constexpr uint32_t SMEM = OFF_BAR + 64;
constexpr uint32_t TMEM_COLS = 64;
constexpr uint32_t WAIT_LIMIT = 1u << 24;
// image of K0 hi / lo in the B layout, built on the host (2 x 768 floats)
constexpr int K0_IMAGE_FLOATS = 2 * 32 * 24;
}  // namespace mftc

struct MfTcGrid {
  MfGrid g;
  int ncy, ncx, nseg, zs;   // columns along y and x; z segments of zs node planes
};

__device__ __forceinline__ void mftc_cp4(void* s, const void* gp, bool in) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gp),
               "r"(in ? 4 : 0));
}
__device__ __forceinline__ void mftc_commit() { asm volatile("cp.async.commit_group;\n" ::); }

// Named barrier of one role (id 1: builders, 2: drainers), returning the OR
// of `fail` over the role.
__device__ __forceinline__ bool mftc_group_sync_or(int id, bool fail) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n"
      " bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)fail), "r"(id), "r"(mftc::GROUP)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void mftc_group_sync(int id) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(mftc::GROUP) : "memory");
}

// Bounded wait on an mbarrier phase that also gives up when the CTA's abort
// flag is set.
__device__ __forceinline__ bool mftc_wait(uint64_t* bar, uint32_t parity,
                                          const volatile int* abort_f) {
  const uint32_t a = tc::smem_u32(bar);
  for (uint32_t i = 0; i < mftc::WAIT_LIMIT; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred P1;\n mbarrier.test_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
        " selp.b32 %0, 1, 0, P1;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 255) == 255 && *abort_f) return false;
  }
  return false;
}

__device__ __forceinline__ void mftc_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(tc::smem_u32(bar))
               : "memory");
}

// Node plane z of the column's halo (builders): x in .xyz, the fixed-DOF
// bits in .w, zeros outside the grid.
__device__ __forceinline__ void mftc_stage_plane(float* P, int z, int y0, int x0, int ny1,
                                                 int nx1, int nz1, int t,
                                                 const float* __restrict__ x,
                                                 const uint32_t* __restrict__ m32) {
  using namespace mftc;
  const bool zin = z >= 0 && z < nz1;
  for (int q = t; q < HY * HX; q += GROUP) {
    const int hy = q % HY, hx = q / HY;
    const int gy = y0 - 1 + hy, gx = x0 - 1 + hx;
    const bool in = zin && gy >= 0 && gy < ny1 && gx >= 0 && gx < nx1;
    const int64_t n = in ? (int64_t)gy + (int64_t)ny1 * (gx + (int64_t)nx1 * z) : 0;
    float* d = P + q * 4;
    mftc_cp4(d + 0, x + n * 3 + 0, in);
    mftc_cp4(d + 1, x + n * 3 + 1, in);
    mftc_cp4(d + 2, x + n * 3 + 2, in);
    mftc_cp4(d + 3, m32 + n, in);
  }
}

// Drainer e's own data for cell layer c and node plane c: the coefficient of
// its cell, and (e < 105) its node's x, flags and b / y.  Every thread reads
// only what it loaded itself.
template <int MODE>
__device__ __forceinline__ void mftc_stage_own(unsigned char* S, int c, int y0, int x0,
                                               const MfGrid& g, int e,
                                               const float* __restrict__ coef,
                                               const float* __restrict__ x,
                                               const uint32_t* __restrict__ m32,
                                               const float* __restrict__ src) {
  using namespace mftc;
  const int ny1 = g.ny + 1, nx1 = g.nx + 1, nz1 = g.nz + 1;
  {
    const int cy = y0 - 1 + (e % CY), cx = x0 - 1 + (e / CY);
    const bool in = c >= 0 && c < g.nz && cy >= 0 && cy < g.ny && cx >= 0 && cx < g.nx;
    const int64_t ce = in ? (int64_t)cy + (int64_t)g.ny * (cx + (int64_t)g.nx * c) : 0;
    mftc_cp4(reinterpret_cast<float*>(S + E_COEF) + e, coef + ce, in);
  }
  if (e < NPN) {
    const int gy = y0 + e % NY, gx = x0 + e / NY;
    const bool in = c >= 0 && c < nz1 && gy < ny1 && gx < nx1;
    const int64_t n = in ? (int64_t)gy + (int64_t)ny1 * (gx + (int64_t)nx1 * c) : 0;
    float* d = reinterpret_cast<float*>(S + E_SELF) + e * 4;
    mftc_cp4(d + 0, x + n * 3 + 0, in);
    mftc_cp4(d + 1, x + n * 3 + 1, in);
    mftc_cp4(d + 2, x + n * 3 + 2, in);
    mftc_cp4(d + 3, m32 + n, in);
    if (MODE != 0) {
      float* s3 = reinterpret_cast<float*>(S + E_SRC) + e * 3;
      mftc_cp4(s3 + 0, src + n * 3 + 0, in);
      mftc_cp4(s3 + 1, src + n * 3 + 1, in);
      mftc_cp4(s3 + 2, src + n * 3 + 2, in);
    }
  }
}

template <int MODE, bool DOT, bool COLMASK>
__global__ void __launch_bounds__(mftc::THREADS, 2)
k_mf_tc(MfTcGrid G, const float* __restrict__ k0img, const float* __restrict__ coef,
        const uint32_t* __restrict__ m32, const float* __restrict__ x,
        const float* __restrict__ b, float* __restrict__ y, double* partials,
        unsigned* counter, double* dot_out, int* err) {
  TOPT_KERNEL_COUNT();
  using namespace mftc;
  extern __shared__ __align__(1024) unsigned char mftc_smem[];
  unsigned char* smem = mftc_smem;
  float* Bs = reinterpret_cast<float*>(smem + OFF_B);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
  uint64_t* empty = full + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + OFF_BAR + 32);
  volatile int* abort_f = reinterpret_cast<volatile int*>(smem + OFF_BAR + 48);
  const int tid = threadIdx.x, warp = tid >> 5;
  const bool builder = tid < GROUP;
  const int t = builder ? tid : tid - GROUP;
  const MfGrid& g = G.g;
  const int ny1 = g.ny + 1, nx1 = g.nx + 1, nz1 = g.nz + 1;
  const float* bsrc = MODE == 1 ? b : y;

  // K0 hi / lo image (already in the B operand layout)
  for (int i = tid; i < K0_IMAGE_FLOATS / 4; i += THREADS)
    reinterpret_cast<float4*>(Bs)[i] = reinterpret_cast<const float4*>(k0img)[i];
  if (tid == 0) {
    tc::mbar_init(&full[0], 1);
    tc::mbar_init(&full[1], 1);
    tc::mbar_init(&empty[0], GROUP);
    tc::mbar_init(&empty[1], GROUP);
    *abort_f = 0;
    tc::mbar_init_fence();
  }
  if (warp == 0) tc::tmem_alloc(tslot, TMEM_COLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  bool fail = false;           // uniform within the role after each role sync
  float tacc = 0.0f;
  uint32_t L = 0;              // running layer count (same sequence in both roles)
  const int nitems = G.ncy * G.ncx * G.nseg;

  if (builder) {
    const uint32_t idesc = tc::idesc_tf32(M, 32);
    for (int item = blockIdx.x; item < nitems && !fail; item += gridDim.x) {
      const int col = item % (G.ncy * G.ncx), seg = item / (G.ncy * G.ncx);
      const int y0 = (col % G.ncy) * NY, x0 = (col / G.ncy) * NX;
      const int z0 = seg * G.zs, z1 = min(nz1, z0 + G.zs);
      auto plane = [&](int z) {
        return reinterpret_cast<float*>(smem + OFF_P + ((z + NPLANE) % NPLANE) * P_BYTES);
      };
      mftc_stage_plane(plane(z0 - 1), z0 - 1, y0, x0, ny1, nx1, nz1, t, x, m32);
      mftc_commit();
      mftc_stage_plane(plane(z0), z0, y0, x0, ny1, nx1, nz1, t, x, m32);
      mftc_commit();
      for (int c = z0 - 1; c < z1; ++c, ++L) {
        if (c + 2 <= z1) mftc_stage_plane(plane(c + 2), c + 2, y0, x0, ny1, nx1, nz1, t, x, m32);
        mftc_commit();
        asm volatile("cp.async.wait_group 1;\n" ::);
        // A[L % 2] is free once the MMAs of layer L-2 have completed
        const bool ok = L < 2 || mftc_wait(&full[L & 1], ((L - 2) >> 1) & 1u, abort_f);
        if (mftc_group_sync_or(1, fail || !ok)) { fail = true; break; }
        // A tile of cell layer c: row t = cell (t % 16, t / 16)
        {
          const int rcy = t % CY, rcx = t / CY;
          const int cy = y0 - 1 + rcy, cx = x0 - 1 + rcx;
          const bool cin = c >= 0 && c < g.nz && cy >= 0 && cy < g.ny && cx >= 0 && cx < g.nx;
          const float4* P0 = reinterpret_cast<const float4*>(plane(c));
          const float4* P1 = reinterpret_cast<const float4*>(plane(c + 1));
          float xv[24];
#pragma unroll
          for (int lb = 0; lb < 8; ++lb) {
            const float4* P = hoff(lb, 2) ? P1 : P0;
            const float4 v = P[(rcx + hoff(lb, 0)) * HY + rcy + hoff(lb, 1)];
            float a0 = v.x, a1 = v.y, a2 = v.z;
            if (COLMASK) {
              const int mk = __float_as_int(v.w);
              a0 = (mk & 1) ? 0.f : a0;
              a1 = (mk & 2) ? 0.f : a1;
              a2 = (mk & 4) ? 0.f : a2;
            }
            xv[3 * lb + 0] = cin ? a0 : 0.f;
            xv[3 * lb + 1] = cin ? a1 : 0.f;
            xv[3 * lb + 2] = cin ? a2 : 0.f;
          }
          unsigned char* A = smem + OFF_A + (L & 1) * A_BYTES;
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            float4 hi, lo;
            hi.x = tc::to_tf32(xv[4 * q + 0]);
            hi.y = tc::to_tf32(xv[4 * q + 1]);
            hi.z = tc::to_tf32(xv[4 * q + 2]);
            hi.w = tc::to_tf32(xv[4 * q + 3]);
            lo.x = tc::to_tf32(xv[4 * q + 0] - hi.x);
            lo.y = tc::to_tf32(xv[4 * q + 1] - hi.y);
            lo.z = tc::to_tf32(xv[4 * q + 2] - hi.z);
            lo.w = tc::to_tf32(xv[4 * q + 3] - hi.w);
            *reinterpret_cast<float4*>(A + tc::kmaj_off(t, 4 * q, SBO_A)) = hi;
            *reinterpret_cast<float4*>(A + tc::kmaj_off(t, 24 + 4 * q, SBO_A)) = lo;
          }
          tc::fence_async_smem();
        }
        mftc_group_sync(1);
        if (t == 0) {
          // TMEM buffer L % 2 is free once the drainers have read layer L-2
          const bool ok0 = L < 2 || mftc_wait(&empty[L & 1], ((L - 2) >> 1) & 1u, abort_f);
          if (ok0) {
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_u32(smem + OFF_A + (L & 1) * A_BYTES);
            const uint32_t bh = tc::smem_u32(Bs), bl = bh + B_BYTES;
            const uint32_t d = tmem + (L & 1) * 32u;
#pragma unroll
            for (int s = 0; s < 6; ++s)
              tc::mma_tf32(d, tc::sdesc(a0 + 256u * s, 128u, SBO_A),
                           tc::sdesc(bh + 256u * (s % 3), 128u, SBO_B), idesc, s > 0 ? 1u : 0u);
#pragma unroll
            for (int s = 0; s < 3; ++s)
              tc::mma_tf32(d, tc::sdesc(a0 + 256u * s, 128u, SBO_A),
                           tc::sdesc(bl + 256u * s, 128u, SBO_B), idesc, 1u);
            tc::mma_commit(&full[L & 1]);
          } else {
            *const_cast<int*>(abort_f) = 1;
            fail = true;
          }
        }
      }
      asm volatile("cp.async.wait_group 0;\n" ::);
    }
  } else {
    const int e = t;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    for (int item = blockIdx.x; item < nitems && !fail; item += gridDim.x) {
      const int col = item % (G.ncy * G.ncx), seg = item / (G.ncy * G.ncx);
      const int y0 = (col % G.ncy) * NY, x0 = (col / G.ncy) * NX;
      const int z0 = seg * G.zs, z1 = min(nz1, z0 + G.zs);
      mftc_stage_own<MODE>(smem + OFF_E, z0 - 1, y0, x0, g, e, coef, x, m32, bsrc);
      mftc_commit();
      int i = 0;
      for (int c = z0 - 1; c < z1; ++c, ++L, ++i) {
        unsigned char* S = smem + OFF_E + (i & 1) * E_BYTES;
        mftc_stage_own<MODE>(smem + OFF_E + ((i + 1) & 1) * E_BYTES, c + 1, y0, x0, g, e,
                             coef, x, m32, bsrc);
        mftc_commit();
        const bool ok = mftc_wait(&full[L & 1], (L >> 1) & 1u, abort_f);
        if (mftc_group_sync_or(2, fail || !ok)) { fail = true; break; }
        tc::fence_after_sync();
        float v[32];
        tc::tmem_ld32(tmem + (L & 1) * 32u + lane_base, v);
        tc::fence_before_sync();
        mftc_arrive(&empty[L & 1]);
        asm volatile("cp.async.wait_group 1;\n" ::);
        const float sc = reinterpret_cast<const float*>(S + E_COEF)[e];
        float* Yr = reinterpret_cast<float*>(smem + OFF_Y + (L & 1) * Y_BYTES) + e * YS;
#pragma unroll
        for (int la = 0; la < 8; ++la)
          *reinterpret_cast<float4*>(Yr + 4 * la) =
              make_float4(sc * v[3 * la], sc * v[3 * la + 1], sc * v[3 * la + 2], 0.f);
        mftc_group_sync(2);
        // node plane c from cell layers c - 1 (Y[(L-1) % 2]) and c (Y[L % 2])
        if (c >= z0 && e < NPN) {
          const int ly = e % NY, lx = e / NY;
          const int iy = y0 + ly, ix = x0 + lx;
          if (iy < ny1 && ix < nx1) {
            const float* Yc = reinterpret_cast<const float*>(smem + OFF_Y + (L & 1) * Y_BYTES);
            const float* Yb =
                reinterpret_cast<const float*>(smem + OFF_Y + ((L + 1) & 1) * Y_BYTES);
            float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f;
#pragma unroll
            for (int la = 0; la < 8; ++la) {
              const int m = (ly + 1 - hoff(la, 1)) + CY * (lx + 1 - hoff(la, 0));
              const float* Yl = hoff(la, 2) ? Yb : Yc;
              const float4 w = *reinterpret_cast<const float4*>(Yl + m * YS + 4 * la);
              acc0 += w.x;
              acc1 += w.y;
              acc2 += w.z;
            }
            const float4 self = reinterpret_cast<const float4*>(S + E_SELF)[e];
            const float* s3 = reinterpret_cast<const float*>(S + E_SRC) + e * 3;
            const int ma = __float_as_int(self.w);
            const int64_t a = (int64_t)iy + (int64_t)ny1 * (ix + (int64_t)nx1 * c);
            const float acc[3] = {acc0, acc1, acc2};
            const float xs[3] = {self.x, self.y, self.z};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              const float ax = ((ma >> d) & 1) ? xs[d] : acc[d];
              const float out = MODE == 0 ? ax : s3[d] - ax;
              y[a * 3 + d] = out;
              if (DOT) tacc += xs[d] * out;
            }
          }
        }
        mftc_group_sync(2);
      }
      asm volatile("cp.async.wait_group 0;\n" ::);
    }
  }
  if (fail) *const_cast<int*>(abort_f) = 1;
  __syncthreads();
  if (*abort_f) {
    // let MMAs still in flight finish before the tensor memory is released
    for (int k = 0; k < 20000; ++k) __nanosleep(1000);
    if (tid == 0) {
      atomicExch(err, 1);
      y[0] = __int_as_float(0x7fc00000);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, TMEM_COLS);
  if (DOT) {
    double dacc[1] = {(double)tacc};
    __shared__ double sh[32];
    block_sum<double, 1>(dacc, sh);
    grid_finish<double, 1>(dacc, partials, counter, dot_out);
  }
}

}  // namespace topt
