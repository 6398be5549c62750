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
// accumulates in tensor memory (9 MMAs of 128 x 32 x 8).  The epilogue scales
// row m by coef_m and stores it to shared memory; each node then sums the
// rows of its 8 cells (two consecutive cell layers) in a fixed order, so the
// result is deterministic.  Cells on the column's border are computed by
// both neighbouring columns (16 x 8 cells for 15 x 7 nodes).
//
// Pipeline per layer iteration i (cell layer c = z0 - 1 + i):
//   prefetch (cp.async) node plane c+2, coefficients of layer c+1, b/y of
//   node plane c; build the A tile of layer c; one thread issues its 9 MMAs
//   into TMEM buffer i%2 and commits them to mbarrier i%2; meanwhile all
//   threads drain layer c-1 (TMEM buffer (i-1)%2) into shared memory and
//   produce node plane c-1.  A, TMEM and Y are double-buffered; node planes
//   and coefficients sit in rings of four.
//
// Every wait on an mbarrier is bounded: on a timeout the CTA writes a NaN
// into y (the solvers then stop with a non-finite status), records the error,
// frees its tensor memory and returns.
#pragma once

#include "tc_sm100.cuh"

namespace topt {

namespace mftc {
constexpr int CY = 16, CX = 8;              // cells per layer tile
constexpr int NY = CY - 1, NX = CX - 1;     // output nodes per plane
constexpr int HY = CY + 1, HX = CX + 1;     // halo nodes per plane
constexpr int M = CY * CX;                  // 128 = MMA rows
constexpr int NPN = NY * NX;                // 105 output nodes per plane
constexpr int THREADS = 128;
constexpr uint32_t SBO_A = 12 * 128;        // 48 K columns = 12 core matrices
constexpr uint32_t SBO_B = 6 * 128;         // 24 K columns
constexpr int YS = 36;                      // floats per Y row (8 x float4 + pad)
constexpr uint32_t A_BYTES = M * 48 * 4;    // 24576
constexpr uint32_t B_BYTES = 32 * 24 * 4;   // 3072 per split part
constexpr uint32_t Y_BYTES = M * YS * 4;    // 18432
constexpr uint32_t P_BYTES = HY * HX * 16;  // 2448 (float4 per halo node)
constexpr uint32_t C_BYTES = M * 4;         // 512
constexpr uint32_t S_BYTES = NPN * 3 * 4;   // 1260
constexpr uint32_t OFF_A = 0;
constexpr uint32_t OFF_B = OFF_A + 2 * A_BYTES;
constexpr uint32_t OFF_Y = OFF_B + 2 * B_BYTES;
constexpr uint32_t OFF_P = OFF_Y + 2 * Y_BYTES;
constexpr uint32_t OFF_C = OFF_P + 4 * P_BYTES;
constexpr uint32_t OFF_S = OFF_C + 4 * C_BYTES;
constexpr uint32_t OFF_BAR = (OFF_S + 4 * S_BYTES + 15) & ~15u;
constexpr uint32_t SMEM = OFF_BAR + 32;
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

// Node plane z of the column's halo: x in .xyz, the fixed-DOF bits in .w,
// zeros outside the grid.
__device__ __forceinline__ void mftc_stage_plane(float* P, int z, int y0, int x0, int ny1,
                                                 int nx1, int nz1, const float* __restrict__ x,
                                                 const uint32_t* __restrict__ m32) {
  using namespace mftc;
  const bool zin = z >= 0 && z < nz1;
  for (int q = threadIdx.x; q < HY * HX; q += THREADS) {
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

// Coefficients of cell layer c (zero outside the grid).
__device__ __forceinline__ void mftc_stage_coef(float* Cs, int c, int y0, int x0,
                                                const MfGrid& g,
                                                const float* __restrict__ coef) {
  using namespace mftc;
  const int m = threadIdx.x;
  const int cy = y0 - 1 + (m % CY), cx = x0 - 1 + (m / CY);
  const bool in = c >= 0 && c < g.nz && cy >= 0 && cy < g.ny && cx >= 0 && cx < g.nx;
  const int64_t e = in ? (int64_t)cy + (int64_t)g.ny * (cx + (int64_t)g.nx * c) : 0;
  mftc_cp4(Cs + m, coef + e, in);
}

// b (MODE 1) or y (MODE 2) of the column's output nodes on plane z.
__device__ __forceinline__ void mftc_stage_src(float* S, int z, int y0, int x0, int ny1,
                                               int nx1, int nz1,
                                               const float* __restrict__ src) {
  using namespace mftc;
  for (int q = threadIdx.x; q < NPN * 3; q += THREADS) {
    const int t = q / 3, d = q % 3;
    const int gy = y0 + t % NY, gx = x0 + t / NY;
    const bool in = z >= 0 && z < nz1 && gy < ny1 && gx < nx1;
    const int64_t n = in ? (int64_t)gy + (int64_t)ny1 * (gx + (int64_t)nx1 * z) : 0;
    mftc_cp4(S + q, src + n * 3 + d, in);
  }
}

template <int MODE, bool DOT, bool COLMASK>
__global__ void __launch_bounds__(mftc::THREADS)
k_mf_tc(MfTcGrid G, const float* __restrict__ k0img, const float* __restrict__ coef,
        const uint32_t* __restrict__ m32, const float* __restrict__ x,
        const float* __restrict__ b, float* __restrict__ y, double* partials,
        unsigned* counter, double* dot_out, int* err) {
  TOPT_KERNEL_COUNT();
  using namespace mftc;
  extern __shared__ __align__(1024) unsigned char mftc_smem[];
  unsigned char* smem = mftc_smem;
  float* Bs = reinterpret_cast<float*>(smem + OFF_B);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + OFF_BAR + 16);
  const int tid = threadIdx.x, warp = tid >> 5;
  const MfGrid& g = G.g;
  const int ny1 = g.ny + 1, nx1 = g.nx + 1, nz1 = g.nz + 1;
  const float* bsrc = MODE == 1 ? b : y;

  // K0 hi / lo image (already in the B operand layout)
  for (int i = tid; i < K0_IMAGE_FLOATS / 4; i += THREADS)
    reinterpret_cast<float4*>(Bs)[i] = reinterpret_cast<const float4*>(k0img)[i];
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_init_fence();
  }
  if (warp == 0) tc::tmem_alloc(tslot, TMEM_COLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
  const uint32_t idesc = tc::idesc_tf32(M, 32);
  // bit b: parity of the next phase of bar[b] / an MMA group committed to
  // bar[b] and not yet waited for
  uint32_t phase = 0u, pend = 0u;
  bool failed = false;
  float tacc = 0.0f;

  const int nitems = G.ncy * G.ncx * G.nseg;
  for (int item = blockIdx.x; item < nitems && !failed; item += gridDim.x) {
    const int col = item % (G.ncy * G.ncx), seg = item / (G.ncy * G.ncx);
    const int y0 = (col % G.ncy) * NY, x0 = (col / G.ncy) * NX;
    const int z0 = seg * G.zs, z1 = min(nz1, z0 + G.zs);
    const int niter = z1 - z0 + 2;
    // prologue: node planes z0-1 and z0, coefficients of cell layer z0-1
    mftc_stage_plane(reinterpret_cast<float*>(smem + OFF_P + ((z0 - 1) & 3) * P_BYTES),
                     z0 - 1, y0, x0, ny1, nx1, nz1, x, m32);
    mftc_stage_plane(reinterpret_cast<float*>(smem + OFF_P + (z0 & 3) * P_BYTES), z0, y0,
                     x0, ny1, nx1, nz1, x, m32);
    mftc_stage_coef(reinterpret_cast<float*>(smem + OFF_C + ((z0 - 1) & 3) * C_BYTES),
                    z0 - 1, y0, x0, g, coef);
    asm volatile("cp.async.commit_group;\n" ::);
    for (int i = 0; i < niter; ++i) {
      const int c = z0 - 1 + i;               // cell layer of this iteration's MMA
      const bool do_mma = i <= z1 - z0;       // layers z0-1 .. z1-1
      const bool mma_valid = do_mma && c >= 0 && c < g.nz;
      asm volatile("cp.async.wait_group 0;\n" ::);
      __syncthreads();
      // prefetch for the next iterations
      if (i + 1 <= z1 - z0)
        mftc_stage_plane(reinterpret_cast<float*>(smem + OFF_P + ((c + 2) & 3) * P_BYTES),
                         c + 2, y0, x0, ny1, nx1, nz1, x, m32);
      mftc_stage_coef(reinterpret_cast<float*>(smem + OFF_C + ((c + 1) & 3) * C_BYTES),
                      c + 1, y0, x0, g, coef);
      if (MODE != 0)
        mftc_stage_src(reinterpret_cast<float*>(smem + OFF_S + (c & 3) * S_BYTES), c, y0,
                       x0, ny1, nx1, nz1, bsrc);
      asm volatile("cp.async.commit_group;\n" ::);
      // A tile of cell layer c: row tid = cell (tid % 16, tid / 16)
      if (mma_valid) {
        const int rcy = tid % CY, rcx = tid / CY;
        const int cy = y0 - 1 + rcy, cx = x0 - 1 + rcx;
        const bool cin = cy >= 0 && cy < g.ny && cx >= 0 && cx < g.nx;
        const float4* P0 =
            reinterpret_cast<const float4*>(smem + OFF_P + (c & 3) * P_BYTES);
        const float4* P1 =
            reinterpret_cast<const float4*>(smem + OFF_P + ((c + 1) & 3) * P_BYTES);
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
        unsigned char* A = smem + OFF_A + (i & 1) * A_BYTES;
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
          *reinterpret_cast<float4*>(A + tc::kmaj_off(tid, 4 * q, SBO_A)) = hi;
          *reinterpret_cast<float4*>(A + tc::kmaj_off(tid, 24 + 4 * q, SBO_A)) = lo;
        }
        tc::fence_async_smem();
      }
      __syncthreads();
      if (mma_valid) pend |= 1u << (i & 1);
      if (mma_valid && tid == 0) {
        tc::fence_after_sync();
        const uint32_t a0 = tc::smem_u32(smem + OFF_A + (i & 1) * A_BYTES);
        const uint32_t bh = tc::smem_u32(Bs), bl = bh + B_BYTES;
        const uint32_t d = tmem + (uint32_t)(i & 1) * 32u;
#pragma unroll
        for (int s = 0; s < 6; ++s)
          tc::mma_tf32(d, tc::sdesc(a0 + 256u * s, 128u, SBO_A),
                       tc::sdesc(bh + 256u * (s % 3), 128u, SBO_B), idesc, s > 0 ? 1u : 0u);
#pragma unroll
        for (int s = 0; s < 3; ++s)
          tc::mma_tf32(d, tc::sdesc(a0 + 256u * s, 128u, SBO_A),
                       tc::sdesc(bl + 256u * s, 128u, SBO_B), idesc, 1u);
        tc::mma_commit(&bar[i & 1]);
      }
      // drain cell layer c-1 (previous iteration's MMA) into Y[(i-1)%2]
      if (i >= 1) {
        const int cp = c - 1;
        const int pb = (i - 1) & 1;
        float* Yr = reinterpret_cast<float*>(smem + OFF_Y + pb * Y_BYTES) + tid * YS;
        if (cp >= 0 && cp < g.nz) {
          const bool ok = tc::mbar_wait(&bar[pb], (phase >> pb) & 1u, WAIT_LIMIT);
          phase ^= 1u << pb;
          pend &= ~(1u << pb);
          if (__syncthreads_or(!ok)) {
            failed = true;
            break;
          }
          tc::fence_after_sync();
          float v[32];
          tc::tmem_ld32(tmem + (uint32_t)pb * 32u + lane_base, v);
          const float s = reinterpret_cast<const float*>(smem + OFF_C +
                                                         (cp & 3) * C_BYTES)[tid];
#pragma unroll
          for (int la = 0; la < 8; ++la)
            *reinterpret_cast<float4*>(Yr + 4 * la) =
                make_float4(s * v[3 * la], s * v[3 * la + 1], s * v[3 * la + 2], 0.f);
          tc::fence_before_sync();
        } else {
#pragma unroll
          for (int la = 0; la < 8; ++la)
            *reinterpret_cast<float4*>(Yr + 4 * la) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
      __syncthreads();
      // node plane j = c - 1 from cell layers j - 1 and j
      const int j = c - 1;
      if (i >= 2 && tid < NPN) {
        const int ly = tid % NY, lx = tid / NY;
        const int iy = y0 + ly, ix = x0 + lx;
        if (iy < ny1 && ix < nx1) {
          const float* Yc = reinterpret_cast<const float*>(smem + OFF_Y + ((i - 1) & 1) * Y_BYTES);
          const float* Yb = reinterpret_cast<const float*>(smem + OFF_Y + (i & 1) * Y_BYTES);
          float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f;
#pragma unroll
          for (int la = 0; la < 8; ++la) {
            const int m = (ly + 1 - hoff(la, 1)) + CY * (lx + 1 - hoff(la, 0));
            const float* Yl = hoff(la, 2) ? Yb : Yc;
            const float4 v = *reinterpret_cast<const float4*>(Yl + m * YS + 4 * la);
            acc0 += v.x;
            acc1 += v.y;
            acc2 += v.z;
          }
          const float4 self = reinterpret_cast<const float4*>(
              smem + OFF_P + (j & 3) * P_BYTES)[(lx + 1) * HY + ly + 1];
          const int ma = __float_as_int(self.w);
          const float* S = reinterpret_cast<const float*>(smem + OFF_S + (j & 3) * S_BYTES);
          const int64_t a = (int64_t)iy + (int64_t)ny1 * (ix + (int64_t)nx1 * j);
          const float acc[3] = {acc0, acc1, acc2};
          const float xs[3] = {self.x, self.y, self.z};
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float ax = ((ma >> d) & 1) ? xs[d] : acc[d];
            const float out = MODE == 0 ? ax : S[tid * 3 + d] - ax;
            y[a * 3 + d] = out;
            if (DOT) tacc += xs[d] * out;
          }
        }
      }
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();
  }
  if (failed) {
    // let the MMAs still in flight finish (bounded) before the tensor
    // memory is released
    for (int bb = 0; bb < 2; ++bb)
      if ((pend >> bb) & 1u) tc::mbar_wait(&bar[bb], (phase >> bb) & 1u, WAIT_LIMIT);
    asm volatile("cp.async.wait_group 0;\n" ::);
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
