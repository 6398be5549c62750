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
// accumulates in tensor memory (9 MMAs of 128 x 32 x 8, the A operand in
// tensor memory, K0 in shared memory).  Row m is then scaled by coef_m and
// stored to shared memory; each node sums the rows of its 8 cells (two
// consecutive cell layers) in a fixed order, so the result is
// deterministic.  Cells on the column's border are computed by both
// neighbouring columns (16 x 8 cells for 15 x 7 nodes); cells outside the
// grid have coefficient 0.  Shared memory carries only the node halo, K0
// and the scaled rows (about 0.4 KB per cell): that traffic, not the tensor
// cores, bounds the operator.
//
// Warp roles (320 threads), so that consecutive layers overlap:
//   stager (warp 9): loads the column's node planes (x and fixed bits) into
//     a ring of NPL slots with cp.async, each plane signalled on mbarrier
//     plane_full[slot] and its slot reused after plane_free[slot];
//   builders (warps 0-3, lanes 0-127 of tensor memory): once planes c, c+1
//     have landed and the MMAs of layer L-2 have released A buffer L % 2
//     (mbarrier full[L % 2]), gather the row of layer L's cell, release
//     plane c, split the row into TF32 hi / lo parts in registers and store
//     it to that buffer in tensor memory; then arrive on mbarrier
//     ready[L % 2];
//   issuer (warp 8, one lane): waits ready[L % 2] and, for the accumulator,
//     empty[L % 2] (layer L-2 drained), issues layer L's 9 MMAs and commits
//     them to full[L % 2];
//   drainers (warps 4-7, lanes 0-127 of tensor memory): wait full[L % 2],
//     load the accumulators, release them (empty[L % 2]), scale by the cell
//     coefficients, store Y[L % 2] and produce the node plane of layer L
//     from Y[L % 2] and Y[(L-1) % 2].
// Drainers synchronise internally with a named barrier; every other hand-off
// is an mbarrier.
//
// Every wait is bounded: on a timeout the CTA sets an abort flag that all
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
constexpr int NHALO = HY * HX;              // 153
constexpr int M = CY * CX;                  // 128 = MMA rows
constexpr int NPN = NY * NX;                // 105 output nodes per plane
constexpr int GROUP = 128;                  // threads per builder / drainer role
constexpr int THREADS = 2 * GROUP + 64;     // + the issuing and the staging warp
constexpr uint32_t SBO_A = 12 * 128;        // 48 K columns = 12 core matrices
constexpr uint32_t SBO_B = 6 * 128;         // 24 K columns
// Y rows: the 24 scaled products of a cell, rows 25 floats apart (an odd
// stride: consecutive rows start in different banks)
constexpr int YS = 25;
constexpr uint32_t B_BYTES = 32 * 24 * 4;   // 3072 per split part
constexpr uint32_t Y_BYTES = M * YS * 4;    // 12800
// node planes: per halo node (x, y, z, fixed bits) as one float4
constexpr uint32_t P_BYTES = NHALO * 16;    // 2448
// drainers' per-layer slot: coefficients (128), own node x + flags (105 x
// float4), b or y of the own node (105 x 3)
constexpr uint32_t E_COEF = 0, E_SELF = M * 4, E_SRC = E_SELF + NPN * 16;
constexpr uint32_t E_BYTES = (E_SRC + NPN * 12 + 15) & ~15u;
constexpr uint32_t OFF_B = 0;
constexpr uint32_t OFF_Y = OFF_B + 2 * B_BYTES;
constexpr uint32_t OFF_P = OFF_Y + 2 * Y_BYTES;
// node planes (NPL) and drainer slots (NEL) in rings: plane c + NPL - 1 and
// the drainers' data of layer c + NEL - 1 are loading while layer c is built
__host__ __device__ constexpr uint32_t off_e(int NPL) { return OFF_P + NPL * P_BYTES; }
// mbarriers full, empty, ready [2], plane_full, plane_free [NPL], then the
// tensor-memory address slot and the abort flag
__host__ __device__ constexpr uint32_t off_bar(int NPL, int NEL) {
  return off_e(NPL) + NEL * E_BYTES;
}
__host__ __device__ constexpr uint32_t off_misc(int NPL, int NEL) {
  return off_bar(NPL, NEL) + 48 + 16 * NPL;
}
__host__ __device__ constexpr uint32_t smem_bytes(int NPL, int NEL) {
  return off_misc(NPL, NEL) + 16;
}
// tensor memory: accumulators in columns [0, 64) (two buffers of 32), A
// tiles in [64, 160) (two buffers of 48: x_hi then x_lo)
constexpr uint32_t TMEM_COLS = 256;
constexpr uint32_t TMEM_A0 = 64;
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
template <int N>
__device__ __forceinline__ void mftc_wait_groups() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

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
// flag is set.  WAITK 0 polls with mbarrier.test_wait (never blocks);
// WAITK 1 uses mbarrier.try_wait, which suspends the warp in hardware until
// the phase completes or a system-dependent time limit passes, so waiting
// warps leave the issue slots to working ones.  Both are bounded by the
// poll count.
template <int WAITK>
__device__ __forceinline__ bool mftc_wait(uint64_t* bar, uint32_t parity,
                                          const volatile int* abort_f) {
  const uint32_t a = tc::smem_u32(bar);
  const uint32_t limit = WAITK == 0 ? mftc::WAIT_LIMIT : (mftc::WAIT_LIMIT >> 8);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    if (WAITK == 0)
      asm volatile(
          "{\n .reg .pred P1;\n mbarrier.test_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
          " selp.b32 %0, 1, 0, P1;\n}\n"
          : "=r"(done)
          : "r"(a), "r"(parity)
          : "memory");
    else
      asm volatile(
          "{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
          " selp.b32 %0, 1, 0, P1;\n}\n"
          : "=r"(done)
          : "r"(a), "r"(parity)
          : "memory");
    if (done) return true;
    if ((WAITK == 1 || (i & 255) == 255) && *abort_f) return false;
  }
  return false;
}

__device__ __forceinline__ void mftc_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(tc::smem_u32(bar))
               : "memory");
}

// Per-phase time stamps for experiments (no-op unless defined before this
// header is included).
#ifndef MFTC_MARK
#define MFTC_MARK(role, ev)
#endif

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

// The work item sequence every role walks: (column origin, z range).
struct MftcItem {
  int y0, x0, z0, z1;
};
__device__ __forceinline__ MftcItem mftc_item(const MfTcGrid& G, int item, int nz1) {
  using namespace mftc;
  const int col = item % (G.ncy * G.ncx), seg = item / (G.ncy * G.ncx);
  MftcItem it;
  it.y0 = (col % G.ncy) * NY;
  it.x0 = (col / G.ncy) * NX;
  it.z0 = seg * G.zs;
  it.z1 = min(nz1, it.z0 + G.zs);
  return it;
}

// 96 registers: two CTAs of 320 threads fit the register file (and two
// CTAs take all 512 columns of tensor memory).
template <int MODE, bool DOT, bool COLMASK, int NPL, int NEL, int WAITK>
__global__ void __maxnreg__(96)
k_mf_tc(MfTcGrid G, const float* __restrict__ k0img, const float* __restrict__ coef,
        const uint32_t* __restrict__ m32, const float* __restrict__ x,
        const float* __restrict__ b, float* __restrict__ y, double* partials,
        unsigned* counter, double* dot_out, int* err) {
  TOPT_KERNEL_COUNT();
  using namespace mftc;
  static_assert(NPL >= 3 && NEL >= 2, "rings too short");
  extern __shared__ __align__(1024) unsigned char mftc_smem[];
  unsigned char* smem = mftc_smem;
  float* Bs = reinterpret_cast<float*>(smem + OFF_B);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + off_bar(NPL, NEL));
  uint64_t* empty = full + 2;
  uint64_t* ready = full + 4;
  uint64_t* pfull = full + 6;
  uint64_t* pfree = pfull + NPL;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + off_misc(NPL, NEL));
  volatile int* abort_f = reinterpret_cast<volatile int*>(smem + off_misc(NPL, NEL) + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
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
    tc::mbar_init(&ready[0], GROUP);
    tc::mbar_init(&ready[1], GROUP);
    for (int i = 0; i < NPL; ++i) {
      tc::mbar_init(&pfull[i], 32);
      tc::mbar_init(&pfree[i], GROUP);
    }
    *abort_f = 0;
    tc::mbar_init_fence();
  }
  if (warp == 0) tc::tmem_alloc(tslot, TMEM_COLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  bool fail = false;           // uniform within a role after each role sync
  float tacc = 0.0f;
  uint32_t L = 0;              // running layer count (the same sequence in every role)
  const int nitems = G.ncy * G.ncx * G.nseg;

  if (warp < 4) {
    // ------------------------------------------------------------ builders
    const int t = tid;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    uint32_t kb = 0;   // running index of the item's first node plane
    for (int item = blockIdx.x; item < nitems && !fail; item += gridDim.x) {
      const MftcItem it = mftc_item(G, item, nz1);
      for (int c = it.z0 - 1; c < it.z1; ++c, ++L) {
        MFTC_MARK(0, 0);
        // planes c and c + 1 (running indices kc, kc + 1) staged by the
        // staging warp; A buffer L % 2 free once the MMAs of layer L-2 are done
        const uint32_t kc = kb + (uint32_t)(c - (it.z0 - 1));
        bool ok = c > it.z0 - 1 ||
                  mftc_wait<WAITK>(&pfull[kc % NPL], (kc / NPL) & 1u, abort_f);
        ok = ok && mftc_wait<WAITK>(&pfull[(kc + 1) % NPL], ((kc + 1) / NPL) & 1u, abort_f);
        ok = ok && (L < 2 || mftc_wait<WAITK>(&full[L & 1], ((L - 2) >> 1) & 1u, abort_f));
        if (!ok) {
          fail = true;
          *const_cast<int*>(abort_f) = 1;
          break;
        }
        MFTC_MARK(0, 2);
        // row t of layer c: cell (t % 16, t / 16), split into hi | lo
        float row[48];
        {
          const int rcy = t % CY, rcx = t / CY;
          const float4* P0 =
              reinterpret_cast<const float4*>(smem + OFF_P + (kc % NPL) * P_BYTES);
          const float4* P1 =
              reinterpret_cast<const float4*>(smem + OFF_P + ((kc + 1) % NPL) * P_BYTES);
#pragma unroll
          for (int lb = 0; lb < 8; ++lb) {
            const float4* P = hoff(lb, 2) ? P1 : P0;
            const float4 v = P[(rcx + hoff(lb, 0)) * HY + rcy + hoff(lb, 1)];
            float a[3] = {v.x, v.y, v.z};
            if (COLMASK) {
              const int mk = __float_as_int(v.w);
#pragma unroll
              for (int d = 0; d < 3; ++d) a[d] = ((mk >> d) & 1) ? 0.f : a[d];
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              const float h = tc::to_tf32(a[d]);
              row[3 * lb + d] = h;
              row[24 + 3 * lb + d] = tc::to_tf32(a[d] - h);
            }
          }
        }
        // plane c is not read again (and, after the item's last layer, nor
        // is plane c + 1): its slot may be refilled
        mftc_arrive(&pfree[kc % NPL]);
        if (c == it.z1 - 1) mftc_arrive(&pfree[(kc + 1) % NPL]);
        MFTC_MARK(0, 5);
        tc::fence_after_sync();
        const uint32_t ta = tmem + TMEM_A0 + (L & 1) * 48u + lane_base;
        tc::tmem_st16(ta, row);
        tc::tmem_st16(ta + 16, row + 16);
        tc::tmem_st16(ta + 32, row + 32);
        tc::tmem_st_wait();
        tc::fence_before_sync();
        mftc_arrive(&ready[L & 1]);
        MFTC_MARK(0, 1);
      }
      kb += (uint32_t)(it.z1 - it.z0 + 2);
    }
  } else if (warp < 8) {
    // ------------------------------------------------------------ drainers
    const int e = tid - GROUP;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    for (int item = blockIdx.x; item < nitems && !fail; item += gridDim.x) {
      const MftcItem it = mftc_item(G, item, nz1);
      auto slot = [&](int i) { return smem + off_e(NPL) + (i % NEL) * E_BYTES; };
      // layers z0-1 .. z0+NEL-3 in flight before the first layer
      for (int i = 0; i < NEL - 1; ++i) {
        mftc_stage_own<MODE>(slot(i), it.z0 - 1 + i, it.y0, it.x0, g, e, coef, x, m32, bsrc);
        mftc_commit();
      }
      int i = 0;
      for (int c = it.z0 - 1; c < it.z1; ++c, ++L, ++i) {
        MFTC_MARK(1, 0);
        unsigned char* S = slot(i);
        mftc_stage_own<MODE>(slot(i + NEL - 1), c + NEL - 1, it.y0, it.x0, g, e, coef, x, m32,
                             bsrc);
        mftc_commit();
        const bool ok = mftc_wait<WAITK>(&full[L & 1], (L >> 1) & 1u, abort_f);
        if (mftc_group_sync_or(2, fail || !ok)) { fail = true; break; }
        MFTC_MARK(1, 1);
        tc::fence_after_sync();
        float o[32];
        tc::tmem_ld32(tmem + (L & 1) * 32u + lane_base, o);
        tc::fence_before_sync();
        mftc_arrive(&empty[L & 1]);
        MFTC_MARK(1, 2);
        mftc_wait_groups<NEL - 1>();          // this layer's slot has landed
        const float sc = reinterpret_cast<const float*>(S + E_COEF)[e];
        float* Yr = reinterpret_cast<float*>(smem + OFF_Y + (L & 1) * Y_BYTES) + e * YS;
#pragma unroll
        for (int k = 0; k < 24; ++k) Yr[k] = sc * o[k];
        mftc_group_sync(2);
        MFTC_MARK(1, 3);
        // node plane c from cell layers c - 1 (Y[(L-1) % 2]) and c (Y[L % 2])
        if (c >= it.z0 && e < NPN) {
          const int ly = e % NY, lx = e / NY;
          const int iy = it.y0 + ly, ix = it.x0 + lx;
          if (iy < ny1 && ix < nx1) {
            const float* Yc = reinterpret_cast<const float*>(smem + OFF_Y + (L & 1) * Y_BYTES);
            const float* Yb =
                reinterpret_cast<const float*>(smem + OFF_Y + ((L + 1) & 1) * Y_BYTES);
            float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f;
#pragma unroll
            for (int la = 0; la < 8; ++la) {
              const int m = (ly + 1 - hoff(la, 1)) + CY * (lx + 1 - hoff(la, 0));
              const float* w = (hoff(la, 2) ? Yb : Yc) + m * YS + 3 * la;
              acc0 += w[0];
              acc1 += w[1];
              acc2 += w[2];
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
        MFTC_MARK(1, 4);
      }
      mftc_wait_groups<0>();
    }
  } else if (tid == 2 * GROUP) {
    // ------------------------------------------------------------ issuer
    const uint32_t idesc = tc::idesc_tf32(M, 32);
    const uint32_t bh = tc::smem_u32(Bs), bl = bh + B_BYTES;
    uint64_t db[6];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      db[s] = tc::sdesc(bh + 256u * s, 128u, SBO_B);
      db[3 + s] = tc::sdesc(bl + 256u * s, 128u, SBO_B);
    }
    for (int item = blockIdx.x; item < nitems && !fail; item += gridDim.x) {
      const MftcItem it = mftc_item(G, item, nz1);
      for (int c = it.z0 - 1; c < it.z1; ++c, ++L) {
        MFTC_MARK(0, 3);
        // the A tile of layer L is built and TMEM buffer L % 2 was drained
        // (layer L-2)
        if (!mftc_wait<WAITK>(&ready[L & 1], (L >> 1) & 1u, abort_f) ||
            !(L < 2 || mftc_wait<WAITK>(&empty[L & 1], ((L - 2) >> 1) & 1u, abort_f))) {
          fail = true;
          *const_cast<int*>(abort_f) = 1;
          break;
        }
        tc::fence_after_sync();
        const uint32_t a0 = tmem + TMEM_A0 + (L & 1) * 48u;
        const uint32_t d = tmem + (L & 1) * 32u;
#pragma unroll
        for (int s = 0; s < 6; ++s)
          tc::mma_tf32_ta(d, a0 + 8u * s, db[s % 3], idesc, s > 0 ? 1u : 0u);
#pragma unroll
        for (int s = 0; s < 3; ++s)
          tc::mma_tf32_ta(d, a0 + 8u * s, db[3 + s], idesc, 1u);
        tc::mma_commit(&full[L & 1]);
        MFTC_MARK(0, 4);
      }
    }
  } else if (warp == 9) {
    // ------------------------------------------------------------ stager
    const int l = tid - (2 * GROUP + 32);
    uint32_t k = 0;    // running index of the plane being staged
    for (int item = blockIdx.x; item < nitems && !fail; item += gridDim.x) {
      const MftcItem it = mftc_item(G, item, nz1);
      for (int z = it.z0 - 1; z <= it.z1; ++z, ++k) {
        // the slot's previous plane (k - NPL) has been released by the builders
        if (k >= (uint32_t)NPL &&
            !mftc_wait<WAITK>(&pfree[k % NPL], ((k / NPL) - 1) & 1u, abort_f)) {
          fail = true;
          *const_cast<int*>(abort_f) = 1;
          break;
        }
        float* P = reinterpret_cast<float*>(smem + OFF_P + (k % NPL) * P_BYTES);
        const bool zin = z >= 0 && z < nz1;
        for (int q = l; q < NHALO; q += 32) {
          const int hy = q % HY, hx = q / HY;
          const int gy = it.y0 - 1 + hy, gx = it.x0 - 1 + hx;
          const bool in = zin && gy >= 0 && gy < ny1 && gx >= 0 && gx < nx1;
          const int64_t n = in ? (int64_t)gy + (int64_t)ny1 * (gx + (int64_t)nx1 * z) : 0;
          float* d = P + q * 4;
          mftc_cp4(d + 0, x + n * 3 + 0, in);
          mftc_cp4(d + 1, x + n * 3 + 1, in);
          mftc_cp4(d + 2, x + n * 3 + 2, in);
          mftc_cp4(d + 3, m32 + n, in);
        }
        // one arrival on plane_full per lane once its copies have landed
        asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" ::"r"(
                         tc::smem_u32(&pfull[k % NPL]))
                     : "memory");
      }
    }
    mftc_wait_groups<0>();
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
