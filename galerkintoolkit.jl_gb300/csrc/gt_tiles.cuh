// gt_tiles.cuh -- scalar CSR SpMV over row tiles staged in shared memory by
// bulk asynchronous copies (TMA engine, cp.async.bulk + mbarrier).
//
// The rows of the matrix are cut into tiles of R = 256 / G consecutive rows.
// The column indices and values of a tile are one contiguous segment of the
// CSR arrays, so each tile is moved into shared memory by two bulk copies
// (16-byte aligned: the segment is widened to 16-byte boundaries, and every
// device block of this library has 16 bytes of slack past its end).  A CTA
// walks its tiles with two buffers: the copy of the next tile is in flight
// while the current one is multiplied, so the value/index stream runs at
// copy-engine speed and the threads only gather x.  Each row is handled by G
// lanes (entries k = gl, gl + G, ... of the row, summed in that order, then
// a butterfly over the G lanes): a fixed summation order per row.
//
// Waits on the mbarrier are bounded; a copy that does not complete within
// the limit sets bit DEV_ERR_TIMEOUT of the error word, the CTA waits once
// more (bounded) for its copies and returns.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gt {

constexpr int TILE_T = 256;          // threads per CTA
constexpr int TILE_CAP = 4096;       // entries per tile buffer (index + value)
constexpr uint32_t DEV_ERR_TIMEOUT = 64u;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// one bounded wait for the phase `parity` of bar; true when it completed
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <class V>
struct TileBuf {
  static constexpr int kIdx = TILE_CAP + 8;                       // int32 slots (16-byte widening)
  static constexpr int kVal = TILE_CAP + 16 / (int)sizeof(V) * 2;  // V slots
  static constexpr size_t kIdxBytes = ((size_t)kIdx * 4 + 15) / 16 * 16;
  static constexpr size_t kBytes = kIdxBytes + ((size_t)kVal * sizeof(V) + 15) / 16 * 16;
};

template <class V>
constexpr size_t tiles_smem_bytes() {
  return 2 * TileBuf<V>::kBytes + 64;
}

// issues the copies of tile t into buffer (idx, val); returns the offsets
// of the tile's first entry inside the buffers and the entry range
template <int R, class V>
__device__ __forceinline__ void tile_issue(const int64_t* rowptr, const int32_t* colind, const V* val, int64_t nrows,
                                           int64_t t, int32_t* sidx, V* sval, uint64_t* bar) {
  const int64_t r0 = t * R, r1 = min(nrows, r0 + R);
  const int64_t s = rowptr[r0], e = rowptr[r1];
  const uintptr_t ci0 = (uintptr_t)(colind + s) & ~(uintptr_t)15, ci1 = ((uintptr_t)(colind + e) + 15) & ~(uintptr_t)15;
  const uintptr_t v0 = (uintptr_t)(val + s) & ~(uintptr_t)15, v1 = ((uintptr_t)(val + e) + 15) & ~(uintptr_t)15;
  const uint32_t bi = (uint32_t)(ci1 - ci0), bv = (uint32_t)(v1 - v0);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(bar, bi + bv);
  if (bi) bulk_copy_g2s(sidx, (const void*)ci0, bi, bar);
  if (bv) bulk_copy_g2s(sval, (const void*)v0, bv, bar);
}

// y = A x (or y = bsub - A x) over tiles of R = TILE_T / G rows; with DOT
// the CTA also returns the partial sum of (A x) . x over its rows (for CG:
// p . A p)
template <int G, class V, class X, bool DOT>
__device__ __forceinline__ bool spmv_tiles(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                           const V* __restrict__ val, const X* __restrict__ x,
                                           const X* __restrict__ bsub, X* __restrict__ y, int64_t nrows,
                                           unsigned char* smem, uint32_t* err, X* dot) {
  constexpr int R = TILE_T / G;
  using B = TileBuf<V>;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  unsigned char* b0 = smem + 64;
  int32_t* sidx[2] = {reinterpret_cast<int32_t*>(b0), reinterpret_cast<int32_t*>(b0 + B::kBytes)};
  V* sval[2] = {reinterpret_cast<V*>(b0 + B::kIdxBytes), reinterpret_cast<V*>(b0 + B::kBytes + B::kIdxBytes)};
  __shared__ int s_fail;
  const int tid = threadIdx.x, gl = tid % G, grp = tid / G;
  const int64_t ntiles = (nrows + R - 1) / R;
  if (tid == 0) {
    mbar_init(&bars[0]);
    mbar_init(&bars[1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
  }
  __syncthreads();
  X acc_dot = (X)0;
  int64_t t = blockIdx.x;
  int b = 0;
  uint32_t ph[2] = {0u, 0u};
  if (tid == 0 && t < ntiles) tile_issue<R, V>(rowptr, colind, val, nrows, t, sidx[0], sval[0], &bars[0]);
  while (t < ntiles) {
    const int64_t tn = t + gridDim.x;
    if (tid == 0) {
      if (tn < ntiles) tile_issue<R, V>(rowptr, colind, val, nrows, tn, sidx[b ^ 1], sval[b ^ 1], &bars[b ^ 1]);
      if (!mbar_wait(&bars[b], ph[b])) s_fail = 1;
    }
    __syncthreads();
    if (s_fail) break;
    mbar_wait(&bars[b], ph[b]);  // completes at once: acquires the copied bytes for this thread
    ph[b] ^= 1u;
    // rows of tile t
    const int64_t r0 = t * R;
    const int64_t s = rowptr[r0];
    const int oi = (int)(((uintptr_t)(colind + s) & 15) / 4);
    const int ov = (int)(((uintptr_t)(val + s) & 15) / sizeof(V));
    const int64_t row = r0 + grp;
    const bool valid = row < nrows;
    X acc = (X)0;
    if (valid) {
      const int64_t kb = rowptr[row] - s, ke = rowptr[row + 1] - s;
      const int32_t* ci = sidx[b] + oi;
      const V* cv = sval[b] + ov;
      int64_t k = kb + gl;
      for (; k + 3 * G < ke; k += 4 * G) {
        const int32_t j0 = ci[k], j1 = ci[k + G], j2 = ci[k + 2 * G], j3 = ci[k + 3 * G];
        const X x0 = x[j0], x1 = x[j1], x2 = x[j2], x3 = x[j3];
        acc = fma((X)cv[k], x0, acc);
        acc = fma((X)cv[k + G], x1, acc);
        acc = fma((X)cv[k + 2 * G], x2, acc);
        acc = fma((X)cv[k + 3 * G], x3, acc);
      }
      for (; k < ke; k += G) acc = fma((X)cv[k], x[ci[k]], acc);
    }
#pragma unroll
    for (int o = G >> 1; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (gl == 0 && valid) {
      y[row] = bsub ? bsub[row] - acc : acc;
      if (DOT) acc_dot = fma(acc, x[row], acc_dot);
    }
    __syncthreads();  // buffer b is free again
    t = tn;
    b ^= 1;
  }
  if (s_fail) {
    if (tid == 0) {
      atomicOr(err, DEV_ERR_TIMEOUT);
      // copies still in flight land before the CTA leaves
      mbar_wait(&bars[0], ph[0]);
      mbar_wait(&bars[1], ph[1]);
    }
    __syncthreads();
    return false;
  }
  if (DOT) *dot = acc_dot;
  return true;
}

}  // namespace gt
