// gt_rowdot.cuh -- one block row of a block-CSR matrix times a vector, with
// G lanes per row (shared by every SpMV of the library).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gt {

// Lanes per block row for a mean of `avg` blocks per row.  Measured on
// GB300 (scalar FP64/FP32 CSR of P1 tetrahedra, Q1 and Q2 hexahedra): few
// lanes per row with several entries per lane in flight beat wide rows --
// the shuffle reduction of a wide row costs FP64 issue slots (GB300 issues
// FP64 at a fixed cost per warp instruction, however many lanes are
// active), and short per-lane runs keep too few loads in flight.
inline int row_lanes(double avg) {
  if (avg <= 8) return 1;
  if (avg <= 40) return 2;
  if (avg <= 160) return 4;
  return 8;
}

// Entries per lane per trip: all index loads, then all value loads, then
// all gathers of a trip are independent and in flight together.
template <int BS, int G>
struct RowUnroll {
  static constexpr int value = BS > 1 ? 2 : (G == 1 ? 8 : 4);
};

// out[c] = sum_k A[r, k] x[col k] for the BS components of block row r.
// All G lanes of the group call it (it ends in shuffles over the group) and
// every lane gets the result; lane gl sums entries gl, gl + G, ... in that
// order (a fixed summation order per row).  V: value type, A: accumulation
// type, XV: type of x.  L2ONLY: gather x through L2 (x written by other CTAs
// of the same launch); otherwise through L1.
template <int BS, int G, class V, class A, class XV, bool L2ONLY>
__device__ __forceinline__ void row_dot(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                        const V* __restrict__ val, const XV* x, int64_t r, int gl, A* out) {
  constexpr int U = RowUnroll<BS, G>::value;
  A acc[BS];
#pragma unroll
  for (int c = 0; c < BS; c++) acc[c] = (A)0;
  const int64_t b = __ldg(rowptr + r), e = __ldg(rowptr + r + 1);
  int64_t k = b + gl;
  for (; k + (U - 1) * G < e; k += U * G) {
    int32_t j[U];
    V a[U][BS * BS];
#pragma unroll
    for (int u = 0; u < U; u++) j[u] = __ldg(colind + k + u * G);
#pragma unroll
    for (int u = 0; u < U; u++)
#pragma unroll
      for (int q = 0; q < BS * BS; q++) a[u][q] = __ldg(val + (k + u * G) * BS * BS + q);
    A xv[U][BS];
#pragma unroll
    for (int u = 0; u < U; u++)
#pragma unroll
      for (int d = 0; d < BS; d++) {
        if constexpr (L2ONLY) xv[u][d] = (A)__ldcg(x + (int64_t)j[u] * BS + d);
        else xv[u][d] = (A)x[(int64_t)j[u] * BS + d];
      }
#pragma unroll
    for (int u = 0; u < U; u++)
#pragma unroll
      for (int c = 0; c < BS; c++)
#pragma unroll
        for (int d = 0; d < BS; d++) acc[c] = fma((A)a[u][c * BS + d], xv[u][d], acc[c]);
  }
  // the lane's remaining entries (at most U - 1 once the loop above ends):
  // one predicated trip, all loads in flight together, added in the same
  // order as a serial loop over them (a short row otherwise pays one
  // index-then-gather latency per leftover entry)
  {
    constexpr int R = U - 1;
    int32_t j[R];
    V a[R][BS * BS];
    A xv[R][BS];
#pragma unroll
    for (int u = 0; u < R; u++) {
      const int64_t kk = k + u * G;
      j[u] = kk < e ? __ldg(colind + kk) : 0;
#pragma unroll
      for (int q = 0; q < BS * BS; q++) a[u][q] = kk < e ? __ldg(val + kk * BS * BS + q) : (V)0;
    }
#pragma unroll
    for (int u = 0; u < R; u++)
#pragma unroll
      for (int d = 0; d < BS; d++) {
        if (k + u * G < e) {
          if constexpr (L2ONLY) xv[u][d] = (A)__ldcg(x + (int64_t)j[u] * BS + d);
          else xv[u][d] = (A)x[(int64_t)j[u] * BS + d];
        } else {
          xv[u][d] = (A)0;
        }
      }
#pragma unroll
    for (int u = 0; u < R; u++)
      if (k + u * G < e)
#pragma unroll
        for (int c = 0; c < BS; c++)
#pragma unroll
          for (int d = 0; d < BS; d++) acc[c] = fma((A)a[u][c * BS + d], xv[u][d], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < BS; c++) {
#pragma unroll
    for (int o = G >> 1; o; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    out[c] = acc[c];
  }
}

}  // namespace gt
