// D3Q19 and D3Q27 lattice constants shared by host and device code.
//
// The population order is the reference's (src/var.cu:29-35): rest, the six faces, the
// twelve edges, then (D3Q27 only) the eight corners, with opposite pairs (1,2), (3,4), ...,
// (25,26). D3Q19 weights are 1/3, 1/18 and 1/36 (src/var.cu:40-45); D3Q27 weights are
// 8/27, 2/27, 1/54 and 1/216 (src/var.cu:47-52); cs^2 = 1/3 for both (src/var.cu:22).
// Every index below is a compile-time constant at its use, so the tables fold away in the
// kernels. g and the phi stencils always use D3Q19; f uses D3Q19 or D3Q27.
#pragma once

#include <type_traits>
#include <utility>

#if defined(__CUDACC__)
#define MCB_HD __host__ __device__ __forceinline__
#else
#define MCB_HD inline
#endif

namespace mcb {

constexpr int kQ = 19;

constexpr int kQ27 = 27;

MCB_HD constexpr int cx(int l) {
  return (l == 1 || l == 7 || l == 9 || l == 13 || l == 15 || l == 19 || l == 21 || l == 23 ||
          l == 26) ? 1
       : (l == 2 || l == 8 || l == 10 || l == 14 || l == 16 || l == 20 || l == 22 || l == 24 ||
          l == 25) ? -1 : 0;
}
MCB_HD constexpr int cy(int l) {
  return (l == 3 || l == 7 || l == 11 || l == 14 || l == 17 || l == 19 || l == 21 || l == 24 ||
          l == 25) ? 1
       : (l == 4 || l == 8 || l == 12 || l == 13 || l == 18 || l == 20 || l == 22 || l == 23 ||
          l == 26) ? -1 : 0;
}
MCB_HD constexpr int cz(int l) {
  return (l == 5 || l == 9 || l == 11 || l == 16 || l == 18 || l == 19 || l == 22 || l == 23 ||
          l == 25) ? 1
       : (l == 6 || l == 10 || l == 12 || l == 15 || l == 17 || l == 20 || l == 21 || l == 24 ||
          l == 26) ? -1 : 0;
}
// Opposite direction: pairs (2k-1, 2k).
MCB_HD constexpr int opp(int l) { return l == 0 ? 0 : ((l & 1) ? l + 1 : l - 1); }
// Weight class: 0 rest, 1 face, 2 edge.
MCB_HD constexpr int wclass(int l) { return l == 0 ? 0 : (l <= 6 ? 1 : 2); }
MCB_HD constexpr float wf(int l) {
  return l == 0 ? (1.0f / 3.0f) : (l <= 6 ? (1.0f / 18.0f) : (1.0f / 36.0f));
}
MCB_HD constexpr double wd(int l) {
  return l == 0 ? (1.0 / 3.0) : (l <= 6 ? (1.0 / 18.0) : (1.0 / 36.0));
}
// Weights of the f lattice (QF = 19 or 27).
template <int QF>
MCB_HD constexpr float wfq(int l) {
  if constexpr (QF == 19) {
    return wf(l);
  } else {
    return l == 0 ? (8.0f / 27.0f)
         : (l <= 6 ? (2.0f / 27.0f) : (l <= 18 ? (1.0f / 54.0f) : (1.0f / 216.0f)));
  }
}

// Exact integer split of a Q2.30 phi value over the 19 weights, for the weight part of the
// 16-bit deviation form:
//   - a face part ~ P/18: the high word of P * ceil(2^32/18), one multiply;
//   - an edge part: half of the face part;
//   - the rest part: the remainder.
// So the 19 parts add back to P exactly. Any deterministic split would keep the phi sum
// exact; this one keeps every part within one unit of W_l * P.
MCB_HD int wsplit_face(int p) {
#if defined(__CUDA_ARCH__)
  return __mulhi(p, 238609295);
#else
  return static_cast<int>((static_cast<long long>(p) * 238609295LL) >> 32);
#endif
}
MCB_HD int wsplit_edge_of_face(int wf) { return wf >> 1; }
MCB_HD int wsplit_edge(int p) { return wsplit_edge_of_face(wsplit_face(p)); }
MCB_HD int wsplit_rest(int p) {
  const int f = wsplit_face(p);
  return p - 6 * f - 12 * wsplit_edge_of_face(f);
}
template <int L>
MCB_HD int wsplit(int p) {
  if constexpr (L == 0) return wsplit_rest(p);
  else if constexpr (L <= 6) return wsplit_face(p);
  else return wsplit_edge(p);
}

// Q2.30 fixed point: 1.0 = 2^30.
constexpr float kQ30 = 1073741824.0f;
constexpr float kInvQ30 = 1.0f / 1073741824.0f;

// Compile-time loop: f(std::integral_constant<int, I>{}) for I in [B, E).
template <int B, int E, class F>
MCB_HD void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

}  // namespace mcb
