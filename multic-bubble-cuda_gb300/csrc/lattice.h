// D3Q19 lattice constants shared by host and device code.
//
// The population order is the reference's (src/var.cu:29-31): rest, the six faces, then
// the twelve edges, with opposite pairs (1,2), (3,4), ..., (17,18). The weights are 1/3,
// 1/18 and 1/36 (src/var.cu:40-45) and cs^2 = 1/3 (src/var.cu:22). Every index below is a
// compile-time constant at its use, so the tables fold away in the kernels.
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

MCB_HD constexpr int cx(int l) {
  return (l == 1 || l == 7 || l == 9 || l == 13 || l == 15) ? 1
       : (l == 2 || l == 8 || l == 10 || l == 14 || l == 16) ? -1 : 0;
}
MCB_HD constexpr int cy(int l) {
  return (l == 3 || l == 7 || l == 11 || l == 14 || l == 17) ? 1
       : (l == 4 || l == 8 || l == 12 || l == 13 || l == 18) ? -1 : 0;
}
MCB_HD constexpr int cz(int l) {
  return (l == 5 || l == 9 || l == 11 || l == 16 || l == 18) ? 1
       : (l == 6 || l == 10 || l == 12 || l == 15 || l == 17) ? -1 : 0;
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
