// stencil.cuh -- device helpers shared by every translation unit of the
// library: the block size and the flux-form operator of ebKernels.m.
#pragma once
#include <cuda_runtime.h>

namespace bsam {

constexpr int kBlock = 256;

// x / h2: a true division, or a multiplication by the exact reciprocal when
// h2 is a power of two (then both round identically)
template <bool kPow2, class T>
__device__ __forceinline__ T divh(T x, T h2, T ih2) {
  return kPow2 ? x * ih2 : x / h2;
}

// op2d (EllipticBSAM/src/ebKernels.m:13-25) at interior cell (li, lj),
// 0-based, of a padded array with leading dimension ldq
template <bool kPow2>
__device__ __forceinline__ double op_cell(const double *__restrict__ Qa, int ldq, const double *__restrict__ DeW,
                                          const double *__restrict__ DnS, double cc, int mx, int li, int lj,
                                          double hx2, double hy2, double ihx2, double ihy2) {
  const int c = (li + 1) + (lj + 1) * ldq;
  const double q = Qa[c];
  const double feE = DeW[(li + 1) + lj * (mx + 1)] * (Qa[c + 1] - q);
  const double feW = DeW[li + lj * (mx + 1)] * (q - Qa[c - 1]);
  const double fnN = DnS[li + (lj + 1) * mx] * (Qa[c + ldq] - q);
  const double fnS = DnS[li + lj * mx] * (q - Qa[c - ldq]);
  return (divh<kPow2>(-(feE - feW), hx2, ihx2) - divh<kPow2>(fnN - fnS, hy2, ihy2)) + cc * q;
}

}  // namespace bsam
