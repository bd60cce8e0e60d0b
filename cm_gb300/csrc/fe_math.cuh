// Device helpers shared by the element kernels of libcm_fe: Voigt maps and
// the per-Gauss-point constitutive routines, written after
// FINITE_ELASTICITY_GAUSS_STRESS_TENSOR (finite_elasticity_routines.f90:
// 4342-4454), FINITE_ELASTICITY_GAUSS_ELASTICITY_TENSOR (:609-835) and the
// push-forward routines (:1182-1253), with the reference's order of
// operations.
#pragma once
#include <cuda_runtime.h>

#include "../../include/cm_fe.h"

namespace {

// ------------------------------------------------------------ constants ----
// TENSOR_TO_VOIGT3 / VOIGT_TO_TENSOR3 (constants.f90:284-285), 0-based:
// 11->0 22->1 33->2 12->3 13->4 23->5.  Written as constexpr functions so
// that fully unrolled loops index registers, not local memory.
__host__ __device__ constexpr int t2v(int i, int j) { return i == j ? i : (i + j == 1 ? 3 : (i + j == 2 ? 4 : 5)); }
__host__ __device__ constexpr int v2t0(int v) { return v < 3 ? v : (v == 5 ? 1 : 0); }
__host__ __device__ constexpr int v2t1(int v) { return v < 3 ? v : (v == 3 ? 1 : 2); }

constexpr double ZERO_TOL = 5.0 * 2.220446049250313e-16;  // ZERO_TOLERANCE (constants.f90:68)

// ------------------------------------------------------- device maths ----
__device__ __forceinline__ void d_inv3(const double a[3][3], double b[3][3], double& det) {
  det = a[0][0] * a[1][1] * a[2][2] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
        a[0][0] * a[2][1] * a[1][2] - a[1][0] * a[0][1] * a[2][2] - a[2][0] * a[1][1] * a[0][2];
  if (fabs(det) > ZERO_TOL) {
    b[0][0] = (a[1][1] * a[2][2] - a[2][1] * a[1][2]) / det;
    b[1][0] = (a[1][2] * a[2][0] - a[2][2] * a[1][0]) / det;
    b[2][0] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]) / det;
    b[0][1] = (a[2][1] * a[0][2] - a[0][1] * a[2][2]) / det;
    b[1][1] = (a[2][2] * a[0][0] - a[0][2] * a[2][0]) / det;
    b[2][1] = (a[2][0] * a[0][1] - a[0][0] * a[2][1]) / det;
    b[0][2] = (a[0][1] * a[1][2] - a[1][1] * a[0][2]) / det;
    b[1][2] = (a[0][2] * a[1][0] - a[1][2] * a[0][0]) / det;
    b[2][2] = (a[0][0] * a[1][1] - a[1][0] * a[0][1]) / det;
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) b[i][j] = 0.0;
  }
}

template <class T>
__device__ __forceinline__ T d_pow_m13(T j);
template <>
__device__ __forceinline__ double d_pow_m13<double>(double j) { return pow(j, -1.0 / 3.0); }
template <>
__device__ __forceinline__ float d_pow_m13<float>(float j) { return powf(j, -1.0f / 3.0f); }
template <class T>
__device__ __forceinline__ T d_exp(T v);
template <>
__device__ __forceinline__ double d_exp<double>(double v) { return exp(v); }
template <>
__device__ __forceinline__ float d_exp<float>(float v) { return expf(v); }

// Push-forward matrix t(F) of FINITE_ELASTICITY_PUSH_*_TENSOR (:1182-1253).
template <class T>
__device__ __forceinline__ void d_push_t(const T F[3][3], T t[6][6]) {
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i][j] = F[v2t0(i)][v2t0(j)] * F[v2t1(i)][v2t1(j)];
#pragma unroll
  for (int j = 3; j < 6; ++j)
#pragma unroll
    for (int i = 0; i < 6; ++i)
      t[i][j] = F[v2t0(i)][v2t0(j)] * F[v2t1(i)][v2t1(j)] +
                F[v2t0(i)][v2t1(j)] * F[v2t1(i)][v2t0(j)];
}

// F_bar = F J^(-1/3), AZL = F_bar^T F_bar, and the fictitious 2nd Piola
// stress (and material tangent when C != nullptr) of MR (:4386-4394,
// :684-699) or Guccione (:4419-4424, :758-781).
template <class T>
__device__ void d_fictitious(int law, const T* c, const T F[3][3], T J, T mod[3][3], T S[6], T (*C)[6]) {
  const T s = d_pow_m13<T>(J);
  T azl[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) mod[i][j] = F[i][j] * s;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) azl[i][j] = mod[0][i] * mod[0][j] + mod[1][i] * mod[1][j] + mod[2][i] * mod[2][j];
  if (law == FE_LAW_MOONEY_RIVLIN) {
    const T I1 = azl[0][0] + azl[1][1] + azl[2][2];
    const T t1 = T(-2.0) * c[1];
    const T t2 = T(2.0) * (c[0] + I1 * c[1]);
    S[0] = t1 * azl[0][0] + t2;
    S[1] = t1 * azl[1][1] + t2;
    S[2] = t1 * azl[2][2] + t2;
    S[3] = t1 * azl[1][0];
    S[4] = t1 * azl[2][0];
    S[5] = t1 * azl[2][1];
    if (C) {
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) C[i][j] = T(0);
      const T a = T(4.0) * c[1], b = T(-2.0) * c[1];
      C[1][0] = a; C[2][0] = a; C[0][1] = a; C[2][1] = a; C[0][2] = a; C[1][2] = a;
      C[3][3] = b; C[4][4] = b; C[5][5] = b;
    }
  } else {
    const T B[6] = {T(2.0) * c[1], T(2.0) * c[2], T(2.0) * c[2], c[3], c[3], c[2]};
    const T E[6] = {T(0.5) * (azl[0][0] - T(1.0)), T(0.5) * (azl[1][1] - T(1.0)), T(0.5) * (azl[2][2] - T(1.0)),
                    azl[1][0], azl[2][0], azl[2][1]};
    T DQ[6];
    T dot = T(0);
#pragma unroll
    for (int i = 0; i < 6; ++i) DQ[i] = B[i] * E[i];
#pragma unroll
    for (int i = 0; i < 6; ++i) dot = dot + E[i] * DQ[i];
    const T t1 = T(0.5) * c[0] * d_exp<T>(T(0.5) * dot);
#pragma unroll
    for (int i = 0; i < 6; ++i) S[i] = t1 * DQ[i];
    if (C) {
#pragma unroll
      for (int j = 0; j < 6; ++j)
#pragma unroll
        for (int i = j; i < 6; ++i) C[i][j] = t1 * DQ[i] * DQ[j];
#pragma unroll
      for (int i = 0; i < 6; ++i) C[i][i] = C[i][i] + t1 * B[i];
#pragma unroll
      for (int j = 1; j < 6; ++j)
#pragma unroll
        for (int i = 0; i < j; ++i) C[i][j] = C[j][i];
    }
  }
}

template <class T>
__device__ __forceinline__ void d_push_stress(T S[6], const T t[6][6], T J) {
  T r[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j < 6; ++j) s = s + t[i][j] * S[j];
    r[i] = s;
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) S[i] = r[i] / J;
}

// FINITE_ELASTICITY_GAUSS_STRESS_TENSOR (:4342-4454): Cauchy stress (Voigt).
__device__ void d_gauss_stress(int law, const double* c, const double F[3][3], double J, double p, double S[6]) {
  double mod[3][3], t[6][6];
  d_fictitious<double>(law, c, F, J, mod, S, nullptr);
  d_push_t<double>(mod, t);
  d_push_stress<double>(S, t, J);
  const double ot = (S[0] + S[1] + S[2]) / 3.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) S[i] = S[i] - ot + p;
}

// FINITE_ELASTICITY_GAUSS_ELASTICITY_TENSOR (:609-835): spatial tangent and
// Cauchy stress (Voigt), in precision T.
template <class T>
__device__ void d_gauss_elasticity(int law, const T* c, const T F[3][3], T J, T p, T C[6][6], T S[6]) {
  const T ONETHIRD = T(1.0) / T(3.0), TWOTHIRDS = T(2.0) / T(3.0);
  const T DP[3][3] = {{TWOTHIRDS, -ONETHIRD, -ONETHIRD}, {-ONETHIRD, TWOTHIRDS, -ONETHIRD},
                      {-ONETHIRD, -ONETHIRD, TWOTHIRDS}};
  T mod[3][3], t[6][6];
  d_fictitious<T>(law, c, F, J, mod, S, C);
  d_push_t<T>(mod, t);
  d_push_stress<T>(S, t, J);
  {  // C <- t C t^T / J
    T A[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) s = s + t[i][k] * C[k][j];
        A[i][j] = s;
      }
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) s = s + A[i][k] * t[j][k];
        C[i][j] = s / J;
      }
  }
  const T trace = S[0] + S[1] + S[2];
#pragma unroll
  for (int i = 0; i < 3; ++i) S[i] = S[i] - ONETHIRD * trace;
  const T tt = TWOTHIRDS * trace;
#pragma unroll
  for (int i = 0; i < 6; ++i) C[i][i] = C[i][i] + tt * (i < 3 ? T(1.0) : T(0.5));
  T M[3][3], N[3][3], Q[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < 3; ++k) s = s + C[i][k] * DP[k][j];
      M[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < 3; ++k) s = s + DP[i][k] * M[k][j];
      N[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < 3; ++k) s = s + DP[i][k] * C[k][3 + j];
      Q[i][j] = s;
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      C[i][j] = N[i][j];
      C[i][3 + j] = Q[i][j];
      C[3 + j][i] = Q[i][j];
    }
#pragma unroll
  for (int j = 0; j < 6; ++j)
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const T ui = i < 3 ? TWOTHIRDS : T(0), uj = j < 3 ? TWOTHIRDS : T(0);
      C[i][j] = C[i][j] - (ui * S[j] + uj * S[i]);
    }
#pragma unroll
  for (int i = 0; i < 3; ++i) S[i] = S[i] + p;
#pragma unroll
  for (int i = 0; i < 6; ++i) C[i][i] = C[i][i] - p;
  C[1][0] = C[1][0] + p; C[2][0] = C[2][0] + p; C[0][1] = C[0][1] + p;
  C[2][1] = C[2][1] + p; C[0][2] = C[0][2] + p; C[1][2] = C[1][2] + p;
}


}  // namespace
