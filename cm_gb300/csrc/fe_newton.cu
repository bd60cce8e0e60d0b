// libcm_fe: Newton load step on the device (sm_103a).
//
// The solve the reference runs around the assembly for one load increment
// (SOLVER_NEWTON_LINESEARCH, solver_routines.f90:17803-17812 and
// 18772-18775): Newton from the given state, the FP64 Jacobian and residual
// of this library, Dirichlet rows and columns dropped from the linear system
// (solver_mapping_routines.f90:1420,1592), each Newton system solved by
// restarted GMRES (the reference's KSP default, solver_routines.f90:
// 10979-10987) with a block-diagonal preconditioner, then a cubic
// backtracking line search (the published Dennis-Schnabel algorithm that
// PETSc's "bt" line search implements) on f = 1/2 ||r_free||^2.
//
// The free-dof system is never extracted: vectors keep the full dof
// numbering with zeros on the fixed dofs, and the matrix-vector product masks
// rows and columns of fixed dofs.  Every reduction is a fixed-order two-pass
// sum, so a solve is bit-identical from run to run.  The host drives the
// iteration; it reads one small array per GMRES iteration (the new
// Hessenberg column) to update the Givens rotations.
#include "fe_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace {

constexpr int NT = 256;
constexpr int RED_BLOCKS = 304;  // partial sums per reduction: two per SM

// y = P A P x on the free dofs (P: the free-dof mask), 0 on the fixed ones;
// one warp per row, lanes over the row's entries, a fixed shuffle tree.
__global__ void k_spmv(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                       const double* __restrict__ val, const uint8_t* __restrict__ free_dof,
                       const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nw) {
    double s = 0.0;
    if (free_dof[i]) {
      for (int64_t j = rp[i] + lane; j < rp[i + 1]; j += 32) {
        const int c = col[j];
        if (free_dof[c]) s = fma(val[j], x[c], s);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) y[i] = s;
  }
}

// Diagonal of A (0 where a row has no diagonal entry).
__global__ void k_diag(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                       const double* __restrict__ val, double* __restrict__ d) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nw) {
    double v = 0.0;
    for (int64_t j = rp[i] + lane; j < rp[i + 1]; j += 32)
      if (col[j] == i) v = val[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) d[i] = v;
  }
}

// Preconditioner: 1/A_ii on free displacement rows; on free pressure rows
// -1/s_i with s_i = sum over free displacement columns j of B_ij^2 / A_jj
// (the diagonal of the Schur complement B diag(A)^-1 B^T), 1 if s_i = 0;
// 0 on fixed dofs.
__global__ void k_precond(int64_t n, int64_t nu3, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                          const double* __restrict__ val, const uint8_t* __restrict__ free_dof,
                          const double* __restrict__ d, double* __restrict__ minv) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nw) {
    if (!free_dof[i]) {
      if (lane == 0) minv[i] = 0.0;
      continue;
    }
    if (i < nu3) {
      if (lane == 0) minv[i] = 1.0 / d[i];
      continue;
    }
    double s = 0.0;
    for (int64_t j = rp[i] + lane; j < rp[i + 1]; j += 32) {
      const int c = col[j];
      if (c < nu3 && free_dof[c]) s += val[j] * val[j] / d[c];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) minv[i] = -1.0 / (s != 0.0 ? s : 1.0);
  }
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
  return t;  // valid in thread 0
}

// part[j * gridDim.x + b] = block b's share of V_j . w for j < m (V row-major,
// leading dimension ld); with V = w and m = 1 it is the squared norm.
__global__ void k_mdot_part(int64_t n, const double* __restrict__ V, int64_t ld, int m, const double* __restrict__ w,
                            double* __restrict__ part) {
  __shared__ double sh[NT / 32];
  for (int j = 0; j < m; ++j) {
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      s = fma(V[j * ld + i], w[i], s);
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) part[j * gridDim.x + blockIdx.x] = t;
  }
}

// out[j] = sum_b part[j * nb + b], one block per j.
__global__ void k_mdot_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double sh[NT / 32];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[blockIdx.x * nb + b];
  const double t = block_sum(s, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = t;
}

// w -= sum_{j < m} h[j] V_j, and acc[j] += h[j] (first thread) when acc is set.
__global__ void k_gs_update(int64_t n, const double* __restrict__ V, int64_t ld, int m, const double* __restrict__ h,
                            double* __restrict__ w, double* __restrict__ acc) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = w[i];
    for (int j = 0; j < m; ++j) s = fma(-h[j], V[j * ld + i], s);
    w[i] = s;
  }
  if (acc && blockIdx.x == 0 && threadIdx.x < m) acc[threadIdx.x] += h[threadIdx.x];
}

// y = a * x, or y = x / sqrt(*den) when den is set (0 when *den is 0: an
// Arnoldi breakdown, after which the vector is not used).
__global__ void k_scale(int64_t n, double a, const double* __restrict__ den, const double* x, double* y) {
  const double s = den ? (*den > 0.0 ? 1.0 / sqrt(*den) : 0.0) : a;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = s * x[i];
}

// y = a * x + b * y
__global__ void k_axpby(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

// z = minv .* v
__global__ void k_precond_apply(int64_t n, const double* __restrict__ minv, const double* __restrict__ v,
                                double* __restrict__ z) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = minv[i] * v[i];
}

// x += sum_{j < m} y[j] Z_j
__global__ void k_combine(int64_t n, const double* __restrict__ Z, int64_t ld, int m, const double* __restrict__ y,
                          double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = x[i];
    for (int j = 0; j < m; ++j) s = fma(y[j], Z[j * ld + i], s);
    x[i] = s;
  }
}

// r <- -r on free dofs, 0 on fixed ones (in place when out == r)
__global__ void k_mask(int64_t n, const uint8_t* __restrict__ free_dof, double sign, const double* r, double* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = free_dof[i] ? sign * r[i] : 0.0;
}

// x[dofs[k]] = values[k]; free[dofs[k]] = 0
__global__ void k_fix(int64_t m, const int32_t* __restrict__ dofs, const double* __restrict__ values,
                      double* __restrict__ x, uint8_t* __restrict__ free_dof) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
    x[dofs[k]] = values[k];
    free_dof[dofs[k]] = 0;
  }
}

int blocks_for(int64_t n) {
  const int64_t b = (n + NT - 1) / NT;
  return (int)(b < 4096 ? (b < 1 ? 1 : b) : 4096);
}

int warp_blocks_for(int64_t n) {
  const int64_t b = (n + (NT / 32) - 1) / (NT / 32);
  return (int)(b < 8192 ? (b < 1 ? 1 : b) : 8192);
}

#define NT_TRY(expr)                                                                                 \
  do {                                                                                              \
    cudaError_t e_ = (expr);                                                                        \
    if (e_ != cudaSuccess) return cmfe::record_error(FE_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Device work space of one call, freed on scope exit.
struct Work {
  std::vector<void*> ptrs;
  ~Work() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  int alloc(T** p, size_t count) {
    *p = nullptr;
    const cudaError_t e = cudaMalloc(p, count * sizeof(T) + 16);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cmfe::record_error(FE_ERR_OUT_OF_MEMORY, std::string("Newton work space: ") + cudaGetErrorString(e));
    }
    ptrs.push_back(*p);
    return FE_NO_ERROR;
  }
};

struct Solver {
  fe_handle h;
  cudaStream_t st;
  int64_t n, nnz, nu3;
  const int32_t *rp, *col;
  double *vals, *r, *rn, *d, *xs, *w, *minv, *diag, *V, *Z, *hbuf, *part, *scal;
  uint8_t* free_dof;
  int restart;

  int spmv(const double* x, double* y) {
    k_spmv<<<warp_blocks_for(n), NT, 0, st>>>(n, rp, col, vals, free_dof, x, y);
    NT_TRY(cudaGetLastError());
    return FE_NO_ERROR;
  }

  // out[0..m) = V_j . w on the device
  int mdot(const double* Vm, int m, const double* wv, double* out) {
    k_mdot_part<<<RED_BLOCKS, NT, 0, st>>>(n, Vm, n, m, wv, part);
    k_mdot_final<<<m, NT, 0, st>>>(part, RED_BLOCKS, out);
    NT_TRY(cudaGetLastError());
    return FE_NO_ERROR;
  }

  int dot_host(const double* a, const double* b, double* out) {
    int rc = mdot(a, 1, b, scal);
    if (rc) return rc;
    NT_TRY(cudaMemcpyAsync(out, scal, sizeof(double), cudaMemcpyDeviceToHost, st));
    NT_TRY(cudaStreamSynchronize(st));
    return FE_NO_ERROR;
  }

  // r_out = -(residual at x) on free dofs; *inverted when an element of x
  // has det F <= 0 or a non-finite stress (the kernels' status word).
  int residual(double* x, double* r_out, bool* inverted) {
    *inverted = false;
    int rc = fe_residual_evaluate(h, x, r_out, st);
    if (rc) return rc;
    rc = fe_check(h, st);
    if (rc == FE_ERR_NUMERICAL) {
      *inverted = true;
      return FE_NO_ERROR;
    }
    if (rc) return rc;
    k_mask<<<blocks_for(n), NT, 0, st>>>(n, free_dof, 1.0, r_out, r_out);
    NT_TRY(cudaGetLastError());
    return FE_NO_ERROR;
  }

  // Right-preconditioned GMRES(restart) for A dx = b (b on free dofs, dx
  // zero on fixed ones); returns the iterations in *its.
  int gmres(const double* b, double* dx, double rtol, int max_it, int64_t* its) {
    *its = 0;
    NT_TRY(cudaMemsetAsync(dx, 0, sizeof(double) * n, st));
    double bnorm2 = 0.0;
    int rc = dot_host(b, b, &bnorm2);
    if (rc) return rc;
    const double bnorm = std::sqrt(bnorm2);
    if (bnorm == 0.0) return FE_NO_ERROR;
    double* res = w;  // current residual b - A dx before each cycle
    NT_TRY(cudaMemcpyAsync(res, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    double beta = bnorm;
    std::vector<double> H((size_t)(restart + 1) * restart), cs(restart), sn(restart), g(restart + 1), y(restart);
    std::vector<double> col_h(restart + 2);
    while (*its < max_it) {
      if (beta <= rtol * bnorm) break;
      k_scale<<<blocks_for(n), NT, 0, st>>>(n, 1.0 / beta, nullptr, res, V);
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int k = 0;
      bool done = false;
      while (k < restart && *its < max_it) {
        double* vk = V + (size_t)k * n;
        double* zk = Z + (size_t)k * n;
        double* wv = V + (size_t)(k + 1) * n;
        k_precond_apply<<<blocks_for(n), NT, 0, st>>>(n, minv, vk, zk);
        if ((rc = spmv(zk, wv))) return rc;
        // classical Gram-Schmidt, twice; hbuf[0..k] accumulates the column
        NT_TRY(cudaMemsetAsync(hbuf, 0, sizeof(double) * (restart + 2), st));
        for (int pass = 0; pass < 2; ++pass) {
          if ((rc = mdot(V, k + 1, wv, hbuf + restart + 2))) return rc;
          k_gs_update<<<blocks_for(n), NT, 0, st>>>(n, V, n, k + 1, hbuf + restart + 2, wv, hbuf);
        }
        if ((rc = mdot(wv, 1, wv, hbuf + k + 1))) return rc;  // squared norm
        k_scale<<<blocks_for(n), NT, 0, st>>>(n, 0.0, hbuf + k + 1, wv, wv);
        NT_TRY(cudaGetLastError());
        NT_TRY(cudaMemcpyAsync(col_h.data(), hbuf, sizeof(double) * (k + 2), cudaMemcpyDeviceToHost, st));
        NT_TRY(cudaStreamSynchronize(st));
        col_h[k + 1] = std::sqrt(col_h[k + 1]);
        // apply the previous rotations, then a new one that zeroes H[k+1][k]
        for (int i = 0; i < k; ++i) {
          const double t = cs[i] * col_h[i] + sn[i] * col_h[i + 1];
          col_h[i + 1] = -sn[i] * col_h[i] + cs[i] * col_h[i + 1];
          col_h[i] = t;
        }
        const double a = col_h[k], bb = col_h[k + 1];
        const double den = std::hypot(a, bb);
        cs[k] = den > 0.0 ? a / den : 1.0;
        sn[k] = den > 0.0 ? bb / den : 0.0;
        for (int i = 0; i <= k; ++i) H[(size_t)i * restart + k] = col_h[i];
        H[(size_t)k * restart + k] = den;
        g[k + 1] = -sn[k] * g[k];
        g[k] = cs[k] * g[k];
        ++k;
        ++*its;
        if (std::fabs(g[k]) <= rtol * bnorm || bb <= 1e-14 * beta) {
          done = true;
          break;
        }
      }
      // back substitution for the rotated upper-triangular system
      for (int i = k - 1; i >= 0; --i) {
        double s = g[i];
        for (int j = i + 1; j < k; ++j) s -= H[(size_t)i * restart + j] * y[j];
        const double hii = H[(size_t)i * restart + i];
        y[i] = hii != 0.0 ? s / hii : 0.0;
      }
      NT_TRY(cudaMemcpyAsync(hbuf, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
      k_combine<<<blocks_for(n), NT, 0, st>>>(n, Z, n, k, hbuf, dx);
      // true residual of the cycle
      if ((rc = spmv(dx, res))) return rc;
      k_axpby<<<blocks_for(n), NT, 0, st>>>(n, 1.0, b, -1.0, res);
      double r2 = 0.0;
      if ((rc = dot_host(res, res, &r2))) return rc;
      beta = std::sqrt(r2);
      if (done && beta <= rtol * bnorm) break;
    }
    return FE_NO_ERROR;
  }
};

}  // namespace

extern "C" {

void fe_newton_options_default(fe_newton_options* o) {
  if (!o) return;
  o->max_iterations = 50;
  o->atol = 1e-10;
  o->alpha = 1e-4;
  o->max_step = 1e8;
  o->min_lambda = 1e-10;
  o->ksp_rtol = 1e-5;
  o->ksp_restart = 30;
  o->ksp_max_iterations = 600;
  o->forcing = 0;
}

int fe_newton_load_step(fe_handle h, const int32_t* fixed_dofs, const double* fixed_values, int64_t num_fixed,
                        double* x, const fe_newton_options* options, fe_newton_report* report, void* stream) {
  if (!h || !x || !report) return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "NULL handle, x or report");
  if (num_fixed < 0 || (num_fixed > 0 && (!fixed_dofs || !fixed_values)))
    return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "fixed dofs and values must be given together");
  fe_newton_options o;
  fe_newton_options_default(&o);
  if (options) o = *options;
  if (o.ksp_restart < 1 || o.ksp_restart > 200 || o.max_iterations < 0 || !(o.atol >= 0.0))
    return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "invalid Newton options");
  std::memset(report, 0, sizeof(*report));
  Solver S;
  S.h = h;
  S.st = (cudaStream_t)stream;
  S.restart = o.ksp_restart;
  int rc = cmfe::device_pattern(h, &S.rp, &S.col, &S.n, &S.nnz, &S.nu3);
  if (rc) return rc;
  const int64_t n = S.n;
  for (int64_t k = 0; k < num_fixed; ++k)
    if (fixed_dofs[k] < 0 || fixed_dofs[k] >= n) return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "fixed dof out of range");
  Work W;
  double *dx_state, *fvals;
  int32_t* fdofs;
  const size_t rs = (size_t)S.restart;
  if ((rc = W.alloc(&S.vals, (size_t)S.nnz)) || (rc = W.alloc(&S.r, n)) || (rc = W.alloc(&S.rn, n)) ||
      (rc = W.alloc(&S.d, n)) || (rc = W.alloc(&S.xs, n)) || (rc = W.alloc(&S.w, n)) || (rc = W.alloc(&S.minv, n)) ||
      (rc = W.alloc(&S.diag, n)) || (rc = W.alloc(&S.V, (rs + 1) * n)) || (rc = W.alloc(&S.Z, rs * n)) ||
      (rc = W.alloc(&S.hbuf, 2 * rs + 4)) || (rc = W.alloc(&S.part, (rs + 2) * RED_BLOCKS)) ||
      (rc = W.alloc(&S.scal, 4)) || (rc = W.alloc(&S.free_dof, n)) || (rc = W.alloc(&dx_state, n)) ||
      (rc = W.alloc(&fvals, num_fixed > 0 ? num_fixed : 1)) || (rc = W.alloc(&fdofs, num_fixed > 0 ? num_fixed : 1)))
    return rc;
  cudaStream_t st = S.st;
  // the state on the device (x may be host memory)
  cudaPointerAttributes pa;
  bool host_x = true;
  if (cudaPointerGetAttributes(&pa, x) == cudaSuccess)
    host_x = !(pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
  else
    cudaGetLastError();
  double* xd = host_x ? dx_state : x;
  if (host_x) NT_TRY(cudaMemcpyAsync(xd, x, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  NT_TRY(cudaMemsetAsync(S.free_dof, 1, n, st));
  if (num_fixed > 0) {
    NT_TRY(cudaMemcpyAsync(fdofs, fixed_dofs, sizeof(int32_t) * num_fixed, cudaMemcpyHostToDevice, st));
    NT_TRY(cudaMemcpyAsync(fvals, fixed_values, sizeof(double) * num_fixed, cudaMemcpyHostToDevice, st));
    k_fix<<<blocks_for(num_fixed), NT, 0, st>>>(num_fixed, fdofs, fvals, xd, S.free_dof);
    NT_TRY(cudaGetLastError());
  }
  auto finish = [&](int code) -> int {
    if (host_x) {
      const cudaError_t e = cudaMemcpyAsync(x, xd, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
      const cudaError_t e2 = cudaStreamSynchronize(st);
      if (!code && (e != cudaSuccess || e2 != cudaSuccess))
        return cmfe::record_error(FE_ERR_CUDA, "copying the state back failed");
    } else {
      cudaStreamSynchronize(st);
    }
    return code;
  };
  bool inverted = false;
  if ((rc = S.residual(xd, S.r, &inverted))) return finish(rc);
  if (inverted) return finish(cmfe::record_error(FE_ERR_NUMERICAL, "the initial state has an element with det F <= 0"));
  double r2 = 0.0;
  if ((rc = S.dot_host(S.r, S.r, &r2))) return finish(rc);
  double fnorm = std::sqrt(r2), fnorm_prev = -1.0, prev_eta = -1.0;
  report->residual_norm_initial = fnorm;
  report->residual_norm = fnorm;
  report->last_lambda = 0.0;
  int it = 0;
  while (fnorm > o.atol && it < o.max_iterations) {
    if ((rc = fe_jacobian_evaluate(h, xd, S.vals, nullptr, st))) return finish(rc);
    k_diag<<<warp_blocks_for(n), NT, 0, st>>>(n, S.rp, S.col, S.vals, S.diag);
    k_precond<<<warp_blocks_for(n), NT, 0, st>>>(n, S.nu3, S.rp, S.col, S.vals, S.free_dof, S.diag, S.minv);
    NT_TRY(cudaGetLastError());
    double eta = o.ksp_rtol;
    if (o.forcing == 1) {
      // Eisenstat & Walker (1996), choice 2 (gamma 0.9, alpha 2) with their safeguard
      eta = fnorm_prev < 0.0 ? 0.5 : 0.9 * (fnorm / fnorm_prev) * (fnorm / fnorm_prev);
      if (prev_eta >= 0.0 && 0.9 * prev_eta * prev_eta > 0.1) eta = std::fmax(eta, 0.9 * prev_eta * prev_eta);
      eta = std::fmin(std::fmax(eta, o.ksp_rtol), 0.5);
      prev_eta = eta;
    }
    // Newton system A d = -r on the free dofs
    k_mask<<<blocks_for(n), NT, 0, st>>>(n, S.free_dof, -1.0, S.r, S.rn);
    int64_t lits = 0;
    if ((rc = S.gmres(S.rn, S.d, eta, o.ksp_max_iterations, &lits))) return finish(rc);
    report->linear_iterations += lits;
    double dn2 = 0.0;
    if ((rc = S.dot_host(S.d, S.d, &dn2))) return finish(rc);
    if (std::sqrt(dn2) > o.max_step) k_scale<<<blocks_for(n), NT, 0, st>>>(n, o.max_step / std::sqrt(dn2), nullptr, S.d, S.d);
    // slope of f = 1/2 ||r||^2 along d: r . (A d)
    if ((rc = S.spmv(S.d, S.w))) return finish(rc);
    double slope = 0.0;
    if ((rc = S.dot_host(S.r, S.w, &slope))) return finish(rc);
    if (slope > 0.0) slope = -slope;
    const double f0 = 0.5 * fnorm * fnorm;
    double lam = 1.0, lam_prev = -1.0, f_prev = 0.0, f1 = 0.0;
    bool accepted = false;
    NT_TRY(cudaMemcpyAsync(S.xs, xd, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    while (true) {
      NT_TRY(cudaMemcpyAsync(xd, S.xs, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      k_axpby<<<blocks_for(n), NT, 0, st>>>(n, lam, S.d, 1.0, xd);  // d is zero on fixed dofs
      if ((rc = S.residual(xd, S.rn, &inverted))) return finish(rc);
      if (inverted) {
        f1 = INFINITY;
      } else {
        double q = 0.0;
        if ((rc = S.dot_host(S.rn, S.rn, &q))) return finish(rc);
        f1 = 0.5 * q;
      }
      if (std::isfinite(f1) && f1 <= f0 + o.alpha * lam * slope) {
        accepted = true;
        break;
      }
      if (lam < o.min_lambda) break;
      double lt;
      if (lam_prev < 0.0 || !std::isfinite(f1)) {
        lt = std::isfinite(f1) ? -slope / (2.0 * (f1 - f0 - slope)) : 0.1 * lam;
      } else {
        const double a1 = f1 - f0 - lam * slope, a2 = f_prev - f0 - lam_prev * slope, den = lam - lam_prev;
        const double a = (a1 / (lam * lam) - a2 / (lam_prev * lam_prev)) / den;
        const double b = (-lam_prev * a1 / (lam * lam) + lam * a2 / (lam_prev * lam_prev)) / den;
        if (a == 0.0) {
          lt = -slope / (2.0 * b);
        } else {
          const double disc = std::fmax(b * b - 3.0 * a * slope, 0.0);
          lt = (-b + std::sqrt(disc)) / (3.0 * a);
        }
      }
      lam_prev = lam;
      f_prev = f1;
      lam = std::fmin(std::fmax(lt, 0.1 * lam), 0.5 * lam);
    }
    report->last_lambda = lam;
    ++it;
    if (!accepted) {
      // No trial step gave sufficient decrease: keep the state, residual and
      // norm from before the step (as PETSc's bt line search leaves X on a
      // failed reduction) and stop.
      NT_TRY(cudaMemcpyAsync(xd, S.xs, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      report->line_search_failed = 1;
      break;
    }
    std::swap(S.r, S.rn);
    fnorm_prev = fnorm;
    fnorm = std::sqrt(2.0 * f1);
  }
  report->iterations = it;
  report->residual_norm = fnorm;
  report->converged = fnorm <= o.atol;
  return finish(FE_NO_ERROR);
}

}  // extern "C"
