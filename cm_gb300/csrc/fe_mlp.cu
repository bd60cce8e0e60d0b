// libcm_fe: kernels of the learned Newton warm start (include/cm_warmstart.h).
//
// Training runs in FP32 on the CUDA cores (the network is 4-256-256-256-64,
// so one training step is a few tens of MFLOP); inference runs the whole
// network in one launch with BF16 weights on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation), one CTA per 16 input rows with the
// activations held in shared memory between layers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "cm_fe.h"
#include "cm_warmstart.h"
#include "fe_internal.h"

namespace {

int cuda_status(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cmfe::record_error(FE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return FE_NO_ERROR;
}

int bad(const char* what) { return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, what); }

// ---------------------------------------------------------------- FP32 GEMM
constexpr int TM = 64, TN = 64, TK = 16;

__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const float* __restrict__ A, int64_t a_sm,
                                                   int64_t a_sk, const float* __restrict__ B, int64_t b_sk,
                                                   int64_t b_sn, float* __restrict__ C, int64_t ldc, float beta) {
  __shared__ float As[TK][TM + 4];
  __shared__ float Bs[TK][TN + 4];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int tr = tid / 16, tc = tid % 16;  // 16 x 16 threads, 4 x 4 outputs each
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int i = tid; i < TM * TK; i += 256) {
      const int mm = i / TK, kk = i % TK;
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[(int64_t)gm * a_sm + (int64_t)gk * a_sk] : 0.0f;
    }
    for (int i = tid; i < TN * TK; i += 256) {
      const int kk = i / TN, nn = i % TN;
      const int gn = n0 + nn, gk = k0 + kk;
      Bs[kk][nn] = (gn < N && gk < K) ? B[(int64_t)gk * b_sk + (int64_t)gn * b_sn] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gm = m0 + tr + 16 * i, gn = n0 + tc + 16 * j;
      if (gm < M && gn < N) {
        float* c = &C[(int64_t)gm * ldc + gn];
        *c = beta == 0.0f ? acc[i][j] : acc[i][j] + beta * *c;
      }
    }
}

__device__ __forceinline__ float act_fwd(float x, int act) { return act == WS_ACT_TANH ? tanhf(x) : x; }

__global__ void bias_act_kernel(float* y, const float* bias, int rows, int cols, int act) {
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % cols);
    y[i] = act_fwd(y[i] + (bias ? bias[j] : 0.0f), act);
  }
}

__global__ void act_backward_kernel(const float* y, const float* dy, float* dz, int64_t n, int act) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g = dy[i];
    dz[i] = act == WS_ACT_TANH ? g * (1.0f - y[i] * y[i]) : g;
  }
}

__global__ void column_sum_kernel(const float* dz, float* db, int rows, int cols) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  float s = 0.0f;
  for (int i = 0; i < rows; ++i) s += dz[(int64_t)i * cols + j];
  db[j] = s;
}

// One CTA: fixed thread-to-element assignment and a fixed-order tree, so the
// loss does not depend on scheduling.
__global__ void __launch_bounds__(1024) mse_kernel(const float* p, const float* t, float* dp, float* loss, int64_t n) {
  __shared__ float part[1024];
  const float inv = 1.0f / (float)n;
  float s = 0.0f;
  for (int64_t i = threadIdx.x; i < n; i += 1024) {
    const float d = p[i] - t[i];
    s = fmaf(d, d, s);
    if (dp) dp[i] = 2.0f * d * inv;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = part[0] * inv;
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void to_bf16_kernel(const float* s, uint16_t* d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const __nv_bfloat16 h = __float2bfloat16_rn(s[i]);
    d[i] = *reinterpret_cast<const uint16_t*>(&h);
  }
}

// ------------------------------------------------------ BF16 inference
constexpr int MAXW = 256;
constexpr int IW = 8;  // warps per CTA

struct MlpArgs {
  int layers;
  int widths[WS_MAX_LAYERS + 1];
  const uint32_t* w[WS_MAX_LAYERS];  // BF16 pairs, [out][in/2]
  const float* b[WS_MAX_LAYERS];
};

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__global__ void __launch_bounds__(32 * IW) mlp_bf16_kernel(MlpArgs a, int n, const float* __restrict__ x,
                                                           float* __restrict__ y, int act) {
  __shared__ float buf[2][16][MAXW + 4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const int row0 = blockIdx.x * 16;
  const int w0 = a.widths[0];
  for (int i = threadIdx.x; i < 16 * w0; i += blockDim.x) {
    const int r = i / w0, c = i % w0;
    buf[0][r][c] = (row0 + r < n) ? x[(int64_t)(row0 + r) * w0 + c] : 0.0f;
  }
  __syncthreads();
  int cur = 0;
  for (int l = 0; l < a.layers; ++l) {
    const int in = a.widths[l], out = a.widths[l + 1];
    const uint32_t* W = a.w[l];
    const float* bias = a.b[l];
    const bool last = l + 1 == a.layers;
    for (int nt = warp; nt < out / 8; nt += IW) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      const int ncol = 8 * nt + gq;  // B column (output feature) this thread loads
      for (int k0 = 0; k0 < in; k0 += 16) {
        const float* A0 = &buf[cur][gq][k0 + 2 * tq];
        const float* A1 = &buf[cur][gq + 8][k0 + 2 * tq];
        const uint32_t a0 = pack2(A0[0], A0[1]);
        const uint32_t a1 = pack2(A1[0], A1[1]);
        const uint32_t a2 = pack2(A0[8], A0[9]);
        const uint32_t a3 = pack2(A1[8], A1[9]);
        const uint32_t* wr = W + ((int64_t)ncol * in + k0) / 2;
        const uint32_t b0 = wr[tq], b1 = wr[tq + 4];
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
      }
      const int c0 = 8 * nt + 2 * tq;
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int r = gq + (h >= 2 ? 8 : 0), c = c0 + (h & 1);
        float v = d[h] + bias[c];
        if (!last) v = act_fwd(v, act);
        if (last) {
          if (row0 + r < n) y[(int64_t)(row0 + r) * out + c] = v;
        } else {
          buf[cur ^ 1][r][c] = v;
        }
      }
    }
    __syncthreads();
    cur ^= 1;
  }
}

int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g < 4096 ? (g < 1 ? 1 : g) : 4096);
}

}  // namespace

extern "C" {

int ws_gemm_f32(int32_t m, int32_t n, int32_t k, const float* a, int64_t a_sm, int64_t a_sk, const float* b,
                int64_t b_sk, int64_t b_sn, float* c, int64_t ldc, float beta, void* stream) {
  if (m < 0 || n < 0 || k < 0 || !a || !b || !c || ldc < n) return bad("ws_gemm_f32: bad sizes or NULL pointer");
  if (m == 0 || n == 0) return FE_NO_ERROR;
  const dim3 grid((n + TN - 1) / TN, (m + TM - 1) / TM);
  gemm_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(m, n, k, a, a_sm, a_sk, b, b_sk, b_sn, c, ldc, beta);
  return cuda_status("ws_gemm_f32");
}

int ws_bias_act(float* y, const float* bias, int32_t rows, int32_t cols, int32_t act, void* stream) {
  if (!y || rows < 0 || cols <= 0 || (act != WS_ACT_IDENTITY && act != WS_ACT_TANH)) return bad("ws_bias_act: bad arguments");
  bias_act_kernel<<<grid_for((int64_t)rows * cols), 256, 0, (cudaStream_t)stream>>>(y, bias, rows, cols, act);
  return cuda_status("ws_bias_act");
}

int ws_act_backward(const float* y, const float* dy, float* dz, int64_t count, int32_t act, void* stream) {
  if (!y || !dy || !dz || count < 0 || (act != WS_ACT_IDENTITY && act != WS_ACT_TANH)) return bad("ws_act_backward: bad arguments");
  if (count == 0) return FE_NO_ERROR;
  act_backward_kernel<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(y, dy, dz, count, act);
  return cuda_status("ws_act_backward");
}

int ws_column_sum(const float* dz, float* db, int32_t rows, int32_t cols, void* stream) {
  if (!dz || !db || rows < 0 || cols <= 0) return bad("ws_column_sum: bad arguments");
  column_sum_kernel<<<(cols + 127) / 128, 128, 0, (cudaStream_t)stream>>>(dz, db, rows, cols);
  return cuda_status("ws_column_sum");
}

int ws_mse(const float* pred, const float* target, float* dpred, float* loss, int64_t count, void* stream) {
  if (!pred || !target || !loss || count <= 0) return bad("ws_mse: bad arguments");
  mse_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(pred, target, dpred, loss, count);
  return cuda_status("ws_mse");
}

int ws_adam(float* param, const float* grad, float* m, float* v, int64_t count, float lr, float beta1, float beta2,
            float eps, int32_t step, void* stream) {
  if (!param || !grad || !m || !v || count < 0 || step < 1) return bad("ws_adam: bad arguments");
  if (count == 0) return FE_NO_ERROR;
  const float c1 = 1.0f - std::pow(beta1, (float)step), c2 = 1.0f - std::pow(beta2, (float)step);
  adam_kernel<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(param, grad, m, v, count, lr, beta1, beta2, eps, c1,
                                                                  c2);
  return cuda_status("ws_adam");
}

int ws_to_bf16(const float* src, uint16_t* dst, int64_t count, void* stream) {
  if (!src || !dst || count < 0) return bad("ws_to_bf16: bad arguments");
  if (count == 0) return FE_NO_ERROR;
  to_bf16_kernel<<<grid_for(count), 256, 0, (cudaStream_t)stream>>>(src, dst, count);
  return cuda_status("ws_to_bf16");
}

int ws_mlp_forward_bf16(int32_t n, int32_t layers, const int32_t* widths, const uint16_t* const* weights,
                        const float* const* bias, const float* x, float* y, int32_t act, void* stream) {
  if (n < 0 || layers < 1 || layers > WS_MAX_LAYERS || !widths || !weights || !bias || !x || !y)
    return bad("ws_mlp_forward_bf16: bad arguments");
  MlpArgs a;
  a.layers = layers;
  for (int l = 0; l <= layers; ++l) {
    if (widths[l] <= 0 || widths[l] % 16 != 0 || widths[l] > MAXW)
      return bad("ws_mlp_forward_bf16: every width must be a positive multiple of 16, at most 256");
    a.widths[l] = widths[l];
  }
  for (int l = 0; l < layers; ++l) {
    if (!weights[l] || !bias[l]) return bad("ws_mlp_forward_bf16: NULL weight or bias");
    if (reinterpret_cast<uintptr_t>(weights[l]) % 4 != 0) return bad("ws_mlp_forward_bf16: weights must be 4-byte aligned");
    a.w[l] = reinterpret_cast<const uint32_t*>(weights[l]);
    a.b[l] = bias[l];
  }
  if (n == 0) return FE_NO_ERROR;
  mlp_bf16_kernel<<<(n + 15) / 16, 32 * IW, 0, (cudaStream_t)stream>>>(a, n, x, y, act);
  return cuda_status("ws_mlp_forward_bf16");
}

}  // extern "C"
