/*
 * cm_warmstart.h — device kernels of the learned Newton warm start
 * (libcm_fe.so).
 *
 * No counterpart in the reference: OpenCMISS-Iron starts every Newton solve
 * from the current field (solver_routines.f90:17812).  These entry points
 * train and evaluate the small multilayer perceptron that maps load and
 * material parameters to POD coefficients of the converged field; the host
 * code in cm_gb300/warmstart.py composes them.  Newton from the reference
 * initial guess stays the fallback.
 *
 * Conventions: int status (0 = success, negative FE_ERR_* of cm_fe.h on
 * failure, text through fe_last_error()); every pointer is device memory of
 * the current CUDA device; calls are asynchronous on `stream` (NULL = legacy
 * default stream).  Matrices are row-major unless strides say otherwise.
 */
#ifndef CM_WARMSTART_H
#define CM_WARMSTART_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WS_ACT_IDENTITY 0
#define WS_ACT_TANH 1
#define WS_MAX_LAYERS 8

/* C[m][n] = sum_k A(m,k) B(k,n) + beta C[m][n] in FP32, with
 * A(m,k) = A[m*a_sm + k*a_sk] and B(k,n) = B[k*b_sk + n*b_sn] (so either
 * operand may be read transposed); C has row stride ldc. */
int ws_gemm_f32(int32_t m, int32_t n, int32_t k, const float* a, int64_t a_sm, int64_t a_sk, const float* b,
                int64_t b_sk, int64_t b_sn, float* c, int64_t ldc, float beta, void* stream);

/* y[i][j] = act(y[i][j] + bias[j]) for a rows x cols row-major block. */
int ws_bias_act(float* y, const float* bias, int32_t rows, int32_t cols, int32_t act, void* stream);

/* dz = dy * act'(.) expressed through the activation output y (tanh: 1 - y^2). */
int ws_act_backward(const float* y, const float* dy, float* dz, int64_t count, int32_t act, void* stream);

/* db[j] = sum_i dz[i][j] (deterministic: one thread per column, rows in order). */
int ws_column_sum(const float* dz, float* db, int32_t rows, int32_t cols, void* stream);

/* Mean squared error over count entries: *loss = sum (p - t)^2 / count,
 * dpred = 2 (p - t) / count (dpred may be NULL).  Deterministic reduction. */
int ws_mse(const float* pred, const float* target, float* dpred, float* loss, int64_t count, void* stream);

/* One Adam step (bias-corrected, step >= 1) on count parameters. */
int ws_adam(float* param, const float* grad, float* m, float* v, int64_t count, float lr, float beta1, float beta2,
            float eps, int32_t step, void* stream);

/* Round FP32 to BF16 (round to nearest even), stored as raw 16-bit words. */
int ws_to_bf16(const float* src, uint16_t* dst, int64_t count, void* stream);

/* Whole-network inference with BF16 weights on the tensor cores (FP32
 * accumulation, FP32 activations between layers).  widths[0..layers] are
 * host integers, every one a multiple of 16 and at most 256; weights[l] is a
 * device pointer to BF16 [widths[l+1]][widths[l]], bias[l] to FP32
 * [widths[l+1]].  Hidden layers use `act`, the last layer is linear.
 * x: [n][widths[0]], y: [n][widths[layers]]. */
int ws_mlp_forward_bf16(int32_t n, int32_t layers, const int32_t* widths, const uint16_t* const* weights,
                        const float* const* bias, const float* x, float* y, int32_t act, void* stream);

#ifdef __cplusplus
}
#endif

#endif
