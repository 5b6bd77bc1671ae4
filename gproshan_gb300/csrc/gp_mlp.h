// Sweep-cost MLP: sizes and device entry points (gp_mlp.cu).
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

namespace gp {

constexpr int MLP_IN = 16;   // field features (see field_features in gp_ptp.cu)
constexpr int MLP_H = 64;    // hidden width
constexpr int MLP_OUT = 2;   // log(sweeps / rings), log(relaxations / vertices)
constexpr int MLP_NPARAM = MLP_IN * MLP_H + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H * MLP_OUT + MLP_OUT;

size_t mlp_workspace_floats(int n);
cudaError_t mlp_grad_device(const float *P, const float *X, const float *T, int n, float *work, float *grads,
                            float *loss, cudaStream_t s);
cudaError_t mlp_forward_f32_device(const float *P, const float *X, int n, float *work, float *Y, cudaStream_t s);
cudaError_t mlp_infer_bf16_device(const float *P, const float *X, int n, float *Y, cudaStream_t s);
cudaError_t mlp_adam_device(float *P, const float *grads, float *m1, float *m2, float lr, int step, cudaStream_t s);

} // namespace gp
