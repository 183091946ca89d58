// msod_mlp.cuh -- activations, output mapping and the one-thread-per-element
// evaluation of the per-element network, used by msod_mlp.cu.
#pragma once

#include <cuda_runtime.h>

#include "msod_kernels.h"

namespace msod {

__device__ __forceinline__ float silu(float a) { return a / (1.0f + __expf(-a)); }
__device__ __forceinline__ float sigmoidf_(float a) { return 1.0f / (1.0f + __expf(-a)); }
__device__ __forceinline__ float softplus(float z) { return z > 20.0f ? z : log1pf(__expf(z)); }
// Heavy-tailed non-negative features enter as logarithms (offset 1e-12).
__device__ __forceinline__ float flog(float v) { return logf(fmaxf(v, 0.0f) + 1e-12f); }
// Hardware approximations (PTX sqrt.approx.f32, lg2.approx.f32; div.full.f32
// through __fdividef), about 1e-7 relative: the per-node statistics of the
// features, far inside the features' own tolerance.
__device__ __forceinline__ float sqrt_approx(float x)
{
    float y;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float log2_approx(float x)
{
    float y;
    asm("lg2.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// The network's output s >= 0 is a number of decades: y = 10^-s.  Targets y
// are mapped to s = -log10(max(y, 1e-12)) for the loss.
__device__ __forceinline__ float y_from_s(float s) { return exp10f(-s); }
__device__ __forceinline__ float s_from_y(float y) { return -log10f(fminf(fmaxf(y, 1e-12f), 1.0f)); }

// The network's output s (decades) for one element's raw features x_raw, one
// thread per element: weights w in the parameter layout (W1[j][k] at
// kOffW1 + j*12 + k, ...; FP16-rounded values in FP32), every sum in the
// order of the training kernel's forward pass, so that all users of the
// network produce the same bits.
__device__ __forceinline__ float mlp_infer(const float *__restrict__ w, const MlpNorm &nm, const float *x_raw)
{
    float x[kMlpIn], h1[kMlpH];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) x[k] = (x_raw[k] - nm.mean[k]) * nm.inv_std[k];
#pragma unroll
    for (int j = 0; j < kMlpH; ++j) {
        float acc = w[kOffB1 + j];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) acc = fmaf(w[kOffW1 + j * kMlpIn + k], x[k], acc);
        h1[j] = silu(acc);
    }
    float z = w[kOffB3];
    for (int j = 0; j < kMlpH; ++j) {
        float acc = w[kOffB2 + j];
#pragma unroll
        for (int k = 0; k < kMlpH; ++k) acc = fmaf(w[kOffW2 + j * kMlpH + k], h1[k], acc);
        z = fmaf(w[kOffW3 + j], silu(acc), z);
    }
    return softplus(z);
}

}  // namespace msod
