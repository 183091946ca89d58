// msod_mlp.cuh -- activations and output mapping of the per-element network,
// shared by the network kernels (msod_mlp.cu) and the diffusion kernel that
// evaluates the network in its prologue (msod_diffu.cu).
#pragma once

#include <cuda_runtime.h>

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

}  // namespace msod
