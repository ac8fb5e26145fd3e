// k_mlp.cu -- training and inference kernels of the warm-start perceptron
// (mlp_impl.cuh). The network has 5187 parameters: every kernel here is
// bound by latency and launches, not by arithmetic, so it runs on the FP32
// pipes with tiles of samples staged in shared memory.
//
//  k_mlp_forward     one thread per sample, de-standardised output
//  k_mlp_tile_grad   64 samples per CTA: forward + backward per sample into
//                    shared memory, then every parameter's gradient summed
//                    over the tile and added to the global gradient
//  k_mlp_adam        Adam step with bias correction; clears the gradient
#include <atomic>

#include "fsi_kernels.h"
#include "mlp_impl.cuh"

namespace fsi {
namespace {

constexpr int TS = 64;  // samples per CTA in the gradient kernel

__global__ void k_mlp_forward(const float *__restrict__ P, const float *__restrict__ nrm, const float *__restrict__ X,
                              float *__restrict__ Y, int n) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float xn[MLP_IN], h1[MLP_H], h2[MLP_H], yn[MLP_OUT];
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) xn[k] = (X[(long long)s * MLP_IN + k] - nrm[k]) / nrm[MLP_IN + k];
    mlp_forward(P, xn, h1, h2, yn);
#pragma unroll
    for (int c = 0; c < MLP_OUT; c++)
        Y[(long long)s * MLP_OUT + c] = yn[c] * nrm[2 * MLP_IN + MLP_OUT + c] + nrm[2 * MLP_IN + c];
}

// Loss L = sum over the batch of |yn - tn|^2 / (3 B), standardised outputs.
__global__ void __launch_bounds__(256) k_mlp_tile_grad(const float *__restrict__ P, const float *__restrict__ nrm,
                                                       const float *__restrict__ X, const float *__restrict__ Y,
                                                       const int *__restrict__ perm, long long b0, int nb,
                                                       float inv3B, float *__restrict__ grad, float *loss) {
    extern __shared__ float sm[];
    float *sx = sm;                       // [TS][12]
    float *sh1 = sx + TS * MLP_IN;        // [TS][64]
    float *sh2 = sh1 + TS * MLP_H;        // [TS][64]
    float *sd1 = sh2 + TS * MLP_H;        // [TS][64]
    float *sd2 = sd1 + TS * MLP_H;        // [TS][64]
    float *sd3 = sd2 + TS * MLP_H;        // [TS][3]
    float *sred = sd3 + TS * MLP_OUT;     // [256]
    const int t = threadIdx.x;
    const int tile0 = blockIdx.x * TS;
    const int ns = min(TS, nb - tile0);
    float my_loss = 0.0f;
    if (t < TS) {
        if (t < ns) {
            long long gi = b0 + tile0 + t;
            long long s = perm ? (long long)perm[gi] : gi;
            float xn[MLP_IN], tn[MLP_OUT], yn[MLP_OUT];
#pragma unroll
            for (int k = 0; k < MLP_IN; k++) {
                xn[k] = (X[s * MLP_IN + k] - nrm[k]) / nrm[MLP_IN + k];
                sx[t * MLP_IN + k] = xn[k];
            }
#pragma unroll
            for (int c = 0; c < MLP_OUT; c++) tn[c] = (Y[s * MLP_OUT + c] - nrm[2 * MLP_IN + c]) / nrm[2 * MLP_IN + MLP_OUT + c];
            float *h1 = sh1 + t * MLP_H, *h2 = sh2 + t * MLP_H;
            mlp_forward(P, xn, h1, h2, yn);
            float d3[MLP_OUT];
#pragma unroll
            for (int c = 0; c < MLP_OUT; c++) {
                const float e = yn[c] - tn[c];
                my_loss += e * e;
                d3[c] = 2.0f * e * inv3B;
                sd3[t * MLP_OUT + c] = d3[c];
            }
            float *d2 = sd2 + t * MLP_H, *d1 = sd1 + t * MLP_H;
            for (int j = 0; j < MLP_H; j++) {
                float s2 = 0.0f;
#pragma unroll
                for (int c = 0; c < MLP_OUT; c++) s2 = fmaf(P[MLP_W3 + c * MLP_H + j], d3[c], s2);
                d2[j] = s2 * (1.0f - h2[j] * h2[j]);
            }
            for (int j = 0; j < MLP_H; j++) {
                float s1 = 0.0f;
                for (int i = 0; i < MLP_H; i++) s1 = fmaf(P[MLP_W2 + i * MLP_H + j], d2[i], s1);
                d1[j] = s1 * (1.0f - h1[j] * h1[j]);
            }
        } else {
            // padding samples contribute nothing
            for (int k = 0; k < MLP_IN; k++) sx[t * MLP_IN + k] = 0.0f;
            for (int j = 0; j < MLP_H; j++) {
                sh1[t * MLP_H + j] = 0.0f; sh2[t * MLP_H + j] = 0.0f;
                sd1[t * MLP_H + j] = 0.0f; sd2[t * MLP_H + j] = 0.0f;
            }
            for (int c = 0; c < MLP_OUT; c++) sd3[t * MLP_OUT + c] = 0.0f;
        }
    }
    sred[t] = my_loss;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) sred[t] += sred[t + o];
        __syncthreads();
    }
    if (t == 0 && loss) atomicAdd(loss, sred[0] * inv3B);
    // gradient of every parameter, summed over the tile
    for (int p = t; p < MLP_NP; p += blockDim.x) {
        float g = 0.0f;
        if (p < MLP_B1) {
            const int j = p / MLP_IN, k = p % MLP_IN;
            for (int s = 0; s < TS; s++) g = fmaf(sd1[s * MLP_H + j], sx[s * MLP_IN + k], g);
        } else if (p < MLP_W2) {
            const int j = p - MLP_B1;
            for (int s = 0; s < TS; s++) g += sd1[s * MLP_H + j];
        } else if (p < MLP_B2) {
            const int i = (p - MLP_W2) / MLP_H, j = (p - MLP_W2) % MLP_H;
            for (int s = 0; s < TS; s++) g = fmaf(sd2[s * MLP_H + i], sh1[s * MLP_H + j], g);
        } else if (p < MLP_W3) {
            const int i = p - MLP_B2;
            for (int s = 0; s < TS; s++) g += sd2[s * MLP_H + i];
        } else if (p < MLP_B3) {
            const int c = (p - MLP_W3) / MLP_H, j = (p - MLP_W3) % MLP_H;
            for (int s = 0; s < TS; s++) g = fmaf(sd3[s * MLP_OUT + c], sh2[s * MLP_H + j], g);
        } else {
            const int c = p - MLP_B3;
            for (int s = 0; s < TS; s++) g += sd3[s * MLP_OUT + c];
        }
        atomicAdd(grad + p, g);
    }
}

__global__ void k_mlp_adam(float *P, float *grad, float *m, float *v, int np, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.0f - b1) * g;
    const float vv = b2 * v[p] + (1.0f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    P[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    grad[p] = 0.0f;
}

}  // namespace

static size_t mlp_tile_smem() { return sizeof(float) * (TS * MLP_IN + 4 * TS * MLP_H + TS * MLP_OUT + 256); }

cudaError_t launch_mlp_forward(const float *P, const float *nrm, const float *X, float *Y, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_mlp_forward<<<(n + 127) / 128, 128, 0, st>>>(P, nrm, X, Y, n);
    return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const float *P, const float *nrm, const float *X, const float *Y, const int *perm,
                            long long b0, int nb, int batch_total, float *grad, float *loss, cudaStream_t st) {
    if (nb <= 0) return cudaSuccess;
    // the tile needs more than the default 48 KB of shared memory; the
    // attribute is set once per device (setting it twice is harmless, so an
    // atomic flag is enough for callers on several host threads)
    static std::atomic<bool> attr[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!attr[dev].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(k_mlp_tile_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_tile_smem());
        if (e != cudaSuccess) return e;
        attr[dev].store(true, std::memory_order_release);
    }
    k_mlp_tile_grad<<<(nb + TS - 1) / TS, 256, mlp_tile_smem(), st>>>(P, nrm, X, Y, perm, b0, nb,
                                                                     1.0f / (3.0f * (float)batch_total), grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float *P, float *grad, float *m, float *v, float lr, int step, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_mlp_adam<<<(MLP_NP + 255) / 256, 256, 0, st>>>(P, grad, m, v, MLP_NP, lr, b1, b2, 1e-8f, c1, c2);
    return cudaGetLastError();
}

}  // namespace fsi
