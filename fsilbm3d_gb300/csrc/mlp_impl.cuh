// mlp_impl.cuh -- the 12 -> 64 -> 64 -> 3 perceptron of the learned
// immersed-boundary warm start (no counterpart in the reference; it feeds the
// penalty loop of Solidbody.f90:893-906 an initial Lagrangian force).
//
// Parameters, one flat FP32 array: W1[64][12], b1[64], W2[64][64], b2[64],
// W3[3][64], b3[3] (rows = outputs). Hidden activations tanh. Inputs are
// standardised with (x - mean)/std and outputs de-standardised with
// y*std + mean; the 30 statistics live in a separate array:
// mean_in[12], std_in[12], mean_out[3], std_out[3].
//
// Features of a Lagrangian point (in this order): velocity mismatch
// U_body - u_interp before any correction of the step (3), body velocity (3),
// body acceleration (3), surface normal (3); all velocities divided by Uref.
// Target: the converged Lagrangian force divided by (area * Uref).
#pragma once

namespace fsi {

constexpr int MLP_IN = 12, MLP_H = 64, MLP_OUT = 3;
constexpr int MLP_W1 = 0, MLP_B1 = MLP_W1 + MLP_H * MLP_IN, MLP_W2 = MLP_B1 + MLP_H,
              MLP_B2 = MLP_W2 + MLP_H * MLP_H, MLP_W3 = MLP_B2 + MLP_H, MLP_B3 = MLP_W3 + MLP_OUT * MLP_H,
              MLP_NP = MLP_B3 + MLP_OUT;
constexpr int MLP_NNORM = 2 * MLP_IN + 2 * MLP_OUT;

// forward pass of one standardised input; h1/h2 receive the activations
__device__ __forceinline__ void mlp_forward(const float *__restrict__ P, const float xn[MLP_IN], float h1[MLP_H],
                                            float h2[MLP_H], float yn[MLP_OUT]) {
    for (int j = 0; j < MLP_H; j++) {
        float s = P[MLP_B1 + j];
#pragma unroll
        for (int k = 0; k < MLP_IN; k++) s = fmaf(P[MLP_W1 + j * MLP_IN + k], xn[k], s);
        h1[j] = tanhf(s);
    }
    for (int j = 0; j < MLP_H; j++) {
        float s = P[MLP_B2 + j];
#pragma unroll 8
        for (int k = 0; k < MLP_H; k++) s = fmaf(P[MLP_W2 + j * MLP_H + k], h1[k], s);
        h2[j] = tanhf(s);
    }
#pragma unroll
    for (int c = 0; c < MLP_OUT; c++) {
        float s = P[MLP_B3 + c];
#pragma unroll 8
        for (int k = 0; k < MLP_H; k++) s = fmaf(P[MLP_W3 + c * MLP_H + k], h2[k], s);
        yn[c] = s;
    }
}

// The same network evaluated by one warp for one raw input x (every lane
// holds all 12 features): lane l owns hidden units l and l+32, the layer-2
// inputs are broadcast by shuffles and the outputs reduced across the warp.
// Returns the de-standardised output on every lane. Summation order differs
// from mlp_forward, so the two agree to FP32 rounding, not bitwise.
__device__ __forceinline__ void mlp_forward_warp(const float *__restrict__ P, const float *__restrict__ nrm,
                                                 const float x[MLP_IN], int lane, float y[MLP_OUT]) {
    float xn[MLP_IN];
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) xn[k] = (x[k] - nrm[k]) / nrm[MLP_IN + k];
    const int ja = lane, jb = lane + 32;
    float ha = P[MLP_B1 + ja], hb = P[MLP_B1 + jb];
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) {
        ha = fmaf(P[MLP_W1 + ja * MLP_IN + k], xn[k], ha);
        hb = fmaf(P[MLP_W1 + jb * MLP_IN + k], xn[k], hb);
    }
    ha = tanhf(ha);
    hb = tanhf(hb);
    float ga = P[MLP_B2 + ja], gb = P[MLP_B2 + jb];
#pragma unroll 8
    for (int k = 0; k < 32; k++) {
        const float h = __shfl_sync(0xffffffffu, ha, k);
        ga = fmaf(P[MLP_W2 + ja * MLP_H + k], h, ga);
        gb = fmaf(P[MLP_W2 + jb * MLP_H + k], h, gb);
    }
#pragma unroll 8
    for (int k = 0; k < 32; k++) {
        const float h = __shfl_sync(0xffffffffu, hb, k);
        ga = fmaf(P[MLP_W2 + ja * MLP_H + 32 + k], h, ga);
        gb = fmaf(P[MLP_W2 + jb * MLP_H + 32 + k], h, gb);
    }
    ga = tanhf(ga);
    gb = tanhf(gb);
#pragma unroll
    for (int c = 0; c < MLP_OUT; c++) {
        float s = fmaf(P[MLP_W3 + c * MLP_H + ja], ga, P[MLP_W3 + c * MLP_H + jb] * gb);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        y[c] = (s + P[MLP_B3 + c]) * nrm[2 * MLP_IN + MLP_OUT + c] + nrm[2 * MLP_IN + c];
    }
}

}  // namespace fsi
