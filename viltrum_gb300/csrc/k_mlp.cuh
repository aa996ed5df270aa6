/*
 * k_mlp.cuh -- the learned control variate's network on the tensor cores.
 *
 * No reference counterpart: the task asks for a small MLP control variate g (frequency encoding with
 * 6 bands, 4 hidden layers of 64, BF16 weights with FP32 accumulation) trained online on the
 * integrand's own samples, integrated per bin by quadrature, with only f - g sampled.
 *
 * Network: u in [0,1]^D (the point mapped into the range) -> features [u_d, sin(2^k pi u_d),
 * cos(2^k pi u_d), k < 6] (13 D, zero-padded to FIN) -> 4 x (64, ReLU) -> linear output.
 *
 * Tensor-core mapping: a warp pushes a tile of 16 points through the network with
 * mma.sync.m16n8k16 (BF16 in, FP32 accumulate).  Activations never leave registers between layers:
 * the FP32 accumulator fragments of two adjacent 8-column tiles are exactly the A fragment of the
 * next layer's 16-column k-tile, so bias + ReLU + BF16 packing happen in place.  Weights sit in
 * shared memory in two BF16 layouts -- out-major for the forward pass, in-major for the backward
 * pass -- with rows padded by 8 elements so the fragment loads of a warp hit 32 different banks.
 * Backward: dZ = dout * w4 * relu'(z) flows back the same way (dh = dZ W^T on the tensor cores);
 * dW = A^T dZ uses the activation and dZ tiles stored transposed in per-warp shared memory
 * (M = layer inputs, N = 64, K = the 16 points), accumulated per block in shared memory (FP32) and
 * once per block in global memory.
 */
#pragma once
#include <cuda_bf16.h>

#include "vcu_internal.cuh"

namespace vcu {
namespace mlp {

constexpr int WIDTH = 64;
constexpr int NT = WIDTH / 8;   /* 8-column n-tiles of a hidden layer  */
constexpr int KTH = WIDTH / 16; /* 16-column k-tiles of a hidden layer */
constexpr int PAD = 8;          /* bf16 elements of row padding        */
constexpr int BANDS = 6;

__host__ __device__ constexpr int fin(int d) { return ((13 * d + 15) / 16) * 16; }
/* fp32 master parameters: W0[FIN][64], b0, W1[64][64], b1, W2, b2, W3, b3, w4[64], b4 */
__host__ __device__ constexpr int n_params(int d) { return fin(d) * WIDTH + WIDTH + 3 * (WIDTH * WIDTH + WIDTH) + WIDTH + 1; }
__host__ __device__ constexpr int layer_in(int l, int d) { return l == 0 ? fin(d) : WIDTH; }
/* offsets of W_l and b_l in the fp32 parameter vector */
__host__ __device__ constexpr int w_off(int l, int d) {
    return l == 0 ? 0 : fin(d) * WIDTH + WIDTH + (l - 1) * (WIDTH * WIDTH + WIDTH);
}
__host__ __device__ constexpr int b_off(int l, int d) { return w_off(l, d) + layer_in(l, d) * WIDTH; }
__host__ __device__ constexpr int w4_off(int d) { return w_off(3, d) + WIDTH * WIDTH + WIDTH; }

/* packed device copy (the shared-memory image), in bf16 elements:
 *   T_l: [64][in_l + PAD] out-major, l = 0..3     (forward B operands)
 *   N_l: [in_l][64 + PAD] in-major,  l = 0..3     (backward B operands)
 * followed by fp32: bias[4][64], w4[64], b4, pad                                       */
__host__ __device__ constexpr int t_off(int l, int d) {
    return l == 0 ? 0 : WIDTH * (fin(d) + PAD) + (l - 1) * WIDTH * (WIDTH + PAD);
}
__host__ __device__ constexpr int t_elems(int d) { return WIDTH * (fin(d) + PAD) + 3 * WIDTH * (WIDTH + PAD); }
__host__ __device__ constexpr int n_off(int l, int d) {
    return t_elems(d) + (l == 0 ? 0 : fin(d) * (WIDTH + PAD) + (l - 1) * WIDTH * (WIDTH + PAD));
}
__host__ __device__ constexpr int bf16_elems(int d) { return 2 * t_elems(d) - WIDTH * (fin(d) + PAD) + fin(d) * (WIDTH + PAD); }
__host__ __device__ constexpr int fp32_off_bytes(int d) { return ((bf16_elems(d) * 2 + 15) / 16) * 16; }
__host__ __device__ constexpr int pack_bytes(int d) { return fp32_off_bytes(d) + (4 * WIDTH + WIDTH + 4) * 4; }
__host__ __device__ constexpr int fwd_bytes(int d) { return t_elems(d) * 2; } /* forward needs T only + fp32 */

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

/* feature column c of the encoding of one point (c >= 13 D: padding) */
template <int D> __device__ __forceinline__ float feature(const float* u, int c) {
    if (c < D) return u[c];
    const int q = c - D;
    if (q >= 12 * D) return 0.0f;
    const int d = q / 12, k = (q % 12) >> 1;
    const float a = u[d] * (float)(1 << k);
    return (q & 1) ? cospif(a) : sinpif(a);
}

/* A fragments of the feature tile: rows g and g+8 of the warp's 16 points (lane = 4g + t) */
template <int D> __device__ __forceinline__ void features_tile(const float* u_g, const float* u_g8, uint32_t (*A)[4]) {
    const int t = threadIdx.x & 3;
#pragma unroll
    for (int kt = 0; kt < fin(D) / 16; ++kt) {
        const int c0 = 16 * kt + 2 * t;
        A[kt][0] = pack_bf16x2(feature<D>(u_g, c0), feature<D>(u_g, c0 + 1));
        A[kt][1] = pack_bf16x2(feature<D>(u_g8, c0), feature<D>(u_g8, c0 + 1));
        A[kt][2] = pack_bf16x2(feature<D>(u_g, c0 + 8), feature<D>(u_g, c0 + 9));
        A[kt][3] = pack_bf16x2(feature<D>(u_g8, c0 + 8), feature<D>(u_g8, c0 + 9));
    }
}

/* one layer: C = A W + b on the tensor cores, then ReLU, packed as the next layer's A fragments */
template <int KT>
__device__ __forceinline__ void layer_forward(const uint32_t (*A)[4], const __nv_bfloat16* T, int stride,
                                              const float* bias, uint32_t (*H)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float C[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const float b0 = bias[8 * j + 2 * t], b1 = bias[8 * j + 2 * t + 1];
        C[j][0] = b0;
        C[j][1] = b1;
        C[j][2] = b0;
        C[j][3] = b1;
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const uint32_t* row = reinterpret_cast<const uint32_t*>(T + (8 * j + g) * stride + 16 * kt);
            mma16816(C[j], A[kt], row[t], row[t + 4]);
        }
#pragma unroll
    for (int kt = 0; kt < KTH; ++kt) {
        H[kt][0] = pack_bf16x2(fmaxf(C[2 * kt][0], 0.0f), fmaxf(C[2 * kt][1], 0.0f));
        H[kt][1] = pack_bf16x2(fmaxf(C[2 * kt][2], 0.0f), fmaxf(C[2 * kt][3], 0.0f));
        H[kt][2] = pack_bf16x2(fmaxf(C[2 * kt + 1][0], 0.0f), fmaxf(C[2 * kt + 1][1], 0.0f));
        H[kt][3] = pack_bf16x2(fmaxf(C[2 * kt + 1][2], 0.0f), fmaxf(C[2 * kt + 1][3], 0.0f));
    }
}

/* output g = w4 . h4 + b4 for rows g (out[0]) and g+8 (out[1]), replicated over the 4 lanes of a row */
__device__ __forceinline__ void output_layer(const uint32_t (*H)[4], const float* w4, float b4, float* out) {
    const int t = threadIdx.x & 3;
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
    for (int kt = 0; kt < KTH; ++kt) {
        const int c = 16 * kt + 2 * t;
        s0 = fmaf(bf16_lo(H[kt][0]), w4[c], s0);
        s0 = fmaf(bf16_hi(H[kt][0]), w4[c + 1], s0);
        s0 = fmaf(bf16_lo(H[kt][2]), w4[c + 8], s0);
        s0 = fmaf(bf16_hi(H[kt][2]), w4[c + 9], s0);
        s1 = fmaf(bf16_lo(H[kt][1]), w4[c], s1);
        s1 = fmaf(bf16_hi(H[kt][1]), w4[c + 1], s1);
        s1 = fmaf(bf16_lo(H[kt][3]), w4[c + 8], s1);
        s1 = fmaf(bf16_hi(H[kt][3]), w4[c + 9], s1);
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    out[0] = s0 + b4;
    out[1] = s1 + b4;
}

/* forward pass of a 16-point tile; H[l] keeps the input activations of layers 1..3 and h4 */
template <int D> struct Acts {
    uint32_t F[fin(D) / 16][4];
    uint32_t H[4][KTH][4];
};

/* shared-memory image of the parameters (loaded once per block) */
template <int D> struct SmemParams {
    const __nv_bfloat16* T[4];
    const __nv_bfloat16* N[4];
    const float* bias[4];
    const float* w4;
    float b4;
};

template <int D> __device__ __forceinline__ SmemParams<D> smem_params(const char* base, bool with_backward) {
    SmemParams<D> p;
    const __nv_bfloat16* bf = reinterpret_cast<const __nv_bfloat16*>(base);
    for (int l = 0; l < 4; ++l) {
        p.T[l] = bf + t_off(l, D);
        p.N[l] = with_backward ? bf + n_off(l, D) : nullptr;
    }
    const int foff = with_backward ? fp32_off_bytes(D) : ((fwd_bytes(D) + 15) / 16) * 16;
    const float* f32 = reinterpret_cast<const float*>(base + foff);
    for (int l = 0; l < 4; ++l) p.bias[l] = f32 + l * WIDTH;
    p.w4 = f32 + 4 * WIDTH;
    p.b4 = f32[5 * WIDTH];
    return p;
}

/* copy the packed image (global) into shared memory; forward-only blocks skip the N layouts */
template <int D> __device__ __forceinline__ void load_params(char* smem, const char* packed, bool with_backward) {
    const int nthreads = blockDim.x;
    if (with_backward) {
        const int n16 = pack_bytes(D) / 16;
        for (int i = threadIdx.x; i < n16; i += nthreads)
            reinterpret_cast<int4*>(smem)[i] = reinterpret_cast<const int4*>(packed)[i];
    } else {
        const int nt16 = (fwd_bytes(D) + 15) / 16;
        for (int i = threadIdx.x; i < nt16; i += nthreads)
            reinterpret_cast<int4*>(smem)[i] = reinterpret_cast<const int4*>(packed)[i];
        const int foff = ((fwd_bytes(D) + 15) / 16) * 16;
        const float* src = reinterpret_cast<const float*>(packed + fp32_off_bytes(D));
        float* dst = reinterpret_cast<float*>(smem + foff);
        for (int i = threadIdx.x; i < 5 * WIDTH + 4; i += nthreads) dst[i] = src[i];
    }
    __syncthreads();
}
template <int D> __host__ __device__ constexpr int smem_fwd_bytes() { return ((fwd_bytes(D) + 15) / 16) * 16 + (5 * WIDTH + 4) * 4; }

template <int D> __device__ __forceinline__ void forward_tile(const SmemParams<D>& P, Acts<D>& a, float* out) {
    layer_forward<fin(D) / 16>(a.F, P.T[0], fin(D) + PAD, P.bias[0], a.H[0]);
    layer_forward<KTH>(a.H[0], P.T[1], WIDTH + PAD, P.bias[1], a.H[1]);
    layer_forward<KTH>(a.H[1], P.T[2], WIDTH + PAD, P.bias[2], a.H[2]);
    layer_forward<KTH>(a.H[2], P.T[3], WIDTH + PAD, P.bias[3], a.H[3]);
    output_layer(a.H[3], P.w4, P.b4, out);
}

}  // namespace mlp
}  // namespace vcu
