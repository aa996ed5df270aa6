/*
 * k_mlp.cu -- learned control variate: online training, per-bin integral of the network, residual.
 *
 * No reference counterpart (the task's learned part; the per-bin wrapper it plugs into is
 * src/integrator-per-bin-parallel.h:17-35).  Pipeline of vcu_learned_control_variates:
 *  1. train: `train_steps` Adam steps on fresh samples of the integrand (Philox points over the
 *     range, the integrand evaluated by the device) minimising mean (g - f)^2; each step is one
 *     sampling kernel, one fused forward+backward kernel (k_mlp_train: every block writes its own
 *     partial gradient, no atomics), one Adam kernel that sums the partials in a fixed order and
 *     rewrites the BF16 image of the weights, and one counter kernel -- captured once in a CUDA
 *     graph and replayed for all steps;
 *  2. k_mlp_integral: per bin, Gauss-Legendre quadrature (q nodes per dimension) of g over the bin;
 *  3. k_mlp_residual: per bin, `samples` Philox points, estimate = integral of g + mean(f - g)
 *     (control variate with weight 1: unbiased up to the quadrature error of the network's
 *     integral); optionally the plain Monte Carlo mean of the same samples is kept instead when
 *     its sample variance is lower (per-bin fallback).
 */
#include "k_mlp.cuh"

namespace vcu {
namespace mlp {

constexpr int TRAIN_WARPS = 8;
constexpr int FWD_WARPS = 4;
constexpr int ROUND = TRAIN_WARPS * 16; /* points of one block round: a 16-point tile per warp      */
constexpr int KS = ROUND + 8;           /* bf16 row stride of the block's transposed tiles (bank skew) */
constexpr int GS = WIDTH + 8;           /* fp32 row stride of the block's dW accumulators            */
constexpr int SLOT = 4 * WIDTH + WIDTH + 4; /* per-warp sums: db[4][64], dw4[64], db4, pad          */
/* rows of the transposed activation tile: the widest layer input (features or a hidden layer) */
__host__ __device__ constexpr int at_rows(int d) { return fin(d) > WIDTH ? fin(d) : WIDTH; }
__host__ __device__ constexpr int gw_floats(int d) { return (fin(d) + 3 * WIDTH) * GS; }

struct RangeCfg {
    float rmin[VCU_MAX_DIM], rmax[VCU_MAX_DIM];
};

struct TrainCfg {
    RangeCfg r;
    uint32_t k0, k1;
    uint32_t rounds;         /* ROUND-point rounds per block */
    float scale;             /* 2 / batch */
    const float* u_in;       /* explicit points (gradient check) or null */
    const float* y_in;
    float* out;              /* outputs of explicit points, or null */
    uint64_t npts;           /* explicit points: count */
};

/* training block: parameter image | dW accumulators (fp32) | per-warp bias/output sums |
 * transposed activation tile AT[in][ROUND] | transposed dZ tile ZT[64][ROUND] (bf16) */
template <int D> __host__ __device__ constexpr int train_smem_bytes() {
    return pack_bytes(D) + (gw_floats(D) + TRAIN_WARPS * SLOT) * 4 + (at_rows(D) + WIDTH) * KS * 2;
}

/* a warp's 16-point tile of layer inputs (A fragments) -> columns col0..col0+15 of AT[input][point] */
template <int KT>
__device__ __forceinline__ void stage_A(__nv_bfloat16* AT, const uint32_t (*A)[4], int col0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat16* p = AT + col0 + g;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
        const int c = 16 * kt + 2 * t;
        p[c * KS] = __ushort_as_bfloat16((unsigned short)(A[kt][0] & 0xffff));
        p[(c + 1) * KS] = __ushort_as_bfloat16((unsigned short)(A[kt][0] >> 16));
        p[c * KS + 8] = __ushort_as_bfloat16((unsigned short)(A[kt][1] & 0xffff));
        p[(c + 1) * KS + 8] = __ushort_as_bfloat16((unsigned short)(A[kt][1] >> 16));
        p[(c + 8) * KS] = __ushort_as_bfloat16((unsigned short)(A[kt][2] & 0xffff));
        p[(c + 9) * KS] = __ushort_as_bfloat16((unsigned short)(A[kt][2] >> 16));
        p[(c + 8) * KS + 8] = __ushort_as_bfloat16((unsigned short)(A[kt][3] & 0xffff));
        p[(c + 9) * KS + 8] = __ushort_as_bfloat16((unsigned short)(A[kt][3] >> 16));
    }
}

/* a warp's dZ tile (C fragments, already BF16-valued) -> columns col0.. of ZT[unit][point]; its
 * column sums (the bias gradient) are added to the warp's own slot db[64] */
__device__ __forceinline__ void stage_Z(__nv_bfloat16* ZT, const float (*dZ)[4], int col0, float* db) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat16* p = ZT + col0 + g;
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int c = 8 * j + 2 * t;
        p[c * KS] = __float2bfloat16_rn(dZ[j][0]);
        p[(c + 1) * KS] = __float2bfloat16_rn(dZ[j][1]);
        p[c * KS + 8] = __float2bfloat16_rn(dZ[j][2]);
        p[(c + 1) * KS + 8] = __float2bfloat16_rn(dZ[j][3]);
        float s0 = dZ[j][0] + dZ[j][2], s1 = dZ[j][1] + dZ[j][3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (g == 0) {
            db[c] += s0;
            db[c + 1] += s1;
        }
    }
}

/* dW[in][64] += AT . ZT^T over the block's ROUND points (M = inputs, N = 64 units, K = points) on the
 * tensor cores; each warp owns whole 16x8 output tiles, so the FP32 accumulators in shared memory
 * are read and written by one warp only (no atomics, fixed summation order) */
template <int MT>
__device__ __forceinline__ void block_dW(const __nv_bfloat16* AT, const __nv_bfloat16* ZT, float* gw) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int tile = warp; tile < MT * NT; tile += TRAIN_WARPS) {
        const int mt = tile / NT, j = tile % NT;
        float* r0 = gw + (16 * mt + g) * GS + 8 * j + 2 * t;
        float* r1 = r0 + 8 * GS;
        float c[4] = {r0[0], r0[1], r1[0], r1[1]};
        const uint32_t* a0 = reinterpret_cast<const uint32_t*>(AT + (16 * mt + g) * KS);
        const uint32_t* a1 = reinterpret_cast<const uint32_t*>(AT + (16 * mt + g + 8) * KS);
        const uint32_t* zb = reinterpret_cast<const uint32_t*>(ZT + (8 * j + g) * KS);
#pragma unroll
        for (int ks = 0; ks < ROUND / 16; ++ks) {
            const uint32_t a[4] = {a0[8 * ks + t], a1[8 * ks + t], a0[8 * ks + t + 4], a1[8 * ks + t + 4]};
            mma16816(c, a, zb[8 * ks + t], zb[8 * ks + t + 4]);
        }
        r0[0] = c[0];
        r0[1] = c[1];
        r1[0] = c[2];
        r1[1] = c[3];
    }
}

/* dh = dZ W^T for layer l (W in-major N_l: [in][64+PAD]), masked by relu'(previous z) */
__device__ __forceinline__ void backprop_layer(const float (*dZ)[4], const __nv_bfloat16* N, const uint32_t (*Hprev)[4],
                                               float (*dH)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t AZ[KTH][4];
#pragma unroll
    for (int kt = 0; kt < KTH; ++kt) {
        AZ[kt][0] = pack_bf16x2(dZ[2 * kt][0], dZ[2 * kt][1]);
        AZ[kt][1] = pack_bf16x2(dZ[2 * kt][2], dZ[2 * kt][3]);
        AZ[kt][2] = pack_bf16x2(dZ[2 * kt + 1][0], dZ[2 * kt + 1][1]);
        AZ[kt][3] = pack_bf16x2(dZ[2 * kt + 1][2], dZ[2 * kt + 1][3]);
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        dH[j][0] = dH[j][1] = dH[j][2] = dH[j][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < KTH; ++kt) {
            const uint32_t* row = reinterpret_cast<const uint32_t*>(N + (8 * j + g) * (WIDTH + PAD) + 16 * kt);
            mma16816(dH[j], AZ[kt], row[t], row[t + 4]);
        }
    }
    /* relu' of the previous layer's pre-activation: its BF16 output is > 0 */
#pragma unroll
    for (int kt = 0; kt < KTH; ++kt) {
        const uint32_t* h = Hprev[kt];
        dH[2 * kt][0] = bf16_lo(h[0]) > 0.0f ? dH[2 * kt][0] : 0.0f;
        dH[2 * kt][1] = bf16_hi(h[0]) > 0.0f ? dH[2 * kt][1] : 0.0f;
        dH[2 * kt][2] = bf16_lo(h[1]) > 0.0f ? dH[2 * kt][2] : 0.0f;
        dH[2 * kt][3] = bf16_hi(h[1]) > 0.0f ? dH[2 * kt][3] : 0.0f;
        dH[2 * kt + 1][0] = bf16_lo(h[2]) > 0.0f ? dH[2 * kt + 1][0] : 0.0f;
        dH[2 * kt + 1][1] = bf16_hi(h[2]) > 0.0f ? dH[2 * kt + 1][1] : 0.0f;
        dH[2 * kt + 1][2] = bf16_lo(h[3]) > 0.0f ? dH[2 * kt + 1][2] : 0.0f;
        dH[2 * kt + 1][3] = bf16_hi(h[3]) > 0.0f ? dH[2 * kt + 1][3] : 0.0f;
    }
    /* round through BF16 once, as the tensor cores will consume it */
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) dH[j][i] = __bfloat162float(__float2bfloat16_rn(dH[j][i]));
}

/* training points of one step: Philox points over the range and the integrand's values there */
template <class F, int D>
__global__ void k_mlp_samples(const __grid_constant__ F f, const TrainCfg cfg, uint64_t n, float* __restrict__ u_out,
                              float* __restrict__ y_out, const uint32_t* __restrict__ step_ctr) {
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t step = *step_ctr;
    float u[D], x[F::DIM];
    for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
#pragma unroll
    for (int blk = 0; blk < (D + 3) / 4; ++blk) {
        const U4 r = philox4x32_10(U4{(uint32_t)s, (uint32_t)(s >> 32), step, 0x7EA10000u + blk}, cfg.k0, cfg.k1);
        const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int d = blk * 4 + k;
            if (d < D) u[d] = u01(rr[k]);
        }
    }
    for (int d = 0; d < D; ++d) {
        x[d] = vadd(vmul(u[d], vsub(cfg.r.rmax[d], cfg.r.rmin[d])), cfg.r.rmin[d]);
        u_out[s * D + d] = u[d];
    }
    float v[1];
    f(x, v);
    y_out[s] = v[0];
}

/* One training step's forward and backward over cfg.rounds x ROUND points per block.  Each warp
 * pushes a 16-point tile through the network in registers (activations stay in the A-fragment
 * layout), then layer by layer from the top: the warp stages its tile's layer inputs and dZ
 * (transposed, BF16) into the block's tiles and computes dh = dZ W^T for the layer below; after a
 * barrier the block computes dW += AT . ZT^T over all its points on the tensor cores.  The block
 * writes its summed gradient to partial[block] (kernel order: W0..W3, b0..b3, w4, b4). */
template <int D>
__global__ void __launch_bounds__(TRAIN_WARPS * 32, 1)
    k_mlp_train(const TrainCfg cfg, const char* __restrict__ packed, float* __restrict__ partial) {
    extern __shared__ __align__(16) char smem[];
    load_params<D>(smem, packed, true);
    const SmemParams<D> P = smem_params<D>(smem, true);
    float* gw = reinterpret_cast<float*>(smem + pack_bytes(D));
    float* slots = gw + gw_floats(D);
    __nv_bfloat16* AT = reinterpret_cast<__nv_bfloat16*>(slots + TRAIN_WARPS * SLOT);
    __nv_bfloat16* ZT = AT + at_rows(D) * KS;
    for (int i = threadIdx.x; i < gw_floats(D) + TRAIN_WARPS * SLOT; i += blockDim.x) gw[i] = 0.0f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float* my = slots + warp * SLOT; /* db[4][64] | dw4[64] | db4 */
    const int col0 = warp * 16;
    for (uint32_t round = 0; round < cfg.rounds; ++round) {
        const uint64_t base = ((uint64_t)blockIdx.x * cfg.rounds + round) * ROUND + col0;
        const uint64_t s0 = base + g, s1 = base + g + 8;
        const bool v0 = s0 < cfg.npts, v1 = s1 < cfg.npts;
        float ug[D], ug8[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            ug[d] = v0 ? cfg.u_in[s0 * D + d] : 0.5f;
            ug8[d] = v1 ? cfg.u_in[s1 * D + d] : 0.5f;
        }
        const float y0 = v0 ? cfg.y_in[s0] : 0.0f, y1 = v1 ? cfg.y_in[s1] : 0.0f;
        Acts<D> a;
        features_tile<D>(ug, ug8, a.F);
        float out[2];
        forward_tile<D>(P, a, out);
        if (cfg.out && t == 0) {
            if (v0) cfg.out[s0] = out[0];
            if (v1) cfg.out[s1] = out[1];
        }
        const float d0 = v0 ? (out[0] - y0) * cfg.scale : 0.0f;
        const float d1 = v1 ? (out[1] - y1) * cfg.scale : 0.0f;
        /* output layer: dw4 = sum d * h4, db4 = sum d (the warp's own slot) */
        {
            float sb = (t == 0) ? d0 + d1 : 0.0f;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) sb += __shfl_xor_sync(0xffffffffu, sb, o);
            if (lane == 0) my[5 * WIDTH] += sb;
#pragma unroll
            for (int kt = 0; kt < KTH; ++kt) {
                const int c = 16 * kt + 2 * t;
                float sw[4] = {d0 * bf16_lo(a.H[3][kt][0]) + d1 * bf16_lo(a.H[3][kt][1]),
                               d0 * bf16_hi(a.H[3][kt][0]) + d1 * bf16_hi(a.H[3][kt][1]),
                               d0 * bf16_lo(a.H[3][kt][2]) + d1 * bf16_lo(a.H[3][kt][3]),
                               d0 * bf16_hi(a.H[3][kt][2]) + d1 * bf16_hi(a.H[3][kt][3])};
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int o = 4; o < 32; o <<= 1) sw[i] += __shfl_xor_sync(0xffffffffu, sw[i], o);
                if (g == 0) {
                    my[4 * WIDTH + c] += sw[0];
                    my[4 * WIDTH + c + 1] += sw[1];
                    my[4 * WIDTH + c + 8] += sw[2];
                    my[4 * WIDTH + c + 9] += sw[3];
                }
            }
        }
        /* dZ4 = dout * w4 * relu'(z4), rounded to BF16 */
        float dZ[NT][4], dH[NT][4];
#pragma unroll
        for (int kt = 0; kt < KTH; ++kt) {
            const int c = 16 * kt + 2 * t;
            const uint32_t* h = a.H[3][kt];
            dZ[2 * kt][0] = bf16_lo(h[0]) > 0.0f ? d0 * P.w4[c] : 0.0f;
            dZ[2 * kt][1] = bf16_hi(h[0]) > 0.0f ? d0 * P.w4[c + 1] : 0.0f;
            dZ[2 * kt][2] = bf16_lo(h[1]) > 0.0f ? d1 * P.w4[c] : 0.0f;
            dZ[2 * kt][3] = bf16_hi(h[1]) > 0.0f ? d1 * P.w4[c + 1] : 0.0f;
            dZ[2 * kt + 1][0] = bf16_lo(h[2]) > 0.0f ? d0 * P.w4[c + 8] : 0.0f;
            dZ[2 * kt + 1][1] = bf16_hi(h[2]) > 0.0f ? d0 * P.w4[c + 9] : 0.0f;
            dZ[2 * kt + 1][2] = bf16_lo(h[3]) > 0.0f ? d1 * P.w4[c + 8] : 0.0f;
            dZ[2 * kt + 1][3] = bf16_hi(h[3]) > 0.0f ? d1 * P.w4[c + 9] : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int i = 0; i < 4; ++i) dZ[j][i] = __bfloat162float(__float2bfloat16_rn(dZ[j][i]));
        /* layer 3 */
        stage_A<KTH>(AT, a.H[2], col0);
        stage_Z(ZT, dZ, col0, my + 3 * WIDTH);
        backprop_layer(dZ, P.N[3], a.H[2], dH);
        __syncthreads();
        block_dW<KTH>(AT, ZT, gw + (fin(D) + 2 * WIDTH) * GS);
        __syncthreads();
        /* layer 2 */
        stage_A<KTH>(AT, a.H[1], col0);
        stage_Z(ZT, dH, col0, my + 2 * WIDTH);
        backprop_layer(dH, P.N[2], a.H[1], dZ);
        __syncthreads();
        block_dW<KTH>(AT, ZT, gw + (fin(D) + WIDTH) * GS);
        __syncthreads();
        /* layer 1 */
        stage_A<KTH>(AT, a.H[0], col0);
        stage_Z(ZT, dZ, col0, my + WIDTH);
        backprop_layer(dZ, P.N[1], a.H[0], dH);
        __syncthreads();
        block_dW<KTH>(AT, ZT, gw + fin(D) * GS);
        __syncthreads();
        /* layer 0 (features) */
        stage_A<fin(D) / 16>(AT, a.F, col0);
        stage_Z(ZT, dH, col0, my);
        __syncthreads();
        block_dW<fin(D) / 16>(AT, ZT, gw);
        __syncthreads();
    }
    /* the block's gradient: W rows are consecutive in gw (W0 rows, then W1..W3); the per-warp sums
     * are added in warp order */
    float* dst = partial + (size_t)blockIdx.x * n_params(D);
    const int nw = (fin(D) + 3 * WIDTH) * WIDTH;
    for (int i = threadIdx.x; i < n_params(D); i += blockDim.x) {
        float v = 0.0f;
        if (i < nw) {
            v = gw[(i / WIDTH) * GS + (i % WIDTH)];
        } else {
            const int k = i - nw; /* db[4][64], dw4[64], db4: the slot layout */
#pragma unroll
            for (int w = 0; w < TRAIN_WARPS; ++w) v += slots[w * SLOT + k];
        }
        dst[i] = v;
    }
}

/* grad[i] = sum over blocks of partial[b][i], in block order */
template <int D>
__global__ void k_mlp_reduce(const float* __restrict__ partial, int nparts, float* __restrict__ grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_params(D)) return;
    float s = 0.0f;
    for (int b = 0; b < nparts; ++b) s += partial[(size_t)b * n_params(D) + i];
    grad[i] = s;
}

/* gradient layout in shared memory / global: gW0..gW3 (W order), gb0..gb3, gw4, gb4 -> parameter index */
template <int D> __device__ __forceinline__ int grad_to_param(int i) {
    const int a = fin(D) * WIDTH, hid = WIDTH * WIDTH;
    if (i < a) return w_off(0, D) + i;
    if (i < a + 3 * hid) {
        const int l = 1 + (i - a) / hid;
        return w_off(l, D) + (i - a) % hid;
    }
    i -= a + 3 * hid;
    if (i < 4 * WIDTH) return b_off(i / WIDTH, D) + i % WIDTH;
    i -= 4 * WIDTH;
    return w4_off(D) + i; /* w4[0..63], then b4 */
}

/* write parameter p (fp32) into the packed shared-memory image */
template <int D> __device__ __forceinline__ void pack_param(char* packed, int p, float v) {
    __nv_bfloat16* bf = reinterpret_cast<__nv_bfloat16*>(packed);
    float* f32 = reinterpret_cast<float*>(packed + fp32_off_bytes(D));
    for (int l = 0; l < 4; ++l) {
        const int in = layer_in(l, D);
        const int w0 = w_off(l, D);
        if (p >= w0 && p < w0 + in * WIDTH) {
            const int k = (p - w0) / WIDTH, n = (p - w0) % WIDTH;
            const __nv_bfloat16 b = __float2bfloat16_rn(v);
            bf[t_off(l, D) + n * (in + PAD) + k] = b;
            bf[n_off(l, D) + k * (WIDTH + PAD) + n] = b;
            return;
        }
        if (p >= b_off(l, D) && p < b_off(l, D) + WIDTH) {
            f32[l * WIDTH + (p - b_off(l, D))] = v;
            return;
        }
    }
    f32[4 * WIDTH + (p - w4_off(D))] = v; /* w4 and b4 */
}

struct AdamCfg {
    float lr, b1, b2, eps;
    int n;
    int nparts; /* per-block partial gradients to add */
};

template <int D>
__global__ void k_mlp_adam(const AdamCfg c, float* __restrict__ theta, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ partial, const uint32_t* __restrict__ step_ctr,
                           char* __restrict__ packed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int p = grad_to_param<D>(i);
    float gr = 0.0f;
    for (int b = 0; b < c.nparts; ++b) gr += partial[(size_t)b * c.n + i];
    const float t = (float)(*step_ctr + 1);
    const float mi = c.b1 * m[p] + (1.0f - c.b1) * gr;
    const float vi = c.b2 * v[p] + (1.0f - c.b2) * gr * gr;
    m[p] = mi;
    v[p] = vi;
    const float mh = mi / (1.0f - powf(c.b1, t));
    const float vh = vi / (1.0f - powf(c.b2, t));
    const float w = theta[p] - c.lr * mh / (sqrtf(vh) + c.eps);
    theta[p] = w;
    pack_param<D>(packed, p, w);
}

__global__ void k_mlp_step_inc(uint32_t* step_ctr) { *step_ctr += 1u; }

template <int D> __global__ void k_mlp_pack(const float* __restrict__ theta, char* __restrict__ packed) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n_params(D)) pack_param<D>(packed, p, theta[p]);
}

/* ---------------------------------------------------------------- per-bin integral of g */
struct BinCfg {
    RangeCfg r;
    float drange[VCU_MAX_DIMBINS];
    uint32_t res[VCU_MAX_DIMBINS];
    int32_t dimbins;
    uint64_t nbins;
    int32_t q;     /* Gauss-Legendre nodes per cell and dimension */
    int32_t cells;          /* composite cells per binned dimension   */
    int32_t cells_unbinned; /* composite cells per unbinned dimension */
    float gl_x[4], gl_w[4];
};

template <int D>
__device__ __forceinline__ void bin_box(const BinCfg& c, uint64_t bin, float* lo, float* hi) {
    uint64_t rem = bin;
    for (int d = 0; d < D; ++d) {
        lo[d] = c.r.rmin[d];
        hi[d] = c.r.rmax[d];
        if (d < c.dimbins) {
            const uint32_t pos = (uint32_t)(rem % c.res[d]);
            rem /= c.res[d];
            lo[d] = vadd(c.r.rmin[d], vmul((float)pos, c.drange[d]));
            hi[d] = vadd(c.r.rmin[d], vmul((float)(pos + 1), c.drange[d]));
        }
    }
}

template <int D>
__global__ void __launch_bounds__(FWD_WARPS * 32)
    k_mlp_integral(const BinCfg c, const char* __restrict__ packed, float* __restrict__ integral) {
    extern __shared__ __align__(16) char smem[];
    load_params<D>(smem, packed, false);
    const SmemParams<D> P = smem_params<D>(smem, false);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2;
    /* per dimension `cells` equal cells of q Gauss-Legendre nodes; the unbinned dimensions, which
     * span the whole range rather than one bin, have their own cell count */
    int qd[D], cd[D];
    int nodes = 1;
    for (int d = 0; d < D; ++d) {
        cd[d] = d < c.dimbins ? c.cells : c.cells_unbinned;
        qd[d] = c.q * cd[d];
        nodes *= qd[d];
    }
    for (uint64_t bin = (uint64_t)blockIdx.x * FWD_WARPS + warp; bin < c.nbins; bin += (uint64_t)gridDim.x * FWD_WARPS) {
        float lo[D], hi[D];
        bin_box<D>(c, bin, lo, hi);
        double acc = 0.0;
        for (int base = 0; base < nodes; base += 16) {
            float ug[D], ug8[D], w0 = 1.0f, w1 = 1.0f;
            const int n0 = base + g, n1 = base + g + 8;
            int r0 = n0, r1 = n1;
            for (int d = 0; d < D; ++d) {
                const int i0 = r0 % qd[d], i1 = r1 % qd[d];
                r0 /= qd[d];
                r1 /= qd[d];
                const float inv_cells = 1.0f / (float)cd[d];
                /* node j of cell k: (k + (1 + x_j) / 2) / cells of the extent */
                const float t0 = ((float)(i0 / c.q) + 0.5f * (1.0f + c.gl_x[i0 % c.q])) * inv_cells;
                const float t1 = ((float)(i1 / c.q) + 0.5f * (1.0f + c.gl_x[i1 % c.q])) * inv_cells;
                const float x0 = lo[d] + (hi[d] - lo[d]) * t0;
                const float x1 = lo[d] + (hi[d] - lo[d]) * t1;
                const float span = c.r.rmax[d] - c.r.rmin[d];
                ug[d] = (x0 - c.r.rmin[d]) / span;
                ug8[d] = (x1 - c.r.rmin[d]) / span;
                w0 *= 0.5f * c.gl_w[i0 % c.q] * inv_cells;
                w1 *= 0.5f * c.gl_w[i1 % c.q] * inv_cells;
            }
            Acts<D> a;
            features_tile<D>(ug, ug8, a.F);
            float out[2];
            forward_tile<D>(P, a, out);
            if ((lane & 3) == 0) acc += (n0 < nodes ? (double)(w0 * out[0]) : 0.0) + (n1 < nodes ? (double)(w1 * out[1]) : 0.0);
        }
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) integral[bin] = (float)acc; /* mean of g over the bin */
    }
}

/* ---------------------------------------------------------------- residual */
struct ResidualCfg {
    BinCfg b;
    uint64_t spp;
    uint32_t k0, k1;
    int32_t fallback;
    float factor; /* prod(res) */
};

template <class F, int D>
__global__ void __launch_bounds__(FWD_WARPS * 32)
    k_mlp_residual(const __grid_constant__ F f, const ResidualCfg c, const char* __restrict__ packed,
                   const float* __restrict__ integral, float* __restrict__ bins, uint32_t* __restrict__ fallback_count,
                   uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) char smem[];
    load_params<D>(smem, packed, false);
    const SmemParams<D> P = smem_params<D>(smem, false);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2;
    for (uint64_t bin = (uint64_t)blockIdx.x * FWD_WARPS + warp; bin < c.b.nbins;
         bin += (uint64_t)gridDim.x * FWD_WARPS) {
        float lo[D], hi[D];
        bin_box<D>(c.b, bin, lo, hi);
        float vol = 1.0f;
        for (int d = 0; d < D; ++d) vol = vmul(vol, vsub(hi[d], lo[d]));
        /* per lane, in FP32: Welford means and squared deviations of f and of f - g; merged across
         * the lanes in FP32 too (Chan's pairwise formulas, one division per step): FP64 runs at a
         * small fraction of the FP32 rate, and the means are only summed into the estimate in FP64 */
        float wn = 0.0f, mf = 0.0f, m2f = 0.0f, mr = 0.0f, m2r = 0.0f;
        for (uint64_t base = 0; base < c.spp; base += 32) {
            const uint64_t s = base + lane;
            const bool valid = s < c.spp;
            float u[D], x[F::DIM];
            for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
#pragma unroll
            for (int blk = 0; blk < (D + 3) / 4; ++blk) {
                const U4 r = philox4x32_10(U4{(uint32_t)s, (uint32_t)bin, (uint32_t)(bin >> 32), 0x5E5D0000u + blk},
                                           c.k0, c.k1);
                const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int d = blk * 4 + k;
                    if (d < D) x[d] = vadd(vmul(u01(rr[k]), vsub(hi[d], lo[d])), lo[d]);
                }
            }
            for (int d = 0; d < D; ++d) u[d] = (x[d] - c.b.r.rmin[d]) / (c.b.r.rmax[d] - c.b.r.rmin[d]);
            float fv[1];
            f(x, fv);
            /* g at the 32 points: two 16-point tiles */
            float gme = 0.0f;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                float ug[D], ug8[D];
                for (int d = 0; d < D; ++d) {
                    ug[d] = __shfl_sync(0xffffffffu, u[d], 16 * half + g);
                    ug8[d] = __shfl_sync(0xffffffffu, u[d], 16 * half + g + 8);
                }
                Acts<D> a;
                features_tile<D>(ug, ug8, a.F);
                float out[2];
                forward_tile<D>(P, a, out);
                /* point p = 16*half + r lives in lanes 4*(r%8).. as out[r/8] */
                const int r = lane - 16 * half;
                const float o0 = __shfl_sync(0xffffffffu, out[0], 4 * (lane & 7));
                const float o1 = __shfl_sync(0xffffffffu, out[1], 4 * (lane & 7));
                if (r >= 0 && r < 16) gme = (r < 8) ? o0 : o1;
            }
            if (valid) {
                const float rv = vsub(fv[0], gme);
                wn = vadd(wn, 1.0f);
                const float inv = vdiv(1.0f, wn);
                const float df = vsub(fv[0], mf);
                mf = vfma(df, inv, mf);
                m2f = vfma(df, vsub(fv[0], mf), m2f);
                const float dr = vsub(rv, mr);
                mr = vfma(dr, inv, mr);
                m2r = vfma(dr, vsub(rv, mr), m2r);
            }
        }
        float n_a = wn, mf_a = mf, m2f_a = m2f, mr_a = mr, m2r_a = m2r;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float n_b = __shfl_xor_sync(0xffffffffu, n_a, o);
            const float mf_b = __shfl_xor_sync(0xffffffffu, mf_a, o);
            const float m2f_b = __shfl_xor_sync(0xffffffffu, m2f_a, o);
            const float mr_b = __shfl_xor_sync(0xffffffffu, mr_a, o);
            const float m2r_b = __shfl_xor_sync(0xffffffffu, m2r_a, o);
            const float nt = vadd(n_a, n_b);
            if (nt > 0.0f) {
                const float r = vdiv(n_b, nt);
                const float w = vmul(n_a, r), df = vsub(mf_b, mf_a), dr = vsub(mr_b, mr_a);
                mf_a = vfma(df, r, mf_a);
                mr_a = vfma(dr, r, mr_a);
                m2f_a = vadd(m2f_a, vfma(vmul(df, df), w, m2f_b));
                m2r_a = vadd(m2r_a, vfma(vmul(dr, dr), w, m2r_b));
                n_a = nt;
            }
        }
        if (lane == 0) {
            const double scale = (double)c.factor * (double)vol;
            const double est_cv = scale * ((double)integral[bin] + (double)mr_a);
            const double est_mc = scale * (double)mf_a;
            const double var_r = n_a > 0.0f ? (double)m2r_a / n_a : 0.0, var_f = n_a > 0.0f ? (double)m2f_a / n_a : 0.0;
            const bool use_mc = c.fallback && var_f < var_r;
            const float o = (float)(use_mc ? est_mc : est_cv);
            bins[bin] = o;
            if (use_mc) atomicAdd(fallback_count, 1u);
            if (isnan(o)) atomicOr(status, VCU_FLAG_NAN);
        }
    }
}

}  // namespace mlp
}  // namespace vcu

/* ------------------------------------------------------------------------------------ host side */
namespace vcu {
namespace mlp {

constexpr float kGLx[4][4] = {{0.0f, 0.0f, 0.0f, 0.0f},
                              {-0.5773502691896258f, 0.5773502691896258f, 0.0f, 0.0f},
                              {-0.7745966692414834f, 0.0f, 0.7745966692414834f, 0.0f},
                              {-0.8611363115940526f, -0.3399810435848563f, 0.3399810435848563f, 0.8611363115940526f}};
constexpr float kGLw[4][4] = {{2.0f, 0.0f, 0.0f, 0.0f},
                              {1.0f, 1.0f, 0.0f, 0.0f},
                              {0.5555555555555556f, 0.8888888888888888f, 0.5555555555555556f, 0.0f},
                              {0.3478548451374538f, 0.6521451548625461f, 0.6521451548625461f, 0.3478548451374538f}};

/* He-uniform initial weights from a SplitMix64 stream, zero biases */
inline void init_params(int d, uint64_t seed, float* theta) {
    uint64_t s = seed ^ 0x243F6A8885A308D3ull;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int i = 0; i < n_params(d); ++i) theta[i] = 0.0f;
    for (int l = 0; l < 4; ++l) {
        const int in = layer_in(l, d);
        const double lim = std::sqrt(6.0 / in);
        for (int i = 0; i < in * WIDTH; ++i) theta[w_off(l, d) + i] = (float)((2.0 * next() - 1.0) * lim);
    }
    const double lim = std::sqrt(6.0 / WIDTH);
    for (int i = 0; i < WIDTH; ++i) theta[w4_off(d) + i] = (float)((2.0 * next() - 1.0) * lim);
}

struct State {
    float *theta, *m, *v, *grad, *partial;
    char* packed;
    uint32_t* step;
    float* integral;
    uint32_t* fallback;
};

template <int D> int alloc_state(vcu_ctx* ctx, uint64_t nbins, uint64_t nparts, State& s) {
    const size_t np = n_params(D), ng = np; /* gradient vector has one entry per parameter */
    size_t o = 0;
    auto a = [&](size_t bytes) {
        const size_t at = o;
        o = (o + bytes + 255) & ~size_t(255);
        return at;
    };
    const size_t o_theta = a(np * 4), o_m = a(np * 4), o_v = a(np * 4), o_g = a(ng * 4), o_p = a(pack_bytes(D)),
                 o_s = a(64), o_i = a(nbins * 4), o_f = a(64), o_pt = a(nparts * ng * 4);
    int rc = ensure(ctx, ctx->scratch, o);
    if (rc) return rc;
    char* b = static_cast<char*>(ctx->scratch.ptr);
    s.theta = reinterpret_cast<float*>(b + o_theta);
    s.m = reinterpret_cast<float*>(b + o_m);
    s.v = reinterpret_cast<float*>(b + o_v);
    s.grad = reinterpret_cast<float*>(b + o_g);
    s.partial = reinterpret_cast<float*>(b + o_pt);
    s.packed = b + o_p;
    s.step = reinterpret_cast<uint32_t*>(b + o_s);
    s.integral = reinterpret_cast<float*>(b + o_i);
    s.fallback = reinterpret_cast<uint32_t*>(b + o_f);
    return VCU_OK;
}

template <int D> int upload_params(vcu_ctx* ctx, const State& s, const float* theta_host, uint32_t& launches) {
    const size_t np = n_params(D);
    VCU_CUDA(ctx, cudaMemcpyAsync(s.theta, theta_host, np * 4, cudaMemcpyHostToDevice, ctx->stream));
    VCU_CUDA(ctx, cudaMemsetAsync(s.m, 0, np * 4, ctx->stream));
    VCU_CUDA(ctx, cudaMemsetAsync(s.v, 0, np * 4, ctx->stream));
    VCU_CUDA(ctx, cudaMemsetAsync(s.grad, 0, np * 4, ctx->stream));
    VCU_CUDA(ctx, cudaMemsetAsync(s.packed, 0, pack_bytes(D), ctx->stream));
    VCU_CUDA(ctx, cudaMemsetAsync(s.step, 0, 64, ctx->stream));
    k_mlp_pack<D><<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(s.theta, s.packed);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());
    return VCU_OK;
}

template <int D> int set_smem_train(vcu_ctx* ctx) {
    const int tb = train_smem_bytes<D>();
    if ((size_t)tb > ctx->smem_optin) return fail(ctx, VCU_UNSUPPORTED, "training block does not fit in shared memory");
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_train<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, tb));
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_integral<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       smem_fwd_bytes<D>()));
    return VCU_OK;
}

template <class F, int D>
int learned(vcu_ctx* ctx, const F& f, const vcu_problem* p, const BinGrid& g, const vcu_learned& opt, float* d_bins,
            float* d_integral, vcu_learned_report* report, uint32_t& launches) {
    /* training grid: at most one block per SM, each doing `rounds` rounds of ROUND points */
    const uint64_t want = ((uint64_t)(opt.batch > 0 ? opt.batch : 1) + ROUND - 1) / ROUND;
    const unsigned train_blocks = (unsigned)(want < (uint64_t)ctx->sm_count ? want : (uint64_t)ctx->sm_count);
    State s;
    int rc = alloc_state<D>(ctx, g.nbins, train_blocks, s);
    if (rc) return rc;
    if ((rc = set_smem_train<D>(ctx))) return rc;
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_residual<F, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       smem_fwd_bytes<D>()));
    std::vector<float> theta(n_params(D));
    init_params(D, opt.seed, theta.data());
    if ((rc = upload_params<D>(ctx, s, theta.data(), launches))) return rc;
    /* 1. training: one graph of (train, adam, step) replayed train_steps times */
    TrainCfg tc{};
    for (int d = 0; d < D; ++d) {
        tc.r.rmin[d] = p->range_min[d];
        tc.r.rmax[d] = p->range_max[d];
    }
    tc.k0 = (uint32_t)(opt.seed * 0x9E3779B97F4A7C15ull >> 32);
    tc.k1 = (uint32_t)(opt.seed >> 32) ^ 0x51ED270Bu;
    tc.rounds = (uint32_t)((want + train_blocks - 1) / train_blocks);
    const uint64_t batch = (uint64_t)tc.rounds * train_blocks * ROUND;
    tc.scale = (float)(2.0 / (double)batch);
    /* the step's training points live in the context's input buffer */
    if ((rc = ensure(ctx, ctx->in, batch * (D + 1) * 4 + 1024))) return rc;
    float* su = static_cast<float*>(ctx->in.ptr);
    float* sy = su + batch * D;
    tc.u_in = su;
    tc.y_in = sy;
    tc.npts = batch;
    AdamCfg ac{opt.learning_rate, 0.9f, 0.999f, 1e-8f, n_params(D), (int)train_blocks};
    cudaEvent_t e0 = ctx->ev_tune[0], e1 = ctx->ev_tune[1];
    VCU_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    if (opt.train_steps > 0) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        VCU_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        k_mlp_samples<F, D><<<(unsigned)((batch + 255) / 256), 256, 0, ctx->stream>>>(f, tc, batch, su, sy, s.step);
        k_mlp_train<D><<<train_blocks, TRAIN_WARPS * 32, train_smem_bytes<D>(), ctx->stream>>>(tc, s.packed,
                                                                                                s.partial);
        k_mlp_adam<D><<<(unsigned)((n_params(D) + 255) / 256), 256, 0, ctx->stream>>>(ac, s.theta, s.m, s.v, s.partial,
                                                                                       s.step, s.packed);
        k_mlp_step_inc<<<1, 1, 0, ctx->stream>>>(s.step);
        const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        if (ie != cudaSuccess) {
            cudaGraphDestroy(graph);
            return cuda_fail(ctx, ie, "cudaGraphInstantiate");
        }
        for (uint32_t i = 0; i < opt.train_steps; ++i) {
            const cudaError_t le = cudaGraphLaunch(exec, ctx->stream);
            if (le != cudaSuccess) {
                cudaGraphExecDestroy(exec);
                cudaGraphDestroy(graph);
                return cuda_fail(ctx, le, "cudaGraphLaunch");
            }
        }
        launches += 4 * opt.train_steps;
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
    }
    VCU_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    float train_ms = 0.0f;
    VCU_CUDA(ctx, cudaEventSynchronize(e1));
    VCU_CUDA(ctx, cudaEventElapsedTime(&train_ms, e0, e1));
    /* 2. per-bin integral of g */
    BinCfg bc{};
    for (int d = 0; d < D; ++d) {
        bc.r.rmin[d] = p->range_min[d];
        bc.r.rmax[d] = p->range_max[d];
    }
    for (int d = 0; d < p->dimbins; ++d) {
        bc.drange[d] = g.drange[d];
        bc.res[d] = g.res[d];
    }
    bc.dimbins = p->dimbins;
    bc.nbins = g.nbins;
    bc.q = (int)opt.quad_nodes;
    bc.cells = opt.quad_cells > 1 ? opt.quad_cells : 1;
    bc.cells_unbinned = opt.quad_cells_unbinned > 0 ? opt.quad_cells_unbinned : bc.cells;
    for (int i = 0; i < 4; ++i) {
        bc.gl_x[i] = kGLx[bc.q - 1][i];
        bc.gl_w[i] = kGLw[bc.q - 1][i];
    }
    int per_sm = 0;
    VCU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlp_integral<D>, FWD_WARPS * 32,
                                                                smem_fwd_bytes<D>()));
    const uint64_t need = (g.nbins + FWD_WARPS - 1) / FWD_WARPS;
    const uint64_t cap = (uint64_t)ctx->sm_count * (per_sm > 0 ? per_sm : 1) * 4;
    const unsigned blocks = (unsigned)(need < cap ? need : cap);
    float* integral = d_integral ? d_integral : s.integral;
    VCU_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    k_mlp_integral<D><<<blocks, FWD_WARPS * 32, smem_fwd_bytes<D>(), ctx->stream>>>(bc, s.packed, integral);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());
    VCU_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    float integral_ms = 0.0f;
    VCU_CUDA(ctx, cudaEventSynchronize(e1));
    VCU_CUDA(ctx, cudaEventElapsedTime(&integral_ms, e0, e1));
    /* 3. residual */
    ResidualCfg rcfg{};
    rcfg.b = bc;
    rcfg.spp = opt.samples_per_bin;
    rcfg.k0 = (uint32_t)opt.seed;
    rcfg.k1 = (uint32_t)(opt.seed >> 32);
    rcfg.fallback = opt.fallback;
    rcfg.factor = g.factor;
    VCU_CUDA(ctx, cudaMemsetAsync(s.fallback, 0, 4, ctx->stream));
    VCU_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    k_mlp_residual<F, D><<<blocks, FWD_WARPS * 32, smem_fwd_bytes<D>(), ctx->stream>>>(f, rcfg, s.packed, integral,
                                                                                        d_bins, s.fallback,
                                                                                        ctx->d_status);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());
    VCU_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    float residual_ms = 0.0f;
    VCU_CUDA(ctx, cudaEventSynchronize(e1));
    VCU_CUDA(ctx, cudaEventElapsedTime(&residual_ms, e0, e1));
    if (opt.theta_out)
        VCU_CUDA(ctx, cudaMemcpyAsync(opt.theta_out, s.theta, n_params(D) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (report) {
        uint32_t fb = 0;
        VCU_CUDA(ctx, cudaMemcpy(&fb, s.fallback, 4, cudaMemcpyDeviceToHost));
        report->fallback_bins = fb;
        report->train_ms = train_ms;
        report->integral_ms = integral_ms;
        report->residual_ms = residual_ms;
    }
    return VCU_OK;
}

/* forward (and gradient) of given points with given parameters: the gradient check */
template <int D>
int eval_grad(vcu_ctx* ctx, const float* theta, const float* u, const float* y, int64_t npts, float* out, float* grad,
              uint32_t& launches) {
    const unsigned blocks = (unsigned)((npts + ROUND - 1) / ROUND);
    State s;
    int rc = alloc_state<D>(ctx, 1, blocks, s);
    if (rc) return rc;
    if ((rc = set_smem_train<D>(ctx))) return rc;
    if ((rc = upload_params<D>(ctx, s, theta, launches))) return rc;
    const size_t in_bytes = (size_t)npts * (D + 2) * 4;
    if ((rc = ensure(ctx, ctx->in, in_bytes + 1024))) return rc;
    float* du = static_cast<float*>(ctx->in.ptr);
    float* dy = du + (size_t)npts * D;
    float* dout = dy + npts;
    VCU_CUDA(ctx, cudaMemcpyAsync(du, u, (size_t)npts * D * 4, cudaMemcpyHostToDevice, ctx->stream));
    if (y) VCU_CUDA(ctx, cudaMemcpyAsync(dy, y, (size_t)npts * 4, cudaMemcpyHostToDevice, ctx->stream));
    else VCU_CUDA(ctx, cudaMemsetAsync(dy, 0, (size_t)npts * 4, ctx->stream));
    TrainCfg tc{};
    tc.rounds = 1;
    tc.u_in = du;
    tc.y_in = dy;
    tc.out = dout;
    tc.npts = (uint64_t)npts;
    tc.scale = (float)(2.0 / (double)npts);
    k_mlp_train<D><<<blocks, TRAIN_WARPS * 32, train_smem_bytes<D>(), ctx->stream>>>(tc, s.packed, s.partial);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());
    k_mlp_reduce<D><<<(unsigned)((n_params(D) + 255) / 256), 256, 0, ctx->stream>>>(s.partial, (int)blocks, s.grad);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());
    VCU_CUDA(ctx, cudaMemcpyAsync(out, dout, (size_t)npts * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (grad) {
        /* the kernel's gradient vector follows its own order (W0..W3, b0..b3, w4, b4): map to parameters */
        std::vector<float> gk(n_params(D));
        VCU_CUDA(ctx, cudaMemcpyAsync(gk.data(), s.grad, gk.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
        VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int a = fin(D) * WIDTH, hid = WIDTH * WIDTH;
        for (int i = 0; i < n_params(D); ++i) {
            int pidx;
            if (i < a) pidx = w_off(0, D) + i;
            else if (i < a + 3 * hid) pidx = w_off(1 + (i - a) / hid, D) + (i - a) % hid;
            else if (i < a + 3 * hid + 4 * WIDTH) pidx = b_off((i - a - 3 * hid) / WIDTH, D) + (i - a - 3 * hid) % WIDTH;
            else pidx = w4_off(D) + (i - a - 3 * hid - 4 * WIDTH);
            grad[pidx] = gk[i];
        }
    }
    return VCU_OK;
}

}  // namespace mlp

int run_learned(vcu_ctx* ctx, const vcu_problem* p, const BinGrid& g, const vcu_learned& opt, float* d_bins,
                float* d_integral, vcu_learned_report* report, uint32_t& launches) {
    return with_integrand(ctx, p->f, p->dim, [&](const auto& f) -> int {
        using F = std::decay_t<decltype(f)>;
        if constexpr (F::CH != 1) {
            return fail(ctx, VCU_UNSUPPORTED, "the learned control variate is built for scalar integrands");
        } else if constexpr (F::DIM == 6) {
            switch (p->dim) {
            case 2: return mlp::learned<F, 2>(ctx, f, p, g, opt, d_bins, d_integral, report, launches);
            case 3: return mlp::learned<F, 3>(ctx, f, p, g, opt, d_bins, d_integral, report, launches);
            case 5: return mlp::learned<F, 5>(ctx, f, p, g, opt, d_bins, d_integral, report, launches);
            default: return fail(ctx, VCU_UNSUPPORTED, "the learned control variate is built for 2, 3 and 5 dimensions");
            }
        } else if constexpr (F::DIM == 2 || F::DIM == 3 || F::DIM == 5) {
            return mlp::learned<F, F::DIM>(ctx, f, p, g, opt, d_bins, d_integral, report, launches);
        } else {
            return fail(ctx, VCU_UNSUPPORTED, "the learned control variate is built for 2, 3 and 5 dimensions");
        }
    });
}

int run_mlp_eval(vcu_ctx* ctx, int dim, const float* theta, const float* u, const float* y, int64_t npts, float* out,
                 float* grad, uint32_t& launches) {
    switch (dim) {
    case 2: return mlp::eval_grad<2>(ctx, theta, u, y, npts, out, grad, launches);
    case 3: return mlp::eval_grad<3>(ctx, theta, u, y, npts, out, grad, launches);
    case 5: return mlp::eval_grad<5>(ctx, theta, u, y, npts, out, grad, launches);
    default: return fail(ctx, VCU_UNSUPPORTED, "network dimension must be 2, 3 or 5");
    }
}

}  // namespace vcu
