/*
 * k_mlp.cu -- learned control variate: online training, the network's interpolant per bin, residual.
 *
 * No reference counterpart (the task's learned part; the per-bin wrapper it plugs into is
 * src/integrator-per-bin-parallel.h:17-35).  Pipeline of vcu_learned_control_variates:
 *  1. train: Adam steps on fresh samples of the integrand (Philox points over the range, the
 *     integrand evaluated by the device) minimising mean (g - f)^2; each step is one sampling
 *     kernel, one fused forward+backward kernel (k_mlp_train: every block writes its own partial
 *     gradient, no atomics), one Adam kernel that sums the partials in a fixed order and rewrites
 *     the BF16 image of the weights, and one counter kernel -- captured once in a CUDA graph and
 *     replayed; every `check_every` steps the mean squared error on a fixed held-out set is summed
 *     per block (k_mlp_heldout) and added in block order on the host, and training stops once it
 *     no longer improves;
 *  2. k_mlp_nodes: the network at the Simpson nodes of every bin's grid (tensor cores, 16-point
 *     tiles), a chunk of bins at a time;
 *  3. k_mlp_cv: per bin, the interpolant h of those node values (piecewise quadratic, Lagrange on
 *     the three nodes of a cell per dimension; constant in a dimension with one node) is the
 *     control variate: its mean over the bin is the composite Simpson sum of the nodes -- exact, so
 *     integral(h) + mean(f - h) over the residual samples is unbiased.  Optionally, separate pilot
 *     samples per bin give the bin's weight alpha = cov(f, h) / var(h) (estimate alpha integral(h) +
 *     mean(f - alpha h); alpha 0 is plain Monte Carlo) and choose a given polynomial control
 *     variate's estimate where its variance is lower.
 */
#include <algorithm>

#include "k_mlp.cuh"
#include "k_mlp_tc.cuh"

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
    const float t = (float)(step_ctr[0] + 1);
    const float lr = c.lr * __uint_as_float(step_ctr[2]); /* step_ctr[2]: the learning-rate scale */
    const float mi = c.b1 * m[p] + (1.0f - c.b1) * gr;
    const float vi = c.b2 * v[p] + (1.0f - c.b2) * gr * gr;
    m[p] = mi;
    v[p] = vi;
    const float mh = mi / (1.0f - powf(c.b1, t));
    const float vh = vi / (1.0f - powf(c.b2, t));
    const float w = theta[p] - lr * mh / (sqrtf(vh) + c.eps);
    theta[p] = w;
    pack_param<D>(packed, p, w);
}

__global__ void k_mlp_step_inc(uint32_t* step_ctr) { *step_ctr += 1u; }

template <int D> __global__ void k_mlp_pack(const float* __restrict__ theta, char* __restrict__ packed) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n_params(D)) pack_param<D>(packed, p, theta[p]);
}

/* ---------------------------------------------------------------- held-out loss */
/* per block: the sum of (g - y)^2 over its points of the held-out set, FP64 in a fixed order */
template <int D>
__global__ void __launch_bounds__(FWD_WARPS * 32)
    k_mlp_heldout(const char* __restrict__ packed, const float* __restrict__ u, const float* __restrict__ y,
                  uint64_t npts, double* __restrict__ partial) {
    extern __shared__ __align__(16) char smem[];
    __shared__ double wsum[FWD_WARPS];
    load_params<D>(smem, packed, false);
    const SmemParams<D> P = smem_params<D>(smem, false);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2;
    double acc = 0.0;
    const uint64_t tiles = (npts + 15) / 16;
    for (uint64_t tile = (uint64_t)blockIdx.x * FWD_WARPS + warp; tile < tiles; tile += (uint64_t)gridDim.x * FWD_WARPS) {
        const uint64_t s0 = tile * 16 + g, s1 = s0 + 8;
        float ug[D], ug8[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            ug[d] = s0 < npts ? u[s0 * D + d] : 0.5f;
            ug8[d] = s1 < npts ? u[s1 * D + d] : 0.5f;
        }
        Acts<D> a;
        features_tile<D>(ug, ug8, a.F);
        float out[2];
        forward_tile<D>(P, a, out);
        if ((lane & 3) == 0) {
            if (s0 < npts) acc += (double)(out[0] - y[s0]) * (double)(out[0] - y[s0]);
            if (s1 < npts) acc += (double)(out[1] - y[s1]) * (double)(out[1] - y[s1]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) wsum[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < FWD_WARPS; ++w) t += wsum[w];
        partial[blockIdx.x] = t;
    }
}

/* ---------------------------------------------------------------- the interpolation grid */
/* Per dimension the grid has n[d] = 2 cells + 1 Simpson nodes (or one node, at the bin centre, for
 * a binned dimension with no cells); the nodes of a bin are numbered dimension 0 fastest. */
struct GridCfg {
    RangeCfg r;
    float drange[VCU_MAX_DIMBINS];
    uint32_t res[VCU_MAX_DIMBINS];
    int32_t dimbins;
    uint64_t nbins;
    int32_t n[VCU_MAX_DIM]; /* nodes per dimension */
    int32_t npb;            /* nodes per bin        */
};

/* lower/upper corner of the box the grid spans in each dimension: the bin in binned dimensions,
 * the range in the others */
template <int D>
__device__ __forceinline__ void grid_box(const GridCfg& c, uint64_t bin, float* lo, float* hi) {
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

/* the network at every grid node of bins [bin0, bin0 + count): out[(bin - bin0) * npb + node] */
template <int D>
__global__ void __launch_bounds__(FWD_WARPS * 32)
    k_mlp_nodes(const GridCfg c, const char* __restrict__ packed, uint64_t bin0, uint64_t count,
                float* __restrict__ out) {
    extern __shared__ __align__(16) char smem[];
    load_params<D>(smem, packed, false);
    const SmemParams<D> P = smem_params<D>(smem, false);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2;
    const uint64_t tiles_per_bin = (uint64_t)(c.npb + 15) / 16, tiles = count * tiles_per_bin;
    for (uint64_t tile = (uint64_t)blockIdx.x * FWD_WARPS + warp; tile < tiles; tile += (uint64_t)gridDim.x * FWD_WARPS) {
        const uint64_t lb = tile / tiles_per_bin;
        const int n0 = (int)(tile % tiles_per_bin) * 16 + g, n1 = n0 + 8;
        float lo[D], hi[D];
        grid_box<D>(c, bin0 + lb, lo, hi);
        float ug[D], ug8[D];
        int r0 = n0 < c.npb ? n0 : 0, r1 = n1 < c.npb ? n1 : 0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int i0 = r0 % c.n[d], i1 = r1 % c.n[d];
            r0 /= c.n[d];
            r1 /= c.n[d];
            /* node i of n: lo + (hi - lo) * i / (n - 1); the centre when n == 1 */
            const float t0 = c.n[d] == 1 ? 0.5f : (float)i0 / (float)(c.n[d] - 1);
            const float t1 = c.n[d] == 1 ? 0.5f : (float)i1 / (float)(c.n[d] - 1);
            const float span = c.r.rmax[d] - c.r.rmin[d];
            ug[d] = (lo[d] + (hi[d] - lo[d]) * t0 - c.r.rmin[d]) / span;
            ug8[d] = (lo[d] + (hi[d] - lo[d]) * t1 - c.r.rmin[d]) / span;
        }
        Acts<D> a;
        features_tile<D>(ug, ug8, a.F);
        float o[2];
        forward_tile<D>(P, a, o);
        if ((lane & 3) == 0) {
            float* dst = out + lb * (uint64_t)c.npb;
            if (n0 < c.npb) dst[n0] = o[0];
            if (n1 < c.npb) dst[n1] = o[1];
        }
    }
}

/* the same on the 5th-generation tensor cores (k_mlp_tc.cuh): one warpgroup per CTA, 128 nodes per
 * tile, persistent over the chunk's nodes */
template <int D>
__global__ void __launch_bounds__(tc::THREADS)
    k_mlp_nodes_tc(const GridCfg c, const char* __restrict__ packed, uint64_t bin0, uint64_t count,
                   float* __restrict__ out, uint32_t* __restrict__ status) {
    auto point = [&](uint64_t i, float* u) -> bool {
        const uint64_t lb = i / (uint64_t)c.npb;
        int r = (int)(i % (uint64_t)c.npb);
        float lo[D], hi[D];
        grid_box<D>(c, bin0 + lb, lo, hi);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int j = r % c.n[d];
            r /= c.n[d];
            const float tt = c.n[d] == 1 ? 0.5f : (float)j / (float)(c.n[d] - 1);
            u[d] = (lo[d] + (hi[d] - lo[d]) * tt - c.r.rmin[d]) / (c.r.rmax[d] - c.r.rmin[d]);
        }
        return true;
    };
    tc::forward_points<D>(packed, count * (uint64_t)c.npb, point, out, status);
}

/* the network at explicit points u[n][D] (vcu_mlp_eval without a gradient), tensor cores */
template <int D>
__global__ void __launch_bounds__(tc::THREADS)
    k_mlp_forward_tc(const char* __restrict__ packed, const float* __restrict__ u_in, uint64_t n,
                     float* __restrict__ out, uint32_t* __restrict__ status) {
    auto point = [&](uint64_t i, float* u) -> bool {
#pragma unroll
        for (int d = 0; d < D; ++d) u[d] = u_in[i * D + d];
        return true;
    };
    tc::forward_points<D>(packed, n, point, out, status);
}

/* ---------------------------------------------------------------- residual */
struct CvCfg {
    GridCfg gr;
    uint64_t spp, pilot;
    uint32_t k0, k1;
    int32_t fallback;
    float factor; /* prod(res) */
    const float* poly_bins;
    const float* poly_var;
};

/* weight of node j (of n) in the composite Simpson mean over [0,1] with (n-1)/2 cells */
__device__ __forceinline__ float simpson_weight(int j, int n) {
    if (n == 1) return 1.0f;
    const float cells = 0.5f * (float)(n - 1);
    const float w = (j == 0 || j == n - 1) ? 1.0f : ((j & 1) ? 4.0f : 2.0f);
    return w / (6.0f * cells);
}

/* sum over the nodes of the point's cell of weight x node value, one dimension per level: a
 * dimension contributes 3 nodes (Lagrange weights w0..w2) or 1 (weight 1) */
template <int d, int D>
__device__ __forceinline__ float interp_level(const float* __restrict__ nodes, const int* off, const int* stride,
                                              const int* nw, const float (*w)[3], int idx, float wacc) {
    if constexpr (d == D) {
        return wacc * __ldg(nodes + idx);
    } else {
        float h = interp_level<d + 1, D>(nodes, off, stride, nw, w, idx + off[d], wacc * w[d][0]);
        if (nw[d] == 3) {
            h += interp_level<d + 1, D>(nodes, off, stride, nw, w, idx + off[d] + stride[d], wacc * w[d][1]);
            h += interp_level<d + 1, D>(nodes, off, stride, nw, w, idx + off[d] + 2 * stride[d], wacc * w[d][2]);
        }
        return h;
    }
}

/* h at a point (normalised coordinates t in [0,1] per dimension of the grid box): Lagrange
 * interpolation on the three nodes of the point's cell in each dimension with cells */
template <int D>
__device__ __forceinline__ float interpolant(const GridCfg& c, const float* __restrict__ nodes, const float* t) {
    int off[D], stride[D], nw[D];
    float w[D][3];
    int st = 1;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        stride[d] = st;
        if (c.n[d] == 1) {
            off[d] = 0;
            nw[d] = 1;
            w[d][0] = 1.0f;
            w[d][1] = w[d][2] = 0.0f;
        } else {
            const int cells = (c.n[d] - 1) >> 1;
            const float sc = t[d] * (float)cells;
            int k = (int)sc;
            k = k < 0 ? 0 : (k > cells - 1 ? cells - 1 : k);
            const float s = sc - (float)k; /* in [0, 1] */
            off[d] = 2 * k * st;
            nw[d] = 3;
            w[d][0] = 2.0f * (s - 0.5f) * (s - 1.0f);
            w[d][1] = -4.0f * s * (s - 1.0f);
            w[d][2] = 2.0f * s * (s - 0.5f);
        }
        st *= c.n[d];
    }
    return interp_level<0, D>(nodes, off, stride, nw, w, 0, 1.0f);
}

/* Welford update of a (count, mean, M2) triple, FP32 */
__device__ __forceinline__ void welford(float& n, float& m, float& m2, float x) {
    n += 1.0f;
    const float dx = x - m;
    m = fmaf(dx, 1.0f / n, m);
    m2 = fmaf(dx, x - m, m2);
}
/* Chan's pairwise merge of two such triples across the lanes of a warp (xor shuffles) */
__device__ __forceinline__ void warp_merge(float& n, float& m, float& m2) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float nb = __shfl_xor_sync(0xffffffffu, n, o);
        const float mb = __shfl_xor_sync(0xffffffffu, m, o);
        const float m2b = __shfl_xor_sync(0xffffffffu, m2, o);
        const float nt = n + nb;
        if (nt > 0.0f) {
            const float r = nb / nt, dm = mb - m;
            m = fmaf(dm, r, m);
            m2 = m2 + m2b + dm * dm * n * r;
            n = nt;
        }
    }
}

/* one warp per bin of the chunk: mean of h by Simpson weights, optional pilot choice, residual */
template <class F, int D>
__global__ void __launch_bounds__(FWD_WARPS * 32)
    k_mlp_cv(const __grid_constant__ F f, const CvCfg c, uint64_t bin0, uint64_t count, const float* __restrict__ nodes,
             float* __restrict__ bins, float* __restrict__ integral, uint32_t* __restrict__ counters,
             uint32_t* __restrict__ status) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint64_t lb = (uint64_t)blockIdx.x * FWD_WARPS + warp; lb < count; lb += (uint64_t)gridDim.x * FWD_WARPS) {
        const uint64_t bin = bin0 + lb;
        const float* nd = nodes + lb * (uint64_t)c.gr.npb;
        float lo[D], hi[D];
        grid_box<D>(c.gr, bin, lo, hi);
        /* the grid box is the bin's integration box: the bin in binned dimensions, the range in the others */
        float vol = 1.0f;
        for (int d = 0; d < D; ++d) vol = vmul(vol, vsub(hi[d], lo[d]));
        /* mean of h over the box: composite Simpson weights of the nodes, FP32 lane sums (relative
         * rounding ~1e-7 of the mean, far below any sampling error; FP64 would occupy the scarce FP64
         * pipe) */
        float mhf = 0.0f;
        for (int k = lane; k < c.gr.npb; k += 32) {
            int r = k;
            float w = 1.0f;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                w *= simpson_weight(r % c.gr.n[d], c.gr.n[d]);
                r /= c.gr.n[d];
            }
            mhf = fmaf(w, __ldg(nd + k), mhf);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mhf += __shfl_xor_sync(0xffffffffu, mhf, o);
        const double mh = (double)mhf;
        const uint32_t blo = (uint32_t)bin, bhi = (uint32_t)(bin >> 32);
        /* samples of stream `tag`: f and r = f - h, Welford per lane */
        auto draw = [&](uint64_t s, uint32_t tag, float* x, float* t) {
            for (int d = 0; d < F::DIM; ++d) x[d] = 0.0f;
#pragma unroll
            for (int blk = 0; blk < (D + 3) / 4; ++blk) {
                const U4 rr4 = philox4x32_10(U4{(uint32_t)s, blo, bhi, tag + blk}, c.k0, c.k1);
                const uint32_t rr[4] = {rr4.x, rr4.y, rr4.z, rr4.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int d = blk * 4 + k;
                    if (d < D) {
                        const float u = u01(rr[k]);
                        x[d] = vadd(vmul(u, vsub(hi[d], lo[d])), lo[d]);
                        t[d] = u;
                    }
                }
            }
        };
        /* samples of stream `tag`, two per lane and round (the integrand's pair form where it has
         * one): Welford moments of f and of f - alpha h; the pilot (P) also those of h */
        /* the scene terms that can be non-zero over the bin's box of the first two coordinates */
        [[maybe_unused]] typename cull_box_of<F>::type cl{};
        if constexpr (has_pair_cull<F>::value && D >= 2) {
            float clo[F::DIM], chi[F::DIM];
            for (int d = 0; d < F::DIM; ++d) clo[d] = chi[d] = 0.0f;
            for (int d = 0; d < D; ++d) {
                clo[d] = lo[d];
                chi[d] = hi[d];
            }
            cl = f.cull_box(clo, chi);
        }
        auto run = [&](auto pilot, uint64_t n, uint32_t tag, float alpha, float* st) {
            constexpr bool P = decltype(pilot)::value;
            float cnt = 0.0f, mf = 0.0f, m2f = 0.0f, mr = 0.0f, m2r = 0.0f, mhs = 0.0f, m2h = 0.0f;
            auto add = [&](float fv, float hv) {
                cnt += 1.0f;
                const float inv = 1.0f / cnt;
                const float rv = fv - alpha * hv;
                const float df = fv - mf, dr = rv - mr;
                mf = fmaf(df, inv, mf);
                m2f = fmaf(df, fv - mf, m2f);
                mr = fmaf(dr, inv, mr);
                m2r = fmaf(dr, rv - mr, m2r);
                if constexpr (P) {
                    const float dh = hv - mhs;
                    mhs = fmaf(dh, inv, mhs);
                    m2h = fmaf(dh, hv - mhs, m2h);
                }
            };
            for (uint64_t s = lane; s < n; s += 64) {
                const bool two = s + 32 < n;
                float x0[F::DIM], x1[F::DIM], t0[D], t1[D], v0[1], v1[1];
                draw(s, tag, x0, t0);
                draw(two ? s + 32 : s, tag, x1, t1);
                if constexpr (has_pair_cull<F>::value && D >= 2) {
                    f.pair_culled(cl, x0, x1, v0, v1);
                } else if constexpr (has_pair<F>::value) {
                    f.pair(x0, x1, v0, v1);
                } else {
                    f(x0, v0);
                    f(x1, v1);
                }
                add(v0[0], interpolant<D>(c.gr, nd, t0));
                if (two) add(v1[0], interpolant<D>(c.gr, nd, t1));
            }
            float n1 = cnt, n2 = cnt, n3 = cnt;
            warp_merge(n1, mf, m2f);
            warp_merge(n2, mr, m2r);
            if constexpr (P) warp_merge(n3, mhs, m2h);
            st[0] = n1;
            st[1] = mf;
            st[2] = m2f;
            st[3] = mr;
            st[4] = m2r;
            st[5] = m2h;
        };
        /* 0: control variate with weight alpha (alpha 0: plain Monte Carlo), 2: polynomial */
        int choice = 0;
        float alpha = 1.0f;
        if (c.fallback) {
            /* pilot (samples of their own stream, not reused): alpha = cov(f, h) / var(h), the
             * variance-minimising weight, clamped to [0, 1.5]; fixed before the residual samples, so
             * the estimate stays unbiased */
            float ps[6];
            run(std::true_type{}, c.pilot, 0x91107000u, 1.0f, ps);
            const float m2f = ps[2], m2r1 = ps[4], m2h = ps[5]; /* sums of squares over the pilot */
            const float cov = 0.5f * (m2f + m2h - m2r1);
            alpha = m2h > 0.0f ? fminf(fmaxf(cov / m2h, 0.0f), 1.5f) : 0.0f;
            if (c.poly_bins) {
                /* variance of this bin's estimate from the pilot, scaled to bin values and to the
                 * residual samples, against the polynomial estimate's own */
                const float m2a = fmaxf(m2f - 2.0f * alpha * cov + alpha * alpha * m2h, 0.0f);
                const double scale = (double)c.factor * (double)vol;
                const double pv = ps[0] > 1.0f ? (double)m2a / (ps[0] - 1.0f) : INFINITY;
                const double v_mine = pv * scale * scale / (double)c.spp;
                if ((double)c.poly_var[bin] < v_mine) choice = 2;
            }
        }
        float ms[6];
        if (choice != 2) run(std::false_type{}, c.spp, 0x5E5D0000u, alpha, ms);
        if (lane == 0) {
            const double scale = (double)c.factor * (double)vol;
            float o;
            if (choice == 2) o = c.poly_bins[bin];
            else o = (float)(scale * ((double)alpha * mh + (double)ms[3]));
            bins[bin] = o;
            if (integral) integral[bin] = (float)mh;
            if (choice == 0 && alpha == 0.0f) atomicAdd(counters, 1u);
            if (choice == 2) atomicAdd(counters + 1, 1u);
            if (isnan(o)) atomicOr(status, VCU_FLAG_NAN);
        }
    }
}

}  // namespace mlp
}  // namespace vcu

/* ------------------------------------------------------------------------------------ host side */
namespace vcu {
namespace mlp {

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
    uint32_t* step;     /* [0]: Adam step counter; [1]: the held-out set's fixed counter; [2]: the
                         * learning-rate scale (float bits) */
    uint32_t* counters; /* [0]: plain Monte Carlo bins, [1]: polynomial control-variate bins */
    double* heldout;    /* per-block partial sums of the held-out squared error */
    float* nodes;       /* a chunk of bins' grid node values */
};

constexpr int HELDOUT_BLOCKS = 64;
constexpr uint64_t HELDOUT_POINTS = 16384;
constexpr size_t NODE_CHUNK_BYTES = size_t(1) << 30; /* grid values held at once */

template <int D> int alloc_state(vcu_ctx* ctx, uint64_t nparts, size_t node_floats, State& s) {
    const size_t np = n_params(D), ng = np; /* gradient vector has one entry per parameter */
    size_t o = 0;
    auto a = [&](size_t bytes) {
        const size_t at = o;
        o = (o + bytes + 255) & ~size_t(255);
        return at;
    };
    const size_t o_theta = a(np * 4), o_m = a(np * 4), o_v = a(np * 4), o_g = a(ng * 4), o_p = a(pack_bytes(D)),
                 o_s = a(64), o_c = a(64), o_h = a(HELDOUT_BLOCKS * 8), o_pt = a(nparts * ng * 4),
                 o_n = a(node_floats * 4);
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
    s.counters = reinterpret_cast<uint32_t*>(b + o_c);
    s.heldout = reinterpret_cast<double*>(b + o_h);
    s.nodes = reinterpret_cast<float*>(b + o_n);
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
    static const float one = 1.0f; /* the learning-rate scale starts at 1 */
    VCU_CUDA(ctx, cudaMemcpyAsync(s.step + 2, &one, 4, cudaMemcpyHostToDevice, ctx->stream));
    k_mlp_pack<D><<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(s.theta, s.packed);
    ++launches;
    VCU_CUDA(ctx, cudaGetLastError());
    return VCU_OK;
}

template <int D> int set_smem_train(vcu_ctx* ctx) {
    const int tb = train_smem_bytes<D>();
    if ((size_t)tb > ctx->smem_optin) return fail(ctx, VCU_UNSUPPORTED, "training block does not fit in shared memory");
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_train<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, tb));
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_nodes<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       smem_fwd_bytes<D>()));
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_heldout<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       smem_fwd_bytes<D>()));
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_nodes_tc<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::Smem<D>::BYTES));
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_forward_tc<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::Smem<D>::BYTES));
    /* all of the unified L1/shared storage as shared memory: 4 CTAs of ~57 KB per SM, so one CTA's
     * tensor-core work overlaps the others' feature and epilogue work */
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_nodes_tc<D>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    VCU_CUDA(ctx, cudaFuncSetAttribute(k_mlp_forward_tc<D>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    return VCU_OK;
}

template <class F, int D>
int learned(vcu_ctx* ctx, const F& f, const vcu_problem* p, const BinGrid& g, const vcu_learned& opt, float* d_bins,
            float* d_integral, vcu_learned_report* report, uint32_t& launches) {
    /* the interpolation grid */
    GridCfg gc{};
    for (int d = 0; d < D; ++d) {
        gc.r.rmin[d] = p->range_min[d];
        gc.r.rmax[d] = p->range_max[d];
        gc.n[d] = d < p->dimbins ? 2 * opt.cells + 1 : 2 * opt.cells_unbinned + 1;
    }
    for (int d = 0; d < p->dimbins; ++d) {
        gc.drange[d] = g.drange[d];
        gc.res[d] = g.res[d];
    }
    gc.dimbins = p->dimbins;
    gc.nbins = g.nbins;
    gc.npb = 1;
    for (int d = 0; d < D; ++d) gc.npb *= gc.n[d];
    uint64_t chunk = NODE_CHUNK_BYTES / (4ull * (uint64_t)gc.npb);
    if (chunk > g.nbins) chunk = g.nbins;
    if (chunk < 1) chunk = 1;
    /* training grid: at most one block per SM, each doing `rounds` rounds of ROUND points */
    const uint64_t want = ((uint64_t)(opt.batch > 0 ? opt.batch : 1) + ROUND - 1) / ROUND;
    const unsigned train_blocks = (unsigned)(want < (uint64_t)ctx->sm_count ? want : (uint64_t)ctx->sm_count);
    State s;
    int rc = alloc_state<D>(ctx, train_blocks, chunk * (uint64_t)gc.npb, s);
    if (rc) return rc;
    if ((rc = set_smem_train<D>(ctx))) return rc;
    std::vector<float> theta(n_params(D));
    init_params(D, opt.seed, theta.data());
    if ((rc = upload_params<D>(ctx, s, theta.data(), launches))) return rc;
    /* 1. training: one graph of (samples, train, adam, step) replayed; held-out checks between */
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
    /* the step's training points and the held-out set live in the context's input buffer */
    const bool early = opt.check_every > 0 && opt.train_steps > 0;
    const uint64_t hn = early ? HELDOUT_POINTS : 0;
    if ((rc = ensure(ctx, ctx->in, (batch + hn) * (D + 1) * 4 + 1024))) return rc;
    float* su = static_cast<float*>(ctx->in.ptr);
    float* sy = su + batch * D;
    float* hu = sy + batch;
    float* hy = hu + hn * D;
    tc.u_in = su;
    tc.y_in = sy;
    tc.npts = batch;
    AdamCfg ac{opt.learning_rate, 0.9f, 0.999f, 1e-8f, n_params(D), (int)train_blocks};
    cudaEvent_t e0 = ctx->ev_tune[0], e1 = ctx->ev_tune[1];
    VCU_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    uint32_t steps_run = 0;
    double heldout_mse = NAN;
    if (early) {
        /* the held-out set: its own Philox key and a fixed counter word (step[1] = 0xFFFFFFFF) */
        TrainCfg hc = tc;
        hc.k0 ^= 0xA5A5A5A5u;
        hc.k1 ^= 0x3C3C3C3Cu;
        VCU_CUDA(ctx, cudaMemsetAsync(s.step + 1, 0xFF, 4, ctx->stream));
        k_mlp_samples<F, D><<<(unsigned)((hn + 255) / 256), 256, 0, ctx->stream>>>(f, hc, hn, hu, hy, s.step + 1);
        ++launches;
        VCU_CUDA(ctx, cudaGetLastError());
    }
    auto heldout = [&](double& mse) -> int {
        k_mlp_heldout<D><<<HELDOUT_BLOCKS, FWD_WARPS * 32, smem_fwd_bytes<D>(), ctx->stream>>>(s.packed, hu, hy, hn,
                                                                                               s.heldout);
        ++launches;
        VCU_CUDA(ctx, cudaGetLastError());
        double part[HELDOUT_BLOCKS];
        VCU_CUDA(ctx, cudaMemcpyAsync(part, s.heldout, sizeof(part), cudaMemcpyDeviceToHost, ctx->stream));
        VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        double t = 0.0;
        for (int b = 0; b < HELDOUT_BLOCKS; ++b) t += part[b]; /* block order: deterministic */
        mse = t / (double)hn;
        return VCU_OK;
    };
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
        double best = INFINITY;
        int stale = 0, drops = 0;
        float lr_scale = 1.0f;
        while (steps_run < opt.train_steps) {
            const uint32_t n = early ? std::min(opt.check_every, opt.train_steps - steps_run) : opt.train_steps;
            for (uint32_t i = 0; i < n; ++i) {
                const cudaError_t le = cudaGraphLaunch(exec, ctx->stream);
                if (le != cudaSuccess) {
                    cudaGraphExecDestroy(exec);
                    cudaGraphDestroy(graph);
                    return cuda_fail(ctx, le, "cudaGraphLaunch");
                }
            }
            steps_run += n;
            launches += 4 * n;
            if (!early) break;
            double mse = 0.0;
            if ((rc = heldout(mse))) {
                cudaGraphExecDestroy(exec);
                cudaGraphDestroy(graph);
                return rc;
            }
            heldout_mse = mse;
            /* after two checks in a row without a 0.5 % improvement on the best, the learning rate
             * drops to 0.3 of itself; the third such plateau ends training */
            if (mse < best * 0.995) {
                best = mse;
                stale = 0;
            } else if (++stale >= 2) {
                if (drops == 2) break;
                ++drops;
                stale = 0;
                lr_scale *= 0.3f;
                VCU_CUDA(ctx, cudaMemcpyAsync(s.step + 2, &lr_scale, 4, cudaMemcpyHostToDevice, ctx->stream));
                VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream)); /* lr_scale is a host local */
            }
        }
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
    } else if (early) {
        if ((rc = heldout(heldout_mse))) return rc;
    }
    VCU_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    float train_ms = 0.0f;
    VCU_CUDA(ctx, cudaEventSynchronize(e1));
    VCU_CUDA(ctx, cudaEventElapsedTime(&train_ms, e0, e1));
    /* 2.-3. per chunk of bins: the network at the grid nodes, then the residual */
    CvCfg cc{};
    cc.gr = gc;
    cc.spp = opt.samples_per_bin;
    cc.pilot = learned_pilot(opt.samples_per_bin, opt.pilot);
    cc.k0 = (uint32_t)opt.seed;
    cc.k1 = (uint32_t)(opt.seed >> 32);
    cc.fallback = opt.fallback;
    cc.factor = g.factor;
    cc.poly_bins = opt.poly_bins;
    cc.poly_var = opt.poly_variance;
    /* persistent: CTAs_PER_SM CTAs per SM (the shared memory of 4 fits with the max-shared carveout; 4 x 64
     * TMEM columns of the 512); the occupancy query is not used here because it ignores the carveout
     * preference and answers 1 */
    const unsigned node_blocks = (unsigned)ctx->sm_count * tc::CTAS_PER_SM;
    int per_sm_cv = 0;
    VCU_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_cv, k_mlp_cv<F, D>, FWD_WARPS * 32, 0));
    VCU_CUDA(ctx, cudaMemsetAsync(s.counters, 0, 8, ctx->stream));
    float integral_ms = 0.0f, residual_ms = 0.0f;
    for (uint64_t b0 = 0; b0 < g.nbins; b0 += chunk) {
        const uint64_t cnt = std::min(chunk, g.nbins - b0);
        VCU_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        k_mlp_nodes_tc<D><<<node_blocks, tc::THREADS, tc::Smem<D>::BYTES, ctx->stream>>>(gc, s.packed, b0, cnt,
                                                                                          s.nodes, ctx->d_status);
        ++launches;
        VCU_CUDA(ctx, cudaGetLastError());
        VCU_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        VCU_CUDA(ctx, cudaEventSynchronize(e1));
        float ms = 0.0f;
        VCU_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        integral_ms += ms;
        const uint64_t need = (cnt + FWD_WARPS - 1) / FWD_WARPS;
        const uint64_t cap = (uint64_t)ctx->sm_count * (per_sm_cv > 0 ? per_sm_cv : 1) * 8;
        const unsigned blocks = (unsigned)(need < cap ? need : cap);
        VCU_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        k_mlp_cv<F, D><<<blocks, FWD_WARPS * 32, 0, ctx->stream>>>(f, cc, b0, cnt, s.nodes, d_bins, d_integral,
                                                                   s.counters, ctx->d_status);
        ++launches;
        VCU_CUDA(ctx, cudaGetLastError());
        VCU_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        VCU_CUDA(ctx, cudaEventSynchronize(e1));
        VCU_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        residual_ms += ms;
    }
    if (opt.theta_out)
        VCU_CUDA(ctx, cudaMemcpyAsync(opt.theta_out, s.theta, n_params(D) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    uint32_t cnts[2] = {0, 0};
    VCU_CUDA(ctx, cudaMemcpyAsync(cnts, s.counters, 8, cudaMemcpyDeviceToHost, ctx->stream));
    VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (report) {
        report->fallback_bins = cnts[0];
        report->polynomial_bins = cnts[1];
        report->train_ms = train_ms;
        report->integral_ms = integral_ms;
        report->residual_ms = residual_ms;
        report->heldout_mse = heldout_mse;
        report->train_steps_run = steps_run;
        report->nodes_per_bin = (uint32_t)gc.npb;
    }
    return VCU_OK;
}

/* forward (and gradient) of given points with given parameters: the gradient check */
template <int D>
int eval_grad(vcu_ctx* ctx, const float* theta, const float* u, const float* y, int64_t npts, float* out, float* grad,
              uint32_t& launches) {
    const unsigned blocks = (unsigned)((npts + ROUND - 1) / ROUND);
    State s;
    int rc = alloc_state<D>(ctx, blocks, 0, s);
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
    if (!grad) {
        const uint64_t tiles = ((uint64_t)npts + tc::TILE - 1) / tc::TILE;
        const uint64_t cap = (uint64_t)ctx->sm_count * tc::CTAS_PER_SM;
        k_mlp_forward_tc<D><<<(unsigned)(tiles < cap ? tiles : cap), tc::THREADS, tc::Smem<D>::BYTES, ctx->stream>>>(
            s.packed, du, (uint64_t)npts, dout, ctx->d_status);
        ++launches;
        VCU_CUDA(ctx, cudaGetLastError());
        VCU_CUDA(ctx, cudaMemcpyAsync(out, dout, (size_t)npts * 4, cudaMemcpyDeviceToHost, ctx->stream));
        return VCU_OK;
    }
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
