/*
 * k_mlp_tc.cuh -- the control-variate network's forward pass on the 5th-generation tensor cores
 * (tcgen05): the learned control variate's grid nodes and vcu_mlp_eval's outputs.
 *
 * One CTA = one warpgroup of 128 threads; a tile is 128 points, thread t owning row t.  Per layer
 * the layer input A (128 x K, BF16) sits in shared memory, the weights B (64 x K, BF16, one row per
 * output unit) too, both in the canonical no-swizzle K-major layout of tcgen05: 8-row x 16-byte
 * core matrices, the K-chunks of a row group adjacent (leading byte offset 128 B), the row groups
 * K/8 x 128 B apart (stride byte offset).  One elected thread issues K/16 tcgen05.mma (kind::f16,
 * BF16 x BF16 -> FP32, M = 128, N = 64) into a 64-column TMEM accumulator and commits them to an
 * mbarrier; every warp then reads its 32 TMEM lanes (= its 32 rows) with tcgen05.ld, adds the bias,
 * applies ReLU, rounds to BF16 and writes the row back as the next layer's A.  The 64 -> 1 output
 * layer is a dot product on the FP32 pipe.  Rounding points are those of the mma.sync kernels and
 * of oracle/mlp_ref.py: features and hidden activations to BF16, accumulation in FP32.
 *
 * Every mbarrier wait is bounded: on expiry the CTA sets VCU_FLAG_TIMEOUT, stops, and still frees
 * its TMEM columns.
 */
#pragma once
#include "k_mlp.cuh"

namespace vcu {
namespace mlp {
namespace tc {

constexpr int TILE = 128;    /* points per tile = M of the MMA */
constexpr int THREADS = 128; /* one warpgroup: thread t owns row t */
constexpr int TMEM_COLS = 64;
constexpr unsigned CTAS_PER_SM = 4; /* persistent grid: 4 x ~57 KB of shared memory, 4 x 64 TMEM columns */
constexpr int MMA_N = 64;

/* byte offset of element (row, k) of a row-major-by-K operand with K columns, in the canonical
 * no-swizzle K-major layout */
__host__ __device__ constexpr int core_off(int row, int k, int K) {
    return ((row >> 3) * (K >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}
/* shared-memory matrix descriptor: start address, leading byte offset (K direction), stride byte
 * offset (8-row groups), descriptor version 1, no swizzle */
__host__ __device__ constexpr uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
/* instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16 (bits 7-9,
 * 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28 */
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

/* shared memory of a CTA: B_0..B_3 (64 x K_l BF16), A (128 x max K BF16), FP32 bias[4][64], w4[64],
 * b4, then the mbarrier and the TMEM address slot */
template <int D> struct Smem {
    static constexpr int K0 = fin(D);
    static constexpr int KA = K0 > WIDTH ? K0 : WIDTH;
    static constexpr int B0 = 0;
    static constexpr int B1 = B0 + MMA_N * K0 * 2;
    static constexpr int B2 = B1 + MMA_N * WIDTH * 2;
    static constexpr int B3 = B2 + MMA_N * WIDTH * 2;
    static constexpr int A = B3 + MMA_N * WIDTH * 2;
    static constexpr int F32 = A + TILE * KA * 2;
    static constexpr int MBAR = F32 + (5 * WIDTH + 4) * 4;
    static constexpr int SLOT = MBAR + 8;
    static constexpr int FLAG = SLOT + 4;
    static constexpr int BYTES = FLAG + 4;
    static_assert(B1 % 16 == 0 && A % 16 == 0 && F32 % 16 == 0 && MBAR % 8 == 0, "operand alignment");
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}
/* bounded wait for the phase with parity `parity` of the mbarrier at `mbar` */
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
/* 32 consecutive FP32 columns of this warp's 32 TMEM lanes: v[j] = row (lane), column col + j */
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

/* The forward pass over the points a functor `point(i, u)` describes (i in [0, n): fills u[D] in
 * [0,1]^D and returns whether point i exists); the result of point i goes to out[i].  Persistent
 * over tiles of 128 points. */
template <int D, class Points>
__device__ __forceinline__ void forward_points(const char* __restrict__ packed, uint64_t n, const Points& point,
                                               float* __restrict__ out, uint32_t* __restrict__ status) {
    using L = Smem<D>;
    extern __shared__ __align__(128) char smem[];
    const int t = threadIdx.x, warp = t >> 5;
    /* weights into the canonical layout (the packed image holds T_l: [64][in + PAD], out-major) */
    {
        const __nv_bfloat16* bf = reinterpret_cast<const __nv_bfloat16*>(packed);
        for (int l = 0; l < 4; ++l) {
            const int K = layer_in(l, D);
            const int base = l == 0 ? L::B0 : (l == 1 ? L::B1 : (l == 2 ? L::B2 : L::B3));
            const __nv_bfloat16* T = bf + t_off(l, D);
            for (int idx = t; idx < MMA_N * K; idx += THREADS) {
                const int nrow = idx / K, k = idx % K;
                *reinterpret_cast<__nv_bfloat16*>(smem + base + core_off(nrow, k, K)) = T[nrow * (K + PAD) + k];
            }
        }
        const float* src = reinterpret_cast<const float*>(packed + fp32_off_bytes(D));
        float* f32 = reinterpret_cast<float*>(smem + L::F32);
        for (int i = t; i < 5 * WIDTH + 1; i += THREADS) f32[i] = src[i];
    }
    const uint32_t mbar = smem_u32(smem + L::MBAR), slot = smem_u32(smem + L::SLOT);
    volatile int* flag = reinterpret_cast<volatile int*>(smem + L::FLAG);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *flag = 0;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + L::SLOT);
    const float* bias = reinterpret_cast<const float*>(smem + L::F32);
    const float* w4 = bias + 4 * WIDTH;
    const float b4 = w4[WIDTH];
    char* A = smem + L::A;
    const uint32_t a_addr = smem_u32(A);
    const uint32_t idesc = instr_desc(TILE, MMA_N);
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16; /* TMEM address of this warp's lanes */
    uint32_t phase = 0;
    const uint64_t tiles = (n + TILE - 1) / TILE;
    bool ok = true;
    for (uint64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const uint64_t i = tile * TILE + (uint64_t)t;
        float u[D];
        const bool valid = i < n && point(i, u);
        if (!valid)
            for (int d = 0; d < D; ++d) u[d] = 0.5f;
        /* features of row t: [u, sin(2^k pi u), cos(2^k pi u)] in feature<D>'s order, zero-padded:
         * sinpi/cospi of the first band, the others by angle doubling (sin 2a = 2 sin a cos a,
         * cos 2a = 1 - 2 sin^2 a; a few ulp of FP32, far below the BF16 the MMA takes) */
        float ft[L::K0];
#pragma unroll
        for (int k = 0; k < L::K0; ++k) ft[k] = 0.0f;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            ft[d] = u[d];
            float sn = sinpif(u[d]), cs = cospif(u[d]);
#pragma unroll
            for (int k = 0; k < BANDS; ++k) {
                ft[D + 12 * d + 2 * k] = sn;
                ft[D + 12 * d + 2 * k + 1] = cs;
                const float s2 = 2.0f * sn * cs, c2 = fmaf(-2.0f * sn, sn, 1.0f);
                sn = s2;
                cs = c2;
            }
        }
#pragma unroll
        for (int kg = 0; kg < L::K0 / 8; ++kg) {
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = pack_bf16x2(ft[8 * kg + 2 * q], ft[8 * kg + 2 * q + 1]);
            *reinterpret_cast<uint4*>(A + core_off(t, 8 * kg, L::K0)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
        float o = 0.0f;
        for (int l = 0; l < 4 && ok; ++l) {
            const int K = l == 0 ? L::K0 : WIDTH;
            const int base = l == 0 ? L::B0 : (l == 1 ? L::B1 : (l == 2 ? L::B2 : L::B3));
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            if (t == 0) {
                tc_fence_after();
                const uint32_t b_addr = smem_u32(smem + base);
                for (int ks = 0; ks < K / 16; ++ks) {
                    /* K = 16 is two adjacent K-chunks: advance both operands by 2 x 128 B */
                    const uint64_t ad = smem_desc(a_addr + ks * 256, 128, (K / 8) * 128);
                    const uint64_t bd = smem_desc(b_addr + ks * 256, 128, (K / 8) * 128);
                    mma_f16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
                }
                mma_commit(mbar);
            }
            const bool got = mbar_wait(mbar, phase);
            phase ^= 1u;
            if (!got) *flag = 1;
            tc_fence_after();
            ok = __syncthreads_and(got) != 0;
            if (!ok) break;
            /* this warp's rows: accumulator + bias, ReLU, BF16 */
            float h[WIDTH];
            tmem_ld32(tmem + lane_base, h);
            tmem_ld32(tmem + lane_base + 32, h + 32);
            const float* bl = bias + l * WIDTH;
            if (l < 3) {
#pragma unroll
                for (int kg = 0; kg < WIDTH / 8; ++kg) {
                    uint32_t w[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int j = 8 * kg + 2 * q;
                        w[q] = pack_bf16x2(fmaxf(h[j] + bl[j], 0.0f), fmaxf(h[j + 1] + bl[j + 1], 0.0f));
                    }
                    *reinterpret_cast<uint4*>(A + core_off(t, 8 * kg, WIDTH)) = make_uint4(w[0], w[1], w[2], w[3]);
                }
            } else {
                /* output layer on the FP32 pipe: w4 . bf16(relu(h)) + b4 */
                float s = 0.0f;
#pragma unroll
                for (int j = 0; j < WIDTH; ++j) s = fmaf(__bfloat162float(__float2bfloat16_rn(fmaxf(h[j] + bl[j], 0.0f))), w4[j], s);
                o = s + b4;
            }
            tc_fence_before();
        }
        if (ok && valid) out[i] = o;
    }
    if (*flag && t == 0) atomicOr(status, VCU_FLAG_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

}  // namespace tc
}  // namespace mlp
}  // namespace vcu
