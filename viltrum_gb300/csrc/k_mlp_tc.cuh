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

/* ---------------------------------------------------------------- training on tcgen05
 * One training step's forward and backward over `rounds` tiles of 128 points per CTA (thread t owns
 * row t), every product on the tensor cores (M = 128, N = 64, BF16 operands in shared memory, FP32
 * accumulators in TMEM):
 *   forward   z_l = a_l W_l          A = a_l (points x inputs, K-major), B = W_l as [units][inputs]
 *   backward  da_l = dz_l W_l^T      A = dz_l (points x units, K-major), B = W_l as [inputs][units]
 *             dW_l += a_l^T dz_l     A = a_l, B = dz_l, both read MN-major (the same bytes: a
 *                                    K-major [point][input] tile is an MN-major [input][point] one)
 *             db_l = 1^T dz_l        A = ones, B = dz_l MN-major (every row of D is the column sum)
 * so no operand is transposed in shared memory.  The dW MMA's M = 128 rows past the layer's inputs
 * read neighbouring shared memory and are discarded.  dW_l of the four layers accumulate in TMEM over
 * the CTA's tiles (64 columns each) and are read once at the end; the output weights' and bias'
 * gradients are FP32 sums in shared memory.  Rounding points are the mma.sync kernels': BF16
 * features and activations, dz rounded to BF16 before its products, FP32 accumulation.  The CTA
 * writes its gradient to partial[block] in the training kernels' order (W0..W3 rows by input,
 * b0..b3, w4, b4). */
template <int D> struct TrainSmem {
    static constexpr int K0 = fin(D);
    static constexpr int W0 = 0;                              /* B of forward layer 0: 64 x K0 */
    static constexpr int W1 = W0 + MMA_N * K0 * 2;            /* B of forward layers 1-3: 64 x 64 */
    static constexpr int W2 = W1 + MMA_N * WIDTH * 2;
    static constexpr int W3 = W2 + MMA_N * WIDTH * 2;
    static constexpr int WT1 = W3 + MMA_N * WIDTH * 2;        /* B of backward layers 1-3: 64 x 64 */
    static constexpr int WT2 = WT1 + WIDTH * WIDTH * 2;
    static constexpr int WT3 = WT2 + WIDTH * WIDTH * 2;
    static constexpr int F = WT3 + WIDTH * WIDTH * 2;         /* features: 128 x K0 */
    static constexpr int H1 = F + TILE * K0 * 2;              /* hidden activations: 128 x 64 each */
    static constexpr int H2 = H1 + TILE * WIDTH * 2;
    static constexpr int H3 = H2 + TILE * WIDTH * 2;
    static constexpr int DZ = H3 + TILE * WIDTH * 2;          /* dz_l (and h4 before dz_3): 128 x 64 */
    static constexpr int ONES = DZ + TILE * WIDTH * 2;        /* 128 x 128 ones */
    /* an MN-major read of a tile strides up to 29 x (its row bytes / 8 x 16) past its start (16
     * core matrices along M, 2 x 8 along the points): F, H_l and DZ are followed by at least that
     * much of the layout, ONES last among the operands, then a pad */
    static constexpr int P32 = ONES + TILE * TILE * 2 + 4096; /* bias[4][64], w4[64], b4 */
    static constexpr int ACC = P32 + (5 * WIDTH + 4) * 4;     /* db[4][64], dw4[64], db4 */
    static constexpr int DV = ACC + (5 * WIDTH + 4) * 4;      /* the tile's output gradients */
    static constexpr int MBAR = DV + TILE * 4;
    static constexpr int SLOT = MBAR + 8;
    static constexpr int FLAG = SLOT + 4;
    static constexpr int BYTES = FLAG + 4;
    static constexpr int TCOLS = 512; /* temp 0-63, dW_l at 64 + 64 l, db 320-383 */
    static_assert(W1 % 16 == 0 && F % 16 == 0 && ONES % 16 == 0 && P32 % 16 == 0 && MBAR % 8 == 0, "alignment");
};

/* The packed parameter image carries, after its mma.sync layouts (pack_bytes), the training CTA's
 * weight operands already in the canonical layouts -- TrainSmem's W0..WT3, byte for byte -- so that
 * a CTA loads them with 16-byte copies. */
template <int D> __host__ __device__ constexpr int tc_pack_off() { return ((pack_bytes(D) + 127) / 128) * 128; }
template <int D> __host__ __device__ constexpr int tc_pack_bytes() { return TrainSmem<D>::F; }
template <int D> __host__ __device__ constexpr int packed_total_bytes() { return tc_pack_off<D>() + tc_pack_bytes<D>(); }
/* W_l[k][n] (input k, unit n) in the canonical sections */
template <int D> __device__ __forceinline__ void pack_tc_weight(char* packed, int l, int k, int n, __nv_bfloat16 b) {
    using L = TrainSmem<D>;
    char* base = packed + tc_pack_off<D>();
    const int K = layer_in(l, D);
    const int wb = l == 0 ? L::W0 : (l == 1 ? L::W1 : (l == 2 ? L::W2 : L::W3));
    *reinterpret_cast<__nv_bfloat16*>(base + wb + core_off(n, k, K)) = b;
    if (l > 0) {
        const int tb = l == 1 ? L::WT1 : (l == 2 ? L::WT2 : L::WT3);
        *reinterpret_cast<__nv_bfloat16*>(base + tb + core_off(k, n, WIDTH)) = b;
    }
}

/* instruction descriptor with A and B MN-major (bits 15 and 16) */
__host__ __device__ constexpr uint32_t instr_desc_mn(int m, int n, bool a_mn, bool b_mn) {
    return instr_desc(m, n) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}
/* issue the K/16 MMAs of D[128 x 64] (+)= A[128 x K] B[64 x K]^T with both operands K-major */
__device__ __forceinline__ void mma_tile(uint32_t tmem_d, uint32_t a_addr, uint32_t b_addr, int K, bool accumulate) {
    const uint32_t idesc = instr_desc(TILE, MMA_N);
    for (int ks = 0; ks < K / 16; ++ks) {
        const uint64_t ad = smem_desc(a_addr + ks * 256, 128, (K / 8) * 128);
        const uint64_t bd = smem_desc(b_addr + ks * 256, 128, (K / 8) * 128);
        mma_f16(tmem_d, ad, bd, idesc, (accumulate || ks > 0) ? 1u : 0u);
    }
}
/* D[128 x 64] (+)= A^T B over the 128 points of a tile, A and B stored K-major as [point][ka] and
 * [point][kb] tiles and read MN-major: along M / N the core matrices are 128 B apart (the stride
 * byte offset of an MN-major no-swizzle descriptor), along the points (K) ka/8 x 128 B and
 * kb/8 x 128 B (its leading byte offset); one MMA consumes 16 points.  a_mn false: A is a K-major
 * [128][128] tile (the ones).  The other assignment of the two offsets fails the gradient check
 * against the FP64 reference (tests/test_gpu_learned.py). */
__device__ __forceinline__ void mma_points(uint32_t tmem_d, uint32_t a_addr, int ka, bool a_mn, uint32_t b_addr, int kb,
                                           bool accumulate) {
    const uint32_t idesc = instr_desc_mn(TILE, MMA_N, a_mn, true);
    const uint32_t a_k = (uint32_t)(ka / 8) * 128u, b_k = (uint32_t)(kb / 8) * 128u;
    for (int ks = 0; ks < TILE / 16; ++ks) {
        const uint64_t ad = a_mn ? smem_desc(a_addr + ks * 2 * a_k, a_k, 128)
                                 : smem_desc(a_addr + ks * 256, 128, (TILE / 8) * 128);
        const uint64_t bd = smem_desc(b_addr + ks * 2 * b_k, b_k, 128);
        mma_f16(tmem_d, ad, bd, idesc, (accumulate || ks > 0) ? 1u : 0u);
    }
}
__device__ __forceinline__ __nv_bfloat16 bf16_of(float v) { return __float2bfloat16_rn(v); }

template <int D>
__device__ __forceinline__ void train_tiles(const float* __restrict__ u_in, const float* __restrict__ y_in,
                                            uint64_t npts, uint32_t rounds, float scale, float* __restrict__ out,
                                            const char* __restrict__ packed, float* __restrict__ partial,
                                            uint32_t* __restrict__ status) {
    using L = TrainSmem<D>;
    constexpr int K0 = L::K0;
    extern __shared__ __align__(128) char smem[];
    const int t = threadIdx.x, warp = t >> 5;
    /* weights (the packed image's canonical sections), FP32 parameters, the ones, zeroed sums */
    {
        const uint4* wsrc = reinterpret_cast<const uint4*>(packed + tc_pack_off<D>());
        uint4* wdst = reinterpret_cast<uint4*>(smem);
        for (int i = t; i < tc_pack_bytes<D>() / 16; i += THREADS) wdst[i] = wsrc[i];
        const float* src = reinterpret_cast<const float*>(packed + fp32_off_bytes(D));
        float* p32 = reinterpret_cast<float*>(smem + L::P32);
        for (int i = t; i < 5 * WIDTH + 1; i += THREADS) p32[i] = src[i];
        float* acc = reinterpret_cast<float*>(smem + L::ACC);
        for (int i = t; i < 5 * WIDTH + 4; i += THREADS) acc[i] = 0.0f;
        const uint32_t one2 = pack_bf16x2(1.0f, 1.0f);
        uint4* ones = reinterpret_cast<uint4*>(smem + L::ONES);
        for (int i = t; i < TILE * TILE * 2 / 16; i += THREADS) ones[i] = make_uint4(one2, one2, one2, one2);
    }
    const uint32_t mbar = smem_u32(smem + L::MBAR), slot = smem_u32(smem + L::SLOT);
    volatile int* flag = reinterpret_cast<volatile int*>(smem + L::FLAG);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(L::TCOLS)
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
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const float* bias = reinterpret_cast<const float*>(smem + L::P32);
    const float* w4 = bias + 4 * WIDTH;
    const float b4 = w4[WIDTH];
    float* acc = reinterpret_cast<float*>(smem + L::ACC); /* db[4][64] | dw4[64] | db4 */
    float* dv = reinterpret_cast<float*>(smem + L::DV);
    char* DZ = smem + L::DZ;
    uint32_t phase = 0;
    bool ok = true;
    /* wait for the committed MMAs; false (and the flag) when the bounded wait ran out */
    auto mma_done = [&]() -> bool {
        const bool got = mbar_wait(mbar, phase);
        phase ^= 1u;
        if (!got) *flag = 1;
        tc_fence_after();
        return __syncthreads_and(got) != 0;
    };
    auto sync_operands = [&]() {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
    };
    /* row t of a K-major [point][unit] 128 x 64 tile from 64 BF16-valued floats */
    auto write_row = [&](char* dst, const float* v) {
#pragma unroll
        for (int kg = 0; kg < WIDTH / 8; ++kg) {
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = pack_bf16x2(v[8 * kg + 2 * q], v[8 * kg + 2 * q + 1]);
            *reinterpret_cast<uint4*>(dst + core_off(t, 8 * kg, WIDTH)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    };
    uint32_t done_tiles = 0;
    for (uint32_t r = 0; r < rounds && ok; ++r) {
        const uint64_t i = ((uint64_t)blockIdx.x * rounds + r) * TILE + (uint64_t)t;
        const bool valid = i < npts;
        float u[D];
        for (int d = 0; d < D; ++d) u[d] = valid ? u_in[i * D + d] : 0.5f;
        const float y = valid ? y_in[i] : 0.0f;
        /* features of row t, as the forward kernel forms them */
        {
            float ft[K0];
#pragma unroll
            for (int k = 0; k < K0; ++k) ft[k] = 0.0f;
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
            for (int kg = 0; kg < K0 / 8; ++kg) {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q] = pack_bf16x2(ft[8 * kg + 2 * q], ft[8 * kg + 2 * q + 1]);
                *reinterpret_cast<uint4*>(smem + L::F + core_off(t, 8 * kg, K0)) = make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        /* forward: masks of the positive activations (relu') per layer, two words of 32 units */
        uint32_t mk[4][2];
        float g = 0.0f;
        for (int l = 0; l < 4 && ok; ++l) {
            const int K = l == 0 ? K0 : WIDTH;
            const int ab = l == 0 ? L::F : (l == 1 ? L::H1 : (l == 2 ? L::H2 : L::H3));
            const int wb = l == 0 ? L::W0 : (l == 1 ? L::W1 : (l == 2 ? L::W2 : L::W3));
            sync_operands();
            if (t == 0) {
                tc_fence_after();
                mma_tile(tmem, smem_u32(smem + ab), smem_u32(smem + wb), K, false);
                mma_commit(mbar);
            }
            ok = mma_done();
            if (!ok) break;
            float h[WIDTH];
            tmem_ld32(tmem + lane_base, h);
            tmem_ld32(tmem + lane_base + 32, h + 32);
            const float* bl = bias + l * WIDTH;
            mk[l][0] = mk[l][1] = 0u;
#pragma unroll
            for (int j = 0; j < WIDTH; ++j) {
                h[j] = __bfloat162float(bf16_of(fmaxf(h[j] + bl[j], 0.0f)));
                if (h[j] > 0.0f) mk[l][j >> 5] |= 1u << (j & 31);
            }
            if (l < 3) {
                write_row(smem + (l == 0 ? L::H1 : (l == 1 ? L::H2 : L::H3)), h);
            } else {
                float s = 0.0f;
#pragma unroll
                for (int j = 0; j < WIDTH; ++j) s = fmaf(h[j], w4[j], s);
                g = s + b4;
                write_row(DZ, h); /* h4, for the output weights' gradient */
            }
            tc_fence_before();
        }
        if (!ok) break;
        if (out && valid) out[i] = g;
        const float d = valid ? (g - y) * scale : 0.0f;
        dv[t] = d;
        __syncthreads();
        /* output layer: dw4[n] = sum d h4[n] (two threads per unit, half the points each) and
         * db4 = sum d (a warp sum per warp) */
        {
            const int n = t & (WIDTH - 1), half = t >> 6;
            float sw = 0.0f;
            for (int b = half * (TILE / 2); b < (half + 1) * (TILE / 2); ++b)
                sw = fmaf(dv[b], __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(DZ + core_off(b, n, WIDTH))), sw);
            float sb = d;
            for (int o = 16; o > 0; o >>= 1) sb += __shfl_xor_sync(0xffffffffu, sb, o);
            __syncthreads();
            float* tmp = dv; /* the output gradients are no longer needed */
            if (half == 1) tmp[n] = sw;
            if ((t & 31) == 0) tmp[WIDTH + warp] = sb;
            __syncthreads();
            if (half == 0) acc[4 * WIDTH + n] += sw + tmp[n];
            if (t == 0) acc[5 * WIDTH] += ((tmp[WIDTH] + tmp[WIDTH + 1]) + tmp[WIDTH + 2]) + tmp[WIDTH + 3];
        }
        /* dz_3 = relu'(z_3) * d * w4, rounded to BF16 (overwrites h4) */
        {
            float z[WIDTH];
#pragma unroll
            for (int n = 0; n < WIDTH; ++n)
                z[n] = ((mk[3][n >> 5] >> (n & 31)) & 1u) ? __bfloat162float(bf16_of(d * w4[n])) : 0.0f;
            __syncthreads(); /* every thread has read h4 */
            write_row(DZ, z);
        }
        for (int l = 3; l >= 0 && ok; --l) {
            const int K = l == 0 ? K0 : WIDTH;
            const int ab = l == 0 ? L::F : (l == 1 ? L::H1 : (l == 2 ? L::H2 : L::H3));
            sync_operands();
            if (t == 0) {
                tc_fence_after();
                /* dW_l += a_l^T dz_l, the bias gradient 1^T dz_l, and (l > 0) da_l = dz_l W_l^T */
                mma_points(tmem + 64 + 64 * l, smem_u32(smem + ab), K, true, smem_u32(DZ), WIDTH, done_tiles > 0);
                mma_points(tmem + 320, smem_u32(smem + L::ONES), TILE, false, smem_u32(DZ), WIDTH, false);
                if (l > 0) {
                    const int tb = l == 1 ? L::WT1 : (l == 2 ? L::WT2 : L::WT3);
                    mma_tile(tmem, smem_u32(DZ), smem_u32(smem + tb), WIDTH, false);
                }
                mma_commit(mbar);
            }
            ok = mma_done();
            if (!ok) break;
            if (warp == 0) { /* row 0 of the ones product: the column sums */
                float db[WIDTH];
                tmem_ld32(tmem + lane_base + 320, db);
                tmem_ld32(tmem + lane_base + 352, db + 32);
                if (t == 0)
                    for (int n = 0; n < WIDTH; ++n) acc[l * WIDTH + n] += db[n];
            }
            if (l > 0) {
                /* dz_{l-1} = relu'(z_{l-1}) * (dz_l W_l^T), rounded to BF16 */
                float da[WIDTH];
                tmem_ld32(tmem + lane_base, da);
                tmem_ld32(tmem + lane_base + 32, da + 32);
#pragma unroll
                for (int k = 0; k < WIDTH; ++k)
                    da[k] = ((mk[l - 1][k >> 5] >> (k & 31)) & 1u) ? __bfloat162float(bf16_of(da[k])) : 0.0f;
                write_row(DZ, da);
            }
            tc_fence_before();
        }
        if (!ok) break;
        ++done_tiles;
        __syncthreads();
    }
    /* the CTA's gradient: dW_l rows (inputs) from TMEM, warp w reading rows 32w..32w+31 */
    float* dst = partial + (size_t)blockIdx.x * n_params(D);
    __syncthreads();
    for (int l = 0; l < 4; ++l) {
        const int K = layer_in(l, D);
        const int woff = l == 0 ? 0 : K0 * WIDTH + (l - 1) * WIDTH * WIDTH;
        float v[WIDTH];
        if (ok && done_tiles > 0) {
            tmem_ld32(tmem + lane_base + 64 + 64 * l, v);
            tmem_ld32(tmem + lane_base + 96 + 64 * l, v + 32);
        } else {
#pragma unroll
            for (int n = 0; n < WIDTH; ++n) v[n] = 0.0f;
        }
        if (t < K)
            for (int n = 0; n < WIDTH; ++n) dst[woff + t * WIDTH + n] = v[n];
    }
    const int nw = (K0 + 3 * WIDTH) * WIDTH;
    for (int k = t; k < 5 * WIDTH + 1; k += THREADS) dst[nw + k] = acc[k];
    if (*flag && t == 0) atomicOr(status, VCU_FLAG_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::TCOLS) : "memory");
}

}  // namespace tc
}  // namespace mlp
}  // namespace vcu
