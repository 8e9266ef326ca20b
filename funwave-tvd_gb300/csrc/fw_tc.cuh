// fw_tc.cuh -- 3x3 convolutions of the learned correction on the fifth-
// generation tensor cores (tcgen05), for sm_100a / sm_103a.
//
// Implicit GEMM per CTA: M = 128 consecutive pixels of one grid row (one
// tcgen05.mma tile), N = the output channels (16 or 32), K = 9 taps x the
// input channels.  A CTA computes TROWS rows of 128 pixels:
//
//   1. one thread issues CINC TMA tensor loads (one per 8-channel chunk) of
//      the (TROWS + 2) x 130-pixel input halo tile -- zero-filled by the
//      TMA unit outside the grid -- and one bulk copy of the packed BF16
//      weight image, all completing on one mbarrier;
//   2. the same thread issues TROWS x 9 x CINC/2 tcgen05.mma (kind::f16,
//      BF16 x BF16 -> FP32) into TMEM, one 128 x N accumulator per output
//      row, and commits them to a second mbarrier;
//   3. the four warps read their 32 TMEM lanes (= pixels) back with
//      tcgen05.ld and apply the epilogue (bias + ReLU -> BF16, bias ->
//      FP32, or the backward ReLU mask -> BF16).
//
// Shared-memory operand layout (no swizzle, K-major canonical layout): the
// input tile is stored as CINC chunk planes, each [row][pixel][8 channels]
// (16 bytes a pixel).  A core matrix -- 8 pixels x 16 bytes -- is then 128
// contiguous bytes, consecutive pixel groups are 128 bytes apart (SBO) and
// consecutive K chunks one plane apart (LBO).  A tap's shift by one pixel
// is a shift of the descriptor's start address by 16 bytes, so all nine
// taps read the same staged tile.  The weight image of one tap is
// [chunk][n][8 channels] (SBO 128 bytes, LBO N x 16 bytes).
//
// Every wait on an mbarrier is bounded: on expiry the kernel records an
// error code, waits (bounded) for its own copies, frees its TMEM and
// returns.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace fwtc {

typedef __nv_bfloat16 bf16;

constexpr int TPX = 128;                 // pixels of an output row tile (the MMA's M)
constexpr int TROWS = 4;                 // output rows per CTA
constexpr int HPX = TPX + 2;             // staged pixels of a row (one halo pixel each side)
constexpr int ROWB = HPX * 16;           // bytes of one staged row of one chunk
constexpr int PLANE = ((TROWS + 2) * ROWB + 127) / 128 * 128;  // bytes of one chunk plane
constexpr int BOX_BYTES = 8 * HPX * (TROWS + 2) * 2;           // bytes one tensor load delivers
constexpr unsigned WAIT_LIMIT = 1u << 22;                      // polls of an mbarrier (~0.3-1 s)

enum { EPI_RELU_BF16 = 0, EPI_LINEAR_F32 = 1, EPI_MASK_BF16 = 2 };

template <int CINC, int N> struct Layout {
    static constexpr int X_BYTES = CINC * PLANE;
    static constexpr int W_BYTES = 9 * CINC * N * 16;
    static constexpr int BAR = X_BYTES + W_BYTES;  // two mbarriers, the TMEM address, a status word
    static constexpr int TMEM_COLS = TROWS * N <= 32 ? 32 : (TROWS * N <= 64 ? 64 : 128);
    // + slack for the 1024-byte alignment; at least 46 KB, so that no more
    // than four CTAs (4 x 128 TMEM columns = all 512) share an SM and no
    // tcgen05.alloc has to wait for another CTA's columns
    static constexpr int NEED = BAR + 32 + 1024;
    static constexpr int BYTES = NEED > 47104 ? NEED : 47104;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned i = 0; i < WAIT_LIMIT; i++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\n"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (i >= 32) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: start, leading (K) and stride (M/N)
// byte offsets, version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D
template <int M, int N> __host__ __device__ constexpr uint32_t idesc_bf16() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const uint32_t l = __bfloat16_as_ushort(__float2bfloat16(lo));
    const uint32_t h = __bfloat16_as_ushort(__float2bfloat16(hi));
    return l | (h << 16);
}

__device__ __forceinline__ float lo_bf(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float hi_bf(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// One CTA: TROWS output rows x 128 pixels of image b.  x: the input through
// its tensor map ([B][H][W][8*CINC] BF16).  wimg: the packed weight image
// (9 x CINC x N x 8 BF16).  EPI_RELU_BF16: y = BF16 relu(acc + bias),
// [pix][32]; EPI_LINEAR_F32: y = FP32 acc + bias, [pix][NOUTF]; EPI_MASK_BF16:
// y = BF16 acc where act > 0 else 0, [pix][32] (act: [pix][32] BF16).
// status: set to 1 (input wait expired) or 2 (MMA wait expired).
template <int CINC, int N, int EPI, int NOUTF>
__global__ void __launch_bounds__(128) k_conv_tc(const __grid_constant__ CUtensorMap xmap,
                                                 const bf16 *__restrict__ wimg, const float *__restrict__ bias,
                                                 const bf16 *__restrict__ act, void *__restrict__ y, int H, int W,
                                                 int *status) {
    static_assert(CINC % 2 == 0 && (N == 16 || N == 32), "K steps of 16 channels; N of 16 or 32");
    using L = Layout<CINC, N>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const uint32_t xs = smem_u32(smem), ws = xs + L::X_BYTES;
    const uint32_t bar_in = xs + L::BAR, bar_mma = bar_in + 8, tptr = bar_in + 16;
    volatile uint32_t *flag = reinterpret_cast<volatile uint32_t *>(smem + L::BAR + 20);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x0 = blockIdx.x * TPX, y0 = blockIdx.y * TROWS, b = blockIdx.z;

    if (threadIdx.x == 0) {
        mbar_init(bar_in, 1);
        mbar_init(bar_mma, 1);
        *flag = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tptr),
                     "r"((uint32_t)L::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t tmem;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(tmem) : "r"(tptr) : "memory");

    if (threadIdx.x == 0) {
        mbar_expect_tx(bar_in, (uint32_t)(CINC * BOX_BYTES + L::W_BYTES));
#pragma unroll
        for (int c = 0; c < CINC; c++) tma_load_4d(xs + c * PLANE, &xmap, c * 8, x0 - 1, y0 - 1, b, bar_in);
        bulk_load(ws, wimg, (uint32_t)L::W_BYTES, bar_in);
        if (mbar_wait(bar_in, 0)) {
            tc_fence_after();
            constexpr uint32_t idesc = idesc_bf16<TPX, N>();
#pragma unroll 1
            for (int r = 0; r < TROWS; r++) {
#pragma unroll
                for (int t = 0; t < 9; t++) {
                    const int ky = t / 3, kx = t % 3;  // staged row and pixel offsets of the tap
#pragma unroll
                    for (int h = 0; h < CINC / 2; h++) {
                        const uint32_t a = xs + 2 * h * PLANE + (r + ky) * ROWB + kx * 16;
                        const uint32_t bw = ws + (t * CINC + 2 * h) * N * 16;
                        tc_mma(tmem + r * N, sdesc(a, PLANE, 128), sdesc(bw, N * 16, 128), idesc,
                               (t | h) != 0 ? 1u : 0u);
                    }
                }
            }
            tc_commit(bar_mma);
        } else {
            *flag = 1u;
            atomicExch(status, 1);
            mbar_wait(bar_in, 0);  // the copies in flight, once more (bounded)
        }
    }
    __syncthreads();
    if (*flag == 0u) {
        const bool done = mbar_wait(bar_mma, 0);
        if (!done) atomicExch(status, 2);
        tc_fence_after();
        const int px = x0 + warp * 32 + lane;
#pragma unroll 1
        for (int r = 0; r < TROWS; r++) {
            uint32_t v[N];
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(r * N);
            tc_ld16(ta, *reinterpret_cast<uint32_t(*)[16]>(&v[0]));
            if constexpr (N == 32) tc_ld16(ta + 16, *reinterpret_cast<uint32_t(*)[16]>(&v[16]));
            tc_wait_ld();
            const int py = y0 + r;
            if (!done || px >= W || py >= H) continue;
            const long long p = ((long long)b * H + py) * W + px;
            if constexpr (EPI == EPI_LINEAR_F32) {
                float *yf = reinterpret_cast<float *>(y) + p * NOUTF;
#pragma unroll
                for (int c = 0; c < NOUTF; c++) yf[c] = __uint_as_float(v[c]) + __ldg(bias + c);
            } else {
                static_assert(EPI == EPI_LINEAR_F32 || N == 32, "BF16 outputs have 32 channels");
                uint4 *yq = reinterpret_cast<uint4 *>(reinterpret_cast<bf16 *>(y) + p * 32);
                if constexpr (EPI == EPI_RELU_BF16) {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float f[8];
#pragma unroll
                        for (int e = 0; e < 8; e++) f[e] = fmaxf(__uint_as_float(v[q * 8 + e]) + __ldg(bias + q * 8 + e), 0.0f);
                        yq[q] = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
                    }
                } else {
                    const uint4 *aq = reinterpret_cast<const uint4 *>(act + p * 32);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const uint4 m = __ldg(aq + q);
                        const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
                        float f[8];
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            f[2 * e] = lo_bf(mw[e]) > 0.0f ? __uint_as_float(v[q * 8 + 2 * e]) : 0.0f;
                            f[2 * e + 1] = hi_bf(mw[e]) > 0.0f ? __uint_as_float(v[q * 8 + 2 * e + 1]) : 0.0f;
                        }
                        yq[q] = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)L::TMEM_COLS)
                     : "memory");
    }
}

// Packed weight image of one convolution for k_conv_tc: [tap][chunk][n][8].
// Forward: K index = the layer's input channel ci, n = its output channel
// co, tap t reads w[t][ci][co].  Backward data gradient (dgrad != 0): the
// convolution runs over dy, so K = co, n = ci, and tap t reads the layer's
// tap 8 - t (the mirrored offset).  Channels beyond cin / cout are zero.
__global__ void k_pack_wimg(const float *__restrict__ w, int cin, int cout, int cinc, int n_img, int dgrad,
                            bf16 *__restrict__ img) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = 9 * cinc * n_img * 8;
    if (e >= total) return;
    const int j = e % 8, n = (e / 8) % n_img, c = (e / (8 * n_img)) % cinc, t = e / (8 * n_img * cinc);
    const int k = c * 8 + j;
    float v = 0.0f;
    if (!dgrad) {
        if (k < cin && n < cout) v = w[((size_t)t * cin + k) * cout + n];
    } else {
        if (n < cin && k < cout) v = w[((size_t)(8 - t) * cin + n) * cout + k];
    }
    img[e] = __float2bfloat16(v);
}

}  // namespace fwtc
