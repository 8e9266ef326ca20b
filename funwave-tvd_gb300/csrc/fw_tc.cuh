// fw_tc.cuh -- 3x3 convolutions of the learned correction on the fifth-
// generation tensor cores (tcgen05), for sm_100a / sm_103a.
//
// Implicit GEMM per CTA: M = 128 consecutive pixels of one grid row (one
// tcgen05.mma tile), N = the output channels (16 or 32), K = 9 taps x the
// input channels.  A CTA computes TROWS rows of 128 pixels:
//
//   1. the lanes of one warp issue (TROWS + 2) x CINC bulk copies (cp.async.bulk),
//      one contiguous 130-pixel run per staged row and 8-channel chunk of
//      the padded activation (below), completing on an mbarrier (with the
//      first tile, one bulk copy of the packed BF16 weight image too);
//   2. one thread of a second warp issues TROWS x 9 x CINC/2 tcgen05.mma
//      (kind::f16, BF16 x BF16 -> FP32) into TMEM, one 128 x N accumulator
//      per output row, and commits them to a second mbarrier;
//   3. the epilogue warps read their 32 TMEM lanes (= pixels) back with
//      tcgen05.ld and apply the epilogue (bias + ReLU -> BF16, bias ->
//      FP32, or the backward ReLU mask -> BF16).
// CTAs are persistent and warp-specialised (a TMA warp, an MMA warp, eight
// epilogue warps) with NSTAGE input stages and two TMEM accumulators, so
// loads, MMAs and epilogues of successive tiles overlap.
//
// Activations in global memory are BF16, chunk-planar and padded:
// [B][H + 2][chunks][W + 2][8 channels], a zero pixel on every side of each
// image (act_idx).  A staged row of one chunk is then 130 contiguous
// 16-byte pixels, and the zero border is the convolution's padding.
//
// Shared-memory operand layout (no swizzle, K-major canonical layout): the
// staged tile is [row][chunk][pixel][8 channels] (16 bytes a pixel).  A
// core matrix -- 8 pixels x 16 bytes -- is then 128 contiguous bytes,
// consecutive pixel groups are 128 bytes apart (SBO) and consecutive K
// chunks one staged row of a chunk apart (LBO).  A tap's shift by one pixel
// is a shift of the descriptor's start address by 16 bytes, so all nine
// taps read the same staged tile.  The weight image of one tap is
// [chunk][n][8 channels] (SBO 128 bytes, LBO N x 16 bytes).
//
// Every wait on an mbarrier is bounded: on expiry the kernel records an
// error code, waits (bounded) for its own copies, frees its TMEM and
// returns.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace fwtc {

typedef __nv_bfloat16 bf16;

constexpr int TPX = 128;                 // pixels of an output row tile (the MMA's M)
constexpr int TROWS = 4;                 // output rows per CTA
constexpr int HPX = TPX + 2;             // staged pixels of a row (one halo pixel each side)
constexpr int ROWB = HPX * 16;           // bytes of one staged row of one chunk
constexpr unsigned WAIT_LIMIT = 1u << 22;  // polls of an mbarrier (~0.3-1 s)

// the padded chunk-planar activation of a B x H x W image batch with CC
// 8-channel chunks, in 16-byte units: [B][H + 2][CC][W + 2]
struct ActGeom {
    int B, H, W, CC;
};
__host__ __device__ __forceinline__ long long act_idx(const ActGeom &a, int b, int y, int c, int x) {
    return (((long long)b * (a.H + 2) + (y + 1)) * a.CC + c) * (a.W + 2) + (x + 1);
}
// bytes of such a buffer, with slack for the staged runs of the last tiles,
// which may read up to 128 pixels past a row's end and TROWS + 2 rows past
// the last image (values that only masked outputs use)
__host__ __device__ __forceinline__ size_t act_bytes(const ActGeom &a) {
    return (size_t)a.B * (a.H + 2) * a.CC * (a.W + 2) * 16 + (size_t)(TROWS + 2) * a.CC * (a.W + 2) * 16 + 4096;
}

enum { EPI_RELU_BF16 = 0, EPI_LINEAR_F32 = 1, EPI_MASK_BF16 = 2 };

constexpr int NSTAGE = 3;                // input stages in flight per CTA
constexpr int EPI_WARPS = 8;             // epilogue warps (two per TMEM lane quadrant)
static_assert(TROWS % 2 == 0, "the epilogue splits a tile's rows in two halves");

template <int CINC, int N> struct Layout {
    static constexpr int X_BYTES = (TROWS + 2) * CINC * ROWB;  // one input stage
    static constexpr int W_BYTES = 9 * CINC * N * 16;
    static constexpr int TMEM_COLS = TROWS * N <= 32 ? 32 : (TROWS * N <= 64 ? 64 : 128);  // one accumulator
    // NSTAGE input stages, the weights, 2 NSTAGE + 4 mbarriers, the TMEM
    // address and a flag, + slack for the 1024-byte alignment
    static constexpr int NEED = NSTAGE * X_BYTES + W_BYTES + 8 * (2 * NSTAGE + 4) + 8 + 1024;
    // CTAs an SM can hold: by shared memory (228 KB, 1 KB reserved each)
    // and by TMEM (512 columns, two accumulators each); the host launches
    // no more than this per SM, so no tcgen05.alloc waits for another CTA
    static constexpr int PER_SM_SMEM = 233472 / (NEED + 1024);
    static constexpr int PER_SM_TMEM = 512 / (2 * TMEM_COLS);
    static constexpr int PER_SM = PER_SM_SMEM < PER_SM_TMEM ? PER_SM_SMEM : PER_SM_TMEM;
    static constexpr int BYTES = NEED;
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
// limit: polls before giving up.  Waits whose expiry the kernel turns into
// an error status take the caller's limit (a run-time setting, so that a
// test can make them run out); the waits that drain a block's own copies
// and MMAs before it frees its shared memory and TMEM always take
// WAIT_LIMIT.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned limit = WAIT_LIMIT) {
    for (unsigned i = 0; i < limit; i++) {
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

// TMA tiled load of a 2-D box at (c0, c1) (elements) through a tensor map
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void *map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
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

// Persistent, warp-specialised CTAs of 320 threads, each walking the tiles
// t = blockIdx.x, + gridDim.x, ... (a tile: TROWS output rows x 128 pixels
// of one image):
//   warp 0              TMA producer: tile i's halo into input stage
//                       i % NSTAGE once the MMAs of tile i - NSTAGE have
//                       released it (the weight image with tile 0);
//   warp 1              allocates TMEM; one lane issues tile i's MMAs into
//                       accumulator i & 1 once its input has landed and
//                       the epilogue of tile i - 2 has drained that
//                       accumulator, then commits to the stage's "empty"
//                       and the accumulator's "full" barriers;
//   warps 2-9           the epilogue: each reads its TMEM lane quadrant
//                       (warp % 4) of half of the finished accumulator's
//                       rows (warps 2-5 the first half, 6-9 the second),
//                       releases it, and stores.
// No CTA-wide barrier sits inside the loop, so loads, MMAs and epilogues of
// successive tiles overlap.  x: the padded input (CINC chunks); wimg: the
// packed weight image (9 x CINC x N x 8 BF16).  EPI_RELU_BF16: y = BF16
// relu(acc + bias), padded with 4 chunks; EPI_LINEAR_F32: y = FP32 acc +
// bias, [pix][NOUTF] unpadded; EPI_MASK_BF16: y = BF16 acc where act > 0
// else 0, padded with 4 chunks (act: padded, 4 chunks).  status: set to
// 1 (an input or accumulator wait expired) or 2 (an MMA wait expired); every
// role then stops.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, volatile uint32_t *flag,
                                                   unsigned limit) {
    for (unsigned i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\n"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 63) == 63 && *flag != 0u) return false;
        if (i >= 32) __nanosleep(32);
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

template <int CINC, int N, int EPI, int NOUTF>
__global__ void __launch_bounds__(320, 1) k_conv_tc(const bf16 *__restrict__ x, const bf16 *__restrict__ wimg,
                                                    const float *__restrict__ bias, const bf16 *__restrict__ act,
                                                    void *__restrict__ y, int H, int W, int B, int *status,
                                                    unsigned wait_limit) {
    static_assert(CINC % 2 == 0 && (N == 16 || N == 32), "K steps of 16 channels; N of 16 or 32");
    using L = Layout<CINC, N>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const uint32_t xs0 = smem_u32(smem), ws = xs0 + NSTAGE * L::X_BYTES;
    const uint32_t bar = ws + L::W_BYTES;
    // barriers: full[NSTAGE], empty[NSTAGE], accf[2], acce[2]
    auto full_bar = [&](int st) { return bar + 8u * st; };
    auto empty_bar = [&](int st) { return bar + 8u * (NSTAGE + st); };
    auto accf_bar = [&](int a) { return bar + 8u * (2 * NSTAGE + a); };
    auto acce_bar = [&](int a) { return bar + 8u * (2 * NSTAGE + 2 + a); };
    const uint32_t tptr = bar + 8u * (2 * NSTAGE + 4);
    volatile uint32_t *flag = reinterpret_cast<volatile uint32_t *>(smem + (tptr + 4u - xs0));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ActGeom gin{B, H, W, CINC}, gout{B, H, W, 4};
    const int tiles_x = (W + TPX - 1) / TPX, tiles_y = (H + TROWS - 1) / TROWS;
    const int ntiles = tiles_x * tiles_y * B;
    const int ntl = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto tile_xyb = [&](int i, int &x0, int &y0, int &b) {
        const int t = (int)blockIdx.x + i * (int)gridDim.x;
        x0 = (t % tiles_x) * TPX;
        y0 = ((t / tiles_x) % tiles_y) * TROWS;
        b = t / (tiles_x * tiles_y);
    };
    auto fail = [&](int code) {
        *flag = 1u;
        atomicExch(status, code);
    };

    if (threadIdx.x == 0) {
        for (int k = 0; k < NSTAGE; k++) {
            mbar_init(full_bar(k), 1);
            mbar_init(empty_bar(k), 1);
        }
        for (int k = 0; k < 2; k++) {
            mbar_init(accf_bar(k), 1);
            mbar_init(acce_bar(k), EPI_WARPS);  // one arrival per epilogue warp
        }
        *flag = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tptr),
                     "r"((uint32_t)(2 * L::TMEM_COLS))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t tmem;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(tmem) : "r"(tptr) : "memory");

    // the last tile issued to each input stage (producer lane) and the last
    // tile whose MMAs were committed (MMA lane): what a block that aborts
    // must wait for before it frees its shared memory and TMEM
    int last[NSTAGE];
#pragma unroll
    for (int k = 0; k < NSTAGE; k++) last[k] = -1;
    int committed = -1;
    if (warp == 0) {
        // lane 0 waits for the stage and sets the bytes to expect, then the
        // warp's lanes issue the tile's copies, one each
        for (int i = 0; i < ntl; i++) {
            const int st = i % NSTAGE;
            int go = 1;
            if (lane == 0) {
                if (i >= NSTAGE &&
                    !mbar_wait_or_abort(empty_bar(st), (uint32_t)(((i / NSTAGE) - 1) & 1), flag, wait_limit)) {
                    if (*flag == 0u) fail(1);
                    go = 0;
                } else {
                    mbar_expect_tx(full_bar(st), (uint32_t)(L::X_BYTES + (i == 0 ? L::W_BYTES : 0)));
                }
            }
            go = __shfl_sync(0xffffffffu, go, 0);
            if (!go) break;
            int x0, y0, b;
            tile_xyb(i, x0, y0, b);
            const uint32_t xs = xs0 + st * L::X_BYTES;
            // staged row rr, chunk c: pixels x0-1 .. x0+128 of image row y0-1+rr
            for (int e = lane; e < (TROWS + 2) * CINC; e += 32) {
                const int rr = e / CINC, c = e % CINC;
                bulk_load(xs + e * ROWB, x + 8 * act_idx(gin, b, y0 - 1 + rr, c, x0 - 1), (uint32_t)ROWB,
                          full_bar(st));
            }
            if (i == 0 && lane == 31) bulk_load(ws, wimg, (uint32_t)L::W_BYTES, full_bar(0));
#pragma unroll
            for (int k = 0; k < NSTAGE; k++)
                if (k == st) last[k] = i;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16<TPX, N>();
            for (int i = 0; i < ntl; i++) {
                const int st = i % NSTAGE, a = i & 1;
                if (!mbar_wait_or_abort(full_bar(st), (uint32_t)((i / NSTAGE) & 1), flag, wait_limit)) {
                    if (*flag == 0u) fail(1);
                    break;
                }
                if (i >= 2 && !mbar_wait_or_abort(acce_bar(a), (uint32_t)(((i >> 1) - 1) & 1), flag, wait_limit)) {
                    if (*flag == 0u) fail(1);
                    break;
                }
                tc_fence_after();
                const uint32_t xs = xs0 + st * L::X_BYTES, acc = tmem + (uint32_t)(a * L::TMEM_COLS);
                // the start address is the descriptors' low field (16-byte
                // units), so each MMA's descriptors are these two plus a
                // compile-time offset (all shared addresses stay below 256 KB,
                // so the field does not overflow)
                const uint64_t a_base = sdesc(xs, ROWB, 128), b_base = sdesc(ws, N * 16, 128);
#pragma unroll 1
                for (int r = 0; r < TROWS; r++) {
                    const uint64_t a_row = a_base + (uint64_t)((r * CINC * ROWB) >> 4);
#pragma unroll
                    for (int t = 0; t < 9; t++) {
                        const int ky = t / 3, kx = t % 3;  // staged row and pixel offsets of the tap
#pragma unroll
                        for (int h = 0; h < CINC / 2; h++) {
                            const uint32_t a_off = (uint32_t)(((ky * CINC + 2 * h) * ROWB + kx * 16) >> 4);
                            const uint32_t b_off = (uint32_t)(((t * CINC + 2 * h) * N * 16) >> 4);
                            tc_mma(acc + r * N, a_row + a_off, b_base + b_off, idesc, (t | h) != 0 ? 1u : 0u);
                        }
                    }
                }
                tc_commit(empty_bar(st));
                tc_commit(accf_bar(a));
                committed = i;
            }
        }
    } else {
        const int q = warp & 3;  // TMEM lane quadrant of this warp
        constexpr int RH = TROWS / 2;
        const int r0 = warp < 6 ? 0 : RH;  // this warp's rows: r0 .. r0 + RH - 1
        float bs[EPI == EPI_MASK_BF16 ? 1 : N];
        if constexpr (EPI != EPI_MASK_BF16) {
#pragma unroll
            for (int c = 0; c < N; c++) bs[c] = (EPI == EPI_LINEAR_F32 && c >= NOUTF) ? 0.0f : __ldg(bias + c);
        }
        for (int i = 0; i < ntl; i++) {
            const int a = i & 1;
            if (!mbar_wait_or_abort(accf_bar(a), (uint32_t)((i >> 1) & 1), flag, wait_limit)) {
                if (*flag == 0u) fail(2);
                break;
            }
            __syncwarp();
            tc_fence_after();
            int x0, y0, b;
            tile_xyb(i, x0, y0, b);
            const int px = x0 + q * 32 + lane;
#pragma unroll 1
            for (int r = r0; r < r0 + RH; r++) {
                uint32_t v[N];
                const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * L::TMEM_COLS + r * N);
                tc_ld16(ta, *reinterpret_cast<uint32_t(*)[16]>(&v[0]));
                if constexpr (N == 32) tc_ld16(ta + 16, *reinterpret_cast<uint32_t(*)[16]>(&v[16]));
                tc_wait_ld();
                if (r == r0 + RH - 1) {
                    // the accumulator is read: release it to tile i + 2
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(acce_bar(a));
                }
                const int py = y0 + r;
                if (px >= W || py >= H) continue;
                const long long p = ((long long)b * H + py) * W + px;
                if constexpr (EPI == EPI_LINEAR_F32) {
                    float *yf = reinterpret_cast<float *>(y) + p * NOUTF;
#pragma unroll
                    for (int c = 0; c < NOUTF; c++) yf[c] = __uint_as_float(v[c]) + bs[c];
                } else {
                    static_assert(EPI == EPI_LINEAR_F32 || N == 32, "BF16 outputs have 32 channels");
                    // chunk qq of this pixel: consecutive lanes write consecutive 16 bytes
                    uint4 *yq = reinterpret_cast<uint4 *>(y);
                    const long long o0 = act_idx(gout, b, py, 0, px), ostep = (long long)(W + 2);
                    if constexpr (EPI == EPI_RELU_BF16) {
#pragma unroll
                        for (int qq = 0; qq < 4; qq++) {
                            float f[8];
#pragma unroll
                            for (int e = 0; e < 8; e++)
                                f[e] = fmaxf(__uint_as_float(v[qq * 8 + e]) + bs[qq * 8 + e], 0.0f);
                            yq[o0 + qq * ostep] = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]),
                                                             pack2(f[6], f[7]));
                        }
                    } else {
                        const uint4 *aq = reinterpret_cast<const uint4 *>(act);
#pragma unroll
                        for (int qq = 0; qq < 4; qq++) {
                            const uint4 m = __ldg(aq + o0 + qq * ostep);
                            const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
                            float f[8];
#pragma unroll
                            for (int e = 0; e < 4; e++) {
                                f[2 * e] = lo_bf(mw[e]) > 0.0f ? __uint_as_float(v[qq * 8 + 2 * e]) : 0.0f;
                                f[2 * e + 1] = hi_bf(mw[e]) > 0.0f ? __uint_as_float(v[qq * 8 + 2 * e + 1]) : 0.0f;
                            }
                            yq[o0 + qq * ostep] = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]),
                                                             pack2(f[6], f[7]));
                        }
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    // Every role has finished or given up, so the abort flag is final here.
    // After an abort, loads and MMAs may still be in flight (a role can give
    // up while another has already issued work, and the producer may have
    // issued its last loads before any role gave up): wait for them
    // (bounded, with the full limit) before the block frees its TMEM and
    // its shared memory.
    if (*flag != 0u) {
        if (warp == 0 && lane == 0) {
#pragma unroll
            for (int k = 0; k < NSTAGE; k++)
                if (last[k] >= 0) mbar_wait(full_bar(k), (uint32_t)((last[k] / NSTAGE) & 1));
        }
        if (warp == 1 && lane == 0 && committed >= 0)
            mbar_wait(accf_bar(committed & 1), (uint32_t)((committed >> 1) & 1));
        __syncwarp();
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"((uint32_t)(2 * L::TMEM_COLS))
                     : "memory");
    }
}

// Packed weight image of one convolution for k_conv_tc: [tap][chunk][n][8].
// Forward: K index = the layer's input channel ci, n = its output channel
// co, tap t reads w[t][ci][co].  Backward data gradient (dgrad != 0): the
// convolution runs over dy, so K = co, n = ci, and tap t reads the layer's
// tap 8 - t (the mirrored offset).  Channels beyond cin / cout are zero.
static __global__ void k_pack_wimg(const float *__restrict__ w, int cin, int cout, int cinc, int n_img, int dgrad,
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

// ---------------------------------------------------------------------------
// Weight and bias gradients on the tensor cores.  For a layer with input x
// and (masked) output gradient dy,
//     dW[t][ci][co] = sum_p x[p + tap t][ci] dy[p][co],   db[co] = sum_p dy[p][co],
// a GEMM whose K is the pixels: D (M x N) += A (M x K) B (K x N) with the
// rows of A (tap, input channel) pairs, N the output channels and one tile
// of WKT = 64 consecutive pixels of a grid row per step of K.
//
// A tile stages, for each of the rows y-1, y, y+1 and each used 8-channel
// chunk c of x, one run of 66 pixels (x0-1 .. x0+64) of the padded
// activation: plane q = ky * CCU + c, 1056 bytes, one bulk copy each.  A
// plane of ones follows the 3 CCU row planes (its row of D is the bias
// gradient) and zero planes fill up to 16.  Both operands are read MN-major
// (the 8 channels of a pixel are the contiguous 16 bytes): a core matrix is
// 8 pixels x 16 bytes = 128 contiguous bytes, consecutive planes are 1056
// bytes apart (the M direction, SBO) and consecutive 8-pixel groups 128
// bytes apart (K, LBO).  The taps of one x offset kx are then the 16 planes
// read from a start address kx * 16 bytes on: three M = 128 MMAs per K step
// (kx = 0, 1, 2), each into its own TMEM accumulator of N columns, whose row
// 8q + ch is tap (q / CCU) * 3 + kx, input channel (q % CCU) * 8 + ch.  B is
// dy, DYCC planes of 64 pixels.  The accumulators add up over all the tiles
// a CTA walks, and the epilogue writes them as one partial per CTA (the
// weight layout [t][ci][co], then the bias).
//
// Warp 0 loads (one copy per lane), warp 1 zeroes the pixels past the grid
// row in a partial tile and one lane issues the MMAs, warps 2-5 read the
// accumulators once at the end.  Every wait is bounded as in k_conv_tc.
// ---------------------------------------------------------------------------
constexpr int WKT = 64;                  // pixels of a tile: four K steps of 16
constexpr int WPLANE = WKT * 16;         // bytes of one staged dy plane
constexpr int WXPLANE = (WKT + 2) * 16;  // bytes of one staged x plane (one halo pixel each side)
constexpr int WNSTAGE = 4;

template <int CCU, int DYCC> struct WLayout {
    static constexpr int NQ = 3 * CCU;                   // row planes of x
    static_assert(NQ + 1 <= 16, "the row planes and the ones plane fill one M = 128 group");
    static constexpr int G = 3;                          // M = 128 groups: one per x offset of the taps
    static constexpr int N = DYCC * 8;
    static constexpr int DYOFF = 16 * WXPLANE;           // dy planes after the 16 x planes
    static constexpr int STAGE = DYOFF + DYCC * WPLANE;
    static constexpr int LOAD = NQ * WXPLANE + DYCC * WPLANE;  // bytes the copies of one tile bring
    static constexpr int TMEM_COLS = G * N <= 32 ? 32 : (G * N <= 64 ? 64 : (G * N <= 128 ? 128 : 256));
    static constexpr int NEED = WNSTAGE * STAGE + 8 * (2 * WNSTAGE + 1) + 8 + 1024;
    static constexpr int PER_SM_SMEM = 233472 / (NEED + 1024);
    static constexpr int PER_SM_TMEM = 512 / TMEM_COLS;
    static constexpr int PER_SM = PER_SM_SMEM < PER_SM_TMEM ? PER_SM_SMEM : PER_SM_TMEM;
    static constexpr int BYTES = NEED;
};

// XCC / DYCC: chunks of the stored x and dy; CCU: chunks of x used (CIN =
// the layer's input channels, <= 8 CCU); COUT: output channels (<= N).
// part: E = 9 CIN COUT + COUT floats per CTA.
template <int XCC, int CCU, int DYCC, int CIN, int COUT>
__global__ void __launch_bounds__(192) k_wgrad_tc(const bf16 *__restrict__ x, const bf16 *__restrict__ dy,
                                                  float *__restrict__ part, int H, int W, int B, int *status,
                                                  unsigned wait_limit) {
    using L = WLayout<CCU, DYCC>;
    constexpr int N = L::N, E = 9 * CIN * COUT + COUT;
    static_assert(N == 16 || N == 32, "N of 16 or 32");
    static_assert(CIN <= 8 * CCU && COUT <= N && CCU <= XCC, "channels");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const uint32_t xs0 = smem_u32(smem);
    const uint32_t bar = xs0 + WNSTAGE * L::STAGE;
    auto full_bar = [&](int st) { return bar + 8u * st; };
    auto empty_bar = [&](int st) { return bar + 8u * (WNSTAGE + st); };
    const uint32_t done_bar = bar + 8u * (2 * WNSTAGE);
    const uint32_t tptr = bar + 8u * (2 * WNSTAGE + 1);
    volatile uint32_t *flag = reinterpret_cast<volatile uint32_t *>(smem + (tptr + 4u - xs0));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ActGeom gx{B, H, W, XCC}, gd{B, H, W, DYCC};
    const int tiles_x = (W + WKT - 1) / WKT;
    const int ntiles = tiles_x * H * B;
    const int ntl = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto tile_xyb = [&](int i, int &x0, int &y, int &b) {
        const int t = (int)blockIdx.x + i * (int)gridDim.x;
        x0 = (t % tiles_x) * WKT;
        y = (t / tiles_x) % H;
        b = t / (tiles_x * H);
    };
    auto fail = [&](int code) {
        *flag = 1u;
        atomicExch(status, code);
    };

    if (threadIdx.x == 0) {
        for (int k = 0; k < WNSTAGE; k++) {
            mbar_init(full_bar(k), 1);
            mbar_init(empty_bar(k), 1);
        }
        mbar_init(done_bar, 1);
        *flag = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tptr),
                     "r"((uint32_t)L::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // the ones plane and the zero planes of every stage, once: the copies
    // never write them
    {
        constexpr int PX = WXPLANE / 16, PER = (16 - L::NQ) * PX;
        for (int e = threadIdx.x; e < WNSTAGE * PER; e += blockDim.x) {
            const int st = e / PER, r = e % PER;
            const int q = L::NQ + r / PX, px = r % PX;
            const uint32_t one2 = 0x3F803F80u;  // two BF16 ones
            const uint4 v = q == L::NQ ? make_uint4(one2, one2, one2, one2) : make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4 *>(smem + st * L::STAGE + q * WXPLANE + px * 16) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t tmem;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(tmem) : "r"(tptr) : "memory");

    int last[WNSTAGE];
#pragma unroll
    for (int k = 0; k < WNSTAGE; k++) last[k] = -1;
    int committed = -1;
    bool done_sent = false;
    if (warp == 0) {
        // lane 0 waits for the stage and sets the bytes to expect, then the
        // warp's lanes issue the tile's copies, one each
        for (int i = 0; i < ntl; i++) {
            const int st = i % WNSTAGE;
            int go = 1;
            if (lane == 0) {
                if (i >= WNSTAGE &&
                    !mbar_wait_or_abort(empty_bar(st), (uint32_t)(((i / WNSTAGE) - 1) & 1), flag, wait_limit)) {
                    if (*flag == 0u) fail(1);
                    go = 0;
                } else {
                    mbar_expect_tx(full_bar(st), (uint32_t)L::LOAD);
                }
            }
            go = __shfl_sync(0xffffffffu, go, 0);
            if (!go) break;
            int x0, y, b;
            tile_xyb(i, x0, y, b);
            const uint32_t xs = xs0 + st * L::STAGE;
            if (lane < L::NQ) {
                const int ky = lane / CCU, c = lane % CCU;
                bulk_load(xs + lane * WXPLANE, x + 8 * act_idx(gx, b, y - 1 + ky, c, x0 - 1), (uint32_t)WXPLANE,
                          full_bar(st));
            } else if (lane < L::NQ + DYCC) {
                const int c = lane - L::NQ;
                bulk_load(xs + L::DYOFF + c * WPLANE, dy + 8 * act_idx(gd, b, y, c, x0), (uint32_t)WPLANE,
                          full_bar(st));
            }
#pragma unroll
            for (int k = 0; k < WNSTAGE; k++)
                if (k == st) last[k] = i;
        }
    } else if (warp == 1) {
        // MN-major A and B (instruction descriptor bits 15 and 16)
        constexpr uint32_t idesc = idesc_bf16<128, N>() | (1u << 15) | (1u << 16);
        bool ok = true;
        for (int i = 0; i < ntl; i++) {
            const int st = i % WNSTAGE;
            int landed = 1;
            if (lane == 0) landed = mbar_wait_or_abort(full_bar(st), (uint32_t)((i / WNSTAGE) & 1), flag, wait_limit);
            landed = __shfl_sync(0xffffffffu, landed, 0);
            if (!landed) {
                if (lane == 0 && *flag == 0u) fail(1);
                ok = false;
                break;
            }
            int x0, y, b;
            tile_xyb(i, x0, y, b);
            const int valid = W - x0 < WKT ? W - x0 : WKT;
            uint8_t *xsg = smem + st * L::STAGE;
            if (valid < WKT) {
                // past the grid row: dy pixels valid.. and x pixels valid+2..
                // (staged pixel s is grid pixel x0 - 1 + s; pixel W is the
                // zero border) are zeroed, once every lane has seen the copies
                // land (the phase is complete, so the first poll succeeds)
                mbar_wait(full_bar(st), (uint32_t)((i / WNSTAGE) & 1), 64);
                const int nz = WKT - valid;
                for (int e = lane; e < (L::NQ + DYCC) * nz; e += 32) {
                    const int qq = e / nz, r = e % nz;
                    const int off = qq < L::NQ ? qq * WXPLANE + (valid + 2 + r) * 16
                                               : L::DYOFF + (qq - L::NQ) * WPLANE + (valid + r) * 16;
                    *reinterpret_cast<uint4 *>(xsg + off) = make_uint4(0u, 0u, 0u, 0u);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            __syncwarp();
            if (lane == 0) {
                tc_fence_after();
                const uint32_t xs = xs0 + st * L::STAGE;
                // no swizzle: the stride between core matrices along M / N in
                // the SBO field, along K in the LBO field
                const uint64_t a_base = sdesc(xs, 128, WXPLANE), b_base = sdesc(xs + L::DYOFF, 128, WPLANE);
#pragma unroll
                for (int ks = 0; ks < WKT / 16; ks++)
#pragma unroll
                    for (int kx = 0; kx < 3; kx++)
                        tc_mma(tmem + (uint32_t)(kx * N), a_base + (uint64_t)((kx * 16 + ks * 256) >> 4),
                               b_base + (uint64_t)((ks * 256) >> 4), idesc, (i | ks) != 0 ? 1u : 0u);
                tc_commit(empty_bar(st));
            }
            committed = i;
            __syncwarp();
        }
        if (lane == 0 && ok && ntl > 0) {
            tc_commit(done_bar);
            done_sent = true;
        }
    } else {
        const int q = warp & 3;  // TMEM lane quadrant
        float *pp = part + (size_t)blockIdx.x * E;
        // 1: the accumulators are final; 0: this CTA had no tile (zeros);
        // 2: a wait gave up (nothing is written).  Decided by lane 0 for the
        // warp, whose TMEM loads are warp-wide.
        int st = 1;
        if (lane == 0) {
            if (ntl == 0) {
                st = 0;
            } else if (!mbar_wait_or_abort(done_bar, 0u, flag, wait_limit)) {
                if (*flag == 0u) fail(2);
                st = 2;
            }
        }
        st = __shfl_sync(0xffffffffu, st, 0);
        tc_fence_after();
        const int row = q * 32 + lane;
#pragma unroll 1
        for (int kx = 0; kx < 3 && st != 2; kx++) {
            uint32_t v[N];
            if (st == 1) {
                const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(kx * N);
                tc_ld16(ta, *reinterpret_cast<uint32_t(*)[16]>(&v[0]));
                if constexpr (N == 32) tc_ld16(ta + 16, *reinterpret_cast<uint32_t(*)[16]>(&v[16]));
                tc_wait_ld();
            } else {
#pragma unroll
                for (int c = 0; c < N; c++) v[c] = 0u;
            }
            const int plane = row / 8, ch = row % 8;
            if (plane < L::NQ) {
                const int t = (plane / CCU) * 3 + kx, ci = (plane % CCU) * 8 + ch;
                if (ci < CIN) {
#pragma unroll
                    for (int co = 0; co < COUT; co++) pp[(t * CIN + ci) * COUT + co] = __uint_as_float(v[co]);
                }
            } else if (plane == L::NQ && kx == 0 && ch == 0) {
#pragma unroll
                for (int co = 0; co < COUT; co++) pp[9 * CIN * COUT + co] = __uint_as_float(v[co]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    // after an abort, wait (bounded, full limit) for this block's own copies
    // and MMAs before its TMEM and shared memory are given up
    if (*flag != 0u) {
        if (warp == 0 && lane == 0) {
#pragma unroll
            for (int k = 0; k < WNSTAGE; k++)
                if (last[k] >= 0) mbar_wait(full_bar(k), (uint32_t)((last[k] / WNSTAGE) & 1));
        }
        if (warp == 1 && lane == 0 && committed >= 0) {
            mbar_wait(empty_bar(committed % WNSTAGE), (uint32_t)((committed / WNSTAGE) & 1));
            if (done_sent) mbar_wait(done_bar, 0u);
        }
        __syncwarp();
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)L::TMEM_COLS)
                     : "memory");
    }
}

}  // namespace fwtc
