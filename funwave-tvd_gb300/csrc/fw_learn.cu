// fw_learn.cu -- the learned coarse-grid correction: a 4-layer 3x3
// convolutional network on the coarse grid (inputs eta, u, v, depth, MASK;
// 32 channels; outputs corrections of eta, u, v), its training (forward,
// backward, Adam) and its application to a running coarse context.
//
// Layout: activations channels-last (pixel-major, the channels of a pixel
// contiguous), pixel p = x + y*W + b*W*H with x the grid's I (cross-shore)
// direction.  Weights and activations are BF16 (weights rounded from an
// FP32 master copy before each use), every sum accumulates in FP32, the
// gradients and the Adam moments are FP32.  Zero padding at the grid edge.
//
// Layers: 5 (stored as 8) -> 32 ReLU -> 32 ReLU -> 32 ReLU -> 3.  Weight
// index [k][ci][co] with k = (ky+1)*3 + (kx+1) for the tap at (x+kx, y+ky).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <vector>

#include "fw_internal.h"

namespace {

constexpr int NL = 4;
constexpr int CIN0 = 8;      // 5 input channels padded to 8
constexpr int NIN = 5;
constexpr int HID = 32;
constexpr int NOUT = 3;
constexpr int LCIN[NL] = {CIN0, HID, HID, HID};
constexpr int LCOUT[NL] = {HID, HID, HID, NOUT};
constexpr int WG_BLOCKS = 304;  // wgrad partial blocks (2 per SM)

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ float bf(bf16 v) { return __bfloat162float(v); }

// Hidden activations (32 channels) are stored with their channel pairs
// permuted: pair P = c/2 sits at word (P % 4) * 4 + P / 4 of the pixel, so
// that the four words a tensor-core lane needs for one tap (pairs t, 4+t,
// 8+t, 12+t) are one 16-byte load and its outputs one 16-byte store.  The
// 8-channel input is stored in natural order.
template <int C> __device__ __forceinline__ int sidx(int c) {
    if constexpr (C == 32) {
        const int P = c >> 1;
        return (((P & 3) << 2) + (P >> 2)) * 2 + (c & 1);
    } else {
        return c;
    }
}

// ---------------------------------------------------------------------------
// forward of the 32-input-channel layers on the tensor cores: implicit GEMM
// with M = pixels (16 per warp tile, consecutive in memory), N = output
// channels (NT tiles of 8), K = 9 taps x 32 channels (18 steps of 16),
// mma.sync m16n8k16 BF16 x BF16 -> FP32.  Each lane loads its A rows (two
// pixels' channel pairs, zero outside the grid) straight from the
// channels-last activations; the weights sit in shared memory as BF16
// pairs [tap][co][ci/2], rows padded to 20 words (conflict-free).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const uint32_t l = __bfloat16_as_ushort(__float2bfloat16(lo));
    const uint32_t h = __bfloat16_as_ushort(__float2bfloat16(hi));
    return l | (h << 16);
}

__device__ __forceinline__ void mma_bf16(float *c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// epilogue of a warp tile: bias, ReLU, then the permuted BF16 layout (one
// 16-byte store per pixel and lane when COUT = 32) or natural FP32
template <int NT, int COUT, bool RELU, bool OUT_BF16>
__device__ __forceinline__ void store_tile(float (&acc)[NT][4], const float *bs, void *y, long long pa, long long pb,
                                           bool ina, bool inb, int t) {
    uint32_t wa[NT], wb[NT];
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        const int c = nt * 8 + 2 * t;
        float v[4] = {acc[nt][0] + bs[c], acc[nt][1] + bs[c + 1], acc[nt][2] + bs[c], acc[nt][3] + bs[c + 1]};
        if (RELU)
#pragma unroll
            for (int q = 0; q < 4; q++) v[q] = v[q] > 0.0f ? v[q] : 0.0f;
        if (OUT_BF16) {
            wa[nt] = pack_bf16(v[0], v[1]);
            wb[nt] = pack_bf16(v[2], v[3]);
        } else {
            float *yf = reinterpret_cast<float *>(y);
            if (ina && c < COUT) yf[pa * COUT + c] = v[0];
            if (ina && c + 1 < COUT) yf[pa * COUT + c + 1] = v[1];
            if (inb && c < COUT) yf[pb * COUT + c] = v[2];
            if (inb && c + 1 < COUT) yf[pb * COUT + c + 1] = v[3];
        }
    }
    if constexpr (OUT_BF16) {
        static_assert(COUT == 32 && NT == 4, "BF16 outputs are the 32-channel permuted layout");
        uint32_t *yw = reinterpret_cast<uint32_t *>(y);
        // pair nt*4 + t sits at word t*4 + nt
        if (ina) *reinterpret_cast<uint4 *>(yw + pa * 16 + 4 * t) = make_uint4(wa[0], wa[1], wa[2], wa[3]);
        if (inb) *reinterpret_cast<uint4 *>(yw + pb * 16 + 4 * t) = make_uint4(wb[0], wb[1], wb[2], wb[3]);
    }
}

// the first layer (8 natural input channels) on the tensor cores: a K step
// of 16 holds two taps (8 channels each), five steps cover the 9 taps plus
// one zero tap
__global__ void __launch_bounds__(128) k_conv8_fwd_mma(const bf16 *__restrict__ x, const float *__restrict__ w,
                                                       const float *__restrict__ bias, bf16 *y, int B, int H, int W) {
    constexpr int CIN = 8, COUT = 32, WS = 12;
    __shared__ uint32_t wT[5][COUT][WS];  // [k step][co][words: 4 of tap 2s, 4 of tap 2s+1]
    __shared__ float bs[COUT];
    for (int e = threadIdx.x; e < 5 * COUT * 8; e += blockDim.x) {
        const int wd = e % 8, co = (e / 8) % COUT, ks = e / (8 * COUT);
        const int tap = 2 * ks + (wd >> 2), cp = wd & 3;
        float lo = 0.0f, hi = 0.0f;
        if (tap < 9) {
            lo = w[((size_t)tap * CIN + 2 * cp) * COUT + co];
            hi = w[((size_t)tap * CIN + 2 * cp + 1) * COUT + co];
        }
        wT[ks][co][wd] = pack_bf16(lo, hi);
    }
    for (int e = threadIdx.x; e < COUT; e += blockDim.x) bs[e] = bias[e];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const long long npix = (long long)B * H * W;
    const long long ntile = (npix + 15) / 16;
    const uint32_t *xw = reinterpret_cast<const uint32_t *>(x);  // 4 words per pixel
    for (long long tile = (long long)blockIdx.x * 4 + warp; tile < ntile; tile += (long long)gridDim.x * 4) {
        const long long pa = tile * 16 + g, pb = pa + 8;
        const bool ina = pa < npix, inb = pb < npix;
        const int xa = (int)(pa % W), ya = (int)((pa / W) % H);
        const int xb = (int)(pb % W), yb = (int)((pb / W) % H);
        float acc[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
        for (int ks = 0; ks < 5; ks++) {
            uint32_t a[4];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int tap = 2 * ks + h;
                const int kx = tap % 3 - 1, ky = tap / 3 - 1;
                const bool va = tap < 9 && ina && xa + kx >= 0 && xa + kx < W && ya + ky >= 0 && ya + ky < H;
                const bool vb = tap < 9 && inb && xb + kx >= 0 && xb + kx < W && yb + ky >= 0 && yb + ky < H;
                a[2 * h] = va ? xw[(pa + (long long)ky * W + kx) * 4 + t] : 0u;
                a[2 * h + 1] = vb ? xw[(pb + (long long)ky * W + kx) * 4 + t] : 0u;
            }
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
                mma_bf16(acc[nt], a[0], a[1], a[2], a[3], wT[ks][nt * 8 + g][t], wT[ks][nt * 8 + g][4 + t]);
        }
        store_tile<4, COUT, true, true>(acc, bs, y, pa, pb, ina, inb, t);
    }
}

template <int NT, int COUT, bool RELU, bool OUT_BF16>
__global__ void __launch_bounds__(128) k_conv32_fwd_mma(const bf16 *__restrict__ x, const float *__restrict__ w,
                                                        const float *__restrict__ bias, void *y, int B, int H,
                                                        int W) {
    constexpr int CIN = 32, WS = 20;
    __shared__ uint32_t wT[9][NT * 8][WS];
    __shared__ float bs[NT * 8];
    for (int e = threadIdx.x; e < 9 * NT * 8 * 16; e += blockDim.x) {
        const int cp = e % 16, co = (e / 16) % (NT * 8), tap = e / (16 * NT * 8);
        float lo = 0.0f, hi = 0.0f;
        if (co < COUT) {
            lo = w[((size_t)tap * CIN + 2 * cp) * COUT + co];
            hi = w[((size_t)tap * CIN + 2 * cp + 1) * COUT + co];
        }
        wT[tap][co][cp] = pack_bf16(lo, hi);
    }
    for (int e = threadIdx.x; e < NT * 8; e += blockDim.x) bs[e] = e < COUT ? bias[e] : 0.0f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const long long npix = (long long)B * H * W;
    const long long ntile = (npix + 15) / 16;
    const uint32_t *xw = reinterpret_cast<const uint32_t *>(x);  // 16 words per pixel
    for (long long tile = (long long)blockIdx.x * 4 + warp; tile < ntile; tile += (long long)gridDim.x * 4) {
        const long long pa = tile * 16 + g, pb = pa + 8;
        const bool ina = pa < npix, inb = pb < npix;
        const int xa = (int)(pa % W), ya = (int)((pa / W) % H);
        const int xb = (int)(pb % W), yb = (int)((pb / W) % H);
        float acc[NT][4];
#pragma unroll
        for (int nt = 0; nt < NT; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
            const int kx = tap % 3 - 1, ky = tap / 3 - 1;
            const bool va = ina && xa + kx >= 0 && xa + kx < W && ya + ky >= 0 && ya + ky < H;
            const bool vb = inb && xb + kx >= 0 && xb + kx < W && yb + ky >= 0 && yb + ky < H;
            // words 4t..4t+3 of the permuted pixel: pairs t, 4+t, 8+t, 12+t
            const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
            const uint4 qa = va ? *reinterpret_cast<const uint4 *>(xw + (pa + (long long)ky * W + kx) * 16 + 4 * t) : z4;
            const uint4 qb = vb ? *reinterpret_cast<const uint4 *>(xw + (pb + (long long)ky * W + kx) * 16 + 4 * t) : z4;
#pragma unroll
            for (int ks = 0; ks < 2; ks++) {
                const uint32_t a0 = ks == 0 ? qa.x : qa.z, a2 = ks == 0 ? qa.y : qa.w;
                const uint32_t a1 = ks == 0 ? qb.x : qb.z, a3 = ks == 0 ? qb.y : qb.w;
#pragma unroll
                for (int nt = 0; nt < NT; nt++) {
                    const uint32_t b0 = wT[tap][nt * 8 + g][ks * 8 + t];
                    const uint32_t b1 = wT[tap][nt * 8 + g][ks * 8 + 4 + t];
                    mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
                }
            }
        }
        store_tile<NT, COUT, RELU, OUT_BF16>(acc, bs, y, pa, pb, ina, inb, t);
    }
}

// ---------------------------------------------------------------------------
// backward: dy of a layer's output (FP32) -> dx of its input (FP32), with the
// layer's ReLU applied to dy first (y = the layer's stored output)
// ---------------------------------------------------------------------------
template <int CIN, int COUT, bool RELU>
__global__ void __launch_bounds__(128) k_conv_dgrad(const float *__restrict__ dy, const bf16 *__restrict__ y,
                                                    const float *__restrict__ w, float *__restrict__ dx, int B,
                                                    int H, int W) {
    __shared__ float ws[9 * CIN * COUT];
    for (int e = threadIdx.x; e < 9 * CIN * COUT; e += blockDim.x) ws[e] = bf(__float2bfloat16(w[e]));
    __syncthreads();
    const long long npix = (long long)B * H * W;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int px = (int)(p % W), py = (int)((p / W) % H);
    float acc[CIN];
#pragma unroll
    for (int ci = 0; ci < CIN; ci++) acc[ci] = 0.0f;
    // output q = p - (kx, ky) read this input through tap k
    for (int ky = -1; ky <= 1; ky++) {
        if (py - ky < 0 || py - ky >= H) continue;
        for (int kx = -1; kx <= 1; kx++) {
            if (px - kx < 0 || px - kx >= W) continue;
            const long long q = p - (long long)ky * W - kx;
            const float *wk = ws + ((ky + 1) * 3 + (kx + 1)) * CIN * COUT;
            for (int co = 0; co < COUT; co++) {
                float g = dy[q * COUT + co];
                if (RELU && !(bf(y[q * COUT + sidx<COUT>(co)]) > 0.0f)) g = 0.0f;
#pragma unroll
                for (int ci = 0; ci < CIN; ci++) acc[ci] += wk[ci * COUT + co] * g;
            }
        }
    }
#pragma unroll
    for (int ci = 0; ci < CIN; ci++) dx[p * CIN + ci] = acc[ci];
}

// weight and bias gradients.  A tile is a row segment of TPX pixels; its
// three input rows (with one pixel of halo on each side, zero outside the
// grid) and its dy (with this layer's ReLU applied) are staged in shared
// memory, then every thread adds its share of the 9*CIN*COUT + COUT
// entries over the tile.  Each of the WG_BLOCKS blocks walks many tiles and
// writes one partial; k_wgrad_reduce adds the partials.
constexpr int TPX = 64;
template <int CIN, int COUT, bool RELU>
__global__ void __launch_bounds__(256) k_conv_wgrad(const bf16 *__restrict__ x, const float *__restrict__ dy,
                                                    const bf16 *__restrict__ y, float *__restrict__ part, int B,
                                                    int H, int W) {
    constexpr int E = 9 * CIN * COUT + COUT;
    constexpr int NE = (E + 255) / 256;
    __shared__ float xs[3][TPX + 2][CIN];
    __shared__ float dys[TPX][COUT];
    float acc[NE];
#pragma unroll
    for (int r = 0; r < NE; r++) acc[r] = 0.0f;
    const int tiles_x = (W + TPX - 1) / TPX;
    const long long ntiles = (long long)B * H * tiles_x;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tx = (int)(tile % tiles_x);
        const long long row = tile / tiles_x;  // b*H + y
        const int py = (int)(row % H);
        const int x0 = tx * TPX;
        __syncthreads();
        for (int e = threadIdx.x; e < 3 * (TPX + 2) * CIN; e += blockDim.x) {
            const int ci = e % CIN, c = (e / CIN) % (TPX + 2), r = e / (CIN * (TPX + 2));
            const int gx = x0 + c - 1, gy = py + r - 1;
            float v = 0.0f;
            if (gx >= 0 && gx < W && gy >= 0 && gy < H)
                v = bf(x[((row + (r - 1)) * W + gx) * CIN + sidx<CIN>(ci)]);
            xs[r][c][ci] = v;
        }
        for (int e = threadIdx.x; e < TPX * COUT; e += blockDim.x) {
            const int co = e % COUT, t = e / COUT;
            float g = 0.0f;
            if (x0 + t < W) {
                const long long q = (row * W + x0 + t) * COUT;
                g = dy[q + co];
                if (RELU && !(bf(y[q + sidx<COUT>(co)]) > 0.0f)) g = 0.0f;
            }
            dys[t][co] = g;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < NE; r++) {
            const int e = threadIdx.x + r * 256;
            if (e >= E) continue;
            float s = 0.0f;
            if (e < 9 * CIN * COUT) {
                const int co = e % COUT, ci = (e / COUT) % CIN, k = e / (COUT * CIN);
                const int kx = k % 3, ky = k / 3;  // 0..2: tap offset + 1
                for (int t = 0; t < TPX; t++) s += xs[ky][t + kx][ci] * dys[t][co];
            } else {
                const int co = e - 9 * CIN * COUT;
                for (int t = 0; t < TPX; t++) s += dys[t][co];
            }
            acc[r] += s;
        }
    }
#pragma unroll
    for (int r = 0; r < NE; r++) {
        const int e = threadIdx.x + r * 256;
        if (e < E) part[(size_t)blockIdx.x * E + e] = acc[r];
    }
}

__global__ void k_wgrad_reduce(const float *part, int nblocks, int E, float *gw, float *gb, int nw) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    float s = 0.0f;
    for (int b = 0; b < nblocks; b++) s += part[(size_t)b * E + e];
    if (e < nw) gw[e] = s;
    else gb[e - nw] = s;
}

// inputs: FP32 [npix][5] -> BF16 [npix][8] (three zero channels)
__global__ void k_pack_input(const float *in, bf16 *x, long long npix) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
#pragma unroll
    for (int c = 0; c < CIN0; c++) x[p * CIN0 + c] = __float2bfloat16(c < NIN ? in[p * NIN + c] : 0.0f);
}

// masked mean squared error and its gradient w.r.t. the output
__global__ void k_loss(const float *out, const float *target, const float *wmask, long long npix, float inv_n,
                       float *dy, double *loss) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (p < npix) {
        const float m = wmask[p];
        for (int c = 0; c < NOUT; c++) {
            const float d = out[p * NOUT + c] - target[p * NOUT + c];
            l += m * d * d;
            dy[p * NOUT + c] = 2.0f * m * d * inv_n;
        }
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)(l * inv_n));
}

__global__ void k_adam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// zero the gradients of the padding input channels 5..7 of layer 0
__global__ void k_zero_pad_grad(float *gw0) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 9 * CIN0 * HID) return;
    const int ci = (e / HID) % CIN0;
    if (ci >= NIN) gw0[e] = 0.0f;
}

// the network's input from a context's interior cells (x = I fastest)
template <typename T>
__global__ void k_corr_input(fw::Grid g, fw::Fields<T> f, float *in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mglob || j >= g.Nglob) return;
    const size_t id = (size_t)(i + g.ib) + (size_t)(j + g.jb) * g.pitch;
    const long long p = (long long)i + (long long)j * g.Mglob;
    in[p * NIN + 0] = (float)f.Eta[id];
    in[p * NIN + 1] = (float)f.U[id];
    in[p * NIN + 2] = (float)f.V[id];
    in[p * NIN + 3] = (float)(f.Depth[id] / (T)FW_NET_DEPTH_SCALE);
    in[p * NIN + 4] = f.MASK[id] ? 1.0f : 0.0f;
}

// sums over the wet interior cells: [0] the eta correction, [1] the count,
// [2] max |correction| (bits of a non-negative double)
template <typename T>
__global__ void k_corr_sums(fw::Grid g, fw::Fields<T> f, const float *out, double *sums) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    float se = 0.0f, sc = 0.0f, mx = 0.0f;
    if (i < g.Mglob && j < g.Nglob) {
        const size_t id = (size_t)(i + g.ib) + (size_t)(j + g.jb) * g.pitch;
        const long long p = (long long)i + (long long)j * g.Mglob;
        if (f.MASK[id]) {
            const float inv = (float)(1.0 / FW_NET_OUT_SCALE);
            se = out[p * NOUT] * inv;
            sc = 1.0f;
            mx = fmaxf(fabsf(out[p * NOUT]), fmaxf(fabsf(out[p * NOUT + 1]), fabsf(out[p * NOUT + 2]))) * inv;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_xor_sync(0xffffffffu, se, o);
        sc += __shfl_xor_sync(0xffffffffu, sc, o);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (((threadIdx.x + threadIdx.y * blockDim.x) & 31) == 0) {
        atomicAdd(&sums[0], (double)se);
        atomicAdd(&sums[1], (double)sc);
        atomicMax((unsigned long long *)&sums[2], (unsigned long long)__double_as_longlong((double)mx));
    }
}

template <typename T>
__global__ void k_corr_apply(fw::Grid g, fw::Fields<T> f, const float *out, const double *sums, double max_corr) {
    // the fallback: a correction above max_corr anywhere leaves the plain step
    if (!(sums[2] <= max_corr) || !(sums[1] == sums[1])) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mglob || j >= g.Nglob) return;
    const size_t id = (size_t)(i + g.ib) + (size_t)(j + g.jb) * g.pitch;
    if (!f.MASK[id]) return;
    const long long p = (long long)i + (long long)j * g.Mglob;
    const double inv = 1.0 / FW_NET_OUT_SCALE;
    const double mean = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
    const T de = (T)(out[p * NOUT] * inv - mean), du = (T)(out[p * NOUT + 1] * inv), dv = (T)(out[p * NOUT + 2] * inv);
    f.Eta[id] += de;
    f.H[id] += de;
    const T h = f.H[id] > (T)0 ? f.H[id] : (T)0;
    f.U[id] += du;
    f.V[id] += dv;
    f.HU[id] += h * du;
    f.HV[id] += h * dv;
    f.Ubar[id] += h * du;
    f.Vbar[id] += h * dv;
}

unsigned long long splitmix(unsigned long long &s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

// ---------------------------------------------------------------------------
// the network object
// ---------------------------------------------------------------------------
struct fw_net {
    size_t woff[NL], boff[NL], nparam = 0;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 master, grads, Adam moments
    long long adam_t = 0;
    // workspace for npix_cap pixels
    long long npix_cap = 0;
    bf16 *act[NL] = {nullptr};  // act[0] = packed input, act[l] = output of layer l-1 (l = 1..3)
    float *out = nullptr;       // output of the last layer, FP32 [npix][3]
    float *dbuf[2] = {nullptr, nullptr};
    float *part = nullptr;
    double *loss = nullptr;
    float *corr_in = nullptr;   // fw_correct's input tensor
};

namespace {

void free_ws(fw_net *n) {
    for (auto &a : n->act) {
        if (a) cudaFree(a);
        a = nullptr;
    }
    for (auto &b : n->dbuf) {
        if (b) cudaFree(b);
        b = nullptr;
    }
    if (n->out) cudaFree(n->out);
    if (n->corr_in) cudaFree(n->corr_in);
    n->out = nullptr;
    n->corr_in = nullptr;
    n->npix_cap = 0;
}

int ensure_ws(fw_net *n, long long npix) {
    if (npix <= n->npix_cap) return FW_OK;
    free_ws(n);
    bool ok = cudaMalloc(&n->act[0], (size_t)npix * CIN0 * sizeof(bf16)) == cudaSuccess;
    for (int l = 1; l < NL && ok; l++) ok = cudaMalloc(&n->act[l], (size_t)npix * HID * sizeof(bf16)) == cudaSuccess;
    ok = ok && cudaMalloc(&n->out, (size_t)npix * NOUT * sizeof(float)) == cudaSuccess;
    for (int k = 0; k < 2 && ok; k++) ok = cudaMalloc(&n->dbuf[k], (size_t)npix * HID * sizeof(float)) == cudaSuccess;
    ok = ok && cudaMalloc(&n->corr_in, (size_t)npix * NIN * sizeof(float)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_ws(n);
        return FW_ERR_OOM;
    }
    n->npix_cap = npix;
    return FW_OK;
}

unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

void forward(fw_net *n, const float *in, long long npix, int B, int H, int W, cudaStream_t s) {
    k_pack_input<<<nblk(npix, 256), 256, 0, s>>>(in, n->act[0], npix);
    // every layer on the tensor cores: a persistent grid of warps over
    // 16-pixel tiles
    const long long ntile = (npix + 15) / 16;
    const unsigned gm = (unsigned)std::min<long long>((ntile + 3) / 4, 152LL * 16);
    k_conv8_fwd_mma<<<gm, 128, 0, s>>>(n->act[0], n->w + n->woff[0], n->w + n->boff[0], n->act[1], B, H, W);
    k_conv32_fwd_mma<4, HID, true, true><<<gm, 128, 0, s>>>(n->act[1], n->w + n->woff[1], n->w + n->boff[1],
                                                             n->act[2], B, H, W);
    k_conv32_fwd_mma<4, HID, true, true><<<gm, 128, 0, s>>>(n->act[2], n->w + n->woff[2], n->w + n->boff[2],
                                                             n->act[3], B, H, W);
    k_conv32_fwd_mma<1, NOUT, false, false><<<gm, 128, 0, s>>>(n->act[3], n->w + n->woff[3], n->w + n->boff[3],
                                                                n->out, B, H, W);
}

template <int CIN, int COUT, bool RELU>
void wgrad(fw_net *n, int l, const bf16 *x, const float *dy, const bf16 *y, long long npix, int B, int H, int W,
           cudaStream_t s) {
    constexpr int E = 9 * CIN * COUT + COUT;
    k_conv_wgrad<CIN, COUT, RELU><<<WG_BLOCKS, 256, 0, s>>>(x, dy, y, n->part, B, H, W);
    k_wgrad_reduce<<<nblk(E, 256), 256, 0, s>>>(n->part, WG_BLOCKS, E, n->g + n->woff[l], n->g + n->boff[l],
                                                 9 * CIN * COUT);
}

void backward(fw_net *n, long long npix, int B, int H, int W, cudaStream_t s) {
    const unsigned gb = nblk(npix, 128);
    float *dy = n->dbuf[0], *dx = n->dbuf[1];
    // dy of the last layer is in dbuf[0] ([npix][3])
    wgrad<HID, NOUT, false>(n, 3, n->act[3], dy, nullptr, npix, B, H, W, s);
    k_conv_dgrad<HID, NOUT, false><<<gb, 128, 0, s>>>(dy, nullptr, n->w + n->woff[3], dx, B, H, W);
    for (int l = 2; l >= 1; l--) {
        std::swap(dy, dx);  // dy: gradient of act[l+1]
        wgrad<HID, HID, true>(n, l, n->act[l], dy, n->act[l + 1], npix, B, H, W, s);
        k_conv_dgrad<HID, HID, true><<<gb, 128, 0, s>>>(dy, n->act[l + 1], n->w + n->woff[l], dx, B, H, W);
    }
    std::swap(dy, dx);  // gradient of act[1]
    wgrad<CIN0, HID, true>(n, 0, n->act[0], dy, n->act[1], npix, B, H, W, s);
    k_zero_pad_grad<<<nblk(9 * CIN0 * HID, 256), 256, 0, s>>>(n->g + n->woff[0]);
}

}  // namespace

namespace {
template <typename T> int correct(fw_ctx *c, fw_net *n, double max_corr, int *applied) {
    const fw::Grid &g = c->g;
    fw::Fields<T> &f = c->F<T>();
    const long long npix = (long long)g.Mglob * g.Nglob;
    int rc = ensure_ws(n, npix);
    if (rc != FW_OK) return rc;
    cudaStream_t s = c->stream;
    const dim3 b(32, 8), gr((g.Mglob + 31) / 32, (g.Nglob + 7) / 8);
    k_corr_input<T><<<gr, b, 0, s>>>(g, f, n->corr_in);
    forward(n, n->corr_in, npix, 1, g.Nglob, g.Mglob, s);
    double *sums = n->loss;  // 3 doubles of scratch after the loss slot
    cudaMemsetAsync(sums, 0, 4 * sizeof(double), s);
    k_corr_sums<T><<<gr, b, 0, s>>>(g, f, n->out, sums + 1);
    k_corr_apply<T><<<gr, b, 0, s>>>(g, f, n->out, sums + 1, max_corr);
    if (applied) {
        // only a caller that asks waits for the decision
        double h[4];
        cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return FW_ERR_CUDA;
        *applied = (h[3] <= max_corr && h[2] == h[2]) ? 1 : 0;
    }
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}
}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int fw_net_create(unsigned long long seed, fw_net **out) {
    if (!out) return FW_ERR_BAD_PARAM;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FW_ERR_NO_DEVICE;
    }
    fw_net *n = new fw_net();
    size_t off = 0;
    for (int l = 0; l < NL; l++) {
        n->woff[l] = off;
        off += (size_t)9 * LCIN[l] * LCOUT[l];
        n->boff[l] = off;
        off += LCOUT[l];
    }
    n->nparam = off;
    // He-normal weights (Box-Muller on SplitMix64), zero biases, zero
    // weights for the padding input channels; the last layer scaled by 0.1
    std::vector<float> h(off, 0.0f);
    unsigned long long s = seed;
    for (int l = 0; l < NL; l++) {
        const int cin_real = l == 0 ? NIN : LCIN[l];
        const double sd = std::sqrt(2.0 / (9.0 * cin_real)) * (l == NL - 1 ? 0.1 : 1.0);
        for (int k = 0; k < 9; k++)
            for (int ci = 0; ci < LCIN[l]; ci++)
                for (int co = 0; co < LCOUT[l]; co++) {
                    const double u1 = ((splitmix(s) >> 11) + 1.0) / 9007199254740993.0;
                    const double u2 = (splitmix(s) >> 11) / 9007199254740992.0;
                    const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
                    h[n->woff[l] + ((size_t)k * LCIN[l] + ci) * LCOUT[l] + co] = ci < cin_real ? (float)(z * sd) : 0.0f;
                }
    }
    bool ok = cudaMalloc(&n->w, off * sizeof(float)) == cudaSuccess && cudaMalloc(&n->g, off * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&n->m, off * sizeof(float)) == cudaSuccess && cudaMalloc(&n->v, off * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&n->part, (size_t)WG_BLOCKS * (9 * HID * HID + HID) * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&n->loss, 4 * sizeof(double)) == cudaSuccess;
    ok = ok && cudaMemcpy(n->w, h.data(), off * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemset(n->g, 0, off * sizeof(float)) == cudaSuccess && cudaMemset(n->m, 0, off * sizeof(float)) == cudaSuccess &&
         cudaMemset(n->v, 0, off * sizeof(float)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        fw_net_destroy(n);
        return FW_ERR_OOM;
    }
    *out = n;
    return FW_OK;
}

int fw_net_destroy(fw_net *n) {
    if (!n) return FW_ERR_BAD_PARAM;
    cudaDeviceSynchronize();
    free_ws(n);
    for (float *p : {n->w, n->g, n->m, n->v, n->part})
        if (p) cudaFree(p);
    if (n->loss) cudaFree(n->loss);
    delete n;
    return FW_OK;
}

long long fw_net_num_params(fw_net *n) { return n ? (long long)n->nparam : -1; }

int fw_net_get_params(fw_net *n, float *host) {
    if (!n || !host) return FW_ERR_BAD_PARAM;
    return cudaMemcpy(host, n->w, n->nparam * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_set_params(fw_net *n, const float *host) {
    if (!n || !host) return FW_ERR_BAD_PARAM;
    return cudaMemcpy(n->w, host, n->nparam * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_get_grads(fw_net *n, float *host) {
    if (!n || !host) return FW_ERR_BAD_PARAM;
    return cudaMemcpy(host, n->g, n->nparam * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_forward(fw_net *n, const float *x, int B, int H, int W, float *y, void *stream) {
    if (!n || !x || !y || B <= 0 || H <= 0 || W <= 0) return FW_ERR_BAD_PARAM;
    const long long npix = (long long)B * H * W;
    int rc = ensure_ws(n, npix);
    if (rc != FW_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    forward(n, x, npix, B, H, W, s);
    cudaMemcpyAsync(y, n->out, (size_t)npix * NOUT * sizeof(float), cudaMemcpyDeviceToDevice, s);
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_loss_grad(fw_net *n, const float *x, const float *target, const float *wmask, int B, int H, int W,
                     double *loss, void *stream) {
    if (!n || !x || !target || !wmask || B <= 0 || H <= 0 || W <= 0) return FW_ERR_BAD_PARAM;
    const long long npix = (long long)B * H * W;
    int rc = ensure_ws(n, npix);
    if (rc != FW_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    forward(n, x, npix, B, H, W, s);
    cudaMemsetAsync(n->loss, 0, sizeof(double), s);
    k_loss<<<nblk(npix, 256), 256, 0, s>>>(n->out, target, wmask, npix, 1.0f / (float)npix, n->dbuf[0], n->loss);
    backward(n, npix, B, H, W, s);
    if (loss) {
        cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
    }
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_adam(fw_net *n, float lr, float beta1, float beta2, float eps, void *stream) {
    if (!n || !(lr > 0.0f)) return FW_ERR_BAD_PARAM;
    n->adam_t++;
    const float c1 = 1.0f - std::pow(beta1, (float)n->adam_t), c2 = 1.0f - std::pow(beta2, (float)n->adam_t);
    k_adam<<<nblk((long long)n->nparam, 256), 256, 0, (cudaStream_t)stream>>>(n->w, n->g, n->m, n->v,
                                                                              (long long)n->nparam, lr, beta1,
                                                                              beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_correct(fw_ctx *c, fw_net *n, double max_corr, int *applied) {
    if (!c || !n || !c->initialized) return FW_ERR_BAD_PARAM;
    if (c->p.precision == FW_PREC_FP64) return correct<double>(c, n, max_corr, applied);
    return correct<float>(c, n, max_corr, applied);
}

}  // extern "C"
