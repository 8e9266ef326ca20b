// fw_learn.cu -- the learned coarse-grid correction: a 4-layer 3x3
// convolutional network on the coarse grid (inputs eta, u, v, depth, MASK;
// 32 channels; outputs corrections of eta, u, v), its training (forward,
// backward, Adam) and its application to a running coarse context.
//
// Layout: the network's FP32 inputs and outputs are channels-last
// ([pixel][channel]), pixel p = x + y*W + b*W*H with x the grid's I
// (cross-shore) direction.  Weights and activations are BF16 (weights
// rounded from an FP32 master copy into packed images before use), every
// sum accumulates in FP32, the weight gradients and the Adam moments are
// FP32.  Zero padding at the grid edge.
//
// Layers: 5 (stored as 16 channels, weights for 8) -> 32 ReLU -> 32 ReLU
// -> 32 ReLU -> 3.  Weight index [k][ci][co] with k = (ky+1)*3 + (kx+1) for
// the tap at (x+kx, y+ky).
//
// The forward convolutions, the data gradients and the weight and bias
// gradients of the backward pass run on the tcgen05 tensor cores
// (fw_tc.cuh).  Their BF16 activations and gradients are stored
// chunk-planar with a zero border (fwtc::act_idx); the network's FP32
// inputs and outputs are plain [pixel][channel].  The backward pass carries
// the gradient of each hidden activation in BF16 with the ReLU mask already
// applied (dy * [act > 0]), as the tensor-core data-gradient kernel writes
// it; the weight gradients sum those BF16 values times the BF16 inputs in
// FP32 (per CTA in TMEM, then over the CTAs).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <vector>

#include "fw_internal.h"
#include "fw_tc.cuh"

namespace {

constexpr int NL = 4;
constexpr int CIN0 = 8;      // 5 input channels padded to 8 (weights)
constexpr int XC0 = 16;      // channels of the stored input (one K step of the tensor cores)
constexpr int GC3 = 16;      // channels of the stored output gradient (3 used)
constexpr int NIN = 5;
constexpr int HID = 32;
constexpr int NOUT = 3;
constexpr int LCIN[NL] = {CIN0, HID, HID, HID};
constexpr int LCOUT[NL] = {HID, HID, HID, NOUT};
constexpr long long WG_PART = 304LL * (9 * 32 * 32 + 32);  // floats of the weight-gradient partials

typedef __nv_bfloat16 bf16;

// BF16 of a float, round to nearest even
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const uint32_t l = __bfloat16_as_ushort(__float2bfloat16(lo));
    const uint32_t h = __bfloat16_as_ushort(__float2bfloat16(hi));
    return l | (h << 16);
}

__global__ void k_wgrad_reduce(const float *part, int nblocks, int E, float *gw, float *gb, int nw) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    float s = 0.0f;
    for (int b = 0; b < nblocks; b++) s += part[(size_t)b * E + e];
    if (e < nw) gw[e] = s;
    else gb[e - nw] = s;
}

// inputs: FP32 [npix][5] -> the padded BF16 input of 2 chunks (channels
// 5..15 zero)
__global__ void k_pack_input(const float *in, bf16 *x, int B, int H, int W) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)B * H * W) return;
    const int px = (int)(p % W), py = (int)((p / W) % H), pb = (int)(p / ((long long)W * H));
    float v[NIN];
#pragma unroll
    for (int c = 0; c < NIN; c++) v[c] = in[p * NIN + c];
    const fwtc::ActGeom g{B, H, W, XC0 / 8};
    uint4 *xq = reinterpret_cast<uint4 *>(x);
    const long long o = fwtc::act_idx(g, pb, py, 0, px);
    xq[o] = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], 0.0f), 0u);
    xq[o + W + 2] = make_uint4(0u, 0u, 0u, 0u);
}

// masked mean squared error and its gradient w.r.t. the output, stored as
// a padded BF16 activation of 2 chunks (channels 3..15 zero)
__global__ void k_loss(const float *out, const float *target, const float *wmask, int B, int H, int W, float inv_n,
                       bf16 *dy, double *loss) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long npix = (long long)B * H * W;
    float l = 0.0f;
    if (p < npix) {
        const float m = wmask[p];
        float g[NOUT];
        for (int c = 0; c < NOUT; c++) {
            const float d = out[p * NOUT + c] - target[p * NOUT + c];
            l += m * d * d;
            g[c] = 2.0f * m * d * inv_n;
        }
        const int px = (int)(p % W), py = (int)((p / W) % H), pb = (int)(p / ((long long)W * H));
        const fwtc::ActGeom ga{B, H, W, GC3 / 8};
        uint4 *dq = reinterpret_cast<uint4 *>(dy);
        const long long o = fwtc::act_idx(ga, pb, py, 0, px);
        dq[o] = make_uint4(pack_bf16(g[0], g[1]), pack_bf16(g[2], 0.0f), 0u, 0u);
        dq[o + W + 2] = make_uint4(0u, 0u, 0u, 0u);
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

// The correction acts on the interior cells whose neighbourhood of
// (2 band + 1) x (2 band + 1) cells is wet (MASK; band 1 by default, at
// most the ghost width 3; 0: every wet cell): not at the shoreline, where
// the wet/dry switch is a threshold the network does not see.  (MASK9 is
// not this test: with VISCOSITY_BREAKING it is 1 on every interior cell,
// dry ones included.)
template <typename T>
__device__ __forceinline__ bool wet_band(const fw::Grid &g, const fw::Fields<T> &f, size_t id, int band) {
    const uint8_t *m = f.MASK;
    const long long p = g.pitch;
    for (int b = -band; b <= band; b++)
        for (int a = -band; a <= band; a++)
            if (!m[(long long)id + a + b * p]) return false;
    return true;
}
// Sums over those cells: [0] the eta correction, [1] the count, [2] max
// |correction|, [3] the largest amount by which a corrected total depth
// would fall below MinDepth (bits of non-negative doubles); [4] the
// decision of k_corr_apply (1 applied, 0 the plain step kept)
template <typename T>
__global__ void k_corr_sums(fw::Grid g, fw::Fields<T> f, const float *out, double *sums, float min_depth,
                            int band) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    float se = 0.0f, sc = 0.0f, mx = 0.0f, dry = 0.0f;
    if (i < g.Mglob && j < g.Nglob) {
        const size_t id = (size_t)(i + g.ib) + (size_t)(j + g.jb) * g.pitch;
        const long long p = (long long)i + (long long)j * g.Mglob;
        if (wet_band(g, f, id, band)) {
            const float inv = (float)(1.0 / FW_NET_OUT_SCALE);
            se = out[p * NOUT] * inv;
            sc = 1.0f;
            mx = fmaxf(fabsf(out[p * NOUT]), fmaxf(fabsf(out[p * NOUT + 1]), fabsf(out[p * NOUT + 2]))) * inv;
            dry = fmaxf(0.0f, min_depth - ((float)f.H[id] + se));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_xor_sync(0xffffffffu, se, o);
        sc += __shfl_xor_sync(0xffffffffu, sc, o);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        dry = fmaxf(dry, __shfl_xor_sync(0xffffffffu, dry, o));
    }
    if (((threadIdx.x + threadIdx.y * blockDim.x) & 31) == 0) {
        atomicAdd(&sums[0], (double)se);
        atomicAdd(&sums[1], (double)sc);
        atomicMax((unsigned long long *)&sums[2], (unsigned long long)__double_as_longlong((double)mx));
        atomicMax((unsigned long long *)&sums[3], (unsigned long long)__double_as_longlong((double)dry));
    }
}

// Whether a correction is applied, the same on every thread from the sums:
// no component above max_corr; a finite result; no wet cell pushed to or
// below MinDepth (the correction would move the shoreline and so change the
// volume through UPDATE_MASK); and a volume drift of the raw eta correction
// (its mean, which the projection removes) of at most half of max_corr:
// a network whose output rises or falls the whole water level is off its
// training data.  Otherwise the plain step stands.
__device__ __forceinline__ bool corr_ok(const double *sums, double max_corr) {
    const double mean = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
    return sums[2] <= max_corr && sums[1] == sums[1] && mean == mean && !(sums[3] > 0.0) &&
           fabs(mean) <= 0.5 * max_corr;
}

template <typename T>
__global__ void k_corr_apply(fw::Grid g, fw::Fields<T> f, const float *out, double *sums, double max_corr,
                             int band) {
    const bool ok = corr_ok(sums, max_corr);
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) sums[4] = ok ? 1.0 : 0.0;
    if (!ok) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mglob || j >= g.Nglob) return;
    const size_t id = (size_t)(i + g.ib) + (size_t)(j + g.jb) * g.pitch;
    if (!wet_band(g, f, id, band)) return;
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
    // packed BF16 weight images of the tensor-core convolutions: the four
    // forward layers, then the data gradients of layers 1..3; rebuilt when
    // the master weights change (wver != img_ver)
    bf16 *img = nullptr;
    size_t img_off[NL + 3] = {0};
    unsigned long long wver = 1, img_ver = 0;
    int *status = nullptr;      // set by a tensor-core kernel whose bounded wait expired
    unsigned wait_limit = fwtc::WAIT_LIMIT;  // polls of those waits (fw_net_set_wait_limit)
    // workspace: FP32 buffers for npix_cap pixels; padded BF16 activations
    // (fwtc::act_idx) of cap16 / cap32 bytes, laid out for the batch shape
    // sB x sH x sW (their zero borders are set when the shape changes)
    long long npix_cap = 0;
    size_t cap16 = 0, cap32 = 0;
    int sB = 0, sH = 0, sW = 0;
    bf16 *act[NL] = {nullptr};  // act[0] = packed input (2 chunks), act[l] = output of layer l-1 (4 chunks)
    float *out = nullptr;       // output of the last layer, FP32 [npix][3]
    bf16 *gout = nullptr;       // gradient of the output (2 chunks)
    bf16 *gbuf[2] = {nullptr, nullptr};  // masked gradients of hidden activations (4 chunks)
    float *part = nullptr;
    double *loss = nullptr;
    float *corr_in = nullptr;   // fw_correct's input tensor
    // the checks of the last fw_correct that reported its decision: mean
    // raw eta correction, cells corrected, max |correction|, MinDepth
    // violation, decision
    double last_check[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    int shore_band = 1;         // fw_correct acts where the (2 band + 1)^2 neighbourhood is wet
    // fw_correct_run's graph of two (step + correction) pairs and what it was
    // captured with
    cudaGraphExec_t cexec = nullptr;
    fw_ctx *cctx = nullptr;
    long long cstate = 0;
    int ctune[FW_TUNE_LEN] = {0};
    double cmax = 0.0;
};

namespace {

// the images: {cin chunks, N} of each
constexpr int IMG_CINC[NL + 3] = {2, 4, 4, 4, 4, 4, 2};
constexpr int IMG_N[NL + 3] = {32, 32, 32, 16, 32, 32, 32};

size_t img_elems(int i) { return (size_t)9 * IMG_CINC[i] * IMG_N[i] * 8; }

void free_ws(fw_net *n) {
    for (auto &a : n->act) {
        if (a) cudaFree(a);
        a = nullptr;
    }
    for (auto &b : n->gbuf) {
        if (b) cudaFree(b);
        b = nullptr;
    }
    for (void *p : {(void *)n->out, (void *)n->corr_in, (void *)n->gout})
        if (p) cudaFree(p);
    n->out = nullptr;
    n->corr_in = nullptr;
    n->gout = nullptr;
    n->npix_cap = 0;
    n->cap16 = n->cap32 = 0;
    n->sB = n->sH = n->sW = 0;
}

// buffers for a batch of B images of H x W; a new shape zeroes the padded
// activations (their borders are the convolutions' zero padding)
int ensure_ws(fw_net *n, int B, int H, int W, cudaStream_t s) {
    const long long npix = (long long)B * H * W;
    const size_t need16 = fwtc::act_bytes(fwtc::ActGeom{B, H, W, 2});
    const size_t need32 = fwtc::act_bytes(fwtc::ActGeom{B, H, W, 4});
    if (npix > n->npix_cap || need16 > n->cap16 || need32 > n->cap32) {
        const long long np = std::max(npix, n->npix_cap);
        const size_t c16 = std::max(need16, n->cap16), c32 = std::max(need32, n->cap32);
        free_ws(n);
        bool ok = cudaMalloc(&n->act[0], c16) == cudaSuccess;
        for (int l = 1; l < NL && ok; l++) ok = cudaMalloc(&n->act[l], c32) == cudaSuccess;
        ok = ok && cudaMalloc(&n->out, (size_t)np * NOUT * sizeof(float)) == cudaSuccess;
        ok = ok && cudaMalloc(&n->gout, c16) == cudaSuccess;
        for (int k = 0; k < 2 && ok; k++) ok = cudaMalloc(&n->gbuf[k], c32) == cudaSuccess;
        ok = ok && cudaMalloc(&n->corr_in, (size_t)np * NIN * sizeof(float)) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            free_ws(n);
            return FW_ERR_OOM;
        }
        n->npix_cap = np;
        n->cap16 = c16;
        n->cap32 = c32;
    }
    if (n->sB != B || n->sH != H || n->sW != W) {
        bool ok = cudaMemsetAsync(n->act[0], 0, n->cap16, s) == cudaSuccess &&
                  cudaMemsetAsync(n->gout, 0, n->cap16, s) == cudaSuccess;
        for (int l = 1; l < NL && ok; l++) ok = cudaMemsetAsync(n->act[l], 0, n->cap32, s) == cudaSuccess;
        for (int k = 0; k < 2 && ok; k++) ok = cudaMemsetAsync(n->gbuf[k], 0, n->cap32, s) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            return FW_ERR_CUDA;
        }
        n->sB = B;
        n->sH = H;
        n->sW = W;
    }
    return FW_OK;
}

unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// the shared-memory size of one tensor-core convolution, set once (outside
// any stream capture: fw_net_create sets every one the network uses)
template <int CINC, int N, int EPI, int NOUTF> bool conv_attr() {
    static bool attr = false;
    if (!attr) {
        using Lt = fwtc::Layout<CINC, N>;
        if (cudaFuncSetAttribute(fwtc::k_conv_tc<CINC, N, EPI, NOUTF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Lt::BYTES) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        attr = true;
    }
    return true;
}

bool conv_attrs_all() {
    using namespace fwtc;
    return conv_attr<2, 32, EPI_RELU_BF16, 0>() && conv_attr<4, 32, EPI_RELU_BF16, 0>() &&
           conv_attr<4, 16, EPI_LINEAR_F32, NOUT>() && conv_attr<2, 32, EPI_MASK_BF16, 0>() &&
           conv_attr<4, 32, EPI_MASK_BF16, 0>();
}

// the weight-gradient kernels' shared-memory size, set once like conv_attr
template <int CIN, int COUT, int XCC, int DYCC> bool wgrad_attr() {
    static bool attr = false;
    if (!attr) {
        constexpr int CCU = (CIN + 7) / 8;
        if (cudaFuncSetAttribute(fwtc::k_wgrad_tc<XCC, CCU, DYCC, CIN, COUT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 fwtc::WLayout<CCU, DYCC>::BYTES) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        attr = true;
    }
    return true;
}

bool wgrad_attrs_all() {
    return wgrad_attr<HID, NOUT, HID / 8, GC3 / 8>() && wgrad_attr<HID, HID, HID / 8, HID / 8>() &&
           wgrad_attr<CIN0, HID, XC0 / 8, HID / 8>();
}

// SMs of the current device (0 on error)
int sm_count() {
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            nsm = 0;
        }
    }
    return nsm;
}

template <int CINC, int N, int EPI, int NOUTF>
int conv_tc(const bf16 *x, const bf16 *img, const float *bias, const bf16 *act, void *y, int B, int H, int W,
            int *status, unsigned wait_limit, cudaStream_t s) {
    using Lt = fwtc::Layout<CINC, N>;
    auto k = fwtc::k_conv_tc<CINC, N, EPI, NOUTF>;
    if (!conv_attr<CINC, N, EPI, NOUTF>()) return FW_ERR_CUDA;
    const int nsm = sm_count();
    if (!nsm) return FW_ERR_CUDA;
    const long long ntiles = (long long)((W + fwtc::TPX - 1) / fwtc::TPX) * ((H + fwtc::TROWS - 1) / fwtc::TROWS) * B;
    const unsigned grid = (unsigned)std::min<long long>(ntiles, (long long)nsm * Lt::PER_SM);
    k<<<grid, 64 + 32 * fwtc::EPI_WARPS, Lt::BYTES, s>>>(x, img, bias, act, y, H, W, B, status,
                                                                      wait_limit);
    return FW_OK;
}

// The status word of the tensor-core kernels, read after the stream's work:
// a bounded wait that ran out becomes FW_ERR_TIMEOUT, and the word is
// cleared so that the network can be used again.
int take_status(fw_net *n, int st, cudaStream_t s) {
    if (st == 0) return FW_OK;
    if (cudaMemsetAsync(n->status, 0, sizeof(int), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        return FW_ERR_CUDA;
    return FW_ERR_TIMEOUT;
}

// the tensor-core kernels number their tiles in an int
bool shape_ok(int B, int H, int W) {
    return B > 0 && H > 0 && W > 0 &&
           (long long)((W + fwtc::TPX - 1) / fwtc::TPX) * ((H + fwtc::TROWS - 1) / fwtc::TROWS) * B < (1LL << 31) &&
           (long long)((W + fwtc::WKT - 1) / fwtc::WKT) * H * B < (1LL << 31);
}

void pack_images(fw_net *n, cudaStream_t s) {
    if (n->img_ver == n->wver) return;
    for (int i = 0; i < NL + 3; i++) {
        const int l = i < NL ? i : i - NL + 1;  // images 4..6 are the data gradients of layers 1..3
        const int tot = (int)img_elems(i);
        fwtc::k_pack_wimg<<<nblk(tot, 256), 256, 0, s>>>(n->w + n->woff[l], LCIN[l], LCOUT[l], IMG_CINC[i], IMG_N[i],
                                                         i >= NL ? 1 : 0, n->img + n->img_off[i]);
    }
    n->img_ver = n->wver;
}

int forward(fw_net *n, const float *in, long long npix, int B, int H, int W, cudaStream_t s) {
    using namespace fwtc;
    pack_images(n, s);
    k_pack_input<<<nblk(npix, 256), 256, 0, s>>>(in, n->act[0], B, H, W);
    const bf16 *im = n->img;
    int rc = conv_tc<2, 32, EPI_RELU_BF16, 0>(n->act[0], im + n->img_off[0], n->w + n->boff[0], nullptr,
                                              n->act[1], B, H, W, n->status, n->wait_limit, s);
    for (int l = 1; l < 3 && rc == FW_OK; l++)
        rc = conv_tc<4, 32, EPI_RELU_BF16, 0>(n->act[l], im + n->img_off[l], n->w + n->boff[l], nullptr,
                                              n->act[l + 1], B, H, W, n->status, n->wait_limit, s);
    if (rc == FW_OK)
        rc = conv_tc<4, 16, EPI_LINEAR_F32, NOUT>(n->act[3], im + n->img_off[3], n->w + n->boff[3], nullptr,
                                                  n->out, B, H, W, n->status, n->wait_limit, s);
    return rc;
}

// weight and bias gradients of layer l on the tensor cores
// (fwtc::k_wgrad_tc): one partial per CTA, then k_wgrad_reduce adds them
template <int CIN, int COUT, int XCC, int DYCC>
int wgrad(fw_net *n, int l, const bf16 *x, const bf16 *dy, int B, int H, int W, cudaStream_t s) {
    constexpr int CCU = (CIN + 7) / 8, E = 9 * CIN * COUT + COUT;
    using Lw = fwtc::WLayout<CCU, DYCC>;
    if (!wgrad_attr<CIN, COUT, XCC, DYCC>()) return FW_ERR_CUDA;
    const int nsm = sm_count();
    if (!nsm) return FW_ERR_CUDA;
    const long long ntiles = (long long)((W + fwtc::WKT - 1) / fwtc::WKT) * H * B;
    // the partial buffer holds WG_PART floats
    const long long cap = WG_PART / E;
    const unsigned grid = (unsigned)std::min<long long>(std::min<long long>(ntiles, (long long)nsm * Lw::PER_SM), cap);
    fwtc::k_wgrad_tc<XCC, CCU, DYCC, CIN, COUT><<<grid, 192, Lw::BYTES, s>>>(x, dy, n->part, H, W, B, n->status,
                                                                            n->wait_limit);
    k_wgrad_reduce<<<nblk(E, 256), 256, 0, s>>>(n->part, (int)grid, E, n->g + n->woff[l], n->g + n->boff[l],
                                                 9 * CIN * COUT);
    return FW_OK;
}

// the output gradient is in gout; the images are current (forward ran)
int backward(fw_net *n, int B, int H, int W, cudaStream_t s) {
    using namespace fwtc;
    const bf16 *im = n->img;
    bf16 *ga = n->gbuf[0], *gb = n->gbuf[1];
    int rc = wgrad<HID, NOUT, HID / 8, GC3 / 8>(n, 3, n->act[3], n->gout, B, H, W, s);
    // gradient of act[3] (the output of layer 2), masked by its ReLU
    if (rc == FW_OK)
        rc = conv_tc<2, 32, EPI_MASK_BF16, 0>(n->gout, im + n->img_off[NL + 2], nullptr, n->act[3], ga, B, H, W,
                                              n->status, n->wait_limit, s);
    for (int l = 2; l >= 1 && rc == FW_OK; l--) {
        rc = wgrad<HID, HID, HID / 8, HID / 8>(n, l, n->act[l], ga, B, H, W, s);
        if (rc == FW_OK)
            rc = conv_tc<4, 32, EPI_MASK_BF16, 0>(ga, im + n->img_off[NL + l - 1], nullptr, n->act[l], gb, B, H, W,
                                                  n->status, n->wait_limit, s);
        std::swap(ga, gb);
    }
    if (rc == FW_OK) rc = wgrad<CIN0, HID, XC0 / 8, HID / 8>(n, 0, n->act[0], ga, B, H, W, s);
    if (rc != FW_OK) return rc;
    k_zero_pad_grad<<<nblk(9 * CIN0 * HID, 256), 256, 0, s>>>(n->g + n->woff[0]);
    return FW_OK;
}

}  // namespace

namespace {
// the correction's launches on the context's stream (no host wait, so a
// stream capture may hold them); the workspace and images are ready
template <typename T> int correct_enqueue(fw_ctx *c, fw_net *n, double max_corr) {
    const fw::Grid &g = c->g;
    fw::Fields<T> &f = c->F<T>();
    const long long npix = (long long)g.Mglob * g.Nglob;
    cudaStream_t s = c->stream;
    const dim3 b(32, 8), gr((g.Mglob + 31) / 32, (g.Nglob + 7) / 8);
    k_corr_input<T><<<gr, b, 0, s>>>(g, f, n->corr_in);
    int rc = forward(n, n->corr_in, npix, 1, g.Nglob, g.Mglob, s);
    if (rc != FW_OK) return rc;
    double *sums = n->loss;  // 5 doubles of scratch after the loss slot
    if (cudaMemsetAsync(sums, 0, 6 * sizeof(double), s) != cudaSuccess) return FW_ERR_CUDA;
    k_corr_sums<T><<<gr, b, 0, s>>>(g, f, n->out, sums + 1, (float)c->p.min_depth, n->shore_band);
    k_corr_apply<T><<<gr, b, 0, s>>>(g, f, n->out, sums + 1, max_corr, n->shore_band);
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

template <typename T> int correct(fw_ctx *c, fw_net *n, double max_corr, int *applied) {
    const fw::Grid &g = c->g;
    if (!shape_ok(1, g.Nglob, g.Mglob)) return FW_ERR_BAD_PARAM;
    cudaStream_t s = c->stream;
    int rc = ensure_ws(n, 1, g.Nglob, g.Mglob, s);
    if (rc != FW_OK) return rc;
    rc = correct_enqueue<T>(c, n, max_corr);
    if (rc != FW_OK) return rc;
    double *sums = n->loss;
    if (applied) {
        // only a caller that asks waits for the decision
        double h[6];
        int st = 0;
        cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&st, n->status, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return FW_ERR_CUDA;
        if (st != 0) return take_status(n, st, s);
        *applied = h[5] == 1.0 ? 1 : 0;
        for (int k = 0; k < 5; k++) n->last_check[k] = h[k + 1];
        n->last_check[0] = h[2] > 0.0 ? h[1] / h[2] : 0.0;  // the mean, not the sum
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
              cudaMalloc(&n->part, (size_t)WG_PART * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&n->loss, 8 * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&n->status, sizeof(int)) == cudaSuccess;
    size_t ioff = 0;
    for (int i = 0; i < NL + 3; i++) {
        n->img_off[i] = ioff;
        ioff += img_elems(i);
    }
    ok = ok && cudaMalloc(&n->img, ioff * sizeof(bf16)) == cudaSuccess;
    ok = ok && conv_attrs_all() && wgrad_attrs_all();
    ok = ok && cudaMemset(n->status, 0, sizeof(int)) == cudaSuccess;
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

int fw_net_set_shore_band(fw_net *n, int cells) {
    if (!n || cells < 0 || cells > 3) return FW_ERR_BAD_PARAM;
    n->shore_band = cells;
    // fw_correct_run's graph holds the old band
    if (n->cexec) {
        cudaGraphExecDestroy(n->cexec);
        n->cexec = nullptr;
    }
    return FW_OK;
}

int fw_net_set_wait_limit(fw_net *n, unsigned polls) {
    if (!n) return FW_ERR_BAD_PARAM;
    n->wait_limit = polls ? polls : fwtc::WAIT_LIMIT;
    // fw_correct_run's graph holds the old limit
    if (n->cexec) {
        cudaGraphExecDestroy(n->cexec);
        n->cexec = nullptr;
    }
    return FW_OK;
}

int fw_net_destroy(fw_net *n) {
    if (!n) return FW_ERR_BAD_PARAM;
    cudaDeviceSynchronize();
    free_ws(n);
    for (float *p : {n->w, n->g, n->m, n->v, n->part})
        if (p) cudaFree(p);
    if (n->loss) cudaFree(n->loss);
    if (n->img) cudaFree(n->img);
    if (n->cexec) cudaGraphExecDestroy(n->cexec);
    if (n->status) cudaFree(n->status);
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
    n->wver++;
    return cudaMemcpy(n->w, host, n->nparam * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_get_grads(fw_net *n, float *host) {
    if (!n || !host) return FW_ERR_BAD_PARAM;
    return cudaMemcpy(host, n->g, n->nparam * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_forward(fw_net *n, const float *x, int B, int H, int W, float *y, void *stream) {
    if (!n || !x || !y || !shape_ok(B, H, W)) return FW_ERR_BAD_PARAM;
    const long long npix = (long long)B * H * W;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = ensure_ws(n, B, H, W, s);
    if (rc != FW_OK) return rc;
    rc = forward(n, x, npix, B, H, W, s);
    if (rc != FW_OK) return rc;
    cudaMemcpyAsync(y, n->out, (size_t)npix * NOUT * sizeof(float), cudaMemcpyDeviceToDevice, s);
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_loss_grad(fw_net *n, const float *x, const float *target, const float *wmask, int B, int H, int W,
                     double *loss, void *stream) {
    if (!n || !x || !target || !wmask || !shape_ok(B, H, W)) return FW_ERR_BAD_PARAM;
    const long long npix = (long long)B * H * W;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = ensure_ws(n, B, H, W, s);
    if (rc != FW_OK) return rc;
    rc = forward(n, x, npix, B, H, W, s);
    if (rc != FW_OK) return rc;
    cudaMemsetAsync(n->loss, 0, sizeof(double), s);
    k_loss<<<nblk(npix, 256), 256, 0, s>>>(n->out, target, wmask, B, H, W, 1.0f / (float)npix, n->gout, n->loss);
    rc = backward(n, B, H, W, s);
    if (rc != FW_OK) return rc;
    if (loss) {
        int st = 0;
        cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&st, n->status, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return FW_ERR_CUDA;
        if (st != 0) return take_status(n, st, s);
    }
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

int fw_net_adam(fw_net *n, float lr, float beta1, float beta2, float eps, void *stream) {
    if (!n || !(lr > 0.0f)) return FW_ERR_BAD_PARAM;
    n->adam_t++;
    n->wver++;
    const float c1 = 1.0f - std::pow(beta1, (float)n->adam_t), c2 = 1.0f - std::pow(beta2, (float)n->adam_t);
    k_adam<<<nblk((long long)n->nparam, 256), 256, 0, (cudaStream_t)stream>>>(n->w, n->g, n->m, n->v,
                                                                              (long long)n->nparam, lr, beta1,
                                                                              beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? FW_OK : FW_ERR_CUDA;
}

// nsteps of (fw_step + fw_correct without waiting), two pairs per replay
// of a captured graph; status as fw_step's
int fw_correct_run(fw_ctx *c, fw_net *n, int nsteps, double max_corr, int *status) {
    if (!c || !n || !c->initialized || nsteps < 0) return FW_ERR_BAD_PARAM;
    if (status) *status = FW_OK;
    if (nsteps == 0) return FW_OK;
    const fw::Grid &g = c->g;
    if (!shape_ok(1, g.Nglob, g.Mglob)) return FW_ERR_BAD_PARAM;
    int rc = ensure_ws(n, 1, g.Nglob, g.Mglob, c->stream);
    if (rc != FW_OK) return rc;
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    pack_images(n, c->stream);  // before any capture: the graph reads the images
    if ((rc = fw::reset_step_max(c)) != FW_OK) return rc;
    auto pair = [&]() -> int {
        int r = fw::enqueue_one_step(c);
        if (r == FW_OK) r = fp64 ? correct_enqueue<double>(c, n, max_corr) : correct_enqueue<float>(c, n, max_corr);
        return r;
    };
    for (int s2 = 0; s2 + 2 <= nsteps; s2 += 2) {
        const bool stale = !n->cexec || n->cctx != c || n->cstate != fw::buffer_state(c) ||
                           std::memcmp(n->ctune, c->tune, sizeof(n->ctune)) != 0 || n->cmax != max_corr;
        if (stale) {
            if (n->cexec) cudaGraphExecDestroy(n->cexec);
            n->cexec = nullptr;
            const long long st = fw::buffer_state(c);
            cudaGraph_t gr;
            if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                cudaGetLastError();
                return FW_ERR_CUDA;
            }
            int r1 = pair();
            if (r1 == FW_OK) r1 = pair();
            const cudaError_t e1 = cudaStreamEndCapture(c->stream, &gr);
            if (r1 != FW_OK || e1 != cudaSuccess) {
                cudaGetLastError();
                if (e1 == cudaSuccess) cudaGraphDestroy(gr);
                return r1 != FW_OK ? r1 : FW_ERR_CUDA;
            }
            const cudaError_t e2 = cudaGraphInstantiate(&n->cexec, gr, 0);
            cudaGraphDestroy(gr);
            if (e2 != cudaSuccess) {
                cudaGetLastError();
                n->cexec = nullptr;
                return FW_ERR_CUDA;
            }
            n->cctx = c;
            n->cstate = st;
            std::memcpy(n->ctune, c->tune, sizeof(n->ctune));
            n->cmax = max_corr;
        }
        if (cudaGraphLaunch(n->cexec, c->stream) != cudaSuccess) {
            cudaGetLastError();
            return FW_ERR_CUDA;
        }
    }
    if (nsteps % 2 && (rc = pair()) != FW_OK) return rc;
    rc = fw::step_status(c, status);
    int st = 0;
    if (cudaMemcpy(&st, n->status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return FW_ERR_CUDA;
    if (st != 0) return take_status(n, st, c->stream);
    return rc;
}

int fw_net_last_check(fw_net *n, double *out) {
    if (!n || !out) return FW_ERR_BAD_PARAM;
    for (int k = 0; k < 5; k++) out[k] = n->last_check[k];
    return FW_OK;
}

int fw_correct(fw_ctx *c, fw_net *n, double max_corr, int *applied) {
    if (!c || !n || !c->initialized) return FW_ERR_BAD_PARAM;
    if (c->p.precision == FW_PREC_FP64) return correct<double>(c, n, max_corr, applied);
    return correct<float>(c, n, max_corr, applied);
}

}  // extern "C"
