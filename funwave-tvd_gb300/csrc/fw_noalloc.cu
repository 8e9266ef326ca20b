// fw_noalloc.cu -- ESTIMATE_DT on caller-owned device arrays, with no device
// allocation at all.
//
// Some callers of this library cannot call cudaMalloc: a Fortran host whose
// device arrays are owned by its own OpenACC or CUDA Fortran runtime, a code
// that runs inside a memory pool it must not grow, or a real-time loop where
// every allocation is forbidden after start-up.  fw_estimate_dt_device gives
// them the CFL time step of ESTIMATE_DT (misc.F:216-296) on arrays they
// already hold on the GPU, with the reference's own argument list
// ESTIMATE_DT(M,N,DX,DY,U,V,H,MinDepthFrc,DT,CFL,TIME).
//
// Its only scratch is the file-scope array fw_dt_scratch below: one double
// per block of FW_DT_CELLS_PER_BLOCK cells, FW_DT_MAX_BLOCKS blocks (512 KB,
// held by every GPU that loads the library until the process exits).  The
// arithmetic per cell is the one of the context path (k_dt_only and
// k_dt_final), so both give the same DT bit for bit.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "funwave_gpu.h"

namespace {

constexpr double GRAV = 9.81;
constexpr double SMALL = 0.000001;
constexpr double LARGE = 999999.0;

constexpr int DT_THREADS = 256;
constexpr int DT_CELLS_PER_THREAD = 8;
constexpr long long FW_DT_CELLS_PER_BLOCK = (long long)DT_THREADS * DT_CELLS_PER_THREAD;  // 2048
constexpr int FW_DT_MAX_BLOCKS = 65536;

// Per-block CFL minima of one call.  Every call writes the slots it reads
// before it reads them, so nothing here has to start at zero.
static __device__ __align__(256) double fw_dt_scratch[FW_DT_MAX_BLOCKS];

constexpr int MAX_DEVICES = 64;
double *g_scratch[MAX_DEVICES] = {nullptr};
std::mutex g_mutex;

// dx / (|u| + sqrt(g max(H, MinDepthFrc))) and the same in y (misc.F:243-262)
__device__ __forceinline__ double cell_dt(double u, double v, double h, double dx, double dy, double mdf) {
    const double c = sqrt(GRAV * fmax(h, mdf));
    double t1 = fabs(u) + c;
    double m = (t1 < SMALL) ? dx / SMALL : dx / t1;
    t1 = fabs(v) + c;
    const double t2 = (t1 < SMALL) ? dy / SMALL : dy / t1;
    return (t2 < m) ? t2 : m;
}

__global__ void __launch_bounds__(DT_THREADS) k_dt_blocks(long long ncell, double dx, double dy, double mdf,
                                                          const double *__restrict__ U,
                                                          const double *__restrict__ V,
                                                          const double *__restrict__ H, double *scratch) {
    __shared__ double sm[DT_THREADS / 32];
    const long long base = (long long)blockIdx.x * FW_DT_CELLS_PER_BLOCK;
    double v = 1.0e30;
    for (int k = 0; k < DT_CELLS_PER_THREAD; k++) {
        const long long id = base + (long long)k * DT_THREADS + threadIdx.x;
        if (id < ncell) v = fmin(v, cell_dt(U[id], V[id], H[id], dx, dy, mdf));
    }
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < DT_THREADS / 32 ? sm[threadIdx.x] : 1.0e30;
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) scratch[blockIdx.x] = v;
    }
}

// DT = CFL * min over the blocks (with the DT_fixed halving of misc.F:266-
// 290 when dt_fixed > 0); TIME += DT (misc.F:294)
__global__ void __launch_bounds__(1024) k_dt_reduce(int nblocks, double cfl, double dt_fixed,
                                                    const double *scratch, double *dt, double *time) {
    __shared__ double sm[32];
    double v = 1.0e30;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v = fmin(v, scratch[b]);
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 1.0e30;
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) {
            double tmp3 = v;
            if (!(tmp3 < LARGE)) tmp3 = LARGE;
            const double dt_tmp = cfl * tmp3;
            double d = dt_tmp;
            if (dt_fixed > 0.0) {
                d = dt_fixed;
                for (int k = 0; k < 4096 && d > dt_tmp; k++) d = d / 2.0;
            }
            *dt = d;
            if (time) *time = *time + d;
        }
    }
}

// The device address of fw_dt_scratch for the current device, looked up
// once per device.  Host code must not pass fw_dt_scratch itself to a
// kernel: on the host that name is only a stand-in for the device array.
int scratch_for_current_device(double **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FW_ERR_NO_DEVICE;
    if (dev < 0 || dev >= MAX_DEVICES) return FW_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, fw_dt_scratch) != cudaSuccess || !p) return FW_ERR_CUDA;
        g_scratch[dev] = (double *)p;
    }
    *out = g_scratch[dev];
    return FW_OK;
}

}  // namespace

extern "C" int fw_estimate_dt_device(int Mloc, int Nloc, double DX, double DY, const double *U, const double *V,
                                     const double *H, double MinDepthFrc, double CFL, double dt_fixed,
                                     double *DT, double *TIME, void *stream) {
    if (Mloc <= 0 || Nloc <= 0 || !U || !V || !H || !DT) return FW_ERR_BAD_PARAM;
    if (!(DX > 0.0) || !(DY > 0.0) || !(CFL > 0.0)) return FW_ERR_BAD_PARAM;
    const long long ncell = (long long)Mloc * (long long)Nloc;
    const long long nblocks = (ncell + FW_DT_CELLS_PER_BLOCK - 1) / FW_DT_CELLS_PER_BLOCK;
    if (nblocks > FW_DT_MAX_BLOCKS) return FW_ERR_BAD_PARAM;  // beyond FW_DT_DEVICE_MAX_CELLS
    double *scratch = nullptr;
    const int st = scratch_for_current_device(&scratch);
    if (st != FW_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    k_dt_blocks<<<(unsigned)nblocks, DT_THREADS, 0, s>>>(ncell, DX, DY, MinDepthFrc, U, V, H, scratch);
    if (cudaGetLastError() != cudaSuccess) return FW_ERR_CUDA;
    k_dt_reduce<<<1, 1024, 0, s>>>((int)nblocks, CFL, dt_fixed, scratch, DT, TIME);
    if (cudaGetLastError() != cudaSuccess) return FW_ERR_CUDA;
    return FW_OK;
}
