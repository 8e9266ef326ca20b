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
#include <cuda.h>
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

// The device address of fw_dt_scratch differs between CUDA contexts: a
// context that is reset (cudaDeviceReset) or a caller's own non-primary
// context loads this module again, at another address, and a reset primary
// context may come back under the same handle.  So the address is cached
// under the context's unique id (cuCtxGetId: never reused in a process).
constexpr int MAX_CONTEXTS = 64;
struct ScratchSlot {
    unsigned long long ctx_id;
    double *ptr;
};
ScratchSlot g_slots[MAX_CONTEXTS] = {};
int g_nslots = 0;
std::mutex g_mutex;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

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

// cuCtxGetCurrent and cuCtxGetId through the runtime's driver entry point
// (the library does not link libcuda).
template <typename F>
F driver_fn(const char *name) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (F)p;
}

// The id of the context current on this thread; 0 when there is none.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        get = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
        get_id = driver_fn<CtxGetIdFn>("cuCtxGetId");
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get || !get_id || get(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// The device address of fw_dt_scratch in the current context, looked up
// with cudaGetSymbolAddress once per context (in the usual case one per
// device: the device's primary context).  Host code must not pass
// fw_dt_scratch itself to a kernel: on the host that name is only a
// stand-in for the device array.
int scratch_for_current_context(double **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return FW_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    unsigned long long id = current_context_id();
    if (id) {
        for (int k = 0; k < g_nslots; k++)
            if (g_slots[k].ctx_id == id) {
                *out = g_slots[k].ptr;
                return FW_OK;
            }
    }
    // The lookup binds the device's primary context to this thread when no
    // context was current, so the id is read again after it.
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, fw_dt_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return FW_ERR_CUDA;
    }
    if (!id) id = current_context_id();
    if (!id) return FW_ERR_CUDA;
    // a small table: when it is full the oldest entry goes
    if (g_nslots == MAX_CONTEXTS) {
        for (int i = 1; i < MAX_CONTEXTS; i++) g_slots[i - 1] = g_slots[i];
        g_nslots--;
    }
    g_slots[g_nslots++] = {id, (double *)p};
    *out = (double *)p;
    return FW_OK;
}

// True when ptr is device (or managed) memory that the current device can
// use as a kernel argument.  Host memory, pinned or not, and memory of
// another GPU are refused, so a wrong pointer becomes FW_ERR_BAD_PARAM
// instead of a fault inside the kernel.
bool on_current_device(const void *ptr, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeDevice) return a.device == dev;
    if (a.type == cudaMemoryTypeManaged) return true;
    return false;
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
    const int st = scratch_for_current_context(&scratch);
    if (st != FW_OK) return st;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FW_ERR_CUDA;
    if (!on_current_device(U, dev) || !on_current_device(V, dev) || !on_current_device(H, dev) ||
        !on_current_device(DT, dev) || (TIME && !on_current_device(TIME, dev)))
        return FW_ERR_BAD_PARAM;
    cudaStream_t s = (cudaStream_t)stream;
    k_dt_blocks<<<(unsigned)nblocks, DT_THREADS, 0, s>>>(ncell, DX, DY, MinDepthFrc, U, V, H, scratch);
    if (cudaGetLastError() != cudaSuccess) return FW_ERR_CUDA;
    k_dt_reduce<<<1, 1024, 0, s>>>((int)nblocks, CFL, dt_fixed, scratch, DT, TIME);
    if (cudaGetLastError() != cudaSuccess) return FW_ERR_CUDA;
    return FW_OK;
}
