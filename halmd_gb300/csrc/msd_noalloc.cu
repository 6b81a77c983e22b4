// msd_noalloc.cu — mean-square displacement of one pair of samples that
// allocates no device memory: the per-block partial sums live in a
// file-scope __device__ array of fixed size instead of a buffer the caller
// or the engine allocates.
//
// Who needs it: callers that must not allocate at the point of the call.
// cudaMalloc and cudaFree synchronise the whole device, so a sampler that
// runs between the asynchronous step launches of a running simulation would
// stall every stream on the GPU for each sample; and a job server that has
// reserved nearly all of HBM for its engine has no room left for per-call
// buffers, so an allocation there can fail in the middle of a run.  This
// entry point takes device pointers, launches two kernels on the caller's
// stream and returns without synchronising or allocating.
//
// The arithmetic per block and the order in which the block results are
// merged are those of the MSD kernels the dynamics path uses (Welford update
// per thread, pairwise Chan merge across the block, blocks of 8192
// particles merged in index order), so both give the same (count, mean,
// variance) for the same two samples.
#include <cuda.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "engine.h"

namespace hmd {

constexpr uint32_t NOALLOC_CHUNK = 8192;    // particles per block
constexpr uint32_t NOALLOC_BLOCKS = 4096;   // most blocks one call may use
constexpr int NOALLOC_MAX_DEVICES = 64;

static_assert((uint64_t)NOALLOC_CHUNK * NOALLOC_BLOCKS == HMD_MSD_NOALLOC_MAX_PARTICLES,
              "the header's particle limit must match the scratch size");

// (count, mean, M2) per block: 4096 x 3 doubles = 96 KiB per device.  Every
// partial a call reads was written earlier in the same call, so nothing here
// has to start at zero.
static __device__ __align__(256) double g_msd_scratch[3 * NOALLOC_BLOCKS];

namespace {

__device__ __forceinline__ void merge(double& n, double& m, double& v, double n2, double m2, double v2)
{
    if (n2 > 0) {
        const double c = n + n2;
        const double diff = m - m2;
        v = v + v2 + diff * diff * n * n2 / c;
        m = (n * m + n2 * m2) / c;
        n = c;
    }
}

__global__ void __launch_bounds__(256) k_msd_noalloc_partial(const double* r1, const double* r2, uint32_t count,
                                                             double* partial)
{
    const uint32_t b = blockIdx.x;
    const uint32_t beg = b * NOALLOC_CHUNK;
    const uint32_t end = min(beg + NOALLOC_CHUNK, count);
    double n = 0, m = 0, v = 0;
    for (uint32_t k = beg + threadIdx.x; k < end; k += blockDim.x) {
        const double dx = r2[3 * (size_t)k] - r1[3 * (size_t)k];
        const double dy = r2[3 * (size_t)k + 1] - r1[3 * (size_t)k + 1];
        const double dz = r2[3 * (size_t)k + 2] - r1[3 * (size_t)k + 2];
        const double x = dx * dx + dy * dy + dz * dz;
        const double t = x - m;
        n += 1;
        m += t / n;
        v += t * (x - m);
    }
    __shared__ double sn[256], sm[256], sv[256];
    sn[threadIdx.x] = n; sm[threadIdx.x] = m; sv[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            double a = sn[threadIdx.x], am = sm[threadIdx.x], av = sv[threadIdx.x];
            merge(a, am, av, sn[threadIdx.x + o], sm[threadIdx.x + o], sv[threadIdx.x + o]);
            sn[threadIdx.x] = a; sm[threadIdx.x] = am; sv[threadIdx.x] = av;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[3 * b] = sn[0]; partial[3 * b + 1] = sm[0]; partial[3 * b + 2] = sv[0];
    }
}

// one thread merges the blocks in index order (a fixed order: the result
// does not depend on scheduling)
__global__ void k_msd_noalloc_merge(const double* partial, uint32_t nblk, double* out)
{
    if (threadIdx.x != 0) return;
    double n = 0, m = 0, v = 0;
    for (uint32_t b = 0; b < nblk; ++b) merge(n, m, v, partial[3 * b], partial[3 * b + 1], partial[3 * b + 2]);
    out[0] = n;
    out[1] = m;
    out[2] = n > 0 ? v / n : 0.0;
}

// Driver calls reached through the runtime's entry-point table, so the
// library does not link the driver library itself (it must still load on
// machines without a GPU driver, where nothing is launched).
struct Driver {
    CUresult (*ctx_get_current)(CUcontext*) = nullptr;
    CUresult (*ctx_get_id)(CUcontext, unsigned long long*) = nullptr;
    CUresult (*mem_get_address_range)(CUdeviceptr*, size_t*, CUdeviceptr) = nullptr;
};

template <typename F>
void driver_entry(const char* name, F& fn)
{
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
        (void)cudaGetLastError();
        throw Error(HMD_ERR_CUDA, std::string("hmd_msd_pair_noalloc: driver entry point ") + name + " unavailable");
    }
    fn = reinterpret_cast<F>(p);
}

std::mutex g_setup_mutex;
Driver g_driver;
bool g_driver_ready = false;

// Scratch addresses by CUDA context.  A __device__ array's address belongs
// to the context that loaded the module, not to the device: after
// cudaDeviceReset the primary context, and with it the module and the
// address, are new, and a context the caller made current through the
// driver API has its own copy.  So the address is looked up once per
// context (by its unique id) and again when the current context is one not
// seen before.
struct ScratchEntry {
    unsigned long long ctx_id;
    double* ptr;
};
ScratchEntry g_scratch[NOALLOC_MAX_DEVICES];
int g_nscratch = 0;

const Driver& driver()
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_driver_ready) {
        driver_entry("cuCtxGetCurrent", g_driver.ctx_get_current);
        driver_entry("cuCtxGetId", g_driver.ctx_get_id);
        driver_entry("cuMemGetAddressRange", g_driver.mem_get_address_range);
        g_driver_ready = true;
    }
    return g_driver;
}

// Device address of g_msd_scratch in the current context.  The first lookup
// in a context may load this library's device code there; host code never
// uses the symbol itself as an address.
double* scratch_for_current_context()
{
    const Driver& drv = driver();
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (drv.ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx || drv.ctx_get_id(ctx, &id) != CUDA_SUCCESS)
        throw Error(HMD_ERR_CUDA, "hmd_msd_pair_noalloc: no current CUDA context");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    for (int k = 0; k < g_nscratch; ++k)
        if (g_scratch[k].ctx_id == id) return g_scratch[k].ptr;
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_msd_scratch);
    if (e != cudaSuccess || !p) {
        (void)cudaGetLastError();
        throw Error(HMD_ERR_CUDA, std::string("hmd_msd_pair_noalloc: cudaGetSymbolAddress of the scratch array "
                                              "failed: ") + cudaGetErrorString(e));
    }
    // a full table reuses a slot (contexts of past resets are gone)
    const int k = g_nscratch < NOALLOC_MAX_DEVICES ? g_nscratch++ : (int)(id % NOALLOC_MAX_DEVICES);
    g_scratch[k] = ScratchEntry{id, static_cast<double*>(p)};
    return g_scratch[k].ptr;
}

// the kernels read `bytes` bytes behind r1 and r2 and write 24 behind out:
// each must be device (or managed) memory of the current device, 8-byte
// aligned, inside one allocation that holds all of those bytes
void check_pointer(const void* p, int dev, const char* what, size_t bytes)
{
    if (!p) throw Error(HMD_ERR_INVALID, std::string("hmd_msd_pair_noalloc: ") + what + " is null");
    if (reinterpret_cast<uintptr_t>(p) % alignof(double))
        throw Error(HMD_ERR_INVALID, std::string("hmd_msd_pair_noalloc: ") + what + " is not 8-byte aligned");
    cudaPointerAttributes a;
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw Error(HMD_ERR_INVALID, std::string("hmd_msd_pair_noalloc: ") + what + ": " + cudaGetErrorString(e));
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
        throw Error(HMD_ERR_INVALID, std::string("hmd_msd_pair_noalloc: ") + what + " is not device memory");
    if (a.type == cudaMemoryTypeDevice && a.device != dev)
        throw Error(HMD_ERR_INVALID, std::string("hmd_msd_pair_noalloc: ") + what + " is on device " +
                                         std::to_string(a.device) + ", the current device is " + std::to_string(dev));
    CUdeviceptr base = 0;
    size_t size = 0;
    const CUdeviceptr at = reinterpret_cast<CUdeviceptr>(p);
    if (driver().mem_get_address_range(&base, &size, at) != CUDA_SUCCESS)
        throw Error(HMD_ERR_INVALID, std::string("hmd_msd_pair_noalloc: ") + what + " is not inside an allocation");
    if (at - base > size || size - (at - base) < bytes)
        throw Error(HMD_ERR_INVALID, std::string("hmd_msd_pair_noalloc: ") + what + " holds " +
                                         std::to_string(size - (at - base)) + " bytes, the call needs " +
                                         std::to_string(bytes));
}

} // namespace

void msd_pair_noalloc(const double* origin, const double* position, uint32_t count, double* out, cudaStream_t st)
{
    if (count > HMD_MSD_NOALLOC_MAX_PARTICLES)
        throw Error(HMD_ERR_INVALID, "hmd_msd_pair_noalloc: " + std::to_string(count) + " particles exceed the limit of " +
                                         std::to_string(HMD_MSD_NOALLOC_MAX_PARTICLES) +
                                         " set by its fixed scratch array; use the dynamics path for larger samples");
    int dev = -1;
    HMD_CUDA(cudaGetDevice(&dev));
    if (count > 0) {
        check_pointer(origin, dev, "origin", 3 * sizeof(double) * (size_t)count);
        check_pointer(position, dev, "position", 3 * sizeof(double) * (size_t)count);
    }
    check_pointer(out, dev, "out", 3 * sizeof(double));
    double* partial = scratch_for_current_context();
    const uint32_t nblk = (count + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK;
    if (nblk > 0) k_msd_noalloc_partial<<<nblk, 256, 0, st>>>(origin, position, count, partial);
    k_msd_noalloc_merge<<<1, 32, 0, st>>>(partial, nblk, out);
    HMD_CUDA(cudaGetLastError());
}

} // namespace hmd
