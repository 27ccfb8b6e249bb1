// fs_noalloc.cu -- RANLUX state-table seeding that allocates no device memory.
//
// fs_ranlux_init stages the caller's 64-bit seed values in a device buffer it allocates
// for the call.  Some callers cannot let a library allocate: a host that hands all device
// memory to its own pool up front and forbids cudaMalloc afterwards, or a foreign-language
// binding whose memory manager must own every device allocation.  fs_ranlux_init_noalloc
// does the same seeding with the values staged in the fixed scratch array below.  The
// table itself is the caller's device buffer.
//
// The scratch array is FS_NOALLOC_MAX_ROWS 64-bit words (2 MiB).  It lives in the
// library's device image, so every GPU that loads the library holds it until the process
// exits.  All calls share it: calls that can overlap on the GPU (different streams with
// no ordering between them) race on it, and the later copy can overwrite seeds the earlier
// kernel is still reading.  The kernel reads only the rows the same call copied in, so
// nothing in the array needs to start at zero, and whatever the previous call left there
// is never read.  The array's device address is looked up once per device and kept for
// the life of the process; a device reset (cudaDeviceReset, or a primary-context reset by
// another library) frees the image that holds the array, so the kept address is stale
// after one and the entry point must not be called again in that process.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/feynsimul.h"
#include "fs_rng.cuh"

#define FS_NOALLOC_MAX_ROWS (1 << 18)
#define FS_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned long long fs_noalloc_seed_scratch[FS_NOALLOC_MAX_ROWS];

// Same seeding as the NVRTC module's fs_ranlux_init (ranluxcl_init per row).
__global__ void fs_ranlux_init_scratch_kernel(fs_u32 *tab, const fs_u64 *xs, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    FsRanlux r;
    fs_rl_seed(r, xs[i]);
    fs_rl_store(r, tab + (size_t)i * 28);
}

extern int fsi_thread_error(int code, const char *msg);

static std::mutex g_noalloc_mu;
static void *g_noalloc_scratch[FS_NOALLOC_MAX_DEVICES];

// Device address of the scratch array on the current device.  The array's name in host
// code is only a host-side stand-in for the symbol, so the address comes from
// cudaGetSymbolAddress, once per device, with that device current.
static int noalloc_scratch(void **ptr)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fsi_thread_error(FS_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= FS_NOALLOC_MAX_DEVICES)
        return fsi_thread_error(FS_ERR_CUDA, "device index out of range for the scratch table");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_scratch[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, fs_noalloc_seed_scratch);
        if (e != cudaSuccess || !p)
            return fsi_thread_error(FS_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e)
                                                                  : "cudaGetSymbolAddress returned null");
        g_noalloc_scratch[dev] = p;
    }
    *ptr = g_noalloc_scratch[dev];
    return FS_OK;
}

extern "C" int fs_ranlux_init_noalloc(uint32_t *table, const uint64_t *xs, size_t n_rows, void *stream)
{
    if (n_rows == 0) return FS_OK;
    if (!table || !xs) return fsi_thread_error(FS_ERR_CONFIG, "fs_ranlux_init_noalloc: null table or seed array");
    if (n_rows > (size_t)FS_NOALLOC_MAX_ROWS)
        return fsi_thread_error(FS_ERR_CONFIG,
                                "fs_ranlux_init_noalloc: at most 262144 rows per call (the fixed scratch "
                                "holds 262144 seed values); seed larger tables in slices of that size");
    void *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(scratch, xs, n_rows * sizeof(uint64_t), cudaMemcpyDefault, s);
    if (e != cudaSuccess) return fsi_thread_error(FS_ERR_CUDA, cudaGetErrorString(e));
    const int n = (int)n_rows;
    fs_ranlux_init_scratch_kernel<<<(n + 127) / 128, 128, 0, s>>>((fs_u32 *)table, (const fs_u64 *)scratch, n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fsi_thread_error(FS_ERR_LAUNCH, cudaGetErrorString(e));
    return FS_OK;
}
