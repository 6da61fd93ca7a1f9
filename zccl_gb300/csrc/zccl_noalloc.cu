/*
 * zccl_noalloc.cu -- zccl_gpu_compress_noalloc: the device compressor with
 * its scratch in a fixed array of this library's device image, for callers
 * that must not allocate device memory.
 *
 * The compressor needs, per call, an error word, a tile ticket and one
 * look-back status word per tile, all zero at launch: 16 + 8 * tiles bytes.
 * Here they live in g_scratch, a file-scope __device__ array that exists
 * once per device from the moment the library's device code is loaded.
 * Its address is looked up with cudaGetSymbolAddress the first time a call
 * runs with that device current, kept per device (so a cudaDeviceReset()
 * between calls is not supported: the module, and the array with it, may
 * move), and then handed to the ordinary compressor as its workspace, which
 * clears the part that must start at zero on the caller's stream and
 * launches the same kernel.  The array's two status words start at zero
 * with the module and collect the errors of every call until
 * zccl_gpu_check() reads and clears them.  No call here allocates: no
 * cudaMalloc, no cudaFree, no allocating library.
 *
 * One array per device is shared by every call on that device, so two calls
 * whose work overlaps in time on that device (two streams, or two host
 * threads) race on it; callers order them, for instance by using one stream.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/zccl_gpu.h"
#include "zgeom.h"

namespace {

static __device__ __align__(256) unsigned char g_scratch[ZCCL_GPU_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices]; /* address of g_scratch per device ordinal, once looked up */

/* Address of g_scratch on the current device (one-time lookup per device). */
int scratch_address(void **addr)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return ZCCL_GPU_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return ZCCL_GPU_EINVAL;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return ZCCL_GPU_ECUDA;
        }
        g_addr[dev] = p;
    }
    *addr = g_addr[dev];
    return ZCCL_GPU_OK;
}

} // namespace

extern "C" int zccl_gpu_compress_noalloc(zccl_gpu_stream *out, const float *d_in, size_t n,
                                         float eb, int L, int T, void *cuda_stream,
                                         void **d_scratch)
{
    if (d_scratch) *d_scratch = nullptr;
    ZGeom g;
    if (L < 1 || T < 1 || zg_init(&g, (uint64_t)n, (uint32_t)L, (uint32_t)T) != 0)
        return ZCCL_GPU_EINVAL;
    /* error word, ticket, padding, one status word per tile */
    if (16ull + 8ull * g.ntiles > (uint64_t)ZCCL_GPU_NOALLOC_SCRATCH_BYTES) return ZCCL_GPU_ESCRATCH;
    void *scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    const int rc = zccl_gpu_compress(out, d_in, n, eb, L, T, scratch, cuda_stream);
    if (rc == ZCCL_GPU_OK && d_scratch) *d_scratch = scratch;
    return rc;
}
