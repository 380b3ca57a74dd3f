// noalloc.cu -- tl_gemm_noalloc: the split-k tensor-core GEMM for callers that cannot allocate device
// memory.  Examples: a plugin that runs inside a host application owning all device memory through
// its own pool (or a fixed reservation made at start-up), code on a latency-critical path where a
// cudaMalloc (which can synchronise the device) is not acceptable, or a caller without a tl_handle
// (creating one allocates).  Its split-k partial tiles, tile counters and error word live in one
// file-scope device array instead of a workspace the library allocates.
//
// Limits and sharing:
//   * kNoallocScratchBytes (64 MiB) in total: 256 bytes of error word, kNoallocCounters tile
//     counters, the rest for fp32 partial tiles (tiles * split_k * 128 * macro_tile0 * 4 bytes).
//     Problems that need more are refused with TL_ERR_UNSUPPORTED before anything is launched.
//   * Every GPU that loads the library holds the array until the process exits.
//   * All calls on a device share the array and it keeps the last call's contents; each call
//     clears the error word and counters it uses (on its stream) before the GEMM.  Two calls whose
//     work overlaps on the GPU (different streams, no ordering between them) race on it.
//   * The first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//     that device current; make that first call before any stream capture.
//   * A kernel whose bounded wait ran out ORs a role mask into the error word and returns early;
//     tl_noalloc_status reads and clears it (a device-to-host copy into a host int, no allocation).
//   * Calls use the caller's current device and context; nothing here calls cudaSetDevice.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "tl_internal.h"

namespace tl {
namespace {

constexpr size_t kNoallocScratchBytes = size_t(64) << 20;
constexpr size_t kNoallocHeaderBytes = 256;                 // error word (+ padding)
constexpr size_t kNoallocCounters = 16384;                  // split-k tile counters
constexpr size_t kNoallocPartialOffset = kNoallocHeaderBytes + kNoallocCounters * sizeof(int);
constexpr size_t kNoallocPartialBytes = kNoallocScratchBytes - kNoallocPartialOffset;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

struct NoallocDevice {
    bool ready = false;
    unsigned char* scratch = nullptr;   // device address of g_noalloc_scratch on this device
    int sm_count = 0;
    size_t smem_optin = 0;
};

std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[kMaxDevices];

// Once per device, with that device current: the array's device address and the device limits.
tl_status noalloc_setup(int dev, NoallocDevice** out)
{
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    NoallocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        int sms = 0, smem = 0;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            return cuda_fail(e, "cudaDeviceGetAttribute(sm count)");
        if ((e = cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess)
            return cuda_fail(e, "cudaDeviceGetAttribute(smem)");
        d.scratch = static_cast<unsigned char*>(ptr);
        d.sm_count = sms;
        d.smem_optin = static_cast<size_t>(smem);
        d.ready = true;
    }
    *out = &d;
    return TL_SUCCESS;
}

}  // namespace
}  // namespace tl

using namespace tl;

extern "C" TL_API tl_status tl_gemm_noalloc(const tl_gemm_problem* problem, const tl_gemm_solution* solution,
                                            void* D, const void* C, const void* A, const void* B, void* stream)
{
    // The caller's current device and context are used as they are (no cudaSetDevice): a caller on
    // the driver API keeps its own current context.  The memset below is a runtime call on that
    // context, so the tensor-map encoding after it always runs with a context current.
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(TL_ERR_UNSUPPORTED, "device ordinal beyond 63");
    NoallocDevice* nd = nullptr;
    tl_status st = noalloc_setup(dev, &nd);
    if (st != TL_SUCCESS) return st;
    TcLaunch L;
    size_t ws_bytes = 0, counters = 0;
    st = plan_tc_noalloc(dev, nd->sm_count, nd->smem_optin, problem, solution, D, C, A, B, &L, &ws_bytes, &counters);
    if (st != TL_SUCCESS) return st;
    if (ws_bytes > kNoallocPartialBytes || counters > kNoallocCounters)
        return fail(TL_ERR_UNSUPPORTED,
                    "tl_gemm_noalloc: this problem needs " + std::to_string(ws_bytes) + " bytes of split-k workspace and " +
                        std::to_string(counters) + " tile counters; the static scratch holds " +
                        std::to_string(kNoallocPartialBytes) + " bytes and " + std::to_string(kNoallocCounters) +
                        " counters (use a smaller split_k or tl_gemm)");
    const tl_gemm_problem& p = *problem;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (p.m == 0 || p.n == 0) return TL_SUCCESS;
    // the error word and the counters this call uses must start at zero
    e = cudaMemsetAsync(nd->scratch, 0, kNoallocHeaderBytes + counters * sizeof(int), s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(noalloc scratch)");
    if (p.k == 0 || L.alpha == 0.0f)
        return aux_scale_c(p.dtype_d, p.out_rounding, D, p.ldd, p.stride_d, C, p.ldc, p.stride_c, p.m, p.n, p.batch,
                           p.beta, s, nullptr);
    L.err = reinterpret_cast<int*>(nd->scratch);
    L.counters = reinterpret_cast<int*>(nd->scratch + kNoallocHeaderBytes);
    L.workspace = reinterpret_cast<float*>(nd->scratch + kNoallocPartialOffset);
    L.timeout_ns = 4000000000ull;
    if (const char* t = getenv("TL_WAIT_TIMEOUT_MS")) {
        long v = strtol(t, nullptr, 10);
        if (v > 0) L.timeout_ns = static_cast<uint64_t>(v) * 1000000ull;
    }
    return tc_gemm_launch(L, s, nullptr);
}

// The error word is the first int of the array; kernels that ran out a bounded wait OR a role mask
// into it.  Read on `stream` (after the calls queued there) into a host int, then cleared.
extern "C" TL_API tl_status tl_noalloc_status(void* stream)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(TL_ERR_UNSUPPORTED, "device ordinal beyond 63");
    NoallocDevice* nd = nullptr;
    tl_status st = noalloc_setup(dev, &nd);
    if (st != TL_SUCCESS) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int v = 0;
    if ((e = cudaMemcpyAsync(&v, nd->scratch, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpyAsync(noalloc error word)");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    if (v != 0) {
        if ((e = cudaMemsetAsync(nd->scratch, 0, sizeof(int), s)) != cudaSuccess)
            return cuda_fail(e, "cudaMemsetAsync(noalloc error word)");
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
        char buf[128];
        snprintf(buf, sizeof(buf), "tl_gemm_noalloc: device wait timed out (role mask 0x%x); D is not valid", v);
        return fail(TL_ERR_TIMEOUT, buf);
    }
    return TL_SUCCESS;
}
