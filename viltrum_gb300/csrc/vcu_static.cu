/*
 * vcu_static.cu -- per-bin adaptive nested quadrature for callers that cannot allocate device
 * memory.
 *
 * Some host programs must not call cudaMalloc at all: plugins loaded into a process whose CUDA
 * memory is owned by another allocator (a renderer or a framework with its own pool), real-time
 * frame loops that cannot take the device-wide synchronisation cudaMalloc/cudaFree may imply, or
 * hosts with a fixed memory budget checked at start-up.  vcu_per_bin_adaptive_nested_static() serves them.  It creates no context and allocates
 * nothing: its only device scratch -- the status word and, for host-memory bins, the staging copy of
 * the bin values -- is the file-scope array below, which every GPU that loads the library holds until
 * the process exits.
 *
 * The array's name is only a host-side stand-in in host code; the kernel receives its device
 * address, taken with cudaGetSymbolAddress with the caller's device current.  The first call on a
 * device does this set-up, so it should come before any stream capture.  Every call on a stream
 * that is not capturing looks the address up again (a cudaDeviceReset in the host process reloads
 * the module and can move the array); the per-device cache serves only calls on a capturing
 * stream.  All calls share the array and it keeps the last call's contents: the status word is
 * cleared at the start of every call, and calls that overlap on the GPU (on different streams, or
 * from different host threads) race on it -- serialise them.
 *
 * Nothing is allocated on the device, on any path.  On success nothing is allocated on the host
 * either; a call that fails inside the launch code shared with the regular entry point formats its
 * message into a host string that is then discarded (this entry point returns only the code).
 */
#include <mutex>

#include "vcu_internal.cuh"

#define VCU_STATIC_MAX_DEVICES 64

namespace {

/* [0, 64): status word (first uint32) and padding; [64, 64 + VCU_STATIC_MAX_BIN_VALUES): staged bins */
static __device__ __align__(256) float g_static_scratch[64 + VCU_STATIC_MAX_BIN_VALUES];

std::mutex g_static_mutex;
float* g_static_ptr[VCU_STATIC_MAX_DEVICES] = {};

/* device address of g_static_scratch on the current device: looked up on every uncaptured call
 * (the module, and the array with it, moves after a cudaDeviceReset), the cached value during a
 * stream capture */
int static_scratch(int device, cudaStream_t stream, float** out) {
    if (device < 0 || device >= VCU_STATIC_MAX_DEVICES) return VCU_UNSUPPORTED;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
        cudaGetLastError();
        return VCU_CUDA_ERROR;
    }
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return VCU_CUDA_ERROR;
        }
        g_static_ptr[device] = static_cast<float*>(p);
    } else if (!g_static_ptr[device]) {
        return VCU_UNSUPPORTED; /* first call on this device inside a capture */
    }
    *out = g_static_ptr[device];
    return VCU_OK;
}

}  // namespace

extern "C" int vcu_per_bin_adaptive_nested_static(const vcu_problem* p, const vcu_nested* nested,
                                                  uint64_t iterations, float* bins, void* stream) {
    using namespace vcu;
    if (!p || !nested || !bins) return VCU_INVALID_ARG;
    const int ch = vcu_channels(p->f.kind);
    if (ch < 0) return VCU_INVALID_ARG;
    if (iterations > 62) return VCU_UNSUPPORTED;
    if (check_per_bin_nested(nullptr, *nested)) return VCU_INVALID_ARG;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return VCU_NO_DEVICE;
    }
    /* a context on the stack: the caller's stream, the device's limits and the static status word;
     * its buffers stay empty (nothing is allocated) */
    vcu_ctx ctx;
    ctx.device = device;
    ctx.tune = 0; /* the autotuner would time extra launches: use the default configuration */
    ctx.stream = static_cast<cudaStream_t>(stream);
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return VCU_CUDA_ERROR;
    ctx.sm_count = v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess)
        return VCU_CUDA_ERROR;
    ctx.smem_optin = (size_t)v;
    BinGrid g;
    int rc = make_grid(&ctx, p, g);
    if (rc) return rc;
    if (g.nbins * (uint64_t)ch > VCU_STATIC_MAX_BIN_VALUES) return VCU_UNSUPPORTED;
    float* scratch = nullptr;
    if ((rc = static_scratch(device, ctx.stream, &scratch))) return rc;
    ctx.d_status = reinterpret_cast<uint32_t*>(scratch);
    if (cudaMemsetAsync(ctx.d_status, 0, sizeof(uint32_t), ctx.stream) != cudaSuccess) return VCU_CUDA_ERROR;
    float* dbins = (p->mem == VCU_MEM_DEVICE) ? bins : scratch + 64;
    uint32_t launches = 0;
    if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_SIMPSON)
        rc = run_nested_bs(&ctx, p, g, *nested, (int)iterations, dbins, nullptr, launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_nested_bt(&ctx, p, g, *nested, (int)iterations, dbins, nullptr, launches);
    else
        rc = run_nested_st(&ctx, p, g, *nested, (int)iterations, dbins, nullptr, launches);
    if (rc) return rc;
    if (p->mem == VCU_MEM_HOST &&
        cudaMemcpyAsync(bins, dbins, g.nbins * ch * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess)
        return VCU_CUDA_ERROR;
    uint32_t flags = 0;
    if (cudaMemcpyAsync(&flags, ctx.d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess)
        return VCU_CUDA_ERROR;
    if (cudaStreamSynchronize(ctx.stream) != cudaSuccess) return VCU_CUDA_ERROR;
    if (flags & VCU_FLAG_NAN) return VCU_NAN_DETECTED;
    return VCU_OK;
}
