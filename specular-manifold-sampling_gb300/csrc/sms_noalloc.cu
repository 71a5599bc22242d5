// sms_noalloc.cu -- allocation-free variant of the single-scatter connection call.
//
// Some callers cannot allocate device memory while they render: a real-time
// loop with a fixed memory budget, or an embedding that owns every allocation
// itself and forbids libraries from calling cudaMalloc.  sms_ss_connect_batch_device may allocate:
// it grows the context's per-query scratch of the unbiased estimator on demand.
// sms_ss_connect_batch_noalloc runs the same kernels, but takes that scratch
// from the fixed device array below and makes no allocating call at all.
#include <cuda.h>

#include <mutex>
#include <string>

#include "../../include/sms_gb300.h"
#include "sms_device.cuh"
#include "sms_kernels.h"

namespace sms {

static sms_status set_last_error(sms_status st, const std::string &msg) {
    return (sms_status)set_last_error_impl((int)st, msg.c_str());
}

// Largest batch the allocation-free entry point accepts.  The scratch holds 32
// bytes per query (stream position, first-walk direction, first-walk
// contribution, trial-queue slot): 262,144 queries = 8 MiB, held by every GPU
// that loads this library until the process exits.
constexpr uint32_t kNoAllocMaxQueries = 1u << 18;

static __device__ __align__(256) unsigned char g_noalloc_scratch[(size_t)kNoAllocMaxQueries * 32];

constexpr int kNoAllocMaxDevices = 64;

// Cached device address of g_noalloc_scratch, per device, with the id of the
// CUDA context it was looked up in.  cudaDeviceReset destroys the primary
// context; the runtime then reloads this library's module in a new context,
// where the array may sit elsewhere, so an address is reused only while the
// device's current context is the one it came from.
struct ScratchAddr {
    unsigned long long ctx_id;
    void *ptr;
};
static ScratchAddr g_scratch_addr[kNoAllocMaxDevices];
static std::mutex g_scratch_mu;

using CuCtxGetCurrentFn = CUresult (*)(CUcontext *);
using CuCtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

// Id of the calling thread's current CUDA context (unique for the life of
// the process); false when the driver cannot tell.
static bool current_ctx_id(unsigned long long *id) {
    static CuCtxGetCurrentFn get_current = nullptr;
    static CuCtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CuCtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CuCtxGetIdFn>(p);
    });
    CUcontext cx = nullptr;
    if (!get_current || !get_id || get_current(&cx) != CUDA_SUCCESS || !cx) return false;
    return get_id(cx, id) == CUDA_SUCCESS;
}

// Device address of g_noalloc_scratch on the current device.  In host code
// the symbol name is only a host-side stand-in; cudaGetSymbolAddress gives
// the address kernels can use.  The lookup runs once per device and context
// (the first one also lets the runtime load the module that holds the array).
static cudaError_t noalloc_scratch(int device, void **out) {
    if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    unsigned long long id = 0;
    const bool have_id = current_ctx_id(&id);
    ScratchAddr &a = g_scratch_addr[device];
    if (have_id && a.ptr && a.ctx_id == id) {
        *out = a.ptr;
        return cudaSuccess;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        a.ptr = nullptr;
        return e;
    }
    // The lookup may have created the context: take its id now.
    if (have_id || current_ctx_id(&id)) {
        a.ctx_id = id;
        a.ptr = p;
    } else {
        a.ptr = nullptr;   // no context id: look the address up on every call
    }
    *out = p;
    return cudaSuccess;
}

}  // namespace sms

using namespace sms;

extern "C" sms_status sms_ss_connect_batch_noalloc(sms_ctx *ctx, const float *queries_dev, uint32_t n,
                                                   uint64_t seed, uint64_t stream_offset, sms_result *out_dev) {
    if (!ctx || !out_dev || (n && (!queries_dev || !out_dev->value || !out_dev->count || !out_dev->walks)))
        return set_last_error(SMS_ERR_INVALID_ARG, "sms_ss_connect_batch_noalloc: null argument");
    if (n > kNoAllocMaxQueries)
        return set_last_error(SMS_ERR_INVALID_ARG,
                              "sms_ss_connect_batch_noalloc: " + std::to_string(n) +
                                  " queries exceed the fixed scratch of " + std::to_string(kNoAllocMaxQueries) +
                                  "; split the batch (stream_offset keeps the results identical)");
    if (n == 0) return SMS_OK;
    CtxView v;
    if (!ctx_view(ctx, v)) return set_last_error(SMS_ERR_INVALID_ARG, "sms_ss_connect_batch_noalloc: bad context");
    if (v.proposal_bound)
        return set_last_error(SMS_ERR_UNSUPPORTED,
                              "sms_ss_connect_batch_noalloc: a bound learned proposal needs per-query mixture "
                              "scratch; use sms_ss_connect_batch_device");
    // Same configuration checks as sms_ss_connect_batch_device, except that a
    // missing LEAN pyramid is reported rather than built.
    if (sms_status st = ctx_ss_check(ctx, false)) return st;
    cudaError_t e = cudaSetDevice(v.device);
    if (e != cudaSuccess) return set_last_error(SMS_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    void *base = nullptr;
    e = noalloc_scratch(v.device, &base);
    if (e != cudaSuccess)
        return set_last_error(SMS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    // Same sub-array layout as the context scratch, with capacity kNoAllocMaxQueries.
    char *b = reinterpret_cast<char *>(base);
    const size_t cap = kNoAllocMaxQueries;
    SsScratch scr;
    scr.pos = reinterpret_cast<uint32_t *>(b);
    scr.dir0 = reinterpret_cast<float *>(b + 4 * cap);
    scr.val = reinterpret_cast<float *>(b + 16 * cap);
    scr.list = reinterpret_cast<uint32_t *>(b + 28 * cap);
    // Nothing in the scratch has to start at zero: every query's entries are
    // written before they are read within the call, and the trial-queue
    // counters live in the context and are cleared by the launch itself.
    // No phase timer: recording it may create CUDA events (an allocation), so
    // these calls do not appear in sms_profile_read.
    e = launch_ss_connect(*v.scene, v.solver, queries_dev, n, seed, stream_offset, out_dev->value, out_dev->count,
                          out_dev->walks, v.counters, scr, v.num_sms, v.blocks_per_sm, nullptr, v.stream, nullptr,
                          v.trial_group);
    if (e != cudaSuccess) return set_last_error(SMS_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return SMS_OK;
}
