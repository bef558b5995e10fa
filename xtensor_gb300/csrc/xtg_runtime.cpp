// xtg_runtime.cpp — device bring-up, memory, streams, options and error
// reporting of the C ABI.  xtensor reports failures by exceptions
// (XTENSOR_THROW, include/xtensor/core/xtensor_config.hpp:27-33); across a C
// ABI they become xtg_status codes plus a thread-local message.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "xtg_internal.h"

namespace xtgh {

static thread_local std::string t_err;

xtg_status fail(xtg_status s, const std::string& msg) {
    t_err = msg;
    return s;
}
xtg_status cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(XTG_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return fail(XTG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
static Drv g_drv;
const Drv& drv() { return g_drv; }

template <class F> static xtg_status resolve(const char* sym, F& fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion(sym, &p, 13000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
        return fail(XTG_ERR_CUDA, std::string("driver entry point not found: ") + sym);
    fn = reinterpret_cast<F>(p);
    return XTG_OK;
}

static xtg_status resolve_driver() {
    XTG_TRY(resolve("cuInit", g_drv.Init));
    XTG_TRY(resolve("cuCtxGetCurrent", g_drv.CtxGetCurrent));
    XTG_TRY(resolve("cuCtxSetCurrent", g_drv.CtxSetCurrent));
    XTG_TRY(resolve("cuModuleLoadData", g_drv.ModuleLoadData));
    XTG_TRY(resolve("cuModuleGetFunction", g_drv.ModuleGetFunction));
    XTG_TRY(resolve("cuLaunchKernel", g_drv.LaunchKernel));
    XTG_TRY(resolve("cuLaunchKernelEx", g_drv.LaunchKernelEx));
    XTG_TRY(resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", g_drv.OccupancyMaxActiveBlocksPerMultiprocessor));
    XTG_TRY(resolve("cuGetErrorString", g_drv.GetErrorString));
    XTG_TRY(resolve("cuFuncSetAttribute", g_drv.FuncSetAttribute));
    return XTG_OK;
}

xtg_status cu_fail(CUresult e, const char* what) {
    const char* s = nullptr;
    if (g_drv.GetErrorString) g_drv.GetErrorString(e, &s);
    if (e == CUDA_ERROR_OUT_OF_MEMORY) return fail(XTG_ERR_OOM, std::string(what) + ": " + (s ? s : "?"));
    return fail(XTG_ERR_CUDA, std::string(what) + ": " + (s ? s : "?"));
}
void clear_error() { t_err.clear(); }

// ---- dtypes -----------------------------------------------------------------------
static const DTypeInfo kDT[XTG_NUM_DTYPES] = {
    {"bool", 1, false, false, true},
    {"signed char", 1, false, true, true},
    {"unsigned char", 1, false, false, true},
    {"short", 2, false, true, true},
    {"unsigned short", 2, false, false, true},
    {"int", 4, false, true, true},
    {"unsigned int", 4, false, false, true},
    {"long long", 8, false, true, true},
    {"unsigned long long", 8, false, false, true},
    {"xtg::bf16", 2, true, true, false},
    {"float", 4, true, true, false},
    {"double", 8, true, true, false},
};
bool valid_dtype(int d) { return d >= 0 && d < XTG_NUM_DTYPES; }
const DTypeInfo& dt(int d) { return kDT[valid_dtype(d) ? d : 0]; }

// ---- device -------------------------------------------------------------------------
static std::mutex g_dev_mu;
static DeviceInfo g_dev;
static CUcontext g_ctx = nullptr;

static xtg_status init_locked(int device) {
    int n = 0;
    XTG_CUDA(cudaGetDeviceCount(&n));
    if (n <= 0) return fail(XTG_ERR_CUDA, "no CUDA device");
    if (device < 0) XTG_CUDA(cudaGetDevice(&device));
    if (device >= n) return fail(XTG_ERR_INVALID, "device index out of range");
    XTG_CUDA(cudaSetDevice(device));
    XTG_CUDA(cudaFree(0));
    XTG_TRY(resolve_driver());
    XTG_CU(g_drv.Init(0));
    XTG_CU(g_drv.CtxGetCurrent(&g_ctx));
    if (!g_ctx) return fail(XTG_ERR_CUDA, "no current CUDA context after runtime init");
    cudaDeviceProp pr;
    XTG_CUDA(cudaGetDeviceProperties(&pr, device));
    g_dev.device = device;
    g_dev.sm_count = pr.multiProcessorCount;
    g_dev.cc_major = pr.major;
    g_dev.cc_minor = pr.minor;
    g_dev.hbm = (int64_t)pr.totalGlobalMem;
    g_dev.max_threads_per_sm = pr.maxThreadsPerMultiProcessor;
    return XTG_OK;
}

bool dry_run() { return opt("jit.dry_run", 0) != 0; }

xtg_status ensure_device(DeviceInfo** info) {
    if (dry_run()) {
        // Planning + NVRTC compilation without a GPU: a GB300-shaped fake device.
        static DeviceInfo fake{0, 152, 10, 3, (int64_t)288 << 30, 2048};
        if (info) *info = &fake;
        return XTG_OK;
    }
    {
        std::lock_guard<std::mutex> lk(g_dev_mu);
        if (g_dev.device < 0) XTG_TRY(init_locked(-1));
    }
    CUcontext cur = nullptr;
    g_drv.CtxGetCurrent(&cur);
    if (cur != g_ctx) {
        XTG_CUDA(cudaSetDevice(g_dev.device));
        XTG_CU(g_drv.CtxSetCurrent(g_ctx));
    }
    if (info) *info = &g_dev;
    return XTG_OK;
}

// ---- options ------------------------------------------------------------------------------
static std::mutex g_opt_mu;
static std::map<std::string, int64_t> g_opts;
static std::atomic<int64_t> g_opt_gen{0};

int64_t opt_generation() { return g_opt_gen.load(); }

int64_t opt(const char* key, int64_t dflt) {
    std::lock_guard<std::mutex> lk(g_opt_mu);
    auto it = g_opts.find(key);
    return it == g_opts.end() ? dflt : it->second;
}

xtg_status scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
    if (bytes == 0) bytes = 16;
    if (Recorder* rec = recorder()) {
        rec->scratch_bytes = bytes;
        rec->scratch_allocs++;
    }
    if (dry_run()) {
        *p = (void*)(uintptr_t)0x7f0000000000ull;
        return XTG_OK;
    }
    XTG_CUDA(cudaMallocAsync(p, bytes, s));
    return XTG_OK;
}
static int* g_err_word = nullptr;

xtg_status device_error_word(int** p) {
    if (dry_run()) {
        *p = (int*)(uintptr_t)0x7e0000000000ull;
        return XTG_OK;
    }
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (!g_err_word) {
        XTG_CUDA(cudaMalloc((void**)&g_err_word, 256));
        XTG_CUDA(cudaMemset(g_err_word, 0, 256));
    }
    *p = g_err_word;
    return XTG_OK;
}

xtg_status scratch_free(void* p, cudaStream_t s) {
    if (dry_run()) return XTG_OK;
    if (p) XTG_CUDA(cudaFreeAsync(p, s));
    return XTG_OK;
}

}  // namespace xtgh

using namespace xtgh;

extern "C" {

const char* xtg_version(void) { return "xtensor-gb300 0.1 (xtensor 0.27.1 hot path, sm_103a)"; }

const char* xtg_status_string(xtg_status s) {
    switch (s) {
        case XTG_OK: return "ok";
        case XTG_ERR_INVALID: return "invalid argument";
        case XTG_ERR_BROADCAST: return "broadcast error";
        case XTG_ERR_AXIS: return "invalid reduction axes";
        case XTG_ERR_OUT_OF_RANGE: return "axis out of range";
        case XTG_ERR_SHAPE: return "shape mismatch";
        case XTG_ERR_CUDA: return "CUDA error";
        case XTG_ERR_JIT: return "kernel compilation failed";
        case XTG_ERR_OOM: return "out of device memory";
        case XTG_ERR_UNSUPPORTED: return "unsupported";
        case XTG_ERR_TIMEOUT: return "timeout";
        case XTG_ERR_REJECTED: return "rejected";
        case XTG_ERR_CANCELLED: return "cancelled";
        case XTG_ERR_NOT_FOUND: return "not found";
    }
    return "unknown status";
}

const char* xtg_last_error(void) { return t_err.c_str(); }

xtg_status xtg_init(int device) {
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (g_dev.device >= 0) {
        if (device >= 0 && device != g_dev.device)
            return fail(XTG_ERR_INVALID, "libxtg is already bound to another device");
        return XTG_OK;
    }
    return init_locked(device);
}

xtg_status xtg_device_count(int* count) {
    if (!count) return fail(XTG_ERR_INVALID, "null count");
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *count = 0;
    }
    return XTG_OK;
}

xtg_status xtg_device_info(int* sm_count, int64_t* hbm_bytes, int* cc_major, int* cc_minor) {
    DeviceInfo* d;
    XTG_TRY(ensure_device(&d));
    if (sm_count) *sm_count = d->sm_count;
    if (hbm_bytes) *hbm_bytes = d->hbm;
    if (cc_major) *cc_major = d->cc_major;
    if (cc_minor) *cc_minor = d->cc_minor;
    return XTG_OK;
}

xtg_status xtg_mem_info(int64_t* free_bytes, int64_t* total_bytes) {
    XTG_TRY(ensure_device(nullptr));
    size_t f = 0, t = 0;
    XTG_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = (int64_t)f;
    if (total_bytes) *total_bytes = (int64_t)t;
    return XTG_OK;
}

xtg_status xtg_malloc(void** ptr, size_t bytes, xtg_stream stream) {
    if (!ptr) return fail(XTG_ERR_INVALID, "null ptr");
    XTG_TRY(ensure_device(nullptr));
    *ptr = nullptr;
    if (bytes == 0) bytes = 1;
    XTG_CUDA(cudaMallocAsync(ptr, bytes, (cudaStream_t)stream));
    return XTG_OK;
}

xtg_status xtg_free(void* ptr, xtg_stream stream) {
    if (!ptr) return XTG_OK;
    XTG_TRY(ensure_device(nullptr));
    XTG_CUDA(cudaFreeAsync(ptr, (cudaStream_t)stream));
    return XTG_OK;
}

xtg_status xtg_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return fail(XTG_ERR_INVALID, "null ptr");
    XTG_TRY(ensure_device(nullptr));
    XTG_CUDA(cudaMallocHost(ptr, bytes ? bytes : 1));
    return XTG_OK;
}

xtg_status xtg_host_free(void* ptr) {
    if (!ptr) return XTG_OK;
    XTG_CUDA(cudaFreeHost(ptr));
    return XTG_OK;
}

xtg_status xtg_memcpy(void* dst, const void* src, size_t bytes, int kind, xtg_stream stream) {
    if (bytes == 0) return XTG_OK;
    if (!dst || !src) return fail(XTG_ERR_INVALID, "null pointer in memcpy");
    XTG_TRY(ensure_device(nullptr));
    cudaMemcpyKind k = cudaMemcpyDefault;
    if (kind == XTG_MEMCPY_H2D) k = cudaMemcpyHostToDevice;
    else if (kind == XTG_MEMCPY_D2H) k = cudaMemcpyDeviceToHost;
    else if (kind == XTG_MEMCPY_D2D) k = cudaMemcpyDeviceToDevice;
    XTG_CUDA(cudaMemcpyAsync(dst, src, bytes, k, (cudaStream_t)stream));
    return XTG_OK;
}

xtg_status xtg_memset(void* dst, int value, size_t bytes, xtg_stream stream) {
    if (bytes == 0) return XTG_OK;
    XTG_TRY(ensure_device(nullptr));
    XTG_CUDA(cudaMemsetAsync(dst, value, bytes, (cudaStream_t)stream));
    return XTG_OK;
}

xtg_status xtg_stream_create(xtg_stream* stream) {
    if (!stream) return fail(XTG_ERR_INVALID, "null stream");
    XTG_TRY(ensure_device(nullptr));
    cudaStream_t s;
    XTG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream = (xtg_stream)s;
    return XTG_OK;
}

xtg_status xtg_stream_destroy(xtg_stream stream) {
    if (!stream) return XTG_OK;
    XTG_CUDA(cudaStreamDestroy((cudaStream_t)stream));
    return XTG_OK;
}

xtg_status xtg_stream_sync(xtg_stream stream) {
    XTG_TRY(ensure_device(nullptr));
    XTG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return XTG_OK;
}

xtg_status xtg_device_sync(void) {
    XTG_TRY(ensure_device(nullptr));
    XTG_CUDA(cudaDeviceSynchronize());
    return XTG_OK;
}

size_t xtg_dtype_size(int32_t dtype) { return valid_dtype(dtype) ? (size_t)dt(dtype).size : 0; }

xtg_status xtg_check_device_errors(void) {
    XTG_TRY(ensure_device(nullptr));
    if (dry_run() || !g_err_word) return XTG_OK;
    int v = 0;
    XTG_CUDA(cudaDeviceSynchronize());
    XTG_CUDA(cudaMemcpy(&v, g_err_word, sizeof v, cudaMemcpyDeviceToHost));
    if (v) {
        XTG_CUDA(cudaMemset(g_err_word, 0, sizeof v));
        if (v == 2) return fail(XTG_ERR_OUT_OF_RANGE, "an index view coordinate was outside the array (element skipped)");
        return fail(XTG_ERR_TIMEOUT, "a kernel's bounded wait gave up (device error word was set)");
    }
    return XTG_OK;
}

xtg_status xtg_event_create(xtg_event* ev) {
    if (!ev) return fail(XTG_ERR_INVALID, "null event");
    XTG_TRY(ensure_device(nullptr));
    cudaEvent_t e;
    XTG_CUDA(cudaEventCreate(&e));
    *ev = (xtg_event)e;
    return XTG_OK;
}

xtg_status xtg_event_destroy(xtg_event ev) {
    if (ev) XTG_CUDA(cudaEventDestroy((cudaEvent_t)ev));
    return XTG_OK;
}

xtg_status xtg_event_record(xtg_event ev, xtg_stream stream) {
    XTG_CUDA(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream));
    return XTG_OK;
}

xtg_status xtg_event_sync(xtg_event ev) {
    XTG_CUDA(cudaEventSynchronize((cudaEvent_t)ev));
    return XTG_OK;
}

xtg_status xtg_event_elapsed_ms(xtg_event start, xtg_event end, float* ms) {
    if (!ms) return fail(XTG_ERR_INVALID, "null output");
    XTG_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)end));
    return XTG_OK;
}

xtg_status xtg_stream_wait_event(xtg_stream stream, xtg_event ev) {
    if (!ev) return fail(XTG_ERR_INVALID, "null event");
    if (dry_run()) return XTG_OK;
    XTG_CUDA(cudaStreamWaitEvent((cudaStream_t)stream, (cudaEvent_t)ev, 0));
    return XTG_OK;
}

xtg_status xtg_set_option(const char* key, int64_t value) {
    if (!key) return fail(XTG_ERR_INVALID, "null key");
    std::lock_guard<std::mutex> lk(g_opt_mu);
    if (value < 0) g_opts.erase(key);
    else g_opts[key] = value;
    g_opt_gen.fetch_add(1);
    return XTG_OK;
}

xtg_status xtg_get_option(const char* key, int64_t* value) {
    if (!key || !value) return fail(XTG_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(g_opt_mu);
    auto it = g_opts.find(key);
    if (it == g_opts.end()) return fail(XTG_ERR_NOT_FOUND, std::string("option not set: ") + key);
    *value = it->second;
    return XTG_OK;
}

}  // extern "C"
