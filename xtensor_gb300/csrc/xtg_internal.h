// xtg_internal.h — shared host-side declarations of libxtg (not installed).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/xtg.h"

namespace xtgh {

// ---- errors ---------------------------------------------------------------
xtg_status fail(xtg_status s, const std::string& msg);
xtg_status cuda_fail(cudaError_t e, const char* what);
xtg_status cu_fail(CUresult e, const char* what);
void clear_error();

#define XTG_CUDA(call)                                         \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return ::xtgh::cuda_fail(_e, #call); \
    } while (0)
#define XTG_CU(call)                                           \
    do {                                                       \
        CUresult _e = (call);                                  \
        if (_e != CUDA_SUCCESS) return ::xtgh::cu_fail(_e, #call); \
    } while (0)
#define XTG_TRY(call)                                          \
    do {                                                       \
        xtg_status _s = (call);                                \
        if (_s != XTG_OK) return _s;                           \
    } while (0)

// ---- driver API (resolved at run time through cudaGetDriverEntryPointByVersion
// so that the library loads on machines without a driver) -------------------------
struct Drv {
    CUresult (*Init)(unsigned int) = nullptr;
    CUresult (*CtxGetCurrent)(CUcontext*) = nullptr;
    CUresult (*CtxSetCurrent)(CUcontext) = nullptr;
    CUresult (*ModuleLoadData)(CUmodule*, const void*) = nullptr;
    CUresult (*ModuleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
    CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**) = nullptr;
    CUresult (*LaunchKernelEx)(const CUlaunchConfig*, CUfunction, void**, void**) = nullptr;
    CUresult (*OccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t) = nullptr;
    CUresult (*GetErrorString)(CUresult, const char**) = nullptr;
    CUresult (*FuncSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
};
const Drv& drv();

// ---- device ----------------------------------------------------------------
struct DeviceInfo {
    int device = -1;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    int64_t hbm = 0;
    int max_threads_per_sm = 0;
};
// Initialises the runtime on the current (or default) device once, makes the
// primary context current on the calling thread.
xtg_status ensure_device(DeviceInfo** info);

// ---- options -----------------------------------------------------------------
int64_t opt(const char* key, int64_t dflt);
// Default work items a ROW reduction is split into (reduce.target_items):
// shared by every planner of a reduction so equal calls partition alike.
constexpr int64_t kReduceTargetItems = 2048;
// Option "jit.dry_run": plan and compile kernels without a GPU (no launches).
bool dry_run();

// ---- dtypes -------------------------------------------------------------------
struct DTypeInfo {
    const char* cname;  // C++ spelling used in kernel names
    int size;
    bool is_float;
    bool is_signed;
    bool is_int;
};
const DTypeInfo& dt(int dtype);
bool valid_dtype(int dtype);

// ---- JIT ------------------------------------------------------------------------
struct Kernel {
    CUfunction fn = nullptr;
    std::string name;
    int max_blocks_per_sm = 0;  // occupancy at the block size it was queried for
    int block = 0;
    size_t dyn_smem = 0;        // dynamic shared memory the occupancy was queried with
    size_t smem_limit = 0;      // the kernel's dynamic shared-memory limit: only ever raised, so
                                // the launches of a cached plan stay within it when replayed
};
// Compiles (or fetches) the kernel whose name expression is `expr`
// (e.g. "xtg::k_assign<...>").  `block` / `dyn_smem` are used for the
// occupancy query (and dyn_smem > 48 KiB raises the kernel's limit).
xtg_status get_kernel(const std::string& expr, int block, Kernel** k, size_t dyn_smem = 0);
// Whether `expr` is compiled and loaded in this process (no compile).
bool kernel_ready(const std::string& expr);
// Compiles and loads `expr` on a background thread (no-op when it is ready
// or being built); callers that must not wait use their other path meanwhile.
void compile_async(const std::string& expr, int block, size_t dyn_smem = 0);
// Waits (bounded) until no background compile is running.
void wait_background_compiles(int64_t timeout_ms);
// Launch with a parameter block of `psize` bytes.  scratch_off >= 0: byte
// offset of a pointer to the call's split-reduction scratch inside the
// block (patched when a cached plan is replayed with fresh scratch).
xtg_status launch_raw(Kernel* k, unsigned grid, unsigned block, const void* params, size_t psize, cudaStream_t stream,
                      size_t dyn_smem, int scratch_off);
template <class P>
xtg_status launch(Kernel* k, unsigned grid, unsigned block, P* params, cudaStream_t stream, size_t dyn_smem = 0,
                  int scratch_off = -1) {
    return launch_raw(k, grid, block, params, sizeof(P), stream, dyn_smem, scratch_off);
}

// ---- plan recording / replay (xtg_plancache.cpp) ------------------------------
struct RecLaunch {
    Kernel* k;
    unsigned grid, block;
    size_t smem;
    std::vector<unsigned char> params;
    int scratch_off;
};
struct Recorder {
    std::vector<RecLaunch> launches;
    size_t scratch_bytes = 0;
    int scratch_allocs = 0;
    bool nocache = false;  // a launch holds a temporary the replay could not patch
};
Recorder*& recorder();  // the calling thread's active recorder (nullptr: none)
int64_t opt_generation();  // increments whenever an option changes
// A device word that kernels set when a bounded wait gives up.
xtg_status device_error_word(int** p);
void count_launch();
// Resets the per-thread record of launched kernels (start of an API call).
void begin_call();

// ---- batches (xtg_batch.cpp) -----------------------------------------------------------
// The kernel xtg_batch_build would launch without autotuning (no device work).
xtg_status batch_planned_kernel(xtg_batch* b, std::string* name);

// ---- pinned staging ring (xtg_npy.cpp) ---------------------------------------------
// Copies `bytes` of pageable host memory to device memory through the pinned
// staging ring (several host threads, one CUDA stream each); the copies start
// after `wait_for` (non-null) and have landed when the call returns.
xtg_status ring_h2d(void* dev, const void* host, size_t bytes, cudaEvent_t wait_for);

// ---- scratch ---------------------------------------------------------------------
xtg_status scratch_alloc(void** p, size_t bytes, cudaStream_t s);
xtg_status scratch_free(void* p, cudaStream_t s);

}  // namespace xtgh
