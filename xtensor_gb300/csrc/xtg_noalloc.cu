// xtg_noalloc.cu — float32 full sum that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they reduce: code
// whose device memory is owned by its own allocator or budget (a framework
// that reserved the device's memory up front, where a cudaMalloc of the
// library would fail or fragment it), or loops with latency limits that must
// never enter an allocator (a stream-ordered allocation can map new memory
// with an unbounded delay).  xtg_reduce gets the scratch for its split
// reduction from the stream-ordered pool; xtg_sum_f32_noalloc runs the same
// two kernels (the split row reduction and its in-order combine, compiled
// here ahead of time for sm_103a) with the partials in a fixed static device
// array instead.
//
// The array below is a module-scope `__device__` buffer: every GPU on which
// this library is used holds XTG_NOALLOC_SCRATCH_BYTES of it until the
// process exits.  All calls on a device share it and it keeps the last
// call's contents; nothing in it needs clearing because each call writes
// every partial it later reads.  Two calls whose kernels overlap on the GPU
// (different streams without ordering between them) race on the array —
// serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "xtg_device.cuh"
#include "xtg_internal.h"
#include "xtg_plan.h"

static __device__ __align__(256) unsigned char g_xtg_noalloc_scratch[XTG_NOALLOC_SCRATCH_BYTES];

namespace {

using namespace xtg;
typedef LeafSet<LeafSpec<float, 0>> LS;
typedef L<0, float> Tree;

#define XTG_NOALLOC_ROW(VEC, GROUP) xtg::k_reduce_row<Tree, LS, AccSumC, float, 0, VEC, 1, 1, GROUP, false>
#define XTG_NOALLOC_COMBINE xtg::k_reduce_combine<AccSumC, float, 0, 1>
#define XTG_NOALLOC_COMBINE_THREAD xtg::k_reduce_combine_thread<AccSumC, float, 0, 1>

// Launch geometry and the array's device address, per CUDA context: the
// address belongs to the context that loaded this module, so a device reset
// (which ends the context) or a second context on the same device gets its
// own entry, keyed by the driver's unique context id.
struct CtxState {
    unsigned long long ctx_id = 0;
    void* scratch = nullptr;  // device address of g_xtg_noalloc_scratch in this context
    int sms = 0;
    int occ[3][2] = {{0, 0}, {0, 0}, {0, 0}};  // [vec 1/2/4][group 32/256]
    int occ_combine = 0;
};
constexpr size_t kMaxContexts = 64;
CtxState g_state[kMaxContexts];
size_t g_nstate = 0;
std::mutex g_mu;

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

template <class F> xtg_status driver_fn(const char* sym, F& fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion(sym, &p, 13000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
        return xtgh::fail(XTG_ERR_CUDA, std::string("driver entry point not found: ") + sym);
    fn = reinterpret_cast<F>(p);
    return XTG_OK;
}

template <class K> int occupancy(K k) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 256, 0) != cudaSuccess) {
        cudaGetLastError();
        n = 1;
    }
    return n > 0 ? n : 1;
}

// The entry of the calling thread's current context; the first call in a
// context resolves the scratch array's device address there
// (cudaGetSymbolAddress, which also loads this library's device code and, on
// a thread with no context yet, creates the device's primary context) and
// the launch geometry.
xtg_status setup(int dev, CtxState** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ctx_get_current) {
        XTG_TRY(driver_fn("cuCtxGetCurrent", g_ctx_get_current));
        XTG_TRY(driver_fn("cuCtxGetId", g_ctx_get_id));
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return xtgh::fail(XTG_ERR_CUDA, "cuCtxGetCurrent failed");
    void* ptr = nullptr;
    if (!ctx) {
        const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_xtg_noalloc_scratch);
        if (e != cudaSuccess) return xtgh::cuda_fail(e, "cudaGetSymbolAddress(g_xtg_noalloc_scratch)");
        if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
            return xtgh::fail(XTG_ERR_CUDA, "no CUDA context after loading the device code");
    }
    unsigned long long id = 0;
    if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return xtgh::fail(XTG_ERR_CUDA, "cuCtxGetId failed");
    for (size_t i = 0; i < g_nstate; ++i)
        if (g_state[i].ctx_id == id) {
            *out = &g_state[i];
            return XTG_OK;
        }
    if (g_nstate == kMaxContexts) return xtgh::fail(XTG_ERR_UNSUPPORTED, "xtg_sum_f32_noalloc: too many CUDA contexts");
    if (!ptr) {
        const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_xtg_noalloc_scratch);
        if (e != cudaSuccess) return xtgh::cuda_fail(e, "cudaGetSymbolAddress(g_xtg_noalloc_scratch)");
    }
    CtxState s;
    s.ctx_id = id;
    s.scratch = ptr;
    XTG_CUDA(cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, dev));
    s.occ[0][0] = occupancy(XTG_NOALLOC_ROW(1, 32));
    s.occ[0][1] = occupancy(XTG_NOALLOC_ROW(1, 256));
    s.occ[1][0] = occupancy(XTG_NOALLOC_ROW(2, 32));
    s.occ[1][1] = occupancy(XTG_NOALLOC_ROW(2, 256));
    s.occ[2][0] = occupancy(XTG_NOALLOC_ROW(4, 32));
    s.occ[2][1] = occupancy(XTG_NOALLOC_ROW(4, 256));
    s.occ_combine = occupancy(XTG_NOALLOC_COMBINE);
    g_state[g_nstate] = s;
    *out = &g_state[g_nstate++];
    return XTG_OK;
}

template <int VEC, int GROUP>
void launch_row(const RedParams& p, unsigned grid, cudaStream_t st) {
    XTG_NOALLOC_ROW(VEC, GROUP)<<<grid, 256, 0, st>>>(p);
}

}  // namespace

extern "C" xtg_status xtg_sum_f32_noalloc(const float* x, int64_t n, float* out, xtg_stream stream) {
    using namespace xtgh;
    if (!out || (n > 0 && !x)) return fail(XTG_ERR_INVALID, "null pointer");
    if (n < 0) return fail(XTG_ERR_INVALID, "negative element count");
    int dev = 0;
    XTG_CUDA(cudaGetDevice(&dev));
    CtxState* S;
    XTG_TRY(setup(dev, &S));

    // The same plan as xtg_reduce(XTG_RED_SUM, all axes) on a contiguous
    // float32 array: vector width, fixed chunking, warp/CTA groups.
    int vec = 4;
    while (vec > 1 && ((n % vec) != 0 || ((uintptr_t)x % (uintptr_t)(vec * 4)) != 0)) vec >>= 1;
    if (n == 0) vec = 1;
    const int64_t nv = n / vec;
    if (nv > 0xFFFFFFF0ll) return fail(XTG_ERR_UNSUPPORTED, "xtg_sum_f32_noalloc: more than 2^32 vectors");
    int64_t nsplit = 1;
    {
        const int64_t target = opt("reduce.target_items", kReduceTargetItems);
        const int64_t minchunk = opt("reduce.min_chunk", 512);
        nsplit = std::max<int64_t>(1, std::min<int64_t>(target, nv / minchunk));
    }
    int64_t chunk = nv > 0 ? (nv + nsplit - 1) / nsplit : 1;
    nsplit = nv > 0 ? (nv + chunk - 1) / chunk : 1;
    const size_t need = (size_t)nsplit * 32;
    if (nsplit > 1 && need > XTG_NOALLOC_SCRATCH_BYTES)
        return fail(XTG_ERR_UNSUPPORTED, "xtg_sum_f32_noalloc: the reduction needs " + std::to_string(need) +
                                             " bytes of scratch, more than the static " +
                                             std::to_string((size_t)XTG_NOALLOC_SCRATCH_BYTES) + "-byte buffer");
    const int group = chunk >= opt("reduce.cta_chunk", 2048) ? 256 : 32;

    RedParams p;
    memset(&p, 0, sizeof p);
    p.oshape[0] = 1;
    p.ofd[0] = make_fd(1);
    p.rshape[0] = nv > 0 ? nv : 1;
    p.rfd[0] = make_fd((uint64_t)(nv > 0 ? nv : 1));
    p.n_out = 1;
    p.n_outv = 1;
    p.n_red = n;
    p.n_redv = nv;
    p.chunk = chunk;
    p.nsplit = nsplit;
    p.leaf[0] = x;
    p.lks[0][0] = 0;
    p.lrs[0][0] = 1;
    p.out = out;
    p.ostr[0] = 0;
    p.partial = nsplit > 1 ? S->scratch : nullptr;

    const int vi = vec == 4 ? 2 : (vec == 2 ? 1 : 0);
    const int gi = group == 256 ? 1 : 0;
    const int64_t items = nsplit;
    const int64_t want = group == 32 ? (items + 7) / 8 : items;
    const int64_t cap = (int64_t)S->occ[vi][gi] * S->sms;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min(want, cap));
    cudaStream_t st = (cudaStream_t)stream;
    if (vec == 4) group == 256 ? launch_row<4, 256>(p, grid, st) : launch_row<4, 32>(p, grid, st);
    else if (vec == 2) group == 256 ? launch_row<2, 256>(p, grid, st) : launch_row<2, 32>(p, grid, st);
    else group == 256 ? launch_row<1, 256>(p, grid, st) : launch_row<1, 32>(p, grid, st);
    XTG_CUDA(cudaGetLastError());
    count_launch();
    if (nsplit > 1 && nsplit <= opt("reduce.thread_combine_max", 64)) {
        XTG_NOALLOC_COMBINE_THREAD<<<1, 256, 0, st>>>(p);
        XTG_CUDA(cudaGetLastError());
        count_launch();
    } else if (nsplit > 1) {
        XTG_NOALLOC_COMBINE<<<1, 256, 0, st>>>(p);
        XTG_CUDA(cudaGetLastError());
        count_launch();
    }
    return XTG_OK;
}
