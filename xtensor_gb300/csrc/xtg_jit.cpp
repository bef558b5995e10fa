// xtg_jit.cpp — instantiates the kernel templates of xtg_device.cuh for one
// expression-tree type at first use.  NVRTC compiles the instantiation to an
// sm_103a cubin (arch-specific target of the running device), the cubin is
// cached on disk and in-process, and launches go through the driver API on
// the runtime's primary context.  This is the "compile-time lowering" of an
// xfunction tree, performed when the tree shape is first seen instead of when
// the caller's translation unit is built.
#include <nvrtc.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <condition_variable>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>

#include <sys/stat.h>
#include <unistd.h>

#include "xtg_internal.h"
#include "_gen/xtg_device_src.h"  // kXtgParamsSrc / kXtgDeviceSrc: texts of the two headers

namespace xtgh {

namespace {

struct JitState {
    std::mutex mu;
    std::condition_variable cv;  // a kernel another thread was building is ready
    std::unordered_map<std::string, std::unique_ptr<Kernel>> kernels;
    std::unordered_set<std::string> building;  // compiled / loaded right now, outside the lock
    int background = 0;                        // compile_async threads still running
    xtg_jit_stats st{};
};
JitState& js() {
    static JitState* s = new JitState();  // never destroyed: a background compile may outlive main()
    return *s;
}
std::atomic<int64_t> g_launches{0};

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

std::string cache_dir() {
    const char* d = getenv("XTG_CACHE_DIR");
    std::string dir;
    if (d && *d) dir = d;
    else {
        const char* home = getenv("HOME");
        dir = std::string(home && *home ? home : "/tmp") + "/.cache/xtensor_gb300";
    }
    return dir;
}

void mkdirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
    }
    mkdir(path.c_str(), 0755);
}

bool read_file(const std::string& p, std::string& out) {
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

void write_file_atomic(const std::string& p, const std::string& data) {
    std::string tmp = p + ".tmp." + std::to_string(getpid());
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f) return;
        f.write(data.data(), (std::streamsize)data.size());
    }
    rename(tmp.c_str(), p.c_str());
}

xtg_status compile(const std::string& expr, const std::string& arch, std::string& cubin, std::string& lowered) {
    const char* hdr_src[2] = {kXtgParamsSrc, kXtgDeviceSrc};
    const char* hdr_name[2] = {"xtg_params.h", "xtg_device.cuh"};
    nvrtcProgram prog;
    const char* src = "#include \"xtg_device.cuh\"\n";
    nvrtcResult r = nvrtcCreateProgram(&prog, src, "xtg_jit.cu", 2, hdr_src, hdr_name);
    if (r != NVRTC_SUCCESS) return fail(XTG_ERR_JIT, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
    std::string name_expr = "&" + expr;
    nvrtcAddNameExpression(prog, name_expr.c_str());
    std::string archopt = "--gpu-architecture=" + arch;
    const char* opts[] = {archopt.c_str(), "--std=c++17", "--fmad=false", "-DXTG_NVRTC=1"};
    r = nvrtcCompileProgram(prog, 4, opts);
    if (r != NVRTC_SUCCESS) {
        size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        nvrtcDestroyProgram(&prog);
        if (log.size() > 4000) log = log.substr(0, 4000) + "...";
        return fail(XTG_ERR_JIT, "NVRTC failed for " + expr + ":\n" + log);
    }
    const char* low = nullptr;
    nvrtcGetLoweredName(prog, name_expr.c_str(), &low);
    lowered = low ? low : "";
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin.assign(n, '\0');
    if (n) nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    if (lowered.empty() || cubin.empty()) return fail(XTG_ERR_JIT, "NVRTC produced no cubin for " + expr);
    return XTG_OK;
}

}  // namespace

// The kernels launched by the calling thread's last evaluation call, as a
// list of kernels (the names are joined only when asked for: they are long).
static thread_local std::vector<const Kernel*> t_last_kernels;
static thread_local std::string t_last_kernels_str;

void begin_call() { t_last_kernels.clear(); }

// Occupancy for a (block, dynamic shared memory) configuration; sets the
// kernel's dynamic shared memory limit to the request.
static xtg_status configure(Kernel* k, int block, size_t dyn_smem) {
    if (dry_run() || !k->fn) {
        k->block = block;
        k->dyn_smem = dyn_smem;
        return XTG_OK;
    }
    if (k->block == block && k->dyn_smem == dyn_smem && k->max_blocks_per_sm > 0) return XTG_OK;
    // the dynamic limit covers the request whatever the kernel's static
    // shared memory (static + dynamic above 48 KiB needs the opt-in); it is
    // raised, never lowered: a kernel whose dynamic size depends on the call
    // (a row length, a segment count) keeps the launches recorded in cached
    // plans for larger calls valid
    if (dyn_smem > k->smem_limit) {
        XTG_CU(drv().FuncSetAttribute(k->fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)dyn_smem));
        k->smem_limit = dyn_smem;
    }
    int nb = 0;
    if (drv().OccupancyMaxActiveBlocksPerMultiprocessor(&nb, k->fn, block, dyn_smem) != CUDA_SUCCESS) nb = 1;
    k->max_blocks_per_sm = nb > 0 ? nb : 1;
    k->block = block;
    k->dyn_smem = dyn_smem;
    return XTG_OK;
}

xtg_status build_kernel(const std::string& expr, DeviceInfo* dev, std::unique_ptr<Kernel>& k, bool& compiled,
                        bool& from_disk, double& secs);

// The cache lock is not held while a kernel is compiled or loaded: other
// threads keep launching cached kernels meanwhile; a second request for a
// kernel that is being built waits for it instead of compiling it again.
xtg_status get_kernel(const std::string& expr, int block, Kernel** out, size_t dyn_smem) {
    DeviceInfo* dev;
    XTG_TRY(ensure_device(&dev));
    JitState& S = js();
    // dry-run kernels have no function handle: keep them apart
    const std::string key = dry_run() ? "dry:" + expr : expr;
    {
        std::unique_lock<std::mutex> lk(S.mu);
        for (;;) {
            auto it = S.kernels.find(key);
            if (it != S.kernels.end()) {
                S.st.memory_hits++;
                *out = it->second.get();
                return configure(*out, block, dyn_smem);
            }
            if (!S.building.count(key)) break;
            S.cv.wait(lk);
        }
        S.building.insert(key);
    }
    struct Done {
        JitState& S;
        const std::string& key;
        ~Done() {
            std::lock_guard<std::mutex> lk(S.mu);
            S.building.erase(key);
            S.cv.notify_all();
        }
    } done{S, key};
    std::unique_ptr<Kernel> k;
    bool compiled = false, disk = false;
    double secs = 0;
    XTG_TRY(build_kernel(expr, dev, k, compiled, disk, secs));
    std::lock_guard<std::mutex> lk(S.mu);
    if (compiled) {
        S.st.compiles++;
        S.st.compile_seconds += secs;
    }
    if (disk) S.st.disk_hits++;
    Kernel* kp = k.get();
    S.kernels.emplace(key, std::move(k));
    *out = kp;
    if (dry_run()) {
        kp->block = block;
        return XTG_OK;
    }
    return configure(kp, block, dyn_smem);
}

bool kernel_ready(const std::string& expr) {
    JitState& S = js();
    std::lock_guard<std::mutex> lk(S.mu);
    return S.kernels.count(dry_run() ? "dry:" + expr : expr) > 0;
}

void compile_async(const std::string& expr, int block, size_t dyn_smem) {
    JitState& S = js();
    {
        std::lock_guard<std::mutex> lk(S.mu);
        const std::string key = dry_run() ? "dry:" + expr : expr;
        if (S.kernels.count(key) || S.building.count(key)) return;
        S.background++;
    }
    std::thread([expr, block, dyn_smem]() {
        Kernel* k = nullptr;
        get_kernel(expr, block, &k, dyn_smem);
        clear_error();
        JitState& S = js();
        std::lock_guard<std::mutex> lk(S.mu);
        S.background--;
        S.cv.notify_all();
    }).detach();
}

void wait_background_compiles(int64_t timeout_ms) {
    JitState& S = js();
    std::unique_lock<std::mutex> lk(S.mu);
    S.cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return S.background == 0; });
}

// Compiles (or reads from the disk cache) and loads one kernel; no shared state.
xtg_status build_kernel(const std::string& expr, DeviceInfo* dev, std::unique_ptr<Kernel>& k, bool& compiled,
                        bool& from_disk, double& secs) {
    char arch[32];
    snprintf(arch, sizeof arch, "sm_%d%da", dev->cc_major, dev->cc_minor);
    int vmaj = 0, vmin = 0;
    nvrtcVersion(&vmaj, &vmin);
    const std::string key_src = expr + "\n" + arch + "\n" + std::to_string(vmaj) + "." + std::to_string(vmin) + "\n";
    uint64_t h = fnv1a(kXtgDeviceSrc, fnv1a(kXtgParamsSrc, fnv1a(key_src)));
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)h);
    const std::string dir = cache_dir();
    const std::string path = dir + "/" + hex + ".cubin";

    std::string blob, cubin, lowered;
    from_disk = false;
    compiled = false;
    if (read_file(path, blob) && blob.size() > 8) {
        uint32_t nl = 0;
        memcpy(&nl, blob.data(), 4);
        if (nl > 0 && 4 + (size_t)nl < blob.size()) {
            lowered.assign(blob.data() + 4, nl);
            cubin.assign(blob.data() + 4 + nl, blob.size() - 4 - nl);
            from_disk = true;
        }
    }
    if (!from_disk) {
        auto t0 = std::chrono::steady_clock::now();
        XTG_TRY(compile(expr, arch, cubin, lowered));
        auto t1 = std::chrono::steady_clock::now();
        compiled = true;
        secs = std::chrono::duration<double>(t1 - t0).count();
        mkdirs(dir);
        uint32_t nl = (uint32_t)lowered.size();
        std::string b(4, '\0');
        memcpy(&b[0], &nl, 4);
        write_file_atomic(path, b + lowered + cubin);
    }
    k.reset(new Kernel);
    k->name = expr;
    if (dry_run()) {
        k->max_blocks_per_sm = 4;
        return XTG_OK;
    }
    CUmodule mod;
    CUresult cr = drv().ModuleLoadData(&mod, cubin.data());
    if (cr != CUDA_SUCCESS) {
        if (from_disk) unlink(path.c_str());
        return cu_fail(cr, "cuModuleLoadData");
    }
    XTG_CU(drv().ModuleGetFunction(&k->fn, mod, lowered.c_str()));
    k->max_blocks_per_sm = 0;
    return XTG_OK;
}

Recorder*& recorder() {
    static thread_local Recorder* r = nullptr;
    return r;
}

xtg_status launch_raw(Kernel* k, unsigned grid, unsigned block, const void* params, size_t psize, cudaStream_t stream,
                      size_t dyn_smem, int scratch_off) {
    if (grid == 0) return XTG_OK;
    if (Recorder* rec = recorder()) {
        RecLaunch l;
        l.k = k;
        l.grid = grid;
        l.block = block;
        l.smem = dyn_smem;
        l.params.assign((const unsigned char*)params, (const unsigned char*)params + psize);
        l.scratch_off = scratch_off;
        rec->launches.push_back(std::move(l));
    }
    t_last_kernels.push_back(k);
    if (dry_run()) {
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return XTG_OK;
    }
    void* args[1] = {const_cast<void*>(params)};
    if (opt("launch.pdl", 1)) {
        // programmatic dependent launch: the kernel may be set up while the
        // one before it drains (every kernel waits for its predecessors on
        // entry, griddepcontrol.wait)
        CUlaunchAttribute at[1];
        memset(at, 0, sizeof at);
        at[0].id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
        at[0].value.programmaticStreamSerializationAllowed = 1;
        CUlaunchConfig cfg;
        memset(&cfg, 0, sizeof cfg);
        cfg.gridDimX = grid;
        cfg.gridDimY = cfg.gridDimZ = 1;
        cfg.blockDimX = block;
        cfg.blockDimY = cfg.blockDimZ = 1;
        cfg.sharedMemBytes = (unsigned)dyn_smem;
        cfg.hStream = (CUstream)stream;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        XTG_CU(drv().LaunchKernelEx(&cfg, k->fn, args, nullptr));
    } else {
        XTG_CU(drv().LaunchKernel(k->fn, grid, 1, 1, block, 1, 1, (unsigned)dyn_smem, (CUstream)stream, args, nullptr));
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return XTG_OK;
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

}  // namespace xtgh

extern "C" const char* xtg_last_kernels(void) {
    std::string& r = xtgh::t_last_kernels_str;
    r.clear();
    for (const xtgh::Kernel* k : xtgh::t_last_kernels) {
        if (!r.empty()) r += ";";
        r += k->name.compare(0, 5, "xtg::") == 0 ? k->name.substr(5) : k->name;
    }
    return r.c_str();
}

extern "C" xtg_status xtg_get_jit_stats(xtg_jit_stats* st) {
    if (!st) return xtgh::fail(XTG_ERR_INVALID, "null stats");
    xtgh::JitState& S = xtgh::js();
    std::lock_guard<std::mutex> lk(S.mu);
    *st = S.st;
    st->launches = xtgh::g_launches.load();
    return XTG_OK;
}
