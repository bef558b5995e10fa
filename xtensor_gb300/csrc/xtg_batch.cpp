// xtg_batch.cpp — the batching layer: one persistent launch (optionally a
// CUDA graph) over thousands of uneven instances of one expression shape,
// with a launch configuration chosen by a measured autotuner.
//
// No counterpart in xtensor: the reference evaluates every expression on its
// own (one assign / one reducer at a time).  Each instance here is exactly the
// reference's 2-D assign `out = tree(leaves)` or `out = sum(tree, {1})`
// (include/xtensor/core/xassign.hpp:439-478, reducers/xreducer.hpp:1778-1828)
// with its own shapes and strides.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "xtg_plan.h"
#include "xtg_params.h"

using namespace xtgh;

struct xtg_batch {
    xtg_expr templ;
    bool reduce = false;
    xtg_reduce_desc rd;
    std::vector<xtg::BatchInst> inst;
    std::vector<int64_t> inst_bytes;
    int out_dtype = -1;
    int64_t elements = 0;
    int64_t bytes = 0;
    // device state (stream-ordered allocations; host copies stay alive until
    // the batch is destroyed, so uploads never wait for the stream)
    xtg::BatchInst* d_inst = nullptr;
    xtg::BatchTile* d_tiles = nullptr;
    int* d_counter = nullptr;
    int64_t ntiles = 0;
    size_t tiles_cap = 0;
    std::vector<std::vector<xtg::BatchTile>> h_tiles;
    cudaStream_t stream = nullptr;  // stream of the last allocation / launch
    cudaEvent_t last = nullptr;     // recorded after every upload and launch: destroy waits on it,
                                    // never on the stream (which may be gone by then)
    // configuration
    int gl = 32, unroll = 4, cpsm = 4;
    int vec = 1;  // reductions: elements per vector load (1: the strided form)
    int64_t tile_elems = 32768;
    int tuned = 0;
    std::string kname;  // kernel name for the current group width
    Kernel* k = nullptr;
    xtg::BatchParams params;
    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool built = false;
};

namespace {

std::mutex g_tune_mu;

std::string tune_dir() {
    const char* d = getenv("XTG_CACHE_DIR");
    if (d && *d) return d;
    const char* home = getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/xtensor_gb300";
}

void mkdir_p(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
    }
    mkdir(path.c_str(), 0755);
}

// the autotuner's cache: "key gl tile_elems cpsm microseconds" per line
bool tune_lookup(const std::string& key, int& gl, int64_t& te, int& cpsm) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::ifstream f(tune_dir() + "/autotune.txt");
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        std::string k;
        int a, c;
        long long b;
        double us;
        if (ss >> k >> a >> b >> c >> us && k == key) {
            gl = a;
            te = b;
            cpsm = c;
            found = true;
        }
    }
    return found;
}

void tune_store(const std::string& key, int gl, int64_t te, int cpsm, double us) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    mkdir_p(tune_dir());
    std::ofstream f(tune_dir() + "/autotune.txt", std::ios::app);
    f << key << " " << gl << " " << te << " " << cpsm << " " << us << "\n";
}

int ilog2(int64_t v) {
    int r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}

xtg_status make_tiles(xtg_batch* b, int64_t te, std::vector<xtg::BatchTile>& tiles) {
    tiles.clear();
    for (size_t i = 0; i < b->inst.size(); ++i) {
        const auto& I = b->inst[i];
        if (I.rows == 0 || I.cols == 0) continue;
        int64_t rpt = std::max<int64_t>(1, te / std::max<int64_t>(I.cols, 1));
        rpt = std::min<int64_t>(rpt, 1 << 20);
        for (int64_t r = 0; r < I.rows; r += rpt) {
            xtg::BatchTile t;
            t.inst = (int)i;
            t.row0 = r;
            t.nrows = (int)std::min<int64_t>(rpt, I.rows - r);
            tiles.push_back(t);
        }
    }
    return XTG_OK;
}

xtg_status upload_tiles(xtg_batch* b, int64_t te, cudaStream_t s) {
    b->h_tiles.emplace_back();
    std::vector<xtg::BatchTile>& tiles = b->h_tiles.back();
    XTG_TRY(make_tiles(b, te, tiles));
    if (tiles.size() > b->tiles_cap) {
        if (b->d_tiles) XTG_CUDA(cudaFreeAsync(b->d_tiles, s));
        b->tiles_cap = tiles.size() + 64;
        XTG_CUDA(cudaMallocAsync((void**)&b->d_tiles, b->tiles_cap * sizeof(xtg::BatchTile), s));
    }
    if (!tiles.empty())
        XTG_CUDA(cudaMemcpyAsync(b->d_tiles, tiles.data(), tiles.size() * sizeof(xtg::BatchTile), cudaMemcpyHostToDevice, s));
    b->stream = s;
    b->ntiles = (int64_t)tiles.size();
    b->tile_elems = te;
    return XTG_OK;
}

std::string kernel_name(xtg_batch* b, const Tree& t, int gl, const AccChoice* ch) {
    std::vector<int> map(t.leaves.size());
    for (size_t l = 0; l < map.size(); ++l) map[l] = (int)l;
    std::string ls = "xtg::LeafSet<";
    for (size_t l = 0; l < t.leaves.size(); ++l) {
        if (l) ls += ", ";
        ls += std::string("xtg::LeafSpec<") + dt(t.leaves[l].dtype).cname + ", 2>";
    }
    ls += ">";
    const std::string tree = tree_type(t, t.root, map);
    if (b->reduce)
        return "xtg::k_batch_rowreduce<" + tree + ", " + ls + ", " + ch->acc + ", " + dt(b->out_dtype).cname + ", " +
               std::to_string(ch->post) + ", " + std::to_string(gl) + ", " +
               std::to_string(b->vec > 1 ? (int)opt("batch.vec_unroll", 3) : b->unroll) + ", " + std::to_string(b->vec) +
               ", " + std::to_string(b->vec > 1 ? (int)opt("batch.vec_minblocks", 4) : 1) + ">";
    return "xtg::k_batch_assign<" + tree + ", " + ls + ", " + dt(b->out_dtype).cname + ", " + std::to_string(gl) + ", " +
           std::to_string(b->unroll) + ">";
}

xtg_status mark(xtg_batch* b, cudaStream_t s) {
    if (dry_run()) return XTG_OK;
    if (!b->last) XTG_CUDA(cudaEventCreateWithFlags(&b->last, cudaEventDisableTiming));
    XTG_CUDA(cudaEventRecord(b->last, s));
    return XTG_OK;
}

xtg_status launch_once(xtg_batch* b, cudaStream_t s) {
    DeviceInfo* dev;
    XTG_TRY(ensure_device(&dev));
    if (!dry_run()) XTG_CUDA(cudaMemsetAsync(b->d_counter, 0, sizeof(int), s));
    b->stream = s;
    int64_t cap = (int64_t)std::min(b->k->max_blocks_per_sm, b->cpsm) * dev->sm_count;
    unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(b->ntiles, cap));
    XTG_TRY(launch(b->k, grid, 256, &b->params, s));
    return mark(b, s);
}

// The parts of a build that decide the kernel: the tree, the accumulator,
// the vector form and the default group width.
xtg_status plan_kernel(xtg_batch* b, Tree& t, AccChoice& ch, int& gl_default, std::vector<int64_t>& cols,
                       std::vector<int64_t>& rows) {
    const bool demote = opt("fp32_compute", 1) != 0 && b->out_dtype != XTG_FLOAT64;
    XTG_TRY(build_tree(&b->templ, demote, t, false));
    if (b->reduce) {
        XTG_TRY(choose_acc(t, &b->rd, ch));
        if (ch.result_dtype != b->out_dtype)
            return fail(XTG_ERR_INVALID, "batch output dtype differs from the reduction's result type");
    }
    // vector form of the row reduction: every leaf of every instance
    // contiguous or broadcast along its rows, all leaves of one element size
    b->vec = 1;
    if (b->reduce && !t.leaves.empty() && opt("batch.vec", 1)) {
        const int esz = dt(t.leaves[0].dtype).size;
        bool ok = esz >= 1 && esz <= 8 && 16 % esz == 0;
        for (auto& L : t.leaves) ok = ok && dt(L.dtype).size == esz;
        for (auto& I : b->inst)
            for (size_t l = 0; ok && l < t.leaves.size(); ++l) ok = I.cs[l] == 0 || I.cs[l] == 1;
        if (ok) b->vec = 16 / esz;
    }
    cols.clear();
    rows.clear();
    for (auto& I : b->inst) {
        cols.push_back(I.cols);
        rows.push_back(I.rows);
    }
    std::sort(cols.begin(), cols.end());
    std::sort(rows.begin(), rows.end());
    gl_default = (int)opt("batch.group_lanes", -1);
    if (gl_default < 0) gl_default = cols[cols.size() / 2] >= 512 ? 32 : (cols[cols.size() / 2] >= 128 ? 16 : 8);
    return XTG_OK;
}

}  // namespace

xtg_status xtgh::batch_planned_kernel(xtg_batch* b, std::string* name) {
    if (!b || b->inst.empty()) return fail(XTG_ERR_INVALID, "empty batch");
    Tree t;
    AccChoice ch;
    int gl;
    std::vector<int64_t> cols, rows;
    XTG_TRY(plan_kernel(b, t, ch, gl, cols, rows));
    *name = kernel_name(b, t, gl, b->reduce ? &ch : nullptr);
    return XTG_OK;
}

extern "C" {

xtg_status xtg_batch_create(const xtg_expr* templ, const xtg_reduce_desc* rd, xtg_batch** out) {
    if (!templ || !out) return fail(XTG_ERR_INVALID, "null argument");
    Tree t;
    XTG_TRY(build_tree(templ, false, t, false));
    if (t.n_rstats) return fail(XTG_ERR_UNSUPPORTED, "row statistics in a batch template");
    if (rd) {
        if (rd->n_axes != 1) return fail(XTG_ERR_UNSUPPORTED, "batched reductions reduce the last axis only");
        if (rd->op == XTG_RED_VARIANCE || rd->op == XTG_RED_STDDEV || rd->op == XTG_RED_PROD)
            return fail(XTG_ERR_UNSUPPORTED, "batched reduction op not supported");
    }
    xtg_batch* b = new xtg_batch();
    b->templ = *templ;
    b->reduce = rd != nullptr;
    if (rd) b->rd = *rd;
    *out = b;
    return XTG_OK;
}

xtg_status xtg_batch_add(xtg_batch* b, const xtg_array* leaves, int32_t n_leaves, const xtg_array* out) {
    if (!b || !out || (n_leaves && !leaves)) return fail(XTG_ERR_INVALID, "null argument");
    if (b->built) return fail(XTG_ERR_INVALID, "batch already built");
    if (n_leaves != b->templ.n_leaves) return fail(XTG_ERR_INVALID, "instance leaf count differs from the template");
    xtg_expr e = b->templ;
    for (int i = 0; i < n_leaves; ++i) {
        if (leaves[i].dtype != b->templ.leaves[i].dtype || leaves[i].rank != b->templ.leaves[i].rank)
            return fail(XTG_ERR_INVALID, "instance leaf dtype/rank differs from the template");
        if (leaves[i].rank > 2) return fail(XTG_ERR_UNSUPPORTED, "batched instances are at most 2-D");
        e.leaves[i] = leaves[i];
    }
    Tree t;
    XTG_TRY(build_tree(&e, false, t, false));
    int64_t rows = t.rank == 2 ? t.shape[0] : 1;
    int64_t cols = t.rank >= 1 ? t.shape[t.rank - 1] : 1;
    xtg::BatchInst I;
    memset(&I, 0, sizeof I);
    I.rows = rows;
    I.cols = cols;
    const int64_t shp[2] = {rows, cols};
    int64_t bytes = 0;
    for (int i = 0; i < e.n_leaves; ++i) {
        int s = t.expr_slot[i];
        if (s < 0) continue;
        int64_t st[2];
        bstrides_to(e.leaves[i], 2, shp, st);
        I.leaf[s] = e.leaves[i].data;
        I.rs[s] = st[0];
        I.cs[s] = st[1];
        int64_t n = 1;
        for (int d = 0; d < e.leaves[i].rank; ++d) n *= e.leaves[i].shape[d];
        bytes += n * dt(e.leaves[i].dtype).size;
    }
    if (b->out_dtype < 0) b->out_dtype = out->dtype;
    if (out->dtype != b->out_dtype) return fail(XTG_ERR_INVALID, "instance output dtype differs from the batch's");
    I.out = out->data;
    if (b->reduce) {
        int64_t on = 1;
        for (int d = 0; d < out->rank; ++d) on *= out->shape[d];
        if (on != rows) return fail(XTG_ERR_SHAPE, "reduction output must hold one value per row");
        I.ors = out->rank >= 1 ? out->strides[0] : 0;
        if (out->rank == 2 && out->shape[0] == 1) I.ors = out->strides[1];
        I.ocs = 0;
        I.divisor = (double)cols;
        bytes += rows * dt(out->dtype).size;
    } else {
        if (out->rank == 2) {
            if (out->shape[0] != rows || out->shape[1] != cols) return fail(XTG_ERR_SHAPE, "instance output shape mismatch");
            I.ors = out->strides[0];
            I.ocs = out->strides[1];
        } else if (out->rank == 1 && rows == 1) {
            if (out->shape[0] != cols) return fail(XTG_ERR_SHAPE, "instance output shape mismatch");
            I.ors = 0;
            I.ocs = out->strides[0];
        } else {
            return fail(XTG_ERR_SHAPE, "instance output shape mismatch");
        }
        bytes += rows * cols * dt(out->dtype).size;
    }
    if (!out->data) return fail(XTG_ERR_INVALID, "null output data");
    b->inst.push_back(I);
    b->elements += rows * cols;
    b->bytes += bytes;
    return XTG_OK;
}

xtg_status xtg_batch_build(xtg_batch* b, int32_t autotune, xtg_stream stream) {
    if (!b) return fail(XTG_ERR_INVALID, "null batch");
    if (b->inst.empty()) return fail(XTG_ERR_INVALID, "empty batch");
    DeviceInfo* dev;
    XTG_TRY(ensure_device(&dev));
    cudaStream_t s = (cudaStream_t)stream;
    Tree t;
    AccChoice ch;
    int gl_default;
    std::vector<int64_t> cols, rows;
    XTG_TRY(plan_kernel(b, t, ch, gl_default, cols, rows));
    // device work list
    if (!dry_run()) {
        if (!b->d_inst) XTG_CUDA(cudaMallocAsync((void**)&b->d_inst, b->inst.size() * sizeof(xtg::BatchInst), s));
        XTG_CUDA(cudaMemcpyAsync(b->d_inst, b->inst.data(), b->inst.size() * sizeof(xtg::BatchInst),
                                 cudaMemcpyHostToDevice, s));
        if (!b->d_counter) XTG_CUDA(cudaMallocAsync((void**)&b->d_counter, 256, s));
        b->stream = s;
    }
    memset(&b->params, 0, sizeof b->params);
    b->params.inst = b->d_inst;
    b->params.counter = b->d_counter;
    for (size_t i = 0; i < t.scalars.size(); ++i) b->params.scal.v[i] = t.scalars[i];
    if (b->reduce) {
        b->params.init_f = ch.init_f;
        b->params.init_i = ch.init_i;
        b->params.has_initial = ch.has_initial;
        b->params.initial_f = ch.initial_f;
        b->params.initial_i = ch.initial_i;
    }
    // shape class for the tuning cache
    const std::string base = kernel_name(b, t, 0, b->reduce ? &ch : nullptr);
    char cls[160];
    snprintf(cls, sizeof cls, "|n%d|c%d|r%d|e%d|sm%d", ilog2((int64_t)b->inst.size()), ilog2(cols[cols.size() / 2]),
             ilog2(rows[rows.size() / 2]), ilog2(b->elements), dev->sm_count);
    std::string key;
    for (char c : base + cls)
        if (c != ' ') key += c;

    int gl = gl_default, cpsm = (int)opt("batch.ctas_per_sm", 4);
    int64_t te = opt("batch.tile_elems", 32768);
    b->tuned = 0;
    if (autotune && !dry_run()) {
        int tg, tc;
        int64_t tt;
        if (tune_lookup(key, tg, tt, tc)) {
            gl = tg;
            te = tt;
            cpsm = tc;
            b->tuned = 2;
        } else {
            // measured search: group width x tile size x CTAs per SM.  Stage
            // 1 times every candidate (median of 5); stage 2 re-times the
            // candidates within 3% of the best (median of 9) and keeps the
            // fastest, where a candidate must beat the one before it in the
            // fixed order by more than 1% to replace it, so that near-ties
            // resolve the same way on every run.
            const int gls[3] = {8, 16, 32};
            const int64_t tes[3] = {8192, 32768, 131072};
            const int cps[3] = {2, 4, 8};
            struct Cand {
                int g;
                int64_t t;
                int c;
                double ms;
            };
            std::vector<Cand> cands;
            double best = 1e30;
            cudaEvent_t e0, e1;
            XTG_CUDA(cudaEventCreate(&e0));
            XTG_CUDA(cudaEventCreate(&e1));
            auto time_cand = [&](const Cand& cd, int reps, double* med) -> xtg_status {
                XTG_TRY(upload_tiles(b, cd.t, s));
                b->params.tiles = b->d_tiles;
                b->params.ntiles = b->ntiles;
                XTG_TRY(get_kernel(kernel_name(b, t, cd.g, b->reduce ? &ch : nullptr), 256, &b->k));
                b->cpsm = cd.c;
                XTG_TRY(launch_once(b, s));  // warm-up
                std::vector<float> ms((size_t)reps);
                for (int r = 0; r < reps; ++r) {
                    XTG_CUDA(cudaEventRecord(e0, s));
                    XTG_TRY(launch_once(b, s));
                    XTG_CUDA(cudaEventRecord(e1, s));
                    XTG_CUDA(cudaEventSynchronize(e1));
                    XTG_CUDA(cudaEventElapsedTime(&ms[(size_t)r], e0, e1));
                }
                std::sort(ms.begin(), ms.end());
                *med = ms[(size_t)reps / 2];
                return XTG_OK;
            };
            for (int64_t tcand : tes)
                for (int gcand : gls)
                    for (int ccand : cps) {
                        Cand cd{gcand, tcand, ccand, 0.0};
                        XTG_TRY(time_cand(cd, 5, &cd.ms));
                        cands.push_back(cd);
                        best = std::min(best, cd.ms);
                    }
            const double cut = best * 1.03;
            int pick = -1;
            for (size_t i = 0; i < cands.size(); ++i) {
                if (cands[i].ms > cut) continue;
                XTG_TRY(time_cand(cands[i], 9, &cands[i].ms));
                if (pick < 0 || cands[i].ms < cands[(size_t)pick].ms * 0.99) pick = (int)i;
            }
            gl = cands[(size_t)pick].g;
            te = cands[(size_t)pick].t;
            cpsm = cands[(size_t)pick].c;
            best = cands[(size_t)pick].ms;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            tune_store(key, gl, te, cpsm, best * 1e3);
            b->tuned = 1;
        }
    }
    b->gl = gl;
    b->cpsm = cpsm;
    if (!dry_run()) {
        XTG_TRY(upload_tiles(b, te, s));
    } else {
        std::vector<xtg::BatchTile> tiles;
        make_tiles(b, te, tiles);
        b->ntiles = (int64_t)tiles.size();
        b->tile_elems = te;
    }
    b->params.tiles = b->d_tiles;
    b->params.ntiles = b->ntiles;
    b->kname = kernel_name(b, t, gl, b->reduce ? &ch : nullptr);
    XTG_TRY(get_kernel(b->kname, 256, &b->k));
    b->built = true;
    XTG_TRY(mark(b, s));  // the uploads are ordered before the event destroy waits on
    return XTG_OK;
}

xtg_status xtg_batch_run(xtg_batch* b, xtg_stream stream) {
    if (!b || !b->built) return fail(XTG_ERR_INVALID, "batch not built");
    begin_call();
    return launch_once(b, (cudaStream_t)stream);
}

xtg_status xtg_batch_capture(xtg_batch* b, xtg_stream stream) {
    if (!b || !b->built) return fail(XTG_ERR_INVALID, "batch not built");
    if (!stream) return fail(XTG_ERR_INVALID, "graph capture needs a created stream");
    cudaStream_t s = (cudaStream_t)stream;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    XTG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    xtg_status st = launch_once(b, s);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (st != XTG_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    b->graph = g;
    XTG_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return XTG_OK;
}

xtg_status xtg_batch_replay(xtg_batch* b, xtg_stream stream) {
    if (!b || !b->exec) return fail(XTG_ERR_INVALID, "no captured graph");
    XTG_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    XTG_TRY(mark(b, (cudaStream_t)stream));
    count_launch();
    return XTG_OK;
}

xtg_status xtg_batch_get_info(const xtg_batch* b, xtg_batch_info* info) {
    if (!b || !info) return fail(XTG_ERR_INVALID, "null argument");
    memset(info, 0, sizeof *info);
    info->instances = (int64_t)b->inst.size();
    info->tiles = b->ntiles;
    info->elements = b->elements;
    info->algorithmic_bytes = b->bytes;
    info->group_lanes = b->gl;
    info->unroll = b->unroll;
    info->ctas_per_sm = b->cpsm;
    info->tuned = b->tuned;
    info->tile_elems = b->tile_elems;
    info->graph_ready = b->exec != nullptr;
    return XTG_OK;
}

xtg_status xtg_batch_destroy(xtg_batch* b) {
    if (!b) return XTG_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (!dry_run()) {
        // wait for the batch's last upload / launch (its own event: the
        // caller may have destroyed the stream it used), then free on the
        // per-thread stream — cudaFree would synchronise the whole device,
        // stalling a server that destroys batches while others run
        if (b->last) {
            cudaEventSynchronize(b->last);
            cudaEventDestroy(b->last);
        } else if (b->stream) {
            cudaDeviceSynchronize();
        }
        if (b->d_inst) cudaFreeAsync(b->d_inst, cudaStreamPerThread);
        if (b->d_tiles) cudaFreeAsync(b->d_tiles, cudaStreamPerThread);
        if (b->d_counter) cudaFreeAsync(b->d_counter, cudaStreamPerThread);
    }
    delete b;
    return XTG_OK;
}

}  // extern "C"
