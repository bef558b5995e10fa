// xtg_plan.h — host-side planning of expression trees (internal).
#pragma once

#include <array>
#include <string>
#include <vector>

#include "xtg_internal.h"
#include "xtg_params.h"

namespace xtgh {

// One node of a parsed expression tree.
struct PNode {
    int op = 0;
    int dtype = -1;   // inferred result type (after fp32 demotion when enabled)
    int cxx_dtype = -1;  // C++ result type before demotion
    int arg = 0, aux = 0;
    xtg_value imm{};
    std::vector<int> kids;
    int scal = -1;    // scalar slot
    int leaf = -1;    // leaf slot (after dedup)
    int stat = -1;    // row-statistic slot (R* nodes)
};

struct Tree {
    std::vector<PNode> nodes;
    int root = -1;
    std::vector<xtg_array> leaves;  // deduplicated
    std::vector<uint64_t> scalars;  // encoded immediates
    int n_rstats = 0;
    int rstat_axes = -1;            // trailing-axis count shared by R* nodes
    bool has_f64_leaf = false;
    int rank = 0;                   // broadcast rank
    int64_t shape[XTG_MAX_RANK] = {0};
    std::vector<int> expr_slot;     // xtg_expr leaf index -> leaf slot (-1: unused)
};

// Parse + type-check + broadcast.  `demote` enables float32 evaluation of
// float64 nodes (only when no leaf is float64).  `dedup` merges leaves that
// describe the same array (off for batch templates, whose leaves are
// placeholders).
xtg_status build_tree(const xtg_expr* e, bool demote, Tree& t, bool dedup = true);
int promote(int a, int b);
bool is_rop(int op);
// Type string of the subtree at node `n` (leaf indices through `leaf_map`).
// recip_div: bit 0 float64, bit 1 float32 — divisions of that type by a
// leaf-free (row-invariant) divisor become a multiplication by its reciprocal
// ((a - m) / s becomes fma(a, 1/s, -(m * (1/s)))), whose row-invariant parts
// take statistic slots *slot, *slot + 1, ... (fused row kernels only; slot
// must then be given and is advanced past the slots used).
std::string tree_type(const Tree& t, int n, const std::vector<int>& leaf_map, int recip_div = 0, int* slot = nullptr);
// Broadcast strides of leaf `l` against the tree's shape (rank t.rank).
void leaf_bstrides(const Tree& t, int l, int64_t* st);
// Broadcast strides of array `a` against a target shape of rank `rank`.
void bstrides_to(const xtg_array& a, int rank, const int64_t* shape, int64_t* st);

// An iteration space with the strides of several arrays over it.
struct Dims {
    int R = 0;
    int64_t shape[XTG_MAX_RANK];
    std::vector<std::array<int64_t, XTG_MAX_RANK>> st;
};
// Drop extent-1 dims and merge dims that are contiguous for every array
// (row-major order of the merged dims is preserved).
void collapse(Dims& D);
xtg::FastDiv make_fd(uint64_t d);

// Scratch for split reductions: stream-ordered allocation unless a fixed
// buffer is supplied.
struct ScratchSpec {
    void* fixed = nullptr;
    size_t fixed_bytes = 0;
};
xtg_status reduce_impl(const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* out, cudaStream_t stream,
                       const ScratchSpec* scratch);
xtg_status assign_tree(const Tree& t, const xtg_array* out, cudaStream_t stream);
// xtg_accumulate without the plan cache (used by the filter views).
xtg_status accumulate_call(const xtg_expr* e, int32_t op, int32_t has_axis, int64_t axis, int32_t acc_dtype,
                           const xtg_array* out, cudaStream_t stream);
// assign_tree, through a temporary when a leaf shares memory with `out` but
// is read at other positions than the ones written.
xtg_status assign_guarded(const Tree& t, const xtg_array* out, cudaStream_t stream);
// True when a leaf shares memory with `out` but is read at other positions
// than the ones written.
bool assign_hazard(const Tree& t, const xtg_array& out);
// True when any leaf's byte range overlaps `out`'s.
bool shares_memory(const Tree& t, const xtg_array& out);

// Chunk grid of a chunked array: chunks per dimension (the edge chunk
// included) and their count.
struct ChunkGrid {
    int rank = 0;
    int64_t shape[XTG_MAX_RANK] = {0};
    int64_t cs[XTG_MAX_RANK] = {0};
    int64_t grid[XTG_MAX_RANK] = {0};
    int64_t n = 0;
};
xtg_status chunk_grid(const xtg_chunked& c, ChunkGrid& g);
// Grid coordinates of chunk i (row-major).
void chunk_coords(const ChunkGrid& g, int64_t i, int64_t* gc);
// Row-major element strides inside a chunk.
void chunk_strides(const ChunkGrid& g, int64_t* st);

// Accumulator type string, post-operation and initial values of a reduction.
struct AccChoice {
    std::string acc;
    int post = 0;
    double init_f = 0;
    int64_t init_i = 0;
    int has_initial = 0;
    double initial_f = 0;
    int64_t initial_i = 0;
    int result_dtype = -1;
};
xtg_status choose_acc(const Tree& t, const xtg_reduce_desc* rd, AccChoice& ch);

// ---- plan cache (xtg_plancache.cpp) -----------------------------------------------
bool plan_cache_enabled();
std::vector<unsigned char>& plan_key(int kind, const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* out,
                                    int32_t a0, int32_t a1, int64_t a2, const xtg_array* out2 = nullptr);
bool plan_replay(const std::vector<unsigned char>& key, cudaStream_t s, xtg_status* st);
void plan_store(const std::vector<unsigned char>& key, Recorder& rec);

// Runs `fn` (a planning + launching call) through the plan cache.
template <class F>
xtg_status with_plan_cache(int kind, const xtg_expr* e, const xtg_reduce_desc* rd, const xtg_array* out, int32_t a0,
                           int32_t a1, int64_t a2, cudaStream_t s, F&& fn, const xtg_array* out2 = nullptr) {
    if (!e || !out || !plan_cache_enabled() || recorder()) return fn();
    xtg_status st;
    if (plan_replay(plan_key(kind, e, rd, out, a0, a1, a2, out2), s, &st)) return st;
    Recorder rec;
    recorder() = &rec;
    st = fn();
    recorder() = nullptr;
    // (the planning call may itself have used the thread's key buffer)
    if (st == XTG_OK) plan_store(plan_key(kind, e, rd, out, a0, a1, a2, out2), rec);
    return st;
}

}  // namespace xtgh
