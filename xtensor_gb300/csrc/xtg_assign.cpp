// xtg_assign.cpp — xtg_assign: the device counterpart of
// xexpression_assigner<Tag>::assign_data (include/xtensor/core/xassign.hpp:439-478).
//
// The reference picks between linear_assigner (all operands share the
// destination's layout), strided_loop_assigner (an outer multi-index loop
// around a contiguous SIMD inner loop) and the scalar stepper_assigner
// (transposes, arbitrary strides).  Here:
//   K1 k_assign     — any tree whose leaves are unit-, zero- or arbitrarily
//                     strided along the destination's innermost dim; 128-bit
//                     vectors when alignment allows.  Covers linear and
//                     strided-loop assignment.
//   K2 k_transpose  — one leaf is unit-stride along another dim than the
//                     destination's (transpose / permuted strided_view):
//                     shared-memory tiles make both sides coalesced.
//   K7 k_rowfused   — trees containing keep-dims statistics over trailing
//                     axes, evaluated in one pass.
#include <algorithm>
#include <cmath>
#include <array>
#include <cstring>
#include <string>

#include "xtg_plan.h"
#include "xtg_params.h"

namespace xtgh {

xtg::FastDiv make_fd(uint64_t d) {
    xtg::FastDiv f;
    f.d = (uint32_t)d;
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < d) ++l;
    f.l = l;
    f.m = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / (d ? d : 1)) + 1);
    return f;
}

void bstrides_to(const xtg_array& a, int rank, const int64_t* shape, int64_t* st) {
    for (int d = 0; d < rank; ++d) {
        int ld = d - (rank - a.rank);
        if (ld < 0 || (a.shape[ld] == 1 && shape[d] != 1)) st[d] = 0;
        else st[d] = a.strides[ld];
        if (shape[d] == 1) st[d] = 0;
    }
}

void collapse(Dims& D) {
    int nr = 0;
    int64_t ns[XTG_MAX_RANK];
    std::vector<std::array<int64_t, XTG_MAX_RANK>> nst(D.st.size());
    for (int d = D.R - 1; d >= 0; --d) {
        if (D.shape[d] == 1) continue;
        bool merge = nr > 0;
        for (size_t a = 0; merge && a < D.st.size(); ++a)
            if (D.st[a][d] != nst[a][nr - 1] * ns[nr - 1]) merge = false;
        if (merge) {
            ns[nr - 1] *= D.shape[d];
        } else {
            ns[nr] = D.shape[d];
            for (size_t a = 0; a < D.st.size(); ++a) nst[a][nr] = D.st[a][d];
            ++nr;
        }
    }
    if (nr == 0) {
        ns[0] = 1;
        for (size_t a = 0; a < D.st.size(); ++a) nst[a][0] = 0;
        nr = 1;
    }
    D.R = nr;
    for (int i = 0; i < nr; ++i) {
        D.shape[i] = ns[nr - 1 - i];
        for (size_t a = 0; a < D.st.size(); ++a) D.st[a][i] = nst[a][nr - 1 - i];
    }
}

static int kind_of(int64_t s) { return s == 1 ? 0 : (s == 0 ? 1 : 2); }

static bool aligned(const void* p, int64_t bytes) { return ((uintptr_t)p % (uintptr_t)bytes) == 0; }

static std::string leafset(const Tree& t, const std::vector<int>& order, const std::vector<int>& kinds) {
    std::string s = "xtg::LeafSet<";
    for (size_t i = 0; i < order.size(); ++i) {
        if (i) s += ", ";
        s += std::string("xtg::LeafSpec<") + dt(t.leaves[order[i]].dtype).cname + ", " + std::to_string(kinds[i]) + ">";
    }
    return s + ">";
}

static void fill_scalars(const Tree& t, xtg::Scalars& s) {
    memset(&s, 0, sizeof s);
    for (size_t i = 0; i < t.scalars.size(); ++i) s.v[i] = t.scalars[i];
}

static unsigned grid_for(Kernel* k, int64_t blocks_needed) {
    DeviceInfo* dev;
    ensure_device(&dev);
    int64_t cap = (int64_t)k->max_blocks_per_sm * dev->sm_count;
    int64_t g = std::min<int64_t>(blocks_needed, cap);
    return (unsigned)std::max<int64_t>(g, 1);
}

// Subtree broadcast shape (right-aligned extents of the leaves below node n).
static void subtree_shape(const Tree& t, int n, int& rank, int64_t* sh) {
    std::vector<int> stack{n};
    rank = 0;
    for (int d = 0; d < XTG_MAX_RANK; ++d) sh[d] = 1;
    std::vector<int> leaves;
    while (!stack.empty()) {
        int k = stack.back();
        stack.pop_back();
        if (t.nodes[k].op == XTG_OP_LEAF) leaves.push_back(t.nodes[k].leaf);
        for (int c : t.nodes[k].kids) stack.push_back(c);
    }
    for (int l : leaves) rank = std::max(rank, (int)t.leaves[l].rank);
    for (int l : leaves) {
        const xtg_array& a = t.leaves[l];
        for (int i = 0; i < a.rank; ++i) {
            int d = rank - a.rank + i;
            if (sh[d] == 1) sh[d] = a.shape[i];
        }
    }
}

static xtg_status assign_rowfused(const Tree& t, const xtg_array& out, int R, const int64_t* shape, cudaStream_t stream);

xtg_status assign_tree(const Tree& t, const xtg_array* out, cudaStream_t stream) {
    DeviceInfo* dev;
    XTG_TRY(ensure_device(&dev));
    // destination shape must be the expression's shape, or a broadcast of it
    const int R = out->rank;
    if (t.rank > R) return fail(XTG_ERR_SHAPE, "destination rank is smaller than the expression's");
    for (int i = 0; i < t.rank; ++i) {
        int d = R - t.rank + i;
        if (t.shape[i] != out->shape[d] && t.shape[i] != 1)
            return fail(XTG_ERR_SHAPE, "destination shape does not match the expression shape");
    }
    int64_t n = 1;
    for (int d = 0; d < R; ++d) n *= out->shape[d];
    if (n == 0) return XTG_OK;
    if (!out->data) return fail(XTG_ERR_INVALID, "null destination data");
    for (auto& a : t.leaves)
        if (!a.data) return fail(XTG_ERR_INVALID, "null leaf data");
    for (int d = 0; d < R; ++d)
        if (out->strides[d] == 0 && out->shape[d] > 1)
            return fail(XTG_ERR_INVALID, "destination has a zero stride (broadcast destination)");

    if (t.n_rstats > 0) return assign_rowfused(t, *out, R, out->shape, stream);

    const int NL = (int)t.leaves.size();
    Dims D;
    D.R = R;
    for (int d = 0; d < R; ++d) D.shape[d] = out->shape[d];
    D.st.resize(1 + NL);
    for (int d = 0; d < R; ++d) D.st[0][d] = out->strides[d];
    for (int l = 0; l < NL; ++l) bstrides_to(t.leaves[l], R, out->shape, D.st[1 + l].data());
    if (R == 0) {
        D.R = 1;
        D.shape[0] = 1;
        for (auto& s : D.st) s[0] = 0;
    }
    collapse(D);
    const int RR = D.R, in = RR - 1;
    const int out_dt = out->dtype;
    const int osz = dt(out_dt).size;

    // K2: exactly one leaf is neither unit- nor zero-stride along the inner
    // dim, and it is unit-stride along another dim.
    int tl = -1, ta = -1, nstrided = 0;
    for (int l = 0; l < NL; ++l) {
        int64_t s = D.st[1 + l][in];
        if (s != 0 && s != 1) {
            ++nstrided;
            tl = l;
        }
    }
    if (nstrided == 1 && D.st[0][in] == 1 && RR >= 2 && opt("transpose.enable", 1)) {
        for (int d = 0; d < in; ++d)
            if (D.st[1 + tl][d] == 1) ta = d;
    }
    if (ta >= 0) {
        // leaf order: the transposed leaf first
        std::vector<int> order{tl};
        for (int l = 0; l < NL; ++l)
            if (l != tl) order.push_back(l);
        std::vector<int> map(NL), kinds(NL, 2);
        for (int i = 0; i < NL; ++i) map[order[i]] = i;
        // 64-wide tiles for <= 4-byte elements (256 B per warp row access),
        // 32-wide for 8-byte ones
        const int esz = dt(t.leaves[tl].dtype).size;
        const int TILE = esz <= 4 ? (int)opt("transpose.tile_small", 64) : 32;
        const int ROWS = esz <= 4 ? 256 / TILE : 8;
        xtg::TransposeParams p;
        memset(&p, 0, sizeof p);
        p.sa = D.shape[ta];
        p.sb = D.shape[in];
        p.ntile_a = (p.sa + TILE - 1) / TILE;
        p.ntile_b = (p.sb + TILE - 1) / TILE;
        int nb = 0;
        int64_t nbatch = 1;
        for (int d = 0; d < RR; ++d) {
            if (d == ta || d == in) continue;
            p.bshape[nb] = D.shape[d];
            p.obs[nb] = D.st[0][d];
            for (int i = 0; i < NL; ++i) p.lbs[i][nb] = D.st[1 + order[i]][d];
            nbatch *= D.shape[d];
            ++nb;
        }
        p.nbd = nb;
        p.n_tiles = nbatch * p.ntile_a * p.ntile_b;
        p.out = out->data;
        p.oa = D.st[0][ta];
        p.ob = D.st[0][in];
        for (int i = 0; i < NL; ++i) {
            p.leaf[i] = t.leaves[order[i]].data;
            p.la[i] = D.st[1 + order[i]][ta];
            p.lb[i] = D.st[1 + order[i]][in];
        }
        fill_scalars(t, p.scal);
        std::string name = "xtg::k_transpose<" + tree_type(t, t.root, map) + ", " + leafset(t, order, kinds) + ", " +
                           dt(out_dt).cname + ", " + std::to_string(nb) + ", " + std::to_string(TILE) + ", " +
                           std::to_string(ROWS) + ">";
        Kernel* k;
        XTG_TRY(get_kernel(name, TILE * ROWS, &k));
        return launch(k, grid_for(k, p.n_tiles), TILE * ROWS, &p, stream);
    }

    // K1
    std::vector<int> kinds(NL);
    int maxsz = osz;
    for (int l = 0; l < NL; ++l) {
        kinds[l] = kind_of(D.st[1 + l][in]);
        if (kinds[l] == 0) maxsz = std::max(maxsz, dt(t.leaves[l].dtype).size);
    }
    const int okind = D.st[0][in] == 1 ? 0 : 2;
    int vec = (int)std::min<int64_t>(opt("assign.max_vec_bytes", 16) / maxsz, 16);
    if (vec < 1) vec = 1;
    auto vec_ok = [&](int v) {
        if (v == 1) return true;
        if (D.shape[in] % v) return false;
        auto arr_ok = [&](const void* p, int sz, const std::array<int64_t, XTG_MAX_RANK>& st) {
            if (!aligned(p, (int64_t)v * sz)) return false;
            for (int d = 0; d < in; ++d)
                if (st[d] % v) return false;
            return true;
        };
        if (okind == 0 && !arr_ok(out->data, osz, D.st[0])) return false;
        for (int l = 0; l < NL; ++l)
            if (kinds[l] == 0 && !arr_ok(t.leaves[l].data, dt(t.leaves[l].dtype).size, D.st[1 + l])) return false;
        return true;
    };
    while (vec > 1 && !vec_ok(vec)) vec >>= 1;
    xtg::AssignParams p;
    memset(&p, 0, sizeof p);
    int64_t nvec = 1;
    for (int d = 0; d < RR; ++d) {
        p.sp.shape[d] = d == in ? D.shape[d] / vec : D.shape[d];
        nvec *= p.sp.shape[d];
    }
    p.sp.nvec = nvec;
    const bool big = nvec > 0xFFFFFFF0ll;
    if (!big)
        for (int d = 0; d < RR; ++d) p.sp.fd[d] = make_fd((uint64_t)p.sp.shape[d]);
    p.out = out->data;
    for (int d = 0; d < RR; ++d) p.out_strides[d] = D.st[0][d];
    for (int l = 0; l < NL; ++l) {
        p.leaf[l] = t.leaves[l].data;
        for (int d = 0; d < RR; ++d) p.leaf_strides[l][d] = D.st[1 + l][d];
    }
    fill_scalars(t, p.scal);
    const int U = (int)opt("assign.unroll", vec * maxsz >= 16 ? 4 : 8);
    const int block = (int)opt("assign.block", 256);
    std::vector<int> order(NL), map(NL);
    for (int l = 0; l < NL; ++l) order[l] = map[l] = l;
    std::string name = "xtg::k_assign<" + tree_type(t, t.root, map) + ", " + leafset(t, order, kinds) + ", " +
                       dt(out_dt).cname + ", " + std::to_string(okind) + ", " + std::to_string(vec) + ", " +
                       std::to_string(RR) + ", " + std::to_string(U) + ", " + (big ? "true" : "false") + ">";
    Kernel* k;
    XTG_TRY(get_kernel(name, block, &k));
    int64_t need = (nvec + (int64_t)block * U - 1) / ((int64_t)block * U);
    return launch(k, grid_for(k, need), block, &p, stream);
}

// ---- K7 -----------------------------------------------------------------------
static xtg_status assign_rowfused(const Tree& t, const xtg_array& out, int R, const int64_t* shape, cudaStream_t stream) {
    const int k = t.rstat_axes;
    const int NL = (int)t.leaves.size();
    // every statistic's operand must span the full trailing extents
    for (size_t i = 0; i < t.nodes.size(); ++i) {
        if (!is_rop(t.nodes[i].op)) continue;
        int sr;
        int64_t sh[XTG_MAX_RANK];
        subtree_shape(t, t.nodes[i].kids[0], sr, sh);
        for (int j = 0; j < k; ++j) {
            int ds = sr - 1 - j, dO = R - 1 - j;
            int64_t e = ds >= 0 ? sh[ds] : 1;
            if (e != shape[dO]) return fail(XTG_ERR_UNSUPPORTED, "row statistic over a broadcast operand");
        }
    }
    // strides of out and leaves over the full shape
    std::vector<std::array<int64_t, XTG_MAX_RANK>> st(1 + NL);
    for (int d = 0; d < R; ++d) st[0][d] = out.strides[d];
    for (int l = 0; l < NL; ++l) bstrides_to(t.leaves[l], R, shape, st[1 + l].data());
    // collapse the trailing k dims into one row stride per array
    int64_t row_len = 1;
    for (int d = R - k; d < R; ++d) row_len *= shape[d];
    std::vector<int64_t> li(1 + NL, 0);
    for (size_t a = 0; a < st.size(); ++a) {
        int64_t cur_st = 0, cur_ext = 1;
        bool first = true;
        for (int d = R - 1; d >= R - k; --d) {
            if (shape[d] == 1) continue;
            if (first) {
                cur_st = st[a][d];
                cur_ext = shape[d];
                first = false;
            } else {
                if (st[a][d] != cur_st * cur_ext)
                    return fail(XTG_ERR_UNSUPPORTED, "row dims of an operand are not collapsible");
                cur_ext *= shape[d];
            }
        }
        li[a] = cur_st;
    }
    // outer dims
    Dims D;
    D.R = R - k;
    for (int d = 0; d < D.R; ++d) D.shape[d] = shape[d];
    D.st.resize(1 + NL);
    for (size_t a = 0; a < st.size(); ++a)
        for (int d = 0; d < D.R; ++d) D.st[a][d] = st[a][d];
    collapse(D);
    int64_t n_rows = 1;
    for (int d = 0; d < D.R; ++d) n_rows *= D.shape[d];
    // vector width
    std::vector<int> kinds(NL);
    const int osz = dt(out.dtype).size;
    int maxsz = osz;
    for (int l = 0; l < NL; ++l) {
        kinds[l] = kind_of(li[1 + l]);
        if (kinds[l] == 0) maxsz = std::max(maxsz, dt(t.leaves[l].dtype).size);
    }
    int vec = 16 / maxsz;
    auto vec_ok = [&](int v) {
        if (v == 1) return true;
        if (row_len % v || li[0] != 1) return false;
        auto arr_ok = [&](const void* p, int sz, const std::array<int64_t, XTG_MAX_RANK>& s) {
            if (!aligned(p, (int64_t)v * sz)) return false;
            for (int d = 0; d < D.R; ++d)
                if (s[d] % v) return false;
            return true;
        };
        if (!arr_ok(out.data, osz, D.st[0])) return false;
        for (int l = 0; l < NL; ++l)
            if (kinds[l] == 0 && !arr_ok(t.leaves[l].data, dt(t.leaves[l].dtype).size, D.st[1 + l])) return false;
        return true;
    };
    while (vec > 1 && !vec_ok(vec)) vec >>= 1;
    const int64_t nvec = (row_len + vec - 1) / vec;
    int group, nv;
    auto p2 = [](int64_t x) {
        int64_t r = 1;
        while (r < x) r <<= 1;
        return (int)r;
    };
    if (nvec <= 32 * 16) {
        group = 32;
        nv = p2((nvec + 31) / 32);
    } else if (nvec <= 256 * 16) {
        group = 256;
        nv = p2((nvec + 255) / 256);
    } else {
        return fail(XTG_ERR_UNSUPPORTED, "row too long for the fused row kernel");
    }
    xtg::RowParams p;
    memset(&p, 0, sizeof p);
    p.n_rows = n_rows;
    p.row_len = row_len;
    for (int d = 0; d < D.R; ++d) p.oshape[d] = D.shape[d];
    for (int l = 0; l < NL; ++l) {
        p.leaf[l] = t.leaves[l].data;
        for (int d = 0; d < D.R; ++d) p.lo[l][d] = D.st[1 + l][d];
        p.li[l] = li[1 + l];
    }
    p.out = out.data;
    for (int d = 0; d < D.R; ++d) p.oo[d] = D.st[0][d];
    p.oi = li[0];
    fill_scalars(t, p.scal);
    // statistics (in postfix order = stat index order)
    std::vector<int> order(NL), map(NL);
    for (int l = 0; l < NL; ++l) order[l] = map[l] = l;
    std::string sl = "xtg::StatList<";
    int ns = 0;
    for (size_t i = 0; i < t.nodes.size(); ++i) {
        const PNode& x = t.nodes[i];
        if (!is_rop(x.op)) continue;
        int mode = x.op - XTG_OP_RSUM;
        int sub_dt = t.nodes[x.kids[0]].dtype;
        const char* c = (mode >= 4) ? dt(sub_dt == XTG_BFLOAT16 ? XTG_FLOAT32 : sub_dt).cname
                                    : (sub_dt == XTG_FLOAT32 || sub_dt == XTG_BFLOAT16 ? "float" : "double");
        if (ns++) sl += ", ";
        sl += "xtg::RStat<" + std::to_string(x.stat) + ", " + std::to_string(mode) + ", " + c + ", " +
              tree_type(t, x.kids[0], map) + ">";
        double div = (double)row_len;
        if (x.op == XTG_OP_RVAR || x.op == XTG_OP_RSTD) {
            int64_t ddof = x.aux;
            int64_t total = n_rows * row_len;
            div = n_rows ? (double)((total - ddof) / n_rows) : 0.0;
        }
        p.div[x.stat] = div;
        p.rdiv[x.stat] = 1.0 / div;
        p.vfac[x.stat] = 1.0 / ((double)row_len * div);
        auto e2 = [](double f) {
            int k;
            const double m = std::frexp(f, &k);  // f = m * 2^k, m in [0.5, 1)
            return (m == 0.5 && k - 1 > -1000 && k - 1 < 1000) ? k - 1 + 100000 : 0;
        };
        p.rdiv_e2[x.stat] = e2(p.rdiv[x.stat]);
        p.vfac_e2[x.stat] = e2(p.vfac[x.stat]);
        p.fdiv[x.stat] = (float)div;
    }
    p.rrow_len = 1.0 / (double)row_len;
    p.frow_len = (float)row_len;
    sl += ">";
    const int recip = (opt("row.recip_div_f64", 1) != 0 ? 1 : 0) | (opt("row.recip_div_f32", 1) != 0 ? 2 : 0);
    int nstat = t.n_rstats;  // real statistics, then the reciprocal nodes' row-invariant slots
    const std::string tree = tree_type(t, t.root, map, recip, &nstat);
    const int full = (int64_t)nv * group * vec == row_len ? 1 : 0;

    // Bulk-copy variant: every leaf contiguous along the row, 16-byte rows,
    // warp-sized groups, output contiguous along the row.
    bool tma = opt("row.tma", 1) != 0 && group == 32 && li[0] == 1 && NL > 0;
    unsigned buf_bytes = 0;
    for (int l = 0; tma && l < NL; ++l) {
        const int sz = dt(t.leaves[l].dtype).size;
        const int64_t rb = row_len * sz;
        if (kinds[l] != 0 || rb % 16 || !aligned(t.leaves[l].data, 16)) tma = false;
        for (int d = 0; tma && d < D.R; ++d)
            if ((D.st[1 + l][d] * sz) % 16) tma = false;
        if (tma) {
            p.loff[l] = buf_bytes;
            p.lbytes[l] = (unsigned)rb;
            buf_bytes += (unsigned)rb;
        }
    }
    const int tma_block = 128;
    // One buffer per warp by default (refilled once the row is in registers),
    // and a register cap that leaves room for 5 blocks per SM when a lane's
    // share of the row takes at most 64 registers (float64 rows of 1024: 376
    // us per 2^27 elements with 96 registers; 388 at 4 blocks, 422 at 3,
    // 519 uncapped with two buffers — the compiler then spends ~210
    // registers; 6 blocks spill).
    const int nbuf = opt("row.tma_buffers", 1) == 2 ? 2 : 1;
    int64_t row_regs = 0;
    for (int l = 0; l < NL; ++l) row_regs += (int64_t)nv * vec * dt(t.leaves[l].dtype).size / 4;
    const int64_t minb_auto = row_regs <= 64 ? 5 : (row_regs <= 96 ? 3 : 2);
    const int minb = (int)std::max<int64_t>(1, std::min<int64_t>(opt("row.tma_min_blocks", minb_auto), 16));
    const size_t dyn = (size_t)buf_bytes * nbuf * (tma_block / 32);
    if (tma && dyn > 200 * 1024) tma = false;
    if (tma) {
        p.buf_bytes = buf_bytes;
        XTG_TRY(device_error_word(&p.err));
        std::string name = "xtg::k_rowfused_tma<" + tree + ", " + sl + ", " + leafset(t, order, kinds) + ", " +
                           dt(out.dtype).cname + ", " + std::to_string(vec) + ", " + std::to_string(nv) + ", " +
                           std::to_string(D.R) + ", " + std::to_string(nstat) + ", " + std::to_string(full) + ", " +
                           std::to_string(nbuf) + ", " + std::to_string(minb) + ">";
        Kernel* kr;
        XTG_TRY(get_kernel(name, tma_block, &kr, dyn));
        int64_t need = (n_rows + 3) / 4;
        return launch(kr, grid_for(kr, need), tma_block, &p, stream, dyn);
    }
    std::string name = "xtg::k_rowfused<" + tree + ", " + sl + ", " + leafset(t, order, kinds) + ", " +
                       dt(out.dtype).cname + ", " + std::to_string(vec) + ", " + std::to_string(nv) + ", " +
                       std::to_string(group) + ", " + std::to_string(D.R) + ", " + std::to_string(nstat) + ", " +
                       std::to_string(full) + ">";
    const int block = 256;
    Kernel* kr;
    XTG_TRY(get_kernel(name, block, &kr));
    const int gpb = block / group;
    int64_t need = (n_rows + gpb - 1) / gpb;
    return launch(kr, grid_for(kr, need), block, &p, stream);
}

// Memory hazards: a leaf sharing memory with the destination but read at
// other positions than the ones being written (a transposed, shifted or
// reinterpreted view of the destination).  Such assignments evaluate into a
// temporary first — what the reference's `a = e` does for every call
// (include/xtensor/core/xsemantic.hpp:620-690).
static void byte_range(const xtg_array& a, int64_t& lo, int64_t& hi) {
    lo = hi = 0;
    for (int d = 0; d < a.rank; ++d) {
        if (a.shape[d] == 0) {
            lo = 1;
            hi = 0;  // empty
            return;
        }
        const int64_t ext = (a.shape[d] - 1) * a.strides[d];
        if (ext < 0) lo += ext;
        else hi += ext;
    }
    const int64_t sz = dt(a.dtype).size;
    lo = (int64_t)(uintptr_t)a.data + lo * sz;
    hi = (int64_t)(uintptr_t)a.data + hi * sz + sz;
}

bool shares_memory(const Tree& t, const xtg_array& out) {
    int64_t olo, ohi;
    byte_range(out, olo, ohi);
    if (olo >= ohi) return false;
    for (const xtg_array& l : t.leaves) {
        int64_t llo, lhi;
        byte_range(l, llo, lhi);
        if (llo < lhi && lhi > olo && llo < ohi) return true;
    }
    return false;
}

bool assign_hazard(const Tree& t, const xtg_array& out) {
    int64_t olo, ohi;
    byte_range(out, olo, ohi);
    if (olo >= ohi) return false;
    for (const xtg_array& l : t.leaves) {
        int64_t llo, lhi;
        byte_range(l, llo, lhi);
        if (llo >= lhi || lhi <= olo || llo >= ohi) continue;
        if (l.data != out.data || l.dtype != out.dtype || l.rank > out.rank) return true;
        int64_t st[XTG_MAX_RANK];
        bstrides_to(l, out.rank, out.shape, st);
        for (int d = 0; d < out.rank; ++d)
            if (out.shape[d] > 1 && st[d] != out.strides[d]) return true;
    }
    return false;
}

xtg_status assign_guarded(const Tree& t, const xtg_array* out, cudaStream_t stream) {
    if (!assign_hazard(t, *out)) return assign_tree(t, out, stream);
    if (recorder()) recorder()->nocache = true;  // the temporary's address is baked into the launches
    int64_t n = 1;
    for (int d = 0; d < out->rank; ++d) n *= out->shape[d];
    void* tmp = nullptr;
    XTG_TRY(scratch_alloc(&tmp, (size_t)std::max<int64_t>(n, 1) * dt(out->dtype).size + 16, stream));
    xtg_array ta = *out;
    ta.data = tmp;
    int64_t m = 1;
    for (int d = out->rank - 1; d >= 0; --d) {
        ta.strides[d] = m;
        m *= out->shape[d];
    }
    xtg_status st = assign_tree(t, &ta, stream);
    if (st == XTG_OK) {
        xtg_expr le;
        memset(&le, 0, sizeof le);
        le.n_nodes = 1;
        le.nodes[0].op = XTG_OP_LEAF;
        le.nodes[0].dtype = out->dtype;
        le.n_leaves = 1;
        le.leaves[0] = ta;
        Tree t2;
        st = build_tree(&le, false, t2);
        if (st == XTG_OK) st = assign_tree(t2, out, stream);
    }
    xtg_status fs = scratch_free(tmp, stream);
    return st != XTG_OK ? st : fs;
}

}  // namespace xtgh

using namespace xtgh;

extern "C" xtg_status xtg_assign(const xtg_expr* e, const xtg_array* out, xtg_stream stream) {
    if (!out) return fail(XTG_ERR_INVALID, "null destination");
    if (!valid_dtype(out->dtype) || out->rank < 0 || out->rank > XTG_MAX_RANK)
        return fail(XTG_ERR_INVALID, "bad destination descriptor");
    begin_call();
    return with_plan_cache(0, e, nullptr, out, 0, 0, 0, (cudaStream_t)stream, [&]() -> xtg_status {
        Tree t;
        const bool demote = opt("fp32_compute", 1) != 0 && out->dtype != XTG_FLOAT64;
        XTG_TRY(build_tree(e, demote, t));
        return assign_guarded(t, out, (cudaStream_t)stream);
    });
}
