// xtg_plan.cpp — parsing, C++ type inference and broadcasting of lowered
// expression trees, and the type-string code generation that turns a tree
// into a kernel template argument.
//
// Type rules follow what `decltype(functor(a, b))` yields in the reference:
// xtensor's functors apply the C++ operator / std:: math function to the
// element values (include/xtensor/core/xoperation.hpp:30-143,
// include/xtensor/core/xmath.hpp:84-99, 295-341), so a node's type is the
// C++ usual-arithmetic-conversion result.  Broadcasting follows
// xt::broadcast_shape (include/xtensor/core/xstrides.hpp:738-794).
#include <algorithm>
#include <cstring>
#include <string>

#include "xtg_plan.h"

namespace xtgh {

static bool is_unary(int op) { return op >= XTG_OP_NEG && op <= XTG_OP_CAST; }
static bool is_binary(int op) { return op >= XTG_OP_ADD && op <= XTG_OP_POW; }
bool is_rop(int op) { return op >= XTG_OP_RSUM && op <= XTG_OP_RMIN; }
static bool is_cmp(int op) { return (op >= XTG_OP_LT && op <= XTG_OP_LOGICAL_OR); }

static int iprom(int a) {  // integral promotion
    if (a == XTG_BOOL || a == XTG_INT8 || a == XTG_UINT8 || a == XTG_INT16 || a == XTG_UINT16) return XTG_INT32;
    if (a == XTG_BFLOAT16) return XTG_FLOAT32;
    return a;
}

int promote(int a, int b) {
    if (a == XTG_FLOAT64 || b == XTG_FLOAT64) return XTG_FLOAT64;
    if (a == XTG_FLOAT32 || b == XTG_FLOAT32 || a == XTG_BFLOAT16 || b == XTG_BFLOAT16) return XTG_FLOAT32;
    a = iprom(a);
    b = iprom(b);
    if (a == b) return a;
    auto rank = [](int t) { return (t == XTG_INT64 || t == XTG_UINT64) ? 2 : 1; };
    bool sa = dt(a).is_signed, sb = dt(b).is_signed;
    if (sa == sb) return rank(a) >= rank(b) ? a : b;
    int u = sa ? b : a, s = sa ? a : b;
    if (rank(u) >= rank(s)) return u;
    return s;  // int64 holds every uint32
}

static int float_fn_type(int a) {  // std::exp(float)->float, std::exp(int)->double
    if (a == XTG_FLOAT32 || a == XTG_BFLOAT16) return XTG_FLOAT32;
    return XTG_FLOAT64;
}

static const char* tname(int op) {
    switch (op) {
        case XTG_OP_NEG: return "Neg";
        case XTG_OP_POS: return "Pos";
        case XTG_OP_EXP: return "Exp";
        case XTG_OP_LOG: return "Log";
        case XTG_OP_SQRT: return "Sqrt";
        case XTG_OP_ABS: return "Abs";
        case XTG_OP_SQUARE: return "Square";
        case XTG_OP_SIN: return "Sin";
        case XTG_OP_COS: return "Cos";
        case XTG_OP_TANH: return "Tanh";
        case XTG_OP_LOGICAL_NOT: return "LogicalNot";
        case XTG_OP_BIT_NOT: return "BitNot";
        case XTG_OP_CAST: return "Cast";
        case XTG_OP_ADD: return "Add";
        case XTG_OP_SUB: return "Sub";
        case XTG_OP_MUL: return "Mul";
        case XTG_OP_DIV: return "Div";
        case XTG_OP_MOD: return "Mod";
        case XTG_OP_MAXIMUM: return "Maximum";
        case XTG_OP_MINIMUM: return "Minimum";
        case XTG_OP_LT: return "Lt";
        case XTG_OP_LE: return "Le";
        case XTG_OP_GT: return "Gt";
        case XTG_OP_GE: return "Ge";
        case XTG_OP_EQ: return "Eq";
        case XTG_OP_NE: return "Ne";
        case XTG_OP_LOGICAL_AND: return "LogicalAnd";
        case XTG_OP_LOGICAL_OR: return "LogicalOr";
        case XTG_OP_BIT_AND: return "BitAnd";
        case XTG_OP_BIT_OR: return "BitOr";
        case XTG_OP_BIT_XOR: return "BitXor";
        case XTG_OP_POW: return "Pow";
        case XTG_OP_WHERE: return "Where";
    }
    return nullptr;
}

static xtg_status infer(Tree& t, int n) {
    PNode& x = t.nodes[n];
    auto kt = [&](int i) { return t.nodes[x.kids[i]].cxx_dtype; };
    int r = -1;
    const int op = x.op;
    if (op == XTG_OP_LEAF) {
        r = t.leaves[x.leaf].dtype;
    } else if (op == XTG_OP_SCALAR) {
        if (!valid_dtype(x.dtype)) return fail(XTG_ERR_INVALID, "scalar node without a valid dtype");
        r = x.dtype;
    } else if (op == XTG_OP_CAST) {
        if (!valid_dtype(x.arg)) return fail(XTG_ERR_INVALID, "cast node without a valid target dtype");
        r = x.arg;
    } else if (op == XTG_OP_NEG || op == XTG_OP_POS || op == XTG_OP_BIT_NOT) {
        r = iprom(kt(0));
        if (op == XTG_OP_BIT_NOT && !dt(r).is_int) return fail(XTG_ERR_INVALID, "bitwise not of a floating value");
    } else if (op == XTG_OP_SQUARE) {
        r = promote(kt(0), kt(0));
    } else if (op == XTG_OP_ABS) {
        int a = kt(0);
        r = (a == XTG_UINT32 || a == XTG_UINT64) ? a : iprom(a);
    } else if (op == XTG_OP_EXP || op == XTG_OP_LOG || op == XTG_OP_SQRT || op == XTG_OP_SIN || op == XTG_OP_COS ||
               op == XTG_OP_TANH) {
        r = float_fn_type(kt(0));
    } else if (op == XTG_OP_LOGICAL_NOT) {
        r = XTG_BOOL;
    } else if (op == XTG_OP_POW) {
        r = (float_fn_type(kt(0)) == XTG_FLOAT32 && float_fn_type(kt(1)) == XTG_FLOAT32 &&
             dt(kt(0)).is_float && dt(kt(1)).is_float)
                ? XTG_FLOAT32
                : XTG_FLOAT64;
    } else if (is_cmp(op)) {
        r = XTG_BOOL;
    } else if (is_binary(op)) {
        r = promote(kt(0), kt(1));
        if ((op == XTG_OP_MOD || op == XTG_OP_BIT_AND || op == XTG_OP_BIT_OR || op == XTG_OP_BIT_XOR) && !dt(r).is_int)
            return fail(XTG_ERR_INVALID, "integer-only operator applied to floating values");
    } else if (op == XTG_OP_WHERE) {
        r = promote(kt(1), kt(2));
    } else if (op == XTG_OP_RSUM) {
        r = promote(kt(0), kt(0));
    } else if (op == XTG_OP_RMEAN || op == XTG_OP_RVAR || op == XTG_OP_RSTD) {
        r = XTG_FLOAT64;
    } else if (op == XTG_OP_RMAX || op == XTG_OP_RMIN) {
        r = kt(0) == XTG_BFLOAT16 ? XTG_FLOAT32 : kt(0);
    } else {
        return fail(XTG_ERR_INVALID, "unknown opcode " + std::to_string(op));
    }
    // A caller-provided result type must agree with the inference.
    if (op != XTG_OP_LEAF && op != XTG_OP_SCALAR && op != XTG_OP_CAST && x.dtype >= 0 && x.dtype != r)
        return fail(XTG_ERR_INVALID, "node " + std::to_string(n) + ": dtype " + std::to_string(x.dtype) +
                                         " disagrees with the C++ result type " + std::to_string(r));
    x.cxx_dtype = r;
    x.dtype = r;
    return XTG_OK;
}

static bool same_array(const xtg_array& a, const xtg_array& b) {
    if (a.data != b.data || a.dtype != b.dtype || a.rank != b.rank) return false;
    for (int d = 0; d < a.rank; ++d)
        if (a.shape[d] != b.shape[d] || a.strides[d] != b.strides[d]) return false;
    return true;
}

xtg_status build_tree(const xtg_expr* e, bool demote, Tree& t, bool dedup) {
    if (!e) return fail(XTG_ERR_INVALID, "null expression");
    if (e->n_nodes <= 0 || e->n_nodes > XTG_MAX_NODES) return fail(XTG_ERR_INVALID, "bad node count");
    if (e->n_leaves < 0 || e->n_leaves > XTG_MAX_LEAVES) return fail(XTG_ERR_INVALID, "bad leaf count");
    t = Tree();
    std::vector<int> leaf_slot(e->n_leaves, -1);
    std::vector<int> st;
    for (int i = 0; i < e->n_nodes; ++i) {
        const xtg_node& in = e->nodes[i];
        PNode x;
        x.op = in.op;
        x.dtype = in.dtype;
        x.arg = in.arg;
        x.aux = in.aux;
        x.imm = in.imm;
        int arity = 0;
        if (in.op == XTG_OP_LEAF || in.op == XTG_OP_SCALAR) arity = 0;
        else if (is_unary(in.op) || is_rop(in.op)) arity = 1;
        else if (is_binary(in.op)) arity = 2;
        else if (in.op == XTG_OP_WHERE) arity = 3;
        else return fail(XTG_ERR_INVALID, "unknown opcode " + std::to_string(in.op));
        if ((int)st.size() < arity) return fail(XTG_ERR_INVALID, "malformed postfix expression (stack underflow)");
        x.kids.assign(st.end() - arity, st.end());
        st.resize(st.size() - arity);
        if (in.op == XTG_OP_LEAF) {
            if (in.arg < 0 || in.arg >= e->n_leaves) return fail(XTG_ERR_INVALID, "leaf index out of range");
            if (leaf_slot[in.arg] < 0) {
                const xtg_array& a = e->leaves[in.arg];
                if (!valid_dtype(a.dtype)) return fail(XTG_ERR_INVALID, "leaf with invalid dtype");
                if (a.rank < 0 || a.rank > XTG_MAX_RANK) return fail(XTG_ERR_INVALID, "leaf rank out of range");
                int found = -1;
                for (size_t k = 0; dedup && k < t.leaves.size(); ++k)
                    if (same_array(t.leaves[k], a)) found = (int)k;
                if (found < 0) {
                    found = (int)t.leaves.size();
                    t.leaves.push_back(a);
                    if (a.dtype == XTG_FLOAT64) t.has_f64_leaf = true;
                }
                leaf_slot[in.arg] = found;
            }
            x.leaf = leaf_slot[in.arg];
        } else if (in.op == XTG_OP_SCALAR) {
            if (t.scalars.size() >= XTG_MAX_SCALARS) return fail(XTG_ERR_UNSUPPORTED, "too many scalars");
            x.scal = (int)t.scalars.size();
            uint64_t enc;
            if (valid_dtype(in.dtype) && dt(in.dtype).is_float) memcpy(&enc, &in.imm.f, 8);
            else enc = in.imm.u;
            t.scalars.push_back(enc);
        }
        t.nodes.push_back(x);
        int id = (int)t.nodes.size() - 1;
        XTG_TRY(infer(t, id));
        if (is_rop(in.op)) {
            // no statistic inside another statistic's operand
            std::vector<int> stack(t.nodes[id].kids);
            while (!stack.empty()) {
                int k = stack.back();
                stack.pop_back();
                if (is_rop(t.nodes[k].op)) return fail(XTG_ERR_UNSUPPORTED, "nested row reductions");
                for (int c : t.nodes[k].kids) stack.push_back(c);
            }
            if (t.rstat_axes >= 0 && t.rstat_axes != in.arg)
                return fail(XTG_ERR_UNSUPPORTED, "row reductions over different axis counts in one tree");
            if (in.arg < 1) return fail(XTG_ERR_INVALID, "row reduction over zero axes");
            t.rstat_axes = in.arg;
            t.nodes[id].stat = t.n_rstats++;
        }
        st.push_back(id);
    }
    if (st.size() != 1) return fail(XTG_ERR_INVALID, "malformed postfix expression (stack not 1 at end)");
    t.root = st[0];
    t.expr_slot = leaf_slot;
    if (t.leaves.empty() && t.nodes[t.root].op != XTG_OP_SCALAR)
        return fail(XTG_ERR_INVALID, "expression without leaves");
    if (t.n_rstats > XTG_MAX_SCALARS) return fail(XTG_ERR_UNSUPPORTED, "too many row reductions");

    // broadcast shape
    int rank = 0;
    for (auto& a : t.leaves) rank = std::max(rank, (int)a.rank);
    int64_t sh[XTG_MAX_RANK];
    for (int d = 0; d < rank; ++d) sh[d] = 1;
    for (auto& a : t.leaves) {
        for (int i = 0; i < a.rank; ++i) {
            int d = rank - a.rank + i;
            int64_t in = a.shape[i];
            if (in < 0) return fail(XTG_ERR_INVALID, "negative extent");
            if (sh[d] == 1) sh[d] = in;
            else if (in != 1 && in != sh[d])
                return fail(XTG_ERR_BROADCAST, "Incompatible dimension of arrays, compile in DEBUG for more info");
        }
    }
    t.rank = rank;
    for (int d = 0; d < rank; ++d) t.shape[d] = sh[d];
    if (t.rstat_axes > rank) return fail(XTG_ERR_AXIS, "row reduction over more axes than the expression has");

    if (demote && !t.has_f64_leaf)
        for (auto& x : t.nodes)
            if (x.dtype == XTG_FLOAT64) x.dtype = XTG_FLOAT32;
    return XTG_OK;
}

void leaf_bstrides(const Tree& t, int l, int64_t* st) {
    const xtg_array& a = t.leaves[l];
    for (int d = 0; d < t.rank; ++d) {
        int ld = d - (t.rank - a.rank);
        if (ld < 0 || (a.shape[ld] == 1 && t.shape[d] != 1)) st[d] = 0;
        else st[d] = a.strides[ld];
        if (t.shape[d] == 1) st[d] = 0;
    }
}

static bool leaf_free(const Tree& t, int n) {
    if (t.nodes[n].op == XTG_OP_LEAF) return false;
    if (is_rop(t.nodes[n].op)) return true;  // a statistic is one value per row
    for (int c : t.nodes[n].kids)
        if (!leaf_free(t, c)) return false;
    return true;
}

std::string tree_type(const Tree& t, int n, const std::vector<int>& map, int recip, int* slot) {
    const PNode& x = t.nodes[n];
    const std::string T = dt(x.dtype).cname;
    auto k = [&](int i) { return tree_type(t, x.kids[i], map, recip, slot); };
    const bool rdt = (x.dtype == XTG_FLOAT64 && (recip & 1)) || (x.dtype == XTG_FLOAT32 && (recip & 2));
    if (slot && rdt && x.op == XTG_OP_DIV && leaf_free(t, x.kids[1])) {
        const PNode& a = t.nodes[x.kids[0]];
        if (a.op == XTG_OP_SUB && a.dtype == x.dtype && leaf_free(t, a.kids[1])) {
            const std::string ta = tree_type(t, a.kids[0], map, recip, slot);
            const std::string tm = tree_type(t, a.kids[1], map, recip, slot);
            const std::string tb = k(1);
            const int kr = (*slot)++, km = (*slot)++;
            return "xtg::FmaRecipSub<" + T + ", " + ta + ", " + tm + ", " + tb + ", " + std::to_string(kr) + ", " +
                   std::to_string(km) + ">";
        }
        const std::string ta = k(0), tb = k(1);
        const int kr = (*slot)++;
        return "xtg::MulRecip<" + T + ", " + ta + ", " + tb + ", " + std::to_string(kr) + ">";
    }
    switch (x.op) {
        case XTG_OP_LEAF:
            return "xtg::L<" + std::to_string(map[x.leaf]) + ", " + dt(t.leaves[x.leaf].dtype).cname + ">";
        case XTG_OP_SCALAR:
            return "xtg::S<" + std::to_string(x.scal) + ", " + T + ">";
        default:
            break;
    }
    if (is_rop(x.op)) return "xtg::Stat<" + std::to_string(x.stat) + ", " + T + ">";
    if (is_cmp(x.op)) {
        std::string ct = (x.op == XTG_OP_LOGICAL_AND || x.op == XTG_OP_LOGICAL_OR)
                             ? std::string("bool")
                             : std::string(dt(promote(t.nodes[x.kids[0]].dtype, t.nodes[x.kids[1]].dtype)).cname);
        return std::string("xtg::") + tname(x.op) + "<" + ct + ", " + k(0) + ", " + k(1) + ">";
    }
    if (x.op == XTG_OP_WHERE) return "xtg::Where<" + T + ", " + k(0) + ", " + k(1) + ", " + k(2) + ">";
    if (is_binary(x.op)) return std::string("xtg::") + tname(x.op) + "<" + T + ", " + k(0) + ", " + k(1) + ">";
    return std::string("xtg::") + tname(x.op) + "<" + T + ", " + k(0) + ">";
}

}  // namespace xtgh

using namespace xtgh;

extern "C" {

xtg_status xtg_broadcast_shape(const xtg_expr* e, int32_t* rank, int64_t* shape) {
    if (!rank || !shape) return fail(XTG_ERR_INVALID, "null output");
    Tree t;
    XTG_TRY(build_tree(e, false, t));
    *rank = t.rank;
    for (int d = 0; d < t.rank; ++d) shape[d] = t.shape[d];
    return XTG_OK;
}

xtg_status xtg_expr_dtype(const xtg_expr* e, int32_t* dtype) {
    if (!dtype) return fail(XTG_ERR_INVALID, "null output");
    Tree t;
    XTG_TRY(build_tree(e, false, t));
    *dtype = t.nodes[t.root].cxx_dtype;
    return XTG_OK;
}

}  // extern "C"
