// Host encoders of the laml_gb300 C ABI: newick -> node table in the
// reference's numbering, character matrix -> device site layout, and the
// level schedule of a batch of trees.  Pure C++ (no CUDA), thread-safe.
#include "laml_gb300.h"

#include <algorithm>
#include <charconv>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <atomic>
#include <climits>
#include <cstdint>
#include <thread>
#include <unordered_map>
#include <vector>

namespace laml {
thread_local std::string g_last_error;
void set_error(const std::string& s) { g_last_error = s; }
}  // namespace laml

extern "C" const char* laml_last_error(void) { return laml::g_last_error.c_str(); }

namespace {

using laml::set_error;

// f(begin, end) over [0, n) split into one contiguous range per host thread
template <class F>
void parallel_for(int64_t n, F f, int64_t min_parallel = 4096) {
    int nt = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 16u);
    if (n < min_parallel || nt <= 1) {
        f((int64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    const int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        const int64_t a = t * chunk, e = std::min(n, a + chunk);
        if (a >= e) break;
        th.emplace_back([&f, a, e]() { f(a, e); });
    }
    for (auto& x : th) x.join();
}


// ---------------------------------------------------------------------------
// newick
// ---------------------------------------------------------------------------
struct PNode {
    std::string label;
    bool has_label = false;
    double length = 0.0;
    bool has_length = false;
    int parent = -1;
    std::vector<int> children;  // newick order
};

bool parse_newick(const char* s, std::vector<PNode>& nodes) {
    nodes.clear();
    nodes.emplace_back();
    int cur = 0;
    std::vector<int> stack;
    const size_t n = std::strlen(s);
    size_t i = 0;
    auto token_end = [&](size_t j) {
        while (j < n && !std::strchr(",():;[", s[j])) ++j;
        return j;
    };
    auto trim = [](const char* b, const char* e) {
        while (b < e && std::isspace((unsigned char)*b)) ++b;
        while (e > b && std::isspace((unsigned char)e[-1])) --e;
        return std::string(b, e);
    };
    while (i < n) {
        char ch = s[i];
        if (ch == '(') {
            int c = (int)nodes.size();
            nodes.emplace_back();
            nodes[c].parent = cur;
            nodes[cur].children.push_back(c);
            stack.push_back(cur);
            cur = c;
            ++i;
        } else if (ch == ',') {
            if (stack.empty()) { set_error("newick: ',' outside parentheses"); return false; }
            int p = stack.back();
            int c = (int)nodes.size();
            nodes.emplace_back();
            nodes[c].parent = p;
            nodes[p].children.push_back(c);
            cur = c;
            ++i;
        } else if (ch == ')') {
            if (stack.empty()) { set_error("newick: unbalanced ')'"); return false; }
            cur = stack.back();
            stack.pop_back();
            ++i;
        } else if (ch == ':') {
            size_t e = token_end(i + 1);
            std::string tok = trim(s + i + 1, s + e);
            char* endp = nullptr;
            double v = std::strtod(tok.c_str(), &endp);
            if (tok.empty() || endp == tok.c_str()) { set_error("newick: bad length '" + tok + "'"); return false; }
            nodes[cur].length = v;
            nodes[cur].has_length = true;
            i = e;
        } else if (ch == ';') {
            break;
        } else if (ch == '[') {
            const char* e = std::strchr(s + i, ']');
            if (!e) { set_error("newick: unterminated comment"); return false; }
            i = (size_t)(e - s) + 1;
        } else if (std::isspace((unsigned char)ch)) {
            ++i;
        } else {
            size_t e = token_end(i);
            std::string tok = trim(s + i, s + e);
            if (!tok.empty()) { nodes[cur].label = tok; nodes[cur].has_label = true; }
            i = e;
        }
    }
    if (!stack.empty()) { set_error("newick: unbalanced '('"); return false; }
    return true;
}

// treeswift preorder: stack, children pushed in newick order, popped last-first
std::vector<int> ts_preorder(const std::vector<PNode>& nodes, int root) {
    std::vector<int> out, st{root};
    out.reserve(nodes.size());
    while (!st.empty()) {
        int v = st.back();
        st.pop_back();
        out.push_back(v);
        for (int c : nodes[v].children) st.push_back(c);
    }
    return out;
}

struct Encoded {
    int N = 0, n = 0;
    std::vector<int> parent, c0, c1;
    std::vector<double> bl;
    std::vector<uint8_t> has;
    std::vector<std::string> labels;
};

int encode_tree(const char* newick, const char* const* leaf_order, int n_order, Encoded& E) {
    std::vector<PNode> nodes;
    if (!parse_newick(newick, nodes)) return LAML_ERR_PARSE;
    std::vector<int> pre = ts_preorder(nodes, 0);
    // unnamed nodes: "node_<preorder index>" (fastEM_solver.py:65-67)
    for (size_t k = 0; k < pre.size(); ++k) {
        PNode& v = nodes[pre[k]];
        if (!v.has_label) { v.label = "node_" + std::to_string(k); v.has_label = true; }
    }
    // graph order = preorder; a unifurcating root is removed (lines 77-80)
    std::vector<int> order = pre;
    int root = pre[0];
    if (nodes[root].children.size() == 1) {
        order.erase(order.begin());
        root = nodes[root].children[0];
    }
    std::vector<int> leaves_pre;
    for (int v : order)
        if (nodes[v].children.empty()) leaves_pre.push_back(v);
    std::vector<int> leaf_seq;
    if (leaf_order) {
        std::unordered_map<std::string, int> by_label;
        for (int v : leaves_pre) by_label.emplace(nodes[v].label, v);
        std::vector<uint8_t> used(nodes.size(), 0);
        for (int k = 0; k < n_order; ++k) {
            auto it = by_label.find(leaf_order[k]);
            if (it != by_label.end() && !used[it->second]) {
                leaf_seq.push_back(it->second);
                used[it->second] = 1;
            }
        }
        if (leaf_seq.size() != leaves_pre.size()) {
            for (int v : leaves_pre)
                if (!used[v]) { set_error("leaf '" + nodes[v].label + "' is not in the leaf order"); break; }
            return LAML_ERR_LEAF;
        }
    } else {
        leaf_seq = leaves_pre;
    }
    std::vector<int> id(nodes.size(), -1);
    int next = 0;
    for (int v : leaf_seq) id[v] = next++;
    E.n = next;
    for (int v : order)
        if (!nodes[v].children.empty()) id[v] = next++;
    E.N = next;
    E.parent.assign(E.N, -1);
    E.c0.assign(E.N, -1);
    E.c1.assign(E.N, -1);
    E.bl.assign(E.N, 0.0);
    E.has.assign(E.N, 0);
    E.labels.assign(E.N, std::string());
    for (int v : order) {
        int i = id[v];
        E.labels[i] = nodes[v].label;
        E.bl[i] = nodes[v].has_length ? nodes[v].length : 0.0;
        E.has[i] = nodes[v].has_length ? 1 : 0;
        const auto& ch = nodes[v].children;
        if (ch.size() > 2 || (ch.size() == 1)) {
            set_error("node '" + nodes[v].label + "' has " + std::to_string(ch.size()) +
                      " children; the PMM kernels need a binary tree");
            return LAML_ERR_NOT_BINARY;
        }
        if (ch.size() == 2) {
            // networkx successor order: the preorder visit order = reversed newick order
            E.c0[i] = id[ch[1]];
            E.c1[i] = id[ch[0]];
            E.parent[id[ch[0]]] = i;
            E.parent[id[ch[1]]] = i;
        }
    }
    (void)root;
    return LAML_OK;
}

}  // namespace

extern "C" int laml_newick_size(const char* newick, int32_t* num_nodes, int32_t* num_leaves,
                                int64_t* label_bytes) {
    if (!newick || !num_nodes || !num_leaves) { set_error("null argument"); return LAML_ERR_ARG; }
    Encoded E;
    int rc = encode_tree(newick, nullptr, 0, E);
    if (rc != LAML_OK) return rc;
    *num_nodes = E.N;
    *num_leaves = E.n;
    if (label_bytes) {
        int64_t b = 0;
        for (auto& s : E.labels) b += (int64_t)s.size() + 1;
        *label_bytes = b;
    }
    return LAML_OK;
}

extern "C" int laml_newick_encode(const char* newick, const char* const* leaf_order,
                                  int32_t n_leaf_order, int32_t* parent, int32_t* child0,
                                  int32_t* child1, double* branch_length, uint8_t* has_length,
                                  char* labels, int64_t* label_offsets) {
    if (!newick || !parent || !child0 || !child1 || !branch_length || !has_length) {
        set_error("null argument");
        return LAML_ERR_ARG;
    }
    Encoded E;
    int rc = encode_tree(newick, leaf_order, n_leaf_order, E);
    if (rc != LAML_OK) return rc;
    std::memcpy(parent, E.parent.data(), sizeof(int32_t) * E.N);
    std::memcpy(child0, E.c0.data(), sizeof(int32_t) * E.N);
    std::memcpy(child1, E.c1.data(), sizeof(int32_t) * E.N);
    std::memcpy(branch_length, E.bl.data(), sizeof(double) * E.N);
    std::memcpy(has_length, E.has.data(), E.N);
    if (labels && label_offsets) {
        int64_t off = 0;
        for (int i = 0; i < E.N; ++i) {
            label_offsets[i] = off;
            std::memcpy(labels + off, E.labels[i].c_str(), E.labels[i].size() + 1);
            off += (int64_t)E.labels[i].size() + 1;
        }
    }
    return LAML_OK;
}

// ---------------------------------------------------------------------------
// batch newick encoding: many trees over one leaf set, one parse each,
// parallel over trees.  The parser is the state machine of parse_newick over
// flat arrays (labels are views into the newick string), so a tree costs no
// per-node allocation.
// ---------------------------------------------------------------------------
namespace {

int64_t raw_node_count(const char* s) {
    int64_t n = 1;
    for (const char* p = s; *p && *p != ';'; ++p) {
        if (*p == '(' || *p == ',') ++n;
        else if (*p == '[') {
            while (*p && *p != ']') ++p;
            if (!*p) break;
        }
    }
    return n;
}

void raw_counts(int32_t n_trees, const char* const* newicks, std::vector<int64_t>& raw) {
    raw.assign((size_t)n_trees + 1, 0);
    parallel_for(n_trees, [&](int64_t a, int64_t e) {
        for (int64_t i = a; i < e; ++i) raw[i + 1] = raw_node_count(newicks[i]);
    }, 8);
    for (int i = 0; i < n_trees; ++i) raw[i + 1] += raw[i];
}

struct FNode {
    int32_t nch, ch0, ch1;
    uint32_t lab_off, lab_len;
    double len;
    uint8_t has_len;
};

struct SV {
    const char* p;
    size_t n;
    bool operator==(const SV& o) const { return n == o.n && std::memcmp(p, o.p, n) == 0; }
};
struct SVHash {
    size_t operator()(const SV& v) const {
        uint64_t h = 1469598103934665603ull;   // FNV-1a
        for (size_t i = 0; i < v.n; ++i) h = (h ^ (unsigned char)v.p[i]) * 1099511628211ull;
        return (size_t)h;
    }
};

// a branch length token: the decimal forms through from_chars, anything else
// (a sign, hex, inf/nan) through strtod, as parse_newick does
bool parse_length(const char* b, const char* e, double* out) {
    bool plain = b < e;
    for (const char* q = b; q < e && plain; ++q)
        plain = (*q >= '0' && *q <= '9') || *q == '.' || *q == 'e' || *q == 'E' || *q == '-';
    if (plain) {
        auto r = std::from_chars(b, e, *out);
        if (r.ec == std::errc() && r.ptr != b) return true;
    }
    std::string tok(b, e);
    char* endp = nullptr;
    *out = std::strtod(tok.c_str(), &endp);
    return !tok.empty() && endp != tok.c_str();
}

bool parse_flat(const char* s, std::vector<FNode>& nodes, std::vector<int>& stack) {
    nodes.clear();
    stack.clear();
    nodes.push_back(FNode{0, -1, -1, 0, 0, 0.0, 0});
    int cur = 0;
    const char* base = s;
    const char* p = s;
    auto is_delim = [](char c) {
        return c == ',' || c == '(' || c == ')' || c == ':' || c == ';' || c == '[' || c == 0;
    };
    auto add_child = [&](int par) {
        const int c = (int)nodes.size();
        nodes.push_back(FNode{0, -1, -1, 0, 0, 0.0, 0});
        FNode& P = nodes[par];
        if (P.nch == 0) P.ch0 = c; else if (P.nch == 1) P.ch1 = c;
        ++P.nch;
        return c;
    };
    for (;;) {
        const char ch = *p;
        if (ch == 0 || ch == ';') break;
        if (ch == '(') {
            const int c = add_child(cur);
            stack.push_back(cur);
            cur = c;
            ++p;
        } else if (ch == ',') {
            if (stack.empty()) { set_error("newick: ',' outside parentheses"); return false; }
            cur = add_child(stack.back());
            ++p;
        } else if (ch == ')') {
            if (stack.empty()) { set_error("newick: unbalanced ')'"); return false; }
            cur = stack.back();
            stack.pop_back();
            ++p;
        } else if (ch == ':') {
            const char* b = p + 1;
            const char* e = b;
            while (!is_delim(*e)) ++e;
            const char* tb = b;
            const char* te = e;
            while (tb < te && std::isspace((unsigned char)*tb)) ++tb;
            while (te > tb && std::isspace((unsigned char)te[-1])) --te;
            double v;
            if (!parse_length(tb, te, &v)) {
                set_error("newick: bad length '" + std::string(tb, te) + "'");
                return false;
            }
            nodes[cur].len = v;
            nodes[cur].has_len = 1;
            p = e;
        } else if (ch == '[') {
            const char* e = std::strchr(p, ']');
            if (!e) { set_error("newick: unterminated comment"); return false; }
            p = e + 1;
        } else if (std::isspace((unsigned char)ch)) {
            ++p;
        } else {
            const char* e = p;
            while (!is_delim(*e)) ++e;
            const char* tb = p;
            const char* te = e;
            while (tb < te && std::isspace((unsigned char)*tb)) ++tb;
            while (te > tb && std::isspace((unsigned char)te[-1])) --te;
            if (te > tb) {
                nodes[cur].lab_off = (uint32_t)(tb - base);
                nodes[cur].lab_len = (uint32_t)(te - tb);
            }
            p = e;
        }
    }
    if (!stack.empty()) { set_error("newick: unbalanced '('"); return false; }
    return true;
}

}  // namespace

extern "C" int laml_newick_batch_measure(int32_t n_trees, const char* const* newicks,
                                         int64_t* raw_nodes_total) {
    if (n_trees < 0 || (n_trees > 0 && !newicks) || !raw_nodes_total) {
        set_error("laml_newick_batch_measure: bad argument");
        return LAML_ERR_ARG;
    }
    std::vector<int64_t> raw;
    raw_counts(n_trees, newicks, raw);
    *raw_nodes_total = raw[n_trees];
    return LAML_OK;
}

extern "C" int laml_newick_encode_batch(int32_t n_trees, const char* const* newicks,
                                        const char* const* leaf_order, int32_t n_leaf_order,
                                        int32_t n_threads, int64_t* node_offsets,
                                        int32_t* num_leaves, int32_t* parent, int32_t* child0,
                                        int32_t* child1, double* branch_length,
                                        uint8_t* has_length) {
    if (n_trees <= 0 || !newicks || !leaf_order || !node_offsets || !num_leaves) {
        set_error("laml_newick_encode_batch: bad argument");
        return LAML_ERR_ARG;
    }
    // raw offsets (upper bounds); compacted offsets are written afterwards
    std::vector<int64_t> raw;
    raw_counts(n_trees, newicks, raw);
    std::unordered_map<SV, int, SVHash> order;
    order.reserve((size_t)n_leaf_order * 2);
    for (int k = 0; k < n_leaf_order; ++k)
        order.emplace(SV{leaf_order[k], std::strlen(leaf_order[k])}, k);
    std::vector<int64_t> used(n_trees, 0);
    std::vector<int> rc(n_trees, LAML_OK);
    std::vector<std::string> msg(n_trees);
    std::atomic<int> next{0};
    auto work = [&]() {
        std::vector<FNode> nodes;
        std::vector<int> stack, pre, id;
        std::vector<uint8_t> seen((size_t)n_leaf_order, 0);
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n_trees) break;
            const char* s = newicks[i];
            if (!parse_flat(s, nodes, stack)) { rc[i] = LAML_ERR_PARSE; msg[i] = laml::g_last_error; continue; }
            const int NN = (int)nodes.size();
            // treeswift preorder: children pushed in newick order, popped last-first
            pre.clear();
            stack.clear();
            stack.push_back(0);
            bool binary = true;
            while (!stack.empty()) {
                const int v = stack.back();
                stack.pop_back();
                pre.push_back(v);
                const FNode& F = nodes[v];
                if (F.nch > 2 || (F.nch == 1 && v != 0)) binary = false;
                if (F.nch >= 1) stack.push_back(F.ch0);
                if (F.nch >= 2) stack.push_back(F.ch1);
            }
            int root = 0;
            size_t first = 0;
            if (nodes[0].nch == 1) { first = 1; root = nodes[0].ch0; }
            if (!binary || nodes[root].nch == 1) {
                rc[i] = LAML_ERR_NOT_BINARY;
                msg[i] = "tree " + std::to_string(i) + ": a node that does not have two children";
                continue;
            }
            // leaves take their leaf-order position; internal nodes follow in preorder
            id.assign(NN, -1);
            std::fill(seen.begin(), seen.end(), 0);
            int nl = 0;
            for (size_t k = first; k < pre.size(); ++k) {
                const FNode& v = nodes[pre[k]];
                if (v.nch == 0) {
                    auto it = v.lab_len ? order.find(SV{s + v.lab_off, v.lab_len}) : order.end();
                    if (it == order.end() || seen[it->second]) {
                        rc[i] = LAML_ERR_LEAF;
                        msg[i] = "leaf '" + std::string(s + v.lab_off, v.lab_len) +
                                 (it == order.end() ? "' is not in the leaf order"
                                                    : "' appears twice");
                        break;
                    }
                    seen[it->second] = 1;
                    id[pre[k]] = it->second;
                    ++nl;
                }
            }
            if (rc[i]) continue;
            if (nl != n_leaf_order) {
                rc[i] = LAML_ERR_LEAF;
                msg[i] = "tree " + std::to_string(i) + " does not have every leaf of the leaf order";
                continue;
            }
            int nxt = nl;
            for (size_t k = first; k < pre.size(); ++k)
                if (nodes[pre[k]].nch) id[pre[k]] = nxt++;
            const int64_t o = raw[i];
            int32_t* P = parent + o; int32_t* A = child0 + o; int32_t* B = child1 + o;
            double* D = branch_length + o; uint8_t* H = has_length + o;
            for (size_t k = first; k < pre.size(); ++k) {
                const FNode& v = nodes[pre[k]];
                const int u = id[pre[k]];
                D[u] = v.has_len ? v.len : 0.0;
                H[u] = v.has_len;
                if (pre[k] == root) P[u] = -1;
                if (v.nch == 2) {
                    // networkx successor order = preorder visit order = reversed newick order
                    A[u] = id[v.ch1];
                    B[u] = id[v.ch0];
                    P[id[v.ch0]] = u;
                    P[id[v.ch1]] = u;
                } else {
                    A[u] = -1;
                    B[u] = -1;
                }
            }
            used[i] = nxt;
            num_leaves[i] = nl;
        }
    };
    int nt = n_threads > 0 ? n_threads : (int)std::thread::hardware_concurrency();
    nt = std::max(1, std::min(nt, std::min(n_trees, 64)));
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
    for (int i = 0; i < n_trees; ++i)
        if (rc[i]) { set_error(msg[i]); return rc[i]; }
    // compact in place (outputs move towards lower offsets only)
    int64_t w = 0;
    for (int i = 0; i < n_trees; ++i) {
        node_offsets[i] = w;
        const int64_t o = raw[i], n = used[i];
        if (w != o) {
            std::memmove(parent + w, parent + o, sizeof(int32_t) * n);
            std::memmove(child0 + w, child0 + o, sizeof(int32_t) * n);
            std::memmove(child1 + w, child1 + o, sizeof(int32_t) * n);
            std::memmove(branch_length + w, branch_length + o, sizeof(double) * n);
            std::memmove(has_length + w, has_length + o, n);
        }
        w += n;
    }
    node_offsets[n_trees] = w;
    return LAML_OK;
}

// ---------------------------------------------------------------------------
// dataset layout
// ---------------------------------------------------------------------------
namespace {

struct SiteEnc {
    std::vector<int> states;     // sorted observed mutated states
    std::vector<double> q;       // per slot 2.. (exact: + lumped state)
    int C = 2;
};

int encode_sites(int n, int K, const int32_t* chars, const int32_t* pp, const int32_t* ps,
                 const double* pq, int compat, std::vector<SiteEnc>& S, int64_t* nmiss,
                 int64_t* nsil) {
    S.assign(K, SiteEnc());
    int64_t miss = 0, sil = 0;
    std::vector<int> col(n);
    for (int c = 0; c < K; ++c) {
        for (int i = 0; i < n; ++i) {
            int x = chars[(int64_t)i * K + c];
            col[i] = x;
            if (x < 0) {
                if (!compat && x == LAML_CHAR_SILENCED) ++sil;
                else ++miss;
            }
        }
        std::vector<int> st;
        for (int i = 0; i < n; ++i)
            if (col[i] > 0) st.push_back(col[i]);
        std::sort(st.begin(), st.end());
        st.erase(std::unique(st.begin(), st.end()), st.end());
        SiteEnc& E = S[c];
        E.states = st;
        double tot = 0.0;
        for (int k = pp[c]; k < pp[c + 1]; ++k) tot += pq[k];
        for (int o : st) {
            int hit = -1;
            for (int k = pp[c]; k < pp[c + 1]; ++k)
                if (ps[k] == o) { hit = k; break; }
            if (hit < 0) {
                set_error("missing mutation prior for character " + std::to_string(c) + ", state " +
                          std::to_string(o));
                return LAML_ERR_PRIOR;
            }
            if (compat) E.q.push_back((double)(float)pq[hit]);
            else E.q.push_back(tot > 0 ? pq[hit] / tot : 0.0);
        }
        if (!compat) {
            double s = 0.0;
            for (double v : E.q) s += v;
            double other = 1.0 - s;
            if (other > 0.0) E.q.push_back(other);   // mass of the unobserved mutated states
        }
        E.C = (int)E.q.size() + 2;
    }
    *nmiss = miss;
    *nsil = sil;
    return LAML_OK;
}

bool check_group(int G) { return G == 8 || G == 16 || G == 32; }

}  // namespace

extern "C" int laml_dataset_measure(int32_t n_leaves, int32_t n_sites, const int32_t* chars,
                                    const int32_t* prior_ptr, const int32_t* prior_state,
                                    const double* prior_prob, int32_t compat, int32_t G,
                                    laml_dataset_info* info) {
    if (!chars || !prior_ptr || !info || n_leaves <= 0 || n_sites <= 0 || !check_group(G)) {
        set_error("laml_dataset_measure: bad argument");
        return LAML_ERR_ARG;
    }
    std::vector<SiteEnc> S;
    int64_t nm, ns;
    int rc = encode_sites(n_leaves, n_sites, chars, prior_ptr, prior_state, prior_prob, compat, S, &nm, &ns);
    if (rc) return rc;
    std::vector<int> Cs;
    for (auto& e : S) Cs.push_back(e.C);
    std::sort(Cs.begin(), Cs.end(), std::greater<int>());
    int Kpad = (n_sites + G - 1) / G * G;
    Cs.resize(Kpad, 2);
    int NG = Kpad / G;
    int64_t row = 0;
    for (int g = 0; g < NG; ++g) row += (int64_t)Cs[g * G] * G;
    info->n_leaves = n_leaves;
    info->n_sites = n_sites;
    info->n_sites_pad = Kpad;
    info->n_groups = NG;
    info->group_sites = G;
    info->row_len = row;
    info->max_states = Cs[0];
    info->n_missing = nm;
    info->n_silenced = ns;
    return LAML_OK;
}

extern "C" int laml_dataset_encode(int32_t n_leaves, int32_t n_sites, const int32_t* chars,
                                   const int32_t* prior_ptr, const int32_t* prior_state,
                                   const double* prior_prob, int32_t compat, int32_t G,
                                   int16_t* codes, float* q, int32_t* site_perm, int32_t* site_C,
                                   float* site_sumq, int32_t* group_off, int32_t* group_C,
                                   int32_t* state_ptr, int32_t* state_map) {
    laml_dataset_info info;
    int rc = laml_dataset_measure(n_leaves, n_sites, chars, prior_ptr, prior_state, prior_prob,
                                  compat, G, &info);
    if (rc) return rc;
    std::vector<SiteEnc> S;
    int64_t nm, ns;
    encode_sites(n_leaves, n_sites, chars, prior_ptr, prior_state, prior_prob, compat, S, &nm, &ns);
    const int K = n_sites, Kpad = info.n_sites_pad, NG = info.n_groups;
    std::vector<int> perm(K);
    for (int c = 0; c < K; ++c) perm[c] = c;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return S[a].C > S[b].C; });
    perm.resize(Kpad, -1);
    int64_t off = 0;
    for (int g = 0; g < NG; ++g) {
        int c0 = perm[g * G];
        int Cg = c0 >= 0 ? S[c0].C : 2;
        group_off[g] = (int32_t)off;
        group_C[g] = Cg;
        off += (int64_t)Cg * G;
    }
    std::memset(q, 0, sizeof(float) * info.row_len);
    for (int c = 0; c < Kpad; ++c) {
        int o = perm[c];
        site_perm[c] = o;
        int g = c / G, lane = c % G;
        if (o < 0) {
            site_C[c] = 2;
            site_sumq[c] = 0.f;
            continue;
        }
        site_C[c] = S[o].C;
        double sq = 0.0;
        for (size_t j = 0; j < S[o].q.size(); ++j) {
            float v = (float)S[o].q[j];
            q[group_off[g] + (int64_t)(j + 2) * G + lane] = v;
            sq += (double)v;
        }
        site_sumq[c] = (float)sq;
    }
    // codes in layout site order
    std::vector<std::unordered_map<int, int>> slot(K);
    for (int c = 0; c < K; ++c)
        for (size_t j = 0; j < S[c].states.size(); ++j) slot[c][S[c].states[j]] = (int)j + 2;
    for (int i = 0; i < n_leaves; ++i) {
        for (int c = 0; c < Kpad; ++c) {
            int o = perm[c];
            int16_t v = 0;
            if (o >= 0) {
                int x = chars[(int64_t)i * K + o];
                if (x < 0) v = (!compat && x == LAML_CHAR_SILENCED) ? -2 : -1;
                else if (x == 0) v = 0;
                else v = (int16_t)slot[o][x];
            }
            codes[(int64_t)i * Kpad + c] = v;
        }
    }
    if (state_ptr && state_map) {
        int64_t p = 0;
        for (int c = 0; c < K; ++c) {
            state_ptr[c] = (int32_t)p;
            for (int s : S[c].states) state_map[p++] = s;
        }
        state_ptr[K] = (int32_t)p;
    }
    return LAML_OK;
}

// ---------------------------------------------------------------------------
// batch plan
// ---------------------------------------------------------------------------
namespace {

struct TreeLevels {
    std::vector<int> height, depth, parent;
};

int tree_levels(int N, int n, const int32_t* c0, const int32_t* c1, TreeLevels& L, int* root) {
    L.height.assign(N, 0);
    L.depth.assign(N, -1);
    L.parent.assign(N, -1);
    for (int u = 0; u < N; ++u) {
        bool leaf = c0[u] < 0;
        if (leaf != (u < n) || (c1[u] < 0) != leaf) {
            set_error("plan: leaves must be 0..n-1 and internal nodes binary");
            return LAML_ERR_ARG;
        }
        if (!leaf) {
            if (c0[u] >= N || c1[u] >= N) { set_error("plan: child id out of range"); return LAML_ERR_ARG; }
            L.parent[c0[u]] = u;
            L.parent[c1[u]] = u;
        }
    }
    int r = -1;
    for (int u = 0; u < N; ++u)
        if (L.parent[u] < 0) {
            if (r >= 0) { set_error("plan: more than one root"); return LAML_ERR_ARG; }
            r = u;
        }
    if (r < 0 || N < 3) { set_error("plan: a tree needs a root and at least two leaves"); return LAML_ERR_ARG; }
    // heights: children have larger ids than their internal parent in the
    // preorder numbering, but do not rely on it: iterate to a fixed point
    std::vector<int> order;   // preorder from the root
    order.reserve(N);
    std::vector<int> st{r};
    L.depth[r] = 0;
    while (!st.empty()) {
        int u = st.back();
        st.pop_back();
        order.push_back(u);
        if (c0[u] >= 0) {
            L.depth[c0[u]] = L.depth[u] + 1;
            L.depth[c1[u]] = L.depth[u] + 1;
            st.push_back(c1[u]);
            st.push_back(c0[u]);
        }
    }
    if ((int)order.size() != N) { set_error("plan: tree is not connected"); return LAML_ERR_ARG; }
    for (int k = N - 1; k >= 0; --k) {
        int u = order[k];
        if (c0[u] >= 0) L.height[u] = 1 + std::max(L.height[c0[u]], L.height[c1[u]]);
    }
    *root = r;
    return LAML_OK;
}

}  // namespace

namespace {

struct PlanScratch {
    std::vector<TreeLevels> lv;
    std::vector<int> root;
    std::vector<int64_t> node_base;
};

int plan_levels(const laml_plan_input* in, PlanScratch& S, laml_plan_sizes* sz) {
    if (!in || !sz || in->n_trees <= 0 || in->n_trees >= (1 << 24)) {
        set_error("plan: bad argument (1 <= n_trees < 2^24)");
        return LAML_ERR_ARG;
    }
    const int T = in->n_trees;
    std::memset(sz, 0, sizeof(*sz));
    S.lv.assign(T, TreeLevels());
    S.root.assign(T, -1);
    S.node_base.assign(T + 1, 0);
    for (int p = 0; p < T; ++p) {
        const int d = in->tree_dataset[p];
        if (d < 0 || d >= in->n_datasets) { set_error("plan: bad dataset id"); return LAML_ERR_ARG; }
        S.node_base[p + 1] = S.node_base[p] + in->tree_nodes[p];
    }
    std::vector<int> rcs(T, LAML_OK);
    std::vector<std::string> msgs(T);
    parallel_for(T, [&](int64_t a, int64_t e) {
        for (int64_t p = a; p < e; ++p) {
            const int64_t nb = S.node_base[p];
            rcs[p] = tree_levels(in->tree_nodes[p], in->tree_leaves[p], in->child0 + nb,
                                 in->child1 + nb, S.lv[p], &S.root[p]);
            if (rcs[p]) msgs[p] = laml::g_last_error;
        }
    }, 8);
    for (int p = 0; p < T; ++p)
        if (rcs[p]) { set_error(msgs[p]); return rcs[p]; }
    int hmax = 0, dmax = 0;
    for (int p = 0; p < T; ++p) {
        const int N = in->tree_nodes[p], n = in->tree_leaves[p], d = in->tree_dataset[p];
        const int32_t* c0 = in->child0 + S.node_base[p];
        const TreeLevels& L = S.lv[p];
        for (int u = 0; u < N; ++u) {
            hmax = std::max(hmax, L.height[u]);
            if (c0[u] >= 0) dmax = std::max(dmax, L.depth[u] + 1);   // levels of internal parents
        }
        const int NG = in->ds_groups[d], Kp = in->ds_sites_pad[d];
        sz->n_nodes += N;
        sz->part_floats += (int64_t)(N - n) * in->ds_row_len[d];
        sz->scalar_len += (int64_t)(N - n) * Kp;
        sz->site_len += Kp;
        sz->count_floats += (int64_t)N * NG * 8;
        sz->post_len += (int64_t)N * Kp;
        sz->n_in_items += (int64_t)(N - n) * NG;
        sz->n_out_items += (int64_t)(N - n) * NG;
        sz->n_root_items += NG;
    }
    sz->n_in_levels = hmax;
    sz->n_out_levels = dmax;
    for (int d = 0; d < in->n_datasets; ++d) sz->n_groups_total += in->ds_groups[d];
    return LAML_OK;
}

}  // namespace

extern "C" int laml_plan_measure(const laml_plan_input* in, laml_plan_sizes* sz) {
    PlanScratch S;
    return plan_levels(in, S, sz);
}

extern "C" int laml_plan_fill(const laml_plan_input* in, laml_plan_output* o) {
    laml_plan_sizes sz;
    PlanScratch S;
    int rc = plan_levels(in, S, &sz);
    if (rc) return rc;
    const int T = in->n_trees;
    const int H = sz.n_in_levels, D = sz.n_out_levels;
    int maxNG = 0;
    std::vector<int64_t> pbase(T), sbase(T), tbase(T), cbase(T), qbase(T);
    {
        int64_t pb = 0, sb = 0, tb = 0, cb = 0, qb = 0;
        for (int p = 0; p < T; ++p) {
            const int N = in->tree_nodes[p], n = in->tree_leaves[p], d = in->tree_dataset[p];
            const int NG = in->ds_groups[d], Kp = in->ds_sites_pad[d];
            maxNG = std::max(maxNG, NG);
            pbase[p] = pb; sbase[p] = sb; tbase[p] = tb; cbase[p] = cb; qbase[p] = qb;
            pb += (int64_t)(N - n) * in->ds_row_len[d];
            sb += (int64_t)(N - n) * Kp;
            tb += Kp;
            cb += (int64_t)N * NG * 8;
            qb += (int64_t)N * Kp;
        }
    }
    // node and tree arrays (parallel over trees)
    parallel_for(T, [&](int64_t a, int64_t e) {
        for (int64_t p = a; p < e; ++p) {
            const int N = in->tree_nodes[p], n = in->tree_leaves[p], d = in->tree_dataset[p];
            const int64_t nb = S.node_base[p];
            const int32_t* c0 = in->child0 + nb;
            const int32_t* c1 = in->child1 + nb;
            const TreeLevels& L = S.lv[p];
            const int Kp = in->ds_sites_pad[d];
            const int64_t R = in->ds_row_len[d];
            o->tr_node_base[p] = (int32_t)nb;
            o->tr_root[p] = (int32_t)(nb + S.root[p]);
            o->tr_quirk[p] = (int32_t)(nb + N - 1);   // parent_sibling[root] = (-1,-1) -> node N-1
            o->tr_site_base[p] = tbase[p];
            o->tr_cnt_base[p] = cbase[p];
            o->tr_post_base[p] = qbase[p];
            for (int u = 0; u < N; ++u) {
                const int64_t g = nb + u;
                o->nd_tree[g] = (int32_t)p;
                o->nd_c0[g] = c0[u] >= 0 ? (int32_t)(nb + c0[u]) : -1;
                o->nd_c1[g] = c1[u] >= 0 ? (int32_t)(nb + c1[u]) : -1;
                const int par = L.parent[u];
                o->nd_parent[g] = par >= 0 ? (int32_t)(nb + par) : -1;
                int sib = -1;
                if (par >= 0) sib = (c0[par] == u) ? c1[par] : c0[par];
                o->nd_sib[g] = sib >= 0 ? (int32_t)(nb + sib) : -1;
                if (u < n) {
                    o->nd_leafrow[g] = u;
                    o->nd_prow[g] = -1;
                    o->nd_srow[g] = -1;
                } else {
                    o->nd_leafrow[g] = -1;
                    o->nd_prow[g] = pbase[p] + (int64_t)(u - n) * R;
                    o->nd_srow[g] = sbase[p] + (int64_t)(u - n) * Kp;
                }
            }
        }
    }, 8);
    // level buckets: inside by height, outside by the depth of the internal
    // parent; within a level, nodes grouped by which of their children are
    // leaves (key 0..3: consecutive items -- the items of one warp -- then
    // take the same specialised state loop), then trees in order and nodes
    // ascending.  Per-(tree, level, key) counts, a prefix over (level, key,
    // tree), then a parallel scatter: the order a stable sort by key of the
    // tree-major level lists gives, without a sort pass.
    const int NL[2] = {H, D};
    constexpr int NK = 4;
    std::vector<int64_t> lcnt[2];
    for (int s2 = 0; s2 < 2; ++s2) lcnt[s2].assign((size_t)T * (NL[s2] + 1) * NK, 0);
    auto level_of = [&](const TreeLevels& L, int u, int side) {
        return side == 0 ? L.height[u] : L.depth[u] + 1;
    };
    auto key_of = [&](const int32_t* c0, const int32_t* c1, int u) {
        return (c0[c0[u]] < 0 ? 1 : 0) | (c0[c1[u]] < 0 ? 2 : 0);
    };
    parallel_for(T, [&](int64_t a, int64_t e) {
        for (int64_t p = a; p < e; ++p) {
            const int N = in->tree_nodes[p], n = in->tree_leaves[p];
            const int64_t nb = S.node_base[p];
            const int32_t* c0 = in->child0 + nb;
            const int32_t* c1 = in->child1 + nb;
            const TreeLevels& L = S.lv[p];
            for (int side = 0; side < 2; ++side) {
                int64_t* c = lcnt[side].data() + (size_t)p * (NL[side] + 1) * NK;
                for (int u = n; u < N; ++u) ++c[level_of(L, u, side) * NK + key_of(c0, c1, u)];
            }
        }
    }, 8);
    std::vector<int64_t> lstart[2];     // [level + 1]: first slot of the level
    std::vector<int32_t> lnodes[2];
    for (int side = 0; side < 2; ++side) {
        const int nl = NL[side];
        lstart[side].assign(nl + 2, 0);
        int64_t acc = 0;
        for (int l = 0; l <= nl; ++l) {
            lstart[side][l] = acc;
            for (int k = 0; k < NK; ++k)
                for (int p = 0; p < T; ++p) {
                    int64_t& c = lcnt[side][((size_t)p * (nl + 1) + l) * NK + k];
                    const int64_t x = c;
                    c = acc;          // becomes the tree's first slot of (level, key)
                    acc += x;
                }
        }
        lstart[side][nl + 1] = acc;
        lnodes[side].assign(acc, 0);
    }
    parallel_for(T, [&](int64_t a, int64_t e) {
        for (int64_t p = a; p < e; ++p) {
            const int N = in->tree_nodes[p], n = in->tree_leaves[p];
            const int64_t nb = S.node_base[p];
            const int32_t* c0 = in->child0 + nb;
            const int32_t* c1 = in->child1 + nb;
            const TreeLevels& L = S.lv[p];
            for (int side = 0; side < 2; ++side) {
                int64_t* c = lcnt[side].data() + (size_t)p * (NL[side] + 1) * NK;
                for (int u = n; u < N; ++u)
                    lnodes[side][c[level_of(L, u, side) * NK + key_of(c0, c1, u)]++] =
                        (int32_t)(nb + u);
            }
        }
    }, 8);
    // items, group-major within a level (groups are sorted by state count)
    bool uniform = true;
    for (int p = 0; p < T; ++p) uniform = uniform && in->ds_groups[in->tree_dataset[p]] == maxNG;
    const bool want_items = o->in_items && o->out_items;
    if (!want_items && !(uniform && o->in_lnodes && o->out_lnodes)) {
        set_error("plan: in_items/out_items are required unless every dataset has the same "
                  "group count and in_lnodes/out_lnodes are given");
        return LAML_ERR_ARG;
    }
    if ((o->in_desc || o->out_desc) && !want_items) {
        set_error("plan: host descriptors need in_items/out_items");
        return LAML_ERR_ARG;
    }
    auto emit = [&](int side, int first, int last, int32_t* off, int32_t* items,
                    int32_t* lout) {
        const int32_t* nodes = lnodes[side].data();
        if (lout)   // the level node lists, first..last (level 0 is empty)
            std::memcpy(lout, nodes + lstart[side][first],
                        sizeof(int32_t) * (size_t)(lstart[side][last + 1] - lstart[side][first]));
        if (uniform) {
            // every tree has maxNG groups: item k of level l is node
            // a_l + (k - off_l) % cnt_l of group (k - off_l) / cnt_l; one
            // parallel pass over all items of all levels
            const int nl = last - first + 1;
            std::vector<int64_t> o64((size_t)nl + 1, 0);
            for (int l = first; l <= last; ++l) {
                const int64_t cnt = lstart[side][l + 1] - lstart[side][l];
                o64[l - first + 1] = o64[l - first] + cnt * maxNG;
                off[l - first] = (int32_t)o64[l - first];
            }
            off[nl] = (int32_t)o64[nl];
            if (!items) return;
            parallel_for(o64[nl], [&](int64_t k0, int64_t k1) {
                int li = (int)(std::upper_bound(o64.begin(), o64.end(), k0) - o64.begin()) - 1;
                for (int64_t k = k0; k < k1; ++k) {
                    while (k >= o64[li + 1]) ++li;
                    const int l = li + first;
                    const int64_t a = lstart[side][l], cnt = lstart[side][l + 1] - a;
                    const int64_t r = k - o64[li];
                    const int64_t g = r / cnt;
                    items[2 * k] = nodes[a + (r - g * cnt)];
                    items[2 * k + 1] = (int32_t)g;
                }
            }, 1 << 15);
            return;
        }
        int64_t k = 0;
        for (int l = first; l <= last; ++l) {
            off[l - first] = (int32_t)k;
            const int64_t a = lstart[side][l], e = lstart[side][l + 1];
            {
                for (int g = 0; g < maxNG; ++g)
                    for (int64_t x = a; x < e; ++x) {
                        const int node = nodes[x];
                        if (g < in->ds_groups[in->tree_dataset[o->nd_tree[node]]]) {
                            items[2 * k] = node;
                            items[2 * k + 1] = g;
                            ++k;
                        }
                    }
            }
        }
        off[last - first + 1] = (int32_t)k;
    };
    emit(0, 1, H, o->in_level_off, o->in_items, o->in_lnodes);
    emit(1, 1, D, o->out_level_off, o->out_items, o->out_lnodes);
    int64_t k = 0;
    for (int g = 0; g < maxNG; ++g)
        for (int p = 0; p < T; ++p) {
            if (g < in->ds_groups[in->tree_dataset[p]]) {
                o->root_items[2 * k] = o->tr_root[p];
                o->root_items[2 * k + 1] = g;
                ++k;
            }
        }
    // global group table and item descriptors (the 32-bit range check holds
    // for descriptors built later on the device as well)
    std::vector<int64_t> site_base(in->n_datasets), q_base(in->n_datasets),
        code_base(in->n_datasets);
    {
        int64_t sb = 0, qb2 = 0, cb2 = 0;
        for (int d = 0; d < in->n_datasets; ++d) {
            site_base[d] = sb;
            q_base[d] = qb2;
            code_base[d] = cb2;
            sb += in->ds_sites_pad[d];
            qb2 += in->ds_row_len[d];
            if (in->ds_leaves) cb2 += (int64_t)in->ds_leaves[d] * in->ds_sites_pad[d];
        }
        if (qb2 >= INT32_MAX || cb2 >= INT32_MAX || sz.part_floats / 8 >= INT32_MAX ||
            sz.scalar_len >= INT32_MAX || sz.n_nodes >= INT32_MAX) {
            set_error("plan: batch too large for 32-bit descriptors");
            return LAML_ERR_ARG;
        }
    }
    if (o->grp_desc || o->in_desc || o->out_desc) {
        if (!in->ds_sites || !in->ds_leaves || !in->group_off) {
            set_error("plan: descriptors need ds_sites, ds_leaves and group_off");
            return LAML_ERR_ARG;
        }
        if (o->grp_desc) {
            for (int d = 0; d < in->n_datasets; ++d)
                for (int g = 0; g < in->ds_groups[d]; ++g) {
                    const int gi = in->ds_group_base[d] + g;
                    const int G = in->ds_sites_pad[d] / in->ds_groups[d];
                    int32_t* e = o->grp_desc + 8 * (int64_t)gi;
                    e[0] = in->group_off[gi];
                    e[1] = (int32_t)(site_base[d] + (int64_t)g * G);
                    e[2] = (int32_t)(q_base[d] + in->group_off[gi]);
                    e[3] = d;
                    e[4] = (int32_t)code_base[d];
                    e[5] = in->ds_sites_pad[d];
                    e[6] = in->ds_sites[d];
                    e[7] = 0;
                }
        }
        auto ref = [&](int x) -> int32_t {
            return o->nd_c0[x] < 0 ? o->nd_leafrow[x] : (int32_t)(o->nd_prow[x] / 8);
        };
        auto fill = [&](const int32_t* items, int64_t n_items, int32_t* desc) {
          parallel_for(n_items, [&](int64_t ka, int64_t ke) {
            for (int64_t k = ka; k < ke; ++k) {
                const int u = items[2 * k], g = items[2 * k + 1];
                const int tree = o->nd_tree[u];
                const int d = in->tree_dataset[tree];
                const int v = o->nd_c0[u], w = o->nd_c1[u];
                int flags = (o->nd_c0[v] < 0 ? 1 : 0) | (o->nd_c0[w] < 0 ? 2 : 0) |
                            (o->tr_root[tree] == u ? 4 : 0);
                int32_t* e = desc + 12 * k;
                e[0] = u; e[1] = v; e[2] = w; e[3] = tree | (flags << 24);
                e[4] = g; e[5] = in->ds_group_base[d] + g;
                e[6] = (int32_t)o->nd_srow[u]; e[7] = (int32_t)(o->nd_prow[u] / 8);
                e[8] = ref(v); e[9] = ref(w);
                e[10] = (int32_t)o->nd_srow[v]; e[11] = (int32_t)o->nd_srow[w];
            }
          });
        };
        if (o->in_desc) fill(o->in_items, sz.n_in_items, o->in_desc);
        if (o->out_desc) fill(o->out_items, sz.n_out_items, o->out_desc);
    }
    return LAML_OK;
}

// Depth schedule of one binary tree for the ultrametric M-step: node ids
// grouped by depth from the root (a breadth-first walk, so each level lists
// its nodes in the order their parents were reached).
extern "C" int laml_ultra_order(const int32_t* parent, int32_t n_nodes, int32_t* out,
                                int64_t out_len, int64_t* written) {
    if (!parent || !out || n_nodes <= 0) {
        set_error("laml_ultra_order: null argument or empty tree");
        return LAML_ERR_ARG;
    }
    if (out_len < 2 * (int64_t)n_nodes + 2) {
        set_error("laml_ultra_order: out_len below 2 * n_nodes + 2");
        return LAML_ERR_ARG;
    }
    const int N = n_nodes;
    std::vector<int32_t> c0(N, -1), c1(N, -1);
    int root = -1;
    for (int v = 0; v < N; ++v) {
        const int p = parent[v];
        if (p < 0) {
            if (root >= 0) {
                set_error("laml_ultra_order: more than one root");
                return LAML_ERR_ARG;
            }
            root = v;
        } else if (p >= N) {
            set_error("laml_ultra_order: parent id out of range");
            return LAML_ERR_ARG;
        } else if (c0[p] < 0) {
            c0[p] = v;
        } else if (c1[p] < 0) {
            c1[p] = v;
        } else {
            set_error("laml_ultra_order: a node with more than two children");
            return LAML_ERR_NOT_BINARY;
        }
    }
    if (root < 0) {
        set_error("laml_ultra_order: no root");
        return LAML_ERR_ARG;
    }
    std::vector<int32_t> ids;
    std::vector<int32_t> off{0};
    ids.reserve(N);
    ids.push_back(root);
    for (size_t a = 0; a < ids.size();) {   // one level per pass
        const size_t e = ids.size();
        off.push_back((int32_t)e);
        for (size_t k = a; k < e; ++k) {
            const int u = ids[k];
            if (c0[u] >= 0) {
                if (c1[u] < 0) {
                    set_error("laml_ultra_order: a node with one child");
                    return LAML_ERR_NOT_BINARY;
                }
                ids.push_back(c0[u]);
                ids.push_back(c1[u]);
            }
        }
        a = e;
    }
    if ((int)ids.size() != N) {
        set_error("laml_ultra_order: the parent array is not one tree");
        return LAML_ERR_ARG;
    }
    const int L = (int)off.size() - 1;
    out[0] = L;
    std::copy(off.begin(), off.end(), out + 1);
    std::copy(ids.begin(), ids.end(), out + L + 2);
    if (written) *written = (int64_t)N + L + 2;
    return LAML_OK;
}

// NNI candidates of one encoded tree, renumbered as the encoder numbers the
// newick of each swapped tree.  The search lists its moves on ONE tree object,
// swapping and swapping back in turn (Topology_search_parallel.py:114-129);
// treeswift appends on add_child, so a swap and its undo leave the topology
// as it was but u's children reading (u's other child, u_child) and v's
// reading (u, w).  Every later candidate's newick -- and so its preorder
// numbering -- sees those orders: the child orders are state, replayed move
// by move (each thread replays the moves before its chunk, O(1) each).
extern "C" int laml_nni_candidates(int32_t n_nodes, int32_t n_leaves, const int32_t* parent,
                                   const int32_t* child0, const int32_t* child1,
                                   const double* branch_length, const uint8_t* has_length,
                                   int32_t n_moves, const int32_t* moves, int32_t n_threads,
                                   int32_t* out_parent, int32_t* out_child0,
                                   int32_t* out_child1, double* out_length,
                                   uint8_t* out_has_length) {
    const int N = n_nodes, n = n_leaves;
    if (N < 3 || n < 2 || n >= N || n_moves < 0 || !parent || !child0 || !child1 ||
        !branch_length || !has_length || (n_moves > 0 && (!moves || !out_parent || !out_child0 ||
                                                          !out_child1 || !out_length ||
                                                          !out_has_length))) {
        set_error("laml_nni_candidates: bad argument");
        return LAML_ERR_ARG;
    }
    int root = -1;
    for (int x = 0; x < N; ++x) {
        const bool internal = child0[x] >= 0;
        if ((x < n) == internal || (internal && (child1[x] < 0 || child0[x] >= N || child1[x] >= N))) {
            set_error("laml_nni_candidates: leaves must be 0..n-1 and internal nodes binary");
            return LAML_ERR_ARG;
        }
        if (parent[x] < 0) {
            if (root >= 0) { set_error("laml_nni_candidates: more than one root"); return LAML_ERR_ARG; }
            root = x;
        }
    }
    if (root < 0) { set_error("laml_nni_candidates: no root"); return LAML_ERR_ARG; }
    for (int m = 0; m < n_moves; ++m) {
        const int u = moves[2 * m], uc = moves[2 * m + 1];
        if (u < n || u >= N || u == root || uc < 0 || uc >= N || parent[uc] != u) {
            set_error("laml_nni_candidates: move " + std::to_string(m) +
                      " is not (internal non-root u, a child of u)");
            return LAML_ERR_ARG;
        }
    }
    auto other = [&](int x, int c) { return child0[x] == c ? child1[x] : child0[x]; };
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int nt = std::max(1, std::min(n_threads > 0 ? n_threads : hw, std::max(1, n_moves / 16)));
    const int chunk = (n_moves + nt - 1) / std::max(1, nt);
    auto work = [&](int t) {
        const int m0 = t * chunk, m1 = std::min(n_moves, m0 + chunk);
        if (m0 >= m1) return;
        // newick order (first, second) of every internal node, as the tree
        // object reads it before move m0
        std::vector<int32_t> fst(child1, child1 + N), snd(child0, child0 + N);
        auto undo_state = [&](int m) {
            const int u = moves[2 * m], uc = moves[2 * m + 1], v = parent[u];
            fst[u] = other(u, uc); snd[u] = uc;
            fst[v] = u; snd[v] = other(v, u);
        };
        for (int m = 0; m < m0; ++m) undo_state(m);
        std::vector<int32_t> id(N), st;
        st.reserve(64);
        for (int m = m0; m < m1; ++m) {
            const int u = moves[2 * m], uc = moves[2 * m + 1];
            const int v = parent[u], w = other(v, u), keep = other(u, uc);
            auto first = [&](int x) { return x == u ? keep : (x == v ? u : fst[x]); };
            auto second = [&](int x) { return x == u ? w : (x == v ? uc : snd[x]); };
            // treeswift preorder: the first newick child is pushed first, so
            // the second is visited first
            int nxt = n;
            st.clear();
            st.push_back(root);
            while (!st.empty()) {
                const int x = st.back();
                st.pop_back();
                if (x < n) { id[x] = x; continue; }
                id[x] = nxt++;
                st.push_back(first(x));
                st.push_back(second(x));
            }
            const int64_t o = (int64_t)m * N;
            int32_t* P = out_parent + o; int32_t* A = out_child0 + o; int32_t* B = out_child1 + o;
            double* D = out_length + o; uint8_t* H = out_has_length + o;
            P[id[root]] = -1;
            for (int x = 0; x < N; ++x) {
                const int i = id[x];
                D[i] = branch_length[x];
                H[i] = has_length[x];
                if (x < n) { A[i] = -1; B[i] = -1; continue; }
                const int f = id[first(x)], s2 = id[second(x)];
                A[i] = s2;   // networkx successor order = reversed newick order
                B[i] = f;
                P[f] = i;
                P[s2] = i;
            }
            undo_state(m);
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& x : th) x.join();
    return LAML_OK;
}
