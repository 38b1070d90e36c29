// sm_103a kernels of the PMM inside / outside / E-step / M-step path.
//
// Layout (per dataset): sites are sorted by state count and packed in groups
// of G sites; a node row holds, per group g, group_C[g] state slots x G
// sites interleaved (slot j of the lane-th site of the group at
// group_off[g] + j*G + lane).  Slot 0 = unmutated, slot 1 = silenced,
// slots 2.. = the observed mutated states (+ one lumped state in the exact
// model).  Only internal nodes own rows; a leaf's inside vector is a function
// of its character code and phi and is never stored.
//
// Work item = (node, group); a thread owns one (node, site) and loops over
// that site's states, so every per-site reduction (the prior-weighted sum for
// the transition out of state 0, the max used for scaling) stays in
// registers.  Values are FP32 in linear space with a power-of-two scale per
// (node, site): a stored row S holds the product of normalised child
// vectors; h = exponent of max(S) is stored beside it and readers use
// S * 2^-h, with the cumulative exponent X kept as an int32.  Per-site
// log-likelihoods are formed in FP64.
//
// Math restated from fast_em/calculations.py (edge products 11-91, leaf init
// 278-334, inside 193-276, outside 135-191, responsibilities 373-454) in
// linear space:
//   E_v[0] = P00 in_v[0] + Pmut sum_a q_a in_v[a] + Psil in_v[s]
//   E_v[a] = Pstay in_v[a] + Psil in_v[s],  E_v[s] = in_v[s]
//   out_v[0] = P00 x0, out_v[a] = Pmut q_a x0 + Pstay x_a,
//   out_v[s] = Psil (x0 + sum_a x_a) + x_s,  x = out_parent * E_sibling
// with P00 = e^{-d(1+nu)}, Pmut = (1-e^{-d}) e^{-nu d}, Pstay = e^{-nu d},
// Psil = 1-e^{-nu d}.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "laml_gb300.h"

namespace laml {
void set_error(const std::string& s);
}

namespace {

constexpr float kEPS = 1e-6f;          // fast_em/calculations.py:9
constexpr double kEPSd = 1e-6;
constexpr double kCalcEps = 1e-10;     // fast_em/laml.py:47
constexpr double kDmin = 0.005, kDmax = 10.0;   // core_constants.py:7-8
constexpr double kEpsS = 1e-6, kEpsNu = 1e-5;   // EM_solver.Mstep defaults (EM_solver.py:307)
constexpr double kLn2 = 0.69314718055994530942;
constexpr int kBlock = 256;
constexpr unsigned kFull = 0xffffffffu;
#ifndef LAML_CHUNK
#define LAML_CHUNK 4
#endif
constexpr int kChunk = LAML_CHUNK;   // states loaded ahead per step of a state loop
#ifndef LAML_MINB
#define LAML_MINB 4
#endif
#ifndef LAML_MINB_OUT
#define LAML_MINB_OUT LAML_MINB   // resident blocks per SM asked of the outside kernel
#endif
constexpr int kMstepStage = 2048;    // branches of a tree staged in shared memory by the M-step

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pow2i(int e) {   // 2^e for e in [-126, 127]
    return __int_as_float((127 + e) << 23);
}

__device__ __forceinline__ int scale_exp(float m) {
    // exponent h with m * 2^-h in [0.5, 1), clamped so 2^-h stays a normal float
    if (!(m > 0.f)) return 0;
    int h;
    frexpf(m, &h);
    return max(-125, min(125, h));
}

struct Leaf {
    float e1, ephi, es;   // max(1-phi, eps), max(phi, eps), eps
};

__device__ __forceinline__ Leaf leaf_params(const laml_batch& b, int tree) {
    double phi = __ldcg(b.tr_phi + tree);
    Leaf L;
    if (b.compat) {
        L.e1 = fmaxf((float)(1.0 - phi), kEPS);
        L.ephi = fmaxf((float)phi, kEPS);
        L.es = kEPS;
    } else {
        L.e1 = (float)(1.0 - phi);
        L.ephi = (float)phi;
        L.es = 0.f;
    }
    return L;
}

// fast_em exponentiates its log-responsibilities in float32 with denormals
// flushed (calculations.py:576-577): in the compat model a per-site count
// term below the smallest normal float is zero
__device__ __forceinline__ void flush_counts(const laml_batch& b, float* c, int n) {
    if (!b.compat) return;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < n && c[k] < FLT_MIN) c[k] = 0.f;
}

// One child's inside vector at one site, normalised.
struct Child {
    const float* row;   // internal: &row[slot 0] of this site (stride G); null for a leaf
    float f;            // 2^-h
    int X;              // cumulative exponent of the normalised vector
    float s0, ss, D;    // slot 0, silenced slot, sum_a q_a * value_a
    int code;           // leaf character code
    float e1, ephi;
};

template <int G>
__device__ __forceinline__ float child_val(const Child& c, int j) {
    if (c.row) return __ldcg(c.row + j * G) * c.f;
    return c.code == j ? c.e1 : (c.code == -1 ? c.ephi : 0.f);
}

template <int G>
__device__ __forceinline__ Child load_child(const laml_batch& b, int x, int ds, int site,
                                            int goff, int lane, const float* qrow, float sumq,
                                            const Leaf& L) {
    Child c;
    c.e1 = L.e1;
    c.ephi = L.ephi;
    if (__ldg(b.nd_c0 + x) < 0) {
        int row = __ldg(b.nd_leafrow + x);
        int code = __ldg(b.codes + __ldg(b.ds_code_base + ds) +
                         (int64_t)row * __ldg(b.ds_sites_pad + ds) + site);
        c.row = nullptr;
        c.f = 1.f;
        c.X = 0;
        c.code = code;
        c.s0 = code == 0 ? L.e1 : (code == -1 ? L.ephi : 0.f);
        c.ss = code < 0 ? 1.f : L.es;
        c.D = code >= 2 ? __ldg(qrow + code * G) * L.e1 : (code == -1 ? L.ephi * sumq : 0.f);
    } else {
        int64_t s = __ldg(b.nd_srow + x) + site;
        int h = __ldcg(b.in_h + s);
        c.f = pow2i(-h);
        c.X = __ldcg(b.in_x + s);
        c.D = __ldcg(b.in_dot + s);
        c.row = b.in_part + __ldg(b.nd_prow + x) + goff + lane;
        c.code = 0;
        c.s0 = __ldcg(c.row) * c.f;
        c.ss = __ldcg(c.row + G) * c.f;
    }
    return c;
}

__device__ __forceinline__ float4 load_bt(const laml_batch& b, int x) {
    return __ldcg(reinterpret_cast<const float4*>(b.nd_bt) + x);
}

struct SiteCtx {
    int tree, ds, site, goff, C;
    const float* qrow;
    float sumq;
};

template <int G>
__device__ __forceinline__ bool site_ctx(const laml_batch& b, int node, int g, int lane,
                                         bool respect_status, SiteCtx& s) {
    s.tree = __ldg(b.nd_tree + node);
    if (respect_status && __ldcg(b.tr_status + s.tree) != LAML_TREE_ACTIVE) return false;
    s.ds = __ldg(b.tr_ds + s.tree);
    s.site = g * G + lane;
    if (s.site >= __ldg(b.ds_sites + s.ds)) return false;
    int gb = __ldg(b.ds_group_base + s.ds) + g;
    s.goff = __ldg(b.group_off + gb);
    int sb = __ldg(b.ds_site_base + s.ds) + s.site;
    s.C = __ldg(b.site_C + sb);
    s.sumq = __ldg(b.site_sumq + sb);
    s.qrow = b.q + __ldg(b.ds_q_base + s.ds) + s.goff + lane;
    return true;
}

// ---------------------------------------------------------------------------
// The root edge in log space.  fast_em's root E-step row reads node N-1
// (parent_sibling[root] = (-1, -1)), so the counts that set the root's branch
// length are not the root's own, and EM can drive that length far past where
// e^{-d(1+nu)} has an FP32 (or FP64) value while the root itself stays in
// state 0 at every site.  Everything that multiplies by a root-edge term is
// therefore formed from the terms' logarithms in FP64: the site likelihood
// (kept as an FP32 mantissa in [0.5, 1) and an int exponent), the root's
// posteriors, its E-step row and the outside inputs of its two children.
// ---------------------------------------------------------------------------
struct RootEdge {
    double l00, lm, lst, ls;   // log P00, log Pmut (without q), log Pstay, log Psil
};

__device__ __forceinline__ RootEdge root_edge_logs(const laml_batch& b, int tree) {
    const int r = __ldg(b.tr_root + tree);
    const double d = __ldcg(b.nd_d + r), nu = __ldcg(b.tr_nu + tree), nd = d * nu;
    RootEdge e;
    e.l00 = -d * (1.0 + nu);
    e.lst = -nd;
    e.lm = log((b.compat && d < kEPSd) ? kEPSd : -expm1(-d)) - nd;
    e.ls = (b.compat && nd < kEPSd) ? log(kEPSd) : log(-expm1(-nd));
    return e;
}

// log of a non-negative FP32 value (-inf at 0)
__device__ __forceinline__ double logz(float x) {
    return x > 0.f ? log((double)x) : -(double)INFINITY;
}

__device__ __forceinline__ double lse3(double a, double b, double c) {
    const double m = fmax(a, fmax(b, c));
    if (m == -(double)INFINITY) return m;
    return m + log(exp(a - m) + exp(b - m) + exp(c - m));
}

// exp(l) as an FP32 value (0 below its range)
__device__ __forceinline__ float expz(double l) { return (float)exp(l); }

// exp(l) = m * 2^e with m in [0.5, 1) (m = 0, e = 0 for l = -inf)
__device__ __forceinline__ float split_exp(double l, int& e) {
    if (!(l > -(double)INFINITY)) {
        e = 0;
        return 0.f;
    }
    e = (int)floor(l / kLn2) + 1;
    return (float)exp(l - (double)e * kLn2);
}

// Root edge from a progenitor in state 0 (calculations.py:270-276, 504): s0,
// dt (= sum_a q_a in_a) and ss are the root's inside values at scale 2^X.
__device__ __forceinline__ void root_site_llh(const laml_batch& b, int tree, int site,
                                              const RootEdge& re, float s0, float dt, float ss,
                                              int X) {
    const double l = lse3(re.l00 + logz(s0), re.lm + logz(dt), re.ls + logz(ss));
    const int64_t t = __ldg(b.tr_site_base + tree) + site;
    int e = 0;
    float m = 0.f;
    if (l > -(double)INFINITY) {
        e = (int)floor(l / kLn2) + 1;
        m = (float)exp(l - (double)e * kLn2);
    }
    __stcg(b.root_lr + t, m);
    __stcg(b.root_x + t, X + e);
    __stcg(b.llh_site + t, l + (double)X * kLn2);
}

// log of 1 / (site likelihood) at scale 2^X
__device__ __forceinline__ double root_log_scale(const laml_batch& b, int tree, int site, int X) {
    const int64_t t = __ldg(b.tr_site_base + tree) + site;
    const float m = __ldcg(b.root_lr + t);
    if (!(m > 0.f)) return -(double)INFINITY;   // a zero likelihood: no responsibilities
    return (double)(X - __ldcg(b.root_x + t)) * kLn2 - log((double)m);
}


// ---------------------------------------------------------------------------
// outside by parent: one internal node u, one site -> the outside rows and
// the expected counts of BOTH children v, w.  For child v the input is
// x^v = out[u] * E[w] (E = edge-inside), for w it is x^w = out[u] * E[v], so
// out[u] and each child's inside row are read once for the pair.
// ---------------------------------------------------------------------------
struct ChildOut {
    float x0, xs, sumx, dot, mx;
    int X;
    float* orow;
};

template <int G>
__device__ __forceinline__ void child_finish(const laml_batch& b, const SiteCtx& s, int v,
                                             const Child& cv, const float4& bv, ChildOut& o,
                                             bool want_post, float lroot, int xroot, float* cnt) {
    const float out0 = bv.x * o.x0;
    const float outs = bv.w * (o.x0 + o.sumx) + o.xs;
    if (o.orow) {
        __stcg(o.orow, out0);
        __stcg(o.orow + G, outs);
        const int h = scale_exp(fmaxf(o.mx, fmaxf(out0, outs)));
        const int64_t sv = __ldg(b.nd_srow + v) + s.site;
        __stcg(b.out_h + sv, h);
        __stcg(b.out_x + sv, o.X + h);
    }
    const int e = o.X + cv.X - xroot;
    const float sc = (lroot > 0.f) ? ldexpf(1.f / lroot, e) : 0.f;
    cnt[0] = o.x0 * cv.s0 * bv.x * sc;
    cnt[1] = o.x0 * bv.y * cv.D * sc;
    cnt[2] = o.x0 * cv.ss * bv.w * sc;
    cnt[3] = bv.z * o.dot * sc;
    cnt[4] = bv.w * cv.ss * o.sumx * sc;
    cnt[5] = o.xs * cv.ss * sc;
    cnt[6] = 0.f;
    cnt[7] = 0.f;
    if (cv.row == nullptr) {   // P(leaf silenced | D): '?' entries and observed entries apart
        const float pl = cv.ss * outs * sc;
        if (cv.code == -1) cnt[6] = pl; else cnt[7] = pl;
    }
    flush_counts(b, cnt, 8);
    if (want_post && b.post0) {
        const int64_t pb = __ldg(b.tr_post_base + s.tree) +
                           (int64_t)(v - __ldg(b.tr_node_base + s.tree)) *
                               __ldg(b.ds_sites_pad + s.ds) + s.site;
        __stcg(b.post0 + pb, cv.s0 * out0 * sc);
        __stcg(b.post1 + pb, cv.ss * outs * sc);
    }
}

template <int G>
__device__ __forceinline__ void write_counts(const laml_batch& b, int tree, int v, int g,
                                             const float* c) {
    const int ds = __ldg(b.tr_ds + tree);
    const int NG = __ldg(b.ds_groups + ds);
    float4* dst = reinterpret_cast<float4*>(
        b.cnt_part + __ldg(b.tr_cnt_base + tree) +
        ((int64_t)(v - __ldg(b.tr_node_base + tree)) * NG + g) * 8);
    __stcg(dst, make_float4(c[0], c[1], c[2], c[3]));
    __stcg(dst + 1, make_float4(c[4], c[5], c[6], c[7]));
}

// ---------------------------------------------------------------------------
// Descriptor-driven items: every address an item needs comes from its 48-byte
// descriptor and the per-group table, so the loads of an item form a chain of
// three (descriptor -> scalars/rows/codes -> state loop) instead of six.
// ---------------------------------------------------------------------------
struct ItemDesc {
    int u, v, w, tree, flags, g, gd, u_srow, u_prow8, v_ref, w_ref, v_srow, w_srow;
};

__device__ __forceinline__ ItemDesc load_desc(const int32_t* base, int64_t it) {
    const int4* p = reinterpret_cast<const int4*>(base) + 3 * it;
    const int4 A = __ldg(p), B = __ldg(p + 1), C = __ldg(p + 2);
    ItemDesc d;
    d.u = A.x; d.v = A.y; d.w = A.z;
    d.tree = A.w & 0xffffff;
    d.flags = (int)((unsigned)A.w >> 24);
    d.g = B.x; d.gd = B.y; d.u_srow = B.z; d.u_prow8 = B.w;
    d.v_ref = C.x; d.w_ref = C.y; d.v_srow = C.z; d.w_srow = C.w;
    return d;
}

struct GroupCtx {
    int code_base, kpad;
};

template <int G>
__device__ __forceinline__ bool site_ctx_d(const laml_batch& b, const ItemDesc& d, int lane,
                                           bool respect_status, SiteCtx& s, GroupCtx& gc) {
    s.tree = d.tree;
    if (respect_status && __ldcg(b.tr_status + s.tree) != LAML_TREE_ACTIVE) return false;
    const int4* gp = reinterpret_cast<const int4*>(b.grp_desc) + 2 * d.gd;
    const int4 G1 = __ldg(gp), G2 = __ldg(gp + 1);
    s.site = d.g * G + lane;
    if (s.site >= G2.z) return false;
    s.goff = G1.x;
    s.ds = G1.w;
    const int sb = G1.y + lane;
    s.C = __ldg(b.site_C + sb);
    s.sumq = __ldg(b.site_sumq + sb);
    s.qrow = b.q + G1.z + lane;
    gc.code_base = G2.x;
    gc.kpad = G2.y;
    return true;
}

template <int G>
__device__ __forceinline__ Child load_child_d(const laml_batch& b, bool leaf, int ref, int srow,
                                              const SiteCtx& s, const GroupCtx& gc, int lane,
                                              const Leaf& L) {
    Child c;
    c.e1 = L.e1;
    c.ephi = L.ephi;
    if (leaf) {
        const int code = __ldg(b.codes + gc.code_base + (int64_t)ref * gc.kpad + s.site);
        c.row = nullptr;
        c.f = 1.f;
        c.X = 0;
        c.code = code;
        c.s0 = code == 0 ? L.e1 : (code == -1 ? L.ephi : 0.f);
        c.ss = code < 0 ? 1.f : L.es;
        c.D = code >= 2 ? __ldg(s.qrow + code * G) * L.e1 : (code == -1 ? L.ephi * s.sumq : 0.f);
    } else {
        const int64_t si = (int64_t)srow + s.site;
        c.row = b.in_part + (int64_t)ref * 8 + s.goff + lane;
        const float r0 = __ldcg(c.row), r1 = __ldcg(c.row + G);   // rows before scalars: both in flight
        const int h = __ldcg(b.in_h + si);
        c.f = pow2i(-h);
        c.X = __ldcg(b.in_x + si);
        c.D = __ldcg(b.in_dot + si);
        c.code = 0;
        c.s0 = r0 * c.f;
        c.ss = r1 * c.f;
    }
    return c;
}

// ---------------------------------------------------------------------------
// Log mode: a tree with a branch whose d (1 + nu) exceeds LAML_LOG_MODE_RATE
// keeps its partials as FP32 natural logs, the reference's representation
// (fast_em/calculations.py:11-133, 373-454), because the state classes of
// such a tree (unmutated, mutated, silenced) lie further apart than one
// power-of-two exponent per (node, site) can hold.  These items are
// __noinline__ so the linear items keep their registers; they do not
// shuffle (the caller reduces the counts).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool tree_log(const laml_batch& b, int tree) {
    return __ldcg(b.tr_mode + tree) == LAML_MODE_LOG;
}

struct EdgeL {
    float l00, lm, lst, ls;   // log P00, log Pmut (without q), log Pstay, log Psil
};

__device__ __forceinline__ EdgeL edge_logs(const laml_batch& b, int x, int tree) {
    const double d = __ldcg(b.nd_d + x), nu = __ldcg(b.tr_nu + tree), nd = d * nu;
    EdgeL e;
    e.l00 = (float)(-d * (1.0 + nu));
    e.lst = (float)(-nd);
    e.lm = (float)(log((b.compat && d < kEPSd) ? kEPSd : -expm1(-d)) - nd);
    e.ls = (float)((b.compat && nd < kEPSd) ? log(kEPSd) : log(-expm1(-nd)));
    return e;
}

__device__ __forceinline__ float lgz(float x) { return x > 0.f ? logf(x) : -INFINITY; }

__device__ __forceinline__ float laddexp(float a, float c) {
    const float m = fmaxf(a, c);
    if (m == -INFINITY) return m;
    return m + log1pf(expf(-fabsf(a - c)));
}

__device__ __forceinline__ float lse3f(float a, float c, float e) {
    const float m = fmaxf(a, fmaxf(c, e));
    if (m == -INFINITY) return m;
    return m + logf(expf(a - m) + expf(c - m) + expf(e - m));
}

// running log-sum-exp
struct Lse {
    float m = -INFINITY, s = 0.f;
    __device__ __forceinline__ void add(float x) {
        if (x == -INFINITY) return;
        if (x > m) {
            s = s * expf(m - x) + 1.f;
            m = x;
        } else {
            s += expf(x - m);
        }
    }
    __device__ __forceinline__ float value() const { return m == -INFINITY ? m : m + logf(s); }
};

// exp(x - lL) for an FP32 log x and an FP64 log-likelihood
__device__ __forceinline__ float rel_exp(float x, double lL) {
    return x == -INFINITY ? 0.f : (float)exp((double)x - lL);
}

struct ChildL {
    const float* row;   // null for a leaf
    float s0, ss, ld;   // log of state 0, silenced, sum_a q_a in_a
    float le1, lephi;
    int code;
};

template <int G>
__device__ __forceinline__ float child_val_log(const ChildL& c, int j) {
    if (c.row) return __ldcg(c.row + j * G);
    return c.code == j ? c.le1 : (c.code == -1 ? c.lephi : -INFINITY);
}

template <int G>
__device__ __forceinline__ ChildL load_child_log(const laml_batch& b, bool leaf, int ref, int srow,
                                                 const SiteCtx& s, const GroupCtx& gc,
                                                 const Leaf& L) {
    ChildL c;
    c.le1 = lgz(L.e1);
    c.lephi = lgz(L.ephi);
    if (leaf) {
        const int code = __ldg(b.codes + gc.code_base + (int64_t)ref * gc.kpad + s.site);
        c.row = nullptr;
        c.code = code;
        c.s0 = code == 0 ? c.le1 : (code == -1 ? c.lephi : -INFINITY);
        c.ss = code < 0 ? 0.f : lgz(L.es);
        c.ld = code >= 2 ? lgz(__ldg(s.qrow + code * G)) + c.le1
                         : (code == -1 ? c.lephi + lgz(s.sumq) : -INFINITY);
    } else {
        c.row = b.in_part + (int64_t)ref * 8 + s.goff + (s.site % G);
        c.code = 0;
        c.s0 = __ldcg(c.row);
        c.ss = __ldcg(c.row + G);
        c.ld = __ldcg(b.in_dot + (int64_t)srow + s.site);
    }
    return c;
}

__device__ __forceinline__ void root_store_log(const laml_batch& b, int tree, int site, double l) {
    const int64_t t = __ldg(b.tr_site_base + tree) + site;
    int e = 0;
    float m = 0.f;
    if (l > -(double)INFINITY) {
        e = (int)floor(l / kLn2) + 1;
        m = (float)exp(l - (double)e * kLn2);
    }
    __stcg(b.root_lr + t, m);
    __stcg(b.root_x + t, e);
    __stcg(b.llh_site + t, l);
}

template <int G>
__device__ __noinline__ void inside_log_item(const laml_batch& b, const ItemDesc& d,
                                             const SiteCtx& s, const GroupCtx& gc) {
    const Leaf L = leaf_params(b, s.tree);
    const ChildL cv = load_child_log<G>(b, d.flags & 1, d.v_ref, d.v_srow, s, gc, L);
    const ChildL cw = load_child_log<G>(b, d.flags & 2, d.w_ref, d.w_srow, s, gc, L);
    const EdgeL ev = edge_logs(b, d.v, s.tree), ew = edge_logs(b, d.w, s.tree);
    float* row = b.in_part + (int64_t)d.u_prow8 * 8 + s.goff + (s.site % G);
    const float s0 = lse3f(ev.l00 + cv.s0, ev.lm + cv.ld, ev.ls + cv.ss) +
                     lse3f(ew.l00 + cw.s0, ew.lm + cw.ld, ew.ls + cw.ss);
    const float ss = cv.ss + cw.ss;
    __stcg(row, s0);
    __stcg(row + G, ss);
    const float kv = ev.ls + cv.ss, kw = ew.ls + cw.ss;
    Lse dot;
    for (int j = 2; j < s.C; ++j) {
        const float x = laddexp(ev.lst + child_val_log<G>(cv, j), kv) +
                        laddexp(ew.lst + child_val_log<G>(cw, j), kw);
        __stcg(row + j * G, x);
        dot.add(lgz(__ldg(s.qrow + j * G)) + x);
    }
    const int64_t sr = (int64_t)d.u_srow + s.site;
    const float ld = dot.value();
    __stcg(b.in_h + sr, 0);
    __stcg(b.in_x + sr, 0);
    __stcg(b.in_dot + sr, ld);
    if (d.flags & 4) {
        const RootEdge re = root_edge_logs(b, s.tree);
        root_store_log(b, s.tree, s.site,
                       lse3(re.l00 + (double)s0, re.lm + (double)ld, re.ls + (double)ss));
    }
}

// the six responsibilities of a child (and its leaf / posterior terms) from
// x = out[parent] + E[sibling] in logs
template <int G>
__device__ __forceinline__ void child_counts_log(const laml_batch& b, const SiteCtx& s, int v,
                                                 const ChildL& cv, const EdgeL& ev, float x0,
                                                 float xs, float lsx, float ldx, float out0,
                                                 float outs, double lL, bool want_post,
                                                 float* cnt) {
    cnt[0] = rel_exp(x0 + cv.s0 + ev.l00, lL);
    cnt[1] = rel_exp(x0 + ev.lm + cv.ld, lL);
    cnt[2] = rel_exp(x0 + cv.ss + ev.ls, lL);
    cnt[3] = rel_exp(ev.lst + ldx, lL);
    cnt[4] = rel_exp(ev.ls + cv.ss + lsx, lL);
    cnt[5] = rel_exp(xs + cv.ss, lL);
    cnt[6] = 0.f;
    cnt[7] = 0.f;
    if (cv.row == nullptr) {
        const float pl = rel_exp(cv.ss + outs, lL);
        if (cv.code == -1) cnt[6] = pl; else cnt[7] = pl;
    }
    flush_counts(b, cnt, 8);
    if (want_post && b.post0) {
        const int64_t pb = __ldg(b.tr_post_base + s.tree) +
                           (int64_t)(v - __ldg(b.tr_node_base + s.tree)) *
                               __ldg(b.ds_sites_pad + s.ds) + s.site;
        __stcg(b.post0 + pb, rel_exp(cv.s0 + out0, lL));
        __stcg(b.post1 + pb, rel_exp(cv.ss + outs, lL));
    }
}

// outside of both children of internal node u (compute_Q_v_product,
// calculations.py:11-45, with x = out[u] + edge-inside of the sibling); for a
// root, out[u] is its edge from a progenitor in state 0 (calculations.py:
// 172-175)
template <int G>
__device__ __noinline__ void outside_log_lane(const laml_batch& b, const ItemDesc& d,
                                              const SiteCtx& s, const GroupCtx& gc,
                                              bool want_post, float* cv_, float* cw_) {
    const int lane = s.site % G;
    const Leaf L = leaf_params(b, s.tree);
    const ChildL cv = load_child_log<G>(b, d.flags & 1, d.v_ref, d.v_srow, s, gc, L);
    const ChildL cw = load_child_log<G>(b, d.flags & 2, d.w_ref, d.w_srow, s, gc, L);
    const EdgeL ev = edge_logs(b, d.v, s.tree), ew = edge_logs(b, d.w, s.tree);
    const bool at_root = d.flags & 4;
    const float* urow = b.out_part + (int64_t)d.u_prow8 * 8 + s.goff + lane;
    float o0, os, olm = 0.f;
    if (at_root) {
        const RootEdge re = root_edge_logs(b, s.tree);
        o0 = (float)re.l00;
        os = (float)re.ls;
        olm = (float)re.lm;
    } else {
        o0 = __ldcg(urow);
        os = __ldcg(urow + G);
    }
    const float E0v = lse3f(ev.l00 + cv.s0, ev.lm + cv.ld, ev.ls + cv.ss);
    const float E0w = lse3f(ew.l00 + cw.s0, ew.lm + cw.ld, ew.ls + cw.ss);
    const float xa0 = o0 + E0w, xas = os + cw.ss;   // child v: x = out[u] + E[w]
    const float xb0 = o0 + E0v, xbs = os + cv.ss;   // child w: x = out[u] + E[v]
    const float kv = ev.ls + cv.ss, kw = ew.ls + cw.ss;
    float* arow = cv.row ? b.out_part + (int64_t)d.v_ref * 8 + s.goff + lane : nullptr;
    float* brow = cw.row ? b.out_part + (int64_t)d.w_ref * 8 + s.goff + lane : nullptr;
    Lse sa, sb, da, db;
    for (int j = 2; j < s.C; ++j) {
        const float lq = lgz(__ldg(s.qrow + j * G));
        const float oj = at_root ? olm + lq : __ldcg(urow + j * G);
        const float av = child_val_log<G>(cv, j), aw = child_val_log<G>(cw, j);
        const float xa = oj + laddexp(ew.lst + aw, kw);
        const float xb = oj + laddexp(ev.lst + av, kv);
        sa.add(xa);
        da.add(xa + av);
        sb.add(xb);
        db.add(xb + aw);
        if (arow) __stcg(arow + j * G, laddexp(lq + ev.lm + xa0, ev.lst + xa));
        if (brow) __stcg(brow + j * G, laddexp(lq + ew.lm + xb0, ew.lst + xb));
    }
    const float lsa = sa.value(), lsb = sb.value();
    const float outa0 = ev.l00 + xa0, outas = laddexp(ev.ls + laddexp(xa0, lsa), xas);
    const float outb0 = ew.l00 + xb0, outbs = laddexp(ew.ls + laddexp(xb0, lsb), xbs);
    if (arow) {
        __stcg(arow, outa0);
        __stcg(arow + G, outas);
        __stcg(b.out_h + (int64_t)d.v_srow + s.site, 0);
        __stcg(b.out_x + (int64_t)d.v_srow + s.site, 0);
    }
    if (brow) {
        __stcg(brow, outb0);
        __stcg(brow + G, outbs);
        __stcg(b.out_h + (int64_t)d.w_srow + s.site, 0);
        __stcg(b.out_x + (int64_t)d.w_srow + s.site, 0);
    }
    const double lL = __ldcg(b.llh_site + __ldg(b.tr_site_base + s.tree) + s.site);
    child_counts_log<G>(b, s, d.v, cv, ev, xa0, xas, lsa, da.value(), outa0, outas, lL,
                        want_post, cv_);
    child_counts_log<G>(b, s, d.w, cw, ew, xb0, xbs, lsb, db.value(), outb0, outbs, lL,
                        want_post, cw_);
}

// the root's E-step row in logs (see root_counts_item for the modes)
template <int G>
__device__ __noinline__ void root_counts_log(const laml_batch& b, int v, const SiteCtx& s,
                                             int mode, float* c) {
    const int lane = s.site % G;
    const Leaf L = leaf_params(b, s.tree);
    const GroupCtx gc{0, 0};
    const ChildL cv = load_child_log<G>(b, false, (int)(__ldg(b.nd_prow + v) / 8),
                                        (int)__ldg(b.nd_srow + v), s, gc, L);
    const RootEdge re = root_edge_logs(b, s.tree);
    float x0 = 0.f, xs = -INFINITY;
    Lse sx, dx;
    if (mode == 1) {
        const int u = __ldg(b.tr_quirk + s.tree);
        const ChildL cu = load_child_log<G>(b, false, (int)(__ldg(b.nd_prow + u) / 8),
                                            (int)__ldg(b.nd_srow + u), s, gc, L);
        const EdgeL eu = edge_logs(b, u, s.tree);
        const float* urow = b.out_part + __ldg(b.nd_prow + u) + s.goff + lane;
        x0 = __ldcg(urow) + lse3f(eu.l00 + cu.s0, eu.lm + cu.ld, eu.ls + cu.ss);
        xs = __ldcg(urow + G) + cu.ss;
        const float ku = eu.ls + cu.ss;
        for (int j = 2; j < s.C; ++j) {
            const float xj = __ldcg(urow + j * G) + laddexp(eu.lst + child_val_log<G>(cu, j), ku);
            sx.add(xj);
            dx.add(xj + child_val_log<G>(cv, j));
        }
    }
    const double lL = __ldcg(b.llh_site + __ldg(b.tr_site_base + s.tree) + s.site);
    c[0] = rel_exp(x0 + cv.s0 + (float)re.l00, lL);
    c[1] = rel_exp(x0 + (float)re.lm + cv.ld, lL);
    c[2] = rel_exp(x0 + cv.ss + (float)re.ls, lL);
    c[3] = rel_exp((float)re.lst + dx.value(), lL);
    c[4] = rel_exp((float)re.ls + cv.ss + sx.value(), lL);
    c[5] = rel_exp(xs + cv.ss, lL);
    flush_counts(b, c, 6);
}

// ---------------------------------------------------------------------------
// E-step row of a root (the root edge's expected counts), one site.
// mode 1: fast_em's row with parent = sibling = node N-1 (fast_em/laml.py:
// 244-246 + calculations.py:418); mode 2: below a progenitor in state 0
// (EM_solver.py:282-286).
// ---------------------------------------------------------------------------
template <int G>
__device__ void root_counts_item(const laml_batch& b, int v, int g, int lane, bool act,
                                 int mode) {
    float c00 = 0.f, c0a = 0.f, c0s = 0.f, caa = 0.f, cas = 0.f, css = 0.f;
    SiteCtx s;
    const bool live = act && site_ctx<G>(b, v, g, lane, true, s);
    if (live && tree_log(b, s.tree)) {
        float c[6];
        root_counts_log<G>(b, v, s, mode, c);
        c00 = c[0]; c0a = c[1]; c0s = c[2]; caa = c[3]; cas = c[4]; css = c[5];
    } else if (live) {
        const Leaf L = leaf_params(b, s.tree);
        const Child cv = load_child<G>(b, v, s.ds, s.site, s.goff, lane, s.qrow, s.sumq, L);
        const RootEdge re = root_edge_logs(b, s.tree);
        float x0 = 1.f, xs = 0.f, sumx = 0.f, dotxv = 0.f;
        int Xx = 0;
        if (mode == 1) {
            const int u = __ldg(b.tr_quirk + s.tree);
            const Child cw = load_child<G>(b, u, s.ds, s.site, s.goff, lane, s.qrow, s.sumq, L);
            const float4 bw = load_bt(b, u);
            const int64_t su = __ldg(b.nd_srow + u) + s.site;
            const float fo = pow2i(-__ldcg(b.out_h + su));
            const float* urow = b.out_part + __ldg(b.nd_prow + u) + s.goff + lane;
            x0 = __ldcg(urow) * fo * (bw.x * cw.s0 + bw.y * cw.D + bw.w * cw.ss);
            xs = __ldcg(urow + G) * fo * cw.ss;
            Xx = __ldcg(b.out_x + su) + cw.X;
            const float kw = bw.w * cw.ss;
            for (int j = 2; j < s.C; ++j) {
                const float xa = __ldcg(urow + j * G) * fo * fmaf(bw.z, child_val<G>(cw, j), kw);
                sumx += xa;
                dotxv = fmaf(xa, child_val<G>(cv, j), dotxv);
            }
        }
        // responsibilities (calculations.py:418-451) over the site likelihood
        const double lsc = root_log_scale(b, s.tree, s.site, Xx + cv.X);
        c00 = expz(logz(x0 * cv.s0) + re.l00 + lsc);
        c0a = expz(logz(x0 * cv.D) + re.lm + lsc);
        c0s = expz(logz(x0 * cv.ss) + re.ls + lsc);
        caa = expz(logz(dotxv) + re.lst + lsc);
        cas = expz(logz(cv.ss * sumx) + re.ls + lsc);
        css = expz(logz(xs * cv.ss) + lsc);
        float c[6] = {c00, c0a, c0s, caa, cas, css};
        flush_counts(b, c, 6);
        c00 = c[0]; c0a = c[1]; c0s = c[2]; caa = c[3]; cas = c[4]; css = c[5];
    }
    // sum over the G sites of the group
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
        c00 += __shfl_xor_sync(kFull, c00, off);
        c0a += __shfl_xor_sync(kFull, c0a, off);
        c0s += __shfl_xor_sync(kFull, c0s, off);
        caa += __shfl_xor_sync(kFull, caa, off);
        cas += __shfl_xor_sync(kFull, cas, off);
        css += __shfl_xor_sync(kFull, css, off);
    }
    if (act && lane == 0) {
        const int tree = __ldg(b.nd_tree + v);
        if (__ldcg(b.tr_status + tree) == LAML_TREE_ACTIVE) {
            const int ds = __ldg(b.tr_ds + tree);
            const int NG = __ldg(b.ds_groups + ds);
            float4* dst = reinterpret_cast<float4*>(
                b.cnt_part + __ldg(b.tr_cnt_base + tree) +
                ((int64_t)(v - __ldg(b.tr_node_base + tree)) * NG + g) * 8);
            __stcg(dst, make_float4(c00, c0a, c0s, caa));
            __stcg(dst + 1, make_float4(cas, css, 0.f, 0.f));
        }
    }
}

template <int G>
__device__ void inside_item_d(const laml_batch& b, const ItemDesc& d, int lane,
                              bool respect_status) {
    SiteCtx s;
    GroupCtx gc;
    if (!site_ctx_d<G>(b, d, lane, respect_status, s, gc)) return;
    if (tree_log(b, s.tree)) {
        inside_log_item<G>(b, d, s, gc);
        return;
    }
    const Leaf L = leaf_params(b, s.tree);
    const Child cv = load_child_d<G>(b, d.flags & 1, d.v_ref, d.v_srow, s, gc, lane, L);
    const Child cw = load_child_d<G>(b, d.flags & 2, d.w_ref, d.w_srow, s, gc, lane, L);
    const float4 bv = load_bt(b, d.v), bw = load_bt(b, d.w);
    const float ev0 = bv.x * cv.s0 + bv.y * cv.D + bv.w * cv.ss;
    const float ew0 = bw.x * cw.s0 + bw.y * cw.D + bw.w * cw.ss;
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    float* row = b.in_part + (int64_t)d.u_prow8 * 8 + s.goff + lane;
    const float s0 = ev0 * ew0, ss = cv.ss * cw.ss;
    __stcg(row, s0);
    __stcg(row + G, ss);
    float mx = fmaxf(s0, ss), dot = 0.f;
    int j = 2;
    for (; j + kChunk <= s.C; j += kChunk) {
        float av[kChunk], aw[kChunk], qv[kChunk];
#pragma unroll
        for (int k = 0; k < kChunk; ++k) {
            av[k] = child_val<G>(cv, j + k);
            aw[k] = child_val<G>(cw, j + k);
            qv[k] = __ldg(s.qrow + (j + k) * G);
        }
#pragma unroll
        for (int k = 0; k < kChunk; ++k) {
            const float x = fmaf(bv.z, av[k], kv) * fmaf(bw.z, aw[k], kw);
            __stcg(row + (j + k) * G, x);
            dot = fmaf(qv[k], x, dot);
            mx = fmaxf(mx, x);
        }
    }
    for (; j < s.C; ++j) {
        const float av = child_val<G>(cv, j), aw = child_val<G>(cw, j);
        const float x = fmaf(bv.z, av, kv) * fmaf(bw.z, aw, kw);
        __stcg(row + j * G, x);
        dot = fmaf(__ldg(s.qrow + j * G), x, dot);
        mx = fmaxf(mx, x);
    }
    const int h = scale_exp(mx);
    const float f = pow2i(-h);
    const int X = cv.X + cw.X + h;
    const int64_t sr = (int64_t)d.u_srow + s.site;
    __stcg(b.in_h + sr, h);
    __stcg(b.in_x + sr, X);
    __stcg(b.in_dot + sr, dot * f);
    if (d.flags & 4)
        root_site_llh(b, s.tree, s.site, root_edge_logs(b, s.tree), s0 * f, dot * f, ss * f, X);
}

template <int G>
__device__ void outside_item_d(const laml_batch& b, const ItemDesc& d, int lane, bool act,
                               bool want_post) {
    float cv_[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cw_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    SiteCtx s;
    GroupCtx gc;
    const bool live = act && site_ctx_d<G>(b, d, lane, true, s, gc);
    if (live && tree_log(b, s.tree)) {
        float tv[8], tw[8];
        outside_log_lane<G>(b, d, s, gc, want_post, tv, tw);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cv_[k] = tv[k];
            cw_[k] = tw[k];
        }
    } else if (live) {
        const Leaf L = leaf_params(b, s.tree);
        const Child cv = load_child_d<G>(b, d.flags & 1, d.v_ref, d.v_srow, s, gc, lane, L);
        const Child cw = load_child_d<G>(b, d.flags & 2, d.w_ref, d.w_srow, s, gc, lane, L);
        const float4 bv = load_bt(b, d.v), bw = load_bt(b, d.w);
        const int64_t su = (int64_t)d.u_srow + s.site;
        const float* urow = b.out_part + (int64_t)d.u_prow8 * 8 + s.goff + lane;
        const float u0 = __ldcg(urow), u1 = __ldcg(urow + G);
        const float fo = pow2i(-__ldcg(b.out_h + su));
        const int Xo = __ldcg(b.out_x + su);
        const float o0 = u0 * fo, os = u1 * fo;
        const float ev0 = bv.x * cv.s0 + bv.y * cv.D + bv.w * cv.ss;
        const float ew0 = bw.x * cw.s0 + bw.y * cw.D + bw.w * cw.ss;
        ChildOut A, B;   // A: child v (uses E[w]), B: child w (uses E[v])
        A.x0 = o0 * ew0; A.xs = os * cw.ss; A.X = Xo + cw.X;
        B.x0 = o0 * ev0; B.xs = os * cv.ss; B.X = Xo + cv.X;
        A.sumx = A.dot = A.mx = 0.f;
        B.sumx = B.dot = B.mx = 0.f;
        A.orow = cv.row ? b.out_part + (int64_t)d.v_ref * 8 + s.goff + lane : nullptr;
        B.orow = cw.row ? b.out_part + (int64_t)d.w_ref * 8 + s.goff + lane : nullptr;
        const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
        const float pxa = bv.y * A.x0, pxb = bw.y * B.x0;
        int j = 2;
        for (; j + kChunk <= s.C; j += kChunk) {
            float ou[kChunk], av[kChunk], aw[kChunk], qv[kChunk];
#pragma unroll
            for (int k = 0; k < kChunk; ++k) {
                ou[k] = __ldcg(urow + (j + k) * G);
                av[k] = child_val<G>(cv, j + k);
                aw[k] = child_val<G>(cw, j + k);
                qv[k] = __ldg(s.qrow + (j + k) * G);
            }
#pragma unroll
            for (int k = 0; k < kChunk; ++k) {
                const float o = ou[k] * fo;
                const float xa = o * fmaf(bw.z, aw[k], kw);
                const float xb = o * fmaf(bv.z, av[k], kv);
                A.sumx += xa;
                A.dot = fmaf(xa, av[k], A.dot);
                B.sumx += xb;
                B.dot = fmaf(xb, aw[k], B.dot);
                if (A.orow) {
                    const float r = fmaf(pxa, qv[k], bv.z * xa);
                    __stcg(A.orow + (j + k) * G, r);
                    A.mx = fmaxf(A.mx, r);
                }
                if (B.orow) {
                    const float r = fmaf(pxb, qv[k], bw.z * xb);
                    __stcg(B.orow + (j + k) * G, r);
                    B.mx = fmaxf(B.mx, r);
                }
            }
        }
        for (; j < s.C; ++j) {
            const float o = __ldcg(urow + j * G) * fo;
            const float av = child_val<G>(cv, j), aw = child_val<G>(cw, j);
            const float qj = __ldg(s.qrow + j * G);
            const float xa = o * fmaf(bw.z, aw, kw);
            const float xb = o * fmaf(bv.z, av, kv);
            A.sumx += xa;
            A.dot = fmaf(xa, av, A.dot);
            B.sumx += xb;
            B.dot = fmaf(xb, aw, B.dot);
            if (A.orow) {
                const float r = fmaf(pxa, qj, bv.z * xa);
                __stcg(A.orow + j * G, r);
                A.mx = fmaxf(A.mx, r);
            }
            if (B.orow) {
                const float r = fmaf(pxb, qj, bw.z * xb);
                __stcg(B.orow + j * G, r);
                B.mx = fmaxf(B.mx, r);
            }
        }
        const int64_t t = __ldg(b.tr_site_base + s.tree) + s.site;
        const float lroot = __ldcg(b.root_lr + t);
        const int xroot = __ldcg(b.root_x + t);
        child_finish<G>(b, s, d.v, cv, bv, A, want_post, lroot, xroot, cv_);
        child_finish<G>(b, s, d.w, cw, bw, B, want_post, lroot, xroot, cw_);
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cv_[k] += __shfl_xor_sync(kFull, cv_[k], off);
            cw_[k] += __shfl_xor_sync(kFull, cw_[k], off);
        }
    }
    if (act && lane == 0 && __ldcg(b.tr_status + d.tree) == LAML_TREE_ACTIVE) {
        write_counts<G>(b, d.tree, d.v, d.g, cv_);
        write_counts<G>(b, d.tree, d.w, d.g, cw_);
    }
}

// Outside of the two children of a root (out level 1).  The root's outside
// vector is the root edge itself, o = (P00, Pmut q_a, Psil), whose terms can
// lie further apart than FP32 spans; each child's inputs x = o * E[sibling]
// are formed from the terms' logs and scaled as one vector, so the class that
// dominates x keeps full precision whatever the branch length.
template <int G>
__device__ void outside_root_item_d(const laml_batch& b, const ItemDesc& d, int lane, bool act,
                                    bool want_post) {
    float cv_[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cw_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    SiteCtx s;
    GroupCtx gc;
    const bool live = act && site_ctx_d<G>(b, d, lane, true, s, gc);
    if (live && tree_log(b, s.tree)) {
        float tv[8], tw[8];
        outside_log_lane<G>(b, d, s, gc, want_post, tv, tw);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cv_[k] = tv[k];
            cw_[k] = tw[k];
        }
    } else if (live) {
        const Leaf L = leaf_params(b, s.tree);
        const Child cv = load_child_d<G>(b, d.flags & 1, d.v_ref, d.v_srow, s, gc, lane, L);
        const Child cw = load_child_d<G>(b, d.flags & 2, d.w_ref, d.w_srow, s, gc, lane, L);
        const float4 bv = load_bt(b, d.v), bw = load_bt(b, d.w);
        const RootEdge re = root_edge_logs(b, s.tree);
        const float ev0 = bv.x * cv.s0 + bv.y * cv.D + bv.w * cv.ss;
        const float ew0 = bw.x * cw.s0 + bw.y * cw.D + bw.w * cw.ss;
        const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
        // largest q_a E[.]_a of each child: the mutated class's share of x
        float ma = 0.f, mb = 0.f;
        for (int j = 2; j < s.C; ++j) {
            const float qj = __ldg(s.qrow + j * G);
            ma = fmaxf(ma, qj * fmaf(bw.z, child_val<G>(cw, j), kw));
            mb = fmaxf(mb, qj * fmaf(bv.z, child_val<G>(cv, j), kv));
        }
        auto scale_of = [](double l) { return l > -(double)INFINITY ? (int)floor(l / kLn2) + 1 : 0; };
        const int Ea = scale_of(fmax(re.l00 + logz(ew0), fmax(re.ls + logz(cw.ss), re.lm + logz(ma))));
        const int Eb = scale_of(fmax(re.l00 + logz(ev0), fmax(re.ls + logz(cv.ss), re.lm + logz(mb))));
        ChildOut A, B;   // A: child v (uses E[w]), B: child w (uses E[v])
        A.x0 = expz(re.l00 - Ea * kLn2 + logz(ew0));
        A.xs = expz(re.ls - Ea * kLn2 + logz(cw.ss));
        A.X = Ea + cw.X;
        B.x0 = expz(re.l00 - Eb * kLn2 + logz(ev0));
        B.xs = expz(re.ls - Eb * kLn2 + logz(cv.ss));
        B.X = Eb + cv.X;
        // exp(re.lm - E ln 2) as an FP32 mantissa times 2^e: the per-state
        // terms q_a E_a exp(re.lm - E ln 2) then need no FP64 (one exact
        // power-of-two scaling each)
        int ea, eb;
        const float fa = split_exp(re.lm - Ea * kLn2, ea), fb = split_exp(re.lm - Eb * kLn2, eb);
        A.sumx = A.dot = A.mx = 0.f;
        B.sumx = B.dot = B.mx = 0.f;
        A.orow = cv.row ? b.out_part + (int64_t)d.v_ref * 8 + s.goff + lane : nullptr;
        B.orow = cw.row ? b.out_part + (int64_t)d.w_ref * 8 + s.goff + lane : nullptr;
        const float pxa = bv.y * A.x0, pxb = bw.y * B.x0;
        for (int j = 2; j < s.C; ++j) {
            const float av = child_val<G>(cv, j), aw = child_val<G>(cw, j);
            const float qj = __ldg(s.qrow + j * G);
            const float xa = ldexpf(fa * (qj * fmaf(bw.z, aw, kw)), ea);
            const float xb = ldexpf(fb * (qj * fmaf(bv.z, av, kv)), eb);
            A.sumx += xa;
            A.dot = fmaf(xa, av, A.dot);
            B.sumx += xb;
            B.dot = fmaf(xb, aw, B.dot);
            if (A.orow) {
                const float r = fmaf(pxa, qj, bv.z * xa);
                __stcg(A.orow + j * G, r);
                A.mx = fmaxf(A.mx, r);
            }
            if (B.orow) {
                const float r = fmaf(pxb, qj, bw.z * xb);
                __stcg(B.orow + j * G, r);
                B.mx = fmaxf(B.mx, r);
            }
        }
        const int64_t t = __ldg(b.tr_site_base + s.tree) + s.site;
        const float lroot = __ldcg(b.root_lr + t);
        const int xroot = __ldcg(b.root_x + t);
        child_finish<G>(b, s, d.v, cv, bv, A, want_post, lroot, xroot, cv_);
        child_finish<G>(b, s, d.w, cw, bw, B, want_post, lroot, xroot, cw_);
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cv_[k] += __shfl_xor_sync(kFull, cv_[k], off);
            cw_[k] += __shfl_xor_sync(kFull, cw_[k], off);
        }
    }
    if (act && lane == 0 && __ldcg(b.tr_status + d.tree) == LAML_TREE_ACTIVE) {
        write_counts<G>(b, d.tree, d.v, d.g, cv_);
        write_counts<G>(b, d.tree, d.w, d.g, cw_);
    }
}

// the root's outside row in logs: its edge from a progenitor in state 0
template <int G>
__device__ __noinline__ void root_init_log(const laml_batch& b, int r, const SiteCtx& s,
                                           float* row, bool want_post) {
    const RootEdge re = root_edge_logs(b, s.tree);
    __stcg(row, (float)re.l00);
    __stcg(row + G, (float)re.ls);
    for (int j = 2; j < s.C; ++j)
        __stcg(row + j * G, (float)re.lm + lgz(__ldg(s.qrow + j * G)));
    const int64_t sr = __ldg(b.nd_srow + r) + s.site;
    __stcg(b.out_h + sr, 0);
    __stcg(b.out_x + sr, 0);
    if (want_post && b.post0) {
        const Leaf L = leaf_params(b, s.tree);
        const GroupCtx gc{0, 0};
        const ChildL cr = load_child_log<G>(b, false, (int)(__ldg(b.nd_prow + r) / 8),
                                            (int)__ldg(b.nd_srow + r), s, gc, L);
        const double lL = __ldcg(b.llh_site + __ldg(b.tr_site_base + s.tree) + s.site);
        const int64_t pb = __ldg(b.tr_post_base + s.tree) +
                           (int64_t)(r - __ldg(b.tr_node_base + s.tree)) *
                               __ldg(b.ds_sites_pad + s.ds) + s.site;
        __stcg(b.post0 + pb, rel_exp(cr.s0 + (float)re.l00, lL));
        __stcg(b.post1 + pb, rel_exp(cr.ss + (float)re.ls, lL));
    }
}

// outside row of a root (calculations.py:172-175) + the root's posteriors
template <int G>
__device__ void root_init_item(const laml_batch& b, int r, int g, int lane, bool want_post) {
    SiteCtx s;
    if (!site_ctx<G>(b, r, g, lane, true, s)) return;
    float* row = b.out_part + __ldg(b.nd_prow + r) + s.goff + lane;
    if (tree_log(b, s.tree)) {
        root_init_log<G>(b, r, s, row, want_post);
        return;
    }
    const float4 br = load_bt(b, r);
    float mx = fmaxf(br.x, br.w);
    __stcg(row, br.x);
    __stcg(row + G, br.w);
    for (int j = 2; j < s.C; ++j) {
        const float o = br.y * __ldg(s.qrow + j * G);
        __stcg(row + j * G, o);
        mx = fmaxf(mx, o);
    }
    const int h = scale_exp(mx);
    const int64_t sr = __ldg(b.nd_srow + r) + s.site;
    __stcg(b.out_h + sr, h);
    __stcg(b.out_x + sr, h);
    if (want_post && b.post0) {
        const Leaf L = leaf_params(b, s.tree);
        const Child cr = load_child<G>(b, r, s.ds, s.site, s.goff, lane, s.qrow, s.sumq, L);
        const RootEdge re = root_edge_logs(b, s.tree);
        const double lsc = root_log_scale(b, s.tree, s.site, cr.X);
        const int64_t pb = __ldg(b.tr_post_base + s.tree) +
                           (int64_t)(r - __ldg(b.tr_node_base + s.tree)) *
                               __ldg(b.ds_sites_pad + s.ds) + s.site;
        __stcg(b.post0 + pb, expz(logz(cr.s0) + re.l00 + lsc));
        __stcg(b.post1 + pb, expz(logz(cr.ss) + re.ls + lsc));
    }
}

// ---------------------------------------------------------------------------
// block-level helpers (FP64)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 block_sum2(double a, double c, double2* sh) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(kFull, a, off);
        c += __shfl_xor_sync(kFull, c, off);
    }
    const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
    __syncthreads();
    if (ln == 0) sh[wid] = make_double2(a, c);
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        r.x += sh[k].x;
        r.y += sh[k].y;
    }
    return r;
}

__device__ __forceinline__ float2 block_sum2f(float a, float c, double2* shd) {
    float2* sh = reinterpret_cast<float2*>(shd);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(kFull, a, off);
        c += __shfl_xor_sync(kFull, c, off);
    }
    const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
    __syncthreads();
    if (ln == 0) sh[wid] = make_float2(a, c);
    __syncthreads();
    float2 r = make_float2(0.f, 0.f);
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        r.x += sh[k].x;
        r.y += sh[k].y;
    }
    return r;
}

__device__ float4 branch_terms_of(double d, double nu, int compat) {
    // FP32 is the storage precision of the terms: compute them in FP32
    const float df = (float)d, nf = (float)nu, nd = df * nf;
    const float p00 = expf(-df * (1.f + nf));
    const float e1md = (compat && d < kEPSd) ? kEPS : -expm1f(-df);
    const float e1mnd = (compat && (double)d * nu < kEPSd) ? kEPS : -expm1f(-nd);
    const float pst = expf(-nd);
    return make_float4(p00, e1md * pst, pst, e1mnd);
}

// Stationarity in d of  -a d + b log(1-e^{-d}) + c log(1-e^{-nu d})  (a
// decreasing function of d).  With h(x) = x / (e^x - 1) and
// k(x) = x / (1 - e^{-x}) (both finite on (0, inf)):
//   F(d) = -a + (b h(d) + c h(nu d)) / d,
//   dF/dlog d = -(b h(d) k(d) + c h(nu d) k(nu d)) / d.
template <typename T>
__device__ __forceinline__ T branch_F(T a, T b, T c, T nu, T d, T* dFdu) {
    // k(x) = x e^x / (e^x - 1) = h(x) + x
    T s = T(0), ds = T(0);
    if (b > T(0)) {
        const T h = d / expm1(d);
        s += b * h;
        ds += b * h * (h + d);
    }
    if (c > T(0)) {
        const T x = nu * d;
        const T h = x / expm1(x);
        s += c * h;
        ds += c * h * (h + x);
    }
    *dFdu = -ds / d;
    return -a + s / d;
}

// One step of a safeguarded Newton iteration for the root of a decreasing
// function (value f, Newton step `step`) in the bracket [lo, hi]; true when
// converged.  A step below `tol` (relative to u) ends the iteration at
// u + step without touching the bracket: such a step can be smaller than the
// FP32 spacing of u, so u + step would round back to u, fail the bracket test
// and send the iterate to the middle of a bracket that may still span the
// whole starting interval.
__device__ __forceinline__ bool newton_step(float f, float step, float tol, float& u, float& lo,
                                            float& hi) {
    if (fabsf(step) <= tol * fmaxf(1.f, fabsf(u))) {
        u += step;
        return true;
    }
    if (f > 0.f) lo = u; else hi = u;
    float un = u + step;
    if (!(un > lo && un < hi)) un = 0.5f * (lo + hi);
    u = un;
    return hi - lo < 1e-6f;
}

// FP32 safeguarded Newton in log d on [lo, hi] from the previous value.
__device__ float solve_branch_f(float a, float bb, float c, float nu, float d0, float lo,
                                float hi) {
    float t;
    // a branch without expected counts has a flat objective: its gradient is
    // zero and fast_em's L-BFGS leaves it where it is
    if (a == 0.f && bb == 0.f && c == 0.f) return fminf(fmaxf(d0, lo), hi);
    if (branch_F<float>(a, bb, c, nu, lo, &t) <= 0.f) return lo;
    if (branch_F<float>(a, bb, c, nu, hi, &t) >= 0.f) return hi;
    float ulo = logf(lo), uhi = logf(hi);
    float u = logf(fminf(fmaxf(d0, lo), hi));
    for (int it = 0; it < 24; ++it) {
        float dF;
        const float f = branch_F<float>(a, bb, c, nu, expf(u), &dF);
        if (newton_step(f, -f / dF, 2e-6f, u, ulo, uhi)) break;
    }
    return fminf(fmaxf(expf(u), lo), hi);
}

// Safeguarded Newton in log d on [lo, hi]: FP32 iterations from the previous
// value, then (``polish``) FP64 Newton steps inside the FP32 bracket.
__device__ double solve_branch(double a, double bb, double c, double nu, double d0, double lo,
                               double hi, bool polish) {
    float t;
    if (a == 0.0 && bb == 0.0 && c == 0.0) return fmin(fmax(d0, lo), hi);   // flat objective
    const float af = (float)a, bf = (float)bb, cf = (float)c, nf = (float)nu;
    if (branch_F<float>(af, bf, cf, nf, (float)lo, &t) <= 0.f) return lo;
    if (branch_F<float>(af, bf, cf, nf, (float)hi, &t) >= 0.f) return hi;
    float ulo = logf((float)lo), uhi = logf((float)hi);
    float u = logf((float)fmin(fmax(d0, lo), hi));
    // warm-started from the previous d: a few Newton steps; the cap stops
    // oscillation at the FP32 noise floor
    for (int it = 0; it < 24; ++it) {
        float dF;
        const float f = branch_F<float>(af, bf, cf, nf, expf(u), &dF);
        if (newton_step(f, -f / dF, 2e-6f, u, ulo, uhi)) break;
    }
    if (!polish) return fmin(fmax((double)expf(u), lo), hi);
    double ud = (double)u;
    {
        const double dl = log(lo), dh = log(hi);
        for (int it = 0; it < 2; ++it) {
            double dF;
            const double f = branch_F<double>(a, bb, c, nu, exp(ud), &dF);
            const double un = ud - f / dF;
            if (!(un > dl && un < dh) || !(fabs(un - ud) < 1e-4 * fmax(1.0, fabs(ud)))) break;
            ud = un;
        }
    }
    return fmin(fmax(exp(ud), lo), hi);
}

// ---------------------------------------------------------------------------
// M-step of one tree (one thread block).  Per-branch data used by every
// round -- {C00, C00+C0a+Caa, C0a, C0s+Cas} and d -- is staged in shared
// memory (global scratch for trees above kMstepStage nodes); the final round
// polishes d and nu with FP64 Newton steps on the FP64 counts.
// ---------------------------------------------------------------------------
__device__ void mstep_tree(const laml_batch& b, int p, int rounds, double2* sh, float4* s_cnt,
                           float* s_d, bool polish) {
    if (__ldcg(b.tr_status + p) != LAML_TREE_ACTIVE) return;
    const int N = __ldg(b.tr_nodes + p), n = __ldg(b.tr_leaves + p), base = __ldg(b.tr_node_base + p);
    const int ds = __ldg(b.tr_ds + p), NG = __ldg(b.ds_groups + ds), K = __ldg(b.ds_sites + ds);
    const int64_t cb = __ldg(b.tr_cnt_base + p);
    const bool compat = b.compat != 0;
    const uint8_t fix = __ldg(b.tr_fix + p);
    double nu = __ldcg(b.tr_nu + p), phi = __ldcg(b.tr_phi + p);
    float4* C4 = s_cnt;
    float* Dd = s_d;
    if (N > kMstepStage) {
        C4 = reinterpret_cast<float4*>(b.nd_stage) + base;
        Dd = b.nd_stage + 4 * b.n_nodes + base;
    }
    // 1. counts summed over site groups (EM_solver.py:342-345 normalisation in
    //    the exact model), d saved
    // (FP32 accumulation: the FP64 pipe of this part is narrow)
    float lr = 0.f, lro = 0.f;
    for (int v = threadIdx.x; v < N; v += blockDim.x) {
        float c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const float4* src = reinterpret_cast<const float4*>(b.cnt_part + cb + (int64_t)v * NG * 8);
        for (int g = 0; g < NG; ++g) {
            const float4 x = __ldcg(src + 2 * g), z = __ldcg(src + 2 * g + 1);
            c[0] += x.x; c[1] += x.y; c[2] += x.z; c[3] += x.w;
            c[4] += z.x; c[5] += z.y; c[6] += z.z; c[7] += z.w;
        }
        double* dst = b.nd_cnt + (int64_t)(base + v) * 6;
        if (!compat) {
            double cd[5], t = 0.0;
#pragma unroll
            for (int k = 0; k < 5; ++k) { cd[k] = fmax((double)c[k], kEpsS); t += cd[k]; }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                cd[k] = cd[k] / t * K;
                __stcg(dst + k, cd[k]);
                c[k] = (float)cd[k];
            }
            __stcg(dst + 5, (double)c[5]);
        } else {
#pragma unroll
            for (int k = 0; k < 6; ++k) __stcg(dst + k, (double)c[k]);
        }
        C4[v] = make_float4(c[0], c[0] + c[1] + c[3], c[1], c[2] + c[4]);
        const double d = __ldcg(b.nd_d + base + v);
        __stcg(b.nd_d_prev + base + v, d);
        Dd[v] = (float)d;
        lr += c[6];
        lro += c[7];
    }
    const float2 LRf = block_sum2f(lr, lro, sh);   // also orders the staging writes
    const double2 LRs = make_double2((double)LRf.x, (double)LRf.y);
    const double LR = LRs.x + LRs.y;
    if (threadIdx.x == 0) {
        b.tr_prev[2 * p] = nu;
        b.tr_prev[2 * p + 1] = phi;
    }
    // 2. phi (fast_em/laml.py:77 stationary point; EM_solver.py:318-326)
    if (!(fix & 2)) {
        const double M = __ldg(b.ds_missing + ds), total = (double)n * K;
        if (compat) {
            const double Bm = M - LR, R = total - M;
            phi = (R + Bm) > 0.0 ? Bm / (R + Bm) : phi;
            phi = fmin(fmax(phi, kCalcEps), 1.0 - kCalcEps);
        } else {
            const double Rt = M - LRs.x, R = total - M;   // '?' entries only
            phi = (R + Rt) > 0.0 ? Rt / (R + Rt) : 0.0;
            if (fabs(phi) < 1.0 / total) phi = 0.0;
        }
    }
    // 3. coordinate rounds: d | nu (per branch), then nu | d
    const int R = compat ? rounds : 1;
    const double dlo = compat ? kCalcEps : kDmin, dhi = compat ? 1.0 / kCalcEps : kDmax;
    for (int r = 0; r < R; ++r) {
        const bool last = r == R - 1;
        const bool use_s = compat || nu > kEpsNu;
        const float nuf = (float)nu;
        for (int v = threadIdx.x; v < N; v += blockDim.x) {
            if (!__ldg(b.nd_mask + base + v)) continue;
            if (last && polish) {   // the FP64 counts for the polished solve
                const double* c = b.nd_cnt + (int64_t)(base + v) * 6;
                const double c0 = __ldcg(c), c1 = __ldcg(c + 1), c2 = __ldcg(c + 2),
                             c3 = __ldcg(c + 3), c4 = __ldcg(c + 4);
                const double dn = solve_branch(c0 + nu * (c0 + c1 + c3), c1,
                                               use_s ? c2 + c4 : 0.0, nu, (double)Dd[v], dlo,
                                               dhi, true);
                Dd[v] = (float)dn;
                __stcg(b.nd_d + base + v, dn);
            } else {
                const float4 q = C4[v];
                const float dn = solve_branch_f(q.x + nuf * q.y, q.z, use_s ? q.w : 0.f, nuf,
                                                Dd[v], (float)dlo, (float)dhi);
                Dd[v] = dn;
                if (last) __stcg(b.nd_d + base + v, (double)dn);
            }
        }
        __syncthreads();
        if (!(fix & 1)) {
            // -A nu + sum_v c_v log(1 - e^{-nu d_v}); compat: every branch,
            // exact: the optimised branches (EM_solver.py:392-407)
            float Af = 0.f, Csf = 0.f;
            for (int v = threadIdx.x; v < N; v += blockDim.x) {
                if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                const float4 q = C4[v];
                Af += q.y * Dd[v];
                Csf += q.w;
            }
            const float2 acf = block_sum2f(Af, Csf, sh);
            const double2 ac = make_double2((double)acf.x, (double)acf.y);
            double A = ac.x;
            const double nlo = compat ? kCalcEps : 1e-30, nhi = compat ? 1.0 - kCalcEps : 1.0;
            // G(nu) = -A + S1 / nu,  dG/dlog nu = -S2 / nu,  S1 = sum c h(nu d),
            // S2 = sum c h k  (h, k as in branch_F)
            auto sums = [&](double x, bool fp64) {
                if (fp64) {
                    double s1 = 0.0, s2 = 0.0;
                    for (int v = threadIdx.x; v < N; v += blockDim.x) {
                        if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                        const double* c = b.nd_cnt + (int64_t)(base + v) * 6;
                        const double cc = __ldcg(c + 2) + __ldcg(c + 4);
                        if (cc <= 0.0) continue;
                        const double y = x * __ldcg(b.nd_d + base + v), h = y / expm1(y);
                        s1 += cc * h;
                        s2 += cc * h * (h + y);
                    }
                    return block_sum2(s1, s2, sh);
                }
                float s1 = 0.f, s2 = 0.f;
                const float xf = (float)x;
                for (int v = threadIdx.x; v < N; v += blockDim.x) {
                    if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                    const float cc = C4[v].w;
                    if (cc <= 0.f) continue;
                    const float y = xf * Dd[v], h = y / expm1f(y);
                    s1 += cc * h;
                    s2 += cc * h * (h + y);
                }
                const float2 r = block_sum2f(s1, s2, sh);
                return make_double2((double)r.x, (double)r.y);
            };
            if (ac.y <= 0.0) {
                nu = compat ? nlo : 0.0;
            } else if (-A * nhi + sums(nhi, false).x >= 0.0) {
                nu = nhi;
            } else if (-A * nlo + sums(nlo, false).x <= 0.0) {
                nu = nlo;
            } else {
                float wlo = logf((float)nlo), whi = logf((float)nhi);
                float w = logf((float)fmin(fmax(nu, nlo), nhi));
                for (int it = 0; it < 20; ++it) {
                    const float x = expf(w);
                    const double2 S = sums(x, false);
                    const float H = (float)(-A * x + S.x);   // same sign as G
                    if (newton_step(H, H / (float)S.y, 1e-6f, w, wlo, whi)) break;
                }
                double wd = (double)w;
                if (last && polish) {   // FP64 Newton polish
                    double A64 = 0.0;
                    for (int v = threadIdx.x; v < N; v += blockDim.x) {
                        if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                        const double* c = b.nd_cnt + (int64_t)(base + v) * 6;
                        A64 += (__ldcg(c) + __ldcg(c + 1) + __ldcg(c + 3)) * __ldcg(b.nd_d + base + v);
                    }
                    A64 = block_sum2(A64, 0.0, sh).x;
                    for (int it = 0; it < 2; ++it) {
                        const double x = exp(wd);
                        const double2 S = sums(x, true);
                        const double wn = wd + (-A64 * x + S.x) / S.y;
                        if (!(wn > log(nlo) && wn < log(nhi)) || !(fabs(wn - wd) < 1e-3)) break;
                        wd = wn;
                    }
                }
                nu = fmin(fmax(polish ? exp(wd) : (double)expf(w), nlo), nhi);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        b.tr_nu[p] = nu;
        b.tr_phi[p] = phi;
    }
    // the arithmetic of the next passes: log mode once a branch's
    // d (1 + nu) leaves the range of the linear partials
    __shared__ int s_rate;
    if (threadIdx.x == 0) s_rate = 0;
    __syncthreads();
    int rate = 0;
    for (int v = threadIdx.x; v < N; v += blockDim.x) {
        reinterpret_cast<float4*>(b.nd_bt)[base + v] = branch_terms_of((double)Dd[v], nu, b.compat);
        rate = max(rate, __float_as_int(fmaxf(Dd[v] * (1.f + (float)nu), 0.f)));
    }
    atomicMax(&s_rate, rate);
    __syncthreads();
    if (threadIdx.x == 0)
        b.tr_mode[p] = __int_as_float(s_rate) > (float)LAML_LOG_MODE_RATE ? LAML_MODE_LOG
                                                                           : LAML_MODE_LINEAR;
    __syncthreads();
}

// per-tree log-likelihood (FP64 sum over sites) and the EM stopping rule
__device__ void tree_llh_item(const laml_batch& b, int p, int mode, double rel_tol, int max_iters) {
    // mode 0: plain sum; 1: init (llh_prev = llh); 2: EM update
    if (mode == 2 && __ldcg(b.tr_status + p) != LAML_TREE_ACTIVE) return;
    const int ds = __ldg(b.tr_ds + p), K = __ldg(b.ds_sites + ds);
    const int64_t t = __ldg(b.tr_site_base + p);
    double s = 0.0;
    for (int c = 0; c < K; ++c) s += __ldcg(b.llh_site + t + c);
    if (mode == 0) { b.tr_llh[p] = s; return; }
    if (mode == 1) {
        b.tr_llh[p] = s;
        b.tr_llh_prev[p] = s;
        b.tr_iter[p] = 0;
        b.tr_status[p] = LAML_TREE_ACTIVE;
        return;
    }
    const double prev = b.tr_llh_prev[p];
    const int it = b.tr_iter[p] + 1;
    b.tr_iter[p] = it;
    if (fabs(s - prev) / fabs(prev) < rel_tol) {
        b.tr_llh[p] = s;
        b.tr_status[p] = LAML_TREE_CONVERGED;
    } else if (isnan(s)) {
        b.tr_llh[p] = prev;
        b.tr_status[p] = LAML_TREE_NAN;
    } else {
        b.tr_llh[p] = s;
        b.tr_llh_prev[p] = s;
        if (it >= max_iters) b.tr_status[p] = LAML_TREE_MAXITER;
    }
}

// ---------------------------------------------------------------------------
// grid barrier with a bounded wait (no trap: on timeout the error word is set
// and every block returns)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const uint32_t* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ bool grid_barrier(const laml_batch& b, unsigned& gen) {
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        const unsigned arrived = atomicAdd(b.barrier, 1u);
        if (arrived == gen * gridDim.x + gridDim.x - 1) {
            atomicExch(b.barrier + 1, gen + 1);
        } else {
            const unsigned long long t0 = gtimer();
            while (ld_acquire(b.barrier + 1) <= gen) {
                if (*(volatile int*)b.error != 0) { ok = 0; break; }
                if (gtimer() - t0 > 2000000000ull) {   // 2 s
                    atomicCAS(b.error, 0, LAML_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
        if (*(volatile int*)b.error != 0) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    ++gen;
    return s_ok != 0;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
template <int G, int KIND>
__device__ __forceinline__ void for_items(const laml_batch& b, const int32_t* items, int64_t n,
                                          int gwarp, int nwarps, bool want_post,
                                          bool respect_status, const int32_t* desc = nullptr) {
    constexpr int kind = KIND;
    constexpr int IPW = 32 / G;
    const int lane32 = threadIdx.x & 31, lane = lane32 % G, sub = lane32 / G;
    const int64_t nw = (n + IPW - 1) / IPW;
    for (int64_t wi = gwarp; wi < nw; wi += nwarps) {
        const int64_t it = wi * IPW + sub;
        const bool act = it < n;
        if constexpr (KIND <= 1 || KIND == 5) {   // descriptor-driven inside / outside
            const ItemDesc d = load_desc(desc, act ? it : 0);
            if constexpr (KIND == 0) {
                if (act) inside_item_d<G>(b, d, lane, respect_status);
            } else if constexpr (KIND == 1) {
                outside_item_d<G>(b, d, lane, act, want_post);
            } else {
                outside_root_item_d<G>(b, d, lane, act, want_post);
            }
        } else {
            const int node = act ? __ldg(items + 2 * it) : 0;
            const int g = act ? __ldg(items + 2 * it + 1) : 0;
            if constexpr (KIND == 2) {
                if (act) root_init_item<G>(b, node, g, lane, want_post);
            } else {
                root_counts_item<G>(b, node, g, lane, act, (b.compat && kind == 3) ? 1 : 2);
            }
        }
    }
}

template <int G, int KIND>
__global__ void __launch_bounds__(kBlock, KIND == 1 ? LAML_MINB_OUT : LAML_MINB) k_items(laml_batch b, const int32_t* items, int64_t n,
                                                   int want_post, int respect_status,
                                                   const int32_t* desc) {
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for_items<G, KIND>(b, items, n, gwarp, nwarps, want_post != 0, respect_status != 0, desc);
}

__global__ void __launch_bounds__(kBlock, 4) k_mstep(laml_batch b, int rounds, int flags) {
    __shared__ double2 sh[kBlock / 32];
    __shared__ float4 s_cnt[kMstepStage];
    __shared__ float s_d[kMstepStage];
    for (int p = blockIdx.x; p < b.n_trees; p += gridDim.x)
        mstep_tree(b, p, rounds, sh, s_cnt, s_d, (flags & LAML_MSTEP_FP64_POLISH) != 0);
}

// d logL / d(d_v, nu, phi) from the expected counts (Fisher's identity: the
// gradient of the expected complete-data log-likelihood at the current
// parameters); with the compat EPS floors a floored term has zero derivative.
__global__ void __launch_bounds__(kBlock) k_gradient(laml_batch b, double* grad_d,
                                                     double* grad_np) {
    __shared__ double2 sh[kBlock / 32];
    for (int p = blockIdx.x; p < b.n_trees; p += gridDim.x) {
        const int N = b.tr_nodes[p], n = b.tr_leaves[p], base = b.tr_node_base[p];
        const int ds = b.tr_ds[p], NG = b.ds_groups[ds], K = b.ds_sites[ds];
        const int64_t cb = b.tr_cnt_base[p];
        const bool compat = b.compat != 0;
        const double nu = b.tr_nu[p], phi = b.tr_phi[p];
        double gnu = 0.0, lrm = 0.0, lro = 0.0;
        for (int v = threadIdx.x; v < N; v += blockDim.x) {
            double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const float4* src = reinterpret_cast<const float4*>(b.cnt_part + cb + (int64_t)v * NG * 8);
            for (int g = 0; g < NG; ++g) {
                const float4 x = src[2 * g], z = src[2 * g + 1];
                c[0] += x.x; c[1] += x.y; c[2] += x.z; c[3] += x.w;
                c[4] += z.x; c[5] += z.y; c[6] += z.z; c[7] += z.w;
            }
            const double d = b.nd_d[base + v], nd = d * nu;
            const double dt3 = (compat && d < kEPSd) ? 0.0 : 1.0 / expm1(d);   // d/dd log(1-e^-d)
            const bool fl2 = (compat && nd < kEPSd) || nu <= 0.0;
            const double en = expm1(nd);
            const double dt2_dd = fl2 ? 0.0 : nu / en, dt2_dnu = fl2 ? 0.0 : d / en;
            const double cs = c[2] + c[4];
            grad_d[base + v] = -c[0] * (1.0 + nu) + c[1] * (dt3 - nu) + cs * dt2_dd - c[3] * nu;
            gnu += -(c[0] + c[1] + c[3]) * d + cs * dt2_dnu;
            lrm += c[6];
            lro += c[7];
        }
        const double gsum = block_sum2(gnu, 0.0, sh).x;
        const double2 L = block_sum2(lrm, lro, sh);
        if (threadIdx.x == 0) {
            const double M = b.ds_missing[ds], R = (double)n * K - M;
            const double de1 = (compat && 1.0 - phi <= kEPSd) ? 0.0 : -1.0 / (1.0 - phi);
            const double dep = (compat && phi <= kEPSd) ? 0.0 : 1.0 / phi;
            grad_np[2 * p] = gsum;
            grad_np[2 * p + 1] = (R - L.y) * de1 + (M - L.x) * dep;
        }
        __syncthreads();
    }
}

__global__ void k_tree_llh(laml_batch b, int mode, double rel_tol, int max_iters) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < b.n_trees) tree_llh_item(b, p, mode, rel_tol, max_iters);
}

// per tree: log mode if some branch has d (1 + nu) > LAML_LOG_MODE_RATE
__global__ void k_tree_mode(laml_batch b) {
    __shared__ int s_rate;
    for (int p = blockIdx.x; p < b.n_trees; p += gridDim.x) {
        if (threadIdx.x == 0) s_rate = 0;
        __syncthreads();
        const int N = b.tr_nodes[p], base = b.tr_node_base[p];
        const double nu = b.tr_nu[p];
        int rate = 0;
        for (int v = threadIdx.x; v < N; v += blockDim.x)
            rate = max(rate, __float_as_int(fmaxf((float)(b.nd_d[base + v] * (1.0 + nu)), 0.f)));
        atomicMax(&s_rate, rate);
        __syncthreads();
        if (threadIdx.x == 0)
            b.tr_mode[p] = __int_as_float(s_rate) > (float)LAML_LOG_MODE_RATE ? LAML_MODE_LOG
                                                                               : LAML_MODE_LINEAR;
        __syncthreads();
    }
}

__global__ void k_branch_terms(laml_batch b) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < b.n_nodes) {
        const int p = b.nd_tree[i];
        reinterpret_cast<float4*>(b.nd_bt)[i] = branch_terms_of(b.nd_d[i], b.tr_nu[p], b.compat);
    }
}

// Item descriptors from the node arrays already on the device: the same 12
// int32 per item that laml_plan_fill writes on the host, three 16-byte stores.
__global__ void k_item_desc(laml_batch b, const int32_t* __restrict__ items, int64_t n,
                            int32_t* __restrict__ desc) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int u = items[2 * k], g = items[2 * k + 1];
        const int tree = b.nd_tree[u];
        const int d = b.tr_ds[tree];
        const int v = b.nd_c0[u], w = b.nd_c1[u];
        const bool vl = b.nd_c0[v] < 0, wl = b.nd_c0[w] < 0;
        const int flags = (vl ? 1 : 0) | (wl ? 2 : 0) | (b.tr_root[tree] == u ? 4 : 0);
        const int32_t rv = vl ? b.nd_leafrow[v] : (int32_t)(b.nd_prow[v] / 8);
        const int32_t rw = wl ? b.nd_leafrow[w] : (int32_t)(b.nd_prow[w] / 8);
        int4* e = reinterpret_cast<int4*>(desc + 12 * k);
        e[0] = make_int4(u, v, w, tree | (flags << 24));
        e[1] = make_int4(g, b.ds_group_base[d] + g, (int32_t)b.nd_srow[u],
                         (int32_t)(b.nd_prow[u] / 8));
        e[2] = make_int4(rv, rw, (int32_t)b.nd_srow[v], (int32_t)b.nd_srow[w]);
    }
}

// Group table: one block per dataset.
__global__ void k_group_desc(laml_batch b, int32_t* __restrict__ grp) {
    const int d = blockIdx.x;
    const int NG = b.ds_groups[d];
    for (int g = threadIdx.x; g < NG; g += blockDim.x) {
        const int gi = b.ds_group_base[d] + g;
        const int off = b.group_off[gi];
        int4* e = reinterpret_cast<int4*>(grp + 8 * (int64_t)gi);
        e[0] = make_int4(off, b.ds_site_base[d] + g * b.group_sites,
                         (int32_t)(b.ds_q_base[d] + off), d);
        e[1] = make_int4((int32_t)b.ds_code_base[d], b.ds_sites_pad[d], b.ds_sites[d], 0);
    }
}

template <int G>
__global__ void __launch_bounds__(kBlock, LAML_MINB) k_em_persistent(laml_batch b, int iters, int rounds,
                                                           double rel_tol, int max_iters, int flags) {
    __shared__ double2 sh[kBlock / 32];
    __shared__ float4 s_cnt[kMstepStage];
    __shared__ float s_d[kMstepStage];
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned gen = 0;
    for (int it = 0; it < iters; ++it) {
        for_items<G, 2>(b, b.root_items, b.n_root_items, gwarp, nwarps, false, true);
        if (!grid_barrier(b, gen)) return;
        for (int l = 0; l < b.n_out_levels; ++l) {
            const int64_t o = b.out_level_off[l], e = b.out_level_off[l + 1];
            if (l == 0)   // the roots
                for_items<G, 5>(b, b.out_items + 2 * o, e - o, gwarp, nwarps, false, true,
                                b.out_desc + 12 * o);
            else
                for_items<G, 1>(b, b.out_items + 2 * o, e - o, gwarp, nwarps, false, true,
                                b.out_desc + 12 * o);
            if (!grid_barrier(b, gen)) return;
        }
        for_items<G, 3>(b, b.root_items, b.n_root_items, gwarp, nwarps, false, true);
        if (!grid_barrier(b, gen)) return;
        for (int p = blockIdx.x; p < b.n_trees; p += gridDim.x)
            mstep_tree(b, p, rounds, sh, s_cnt, s_d, (flags & LAML_MSTEP_FP64_POLISH) != 0);
        if (!grid_barrier(b, gen)) return;
        for (int l = 0; l < b.n_in_levels; ++l) {
            const int64_t o = b.in_level_off[l], e = b.in_level_off[l + 1];
            for_items<G, 0>(b, b.in_items + 2 * o, e - o, gwarp, nwarps, false, true,
                            b.in_desc + 12 * o);
            if (!grid_barrier(b, gen)) return;
        }
        for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < b.n_trees;
             p += gridDim.x * blockDim.x)
            tree_llh_item(b, p, 2, rel_tol, max_iters);
        if (!grid_barrier(b, gen)) return;
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
int g_num_sms = 0;

int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

int check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        laml::set_error(std::string(what) + ": " + cudaGetErrorString(e));
        return LAML_ERR_CUDA;
    }
    return LAML_OK;
}

int validate(const laml_batch* b) {
    if (!b || b->n_trees <= 0 || b->n_nodes <= 0) {
        laml::set_error("laml_batch: empty or null batch");
        return LAML_ERR_ARG;
    }
    if (b->group_sites != 8 && b->group_sites != 16 && b->group_sites != 32) {
        laml::set_error("laml_batch: group_sites must be 8, 16 or 32");
        return LAML_ERR_ARG;
    }
    if (!b->tr_mode) {
        laml::set_error("laml_batch: tr_mode (one int32 per tree) is required");
        return LAML_ERR_ARG;
    }
    if (!b->in_desc || !b->out_desc || !b->grp_desc) {
        laml::set_error("laml_batch: in_desc, out_desc and grp_desc (laml_plan_fill) are required");
        return LAML_ERR_ARG;
    }
    return LAML_OK;
}

template <int G>
int launch_items(const laml_batch& b, const int32_t* items, int64_t n, int kind, int want_post,
                 int respect_status, cudaStream_t st, const int32_t* desc = nullptr) {
    if (n <= 0) return LAML_OK;
    const int ipb = (kBlock / 32) * (32 / G);
    int64_t blocks = (n + ipb - 1) / ipb;
    const int64_t cap = (int64_t)num_sms() * 16;
    if (blocks > cap) blocks = cap;
    switch (kind) {
        case 0: k_items<G, 0><<<(unsigned)blocks, kBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        case 1: k_items<G, 1><<<(unsigned)blocks, kBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        case 2: k_items<G, 2><<<(unsigned)blocks, kBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        case 3: k_items<G, 3><<<(unsigned)blocks, kBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        case 5: k_items<G, 5><<<(unsigned)blocks, kBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        default: k_items<G, 4><<<(unsigned)blocks, kBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
    }
    return check(cudaGetLastError(), "k_items launch");
}

// host copies of the level offsets (tiny) are needed to launch per level
struct Levels {
    std::vector<int32_t> in, out;
};

int fetch_levels(const laml_batch& b, Levels& L, cudaStream_t st) {
    L.in.resize(b.n_in_levels + 1);
    L.out.resize(b.n_out_levels + 1);
    if (b.h_in_level_off && b.h_out_level_off) {
        std::copy(b.h_in_level_off, b.h_in_level_off + L.in.size(), L.in.begin());
        std::copy(b.h_out_level_off, b.h_out_level_off + L.out.size(), L.out.begin());
        return LAML_OK;
    }
    int rc = check(cudaMemcpyAsync(L.in.data(), b.in_level_off, sizeof(int32_t) * L.in.size(),
                                   cudaMemcpyDeviceToHost, st), "level offsets");
    if (rc) return rc;
    rc = check(cudaMemcpyAsync(L.out.data(), b.out_level_off, sizeof(int32_t) * L.out.size(),
                               cudaMemcpyDeviceToHost, st), "level offsets");
    if (rc) return rc;
    return check(cudaStreamSynchronize(st), "level offsets");
}

template <int G>
int inside_t(const laml_batch& b, int update_em, cudaStream_t st, const Levels& L,
             int respect_status) {
    for (int l = 0; l < b.n_in_levels; ++l) {
        int rc = launch_items<G>(b, b.in_items + 2 * (int64_t)L.in[l], L.in[l + 1] - L.in[l], 0, 0,
                                 respect_status, st,
                                 b.in_desc + 12 * (int64_t)L.in[l]);
        if (rc) return rc;
    }
    return LAML_OK;
}

template <int G>
int outside_t(const laml_batch& b, int flags, cudaStream_t st, const Levels& L) {
    const int want_post = flags & LAML_OUT_POSTERIORS;
    int rc = launch_items<G>(b, b.root_items, b.n_root_items, 2, want_post, 1, st);
    if (rc) return rc;
    for (int l = 0; l < b.n_out_levels; ++l) {
        // level 0 holds the roots (parents at depth 0)
        rc = launch_items<G>(b, b.out_items + 2 * (int64_t)L.out[l], L.out[l + 1] - L.out[l],
                             l == 0 ? 5 : 1, want_post, 1, st,
                             b.out_desc + 12 * (int64_t)L.out[l]);
        if (rc) return rc;
    }
    // kind 3: the E-step row of the root (compat: from node N-1); kind 4: from
    // the progenitor in state 0 (the true posterior counts, for gradients)
    return launch_items<G>(b, b.root_items, b.n_root_items,
                           (flags & LAML_OUT_TRUE_ROOT) ? 4 : 3, 0, 1, st);
}

template <int G>
int em_levels_t(const laml_batch& b, int iters, int rounds, double tol, int max_iters,
                int flags, cudaStream_t st) {
    Levels L;
    int rc = fetch_levels(b, L, st);
    if (rc) return rc;
    const int tb = (b.n_trees + 127) / 128;
    for (int it = 0; it < iters; ++it) {
        if ((rc = outside_t<G>(b, 0, st, L))) return rc;
        k_mstep<<<b.n_trees, kBlock, 0, st>>>(b, rounds, flags);
        if ((rc = check(cudaGetLastError(), "k_mstep"))) return rc;
        if ((rc = inside_t<G>(b, 0, st, L, 1))) return rc;
        k_tree_llh<<<tb, 128, 0, st>>>(b, 2, tol, max_iters);
        if ((rc = check(cudaGetLastError(), "k_tree_llh"))) return rc;
    }
    return LAML_OK;
}

template <int G>
int em_persistent_t(const laml_batch& b, int iters, int rounds, double tol, int max_iters,
                    int flags, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    int per_sm = 0;
    int rc = check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_em_persistent<G>,
                                                                 kBlock, 0), "occupancy");
    if (rc) return rc;
    if (!coop || per_sm <= 0) {
        laml::set_error("cooperative launch unavailable for the persistent EM kernel");
        return LAML_ERR_CUDA;
    }
    const int grid = per_sm * num_sms();
    if ((rc = check(cudaMemsetAsync(b.barrier, 0, 2 * sizeof(uint32_t), st), "barrier reset")))
        return rc;
    laml_batch bb = b;
    void* args[] = {&bb, &iters, &rounds, &tol, &max_iters, &flags};
    return check(cudaLaunchCooperativeKernel((const void*)k_em_persistent<G>, dim3(grid),
                                             dim3(kBlock), args, 0, st),
                 "k_em_persistent launch");
}

struct GraphHolder {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

#define DISPATCH_G(b, call)                                   \
    switch ((b).group_sites) {                                \
        case 8: { constexpr int GG = 8; return call; }        \
        case 16: { constexpr int GG = 16; return call; }      \
        default: { constexpr int GG = 32; return call; }      \
    }

}  // namespace

extern "C" int laml_supported_group_sites(void) { return 8 | 16 | 32; }

extern "C" int laml_gradient(const laml_batch* b, double* grad_d, double* grad_nu_phi,
                             void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    if (!grad_d || !grad_nu_phi) {
        laml::set_error("laml_gradient: null output");
        return LAML_ERR_ARG;
    }
    k_gradient<<<b->n_trees, kBlock, 0, (cudaStream_t)stream>>>(*b, grad_d, grad_nu_phi);
    return check(cudaGetLastError(), "k_gradient");
}

extern "C" int laml_branch_terms(const laml_batch* b, void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t blocks = (b->n_nodes + kBlock - 1) / kBlock;
    k_branch_terms<<<(unsigned)blocks, kBlock, 0, st>>>(*b);
    if ((rc = check(cudaGetLastError(), "k_branch_terms"))) return rc;
    const int tb = std::min(b->n_trees, num_sms() * 8);
    k_tree_mode<<<tb, 128, 0, st>>>(*b);
    return check(cudaGetLastError(), "k_tree_mode");
}

extern "C" int laml_plan_descriptors(const laml_batch* b, int32_t* in_desc, int32_t* out_desc,
                                     int32_t* grp_desc, void* stream) {
    if (!b || b->n_trees <= 0 || b->n_nodes <= 0 || b->n_datasets <= 0) {
        laml::set_error("laml_plan_descriptors: empty or null batch");
        return LAML_ERR_ARG;
    }
    const uintptr_t mis = (uintptr_t)in_desc | (uintptr_t)out_desc | (uintptr_t)grp_desc;
    if (!in_desc || !out_desc || !grp_desc || (mis & 15)) {
        laml::set_error("laml_plan_descriptors: null or misaligned (16 B) output");
        return LAML_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t cap = (int64_t)num_sms() * 8;
    auto blocks = [&](int64_t n) { return (unsigned)std::max<int64_t>(1, std::min(cap, (n + kBlock - 1) / kBlock)); };
    if (b->n_in_items > 0)
        k_item_desc<<<blocks(b->n_in_items), kBlock, 0, st>>>(*b, b->in_items, b->n_in_items, in_desc);
    if (b->n_out_items > 0)
        k_item_desc<<<blocks(b->n_out_items), kBlock, 0, st>>>(*b, b->out_items, b->n_out_items, out_desc);
    k_group_desc<<<b->n_datasets, 128, 0, st>>>(*b, grp_desc);
    return check(cudaGetLastError(), "laml_plan_descriptors");
}

extern "C" int laml_inside(const laml_batch* b, int32_t update_em, void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Levels L;
    if ((rc = fetch_levels(*b, L, st))) return rc;
    auto run = [&]() -> int { DISPATCH_G(*b, (inside_t<GG>(*b, update_em, st, L, 0))); };
    if ((rc = run())) return rc;
    const int tb = (b->n_trees + 127) / 128;
    k_tree_llh<<<tb, 128, 0, st>>>(*b, update_em ? 1 : 0, 0.0, 0);
    return check(cudaGetLastError(), "k_tree_llh");
}

extern "C" int laml_outside(const laml_batch* b, int32_t flags, void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    if ((flags & LAML_OUT_POSTERIORS) && (!b->post0 || !b->post1)) {
        laml::set_error("laml_outside: want_post needs post0/post1 buffers");
        return LAML_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    Levels L;
    if ((rc = fetch_levels(*b, L, st))) return rc;
    DISPATCH_G(*b, (outside_t<GG>(*b, flags, st, L)));
}

extern "C" int laml_mstep(const laml_batch* b, int32_t rounds, int32_t flags, void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    k_mstep<<<b->n_trees, kBlock, 0, (cudaStream_t)stream>>>(*b, rounds, flags);
    return check(cudaGetLastError(), "k_mstep");
}

extern "C" int laml_em_run(const laml_batch* b, int32_t iters, int32_t rounds, double rel_tol,
                           int32_t max_iters, int32_t flags, void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    if (iters <= 0) return LAML_OK;
    DISPATCH_G(*b, (em_persistent_t<GG>(*b, iters, rounds, rel_tol, max_iters, flags,
                                        (cudaStream_t)stream)));
}

extern "C" int laml_em_graph_create(const laml_batch* b, int32_t iters, int32_t rounds,
                                    double rel_tol, int32_t max_iters, int32_t flags,
                                    int32_t persistent, void** graph) {
    int rc = validate(b);
    if (rc) return rc;
    if (!graph || iters <= 0) {
        laml::set_error("laml_em_graph_create: bad argument");
        return LAML_ERR_ARG;
    }
    if (!persistent && (!b->h_in_level_off || !b->h_out_level_off)) {
        laml::set_error("laml_em_graph_create: per-level capture needs the host level offsets");
        return LAML_ERR_ARG;
    }
    cudaStream_t st;
    if ((rc = check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream"))) return rc;
    GraphHolder* g = new GraphHolder();
    rc = check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (!rc) {
        auto body = [&]() -> int {
            if (persistent) {
                DISPATCH_G(*b, (em_persistent_t<GG>(*b, iters, rounds, rel_tol, max_iters, flags, st)));
            }
            DISPATCH_G(*b, (em_levels_t<GG>(*b, iters, rounds, rel_tol, max_iters, flags, st)));
        };
        int brc = body();
        cudaGraph_t gr = nullptr;
        int erc = check(cudaStreamEndCapture(st, &gr), "end capture");
        rc = brc ? brc : erc;
        g->graph = gr;
        if (!rc) rc = check(cudaGraphInstantiate(&g->exec, gr, 0), "graph instantiate");
    }
    cudaStreamDestroy(st);
    if (rc) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        delete g;
        return rc;
    }
    *graph = g;
    return LAML_OK;
}

extern "C" int laml_graph_launch(void* graph, void* stream) {
    if (!graph) {
        laml::set_error("laml_graph_launch: null graph");
        return LAML_ERR_ARG;
    }
    GraphHolder* g = static_cast<GraphHolder*>(graph);
    return check(cudaGraphLaunch(g->exec, (cudaStream_t)stream), "graph launch");
}

extern "C" void laml_graph_destroy(void* graph) {
    if (!graph) return;
    GraphHolder* g = static_cast<GraphHolder*>(graph);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
}

extern "C" int laml_em_run_levels(const laml_batch* b, int32_t iters, int32_t rounds,
                                  double rel_tol, int32_t max_iters, int32_t flags, void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    if (iters <= 0) return LAML_OK;
    DISPATCH_G(*b, (em_levels_t<GG>(*b, iters, rounds, rel_tol, max_iters, flags,
                                    (cudaStream_t)stream)));
}

// ---------------------------------------------------------------------------
// laml_inside_noalloc: the inside pass for callers that cannot allocate
// device memory.  Its scratch (the inside partial rows and the per-(node,
// site) scale exponents and prior-weighted sums) is a fixed array of the
// library, not a caller buffer.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;   // 32 MiB per device
// Device storage of the no-allocation entry point.  In host code this name is
// only a stand-in: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[128] = {};   // device address of the scratch, per device ordinal

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

template <int G>
__global__ void __launch_bounds__(kBlock, LAML_MINB) k_inside_level(laml_batch b, int level) {
    const int32_t o = b.in_level_off[level], e = b.in_level_off[level + 1];
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for_items<G, 0>(b, b.in_items + 2 * (int64_t)o, e - o, gwarp, nwarps, false, false,
                    b.in_desc + 12 * (int64_t)o);
}

template <int G>
int inside_noalloc_t(const laml_batch& b, cudaStream_t st) {
    const unsigned grid = (unsigned)num_sms() * 8;
    for (int l = 0; l < b.n_in_levels; ++l) {
        k_inside_level<G><<<grid, kBlock, 0, st>>>(b, l);
        int rc = check(cudaGetLastError(), "k_inside_level");
        if (rc) return rc;
    }
    const int tb = (b.n_trees + 127) / 128;
    k_tree_llh<<<tb, 128, 0, st>>>(b, 0, 0.0, 0);
    return check(cudaGetLastError(), "k_tree_llh");
}

}  // namespace

extern "C" int laml_inside_noalloc(const laml_batch* b, int64_t part_floats, int64_t scalar_len,
                                   void* stream) {
    int rc = validate(b);
    if (rc) return rc;
    if (part_floats < 0 || scalar_len < 0) {
        laml::set_error("laml_inside_noalloc: negative size");
        return LAML_ERR_ARG;
    }
    const size_t need = align256((size_t)part_floats * sizeof(float)) +
                        3 * align256((size_t)scalar_len * sizeof(float));
    if (need > kNoAllocScratchBytes) {
        laml::set_error("laml_inside_noalloc: the batch needs " + std::to_string(need) +
                        " bytes of scratch; the library's fixed scratch holds " +
                        std::to_string(kNoAllocScratchBytes) + " bytes (use laml_inside)");
        return LAML_ERR_ARG;
    }
    int dev = 0;
    if ((rc = check(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
    if (dev < 0 || dev >= 128) {
        laml::set_error("laml_inside_noalloc: device ordinal out of range");
        return LAML_ERR_ARG;
    }
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            // once per device, with that device current
            void* p = nullptr;
            if ((rc = check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress")))
                return rc;
            g_noalloc_addr[dev] = p;
        }
        base = g_noalloc_addr[dev];
    }
    unsigned char* s = static_cast<unsigned char*>(base);
    laml_batch bb = *b;
    bb.in_part = reinterpret_cast<float*>(s);
    s += align256((size_t)part_floats * sizeof(float));
    bb.in_x = reinterpret_cast<int32_t*>(s);
    s += align256((size_t)scalar_len * sizeof(float));
    bb.in_h = reinterpret_cast<int32_t*>(s);
    s += align256((size_t)scalar_len * sizeof(float));
    bb.in_dot = reinterpret_cast<float*>(s);
    cudaStream_t st = (cudaStream_t)stream;
    DISPATCH_G(bb, (inside_noalloc_t<GG>(bb, st)));
}
