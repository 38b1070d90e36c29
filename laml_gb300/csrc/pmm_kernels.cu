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
#include <cooperative_groups.h>
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
constexpr double kLogEps = -13.815510557964274;   // log(1e-6)
constexpr int kBlock = 256;
#ifndef LAML_ITEMS_BLOCK
#define LAML_ITEMS_BLOCK 128   // threads per block of the per-level item kernels
#endif
constexpr int kItemsBlock = LAML_ITEMS_BLOCK;
constexpr unsigned kFull = 0xffffffffu;
#ifndef LAML_CHUNK
#define LAML_CHUNK 4
#endif
constexpr int kChunk = LAML_CHUNK;   // states loaded ahead per step of a state loop
#ifndef LAML_OCHUNK
#define LAML_OCHUNK LAML_CHUNK
#endif
constexpr int kOChunk = LAML_OCHUNK;   // the same for the outside items' state loop
#ifndef LAML_MINB
#define LAML_MINB 4
#endif
#ifndef LAML_MINB_IN
#define LAML_MINB_IN 8   // resident blocks per SM asked of the other item kernels (64 registers)
#endif
// resident blocks per SM asked of the wide outside kernel: 8 (64 registers)
// for batches of up to kOutBlocksStates states per site, 6 (80 registers)
// above -- longer state loops reload more of what 64 registers spill and
// leave less L1 beside 8 blocks' stashes (measured: 512 candidates of 40
// sites and 7-52 states, outside pass 1.85 ms at 8 blocks, 1.98 at 6; one
// 50,000-leaf tree of 300 sites and 22-102 states, 2.81 ms at 8, 2.27 at 6)
constexpr int kOutBlocksStates = 64;
constexpr int kMstepStage = 2048;    // branches of a tree staged in shared memory by the M-step
constexpr int kOStash = 34;          // words per thread the outside item parks in shared memory

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pow2i(int e) {   // 2^e for e in [-126, 127]
    return __int_as_float((127 + e) << 23);
}

// bulk prefetch of [p, p + bytes) into L2 (16-byte aligned, a multiple of
// 16 bytes); a hint with no completion to wait for
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Sums of products in the level kernels' shared arithmetic are written with
// the round-to-nearest intrinsics: the compiler may not fuse them into FMAs
// on its own, which it could do differently in each kernel that inlines
// them, so every path (direct, bulk-staged, persistent) rounds alike and
// their results stay bitwise equal.
__device__ __forceinline__ float mulr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float addr(float a, float b) { return __fadd_rn(a, b); }
// the transition out of state 0 applied to a child's vector: P00 s0 + Pmut D + Psil ss
__device__ __forceinline__ float edge0(const float4& bt, float s0, float D, float ss) {
    return addr(addr(mulr(bt.x, s0), mulr(bt.y, D)), mulr(bt.w, ss));
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

// the leaf emission terms of a tree's phi (FP32 pair in tr_leaf when the
// batch keeps one: GB300's FP64 pipe is narrow, and every item reads them)
__device__ __forceinline__ float2 leaf_pair(double phi, int compat) {
    return compat ? make_float2(fmaxf((float)(1.0 - phi), kEPS), fmaxf((float)phi, kEPS))
                  : make_float2((float)(1.0 - phi), (float)phi);
}

__device__ __forceinline__ Leaf leaf_params(const laml_batch& b, int tree) {
    Leaf L;
    if (b.tr_leaf) {
        const float2 e = __ldcg(reinterpret_cast<const float2*>(b.tr_leaf) + tree);
        L.e1 = e.x;
        L.ephi = e.y;
        L.es = b.compat ? kEPS : 0.f;
        return L;
    }
    double phi = __ldcg(b.tr_phi + tree);
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
// FP64 carries the large parts (exponents, d (1 + nu), nu d) and the sums;
// the transcendental parts, whose arguments lie in a small range after that
// split, run in FP32 (GB300's FP64 pipe is narrow): each result is rounded
// to FP32 anyway.
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
    e.lm = (double)logf((b.compat && d < kEPSd) ? kEPS : -expm1f(-(float)d)) - nd;
    e.ls = (b.compat && nd < kEPSd) ? kLogEps : (double)logf(-expm1f(-(float)nd));
    return e;
}

// log of a non-negative FP32 value (-inf at 0): the binary exponent exactly,
// the mantissa in [0.5, 1) through logf
__device__ __forceinline__ double logz(float x) {
    if (!(x > 0.f)) return -(double)INFINITY;
    int e;
    const float m = frexpf(x, &e);
    return (double)e * kLn2 + (double)logf(m);
}

// exp(l) rounded to FP32 (0 below its range): 2^k exactly times expf of the
// remainder in [0, ln 2)
__device__ __forceinline__ float expz(double l) {
    if (isnan(l)) return NAN;
    if (!(l > -110.0)) return 0.f;
    if (l > 89.0) return INFINITY;
    const double k = floor(l / kLn2);
    return ldexpf(expf((float)(l - k * kLn2)), (int)k);
}

__device__ __forceinline__ double lse3(double a, double b, double c) {
    const double m = fmax(a, fmax(b, c));
    if (m == -(double)INFINITY) return m;
    const float s = expf((float)(a - m)) + expf((float)(b - m)) + expf((float)(c - m));
    return m + (double)logf(s);
}

// exp(l) = m * 2^e with m in [0.5, 1) (m = 0, e = 0 for l = -inf)
__device__ __forceinline__ float split_exp(double l, int& e) {
    if (!(l > -(double)INFINITY)) {
        e = 0;
        return 0.f;
    }
    e = (int)floor(l / kLn2) + 1;
    return expf((float)(l - (double)e * kLn2));
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
    if (l > -(double)INFINITY) m = split_exp(l, e);
    __stcg(b.root_lr + t, m);
    __stcg(b.root_x + t, X + e);
    __stcg(b.llh_site + t, l + (double)X * kLn2);
}

// log of 1 / (site likelihood) at scale 2^X
__device__ __forceinline__ double root_log_scale(const laml_batch& b, int tree, int site, int X) {
    const int64_t t = __ldg(b.tr_site_base + tree) + site;
    const float m = __ldcg(b.root_lr + t);
    if (!(m > 0.f)) return -(double)INFINITY;   // a zero likelihood: no responsibilities
    return (double)(X - __ldcg(b.root_x + t)) * kLn2 - logz(m);
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
    const float outs = addr(mulr(bv.w, addr(o.x0, o.sumx)), o.xs);
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

// The two children's 8 count sums over an item's G lanes, reduce-scattered:
// each round a lane keeps half of the values it holds, adds its partner's
// copy of that half and hands over the other half, so after log2(G) rounds
// lane l holds the totals of 16/G of the 16 values and stores them itself.
// Every total comes from the same pairs in the same order as a full
// butterfly (x_l + x_{l^off}, commutative), so the bits are those of an
// all-reduce, with 14 exchanges instead of 48 for G = 8.
template <int G>
__device__ __forceinline__ void scatter_counts(const laml_batch& b, int tree, int v, int w, int g,
                                               int lane, bool act, const float* cv,
                                               const float* cw) {
    float x[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        x[k] = cv[k];
        x[8 + k] = cw[k];
    }
    int base = 0;
#pragma unroll
    for (int off = G / 2, n = 16; off > 0; off >>= 1) {
        if (n > 1) {
            const bool up = (lane & off) != 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (i < n / 2) {
                    const float keep = up ? x[i + n / 2] : x[i];
                    const float give = up ? x[i] : x[i + n / 2];
                    x[i] = keep + __shfl_xor_sync(kFull, give, off);
                }
            }
            base += up ? n / 2 : 0;
            n /= 2;
        } else {   // G = 32: the last round adds the one value both lanes hold
            x[0] += __shfl_xor_sync(kFull, x[0], off);
        }
    }
    if (!act || __ldcg(b.tr_status + tree) != LAML_TREE_ACTIVE) return;
    constexpr int PER = G >= 16 ? 1 : 16 / G;   // totals a lane stores
    if (G == 32 && (lane & 1)) return;          // lanes 2m, 2m + 1 hold the same total
    const int ds = __ldg(b.tr_ds + tree);
    const int NG = __ldg(b.ds_groups + ds);
    const int node = base < 8 ? v : w;
    float* dst = b.cnt_part + __ldg(b.tr_cnt_base + tree) +
                 ((int64_t)(node - __ldg(b.tr_node_base + tree)) * NG + g) * 8 + (base & 7);
    if (PER == 2) __stcg(reinterpret_cast<float2*>(dst), make_float2(x[0], x[1]));
    else __stcg(dst, x[0]);
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
    e.lm = logf((b.compat && d < kEPSd) ? kEPS : -expm1f(-(float)d)) - (float)nd;
    e.ls = (b.compat && nd < kEPSd) ? (float)kLogEps : logf(-expm1f(-(float)nd));
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
    return x == -INFINITY ? 0.f : expz((double)x - lL);
}

// exp(x + y - lL) with an FP32 log x and FP64 logs y, lL: a root-edge term y
// can be thousands in magnitude, far beyond the FP32 spacing it would get
// folded into x
__device__ __forceinline__ float rel_exp2(float x, double y, double lL) {
    return (x == -INFINITY || y == -(double)INFINITY) ? 0.f : expz((double)x + y - lL);
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
    if (l > -(double)INFINITY) m = split_exp(l, e);
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
    const float E0v = lse3f(ev.l00 + cv.s0, ev.lm + cv.ld, ev.ls + cv.ss);
    const float E0w = lse3f(ew.l00 + cw.s0, ew.lm + cw.ld, ew.ls + cw.ss);
    const float kv = ev.ls + cv.ss, kw = ew.ls + cw.ss;
    // Outside rows in log mode are stored relative to XoA / XoB * ln 2 (the
    // children's out_x).  Below a root the offset is the parent's; at a root
    // the outside vector is the root edge (FP64 logs, thousands in magnitude
    // after a blow-up), so each child's inputs x = out[root] + E[sibling] are
    // formed in FP64 and offset by their own maximum: the class that carries
    // the likelihood keeps full FP32 precision.
    float xa0, xas, xb0, xbs;      // child v: x = out[u] + E[w]; child w: x = out[u] + E[v]
    double lmA = 0.0, lmB = 0.0;   // at a root: log Pmut - offset, per child
    int XoA, XoB;
    if (at_root) {
        const RootEdge re = root_edge_logs(b, s.tree);
        // each child's offset: the largest class of x + the child's own
        // inside vector -- the class that carries the site's likelihood --
        // so every posterior below is formed from values near 0.  (The
        // largest class of x alone can be one the child's data rule out,
        // e.g. silenced above an observed state in the exact model, and
        // lie a thousand nats above the likelihood after a blow-up.)
        float ta = -INFINITY, tb = -INFINITY;   // max_j log q_j + E[sibling]_j + in_j
        for (int j = 2; j < s.C; ++j) {
            const float lq = lgz(__ldg(s.qrow + j * G));
            const float av = child_val_log<G>(cv, j), aw = child_val_log<G>(cw, j);
            ta = fmaxf(ta, lq + laddexp(ew.lst + aw, kw) + av);
            tb = fmaxf(tb, lq + laddexp(ev.lst + av, kv) + aw);
        }
        auto offset = [](double a, double c, double e) {
            const double m = fmax(a, fmax(c, e));
            return m > -(double)INFINITY ? (int)floor(m / kLn2) + 1 : 0;
        };
        XoA = offset(re.l00 + (double)E0w + (double)cv.s0, re.ls + (double)cw.ss + (double)cv.ss,
                     re.lm + (double)ta);
        XoB = offset(re.l00 + (double)E0v + (double)cw.s0, re.ls + (double)cv.ss + (double)cw.ss,
                     re.lm + (double)tb);
        // x is summed in FP64: a root-edge term and its offset can each be
        // thousands while their sum is what carries the likelihood
        const double offA = XoA * kLn2, offB = XoB * kLn2;
        xa0 = (float)(re.l00 + (double)E0w - offA);
        xas = (float)(re.ls + (double)cw.ss - offA);
        xb0 = (float)(re.l00 + (double)E0v - offB);
        xbs = (float)(re.ls + (double)cv.ss - offB);
        lmA = re.lm - offA;
        lmB = re.lm - offB;
    } else {
        XoA = XoB = __ldcg(b.out_x + (int64_t)d.u_srow + s.site);
        const float o0 = __ldcg(urow), os = __ldcg(urow + G);
        xa0 = o0 + E0w;
        xas = os + cw.ss;
        xb0 = o0 + E0v;
        xbs = os + cv.ss;
    }
    float* arow = cv.row ? b.out_part + (int64_t)d.v_ref * 8 + s.goff + lane : nullptr;
    float* brow = cw.row ? b.out_part + (int64_t)d.w_ref * 8 + s.goff + lane : nullptr;
    Lse sa, sb, da, db;
    for (int j = 2; j < s.C; ++j) {
        const float lq = lgz(__ldg(s.qrow + j * G));
        const float oj = at_root ? 0.f : __ldcg(urow + j * G);
        const float av = child_val_log<G>(cv, j), aw = child_val_log<G>(cw, j);
        const float ea = laddexp(ew.lst + aw, kw), eb = laddexp(ev.lst + av, kv);
        const float xa = at_root ? (float)(lmA + (double)(lq + ea)) : oj + ea;
        const float xb = at_root ? (float)(lmB + (double)(lq + eb)) : oj + eb;
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
        __stcg(b.out_x + (int64_t)d.v_srow + s.site, XoA);
    }
    if (brow) {
        __stcg(brow, outb0);
        __stcg(brow + G, outbs);
        __stcg(b.out_h + (int64_t)d.w_srow + s.site, 0);
        __stcg(b.out_x + (int64_t)d.w_srow + s.site, XoB);
    }
    const double lL = __ldcg(b.llh_site + __ldg(b.tr_site_base + s.tree) + s.site);
    child_counts_log<G>(b, s, d.v, cv, ev, xa0, xas, lsa, da.value(), outa0, outas,
                        lL - XoA * kLn2, want_post, cv_);
    child_counts_log<G>(b, s, d.w, cw, ew, xb0, xbs, lsb, db.value(), outb0, outbs,
                        lL - XoB * kLn2, want_post, cw_);
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
    int Xo = 0;   // offset of node u's outside row (log mode: out_x in ln 2 units)
    Lse sx, dx;
    if (mode == 1) {
        const int u = __ldg(b.tr_quirk + s.tree);
        const ChildL cu = load_child_log<G>(b, false, (int)(__ldg(b.nd_prow + u) / 8),
                                            (int)__ldg(b.nd_srow + u), s, gc, L);
        const EdgeL eu = edge_logs(b, u, s.tree);
        const float* urow = b.out_part + __ldg(b.nd_prow + u) + s.goff + lane;
        Xo = __ldcg(b.out_x + __ldg(b.nd_srow + u) + s.site);
        x0 = __ldcg(urow) + lse3f(eu.l00 + cu.s0, eu.lm + cu.ld, eu.ls + cu.ss);
        xs = __ldcg(urow + G) + cu.ss;
        const float ku = eu.ls + cu.ss;
        for (int j = 2; j < s.C; ++j) {
            const float xj = __ldcg(urow + j * G) + laddexp(eu.lst + child_val_log<G>(cu, j), ku);
            sx.add(xj);
            dx.add(xj + child_val_log<G>(cv, j));
        }
    }
    const double lL = __ldcg(b.llh_site + __ldg(b.tr_site_base + s.tree) + s.site) - Xo * kLn2;
    c[0] = rel_exp2(x0 + cv.s0, re.l00, lL);
    c[1] = rel_exp2(x0 + cv.ld, re.lm, lL);
    c[2] = rel_exp2(x0 + cv.ss, re.ls, lL);
    c[3] = rel_exp2(dx.value(), re.lst, lL);
    c[4] = rel_exp2(cv.ss + sx.value(), re.ls, lL);
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
            x0 = __ldcg(urow) * fo * (edge0(bw, cw.s0, cw.D, cw.ss));
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

// State loops of the per-thread items, specialised on which children are
// leaves (a leaf's slots come from its code, an internal child's from its
// row).  Every pointer is __restrict__: the rows read (children's inside rows,
// the parent's outside row, priors) and the rows written are distinct, so the
// loads of later slots need not wait for the stores of earlier ones.
template <int G, bool LEAF>
__device__ __forceinline__ float slot_val(const float* __restrict__ row, float f, int code,
                                          float e1, float cst, int j) {
    if (LEAF) return code == j ? e1 : cst;
    return __ldcg(row + j * G) * f;
}

template <int G, bool VL, bool WL>
__device__ __forceinline__ void inside_states(const Child& cv, const Child& cw, const float4& bv,
                                              const float4& bw, const float* __restrict__ qrow,
                                              float* __restrict__ row, int C, float& dot,
                                              float& mx) {
    const float* __restrict__ rv = cv.row;
    const float* __restrict__ rw = cw.row;
    const float cstv = cv.code == -1 ? cv.ephi : 0.f, cstw = cw.code == -1 ? cw.ephi : 0.f;
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    // a leaf's factor b.z a_j + k takes two values (a_j = e1 at the leaf's
    // state, the constant elsewhere): formed once, selected per state
    const float fev = fmaf(bv.z, cv.e1, kv), fcv = fmaf(bv.z, cstv, kv);
    const float few = fmaf(bw.z, cw.e1, kw), fcw = fmaf(bw.z, cstw, kw);
    auto fac_v = [&](int jj, float a) { return VL ? (cv.code == jj ? fev : fcv) : fmaf(bv.z, a, kv); };
    auto fac_w = [&](int jj, float a) { return WL ? (cw.code == jj ? few : fcw) : fmaf(bw.z, a, kw); };
    int j = 2;
    for (; j + kChunk <= C; j += kChunk) {
        float av[kChunk], aw[kChunk], qv[kChunk];
#pragma unroll
        for (int k = 0; k < kChunk; ++k) {
            av[k] = VL ? 0.f : slot_val<G, VL>(rv, cv.f, cv.code, cv.e1, cstv, j + k);
            aw[k] = WL ? 0.f : slot_val<G, WL>(rw, cw.f, cw.code, cw.e1, cstw, j + k);
            qv[k] = __ldg(qrow + (j + k) * G);
        }
#pragma unroll
        for (int k = 0; k < kChunk; ++k) {
            const float x = fac_v(j + k, av[k]) * fac_w(j + k, aw[k]);
            __stcg(row + (j + k) * G, x);
            dot = fmaf(qv[k], x, dot);
            mx = fmaxf(mx, x);
        }
    }
    for (; j < C; ++j) {
        const float av = VL ? 0.f : slot_val<G, VL>(rv, cv.f, cv.code, cv.e1, cstv, j);
        const float aw = WL ? 0.f : slot_val<G, WL>(rw, cw.f, cw.code, cw.e1, cstw, j);
        const float x = fac_v(j, av) * fac_w(j, aw);
        __stcg(row + j * G, x);
        dot = fmaf(__ldg(qrow + j * G), x, dot);
        mx = fmaxf(mx, x);
    }
}

template <int G, bool VL, bool WL>
__device__ __forceinline__ void outside_states(const float* __restrict__ urow, float fo,
                                               const Child& cv, const Child& cw, const float4& bv,
                                               const float4& bw, const float* __restrict__ qrow,
                                               int C, ChildOut& A, ChildOut& B) {
    const float* __restrict__ rv = cv.row;
    const float* __restrict__ rw = cw.row;
    float* __restrict__ ra = A.orow;
    float* __restrict__ rb = B.orow;
    const float cstv = cv.code == -1 ? cv.ephi : 0.f, cstw = cw.code == -1 ? cw.ephi : 0.f;
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    const float pxa = bv.y * A.x0, pxb = bw.y * B.x0;
    float sa = 0.f, da = 0.f, ma = 0.f, sb = 0.f, db = 0.f, mb = 0.f;
    auto step = [&](float o, float av, float aw, float qj, int j) {
        const float xa = mulr(o, fmaf(bw.z, aw, kw));
        const float xb = mulr(o, fmaf(bv.z, av, kv));
        sa = addr(sa, xa);
        da = fmaf(xa, av, da);
        sb = addr(sb, xb);
        db = fmaf(xb, aw, db);
        if (!VL) {
            const float r = fmaf(pxa, qj, mulr(bv.z, xa));
            __stcg(ra + j * G, r);
            ma = fmaxf(ma, r);
        }
        if (!WL) {
            const float r = fmaf(pxb, qj, mulr(bw.z, xb));
            __stcg(rb + j * G, r);
            mb = fmaxf(mb, r);
        }
    };
    int j = 2;
    for (; j + kOChunk <= C; j += kOChunk) {
        float ou[kOChunk], av[kOChunk], aw[kOChunk], qv[kOChunk];
#pragma unroll
        for (int k = 0; k < kOChunk; ++k) {
            ou[k] = __ldcg(urow + (j + k) * G) * fo;
            av[k] = slot_val<G, VL>(rv, cv.f, cv.code, cv.e1, cstv, j + k);
            aw[k] = slot_val<G, WL>(rw, cw.f, cw.code, cw.e1, cstw, j + k);
            qv[k] = __ldg(qrow + (j + k) * G);
        }
#pragma unroll
        for (int k = 0; k < kOChunk; ++k) step(ou[k], av[k], aw[k], qv[k], j + k);
    }
    for (; j < C; ++j)
        step(__ldcg(urow + j * G) * fo, slot_val<G, VL>(rv, cv.f, cv.code, cv.e1, cstv, j),
             slot_val<G, WL>(rw, cw.f, cw.code, cw.e1, cstw, j), __ldg(qrow + j * G), j);
    A.sumx = sa; A.dot = da; A.mx = ma;
    B.sumx = sb; B.dot = db; B.mx = mb;
}

// ---------------------------------------------------------------------------
// Per-thread asynchronous staging of the inside state loop (wide levels).  Each
// thread copies its own coming slots of the rows it reads (cp.async, 4 bytes
// each, into its own column of shared memory: word w of thread t at
// sm[w * S + t], S = block size) kAsStages - 1 chunks of kAsChunk slots
// ahead of the chunk it computes, so the memory latency of a slot is paid
// once per item rather than once per chunk, without holding the data in
// flight in registers.  No thread reads another's column, so the only
// synchronisation is the thread's own cp.async.wait_group.
// ---------------------------------------------------------------------------
#ifndef LAML_AS_CHUNK
#define LAML_AS_CHUNK 4
#endif
#ifndef LAML_AS_STAGES
#define LAML_AS_STAGES 4
#endif
constexpr int kAsChunk = LAML_AS_CHUNK;
constexpr int kAsStages = LAML_AS_STAGES;
static_assert(kAsStages >= 2, "at least one chunk in flight");

__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n"
                 :: "r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" :: "n"(N) : "memory");
}

// the rows of slots j0 .. j0 + kAsChunk - 1 (those below C) into one stage
// of NR words per slot; row r is skipped when it is a leaf's (computed)
template <int G, int NR>
__device__ __forceinline__ void as_issue(float* st, int S, int j0, int C,
                                         const float* const (&rows)[NR], const bool (&live)[NR]) {
#pragma unroll
    for (int k = 0; k < kAsChunk; ++k) {
        const int j = j0 + k;
        if (j < C) {
#pragma unroll
            for (int r = 0; r < NR; ++r)
                if (live[r]) cp_async4(st + (k * NR + r) * S, rows[r] + j * G);
        }
    }
    cp_async_commit();   // every call commits a group, so wait counts stay uniform
}

template <int G, bool VL, bool WL>
__device__ __forceinline__ void inside_states_as(const Child& cv, const Child& cw,
                                                 const float4& bv, const float4& bw,
                                                 const float* __restrict__ qrow,
                                                 float* __restrict__ row, int C, float& dot,
                                                 float& mx, float* sm, int S) {
    constexpr int NR = 2, per = kAsChunk * NR;
    const float* const rows[NR] = {cv.row, cw.row};
    const bool live[NR] = {!VL, !WL};
    const float cstv = cv.code == -1 ? cv.ephi : 0.f, cstw = cw.code == -1 ? cw.ephi : 0.f;
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    const float fev = fmaf(bv.z, cv.e1, kv), fcv = fmaf(bv.z, cstv, kv);   // a leaf's two factors
    const float few = fmaf(bw.z, cw.e1, kw), fcw = fmaf(bw.z, cstw, kw);
    const int nch = (C - 2 + kAsChunk - 1) / kAsChunk;
#pragma unroll
    for (int c = 0; c < kAsStages - 1; ++c) {
        if (c < nch) as_issue<G, NR>(sm + (c % kAsStages) * per * S, S, 2 + c * kAsChunk, C, rows, live);
        else cp_async_commit();
    }
    for (int ch = 0; ch < nch; ++ch) {
        cp_async_wait<kAsStages - 2>();
        const float* st = sm + (ch % kAsStages) * per * S;
        const int j0 = 2 + ch * kAsChunk;
#pragma unroll
        for (int k = 0; k < kAsChunk; ++k) {
            const int j = j0 + k;
            if (j < C) {
                const float fv = VL ? (cv.code == j ? fev : fcv)
                                    : fmaf(bv.z, st[(k * NR) * S] * cv.f, kv);
                const float fw = WL ? (cw.code == j ? few : fcw)
                                    : fmaf(bw.z, st[(k * NR + 1) * S] * cw.f, kw);
                const float x = fv * fw;
                __stcg(row + j * G, x);
                dot = fmaf(__ldg(qrow + j * G), x, dot);
                mx = fmaxf(mx, x);
            }
        }
        const int nx = ch + kAsStages - 1;
        if (nx < nch) as_issue<G, NR>(sm + (nx % kAsStages) * per * S, S, 2 + nx * kAsChunk, C, rows, live);
        else cp_async_commit();
    }
}

// shared-memory words per thread of the wide-level item kernels: the inside
// item's staging ring, the outside item's stash (its state loop reads global
// memory directly: staging it doubled the load/store unit's work per element
// and measured slower)
template <int KIND>
constexpr int as_words() {
    return KIND == 1 ? kOStash : kAsStages * kAsChunk * 2;
}

template <int G, bool AS = false>
__device__ void inside_item_d(const laml_batch& b, const ItemDesc& d, int lane,
                              bool respect_status, float* sm = nullptr) {
    SiteCtx s;
    GroupCtx gc;
    if (!site_ctx_d<G>(b, d, lane, respect_status, s, gc)) return;
    if (lane == 0) {   // the children's rows into L2 while the first slots load
        const uint32_t bytes = (uint32_t)s.C * G * sizeof(float);
        if (!(d.flags & 1)) prefetch_l2(b.in_part + (int64_t)d.v_ref * 8 + s.goff, bytes);
        if (!(d.flags & 2)) prefetch_l2(b.in_part + (int64_t)d.w_ref * 8 + s.goff, bytes);
    }
    if (tree_log(b, s.tree)) {   // copies: the linear path's structs stay in registers
        const ItemDesc dl = d;
        const SiteCtx sl = s;
        const GroupCtx gl = gc;
        inside_log_item<G>(b, dl, sl, gl);
        return;
    }
    const Leaf L = leaf_params(b, s.tree);
    const Child cv = load_child_d<G>(b, d.flags & 1, d.v_ref, d.v_srow, s, gc, lane, L);
    const Child cw = load_child_d<G>(b, d.flags & 2, d.w_ref, d.w_srow, s, gc, lane, L);
    const float4 bv = load_bt(b, d.v), bw = load_bt(b, d.w);
    const float ev0 = edge0(bv, cv.s0, cv.D, cv.ss);
    const float ew0 = edge0(bw, cw.s0, cw.D, cw.ss);
    float* row = b.in_part + (int64_t)d.u_prow8 * 8 + s.goff + lane;
    const float s0 = ev0 * ew0, ss = cv.ss * cw.ss;
    __stcg(row, s0);
    __stcg(row + G, ss);
    float mx = fmaxf(s0, ss), dot = 0.f;
    if constexpr (AS) {
        float* tsm = sm + threadIdx.x;
        constexpr int S = kItemsBlock;   // k_items runs kItemsBlock threads a block
        switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {   // warp-uniform: items are sorted by it
            case 0: inside_states_as<G, false, false>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx, tsm, S); break;
            case 1: inside_states_as<G, true, false>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx, tsm, S); break;
            case 2: inside_states_as<G, false, true>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx, tsm, S); break;
            default: inside_states<G, true, true>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx); break;
        }
    } else {
        switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {   // warp-uniform: items are sorted by it
            case 0: inside_states<G, false, false>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx); break;
            case 1: inside_states<G, true, false>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx); break;
            case 2: inside_states<G, false, true>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx); break;
            default: inside_states<G, true, true>(cv, cw, bv, bw, s.qrow, row, s.C, dot, mx); break;
        }
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

template <int G, bool AS = false>
__device__ void outside_item_d(const laml_batch& b, const ItemDesc& d, int lane, bool act,
                               bool want_post, float* sm = nullptr) {
    float cv_[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cw_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    SiteCtx s;
    GroupCtx gc;
    const bool live = act && site_ctx_d<G>(b, d, lane, true, s, gc);
    // the descriptor and site fields the item needs after its state loop
    // wait in this thread's shared-memory column (AS), not in registers
    constexpr int S_ = kItemsBlock;
    float* sq_ = AS ? sm + threadIdx.x : nullptr;
    if constexpr (AS) {
        sq_[24 * S_] = __int_as_float(d.v); sq_[25 * S_] = __int_as_float(d.w);
        sq_[26 * S_] = __int_as_float(d.tree); sq_[27 * S_] = __int_as_float(d.g);
        sq_[28 * S_] = __int_as_float(d.flags); sq_[29 * S_] = __int_as_float(d.v_ref);
        sq_[30 * S_] = __int_as_float(d.w_ref); sq_[31 * S_] = __int_as_float(s.site);
        sq_[32 * S_] = __int_as_float(s.ds); sq_[33 * S_] = __int_as_float(s.goff);
    }
    if (live && lane == 0) {   // the parent's outside row and the children's rows into L2
        const uint32_t bytes = (uint32_t)s.C * G * sizeof(float);
        prefetch_l2(b.out_part + (int64_t)d.u_prow8 * 8 + s.goff, bytes);
        if (!(d.flags & 1)) prefetch_l2(b.in_part + (int64_t)d.v_ref * 8 + s.goff, bytes);
        if (!(d.flags & 2)) prefetch_l2(b.in_part + (int64_t)d.w_ref * 8 + s.goff, bytes);
    }
    if (live && tree_log(b, s.tree)) {   // copies: the linear path's structs stay in registers
        float tv[8], tw[8];
        const ItemDesc dl = d;
        const SiteCtx sl = s;
        const GroupCtx gl = gc;
        outside_log_lane<G>(b, dl, sl, gl, want_post, tv, tw);
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
        const float ev0 = edge0(bv, cv.s0, cv.D, cv.ss);
        const float ew0 = edge0(bw, cw.s0, cw.D, cw.ss);
        ChildOut A, B;   // A: child v (uses E[w]), B: child w (uses E[v])
        A.x0 = o0 * ew0; A.xs = os * cw.ss; A.X = Xo + cw.X;
        B.x0 = o0 * ev0; B.xs = os * cv.ss; B.X = Xo + cv.X;
        A.sumx = A.dot = A.mx = 0.f;
        B.sumx = B.dot = B.mx = 0.f;
        A.orow = cv.row ? b.out_part + (int64_t)d.v_ref * 8 + s.goff + lane : nullptr;
        B.orow = cw.row ? b.out_part + (int64_t)d.w_ref * 8 + s.goff + lane : nullptr;
        if constexpr (AS) {
            // what child_finish needs after the state loop waits in this
            // thread's shared-memory column, read back through volatile loads,
            // so it does not stay live in registers across the loop (which
            // otherwise spills at this kernel's 80-register budget)
            constexpr int S = kItemsBlock;   // k_items runs kItemsBlock threads a block
            float* sp = sm + threadIdx.x;
            sp[0 * S] = cv.s0; sp[1 * S] = cv.ss; sp[2 * S] = cv.D;
            sp[3 * S] = __int_as_float(cv.X); sp[4 * S] = __int_as_float(cv.code);
            sp[5 * S] = cw.s0; sp[6 * S] = cw.ss; sp[7 * S] = cw.D;
            sp[8 * S] = __int_as_float(cw.X); sp[9 * S] = __int_as_float(cw.code);
            sp[10 * S] = bv.x; sp[11 * S] = bv.y; sp[12 * S] = bv.w;
            sp[13 * S] = bw.x; sp[14 * S] = bw.y; sp[15 * S] = bw.w;
            sp[16 * S] = A.x0; sp[17 * S] = A.xs; sp[18 * S] = __int_as_float(A.X);
            sp[19 * S] = B.x0; sp[20 * S] = B.xs; sp[21 * S] = __int_as_float(B.X);
            sp[22 * S] = bv.z; sp[23 * S] = bw.z;
            switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {   // warp-uniform: items are sorted by it
                case 0: outside_states<G, false, false>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
                case 1: outside_states<G, true, false>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
                case 2: outside_states<G, false, true>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
                default: outside_states<G, true, true>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
            }
            const volatile float* vp = sp;
            const int dflags = __float_as_int(vp[28 * S]);
            Child cv2, cw2;   // child_finish reads row only as "leaf or not"
            cv2.s0 = vp[0 * S]; cv2.ss = vp[1 * S]; cv2.D = vp[2 * S];
            cv2.X = __float_as_int(vp[3 * S]); cv2.code = __float_as_int(vp[4 * S]);
            cv2.row = (dflags & 1) ? nullptr : b.in_part;
            cw2.s0 = vp[5 * S]; cw2.ss = vp[6 * S]; cw2.D = vp[7 * S];
            cw2.X = __float_as_int(vp[8 * S]); cw2.code = __float_as_int(vp[9 * S]);
            cw2.row = (dflags & 2) ? nullptr : b.in_part;
            const float4 bv2 = make_float4(vp[10 * S], vp[11 * S], vp[22 * S], vp[12 * S]);
            const float4 bw2 = make_float4(vp[13 * S], vp[14 * S], vp[23 * S], vp[15 * S]);
            A.x0 = vp[16 * S]; A.xs = vp[17 * S]; A.X = __float_as_int(vp[18 * S]);
            B.x0 = vp[19 * S]; B.xs = vp[20 * S]; B.X = __float_as_int(vp[21 * S]);
            const int dv = __float_as_int(vp[24 * S]), dw = __float_as_int(vp[25 * S]);
            SiteCtx s2;   // child_finish reads the site, its tree and dataset
            s2.tree = __float_as_int(vp[26 * S]);
            s2.site = __float_as_int(vp[31 * S]);
            s2.ds = __float_as_int(vp[32 * S]);
            const int64_t ro = (int64_t)__float_as_int(vp[33 * S]) + lane;   // group offset + lane
            A.orow = (dflags & 1) ? nullptr
                                  : b.out_part + (int64_t)__float_as_int(vp[29 * S]) * 8 + ro;
            B.orow = (dflags & 2) ? nullptr
                                  : b.out_part + (int64_t)__float_as_int(vp[30 * S]) * 8 + ro;
            const int64_t t = __ldg(b.tr_site_base + s2.tree) + s2.site;
            const float lroot = __ldcg(b.root_lr + t);
            const int xroot = __ldcg(b.root_x + t);
            child_finish<G>(b, s2, dv, cv2, bv2, A, want_post, lroot, xroot, cv_);
            child_finish<G>(b, s2, dw, cw2, bw2, B, want_post, lroot, xroot, cw_);
        } else {
            const int64_t t = __ldg(b.tr_site_base + s.tree) + s.site;
            switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {   // warp-uniform: items are sorted by it
                case 0: outside_states<G, false, false>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
                case 1: outside_states<G, true, false>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
                case 2: outside_states<G, false, true>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
                default: outside_states<G, true, true>(urow, fo, cv, cw, bv, bw, s.qrow, s.C, A, B); break;
            }
            const float lroot = __ldcg(b.root_lr + t);
            const int xroot = __ldcg(b.root_x + t);
            child_finish<G>(b, s, d.v, cv, bv, A, want_post, lroot, xroot, cv_);
            child_finish<G>(b, s, d.w, cw, bw, B, want_post, lroot, xroot, cw_);
        }
    }
    if constexpr (AS) {
        const volatile float* vq = sq_;
        const int tr = __float_as_int(vq[26 * S_]), g = __float_as_int(vq[27 * S_]);
        scatter_counts<G>(b, tr, __float_as_int(vq[24 * S_]), __float_as_int(vq[25 * S_]), g,
                          lane, act, cv_, cw_);
    } else {
        scatter_counts<G>(b, d.tree, d.v, d.w, d.g, lane, act, cv_, cw_);
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
    if (live && tree_log(b, s.tree)) {   // copies: the linear path's structs stay in registers
        float tv[8], tw[8];
        const ItemDesc dl = d;
        const SiteCtx sl = s;
        const GroupCtx gl = gc;
        outside_log_lane<G>(b, dl, sl, gl, want_post, tv, tw);
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
        const float ev0 = edge0(bv, cv.s0, cv.D, cv.ss);
        const float ew0 = edge0(bw, cw.s0, cw.D, cw.ss);
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
            A.sumx = addr(A.sumx, xa);
            A.dot = fmaf(xa, av, A.dot);
            B.sumx = addr(B.sumx, xb);
            B.dot = fmaf(xb, aw, B.dot);
            if (A.orow) {
                const float r = fmaf(pxa, qj, mulr(bv.z, xa));
                __stcg(A.orow + j * G, r);
                A.mx = fmaxf(A.mx, r);
            }
            if (B.orow) {
                const float r = fmaf(pxb, qj, mulr(bw.z, xb));
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
        __stcg(b.post0 + pb, rel_exp2(cr.s0, re.l00, lL));
        __stcg(b.post1 + pb, rel_exp2(cr.ss, re.ls, lL));
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

// block-wide max of an int
__device__ __forceinline__ int block_maxi(int x, double2* shd) {
    int* sh = reinterpret_cast<int*>(shd);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x = max(x, __shfl_xor_sync(kFull, x, off));
    const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
    __syncthreads();
    if (ln == 0) sh[wid] = x;
    __syncthreads();
    int r = sh[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) r = max(r, sh[k]);
    return r;
}

// block-wide min of a double
__device__ __forceinline__ double block_mind(double x, double2* sh) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x = fmin(x, __shfl_xor_sync(kFull, x, off));
    const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
    __syncthreads();
    if (ln == 0) sh[wid].x = x;
    __syncthreads();
    double r = sh[0].x;
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) r = fmin(r, sh[k].x);
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
// The thread teams an M-step runs on: one block (trees up to kClusterNodes
// nodes), or a cluster of kMstepCluster blocks of 1024 threads whose
// reductions go through distributed shared memory (larger trees).  Either
// way every thread owns the branches v = tid, tid + size, ... in every phase,
// so the only data threads exchange are the reductions, which are summed in
// a fixed order (warp, then block, then cluster rank).
struct BlockTeam {
    double2* sh;
    __device__ int tid() const { return threadIdx.x; }
    __device__ int size() const { return blockDim.x; }
    __device__ bool leader() const { return threadIdx.x == 0; }
    __device__ void sync() const { __syncthreads(); }
    __device__ float2 sum2f(float a, float c) const { return block_sum2f(a, c, sh); }
    __device__ double2 sum2(double a, double c) const { return block_sum2(a, c, sh); }
    __device__ int maxi(int x) const { return block_maxi(x, sh); }
    __device__ double mind(double x) const { return block_mind(x, sh); }
};

constexpr int kMstepCluster = 8;        // blocks per cluster (the portable size)
constexpr int kMstepClusterThreads = 1024;
constexpr int kClusterNodes = 16384;    // trees above this many nodes take a cluster

struct ClusterTeam {
    double2* sh;      // this block's warp partials
    double2* part;    // [kMstepCluster] block partials, read from the rank-0 block
    __device__ int rank() const { return (int)cooperative_groups::this_cluster().block_rank(); }
    __device__ int tid() const { return rank() * (int)blockDim.x + (int)threadIdx.x; }
    __device__ int size() const { return kMstepCluster * (int)blockDim.x; }
    __device__ bool leader() const { return threadIdx.x == 0 && rank() == 0; }
    __device__ void sync() const { cooperative_groups::this_cluster().sync(); }
    __device__ double2 gather(double2 mine) const {
        auto cl = cooperative_groups::this_cluster();
        double2* p0 = cl.map_shared_rank(part, 0);
        if (threadIdx.x == 0) p0[cl.block_rank()] = mine;
        cl.sync();
        double2 r = make_double2(0.0, 0.0);
        for (int k = 0; k < kMstepCluster; ++k) {
            const double2 x = p0[k];
            r.x += x.x;
            r.y += x.y;
        }
        cl.sync();   // every rank has read before the slots are written again
        return r;
    }
    __device__ float2 sum2f(float a, float c) const {
        const float2 m = block_sum2f(a, c, sh);
        const double2 r = gather(make_double2((double)m.x, (double)m.y));
        return make_float2((float)r.x, (float)r.y);
    }
    __device__ double2 sum2(double a, double c) const { return gather(block_sum2(a, c, sh)); }
    __device__ int maxi(int x) const {
        auto cl = cooperative_groups::this_cluster();
        const int m = block_maxi(x, sh);
        double2* p0 = cl.map_shared_rank(part, 0);
        if (threadIdx.x == 0) p0[cl.block_rank()] = make_double2((double)m, 0.0);
        cl.sync();
        int r = 0;
        for (int k = 0; k < kMstepCluster; ++k) r = max(r, (int)p0[k].x);
        cl.sync();
        return r;
    }
    __device__ double mind(double x) const {
        auto cl = cooperative_groups::this_cluster();
        const double m = block_mind(x, sh);
        double2* p0 = cl.map_shared_rank(part, 0);
        if (threadIdx.x == 0) p0[cl.block_rank()] = make_double2(m, 0.0);
        cl.sync();
        double r = p0[0].x;
        for (int k = 1; k < kMstepCluster; ++k) r = fmin(r, p0[k].x);
        cl.sync();
        return r;
    }
};

// ---------------------------------------------------------------------------
// Ultrametric branch lengths (EM_solver.Mstep with ultra_constr_cache,
// EM_solver.py:349-366, under the equalities of ultrametric_constr, 53-89).
// Given nu, maximise over the optimised branches
//   sum_v f_v(d_v),  f_v(d) = -a_v d + b_v log(1 - e^{-d}) + c_v log(1 - e^{-nu d})
// with d in [dmin, dmax] and every root-to-leaf path of the tree equally
// long.  The solve works on node heights P (the path length from a node down
// to its leaves, 0 at a leaf): d_x = P_parent(x) - P_x for every non-root x,
// so the equalities hold by construction; a fixed branch (mask 0) ties
// P_x = P_parent - d_x, as the reference's node.constant does, and a node
// tied to a leaf through fixed branches is pinned (its height is a
// constant).  The root's own branch is in no equality of a single tree and
// is solved alone.
//
// Method: a primal-dual interior point (Mehrotra predictor-corrector,
// section 4a below) on the bounds; if it has not converged in kPdMax
// iterations, a log-barrier interior point continues from its point.  Both
// solve, per iteration, the Newton system of the heights: a weighted tree
// Laplacian (edge weight W_x),
// solved exactly by eliminating nodes from the deepest level up and
// substituting back down, one depth level (nd_uorder) per team sync; a
// node's reduced diagonal is kept as the sum of positive terms
// W_c E_c / (W_c + E_c), which loses nothing to cancellation however large
// the weights grow.  In the barrier phase a backtracking line search tests
// the barrier objective's change summed branch by branch from log1p/expm1
// differences, so no difference of large totals is taken.  Heights, branch
// lengths, the elimination and every sum are FP64; in the barrier phase the
// transcendental and reciprocal cores (expm1, log1p, 1/x of values formed in
// FP64) run in FP32, since
// GB300's FP64 pipe is narrow and each enters only a gradient, a weight or a
// line-search term at FP32 relative precision (the solution moves by ~1e-7
// relative).  Centring ends when lambda^2 / 2 < 1e-6 or, in the quadratic
// phase, when lambda^2 stops falling (the rounding floor of large t).
// Returns false when the constraints admit no branch lengths (an empty
// height interval at some node).
// ---------------------------------------------------------------------------
namespace ultra {
// per-node FP64 slots of nd_uwork (LAML_UWORK_SLOTS per node)
constexpr int kP = 0;     // height (the warm start during the interval pass)
constexpr int kW = 1;     // weight of the node's own branch (lo during the interval pass)
constexpr int kG = 2;     // barrier-objective slope of that branch (hi during the interval pass)
constexpr int kE = 3;     // reduced diagonal excess of the node's subtree
constexpr int kR = 4;     // reduced right-hand side
constexpr int kDel = 5;   // Newton step of the height
constexpr int kPin = 6;   // 1: height fixed (leaves, nodes tied to a leaf by fixed branches)
constexpr int kRaw = 7;   // gradient of the barrier objective in the height (during the
                          // interval pass: 1 when the path down child1 is all fixed)
constexpr int kA = 8, kB = 9, kC = 10;   // objective coefficients of the node's branch
constexpr int kIE = 11, kIEN = 12;       // 1 / expm1(d), 1 / expm1(nu d) at the current d
constexpr int kRL = 13, kRH = 14;        // 1 / (d - dmin), 1 / (dmax - d)
constexpr int kStat = 15;   // root: Newton steps of the last solve; node 0: line-search passes
constexpr int kBak = 16;    // the primal-dual phase's last heights with every slack positive
constexpr int kSlots = LAML_UWORK_SLOTS;
static_assert(kSlots >= 17, "nd_uwork slots");
constexpr double kTheta = 0.1;        // pull of the start point toward its interval's middle
constexpr double kMu = 20.0;          // barrier weight growth per centring
constexpr double kGapRel = 1e-10;     // objective suboptimality m / t, relative
constexpr double kNewtonTol = 1e-6;   // centred when lambda^2 / 2 is below this
constexpr int kOuterMax = 30, kNewtonMax = 60, kLineMax = 60;
// primal-dual phase (slots 11..14 hold z_lo, z_hi, the predictor's branch
// step and f'(d) while it runs; the barrier phase reuses them)
constexpr int kZL = 11, kZH = 12, kAD = 13, kF1 = 14;
constexpr int kPdMax = 60;            // iterations before the barrier phase takes over
constexpr int kPdShort = 3;           // the same with LAML_MSTEP_ULTRA_PD_SHORT
constexpr double kPdMu = 1e-13;       // mean complementarity, relative to 1 + max a
constexpr double kPdMove = 1e-9;      // largest branch move of the last step, relative to 1 + d
constexpr double kPdFloor = 1e-14;    // smallest slack to a bound, relative to 1 + d

__device__ __forceinline__ double rcp32(double x) { return (double)(1.f / (float)x); }
// 1 / x for a positive normal x to ~1e-14: an FP32 seed of the mantissa (the
// binary exponent split off, so no range is lost) and one FP64 Newton step.
// The level passes of the elimination divide on their critical path, where
// GB300's narrow FP64 pipe makes a full FP64 division a long dependent chain.
__device__ __forceinline__ double rcp64(double x) {
    int e;
    const double m = frexp(x, &e);   // x = m 2^e, m in [0.5, 1)
    double r = (double)(1.f / (float)m);
    r = r * fma(-m, r, 2.0);
    return ldexp(r, -e);
}
__device__ __forceinline__ double log1p32(double x) { return (double)log1pf((float)x); }
__device__ __forceinline__ double expm132(double x) { return (double)expm1f((float)x); }
__device__ __forceinline__ double log1mexp32(double x) {   // log(1 - e^{-x}), x > 0
    return (double)logf(-expm1f(-(float)x));
}
}  // namespace ultra

// SH: the eight slots threads exchange (kP .. kRaw) live slot-major in
// shared memory (hot[k * N + v]); the per-branch terms only their owner
// thread touches stay in nd_uwork.  Each level of the elimination is a chain
// of dependent loads of these slots, which shared memory serves in tens of
// cycles instead of a round trip to L2.
// Returns kUltraOk, kUltraInfeasible (the constraints admit no lengths in
// [dmin, dmax]) or kUltraNaN (a height is not finite: nothing is written).
// pd_iters: iterations of the primal-dual phase (0: the barrier phase alone).
constexpr int kUltraOk = 0, kUltraInfeasible = 1, kUltraNaN = 2;
template <class Team, bool SH>
__device__ __noinline__ int ultra_dstep(const laml_batch& b, int p, Team& T, double nu,
                                        bool use_s, float* Dd, double* hot, int pd_iters) {
    using namespace ultra;
    const int N = __ldg(b.tr_nodes + p), base = __ldg(b.tr_node_base + p);
    const int root = __ldg(b.tr_root + p) - base;
    const int32_t* ord = b.nd_uorder + 2 * (int64_t)base + 2 * (int64_t)p;
    const int L = __ldg(ord);
    const int32_t* off = ord + 1;
    const int32_t* ids = ord + L + 2;
    double* U = b.nd_uwork + (int64_t)kSlots * base;
    const double dlo = kDmin, dhi = kDmax;
    auto at = [&](int v, int k) -> double& {
        if (SH && k <= kRaw) return hot[(int64_t)k * N + v];
        return U[(int64_t)kSlots * v + k];
    };
    auto leaf = [&](int v) { return __ldg(b.nd_c0 + base + v) < 0; };
    auto c0_ = [&](int v) { return __ldg(b.nd_c0 + base + v) - base; };
    auto c1_ = [&](int v) { return __ldg(b.nd_c1 + base + v) - base; };
    auto par = [&](int v) { return __ldg(b.nd_parent + base + v) - base; };
    auto freeb = [&](int v) { return __ldg(b.nd_mask + base + v) != 0; };
    auto dold = [&](int v) { return __ldcg(b.nd_d + base + v); };
    // a free branch between two pinned heights is as good as fixed
    auto active = [&](int x) {
        return x != root && freeb(x) && !(at(x, kPin) != 0.0 && at(par(x), kPin) != 0.0);
    };

    // 1. leaves, the branches' coefficients; then height intervals [lo, hi]
    //    bottom-up, with the warm start (the mean over the children used of
    //    d_c + P_c at the current d)
    for (int v = T.tid(); v < N; v += T.size()) {
        const double* q = b.nd_cnt + (int64_t)(base + v) * 6;
        const double q0 = __ldcg(q), q1 = __ldcg(q + 1), q3 = __ldcg(q + 3);
        at(v, kA) = q0 + nu * (q0 + q1 + q3);
        at(v, kB) = q1;
        at(v, kC) = use_s ? __ldcg(q + 2) + __ldcg(q + 4) : 0.0;
        if (!leaf(v)) continue;
        at(v, kP) = 0.0; at(v, kW) = 0.0; at(v, kG) = 0.0; at(v, kE) = 0.0;
        at(v, kR) = 0.0; at(v, kDel) = 0.0; at(v, kPin) = 1.0; at(v, kRaw) = 1.0;
    }
    T.sync();
    int bad = 0;
    for (int l = L - 1; l >= 0; --l) {
        for (int k = __ldg(off + l) + T.tid(); k < __ldg(off + l + 1); k += T.size()) {
            const int u = __ldg(ids + k);
            if (leaf(u)) continue;
            double lo = -INFINITY, hi = INFINITY, pinv = NAN, warm = 0.0;
            const int cs[2] = {c0_(u), c1_(u)};
            // a child's path (its branch, then first children down to a leaf;
            // treeswift's first child is child1 here) that holds no free
            // branch is a constant; ultrametric_constr keeps no row between
            // two constants (EM_solver.py:70-72), and the node's own path
            // continues down child1 (EM_solver.py:73)
            const bool cp0 = !freeb(cs[0]) && at(cs[0], kRaw) != 0.0;
            const bool cp1 = !freeb(cs[1]) && at(cs[1], kRaw) != 0.0;
            const int first = (cp0 && cp1) ? 1 : 0;
            for (int i = first; i < 2; ++i) {
                const int c = cs[i];
                const double lc = at(c, kW), hc = at(c, kG);
                if (freeb(c)) {
                    lo = fmax(lo, lc + dlo);
                    hi = fmin(hi, hc + dhi);
                } else {
                    const double df = dold(c);
                    lo = fmax(lo, lc + df);
                    hi = fmin(hi, hc + df);
                    if (at(c, kPin) != 0.0) pinv = lc + df;
                }
                warm += (dold(c) + at(c, kP)) / (double)(2 - first);
            }
            const double tol = 1e-9 * fmax(1.0, fabs(hi));
            bool pin = !isnan(pinv);
            if (pin) {   // every other constraint must admit the pinned height
                if (pinv < lo - tol || pinv > hi + tol) bad = 1;
                lo = hi = pinv;
            } else if (lo > hi + tol) {
                bad = 1;
            } else if (!(hi - lo > 1e-12 * fmax(1.0, fabs(hi)))) {
                pin = true;   // a single admissible height
                lo = hi = 0.5 * (lo + hi);
            }
            at(u, kW) = lo;
            at(u, kG) = hi;
            at(u, kPin) = pin ? 1.0 : 0.0;
            at(u, kP) = warm;
            at(u, kDel) = 0.0;
            at(u, kRaw) = cp1 ? 1.0 : 0.0;
        }
        T.sync();
    }
    if (T.maxi(bad)) return kUltraInfeasible;

    // 2. strictly feasible start, top-down: each height the warm start
    //    clamped to what its parent's height leaves, pulled kTheta toward the
    //    middle of that range
    for (int l = 0; l < L; ++l) {
        for (int k = __ldg(off + l) + T.tid(); k < __ldg(off + l + 1); k += T.size()) {
            const int x = __ldg(ids + k);
            if (leaf(x)) continue;
            double lo = at(x, kW), hi = at(x, kG), P;
            if (at(x, kPin) != 0.0) {
                P = lo;
            } else if (x != root && !freeb(x)) {
                P = at(par(x), kP) - dold(x);
            } else {
                if (x != root) {
                    const double Pu = at(par(x), kP);
                    lo = fmax(lo, Pu - dhi);
                    hi = fmin(hi, Pu - dlo);
                }
                const double w = fmin(fmax(at(x, kP), lo), hi);
                P = (1.0 - kTheta) * w + kTheta * 0.5 * (lo + hi);
            }
            at(x, kP) = P;
        }
        T.sync();
    }

    // 3. barrier objective scale: m (bound constraints) and |F| at the start
    double m_loc = 0.0, F_loc = 0.0;
    for (int x = T.tid(); x < N; x += T.size()) {
        if (!active(x)) continue;
        const double a = at(x, kA), bb = at(x, kB), c = at(x, kC);
        const double d = at(par(x), kP) - at(x, kP);
        F_loc += -a * d + (bb > 0.0 ? bb * log1mexp32(d) : 0.0) +
                 (c > 0.0 ? c * log1mexp32(nu * d) : 0.0);
        m_loc += 2.0;
    }
    const double2 mF = T.sum2(m_loc, F_loc);
    const double m = mF.x;
    const double gap_tol = kGapRel * (fabs(mF.y) + 1.0);
    double t = 1.0;
    int n_newton = 0, n_line = 0;

    // the tree system's elimination, deepest level first, and substitution,
    // root first (the latter returns this thread's share of gradient . step)
    auto eliminate = [&]() {
        for (int l = L - 1; l >= 0; --l) {
            for (int k = __ldg(off + l) + T.tid(); k < __ldg(off + l + 1); k += T.size()) {
                const int u = __ldg(ids + k);
                if (leaf(u)) continue;
                const int cs[2] = {c0_(u), c1_(u)};
                double raw = at(cs[0], kG) + at(cs[1], kG) - (u == root ? 0.0 : at(u, kG));
                at(u, kRaw) = raw;
                if (at(u, kPin) != 0.0) {
                    at(u, kE) = 0.0;
                    at(u, kR) = 0.0;
                    continue;
                }
                double E = 0.0, R = raw;
                for (int i = 0; i < 2; ++i) {
                    const int c = cs[i];
                    const double Wc = at(c, kW);
                    if (at(c, kPin) != 0.0) {
                        E += Wc;
                    } else if (freeb(c)) {
                        const double Ec = at(c, kE), iD = rcp64(Wc + Ec);
                        E += Wc * (Ec * iD);
                        R += Wc * (at(c, kR) * iD);
                    } else {   // fixed branch: the child's height moves with this one
                        E += at(c, kE);
                        R += at(c, kR);
                    }
                }
                at(u, kE) = E;
                at(u, kR) = R;
            }
            T.sync();
        }
    };
    auto substitute = [&]() -> double {
        double lam = 0.0;
        for (int l = 0; l < L; ++l) {
            for (int k = __ldg(off + l) + T.tid(); k < __ldg(off + l + 1); k += T.size()) {
                const int x = __ldg(ids + k);
                if (leaf(x)) continue;
                double del;
                if (at(x, kPin) != 0.0) {
                    del = 0.0;
                } else if (x == root) {
                    const double E = at(x, kE);
                    del = E > 0.0 ? at(x, kR) * rcp64(E) : 0.0;
                } else if (!freeb(x)) {
                    del = at(par(x), kDel);
                } else {
                    const double W = at(x, kW);
                    del = (at(x, kR) + W * at(par(x), kDel)) * rcp64(W + at(x, kE));
                }
                at(x, kDel) = del;
                lam += at(x, kRaw) * del;
            }
            T.sync();
        }
        return lam;
    };

    // 4a. primal-dual interior point (Mehrotra predictor-corrector) on the
    //     same tree system: duals z_lo, z_hi of every active branch's
    //     bounds; each iteration solves the system twice (predictor with
    //     complementarity target 0, corrector with sigma mu and the
    //     predictor's second-order term) and steps 99% of the way to the
    //     nearest bound.  FP64 throughout: it takes ~16 passes of
    //     transcendentals where the barrier phase takes hundreds.  Done when
    //     the mean complementarity is below kPdMu (1 + max a) and the last
    //     step moved no branch by more than kPdMove (1 + d); otherwise the
    //     barrier phase below continues from the point reached.
    bool pd_done = !(m > 0.0);
    if (!pd_done && pd_iters > 0) {
        auto derivs = [&](int x, double d, double& g, double& h) {
            const double a = at(x, kA), bb = at(x, kB), c = at(x, kC);
            g = -a;
            h = 0.0;
            if (bb > 0.0) {
                const double e = expm1(d);
                g += bb / e;
                h -= bb * (e + 1.0) / (e * e);
            }
            if (c > 0.0) {
                const double e = expm1(nu * d);
                g += c * nu / e;
                h -= c * nu * nu * (e + 1.0) / (e * e);
            }
        };
        auto bdist = [&](int x, double& d, double& slo, double& shi) {
            d = at(par(x), kP) - at(x, kP);
            slo = d - dlo;
            shi = dhi - d;
        };
        // starting duals: z = mu0 / s, mu0 the mean |f'| times the distance
        // to the nearer bound
        double s_loc = 0.0, na = 0.0;
        for (int x = T.tid(); x < N; x += T.size()) {
            if (!active(x)) continue;
            double d, slo, shi, g, h;
            bdist(x, d, slo, shi);
            derivs(x, d, g, h);
            s_loc += fabs(g) * fmin(slo, shi);
            na = fmax(na, at(x, kA));
        }
        const double mu0 = fmax(1e-8, T.sum2(s_loc, 0.0).x / (0.5 * m));
        const double scale = 1.0 - T.mind(-na);
        for (int x = T.tid(); x < N; x += T.size()) {
            if (!active(x)) continue;
            double d, slo, shi;
            bdist(x, d, slo, shi);
            at(x, kZL) = mu0 / slo;
            at(x, kZH) = mu0 / shi;
        }
        T.sync();
        double move = INFINITY;
        for (int it = 0; it < pd_iters; ++it) {
            // (i) f', the weights -f'' + z_lo/s_lo + z_hi/s_hi, the
            //     predictor's right-hand sides f', and mu.  The heights of a
            //     branch move separately, so its length can round onto or
            //     past a bound although the step stopped 99% of the way
            //     there: then the phase ends at the heights of the previous
            //     iteration (kBak, every slack positive there) and the
            //     barrier phase continues from them
            double mu_loc = 0.0, smin = INFINITY;
            int lost = 0;
            for (int x = T.tid(); x < N; x += T.size()) {
                if (x == root) continue;
                if (!active(x)) {
                    at(x, kW) = 0.0;
                    at(x, kG) = 0.0;
                    continue;
                }
                double d, slo, shi, g, h;
                bdist(x, d, slo, shi);
                if (!(slo > 0.0 && shi > 0.0)) {   // also NaN
                    lost = 1;
                    continue;
                }
                smin = fmin(smin, fmin(slo, shi) / (1.0 + d));
                derivs(x, d, g, h);
                const double zl = at(x, kZL), zh = at(x, kZH);
                at(x, kF1) = g;
                at(x, kW) = -h + zl / slo + zh / shi;
                at(x, kG) = g;
                mu_loc += zl * slo + zh * shi;
            }
            if (T.maxi(lost)) {   // it > 0: the start point is strictly feasible
                for (int x = T.tid(); x < N; x += T.size())
                    if (!leaf(x) && at(x, kPin) == 0.0) at(x, kP) = at(x, kBak);
                T.sync();
                break;
            }
            const double mu = T.sum2(mu_loc, 0.0).x / m;   // also orders the writes
            smin = T.mind(smin);
            ++n_newton;
            // done: complementarity small and either nothing moves any more
            // or a branch sits at its bound to the heights' rounding (its
            // slack would next round to zero)
            if (it > 0 && mu < kPdMu * scale && (move < kPdMove || smin < kPdFloor)) {
                pd_done = true;
                break;
            }
            if (!isfinite(mu)) break;   // not expected; the barrier phase takes over
            // (ii) predictor: solve, keep each branch's step, longest steps
            eliminate();
            substitute();
            auto zsteps = [&](int x, double dd, double slo, double shi, double tlo, double thi,
                              double& dzl, double& dzh) {
                const double zl = at(x, kZL), zh = at(x, kZH);
                dzl = (tlo - zl * slo - zl * dd) / slo;
                dzh = (thi - zh * shi + zh * dd) / shi;
            };
            auto limits = [&](int x, double dd, double slo, double shi, double dzl, double dzh,
                              double& ap, double& ad) {
                if (dd < 0.0) ap = fmin(ap, slo / -dd);
                if (dd > 0.0) ap = fmin(ap, shi / dd);
                if (dzl < 0.0) ad = fmin(ad, at(x, kZL) / -dzl);
                if (dzh < 0.0) ad = fmin(ad, at(x, kZH) / -dzh);
            };
            double ap = INFINITY, ad = INFINITY;
            for (int x = T.tid(); x < N; x += T.size()) {
                if (!active(x)) continue;
                double d, slo, shi, dzl, dzh;
                bdist(x, d, slo, shi);
                const double dd = at(par(x), kDel) - at(x, kDel);
                at(x, kAD) = dd;
                zsteps(x, dd, slo, shi, 0.0, 0.0, dzl, dzh);
                limits(x, dd, slo, shi, dzl, dzh, ap, ad);
            }
            ap = fmin(1.0, T.mind(ap));
            ad = fmin(1.0, T.mind(ad));
            // (iii) mu after the predictor's step; sigma = (mu_aff / mu)^3
            double maff = 0.0;
            for (int x = T.tid(); x < N; x += T.size()) {
                if (!active(x)) continue;
                double d, slo, shi, dzl, dzh;
                bdist(x, d, slo, shi);
                const double dd = at(x, kAD);
                zsteps(x, dd, slo, shi, 0.0, 0.0, dzl, dzh);
                maff += (at(x, kZL) + ad * dzl) * (slo + ap * dd) +
                        (at(x, kZH) + ad * dzh) * (shi - ap * dd);
            }
            maff = T.sum2(maff, 0.0).x / m;
            const double r = maff / mu, sigma = fmin(1.0, r * r * r);
            // (iv) corrector: complementarity targets sigma mu less the
            //      predictor's second-order term
            auto targets = [&](int x, double slo, double shi, double& tlo, double& thi) {
                const double dd = at(x, kAD);
                double dzl, dzh;
                zsteps(x, dd, slo, shi, 0.0, 0.0, dzl, dzh);
                tlo = sigma * mu - dd * dzl;
                thi = sigma * mu + dd * dzh;
            };
            for (int x = T.tid(); x < N; x += T.size()) {
                if (!active(x)) continue;
                double d, slo, shi, tlo, thi;
                bdist(x, d, slo, shi);
                targets(x, slo, shi, tlo, thi);
                at(x, kG) = at(x, kF1) + tlo / slo - thi / shi;
            }
            T.sync();
            eliminate();
            substitute();
            // (v) one step length for heights and duals, 99% of the way to
            //     the nearest bound
            ap = INFINITY;
            ad = INFINITY;
            for (int x = T.tid(); x < N; x += T.size()) {
                if (!active(x)) continue;
                double d, slo, shi, tlo, thi, dzl, dzh;
                bdist(x, d, slo, shi);
                targets(x, slo, shi, tlo, thi);
                const double dd = at(par(x), kDel) - at(x, kDel);
                zsteps(x, dd, slo, shi, tlo, thi, dzl, dzh);
                limits(x, dd, slo, shi, dzl, dzh, ap, ad);
            }
            const double al = fmin(1.0, 0.99 * fmin(T.mind(ap), T.mind(ad)));
            if (!(al > 0.0)) break;   // no step: the barrier phase takes over
            // (vi) duals and the largest move, then the heights
            double mv = 0.0;
            for (int x = T.tid(); x < N; x += T.size()) {
                if (!active(x)) continue;
                double d, slo, shi, tlo, thi, dzl, dzh;
                bdist(x, d, slo, shi);
                targets(x, slo, shi, tlo, thi);
                const double dd = at(par(x), kDel) - at(x, kDel);
                zsteps(x, dd, slo, shi, tlo, thi, dzl, dzh);
                at(x, kZL) += al * dzl;
                at(x, kZH) += al * dzh;
                mv = fmax(mv, fabs(al * dd) / (1.0 + d));
            }
            move = -T.mind(-mv);   // every thread has read the heights
            for (int x = T.tid(); x < N; x += T.size())
                if (!leaf(x) && at(x, kPin) == 0.0) {
                    at(x, kBak) = at(x, kP);
                    at(x, kP) += al * at(x, kDel);
                }
            T.sync();
        }
    }

    for (int outer = 0; outer < kOuterMax && !pd_done; ++outer) {
        double lam_prev = INFINITY;
        for (int it = 0; it < kNewtonMax; ++it) {
            // (a) slope and weight of every branch in the barrier objective
            //     t f(d) + log(d - dmin) + log(dmax - d); the terms the line
            //     search reuses are kept
            for (int x = T.tid(); x < N; x += T.size()) {
                if (x == root) continue;
                if (!active(x)) {
                    at(x, kW) = 0.0;
                    at(x, kG) = 0.0;
                    continue;
                }
                const double a = at(x, kA), bb = at(x, kB), c = at(x, kC);
                const double d = at(par(x), kP) - at(x, kP);
                double g = -a, h = 0.0, ie = 0.0, ien = 0.0;
                if (bb > 0.0) {
                    const double e = expm132(d);
                    ie = rcp32(e);
                    g += bb * ie;
                    h -= bb * (e + 1.0) * ie * ie;
                }
                if (c > 0.0) {
                    const double e = expm132(nu * d);
                    ien = rcp32(e);
                    g += c * nu * ien;
                    h -= c * nu * nu * (e + 1.0) * ien * ien;
                }
                const double rl = rcp32(d - dlo), rh = rcp32(dhi - d);
                at(x, kG) = t * g + rl - rh;
                at(x, kW) = -(t * h) + rl * rl + rh * rh;
                at(x, kIE) = ie;
                at(x, kIEN) = ien;
                at(x, kRL) = rl;
                at(x, kRH) = rh;
            }
            T.sync();
            eliminate();
            const double lam = substitute();
            const double lam2 = T.sum2(lam, 0.0).x;
            ++n_newton;
            if (!(lam2 * 0.5 > kNewtonTol)) break;
            // quadratic phase without progress: the rounding floor of this t
            if (lam2 * 0.5 < 1e-2 && lam2 > 0.25 * lam_prev) break;
            lam_prev = lam2;
            // (d) the longest step that keeps every branch inside its bounds
            double amax = INFINITY;
            for (int x = T.tid(); x < N; x += T.size()) {
                if (!active(x)) continue;
                const int u = par(x);
                const double d = at(u, kP) - at(x, kP);
                const double s = at(u, kDel) - at(x, kDel);
                if (s > 0.0) amax = fmin(amax, (dhi - d) * rcp64(s));
                else if (s < 0.0) amax = fmin(amax, (d - dlo) * rcp64(-s));
            }
            amax = T.mind(amax);
            double alpha = fmin(1.0, 0.99 * amax);
            // (e) backtracking (Armijo) on the change of the barrier objective
            bool ok = false;
            for (int ls = 0; ls < kLineMax; ++ls) {
                double dphi = 0.0;
                for (int x = T.tid(); x < N; x += T.size()) {
                    if (!active(x)) continue;
                    const int u = par(x);
                    const double s = alpha * (at(u, kDel) - at(x, kDel));
                    const double bb = at(x, kB), c = at(x, kC);
                    double df = -at(x, kA) * s;
                    if (bb > 0.0) df += bb * log1p32(-expm132(-s) * at(x, kIE));
                    if (c > 0.0) df += c * log1p32(-expm132(-nu * s) * at(x, kIEN));
                    dphi += t * df + log1p32(s * at(x, kRL)) + log1p32(-s * at(x, kRH));
                }
                dphi = T.sum2(dphi, 0.0).x;
                ++n_line;
                if (dphi >= 0.25 * alpha * lam2) {
                    ok = true;
                    break;
                }
                alpha *= 0.5;
            }
            if (!ok) break;   // no measurable ascent left at this t
            for (int x = T.tid(); x < N; x += T.size())
                if (!leaf(x) && at(x, kPin) == 0.0) at(x, kP) += alpha * at(x, kDel);
            T.sync();
        }
        if (m / t <= gap_tol) break;
        t *= kMu;
    }

    // 4. branch lengths from the heights; the root's branch alone.  A height
    //    that is not finite (not expected) ends the solve with nothing
    //    written, instead of clamping a NaN length onto a bound
    int nonfinite = 0;
    for (int x = T.tid(); x < N; x += T.size())
        if (!isfinite(at(x, kP))) nonfinite = 1;
    if (T.maxi(nonfinite)) return kUltraNaN;
    if (T.leader()) {
        at(root, kStat) = (double)n_newton;
        at(0, kStat) = (double)n_line;
    }
    for (int x = T.tid(); x < N; x += T.size()) {
        if (x == root) {
            if (!freeb(x)) continue;
            const double dn = solve_branch(at(x, kA), at(x, kB), at(x, kC), nu, (double)Dd[x],
                                           dlo, dhi, true);
            Dd[x] = (float)dn;
            __stcg(b.nd_d + base + x, dn);
        } else if (freeb(x)) {
            const double dn = fmin(fmax(at(par(x), kP) - at(x, kP), dlo), dhi);
            Dd[x] = (float)dn;
            __stcg(b.nd_d + base + x, dn);
        }
    }
    T.sync();
    return kUltraOk;
}

// ---------------------------------------------------------------------------
// fastEM's own M-step (LAML_MSTEP_LBFGS, compat model): 100 steps of
// L-BFGS on M_step_loss_fn over x = (log d, logit nu, logit phi) in FP32, as
// fast_em/laml.py:49-110 runs it with optax (optax.lbfgs with
// scale_init_precond=True: the two-loop recursion over the last 10 pairs,
// the initial inverse Hessian <s, y> / <y, y> of the newest pair; its zoom
// line search for the strong Wolfe conditions, c1 = 1e-4, c2 = 0.9, first
// trial 1, at most 20 evaluations; chained with a backtracking Armijo test,
// factor 0.8, at most 15 times).  The published methods restated (Nocedal &
// Wright, algorithms 3.5, 3.6 and 7.4), not optax's code: iterates agree
// with the oracle's restatement to FP32 rounding, not bit for bit with optax.
// One team per tree; the vectors live in nd_lbfgs (LAML_LBFGS_SLOTS floats
// per node and per tree parameter), the scalars in every thread's registers.
// ---------------------------------------------------------------------------
namespace lbfgs {
constexpr int kM = 10, kSteps = 100, kZoom = 20, kBack = 15;
constexpr float kC1 = 1e-4f, kC2 = 0.9f, kBackFactor = 0.8f;
constexpr int kX = 0, kG = 1, kP = 2, kXT = 3, kGT = 4, kS = 5, kY = 5 + kM;
static_assert(kY + kM <= LAML_LBFGS_SLOTS, "nd_lbfgs slots");

// log(1 - e^-z) for z > 0 as fast_em's log1mexp_pos
__device__ __forceinline__ float l1m(float z) {
    return z > 0.69314718f ? log1pf(-expf(-z)) : logf(-expm1f(-z));
}
}  // namespace lbfgs

template <class Team>
__device__ __noinline__ void lbfgs_mstep(const laml_batch& b, int p, Team& T, int N, int base, double Mm,
                            double Rr, double LRd, uint8_t fix, double& nu, double& phi,
                            float* Dd) {
    using namespace lbfgs;
    const int64_t stride = b.n_nodes + 2 * (int64_t)b.n_trees;
    float* W = b.nd_lbfgs;
    const int NP = N + 2;
    auto at = [&](int slot, int i) -> float& {   // i < N: branch i; N: nu; N + 1: phi
        const int64_t idx = i < N ? (int64_t)base + i : b.n_nodes + 2 * (int64_t)p + (i - N);
        return W[(int64_t)slot * stride + idx];
    };
    const float lo = logf((float)kCalcEps), feps = (float)kCalcEps;
    const float M = (float)Mm, R = (float)Rr, LR = (float)LRd;
    const bool fnu = fix & 1, fphi = fix & 2;
    // loss and gradient at slot Z into slot Gs; with dir >= 0 also the
    // slope along slot dir
    auto eval = [&](int Z, int Gs, int dir, float& f, float& slope) {
        const float zn = at(Z, N), zp = at(Z, N + 1);
        const float sn = 1.f / (1.f + expf(-zn)), sp = 1.f / (1.f + expf(-zp));
        const float vn = fminf(fmaxf(sn, feps), 1.f - feps), vp = fminf(fmaxf(sp, feps), 1.f - feps);
        const bool inn = sn > feps && sn < 1.f - feps, inp = sp > feps && sp < 1.f - feps;
        float ls = 0.f, dfn = 0.f, dot = 0.f;
        for (int v = T.tid(); v < N; v += T.size()) {
            const double* c = b.nd_cnt + (int64_t)(base + v) * 6;
            const float c0 = (float)__ldcg(c), c1 = (float)__ldcg(c + 1), c2 = (float)__ldcg(c + 2),
                        c3 = (float)__ldcg(c + 3), c4 = (float)__ldcg(c + 4);
            const float u = at(Z, v);
            const float d = expf(fminf(fmaxf(u, lo), -lo));
            const float dn = d * vn;
            const float a1 = l1m(d), an = l1m(dn);
            ls += -c0 * d * (1.f + vn) + c1 * (a1 - d * vn) + c2 * an - c3 * d * vn + c4 * an;
            const float ie = 1.f / expm1f(d), ien = 1.f / expm1f(dn), cs = c2 + c4;
            const float dfd = -c0 * (1.f + vn) + c1 * (ie - vn) + cs * vn * ien - c3 * vn;
            dfn += -(c0 + c1 + c3) * d + cs * d * ien;
            const bool free = u > lo && u < -lo && __ldg(b.nd_mask + base + v);
            const float g = free ? -dfd * d : 0.f;
            at(Gs, v) = g;
            if (dir >= 0) dot += g * at(dir, v);
        }
        const float2 r = T.sum2f(ls, dfn);
        const float dsum = dir >= 0 ? T.sum2f(dot, 0.f).x : 0.f;
        const float c6 = R * logf(1.f - vp) + (M - LR) * logf(vp);
        f = -(r.x + c6);
        const float gn = (fnu || !inn) ? 0.f : -r.y * vn * (1.f - vn);
        const float gp = (fphi || !inp) ? 0.f : -(-R / (1.f - vp) + (M - LR) / vp) * vp * (1.f - vp);
        slope = dir >= 0 ? dsum + gn * at(dir, N) + gp * at(dir, N + 1) : 0.f;
        T.sync();   // every thread has read the parameters' slots
        if (T.leader()) {
            at(Gs, N) = gn;
            at(Gs, N + 1) = gp;
        }
        T.sync();
    };
    auto dotv = [&](int A, int B) {
        float s = 0.f;
        for (int i = T.tid(); i < NP; i += T.size()) s += at(A, i) * at(B, i);
        return T.sum2f(s, 0.f).x;
    };
    auto axpy = [&](int Yv, float a, int Xv) {   // Y += a X
        for (int i = T.tid(); i < NP; i += T.size()) at(Yv, i) += a * at(Xv, i);
        T.sync();
    };
    auto set = [&](int Yv, float a, int Xv, float c, int Zv) {   // Y = a X + c Z
        for (int i = T.tid(); i < NP; i += T.size())
            at(Yv, i) = a * at(Xv, i) + (Zv >= 0 ? c * at(Zv, i) : 0.f);
        T.sync();
    };
    // the EM loop's parameter vector (laml.py:126-139; kept across
    // iterations there, recovered here from d, nu, phi in FP64)
    for (int v = T.tid(); v < N; v += T.size()) at(kX, v) = (float)log(__ldcg(b.nd_d + base + v));
    if (T.leader()) {
        at(kX, N) = (float)log(nu / (1.0 - nu));
        at(kX, N + 1) = (float)log(phi / (1.0 - phi));
    }
    T.sync();
    float f, s0;
    eval(kX, kG, -1, f, s0);
    float rho[kM], alpha[kM];
    int cnt = 0, head = 0;
    float gamma = 1.f;
    for (int step = 0; step < kSteps; ++step) {
        // direction: two-loop recursion into kP
        set(kP, 1.f, kG, 0.f, -1);
        for (int h = cnt - 1; h >= 0; --h) {
            const int q = (head + h) % kM;
            alpha[q] = rho[q] * dotv(kS + q, kP);
            axpy(kP, -alpha[q], kY + q);
        }
        if (cnt > 0) set(kP, gamma, kP, 0.f, -1);
        for (int h = 0; h < cnt; ++h) {
            const int q = (head + h) % kM;
            const float beta = rho[q] * dotv(kY + q, kP);
            axpy(kP, alpha[q] - beta, kS + q);
        }
        set(kP, -1.f, kP, 0.f, -1);
        float d0 = dotv(kG, kP);
        if (!(d0 < 0.f)) {   // not a descent direction: the gradient, memory cleared
            set(kP, -1.f, kG, 0.f, -1);
            cnt = 0;
            head = 0;
            d0 = dotv(kG, kP);
            if (!(d0 < 0.f)) break;   // stationary under the masks
        }
        // zoom line search: trial a evaluated into kXT / kGT
        int nev = 0;
        float best_a = -1.f, best_f = 0.f;
        auto trial = [&](float a, float& fa, float& da) {
            set(kXT, 1.f, kX, a, kP);
            eval(kXT, kGT, kP, fa, da);
            ++nev;
            if (isfinite(fa) && fa <= f + kC1 * a * d0 && (best_a < 0.f || fa < best_f)) {
                best_a = a;
                best_f = fa;
            }
        };
        float acc_a = -1.f, acc_f = 0.f;   // accepted step; kXT / kGT hold it when set
        bool have = false;
        float ap = 0.f, fp = f, dp = d0, a = 1.f;
        float lo_a = 0.f, lo_f = 0.f, lo_d = 0.f, hi_a = 0.f, hi_f = 0.f, hi_d = 0.f;
        bool zoom = false;
        while (nev < kZoom) {
            float fa, da;
            trial(a, fa, da);
            if (!isfinite(fa) || fa > f + kC1 * a * d0 || (ap > 0.f && fa >= fp)) {
                lo_a = ap; lo_f = fp; lo_d = dp; hi_a = a; hi_f = fa; hi_d = da;
                zoom = true;
                break;
            }
            if (fabsf(da) <= -kC2 * d0) { acc_a = a; acc_f = fa; have = true; break; }
            if (da >= 0.f) {
                lo_a = a; lo_f = fa; lo_d = da; hi_a = ap; hi_f = fp; hi_d = dp;
                zoom = true;
                break;
            }
            ap = a; fp = fa; dp = da;
            a = 2.f * a;
        }
        while (zoom && !have && nev < kZoom) {
            // cubic through the bracket's ends (Nocedal & Wright eq. 3.59),
            // kept 10% inside it, else the midpoint
            float at_ = 0.5f * (lo_a + hi_a);
            const float w = fabsf(hi_a - lo_a);
            if (isfinite(hi_f) && isfinite(hi_d) && w > 0.f) {
                const float d1 = lo_d + hi_d - 3.f * (lo_f - hi_f) / (lo_a - hi_a);
                const float rad = d1 * d1 - lo_d * hi_d;
                if (rad >= 0.f) {
                    const float d2 = copysignf(sqrtf(rad), hi_a - lo_a);
                    const float den = hi_d - lo_d + 2.f * d2;
                    if (den != 0.f) {
                        const float c = hi_a - (hi_a - lo_a) * (hi_d + d2 - d1) / den;
                        if (c >= fminf(lo_a, hi_a) + 0.1f * w && c <= fmaxf(lo_a, hi_a) - 0.1f * w)
                            at_ = c;
                    }
                }
            }
            float fa, da;
            trial(at_, fa, da);
            if (!isfinite(fa) || fa > f + kC1 * at_ * d0 || fa >= lo_f) {
                hi_a = at_; hi_f = fa; hi_d = da;
            } else {
                if (fabsf(da) <= -kC2 * d0) { acc_a = at_; acc_f = fa; have = true; break; }
                if (da * (hi_a - lo_a) >= 0.f) { hi_a = lo_a; hi_f = lo_f; hi_d = lo_d; }
                lo_a = at_; lo_f = fa; lo_d = da;
            }
        }
        if (!have) {   // exhausted: the best sufficient-decrease point seen, else the last
            if (best_a >= 0.f) {
                acc_a = best_a;
                float fa, da;
                set(kXT, 1.f, kX, acc_a, kP);
                eval(kXT, kGT, kP, fa, da);
                acc_f = fa;
            } else {
                acc_a = a;
                float fa, da;
                set(kXT, 1.f, kX, acc_a, kP);
                eval(kXT, kGT, kP, fa, da);
                acc_f = fa;
            }
        }
        // the chained backtracking test on the step found
        const float slope = acc_a * d0;
        float t = 1.f;
        for (int k = 0; k < kBack; ++k) {
            if (isfinite(acc_f) && acc_f <= f + kC1 * t * slope) break;
            t *= kBackFactor;
            float da;
            set(kXT, 1.f, kX, t * acc_a, kP);
            eval(kXT, kGT, kP, acc_f, da);
        }
        // memory: s = x_new - x, y = g_new - g
        const int q = cnt < kM ? (head + cnt) % kM : head;
        set(kS + q, 1.f, kXT, -1.f, kX);
        set(kY + q, 1.f, kGT, -1.f, kG);
        const float sy = dotv(kS + q, kY + q), yy = dotv(kY + q, kY + q);
        rho[q] = sy == 0.f ? 0.f : 1.f / sy;
        gamma = yy > 0.f ? sy / yy : 1.f;
        if (cnt < kM) ++cnt;
        else head = (head + 1) % kM;
        set(kX, 1.f, kXT, 0.f, -1);
        set(kG, 1.f, kGT, 0.f, -1);
        f = acc_f;
    }
    // back to d, nu, phi as the EM loop reads them (exp, sigmoid; laml.py:151-156)
    for (int v = T.tid(); v < N; v += T.size()) {
        if (!__ldg(b.nd_mask + base + v)) continue;
        const double d = exp((double)at(kX, v));
        Dd[v] = (float)d;
        __stcg(b.nd_d + base + v, d);
    }
    nu = 1.0 / (1.0 + exp(-(double)at(kX, N)));
    phi = 1.0 / (1.0 + exp(-(double)at(kX, N + 1)));
    T.sync();
}

template <class Team>
__device__ void mstep_tree(const laml_batch& b, int p, int rounds, Team& T, float4* s_cnt,
                           float* s_d, int flags, double* usm = nullptr, int ucap = 0) {
    const bool polish = (flags & LAML_MSTEP_FP64_POLISH) != 0;
    const bool ultra = (flags & LAML_MSTEP_ULTRAMETRIC) != 0 && !b.compat;
    // primal-dual phase first (capped at kPdShort iterations to test the
    // barrier phase's continuation from its point)
    const int upd = (flags & LAML_MSTEP_ULTRA_BARRIER) ? 0
                    : (flags & LAML_MSTEP_ULTRA_PD_SHORT) ? ultra::kPdShort : ultra::kPdMax;
    if (__ldcg(b.tr_status + p) != LAML_TREE_ACTIVE) return;
    const int N = __ldg(b.tr_nodes + p), n = __ldg(b.tr_leaves + p), base = __ldg(b.tr_node_base + p);
    const int ds = __ldg(b.tr_ds + p), NG = __ldg(b.ds_groups + ds);
    // the whole tree's sites and '?' entries (all ranks' when its sites are split)
    const int K = b.tr_mstats ? (int)__ldg(b.tr_mstats + 2 * p + 1) : __ldg(b.ds_sites + ds);
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
    for (int v = T.tid(); v < N; v += T.size()) {
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
    const float2 LRf = T.sum2f(lr, lro);   // also orders the staging writes
    const double2 LRs = make_double2((double)LRf.x, (double)LRf.y);
    const double LR = LRs.x + LRs.y;
    if (T.leader()) {
        b.tr_prev[2 * p] = nu;
        b.tr_prev[2 * p + 1] = phi;
    }
    if (compat && (flags & LAML_MSTEP_LBFGS)) {   // fastEM's own M-step
        const double Mm = b.tr_mstats ? __ldg(b.tr_mstats + 2 * p) : __ldg(b.ds_missing + ds);
        lbfgs_mstep<Team>(b, p, T, N, base, Mm, (double)n * K - Mm, LR, fix, nu, phi, Dd);
    } else {
    // 2. phi (fast_em/laml.py:77 stationary point; EM_solver.py:318-326)
    if (!(fix & 2)) {
        const double M = b.tr_mstats ? __ldg(b.tr_mstats + 2 * p) : __ldg(b.ds_missing + ds);
        const double total = (double)n * K;
        if (compat) {
            // stationary point of R log(1 - phi) + B log(phi); with B <= 0
            // (leaf silencing explains every '?') the objective decreases in
            // phi and the bound is the maximum -- also when B < -R, where the
            // closed form's denominator changes sign
            const double Bm = M - LR, R = total - M;
            phi = Bm <= 0.0 ? kCalcEps : ((R + Bm) > 0.0 ? Bm / (R + Bm) : phi);
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
        if (ultra) {
            // EM_solver.Mstep returns "d_infeasible" before it places any
            // parameter (EM_solver.py:419-420): the tree keeps d, nu and phi
            const int us = (usm && N <= ucap)
                               ? ultra_dstep<Team, true>(b, p, T, nu, use_s, Dd, usm, upd)
                               : ultra_dstep<Team, false>(b, p, T, nu, use_s, Dd, nullptr, upd);
            if (us != kUltraOk) {
                if (T.leader())
                    b.tr_status[p] = us == kUltraNaN ? LAML_TREE_NAN : LAML_TREE_INFEASIBLE;
                T.sync();
                return;
            }
        } else if (last && polish) {
            for (int v = T.tid(); v < N; v += T.size()) {
                if (!__ldg(b.nd_mask + base + v)) continue;
                // the FP64 counts for the polished solve
                const double* c = b.nd_cnt + (int64_t)(base + v) * 6;
                const double c0 = __ldcg(c), c1 = __ldcg(c + 1), c2 = __ldcg(c + 2),
                             c3 = __ldcg(c + 3), c4 = __ldcg(c + 4);
                const double dn = solve_branch(c0 + nu * (c0 + c1 + c3), c1,
                                               use_s ? c2 + c4 : 0.0, nu, (double)Dd[v], dlo,
                                               dhi, true);
                Dd[v] = (float)dn;
                __stcg(b.nd_d + base + v, dn);
            }
        } else {
            for (int v = T.tid(); v < N; v += T.size()) {
                if (!__ldg(b.nd_mask + base + v)) continue;
                const float4 q = C4[v];
                const float dn = solve_branch_f(q.x + nuf * q.y, q.z, use_s ? q.w : 0.f, nuf,
                                                Dd[v], (float)dlo, (float)dhi);
                Dd[v] = dn;
                if (last) __stcg(b.nd_d + base + v, (double)dn);
            }
        }
        T.sync();
        if (!(fix & 1)) {
            // -A nu + sum_v c_v log(1 - e^{-nu d_v}); compat: every branch,
            // exact: the optimised branches (EM_solver.py:392-407)
            float Af = 0.f, Csf = 0.f;
            for (int v = T.tid(); v < N; v += T.size()) {
                if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                const float4 q = C4[v];
                Af += q.y * Dd[v];
                Csf += q.w;
            }
            const float2 acf = T.sum2f(Af, Csf);
            const double2 ac = make_double2((double)acf.x, (double)acf.y);
            double A = ac.x;
            const double nlo = compat ? kCalcEps : 1e-30, nhi = compat ? 1.0 - kCalcEps : 1.0;
            // G(nu) = -A + S1 / nu,  dG/dlog nu = -S2 / nu,  S1 = sum c h(nu d),
            // S2 = sum c h k  (h, k as in branch_F)
            auto sums = [&](double x, bool fp64) {
                if (fp64) {
                    double s1 = 0.0, s2 = 0.0;
                    for (int v = T.tid(); v < N; v += T.size()) {
                        if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                        const double* c = b.nd_cnt + (int64_t)(base + v) * 6;
                        const double cc = __ldcg(c + 2) + __ldcg(c + 4);
                        if (cc <= 0.0) continue;
                        const double y = x * __ldcg(b.nd_d + base + v), h = y / expm1(y);
                        s1 += cc * h;
                        s2 += cc * h * (h + y);
                    }
                    return T.sum2(s1, s2);
                }
                float s1 = 0.f, s2 = 0.f;
                const float xf = (float)x;
                for (int v = T.tid(); v < N; v += T.size()) {
                    if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                    const float cc = C4[v].w;
                    if (cc <= 0.f) continue;
                    const float y = xf * Dd[v], h = y / expm1f(y);
                    s1 += cc * h;
                    s2 += cc * h * (h + y);
                }
                const float2 r = T.sum2f(s1, s2);
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
                    for (int v = T.tid(); v < N; v += T.size()) {
                        if (!compat && !__ldg(b.nd_mask + base + v)) continue;
                        const double* c = b.nd_cnt + (int64_t)(base + v) * 6;
                        A64 += (__ldcg(c) + __ldcg(c + 1) + __ldcg(c + 3)) * __ldcg(b.nd_d + base + v);
                    }
                    A64 = T.sum2(A64, 0.0).x;
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
        T.sync();
    }
    }   // the stationary-point M-step
    if (T.leader()) {
        b.tr_nu[p] = nu;
        b.tr_phi[p] = phi;
        if (b.tr_leaf) reinterpret_cast<float2*>(b.tr_leaf)[p] = leaf_pair(phi, b.compat);
    }
    // the arithmetic of the next passes: log mode once a branch's
    // d (1 + nu) leaves the range of the linear partials
    int rate = 0;
    for (int v = T.tid(); v < N; v += T.size()) {
        reinterpret_cast<float4*>(b.nd_bt)[base + v] = branch_terms_of((double)Dd[v], nu, b.compat);
        rate = max(rate, __float_as_int(fmaxf(Dd[v] * (1.f + (float)nu), 0.f)));
    }
    rate = T.maxi(rate);
    if (T.leader())
        b.tr_mode[p] = __int_as_float(rate) > (float)LAML_LOG_MODE_RATE ? LAML_MODE_LOG
                                                                        : LAML_MODE_LINEAR;
    T.sync();
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

// limit of the device-side waits (grid barrier, mbarrier phases) in ns:
// laml_batch.wait_limit_ns, 0 = 2 s; negative = give up at the first check
// that finds the wait unsatisfied
__device__ __forceinline__ long long wait_limit(const laml_batch& b) {
    return b.wait_limit_ns == 0 ? 2000000000ll : b.wait_limit_ns;
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
            const long long lim = wait_limit(b);
            while (ld_acquire(b.barrier + 1) <= gen) {
                if (*(volatile int*)b.error != 0) { ok = 0; break; }
                if (lim < 0 || (long long)(gtimer() - t0) > lim) {
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
// Staged warp-per-item levels (linear partials, inside and non-root outside).
//
// A warp owns one (node, group) item at a time.  Lane = p * G + l works on
// site l of the group and on the state slots j = 2 + p, 2 + p + P, ...
// (P = 32 / G lanes per site), so a warp load or store of a slot range covers
// P consecutive slots of all G sites: 32 consecutive floats.  The item's
// partial rows (C * G floats each, contiguous in HBM) are copied into shared
// memory by the bulk-copy engine (cp.async.bulk, completion counted on an
// mbarrier) while the warp computes the previous item; descriptors are read
// two items ahead.  A descriptor lives spread over the warp: lanes 0..11 hold
// the item's 12 words, lanes 12..19 its group's 8 words, lane 20 the group's
// state count, lanes 21, 22 its tree's status and mode; fields are read with a
// shuffle.
// Trees in log mode take the per-lane path (global loads) on the first G
// lanes.  Every wait is bounded: on timeout the warp records
// LAML_ERR_TIMEOUT, waits (bounded) for its own copies and returns.
// ---------------------------------------------------------------------------
constexpr int kWWarps = 4;   // warps per block of the staged kernels

// A level is narrow when it has fewer items than a few per SM: its time is
// the latency of one item, which the one-warp-per-item kernels minimise; the
// wide levels are throughput-bound and run G sites x (32 / G) items per warp.
// The rule depends on the item count only, so every path (staged, direct,
// persistent) makes the same choice and computes the same values.
constexpr int64_t kNarrowItems = 8192;
__host__ __device__ __forceinline__ bool narrow_level(int64_t n) { return n <= kNarrowItems; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// non-blocking test of a phase (try_wait may suspend the thread for a while)
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// order this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy (bulk copy) writes
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for a phase of an mbarrier (the batch's wait limit, then
// LAML_ERR_TIMEOUT)
__device__ __forceinline__ bool mbar_wait(const laml_batch& b, uint64_t* bar, uint32_t parity) {
    const long long lim = wait_limit(b);
    if (lim < 0) {   // one check, without the suspension try_wait may take
        if (mbar_test_wait(bar, parity)) return true;
        atomicCAS(b.error, 0, LAML_ERR_TIMEOUT);
        return false;
    }
    if (mbar_try_wait(bar, parity)) return true;
    {
        const unsigned long long t0 = gtimer();
        for (uint32_t it = 0; it < (1u << 26); ++it) {
            if (mbar_try_wait(bar, parity)) return true;
            if ((it & 63) == 0 && (long long)(gtimer() - t0) > lim) break;
        }
    }
    atomicCAS(b.error, 0, LAML_ERR_TIMEOUT);
    return false;
}

// after a wait gave up: wait (2 s at most, whatever the batch's limit) for a
// phase whose bulk copies are in flight, so none lands after the block exits
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity) {
    const unsigned long long t0 = gtimer();
    for (uint32_t it = 0; it < (1u << 26); ++it) {
        if (mbar_try_wait(bar, parity)) return;
        if ((it & 63) == 0 && gtimer() - t0 > 2000000000ull) return;
    }
}

struct WItem {
    int u, v, w, tree, flags, g, gd, u_srow, u_prow8, v_ref, w_ref, v_srow, w_srow;
    int goff, site0, qoff, ds, code_base, kpad, nsites, C, status, mode;
};

__device__ __forceinline__ int wf(int r, int k) { return __shfl_sync(kFull, r, k); }

__device__ __forceinline__ WItem witem(int r) {
    WItem t;
    t.u = wf(r, 0); t.v = wf(r, 1); t.w = wf(r, 2);
    const int a3 = wf(r, 3);
    t.tree = a3 & 0xffffff;
    t.flags = (int)((unsigned)a3 >> 24);
    t.g = wf(r, 4); t.gd = wf(r, 5); t.u_srow = wf(r, 6); t.u_prow8 = wf(r, 7);
    t.v_ref = wf(r, 8); t.w_ref = wf(r, 9); t.v_srow = wf(r, 10); t.w_srow = wf(r, 11);
    t.goff = wf(r, 12); t.site0 = wf(r, 13); t.qoff = wf(r, 14); t.ds = wf(r, 15);
    t.code_base = wf(r, 16); t.kpad = wf(r, 17); t.nsites = wf(r, 18);
    t.C = wf(r, 20); t.status = wf(r, 21); t.mode = wf(r, 22);
    return t;
}

__device__ __forceinline__ int wload_desc(const int32_t* desc, int64_t it, int lane) {
    return lane < 12 ? __ldg(desc + 12 * it + lane) : 0;
}

// group words, state count, tree status and tree mode of the item whose
// descriptor words r holds
__device__ __forceinline__ int wload_grp(const laml_batch& b, int r, int lane) {
    const int gd = __shfl_sync(kFull, r, 5);
    const int tree = __shfl_sync(kFull, r, 3) & 0xffffff;
    if (lane >= 12 && lane < 20) return __ldg(b.grp_desc + 8 * (int64_t)gd + (lane - 12));
    if (lane == 20) return __ldg(b.group_C + gd);
    if (lane == 21) return __ldcg(b.tr_status + tree);
    if (lane == 22) return __ldcg(b.tr_mode + tree);
    return r;
}

// start the bulk copies of an item's rows: KIND 1 (outside) the parent's
// outside row, then the children's inside rows (internal children only);
// KIND 0 (inside) the children's inside rows.  All lanes call (shuffles).
template <int KIND, int G>
__device__ __forceinline__ void wissue(const laml_batch& b, int r, float* buf, int cmax,
                                       uint64_t* bar, int lane, bool respect_status) {
    const int flags = (int)((unsigned)wf(r, 3) >> 24);
    const int u_prow8 = wf(r, 7), v_ref = wf(r, 8), w_ref = wf(r, 9);
    const int goff = wf(r, 12), C = wf(r, 20), status = wf(r, 21), mode = wf(r, 22);
    if (lane != 0) return;
    const bool skip = C > cmax || (respect_status && status != LAML_TREE_ACTIVE) ||
                      mode == LAML_MODE_LOG;
    if (C > cmax) atomicCAS(b.error, 0, LAML_ERR_ARG);
    const uint32_t rb = (uint32_t)C * G * 4;
    const bool uin = KIND == 1, vin = !(flags & 1), win = !(flags & 2);
    const uint32_t tx = skip ? 0u : (uin ? rb : 0u) + (vin ? rb : 0u) + (win ? rb : 0u);
    fence_proxy_async_smem();
    mbar_arrive_tx(bar, tx);
    if (skip) return;
    const int cmaxG = cmax * G;
    if (uin) bulk_g2s(buf, b.out_part + (int64_t)u_prow8 * 8 + goff, rb, bar);
    float* dv = buf + (uin ? cmaxG : 0);
    if (vin) bulk_g2s(dv, b.in_part + (int64_t)v_ref * 8 + goff, rb, bar);
    if (win) bulk_g2s(dv + cmaxG, b.in_part + (int64_t)w_ref * 8 + goff, rb, bar);
}

__device__ __forceinline__ ItemDesc witem_desc(const WItem& t) {
    ItemDesc d;
    d.u = t.u; d.v = t.v; d.w = t.w; d.tree = t.tree; d.flags = t.flags; d.g = t.g; d.gd = t.gd;
    d.u_srow = t.u_srow; d.u_prow8 = t.u_prow8; d.v_ref = t.v_ref; d.w_ref = t.w_ref;
    d.v_srow = t.v_srow; d.w_srow = t.w_srow;
    return d;
}

template <int G>
__device__ __forceinline__ void witem_ctx(const laml_batch& b, const WItem& t, int l, SiteCtx& s,
                                          GroupCtx& gc) {
    s.tree = t.tree;
    s.ds = t.ds;
    s.site = t.g * G + l;
    s.goff = t.goff;
    s.C = __ldg(b.site_C + t.site0 + l);
    s.sumq = __ldg(b.site_sumq + t.site0 + l);
    s.qrow = b.q + t.qoff + l;
    gc.code_base = t.code_base;
    gc.kpad = t.kpad;
}

// one child of a staged item at site l: inside values from shared memory
// (internal) or from the leaf's character code
template <int G, bool LEAF>
__device__ __forceinline__ Child wchild(const laml_batch& b, const WItem& t, int ref, int srow,
                                        const float* srow_smem, const SiteCtx& s, const Leaf& L,
                                        bool act) {
    Child c;
    c.e1 = L.e1;
    c.ephi = L.ephi;
    if (LEAF) {
        const int code = act ? __ldg(b.codes + t.code_base + (int64_t)ref * t.kpad + s.site) : 0;
        c.row = nullptr;
        c.f = 1.f;
        c.X = 0;
        c.code = code;
        c.s0 = code == 0 ? L.e1 : (code == -1 ? L.ephi : 0.f);
        c.ss = code < 0 ? 1.f : L.es;
        c.D = code >= 2 ? __ldg(s.qrow + code * G) * L.e1 : (code == -1 ? L.ephi * s.sumq : 0.f);
    } else {
        const int64_t si = (int64_t)srow + s.site;
        const int h = act ? __ldcg(b.in_h + si) : 0;
        c.f = pow2i(-h);
        c.X = act ? __ldcg(b.in_x + si) : 0;
        c.D = act ? __ldcg(b.in_dot + si) : 0.f;
        c.row = srow_smem;   // marks an internal child; values come from shared memory
        c.code = 0;
    }
    return c;
}

// slot j of a child of a staged item (leaf: from its code)
template <int G, bool LEAF, bool STAGED>
__device__ __forceinline__ float wval(const Child& c, const float* r, int j, float cst) {
    if (LEAF) return c.code == j ? c.e1 : cst;
    return (STAGED ? r[j * G] : __ldcg(r + j * G)) * c.f;
}

template <bool STAGED>
__device__ __forceinline__ float wrow(const float* r, int k) {
    return STAGED ? r[k] : __ldcg(r + k);
}

// STAGED: the children's rows are in shared memory (buf, after waiting on
// bar); otherwise they are read from HBM (persistent kernel)
template <int G, bool VL, bool WL, bool STAGED>
__device__ void inside_w(const laml_batch& b, const WItem& t, const float* buf, int cmax, int lane,
                         bool& waited, uint64_t* bar, uint32_t parity) {
    constexpr int P = 32 / G;
    const int l = lane % G, p = lane / G;
    SiteCtx s;
    GroupCtx gc;
    witem_ctx<G>(b, t, l, s, gc);
    const bool act = s.site < t.nsites;
    if (!act) s.C = 0;
    const Leaf L = leaf_params(b, t.tree);
    const int cmaxG = cmax * G;
    const float* rv = STAGED ? buf + l : b.in_part + (int64_t)t.v_ref * 8 + t.goff + l;
    const float* rw = STAGED ? buf + cmaxG + l : b.in_part + (int64_t)t.w_ref * 8 + t.goff + l;
    Child cv = wchild<G, VL>(b, t, t.v_ref, t.v_srow, rv, s, L, act);
    Child cw = wchild<G, WL>(b, t, t.w_ref, t.w_srow, rw, s, L, act);
    const float4 bv = load_bt(b, t.v), bw = load_bt(b, t.w);
    if (STAGED) {
        waited = mbar_wait(b, bar, parity);
        if (!waited) return;
    }
    if (!VL) { cv.s0 = wrow<STAGED>(rv, 0) * cv.f; cv.ss = wrow<STAGED>(rv, G) * cv.f; }
    if (!WL) { cw.s0 = wrow<STAGED>(rw, 0) * cw.f; cw.ss = wrow<STAGED>(rw, G) * cw.f; }
    const float ev0 = edge0(bv, cv.s0, cv.D, cv.ss);
    const float ew0 = edge0(bw, cw.s0, cw.D, cw.ss);
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    const float cstv = cv.code == -1 ? L.ephi : 0.f, cstw = cw.code == -1 ? L.ephi : 0.f;
    float* row = b.in_part + (int64_t)t.u_prow8 * 8 + t.goff + l;
    const float s0 = ev0 * ew0, ss = cv.ss * cw.ss;
    float mx = 0.f, dot = 0.f;
    if (act && p == 0) {
        __stcg(row, s0);
        __stcg(row + G, ss);
        mx = fmaxf(s0, ss);
    }
#pragma unroll 4
    for (int j = 2 + p; j < s.C; j += P) {
        const float av = wval<G, VL, STAGED>(cv, rv, j, cstv);
        const float aw = wval<G, WL, STAGED>(cw, rw, j, cstw);
        const float x = fmaf(bv.z, av, kv) * fmaf(bw.z, aw, kw);
        __stcg(row + j * G, x);
        dot = fmaf(__ldg(s.qrow + j * G), x, dot);
        mx = fmaxf(mx, x);
    }
#pragma unroll
    for (int off = G; off < 32; off <<= 1) {
        dot += __shfl_xor_sync(kFull, dot, off);
        mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, off));
    }
    if (act && p == 0) {
        const int h = scale_exp(mx);
        const float f = pow2i(-h);
        const int X = cv.X + cw.X + h;
        const int64_t sr = (int64_t)t.u_srow + s.site;
        __stcg(b.in_h + sr, h);
        __stcg(b.in_x + sr, X);
        __stcg(b.in_dot + sr, dot * f);
        if (t.flags & 4)
            root_site_llh(b, t.tree, s.site, root_edge_logs(b, t.tree), s0 * f, dot * f, ss * f,
                          X);
    }
}

template <int G, bool VL, bool WL, bool STAGED>
__device__ void outside_w(const laml_batch& b, const WItem& t, const float* buf, int cmax,
                          int lane, bool want_post, bool& waited, uint64_t* bar,
                          uint32_t parity) {
    constexpr int P = 32 / G;
    const int l = lane % G, p = lane / G;
    SiteCtx s;
    GroupCtx gc;
    witem_ctx<G>(b, t, l, s, gc);
    const bool act = s.site < t.nsites;
    if (!act) s.C = 0;
    const Leaf L = leaf_params(b, t.tree);
    const int cmaxG = cmax * G;
    const float* ru = STAGED ? buf + l : b.out_part + (int64_t)t.u_prow8 * 8 + t.goff + l;
    const float* rv = STAGED ? buf + cmaxG + l : b.in_part + (int64_t)t.v_ref * 8 + t.goff + l;
    const float* rw = STAGED ? buf + 2 * cmaxG + l : b.in_part + (int64_t)t.w_ref * 8 + t.goff + l;
    Child cv = wchild<G, VL>(b, t, t.v_ref, t.v_srow, rv, s, L, act);
    Child cw = wchild<G, WL>(b, t, t.w_ref, t.w_srow, rw, s, L, act);
    const float4 bv = load_bt(b, t.v), bw = load_bt(b, t.w);
    const int64_t su = (int64_t)t.u_srow + s.site;
    const float fo = pow2i(act ? -__ldcg(b.out_h + su) : 0);
    const int Xo = act ? __ldcg(b.out_x + su) : 0;
    const int64_t ts = __ldg(b.tr_site_base + t.tree) + s.site;
    const float lroot = act ? __ldcg(b.root_lr + ts) : 0.f;
    const int xroot = act ? __ldcg(b.root_x + ts) : 0;
    if (STAGED) {
        waited = mbar_wait(b, bar, parity);
        if (!waited) return;
    }
    if (!VL) { cv.s0 = wrow<STAGED>(rv, 0) * cv.f; cv.ss = wrow<STAGED>(rv, G) * cv.f; }
    if (!WL) { cw.s0 = wrow<STAGED>(rw, 0) * cw.f; cw.ss = wrow<STAGED>(rw, G) * cw.f; }
    const float o0 = wrow<STAGED>(ru, 0) * fo, os = wrow<STAGED>(ru, G) * fo;
    const float ev0 = edge0(bv, cv.s0, cv.D, cv.ss);
    const float ew0 = edge0(bw, cw.s0, cw.D, cw.ss);
    ChildOut A, B;   // A: child v (uses E[w]), B: child w (uses E[v])
    A.x0 = o0 * ew0; A.xs = os * cw.ss; A.X = Xo + cw.X;
    B.x0 = o0 * ev0; B.xs = os * cv.ss; B.X = Xo + cv.X;
    A.sumx = A.dot = A.mx = 0.f;
    B.sumx = B.dot = B.mx = 0.f;
    A.orow = VL ? nullptr : b.out_part + (int64_t)t.v_ref * 8 + t.goff + l;
    B.orow = WL ? nullptr : b.out_part + (int64_t)t.w_ref * 8 + t.goff + l;
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    const float pxa = bv.y * A.x0, pxb = bw.y * B.x0;
    const float cstv = cv.code == -1 ? L.ephi : 0.f, cstw = cw.code == -1 ? L.ephi : 0.f;
#pragma unroll 4
    for (int j = 2 + p; j < s.C; j += P) {
        const float o = wrow<STAGED>(ru, j * G) * fo;
        const float av = wval<G, VL, STAGED>(cv, rv, j, cstv);
        const float aw = wval<G, WL, STAGED>(cw, rw, j, cstw);
        const float qj = __ldg(s.qrow + j * G);
        const float xa = mulr(o, fmaf(bw.z, aw, kw));
        const float xb = mulr(o, fmaf(bv.z, av, kv));
        A.sumx = addr(A.sumx, xa);
        A.dot = fmaf(xa, av, A.dot);
        B.sumx = addr(B.sumx, xb);
        B.dot = fmaf(xb, aw, B.dot);
        if (!VL) {
            const float r = fmaf(pxa, qj, mulr(bv.z, xa));
            __stcg(A.orow + j * G, r);
            A.mx = fmaxf(A.mx, r);
        }
        if (!WL) {
            const float r = fmaf(pxb, qj, mulr(bw.z, xb));
            __stcg(B.orow + j * G, r);
            B.mx = fmaxf(B.mx, r);
        }
    }
#pragma unroll
    for (int off = G; off < 32; off <<= 1) {
        A.sumx += __shfl_xor_sync(kFull, A.sumx, off);
        A.dot += __shfl_xor_sync(kFull, A.dot, off);
        A.mx = fmaxf(A.mx, __shfl_xor_sync(kFull, A.mx, off));
        B.sumx += __shfl_xor_sync(kFull, B.sumx, off);
        B.dot += __shfl_xor_sync(kFull, B.dot, off);
        B.mx = fmaxf(B.mx, __shfl_xor_sync(kFull, B.mx, off));
    }
    // child v's finish on phase 0, child w's on phase 1 (both on phase 0 when
    // a site has one lane)
    constexpr int PW = P > 1 ? 1 : 0;
    float cv_[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cw_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (act && p == 0) child_finish<G>(b, s, t.v, cv, bv, A, want_post, lroot, xroot, cv_);
    if (act && p == PW) child_finish<G>(b, s, t.w, cw, bw, B, want_post, lroot, xroot, cw_);
    if (P > 1) {
        float c[8];   // phase 0 lanes carry child v's counts, phase 1 lanes child w's
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k] = p == 0 ? cv_[k] : cw_[k];
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1)
#pragma unroll
            for (int k = 0; k < 8; ++k) c[k] += __shfl_xor_sync(kFull, c[k], off);
        if (l == 0 && p < 2) write_counts<G>(b, t.tree, p == 0 ? t.v : t.w, t.g, c);
    } else {
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1)
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                cv_[k] += __shfl_xor_sync(kFull, cv_[k], off);
                cw_[k] += __shfl_xor_sync(kFull, cw_[k], off);
            }
        if (l == 0) {
            write_counts<G>(b, t.tree, t.v, t.g, cv_);
            write_counts<G>(b, t.tree, t.w, t.g, cw_);
        }
    }
}

// one staged or direct item of kind 0 (inside) / 1 (outside below the roots),
// dispatched on which children are leaves; log-mode trees take the per-lane
// path on lanes 0..G-1
template <int G, int KIND, bool STAGED>
__device__ __forceinline__ bool witem_run(const laml_batch& b, const WItem& t, const float* buf,
                                          int cmax, int lane, bool want_post, bool respect_status,
                                          uint64_t* bar, uint32_t parity) {
    const bool skip = (STAGED && t.C > cmax) ||
                      ((KIND == 1 || respect_status) && t.status != LAML_TREE_ACTIVE);
    bool waited = true;
    if (skip || t.mode == LAML_MODE_LOG) {
        if (STAGED) waited = mbar_wait(b, bar, parity);
        if (!waited || skip) return waited;
        const int l = lane % G, p = lane / G;
        SiteCtx s;
        GroupCtx gc;
        witem_ctx<G>(b, t, l, s, gc);
        const bool act = p == 0 && s.site < t.nsites;
        const ItemDesc d = witem_desc(t);
        if (KIND == 0) {
            if (act) inside_log_item<G>(b, d, s, gc);
        } else {
            float cv_[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cw_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (act) outside_log_lane<G>(b, d, s, gc, want_post, cv_, cw_);
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1)
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    cv_[k] += __shfl_xor_sync(kFull, cv_[k], off);
                    cw_[k] += __shfl_xor_sync(kFull, cw_[k], off);
                }
            if (lane == 0) {
                write_counts<G>(b, t.tree, t.v, t.g, cv_);
                write_counts<G>(b, t.tree, t.w, t.g, cw_);
            }
        }
        return true;
    }
    const int leaves = t.flags & 3;
#define LAML_W_CALL(VL, WL)                                                                  \
    if (KIND == 0)                                                                           \
        inside_w<G, VL, WL, STAGED>(b, t, buf, cmax, lane, waited, bar, parity);             \
    else                                                                                     \
        outside_w<G, VL, WL, STAGED>(b, t, buf, cmax, lane, want_post, waited, bar, parity);
    switch (leaves) {
        case 0: LAML_W_CALL(false, false) break;
        case 1: LAML_W_CALL(true, false) break;
        case 2: LAML_W_CALL(false, true) break;
        default: LAML_W_CALL(true, true) break;
    }
#undef LAML_W_CALL
    return waited;
}

// Staged level kernel: dynamic shared memory holds, per warp, two buffers of
// NR rows of cmax * G floats (NR = 3 outside, 2 inside) and two mbarriers.
template <int G, int KIND>
__global__ void __launch_bounds__(kWWarps * 32) k_items_w(laml_batch b, const int32_t* desc,
                                                          int64_t n, int cmax, int want_post,
                                                          int respect_status) {
    extern __shared__ __align__(128) unsigned char wsm[];
    constexpr int NR = KIND == 1 ? 3 : 2;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t per = (int64_t)NR * cmax * G;   // floats of one buffer
    float* bufs = reinterpret_cast<float*>(wsm) + (int64_t)wib * 2 * per;
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<float*>(wsm) +
                                                 (int64_t)kWWarps * 2 * per) + 2 * wib;
    const int64_t gw = (int64_t)blockIdx.x * kWWarps + wib;
    const int64_t nw = (int64_t)gridDim.x * kWWarps;
    if (gw >= n) return;
    if (lane == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        fence_mbar_init();
    }
    __syncwarp();
    int r0 = wload_grp(b, wload_desc(desc, gw, lane), lane);
    int r1 = gw + nw < n ? wload_grp(b, wload_desc(desc, gw + nw, lane), lane) : 0;
    int r2 = gw + 2 * nw < n ? wload_desc(desc, gw + 2 * nw, lane) : 0;
    wissue<KIND, G>(b, r0, bufs, cmax, bars, lane, KIND == 1 || respect_status);
    uint32_t ph = 0;   // bit k: phase parity of buffer k
    int cur = 0;
    for (int64_t it = gw; it < n; it += nw) {
        const bool has1 = it + nw < n, has2 = it + 2 * nw < n, has3 = it + 3 * nw < n;
        if (has2) r2 = wload_grp(b, r2, lane);
        if (has1)
            wissue<KIND, G>(b, r1, bufs + (cur ^ 1) * per, cmax, bars + (cur ^ 1), lane,
                            KIND == 1 || respect_status);
        const int r3 = has3 ? wload_desc(desc, it + 3 * nw, lane) : 0;
        const WItem t = witem(r0);
        const uint32_t par = (ph >> cur) & 1u;
        ph ^= 1u << cur;
        if (!witem_run<G, KIND, true>(b, t, bufs + cur * per, cmax, lane, want_post != 0,
                                      respect_status != 0, bars + cur, par)) {
            // timed out: wait (bounded) for this warp's copies still in flight
            mbar_drain(bars + cur, par);
            if (has1) mbar_drain(bars + (cur ^ 1), (ph >> (cur ^ 1)) & 1u);
            return;
        }
        __syncwarp();
        r0 = r1;
        r1 = r2;
        r2 = r3;
        cur ^= 1;
    }
}

// ---------------------------------------------------------------------------
// Bulk-staged wide levels (inside, and outside below the roots; linear
// partials).  The item mapping of the wide kernels -- G sites x 32 / G items
// per warp, one thread per (item, site) -- with the partial rows a thread
// reads arriving in shared memory from the bulk-copy engine.  Each warp runs
// a ring of kSSlots / CH stages; a stage holds CH state slots of every row
// of the warp's 32 / G items (one cp.async.bulk per row and chunk, issued by
// the item's first lane, completion counted on the stage's mbarrier), and is
// refilled as soon as the warp has consumed it.  So up to kSSlots / CH chunks of
// rows are in flight per warp whatever the items' state counts, the
// load/store unit reads only shared memory for them, and no register holds
// a load in flight.  A warp takes every nw-th slab (32 / G consecutive
// items) of the level; each slab's descriptors are read two slabs ahead and
// its scalars one slab ahead.  Every thread's arithmetic is the direct wide
// kernels', in the same order, so the results are bitwise equal.
// ---------------------------------------------------------------------------
constexpr int kSWarps = 4;     // warps per block
constexpr int kSSlots = 32;    // state slots of each row a warp's ring holds
constexpr int kSMinBlocks = 4; // resident blocks per SM asked (<= 128 registers)
// CH state slots of a row per stage, max(2, kSSlots / CH) stages per warp:
// the autotuner's states-per-stage axis (laml_batch.wide_chunk)

template <int G, int NR, int CH>
struct SGeom {
    static constexpr int P = 32 / G;                 // items per warp
    static constexpr int S = kSSlots / CH > 2 ? kSSlots / CH : 2;   // stages per warp
    static constexpr int row = CH * G;               // floats of one row's chunk
    static constexpr int item = NR * row + G;        // + G floats: items start G banks apart
    static constexpr int stage = P * item;
    static constexpr size_t warp_bytes = (size_t)S * stage * sizeof(float);
    static constexpr size_t block_bytes = kSWarps * (warp_bytes + S * sizeof(uint64_t));
};

// one thread's item of a slab: descriptor, site, the group's slot count and
// the scalars its state loop needs (internal children's slots 0 and 1 come
// from the first stage)
struct SItem {
    ItemDesc d;
    SiteCtx s;
    GroupCtx gc;
    int Cg;                    // slots of each of the item's rows (the group's)
    bool valid, live, staged;  // it < n; a real site of an active tree; rows staged
    bool logm;                 // the tree keeps log partials (per-lane global path)
    Child cv, cw;
    float4 bv, bw;
    float fo, lroot;           // outside: 2^-h of the parent's outside row; site likelihood mantissa
    int Xo, xroot;
};

template <int G>
__device__ __forceinline__ Child s_child(const laml_batch& b, bool leaf, int ref, int srow,
                                         const SiteCtx& s, const GroupCtx& gc, const Leaf& L) {
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
        c.f = pow2i(-__ldcg(b.in_h + si));
        c.X = __ldcg(b.in_x + si);
        c.D = __ldcg(b.in_dot + si);
        c.row = b.in_part;   // marks an internal child; its slots come from the stages
        c.code = 0;
        c.s0 = c.ss = 0.f;
    }
    return c;
}

template <int G, int KIND>
__device__ __forceinline__ void s_load(const laml_batch& b, const ItemDesc& d, bool valid,
                                       int lane, bool respect_status, SItem& t) {
    const bool rs = KIND == 1 || respect_status;
    t.d = d;
    t.valid = valid;
    t.live = valid && site_ctx_d<G>(b, d, lane, rs, t.s, t.gc);
    t.Cg = valid ? __ldg(b.group_C + d.gd) : 0;
    const bool active = valid && (!rs || __ldcg(b.tr_status + d.tree) == LAML_TREE_ACTIVE);
    t.logm = valid && tree_log(b, d.tree);
    t.staged = active && !t.logm;
    if (!(t.live && t.staged)) return;
    const Leaf L = leaf_params(b, t.s.tree);
    t.cv = s_child<G>(b, d.flags & 1, d.v_ref, d.v_srow, t.s, t.gc, L);
    t.cw = s_child<G>(b, d.flags & 2, d.w_ref, d.w_srow, t.s, t.gc, L);
    t.bv = load_bt(b, d.v);
    t.bw = load_bt(b, d.w);
    if (KIND == 1) {
        const int64_t su = (int64_t)d.u_srow + t.s.site;
        t.fo = pow2i(-__ldcg(b.out_h + su));
        t.Xo = __ldcg(b.out_x + su);
        const int64_t ts = __ldg(b.tr_site_base + t.s.tree) + t.s.site;
        t.lroot = __ldcg(b.root_lr + ts);
        t.xroot = __ldcg(b.root_x + ts);
    }
}

// what an item's leader lane needs to copy the item's rows: row offsets,
// the group's offset and slot count, whether the rows are staged at all
struct SIss {
    int u_prow8, v_ref, w_ref, flags, goff, Cg;
    bool staged;
};

template <int KIND>
__device__ __forceinline__ SIss s_iss(const laml_batch& b, const ItemDesc& d, bool valid,
                                      bool respect_status) {
    const bool rs = KIND == 1 || respect_status;
    SIss t;
    t.u_prow8 = d.u_prow8;
    t.v_ref = d.v_ref;
    t.w_ref = d.w_ref;
    t.flags = d.flags;
    t.goff = __ldg(b.grp_desc + 8 * (int64_t)d.gd);
    t.Cg = valid ? __ldg(b.group_C + d.gd) : 0;
    const bool active = valid && (!rs || __ldcg(b.tr_status + d.tree) == LAML_TREE_ACTIVE);
    t.staged = active && !tree_log(b, d.tree);
    return t;
}

// chunks of a slab: its staged items' largest slot count over CH
template <int CH>
__device__ __forceinline__ int s_chunks(const SIss& t) {
    const int c = t.staged ? t.Cg : 0;
    const int m = __reduce_max_sync(kFull, c);
    return (m + CH - 1) / CH;
}

// the item's leader lane: arrive on the stage's mbarrier with the bytes of
// chunk c of the item's rows (0 when it has none) and start their copies
template <int G, int KIND, int CH>
__device__ __forceinline__ void s_issue(const laml_batch& b, const SIss& t, int c, float* dst,
                                        uint64_t* bar) {
    constexpr int R = CH * G;
    const int j0 = c * CH;
    const int ns = t.staged ? min(CH, t.Cg - j0) : 0;
    const uint32_t bytes = ns > 0 ? (uint32_t)ns * G * 4u : 0u;
    const bool uin = KIND == 1, vin = !(t.flags & 1), win = !(t.flags & 2);
    const uint32_t tx = bytes ? (uin ? bytes : 0u) + (vin ? bytes : 0u) + (win ? bytes : 0u) : 0u;
    fence_proxy_async_smem();   // this warp's reads of the stage's last use come first
    mbar_arrive_tx(bar, tx);
    if (!tx) return;
    const int64_t off = (int64_t)t.goff + (int64_t)j0 * G;
    if (uin) bulk_g2s(dst, b.out_part + (int64_t)t.u_prow8 * 8 + off, bytes, bar);
    if (vin) bulk_g2s(dst + (uin ? 1 : 0) * R, b.in_part + (int64_t)t.v_ref * 8 + off, bytes, bar);
    if (win) bulk_g2s(dst + (uin ? 2 : 1) * R, b.in_part + (int64_t)t.w_ref * 8 + off, bytes, bar);
}

// one state slot of a staged outside chunk (k: the slot's offset in the stage)
template <int G, bool VL, bool WL>
__device__ __forceinline__ void s_outside_slot(const float* su, const float* sv, const float* sw,
                                               int k, int j, float fo, const Child& cv,
                                               const Child& cw, float bvz, float bwz, float kv,
                                               float kw, float cstv, float cstw, float qj,
                                               float pxa, float pxb, float* __restrict__ ra,
                                               float* __restrict__ rb, float& sa, float& da,
                                               float& ma, float& sb, float& db, float& mb) {
    const float o = su[k] * fo;
    const float av = VL ? (cv.code == j ? cv.e1 : cstv) : sv[k] * cv.f;
    const float aw = WL ? (cw.code == j ? cw.e1 : cstw) : sw[k] * cw.f;
    const float xa = mulr(o, fmaf(bwz, aw, kw));
    const float xb = mulr(o, fmaf(bvz, av, kv));
    sa = addr(sa, xa);
    da = fmaf(xa, av, da);
    sb = addr(sb, xb);
    db = fmaf(xb, aw, db);
    if (!VL) {
        const float r = fmaf(pxa, qj, mulr(bvz, xa));
        __stcg(ra, r);
        ma = fmaxf(ma, r);
    }
    if (!WL) {
        const float r = fmaf(pxb, qj, mulr(bwz, xb));
        __stcg(rb, r);
        mb = fmaxf(mb, r);
    }
}

// slots jlo .. jhi - 1 of a staged chunk starting at slot j0; a full chunk
// (jlo = j0, jhi = j0 + CH) runs unrolled at fixed offsets
template <int G, int CH, bool VL, bool WL>
__device__ __forceinline__ void s_outside_chunk(const float* su, const float* sv, const float* sw,
                                                int j0, int jlo, int jhi, float fo,
                                                const Child& cv, const Child& cw,
                                                const float4& bv, const float4& bw,
                                                const float* __restrict__ qrow, float pxa,
                                                float pxb, float* __restrict__ ra,
                                                float* __restrict__ rb, float& sa, float& da,
                                                float& ma, float& sb, float& db, float& mb) {
    const float cstv = cv.code == -1 ? cv.ephi : 0.f, cstw = cw.code == -1 ? cw.ephi : 0.f;
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    if (jlo == j0 && jhi == j0 + CH) {
        const float* q0 = qrow + j0 * G;
        float* a0 = VL ? nullptr : ra + j0 * G;
        float* b0 = WL ? nullptr : rb + j0 * G;
#pragma unroll
        for (int k = 0; k < CH; ++k)
            s_outside_slot<G, VL, WL>(su, sv, sw, k * G, j0 + k, fo, cv, cw, bv.z, bw.z, kv, kw,
                                      cstv, cstw, __ldg(q0 + k * G), pxa, pxb,
                                      VL ? nullptr : a0 + k * G, WL ? nullptr : b0 + k * G,
                                      sa, da, ma, sb, db, mb);
        return;
    }
#pragma unroll 4
    for (int j = jlo; j < jhi; ++j)
        s_outside_slot<G, VL, WL>(su, sv, sw, (j - j0) * G, j, fo, cv, cw, bv.z, bw.z, kv, kw,
                                  cstv, cstw, __ldg(qrow + j * G), pxa, pxb,
                                  VL ? nullptr : ra + j * G, WL ? nullptr : rb + j * G, sa, da,
                                  ma, sb, db, mb);
}

template <int G, bool VL, bool WL>
__device__ __forceinline__ void s_inside_slot(const float* sv, const float* sw, int k, int j,
                                              const Child& cv, const Child& cw, float bvz,
                                              float bwz, float kv, float kw, float cstv,
                                              float cstw, float qj, float* __restrict__ r,
                                              float& dot, float& mx) {
    const float av = VL ? (cv.code == j ? cv.e1 : cstv) : sv[k] * cv.f;
    const float aw = WL ? (cw.code == j ? cw.e1 : cstw) : sw[k] * cw.f;
    const float x = fmaf(bvz, av, kv) * fmaf(bwz, aw, kw);
    __stcg(r, x);
    dot = fmaf(qj, x, dot);
    mx = fmaxf(mx, x);
}

template <int G, int CH, bool VL, bool WL>
__device__ __forceinline__ void s_inside_chunk(const float* sv, const float* sw, int j0, int jlo,
                                               int jhi, const Child& cv, const Child& cw,
                                               const float4& bv, const float4& bw,
                                               const float* __restrict__ qrow,
                                               float* __restrict__ row, float& dot, float& mx) {
    const float cstv = cv.code == -1 ? cv.ephi : 0.f, cstw = cw.code == -1 ? cw.ephi : 0.f;
    const float kv = bv.w * cv.ss, kw = bw.w * cw.ss;
    if (jlo == j0 && jhi == j0 + CH) {
        const float* q0 = qrow + j0 * G;
        float* r0 = row + j0 * G;
#pragma unroll
        for (int k = 0; k < CH; ++k)
            s_inside_slot<G, VL, WL>(sv, sw, k * G, j0 + k, cv, cw, bv.z, bw.z, kv, kw, cstv,
                                     cstw, __ldg(q0 + k * G), r0 + k * G, dot, mx);
        return;
    }
#pragma unroll 4
    for (int j = jlo; j < jhi; ++j)
        s_inside_slot<G, VL, WL>(sv, sw, (j - j0) * G, j, cv, cw, bv.z, bw.z, kv, kw, cstv, cstw,
                                 __ldg(qrow + j * G), row + j * G, dot, mx);
}

template <int G, int KIND, int CH>
__global__ void __launch_bounds__(kSWarps * 32, kSMinBlocks) k_items_ws(laml_batch b,
                                                                        const int32_t* desc,
                                                                        int64_t n, int want_post,
                                                                        int respect_status) {
    constexpr int NR = KIND == 1 ? 3 : 2;
    using Geo = SGeom<G, NR, CH>;
    constexpr int P = Geo::P, R = Geo::row, kSStages = Geo::S;
    extern __shared__ __align__(128) unsigned char ssm[];
    const int lane32 = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int sub = lane32 / G, l = lane32 % G;
    const bool leader = l == 0;
    float* ring = reinterpret_cast<float*>(ssm) + (size_t)wib * kSStages * Geo::stage;
    uint64_t* bars = reinterpret_cast<uint64_t*>(ssm + kSWarps * Geo::warp_bytes) + wib * kSStages;
    const int64_t nslab = (n + P - 1) / P;
    const int64_t nw = (int64_t)gridDim.x * kSWarps;
    int64_t sc = (int64_t)blockIdx.x * kSWarps + wib;   // this warp's current slab
    if (sc >= nslab) return;
    if (lane32 == 0) {
        for (int k = 0; k < kSStages; ++k) mbar_init(bars + k, P);
        fence_mbar_init();
    }
    __syncwarp();
    const bool rs = respect_status != 0;
    auto item_of = [&](int64_t slab) { return slab * P + sub; };
    auto desc_of = [&](int64_t slab) {
        const int64_t i = item_of(slab);
        return load_desc(desc, i < n ? i : 0);
    };
    // the current slab's descriptor and copy state; the next slab's copy
    // state (its rows are copied while this one computes); the slab after
    // that's descriptor (read ahead)
    ItemDesc dc = desc_of(sc), dn = desc_of(sc + nw), dnn = desc_of(sc + 2 * nw);
    SIss ic_ = s_iss<KIND>(b, dc, item_of(sc) < n, rs);
    SIss in_ = s_iss<KIND>(b, dn, item_of(sc + nw) < n, rs);
    int nch_cur = s_chunks<CH>(ic_), nch_nxt = s_chunks<CH>(in_);
    int iw = 0, ic = 0;   // next chunk to issue: slab (0 current, 1 next), chunk
    int qi = 0, qc = 0;   // chunks issued / consumed by this warp
    auto issue_more = [&]() {
        while (qi - qc < kSStages) {
            if (iw == 0 && ic >= nch_cur) {
                iw = 1;
                ic = 0;
            }
            if (iw == 1 && ic >= nch_nxt) break;   // the rest after the next rotation
            float* dst = ring + (qi % kSStages) * Geo::stage + sub * Geo::item;
            uint64_t* bar = bars + (qi % kSStages);
            if (leader) {
                if (iw == 0) s_issue<G, KIND, CH>(b, ic_, ic, dst, bar);
                else s_issue<G, KIND, CH>(b, in_, ic, dst, bar);
            }
            ++qi;
            ++ic;
        }
    };
    for (;;) {
        issue_more();   // this slab's rows (and the next's) in flight first
        SItem cur;
        s_load<G, KIND>(b, dc, item_of(sc) < n, l, rs, cur);
        float cv_[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cw_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const bool run = cur.live && cur.staged;
        const int C = run ? cur.s.C : 0;
        // outside accumulators (A: child v, B: child w) / inside running values
        ChildOut A, B;
        float pxa = 0.f, pxb = 0.f;
        float* row = nullptr;
        float dot = 0.f, mx = 0.f, s0 = 0.f, ss = 0.f;
        for (int c = 0; c < nch_cur; ++c) {
            issue_more();
            const int stg = qc % kSStages;
            if (!mbar_wait(b, bars + stg, (uint32_t)(qc / kSStages) & 1u)) {
                // gave up: wait (bounded) for this warp's copies in flight,
                // the stage waited on included, then leave
                for (int q = qc; q < qi; ++q)
                    mbar_drain(bars + (q % kSStages), (uint32_t)(q / kSStages) & 1u);
                return;
            }
            const float* st = ring + stg * Geo::stage + sub * Geo::item + l;
            const int j0 = c * CH;
            if (run && j0 < C) {
                const float* su = st;
                const float* sv = st + (KIND == 1 ? R : 0);
                const float* sw = st + (KIND == 1 ? 2 : 1) * R;
                Child& cv = cur.cv;
                Child& cw = cur.cw;
                const float4 bv = cur.bv, bw = cur.bw;
                if (c == 0) {   // slots 0 and 1: the item's heads
                    if (cv.row) { cv.s0 = sv[0] * cv.f; cv.ss = sv[G] * cv.f; }
                    if (cw.row) { cw.s0 = sw[0] * cw.f; cw.ss = sw[G] * cw.f; }
                    const float ev0 = edge0(bv, cv.s0, cv.D, cv.ss);
                    const float ew0 = edge0(bw, cw.s0, cw.D, cw.ss);
                    if (KIND == 1) {
                        const float o0 = su[0] * cur.fo, os = su[G] * cur.fo;
                        A.x0 = o0 * ew0; A.xs = os * cw.ss; A.X = cur.Xo + cw.X;
                        B.x0 = o0 * ev0; B.xs = os * cv.ss; B.X = cur.Xo + cv.X;
                        A.sumx = A.dot = A.mx = 0.f;
                        B.sumx = B.dot = B.mx = 0.f;
                        const int64_t ro = (int64_t)cur.s.goff + l;
                        A.orow = cv.row ? b.out_part + (int64_t)cur.d.v_ref * 8 + ro : nullptr;
                        B.orow = cw.row ? b.out_part + (int64_t)cur.d.w_ref * 8 + ro : nullptr;
                        pxa = bv.y * A.x0;
                        pxb = bw.y * B.x0;
                    } else {
                        row = b.in_part + (int64_t)cur.d.u_prow8 * 8 + cur.s.goff + l;
                        s0 = ev0 * ew0;
                        ss = cv.ss * cw.ss;
                        __stcg(row, s0);
                        __stcg(row + G, ss);
                        mx = fmaxf(s0, ss);
                        dot = 0.f;
                    }
                }
                const int jlo = max(j0, 2), jhi = min(j0 + CH, C);
                if (KIND == 1) {
#define LAML_S_OUT(VL, WL)                                                                     \
    s_outside_chunk<G, CH, VL, WL>(su, sv, sw, j0, jlo, jhi, cur.fo, cv, cw, bv, bw, cur.s.qrow,  \
                               pxa, pxb, A.orow, B.orow, A.sumx, A.dot, A.mx, B.sumx, B.dot,  \
                               B.mx)
                    switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {
                        case 0: LAML_S_OUT(false, false); break;
                        case 1: LAML_S_OUT(true, false); break;
                        case 2: LAML_S_OUT(false, true); break;
                        default: LAML_S_OUT(true, true); break;
                    }
#undef LAML_S_OUT
                } else {
#define LAML_S_IN(VL, WL) \
    s_inside_chunk<G, CH, VL, WL>(sv, sw, j0, jlo, jhi, cv, cw, bv, bw, cur.s.qrow, row, dot, mx)
                    switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {
                        case 0: LAML_S_IN(false, false); break;
                        case 1: LAML_S_IN(true, false); break;
                        case 2: LAML_S_IN(false, true); break;
                        default: LAML_S_IN(true, true); break;
                    }
#undef LAML_S_IN
                }
            }
            __syncwarp();
            ++qc;
        }
        // finish the slab's items
        if (KIND == 1) {
            if (run) {
                child_finish<G>(b, cur.s, cur.d.v, cur.cv, cur.bv, A, want_post != 0, cur.lroot,
                                cur.xroot, cv_);
                child_finish<G>(b, cur.s, cur.d.w, cur.cw, cur.bw, B, want_post != 0, cur.lroot,
                                cur.xroot, cw_);
            } else if (cur.live && cur.logm) {
                float tv[8], tw[8];
                const ItemDesc dl = cur.d;
                const SiteCtx sl = cur.s;
                const GroupCtx gl = cur.gc;
                outside_log_lane<G>(b, dl, sl, gl, want_post != 0, tv, tw);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    cv_[k] = tv[k];
                    cw_[k] = tw[k];
                }
            }
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1) {
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    cv_[k] += __shfl_xor_sync(kFull, cv_[k], off);
                    cw_[k] += __shfl_xor_sync(kFull, cw_[k], off);
                }
            }
            if (cur.valid && leader && __ldcg(b.tr_status + cur.d.tree) == LAML_TREE_ACTIVE) {
                write_counts<G>(b, cur.d.tree, cur.d.v, cur.d.g, cv_);
                write_counts<G>(b, cur.d.tree, cur.d.w, cur.d.g, cw_);
            }
        } else {
            if (run) {
                const int h = scale_exp(mx);
                const float f = pow2i(-h);
                const int X = cur.cv.X + cur.cw.X + h;
                const int64_t sr = (int64_t)cur.d.u_srow + cur.s.site;
                __stcg(b.in_h + sr, h);
                __stcg(b.in_x + sr, X);
                __stcg(b.in_dot + sr, dot * f);
                if (cur.d.flags & 4)
                    root_site_llh(b, cur.s.tree, cur.s.site, root_edge_logs(b, cur.s.tree),
                                  s0 * f, dot * f, ss * f, X);
            } else if (cur.live && cur.logm) {
                const ItemDesc dl = cur.d;
                const SiteCtx sl = cur.s;
                const GroupCtx gl = cur.gc;
                inside_log_item<G>(b, dl, sl, gl);
            }
        }
        // rotate: the next slab becomes current
        sc += nw;
        if (sc >= nslab) break;
        dc = dn;
        ic_ = in_;
        nch_cur = nch_nxt;
        dn = dnn;
        in_ = s_iss<KIND>(b, dn, item_of(sc + nw) < n, rs);
        nch_nxt = s_chunks<CH>(in_);
        dnn = desc_of(sc + 2 * nw);
        if (iw == 1) iw = 0;   // the issue position moves with the slab
        else { iw = 0; ic = 0; }
    }
}

// ---------------------------------------------------------------------------
// Wide levels on producer/consumer warp pairs.  The per-thread kernels wait
// on chains of dependent loads (descriptor -> group -> rows and scalars ->
// state loop) with every byte in flight held in registers; at the 80
// registers the outside item needs, 24 warps per SM keep DRAM about a third
// busy.  Here a producer warp reads each slab's descriptors (32 / G items)
// and per-site scalars one slab ahead and stores them into a slab header
// (two per pair, so one fills while the other is read), and has the
// bulk-copy engine move the slab's rows, CH state slots at a time, into a
// ring of S stages.  The consumer then waits on mbarriers only, and the row
// bytes in flight sit in shared memory.  (Bulk copies issued from several
// lanes of one instruction go out one lane at a time, so the per-site
// scalars, 32 bytes per array and item, are moved by plain loads instead.)
// Every thread's arithmetic is the per-thread kernels' (the same chunk loops
// and child_finish), so the results are bitwise equal.
//
// Header of one item (ints; written by the producer's plain stores, released
// to the consumer by the header's mbarrier):
//   [0, 12) descriptor, [12, 20) group descriptor, [20, 24) status, mode,
//   the group's slot count, valid | staged << 1; [24, 28) leaf terms e1,
//   ephi, es; [32, 36) and [36, 40) branch terms of v and w; from 40 twelve
//   G-int slots: parent's out_h, out_x; v's in_h (its codes when a leaf),
//   in_x, in_dot; w's likewise; root_lr, root_x; site_C, site_sumq.
// ---------------------------------------------------------------------------
constexpr int kPcPairs = 4;     // producer/consumer warp pairs per block
constexpr int kPcMinBlocks = 2; // resident blocks per SM asked (<= 128 registers)

template <int G, int NR, int CH>
struct PGeom {
    static constexpr int P = 32 / G;                 // items per slab
    static constexpr int S = CH <= 8 ? 4 : 3;        // stages per pair
    static constexpr int row = CH * G;               // floats of one row's chunk
    static constexpr int item = NR * row + G;        // + G floats: items start G banks apart
    static constexpr int stage = P * item;
    static constexpr int HI = 40 + 12 * G;           // header ints per item
    static constexpr int hdr = P * HI;
    static constexpr size_t pair_floats = (size_t)S * stage + 2 * hdr;
    static constexpr int nbar = 2 * S + 4;           // full[S], empty[S], hfull[2], hempty[2]
    static constexpr size_t block_bytes =
        kPcPairs * (pair_floats * sizeof(float) + nbar * sizeof(uint64_t));
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}"
                 ::"r"(smem_u32(bar))
                 : "memory");
}

// a phase wait that sleeps between tries (32 ns doubling to kPcSleepNs), so
// that a warp waiting on its partner leaves the issue slots to the warps
// with work; bounded by the batch's wait limit like mbar_wait
constexpr uint32_t kPcSuspendNs = 20000;
constexpr unsigned kPcSleepNs = 512;

__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity), "r"(kPcSuspendNs)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool pc_wait(const laml_batch& b, uint64_t* bar, uint32_t parity) {
    const long long lim = wait_limit(b);
    if (lim < 0) {   // one check, without suspending
        if (mbar_test_wait(bar, parity)) return true;
        atomicCAS(b.error, 0, LAML_ERR_TIMEOUT);
        return false;
    }
    if (mbar_try_wait_hint(bar, parity)) return true;
    const unsigned long long t0 = gtimer();
    unsigned ns = 32;
    for (uint32_t it = 0; it < (1u << 26); ++it) {
        __nanosleep(ns);
        if (ns < kPcSleepNs) ns <<= 1;
        if (mbar_try_wait_hint(bar, parity)) return true;
        if ((long long)(gtimer() - t0) > lim) break;
    }
    atomicCAS(b.error, 0, LAML_ERR_TIMEOUT);
    return false;
}

// the producer's view of one item of a slab: its descriptor, group, tree
// state and leaf terms (read one slab ahead), then this lane's site's
// scalars and the branch terms (read while the slab before is issued)
struct PItem {
    ItemDesc d;
    int4 G1, G2;
    int Cg, status, mode, tsite;
    float e1, ephi, es;
    bool valid, staged;
    int sc[12];      // the header's per-site slots at this lane's site
    float4 bt;       // lane 0: v's branch terms, lane 1: w's
};

template <int KIND>
__device__ __forceinline__ void pc_fetch(const laml_batch& b, const int32_t* desc, int64_t n,
                                         bool rs, int64_t it, PItem& t) {
    t.valid = it < n;
    t.d = load_desc(desc, t.valid ? it : 0);
    const int4* gp = reinterpret_cast<const int4*>(b.grp_desc) + 2 * t.d.gd;
    t.G1 = __ldg(gp);
    t.G2 = __ldg(gp + 1);
    t.Cg = __ldg(b.group_C + t.d.gd);
    t.status = __ldcg(b.tr_status + t.d.tree);
    t.mode = __ldcg(b.tr_mode + t.d.tree);
    t.tsite = KIND == 1 ? __ldg(b.tr_site_base + t.d.tree) : 0;
    const Leaf L = leaf_params(b, t.d.tree);
    t.e1 = L.e1;
    t.ephi = L.ephi;
    t.es = L.es;
    const bool active = t.valid && (!(KIND == 1 || rs) || t.status == LAML_TREE_ACTIVE);
    t.staged = active && t.mode != LAML_MODE_LOG;
}

// slot k of the header at lane l's site: parent's out_h, out_x; v's in_h
// (its code when a leaf), in_x, in_dot; w's likewise; root_lr, root_x;
// site_C, site_sumq
template <int G, int KIND>
__device__ __forceinline__ void pc_scalars(const laml_batch& b, int l, PItem& t) {
    if (!t.staged) return;
    const ItemDesc& d = t.d;
    const int s = d.g * G + l;
    const bool vl = d.flags & 1, wl = d.flags & 2;
    if (KIND == 1) {
        t.sc[0] = __ldcg(b.out_h + (int64_t)d.u_srow + s);
        t.sc[1] = __ldcg(b.out_x + (int64_t)d.u_srow + s);
        t.sc[8] = __float_as_int(__ldcg(b.root_lr + (int64_t)t.tsite + s));
        t.sc[9] = __ldcg(b.root_x + (int64_t)t.tsite + s);
    }
    if (vl) {
        t.sc[2] = __ldg(b.codes + t.G2.x + (int64_t)d.v_ref * t.G2.y + s);
    } else {
        t.sc[2] = __ldcg(b.in_h + (int64_t)d.v_srow + s);
        t.sc[3] = __ldcg(b.in_x + (int64_t)d.v_srow + s);
        t.sc[4] = __float_as_int(__ldcg(b.in_dot + (int64_t)d.v_srow + s));
    }
    if (wl) {
        t.sc[5] = __ldg(b.codes + t.G2.x + (int64_t)d.w_ref * t.G2.y + s);
    } else {
        t.sc[5] = __ldcg(b.in_h + (int64_t)d.w_srow + s);
        t.sc[6] = __ldcg(b.in_x + (int64_t)d.w_srow + s);
        t.sc[7] = __float_as_int(__ldcg(b.in_dot + (int64_t)d.w_srow + s));
    }
    t.sc[10] = __ldg(b.site_C + t.G1.y + l);
    t.sc[11] = __float_as_int(__ldg(b.site_sumq + t.G1.y + l));
    if (l < 2) t.bt = load_bt(b, l == 0 ? d.v : d.w);
}

// the slab's largest staged slot count over CH (every lane of the warp)
template <int CH>
__device__ __forceinline__ int pc_chunks(bool staged, int Cg) {
    const int m = __reduce_max_sync(kFull, staged ? Cg : 0);
    return (m + CH - 1) / CH;
}

// producer warp of a pair: headers (plain stores) and row chunks (bulk
// copies) of the pair's slabs
template <int G, int KIND, int CH>
__device__ void pc_produce(const laml_batch& b, const int32_t* desc, int64_t n, bool rs,
                           int64_t pid, int64_t npairs, float* ring, int* hdr, uint64_t* bars) {
    using Geo = PGeom<G, KIND == 1 ? 3 : 2, CH>;
    constexpr int P = Geo::P, S = Geo::S, R = Geo::row;
    uint64_t* full = bars;
    uint64_t* empty = bars + S;
    uint64_t* hfull = bars + 2 * S;
    uint64_t* hempty = bars + 2 * S + 2;
    const int lane32 = threadIdx.x & 31, sub = lane32 / G, l = lane32 % G;
    const int64_t nslab = (n + P - 1) / P;
    int64_t q = 0, kh = 0;   // stages issued, headers written
    PItem t, tn;
    if (pid < nslab) {
        pc_fetch<KIND>(b, desc, n, rs, pid * P + sub, t);
        pc_scalars<G, KIND>(b, l, t);
    }
    for (int64_t slab = pid; slab < nslab; slab += npairs) {
        const bool more = slab + npairs < nslab;
        // the next slab's items load while this one goes out
        if (more) pc_fetch<KIND>(b, desc, n, rs, (slab + npairs) * P + sub, tn);
        // header kh & 1 of the pair: wait until its consumer has read it
        const int h = (int)(kh & 1);
        if (!pc_wait(b, hempty + h, (uint32_t)((kh >> 1) & 1) ^ 1u)) break;
        int* H = hdr + h * Geo::hdr + sub * Geo::HI;
        const ItemDesc& d = t.d;
        if (l == 0) reinterpret_cast<int4*>(H)[0] = make_int4(d.u, d.v, d.w, d.tree | (d.flags << 24));
        if (l == 1) reinterpret_cast<int4*>(H)[1] = make_int4(d.g, d.gd, d.u_srow, d.u_prow8);
        if (l == 2) reinterpret_cast<int4*>(H)[2] = make_int4(d.v_ref, d.w_ref, d.v_srow, d.w_srow);
        if (l == 3) reinterpret_cast<int4*>(H)[3] = t.G1;
        if (l == 4) reinterpret_cast<int4*>(H)[4] = t.G2;
        if (l == 5) reinterpret_cast<int4*>(H)[5] =
            make_int4(t.status, t.mode, t.Cg, (t.valid ? 1 : 0) | (t.staged ? 2 : 0));
        if (l == 6) reinterpret_cast<float4*>(H)[6] = make_float4(t.e1, t.ephi, t.es, 0.f);
        if (t.staged) {
            if (l < 2) reinterpret_cast<float4*>(H)[8 + l] = t.bt;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (k == 2 && (d.flags & 1))
                    reinterpret_cast<int16_t*>(H + 40 + 2 * G)[l] = (int16_t)t.sc[2];
                else if (k == 5 && (d.flags & 2))
                    reinterpret_cast<int16_t*>(H + 40 + 5 * G)[l] = (int16_t)t.sc[5];
                else
                    H[40 + k * G + l] = t.sc[k];
            }
        }
        __syncwarp();
        if (lane32 == 0) mbar_arrive(hfull + h);   // releases the header's stores
        ++kh;
        // the rows, CH slots per stage: lane l < NR of each item copies row
        // l -- the parent's outside row (outside only), then the internal
        // children's inside rows
        const float* rsrc = nullptr;
        if (t.staged) {
            const int64_t off = t.G1.x;
            if (KIND == 1) {
                if (l == 0) rsrc = b.out_part + (int64_t)d.u_prow8 * 8 + off;
                if (l == 1 && !(d.flags & 1)) rsrc = b.in_part + (int64_t)d.v_ref * 8 + off;
                if (l == 2 && !(d.flags & 2)) rsrc = b.in_part + (int64_t)d.w_ref * 8 + off;
            } else {
                if (l == 0 && !(d.flags & 1)) rsrc = b.in_part + (int64_t)d.v_ref * 8 + off;
                if (l == 1 && !(d.flags & 2)) rsrc = b.in_part + (int64_t)d.w_ref * 8 + off;
            }
        }
        float* rdst = ring + sub * Geo::item + l * R;
        const int nch = pc_chunks<CH>(t.staged, t.Cg);
        bool ok = true;
        for (int c = 0; c < nch; ++c) {
            const int st = (int)(q % S);
            if (!pc_wait(b, empty + st, (uint32_t)((q / S) & 1) ^ 1u)) { ok = false; break; }
            const int j0 = c * CH;
            const int ns = rsrc ? min(CH, t.Cg - j0) : 0;
            const uint32_t by = ns > 0 ? (uint32_t)ns * G * 4u : 0u;
            const uint32_t stot = __reduce_add_sync(kFull, by);
            __syncwarp();
            if (lane32 == 0) mbar_arrive_tx(full + st, stot);
            __syncwarp();
            if (by) bulk_g2s(rdst + st * Geo::stage, rsrc + (int64_t)j0 * G, by, full + st);
            ++q;
        }
        if (!ok) break;
        if (more) {
            t = tn;
            pc_scalars<G, KIND>(b, l, t);
        }
    }
    // every copy this warp started lands before the block may exit: the
    // last S stages (bounded waits)
    if (lane32 == 0)
        for (int64_t qq = (q > S ? q - S : 0); qq < q; ++qq)
            mbar_drain(full + (qq % S), (uint32_t)((qq / S) & 1));
    __syncwarp();
}

// consumer warp of a pair
template <int G, int KIND, int CH>
__device__ void pc_consume(const laml_batch& b, const int32_t* desc, int64_t n, bool rs,
                           bool want_post, int64_t pid, int64_t npairs, const float* ring,
                           const int* hdr, uint64_t* bars) {
    using Geo = PGeom<G, KIND == 1 ? 3 : 2, CH>;
    constexpr int P = Geo::P, S = Geo::S, R = Geo::row;
    uint64_t* full = bars;
    uint64_t* empty = bars + S;
    uint64_t* hfull = bars + 2 * S;
    uint64_t* hempty = bars + 2 * S + 2;
    const int lane32 = threadIdx.x & 31, sub = lane32 / G, l = lane32 % G;
    const bool leader = l == 0;
    const int64_t nslab = (n + P - 1) / P;
    int64_t q = 0, k = 0;
    for (int64_t slab = pid; slab < nslab; slab += npairs, ++k) {
        const int h = (int)(k & 1);
        if (!pc_wait(b, hfull + h, (uint32_t)((k >> 1) & 1))) return;
        const int* H = hdr + h * Geo::hdr + sub * Geo::HI;
        SItem cur;
        {
            const int4 A = reinterpret_cast<const int4*>(H)[0];
            const int4 B = reinterpret_cast<const int4*>(H)[1];
            const int4 C = reinterpret_cast<const int4*>(H)[2];
            ItemDesc& d = cur.d;
            d.u = A.x; d.v = A.y; d.w = A.z;
            d.tree = A.w & 0xffffff;
            d.flags = (int)((unsigned)A.w >> 24);
            d.g = B.x; d.gd = B.y; d.u_srow = B.z; d.u_prow8 = B.w;
            d.v_ref = C.x; d.w_ref = C.y; d.v_srow = C.z; d.w_srow = C.w;
        }
        const int4 G1 = reinterpret_cast<const int4*>(H)[3];
        const int4 G2 = reinterpret_cast<const int4*>(H)[4];
        const int4 X = reinterpret_cast<const int4*>(H)[5];
        cur.valid = X.w & 1;
        cur.staged = (X.w & 2) != 0;
        cur.Cg = X.z;
        cur.logm = cur.valid && X.y == LAML_MODE_LOG;
        const bool act_ok = !(KIND == 1 || rs) || X.x == LAML_TREE_ACTIVE;
        if (cur.staged) {
            SiteCtx& s = cur.s;
            s.tree = cur.d.tree;
            s.site = cur.d.g * G + l;
            cur.live = s.site < G2.z;
            s.goff = G1.x;
            s.ds = G1.w;
            s.C = H[40 + 10 * G + l];
            s.sumq = __int_as_float(H[40 + 11 * G + l]);
            s.qrow = b.q + G1.z + l;
            cur.gc.code_base = G2.x;
            cur.gc.kpad = G2.y;
            const float4 Lf = reinterpret_cast<const float4*>(H)[6];
            Leaf L;
            L.e1 = Lf.x; L.ephi = Lf.y; L.es = Lf.z;
            auto child = [&](bool leaf, int base) {
                Child c;
                c.e1 = L.e1;
                c.ephi = L.ephi;
                if (leaf) {
                    const int code = reinterpret_cast<const int16_t*>(H + base)[l];
                    c.row = nullptr;
                    c.f = 1.f;
                    c.X = 0;
                    c.code = code;
                    c.s0 = code == 0 ? L.e1 : (code == -1 ? L.ephi : 0.f);
                    c.ss = code < 0 ? 1.f : L.es;
                    c.D = code >= 2 ? __ldg(s.qrow + code * G) * L.e1
                                    : (code == -1 ? L.ephi * s.sumq : 0.f);
                } else {
                    c.f = pow2i(-H[base + l]);
                    c.X = H[base + G + l];
                    c.D = __int_as_float(H[base + 2 * G + l]);
                    c.row = b.in_part;   // marks an internal child; its slots come from the stages
                    c.code = 0;
                    c.s0 = c.ss = 0.f;
                }
                return c;
            };
            if (cur.live) {
                cur.cv = child(cur.d.flags & 1, 40 + 2 * G);
                cur.cw = child(cur.d.flags & 2, 40 + 5 * G);
                cur.bv = reinterpret_cast<const float4*>(H)[8];
                cur.bw = reinterpret_cast<const float4*>(H)[9];
                if (KIND == 1) {
                    cur.fo = pow2i(-H[40 + l]);
                    cur.Xo = H[40 + G + l];
                    cur.lroot = __int_as_float(H[40 + 8 * G + l]);
                    cur.xroot = H[40 + 9 * G + l];
                }
            }
        } else {
            cur.live = cur.valid && act_ok && site_ctx_d<G>(b, cur.d, l, KIND == 1 || rs, cur.s, cur.gc);
        }
        // the header is read: hand it back (generic reads before the next
        // bulk writes into it)
        fence_proxy_async_smem();
        __syncwarp();
        if (lane32 == 0) mbar_arrive(hempty + h);
        float cv_[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cw_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const bool run = cur.live && cur.staged;
        const int C = run ? cur.s.C : 0;
        ChildOut A, B;
        float pxa = 0.f, pxb = 0.f;
        float* row = nullptr;
        float dot = 0.f, mx = 0.f, s0 = 0.f, ss = 0.f;
        const int nch = pc_chunks<CH>(cur.staged, cur.Cg);
        for (int c = 0; c < nch; ++c, ++q) {
            const int stg = (int)(q % S);
            if (!pc_wait(b, full + stg, (uint32_t)((q / S) & 1))) return;
            const float* st = ring + stg * Geo::stage + sub * Geo::item + l;
            const int j0 = c * CH;
            if (run && j0 < C) {
                const float* su = st;
                const float* sv = st + (KIND == 1 ? R : 0);
                const float* sw = st + (KIND == 1 ? 2 : 1) * R;
                Child& cv = cur.cv;
                Child& cw = cur.cw;
                const float4 bv = cur.bv, bw = cur.bw;
                if (c == 0) {   // slots 0 and 1: the item's heads
                    if (cv.row) { cv.s0 = sv[0] * cv.f; cv.ss = sv[G] * cv.f; }
                    if (cw.row) { cw.s0 = sw[0] * cw.f; cw.ss = sw[G] * cw.f; }
                    const float ev0 = edge0(bv, cv.s0, cv.D, cv.ss);
                    const float ew0 = edge0(bw, cw.s0, cw.D, cw.ss);
                    if (KIND == 1) {
                        const float o0 = su[0] * cur.fo, os = su[G] * cur.fo;
                        A.x0 = o0 * ew0; A.xs = os * cw.ss; A.X = cur.Xo + cw.X;
                        B.x0 = o0 * ev0; B.xs = os * cv.ss; B.X = cur.Xo + cv.X;
                        A.sumx = A.dot = A.mx = 0.f;
                        B.sumx = B.dot = B.mx = 0.f;
                        const int64_t ro = (int64_t)cur.s.goff + l;
                        A.orow = cv.row ? b.out_part + (int64_t)cur.d.v_ref * 8 + ro : nullptr;
                        B.orow = cw.row ? b.out_part + (int64_t)cur.d.w_ref * 8 + ro : nullptr;
                        pxa = bv.y * A.x0;
                        pxb = bw.y * B.x0;
                    } else {
                        row = b.in_part + (int64_t)cur.d.u_prow8 * 8 + cur.s.goff + l;
                        s0 = ev0 * ew0;
                        ss = cv.ss * cw.ss;
                        __stcg(row, s0);
                        __stcg(row + G, ss);
                        mx = fmaxf(s0, ss);
                        dot = 0.f;
                    }
                }
                const int jlo = max(j0, 2), jhi = min(j0 + CH, C);
                if (KIND == 1) {
#define LAML_P_OUT(VL, WL)                                                                     \
    s_outside_chunk<G, CH, VL, WL>(su, sv, sw, j0, jlo, jhi, cur.fo, cv, cw, bv, bw, cur.s.qrow,  \
                               pxa, pxb, A.orow, B.orow, A.sumx, A.dot, A.mx, B.sumx, B.dot,  \
                               B.mx)
                    switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {
                        case 0: LAML_P_OUT(false, false); break;
                        case 1: LAML_P_OUT(true, false); break;
                        case 2: LAML_P_OUT(false, true); break;
                        default: LAML_P_OUT(true, true); break;
                    }
#undef LAML_P_OUT
                } else {
#define LAML_P_IN(VL, WL) \
    s_inside_chunk<G, CH, VL, WL>(sv, sw, j0, jlo, jhi, cv, cw, bv, bw, cur.s.qrow, row, dot, mx)
                    switch ((cv.row ? 0 : 1) | (cw.row ? 0 : 2)) {
                        case 0: LAML_P_IN(false, false); break;
                        case 1: LAML_P_IN(true, false); break;
                        case 2: LAML_P_IN(false, true); break;
                        default: LAML_P_IN(true, true); break;
                    }
#undef LAML_P_IN
                }
            }
            // the stage is read: hand it back to the producer
            fence_proxy_async_smem();
            __syncwarp();
            if (lane32 == 0) mbar_arrive(empty + stg);
        }
        // finish the slab's items
        if (KIND == 1) {
            if (run) {
                child_finish<G>(b, cur.s, cur.d.v, cur.cv, cur.bv, A, want_post, cur.lroot,
                                cur.xroot, cv_);
                child_finish<G>(b, cur.s, cur.d.w, cur.cw, cur.bw, B, want_post, cur.lroot,
                                cur.xroot, cw_);
            } else if (cur.live && cur.logm) {
                float tv[8], tw[8];
                const ItemDesc dl = cur.d;
                const SiteCtx sl = cur.s;
                const GroupCtx gl = cur.gc;
                outside_log_lane<G>(b, dl, sl, gl, want_post, tv, tw);
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    cv_[kk] = tv[kk];
                    cw_[kk] = tw[kk];
                }
            }
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1) {
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    cv_[kk] += __shfl_xor_sync(kFull, cv_[kk], off);
                    cw_[kk] += __shfl_xor_sync(kFull, cw_[kk], off);
                }
            }
            if (cur.valid && leader && X.x == LAML_TREE_ACTIVE) {
                write_counts<G>(b, cur.d.tree, cur.d.v, cur.d.g, cv_);
                write_counts<G>(b, cur.d.tree, cur.d.w, cur.d.g, cw_);
            }
        } else {
            if (run) {
                const int hh = scale_exp(mx);
                const float f = pow2i(-hh);
                const int Xs = cur.cv.X + cur.cw.X + hh;
                const int64_t sr = (int64_t)cur.d.u_srow + cur.s.site;
                __stcg(b.in_h + sr, hh);
                __stcg(b.in_x + sr, Xs);
                __stcg(b.in_dot + sr, dot * f);
                if (cur.d.flags & 4)
                    root_site_llh(b, cur.s.tree, cur.s.site, root_edge_logs(b, cur.s.tree),
                                  s0 * f, dot * f, ss * f, Xs);
            } else if (cur.live && cur.logm) {
                const ItemDesc dl = cur.d;
                const SiteCtx sl = cur.s;
                const GroupCtx gl = cur.gc;
                inside_log_item<G>(b, dl, sl, gl);
            }
        }
    }
}

template <int G, int KIND, int CH>
__global__ void __launch_bounds__(kPcPairs * 64, kPcMinBlocks) k_items_pc(laml_batch b,
                                                                          const int32_t* desc,
                                                                          int64_t n,
                                                                          int want_post,
                                                                          int respect_status) {
    using Geo = PGeom<G, KIND == 1 ? 3 : 2, CH>;
    extern __shared__ __align__(128) unsigned char psm[];
    const int wib = threadIdx.x >> 5;
    const int pair = wib % kPcPairs;
    const bool producer = wib >= kPcPairs;
    float* base = reinterpret_cast<float*>(psm) + (size_t)pair * Geo::pair_floats;
    float* ring = base;
    int* hdr = reinterpret_cast<int*>(base + (size_t)Geo::S * Geo::stage);
    uint64_t* bars = reinterpret_cast<uint64_t*>(psm + kPcPairs * Geo::pair_floats * sizeof(float)) +
                     pair * Geo::nbar;
    if ((threadIdx.x & 31) == 0 && !producer) {
        for (int k = 0; k < Geo::nbar; ++k) mbar_init(bars + k, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int64_t pid = (int64_t)blockIdx.x * kPcPairs + pair;
    const int64_t npairs = (int64_t)gridDim.x * kPcPairs;
    if (producer)
        pc_produce<G, KIND, CH>(b, desc, n, respect_status != 0, pid, npairs, ring, hdr, bars);
    else
        pc_consume<G, KIND, CH>(b, desc, n, respect_status != 0, want_post != 0, pid, npairs,
                                ring, hdr, bars);
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
template <int G, int KIND, bool AS = false>
__device__ __forceinline__ void for_items(const laml_batch& b, const int32_t* items, int64_t n,
                                          int gwarp, int nwarps, bool want_post,
                                          bool respect_status, const int32_t* desc = nullptr,
                                          float* sm = nullptr) {
    constexpr int kind = KIND;
    if constexpr (KIND <= 1) {
        if (narrow_level(n)) {   // one item per warp: the shortest latency per item
            const int lane = threadIdx.x & 31;
            for (int64_t it = gwarp; it < n; it += nwarps) {
                const WItem t = witem(wload_grp(b, wload_desc(desc, it, lane), lane));
                witem_run<G, KIND, false>(b, t, nullptr, 0, lane, want_post, respect_status,
                                          nullptr, 0);
            }
            return;
        }
    }
    constexpr int IPW = 32 / G;
    const int lane32 = threadIdx.x & 31, lane = lane32 % G, sub = lane32 / G;
    // a level's items are int32-indexed (the plan's level offsets are int32)
    const int n32 = (int)n;
    const int nw = (n32 + IPW - 1) / IPW;
    for (int wi = gwarp; wi < nw; wi += nwarps) {
        const int it = wi * IPW + sub;
        const bool act = it < n32;
        if constexpr (KIND <= 1 || KIND == 5) {   // descriptor-driven inside / outside
            const ItemDesc d = load_desc(desc, act ? it : 0);
            if constexpr (KIND == 0) {
                if (act) inside_item_d<G, AS>(b, d, lane, respect_status, sm);
            } else if constexpr (KIND == 1) {
                outside_item_d<G, AS>(b, d, lane, act, want_post, sm);
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

template <int G, int KIND, int MB = KIND == 1 ? 8 : LAML_MINB_IN>
__global__ void __launch_bounds__(kItemsBlock, MB) k_items(laml_batch b, const int32_t* items, int64_t n,
                                                   int want_post, int respect_status,
                                                   const int32_t* desc) {
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    if constexpr (KIND <= 1) {   // wide levels stage their state loops (dynamic shared memory)
        extern __shared__ float ksm[];
        for_items<G, KIND, true>(b, items, n, gwarp, nwarps, want_post != 0, respect_status != 0,
                                 desc, ksm);
    } else {
        for_items<G, KIND>(b, items, n, gwarp, nwarps, want_post != 0, respect_status != 0, desc);
    }
}

// M-step, one block per tree; with skip_big the trees above kClusterNodes
// nodes are left to k_mstep_cluster
__global__ void __launch_bounds__(kBlock, 4) k_mstep(laml_batch b, int rounds, int flags,
                                                    int skip_big, int ucap) {
    __shared__ double2 sh[kBlock / 32];
    __shared__ float4 s_cnt[kMstepStage];
    __shared__ float s_d[kMstepStage];
    extern __shared__ double usm[];   // ultrametric solve: 8 slots for trees up to ucap nodes
    BlockTeam T{sh};
    for (int p = blockIdx.x; p < b.n_trees; p += gridDim.x) {
        if (skip_big && __ldg(b.tr_nodes + p) > kClusterNodes) continue;
        mstep_tree(b, p, rounds, T, s_cnt, s_d, flags, ucap > 0 ? usm : nullptr, ucap);
    }
}

// M-step of the trees above kClusterNodes nodes, one cluster of
// kMstepCluster blocks per tree
__global__ void __cluster_dims__(kMstepCluster, 1, 1) __launch_bounds__(kMstepClusterThreads, 1)
    k_mstep_cluster(laml_batch b, int rounds, int flags) {
    __shared__ double2 sh[kMstepClusterThreads / 32];
    __shared__ double2 part[kMstepCluster];
    ClusterTeam T{sh, part};
    const int ncl = gridDim.x / kMstepCluster;
    for (int p = blockIdx.x / kMstepCluster; p < b.n_trees; p += ncl) {
        if (__ldg(b.tr_nodes + p) <= kClusterNodes) continue;   // uniform over the cluster
        mstep_tree(b, p, rounds, T, nullptr, nullptr, flags);
    }
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
    if (b.tr_leaf && i < b.n_trees)
        reinterpret_cast<float2*>(b.tr_leaf)[i] = leaf_pair(b.tr_phi[i], b.compat);
}

// Item descriptors from the node arrays already on the device: the same 12
// int32 per item that laml_plan_fill writes on the host, three 16-byte stores.
__device__ __forceinline__ void item_desc(const laml_batch& b, int u, int g, int64_t k,
                                          int32_t* __restrict__ desc) {
    {
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

__global__ void k_item_desc(laml_batch b, const int32_t* __restrict__ items, int64_t n,
                            int32_t* __restrict__ desc) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        item_desc(b, items[2 * k], items[2 * k + 1], k, desc);
}

// The same descriptors from the level node lists (every dataset with NG
// groups): item k of level l, with item offset o_l and c_l = (o_{l+1} - o_l)
// / NG nodes, is node lnodes[o_l / NG + (k - o_l) % c_l] of group
// (k - o_l) / c_l -- the plan's group-major order within a level.
__global__ void k_item_desc_nodes(laml_batch b, const int32_t* __restrict__ lnodes,
                                  const int32_t* __restrict__ level_off, int n_levels, int64_t n,
                                  int32_t* __restrict__ desc) {
    const int NG = b.ds_groups[0];
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_levels;   // the level: level_off[lo] <= k < level_off[lo + 1]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (level_off[mid] <= k) lo = mid; else hi = mid;
        }
        const int64_t o = level_off[lo];
        const int64_t c = (level_off[lo + 1] - o) / NG;
        const int64_t r = k - o;
        const int64_t g = r / c;
        item_desc(b, lnodes[o / NG + (r - g * c)], (int)g, k, desc);
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
    BlockTeam T{sh};   // one block per tree here, whatever its size
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
            mstep_tree(b, p, rounds, T, s_cnt, s_d, flags);
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
    if (b->wide_chunk != 0 && b->wide_chunk != 8 && b->wide_chunk != 16) {
        laml::set_error("laml_batch: wide_chunk must be 0, 8 or 16");
        return LAML_ERR_ARG;
    }
    if (b->wide_pc && ((((uintptr_t)b->in_part) | ((uintptr_t)b->out_part)) & 15u) != 0) {
        // the bulk copies of rows start on 16-byte boundaries
        laml::set_error("laml_batch: wide_pc needs 16-byte aligned in_part and out_part");
        return LAML_ERR_ARG;
    }
    return LAML_OK;
}

// an M-step flag set the batch cannot serve
int validate_mstep_flags(const laml_batch* b, int32_t flags, const char* who) {
    if ((flags & LAML_MSTEP_LBFGS) && b->compat && !b->nd_lbfgs) {
        laml::set_error(std::string(who) + ": LAML_MSTEP_LBFGS needs nd_lbfgs");
        return LAML_ERR_ARG;
    }
    if ((flags & LAML_MSTEP_ULTRAMETRIC) && !b->compat && (!b->nd_uorder || !b->nd_uwork)) {
        laml::set_error(std::string(who) + ": LAML_MSTEP_ULTRAMETRIC needs nd_uorder and nd_uwork");
        return LAML_ERR_ARG;
    }
    return LAML_OK;
}

// shared memory of a staged level kernel: per warp two buffers of NR rows of
// max_states * G floats, then two 8-byte mbarriers per warp
size_t staged_smem(const laml_batch& b, int kind) {
    const size_t NR = kind == 1 ? 3 : 2;
    return (size_t)kWWarps * (2 * NR * (size_t)b.max_states * b.group_sites * sizeof(float) + 16);
}

constexpr size_t kStagedSmemMax = 200 * 1024;

template <int G, int KIND>
int launch_staged(const laml_batch& b, const int32_t* desc, int64_t n, int want_post,
                  int respect_status, cudaStream_t st) {
    static bool attr_set = false;   // per process: the opt-in limit is a function attribute
    if (!attr_set) {
        int rc = check(cudaFuncSetAttribute(k_items_w<G, KIND>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kStagedSmemMax),
                       "staged kernel shared memory limit");
        if (rc) return rc;
        attr_set = true;
    }
    const size_t smem = staged_smem(b, KIND);
    int per_sm = 0;
    int rc = check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_items_w<G, KIND>,
                                                                 kWWarps * 32, smem),
                   "staged kernel occupancy");
    if (rc) return rc;
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = (n + kWWarps - 1) / kWWarps;
    const int64_t cap = (int64_t)per_sm * num_sms();
    if (blocks > cap) blocks = cap;
    k_items_w<G, KIND><<<(unsigned)blocks, kWWarps * 32, smem, st>>>(b, desc, n, b.max_states,
                                                                     want_post, respect_status);
    return check(cudaGetLastError(), "k_items_w launch");
}

template <int G, int KIND, int CH>
int launch_staged_wide_t(const laml_batch& b, const int32_t* desc, int64_t n, int want_post,
                         int respect_status, cudaStream_t st) {
    using Geo = SGeom<G, KIND == 1 ? 3 : 2, CH>;
    static bool attr_set = false;
    if (!attr_set) {
        int rc = check(cudaFuncSetAttribute(k_items_ws<G, KIND, CH>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)Geo::block_bytes),
                       "staged wide kernel shared memory limit");
        if (rc) return rc;
        attr_set = true;
    }
    static int per_sm = 0;
    if (!per_sm) {
        int rc = check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &per_sm, k_items_ws<G, KIND, CH>, kSWarps * 32, Geo::block_bytes),
                       "staged wide kernel occupancy");
        if (rc) return rc;
        if (per_sm < 1) per_sm = 1;
    }
    const int64_t slabs = (n + Geo::P - 1) / Geo::P;
    int64_t blocks = (slabs + kSWarps - 1) / kSWarps;
    const int64_t cap = (int64_t)per_sm * num_sms();
    if (blocks > cap) blocks = cap;
    k_items_ws<G, KIND, CH><<<(unsigned)blocks, kSWarps * 32, Geo::block_bytes, st>>>(
        b, desc, n, want_post, respect_status);
    return check(cudaGetLastError(), "k_items_ws launch");
}

template <int G, int KIND>
int launch_staged_wide(const laml_batch& b, const int32_t* desc, int64_t n, int want_post,
                       int respect_status, cudaStream_t st) {
    if (b.wide_chunk == 8)
        return launch_staged_wide_t<G, KIND, 8>(b, desc, n, want_post, respect_status, st);
    return launch_staged_wide_t<G, KIND, 16>(b, desc, n, want_post, respect_status, st);
}

template <int G, int KIND, int CH>
int launch_pc_wide_t(const laml_batch& b, const int32_t* desc, int64_t n, int want_post,
                     int respect_status, cudaStream_t st) {
    using Geo = PGeom<G, KIND == 1 ? 3 : 2, CH>;
    static bool attr_set = false;
    if (!attr_set) {
        int rc = check(cudaFuncSetAttribute(k_items_pc<G, KIND, CH>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)Geo::block_bytes),
                       "producer/consumer kernel shared memory limit");
        if (rc) return rc;
        attr_set = true;
    }
    static int per_sm = 0;
    if (!per_sm) {
        int rc = check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &per_sm, k_items_pc<G, KIND, CH>, kPcPairs * 64, Geo::block_bytes),
                       "producer/consumer kernel occupancy");
        if (rc) return rc;
        if (per_sm < 1) per_sm = 1;
    }
    const int64_t slabs = (n + Geo::P - 1) / Geo::P;
    int64_t blocks = (slabs + kPcPairs - 1) / kPcPairs;
    const int64_t cap = (int64_t)per_sm * num_sms();
    if (blocks > cap) blocks = cap;
    k_items_pc<G, KIND, CH><<<(unsigned)blocks, kPcPairs * 64, Geo::block_bytes, st>>>(
        b, desc, n, want_post, respect_status);
    return check(cudaGetLastError(), "k_items_pc launch");
}

template <int G, int KIND>
int launch_pc_wide(const laml_batch& b, const int32_t* desc, int64_t n, int want_post,
                   int respect_status, cudaStream_t st) {
    if (b.wide_chunk == 16)
        return launch_pc_wide_t<G, KIND, 16>(b, desc, n, want_post, respect_status, st);
    return launch_pc_wide_t<G, KIND, 8>(b, desc, n, want_post, respect_status, st);
}

template <int G>
int launch_items(const laml_batch& b, const int32_t* items, int64_t n, int kind, int want_post,
                 int respect_status, cudaStream_t st, const int32_t* desc = nullptr) {
    if (n <= 0) return LAML_OK;
    // wide inside / outside levels below the roots on producer/consumer
    // warp pairs when the batch asks for them (wide_pc)
    if ((kind == 0 || kind == 1) && !narrow_level(n) && b.wide_pc) {
        return kind == 0 ? launch_pc_wide<G, 0>(b, desc, n, want_post, respect_status, st)
                         : launch_pc_wide<G, 1>(b, desc, n, want_post, respect_status, st);
    }
    // wide inside / outside levels below the roots: bulk-staged rows when
    // the batch asks for them (wide_chunk), else per-thread loads
    if ((kind == 0 || kind == 1) && !narrow_level(n) && b.max_states > 0 && b.wide_chunk > 0) {
        return kind == 0 ? launch_staged_wide<G, 0>(b, desc, n, want_post, respect_status, st)
                         : launch_staged_wide<G, 1>(b, desc, n, want_post, respect_status, st);
    }
    // inside / outside below the roots: the staged kernels when the batch
    // states its largest group and the buffers fit in shared memory
    if ((kind == 0 || kind == 1) && narrow_level(n) && b.max_states > 0 &&
        staged_smem(b, kind) <= kStagedSmemMax) {
        return kind == 0 ? launch_staged<G, 0>(b, desc, n, want_post, respect_status, st)
                         : launch_staged<G, 1>(b, desc, n, want_post, respect_status, st);
    }
    const int ipb = ((kind == 0 || kind == 1) && narrow_level(n)) ? kItemsBlock / 32
                                                                   : (kItemsBlock / 32) * (32 / G);
    int64_t blocks = (n + ipb - 1) / ipb;
    const int64_t cap = (int64_t)num_sms() * 16;
    if (blocks > cap) blocks = cap;
    const size_t sm0 = sizeof(float) * as_words<0>() * kItemsBlock;
    const size_t sm1 = sizeof(float) * as_words<1>() * kItemsBlock;
    switch (kind) {
        case 0: k_items<G, 0><<<(unsigned)blocks, kItemsBlock, sm0, st>>>(b, items, n, want_post, respect_status, desc); break;
        case 1:
            if (b.max_states > 0 && b.max_states <= kOutBlocksStates)
                k_items<G, 1, 8><<<(unsigned)blocks, kItemsBlock, sm1, st>>>(b, items, n, want_post, respect_status, desc);
            else
                k_items<G, 1, 6><<<(unsigned)blocks, kItemsBlock, sm1, st>>>(b, items, n, want_post, respect_status, desc);
            break;
        case 2: k_items<G, 2><<<(unsigned)blocks, kItemsBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        case 3: k_items<G, 3><<<(unsigned)blocks, kItemsBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        case 5: k_items<G, 5><<<(unsigned)blocks, kItemsBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
        default: k_items<G, 4><<<(unsigned)blocks, kItemsBlock, 0, st>>>(b, items, n, want_post, respect_status, desc); break;
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

// the M-step launches: every tree up to kClusterNodes nodes in k_mstep, the
// larger ones (when the batch may hold any) in k_mstep_cluster
constexpr int kUltraSmemNodes = 2816;   // 8 FP64 slots a node: 176 KB beside k_mstep's 41 KB

int launch_mstep(const laml_batch& b, int rounds, int flags, cudaStream_t st) {
    const bool big = b.max_tree_nodes <= 0 || b.max_tree_nodes > kClusterNodes;
    int ucap = 0;
    size_t usmem = 0;
    if ((flags & LAML_MSTEP_ULTRAMETRIC) && !b.compat) {
        ucap = b.max_tree_nodes > 0 ? std::min(b.max_tree_nodes, kUltraSmemNodes) : kUltraSmemNodes;
        usmem = sizeof(double) * 8 * (size_t)ucap;
        static bool attr_set = false;
        if (!attr_set) {
            const int rc = check(cudaFuncSetAttribute(k_mstep, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      (int)(sizeof(double) * 8 * kUltraSmemNodes)),
                                 "k_mstep shared memory limit");
            if (rc) return rc;
            attr_set = true;
        }
    }
    k_mstep<<<b.n_trees, kBlock, usmem, st>>>(b, rounds, flags, big ? 1 : 0, ucap);
    int rc = check(cudaGetLastError(), "k_mstep");
    if (rc || !big) return rc;
    const int clusters = std::max(1, std::min(b.n_trees, num_sms() / kMstepCluster));
    k_mstep_cluster<<<clusters * kMstepCluster, kMstepClusterThreads, 0, st>>>(b, rounds, flags);
    return check(cudaGetLastError(), "k_mstep_cluster");
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
        if ((rc = launch_mstep(b, rounds, flags, st))) return rc;
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

// The condition of a looping EM graph, run after every chunk: another chunk
// while some tree is still ACTIVE, no error is recorded and fewer than
// max_chunks chunks ran in this launch.  The counter returns to 0 when the
// loop ends, so every launch starts from 0; max_chunks bounds the loop
// whatever the trees' state.
__global__ void k_em_loop_cond(laml_batch b, cudaGraphConditionalHandle h, int32_t* counter,
                               int max_chunks) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < b.n_trees; t += blockDim.x)
        if (__ldcg(b.tr_status + t) == LAML_TREE_ACTIVE) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        const int c = *counter + 1;
        const bool more = any && c < max_chunks && __ldcg(b.error) == 0;
        *counter = more ? c : 0;
        cudaGraphSetConditional(h, more ? 1u : 0u);
    }
}

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
    if ((!b->in_items && !b->in_lnodes) || (!b->out_items && !b->out_lnodes)) {
        laml::set_error("laml_plan_descriptors: the batch needs items or level node lists");
        return LAML_ERR_ARG;
    }
    if (b->n_in_items > 0) {
        if (b->in_items)
            k_item_desc<<<blocks(b->n_in_items), kBlock, 0, st>>>(*b, b->in_items, b->n_in_items, in_desc);
        else
            k_item_desc_nodes<<<blocks(b->n_in_items), kBlock, 0, st>>>(
                *b, b->in_lnodes, b->in_level_off, b->n_in_levels, b->n_in_items, in_desc);
    }
    if (b->n_out_items > 0) {
        if (b->out_items)
            k_item_desc<<<blocks(b->n_out_items), kBlock, 0, st>>>(*b, b->out_items, b->n_out_items, out_desc);
        else
            k_item_desc_nodes<<<blocks(b->n_out_items), kBlock, 0, st>>>(
                *b, b->out_lnodes, b->out_level_off, b->n_out_levels, b->n_out_items, out_desc);
    }
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
    if (!rc) rc = validate_mstep_flags(b, flags, "laml_mstep");
    if (rc) return rc;
    return launch_mstep(*b, rounds, flags, (cudaStream_t)stream);
}

extern "C" int laml_em_run(const laml_batch* b, int32_t iters, int32_t rounds, double rel_tol,
                           int32_t max_iters, int32_t flags, void* stream) {
    int rc = validate(b);
    if (!rc) rc = validate_mstep_flags(b, flags, "laml_em_run");
    if (rc) return rc;
    if (iters <= 0) return LAML_OK;
    DISPATCH_G(*b, (em_persistent_t<GG>(*b, iters, rounds, rel_tol, max_iters, flags,
                                        (cudaStream_t)stream)));
}

extern "C" int laml_em_graph_create(const laml_batch* b, int32_t iters, int32_t rounds,
                                    double rel_tol, int32_t max_iters, int32_t flags,
                                    int32_t persistent, void** graph) {
    int rc = validate(b);
    if (!rc) rc = validate_mstep_flags(b, flags, "laml_em_graph_create");
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

extern "C" int laml_em_graph_loop_create(const laml_batch* b, int32_t chunk, int32_t rounds,
                                         double rel_tol, int32_t max_iters, int32_t flags,
                                         int32_t max_chunks, int32_t* counter, void** graph) {
    int rc = validate(b);
    if (!rc) rc = validate_mstep_flags(b, flags, "laml_em_graph_loop_create");
    if (rc) return rc;
    if (!graph || !counter || chunk <= 0 || max_chunks <= 0) {
        laml::set_error("laml_em_graph_loop_create: bad argument");
        return LAML_ERR_ARG;
    }
    if (!b->h_in_level_off || !b->h_out_level_off) {
        laml::set_error("laml_em_graph_loop_create: per-level capture needs the host level offsets");
        return LAML_ERR_ARG;
    }
    GraphHolder* g = new GraphHolder();
    auto fail = [&](int code) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        delete g;
        return code;
    };
    if ((rc = check(cudaGraphCreate(&g->graph, 0), "graph create"))) return fail(rc);
    cudaGraphConditionalHandle h;
    if ((rc = check(cudaGraphConditionalHandleCreate(&h, g->graph, 1, cudaGraphCondAssignDefault),
                    "conditional handle")))
        return fail(rc);
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if ((rc = check(cudaGraphAddNode(&node, g->graph, nullptr, nullptr, 0, &cp),
                    "conditional node")))
        return fail(rc);
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t st;
    if ((rc = check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")))
        return fail(rc);
    rc = check(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal),
               "begin capture");
    if (!rc) {
        auto run = [&]() -> int {
            DISPATCH_G(*b, (em_levels_t<GG>(*b, chunk, rounds, rel_tol, max_iters, flags, st)));
        };
        int brc = run();
        if (!brc) {
            k_em_loop_cond<<<1, 256, 0, st>>>(*b, h, counter, max_chunks);
            brc = check(cudaGetLastError(), "k_em_loop_cond");
        }
        cudaGraph_t out = nullptr;
        int erc = check(cudaStreamEndCapture(st, &out), "end capture");
        rc = brc ? brc : erc;
    }
    cudaStreamDestroy(st);
    if (!rc) rc = check(cudaGraphInstantiate(&g->exec, g->graph, 0), "graph instantiate");
    if (rc) return fail(rc);
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
    if (!rc) rc = validate_mstep_flags(b, flags, "laml_em_run_levels");
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
    // the level kernels write at the plan's row offsets: sizes below the
    // plan's would put those writes past the carve-outs below
    if (b->plan_part_floats <= 0 || part_floats < b->plan_part_floats ||
        scalar_len < b->plan_scalar_len) {
        laml::set_error("laml_inside_noalloc: part_floats / scalar_len must be at least the "
                        "batch's plan sizes (laml_batch.plan_part_floats = " +
                        std::to_string(b->plan_part_floats) + ", plan_scalar_len = " +
                        std::to_string(b->plan_scalar_len) + ")");
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
