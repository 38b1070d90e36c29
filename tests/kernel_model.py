"""Scalar CPU model of the device kernels' addressing and arithmetic.

Walks the same plan (items, level offsets, row/scalar offsets) and the same
flat buffers as laml_gb300/csrc/pmm_kernels.cu, item by item and lane by lane,
in float32, with explicit bounds checks on every access.  It exists so the
index arithmetic of a plan and the power-of-two scaling scheme can be checked
on a CPU before any kernel runs; tests compare it with the oracle.
"""
import math

import numpy as np

from laml_gb300 import encoding as E

f32 = np.float32
EPS = f32(1e-6)


class Buf:
    def __init__(self, n, dtype, name):
        self.a = np.full(max(int(n), 1), np.nan if dtype in (np.float32, np.float64) else -7777,
                         dtype=dtype)
        self.name = name

    def __getitem__(self, i):
        if not (0 <= i < len(self.a)):
            raise IndexError(f"{self.name}[{i}] out of [0, {len(self.a)})")
        return self.a[i]

    def __setitem__(self, i, v):
        if not (0 <= i < len(self.a)):
            raise IndexError(f"{self.name}[{i}] out of [0, {len(self.a)})")
        self.a[i] = v


def scale_exp(m):
    if not (m > 0):
        return 0
    _, h = math.frexp(float(m))
    return max(-125, min(125, h))


def pow2(e):
    return f32(2.0 ** e)


def logz(x):
    return math.log(float(x)) if x > 0 else -math.inf


def expz(l):
    return f32(math.exp(l)) if l > -745 else f32(0)


def lse3(a, b, c):
    m = max(a, b, c)
    if m == -math.inf:
        return m
    return m + math.log(math.exp(a - m) + math.exp(b - m) + math.exp(c - m))


def scale_of(l):
    return int(math.floor(l / math.log(2))) + 1 if l > -math.inf else 0


class Model:
    def __init__(self, datasets, trees, tree_ds, d, nu, phi, compat):
        self.G = G = datasets[0].group_sites
        self.compat = compat
        self.ds = datasets
        self.trees = trees
        self.sizes, self.p = E.plan_batch(trees, tree_ds, datasets)
        self.tree_ds = list(tree_ds)
        self.nu = [float(x) for x in nu]
        self.phi = [float(x) for x in phi]
        self.d = np.concatenate(d)
        s = self.sizes
        self.in_part = Buf(s["part_floats"], np.float32, "in_part")
        self.out_part = Buf(s["part_floats"], np.float32, "out_part")
        self.in_h = Buf(s["scalar_len"], np.int64, "in_h")
        self.in_x = Buf(s["scalar_len"], np.int64, "in_x")
        self.in_dot = Buf(s["scalar_len"], np.float32, "in_dot")
        self.out_h = Buf(s["scalar_len"], np.int64, "out_h")
        self.out_x = Buf(s["scalar_len"], np.int64, "out_x")
        self.llh_site = Buf(s["site_len"], np.float64, "llh_site")
        self.root_lr = Buf(s["site_len"], np.float32, "root_lr")
        self.root_x = Buf(s["site_len"], np.int64, "root_x")
        self.cnt = Buf(s["count_floats"], np.float32, "cnt_part")
        self.q_base = np.concatenate([[0], np.cumsum([x.row_len for x in datasets])[:-1]])
        self.bt = [self.bterm(i) for i in range(s["n_nodes"])]

    def bterm(self, i):
        t = self.p["nd_tree"][i]
        d, nu = self.d[i], self.nu[t]
        nd = d * nu
        e1md = 1e-6 if (self.compat and d < 1e-6) else -math.expm1(-d)
        e1mnd = 1e-6 if (self.compat and nd < 1e-6) else -math.expm1(-nd)
        pst = math.exp(-nd)
        return (f32(math.exp(-d * (1 + nu))), f32(e1md * pst), f32(pst), f32(e1mnd))

    def root_edge(self, t):
        """log P00, log Pmut (without q), log Pstay, log Psil of tree t's root
        edge, in float64 (the kernels form every root-edge product from these)."""
        r = int(self.p["tr_root"][t])
        d, nu = float(self.d[r]), self.nu[t]
        nd = d * nu
        lm = math.log(1e-6 if (self.compat and d < 1e-6) else -math.expm1(-d)) - nd
        if self.compat and nd < 1e-6:
            ls = math.log(1e-6)
        else:
            e = -math.expm1(-nd)
            ls = math.log(e) if e > 0 else -math.inf
        return -d * (1 + nu), lm, -nd, ls

    def leaf(self, t):
        phi = self.phi[t]
        if self.compat:
            return max(f32(1 - phi), EPS), max(f32(phi), EPS), EPS
        return f32(1 - phi), f32(phi), f32(0)

    def ctx(self, node, g, lane):
        p = self.p
        t = p["nd_tree"][node]
        ds = self.ds[self.tree_ds[t]]
        site = g * self.G + lane
        if site >= ds.n_sites:
            return None
        goff = int(ds.group_off[g])
        return dict(t=t, ds=ds, dsi=self.tree_ds[t], site=site, goff=goff,
                    C=int(ds.site_C[site]), sumq=ds.site_sumq[site],
                    qb=int(self.q_base[self.tree_ds[t]]) + goff + lane)

    def q(self, c, j):
        ds = c["ds"]
        k = c["qb"] - int(self.q_base[c["dsi"]]) + j * self.G
        if not (0 <= k < ds.row_len):
            raise IndexError("q")
        return ds.q[k]

    def child(self, x, c, lane):
        p, G = self.p, self.G
        e1, ephi, es = self.leaf(c["t"])
        if p["nd_c0"][x] < 0:
            row = p["nd_leafrow"][x]
            ds = c["ds"]
            if not (0 <= row < ds.n_leaves):
                raise IndexError("leaf row")
            code = int(ds.codes[row, c["site"]])
            s0 = e1 if code == 0 else (ephi if code == -1 else f32(0))
            ss = f32(1) if code < 0 else es
            D = self.q(c, code) * e1 if code >= 2 else (ephi * c["sumq"] if code == -1 else f32(0))
            return dict(leaf=True, code=code, s0=s0, ss=ss, D=f32(D), X=0, f=f32(1), e1=e1,
                        ephi=ephi)
        s = int(p["nd_srow"][x]) + c["site"]
        h = int(self.in_h[s])
        f = pow2(-h)
        base = int(p["nd_prow"][x]) + c["goff"] + lane
        return dict(leaf=False, base=base, f=f, X=int(self.in_x[s]), D=self.in_dot[s],
                    s0=self.in_part[base] * f, ss=self.in_part[base + G] * f)

    def val(self, ch, j):
        if ch["leaf"]:
            return ch["e1"] if ch["code"] == j else (ch["ephi"] if ch["code"] == -1 else f32(0))
        return self.in_part[ch["base"] + j * self.G] * ch["f"]

    def inside_item(self, u, g, lane):
        c = self.ctx(u, g, lane)
        if c is None:
            return
        p, G = self.p, self.G
        v, w = p["nd_c0"][u], p["nd_c1"][u]
        cv, cw = self.child(v, c, lane), self.child(w, c, lane)
        bv, bw = self.bt[v], self.bt[w]
        ev0 = bv[0] * cv["s0"] + bv[1] * cv["D"] + bv[3] * cv["ss"]
        ew0 = bw[0] * cw["s0"] + bw[1] * cw["D"] + bw[3] * cw["ss"]
        kv, kw = bv[3] * cv["ss"], bw[3] * cw["ss"]
        row = int(p["nd_prow"][u]) + c["goff"] + lane
        s0, ss = f32(ev0 * ew0), f32(cv["ss"] * cw["ss"])
        self.in_part[row] = s0
        self.in_part[row + G] = ss
        mx, dot = max(s0, ss), f32(0)
        for j in range(2, c["C"]):
            x = f32((bv[2] * self.val(cv, j) + kv) * (bw[2] * self.val(cw, j) + kw))
            self.in_part[row + j * G] = x
            dot = f32(dot + self.q(c, j) * x)
            mx = max(mx, x)
        h = scale_exp(mx)
        f = pow2(-h)
        X = cv["X"] + cw["X"] + h
        sr = int(p["nd_srow"][u]) + c["site"]
        self.in_h[sr] = h
        self.in_x[sr] = X
        self.in_dot[sr] = dot * f
        t = c["t"]
        if u == p["tr_root"][t]:
            l00, lm, _, ls = self.root_edge(t)
            lv = lse3(l00 + logz(s0 * f), lm + logz(dot * f), ls + logz(ss * f))
            k = int(p["tr_site_base"][t]) + c["site"]
            e = scale_of(lv)
            self.root_lr[k] = f32(math.exp(lv - e * math.log(2))) if lv > -math.inf else f32(0)
            self.root_x[k] = X + e
            self.llh_site[k] = lv + X * math.log(2)

    def run_inside(self):
        p, s, G = self.p, self.sizes, self.G
        items = p["in_items"]
        for l in range(s["n_in_levels"]):
            for k in range(p["in_level_off"][l], p["in_level_off"][l + 1]):
                for lane in range(G):
                    self.inside_item(int(items[2 * k]), int(items[2 * k + 1]), lane)

    def root_init(self, r, g, lane):
        c = self.ctx(r, g, lane)
        if c is None:
            return
        p, G = self.p, self.G
        br = self.bt[r]
        row = int(p["nd_prow"][r]) + c["goff"] + lane
        mx = max(br[0], br[3])
        self.out_part[row] = br[0]
        self.out_part[row + G] = br[3]
        for j in range(2, c["C"]):
            o = f32(br[1] * self.q(c, j))
            self.out_part[row + j * G] = o
            mx = max(mx, o)
        h = scale_exp(mx)
        sr = int(p["nd_srow"][r]) + c["site"]
        self.out_h[sr] = h
        self.out_x[sr] = h

    def outside_item(self, v, g, lane, mode):
        c = self.ctx(v, g, lane)
        zero = [f32(0)] * 7
        if c is None:
            return zero
        p, G = self.p, self.G
        cv = self.child(v, c, lane)
        bv = self.bt[v]
        sumx, dotxv, mx = f32(0), f32(0), f32(0)
        orow = None
        t = c["t"]
        u = p["nd_parent"][v] if mode == 0 else p["tr_quirk"][t]
        at_root = mode == 0 and u == p["tr_root"][t]
        if mode == 2:
            x0, xs, Xx = f32(1), f32(0), 0
        else:
            w = p["nd_sib"][v] if mode == 0 else u
            cw = self.child(w, c, lane)
            bw = self.bt[w]
            kw = bw[3] * cw["ss"]
            ew0 = f32(bw[0] * cw["s0"] + bw[1] * cw["D"] + bw[3] * cw["ss"])
            if at_root:
                # the root's outside is its edge: x = o * E[w] from the logs
                l00, lm, _, ls = self.root_edge(t)
                ma = max([f32(self.q(c, j) * (bw[2] * self.val(cw, j) + kw))
                          for j in range(2, c["C"])] + [f32(0)])
                E = scale_of(max(l00 + logz(ew0), ls + logz(cw["ss"]), lm + logz(ma)))
                x0 = expz(l00 - E * math.log(2) + logz(ew0))
                xs = expz(ls - E * math.log(2) + logz(cw["ss"]))
                Xx = E + cw["X"]
                lmE = lm - E * math.log(2)
            else:
                su = int(p["nd_srow"][u]) + c["site"]
                fo = pow2(-int(self.out_h[su]))
                Xo = int(self.out_x[su])
                urow = int(p["nd_prow"][u]) + c["goff"] + lane
                o0, os_ = self.out_part[urow] * fo, self.out_part[urow + G] * fo
                x0 = f32(o0 * ew0)
                xs = f32(os_ * cw["ss"])
                Xx = Xo + cw["X"]
            write = mode == 0 and not cv["leaf"]
            if write:
                orow = int(p["nd_prow"][v]) + c["goff"] + lane
            px = bv[1] * x0
            for j in range(2, c["C"]):
                if at_root:
                    xa = expz(lmE + logz(f32(self.q(c, j) * (bw[2] * self.val(cw, j) + kw))))
                    sumx = f32(sumx + xa)
                    dotxv = f32(dotxv + xa * self.val(cv, j))
                    if write:
                        o = f32(px * self.q(c, j) + bv[2] * xa)
                        self.out_part[orow + j * G] = o
                        mx = max(mx, o)
                    continue
                ou = self.out_part[urow + j * G] * fo
                xa = f32(ou * (bw[2] * self.val(cw, j) + kw))
                sumx = f32(sumx + xa)
                dotxv = f32(dotxv + xa * self.val(cv, j))
                if write:
                    o = f32(px * self.q(c, j) + bv[2] * xa)
                    self.out_part[orow + j * G] = o
                    mx = max(mx, o)
        out0 = f32(bv[0] * x0)
        outs = f32(bv[3] * (x0 + sumx) + xs)
        if orow is not None:
            self.out_part[orow] = out0
            self.out_part[orow + G] = outs
            h = scale_exp(max(mx, out0, outs))
            sv = int(p["nd_srow"][v]) + c["site"]
            self.out_h[sv] = h
            self.out_x[sv] = Xx + h
        k = int(p["tr_site_base"][c["t"]]) + c["site"]
        lroot = self.root_lr[k]
        if mode != 0:
            # the root's own row: every root-edge product from the logs
            l00, lm, lst, ls = self.root_edge(t)
            lsc = ((Xx + cv["X"] - int(self.root_x[k])) * math.log(2) - math.log(float(lroot))
                   if lroot > 0 else -math.inf)
            return [expz(logz(f32(x0 * cv["s0"])) + l00 + lsc),
                    expz(logz(f32(x0 * cv["D"])) + lm + lsc),
                    expz(logz(f32(x0 * cv["ss"])) + ls + lsc),
                    expz(logz(dotxv) + lst + lsc),
                    expz(logz(f32(cv["ss"] * sumx)) + ls + lsc),
                    expz(logz(f32(xs * cv["ss"])) + lsc), f32(0)]
        e = Xx + cv["X"] - int(self.root_x[k])
        sc = f32(math.ldexp(1.0 / float(lroot), e)) if lroot > 0 else f32(0)
        res = [x0 * cv["s0"] * bv[0] * sc, x0 * bv[1] * cv["D"] * sc, x0 * cv["ss"] * bv[3] * sc,
               bv[2] * dotxv * sc, bv[3] * cv["ss"] * sumx * sc, xs * cv["ss"] * sc,
               cv["ss"] * outs * sc if cv["leaf"] else f32(0)]
        return [f32(x) for x in res]

    def run_outside(self):
        """Returns counts [n_nodes, 6] and leaf responsibilities [n_nodes]."""
        p, s, G = self.p, self.sizes, self.G
        n = s["n_nodes"]
        counts = np.zeros((n, 7))
        for k in range(s["n_root_items"]):
            for lane in range(G):
                self.root_init(int(p["root_items"][2 * k]), int(p["root_items"][2 * k + 1]), lane)
        items = p["out_items"]

        def acc(node, g, mode):
            tot = np.zeros(7)
            for lane in range(G):
                tot += np.asarray(self.outside_item(node, g, lane, mode), np.float64)
            t = p["nd_tree"][node]
            ds = self.ds[self.tree_ds[t]]
            base = int(p["tr_cnt_base"][t]) + ((node - int(p["tr_node_base"][t])) * ds.n_groups
                                               + g) * 8
            for kk in range(7):
                self.cnt[base + kk] = tot[kk]
            counts[node] += tot

        for l in range(s["n_out_levels"]):
            for k in range(p["out_level_off"][l], p["out_level_off"][l + 1]):
                # one item per internal parent: both children (outside_parent_item)
                u, g = int(items[2 * k]), int(items[2 * k + 1])
                acc(int(p["nd_c0"][u]), g, 0)
                acc(int(p["nd_c1"][u]), g, 0)
        for k in range(s["n_root_items"]):
            acc(int(p["root_items"][2 * k]), int(p["root_items"][2 * k + 1]),
                1 if self.compat else 2)
        return counts[:, :6], counts[:, 6]

    def site_llh(self, t):
        ds = self.ds[self.tree_ds[t]]
        base = int(self.p["tr_site_base"][t])
        out = np.empty(ds.n_sites)
        for c in range(ds.n_sites_pad):
            o = ds.site_perm[c]
            if o >= 0:
                out[o] = self.llh_site[base + c]
        return out
