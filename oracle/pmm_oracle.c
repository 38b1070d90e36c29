/*
 * FP64 C restatement of LAML's fastEM path (compat semantics) -- TEST
 * INFRASTRUCTURE: the timed CPU baseline of bench.py and a cross-check of the
 * NumPy oracle (oracle/pmm_oracle.py).  Never linked into the product.
 *
 * Follows, in log space with the reference's state order (0, 1..k, silenced)
 * and EPS floors:
 *   leaf init            fast_em/calculations.py:278-334
 *   edge-inside Q^T v    fast_em/calculations.py:47-91
 *   inside pass          fast_em/calculations.py:193-276 (postorder instead of
 *                        the level-masked vmap: same values, O(N) work)
 *   outside Q v          fast_em/calculations.py:11-45, 135-191
 *   responsibilities     fast_em/calculations.py:373-454 (root row -> node N-1)
 *   M-step objective     fast_em/laml.py:62-78, maximised by coordinate ascent
 *                        (closed-form phi, bisection in log d, bisection in nu)
 *   EM iteration         fast_em/laml.py:153-192
 * One tree per OpenMP thread.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define EPS 1e-6
#define CEPS 1e-10

typedef struct {
    int N, n, K;            /* nodes, leaves, sites */
    const int* c0;          /* [N] first child (local), -1 at leaves */
    const int* c1;
    const int* parent;      /* [N] -1 at the root */
    const int* chars;       /* [n*K]: 0, 1..k_c, -1 missing */
    const int* kc;          /* [K] observed mutated states per site */
    const double* q;        /* [K*kmax] raw priors */
    int kmax;
    double* d;              /* [N] in/out */
    double nu, phi;         /* in/out */
    double llh;             /* out: log-likelihood after the last iteration */
} ora_tree;

static double lse2(double a, double b) {
    if (a == -INFINITY) return b;
    if (b == -INFINITY) return a;
    double m = a > b ? a : b;
    return m + log1p(exp(-fabs(a - b)));
}

/* fast_em exponentiates its log-responsibilities in float32 with denormals
 * flushed (calculations.py:576-577): a per-site term below the smallest
 * normal float is zero */
static double ftz(double x) { return x < 1.1754943508222875e-38 ? 0.0 : x; }

typedef struct {
    int R;          /* doubles per node row: sum_c (k_c + 2) */
    int* off;       /* [K] */
    double *ins, *ein, *out;   /* [N*R] */
    double *t1, *t2, *t3, *a0; /* [N] */
    double* logq;   /* [R] (slot 0 and slot s unused) */
    double* L;      /* [K] */
} work;

static void terms(const ora_tree* T, work* W) {
    for (int v = 0; v < T->N; ++v) {
        double d = T->d[v], nd = d * T->nu;
        W->t1[v] = -nd;
        W->t2[v] = nd < EPS ? log(EPS) : log(-expm1(-nd));
        W->t3[v] = d < EPS ? log(EPS) : log(-expm1(-d));
        W->a0[v] = -d * (1.0 + T->nu);
    }
}

static void edge_in(const ora_tree* T, const work* W, int v, const double* x, double* e) {
    for (int c = 0; c < T->K; ++c) {
        const int k = T->kc[c], o = W->off[c], s = o + k + 1;
        double m = W->a0[v] + x[o];
        double tmp[1];
        (void)tmp;
        /* log-sum-exp over {a0 + x0, t1 + logq + t3 + x_a, t2 + x_s} */
        double acc_m = m;
        for (int a = 1; a <= k; ++a) {
            double z = W->t1[v] + W->logq[o + a] + W->t3[v] + x[o + a];
            if (z > acc_m) acc_m = z;
        }
        double zs = W->t2[v] + x[s];
        if (zs > acc_m) acc_m = zs;
        double sum = 0.0;
        if (acc_m != -INFINITY) {
            sum += exp(m - acc_m);
            for (int a = 1; a <= k; ++a)
                sum += exp(W->t1[v] + W->logq[o + a] + W->t3[v] + x[o + a] - acc_m);
            sum += exp(zs - acc_m);
            e[o] = acc_m + log(sum);
        } else {
            e[o] = -INFINITY;
        }
        for (int a = 1; a <= k; ++a) e[o + a] = lse2(W->t1[v] + x[o + a], W->t2[v] + x[s]);
        e[s] = x[s];
    }
}

static void leaf_row(const ora_tree* T, const work* W, int v, double* x) {
    const double e1 = log(fmax(1.0 - T->phi, EPS)), ep = log(fmax(T->phi, EPS));
    for (int c = 0; c < T->K; ++c) {
        const int k = T->kc[c], o = W->off[c], s = o + k + 1, ch = T->chars[v * T->K + c];
        for (int a = 0; a <= k; ++a)
            x[o + a] = (a == ch) ? e1 : (ch == -1 ? ep : -INFINITY);
        x[s] = ch == -1 ? 0.0 : log(EPS);
    }
}

static double inside(const ora_tree* T, work* W) {
    const int R = W->R;
    for (int v = 0; v < T->n; ++v) leaf_row(T, W, v, W->ins + (size_t)v * R);
    double* e = (double*)malloc(sizeof(double) * 2 * R);
    for (int u = T->N - 1; u >= T->n; --u) {
        edge_in(T, W, T->c0[u], W->ins + (size_t)T->c0[u] * R, e);
        edge_in(T, W, T->c1[u], W->ins + (size_t)T->c1[u] * R, e + R);
        double* r = W->ins + (size_t)u * R;
        for (int j = 0; j < R; ++j) r[j] = e[j] + e[R + j];
    }
    int root = -1;
    for (int v = 0; v < T->N; ++v)
        if (T->parent[v] < 0) root = v;
    edge_in(T, W, root, W->ins + (size_t)root * R, e);
    double tot = 0.0;
    for (int c = 0; c < T->K; ++c) {
        W->L[c] = e[W->off[c]];
        tot += W->L[c];
    }
    free(e);
    return tot;
}

/* outside + counts; returns the leaf-silenced responsibility total */
static double outside_counts(const ora_tree* T, work* W, double* cnt) {
    const int R = W->R, N = T->N;
    int root = -1;
    for (int v = 0; v < N; ++v)
        if (T->parent[v] < 0) root = v;
    for (int v = 0; v < N; ++v) edge_in(T, W, v, W->ins + (size_t)v * R, W->ein + (size_t)v * R);
    double* o = W->out + (size_t)root * R;
    for (int c = 0; c < T->K; ++c) {
        const int k = T->kc[c], of = W->off[c];
        o[of] = W->a0[root];
        for (int a = 1; a <= k; ++a) o[of + a] = W->t1[root] + W->logq[of + a] + W->t3[root];
        o[of + k + 1] = W->t2[root];
    }
    double* x = (double*)malloc(sizeof(double) * R);
    /* internal ids increase down the tree (preorder numbering) */
    for (int u = T->n; u < N; ++u) {
        int ch[2] = {T->c0[u], T->c1[u]};
        for (int z = 0; z < 2; ++z) {
            const int v = ch[z], w = ch[1 - z];
            const double* ou = W->out + (size_t)u * R;
            const double* ew = W->ein + (size_t)w * R;
            double* ov = W->out + (size_t)v * R;
            for (int j = 0; j < R; ++j) x[j] = ou[j] + ew[j];
            for (int c = 0; c < T->K; ++c) {
                const int k = T->kc[c], of = W->off[c], s = of + k + 1;
                ov[of] = W->a0[v] + x[of];
                double m = -INFINITY;
                for (int a = 0; a <= k; ++a) if (x[of + a] > m) m = x[of + a];
                double sm = 0.0;
                if (m != -INFINITY) {
                    for (int a = 0; a <= k; ++a) sm += exp(x[of + a] - m);
                    sm = m + log(sm);
                } else {
                    sm = -INFINITY;
                }
                ov[s] = lse2(W->t2[v] + sm, x[s]);
                for (int a = 1; a <= k; ++a)
                    ov[of + a] = lse2(W->logq[of + a] + W->t1[v] + W->t3[v] + x[of], W->t1[v] + x[of + a]);
            }
        }
    }
    double lr = 0.0;
    for (int v = 0; v < N; ++v) {
        int u, w;
        if (v == root) { u = N - 1; w = N - 1; }   /* parent_sibling[root] = (-1, -1) */
        else {
            u = T->parent[v];
            w = T->c0[u] == v ? T->c1[u] : T->c0[u];
        }
        const double* ou = W->out + (size_t)u * R;
        const double* ew = W->ein + (size_t)w * R;
        const double* iv = W->ins + (size_t)v * R;
        for (int j = 0; j < R; ++j) x[j] = ou[j] + ew[j];
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int c = 0; c < T->K; ++c) {
            const int k = T->kc[c], of = W->off[c], s = of + k + 1;
            const double L = W->L[c];
            acc[0] += ftz(exp(x[of] + iv[of] + W->a0[v] - L));
            double s1 = 0, s3 = 0, s4 = 0;
            for (int a = 1; a <= k; ++a) {
                s1 += exp(x[of] + iv[of + a] + W->t1[v] + W->logq[of + a] + W->t3[v] - L);
                s3 += exp(x[of + a] + iv[of + a] + W->t1[v] - L);
                s4 += exp(x[of + a] + iv[s] + W->t2[v] - L);
            }
            acc[1] += ftz(s1);
            acc[2] += ftz(exp(x[of] + iv[s] + W->t2[v] - L));
            acc[3] += ftz(s3);
            acc[4] += ftz(s4);
            acc[5] += ftz(exp(x[s] + iv[s] - L));
            if (v < T->n) lr += ftz(exp(iv[s] + W->out[(size_t)v * R + s] - L));
        }
        for (int i = 0; i < 6; ++i) cnt[(size_t)v * 6 + i] = acc[i];
    }
    free(x);
    return lr;
}

static double inv_em1(double x) { return 1.0 / expm1(x); }

static void mstep(ora_tree* T, const double* cnt, double lr, int rounds) {
    double M = 0, Rn = 0;
    for (int i = 0; i < T->n * T->K; ++i) {
        if (T->chars[i] == -1) M += 1; else Rn += 1;
    }
    double B = M - lr;
    double phi = (Rn + B) > 0 ? B / (Rn + B) : T->phi;
    T->phi = fmin(fmax(phi, CEPS), 1 - CEPS);
    double nu = T->nu;
    for (int r = 0; r < rounds; ++r) {
        for (int v = 0; v < T->N; ++v) {
            const double* e = cnt + (size_t)v * 6;
            const double a = e[0] * (1 + nu) + (e[1] + e[3]) * nu, b = e[1], c = e[2] + e[4];
#define FP(x) (-a + b * inv_em1(x) + c * nu * inv_em1(nu * (x)))
            double lo = CEPS, hi = 1.0 / CEPS, res;
            if (a == 0 && b == 0 && c == 0) res = T->d[v];   /* flat: a zero gradient keeps d */
            else if (FP(lo) <= 0) res = lo;
            else if (FP(hi) >= 0) res = hi;
            else {
                double ul = log(lo), uh = log(hi);
                for (int it = 0; it < 200; ++it) {
                    double um = 0.5 * (ul + uh);
                    if (FP(exp(um)) > 0) ul = um; else uh = um;
                }
                res = exp(0.5 * (ul + uh));
            }
#undef FP
            T->d[v] = res;
        }
        double A = 0, Cs = 0;
        for (int v = 0; v < T->N; ++v) {
            const double* e = cnt + (size_t)v * 6;
            A += (e[0] + e[1] + e[3]) * T->d[v];
            Cs += e[2] + e[4];
        }
#define GP(x) ({ double _s = -A; for (int v = 0; v < T->N; ++v) { const double* e = cnt + (size_t)v * 6; \
        double cc = e[2] + e[4]; if (cc > 0) _s += cc * T->d[v] * inv_em1((x) * T->d[v]); } _s; })
        double lo = CEPS, hi = 1 - CEPS;
        if (Cs <= 0) nu = lo;
        else if (GP(hi) >= 0) nu = hi;
        else if (GP(lo) <= 0) nu = lo;
        else {
            double ul = log(lo), uh = log(hi);
            for (int it = 0; it < 200; ++it) {
                double um = 0.5 * (ul + uh);
                if (GP(exp(um)) > 0) ul = um; else uh = um;
            }
            nu = exp(0.5 * (ul + uh));
        }
#undef GP
    }
    T->nu = nu;
}

static void work_init(const ora_tree* T, work* W) {
    W->off = (int*)malloc(sizeof(int) * T->K);
    int R = 0;
    for (int c = 0; c < T->K; ++c) { W->off[c] = R; R += T->kc[c] + 2; }
    W->R = R;
    size_t sz = (size_t)T->N * R;
    W->ins = (double*)malloc(sizeof(double) * sz);
    W->ein = (double*)malloc(sizeof(double) * sz);
    W->out = (double*)malloc(sizeof(double) * sz);
    W->t1 = (double*)malloc(sizeof(double) * T->N);
    W->t2 = (double*)malloc(sizeof(double) * T->N);
    W->t3 = (double*)malloc(sizeof(double) * T->N);
    W->a0 = (double*)malloc(sizeof(double) * T->N);
    W->logq = (double*)malloc(sizeof(double) * R);
    W->L = (double*)malloc(sizeof(double) * T->K);
    for (int c = 0; c < T->K; ++c)
        for (int a = 1; a <= T->kc[c]; ++a) {
            double qv = T->q[c * T->kmax + a - 1];
            W->logq[W->off[c] + a] = qv > 0 ? log(qv) : -INFINITY;
        }
}

static void work_free(work* W) {
    free(W->off); free(W->ins); free(W->ein); free(W->out); free(W->t1); free(W->t2);
    free(W->t3); free(W->a0); free(W->logq); free(W->L);
}

/* Log-likelihood of each tree at its current parameters. */
void ora_loglik(ora_tree* trees, int n_trees) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int p = 0; p < n_trees; ++p) {
        work W;
        work_init(&trees[p], &W);
        terms(&trees[p], &W);
        trees[p].llh = inside(&trees[p], &W);
        work_free(&W);
    }
}

/* Per-site log-likelihood of one tree, sites in parallel (one site's column
 * of inside rows at a time per thread: N * (k_c + 2) doubles), so trees too
 * large for ora_loglik's whole-tree rows (50,000 leaves x 300 sites) fit.
 * Same arithmetic as inside() restricted to site c: leaf rows
 * (calculations.py:278-334), edge-inside (calculations.py:47-91) summed over
 * the two children in postorder (calculations.py:240-251), the root's own
 * edge from state 0 (calculations.py:270-276). */
void ora_site_loglik(const ora_tree* T, double* per_site) {
    int root = -1;
    for (int v = 0; v < T->N; ++v)
        if (T->parent[v] < 0) root = v;
#pragma omp parallel
    {
        int kmax = 0;
        for (int c = 0; c < T->K; ++c) if (T->kc[c] > kmax) kmax = T->kc[c];
        const int Rm = kmax + 2;
        double* col = (double*)malloc(sizeof(double) * (size_t)T->N * Rm);
        double* e = (double*)malloc(sizeof(double) * 2 * Rm);
        double* lq = (double*)malloc(sizeof(double) * Rm);
        double *t1 = (double*)malloc(sizeof(double) * T->N), *t2 = (double*)malloc(sizeof(double) * T->N);
        double *t3 = (double*)malloc(sizeof(double) * T->N), *a0 = (double*)malloc(sizeof(double) * T->N);
        for (int v = 0; v < T->N; ++v) {
            double d = T->d[v], nd = d * T->nu;
            t1[v] = -nd;
            t2[v] = nd < EPS ? log(EPS) : log(-expm1(-nd));
            t3[v] = d < EPS ? log(EPS) : log(-expm1(-d));
            a0[v] = -d * (1.0 + T->nu);
        }
        const double e1 = log(fmax(1.0 - T->phi, EPS)), ep = log(fmax(T->phi, EPS));
#pragma omp for schedule(dynamic, 1)
        for (int c = 0; c < T->K; ++c) {
            const int k = T->kc[c], R = k + 2, s = k + 1;
            for (int a = 1; a <= k; ++a) {
                double qv = T->q[c * T->kmax + a - 1];
                lq[a] = qv > 0 ? log(qv) : -INFINITY;
            }
            for (int v = 0; v < T->n; ++v) {
                const int ch = T->chars[(size_t)v * T->K + c];
                double* x = col + (size_t)v * R;
                for (int a = 0; a <= k; ++a) x[a] = (a == ch) ? e1 : (ch == -1 ? ep : -INFINITY);
                x[s] = ch == -1 ? 0.0 : log(EPS);
            }
            /* children before parents: internal ids grow down the tree */
            for (int u = T->N - 1; u >= T->n; --u) {
                const int kids[2] = {T->c0[u], T->c1[u]};
                for (int z = 0; z < 2; ++z) {
                    const int v = kids[z];
                    const double* x = col + (size_t)v * R;
                    double* ev = e + z * Rm;
                    double m = a0[v] + x[0];
                    for (int a = 1; a <= k; ++a) {
                        double y = t1[v] + lq[a] + t3[v] + x[a];
                        if (y > m) m = y;
                    }
                    if (t2[v] + x[s] > m) m = t2[v] + x[s];
                    if (m == -INFINITY) {
                        ev[0] = -INFINITY;
                    } else {
                        double sum = exp(a0[v] + x[0] - m) + exp(t2[v] + x[s] - m);
                        for (int a = 1; a <= k; ++a) sum += exp(t1[v] + lq[a] + t3[v] + x[a] - m);
                        ev[0] = m + log(sum);
                    }
                    for (int a = 1; a <= k; ++a) ev[a] = lse2(t1[v] + x[a], t2[v] + x[s]);
                    ev[s] = x[s];
                }
                double* r = col + (size_t)u * R;
                for (int j = 0; j < R; ++j) r[j] = e[j] + e[Rm + j];
            }
            /* the root's own edge, from a progenitor in state 0 */
            const double* x = col + (size_t)root * R;
            double m = a0[root] + x[0];
            for (int a = 1; a <= k; ++a) {
                double y = t1[root] + lq[a] + t3[root] + x[a];
                if (y > m) m = y;
            }
            if (t2[root] + x[s] > m) m = t2[root] + x[s];
            double sum = exp(a0[root] + x[0] - m) + exp(t2[root] + x[s] - m);
            for (int a = 1; a <= k; ++a) sum += exp(t1[root] + lq[a] + t3[root] + x[a] - m);
            per_site[c] = m + log(sum);
        }
        free(col); free(e); free(lq); free(t1); free(t2); free(t3); free(a0);
    }
}

/* `iters` EM iterations per tree (E-step, M-step, log-likelihood), with the
 * starting inside pass outside the timed part.  Returns the seconds spent in
 * the iterations (max over threads = wall time of the parallel region). */
double ora_em(ora_tree* trees, int n_trees, int iters, int rounds) {
    double t_iter = 0.0;
#pragma omp parallel
    {
        double mine = 0.0;
#pragma omp for schedule(dynamic, 1)
        for (int p = 0; p < n_trees; ++p) {
            ora_tree* T = &trees[p];
            work W;
            work_init(T, &W);
            for (int v = 0; v < T->N; ++v) T->d[v] = fmax(T->d[v], EPS);
            T->nu = fmin(fmax(T->nu, EPS), 1 - EPS);
            T->phi = fmin(fmax(T->phi, EPS), 1 - EPS);
            terms(T, &W);
            T->llh = inside(T, &W);
            double* cnt = (double*)malloc(sizeof(double) * 6 * T->N);
            double t0 = omp_get_wtime();
            for (int it = 0; it < iters; ++it) {
                double lr = outside_counts(T, &W, cnt);
                mstep(T, cnt, lr, rounds);
                terms(T, &W);
                T->llh = inside(T, &W);
            }
            mine += omp_get_wtime() - t0;
            free(cnt);
            work_free(&W);
        }
#pragma omp critical
        if (mine > t_iter) t_iter = mine;
    }
    return t_iter;
}

int ora_num_threads(void) { return omp_get_max_threads(); }
