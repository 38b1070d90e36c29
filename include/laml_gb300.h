/*
 * laml_gb300 -- C ABI of the GB300 (sm_103a) engine for LAML's PMM
 * likelihood / EM path.
 *
 * Plain pointers and sizes only.  Host-side encoders run on the CPU and fill
 * caller-allocated arrays; device entry points take a `laml_batch` whose
 * pointers are device addresses and launch on the given CUDA stream
 * (`stream` is a cudaStream_t passed as void*; NULL = legacy default stream).
 *
 * The reference surface each entry point replaces is cited beside it
 * (paths are relative to the LAML repository).
 *
 * Return codes: LAML_OK (0) or a negative LAML_ERR_*; laml_last_error()
 * returns a message for the calling thread's last failure.
 */
#ifndef LAML_GB300_H
#define LAML_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LAML_OK 0
#define LAML_ERR_ARG -1        /* bad argument / size */
#define LAML_ERR_CUDA -2       /* a CUDA runtime call failed */
#define LAML_ERR_PARSE -3      /* malformed newick */
#define LAML_ERR_PRIOR -4      /* an observed state has no prior (phylogeny.py:91-93) */
#define LAML_ERR_TIMEOUT -5    /* a device-side wait (grid barrier, mbarrier) gave up */
#define LAML_ERR_NOT_BINARY -6 /* a node with more than two children */
#define LAML_ERR_LEAF -7       /* a leaf label missing from the leaf order */

/* Character codes of the encoded matrix (int32 input to laml_dataset_*). */
#define LAML_CHAR_MISSING (-1)  /* '?' */
#define LAML_CHAR_SILENCED (-2) /* an explicit -1 in the exact (EM_solver) model */

/* ------------------------------------------------------------------------
 * Host encoders (no GPU needed)
 * --------------------------------------------------------------------- */

/* Sizes of a newick tree as fastEM_solver.parse_tree numbers it
 * (laml_libs/fastEM_solver.py:46-146): a unifurcating root is dropped.
 * label_bytes counts the labels' bytes including one NUL each. */
int laml_newick_size(const char* newick, int32_t* num_nodes, int32_t* num_leaves,
                     int64_t* label_bytes);

/* Encode a newick tree in the node order of fastEM_solver.parse_tree:
 * leaves 0..n-1 in `leaf_order` order (or treeswift preorder when
 * leaf_order == NULL), internal nodes n..N-1 in treeswift preorder, children
 * in networkx successor order (child0, child1; -1 for leaves).  Missing edge
 * lengths give has_length = 0 and branch_length = 0.  Labels are written
 * NUL-terminated into `labels` with their start offsets in label_offsets[N];
 * unlabelled nodes are named "node_<preorder index>" (fastEM_solver.py:65-67).
 * Replaces: fastEM_solver.parse_tree + the networkx traversals of
 * EMOptimizer.optimize (fast_em/laml.py:234-251). */
int laml_newick_encode(const char* newick, const char* const* leaf_order, int32_t n_leaf_order,
                       int32_t* parent, int32_t* child0, int32_t* child1,
                       double* branch_length, uint8_t* has_length,
                       char* labels, int64_t* label_offsets);

/* Batch form of laml_newick_encode for many trees over one leaf set (the
 * candidates of a topology search): every tree must have exactly the leaves
 * of `leaf_order`, which numbers them 0..n-1.  laml_newick_batch_measure gives
 * an upper bound of the total node count to size the outputs; node_offsets
 * [n_trees + 1] receives the compacted start of each tree.  Parses once per
 * tree on `n_threads` host threads (0 = all); no labels are produced. */
int laml_newick_batch_measure(int32_t n_trees, const char* const* newicks,
                              int64_t* raw_nodes_total);
int laml_newick_encode_batch(int32_t n_trees, const char* const* newicks,
                             const char* const* leaf_order, int32_t n_leaf_order,
                             int32_t n_threads, int64_t* node_offsets, int32_t* num_leaves,
                             int32_t* parent, int32_t* child0, int32_t* child1,
                             double* branch_length, uint8_t* has_length);

/* NNI candidates of one binary tree without writing or parsing newick.
 * Topology_search's move (laml_libs/Topology_search.py:242-322,
 * Topology_search_parallel.py:65-130) trades u's child `u_child` with u's
 * sibling w; treeswift's child lists then read u: (u's other child, w) and
 * v = parent(u): (u, u_child).  Moves are taken in order on one tree whose
 * child lists each swap-and-undo leaves reading u: (u's other child,
 * u_child), v: (u, w) -- the order the search's own listing leaves its tree
 * object in -- and every later candidate's numbering follows from that
 * state.  Each candidate is written in the numbering
 * laml_newick_encode gives the newick Topology_search writes for it: leaves
 * keep their ids (the input's leaf order), internal nodes are renumbered in
 * treeswift preorder of the new tree, child0/child1 in networkx successor
 * order; every node keeps its own branch length.  Input: the tree as
 * laml_newick_encode wrote it; moves[2 * n_moves] = (u, u_child) pairs of
 * node ids (u internal, not the root).  Outputs hold n_moves * n_nodes
 * entries, candidate m at offset m * n_nodes.  n_threads = 0: all host
 * threads. */
int laml_nni_candidates(int32_t n_nodes, int32_t n_leaves, const int32_t* parent,
                        const int32_t* child0, const int32_t* child1,
                        const double* branch_length, const uint8_t* has_length,
                        int32_t n_moves, const int32_t* moves, int32_t n_threads,
                        int32_t* out_parent, int32_t* out_child0, int32_t* out_child1,
                        double* out_length, uint8_t* out_has_length);

/* Site layout of a character matrix for the device kernels.
 * chars: n_leaves x n_sites int32 in leaf order (LAML_CHAR_* or >= 0 raw
 * states); priors as CSR over sites: prior_ptr[n_sites+1], prior_state[],
 * prior_prob[].  compat = 1 recodes as fast_em/phylogeny.py:62-94 (observed
 * states only, raw float32 priors, '?' and -1 both missing); compat = 0 as
 * ML_solver.py:69-74 (priors normalised over each site's dict, the mass of
 * unobserved mutated states kept as one extra state, -1 = silenced).
 * Sites are sorted by state count (descending) and packed into groups of
 * `group_sites` (8, 16 or 32) sites; see laml_dataset_encode. */
typedef struct laml_dataset_info {
    int32_t n_leaves, n_sites, n_sites_pad, n_groups, group_sites;
    int64_t row_len;     /* floats per node row (sum over groups of max_C * group_sites) */
    int32_t max_states;  /* max over sites of (mutated states + 2) */
    int64_t n_missing;   /* '?' entries */
    int64_t n_silenced;  /* LAML_CHAR_SILENCED entries */
} laml_dataset_info;

int laml_dataset_measure(int32_t n_leaves, int32_t n_sites, const int32_t* chars,
                         const int32_t* prior_ptr, const int32_t* prior_state,
                         const double* prior_prob, int32_t compat, int32_t group_sites,
                         laml_dataset_info* info);

/* Fill the layout: codes[n_leaves * n_sites_pad] (int16, layout site order:
 * 0 = unmutated, >= 2 = state slot, -1 missing, -2 silenced), q[row_len]
 * (prior of slot j of layout site c at group_off[g] + j*group_sites + lane),
 * site_perm[n_sites_pad] (original site of each layout site, -1 padding),
 * site_C[n_sites_pad] (states incl. unmutated and silenced), site_sumq[],
 * group_off[n_groups], group_C[n_groups], state_map[] (CSR by original site:
 * the original state of slot 2+i; offsets in state_ptr[n_sites+1]).
 * Returns LAML_ERR_PRIOR (with the site and state in laml_last_error) when an
 * observed state has no prior. Replaces fast_em/phylogeny.py:48-114. */
int laml_dataset_encode(int32_t n_leaves, int32_t n_sites, const int32_t* chars,
                        const int32_t* prior_ptr, const int32_t* prior_state,
                        const double* prior_prob, int32_t compat, int32_t group_sites,
                        int16_t* codes, float* q, int32_t* site_perm, int32_t* site_C,
                        float* site_sumq, int32_t* group_off, int32_t* group_C,
                        int32_t* state_ptr, int32_t* state_map);

/* Batch plan: the level schedule and buffer offsets of many trees.
 * Trees are given in the laml_newick_encode numbering, concatenated. */
typedef struct laml_plan_input {
    int32_t n_trees;
    const int32_t* tree_nodes;     /* [T] N_p */
    const int32_t* tree_leaves;    /* [T] n_p */
    const int32_t* tree_dataset;   /* [T] */
    const int32_t* child0;         /* [sum N_p] local ids, -1 for leaves */
    const int32_t* child1;
    int32_t n_datasets;
    const int32_t* ds_groups;      /* [D] */
    const int32_t* ds_sites_pad;   /* [D] */
    const int64_t* ds_row_len;     /* [D] */
    const int32_t* ds_group_base;  /* [D] offset of the dataset's groups in group_C */
    const int32_t* group_C;        /* [sum groups] */
    const int32_t* ds_sites;       /* [D] real sites */
    const int32_t* ds_leaves;      /* [D] rows of the dataset's code matrix */
    const int32_t* group_off;      /* [sum groups] offset of each group in a row */
} laml_plan_input;

typedef struct laml_plan_sizes {
    int64_t n_nodes;
    int64_t part_floats;   /* floats of one partial buffer (internal nodes only) */
    int64_t scalar_len;    /* per-(internal node, site) scalars */
    int64_t site_len;      /* per-(tree, site) slots */
    int64_t count_floats;  /* count partials: 8 per (node, group) */
    int64_t post_len;      /* per-(node, site) posterior slots */
    int32_t n_in_levels, n_out_levels;
    int64_t n_in_items, n_out_items, n_root_items;
    int64_t n_groups_total;
} laml_plan_sizes;

typedef struct laml_plan_output {
    /* trees [T] */
    int32_t *tr_node_base, *tr_root, *tr_quirk;
    int64_t *tr_site_base, *tr_cnt_base, *tr_post_base;
    /* nodes [n_nodes] */
    int32_t *nd_tree, *nd_c0, *nd_c1, *nd_parent, *nd_sib, *nd_leafrow;
    int64_t *nd_prow, *nd_srow;
    /* schedule */
    int32_t* in_level_off;   /* [n_in_levels + 1] */
    int32_t* in_items;       /* [2 * n_in_items] (node, group), inside by height */
    int32_t* out_level_off;  /* [n_out_levels + 1] */
    int32_t* out_items;      /* [2 * n_out_items] (internal parent, group), by parent depth */
    int32_t* root_items;     /* [2 * n_root_items] */
    /* item descriptors, 12 int32 per item, parallel to in_items / out_items:
     * {u, v, w, tree | flags << 24}, {group, global group, srow(u), prow(u)/8},
     * {ref(v), ref(w), srow(v), srow(w)} with ref = prow/8 for an internal
     * child and the leaf row for a leaf; flags: 1 v is a leaf, 2 w is a leaf,
     * 4 u is the root */
    int32_t* in_desc;
    int32_t* out_desc;
    /* per global group, 8 int32: {group_off, first site (global), q offset,
     * dataset}, {code offset, sites_pad, real sites, 0} */
    int32_t* grp_desc;
    /* optional, instead of in_items / out_items (left NULL) when every
     * dataset of the batch has the same group count NG: the internal nodes
     * in the schedule's order, [internal nodes] each.  Item k of a level
     * with item offset o and c nodes is node lnodes[o / NG + (k - o) % c]
     * of group (k - o) / c -- laml_plan_descriptors expands them on the
     * device (4 bytes a node to copy instead of 8 a (node, group) item). */
    int32_t* in_lnodes;
    int32_t* out_lnodes;
} laml_plan_output;

int laml_plan_measure(const laml_plan_input* in, laml_plan_sizes* sizes);
int laml_plan_fill(const laml_plan_input* in, laml_plan_output* out);

/* Depth schedule of one binary tree for the ultrametric M-step
 * (LAML_MSTEP_ULTRAMETRIC): parent[N] holds tree-local parent ids (-1 at the
 * root).  Writes out[0] = L (levels: depths 0..L-1), out[1..L+1] = level
 * offsets, then the N node ids grouped by depth from the root down (level l
 * is out[L + 2 + out[1 + l] .. L + 2 + out[2 + l])).  `out_len` must be at
 * least 2 * N + 2; *written receives N + L + 2.  The schedule stands in for
 * the treeswift postorder walk of EM_solver.ultrametric_constr
 * (EM_solver.py:53-89): the equalities it builds at every internal node are
 * met by construction when the solve works on node heights, and the
 * elimination of the heights' Newton systems runs one depth level at a
 * time. */
int laml_ultra_order(const int32_t* parent, int32_t n_nodes, int32_t* out, int64_t out_len,
                     int64_t* written);

/* ------------------------------------------------------------------------
 * Device batch: every pointer is a device address
 * --------------------------------------------------------------------- */
typedef struct laml_batch {
    int32_t group_sites;     /* G: 8, 16 or 32 (must match the datasets) */
    int32_t compat;          /* 1 fast_em semantics, 0 EM_solver semantics */
    int32_t n_trees, n_datasets;
    int64_t n_nodes;
    int32_t n_in_levels, n_out_levels;
    int64_t n_in_items, n_out_items, n_root_items;
    /* datasets [D] */
    const int32_t *ds_sites, *ds_sites_pad, *ds_groups, *ds_group_base, *ds_site_base;
    const int64_t *ds_q_base, *ds_code_base;
    const double *ds_missing, *ds_silenced;      /* counts over the real sites */
    const int32_t *group_off, *group_C, *site_C;
    const float *site_sumq, *q;
    const int16_t* codes;
    /* trees [T] */
    const int32_t *tr_ds, *tr_node_base, *tr_nodes, *tr_leaves, *tr_root, *tr_quirk;
    const int64_t *tr_site_base, *tr_cnt_base, *tr_post_base;
    double *tr_nu, *tr_phi;
    double* tr_prev;               /* [2T] nu, phi before the last M-step */
    const uint8_t* tr_fix;         /* bit0: nu fixed, bit1: phi fixed */
    double *tr_llh, *tr_llh_prev;
    int32_t *tr_iter, *tr_status;  /* status: LAML_TREE_* */
    int32_t* tr_mode;              /* arithmetic of the tree's partials, set by
                                    * laml_branch_terms and the M-step:
                                    * LAML_MODE_LINEAR or LAML_MODE_LOG */
    /* nodes [n_nodes] */
    const int32_t *nd_tree, *nd_c0, *nd_c1, *nd_parent, *nd_sib, *nd_leafrow;
    const int64_t *nd_prow, *nd_srow;
    double *nd_d, *nd_d_prev;
    const uint8_t* nd_mask;        /* 1 = branch length is optimised */
    float* nd_bt;                  /* [4 * n_nodes] P00, Pmut, Pstay, Psil */
    double* nd_cnt;                /* [6 * n_nodes] expected counts summed over sites */
    float* nd_stage;               /* [5 * n_nodes] M-step scratch (trees over 2048 nodes) */
    /* work buffers */
    float *in_part, *out_part, *in_dot;
    int32_t *in_x, *in_h, *out_x, *out_h;
    double* llh_site;              /* [site_len] per (tree, layout site) */
    float* root_lr;
    int32_t* root_x;
    float* cnt_part;               /* [count_floats] */
    float *post0, *post1;          /* [post_len] or NULL */
    /* schedule */
    const int32_t *in_level_off, *in_items, *out_level_off, *out_items, *root_items;
    const int32_t *in_desc, *out_desc, *grp_desc;   /* laml_plan_output's descriptors */
    /* optional HOST copies of in_level_off / out_level_off: when set, the
     * per-level entry points launch without reading the offsets back from the
     * device (no stream synchronisation) */
    const int32_t *h_in_level_off, *h_out_level_off;
    /* control */
    uint32_t* barrier;             /* 2 words, zeroed by the library before each persistent launch */
    int32_t* error;                /* 1 word: 0 or a negative LAML_ERR_* set on the device */
    /* the largest group_C of the batch's datasets (states incl. unmutated and
     * silenced).  > 0 selects the staged per-level kernels, which copy each
     * item's partial rows into shared memory with the bulk-copy engine
     * (cp.async.bulk) one item ahead of the computation; 0 keeps the direct
     * kernels.  A group above it sets LAML_ERR_ARG in the error word. */
    int32_t max_states;
    /* the largest tree's node count.  The M-step runs trees above 16384 nodes
     * on a cluster of 8 blocks each (reductions through distributed shared
     * memory); 0 = unknown, in which case that kernel is launched every
     * M-step and skips the smaller trees. */
    int32_t max_tree_nodes;
    /* [2T] FP32 leaf emission terms of each tree's phi (max(1-phi, eps),
     * max(phi, eps) in compat; 1-phi, phi in exact), kept by
     * laml_branch_terms and the M-step; NULL = derived from tr_phi wherever
     * needed */
    float* tr_leaf;
    /* Ultrametric M-step (LAML_MSTEP_ULTRAMETRIC) only, else NULL:
     * nd_uorder [2 * n_nodes + 2 * n_trees] -- tree p's depth schedule from
     * laml_ultra_order at offset 2 * tr_node_base[p] + 2 * p;
     * nd_uwork [LAML_UWORK_SLOTS * n_nodes] -- FP64 scratch of the solve. */
    const int32_t* nd_uorder;
    double* nd_uwork;
    /* the plan's part_floats and scalar_len (laml_plan_sizes): the sizes of
     * in_part and of in_x / in_h / in_dot; laml_inside_noalloc refuses a
     * batch without them */
    int64_t plan_part_floats, plan_scalar_len;
    /* [2T] or NULL: per tree, the '?' entry count and the site count the
     * M-step uses for phi and for the exact model's count normalisation in
     * place of its dataset's -- the totals over all ranks when the tree's
     * sites are split across ranks and cnt_part holds the reduced counts */
    const double* tr_mstats;
    /* the wide levels' kernel (more than 8192 items): 0 = per-thread row
     * loads; 8 or 16 = rows copied into per-warp shared-memory stages by the
     * bulk-copy engine, that many state slots per stage (4 or 2 stages).  A
     * tiling choice only (laml_gb300/tune.py picks it): results are bitwise
     * the same. */
    int32_t wide_chunk;
    /* limit in ns of every device-side wait (the persistent kernel's grid
     * barrier, the staged kernels' mbarrier phases): 0 = 2 s.  A wait that
     * runs out sets LAML_ERR_TIMEOUT in the error word, waits (2 s at most)
     * for its own copies in flight and returns; the context stays usable.
     * Negative: give up at the first check that finds the wait unsatisfied
     * (to exercise that path). */
    int64_t wait_limit_ns;
    /* LAML_MSTEP_LBFGS only, else NULL: [LAML_LBFGS_SLOTS * (n_nodes + 2 T)]
     * FP32 vectors of the L-BFGS solve */
    float* nd_lbfgs;
    /* nonzero: the wide levels run on producer/consumer warp pairs -- a
     * producer warp copies each slab's rows (wide_chunk state slots per
     * stage, 0 = 8) into shared memory with the bulk-copy engine, and
     * stores the per-site scalars there, while its consumer warp computes
     * the previous slabs from there.  Overrides the wide_chunk kernel choice; results are
     * bitwise the same.  in_part and out_part must start on 16-byte
     * boundaries. */
    int32_t wide_pc;
    /* laml_plan_output's in_lnodes / out_lnodes on the device, read by
     * laml_plan_descriptors when in_items / out_items are NULL (every
     * dataset with the same group count) */
    const int32_t *in_lnodes, *out_lnodes;
} laml_batch;

/* A tree's partials are FP32 values with power-of-two exponents (linear)
 * unless some branch has d (1 + nu) > LAML_LOG_MODE_RATE: then they are FP32
 * natural logs (the reference's own representation), whose range covers the
 * branch lengths fast_em's root row can produce. */
#define LAML_MODE_LINEAR 0
#define LAML_MODE_LOG 1
#define LAML_LOG_MODE_RATE 30.0

#define LAML_TREE_ACTIVE 0
#define LAML_TREE_CONVERGED 1
#define LAML_TREE_NAN 2
#define LAML_TREE_MAXITER 3
/* the ultrametric M-step's constraints admit no branch lengths in
 * [dmin, dmax] (EM_solver.Mstep's "d_infeasible", EM_solver.py:419-420,
 * 491-495): the tree keeps the parameters and log-likelihood it had before
 * that M-step */
#define LAML_TREE_INFEASIBLE 4

/* Number of sites per group the kernels were built for (bit mask of 8|16|32). */
int laml_supported_group_sites(void);

/* Builds in_desc / out_desc / grp_desc (laml_plan_output's layout, byte for
 * byte) on the device from the batch's node arrays, items (or level node
 * lists, in_lnodes / out_lnodes, when the items are NULL) and dataset
 * tables, so a caller uploads the node arrays only (the descriptors are 48
 * bytes per item, most of a batch's host->device bytes otherwise).  Outputs
 * are device buffers of 12 * n_in_items, 12 * n_out_items and
 * 8 * (total groups) int32, 16-byte aligned; the batch's own descriptor
 * pointers are not read.  laml_plan_fill must have accepted the batch (its
 * 32-bit range check covers these descriptors).  No reference counterpart:
 * the reference walks the tree objects on the host for every pass. */
int laml_plan_descriptors(const laml_batch* b, int32_t* in_desc, int32_t* out_desc,
                          int32_t* grp_desc, void* stream);

/* Branch transition terms from nd_d, tr_nu (compat adds the EPS floors of
 * fast_em/calculations.py:153-157).  Replaces the t1/t2/t3/alpha0 arrays. */
int laml_branch_terms(const laml_batch* b, void* stream);

/* Inside pass of every tree + per-site and per-tree log-likelihood (FP64 sum
 * over sites); with `update_em` = 1 it also records llh_prev = llh.
 * Replaces calc.compute_log_likelihood / jit_compute_log_likelihood
 * (fast_em/calculations.py:456-504, fast_em/laml.py:80) and the inside half
 * of EM_solver.Estep_in_llh / lineage_llh (laml_libs/EM_solver.py:91-141). */
int laml_inside(const laml_batch* b, int32_t update_em, void* stream);

/* laml_outside flags */
#define LAML_OUT_POSTERIORS 1  /* also P(v = 0 | D), P(v = silenced | D) into post0/post1 */
#define LAML_OUT_TRUE_ROOT 2   /* root counts from the progenitor in state 0 even in compat */

/* Outside pass + expected transition counts per (node, site group) in
 * cnt_part (C00, C0a, C0s, Caa, Cas, Css, P(silenced|D) at '?' leaf entries,
 * at observed leaf entries).  Requires laml_inside first.  In compat mode the
 * root's row follows parent_sibling[root] = (-1, -1) -> node N-1 unless
 * LAML_OUT_TRUE_ROOT.  Replaces calc.compute_E_step
 * (fast_em/calculations.py:506-577) and EM_solver.Estep_out_llh /
 * Estep_posterior (laml_libs/EM_solver.py:143-300). */
int laml_outside(const laml_batch* b, int32_t flags, void* stream);

/* d logL / d branch length (grad_d[n_nodes], device) and d logL / d(nu, phi)
 * per tree (grad_nu_phi[2T], device) from the counts of
 * laml_outside(LAML_OUT_TRUE_ROOT).  No reference counterpart computes the
 * exact gradient; it is the adjoint of the inside pass (the outside pass
 * reused as the backward) and equals the gradient of the M-step objective
 * (fast_em/laml.py:62-78) at the current parameters with true root counts. */
int laml_gradient(const laml_batch* b, double* grad_d, double* grad_nu_phi, void* stream);

/* M-step flags: FP64 Newton polish of the final branch-length and nu solves
 * (the solves otherwise run FP32 Newton iterations with FP64 accumulation). */
#define LAML_MSTEP_FP64_POLISH 1
/* Exact model only: branch lengths maximise the M-step objective jointly
 * under EM_solver's ultrametric equalities (every root-to-leaf path of a
 * tree has the same length; EM_solver.ultrametric_constr, EM_solver.py:53-89,
 * used at 358-361) and the bounds [dmin, dmax]; the root's own branch is in
 * no equality and is solved alone.  Needs nd_uorder and nd_uwork.  Fixed
 * branches (nd_mask = 0) enter the equalities with their lengths, as the
 * reference's node.constant does; a tree whose constraints admit no solution
 * gets LAML_TREE_INFEASIBLE.  Ignored in compat mode (the fastEM path has no
 * such constraint). */
#define LAML_MSTEP_ULTRAMETRIC 2
/* With LAML_MSTEP_ULTRAMETRIC: solve with the log-barrier method alone (the
 * primal-dual method's fallback) instead of the primal-dual method first --
 * slower, kept selectable so both stay checked. */
#define LAML_MSTEP_ULTRA_BARRIER 4
/* With LAML_MSTEP_ULTRAMETRIC: stop the primal-dual method after 3 iterations
 * and let the log-barrier method continue from the point it reached (the
 * fallback the solve takes when the primal-dual method has not converged in
 * 60 iterations), so that path stays checked. */
#define LAML_MSTEP_ULTRA_PD_SHORT 8
/* Compat model only: the M-step the reference itself runs -- 100 FP32
 * L-BFGS steps (memory 10, zoom line search for the strong Wolfe conditions,
 * a chained backtracking test) on the M_step_loss_fn objective over
 * (log d, logit nu, logit phi) (fast_em/laml.py:49-110, optax.lbfgs) --
 * instead of solving that objective to its stationary point.  Needs
 * nd_lbfgs.  One team per tree, ~60 block synchronisations per step: meant
 * for trees of a few thousand nodes. */
#define LAML_MSTEP_LBFGS 16
/* floats per node and per tree parameter of laml_batch.nd_lbfgs */
#define LAML_LBFGS_SLOTS 25
/* doubles per node of laml_batch.nd_uwork */
#define LAML_UWORK_SLOTS 17

/* M-step of every active tree: compat maximises the fastEM objective
 * (fast_em/laml.py:62-78) by `rounds` coordinate-ascent rounds; exact follows
 * EM_solver.Mstep (laml_libs/EM_solver.py:307-459) with bounded 1-D solves.
 * Writes nd_d (old values to nd_d_prev), tr_nu, tr_phi and the branch terms. */
int laml_mstep(const laml_batch* b, int32_t rounds, int32_t flags, void* stream);

/* `iters` fused EM iterations (outside+counts -> M-step -> inside ->
 * convergence test per tree) in ONE persistent cooperative launch with a
 * bounded grid barrier; trees whose status leaves ACTIVE stop changing.
 * `rel_tol` is the stopping rule (1e-5 in fast_em/laml.py:183, 1e-8 in
 * EM_solver.py:503); max_iters caps tr_iter.  Requires laml_inside(update_em=1)
 * once before the first call.  Replaces the host EM loop of
 * fast_em/laml.py:112-194 / EM_solver.EM_optimization. */
int laml_em_run(const laml_batch* b, int32_t iters, int32_t rounds, double rel_tol,
                int32_t max_iters, int32_t flags, void* stream);

/* Same iterations as laml_em_run, one kernel launch per tree level (no grid
 * barrier); the reference-shaped "plain" path. */
int laml_em_run_levels(const laml_batch* b, int32_t iters, int32_t rounds, double rel_tol,
                       int32_t max_iters, int32_t flags, void* stream);

/* The inside pass (per-tree log-likelihood into tr_llh, per-site values into
 * llh_site / root_lr / root_x) without allocating any device memory.  No
 * counterpart exists in the reference: it is for callers that must not call
 * cudaMalloc -- a host runtime that owns the device memory budget and forbids
 * a library from growing its footprint, or a latency-bound scoring loop that
 * cannot afford the device-wide synchronisation cudaMalloc/cudaFree imply.
 * The inside partials and per-(node, site) scalars (b->in_part, in_x, in_h,
 * in_dot are ignored) live in one fixed 32 MiB array inside the library that
 * every GPU which loads the library holds until the process exits; the caller
 * passes the batch's plan sizes (laml_plan_sizes.part_floats / scalar_len) and
 * a batch whose 4 * part_floats + 12 * scalar_len bytes (plus alignment)
 * exceed 32 MiB is rejected with LAML_ERR_ARG, and so are sizes below the
 * batch's own plan sizes (laml_batch.plan_part_floats / plan_scalar_len,
 * which must be filled).  The first call on each device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  The address is
 * kept for the life of the process: it does not survive cudaDeviceReset (or
 * any other teardown of the device's primary context) in the same process,
 * after which this entry point must not be called on that device.  Every call shares
 * the one array: calls whose work overlaps on the GPU race and must be
 * serialised by the caller (one stream, or events).  Nothing in the array has
 * to start at zero: the pass writes every word it reads. */
int laml_inside_noalloc(const laml_batch* b, int64_t part_floats, int64_t scalar_len,
                        void* stream);

/* Capture `iters` EM iterations (as laml_em_run, or as laml_em_run_levels when
 * `persistent` = 0, which needs h_in_level_off / h_out_level_off) into a CUDA
 * graph bound to the buffers of `b`; laml_graph_launch replays it on a stream
 * (one graph launch per call).  The graph must be destroyed before the
 * batch's buffers are freed.  Replaces the per-iteration dispatch of the
 * reference's host EM loop (fast_em/laml.py:153-192). */
int laml_em_graph_create(const laml_batch* b, int32_t iters, int32_t rounds, double rel_tol,
                         int32_t max_iters, int32_t flags, int32_t persistent, void** graph);
/* The EM loop itself as one CUDA graph: a conditional WHILE node repeats
 * `chunk` fused EM iterations (laml_em_graph_create's body) while some tree
 * is LAML_TREE_ACTIVE, no error is recorded and fewer than max_chunks
 * chunks ran in this launch -- the convergence test runs on the device
 * after every chunk, so one laml_graph_launch runs EM to convergence with no
 * host round trip (fast_em/laml.py:141-194's loop; the reference syncs the
 * host every iteration).  `counter` is one device int32, zero when the graph
 * is created, that the graph counts its chunks in (and leaves at zero after
 * every launch); it must outlive the graph and not be shared by two graphs
 * launched concurrently.  Destroy with laml_graph_destroy. */
int laml_em_graph_loop_create(const laml_batch* b, int32_t chunk, int32_t rounds,
                              double rel_tol, int32_t max_iters, int32_t flags,
                              int32_t max_chunks, int32_t* counter, void** graph);
int laml_graph_launch(void* graph, void* stream);
void laml_graph_destroy(void* graph);

/* Message of the calling thread's last error ("" if none). */
const char* laml_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* LAML_GB300_H */
