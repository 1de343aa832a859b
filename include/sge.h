/*
 * sge.h — C ABI of the GB300 subgraph-enumeration executor (libsge.so).
 *
 * The library replaces the execution half of the reference's
 * `graph_mining_system`: everything after the plan hand-off
 * (main.cpp:64-86 serial, main.cpp:171-193 OpenMP), i.e. the calls
 *   sharedJoin(t, pt, query, cs, trieLevels, visited, result, count, ...)
 *       (matching/join.h:39-41, matching/join.cpp:812-1200)
 *   parSharedJoin(t, pt, query, [DataGraph g,] cs, trieLevels, visited, result, count, traverse)
 *       (matching/parallel.h:88-94, matching/parallel.cpp:1154-1844)
 * and the data structures those read: the CSR data graph
 * (relation/graph.h:113-213), the candidate-space accessors of unlabeled mode
 * (relation/candidate_space.cpp:763-799) and the plan facts produced by
 * plan/optimizer.cpp + plan/decomposition.cpp (flattened into sge_plan_blob).
 *
 * Conventions
 *  - Every entry point returns an sge_status; on failure sge_last_error()
 *    returns a one-line message (thread-local).  The library never calls exit().
 *  - Vertex ids and CSR offsets are uint32 (the reference's VertexID/EdgeID,
 *    config/config.h:42-44); counts are uint64 and wrap like the reference's
 *    size_t accumulator.
 *  - Handles are not thread-safe; calls are stream-ordered on one internal
 *    CUDA stream per graph handle.
 *  - No torch types, no C++ types: plain pointers and sizes only.
 */
#ifndef SGE_H
#define SGE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGE_ABI_VERSION 2u
#define SGE_MAX_K 16u          /* pattern vertices supported by the device executor */
#define SGE_MAX_TAIL 4u        /* levels counted (not enumerated) at the leaf */
#define SGE_MAX_PARTITIONS 15u /* set partitions of a 4-vertex tail (Bell(4)) */
#define SGE_PLAN_MAGIC 0x4E4C5053u /* "SPLN" */

typedef enum sge_status {
    SGE_OK = 0,
    SGE_BAD_INPUT = 1,      /* malformed graph/pattern/plan/argument */
    SGE_OOM = 2,            /* host or device allocation failed */
    SGE_TIMEOUT = 3,        /* a launch exceeded its time budget (partial count kept) */
    SGE_STACK_OVERFLOW = 4, /* a per-warp buffer would have overflowed (never silently) */
    SGE_CUDA_ERROR = 5,     /* a CUDA runtime call failed */
    SGE_UNSUPPORTED = 6,    /* pattern/plan shape outside the executor's limits */
    SGE_IO_ERROR = 7,       /* file could not be opened or was truncated */
    SGE_NO_DEVICE = 8       /* no CUDA device visible */
} sge_status;

/* Leaf counting modes (how the last tail_len levels are counted without
 * enumerating them).  They restate the reference's traverse() variants,
 * matching/join.cpp:1520-1691:
 *   SINGLE  = TrieLevel::numResults on one last level (relation/relation.cpp:301-338)
 *   CHOOSE  = symmLastLevel: choosec(num, r)              (join.cpp:1534-1538, utils.cpp:80-94)
 *   IEP     = groups / numUniqueCombine inclusion–exclusion (join.cpp:1556-1568, utils.cpp:290-350) */
typedef enum sge_tail_mode {
    SGE_TAIL_SINGLE = 1,
    SGE_TAIL_CHOOSE = 2,
    SGE_TAIL_IEP = 3
} sge_tail_mode;

/* Join style.  WCOJ computes a level's candidates when the level is reached
 * (generateCandidates, join.cpp:180-242); EXPLORATION intersects N(v) into the
 * running candidate list of every later neighbour as soon as v is matched and
 * prunes on an empty list (generateCandidates(DataGraph…), join.cpp:266-307;
 * the reference's -i flag).  Counts are identical by construction. */
typedef enum sge_join_style {
    SGE_JOIN_WCOJ = 0,
    SGE_JOIN_EXPLORATION = 1
} sge_join_style;

/* Root restriction between level 0 and level 1 (the two ends of the root edge). */
typedef enum sge_root_kind {
    SGE_ROOT_ANY = 0,      /* both orientations of every undirected edge */
    SGE_ROOT_ASC = 1,      /* only m[0] < m[1] (getEdges(type), candidate_space.cpp:787-799) */
    SGE_ROOT_DESC = 2      /* only m[0] > m[1] */
} sge_root_kind;

/*
 * Plan blob: POD flattening of the facts the executor reads (the role of
 * HyperTree + PrefixNode after refineIntersectionInfo, plan/decomposition.h:53-207).
 * Levels are positions in the matching order; masks are over levels.
 *
 *   candidates(i) = ∩_{j ∈ parents[i]} N(m[j])
 *                   ∩ { x : x > m[j] ∀ j ∈ lower[i] }        (largerAttrs, setBeginPos)
 *                   ∩ { x : x < m[j] ∀ j ∈ upper[i] }        (smallerAttrs, setEndPos)
 *                   \ { m[j] : j ∈ check[i] }                 (visited[] / checkExists)
 *   base[i] (>=0): a level whose stored candidate list is a superset of level i's
 *   list (candidatesBefore, plan/decomposition.h:32); rest[i] = the parents
 *   still to intersect.  base[i] == -1: start from N(m[first_parent[i]]).
 *
 * Levels [0, num_enum) are enumerated; levels [num_enum, k) form the tail,
 * counted by tail_mode.  For SGE_TAIL_IEP the count is
 *   Σ_p coef[p] · Π_{b < nblocks[p]} S[block[p][b]]
 * where S[mask] = |∩_{t ∈ mask} candidates(num_enum + t)|.
 * The result per root is multiplied by count_multiplier (1, or |Aut| for
 * single-bag plans: the reference counts embeddings there, instances elsewhere).
 */
typedef struct sge_plan_blob {
    uint32_t magic;             /* SGE_PLAN_MAGIC */
    uint32_t abi_version;       /* SGE_ABI_VERSION */
    uint32_t k;                 /* pattern vertices, 3..SGE_MAX_K */
    uint32_t num_enum;          /* enumerated levels, 2..k-1 */
    uint32_t tail_mode;         /* sge_tail_mode */
    uint32_t tail_len;          /* k - num_enum, 1..SGE_MAX_TAIL */
    uint32_t join_style;        /* sge_join_style */
    uint32_t root_kind;         /* sge_root_kind */
    uint32_t order[SGE_MAX_K];  /* pattern vertex matched at level i */
    uint32_t parents[SGE_MAX_K];
    uint32_t lower[SGE_MAX_K];
    uint32_t upper[SGE_MAX_K];
    uint32_t check[SGE_MAX_K];
    int32_t  base[SGE_MAX_K];
    uint32_t rest[SGE_MAX_K];
    uint32_t first_parent[SGE_MAX_K]; /* used when base[i] == -1 */
    /* IEP partitions of the tail (only for SGE_TAIL_IEP) */
    uint32_t num_partitions;
    int32_t  part_coef[SGE_MAX_PARTITIONS];
    uint32_t part_nblocks[SGE_MAX_PARTITIONS];
    uint32_t part_block[SGE_MAX_PARTITIONS][SGE_MAX_TAIL]; /* masks over tail positions */
    /* count semantics */
    uint64_t count_multiplier;  /* 1 (instances) or |Aut| (single-bag: embeddings) */
    uint64_t aut_size;          /* |Aut(pattern)| */
    uint32_t single_bag;        /* 1 if the reference would run a one-bag plan */
    uint32_t num_restrictions;  /* symmetry-breaking restrictions installed */
    double   est_cost;          /* planner cost estimate (informational) */
    /* CHOOSE leaves: 0 = the exact binomial C(n, r) mod 2^64; 1 = the
     * reference's choosec (utility/utils.cpp:80-94): n(n-1)…(n-r+1) kept in
     * uint64, which wraps once the product reaches 2^64 (from n = 65,538 at r = 4),
     * then divided by r!.  Plans imported from the reference's own planner
     * (sge_plan_from_order_text) use 1, so their "Number of matches" is the
     * reference's even where it wraps.  Either way a product that reaches
     * 2^64 sets bit 2 of sge_stats.status_flags. */
    uint32_t choose_wrap;
    /* 1: planned for vertex labels (sge_plan_opts.vertex_labels): symmetry
     * restrictions from label-preserving automorphisms only, count_multiplier
     * = their number; sge_plan_set_labels must attach the same labels to the
     * plan and sge_graph_set_labels the data graph's before counting. */
    uint32_t labeled;
} sge_plan_blob;

/* Planner options */
typedef struct sge_plan_opts {
    uint32_t join_style;        /* sge_join_style */
    uint32_t use_iep;           /* 0: tails of length 1 only (no -u); 1: longest valid tail (-u) */
    uint32_t max_tail;          /* cap on tail_len (<= SGE_MAX_TAIL) */
    uint64_t seed;              /* seed for sampling-based cost estimates */
    const uint32_t *force_order;/* optional: a full matching order to use (k entries) */
    /* optional: k pattern vertices; every candidate's symmetry restrictions
     * come from the stabilizer chain of this one sequence instead of from its
     * own order.  With root_edge fixed too, all candidates keep the same
     * representative of each instance on the same root pattern edge, so they
     * count the same instances on any root sample (root_stride). */
    const uint32_t *symmetry_seq;
    /* optional: 2 adjacent pattern vertices every candidate order starts
     * with, in either orientation */
    const uint32_t *root_edge;
    /* optional: k pattern vertex labels (labeled matching: a pattern vertex
     * maps only to data vertices with its label; the reference's LabeledGraph
     * and candidate space, relation/candidate_space.cpp:112-760) */
    const uint32_t *vertex_labels;
} sge_plan_opts;

/* Execution options */
typedef struct sge_count_opts {
    uint32_t blocks_per_sm;     /* 0 = occupancy-derived */
    uint32_t warps_per_block;   /* 0 = occupancy-derived (at most 4) */
    uint32_t chunk;             /* root tasks per queue grab; 0 = auto */
    double   time_budget_s;     /* 0 = unlimited; otherwise kernels stop and report SGE_TIMEOUT */
    uint32_t max_level_capacity;/* 0 = graph max degree; smaller values exercise the overflow path */
    uint64_t root_stride;       /* 0/1 = every root edge; s > 1: only the undirected root edges e ≡ root_offset
                                   (mod s), in CSR order (both orientations when a plan's root is unordered) */
    uint64_t root_offset;       /* (root-range sharding across ranks, or sampled runs) */
    uint32_t collect_counters;  /* 1: run the instrumented kernel (set_ops, alg_bytes, partial matches) */
    uint32_t heavy_threshold;   /* 0 = auto (a quarter of a warp's share of the launch's level-2
                                   candidates, at least 32); otherwise roots whose level-2 list may
                                   exceed it are deferred to a second launch that splits each into tasks
                                   of one level-2 candidate and a part of its level-3 list (or, where
                                   level 3 is not enumerated, of up to 128 level-2 candidates) */
    uint32_t no_hub_bitmaps;    /* 1: probe every adjacency list by binary search, ignoring the graph's
                                   hub bitmaps (for comparison runs); 0 = use them */
    uint32_t root_max_degree;   /* 0 = every sampled root; d > 0: only roots whose two endpoints both have
                                   degree <= d (a bounded sub-sample, e.g. for a CPU check) */
    uint32_t pin_tables;        /* per-warp shared-memory tables for the root's lists: 0 = automatic (a
                                   bitmap when n <= 32768; none on larger graphs with a hub index, whose
                                   bitmaps serve the long lists, so more warps stay resident); 1 = none;
                                   2 = 512-slot hashes of the lists of at most 256 on larger graphs */
} sge_count_opts;

/* Statistics of one sge_count call (per call, summed over plans).  kernel_ms,
 * total_ms, gpu_launches and status_flags are always filled; the counters
 * only with sge_count_opts.collect_counters. */
typedef struct sge_stats {
    double   kernel_ms;         /* device time of the counting kernels (CUDA events) */
    double   total_ms;          /* host wall time of the call */
    uint64_t root_tasks;        /* root edges processed */
    uint64_t set_ops;           /* intersections/counting passes executed */
    uint64_t alg_bytes;         /* algorithmic bytes: 4·(|A'|+|B'|) per set operation + 8 B per offset pair */
    uint64_t partial_matches;   /* enumerated partial matches (all levels) */
    uint32_t gpu_launches;      /* kernels launched by this call */
    uint32_t status_flags;      /* bit0 overflow, bit1 timeout, bit2 a CHOOSE leaf's falling product
                                   n(n-1)…(n-r+1) reached 2^64 (the reference's choosec wraps there;
                                   see sge_plan_blob.choose_wrap) */
} sge_stats;

typedef struct sge_graph_info {
    uint32_t num_vertices;
    uint64_t num_directed_edges;  /* 2m */
    uint32_t max_degree;
    uint64_t device_bytes;        /* HBM held by the graph handle (CSR, root edges, hub index) */
    uint32_t hub_count;           /* vertices with a neighbour bitmap in HBM (degree >= hub_min_degree) */
    uint32_t hub_min_degree;      /* 0xFFFFFFFF: no hub index */
} sge_graph_info;

typedef struct sge_graph sge_graph;
typedef struct sge_plan sge_plan;

/* ---- diagnostics ---- */
/* sizeof of the ABI structs, for binding checks: 0 sge_plan_blob,
 * 1 sge_plan_opts, 2 sge_count_opts, 3 sge_stats, 4 sge_graph_info,
 * 5 sge_graph_stats, 6 sge_trie, 7 sge_plan_tuning. */
size_t sge_struct_size(int which);
const char *sge_last_error(void);
const char *sge_version(void);
int sge_device_count(void);

/* ---- host-side graph I/O (replaces DataGraph::loadDataGraph / loadBinaryGraph,
 *      relation/graph.cpp:255-419, and PatternGraph::loadPatternGraph, :661-770) ----
 * Results are malloc'ed; release them with sge_free_host. */
sge_status sge_load_graph_file(const char *path, uint32_t **offsets, uint32_t **nbrs,
                               uint32_t *num_vertices, uint64_t *num_directed_edges);
sge_status sge_save_graph_binary(const char *path, const uint32_t *offsets, const uint32_t *nbrs,
                                 uint32_t num_vertices);
sge_status sge_load_pattern_file(const char *path, uint32_t *k, uint32_t *m, uint32_t *edges /* 2*m, cap 2*SGE_MAX_K*SGE_MAX_K */);
/* Labeled graph in the reference's text format (LabeledGraph::loadLabeldGraphFromText,
 * relation/labeled_graph.cpp:63-143): "t n m", then "v id label degree" per
 * vertex and "e u v" per undirected edge.  Returns the symmetric CSR with
 * lists sorted by id (as sge_load_graph_file) and one label per vertex; all
 * three arrays are malloc'ed (sge_free_host).  Degrees must match the edges. */
sge_status sge_load_labeled_graph_file(const char *path, uint32_t **offsets, uint32_t **nbrs, uint32_t **labels,
                                       uint32_t *num_vertices, uint64_t *num_directed_edges);
/* CSR from an undirected edge list (u,v pairs): symmetric, per-list sorted
 * (Graph::addDirectedEdges, graph.cpp:143-173).  dedup!=0 also removes
 * duplicates and self-loops (the reference does not; its inputs must be clean). */
sge_status sge_csr_from_edges(const uint32_t *edges, uint64_t m, uint32_t num_vertices, int dedup,
                              uint32_t **offsets, uint32_t **nbrs, uint64_t *num_directed_edges);
void sge_free_host(void *p);

/* ---- seeded synthetic generators (deterministic on every host) ---- */
/* R-MAT: 2^scale vertices, m undirected edge draws; a,b,c in units of 1e-6 (d = rest).
 * Output: deduplicated, self-loop-free undirected edges with u<v, sorted. */
sge_status sge_gen_rmat(uint32_t scale, uint64_t m, uint32_t a_ppm, uint32_t b_ppm, uint32_t c_ppm,
                        uint64_t seed, uint32_t **edges, uint64_t *m_out);
/* Chung-Lu: expected degrees ∝ (i+1)^(-1/(gamma-1)), mean 2m/n, capped at
 * max_deg (0 = n-1); m distinct undirected edges, u<v, sorted. */
sge_status sge_gen_chung_lu(uint32_t n, uint64_t m, uint32_t gamma_milli, uint32_t max_deg, uint64_t seed,
                            uint32_t **edges, uint64_t *m_out);
/* Random connected pattern with k vertices and m edges (k-1 <= m <= k(k-1)/2). */
sge_status sge_gen_pattern(uint32_t k, uint32_t m, uint64_t seed, uint32_t *edges /* 2*m */);

/* Degree/clustering statistics the planner's cost model reads (host only). */
typedef struct sge_graph_stats {
    double num_vertices;
    double num_directed_edges;
    double moments[SGE_MAX_K + 2];  /* M_j = Σ_v deg(v)^j */
    double clustering;              /* sampled global clustering coefficient */
    double max_degree;
} sge_graph_stats;
sge_status sge_graph_stats_compute(const uint32_t *offsets, const uint32_t *nbrs, uint32_t num_vertices,
                                   sge_graph_stats *out);

/* ---- planner (host; stands in for optCostPlan + selectSymmetry +
 *      buildTraverseUnlabeled + refineIntersectionInfo, main.cpp:60-69) ---- */
sge_status sge_plan_pattern(uint32_t k, uint32_t m, const uint32_t *edges,
                            const sge_graph *g /* may be NULL: degree stats unknown */,
                            const sge_plan_opts *opts, sge_plan_blob *out);
/* Same, from precomputed statistics (no device needed). */
sge_status sge_plan_pattern_stats(uint32_t k, uint32_t m, const uint32_t *edges, const sge_graph_stats *stats,
                                  const sge_plan_opts *opts, sge_plan_blob *out);
/* |Aut(P)| and whether the reference would run a single-bag plan. */
sge_status sge_pattern_info(uint32_t k, uint32_t m, const uint32_t *edges,
                            uint64_t *aut_size, uint32_t *single_bag);
/* Every executable plan of the pattern, cheapest first by the cost model
 * (at most cap; the chosen plan of sge_plan_pattern_stats is element 0). */
sge_status sge_plan_candidates(uint32_t k, uint32_t m, const uint32_t *edges, const sge_graph_stats *stats,
                               const sge_plan_opts *opts, sge_plan_blob *out, uint32_t cap, uint32_t *n_out);
/* Fixed-length feature vector of a plan for the learned scorer. */
#define SGE_FEATURES 64u
sge_status sge_plan_features(const sge_plan_blob *blob, const sge_graph_stats *stats, float *out);

/* ---- learned plan scorer (the cost slot of optCostOrder, plan/optimizer.cpp:441-577) ----
 * A 3-layer MLP (in → hidden → hidden → 1, ReLU) predicting a plan's log
 * runtime.  Trained on the GPU in FP32 (Adam, MSE); batched inference in BF16
 * on the tensor cores.  Parameters are one flat FP32 array: W1[h×in], b1[h],
 * W2[h×h], b2[h], W3[h], b3[1]. */
typedef struct sge_mlp sge_mlp;
sge_status sge_mlp_create(uint32_t in_dim, uint32_t hidden, uint64_t seed, int device, sge_mlp **out);
sge_status sge_mlp_destroy(sge_mlp *m);
sge_status sge_mlp_num_params(const sge_mlp *m, size_t *n);
sge_status sge_mlp_get_params(const sge_mlp *m, float *out);
sge_status sge_mlp_set_params(sge_mlp *m, const float *in);
sge_status sge_mlp_forward(sge_mlp *m, const float *x, uint32_t batch, float *y);       /* FP32 */
sge_status sge_mlp_forward_bf16(sge_mlp *m, const float *x, uint32_t batch, float *y);  /* BF16 tensor cores */
sge_status sge_mlp_loss_grad(sge_mlp *m, const float *x, const float *t, uint32_t batch, float *loss, float *grads);
sge_status sge_mlp_train(sge_mlp *m, const float *x, const float *t, uint32_t n, uint32_t epochs, uint32_t batch,
                         float lr, uint64_t seed, float *final_loss);
/* Plans with the learned scorer: the cost model's best `shortlist` candidates
 * are scored by the MLP (BF16) and the lowest predicted runtime wins. */
sge_status sge_plan_pattern_learned(uint32_t k, uint32_t m, const uint32_t *edges, const sge_graph_stats *stats,
                                    const sge_plan_opts *opts, sge_mlp *scorer, uint32_t shortlist,
                                    sge_plan_blob *out);

/* Plans with GPU root sampling (the sampled-cardinality cost slot of
 * optCostOrder / cardEstimateUnlabeled, plan/optimizer.cpp:441-577,
 * plan/estimator.cpp:562-661): the cost model's best `shortlist` candidates
 * (0 = 8) each count the root sample t ≡ 0 (mod sample_stride) on g with the
 * instrumented kernel, and the least sampled work (algorithmic bytes + 64 B
 * per set operation) wins.  A candidate is cut off past 0.5 s or four times
 * the fastest sample; if all are, the cost model's choice stands.  sampled_ms
 * (may be NULL; shortlist entries) receives each sample's time, -1 when cut
 * off or absent. */
sge_status sge_plan_pattern_sampled(uint32_t k, uint32_t m, const uint32_t *edges, sge_graph *g,
                                    const sge_plan_opts *opts, uint32_t shortlist, uint64_t sample_stride,
                                    sge_plan_blob *out, double *sampled_ms);

/* Imports the reference's own plan: `text` is the block
 * HyperTree::writeToStream prints after optCostPlan ("num bags: N", then one
 * comma-separated attribute order per bag, the global bag last;
 * plan/decomposition.cpp:537-552, main.cpp:64-66), a whole reference log
 * holding it, or an order file in buildTreesFromOrderFile's format
 * (plan/optimizer.cpp:724-752).  Replaces the planning half of main.cpp:60-69
 * for callers that keep the reference's planner: the global bag's order runs
 * first, then each other bag's own attributes in its order (as the trie join
 * of sharedJoin/globalJoin visits them), with this library's symmetry
 * restrictions for that order; the own attributes are counted at the leaf
 * (the longest tail they allow when opts->use_iep, one level otherwise).  "Number of matches"
 * follows the imported plan's shape: embeddings for one bag, instances for
 * several (relation/graph.cpp:910-1077).  The bags must cover every vertex
 * and every edge of the pattern.  stats may be NULL; opts (may be NULL)
 * gives the join style and whether the leaf may count several levels (-u).
 * num_bags (may be NULL) receives the number of bags read. */
sge_status sge_plan_from_order_text(uint32_t k, uint32_t m, const uint32_t *edges, const char *text,
                                    const sge_graph_stats *stats, const sge_plan_opts *opts, sge_plan_blob *out,
                                    uint32_t *num_bags);

/* Check a plan blob for internal consistency (levels, masks, tail validity). */
sge_status sge_plan_validate(const sge_plan_blob *blob);

/* ---- device graph (replaces the DataGraph/CandidateSpace the join reads) ----
 * Every graph handle also builds a hub index in HBM: a neighbour bitmap for
 * each vertex of degree >= hub_min_degree (sge_graph_info), the smallest
 * threshold whose bitmaps fit in min(4 GB, 1/16 of free device memory, and
 * SGE_HUB_INDEX_MB megabytes when that environment variable is set), so that
 * a membership test in a high-degree vertex's list is one load. */
sge_status sge_graph_create(const uint32_t *offsets, const uint32_t *nbrs, uint32_t num_vertices,
                            uint64_t num_directed_edges, int device, sge_graph **out);
sge_status sge_graph_destroy(sge_graph *g);
sge_status sge_graph_get_info(const sge_graph *g, sge_graph_info *info);
/* ---- device graph ingest (replaces Graph::addDirectedEdges / loadDataGraph's
 *      CSR build on the host, relation/graph.cpp:143-173,255-419) ----
 * Builds the symmetric CSR on the GPU from m undirected edges (u,v) held in
 * device memory on `device` (d_edges: 2m uint32, any order).  Self-loops and
 * duplicates are dropped; an id >= num_vertices is SGE_BAD_INPUT.  No
 * counterpart takes device input in the reference. */
sge_status sge_graph_create_from_device_edges(const uint32_t *d_edges, uint64_t m, uint32_t num_vertices, int device,
                                              sge_graph **out);
/* R-MAT generated on the GPU: the graph of sge_gen_rmat's edges for the same
 * arguments (the same counter-based stream), built as a device graph without
 * a host round trip of the edges.  No counterpart in the reference, whose
 * data graphs come from files. */
sge_status sge_graph_create_rmat(uint32_t scale, uint64_t m, uint32_t a_ppm, uint32_t b_ppm, uint32_t c_ppm,
                                 uint64_t seed, int device, sge_graph **out);
/* Copies a graph's CSR to host arrays (num_vertices+1 offsets, num_directed_edges neighbours);
 * the counterpart of reading DataGraph's offsets/neighbours (relation/graph.h:113-213). */
sge_status sge_graph_copy_csr(const sge_graph *g, uint32_t *offsets, uint32_t *nbrs);

/* ---- compiled plans ---- */
sge_status sge_plan_create(const sge_plan_blob *blob, sge_plan **out);
sge_status sge_plan_destroy(sge_plan *p);
/* Execution choices of one plan, set by an autotuner from a short sampled run
 * (sge_tune.py) or left automatic (all zero).  No counterpart in the
 * reference, whose OpenMP split is fixed at one task per root
 * (matching/parallel.cpp:1270-1273).  Counts never depend on them. */
typedef struct sge_plan_tuning {
    uint32_t heavy_threshold;   /* 0 = automatic; roots whose level-2 bound exceeds it are split */
    uint32_t level3_parts;      /* 0 = automatic; parts of each level-3 list per split task (1 = none) */
    uint32_t no_hub_bitmaps;    /* 1: this plan probes adjacency lists by binary search only */
} sge_plan_tuning;
sge_status sge_plan_set_tuning(sge_plan *p, const sge_plan_tuning *t);
/* Labeled matching.  sge_graph_set_labels uploads one label per data vertex
 * (n values; NULL removes them); sge_plan_set_labels attaches k pattern
 * labels (pattern vertex order; NULL detaches) to a plan planned with the
 * same labels (blob.labeled).  A labeled plan then matches pattern vertex u
 * only to data vertices of label labels[u]: the root edge's ends and every
 * enumerated candidate are checked, and tail levels are counted by a scan
 * that checks labels (not by range size).  WCOJ plans only; bag relations,
 * sge_enumerate, sge_count_host and sge_count_noalloc take unlabeled plans. */
sge_status sge_graph_set_labels(sge_graph *g, const uint32_t *labels);
sge_status sge_plan_set_labels(sge_plan *p, const uint32_t *labels);

/* ---- execution (replaces sharedJoin / parSharedJoin) ----
 * Counts nplans patterns over g in one persistent launch (the batch shares
 * the graph and a global work queue).  counts[i] receives the reference's
 * "Number of matches" for plan i; instances[i] (may be NULL) the count of
 * subgraph instances (embeddings / |Aut|). */
sge_status sge_count(sge_graph *g, const sge_plan *const *plans, uint32_t nplans,
                     const sge_count_opts *opts, uint64_t *counts, uint64_t *instances,
                     sge_stats *stats);
/* sge_count plus, per plan, the warp-milliseconds its roots took inside the
 * batched launch (busy_ms[i]: summed over the warps that ran plan i's roots,
 * both launch phases); what an autotuner compares.  No counterpart in the
 * reference. */
sge_status sge_count_plan_times(sge_graph *g, const sge_plan *const *plans, uint32_t nplans,
                                const sge_count_opts *opts, uint64_t *counts, double *busy_ms, sge_stats *stats);
/* A batch prepared once and replayed from a captured CUDA graph: the plans
 * are uploaded and the launch sequence (counter reset, both launch phases,
 * read-back of counts, flags and counters) is captured at creation; each run
 * is one graph launch.  The batch owns its device buffers; g must outlive it. */
typedef struct sge_batch sge_batch;
sge_status sge_batch_create(sge_graph *g, const sge_plan *const *plans, uint32_t nplans, const sge_count_opts *opts,
                            sge_batch **out);
sge_status sge_batch_run(sge_batch *b, uint64_t *counts, uint64_t *instances, sge_stats *stats);
sge_status sge_batch_destroy(sge_batch *b);
/* ---- enumeration and bag relations (nodeJoin + buildTrie, matching/join.cpp:309-421,1713-1717;
 *      TrieLevel::buildTrieFromSortedMatchesBatch, relation/relation.cpp:340-379) ---- */
/* Writes every match of p (one per automorphism class: the representative
 * the plan's restrictions keep) as k uint32 vertex ids in pattern-vertex
 * order into the device buffer d_out (capacity rows).  *n_matches receives
 * the number of matches; more than capacity returns SGE_OOM (rows past
 * capacity are dropped).  The plan must have a one-level tail (no IEP). */
sge_status sge_enumerate(sge_graph *g, const sge_plan *p, uint32_t *d_out, uint64_t capacity, uint64_t *n_matches);
/* Automorphisms of a pattern: naut rows of k vertex images (cap rows max). */
sge_status sge_pattern_automorphisms(uint32_t k, uint32_t m, const uint32_t *edges, uint8_t *out, uint32_t cap,
                                     uint32_t *naut);
/* Replaces each device row (k ids, pattern-vertex order) by the
 * lexicographically smallest of its images under the automorphisms (perms:
 * host array naut×k), i.e. a plan-independent form of each instance. */
sge_status sge_canonicalize(uint32_t *d_tuples, uint64_t n, uint32_t k, const uint8_t *perms, uint32_t naut);
/* Lexicographic sort of n device rows of `arity` uint32 (LSD radix sort). */
sge_status sge_sort_tuples(uint32_t *d_tuples, uint64_t n, uint32_t arity);
/* Trie of sorted rows: level l holds level_len[l] values (device);
 * node p of level l < arity-1 owns children [child[l][p], child[l][p+1]). */
#define SGE_TRIE_MAX_LEVELS 16u
typedef struct sge_trie {
    uint32_t arity;
    uint64_t level_len[SGE_TRIE_MAX_LEVELS];
    uint32_t *values[SGE_TRIE_MAX_LEVELS];
    unsigned long long *child[SGE_TRIE_MAX_LEVELS];
} sge_trie;
sge_status sge_trie_build(const uint32_t *d_sorted, uint64_t n, uint32_t arity, sge_trie *out);
sge_status sge_trie_free(sge_trie *t);
/* Copies level `level` of a trie to host: level_len[level] values and, below
 * the last level, level_len[level]+1 child offsets (child may be NULL). */
sge_status sge_trie_copy_level(const sge_trie *t, uint32_t level, uint32_t *values, unsigned long long *child);
/* The sorted instance set (what -r writes; the reference never writes one):
 * one row per instance, each row the lexicographically smallest image of an
 * embedding under the automorphisms, rows sorted.  p must have a one-level
 * tail.  *n_rows receives the instance count; SGE_OOM when above cap_rows. */
sge_status sge_match_set(sge_graph *g, const sge_plan *p, uint32_t k, uint32_t m, const uint32_t *edges,
                         uint32_t *host_out, uint64_t cap_rows, uint64_t *n_rows);

/* ---- the bag-relation join (sharedJoin's trie lookups, matching/join.cpp:812-1200) ----
 * sge_bags_create materialises, on graph g, the relation of every bag of the
 * decomposition in plan_text (the text sge_plan_from_order_text reads) that
 * has exactly one attribute of its own and 3 or 4 attributes: all embeddings
 * of the bag's sub-pattern (nodeJoin, join.cpp:309-421), sorted into a trie
 * (buildTrie, join.cpp:1713-1717) keyed by the bag's other attributes in
 * ascending vertex order, the bag's own attribute last.  The first key level
 * is indexed by vertex id.  Other bags are skipped, and so is a bag whose
 * relation holds more than max_rows tuples (0 = no limit; 2^32 - 1 at most):
 * its tail level keeps intersecting adjacency lists.
 *
 * sge_plan_use_bags makes up to two tail levels of a WCOJ plan read their
 * candidate list from a relation: the level of a bag's own vertex, when every
 * key of the bag is an enumerated level.  Each leaf candidate then looks its
 * key tuple up once (one dense step, one binary search per further key) and
 * counts or probes that range in place of intersecting the vertex's
 * adjacency lists.  The counts do not change.  *levels (may be NULL)
 * receives the number of such levels; b = NULL detaches.  The bags must
 * outlive every count and batch that uses the plan, on the graph they were
 * built on (another graph returns SGE_BAD_INPUT). */
typedef struct sge_bags sge_bags;
sge_status sge_bags_create(sge_graph *g, uint32_t k, uint32_t m, const uint32_t *edges, const char *plan_text,
                           uint64_t max_rows, sge_bags **out);
/* Relations built, their total tuples and device bytes, and the bags skipped
 * for max_rows; own_vertices (may be NULL, one entry per relation) receives
 * each relation's own pattern vertex.  Every output may be NULL. */
sge_status sge_bags_info(const sge_bags *b, uint32_t *num_relations, uint64_t *rows, uint64_t *device_bytes,
                         uint32_t *own_vertices, uint32_t *num_skipped);
sge_status sge_bags_destroy(sge_bags *b);
sge_status sge_plan_use_bags(sge_plan *p, const sge_bags *b, uint32_t *levels);

/* End-to-end convenience: host CSR in, counts out (H2D copy, count, D2H read
 * and release all inside the call). */
sge_status sge_count_host(const uint32_t *offsets, const uint32_t *nbrs, uint32_t num_vertices,
                          uint64_t num_directed_edges, const sge_plan_blob *blobs, uint32_t nplans,
                          const sge_count_opts *opts, uint64_t *counts, sge_stats *stats);

/* ---- counting without any device allocation ----
 * No counterpart in the reference.  For callers that must not allocate
 * device memory after set-up: code running under a host framework that owns
 * the GPU's memory pool, real-time callers with a fixed memory budget, or
 * callers between graph-capture boundaries.  The caller owns every input and
 * output buffer.  The working memory of the launch is a file-scope device
 * array of SGE_NOALLOC_SCRATCH_BYTES that every GPU which loads the library
 * keeps until the process exits.
 *   d_offsets, d_nbrs: device CSR (symmetric, sorted lists, uint32)
 *   max_degree:        an upper bound on the largest list (a smaller value is
 *                      reported as SGE_STACK_OVERFLOW, never silently wrong)
 *   plans:             host plan blobs (at most SGE_NOALLOC_MAX_PLANS)
 *   d_counts:          device uint64[nplans]; receives "Number of matches"
 *   stream:            a cudaStream_t (NULL = the default stream)
 * The call is synchronous on `stream` (it reads back the status).  Each call
 * looks up the array's device address with the current device selected, so
 * a context that was torn down and rebuilt (cudaDeviceReset) is picked up; a
 * call made while `stream` is capturing reuses the address of the device's
 * last call outside capture, so make the first call on a device before any
 * stream capture.  All calls share
 * the one array, so calls whose launches overlap on the GPU race: serialise
 * them (one stream, or one call at a time per device).  A graph or plan batch
 * whose per-warp lists do not fit in the array is rejected with
 * SGE_UNSUPPORTED. */
#define SGE_NOALLOC_SCRATCH_BYTES (32u << 20)
#define SGE_NOALLOC_MAX_PLANS 64u
sge_status sge_count_noalloc(const uint32_t *d_offsets, const uint32_t *d_nbrs, uint32_t num_vertices,
                             uint64_t num_directed_edges, uint32_t max_degree, const sge_plan_blob *plans,
                             uint32_t nplans, uint64_t *d_counts, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SGE_H */
