/* argweaver_gb300 — the chromosome-threading HMM of ARGweaver on one GB300 (sm_103a).
 *
 * Two groups of entry points:
 *
 *  1. The reference's C ABI for the threading HMM, same names, signatures and ownership
 *     rules (libargweaver.so, declared by the reference's ctypes prototypes in
 *     argweaver/argweaverc.py:133-167). A ctypes or C caller of the reference switches
 *     libraries without code changes. Results are host memory allocated with new[], freed
 *     by the matching delete_* export of this library.
 *
 *  2. A flat batch API (awg_*) over plain arrays: many problems per call, FP64 or FP32
 *     compute, explicit uniforms, device-resident sessions for serving.
 *
 * Threading and randomness: as in the reference, the C-ABI samplers draw their uniforms
 * from libc rand() (one per column, last column first: common.h:103-110,
 * sample_thread.cpp:522-569), so srand(seed) reproduces the reference's draws. Calls are
 * synchronous. Errors: the reference returns no codes (it asserts); these entry points
 * log to stderr and return NULL / leave outputs untouched, and awg_last_error() holds the
 * message. Nothing here traps the device.
 */
#ifndef ARGWEAVER_GB300_H
#define ARGWEAVER_GB300_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------
 * Reference-compatible C ABI
 * --------------------------------------------------------------------------------- */

/* A (node, time) state, as the reference's intstate (states.h:135). */
typedef int awg_intstate[2];

/* Opaque local-tree set. Replaces LocalTrees* (local_tree.h:504) on the C-ABI surface. */
typedef struct awg_local_trees awg_local_trees;

/* arghmm_new_trees (local_tree.cpp:1817): trees from parent arrays (leaves first), age
 * indices, SPRs (recomb_node, recomb_time, coal_node, coal_time) and block lengths; node
 * mappings follow make_node_mapping (local_tree.h:767). */
awg_local_trees *arghmm_new_trees(int **ptrees, int **ages, int **sprs, int *blocklens,
                                  int ntrees, int nnodes, int start_coord);
/* delete_local_trees (local_tree.cpp:1895) */
void delete_local_trees(awg_local_trees *trees);
/* get_local_trees_ntrees / _nnodes (local_tree.cpp:1838-1847) */
int get_local_trees_ntrees(awg_local_trees *trees);
int get_local_trees_nnodes(awg_local_trees *trees);

/* get_local_trees_ptrees (local_tree.cpp:1846-1890): parents, ages, SPRs and block lengths
 * of every tree, into ntrees rows of the caller's arrays. Leaf i is named by the sequence
 * it holds (awg_local_trees_seqids) when those ids are a permutation of the leaves, as the
 * reference names them; otherwise by its own index. */
void get_local_trees_ptrees(awg_local_trees *trees, int **ptrees, int **ages, int **sprs,
                            int *blocklens);

/* The sequence each leaf holds (LocalTrees::seqids, local_tree.h:673) into nleaves ints
 * (NULL: count only). Returns nleaves, or -1 (awg_last_error). */
int awg_local_trees_seqids(awg_local_trees *trees, int *seqids);

/* The node mappings from each previous tree (ntrees x nnodes, row 0 all -1), in the names
 * get_local_trees_ptrees shows: after awg_add_arg_thread or awg_remove_arg_thread they are
 * no longer the default. 0, or -1 (awg_last_error). */
int awg_local_trees_mapping(awg_local_trees *trees, int *mapping);

/* Each node's two children (ntrees x nnodes each, -1 for none) in the order the trees keep
 * them, in the names get_local_trees_ptrees shows. 0, or -1 (awg_last_error). */
int awg_local_trees_children(awg_local_trees *trees, int *c0, int *c1);

/* Node mappings (ntrees x nnodes, row 0 ignored; NULL: make_node_mapping) and each root's
 * child[0] (NULL: children in index order) of trees whose structure the parent arrays do
 * not carry (an ARG after surgery). 0, or -1 (awg_last_error). */
int awg_local_trees_set_structure(awg_local_trees *trees, const int *mapping,
                                  const int *root_child0);

/* add_arg_thread (thread.cpp:272-422), on the host: the thread of a new last leaf (a state
 * path over the trees' columns, external trees) and its recombinations (columns, nodes
 * (-1: the new branch), times; e.g. from awg_sample_recombinations) added to the trees,
 * which grow by two nodes and one tree per recombination. 0, or -1 (awg_last_error). */
int awg_add_arg_thread(awg_local_trees *trees, int ntimes, const int *path, int seqlen,
                       const int *rec_pos, const int *rec_node, const int *rec_time, int nrec);

/* remove_arg_thread (thread.cpp:425-556), on the host: the leaf holding sequence `seqid`
 * leaves every tree (the last leaf takes its index, with its sequence id), SPRs on the
 * removed branch vanish and trees left without an SPR merge into the next
 * (remove_null_sprs, local_tree.cpp:409-469). 0, or -1 (awg_last_error). */
int awg_remove_arg_thread(awg_local_trees *trees, int seqid);

/* Removal paths (thread.cpp:1681-1703): one node per tree, in the trees' own node names, into
 * `path` (ntrees ints), drawn from libc rand() as the reference draws them. From `node` of the
 * first tree forward (sample_arg_removal_path, :793-799); through `node` of the block holding
 * coordinate `pos`, forward and backward (:772-790); the leaf path, no draws (:672-700).
 * Errors: awg_last_error(). */
void arghmm_sample_arg_removal_path(awg_local_trees *trees, int node, int *path);
void arghmm_sample_arg_removal_path2(awg_local_trees *trees, int node, int pos, int *path);
void arghmm_sample_arg_removal_leaf_path(awg_local_trees *trees, int node, int *path);

/* A removal path that prefers branches carrying recombinations (weight recomb_preference
 * where the SPR recombines, 1 - recomb_preference elsewhere; thread.cpp:800-912, bound at
 * :1698-1702), drawn from libc rand(). Errors: awg_last_error(). */
void arghmm_sample_arg_removal_path_recomb(awg_local_trees *trees, double recomb_preference,
                                           int *path);

/* A removal path drawn uniformly over all of them (sample_arg_removal_path_uniform,
 * thread.cpp:963-1002, which arg-sample's subtree cuts use); returns the log number of paths,
 * NaN on error. */
double awg_sample_arg_removal_path_uniform(awg_local_trees *trees, int *path);

/* remove_arg_thread_path (thread.cpp:1481-1668, bound at :1705-1709): the ARG cut along a
 * removal path into subtree/main-tree form (each cut regrafted above the root at `maxtime`,
 * ntimes + 1 in arg-sample), trees without an SPR merged. Errors: awg_last_error(). */
void arghmm_remove_arg_thread_path(awg_local_trees *trees, int *removal_path, int maxtime);

/* arghmm_remove_arg_thread_path2 (thread.cpp:1711-1715): the same cut, and the removed
 * thread as state indices of the cut trees into original_thread (one int per column; 0
 * where a tree has no states). */
void arghmm_remove_arg_thread_path2(awg_local_trees *trees, int *removal_path, int maxtime,
                                    int *original_thread);

/* arghmm_get_thread_times (thread.cpp:1718-1733): the time of each column's internal state
 * along a thread path; like the reference, path and path_times are indexed by coordinate
 * (start_coord + column). Columns of a whole tree (no states) get -1, where the reference
 * reads past its empty state list. Errors: awg_last_error(). */
void arghmm_get_thread_times(awg_local_trees *trees, int ntimes, int *path, int *path_times);

/* add_arg_thread_path (thread.cpp:1314-1449), on the host: every partial tree's cut subtree
 * regrafted at the state its internal thread path (internal states with `minage`; e.g. from
 * arghmm_sample_arg_thread_internal) takes at the tree's first column, the trees split at
 * the path's recombinations (columns, nodes, times; e.g. from awg_sample_recombinations on
 * the internal problem). 0, or -1 (awg_last_error). */
int awg_add_arg_thread_path(awg_local_trees *trees, int ntimes, int minage, const int *path,
                            int seqlen, const int *rec_pos, const int *rec_node,
                            const int *rec_time, int nrec);

/* sample_arg_thread (sample_thread.cpp:575-625) for sequence new_chrom of the full sequence
 * set (nseqs rows; the leaves read the rows of their sequence ids): the threading step of
 * arghmm_sample_thread, the new leaf holding new_chrom (resample_arg_leaf's re-threading,
 * sample_arg.cpp:66-86, after awg_remove_arg_thread). 0, or -1 (awg_last_error). */
int awg_sample_arg_thread(awg_local_trees *trees, double *times, int ntimes, double *popsizes,
                          double rho, double mu, char **seqs, int nseqs, int seqlen,
                          int new_chrom);

/* sample_arg_thread_internal (sample_thread.cpp:635-692): the cut subtree of trees in
 * subtree/main-tree form re-threaded in place, forward, traceback and recombinations on the
 * device (draws from libc rand()), the regraft on the host; the thread path into thread_path
 * (seqlen ints) when not NULL. 0, or -1 (awg_last_error). */
int awg_sample_arg_thread_internal(awg_local_trees *trees, double *times, int ntimes,
                                   double *popsizes, double rho, double mu, char **seqs,
                                   int nseqs, int seqlen, int minage, int *thread_path);

/* get_state_spaces (states.cpp:228-251): each tree's states as (node, time) pairs, one new[]
 * row per tree (arghmm_get_nstates' counts per column give the row lengths); free with
 * delete_state_spaces (:255-260). As the reference's, `internal` is accepted and the
 * external states are listed. */
typedef int awg_intstate[2]; /* intstate (states.h:135) */
awg_intstate **get_state_spaces(awg_local_trees *trees, int ntimes, bool internal);
void delete_state_spaces(awg_intstate **all_states, int ntrees);

/* read_local_trees (local_tree.cpp:1908-1932): a trees handle from an SMC file (.gz read
 * through gzip), times snapped to the given grid; NULL and awg_last_error() on failure. */
awg_local_trees *read_local_trees(const char *filename, const double *times, int ntimes);

/* arghmm_copy_trees (local_tree.cpp:1827-1832): an independent copy of the handle. */
awg_local_trees *arghmm_copy_trees(awg_local_trees *trees);

/* get_local_trees_blocks (local_tree.cpp:1946-1958): [start, end) of every tree. */
void get_local_trees_blocks(awg_local_trees *trees, int *starts, int *ends);

/* get_treelens (local_tree.cpp:1935-1943): every tree's total branch length (times[] units,
 * no basal stub). */
void get_treelens(awg_local_trees *trees, const double *times, int ntimes, double *treelens);

/* arghmm_get_nstates (states.cpp:209): states of every column. */
void arghmm_get_nstates(awg_local_trees *trees, int ntimes, bool internal, int *nstates);

/* arghmm_forward_alg (sample_thread.cpp:887-926): FP64 forward table, seqlen rows of
 * max(nstates,1) doubles; free with delete_forward_matrix. slow: the reference's dense
 * S x S test step (arghmm_forward_block_slow, sample_thread.cpp:301-337) instead of the
 * structured one; the same table up to rounding. */
double **arghmm_forward_alg(awg_local_trees *trees, double *times, int ntimes,
                            double *popsizes, double rho, double mu, char **seqs, int nseqs,
                            int seqlen, bool prior_given, double *prior, bool internal,
                            bool slow);

/* arghmm_backward_alg: NEW (the reference has no backward pass for the threading HMM).
 * Same arguments as arghmm_forward_alg minus prior/slow; table layout as the forward
 * table, each column normalised to sum 1; free with delete_forward_matrix. */
double **arghmm_backward_alg(awg_local_trees *trees, double *times, int ntimes,
                             double *popsizes, double rho, double mu, char **seqs, int nseqs,
                             int seqlen, bool internal);

/* arghmm_posterior_marginals: NEW. Posterior state marginals P(state at column i | data)
 * from forward-backward, layout as the forward table; free with delete_forward_matrix. */
double **arghmm_posterior_marginals(awg_local_trees *trees, double *times, int ntimes,
                                    double *popsizes, double rho, double mu, char **seqs,
                                    int nseqs, int seqlen, bool internal);

/* arghmm_sample_posterior (sample_thread.cpp:930-977): forward + stochastic traceback on
 * trees given as arrays; returns (node, time) per column (allocated when path == NULL).
 * The reference converts every block over [start, start+blocklen) of the block start
 * (an inner `end` shadows the outer one, sample_thread.cpp:959-962); this export converts
 * each column with its own block's state space. Free with delete_path. */
awg_intstate *arghmm_sample_posterior(int **ptrees, int **ages, int **sprs, int *blocklens,
                                      int ntrees, int nnodes, double *times, int ntimes,
                                      double *popsizes, double rho, double mu, char **seqs,
                                      int nseqs, int seqlen, awg_intstate *path);

/* arghmm_sample_arg_thread_internal (sample_thread.cpp:981-1006): forward + traceback for
 * an internal branch; writes the state index of every column into thread_path[seqlen]. */
void arghmm_sample_arg_thread_internal(awg_local_trees *trees, double *times, int ntimes,
                                       double *popsizes, double rho, double mu, char **seqs,
                                       int nseqs, int seqlen, int *thread_path);

/* arghmm_sample_thread (sample_thread.cpp:1010-1023): threads the last sequence (nseqs =
 * the trees' leaves + 1) into the trees, in place: forward and traceback on the device
 * (rand() draws as arghmm_sample_posterior), recombinations along the thread on the device
 * (draws continuing rand(); 2 * seqlen + 2 are taken, the reference's number used) and the
 * thread added on the host (add_arg_thread). Returns trees; on failure they are unchanged
 * and awg_last_error() says why. */
awg_local_trees *arghmm_sample_thread(awg_local_trees *trees, double *times, int ntimes,
                                      double *popsizes, double rho, double mu, char **seqs,
                                      int nseqs, int seqlen);

/* delete_path / delete_double_matrix / delete_forward_matrix (sample_thread.cpp:1026-1042) */
void delete_path(int *path);
void delete_double_matrix(double **mat, int nrows);
void delete_forward_matrix(double **mat, int nrows);

/* The reference's dense helper matrices (its ctypes layer's aids for tests and plots),
 * formed by the table kernel (and, for emissions, the emission kernel) on the GPU in FP64
 * and gathered into the caller's state order. istates are (node, time) pairs of the tree's
 * coalescence states in any order (a pair that is no state of the tree is an error: NULL,
 * awg_last_error). treelen, time_steps and the lineage counts are accepted and not read:
 * the kernels derive them from the tree, as the reference recomputes them.
 *
 * new_transition_probs (trans.cpp:1190-1208): [nstates][nstates], log P(i -> j) within
 * the tree (TransMatrix::get_log, trans.h:64-83, 130-133). Free with
 * delete_transition_probs (trans.cpp:1248-1251). */
double **new_transition_probs(int nnodes, int *ptree, int *ages, double treelen,
                              awg_intstate *istates, int nstates, int ntimes, double *times,
                              double *time_steps, int *nbranches, int *nrecombs, int *ncoals,
                              double *popsizes, double rho);
/* new_transition_probs_switch (trans.cpp:1212-1245): [nstates1][nstates2], log P(i -> j)
 * from last_ptree's states to ptree's across the SPR (TransMatrixSwitch::get_log,
 * trans.h:200-219), the node mapping make_node_mapping's (local_tree.h:767-778). */
double **new_transition_probs_switch(int *ptree, int *last_ptree, int nnodes, int recomb_node,
                                     int recomb_time, int coal_node, int coal_time,
                                     int *ages_index, int *last_ages_index, double treelen,
                                     double last_treelen, awg_intstate *istates1, int nstates1,
                                     awg_intstate *istates2, int nstates2, int ntimes,
                                     double *times, double *time_steps, int *nbranches,
                                     int *nrecombs, int *ncoals, double *popsizes, double rho);
void delete_transition_probs(double **transmat, int nstates);
/* new_emissions (emit.cpp:1288-1301): [seqlen][nstates], P(column i | state j) of the
 * threaded sequence seqs[nseqs - 1] on the tree (calc_emissions_external, emit.cpp:
 * 650-845; not in log). Free with delete_emissions (emit.cpp:1304-1307). */
double **new_emissions(awg_intstate *istates, int nstates, int *ptree, int nnodes,
                       int *ages_index, char **seqs, int nseqs, int seqlen, double *times,
                       int ntimes, double mu);
void delete_emissions(double **emit, int seqlen);

/* Probabilities of a whole ARG (total_prob.cpp:315-382; bound by
 * argweaver/argweaverc.py:219-245), computed on the device. arghmm_likelihood: log P(seqs |
 * ARG), sequences one per leaf (leaf i = seqs[i]) covering start_coord .. end of the trees;
 * arghmm_prior_prob: log P(ARG) of the recombination spacing and SPRs; arghmm_tree_prior_prob:
 * the first tree's coalescent prior; arghmm_joint_prob: likelihood + prior. NaN and
 * awg_last_error() on invalid input. */
double arghmm_likelihood(awg_local_trees *trees, double *times, int ntimes, double mu,
                         char **seqs, int nseqs, int seqlen);
double arghmm_prior_prob(awg_local_trees *trees, double *times, int ntimes, double *popsizes,
                         double rho);
double arghmm_tree_prior_prob(awg_local_trees *trees, double *times, int ntimes,
                              double *popsizes);
double arghmm_joint_prob(awg_local_trees *trees, double *times, int ntimes, double *popsizes,
                         double mu, double rho, char **seqs, int nseqs, int seqlen);

/* Input formats, on the host (arg-sample's ingest, arg-sample.cpp:996-1155): a sites file
 * (sequences.cpp:172-297) compressed by `compress` bases per non-variant column
 * (find_compress_cols, sequences.cpp:523-592; make_sequences_from_sites, :315-343, default
 * base 'A'), and optionally an SMC file of local trees (read_local_trees,
 * local_tree.cpp:1422-1540; ages snapped to `times`) compressed the same way
 * (compress_local_trees, local_tree.cpp:818-850). Leaves come out permuted so leaf i is
 * sequence i (get_local_trees_ptrees, local_tree.cpp:1846); the SMC's leaves must be the
 * first sequences of the sites file. ".gz" files are read through gzip. NULL and
 * awg_formats_last_error() on failure. */
typedef struct awg_arg_input awg_arg_input;
awg_arg_input *awg_read_arg_input(const char *sites_path, const char *smc_path, int compress,
                                  const double *times, int ntimes);
int awg_arg_input_dims(const awg_arg_input *in, int *nseqs, int *seqlen, int *ntrees,
                       int *nnodes, int *start_coord);
const char *awg_arg_input_name(const awg_arg_input *in, int i);
/* seqs: nseqs x seqlen; ptrees, ages: ntrees x nnodes; sprs: ntrees x 4; any may be NULL */
int awg_arg_input_copy(const awg_arg_input *in, char *seqs, int *ptrees, int *ages, int *sprs,
                       int *blocklens);
void awg_free_arg_input(awg_arg_input *in);
/* write_sites (sequences.cpp:133-157): the columns whose bases differ, 1-based */
int awg_write_sites(const char *path, const char *const *names, int nseqs, const char *chrom,
                    int start_coord, int seqlen, const char *seqs);
/* write_local_trees (local_tree.cpp:1286-1362) for trees numbered by the default node
 * mapping (a tree keeps the previous tree's node numbers; the broken node recoalesces) */
int awg_write_smc(const char *path, const char *const *names, const char *chrom,
                  int start_coord, const int *ptrees, const int *ages, const int *sprs,
                  const int *blocklens, int ntrees, int nnodes, const double *times,
                  int ntimes);
const char *awg_formats_last_error(void);

/* The dense HMM over a full nstates x nstates log transition matrix (hmm.h:14-19,
 * hmm.cpp:27-85; bound by argweaver/argweaverc.py:42-56). Tables are n row pointers of
 * nstates doubles, in natural log. As in the reference the caller fills the boundary:
 * fw[0] before forward_alg, bw[n-1] before backward_alg, path[n-1] before
 * sample_hmm_posterior, which draws one rand() per column from n-2 down to 0. */
void forward_alg(int n, int nstates, double **trans, double **emit, double **fw);
void backward_alg(int n, int nstates, double **trans, double **emit, double **bw);
void sample_hmm_posterior(int n, int nstates, double **trans, double **fw, int *path);

/* ---------------------------------------------------------------------------------
 * Flat batch API
 * --------------------------------------------------------------------------------- */

/* One threading problem over plain arrays (the arrays arghmm_new_trees takes). */
typedef struct {
    int ntrees, nnodes, ntimes, nseqs, seqlen, internal, start_coord, minage;
    const int *ptrees;      /* [ntrees*nnodes] parent (-1 for the root), leaves first */
    const int *ages;        /* [ntrees*nnodes] age as a time index */
    const int *sprs;        /* [ntrees*4] SPR to the left of each tree (row 0 unused) */
    const int *blocklens;   /* [ntrees] columns of each tree */
    const int *mapping;     /* [ntrees*nnodes] node map from the previous tree, or NULL */
    const int *root_child0; /* [ntrees] child[0] of each root, or NULL (index order);
                               internal-branch trees name their cut subtree there */
    const double *times;    /* [ntimes] time points */
    const double *popsizes; /* [ntimes] population sizes (diploid N, as the reference) */
    double rho, mu;         /* per column */
    const char *seqs;       /* [nseqs*seqlen] rows: leaves in leaf order, then (external)
                               the sequence being threaded; bytes A,C,G,T (either case), N */
    double infsites_penalty; /* ArgModel::infsites_penalty (model.h:53, arg-sample
                               --infsites: 1e-100): the emissions of states that break the
                               infinite-sites model are multiplied by it (emit.cpp:847-862);
                               outside (0, 1), e.g. 0 from a zeroed struct: off */
} awg_problem;

enum { AWG_FP64 = 0, AWG_FP32 = 1 };

/* Outputs of one problem in a batch. Any pointer may be NULL (not wanted). Tables are
 * packed column after column, max(nstates,1) entries per column. */
typedef struct {
    double *forward;        /* [cells] forward table (FP64 compute) */
    float *forward32;       /* [cells] forward table (FP32 compute) */
    double *posterior;      /* [cells] posterior marginals */
    int *path;              /* [seqlen] sampled state index per column */
    double *loglik;         /* [1] sum over columns i>=1 of log(column norm) */
    const double *uniforms; /* [seqlen] input: u[i] drives the draw at column i; NULL
                               draws from libc rand() in the reference's order */
} awg_outputs;

/* Number of forward-table cells of a problem (sum over columns of max(nstates,1)),
 * or -1 when the problem is invalid. */
long long awg_problem_cells(const awg_problem *p);

/* awg_problem_cells of n problems at once into cells[n], the problems checked in parallel
 * (all but their sequence bytes, which awg_run_batch checks). Returns 0, or -1 with
 * awg_last_error() naming the first invalid problem. */
int awg_problems_cells(const awg_problem *problems, int n, long long *cells);

/* Run forward (+ traceback when path is wanted, + backward when posterior is wanted) for
 * n problems in one batch on the current device. precision: AWG_FP64 or AWG_FP32.
 * Returns 0 on success, a negative code on error (awg_last_error() has the message). */
int awg_run_batch(const awg_problem *problems, awg_outputs *outputs, int n, int precision);

/* Batches in flight from one thread (no counterpart in the reference): a context plans,
 * uploads and enqueues a batch (awg_batch_launch returns once its kernels are queued), and
 * awg_batch_finish waits for it and hands its outputs to the caller's buffers. Two contexts
 * used in turn keep the GPU busy while the host plans and uploads the next batch. Each
 * context owns its own streams, page-locked staging and device arena (grown as needed and
 * kept), and replays a batch shape it has seen from a CUDA graph. The output buffers and
 * uniforms must stay valid until awg_batch_finish; a context runs one batch at a time
 * (launch, finish, launch, ...). Both return 0 or a negative code (awg_last_error); results
 * equal awg_run_batch's. */
typedef struct awg_batch_ctx awg_batch_ctx;
awg_batch_ctx *awg_batch_ctx_create(void);
int awg_batch_launch(awg_batch_ctx *ctx, const awg_problem *problems, awg_outputs *outputs,
                     int n, int precision);
int awg_batch_finish(awg_batch_ctx *ctx);
void awg_batch_ctx_destroy(awg_batch_ctx *ctx);

/* Device bytes awg_run_batch needs for this batch with these outputs wanted (the size of a
 * server pool or of a region to set aside), or a negative code (awg_last_error). */
long long awg_batch_device_bytes(const awg_problem *problems, int n, int precision, int want_path,
                                 int want_posterior);

/* sample_recombinations (recomb.cpp:151-235), on the device, external or internal-branch:
 * the recombinations along a sampled thread path (path: the state index of every column, as
 * awg_outputs.path and the reference's thread_path hold it). The draws are the caller's
 * uniforms, consumed in order, one per draw: rand()/RAND_MAX after srand(seed) reproduces
 * the reference's recombinations. Returns their count, their columns, nodes (-1: the new
 * thread's branch of an external problem; internal ones name the cut subtree's root) and
 * times in pos/node/time (cap entries), and the uniforms used; or a negative code
 * (awg_last_error). At most 2 * seqlen uniforms are used. */
int awg_sample_recombinations(const awg_problem *problem, const int *path,
                              const double *uniforms, int n_uniforms, int *pos, int *node,
                              int *time, int cap, int *used);

/* Autotuner (no counterpart in the reference): runs the batch under each candidate
 * schedule (states per owner thread of the forward kernel, i.e. its CTA size; instance
 * group cap of the pipelined schedule; trees per work unit of the persistent per-tree
 * kernels; persistent or one CTA per tree), each `trials` times, coordinate by coordinate
 * from the defaults, and keeps the fastest for the batch's shape class (precision, path
 * wanted, ntimes, binary magnitudes of the largest state count and of the batch size);
 * later awg_run_batch calls of that class use it. outputs receive the last run's results.
 * report (optional) receives "kpt=.. group_div=.. chunk=.. persistent=.. ms=..".
 * Returns 0 or a negative code as awg_run_batch. */
int awg_autotune(const awg_problem *problems, awg_outputs *outputs, int n, int precision,
                 int trials, char *report, int report_len);

/* Forward (FP64) and stochastic traceback of ONE problem conditioned at its ends, for the
 * reference's conditioned samplers (cond_sample_arg_thread[_internal],
 * sample_thread.cpp:708-865, which fill the first forward column and fix the last state
 * before calling arghmm_forward_alg and stochastic_traceback). prior: the first column's
 * max(S0,1) values (NULL: the state prior); last_state: the last column's state (-1: drawn
 * from the last column, as usual). uniforms: seqlen draws as awg_outputs.uniforms (u[L-1]
 * unused when last_state >= 0); NULL draws libc rand() as the reference does: one per column
 * from the last drawn column down to column 0. path: seqlen state indices; loglik optional.
 * Returns 0 or a negative code (awg_last_error). */
int awg_sample_path_conditioned(const awg_problem *problem, const double *prior,
                                int last_state, const double *uniforms, int *path,
                                double *loglik);

/* Frees the batch engine's grow-only device arena, its page-locked staging and captured
 * graph (the next awg_run_batch allocates again). Returns 0. */
int awg_release_memory(void);

/* CUDA graphs (no counterpart in the reference): awg_run_batch captures the device part of
 * a step (kernels, memsets, cross-stream dependencies) once and replays it while a batch
 * has the same launch parameters (sizes, buffers, schedule); on by default. */
void awg_set_graphs(int on);
/* The default schedule (what the autotuner chooses among): kpt = states per owner thread
 * of the forward kernel (1, 2, 4, 8; 0 = by the largest state count), group_div, chunk as
 * awg_autotune; persistent 0 launches one CTA per tree. Forgets the autotuner's choices.
 * Results do not depend on the schedule (every sum has an order fixed by the tree). */
void awg_set_schedule(int kpt, int group_div, int chunk, int persistent);
long long awg_graph_replays(void);
long long awg_graph_captures(void);

/* ---------------------------------------------------------------------------------
 * Serving loop (no counterpart in the reference): continuous batching of threading
 * requests. Requests from any thread queue FIFO; a worker forms batches from the queue head
 * (one precision and one set of wanted outputs, as many as fit the free device memory and
 * max_batch) and keeps up to max_inflight of them on the GPU at once, each on its own
 * streams and region of one device pool allocated at creation (no allocation while
 * serving). Requests arriving while others run are admitted as a batch slot and memory
 * free up; their kernels overlap the running ones. A request's results equal those of the
 * same problem run alone.
 * --------------------------------------------------------------------------------- */
typedef struct awg_server awg_server;
typedef struct {
    size_t device_bytes;  /* device pool for batches in flight (and resident requests) */
    int max_inflight;     /* batches on the GPU at once */
    int max_batch;        /* problems per batch */
    double length_ratio;  /* a batch's requests have column counts within this factor of its
                             oldest request's (a batch lasts as long as its longest chain);
                             <= 1, e.g. 0 from a zeroed struct: 2 */
} awg_server_options;
typedef struct {
    long long submitted, completed, failed, cells;  /* cells: forward cells of completed */
    double p50_ms, p99_ms, mean_ms, max_ms;  /* latency, submission to results in place */
    double span_s;        /* first submission to last completion */
    double busy_s;        /* time with at least one batch on the GPU */
    double launch_s;      /* server thread time spent planning and launching batches */
    int inflight_max;     /* most batches on the GPU at once */
    double queue_p50_ms, queue_p99_ms;      /* submission to admission into a batch */
    double service_p50_ms, service_p99_ms;  /* admission to results in place */
} awg_server_stats;

awg_server *awg_server_create(const awg_server_options *opt);  /* NULL: awg_server_last_error */
void awg_server_destroy(awg_server *s);  /* finishes queued and running requests first */
/* Queues one problem; its arrays (and out->uniforms) are copied, out's result buffers must
 * stay valid until the request completes. resident: keep the request's device data after
 * it completes for awg_server_resample, until awg_server_release (a path must be wanted).
 * Returns the request id (> 0) or -1 (awg_server_last_error). */
long long awg_server_submit(awg_server *s, const awg_problem *p, const awg_outputs *out,
                            int precision, int resident);
/* Waits up to timeout_ms (< 0: no limit): 1 done (results in place), 0 still pending,
 * < 0 failed (awg_server_last_error). */
int awg_server_wait(awg_server *s, long long id, int timeout_ms);
/* submission, start (admitted to a batch) and completion times (seconds, steady clock) */
int awg_server_request_times(awg_server *s, long long id, double *times3);
/* forgets a finished, non-resident request (its id becomes unknown) */
int awg_server_forget(awg_server *s, long long id);
int awg_server_stats_get(awg_server *s, awg_server_stats *out);
/* A new path from a completed resident request: the traceback alone over its resident
 * forward table with these uniforms (NULL: libc rand(), the reference's order). */
int awg_server_resample(awg_server *s, long long id, const double *uniforms, int *path);
int awg_server_release(awg_server *s, long long id);
const char *awg_server_last_error(void);

/* Bytes of device memory awg_forward_static draws all of its buffers from. */
#define AWG_STATIC_SCRATCH_BYTES (64ull << 20)

/* Forward table and log-likelihood of ONE problem, allocating nothing: no cudaMalloc or
 * cudaFree, no page-locked host memory, no memory pool. No counterpart in the reference.
 * The results equal awg_run_batch's for the same problem and precision.
 *
 * For callers that cannot allocate device memory: a process whose device memory belongs
 * to another allocator (a framework's caching allocator, a per-process memory cap), or a
 * loop on its own stream that cannot afford cudaFree's implicit device-wide
 * synchronisation, which awg_run_batch incurs when its arena grows.
 *
 * Every device buffer (inputs, tables, forward table, error record) is carved out of one
 * file-scope device array of AWG_STATIC_SCRATCH_BYTES (64 MiB). A problem whose buffers
 * exceed it is rejected before any device work: return -5, awg_last_error() gives both
 * sizes. (FP64, a problem of S states per column and L columns needs a little over 8*S*L
 * bytes: S = 300 fits about 25,000 columns.)
 *
 * Set-up: the first call on each device, with that device current, loads the module that
 * holds the array (cudaGetSymbolAddress). Every call resolves the array's address again in
 * the current context, so a context destroyed and recreated in between (cudaDeviceReset)
 * is safe. Each call copies from pageable host memory and waits for its stream.
 * Zeroing: only the 16-byte error record has to start at zero, and each call clears it
 * itself (cudaMemsetAsync). Every other byte of the array is written before it is read.
 * Concurrency: the array is shared by every call on a device. Calls that overlap in time
 * (from several host threads, or streams of several threads) race on it and corrupt each
 * other's results: serialise them. A call returns after its stream has finished its work,
 * also when it fails after work was enqueued.
 *
 * output: forward (AWG_FP64) or forward32 (AWG_FP32) and loglik may be set, as in
 * awg_outputs; path and posterior must be NULL. stream: a cudaStream_t, NULL for the
 * default stream. Returns 0, or a negative code with awg_last_error() set. */
int awg_forward_static(const awg_problem *problem, awg_outputs *output, int precision,
                       void *stream);

/* Message of the last error on this thread ("" when none). */
const char *awg_last_error(void);

/* Device and library information: device name and the number of kernels launched by
 * this process so far (every kernel of this library counts). */
int awg_device_name(char *buf, int len);
long long awg_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* ARGWEAVER_GB300_H */
