/* CPU restatement of the reference's chromosome-threading HMM (ARGweaver).
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library: as the checker the CUDA path is compared against,
 * and as the timed CPU port of the reference. It is pinned against the compiled
 * reference through the golden fixtures in tests/golden/ (see tests/golden/make_golden.py).
 *
 * All functions return 0 on success and a negative code on invalid input.
 */
#ifndef AWG_ORACLE_H
#define AWG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* One threading problem (same layout as awg_problem in include/argweaver_gb300.h). */
typedef struct {
    int ntrees, nnodes, ntimes, nseqs, seqlen, internal, start_coord, minage;
    const int *ptrees;      /* [ntrees*nnodes] parent (-1 for the root) */
    const int *ages;        /* [ntrees*nnodes] age as a time index */
    const int *sprs;        /* [ntrees*4] recomb_node, recomb_time, coal_node, coal_time */
    const int *blocklens;   /* [ntrees] */
    const int *mapping;     /* [ntrees*nnodes] or NULL (make_node_mapping) */
    const int *root_child0; /* [ntrees] or NULL (children in index order) */
    const double *times;    /* [ntimes] */
    const double *popsizes; /* [ntimes] */
    double rho, mu;         /* per column */
    const char *seqs;       /* [nseqs*seqlen] */
    double infsites_penalty; /* ArgModel::infsites_penalty (model.h:53); outside (0, 1): off */
} oracle_problem;

/* Number of states of every column (arghmm_get_nstates, states.cpp:209). */
int oracle_nstates(const oracle_problem *p, int *nstates);

/* Forward table (arghmm_forward_alg, sample_thread.cpp:394-460): column i holds
 * max(nstates_i,1) doubles, columns packed back to back. Column 0 is the state prior
 * (no emission); every later column is normalised to sum 1. When loglik is not NULL it
 * receives sum over columns i>=1 of log(norm_i). */
int oracle_forward(const oracle_problem *p, double *fw, double *loglik);
/* The same with column 0 given (prior: max(S0,1) values), or the state priors when NULL. */
int oracle_forward_prior(const oracle_problem *p, const double *prior, double *fw,
                         double *loglik);

/* Stochastic traceback (stochastic_traceback, sample_thread.cpp:522-569) with explicit
 * uniforms: u[i] in [0,1] is the draw used for column i (the reference draws
 * rand()/RAND_MAX once per column, last column first). */
int oracle_traceback(const oracle_problem *p, const double *fw, const double *u, int *path);
int oracle_traceback_given(const oracle_problem *p, const double *fw, const double *u,
                           const int *given, int *path);
/* last_state >= 0: the last column's state is given and takes no draw. */
int oracle_traceback_last(const oracle_problem *p, const double *fw, const double *u,
                          const int *given, int last_state, int *path);

/* Backward table, same layout as the forward table, each column normalised to sum 1;
 * the transition into column i+1 is the one the forward pass used (block matrix or
 * switch matrix). Posterior marginals: fw*bw renormalised per column. */
int oracle_backward(const oracle_problem *p, double *bw);
int oracle_posterior(const oracle_problem *p, const double *fw, const double *bw,
                     double *post);

/* Per-block tables for kernel-level checks. For block b: out_terms[b*9*T + a*T + t] is
 * TransMatrix array a (D,E,lnB,lnE2,lnNegG1,G2,G3,lnG4,norecombs) at time t (t<T-1). */
int oracle_block_terms(const oracle_problem *p, double *out_terms, int *out_minage);

/* Emissions of every column, packed like the forward table. */
int oracle_emissions(const oracle_problem *p, double *emit);
// Dense log matrices of tree b: trans [S][S] within it and (b > 0, sw non-NULL) the switch
// [S1][S2] from tree b - 1; NULL skips one.
int oracle_dense_matrices(const oracle_problem *p, int b, double *trans, double *sw);

/* The tables of the GPU table kernel, same layouts (for kernel-level checks): tmatrix
 * [ntrees][T-1][T-1]; same-branch entries get_time(a_y, b_x, c, minage, true) of each node
 * (states x, y of the node, nodes in index order), entry (x, y) at y * m + x,
 * [sum over trees of sum over nodes of m^2];
 * invariant-site emissions [sum over trees of max(S,1)]; column-0 prior [max(S0,1)]. */
int oracle_debug_tables(const oracle_problem *p, double *tm, double *gts, double *inv,
                        double *prior);

/* The dense HMM over a full log transition matrix trans[S][S] (hmm.cpp:27-85), tables
 * row-major n x S: fill fw[1..n-1] from fw[0]; bw[0..n-2] from bw[n-1]; path[0..n-2] from
 * path[n-1] with u[i] the uniform of column i. */
int oracle_dense_forward(int n, int S, const double *trans, const double *emit, double *fw);
int oracle_dense_backward(int n, int S, const double *trans, const double *emit, double *bw);
int oracle_dense_sample(int n, int S, const double *trans, const double *fw, const double *u,
                        int *path);

/* Probabilities of the problem's ARG (total_prob.cpp): out[0] log-likelihood of the
 * sequences (one per leaf, columns = the trees' sites), out[1] the ARG prior, out[2] the
 * first tree's coalescent prior. */
int oracle_arg_prob(const oracle_problem *p, double *out);

/* sample_recombinations (recomb.cpp:151-235) along a state path: u holds the draws in
 * order; the count of recombinations (columns, nodes, times in pos/node/time, cap entries)
 * and the draws used; negative on a bad path (-1), too few draws (-2), a full output (-3). */
int oracle_sample_recombinations(const oracle_problem *p, const int *path, const double *u,
                                 int nu, int *pos, int *node, int *time, int cap, int *used);

/* Total cells: sum over columns of max(nstates,1). */
long long oracle_cells(const oracle_problem *p);

#ifdef __cplusplus
}
#endif
#endif
