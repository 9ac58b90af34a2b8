/*
 * pairhmm.h -- C ABI of the GB300 (sm_103a) batched 2D pair-HMM
 * forward / backward / E-step library.
 *
 * The library replaces the device side of the reference's 2D pair-HMM
 * dynamic programme (evoldoers/tkf-mixdom, python/tkfmixdom/jax/dp/hmm.py)
 * for batches of sequence pairs.  Every entry point is stream-ordered, takes
 * plain pointers and sizes, and returns 0 on success or a negative PHMM_E_*
 * code (message via phmm_last_error).
 *
 * Conventions shared with the reference:
 *   - state types: 0 = S (start), 1 = M, 2 = I, 3 = D, 4 = E
 *     (core/params.py:21); state index 0 is the start state
 *     (dp/hmm.py:1212, 1236) and the End column is the first E-typed state
 *     (dp/hmm.py:17-23);
 *   - residues are 0..19 plus the wildcard 20 whose emission factor is 1
 *     (dp/hmm.py:646-648);
 *   - transitions are given in linear probability space (the exponential of
 *     the reference's log_trans; NEG_INF entries become 0);
 *   - per-emission-group tables: M[g][a][b] = P(emit x=a, y=b), I[g][b],
 *     D[g][a] (linear, 21 x 21 / 21 entries including the wildcard row and
 *     column), one group per MixDom (domain, fragment) location, one group
 *     for TKF91/TKF92 (dp/hmm.py:628-851 build these as log tables).
 */
#ifndef PAIRHMM_H_
#define PAIRHMM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHMM_OK 0
#define PHMM_E_ARG -1      /* bad argument / unsupported model shape */
#define PHMM_E_CUDA -2     /* CUDA runtime error (allocation, launch) */
#define PHMM_E_KERNEL -3   /* a kernel reported a failure in status[] */

/* per-pair status bits written by the kernels */
#define PHMM_ST_TIMEOUT 1      /* a bounded inter-CTA wait gave up */
#define PHMM_ST_ZERO_LL 2      /* likelihood underflowed to 0 or is not finite */
#define PHMM_ST_BAD_RESIDUE 4  /* residue > 20 (clamped to the wildcard) */
#define PHMM_ST_SCALE_CLAMP 8  /* a posterior scale exponent was clamped */

/* Model description: the state space of one pair HMM.  Replaces the
 * (log_trans.shape, state_types) pair of dp/hmm.py:1775/1834 plus the
 * state -> emission-group map of dp/hmm.py:719-729 (MixDom2) /
 * dp/hmm.py:820-823 (MixDom1). */
typedef struct phmm_model_desc {
    int32_t n_states;            /* N */
    const int8_t *state_types;   /* host [N] */
    const int32_t *state_group;  /* host [N]; group of each M/I/D state, ignored otherwise */
    int32_t n_groups;            /* G */
} phmm_model_desc;

/* A batch of pairs.  Device pointers unless noted.  Replaces the bucketed
 * (xs_pad, ys_pad, Lx_real, Ly_real, log_chis, sub stacks) arguments of the
 * reference's jit(vmap(forward_backward_2d)) callers
 * (train/tkf92_svi_bw.py:263-334, train_pfam.py:1674-1741); no padding is
 * needed: every pair runs at its real lengths. */
typedef struct phmm_batch {
    int32_t n_pairs;
    const int32_t *Lx_host;      /* host [P] ancestor lengths */
    const int32_t *Ly_host;      /* host [P] descendant lengths */
    const uint8_t *residues;     /* device: concatenated residues */
    const int64_t *x_off_host;   /* host [P] offset of x_p in residues */
    const int64_t *y_off_host;   /* host [P] offset of y_p in residues */
    const float *chi;            /* device [P or 1][N][N] transition matrix */
    int32_t chi_per_pair;        /* 1: one matrix per pair, 0: shared */
    const float *emit_M;         /* device [P or 1][G][21][21] */
    const float *emit_I;         /* device [P or 1][G][21] */
    const float *emit_D;         /* device [P or 1][G][21] */
    int32_t emit_per_pair;       /* 1: tables per pair, 0: shared */
    /* device, may be NULL: one byte per lattice cell, pairs concatenated in
     * batch order, each pair row-major (Lx+1) x (Ly+1); bit 0 lets the
     * M-type states emit at the cell, bit 1 the I-type, bit 2 the D-type
     * (a cleared bit is the reference's NEG_INF emission), and a zero byte
     * at (0, 0) removes the start.  Expresses mask_emissions_match_aligned
     * (dp/hmm.py:1085-1117: bit 0 only at the alignment's match cells) and
     * the banded recursions (dp/hmm.py:2104-2492: zero bytes off the band).
     * Honoured by the generic and two-warp kernels (variants 0, 1, 7; the
     * automatic choice takes these for a masked batch), by
     * phmm_estep_tables, and by phmm_viterbi as an envelope (nonzero =
     * inside). */
    const uint8_t *cell_mask;
    /* > 0: beam pruning of the forward recursion (dp/hmm_beam.py:85-203):
     * at every cell the states below the cell's maximum times
     * exp(-beam_log_width) are set to zero, and the backward recursion then
     * runs on the cells the pruned forward left active (hmm_beam.py:206-318;
     * posteriors capped at 1).  0 = off.  Honoured by the generic kernels
     * (variants 0 and 1; the automatic choice takes them for a pruned batch)
     * and by phmm_estep_tables. */
    double beam_log_width;
    /* device, may be NULL: the MixDom transitions of chi in factored form
     * (build_nested_trans, models/mixdom.py:343-394), one record per pair
     * (or one shared, as chi), 20*K*F + 25*K*F*F floats, body state
     * q = 0..5KF-1 being state 2 + q:
     *   exit[q]; cin[a][q] for the top-level types a = M, I, D
     *   (= dest[q] * T_exit_k[d_q][a][U(q)]); intra[d][5F][5F], the
     *   same-domain block without its inter-domain part,
     * so that chi[2+s][2+k] = exit[s] cin[U(s)][k] + [same domain] intra.
     * The dense chi is still required (start row, end column, counts).
     * With it the two-warp stripes of a compiled layout (K = 3, F = 1)
     * contract each cell in about 6N + 11KF^2 multiply-adds instead of N^2,
     * and the wide kernels at F = 4 (K = 4..8; not with checkpointing or the
     * tensor-core forward) in about 3N + 11KF^2 per pass; other layouts,
     * masked and pruned batches use the dense chi.
     * phmm_mixdom2_nest builds it.  nest_dom = K, nest_frag = F. */
    const float *nest;
    int32_t nest_dom, nest_frag;
} phmm_batch;

typedef struct phmm_plan phmm_plan;

/* Create a plan for one state space.  Scratch memory is allocated lazily
 * by the first batch that needs it and reused afterwards. */
int phmm_plan_create(const phmm_model_desc *model, phmm_plan **out);
void phmm_plan_destroy(phmm_plan *plan);

/* Forward pass only: ll_out[p] = log P(x_p, y_p) (float64).
 * Replaces forward_2d (dp/hmm.py:1775-1801) and
 * forward_backward_2d(..., forward_only=True) (dp/hmm.py:1834-1914);
 * stream is a cudaStream_t. */
int phmm_forward(phmm_plan *plan, const phmm_batch *batch,
                 double *ll_out, int32_t *status_out, void *stream);

/* Full E-step: log-likelihood, expected transition counts and the
 * per-group character-indexed expected emission counts.
 *   ll_out    [P]           float64
 *   n_trans   [P][N][N]     float64, reference state order
 *                           (forward_backward_2d's expected_trans,
 *                           dp/hmm.py:1940-1971)
 *   cnt_M     [P][G][21][21] sum of M-type posteriors by (x_i, y_j)
 *   cnt_I     [P][G][21]     sum of I-type posteriors by y_j
 *   cnt_D     [P][G][21]     sum of D-type posteriors by x_i
 * The per-class counts of train/likelihood.py:279-344 and the VJP counts of
 * train/vjp.py:513-625 follow from cnt_* in a small float64 epilogue.
 * Replaces forward_backward_2d (dp/hmm.py:1834-1973) as called by
 * e_step / e_step_mixdom2 (train/likelihood.py:49-373). */
int phmm_estep(phmm_plan *plan, const phmm_batch *batch,
               double *ll_out, double *n_trans, double *cnt_M, double *cnt_I,
               double *cnt_D, int32_t *status_out, void *stream);

/* E-step that also writes full lattice tables (optional, nullable):
 *   log_F, log_B [sum_p (Lx+1)(Ly+1)][N] float64 log forward / backward
 *   post         [sum_p (Lx+1)(Ly+1)][N] float64 posteriors
 * pair p's block starts at cell offset sum_{q<p} (Lx_q+1)(Ly_q+1), row-major
 * (i, j).  For API parity with forward_2d / backward_2d /
 * forward_backward_2d (dp/hmm.py:1775-1973); not a fast path. */
int phmm_estep_tables(phmm_plan *plan, const phmm_batch *batch,
                      double *ll_out, double *n_trans, double *cnt_M,
                      double *cnt_I, double *cnt_D, int32_t *status_out,
                      double *log_F, double *log_B, double *post, void *stream);

/* E-step of a banded batch with the posteriors in band layout.  Replaces
 * forward_backward_2d_banded (dp/hmm.py:2395-2491), which returns the
 * log-likelihood, the band posteriors and the expected transitions of one
 * pair; here for a batch.  batch->cell_mask must hold the band (nonzero
 * where |j - band_center[i]| <= band_half_width); the E-step runs on the
 * two-warp kernels, whose stripes skip the anti-diagonal steps outside their
 * rows' band, so the work is O(L * W) per pair.
 *   band_center     device int32, Lx+1 entries per pair, pairs concatenated
 *   band_half_width W of the output layout (2W + 1 columns per row)
 *   post_band       device float64 [sum over pairs of (Lx+1)][2W+1][N]:
 *                   position (i, b) holds F B / P at column
 *                   band_center[i] - W + b (0 off the lattice or off the band;
 *                   the start state's posterior at the origin is 1)
 * and ll_out, n_trans, cnt_*, status_out as phmm_estep.  Fails with
 * PHMM_E_ARG when the state space has no two-warp kernels (use
 * phmm_estep_tables on the generic kernels then), without a cell mask, or on
 * a plan forced to another kernel family. */
int phmm_estep_band(phmm_plan *plan, const phmm_batch *batch,
                    const int32_t *band_center, int32_t band_half_width,
                    double *ll_out, double *n_trans, double *cnt_M,
                    double *cnt_I, double *cnt_D, int32_t *status_out,
                    double *post_band, void *stream);

/* Caller-owned workspace.  phmm_workspace_bytes stores in *bytes the device
 * scratch one phmm_forward_ws (estep 0) or phmm_estep_ws (estep 1) call on
 * this batch needs; only the batch's host fields (n_pairs, Lx_host, Ly_host,
 * x_off_host, y_off_host) are read.  The _ws calls then run exactly as
 * phmm_forward / phmm_estep, with all scratch carved from `workspace`
 * (256-byte aligned, at least that many bytes) instead of plan-owned
 * buffers, and allocate no device memory (the split E-step creates its side
 * streams and events once per caller stream).  Calls on one plan with distinct workspaces
 * may be in flight on different streams at the same time (issue them from
 * one host thread).  No counterpart in the reference, whose XLA runtime owns
 * the scratch; this is what a serving loop budgets HBM with when it admits
 * requests. */
int phmm_workspace_bytes(phmm_plan *plan, const phmm_batch *batch, int estep,
                         size_t *bytes);
int phmm_forward_ws(phmm_plan *plan, const phmm_batch *batch, void *workspace,
                    size_t workspace_bytes, double *ll_out, int32_t *status_out,
                    void *stream);
int phmm_estep_ws(phmm_plan *plan, const phmm_batch *batch, void *workspace,
                  size_t workspace_bytes, double *ll_out, double *n_trans,
                  double *cnt_M, double *cnt_I, double *cnt_D,
                  int32_t *status_out, void *stream);

/* phmm_estep_ws in two halves, for a caller that captures the E-step in a
 * CUDA graph: phmm_estep_ws_prepare copies the batch's work description
 * (pair metadata and work lists, built on the host from the lengths) into
 * the workspace, stream-ordered; phmm_estep_ws_launch then issues only the
 * device work of phmm_estep_ws (clearing counters and outputs, the kernels)
 * and copies nothing from the host, so it can be captured and replayed
 * while the workspace keeps that description -- the same batch lengths,
 * plan and workspace on every launch (the residues, tables and outputs may
 * change between launches).  No counterpart in the reference, whose
 * per-shape jit cache (train_pfam.py:1674-1741) plays this role. */
int phmm_estep_ws_prepare(phmm_plan *plan, const phmm_batch *batch, void *workspace, size_t workspace_bytes,
                          void *stream);
int phmm_estep_ws_launch(phmm_plan *plan, const phmm_batch *batch, void *workspace, size_t workspace_bytes,
                         double *ll_out, double *n_trans, double *cnt_M, double *cnt_I, double *cnt_D,
                         int32_t *status_out, void *stream);

/* E-step that allocates nothing: no cudaMalloc, cudaFree or other allocating
 * call.  No counterpart in the reference.
 *
 * Who needs it: a caller whose process already owns the GPU's memory.  The
 * reference's own training code runs under JAX, whose runtime by default
 * reserves most of the device memory for its own pool when it starts, and
 * serving processes often run under a framework allocator with a fixed
 * budget; a cudaMalloc issued behind such an allocator's back can fail or
 * fragment its pool, so these callers cannot rely on phmm_plan_create /
 * phmm_estep growing scratch on demand.
 *
 * How: the kernels of phmm_estep run with all their scratch (work list,
 * progress counters, edge rows, forward lattice) in one file-scope
 * __device__ array of PHMM_STATIC_SCRATCH_BYTES, which every GPU that loads
 * this library holds until the process exits.  The caller still provides the
 * inputs and outputs (same meaning as phmm_estep; the model is passed
 * directly, no plan).  The first call on a device looks the array's device
 * address up (cudaGetSymbolAddress, with that device current); make that
 * first call before any stream capture.  A batch whose scratch would exceed
 * the array is rejected with PHMM_E_ARG and a message giving the bytes it
 * needs.  Capacity at 17 states: the lattice is kept in 64-row stripes of
 * (64 + Ly) x 64 cells at 68 bytes a cell (16 floats and an exponent), so
 * the array holds about 490 k stripe cells -- e.g. 11 pairs of 150 x 150
 * (3 stripes each), or one pair of about 1000 x 1000.  Every call shares the
 * array and the static host staging it uses, and the array keeps the last
 * call's contents: each call clears the counters it needs, but calls that
 * overlap -- on the GPU, on different streams, or from different host
 * threads -- race and must be serialised by the caller.  The device address
 * is cached per device ordinal for the life of the process: after
 * cudaDeviceReset (or any other re-creation of the device's primary
 * context) the cached address belongs to the old context, and calls on that
 * device are not supported. */
#define PHMM_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)
int phmm_estep_static(const phmm_model_desc *model, const phmm_batch *batch,
                      double *ll_out, double *n_trans, double *cnt_M, double *cnt_I,
                      double *cnt_D, int32_t *status_out, void *stream);

/* MixDom2 parameters (host float64 arrays), the parameter pytree of the
 * reference's MixDom2 model (models/mixdom.py:52-77, train/likelihood.py:143-190):
 * main_ins / main_del, dom_ins / dom_del / dom_weights [K], frag_weights
 * [K][F], ext_rates [K][F][F] (fragment f to g extension; a [K][F] vector
 * is its diagonal), class_pis [C][A], class_S_exch [C][A][A] (symmetric
 * exchangeabilities), classdist [K][F][C]. */
typedef struct phmm_mixdom2_params {
    int32_t n_dom, n_frag, n_classes, alphabet;   /* K, F, C, A (A = 20) */
    double main_ins, main_del;
    const double *dom_ins, *dom_del, *dom_weights;
    const double *frag_weights;
    const double *ext_rates;
    const double *class_pis;
    const double *class_S_exch;
    const double *classdist;
} phmm_mixdom2_params;

/* Device prologue of the MixDom2 E-step: from the parameters and per-pair
 * times t (device [P] float64) write each pair's collapsed transition matrix
 * chi (device float32 [P][N][N], N = 2 + 5KF), its emission tables
 * (emit_M float32 [P][KF][21][21], emit_I / emit_D [P][KF][21], the layout
 * phmm_batch takes with chi_per_pair = emit_per_pair = 1) and the class
 * substitution matrices P_c(t) = expm(t Q_c) (device float64 [P][C][A][A],
 * phmm_mixdom2_class_subs_count doubles).  Replaces the per-pair builders
 * the reference runs inside its E-step (models/mixdom.py:104-423 via
 * train/likelihood.py:143-190; core/ctmc.py:31-60; dp/hmm.py:673-783).
 * Requires K*F <= 33; stream-ordered; allocates nothing. */
size_t phmm_mixdom2_class_subs_count(const phmm_mixdom2_params *prm, int32_t n_pairs);
int phmm_mixdom2_tables(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t,
                        float *chi, float *emit_M, float *emit_I, float *emit_D,
                        double *class_subs, void *stream);

/* The same prologue with the parameters in device memory, for a captured
 * CUDA graph (a by-value parameter block would be frozen in the graph):
 * phmm_mixdom2_param_block fills a host block of
 * phmm_mixdom2_param_block_bytes() bytes from the parameters (the same
 * checks as phmm_mixdom2_tables); the caller copies it to a device block
 * (stream-ordered, e.g. from pinned memory inside the graph) and passes that
 * to phmm_mixdom2_tables_dp / phmm_mixdom2_class_counts_dp with the n_dom,
 * n_frag and n_classes it was filled from.  Outputs as phmm_mixdom2_tables
 * and phmm_mixdom2_class_counts. */
size_t phmm_mixdom2_param_block_bytes(void);
int phmm_mixdom2_param_block(const phmm_mixdom2_params *prm, void *host_block, size_t bytes);
int phmm_mixdom2_tables_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                           int32_t n_pairs, const double *t, float *chi, float *emit_M, float *emit_I,
                           float *emit_D, double *class_subs, void *stream);
int phmm_mixdom2_class_counts_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                                 int32_t n_pairs, const double *class_subs, const double *cnt_M,
                                 const double *cnt_I, const double *cnt_D, double *class_match,
                                 double *class_insert, double *class_delete, double *classdist_counts,
                                 void *stream);

/* The factored form of the collapsed chi (phmm_batch.nest), float32
 * [P][20KF + 25KF^2] on the device, for per-pair times t [P] (device float64):
 * the exit factors, entry-weighted top-level transitions and same-domain
 * blocks that build_nested_trans (models/mixdom.py:252-423) assembles chi
 * from.  The _dp form reads the parameter block of phmm_mixdom2_param_block
 * from device memory (capturable, as phmm_mixdom2_tables_dp). */
int phmm_mixdom2_nest(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *nest, void *stream);
int phmm_mixdom2_nest_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                         int32_t n_pairs, const double *t, float *nest, void *stream);
/* phmm_mixdom2_tables / _dp that also write the factored record (one build
 * of chi serves both). */
int phmm_mixdom2_tables_nest(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *chi,
                             float *emit_M, float *emit_I, float *emit_D, double *class_subs, float *nest,
                             void *stream);
int phmm_mixdom2_tables_nest_dp(const void *param_block, int32_t n_dom, int32_t n_frag, int32_t n_classes,
                                int32_t n_pairs, const double *t, float *chi, float *emit_M, float *emit_I,
                                float *emit_D, double *class_subs, float *nest, void *stream);
/* 1 when the E-step kernels have a factored instantiation for the MixDom
 * layout (n_dom, n_frag): the 17-state two-warp stripes (3, 1) and the wide
 * kernels at n_frag = 4, n_dom = 4..8 (otherwise a batch's nest record is
 * ignored). */
int phmm_nest_supported(int32_t n_dom, int32_t n_frag);

/* The collapsed chi alone (float32 and, when chi64 is not null, float64
 * [P][N][N]) for the gradient path, and its vector-Jacobian product:
 * grad[p][d] = sum_{s,k} grad_chi[p][s][k] dchi_p[s][k]/dtheta_d (device
 * float64), one forward-mode pass per (pair, direction), for the directions
 * 0 main_ins, 1 main_del, 2 the pair's t, 3 + j the j-th entry of
 * (dom_ins, dom_del, dom_weights, frag_weights, ext_rates [K][F][F]) --
 * phmm_mixdom2_chi_vjp_dirs of them.  With grad_chi = n_trans / chi (the
 * score identity) this is the chi part of the gradient of the reference's
 * mixdom2_log_prob custom VJP (train/vjp.py:627-680). */
int phmm_mixdom2_chi(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t, float *chi,
                     double *chi64, void *stream);
int phmm_mixdom2_chi_vjp_dirs(const phmm_mixdom2_params *prm);
int phmm_mixdom2_chi_vjp(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *t,
                         const double *grad_chi, double *grad, void *stream);

/* 1D alignment-conditioned forward-backward (dp/hmm.py:127-250, 471-607):
 * along a fixed alignment the pair HMM is an HMM over the alignment columns.
 * Per pair p: columns off_host[p] .. off_host[p] + L_host[p] - 1 of emit
 * (device float32 [columns][N], linear; 0 where the reference's log
 * emission is NEG_INF); chi [P or 1][N][N] linear.  Outputs: ll_out [P]
 * float64 (log P; logchi[init][final] for L = 0), n_trans [P][N][N] float64
 * (initial, interior and terminal transition posteriors), posteriors
 * (nullable, float32 [columns][N]), status [P].  N <= 64.  Scratch comes from
 * the caller's workspace (phmm_fb1d_workspace_bytes, 256-byte aligned). */
typedef struct phmm_fb1d_batch {
    int32_t n_pairs, n_states;
    const int32_t *L_host;
    const int64_t *off_host;
    const float *emit;
    const float *chi;
    int32_t chi_per_pair;
    int32_t init_state, final_state;
} phmm_fb1d_batch;
int phmm_fb1d_workspace_bytes(const phmm_fb1d_batch *batch, size_t *bytes);
int phmm_fb1d(const phmm_fb1d_batch *batch, void *workspace, size_t workspace_bytes, double *ll_out,
              double *n_trans, float *posteriors, int32_t *status_out, void *stream);

/* Per-column emissions of alignments for phmm_fb1d (dp/hmm.py:854-1082):
 * cols / anc / desc are device uint8 per column (column type 1 M, 2 I, 3 D;
 * characters 0..20, 20 the wildcard); a column of type c emits through the
 * states of type c with the per-group tables of phmm_batch (M:
 * emit_M[g][anc][desc], I: emit_I[g][desc], D: emit_D[g][anc]), every other
 * state gets 0.  workspace: at least 16 * n_pairs bytes. */
int phmm_fb1d_emissions(const phmm_model_desc *model, int32_t n_pairs, const int32_t *L_host,
                        const int64_t *off_host, const uint8_t *cols, const uint8_t *anc,
                        const uint8_t *desc, const float *emit_M, const float *emit_I,
                        const float *emit_D, int32_t emit_per_pair, void *workspace,
                        size_t workspace_bytes, float *emit, int32_t *status_out, void *stream);

/* Viterbi path of each pair (dp/hmm.py:1976-2040), float64 log space: the
 * batch's sequences (residues, offsets, lengths; chi_per_pair / emit_per_pair
 * select per-pair or shared tables below), log_chi [P or 1][N][N] (NEG_INF
 * = -1e30 for structural zeros), log emission tables per group log_emit_M
 * [P or 1][G][21][21], log_emit_I / log_emit_D [P or 1][G][21] (index 20 the
 * wildcard, log 1).  Outputs: ll_out [P] (log-probability of the best path),
 * path [sum_p (Lx+Ly+1)][3] int32 (i, j, state) triples from (0, 0, S) to
 * (Lx, Ly, best final state), pair p's block starting at sum_{q<p}
 * (Lx_q+Ly_q+1), path_len [P] (entries used), status [P].  N <= 64.
 * With the batch's cell_mask set, a nonzero byte marks a cell inside the
 * envelope of beam_viterbi_2d (dp/hmm_beam.py:397-490): a state whose cell
 * or predecessor cell lies outside keeps NEG_INF and points to the origin.
 * Scratch from the caller's workspace (phmm_viterbi_workspace_bytes:
 * three diagonals and one backpointer byte per cell and state). */
int phmm_viterbi_workspace_bytes(const phmm_model_desc *model, const phmm_batch *batch, size_t *bytes);
int phmm_viterbi(const phmm_model_desc *model, const phmm_batch *batch, const double *log_chi,
                 const double *log_emit_M, const double *log_emit_I, const double *log_emit_D,
                 void *workspace, size_t workspace_bytes, double *ll_out, int32_t *path,
                 int32_t *path_len, int32_t *status_out, void *stream);

/* Stochastic forward traceback (replaces dp/hmm.py:2043-2101
 * sample_traceback_2d, batched over pairs and samples): the float64 log-space
 * forward table of every pair (inputs as phmm_viterbi), then n_samples paths
 * per pair drawn from the posterior over alignments -- the final state with
 * probability proportional to exp(F[Lx][Ly][s] + logchi[s][E]), each
 * predecessor state proportional to exp(F[pred][s] + logchi[s][k]).
 * Random numbers come from a counter-based stream keyed by (seed, pair,
 * sample, draw): the same seed gives the same paths.  Outputs: ll_out [P]
 * (the forward log-likelihood), paths [sum_p n_samples (Lx+Ly+1)][3] int32
 * (i, j, state) from (0, 0, S) on, sample s of pair p at triple
 * n_samples * sum_{q<p} (Lx_q+Ly_q+1) + s (Lx_p+Ly_p+1), path_len
 * [P][n_samples], status [P].  N <= 64.  Scratch (phmm_sample_workspace_bytes):
 * the forward tables, (Lx+1)(Ly+1)N doubles per pair. */
int phmm_sample_workspace_bytes(const phmm_model_desc *model, const phmm_batch *batch, size_t *bytes);
int phmm_sample_paths(const phmm_model_desc *model, const phmm_batch *batch, const double *log_chi,
                      const double *log_emit_M, const double *log_emit_I, const double *log_emit_D,
                      int32_t n_samples, uint64_t seed, void *workspace, size_t workspace_bytes,
                      double *ll_out, int32_t *paths, int32_t *path_len, int32_t *status_out, void *stream);

/* Precompiled X/A/Y pair records (util/pair_format.py; the shards read by
 * train_pfam.py:984-1029 once decompressed): JSON lines with the ancestor
 * "x" and descendant "y" as letters of ACDEFGHIKLMNPQRSTVWY, the alignment
 * "a" as M/I/D runs ("M5I1M3D2"), the time "t" and the family "fam".  A
 * host-side reader in two passes: phmm_pairs_count gives the sizes,
 * phmm_pairs_decode fills caller arrays -- residues in phmm_batch's layout
 * (pair p: x at x_off[p], y at y_off[p] = x_off[p] + Lx[p]), t [P], and the
 * alignment columns (n_cols / col_off per pair; col_state 1 M, 2 I, 3 D;
 * col_anc / col_desc the column's characters, 20 where it has none), the
 * family as a span of the text (fam_off = -1 without one).  A record that
 * fails validate_record (util/pair_format.py:194-223) is PHMM_E_ARG with the
 * line number in phmm_last_error.  Blank lines are skipped. */
typedef struct phmm_pair_counts {
    int32_t n_pairs;
    int64_t n_residues;   /* sum of |x| + |y| */
    int64_t n_columns;    /* sum of alignment columns */
} phmm_pair_counts;

int phmm_pairs_count(const char *text, size_t len, phmm_pair_counts *out);
int phmm_pairs_decode(const char *text, size_t len, const phmm_pair_counts *sizes, int32_t *Lx, int32_t *Ly,
                      int64_t *x_off, int64_t *y_off, uint8_t *residues, double *t, int32_t *n_cols,
                      int64_t *col_off, int8_t *col_state, uint8_t *col_anc, uint8_t *col_desc,
                      int64_t *fam_off, int32_t *fam_len);

/* TKF91 / TKF92 parameters (host float64): insertion and deletion rates,
 * fragment extension probability (0 for TKF91), the substitution rate
 * matrix Q [A][A] (rows summing to zero) and its equilibrium pi [A]; A = 20. */
typedef struct phmm_tkf92_params {
    double ins_rate, del_rate, ext;
    int32_t alphabet;
    const double *Q;
    const double *pi;
} phmm_tkf92_params;

/* Device prologue of the batched TKF92 E-step / forward: for per-pair times
 * t (device [P] float64) write chi (device float32 [P][5][5], the TKF92
 * matrix floored at 1e-30 as train/tkf92_svi_bw.py:164 takes
 * log(max(tau, 1e-30))), the emission tables (emit_M [P][1][21][21],
 * emit_I / emit_D [P][1][21], dp/hmm.py:628-670) and P(t) = expm(t Q)
 * (device float64 [P][A][A]).  Replaces the per-pair builders of
 * train/tkf92_svi_bw.py:263-365.  Stream-ordered; allocates nothing. */
int phmm_tkf92_tables(const phmm_tkf92_params *prm, int32_t n_pairs, const double *t, float *chi,
                      float *emit_M, float *emit_I, float *emit_D, double *sub, void *stream);

/* Device epilogue of the MixDom2 E-step: the per-class sufficient statistics
 * of train/likelihood.py:279-344 from phmm_estep's per-group character
 * counts (cnt_M [P][KF][21][21], cnt_I / cnt_D [P][KF][21]) and the
 * class_subs phmm_mixdom2_tables wrote.  Outputs (device float64):
 * class_match [P][C][20][20], class_insert / class_delete [P][C][20],
 * classdist_counts [P][K][F][C].  The class posterior of a cell depends on
 * it only through its characters, so no lattice-sized joint is formed;
 * character 20 (wildcard) reads the class factors of character 19 (the
 * reference's clamped gather) and is left out of the character-indexed
 * outputs.  At most 8 classes. */
int phmm_mixdom2_class_counts(const phmm_mixdom2_params *prm, int32_t n_pairs, const double *class_subs,
                              const double *cnt_M, const double *cnt_I, const double *cnt_D,
                              double *class_match, double *class_insert, double *class_delete,
                              double *classdist_counts, void *stream);

/* Holmes-Rubin substitution statistics of every (pair, class), float64 on
 * the device (replaces core/ctmc.py:285-326 holmes_rubin_weighted_stats and
 * its integrals core/ctmc.py:173-230, called once per class per pair by
 * train/likelihood.py:279-344):
 *   W[p,c,i]   = sum_ab n[p,c,a,b] I_c[a,b,i,i](t_p) / P_c,ab(t_p)
 *   U[p,c,i,j] = Q_c[i,j] sum_ab n[p,c,a,b] I_c[a,b,i,j](t_p) / P_c,ab(t_p),
 *                zero diagonal,
 * contracted through the eigendecomposition of the symmetrised rate matrix
 * (no A^4 integral tensor).  class_Q [C,A,A] and class_pis [C,A] are HOST
 * arrays (Q reversible with respect to pi, pi > 0); t [P],
 * class_match_counts [P,C,A,A], W [P,C,A] and U [P,C,A,A] are device
 * arrays.  A <= 32.  Enqueued on the stream; PHMM_E_ARG on bad arguments. */
int phmm_holmes_rubin(int32_t n_classes, int32_t alphabet, const double *class_Q, const double *class_pis,
                      int32_t n_pairs, const double *t, const double *class_match_counts, double *W, double *U,
                      void *stream);

/* phmm_holmes_rubin with its per-class blocks (the host eigendecomposition
 * of each class rate matrix) in device memory, for a captured CUDA graph:
 * phmm_holmes_rubin_block fills phmm_holmes_rubin_block_bytes(n_classes)
 * host bytes; the caller copies them to the device block passed to
 * phmm_holmes_rubin_dp.  Results as phmm_holmes_rubin. */
size_t phmm_holmes_rubin_block_bytes(int32_t n_classes);
int phmm_holmes_rubin_block(int32_t n_classes, int32_t alphabet, const double *class_Q, const double *class_pis,
                            void *host_block, size_t bytes);
int phmm_holmes_rubin_dp(const void *block, int32_t n_classes, int32_t n_pairs, const double *t,
                         const double *class_match_counts, double *W, double *U, void *stream);

/* Per-kernel CUDA-event timing on the launching stream (diagnostics and
 * benchmarking; no counterpart in the reference, which has no kernels).
 * phmm_kernel_times waits for the last call's events and returns the forward
 * and backward kernel durations in milliseconds (backward 0 after
 * phmm_forward). */
int phmm_set_timing(phmm_plan *plan, int enable);
int phmm_kernel_times(phmm_plan *plan, float *fwd_ms, float *bwd_ms);
/* Device time of one kernel of the last timed call: which = 0 forward,
 * 1 backward (fused backward + counts, or the backward recursion of the
 * split E-step), 2 the split E-step's count pass (0 when it did not run).
 * A call that ran in groups (a batch larger than free memory) reports each
 * kernel's time summed over its groups. */
int phmm_kernel_time(phmm_plan *plan, int which, float *ms);

/* Kernel family: 0 = automatic (default), 1 = generic kernels (any state
 * space of up to 60 emitting states), 2 = register-resident warp kernels,
 * 3 = quad-per-warp block kernels, 4 = split E-step on the warp kernels
 * (forward and backward recursion at the same time on two streams, then a
 * count pass over both lattices), 5 = split E-step on the block kernels
 * (2 to 5 for state spaces with a compiled shape), 6 = the wide kernels
 * (any state space of up to 164 emitting states; the automatic choice above
 * 60 emitting states), 7 = split E-step on two-warp stripes (one lattice row
 * per thread, 64-thread CTAs; the shapes of 2 and 4).  phmm_last_variant
 * reports the family the last call used.  No
 * counterpart in the reference (it has no kernels). */
int phmm_set_variant(phmm_plan *plan, int variant);
int phmm_last_variant(const phmm_plan *plan);

/* Bound of every inter-CTA wait of this plan's kernels, in polling
 * iterations (each a poll and a 128 ns sleep); 0 restores the default of
 * 40 M (about 5 s).  A wait that reaches the bound sets PHMM_ST_TIMEOUT on
 * its pair, releases the stripes waiting on it and returns, so the launch
 * always completes; after the call such a pair's log-likelihood is NEG_INF
 * (-1e30) and its counts are undefined.  Diagnostic (a test shortens the
 * bound to exercise that path); no counterpart in the reference. */
int phmm_set_spin_limit(phmm_plan *plan, long long iterations);

/* Launch configuration of a plan (what the project's autotuner searches,
 * pairhmm/autotune.py; no counterpart in the reference, whose XLA compiler
 * chooses its own):
 *   variant       kernel family as phmm_set_variant (0 automatic);
 *   wave_per_sm   resident CTAs per SM of each persistent wavefront grid
 *                 (0: half the slots each for the split E-step's two
 *                 wavefronts, all of them for the wide family);
 *   count_per_sm  CTAs per SM of the split E-step's count grid that runs
 *                 beside the wavefronts (-1: half the slots; 0: none, every
 *                 count item then runs once both wavefronts are done);
 *   priorities    1: the wavefronts run on streams of the greatest priority
 *                 and the count grids on streams of the least, so SM slots
 *                 freed while both wait go to the critical path first.
 *   checkpoint    E-step on the wide kernels (more than 60 emitting
 *                 states): 1 keeps no lattice -- the wavefronts keep only
 *                 the edge rows every 32 rows (the checkpoints, about
 *                 sqrt(L) of them for L x L), and the count pass recomputes
 *                 each stripe from the edge rows above and below it, in
 *                 groups of two stripes per SM; scratch is the edge rows plus
 *                 one group instead of two whole lattices, for about a third
 *                 more arithmetic.  2 never does this (a batch larger than
 *                 the free memory runs as consecutive groups of pairs);
 *                 0 (automatic) does it when one pair's lattices alone
 *                 exceed 40 % of the device's memory.  The reference keeps
 *                 its 2D tables within memory by recomputation too
 *                 (jax.checkpoint on its log-likelihood VJPs,
 *                 train/vjp.py:109-124).
 *   tensor        wide kernels, phmm_forward only: 1 runs the forward
 *                 recursion's per-step contraction ([32 rows x NS sources] x
 *                 [NS x 4NQ destinations]) on the tensor cores as 3xTF32
 *                 (each float split into a TF32 high part and a TF32
 *                 remainder; hi*hi + hi*lo + lo*hi accumulated in float32 by
 *                 mma.sync m16n8k8), where the state space allows it
 *                 (destination quads a multiple of 4, each warp's 16
 *                 destinations of one type).  Measured at 162 states: the
 *                 forward 15 % faster, log-likelihoods within 4e-7 relative
 *                 of the float64 oracle (1e-10 with the default float32
 *                 contraction and its compensated sums).  E-steps always run
 *                 the float32 contraction: with a 3xTF32 forward against a
 *                 float32 backward the counts were 1e-3 off.  0 (default):
 *                 float32 everywhere.
 * Results do not depend on the tuning (the same kernels and arithmetic on
 * the same work items; the count sums' order may differ), except for
 * `tensor`.  Defaults {0, 0, -1, 0, 0, 0}. */
typedef struct phmm_tuning {
    int32_t variant;
    int32_t wave_per_sm;
    int32_t count_per_sm;
    int32_t priorities;
    int32_t checkpoint;
    int32_t tensor;
} phmm_tuning;
int phmm_set_tuning(phmm_plan *plan, const phmm_tuning *tuning);
int phmm_get_tuning(const phmm_plan *plan, phmm_tuning *tuning);

/* Number of kernel launches issued by the last call on this plan. */
int phmm_last_launch_count(const phmm_plan *plan);

/* Last error message (thread-local); returns its length. */
int phmm_last_error(char *buf, size_t len);

/* ABI version of this library. */
int phmm_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PAIRHMM_H_ */
