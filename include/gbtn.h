/*
 * gbtn.h -- C ABI of the GB300 belief-propagation library (libgbtn.so).
 *
 * Drop-in boundary for the belief-propagation hot path of ITensorNetworks.jl.
 * A Julia package extension (or the Python host package shipped beside this
 * library) binds these entry points with ccall / ctypes.  Plain C types only:
 * pointers, sizes and status codes; no exceptions cross the boundary and no
 * call aborts the process.
 *
 * Data conventions (identical on host and device):
 *   - vertices 0..nv-1; undirected edges 0..ne-1 with endpoints (edge_u[e],
 *     edge_v[e]); directed edge 2e is edge_u -> edge_v, 2e+1 the reverse.
 *   - the tensor of vertex v has shape (d_v, chi_{leg_edge[leg_ptr[v]]}, ...)
 *     in column-major order (site index fastest), i.e. NDTensors Dense order
 *     with the site index first and the links in the vertex's leg order.
 *     All vertex tensors are concatenated in vertex order.
 *   - the message of a directed edge u -> v is a chi x chi matrix M[b, a]
 *     (b = bra/primed link, a = ket link), column-major, concatenated in
 *     directed-edge order (2e, 2e+1, ...).
 *   - every entry point that takes or returns numbers uses float64 on the
 *     host side; reduced precisions exist only inside the library.
 *
 * Return value of every int function: GBTN_OK (0) or an error code; the
 * message is available from gbtn_last_error(ctx).
 */
#ifndef GBTN_H
#define GBTN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBTN_ABI_VERSION 2

enum gbtn_status {
  GBTN_OK = 0,
  GBTN_ERR_INVALID = 1,     /* bad argument (maps to the reference's error()) */
  GBTN_ERR_CUDA = 2,        /* CUDA runtime error */
  GBTN_ERR_UNSUPPORTED = 3, /* shape outside the compiled kernel limits */
  GBTN_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  GBTN_ERR_NUMERIC = 5,     /* non-finite value where one is not allowed */
  GBTN_ERR_NOMEM = 6
};

enum gbtn_mem { GBTN_HOST = 0, GBTN_DEVICE = 1 };

/* Message-update schedules.
 *   SEQUENTIAL: directed edges in the order given by edge_sequence, each
 *               update seeing every earlier one (update_iteration,
 *               abstractbeliefpropagationcache.jl:272-287).
 *   PARALLEL:   every message of a sweep computed from the previous sweep
 *               (update_iteration over edge groups, :294-308).
 *   COLORED:    vertices in colour classes; all out-messages of one class
 *               computed from the current messages, class after class. */
enum gbtn_schedule { GBTN_SCHED_SEQUENTIAL = 0, GBTN_SCHED_PARALLEL = 1, GBTN_SCHED_COLORED = 2 };

/* Arithmetic of the message contractions.  MIXED runs BF16 tensor-core
 * sweeps (FP32 accumulation), then FP32 sweeps, then refinement sweeps (DF32
 * by default, or FP64: gbtn_bp_opts.refine), each phase started from the
 * previous phase's fixed point.  DF32 is double-FP32 arithmetic (a value is
 * the unevaluated sum of two floats, ~48 significant bits, on the FP32 pipe)
 * on FP64 tensors and messages, with message norms and diffs in FP64.  BF16
 * runs the PARALLEL and COLORED schedules (SEQUENTIAL returns
 * GBTN_ERR_UNSUPPORTED: the tensor-core kernel computes every message of a
 * vertex at once); MIXED with SEQUENTIAL runs its FP32 and refinement phases
 * in waves, without the BF16 phase.  FP32 and FP64 run all three schedules
 * on any plan, DF32 and MIXED SEQUENTIAL on plans without vertices of the
 * global-memory path.  Complex plans have no BF16 or DF32 path: their MIXED
 * pipeline is FP32 then FP64. */
enum gbtn_precision { GBTN_F64 = 0, GBTN_F32 = 1, GBTN_BF16 = 2, GBTN_MIXED = 3, GBTN_DF32 = 4 };
/* Refinement arithmetic of MIXED after its FP32 phase. */
enum gbtn_refine { GBTN_REFINE_DF32 = 0, GBTN_REFINE_F64 = 1 };

enum gbtn_message_init { GBTN_INIT_IDENTITY = 0, GBTN_INIT_ONES = 1 };

typedef struct gbtn_ctx gbtn_ctx;
typedef struct gbtn_plan gbtn_plan;

/* Network structure of one or many independent networks (a disjoint union;
 * vertex_network[v] names the network of v, NULL means one network). */
typedef struct gbtn_graph_desc {
  int32_t nv;
  int32_t ne;
  const int32_t* edge_u;         /* [ne] */
  const int32_t* edge_v;         /* [ne] */
  const int32_t* edge_dim;       /* [ne] bond dimension chi_e >= 1 */
  const int32_t* site_dim;       /* [nv] physical dimension d_v >= 1 */
  const int32_t* leg_ptr;        /* [nv+1] CSR offsets into leg_edge */
  const int32_t* leg_edge;       /* [leg_ptr[nv]] edges of v in tensor leg order */
  const int32_t* vertex_network; /* [nv] or NULL */
  int32_t n_networks;            /* >= 1 (ignored when vertex_network is NULL) */
  int32_t separate_bra;          /* 0: bra = conj(ket) (QuadraticFormNetwork);
                                    1: bra tensors are set separately
                                    (LinearFormNetwork / inner(phi, psi)) */
  int32_t complex_values;        /* 0: real tensors; 1: complex: every
                                    tensor, message, RDM and scalar array
                                    holds interleaved (re, im) doubles, twice
                                    the element count.  Complex plans run
                                    sweeps in FP64 (ComplexF64), FP32
                                    (ComplexF32 arithmetic) or MIXED (FP32
                                    sweeps, then FP64 ones), any schedule;
                                    environments, updated_message, one- and
                                    two-site RDMs,
                                    expect / expect2 (real part of <O>, O
                                    real), vertex and edge scalars,
                                    logscalar, rescale_messages and
                                    rescale_partitions, and the energy and
                                    gradient entry points (the real part of
                                    the loss; gradients dL/dRe + i dL/dIm).
                                    BF16 sweeps return GBTN_ERR_UNSUPPORTED.
                                    (test/test_belief_propagation.jl:18-20) */
} gbtn_graph_desc;

typedef struct gbtn_bp_opts {
  int32_t schedule;              /* gbtn_schedule */
  int32_t precision;             /* gbtn_precision */
  int32_t maxiter;               /* > 0 (the reference errors when absent) */
  int32_t normalize;             /* 1: divide each new message by its norm */
  double tol;                    /* < 0: no convergence test (tol = nothing) */
  const int32_t* edge_sequence;  /* SEQUENTIAL: directed edges, per sweep */
  int32_t edge_sequence_len;     /*   (one sequence shared by all networks is
                                      not allowed; give the full sequence) */
  /* MIXED only: per-phase limits; zeros select the defaults.  The BF16 and
     FP32 phases also stop at their noise floor: when a network's mean diff
     has not dropped below 0.9x its best value for 3 sweeps. */
  double tol_bf16;               /* default 1e-6 */
  double tol_f32;                /* default 1e-13 */
  int32_t maxiter_bf16;          /* default maxiter */
  int32_t maxiter_f32;           /* default maxiter */
  int32_t refine_f64;            /* cap on the refinement sweeps after FP32
                                    (they stop at tol), default maxiter */
  int32_t refine;                /* gbtn_refine, default DF32 */
  int32_t confirm_f64;           /* FP64 sweeps after a DF32 refinement
                                    (they stop at tol), default 0 */
} gbtn_bp_opts;

/* ---- context ----------------------------------------------------------- */
/* Replaces: the host process of ITensorNetworks (no counterpart; one context
 * per host thread, bound to one CUDA device). */
int gbtn_ctx_create(int device, gbtn_ctx** out);
int gbtn_ctx_destroy(gbtn_ctx* ctx);
const char* gbtn_last_error(const gbtn_ctx* ctx);
/* Stream used by every later launch of this context (NULL = the context's own). */
int gbtn_ctx_set_stream(gbtn_ctx* ctx, void* cuda_stream);
void* gbtn_ctx_get_stream(const gbtn_ctx* ctx);
int gbtn_abi_version(void);
/* Instrumentation (no counterpart in the reference): with profiling on, every
 * message-kernel launch of the context is bracketed by CUDA events on the
 * context's stream.  gbtn_ctx_kernel_time returns, and forgets, the summed
 * device time and the launch count of one kernel class. */
enum gbtn_kernel_class {
  GBTN_KCLASS_TENSOR_CORE = 0,
  GBTN_KCLASS_SIMT_F32 = 1,
  GBTN_KCLASS_SIMT_F64 = 2,
  GBTN_KCLASS_GAUGE = 3, /* rescale_messages: message normalisation and gauge scaling */
  GBTN_KCLASS_SIMT_DF32 = 4,
  GBTN_KCLASS_LARGE = 5 /* global-memory path of vertices beyond the shared-memory kernels */
};
int gbtn_ctx_set_profiling(gbtn_ctx* ctx, int on);
/* Failure-detection test of the bounded device waits.  on = 1 makes every
 * tensor-core image copy launched afterwards (any context of the process;
 * CUDA graphs captured before keep their launches) expect 16 bytes more than it
 * delivers: the copy lands, its mbarrier never completes, the kernel's 1 s
 * bounded wait gives up, the CTA drains its own copies, frees its TMEM and
 * returns, and the BF16 sweep returns GBTN_ERR_TIMEOUT (the plan and context
 * stay usable).  No fault, trap or hang.  on = 0 (the default) restores
 * normal operation.  Not for production use. */
int gbtn_ctx_test_wait_timeout(gbtn_ctx* ctx, int on);
int gbtn_ctx_kernel_time(gbtn_ctx* ctx, int kernel_class, double* total_ms, int64_t* launches);

/* ---- plan (BeliefPropagationCache storage) ------------------------------ */
/* Replaces: BeliefPropagationCache(ptn; messages) and initialize_cache
 * (src/caches/beliefpropagationcache.jl:20-35, src/initialize_cache.jl:14-28):
 * validates the graph (no self loops, legs consistent with edges) and
 * allocates device storage for tensors and messages. */
int gbtn_plan_create(gbtn_ctx* ctx, const gbtn_graph_desc* desc, gbtn_plan** out);
int gbtn_plan_destroy(gbtn_plan* plan);
/* Element counts of the concatenated tensor and message arrays. */
int gbtn_plan_sizes(const gbtn_plan* plan, int64_t* n_factor, int64_t* n_message);
/* Instrumentation (no counterpart in the reference): how often the plan's
 * arrays crossed the host boundary since it was made: counts[0] tensor
 * uploads (gbtn_set_factors), [1] message uploads (gbtn_set_messages),
 * [2] message read-backs (gbtn_get_messages), [3] tensor read-backs
 * (gbtn_get_factors).  A caller that keeps one plan for update, expect,
 * logscalar and normalize sees one tensor upload and no message traffic. */
int gbtn_plan_counters(const gbtn_plan* plan, int64_t counts[4]);
/* Tensor-core routing of the BF16 phase (no counterpart in the reference,
 * which contracts every vertex the same way; the "autotuner keyed on chi, d
 * and degree").  Vertices with d = 2, at most four legs and chi <= 8 can run
 * the tensor-core kernel zero-padded to degree 4, chi = 8; the rest run the
 * FP32 SIMT kernel.  AUTO (default) times splits of the candidates, ordered
 * by their algorithmic flops, on the plan's own vertices at the first BF16 /
 * MIXED run after the policy is set; ALL routes every candidate, NATIVE only
 * degree-4 chi = 8 vertices, OFF none.  gbtn_plan_tc_split writes 1 per
 * tensor-core vertex into is_tc[nv] (tuning first if needed) and, when
 * tuned_ms is not NULL, the measured time of the chosen split (0 if the
 * policy is not AUTO). */
enum gbtn_tc_policy { GBTN_TC_AUTO = 0, GBTN_TC_ALL = 1, GBTN_TC_NATIVE = 2, GBTN_TC_OFF = 3 };
int gbtn_plan_set_tc_policy(gbtn_plan* plan, int32_t policy);
int gbtn_plan_tc_split(gbtn_plan* plan, int32_t* is_tc, double* tuned_ms);

/* SIMT team widths (no counterpart in the reference).  Before the first
 * parallel or coloured sweeps of each arithmetic, the plan times the vertex
 * kernel with 32 (four vertices per block), 128 and 256 threads per vertex on
 * up to 2048 vertices of every size class of its own network (vertex size n
 * up to a power of two; CUDA events, best of two) and keeps the fastest width
 * per class -- the results equal those of any width up to rounding in the
 * close reductions.  gbtn_plan_set_simt_tuning(plan, mode) forgets the
 * choices; mode 0 restores the fixed rule (32 threads up to n = 1024, else
 * 256), 1 (the default) measures again at the next run, and 32, 128 or 256
 * takes that width for every class whose shared memory allows it.  gbtn_plan_simt_teams writes the
 * width chosen for arithmetic `arith` (0 FP64, 1 FP32, 2 df32, 3 complex FP64,
 * 4 complex FP32) into teams[k] for the classes n <= 2^k, k < 32 (0: not
 * measured). */
int gbtn_plan_set_simt_tuning(gbtn_plan* plan, int32_t on);
int gbtn_plan_simt_teams(const gbtn_plan* plan, int32_t arith, int32_t teams[32]);
/* CUDA graphs for the parallel / coloured sweeps (no counterpart in the
 * reference): with on = 1, a run of three or more sweeps launches its first
 * sweep directly and replays the rest from a CUDA graph of two sweeps, kept
 * in the plan per launch configuration.  Off by default; event profiling
 * (gbtn_ctx_set_profiling) bypasses the graphs. */
int gbtn_plan_set_graphs(gbtn_plan* plan, int32_t on);

/* Replaces: bpc[v] = tensor (update_factors, abstractbeliefpropagationcache.jl:158-171).
 * bra may be NULL unless the plan has separate_bra. */
int gbtn_set_factors(gbtn_plan* plan, const double* ket, const double* bra, int mem);
int gbtn_get_factors(gbtn_plan* plan, double* ket, int mem);
/* Replaces: set_messages! / messages (abstractbeliefpropagationcache.jl:173-191). */
int gbtn_set_messages(gbtn_plan* plan, const double* msgs, int mem);
int gbtn_get_messages(gbtn_plan* plan, double* msgs, int mem);
/* message_diff (abstractbeliefpropagationcache.jl:32-36) of every directed
   edge from the last sweep that ran with a tolerance (tol >= 0): 2*ne doubles
   in directed-edge order (NaN before the first such sweep).  A caller that
   splits one network across processes sums the diffs of the edges it owns
   (the reference's update loop sums them over the whole sweep, :313-329). */
int gbtn_get_edge_diffs(gbtn_plan* plan, double* diffs, int mem);
/* Replaces: identity_messages (src/formnetworks/quadraticformnetwork.jl:96-124);
 * GBTN_INIT_ONES gives all-ones messages of unit Frobenius norm. */
int gbtn_init_messages(gbtn_plan* plan, int kind);

/* ---- message passing ------------------------------------------------------ */
/* Replaces: update(bpc; maxiter, tol, edge_sequence, message_update_alg)
 * (abstractbeliefpropagationcache.jl:313-337, message update :225-239).
 * iters[n_networks] and mean_diff[n_networks] (may be NULL) receive, per
 * network, the sweeps run and sum(diff)/len(sequence) of the last sweep
 * (NaN when tol < 0). */
int gbtn_bp_run(gbtn_plan* plan, const gbtn_bp_opts* opts, int32_t* iters, double* mean_diff);
/* Instrumentation (no counterpart in the reference): the sweeps each phase of
 * the last gbtn_bp_run took, the most over the plan's networks:
 * sweeps[0..3] = BF16, FP32, refinement (DF32 or FP64), FP64 confirmation
 * (0 for a phase that did not run; a single-precision run counts in its
 * own slot, FP64 in slot 3). */
int gbtn_plan_phase_sweeps(gbtn_plan* plan, int32_t sweeps[4]);
/* Replaces: updated_message(bpc, edge) (abstractbeliefpropagationcache.jl:225-239,
 * 254-261): the normalised new message of one directed edge, FP64, written to
 * out (chi*chi) without changing the cache. */
int gbtn_updated_message(gbtn_plan* plan, int32_t directed_edge, double* out);

/* ---- environments, scalars, expectation values (FP64) ------------------- */
/* Replaces: environment(bpc, [operator_vertex(v)]) contracted with the ket and
 * bra of v (expect.jl:5-19): rho_v[s', s], d_v*d_v per vertex, concatenated. */
int gbtn_vertex_rdms(gbtn_plan* plan, double* out);
/* Replaces: expect(psi, op; alg="bp") over all vertices (expect.jl:21-41).
 * ops: d*d matrix O[s', s] shared by all vertices (per_vertex = 0) or one per
 * vertex concatenated (per_vertex = 1).  out[nv] = tr(rho O)/tr(rho). */
int gbtn_expect1(gbtn_plan* plan, const double* ops, int per_vertex, double* out);
/* Replaces: the two-site RDM of test/test_belief_propagation.jl:64-91 on the
 * listed undirected edges: (du*dv)^2 per edge, row s'_u + du*s'_v, column
 * s_u + du*s_v. */
int gbtn_edge_rdms(gbtn_plan* plan, const int32_t* edges, int32_t n_edges, double* out);
/* Two-site expectation values with one shared (du*dv)^2 operator. */
int gbtn_expect2(gbtn_plan* plan, const int32_t* edges, int32_t n_edges, const double* op,
                 double* out);
/* Replaces: vertex_scalars / edge_scalars (abstractbeliefpropagationcache.jl:83-97,
 * beliefpropagationcache.jl:107-119). */
int gbtn_vertex_scalars(gbtn_plan* plan, double* out);
int gbtn_edge_scalars(gbtn_plan* plan, double* out);
/* Replaces: logscalar(bpc) (abstractbeliefpropagationcache.jl:397-408), FP64
 * accumulation per network: re[n] + i*im[n]; -Inf real part when an edge
 * scalar is zero. */
int gbtn_logscalar(gbtn_plan* plan, double* re, double* im);
/* Replaces: rescale_messages (beliefpropagationcache.jl:121-139). */
int gbtn_rescale_messages(gbtn_plan* plan);
/* Replaces: rescale_partitions on ket+bra vertices (abstractbeliefpropagationcache.jl:349-379,
 * normalize.jl:77): every vertex scalar becomes 1.  Both tensors are divided
 * by their norms, then with r = z^(-1/2) (principal root) of the partition
 * scalar z and s = sign(z) for a real z (else 1) the ket is scaled by s*r and
 * the bra by s*s*r, as in the reference (whose partitions list the bra first).
 * With bra = conj(ket) only the ket is scaled (a real network with a negative
 * z gets NaN tensors; with a separate real bra, where the reference raises a
 * DomainError, the sign goes on the bra and the scalar still becomes 1); for
 * complex tensors the remaining phases z/|z| are then
 * moved onto the messages, which carry a free phase (m_{u->v} by e^{i psi},
 * m_{v->u} by e^{-i psi} on the edges of a spanning forest, which keeps every
 * edge scalar), so vertex scalars become 1 as in the reference. */
int gbtn_rescale_partitions(gbtn_plan* plan);

/* ---- simple update / apply (FP64) ------------------------------------------- */
/* Replaces: the network state updated by apply(o, psi; envs, maxdim, cutoff,
 * normalize) (src/apply.jl:97-160, simple_update_bp :33-95) and tebd
 * (src/tebd.jl:2-31).  Site tensors keep their current bond dimensions, which
 * grow up to chi_max; the graph descriptor's edge_dim gives the initial ones.
 * With complex_values set in the descriptor, tensors, gates and environments
 * are interleaved (re, im) doubles (ComplexF64; e.g. the RandomUnitary gates
 * of test/test_apply.jl), run by a one-kernel complex path limited to site
 * tensors of <= 4096 elements (also with the bond at chi_max) and theta
 * <= 32 x 32; larger gates report GBTN_ERR_UNSUPPORTED.  Real tensors: a site
 * tensor, also rebuilt with the gate's bond at maxdim, holds <= 8192 elements
 * and theta <= 64 x 64; a call with a gate beyond that returns
 * GBTN_ERR_UNSUPPORTED before any of its gates runs. */
typedef struct gbtn_su gbtn_su;
int gbtn_su_create(gbtn_ctx* ctx, const gbtn_graph_desc* desc, int32_t chi_max, gbtn_su** out);
int gbtn_su_destroy(gbtn_su* su);
/* Current bond dimension of every edge. */
int gbtn_su_edge_dims(gbtn_su* su, int32_t* dims);
/* Tensors with the current bond dimensions, concatenated in vertex order (host). */
int gbtn_su_set_factors(gbtn_su* su, const double* ket);
int gbtn_su_get_factors(gbtn_su* su, double* ket, int64_t capacity);
/* Apply two-site gates in the given order (consecutive vertex-disjoint gates
 * run concurrently).  Gate j acts on edge edges[j] = (u, v) as a (du*dv)^2
 * matrix, row s'_u + du*s'_v, column s_u + du*s_v; per_gate = 0 shares one
 * gate.  envs: NULL (tebd) or 2*ne messages of chi_max^2 values each, the
 * current chi x chi message M[b, a] of every directed edge in its leading
 * chi*chi entries.  maxdim <= chi_max, cutoff < 0 disables the cutoff.
 * truncerr[n_gates] and svals[n_gates * maxdim] (kept singular values, zero
 * padded) may be NULL. */
int gbtn_su_apply(gbtn_su* su, int32_t n_gates, const int32_t* edges, const double* gates, int32_t per_gate,
                  const double* envs, int32_t maxdim, double cutoff, int32_t normalize, double* truncerr,
                  double* svals);
/* Set every bond dimension (1..chi_max), e.g. to restore a saved state before
 * gbtn_su_set_factors. */
int gbtn_su_set_edge_dims(gbtn_su* su, const int32_t* dims);
/* Adjoint of gbtn_su_apply (no counterpart in the reference), real tensors:
 * the current tensors are the gates' inputs (they are not changed).  The
 * gates of one call act on disjoint vertices (apply the adjoints of a longer
 * gate sequence batch by batch, in reverse order, from saved states).
 * post_edge_dims: the bond dimensions gbtn_su_apply left (checked against
 * the recomputed truncation).  cot_out: dL/d(tensors after the gates),
 * concatenated in vertex order with post_edge_dims; cot_in receives
 * dL/d(current tensors) in the current shapes (sites without a gate pass
 * theirs through); gate_cot (may be NULL): n_gates (du dv)^2 matrices dL/dG
 * (with per_gate = 0 the shared gate's cotangent is their sum); env_cot
 * (may be NULL): dL/d(envs) in the layout of envs (2 ne messages of chi_max^2
 * values, each chi x chi message's leading entries; zeros without envs),
 * through the square-root and inverse-square-root environments (positive
 * semi-definite messages, as BP's are).  Degenerate singular values (closer
 * than 1e-14 sigma_max^2) and kept zero singular values contribute no
 * derivative. */
int gbtn_su_apply_vjp(gbtn_su* su, int32_t n_gates, const int32_t* edges, const double* gates, int32_t per_gate,
                      const double* envs, int32_t maxdim, double cutoff, int32_t normalize,
                      const int32_t* post_edge_dims, const double* cot_out, double* cot_in, double* gate_cot,
                      double* env_cot);
/* gbtn_su_apply that also records a tape for the adjoint of the whole gate
 * sequence (real tensors): the state before every batch of consecutive
 * vertex-disjoint gates (device copies of the tensors and bond dimensions),
 * the final state, the gates, environments and options.  Memory: one copy of
 * the state's tensor storage per batch, plus one. */
typedef struct gbtn_su_tape gbtn_su_tape;
int gbtn_su_apply_taped(gbtn_su* su, int32_t n_gates, const int32_t* edges, const double* gates, int32_t per_gate,
                        const double* envs, int32_t maxdim, double cutoff, int32_t normalize, double* truncerr,
                        double* svals, gbtn_su_tape** tape);
/* The pullback of a taped apply: cot_out = dL/d(tensors it left), in their
 * shapes; cot_in = dL/d(tensors before it), in those shapes; gate_cot
 * (may be NULL): n_gates (du dv)^2 matrices dL/dG in the order given;
 * env_cot (may be NULL): dL/d(envs), summed over the batches, as in
 * gbtn_su_apply_vjp.  The batches run backwards on the device (each batch's
 * saved state restored, the cotangents kept in device memory); the state is
 * left as the taped apply left it.  The tape can be pulled back more than
 * once. */
int gbtn_su_tape_vjp(gbtn_su* su, const gbtn_su_tape* tape, const double* cot_out, double* cot_in,
                     double* gate_cot, double* env_cot);
int gbtn_su_tape_destroy(gbtn_su_tape* tape);

/* ---- energies and gradients (FP64) ------------------------------------------ */
/* Two-site energy sum_e sum_t coef[t] <O_t (x) O_t>_e with BP reduced density
 * matrices (the pattern of test/test_belief_propagation.jl:64-91 applied to
 * every edge); ops holds n_terms d x d matrices O[s', s] (all vertices share d).
 * energy[n_networks] receives each network's sum.  No counterpart to the
 * gradient exists in the reference (it has no automatic differentiation). */
enum gbtn_grad_mode { GBTN_GRAD_IMPLICIT = 0, GBTN_GRAD_UNROLLED = 1 };
typedef struct gbtn_grad_opts {
  int32_t mode;        /* IMPLICIT: through the converged messages already in the
                          plan (adjoint BP solve); UNROLLED: through `unroll`
                          parallel sweeps from identity messages, which also
                          leave their messages in the plan */
  int32_t maxiter;     /* IMPLICIT: adjoint iterations (default 500) */
  double tol;          /* IMPLICIT: stop at |l_new - l| <= tol |l_new| (default 1e-12) */
  int32_t unroll;      /* UNROLLED: number of sweeps */
  int32_t checkpoint;  /* UNROLLED: keep every k-th sweep (0 = ceil(sqrt(unroll))) */
} gbtn_grad_opts;
int gbtn_energy2(gbtn_plan* plan, int32_t n_terms, const double* coef, const double* ops, double* energy);
/* Energy and its gradient with respect to every site tensor (n_factor values,
 * same layout as gbtn_set_factors).  iters / resid (may be NULL): adjoint
 * iterations and final relative residual (IMPLICIT), or sweeps (UNROLLED).
 * Complex plans: ops are complex d x d matrices (interleaved), the energy is
 * the real part of sum_e sum_t c_t <O_t (x) O_t>_e, and the gradient is
 * dE/dRe + i dE/dIm (interleaved). */
int gbtn_energy2_grad(gbtn_plan* plan, int32_t n_terms, const double* coef, const double* ops,
                      const gbtn_grad_opts* opts, double* energy, double* grad, int32_t* iters, double* resid);
/* Vector-Jacobian product of the BP messages: given dL/dm (n_message
 * values), the gradient dL/dA (n_factor values).  IMPLICIT: through the fixed
 * point, the converged messages in the plan (implicit differentiation, the
 * adjoint BP solve).  UNROLLED: through opts->unroll normalised Jacobi sweeps
 * from identity messages (dL/dm of their final messages, checkpointed every
 * opts->checkpoint sweeps, 0 = ceil(sqrt(unroll))); those final messages are
 * left in the plan.  Complex plans: both are dL/dRe + i dL/dIm of a real loss
 * L, interleaved (re, im). */
int gbtn_bp_vjp(gbtn_plan* plan, const double* msg_cot, const gbtn_grad_opts* opts, double* grad, int32_t* iters,
                double* resid);

/* Gradients of the BP log-norm and of one-site expectation values with
 * respect to every site tensor (no counterpart in the reference, which has no
 * automatic differentiation), at the messages in the plan, which must be a
 * converged fixed point: the direct derivatives (messages held) plus the
 * implicit part through the fixed point (the adjoint BP solve of
 * gbtn_bp_vjp; opts may be NULL for its defaults, mode is ignored).
 *   gbtn_logscalar_grad: value[n] = Re logscalar of network n
 *     (abstractbeliefpropagationcache.jl:397-408) and grad = d/dA of the sum;
 *   gbtn_expect1_grad: value[n] = sum_v <O_v> over network n's vertices
 *     (expect.jl:5-19, one d x d operator O[s', s] for all) and its gradient.
 * Complex plans take the real part of the value (log|.| for the log-norm)
 * and return the gradient as dL/dRe + i dL/dIm (interleaved, the tensors'
 * layout); op is then complex too.  FP64 quadratic-form plans whose vertices
 * all have a link and fit the shared-memory kernels; others return
 * GBTN_ERR_UNSUPPORTED. */
int gbtn_logscalar_grad(gbtn_plan* plan, const gbtn_grad_opts* opts, double* value, double* grad, int32_t* iters,
                        double* resid);
int gbtn_expect1_grad(gbtn_plan* plan, const double* op, const gbtn_grad_opts* opts, double* value, double* grad,
                      int32_t* iters, double* resid);

/* ---- charge-conserving (QN) block-sparse networks ------------------------ */
/* Replaces: BP on QN-conserving ITensors (ITensors' conserve_qns = true, e.g.
 * the QN-graded loopy network of test/test_belief_propagation.jl:103-116).
 * Every index carries sectors of one U(1) charge: the sectors of a link are
 * contiguous ranges of its dense index (sec_dim of them, in order, summing to
 * edge_dim), likewise those of a site index.  A vertex tensor is nonzero only
 * in the blocks whose charges balance its flux:
 *   charge(site sector) + sum_{legs into v} q - sum_{legs out of v} q = flux[v],
 * where a link's sector charge q is counted out of edge_u[e] and into
 * edge_v[e].  Messages of such a network stay block-diagonal in the link
 * sectors, so the plan stores only the nonzero blocks of the tensors and the
 * diagonal sector blocks of the messages, and contracts block by block.
 * Real FP64 tensors; sector dimensions <= 8, degree <= 8; the sectors of one
 * index carry distinct charges (merge equal-charge sectors first). */
typedef struct gbtn_qn_desc {
  const int32_t* edge_sec_ptr;    /* [ne+1] CSR offsets into sec_dim / sec_charge */
  const int32_t* sec_dim;         /* link sector dimensions */
  const int32_t* sec_charge;      /* link sector charges (out of edge_u, into edge_v) */
  const int32_t* site_sec_ptr;    /* [nv+1] CSR offsets into site_sec_dim / site_sec_charge */
  const int32_t* site_sec_dim;    /* site sector dimensions */
  const int32_t* site_sec_charge; /* site sector charges */
  const int32_t* flux;            /* [nv] flux of every vertex tensor */
} gbtn_qn_desc;
typedef struct gbtn_qn_plan gbtn_qn_plan;
/* Replaces: BeliefPropagationCache / initialize_cache for a QN network. */
int gbtn_qn_plan_create(gbtn_ctx* ctx, const gbtn_graph_desc* desc, const gbtn_qn_desc* qn, gbtn_qn_plan** out);
int gbtn_qn_plan_destroy(gbtn_qn_plan* plan);
/* Counts: nonzero blocks, their elements, and the elements of the sector-packed messages. */
int gbtn_qn_plan_sizes(const gbtn_qn_plan* plan, int32_t* n_blocks, int64_t* n_block_elems, int64_t* n_message);
/* The blocks in storage order: for block i, blocks[i*10 + 0] = vertex,
 * [i*10 + 1] = its site sector, [i*10 + 2 + p] = its sector on leg p (-1 past
 * the degree); offsets[i] = its first element.  A block is a dense tensor of
 * shape (site sector dim, leg sector dims...) in column-major order. */
int gbtn_qn_blocks(const gbtn_qn_plan* plan, int32_t* blocks, int64_t* offsets);
/* Replaces: bpc[v] = tensor for every vertex (update_factors). */
int gbtn_qn_set_blocks(gbtn_qn_plan* plan, const double* data, int mem);
/* Replaces: identity_messages (quadraticformnetwork.jl:96-124): the identity in every sector block. */
int gbtn_qn_init_messages(gbtn_qn_plan* plan);
/* Sector-packed messages: directed edge after directed edge (2e = u -> v),
 * within one the sector blocks of its link in order, each dim x dim M[b, a]
 * column-major (the dense message is block-diagonal with these blocks). */
int gbtn_qn_set_messages(gbtn_qn_plan* plan, const double* msgs, int mem);
int gbtn_qn_get_messages(gbtn_qn_plan* plan, double* msgs, int mem);
/* Replaces: update(bpc; maxiter, tol) with the parallel (Jacobi) schedule;
 * message_diff and its mean as the dense plan (abstractbeliefpropagationcache.jl:32-36, 313-329). */
int gbtn_qn_bp_run(gbtn_qn_plan* plan, int32_t maxiter, double tol, int32_t* iters, double* mean_diff);
/* Replaces: update(bpc; maxiter, tol, edge_sequence) with the reference's
 * default sequential schedule (abstractbeliefpropagationcache.jl:272-287):
 * the messages of edge_sequence (directed edges, repeats allowed) updated in
 * order, each seeing every earlier update; executed in waves of messages that
 * do not depend on one another, so the result is the strictly sequential one.
 * The mean diff is over the sequence positions. */
int gbtn_qn_bp_run_sequential(gbtn_qn_plan* plan, const int32_t* edge_sequence, int32_t edge_sequence_len,
                              int32_t maxiter, double tol, int32_t* iters, double* mean_diff);
/* Replaces: update(bpc; maxiter, tol, ...) on a block-sparse network, with
 * the precision and schedule choices of gbtn_bp_run: PARALLEL or SEQUENTIAL
 * (edge_sequence as above); F64, F32 (FP32 blocks and messages, FP64 norms
 * and diffs), DF32 (double-FP32 arithmetic on the FP64 blocks), or MIXED
 * (FP32 sweeps to tol_f32 or their noise floor, then DF32 -- or FP64 with
 * refine = GBTN_REFINE_F64 -- sweeps to tol, optional FP64 confirm_f64
 * sweeps).  BF16 and COLORED are refused (GBTN_ERR_UNSUPPORTED /
 * GBTN_ERR_INVALID): block-sparse vertices have no tensor-core path.
 * iters: sweeps of the last phase. */
int gbtn_qn_bp_run_ex(gbtn_qn_plan* plan, const gbtn_bp_opts* opts, int32_t* iters, double* mean_diff);
/* Sweeps each phase of the last QN run took: [BF16 (always 0), FP32,
 * refinement, FP64]. */
int gbtn_qn_phase_sweeps(const gbtn_qn_plan* plan, int32_t* sweeps);
/* Replaces: the one-site environments of expect (expect.jl:5-19): dense
 * rho_v[s', s] (d x d, block-diagonal in the site sectors) per vertex. */
int gbtn_qn_vertex_rdms(gbtn_qn_plan* plan, double* out);
/* Replaces: logscalar(bpc) (abstractbeliefpropagationcache.jl:397-408). */
int gbtn_qn_logscalar(gbtn_qn_plan* plan, double* re, double* im);

/* ---- allocation-free sweep ------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need a message update (a framework capturing its stream
 * into a CUDA graph, or an application that gives the library a fixed memory
 * budget): one FP64 parallel (Jacobi) sweep, msg_in -> msg_out, with the mean
 * message diff over all directed edges written to *mean_diff.  Every pointer,
 * including the arrays inside *dev_graph (the struct itself stays on the
 * host), is DEVICE memory owned by the caller; the library allocates
 * nothing and keeps its scratch in a fixed ~1.2 MiB device array.  The first
 * call on a device sets that array up (make it before any stream capture; a
 * set-up that fails returns GBTN_ERR_CUDA and is tried again by the next
 * call); calls that overlap on the GPU share the array and race.
 * Asynchronous on `stream` (NULL = the legacy default stream).
 * Returns GBTN_ERR_UNSUPPORTED when nv > GBTN_STATIC_MAX_VERTICES,
 * 2*ne > GBTN_STATIC_MAX_DIRECTED_EDGES, complex_values is set (real
 * tensors only) or separate_bra is set (the bra is always the ket here).
 * The descriptor is checked on the device, since the call does not wait for
 * the GPU: a vertex beyond the kernel limits (degree > 8, chi > 8, d > 8,
 * d*prod(chi) > 8192) or one that fails a structural check (leg_ptr
 * decreasing or not starting at 0, a leg edge outside 0..ne-1 or not incident
 * to the vertex, a dimension < 1) is skipped without reading out of bounds:
 * its outgoing entries of msg_out are left unwritten (they keep whatever the
 * buffer held) and *mean_diff becomes NaN, while every other vertex's
 * messages are computed as usual.  The call itself still returns GBTN_OK. */
#define GBTN_STATIC_MAX_VERTICES 16384
#define GBTN_STATIC_MAX_DIRECTED_EDGES 65536
int gbtn_bp_sweep_static(int device, const gbtn_graph_desc* dev_graph, const double* factors,
                         const double* msg_in, double* msg_out, double* mean_diff, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBTN_H */
