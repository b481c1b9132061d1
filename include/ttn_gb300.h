/* ttn_gb300.h -- C-ABI of the GB300-native one-site projector-splitting TDVP sweep.
 *
 * The entry points replace the objects a caller of ttns_lib builds around the sweep
 * (paths are relative to the ttns_lib project root):
 *
 *   ttn_tree_*        <- ntree<size_t> topology + httensor(topology, capacity)
 *                        include/ttns_lib/httensor.hpp:51, :129-288
 *   ttn_sop_*         <- sop_operator<T>(nterms, mode_dims), bind(op, r, mode), coeff(r)
 *                        include/ttns_lib/operators/sop_operator.hpp:262, :323-392, :471-473
 *   ttn_state_*       <- the httensor node matrices A[i]().as_matrix()
 *                        include/ttns_lib/ttn_nodes/httensor_node.hpp:150-153
 *   ttn_integrator_*  <- fixed_step_projector_splitting_integrator<T>
 *                        include/ttns_lib/integrators/projector_splitting_integrator.hpp:76-218
 *                        (initialise :115-129, operator() :136-169, dt() :187-188,
 *                         nh_applications() :190)
 *   ttn_expect_leaf / ttn_norm2
 *                     <- matrix_element::operator()(op, mode, psi) and operator()(psi)
 *                        include/ttns_lib/observables/matrix_element.hpp:153-187, :264-314
 *
 * Conventions
 *   * complex numbers are interleaved double pairs (re, im);
 *   * a node matrix is row-major (dimen x hrank) with the children's indices in child
 *     order, the last child fastest, exactly the reference's as_matrix() layout;
 *   * nodes are numbered in pre-order (parent[0] = -1, parent[i] < i) and the
 *     children of a node are ordered by id;
 *   * every call returns TTN_OK or an error code; ttn_last_error() gives the message
 *     of the last failure on the calling thread.  No C++ exception crosses the ABI.
 *   * objects are not thread-safe; use one integrator per host thread.  Each
 *     integrator owns its CUDA stream and device workspaces.
 */
#ifndef TTN_GB300_H
#define TTN_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TTN_OK = 0,
  TTN_EINVAL = 1,     /* bad argument or ill-formed tree / operator */
  TTN_ECAPACITY = 2,  /* a size exceeds an allocated capacity */
  TTN_ENUMERIC = 3,   /* non-finite values or a failed Krylov / eigen solve */
  TTN_ECUDA = 4,      /* a CUDA runtime call failed */
  TTN_ETIMEOUT = 5,   /* a bounded device-side wait gave up */
  TTN_ENOTSUP = 6     /* valid request outside what the library implements */
};

/* precision of the contractions in the sweep */
enum { TTN_PREC_FP64 = 0, TTN_PREC_MIXED = 1 };

typedef struct ttn_tree ttn_tree;
typedef struct ttn_sop ttn_sop;
typedef struct ttn_state ttn_state;
typedef struct ttn_integrator ttn_integrator;

typedef struct ttn_integ_cfg {
  int krylov_dim;          /* Lanczos dimension m (reference default 4; driver default 6) */
  double krylov_tol;       /* local error tolerance of the exponential (reference 1e-12) */
  int precision;           /* TTN_PREC_FP64 or TTN_PREC_MIXED */
  int device;              /* CUDA device ordinal */
} ttn_integ_cfg;

const char* ttn_last_error(void);
const char* ttn_version(void);

/* ---- tree ---------------------------------------------------------------------- */
/* parent[nnodes] (pre-order), hrank[nnodes]; leaf_mode[i] >= 0 and leaf_dim[i] > 0 on
 * leaves, -1 / 0 on branch nodes.  hrank must not exceed the product of the node's
 * child dimensions (ntree_builder::sanitise_tree, include/ttns_lib/tree/ntree_builder.hpp:215-233). */
int ttn_tree_create(int nnodes, const int* parent, const int* hrank, const int* leaf_mode,
                    const int* leaf_dim, ttn_tree** out);
int ttn_tree_destroy(ttn_tree* t);
int ttn_tree_num_nodes(const ttn_tree* t, int* out);
int ttn_tree_node_shape(const ttn_tree* t, int node, long long* dimen, int* hrank);
int ttn_tree_state_size(const ttn_tree* t, long long* n_complex);

/* ---- sum-of-product operator --------------------------------------------------- */
int ttn_sop_create(int nterms, int nmodes, const int* mode_dims, ttn_sop** out);
int ttn_sop_destroy(ttn_sop* s);
/* bind one operator on `mode` to the terms r[0..nr) (sop_operator::bind) */
int ttn_sop_bind_dense(ttn_sop* s, int mode, const double* mat, const int* r, int nr);
int ttn_sop_bind_diag(ttn_sop* s, int mode, const double* diag, const int* r, int nr);
int ttn_sop_bind_csr(ttn_sop* s, int mode, const int* rowptr, const int* colind,
                     const double* vals, const int* r, int nr);
int ttn_sop_set_coeff(ttn_sop* s, int r, double re, double im);

/* ---- state (device resident) ---------------------------------------------------- */
int ttn_state_create(const ttn_tree* t, int device, ttn_state** out);
int ttn_state_destroy(ttn_state* s);
/* host <-> device copies of the node matrices; `data` holds all nodes concatenated
 * in node order (ttn_tree_state_size complex numbers) */
int ttn_state_upload(ttn_state* s, const double* data);
int ttn_state_download(ttn_state* s, double* data);
int ttn_state_upload_node(ttn_state* s, int node, const double* data);
int ttn_state_download_node(ttn_state* s, int node, double* data);
/* The spin-boson driver's start state (src/spin_boson.cpp:584-649): leaf SPF 0 is psi0
 * on mode 0 and the vacuum elsewhere, the other leaf SPFs are random orthonormal
 * vectors drawn with std::mt19937(seed), interior nodes are identities and the root
 * is e_0.  Generated on the host, then uploaded.  psi0 may be NULL (vacuum). */
int ttn_state_init_product(ttn_state* s, const double* psi0, unsigned int seed);

/* ---- integrator ---------------------------------------------------------------- */
int ttn_integrator_create(const ttn_tree* t, const ttn_sop* h, const ttn_integ_cfg* cfg,
                          ttn_integrator** out);
int ttn_integrator_destroy(ttn_integrator* it);
int ttn_integrator_set_dt(ttn_integrator* it, double dt);
int ttn_integrator_dt(const ttn_integrator* it, double* out);
int ttn_integrator_t(const ttn_integrator* it, double* out);
/* Batched form: advance n independent instances by one step each (instance k = its[k]
 * with states[k]; distinct integrators and states, any mix of trees, operators and
 * devices).  Instances are stepped from `threads` host threads (0: the hardware
 * concurrency), each integrator on its own stream, so small instances overlap on the GPU.
 * Equivalent to calling ttn_integrator_step on each instance in turn (same results); on
 * failure returns the first failing instance's status and message and its index in
 * *failed (-1 when all succeed).  The reference steps one instance per
 * projector_splitting_integrator::operator() (projector_splitting_integrator.hpp:136-169)
 * from its driver loop (src/spin_boson.cpp:81-105); it has no batched call. */
int ttn_batch_step(ttn_integrator* const* its, ttn_state* const* states, int n, double coeff_re, double coeff_im,
                   int threads, int* failed);
/* One call = one step of dt of exp(coeff * H t) (coeff = -i for Schroedinger
 * dynamics); the first call prepares the environments and sub-steps dt as
 * dt*1e-5, dt*1e-4, ... exactly as the reference integrator does. */
int ttn_integrator_step(ttn_integrator* it, ttn_state* psi, double coeff_re, double coeff_im,
                        double* dt_out);
int ttn_integrator_nh_applications(const ttn_integrator* it, long long* out);
/* How a Krylov sub-step ends (the reference's utils::krylov_integrator, called at
 * include/ttns_lib/tdvp_core/projector_splitting_engine.hpp:124-163): mode 0 (default)
 * builds the full krylov_dim space and controls the step size with Sidje's error estimate;
 * mode 1 ends the Lanczos recurrence as soon as beta_0 beta_{j+1} |e_j^T exp(c tau T) e_1|
 * for the whole remaining interval is below krylov_tol, which reproduces the reference's
 * H-application counts on its examples.  Both precisions; the adjoint sweep takes mode 0. */
int ttn_integrator_set_krylov_stop(ttn_integrator* it, int mode);
/* one-site and two-site subspace expansions so far (Nonesite / Ntwosite,
 * include/ttns_lib/tdvp_core/subspace_expansion_projector_splitting_engine.hpp:513-514):
 * the descent counts every two-site attempt, the ascent only the attempts that grew a
 * bond, as the reference does; both zero without expansion */
int ttn_integrator_expansion_counts(const ttn_integrator* it, long long* onesite, long long* twosite);
int ttn_integrator_reset(ttn_integrator* it);
/* Checkpoints (the reference serialises integrator and state with cereal,
 * include/ttns_lib/integrators/projector_splitting_integrator.hpp:50-68, :198-216 and
 * include/ttns_lib/httensor.hpp:101-118): the tree, the integrator's step count, dt,
 * time, coefficient and H-application count, and every node tensor, in one little-endian
 * file.  Loading into an integrator and state of the same tree resumes the run exactly
 * (the environments the next step carries in are recomputed from the tensors).  Not for
 * integrators with subspace expansion. */
int ttn_integrator_save(ttn_integrator* it, ttn_state* psi, const char* path);
int ttn_integrator_load(ttn_integrator* it, ttn_state* psi, const char* path);
/* wait for all queued device work of this integrator */
int ttn_integrator_synchronize(ttn_integrator* it);

/* Environments and gauge passes of the first step without its evolution (the
 * prepare_evolution half of the first call).  Subsequent steps are then full dt
 * steps; used to time steady-state sweeps without the first-step sub-stepping. */
int ttn_integrator_prepare(ttn_integrator* it, ttn_state* psi);
/* algorithmic flops enqueued so far (complex multiply-add = 8 flops) */
int ttn_integrator_flops(const ttn_integrator* it, double* out);
/* device timer on the integrator's stream: start=1 records, start=0 records and
 * returns the elapsed milliseconds since the last start */
int ttn_integrator_timer(ttn_integrator* it, int start, double* ms);

/* ---- observables ----------------------------------------------------------------- */
/* Schmidt values ("pops") across the bond above `node` (1 <= node < nodes), descending,
 * hrank[node] values into out (count in *n); the state must be in the orthogonalised form
 * the sweep leaves.  Replaces the bond singular values of decomposition_engine
 * (include/ttns_lib/tdvp_core/decomposition_engine.hpp:111-205,
 * the S() read after a step) as reported by the reference driver. */
int ttn_bond_singular_values(ttn_integrator* it, ttn_state* psi, int node, double* out, int* n);
/* <psi| O_mode |psi> with a dense d x d operator on one leaf mode */
int ttn_expect_leaf(ttn_integrator* it, ttn_state* psi, int mode, const double* op, double* re,
                    double* im);
int ttn_norm2(ttn_integrator* it, ttn_state* psi, double* out);
/* <bra|ket> of two states of the integrator's tree (matrix_element::operator()(bra, ket),
 * include/ttns_lib/observables/matrix_element.hpp:223-259) */
int ttn_overlap(ttn_integrator* it, ttn_state* bra, ttn_state* ket, double* re, double* im);
/* <bra| prod_k O_k |ket> with dense operators ops[k] (d x d of mode modes[k], concatenated,
 * interleaved) on distinct modes and the identity elsewhere; bra may be ket
 * (matrix_element::operator()(product operator, bra, ket), matrix_element.hpp:318-356,
 * :441-481) */
int ttn_expect_product(ttn_integrator* it, ttn_state* bra, ttn_state* ket, int nops, const int* modes,
                       const double* ops, double* re, double* im);
/* <bra| H |ket> of a sum-of-product operator (matrix_element::operator()(sop, ...),
 * matrix_element.hpp:358-379, :483-500): the sum of the terms' product contractions */
int ttn_expect_sop(ttn_integrator* it, ttn_state* bra, ttn_state* ket, const ttn_sop* op, double* re, double* im);

/* ---- time-dependent primitive operators --------------------------------------------- */
/* fn(user, mode, op, t, dt, mat) is called before every leaf evolution for each operator
 * bound on the leaf's mode -- the reference's primitive::update(t, dt) hook
 * (include/ttns_lib/tdvp_core/projector_splitting_engine.hpp:139, called with the engine
 * time and dt/2): op is the operator's binding index, mat its d x d matrix (interleaved),
 * updated in place on the host and copied to the device.  fn = NULL removes the hook.
 * FP64 integrators only. */
typedef void (*ttn_op_update_fn)(void* user, int mode, int op, double t, double dt, double* mat);
int ttn_integrator_set_op_update(ttn_integrator* it, ttn_op_update_fn fn, void* user);

/* ---- subspace expansion ------------------------------------------------------------ */
/* Adaptive bond dimension for the following steps, replacing
 * subspace_expansion_projector_splitting_integrator
 * (include/ttns_lib/integrators/projector_splitting_integrator.hpp:221-393; engine
 * include/ttns_lib/tdvp_core/subspace_expansion_projector_splitting_engine.hpp:207-585):
 * capacity[nnodes] is the largest bond dimension above every node (the httensor capacity;
 * capacity[0] equals the root's rank), spawning_threshold / unoccupied_threshold /
 * minimum_unoccupied / neigenvalues / only_when_no_unoccupied are the reference's
 * parameters of the same names, seed starts the random generator of the one-site
 * fallback.  psi is re-laid in slabs sized for the capacities and must be the state
 * stepped afterwards; its bond dimensions (ttn_state_hrank) grow during the steps.  FP64
 * integrators at step 0 only; TTN_EINVAL otherwise. */
int ttn_integrator_set_expansion(ttn_integrator* it, ttn_state* psi, const int* capacity, double spawning_threshold,
                                 double unoccupied_threshold, int minimum_unoccupied, int neigenvalues,
                                 int only_when_no_unoccupied, unsigned seed);
/* current bond dimension above every node (out[nnodes]) */
int ttn_state_hrank(const ttn_state* s, int* out);
/* orthogonaliser::operator() (include/ttns_lib/decompositions/orthogonaliser.hpp:83-112):
 * makes every non-root node of psi an isometry (children before parents: A = Q R, A <- Q,
 * R into the parent's slot), leaving the state unchanged and its norm at the root, so
 * that an arbitrary, non-orthogonal state can be stepped.  Uses the integrator's device
 * QR; psi must have the integrator's tree.  After the first step the integrator's
 * environments are refreshed for the new gauge. */
int ttn_state_orthogonalise(ttn_integrator* it, ttn_state* psi);

/* ---- adjoint sweep ----------------------------------------------------------------- */
/* Gradient of J = sum_k weights[k] Re <psi(t_k)| O_mode |psi(t_k)>, t_k the end of step k,
 * over nsteps integrator steps of dt from psi (the first step sub-stepped like
 * ttn_integrator_step; psi prepared first unless skip_prepare).  No counterpart in the
 * reference: it differentiates the sweep of ttn_integrator_step
 * (include/ttns_lib/integrators/projector_splitting_integrator.hpp:136-169) by the
 * reverse of every operation, with the state checkpointed every checkpoint_every steps
 * and the segments recomputed.  op: dense d x d operator on `mode` (interleaved complex).
 * Out: *J; grad_coeff[nterms] = dJ/dc_r for real perturbations of the term coefficients;
 * grad_ops = cotangent of every operator matrix in binding order (d x d interleaved
 * complex each; for an operator p B, dJ/dp = Re sum conj(grad) * B); grad_state (optional)
 * = cotangent of the state psi is prepared into, node by node as ttn_state_download.
 * Requires an FP64 integrator at step 0 and gauge factors of full rank (a generic state,
 * not a product state); psi is left at the final state and the integrator at step nsteps.
 * TTN_EINVAL on bad arguments, TTN_ENUMERIC on a singular gauge factor or a failed
 * exponential. */
int ttn_adjoint_grad(ttn_integrator* it, ttn_state* psi, double dt, double coeff_re, double coeff_im, int nsteps,
                     const double* weights, int mode, const double* op, int checkpoint_every, int skip_prepare,
                     double* J, double* grad_coeff, double* grad_ops, double* grad_state);

/* ---- measurement entry points (benchmarks and profiles); the kernel-level entry points
 * that only the parity tests use are declared in ttn_gb300_testing.h ------------------ */
/* Krylov kernel phase times accumulated since the last call (TTN_PROFILE set at creation,
 * else zeros), out[16]: out[0..7] ms in begin, matvec, alpha, re-orthogonalisation
 * coefficients, re-orthogonalisation + norm, ||H V_m||, control, combine; out[8] sub-steps,
 * out[9] launches; out[10..13] ms inside the tensor-core contractions (row exponents,
 * chunk pipeline, TMEM drain, output), out[14] tensor-core tiles (as seen by CTA 0) */
int ttn_integrator_kernel_phases(ttn_integrator* it, double* out);
/* time `reps` repetitions of one node operation on the device (kind 0: H_eff
 * application, 1: Krylov exponential of the node over dt/2 (persistent kernel),
 * 2: leaf-to-root Householder QR, 3: Krylov exponential of the node's bond matrix);
 * returns milliseconds and algorithmic flops per repetition */
int ttn_bench_node_op(ttn_integrator* it, ttn_state* psi, int node, int kind, int reps, double* ms_per_rep,
                      double* flops_per_rep);
/* Turns the synchronising per-operation breakdown below on (1) or off (0) and clears it
 * (TTN_PROFILE in the environment turns it on at creation).  It synchronises the stream
 * after every operation, so a step runs slower while it is on. */
int ttn_integrator_set_profiling(ttn_integrator* it, int on);
/* With the breakdown on (TTN_PROFILE or ttn_integrator_set_profiling), synchronising wall-clock seconds and
 * call counts per operation kind (8: node exponential, bond exponential, root-to-leaf
 * QR, leaf-to-root QR, mean-field update, spf update, apply-to-parent,
 * apply-from-parent) and node-size class (4: <1K, <64K, <1M, >=1M elements);
 * 32 doubles and 32 counts. */
int ttn_integrator_profile(ttn_integrator* it, double* seconds, long long* counts);
/* host<->device bytes moved by this integrator's step and observable calls */
int ttn_integrator_io_bytes(const ttn_integrator* it, long long* h2d, long long* d2h);
/* page-locked host memory for callers that keep node tensors on the host between steps */
int ttn_host_alloc(long long bytes, void** out);
int ttn_host_free(void* p);
/* kernel launches issued by this library since it was loaded */
int ttn_launch_count(unsigned long long* out);
/* FP64 FMA throughput of a device in TFLOP/s (long independent FMA chains) */
int ttn_device_fp64_peak(int device, double* tflops);

/* No counterpart in the reference: it is the one entry point that allocates no device
 * memory, for callers that cannot allocate where they factorise (all their device memory
 * comes from their own pool or arena, or a cudaMalloc/cudaFree device synchronisation
 * is not affordable).  Householder QR (LAPACK zgeqrf/zungqr conventions, the
 * column-by-column cooperative kernel; the sweep's gauge moves use its panel-blocked
 * variant, equal to rounding) of an m x n row-major complex matrix
 * already on `device`: a <- Q (m x n), r <- R (n x n, upper triangular); a and r are
 * device pointers to interleaved complex doubles, 16-byte aligned; stream is a
 * cudaStream_t (NULL: the legacy default stream).  The workspace (about 0.52 MB) is one
 * static device array holding the partials of up to 256 CTAs and 64 columns: n > 64
 * returns TTN_ECAPACITY.  The first call on a device looks the array up (set-up); make
 * it before any stream capture.  All calls share the array, so calls that overlap on
 * the GPU race.  Returns after the stream has finished the QR (TTN_ETIMEOUT if a grid
 * barrier gave up).  The calling thread's current device is the same on return as on
 * entry. */
int ttn_qr_noalloc(int m, int n, double* a, double* r, void* stream, int device);

#ifdef __cplusplus
}
#endif
#endif
