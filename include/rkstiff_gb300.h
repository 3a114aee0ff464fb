/*
 * rkstiff_gb300 -- C ABI of the GB300 (sm_103a) stepping kernels.
 *
 * The reference (whalenpt/rkstiff) is pure Python and has no FFI; its boundary is the
 * solver-object API.  This header is what a binding of that API binds: every entry
 * point below replaces one reference routine, cited as file:line within the rkstiff
 * project.  Plain C types only; every pointer marked [device] is a CUDA device pointer
 * on the current device; `stream` is a cudaStream_t passed as void*.
 *
 * Return convention: 0 on success, a negative RK_E* code on an API/CUDA error
 * (rk_last_error() gives the message).  Per-instance outcomes of a run are written to
 * rk_inst_state.status (RK_ST_*), never returned.
 */
#ifndef RKSTIFF_GB300_H
#define RKSTIFF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RK_ABI_VERSION 2

/* twiddle table length: supports complex FFTs and real grids up to this many points */
#define RK_TW_N 8192

/* methods: the seven solver classes of the reference */
enum {
  RK_IF34 = 0,   /* rkstiff/if34.py:260   (adaptive, q=4, FSAL)                 */
  RK_ETD35 = 1,  /* rkstiff/etd35.py:723  (adaptive, q=4, N1 recomputed)        */
  RK_ETD34 = 2,  /* rkstiff/etd34.py:439  (adaptive, q=4, FSAL)                 */
  RK_IF45DP = 3, /* rkstiff/if45dp.py:8   (adaptive, q=5, FSAL, diagonal only)  */
  RK_ETD4 = 4,   /* rkstiff/etd4.py:311   (constant step)                       */
  RK_ETD5 = 5,   /* rkstiff/etd5.py       (constant step)                       */
  RK_IF4 = 6     /* rkstiff/if4.py:202    (constant step)                       */
};

enum { RK_FP64 = 0, RK_FP32 = 1 };

/* built-in fused nonlinearities (the nl_func closures of rkstiff/models.py and README) */
enum {
  RK_NL_NONE = 0, /* N(u) = 0 (pure linear problem)                                     */
  RK_NL_UUX = 1,  /* N(u) = c rfft(irfft(u) * irfft(i kx u)) on a real grid:
                     KS (README.md:94-97, c=-1), Burgers (models.py:189-192, c=-1),
                     KdV (models.py:140-143, c=-6)                                    */
  RK_NL_NLS = 2,  /* N(u) = fft(i c |v|^2 v), v = ifft(u), on a complex grid (c=1)    */
  RK_NL_ALLEN_CAHN = 3 /* dense path: N(w) = x - (w + x)^3 on the interior Chebyshev points
                          x (models.py:242-244, the lifted form u = w + x)            */
};

enum { RK_RUN_EVOLVE = 0, RK_RUN_STEP = 1 };

/* per-instance outcome codes */
enum {
  RK_ST_RUNNING = -1, /* not started / resumable                                      */
  RK_ST_DONE = 0,     /* reached tf                                                   */
  RK_ST_MAX_LOOPS = 1,/* more than 50 retries in one step (solveras.py:399-406)        */
  RK_ST_MIN_STEP = 2, /* h < minh after a reject (solveras.py:407-410)                 */
  RK_ST_ITER_CAP = 4, /* the launch's accepted-step bound was hit (resumable)          */
  RK_ST_SNAP_FULL = 5,/* the snapshot buffer filled (resumable)                        */
  RK_ST_STEP_DONE = 6,/* RK_RUN_STEP: one accepted step was taken                      */
  RK_ST_BAD_SIZE = 7, /* the instance's n[i] is not a power of two in [4, n_max] (or not the
                         size of its class); the instance was not stepped               */
  RK_ST_WAIT_TIMEOUT = 8 /* rk_dense_eig_evolve: a bounded device wait ran out; the
                            instances of that CTA stopped where they were             */
};

/* error codes */
enum {
  RK_OK = 0,
  RK_E_ARG = -1,
  RK_E_CUDA = -2,
  RK_E_UNSUPPORTED = -3,
  RK_E_SIZE = -4
};

/* adaptive controller settings: SolverConfig, rkstiff/solveras.py:27-169 */
typedef struct rk_controller {
  double epsilon, incr_f, decr_f, safety_f, adapt_cutoff, minh;
} rk_controller;

/* psi-function settings: ETDConfig, rkstiff/etd.py:46-131.  contour_at_zero = 1 evaluates
 * every mode's psi values as the reference's non-diagonal strategies do for a matrix
 * operator: the mean over the contour nodes r_j (radius contour_radius, centred at 0) of
 * r_j psi(r_j) / (r_j - c z) for each scaled argument c z (etd35.py:602-658,
 * etd34.py:366-383, etd4.py:245-262, etd5.py); applied to the eigenvalues of a
 * diagonalizable lin_op this reproduces the reference's psi-matrices
 * S diag(.) S^-1 (rk_coeffs; rk_evolve refuses it).  0: the diagonal rule (direct formula,
 * contour around z below modecutoff). */
typedef struct rk_etd_config {
  double modecutoff;
  double contour_radius;
  int32_t contour_points;
  int32_t contour_at_zero;
} rk_etd_config;

/* per-instance controller state (the attributes rkstiff keeps on the solver object:
 * __tc/__tf and _accept of solveras.py:281-282, _h_coeff of etd.py:226) plus counters */
typedef struct rk_inst_state {
  double t;          /* current time                                               */
  double tf;         /* final time                                                 */
  double h;          /* step size of the next attempt                              */
  double h_coeff;    /* step size the cached coefficients were built for (NaN: none)*/
  double h_used;     /* step size of the last accepted step                        */
  double h_suggest;  /* suggestion after the last accepted step                    */
  double s_last;     /* controller factor s of the last attempt                    */
  double reserved_d;
  int32_t status;    /* RK_ST_*                                                    */
  int32_t accept;    /* last attempt accepted (reference _accept)                  */
  int32_t snap_count;/* snapshots written in the current launch                     */
  int32_t reserved_i;/* diagonal kernels: 1 once a launch saved the low words of a double-float
                        state (FP32 ETD35 / ETD5); a fresh state has 0 */
  int64_t steps, attempts, rejects, nl_evals, coeff_updates, reserved_l;
} rk_inst_state;

/* One batched run over independent diagonal-operator instances.
 * Modes of instance i live at [mode_off[i], mode_off[i] + m_i) of lin_op / kx / u,
 * m_i = n_i/2 + 1 for RK_NL_UUX (real grid), n_i otherwise.  Every n[i] must be a power of
 * two with 4 <= n[i] <= n_max (and, with classes, equal to its class's class_n): the kernels
 * size their shared-memory transforms and, in rk_evolve_noalloc, the scratch slabs from
 * n_max.  An instance that breaks this is not stepped and ends with RK_ST_BAD_SIZE. */
typedef struct rk_batch {
  int32_t method;        /* RK_IF34 ... RK_IF4                                        */
  int32_t precision;     /* RK_FP64 / RK_FP32                                         */
  int32_t coef_complex;  /* 0: the operator is real, coefficients stored real         */
  int32_t nl_kind;       /* RK_NL_*                                                   */
  double nl_coef;        /* constant c of the nonlinearity                            */
  int64_t n_inst;
  int32_t n_max;           /* largest n over the instances (sizes the FFT buffers)    */
  int32_t reserved0;
  const int32_t* n;        /* [device] grid points per instance (power of two)       */
  const int64_t* mode_off; /* [device] first mode of each instance                   */
  const int32_t* order;    /* [device] processing order (NULL: 0..n_inst-1)           */
  const double* lin_op;    /* [device] complex128 interleaved operator per mode       */
  const double* kx;        /* [device] wavenumber per mode (RK_NL_UUX)               */
  void* u;                 /* [device] complex64/complex128 state, in/out             */
  rk_inst_state* state;    /* [device] per-instance state, in/out                     */
  void* slab;              /* [device] scratch: coefficient, stage and work arrays    */
  const int64_t* slab_off; /* [device] byte offset of each instance's scratch         */
  const void* twiddle;     /* [device] RK_TW_N twiddles exp(-2 pi i k/RK_TW_N), in T  */
  int32_t* queue;          /* [device] one int32 work counter, zeroed by rk_evolve    */
  int32_t store_freq;      /* snapshot every store_freq accepted steps; 0 = never     */
  int32_t snap_cap;        /* snapshots per instance per launch                       */
  void* snap_u;            /* [device] snap_cap*m_i states per instance at snap_cap*mode_off */
  double* snap_t;          /* [device] snap_cap times per instance                     */
  int64_t max_steps;       /* accepted steps per instance per launch (safety bound)    */
  int32_t run_mode;        /* RK_RUN_EVOLVE / RK_RUN_STEP                              */
  int32_t threads;         /* threads per instance group: 32, 64, 128 or 256 (0: auto)  */
  rk_controller ctl;
  rk_etd_config etd;
  /* Optional split of `order` into classes of equal grid size, each launched as its own
   * kernel on a stream forked from `stream` (joined before rk_evolve returns to the
   * stream's order), sized for its n.  n_classes = 0: one launch over all instances,
   * and `queue` needs one counter; otherwise n_classes counters. */
  int32_t n_classes;
  int32_t placement;            /* RK_PLACE_* for every class (RK_PLACE_AUTO: per class)  */
  const int32_t* class_n;       /* [host] grid size of each class                         */
  const int64_t* class_start;   /* [host] n_classes+1 offsets into `order`                */
  const int32_t* class_threads; /* [host] threads per instance per class (NULL: auto)     */
  const int32_t* class_place;   /* [host] placement per class (NULL: `placement`)         */
  const int32_t* class_groups;  /* [host] instance groups per block per class, threads x groups <= 512 (NULL: auto) */
  /* Optional per-attempt log: instance i writes RK_LOG_FIELDS floats per attempt at
   * attempt_log + (i * log_cap + k) * RK_LOG_FIELDS for its attempts k < log_cap
   * (counted over the whole evolve).  NULL: no log. */
  float* attempt_log;
  int32_t log_cap;
  /* Learned step-size controller (adaptive methods): after an accepted attempt the next
   * step is h * exp(y) / mlp_target, y the output of the MLP in `mlp` (RK_MLP_* layout,
   * bf16 weights), the factor clamped to [0.5, 4]; a rejected attempt keeps the
   * reference's rule.  NULL: the reference's controller (solveras.py:508-554). */
  float mlp_target;
  const void* mlp;
  /* Optional snapshot stream (replaces the list append of solveras.py:643-646 for long
   * runs): with ring_data set, each snapshot (every store_freq accepted steps) goes to the
   * next slot of a ring in mapped, pinned host memory (rk_ring_create) while the launch
   * runs, instead of snap_u / snap_t; the host drains it with rk_ring_take.  A writer claims
   * slot k with an atomic add on *ring_head and waits (bounded by ring_timeout_ms) until the
   * host has taken slot k - ring_slots (*ring_tail > k - ring_slots); if that wait runs out
   * the instance pauses with RK_ST_SNAP_FULL and slot k is never completed (the host sees
   * the stream as overrun).  Slot layout: RK_RING_HEADER bytes {int64 ready (k + 1 once
   * the slot is complete), int64 instance, double t, int64 step} then m_i complex states. */
  void* ring_data;           /* [mapped host] ring_slots * ring_slot_bytes, or NULL     */
  int64_t ring_slot_bytes;   /* >= RK_RING_HEADER + m_max * sizeof(complex T)           */
  int32_t ring_slots;
  int32_t ring_timeout_ms;
  unsigned long long* ring_head; /* [mapped host] slots claimed by the kernels            */
  const int64_t* ring_tail;      /* [mapped host] slots taken by the host                 */
  /* Coefficient cache: 0 or 1 keeps one coefficient block per instance, rebuilt whenever h
   * changes (the reference's exact-compare cache, etd35.py:851); 2..RK_COEF_BLOCKS_MAX keeps
   * that many blocks keyed by their exact h (adaptive methods; the slab must then hold
   * rk_slab_bytes_blocks(..., coef_blocks) bytes per instance; placement RK_PLACE_SMEM_ALL
   * keeps one block).  ladder = 1 (adaptive methods with the learned controller only) puts
   * every step size proposed after the first on the geometric ladder h0 * 2^(k/16) (h0: the
   * instance's first step size): the nearest rung after an accepted attempt, the rung below
   * after a rejection, so a cached block serves every return to a rung. */
  int32_t coef_blocks;
  int32_t ladder;
} rk_batch;

#define RK_COEF_BLOCKS_MAX 4

#define RK_RING_HEADER 32

/* Snapshot ring in mapped, pinned host memory (cudaHostAlloc with cudaHostAllocMapped):
 * rk_ring_create sets r->data / head / tail to device-visible pointers of `slots` slots of
 * `slot_bytes` bytes, zeroed.  rk_ring_take copies slot k (the k-th snapshot written since
 * creation, k counted from 0) to dst (at most `bytes` bytes) and returns 1 if it is
 * complete, 0 if it is not yet; taking it frees the slot for the writer that claims slot
 * k + slots.  Slots must be taken in order.  (No counterpart in the reference: it appends
 * each snapshot to the solver's Python lists, solveras.py:643-646.) */
typedef struct rk_ring {
  void* data;
  unsigned long long* head;
  int64_t* tail;
  int64_t slot_bytes;
  int32_t slots;
  int32_t reserved;
} rk_ring;
int rk_ring_create(int64_t slots, int64_t slot_bytes, rk_ring* r);
int rk_ring_take(rk_ring* r, int64_t k, void* dst, int64_t bytes);
int rk_ring_reset(rk_ring* r);
int rk_ring_destroy(rk_ring* r);

/* per-attempt log record: t, h, s (inf/NaN stored as 1e30 / -1), accepted (0/1), fraction
 * of |unew|^2 in the top quarter of the modes, rejects so far in the step, grid n, method */
#define RK_LOG_FIELDS 8

/* learned controller: MLP with RK_MLP_IN inputs, two tanh layers of RK_MLP_H units and one
 * linear output.  Training parameters (FP32, flat): W1[H][IN], b1[H], W2[H][H], b2[H],
 * w3[H], b3 -- RK_MLP_NPARAM floats.  Inference buffer (rk_mlp_pack): float mu[IN],
 * inv_sd[IN], b1[H], b2[H], b3, pad[3], then bf16 W1[H][IN], W2 transposed ([k][j] holds
 * W2[j][k], so that consecutive units read consecutive weights), w3[H]. */
#define RK_MLP_IN 8
#define RK_MLP_H 64
#define RK_MLP_NPARAM (RK_MLP_H * RK_MLP_IN + RK_MLP_H + RK_MLP_H * RK_MLP_H + RK_MLP_H + RK_MLP_H + 1)
#define RK_MLP_PACK_BYTES ((2 * RK_MLP_IN + 2 * RK_MLP_H + 4) * 4 + (RK_MLP_H * RK_MLP_IN + RK_MLP_H * RK_MLP_H + RK_MLP_H) * 2)

/* where an instance's scratch arrays live during a launch */
enum {
  RK_PLACE_AUTO = -1,
  RK_PLACE_GLOBAL = 0,     /* all arrays in the global scratch slab                       */
  RK_PLACE_SMEM_STATE = 1, /* u, unew and stage arrays in shared memory, coefficients global */
  RK_PLACE_SMEM_ALL = 2,   /* all arrays in shared memory (coefficients rebuilt per launch) */
  RK_PLACE_SMEM_U = 3      /* u and the new-state array in shared memory, the other stage
                              arrays and the coefficients in the global slab (compile-time
                              ETD35 kernels, n = 256 .. 2048, only)                          */
};

/* ABI version and last error message (thread-local). */
int rk_abi_version(void);
const char* rk_last_error(void);

/* Fill twiddle tables exp(-2 pi i k/RK_TW_N), k < RK_TW_N, in FP64 (tw64, complex128)
 * and rounded to FP32 (tw32, complex64).  Either pointer may be NULL. [device] */
int rk_fill_twiddles(void* tw64, void* tw32, void* stream);

/* Bytes of per-instance scratch rk_evolve needs for an instance with m modes.
 * Replaces the coefficient / stage arrays the reference allocates per solver object
 * (e.g. rkstiff/etd35.py:129-155).  FP32 ETD35 / ETD5 also hold the low FP32 words of a
 * double-float state (u and the new state) and of e^z (one more array per coefficient block). */
int64_t rk_slab_bytes(int32_t method, int32_t precision, int32_t coef_complex, int64_t m);
/* The same with `blocks` coefficient blocks (rk_batch.coef_blocks, 1..RK_COEF_BLOCKS_MAX). */
int64_t rk_slab_bytes_blocks(int32_t method, int32_t precision, int32_t coef_complex, int64_t m, int32_t blocks);

/* Coefficient arrays of `method` at step h for a diagonal operator, FP64 math stored in
 * `precision`: the diagonal update_coeffs routines rkstiff/etd35.py:169-288,
 * etd34.py:96-149, etd4.py:87-139, etd5.py:115-203, if34.py:81-93, if4.py:72-83,
 * if45dp.py:183-238.  lin_op: m complex128 [device]; out: rk_num_coeffs(method) arrays of
 * m entries each (real or complex T per coef_complex), array c at out + c*m. */
int rk_num_coeffs(int32_t method);
int rk_coeffs(int32_t method, int32_t precision, int32_t coef_complex, int64_t m, const double* lin_op,
              double h, const rk_etd_config* etd, void* out, void* stream);

/* Run (or resume) the adaptive or constant-step evolve loop of every instance on the
 * device: BaseSolverAS.evolve/step (rkstiff/solveras.py:336-650) with _compute_s,
 * _reject_step_size and _accept_step_size, or BaseSolverCS.evolve/step
 * (rkstiff/solvercs.py:163-279), each attempt running the method's stage program
 * (_update_stages) with the built-in nonlinearity fused between in-shared-memory FFTs. */
int rk_evolve(const rk_batch* b, void* stream);

/* Size of the device scratch array rk_evolve_noalloc places its scratch in: 8 MiB, held by
 * every GPU that loads the library until the process exits. */
#define RK_NOALLOC_SCRATCH_BYTES (8u << 20)

/* No counterpart in the reference.  rk_evolve for callers that cannot allocate device
 * memory -- code running inside another component's CUDA stream capture, plugins whose
 * host application owns every device allocation, hosts that forbid allocation after
 * start-up.  Same batch and results as rk_evolve (every n[i] <= n_max, as there), but the
 * batch's `slab`, `slab_off` and
 * `queue` fields are ignored: that scratch is carved from one library-owned device array of
 * RK_NOALLOC_SCRATCH_BYTES (uniform slabs sized for n_max, the offset table and the queue
 * counters), and all instances run as one launch of the runtime-size kernel (no per-size
 * class split, so no side streams are created).  Batches that need more scratch are
 * rejected with RK_E_SIZE before anything is launched, as are batches that fail rk_evolve's
 * argument checks.  The call allocates nothing (no cudaMalloc/cudaFree, no stream or
 * event creation).  The first call on a device looks up the array's device address with
 * cudaGetSymbolAddress, so make that first call before any stream capture; the address is
 * looked up again only when the device's context changed (after cudaDeviceReset, say), so
 * do not reset the device between a capture and the graph's replays.  Every call
 * shares the array and it keeps the previous call's contents: the call resets each
 * instance's cached-coefficient key (state[i].h_coeff = NaN) and the queue counters itself,
 * and calls whose work overlaps on the GPU (other streams, other host threads) race on it. */
int rk_evolve_noalloc(const rk_batch* b, void* stream);

/* Stepping with a user-supplied nonlinearity.  The reference accepts any callable nl_func
 * (solver.py:104-115); this build evaluates such a callable on the device between two
 * kernels of its own:
 *   rk_combine: out[j] = sum_i w_i * coef_i[j] * v_i[j] (coef_i NULL: w_i * v_i[j]) for 1..8
 *               terms - the stage combinations of the _update_stages methods
 *               (etd35.py:320-345, etd34.py:182-190, if34.py:120-130, if45dp.py:140-179,
 *               etd4.py:167-174, etd5.py:236-260, if4.py:112-121) as one pass; vectors
 *               complex (complex128 / complex64 per precision), coefficients real or
 *               complex per coef_complex in the same precision
 *   rk_error_s: *s_out = safety (eps |u[mask]| / |err[mask]|)^(1/q), the mask and norms of
 *               solveras.py:412-455, in FP64 on the device
 *   rk_cgemv:   y = M x, M a dense n x n complex matrix (row-major) in the precision's
 *               complex type, y not aliasing x: the basis changes S v and S^-1 N of a dense
 *               lin_op stepped in its eigenbasis (the S.dot / Sinv.dot of the diagonalized
 *               strategies, etd35.py:348-495, etd34.py:194-304, if34.py:137-199)
 * All pointers [device] except terms (host array) and ctl (host). */
typedef struct rk_term {
  const void* coef;
  const void* v;
  double w;
} rk_term;
int rk_combine(int32_t precision, int32_t coef_complex, int64_t m, const rk_term* terms, int32_t nterms, void* out,
               void* stream);
int rk_error_s(int32_t precision, int64_t m, const void* unew, const void* err, const rk_controller* ctl, int32_t q,
               double* s_out, void* stream);
int rk_cgemv(int32_t precision, int64_t n, const void* M, const void* x, void* y, void* stream);

/* Learned step-size controller (no counterpart in the reference).  Training kernels on a
 * batch of `batch` samples X[batch][RK_MLP_IN] with targets T[batch], FP32:
 *   rk_mlp_forward: Y[batch] = MLP(params; X)
 *   rk_mlp_grad:    grad += d/dparams of sum_i (Y_i - T_i)^2 / norm over this batch
 *                   (caller zeroes grad), *loss += sum_i (Y_i - T_i)^2 / norm
 *   rk_mlp_adam:    one Adam update of params (m, v moments, step >= 1)
 *   rk_mlp_pack:    inference buffer (RK_MLP_PACK_BYTES) from params and the feature
 *                   normalisation mu / sd (RK_MLP_IN each)
 * All pointers [device]. */
int rk_mlp_forward(const float* params, const float* X, int64_t batch, float* Y, void* stream);
int rk_mlp_grad(const float* params, const float* X, const float* T, int64_t batch, float norm, float* grad,
                float* loss, void* stream);
int rk_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t step, float lr, float beta1,
                float beta2, float eps, void* stream);
int rk_mlp_pack(const float* params, const float* mu, const float* sd, void* out, void* stream);

/* Dense (non-diagonal) lin_op path: ETD35 for a batch of n_inst instances sharing one
 * operator lin_op (n x n, n <= RK_DENSE_NMAX) with real eigenvalues, lin_op = S diag(eig)
 * S^-1.  Replaces rkstiff/etd35.py:_Etd35NonDiagonal (etd35.py:498-720) for the
 * Allen-Cahn Chebyshev operator of models.py:202-247.  The coefficient matrices (the
 * psi-matrices of etd35.py:602-658) are formed in FP64 on the device whenever h changes,
 * as S diag(c(h eig)) S^-1 with the diagonal ETD35 coefficient functions (the arithmetic of
 * the reference's diagonalized form, etd35.py:348-495); the stages run as 3xTF32 tensor-core
 * GEMMs with FP32 accumulation, one K-concatenated GEMM per stage.
 * The batch steps in lockstep: one h for every instance, an attempt is accepted when every
 * instance passes the reference's error test (the smallest s of the batch decides), so a
 * batch of one instance follows the reference's controller exactly. */
#define RK_DENSE_NMAX 128
#define RK_DENSE_TILE 64 /* instances per CTA */

typedef struct rk_dense_state {
  double t, tf, h, h_coeff, h_suggest, s_last; /* h_coeff: h of the current matrices (NaN: none) */
  int32_t status;                              /* RK_ST_*                                        */
  int32_t cur;                                 /* internal: current state buffer                 */
  int32_t numloops, accept, need_matrix, error; /* error != 0: a device wait timed out            */
  int32_t n1_fresh, reserved_i;                /* internal: N1 is re-evaluated this attempt      */
  int64_t steps, attempts, rejects, nl_evals, coeff_updates, reserved;
} rk_dense_state; /* 128 bytes */

typedef struct rk_dense_batch {
  int32_t method;        /* RK_ETD35                                                      */
  int32_t n;             /* vector length, 1..RK_DENSE_NMAX                               */
  int64_t n_inst;        /* instances                                                     */
  int32_t nl_kind;       /* RK_NL_ALLEN_CAHN                                              */
  int32_t err_eigen;     /* 0: error vector in physical space (etd35.py:719, the
                            non-diagonal form); 1: in the eigenbasis, S^-1 applied, as the
                            diagonalized form returns it (etd35.py:495) - the mask still
                            comes from the physical state                                  */
  const double* eig;     /* [device] n real eigenvalues of lin_op                        */
  const double* S;       /* [device] n x n eigenvectors, row-major                       */
  const double* Sinv;    /* [device] n x n inverse of S, row-major                       */
  const double* shift;   /* [device] n points x of the nonlinearity                      */
  float* u;              /* [device] n_inst x n states, instance-major; in/out            */
  void* work;            /* [device] rk_dense_work_bytes(n_inst) bytes, 1024-byte aligned */
  rk_dense_state* state; /* [device] one record; the caller sets t, tf, h, h_coeff = NaN,
                            status = RK_ST_RUNNING, cur = 0 and zero counters before the
                            first call                                                   */
  rk_controller ctl;
  rk_etd_config etd;
  int64_t max_attempts;  /* attempts this call may run before returning                   */
} rk_dense_batch;

int64_t rk_dense_work_bytes(int64_t n_inst);
/* Runs attempts until the state leaves RK_ST_RUNNING or max_attempts attempts ran; returns
 * after the stream has completed them (u holds the current states). */
int rk_dense_evolve(const rk_dense_batch* b, void* stream);
/* Dense lin_op path with a per-instance controller: every instance follows the reference's
 * accept/reject rule with its own h (the rule of solveras.py:457-554 per instance, as a
 * loop of single-instance solvers would), stepped in the eigenbasis of lin_op = S diag(eig)
 * S^-1 as the reference's diagonalized ETD35 / ETD34 / IF34 do (etd35.py:348-495,
 * etd34.py:274-304, if34.py:164-196; ETD34 and IF34 carry N(unew) into the next attempt,
 * first same as last): stage combinations
 * elementwise with per-instance diagonal coefficients (rebuilt for an instance when its h
 * changes), the basis changes S k and S^-1 N(S k) as 3xTF32 tensor-core GEMMs, one
 * persistent launch per call.  Same operator limits as rk_dense_evolve (real spectrum,
 * n <= RK_DENSE_NMAX, the Allen-Cahn nonlinearity).  The error vector is formed in
 * physical space (err_eigen = 0, the non-diagonal form etd35.py:719) or in the eigenbasis
 * (err_eigen = 1, etd35.py:495); the mask comes from the physical state either way.  An
 * FP32 error vector that is exactly zero while |u| > 0 is accepted with s = 4 (below FP32
 * resolution; the reference's x/0 = inf would reject it). */
typedef struct rk_dense_eig_batch {
  int32_t method;        /* RK_ETD35, RK_ETD34 or RK_IF34                                 */
  int32_t n;             /* vector length, 1..RK_DENSE_NMAX                               */
  int64_t n_inst;        /* instances                                                     */
  int32_t nl_kind;       /* RK_NL_ALLEN_CAHN                                              */
  int32_t err_eigen;     /* 0: physical error vector; 1: eigenbasis error vector          */
  const double* eig;     /* [device] n real eigenvalues of lin_op.  err_eigen = 0: any
                            order gives the same results, descending order balances the
                            coefficient rebuilds; err_eigen = 1: the order decides which
                            components the mask keeps (numpy.linalg.eig's order is the
                            reference's)                                                  */
  const double* S;       /* [device] n x n eigenvectors, row-major                       */
  const double* Sinv;    /* [device] n x n inverse of S, row-major                       */
  const double* shift;   /* [device] n points x of the nonlinearity                      */
  float* u;              /* [device] n_inst x n physical states, instance-major: read when
                            first = 1, written by every call                              */
  void* work;            /* [device] rk_dense_eig_work_bytes(n_inst) bytes, 1024-byte
                            aligned; holds the eigenbasis state between calls            */
  rk_inst_state* state;  /* [device] n_inst records: t, tf, h, h_coeff = NaN, status =
                            RK_ST_RUNNING, zero counters and reserved_i (attempts since the
                            last accepted step) before the first call                    */
  rk_controller ctl;
  rk_etd_config etd;
  int32_t first;         /* 1: start from u (and set up the work buffer); 0: continue      */
  int32_t max_attempts;  /* attempts each running instance may make in this call          */
} rk_dense_eig_batch;
int64_t rk_dense_eig_work_bytes(int64_t n_inst);
/* Runs until every instance has left RK_ST_RUNNING or made max_attempts attempts; returns
 * after the stream has completed them.  If a bounded device wait ran out, the instances of
 * that CTA end with status RK_ST_WAIT_TIMEOUT (the call itself still returns 0). */
int rk_dense_eig_evolve(const rk_dense_eig_batch* b, void* stream);

/* The 3xTF32 tensor-core product of the dense path on its own (no counterpart in the
 * reference; a check of the GEMM): D[N][128] = B[N][K] * A[128][K]^T, FP32, K a multiple of
 * 32, N a multiple of RK_DENSE_TILE; work holds rk_tf32x3_work_bytes(K, N) bytes. */
int64_t rk_tf32x3_work_bytes(int64_t K, int64_t N);
int rk_tf32x3_gemm(const float* A, const float* B, float* D, int64_t K, int64_t N, void* work, void* stream);

/* Device grids and spectral derivatives (set-up helpers, so that a problem's operators and
 * initial data can be built without leaving the GPU).  FP64, all arrays [device].
 *   rk_fourier_grid: x[n] = a + j*delta, delta = (a + dx) - a, and kx = 2 pi k / (n dx) with
 *       k the rfft (real_grid = 1, n/2 + 1 entries) or fft (n entries) frequency integers:
 *       construct_x_kx_rfft / construct_x_kx_fft, rkstiff/grids.py:40-85 / 88-131 (the
 *       caller passes dx = (b - a)/n, as the reference computes it); bitwise NumPy's values.
 *       Either output may be NULL.
 *   rk_cheb_grid: the n + 1 Chebyshev extreme points on [a, b] and (D not NULL) the
 *       (n+1) x (n+1) row-major first-derivative matrix: construct_x_cheb /
 *       construct_x_dx_cheb, rkstiff/grids.py:134-219.
 *   rk_dx_fourier: `rows` rows of n points (2 <= n <= 4096; powers of two by FFT, other
 *       n by direct DFT over the n roots of unity): the order-th
 *       derivative irfft((i kx)^order rfft(u)) of real rows (real_grid = 1, u and out
 *       float64, kx n/2 + 1 entries; dx_rfft, rkstiff/derivatives.py:47-124) or
 *       ifft((i kx)^order fft(u)) of complex rows (real_grid = 0, complex128, kx n entries;
 *       dx_fft, rkstiff/derivatives.py:126-180).  twiddle64: the RK_TW_N FP64 table of
 *       rk_fill_twiddles.
 *   rk_dx_cheb: out = D^order u, D n x n, u n x cols (row-major, cols = 1 for a vector):
 *       dx_cheb, rkstiff/derivatives.py:182-253 (D^order formed first by repeated products,
 *       as numpy.linalg.matrix_power; work holds rk_dx_cheb_work_bytes(n) bytes when
 *       order > 1). */
int rk_fourier_grid(int32_t real_grid, int64_t n, double a, double dx, double* x, double* kx, void* stream);
int rk_cheb_grid(int64_t n, double a, double b, double* x, double* D, void* stream);
int rk_dx_fourier(int32_t real_grid, int32_t order, int64_t n, int64_t rows, const double* kx, const void* u,
                  void* out, const void* twiddle64, void* stream);
int64_t rk_dx_cheb_work_bytes(int64_t n);
int rk_dx_cheb(int32_t order, int64_t n, int64_t cols, const double* D, const double* u, double* out, void* work,
               void* stream);

/* Multi-dimensional NLS nonlinearities of the reference's NLS demo (demos/nls.ipynb cells
 * 6-29, which evaluate them with numpy.fft and the Hankel matrix product of
 * rkstiff/transforms.py:178-240) on the library's own kernels.  [device] arrays, complex in
 * the precision's type (complex128 / complex64).
 *   rk_nls_lines: along each of `lines` lines of n points (a power of two <= RK_TW_N; FP64 <=
 *       4096), line l's point j at in[l * line_stride + j * elem_stride]: mode 0 the inverse
 *       FFT (scaled by 1/n, numpy.fft.ifft), 1 the forward FFT, 2 the NLS step
 *       fft(i gamma |v|^2 v) with v = ifft(x) -- one launch, the line held in shared memory.
 *       n = 1 with mode 2 is the product i gamma |x|^2 x over `lines` contiguous points.  out
 *       may alias in.  twiddle: the RK_TW_N table of rk_fill_twiddles in the precision.
 *   rk_dht: the discrete Hankel transform over the radial axis: out = (Y in) * scale
 *       (divide = 0, ht) or (Y in) / scale (divide = 1, iht) for Y the real n x n matrix
 *       (row-major, in the precision's real type) and in / out n x w real, row-major (a
 *       complex array of c columns is w = 2c real columns); out must not alias in. */
int rk_nls_lines(int32_t precision, int32_t mode, int64_t n, int64_t lines, int64_t elem_stride, int64_t line_stride,
                 double gamma, const void* in, void* out, const void* twiddle, void* stream);
int rk_dht(int32_t precision, int32_t divide, int64_t n, int64_t w, const void* Y, double scale, const void* in,
           void* out, void* stream);

/* Measurement utility (no counterpart in the reference): `blocks` x `threads` threads
 * each run 8 independent FP32 FMA chains of `iters` steps and write one float to
 * out[blocks*threads] [device].  FLOPs = 16 * blocks * threads * iters; timing it gives the
 * FP32 CUDA-core peak the spectral kernels are measured against. */
int rk_probe_fp32(float* out, int32_t blocks, int32_t threads, int32_t iters, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RKSTIFF_GB300_H */
