/*
 * gwgb.h — C ABI of the GB300 symmetry-adapted GW engine.
 *
 * The engine replaces the GPU half of SymmetryMBPT's cuGW solver for one GW
 * iteration over the irrep-blocked ("flat block") layout:
 *
 *   P0 contraction -> P~ = (1 - P~0)^-1 P~0 solve -> Sigma contraction -> Dyson,
 *   with the tau <-> i omega sparse-grid (IR) transforms in between.
 *
 * Every entry point takes plain pointers and sizes; complex numbers are
 * interleaved (re, im) doubles, i.e. the memory layout of
 * std::complex<double>.  Every call returns 0 on success or a GWGB_E* code;
 * gwgb_last_error() returns the message of the last failure on the calling
 * thread.  A handle owns one CUDA device context slice (its device buffers,
 * one stream, its CUDA graphs); calls on one handle are serialised by an
 * internal mutex and distinct handles are independent.
 *
 * Host layouts are exactly the reference's host layouts:
 *   G(tau), Sigma(tau):  [nts][ns][flat_ao]      (irreducible k slices)
 *   P0(tau), P~(tau):    [ink][nts][qslice]      (irreducible q slices)
 *   F, S, H:             [ns][flat_ao]
 *   V:                   flat block-sparse, pair k1*nk+k2 slices
 */
#ifndef GWGB_H
#define GWGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GWGB_OK              0
#define GWGB_E_INVALID       1  /* bad argument, inconsistent layout, odd nts */
#define GWGB_E_NOMEM         2  /* device or host allocation failed */
#define GWGB_E_CUDA          3  /* CUDA runtime error */
#define GWGB_E_TIMEOUT       4  /* a bounded device-side wait ran out */
#define GWGB_E_NUMERIC       5  /* singular block in Dyson or W~ solve */
#define GWGB_E_STATE         6  /* call order violated (e.g. solve before upload) */
#define GWGB_E_UNSUPPORTED   7  /* shape beyond the limits of the built kernels */

/* ---- contraction precision -------------------------------------------- */
#define GWGB_PREC_FP64       0  /* complex128 everywhere: the drop-in path */
#define GWGB_PREC_TF32X3     1  /* P0/Sigma on tcgen05 kind::tf32, 3-pass split, FP32 accumulate */
#define GWGB_PREC_BF16X3     2  /* P0/Sigma on tcgen05 kind::f16 (BF16), 3-way split, 6 products, FP32 accumulate */
#define GWGB_PREC_OZAKI      3  /* P0/Sigma on tcgen05 kind::f16 (BF16): four fixed-point slices per operand row
                                   (Ozaki scheme), 10 products, exact FP32 partial sums, float-float accumulation
                                   and intermediates; Sigma error about 1e-9 of the FP64 path */

typedef struct gwgb_handle_s *gwgb_handle;

/* Solver parameters; the subset of params_t the GW solver reads
 * (SymmetryMBPT/include/common/params_t.h:20-74, cugw_solver_block.h:117-142). */
typedef struct gwgb_params {
  int32_t ns;        /* spins, 1 or 2 */
  int32_t nts;       /* tau points including 0 and beta (= ni + 2); must be even */
  int32_t nw;        /* fermionic Matsubara sampling points */
  int32_t nw_b;      /* bosonic Matsubara sampling points */
  double  beta;      /* inverse temperature */
  int32_t precision; /* GWGB_PREC_* */
  int32_t device;    /* CUDA device ordinal */
  int32_t nt_batch;  /* accepted for params_t compatibility; the kernels choose their own tau tiles */
  int32_t flags;     /* reserved, 0 */
  /* Tile-shape settings of the tcgen05 Sigma path, 0 = the built-in choice;
   * mbsymmetry_gb300/autotune.py picks them by timing a workload. */
  int32_t uvt_smem_kb; /* shared memory per U/Sigma CTA (60..227 KB; sets tau per tile and aux rows per chunk) */
  int32_t sw_npk_max;  /* widest W-GEMM column pack (16, 32 or 64 complex columns) */
  int32_t uv_waves;    /* U/Sigma contribution slices per tau, in units of the SM count (1..16; default 8) */
  int32_t uv_simt;     /* 1: all U/Sigma tiles on the FP32 SIMT kernels (the path for AO blocks above 64) */
  /* Sliced path (GWGB_PREC_OZAKI): block GEMMs with at most this many output
   * columns run on the CUDA-core float-float kernel instead of tcgen05
   * (0: the built-in 8; -1: none; at most 1024). */
  int32_t oz_simt_cols;
} gwgb_params;

/* Block layout: the arrays symmetry_utils_t reads from symmetry_info.h5,
 * symmetry_rot.h5 and df_int/meta.h5
 * (SymmetryMBPT/src/common/symmetry_utils.cpp:6-218).  Lists per k point are
 * passed CSR style: entries [ptr[k], ptr[k+1]).  Offsets are derived inside
 * the library with the reference's packing rule (blocks in list order, each
 * b*b row-major; V blocks [q_b][k1_b][k2_b] with q = k2 - k1). */
typedef struct gwgb_layout {
  int32_t nk;                       /* k points in the full BZ */
  int32_t ink;                      /* stored (irreducible) k points */
  const int32_t *irre_list;         /* [ink]  full-BZ index of stored k      (irre_conj_list_) */
  const int32_t *index;             /* [nk]   full-BZ index of the representative (index_) */
  const int32_t *irre_index;        /* [nk]   position of the representative in irre_list */
  const int32_t *conj_index;        /* [nk]   time-reversal partner used for rotation */
  const int32_t *q_ind;             /* [nk*nk] q_ind_(j, q), row-major */
  const int32_t *q_ind2;            /* [nk*nk] q_ind2_(i, j), row-major */
  const int32_t *ao_block_ptr;      /* [nk+1] */
  const int32_t *ao_sizes;          /* AO irrep block sizes per k */
  const int32_t *aux_block_ptr;     /* [nk+1] */
  const int32_t *aux_sizes;         /* aux irrep block sizes per q */
  const int32_t *kpair_block_ptr;   /* [nk*nk+1] */
  const int32_t *tensor_irreps;     /* 3 ints per V block: (iq, ik1, ik2) */
  const int32_t *orep_block_ptr;    /* [nk+1] */
  const int32_t *orep_irreps;       /* 2 ints per block: (block at k, block at irreducible k) */
  const int32_t *auxrep_block_ptr;  /* [nk+1] */
  const int32_t *auxrep_irreps;     /* 2 ints per block */
} gwgb_layout;

/* Per-stage device times of the last solve, milliseconds (CUDA events).
 * Names follow the reference's execution_statistic_t events
 * (SymmetryMBPT/include/solver/cugw_solver_block.h:248-262). */
typedef struct gwgb_stats {
  double rotate_G_ms;     /* "Copy data": iBZ -> BZ rotation of G */
  double p0_ms;           /* "P0_contraction" */
  double pq_ms;           /* "Compute P": tau->Omega, W~ solve, Omega->tau */
  double rotate_P_ms;     /* P~(q_irr) -> P~(q) */
  double sigma_ms;        /* "Sigma_contraction" */
  double dyson_ms;        /* Dyson: tau->omega, block inverses, omega->tau */
  double total_ms;
  double p0_flops;        /* algorithmic FLOPs (8MNK per complex GEMM) of the P0 stage */
  double sigma_flops;     /* algorithmic FLOPs of the Sigma stage */
  double leakage;         /* max|c_{n-1}| / max|c_0| of G after the last Dyson */
  int64_t kernel_launches;/* kernels launched by the last solve/iteration */
  int64_t device_bytes;   /* device memory held by the buffers of all live handles of this process */
  double transform_ms;    /* tau <-> omega transforms of the W~ solve and Dyson that ran */
  double transform_bytes; /* their algorithmic bytes: 16 (n_in + n_out) per column + the matrix */
  double solve_ms;        /* block solves: W~ (inverse + product) and Dyson (inverse) */
  double solve_flops;     /* 16 n^3 per W~ block, 8 n^3 per Dyson block */
  double transform_flops; /* 8 n_in n_out per complex column (FP64: with n ~ 100 the transforms are
                             bound by the FP64 pipe, not by HBM) */
} gwgb_stats;

/* Library version string. */
const char *gwgb_version(void);

/* Message of the last failed call on this thread (never NULL). */
const char *gwgb_last_error(void);

/* Create a handle: validates the layout, builds the (q,k) / (k,q) work lists
 * and allocates the device buffers.  Replaces solver_factory_t::construct_solver
 * with scf_type == cuGW (SymmetryMBPT/include/solver/solver_factory_t.h:34-55)
 * and the cugw_routine_block constructor
 * (SymmetryMBPT/src/cuda/cugw_routines_block.cu:6-44). */
int gwgb_create(const gwgb_params *params, const gwgb_layout *layout, gwgb_handle *out);

/* Release every device buffer of the handle. */
int gwgb_destroy(gwgb_handle h);

/* Select the contraction precision for subsequent solves. Replaces
 * solver_block_t::single_prec_run (SymmetryMBPT/include/solver/solver_block_t.h:48). */
int gwgb_set_precision(gwgb_handle h, int32_t precision);

/* Upload V (flat_V_size complex) into HBM; the host buffer is only read
 * during the call.  Replaces set_shared_Coulomb/read_entire_Coulomb_integrals
 * (SymmetryMBPT/include/solver/cuhf_solver_block.h:43-53, 106-118) and the
 * per-pair reader callback (SymmetryMBPT/include/cuda/cugw_routines_block.h:17-20). */
int gwgb_upload_V(gwgb_handle h, const double *V_flat, int64_t n_complex);

/* Upload the rotation matrices orep / auxrep (flat block form, all nk).
 * Replaces copy_ORep_host_to_device / copy_AuxRep_host_to_device
 * (SymmetryMBPT/src/cuda/cugw_routines_block.cu:214-234). */
int gwgb_set_reps(gwgb_handle h, const double *orep, int64_t n_orep,
                  const double *auxrep, int64_t n_auxrep);

/* IR transform matrices built on the host in FP64 (transformer_t,
 * SymmetryMBPT/src/common/transformer_t.cpp:48-82), row-major complex:
 *   Tnt [nw][nts-2], Ttn [nts][nw], Tnt_BF [nw_b][nts-2], Ttn_FB [nts][nw_b];
 * wsample_fermi [nw] Matsubara indices n (omega_n = (2n+1) pi / beta);
 * tct_first / tct_last: rows 0 and nts-3 of the real Tct matrix (leakage check,
 * SymmetryMBPT/src/scmbpt/sc_type_block.cpp:66-71); may be NULL. */
int gwgb_set_transforms(gwgb_handle h, const double *Tnt, const double *Ttn,
                        const double *Tnt_BF, const double *Ttn_FB,
                        const int64_t *wsample_fermi,
                        const double *tct_first, const double *tct_last);

/* One-electron inputs F, S [ns][flat_ao] (already Bz-shifted and
 * Hermitised as sc_loop_block_t::read_input_data does,
 * SymmetryMBPT/src/scmbpt/sc_loop_block_t.cpp:64-109). */
int gwgb_set_fock(gwgb_handle h, const double *F, const double *S);

/* G(tau) host <-> device, layout [nts][ns][flat_ao].  Replaces
 * copy_G_host_to_device (SymmetryMBPT/src/cuda/cugw_routines_block.cu:100-201);
 * the iBZ -> BZ rotation and the G(-tau) view happen on the device. */
int gwgb_set_G(gwgb_handle h, const double *G_ts_kij);
int gwgb_get_G(gwgb_handle h, double *G_ts_kij);

/* Sigma(tau) host <-> device, layout [nts][ns][flat_ao].  get overwrites the
 * host buffer (the reference's D2H copy adds into a zeroed buffer,
 * SymmetryMBPT/src/cuda/cugw_routines_block.cu:249-274). */
int gwgb_set_sigma(gwgb_handle h, const double *Sigma_ts_kij);
int gwgb_get_sigma(gwgb_handle h, double *Sigma_ts_kij);

/* P0 / P~ host <-> device, layout [ink][nts][qslice]
 * (cugw_solver_block_t::P0_q_t_QP, SymmetryMBPT/include/solver/cugw_solver_block.h:180). */
int gwgb_set_P0(gwgb_handle h, const double *P_q_t_QP);
int gwgb_get_P0(gwgb_handle h, double *P_q_t_QP);

/* P0 only: after the call the P0 buffer holds c/nk * sum for t < nts/2 and
 * zeros above, as cugw_solver_block_t::solve_P0 leaves it
 * (SymmetryMBPT/src/solver/cugw_solver_block.cpp:67-84, 139-190). */
int gwgb_solve_P0(gwgb_handle h);

/* P~ = (1 - P~0)^-1 P~0 from the P0 buffer, in place, all nts.  Replaces
 * cugw_solver_block_t::compute_Pq_from_P0q (cugw_solver_block.cpp:385-439). */
int gwgb_solve_Pq(gwgb_handle h);

/* Sigma from P0 (test hook): mirrors P0 in tau, then the Sigma contraction.
 * Replaces cugw_solver_block_t::solve_sigma (cugw_solver_block.cpp:86-112, 192-252). */
int gwgb_solve_sigma(gwgb_handle h);

/* The Sigma contraction alone, from the handle's G and its P buffer as it is
 * (gwgb_set_P0 or the last gwgb_solve_Pq), without recomputing P0: the Sigma
 * half of cugw_solver_block_t::solve (cugw_solver_block.cpp:192-252).  With
 * P = identity at tau = 0 and G = a density matrix at tau = 0, Sigma(tau = 0)
 * is the Hartree-Fock exchange on the block engine (mbsymmetry_gb300
 * solver.hf_exchange). */
int gwgb_solve_sigma_from_P(gwgb_handle h);

/* Hartree (direct) term of HF from the handle's G at tau = 0 taken as the
 * density matrix rho: J(k)_ij = sum_Q V^Q_ij(k, k) c_Q with
 * c_Q = (f / nk) sum_{k', s} sum_ab V^Q_ab(k', k') rho_s(k')_ba over the full
 * BZ (f = 2 for ns = 1, 1 for ns = 2), for the diagonal AO blocks of the
 * stored k; J: flat_ao complex (spin independent).  With the exchange of
 * gwgb_solve_sigma_from_P this is HF on the block layout (the reference's HF
 * solver is a stub, SymmetryMBPT/include/solver/cuhf_solver_block.h:36-39). */
int gwgb_hf_hartree(gwgb_handle h, double *J);

/* Full GW self-energy: P0 -> P~ -> Sigma.  Replaces
 * cugw_solver_block_t::solve (cugw_solver_block.cpp:34-65, 254-315). */
int gwgb_solve(gwgb_handle h);

/* Dyson: G(tau) from Sigma(tau), F, S at chemical potential mu.  Replaces
 * dyson_sc_block_t::compute_G (SymmetryMBPT/src/scmbpt/sc_type_block.cpp:6-87). */
int gwgb_dyson(gwgb_handle h, double mu);

/* One GW iteration on resident data: solve() then Dyson at mu; captured as
 * one CUDA graph on first use and replayed afterwards. */
int gwgb_iteration(gwgb_handle h, double mu);

/* Per-stage timings and algorithmic FLOPs of the last solve/iteration. */
int gwgb_get_stats(gwgb_handle h, gwgb_stats *out);

/* Block until all work of the handle is done. */
int gwgb_synchronize(gwgb_handle h);

/* ---- per-launch profile of the sliced path (GWGB_PREC_OZAKI) ----
 * With timing on, every GEMM and reduction launch of the P0 and Sigma stages
 * is bracketed by CUDA events (recorded into the iteration's graph); after a
 * solve or iteration gwgb_get_launch_stats returns one entry per launch, in
 * launch order.  Off by default: the events add a few microseconds per launch.
 * Switching it re-captures the iteration graph. */
typedef struct gwgb_launch_stat {
  int32_t stage;    /* 0 Z1 (V G2), 1 Z (G1 Z1), 2 P0 (final), 3 W (P~ V), 4 U (W G2), 5 Sigma (final) */
  int32_t kernel;   /* 0 oz_gemm_kernel (tcgen05), 1 oz_simt_kernel (CUDA cores), 2 reduce_slices_kernel,
                       3 oz_perm_kernel (a chunk's copy of V blocks into a concatenated operand) */
  int32_t tasks;    /* CTA work items (kernels 0, 1) or reduced blocks (kernel 2) */
  int32_t ran;      /* 1 when the launch ran in the last solve / iteration */
  double ms;        /* CUDA-event time of the launch */
  double flops;     /* algorithmic: 8 M N K per complex block GEMM (0 for reductions) */
  double mma_flops; /* kernel 0: BF16 MMA FLOPs issued (128-row tiles, N and K padded to the MMA shape,
                       10 slice products, real embedding); kernel 1: FP32 instructions (48 per complex MAC) */
  double bytes;     /* kernels 2, 3: bytes read + written */
} gwgb_launch_stat;

int gwgb_set_launch_timing(gwgb_handle h, int32_t on);

/* Entries of the last run (at most max); *n = the number of launches. */
int gwgb_get_launch_stats(gwgb_handle h, gwgb_launch_stat *out, int32_t max, int32_t *n);

/* ---- reference-GPU proxy (measurement only, not on the drop-in path) ----
 * Replays the reference's cuBLAS call sequence for the two contractions of one
 * GW iteration on this GPU, for the comparison "reference call sequence vs
 * these kernels" on the same hardware: the G rotation and G(-tau) copies
 * (SymmetryMBPT/src/cuda/cugw_routines_block.cu:164-199), per (q_irr, k) pair
 * the V transposes and the three strided-batched ZGEMMs of P0 per V block and
 * tau batch (cugw_qkpt_block.cu:119-130, 195-284), per (k_irr, q) pair the P~
 * rotation, the V conj-transposes and the three ZGEMMs of Sigma
 * (cugw_qkpt_block.cu:140-192, 288-436), round-robin over nstreams streams
 * (the reference's nqkpt streams), nt_batch tau per batch (its nt_batch).
 * V stays in HBM and the per-pair accumulation locks become per-stream
 * accumulators (both in the reference's favour).  P0 is computed from the
 * handle's G, Sigma from its G and its P~ (the state after gwgb_solve).
 * cuBLAS is loaded when this runs (GWGB_E_UNSUPPORTED if it cannot be). */
typedef struct gwgb_proxy_stats {
  double p0_ms;        /* G set-up + P0 pair loop, CUDA events */
  double sigma_ms;     /* P~ rotation + Sigma pair loop */
  int64_t gemm_calls;  /* cuBLAS ZGEMM_SB calls */
  int64_t other_calls; /* GEAM, SCAL, AXPY, memset and D2D copy calls */
} gwgb_proxy_stats;

int gwgb_refproxy_run(gwgb_handle h, int32_t nt_batch, int32_t nstreams, gwgb_proxy_stats *out);

/* The proxy's P0 ([q_irr][t][qslice], t < nts/2) and Sigma ([t][s][flat_ao]);
 * either pointer may be NULL. */
int gwgb_refproxy_get(gwgb_handle h, double *P0, double *Sigma);

/* ---- self-consistent loop ----------------------------------------------
 * No counterpart in the reference: sc_loop_block_t keeps mu fixed
 * (sc_loop_block_t.h:25), never assigns its energy (:123), does not mix and
 * does not iterate (params_t.cpp:74).  These entry points add, on the device:
 *   N(mu)  = -(2/ns)/nk sum_{s,k} Re Tr[G_k,s(beta) S_k,s]       (electrons)
 *   E_corr = -(1/ns)/nk sum_{s,k} Re sum_{ij} M_ij Tr[Sigma_k,s(tau_i) G_k,s(tau_j)]
 *            (Galitskii-Migdal; M is the caller's interior-tau quadrature of
 *             int_0^beta Sigma(tau) G(beta - tau) dtau)
 *   E_one  = -(1/ns)/nk sum_{s,k} Re Tr[G_k,s(beta) (H_k,s + F_k,s)]  (when H is set)
 * with k summed over the full mesh through the irreducible weights
 * (#k mapped to each stored k), and linear mixing
 *   Sigma <- alpha Sigma_new + (1 - alpha) Sigma_old.                     */

/* Core Hamiltonian H [ns][flat_ao] (complex); enables E_one. */
int gwgb_set_hcore(gwgb_handle h, const double *H);

/* Galitskii-Migdal weights M [(nts-2) x (nts-2)] (real, row-major). */
int gwgb_set_energy_matrix(gwgb_handle h, const double *M, int32_t n);

typedef struct gwgb_mu_search {
  double n_electrons;  /* target N */
  double mu0;          /* first trial */
  double step;         /* first bracket step (> 0); doubled while the root is not bracketed */
  double tol;          /* |N - target| accepted; later evaluations are skipped */
  int32_t max_evals;   /* Dyson evaluations per search (fixed in the graph), 2..64 */
  int32_t pad;
} gwgb_mu_search;

typedef struct gwgb_sc_record {
  double mu;           /* chemical potential used by the iteration's Dyson */
  double n_electrons;  /* N(mu) of the new G */
  double e_corr;       /* Galitskii-Migdal energy of (Sigma, new G) */
  double e_one;        /* one-body energy of the new G (0 without H) */
  double leakage;      /* max |c_last| / max |c_0| of the new G (0 without tct) */
  int32_t mu_evals;    /* Dyson evaluations the search used */
  int32_t precision;   /* GWGB_PREC_* of the iteration's contractions */
} gwgb_sc_record;

/* Dyson with a device-side search for mu (bracketed Illinois regula falsi,
 * at most max_evals Dyson evaluations): the G at the best mu found.  Writes
 * the mu used and N to mu_out / n_out (either may be NULL). */
int gwgb_find_mu(gwgb_handle h, const gwgb_mu_search *ms, double *mu_out, double *n_out);

/* E_corr and E_one of the resident Sigma and G (either pointer may be NULL). */
int gwgb_energy(gwgb_handle h, double *e_corr, double *e_one);

/* niter self-consistent iterations, each one CUDA graph launch with no host
 * synchronisation in between: GW Sigma from G, Sigma mixed with the previous
 * Sigma (alpha), mu search (ms, starting from the previous iteration's mu),
 * Dyson, energies.  The Sigma resident at the call is the first Sigma_old.
 * final_fp64 != 0 runs the last iteration with the FP64 contractions whatever
 * the handle's precision.  One record per iteration goes to out[niter]. */
int gwgb_sc_loop(gwgb_handle h, int32_t niter, double alpha, const gwgb_mu_search *ms, int32_t final_fp64,
                 gwgb_sc_record *out);

/* ---- test hooks (no counterpart in the reference) ----------------------
 * Failure paths exercised without faulting, trapping or hanging a GPU. */

/* Raise one of the handle's device status words as a kernel would
 * (0: singular W~ block, 1: singular Dyson block, 2: tensor-core completion
 * wait ran out).  The next call that reads them (gwgb_synchronize, any solve)
 * returns the mapped error (GWGB_E_NUMERIC / GWGB_E_TIMEOUT) and clears them. */
int gwgb_test_raise_status(gwgb_handle h, int32_t which);

/* Launch a kernel whose bounded wait on an mbarrier that nothing arrives on
 * gives up after `polls` polls (1..10^7) and records that in a device status
 * word; returns GWGB_E_TIMEOUT when the host read the status back, GWGB_OK if
 * the wait did not run out. */
int gwgb_test_wait_timeout(int32_t device, int32_t polls);

/* ---- W~ solve without device allocation -------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they run (a host code whose own pool owns all of HBM, a plugin
 * called where new allocations are forbidden, code that must avoid the
 * implicit synchronisation of cudaMalloc/cudaFree): P~ = (1 - P~0)^-1 P~0 for
 * ONE irreducible q on caller-owned device buffers.  Its work space (the
 * P(i Omega) buffer and the task lists) lives in one static device array of
 * GWGB_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit; the call allocates nothing.  The first call on a device performs the
 * set-up (looks up the array's device address, sets the block-inverse kernels'
 * shared-memory limits).  All calls share the array: calls that overlap on
 * the GPU race, so serialise them.  Every call reads a status word back to
 * the host and synchronises `stream`, so no call (first or later) can be
 * recorded into a CUDA graph.  The host thread's current device is restored
 * before the call returns.
 *   P0_t   device, [nts][qslice] complex: P0(tau) of the q slice, all nts rows
 *          (mirrored, as after gwgb_solve); may alias P_t
 *   P_t    device, [nts][qslice] complex output P~(tau)
 *   Tnt_BF device, [nw_b][nts-2]; Ttn_FB device, [nts][nw_b] (see gwgb_set_transforms)
 *   block_sizes host, [nblocks] aux block sizes of the q (1..64 each)
 *   stream  a cudaStream_t (NULL = legacy default stream)
 * Limits: nblocks <= GWGB_NOALLOC_MAX_BLOCKS and
 *   nw_b*qslice*16 + nw_b*nblocks*32 + 512 <= GWGB_NOALLOC_SCRATCH_BYTES,
 *   otherwise GWGB_E_UNSUPPORTED; a singular block returns GWGB_E_NUMERIC. */
#define GWGB_NOALLOC_SCRATCH_BYTES (8u << 20)
#define GWGB_NOALLOC_MAX_BLOCKS 64
int gwgb_wsolve_noalloc(int32_t device, const double *P0_t, double *P_t, const double *Tnt_BF,
                        const double *Ttn_FB, int32_t nts, int32_t nw_b, const int32_t *block_sizes,
                        int32_t nblocks, void *stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* GWGB_H */
