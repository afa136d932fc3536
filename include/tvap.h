/*
 * tvap.h -- C ABI of the GB300 (sm_103a) PNVAP hot path.
 *
 * Drop-in for the three Fortran call sites of TAURUS_vap's gradient loop:
 *
 *   call calculate_fields(rhoLR,kappaLR,kappaRL,gammaLR,hspLR,deltaLR,deltaRL,ndim)
 *        src/module_fields.f90:99-105           -> tvap_calculate_fields
 *   call project_wavefunction(0,iprint,Mphip,Mphin,ndim)
 *        src/module_projection.f90:201-203      -> tvap_project
 *   call calculate_gradient(ndim)
 *        src/module_gradient.f90:79-81          -> tvap_calculate_gradient
 *
 * plus the Thouless evolution used by adjust_constraints
 * (cholesky_factorization + evolve_wavefunction,
 * src/module_constraints.f90:497-590 -> tvap_evolve) and the adjoint of the
 * projected energy with respect to the Thouless matrix (tvap_energy_adjoint,
 * no counterpart in the reference).
 *
 * Conventions
 *   - all matrices are column-major (Fortran order); complex(r64) arguments
 *     are arrays of interleaved (re, im) doubles, exactly the memory layout of
 *     a Fortran complex(r64) array;
 *   - pointers may be host or device memory; the library detects which;
 *   - the module globals the Fortran routines read implicitly (HOsp_2mj,
 *     HOsp_tr, HOsp_l, hamil_abcd, hamil_H2, hamil_trperm, hamil_H1,
 *     hamil_H0, src/module_basis.f90:33-41, src/module_hamiltonian.f90:53-58)
 *     are handed over once through tvap_init / tvap_set_hamiltonian;
 *   - every call returns a status code; the Fortran shim turns a non-zero
 *     code into the reference's `stop` (the reference has no status codes).
 *   - one context per host thread; a context is not re-entrant.  Contexts on
 *     different threads (and devices) may run at the same time: the settings
 *     a call takes from its context are kept per thread, and each kernel's
 *     shared-memory limit is raised once per device; every call works on the
 *     device that is current on its thread, which tvap_init selects.
 */
#ifndef TVAP_H
#define TVAP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tvap_ctx tvap_ctx;

enum {
  TVAP_OK = 0,
  TVAP_ERR_ARG = 1,           /* bad argument or size */
  TVAP_ERR_CUDA = 2,          /* CUDA runtime error (tvap_last_error has text) */
  TVAP_ERR_NOT_READY = 3,     /* tvap_set_hamiltonian not called */
  TVAP_ERR_SINGULAR_UPHI = 10,/* U_phi singular (calculate_thouless) */
  TVAP_ERR_SINGULAR_RN = 11,  /* canonical overlap matrix singular: the reference
                                 stops with 'got info from zgetrf'
                                 (module_projection.f90:860-864) */
  TVAP_ERR_IMAG_GRADIENT = 13,/* Im(gradient) > 1e-8 (module_projection.f90:751-755) */
  TVAP_ERR_CHOLESKY = 14,     /* dpbtrf failed (module_constraints.f90:528-531) */
  TVAP_ERR_TRTRI = 15,        /* dtrtri failed (module_constraints.f90:568-571) */
  TVAP_ERR_CANONICAL = 16,    /* canonical basis: eigen solver did not converge, a
                                 degenerate subspace larger than 64 or not reducible
                                 to 2 x 2 blocks, or an odd number of paired states */
  TVAP_ERR_NUMBER_DRIFT = 18, /* particle numbers wrong 3 times in 5 iterations
                                 (module_gradient.f90:528-545) */
  TVAP_ERR_DEVICE_TIMEOUT = 19 /* a bounded wait inside a tensor-core kernel ran out
                                  (the kernel stopped and freed its tensor memory) */
};

/* Projected sums of one call of the gauge-angle loop: pnp_over, pnp_ener,
 * pnp_prot, pnp_neut, pnp_prot2, pnp_neut2 (module_projection.f90:58-66) and
 * the canonical-basis counts nocc/nemp of the projected state. */
typedef struct {
  double over[2], ener[2], prot[2], neut[2], prot2[2], neut2[2];
  int nocc, nemp;
} tvap_pnp;

/* Gauge sums of project_wavefunction with iopt = 1 (the observables that
 * print_results prints, src/module_projection.f90:990-1322): the pnp_*
 * accumulators of sum_gauge (src/module_projection.f90:425-458), complex, not
 * divided by the overlap.  ener is the projected energy (the reference leaves
 * rot_ener unset in this mode and prints the sum of ecomp and H0, equal to it
 * up to rounding); pari = sum of weight x <Phi| P R(phi) |Phi> (rot_pari,
 * :279-283); ecomp = calculate_decompo_energy's components
 * (src/module_hamiltonian.f90:1134-1260): 1-body p, n; 2-body PH pp, pn, np,
 * nn; PP pp, pn, np, nn; energy p, n. */
typedef struct {
  double over[2], ener[2], prot[2], neut[2], prot2[2], neut2[2], pari[2];
  double ecomp[12][2];
  int nocc, nemp;
} tvap_pnp_obs;

/* Options of the projection that the reference reads from module globals. */
typedef struct {
  int Mphip, Mphin;      /* proj_Mphip, proj_Mphin */
  double facpi;          /* proj_facpi (2 pi, or pi for separate N/Z) */
  double valence_Z, valence_N;
  double factor_delta;   /* factor_delta (module_fields.f90:40) */
  double seed_occeps;    /* cutoff of occupied states (0 -> 1e-8) */
  int seed_allemp;       /* include all empty sp states in the overlap */
  int mode;              /* 0: batched (all angles per launch, conjugate
                            folding), 1: plain (one angle per launch sequence) */
} tvap_proj_opts;

/* Context: basis size n = HOsp_dim and the single-particle tables
 * (src/module_basis.f90:209-238).  device < 0 selects the current device. */
int tvap_init(tvap_ctx** ctx, int64_t n, const int32_t* sp_2mj, const int32_t* sp_tr, const int32_t* sp_l,
              int device);
void tvap_destroy(tvap_ctx* ctx);
int tvap_set_stream(tvap_ctx* ctx, void* cuda_stream);
const char* tvap_last_error(void);
/* Number of kernels the last top-level call launched: every launch of this
 * library (counted where it is issued); the CUB sort and scan inside
 * tvap_set_hamiltonian launch kernels of their own that are not counted. */
int tvap_kernel_launches(const tvap_ctx* ctx);
/* Optional per-section timing with CUDA events on the streams the sections
 * run on (sections, in this order: canonical basis, angle-independent
 * blocks, Thouless solve, U~/V~, densities, Gamma field, Delta field,
 * traces, H20, overlap, Pfaffian, sums, gradient, evolve, and the tcgen05
 * launches of H20).  tvap_set_timing resets the totals; tvap_get_timing
 * returns milliseconds and call counts per section. */
int tvap_set_timing(tvap_ctx* ctx, int on);
/* Arithmetic of the dense products: 0 = the FP64 pipe (DFMA);
 * 1 = FP64 emulated on the bf16 tensor cores by integer splitting (8
 * balanced 7-bit digits per FP64 value under one power-of-two scale per row
 * or column, exact FP32 partial sums, integer recombination; error bound at
 * tvap_zgemm) with warp-level mma.sync; 2 (default) = the same splitting
 * with tcgen05 MMAs and tensor-memory accumulators for the batched products
 * (small single products keep the mma.sync kernel).  In modes 1 and 2 the
 * field contraction over 16 or more gauge angles also runs on the tensor
 * cores (dense symmetry blocks of the interaction); the factorisations and
 * all reductions run on the FP64 pipe in every mode. */
int tvap_set_gemm_mode(tvap_ctx* ctx, int mode);
int tvap_get_timing(tvap_ctx* ctx, double* ms, long long* calls, int nsec);
/* Mean start and end of every timed section in milliseconds from the start
 * of the projection it belongs to (the gradient and the evolution count
 * from the projection before them).  No reference counterpart. */
int tvap_get_timeline(tvap_ctx* ctx, double* start_ms, double* end_ms, int nsec);
/* Diagnostic counters since the last tvap_set_timing, for the canonical
 * basis: [0] FP32 Jacobi + FP64 refinement attempts, [1] of them accepted by
 * the final check, [2] exact FP64 Jacobi runs, [3] FP32 Jacobi sweeps in
 * total, [4..6] attempts rejected because clusters stayed coupled / the
 * basis was not orthonormal / the clusters of near-degenerate levels could
 * not be diagonalised (more large ones than the list holds, or a block's
 * Jacobi did not converge), [7] large clusters diagonalised by the FP64
 * Jacobi of their block, [8] refinements continued by two second-order
 * steps after a failed check ([4..6] count each failed check).  No
 * reference counterpart. */
int tvap_get_counters(tvap_ctx* ctx, long long* out, int nout);

/* One upload of the reduced two-body list and the one-body part:
 * hamil_H2dim, hamil_abcd (i16, 1-based, 4 per element), hamil_H2 (f32),
 * hamil_trperm (i8), hamil_H1 (complex n x n), hamil_H0 (complex).
 * (src/module_hamiltonian.f90:53-58; read_hamiltonian_reduced :533-599)
 * The list is decoded on the device -- time-reversal pass included -- into
 * the gather form used by tvap_calculate_fields. */
int tvap_set_hamiltonian(tvap_ctx* ctx, int64_t S, const int16_t* abcd, const float* h2, const int8_t* trperm,
                         const double* H1, const double* H0);

/* calculate_fields (src/module_fields.f90:99-189), same arguments and
 * semantics: rho, kappaLR, kappaRL in; gamma, h = gamma + H1, deltaLR,
 * deltaRL out (complex n x n each). */
int tvap_calculate_fields(tvap_ctx* ctx, const double* rhoLR, const double* kappaLR, const double* kappaRL,
                          double* gammaLR, double* hspLR, double* deltaLR, double* deltaRL);

/* calculate_fields for `ncol` (1..256) independent density sets stored one
 * after the other (matrix c at offset c*n*n complex elements).  The call
 * allocates its staging buffers (8 ncol n^2 complex values) and frees them
 * before it returns; cudaFree waits for the whole device. */
int tvap_calculate_fields_batched(tvap_ctx* ctx, int ncol, const double* rhoLR, const double* kappaLR,
                                  const double* kappaRL, double* gammaLR, double* hspLR, double* deltaLR,
                                  double* deltaRL);

/* project_wavefunction(iopt=0) + calculate_projected_H20
 * (src/module_projection.f90:201-373,729-759): from the real Bogoliubov
 * matrices U0, V0 (n x n) computes the projected sums and
 * field_H20v (n*n reals, may be NULL).  A host H20v is complete on return; a
 * device H20v is written in the order of the context's stream. */
int tvap_project(tvap_ctx* ctx, const double* U0, const double* V0, const tvap_proj_opts* opts, tvap_pnp* out,
                 double* H20v);
/* tvap_project for nstates states of the same basis (multi-state batches:
 * seeds, constraint points): state s reads U0s/V0s + s*n*n and opts[s], and
 * writes outs[s] and H20vs + s*n*n (H20vs may be NULL).  The states run one
 * after the other in the context, each on all of the device; the first
 * failing state's code is returned (its outputs and the later ones are not
 * written).  No reference counterpart (the reference projects one state per
 * process). */
int tvap_project_batched(tvap_ctx* ctx, int nstates, const double* U0s, const double* V0s,
                         const tvap_proj_opts* opts, tvap_pnp* outs, double* H20vs);

/* calculate_gradient with gradient_type 0 (src/module_gradient.f90:79-143):
 * Zi = -eta (H20v - sum_j lambda_j C20_j) + mu Zim1, and
 * gradient_norm = |Zi|_F / eta.  C20 holds cdim operators of n*n reals. */
int tvap_calculate_gradient(tvap_ctx* ctx, const double* H20v, int cdim, const double* lambda, const double* C20,
                            const double* Zim1, double eta, double mu, double* Zi, double* gradient_norm);

/* Thouless evolution (cholesky_factorization + evolve_wavefunction,
 * src/module_constraints.f90:497-590): U1 = (U0 + V0 Z) L^-T,
 * V1 = (V0 + U0 Z) L^-T with L L^T = 1 + Z^T Z. */
int tvap_evolve(tvap_ctx* ctx, const double* U0, const double* V0, const double* Z, double* U1, double* V1);

/* tvap_evolve for callers that cannot allocate device memory: the same
 * Thouless evolution, with every matrix (U0, V0, Z in; U1, V1 out) in device
 * memory and the work buffers taken from a fixed array inside the library
 * instead of cudaMalloc.  tvap_evolve keeps its work buffer in the context,
 * allocated on first use and replaced when a larger one is needed (cudaFree
 * of the old one waits for the whole device); a caller whose device memory
 * is owned by its own pool allocator, or that cannot accept such a wait,
 * uses this variant.  No counterpart in the reference.
 *   - limit: n <= 336 (the array holds 3 n^2 + n doubles for n = 336, about
 *     2.6 MB, kept on every GPU that loads the library until the process ends);
 *     larger n is rejected with TVAP_ERR_ARG;
 *   - the first call on a device looks up the array's device address; make
 *     that first call before any stream capture;
 *   - all calls share the array: calls that overlap on the GPU (from several
 *     contexts or streams at once) race on it;
 *   - the dense products run on the FP64 pipe in this variant;
 *   - the context's device must be the current device, and all five
 *     pointers must be device (or managed) memory of that device;
 *   - the call works on the context's stream (tvap_set_stream): the inputs
 *     must be complete in that stream's order when it is called, and the
 *     outputs are complete when it returns (it ends with a synchronisation
 *     of that stream). */
int tvap_evolve_noalloc(tvap_ctx* ctx, const double* U0, const double* V0, const double* Z, double* U1, double* V1);

/* One gradient iteration of the reference's main loop for gradient_type 0
 * without constraints (src/taurus_vap.f90:86-113: project_wavefunction +
 * calculate_projected_H20, calculate_gradient, and the Thouless evolution
 * that adjust_constraints applies when constraint_dim = 0 -- the PNVAP case,
 * src/module_constraints.f90:84-100,270-373) in one call with a single host
 * round trip at the end: out receives the projected sums of (U0, V0), H20v
 * (may be NULL) field_H20v, Zi = -eta H20v + mu Zim1, gradient_norm =
 * |Zi|_F / eta, and (U1, V1) = evolve(U0, V0, Zi).  The evolution is always
 * computed: a caller whose convergence test (gradient_norm <= eps) stops
 * the loop keeps (U0, V0), as the reference does.  Separate input and output
 * buffers; host or device memory.  No single counterpart in the reference
 * (it makes three calls). */
int tvap_iterate(tvap_ctx* ctx, const double* U0, const double* V0, const tvap_proj_opts* opts, double eta,
                 double mu, const double* Zim1, double* Zi, double* U1, double* V1, tvap_pnp* out, double* H20v,
                 double* gradient_norm);

/* diagonalize_hsp_and_H11 with opt = 0 (src/module_gradient.f90:158-453):
 * the eigenvalues (ascending) of h^RR - sum_m lambda_m C_m and of
 * H11 - sum_m lambda_m C11_m for the state (U0, V0), where h and Delta are
 * the fields of the real densities, H11 = U^T h U - V^T h^T V + (U^T Delta V
 * + (U^T Delta V)^T) factor_delta (calculate_H11_real,
 * src/module_fields.f90:327-354), C_m the cdim constraint operators
 * constraint_HO (n*n reals each, the last cpair of them pair operators, whose
 * C11 term is zero as in the reference) with multipliers lambda.  info[0],
 * info[1] take the place of the DSYEV infos of the two (non-zero for a
 * non-finite matrix).  Replaces the two DSYEV calls by an FP64 Householder
 * reduction and Sturm multisection on the device; n <= 512. */
int tvap_diagonalize_hsp_and_H11(tvap_ctx* ctx, const double* U0, const double* V0, int cdim, int cpair,
                                 const double* lambda, const double* constraint_HO, double factor_delta,
                                 double* eigen_hsp, double* eigen_H11, int* info);
/* The step sizes of calculate_gradient (src/module_gradient.f90:86-119):
 * gradient_type 0 returns eta_in, mu_in; 1 takes the H11 spectrum
 * (eigen_max = 4 max|e|, eigen_min = 2 min|e|), 2 that of h (2 max|e|,
 * 2 min|e|), with eta = (2 / (sqrt(eigen_max) + sqrt(eigen_min)))^2 and
 * mu = ((sqrt(c) - 1) / (sqrt(c) + 1))^2, c = eigen_max / eigen_min; a failed
 * diagonalisation (info) falls back to type 0, as in the reference.  Host
 * arithmetic only. */
int tvap_gradient_parameters(int gradient_type, int n, const double* eigen_hsp, const double* eigen_H11,
                             const int* info, double eta_in, double mu_in, double* eta, double* mu);

/* adjust_constraints (src/module_constraints.f90:270-373): up to 100 Newton
 * steps that move the Thouless step Zi (n*n reals, updated in place) until
 * the constraint expectation values of (U1, V1) = evolve(U0, V0, Zi) reach
 * `values` within eps: Tr(C_m rho) for the first cdim - cpair operators of
 * constraint_HO, Tr(C_m kappa^T) for the last cpair (pair operators), with
 * the update Zi += sum_m x_m C20_m, A x = values - <C>, A_ij =
 * Tr(C20_i^T C20_j) and C20_m the 20 part of C_m at (U1, V1) (f20 / g20 of
 * set_operator_qpbasis).  Writes U1, V1, C20 (cdim n*n reals, may be NULL)
 * of the last step and the number of steps; cdim = 0 is one evolution.  All
 * but the cdim x cdim solve runs on the device; cdim <= 64. */
int tvap_adjust_constraints(tvap_ctx* ctx, const double* U0, const double* V0, double* Zi, int cdim, int cpair,
                            const double* constraint_HO, const double* values, double eps, double* U1, double* V1,
                            double* C20, int* iterations);

/* Many independent states iterated at once (the seeds of a minima search,
 * the points of a constraint sweep; no counterpart in the reference, which
 * runs one state per process): state s makes one tvap_iterate step on
 * context ctx[s] with U0[s], V0[s], opts[s], eta[s], mu[s], Zim1[s] and
 * writes Zi[s], U1[s], V1[s], out[s], gradient_norm[s] and status[s].  The
 * states of one context run in order on one host thread; distinct contexts
 * (each with its own streams; bases of different sizes allowed) run on
 * concurrent host threads, so their kernels share the device.  The first
 * failing state's status is returned. */
int tvap_iterate_many(int nstates, tvap_ctx* const* ctx, const double* const* U0, const double* const* V0,
                      const tvap_proj_opts* opts, const double* eta, const double* mu, const double* const* Zim1,
                      double* const* Zi, double* const* U1, double* const* V1, tvap_pnp* out,
                      double* gradient_norm, int* status);

/* project_wavefunction(1, 0, Mphip, Mphin, ndim) as print_results calls it
 * (src/module_projection.f90:1059, the branch :279-354): per gauge angle the
 * transition densities and fields, then the traces the printed observables
 * need, summed over the angles with weight x overlap.
 *   obo:   nobo complex n x n one-body operators B_k (column-major, as the
 *          reference passes its vectorised tables: Jx, i Jy, Jz, the
 *          spin-orbit term, the Q_lm, r^2); obo_sum[k] = (proton, neutron)
 *          sums of Tr(B_k rho^LR) over those rows (calculate_expectval_obo_
 *          cplx, src/module_operators.f90:146-164), 2 x nobo complex;
 *   sq:    nsq pairs (O_k, O2_k) of complex n x n matrices, one after the
 *          other; sq_sum[k] = the sum of <O_k^2> (calculate_expectval_obos_
 *          cplx, src/module_operators.f90:227-257), nsq complex;
 *   sp_parity: (-1)^l of each state (host; NULL: no parity overlap, pari 0);
 *   shell_size: 2j+1 of each of the nshell shells (host); occnum = the
 *          (proton, neutron) occupations of the shells (calculate_occupation_
 *          number, src/module_particlenumber.f90:157-176), 2 x nshell complex;
 *   rho:   pnp_rho, n x n complex (host or device; may be NULL).
 * All Mphip x Mphin angles are computed (no conjugate folding).  obo and sq
 * may be host or device arrays; the sums are host arrays. */
int tvap_project_observables(tvap_ctx* ctx, const double* U0, const double* V0, const tvap_proj_opts* opts,
                             int nobo, const double* obo, int nsq, const double* sq, const int32_t* sp_parity,
                             int nshell, const int32_t* shell_size, tvap_pnp_obs* out, double* obo_sum,
                             double* sq_sum, double* occnum, double* rho);

/* Launch shapes of the projection, chosen by measurement (no counterpart
 * in the reference).  tvap_autotune times `reps` projections of (U0, V0)
 * with opts for each candidate -- B' tile policy of the tcgen05 products (0:
 * the width that pads the output columns less, 1: 64 rows, 2: 48 rows) x the
 * groups of angles in the Thouless solve (2 staggered on two streams, or 1)
 * x the cap on the tcgen05 CTAs beside the second group's panels (0: the
 * SMs the panels leave, 1: half the SMs, 2: none; 2 groups only) x the
 * look-ahead of the solve's panels (the bulk of each elimination product on
 * a stream of its own while the next panel is factored: on, off) x the form
 * of the overlap's Pfaffian (the shared-memory elimination where it fits, or
 * always the blocked one: the same pivots, another summation order) -- 48
 * candidates, CUDA events on the context's stream, and keeps the fastest in
 * the context.  table_ms (may be NULL) receives the ms per projection of the
 * first ntable candidates in the order Pfaffian form 0, then 1, each with
 * look-ahead on, then off, each with groups 2 (cap 0, 1, 2), then groups 1,
 * each with bn 0, 1, 2.  Results do not depend on the tile and launch
 * shapes (the same FP64 emulation in every product); the Pfaffian form
 * changes the order of its rounding.  tvap_set_tuning and tvap_get_tuning
 * (knobs[3] = bn, groups, cap), tvap_set_option and tvap_get_option (the
 * look-ahead and the Pfaffian form, 0 or 1; 0 unless set or chosen by the
 * tuner; tvap_get_option returns -1 for an unknown option) set and read
 * them. */
int tvap_autotune(tvap_ctx* ctx, const double* U0, const double* V0, const tvap_proj_opts* opts, int reps,
                  double* table_ms, int ntable);
int tvap_set_tuning(tvap_ctx* ctx, int bn_policy, int solve_groups, int solve_cap);
int tvap_get_tuning(const tvap_ctx* ctx, int* knobs);
/* TVAP_OPT_COMPLEX_PAIRS = k >= 0: the complex x complex products on the
 * tensor cores whose contraction length is at least k (and whose batch
 * entries share no operand) take the paired form
 * (real and imaginary rows interleaved in both operands, the four real
 * products of each element combined on the exact integer accumulators:
 * half the digit planes of the left operand, twice the tiles of half the
 * k-steps), the others the real representation [[Re, -Im], [Im, Re]] x
 * [Re, Im]; 0: none.  Both forms give the same bits. */
enum { TVAP_OPT_SOLVE_LOOKAHEAD = 1, TVAP_OPT_PFAFFIAN_BLOCKED = 2, TVAP_OPT_COMPLEX_PAIRS = 3 };
int tvap_set_option(tvap_ctx* ctx, int option, int value);
int tvap_get_option(const tvap_ctx* ctx, int option);

/* Test hook, no counterpart in the reference: the next tvap_evolve on this
 * context runs its cooperative launch with one CTA that leaves before the
 * first grid-wide barrier, so that the other CTAs' bounded waits there run
 * out (after about a second); they raise the status word and return, and
 * that tvap_evolve returns TVAP_ERR_DEVICE_TIMEOUT.  Nothing faults or
 * hangs, and the context stays usable.  It shows that a wait which is never
 * released ends in a status the caller can read. */
int tvap_test_wait_timeout(tvap_ctx* ctx);

/* Adjoint of the projected energy E(Z) = <Phi(Z)|H P|Phi(Z)>/<Phi(Z)|P|Phi(Z)>
 * of the state Phi(Z) = evolve(U0, V0, Z) with respect to the real Thouless
 * matrix Z: writes E and dE/dZ (n*n reals).  The per-angle densities are
 * recomputed, not stored.  No counterpart in the reference. */
int tvap_energy_adjoint(tvap_ctx* ctx, const double* U0, const double* V0, const double* Z,
                        const tvap_proj_opts* opts, double* energy, double* dEdZ);

/* ZSKPFA('U', 'P', n, A, n, PFAFF, ...) of PFAPACK
 * (src/subroutines_pfaffian.f:12-258; called by calculate_overlap,
 * src/module_projection.f90:921) for `batch` complex skew-symmetric n x n
 * matrices stored one after the other (column-major, interleaved re/im; only
 * the upper triangle is read).  pfaff receives batch complex values.  As in
 * ZSKPFA: Pf = 1 for n = 0, Pf = 0 for odd n, and a zero pivot of the
 * Parlett-Reid elimination gives Pf = 0 with a successful status.  A is not
 * modified (ZSKPFA overwrites it).  n <= 512; host or device memory. */
int tvap_zskpfa_batched(tvap_ctx* ctx, int batch, int64_t n, const double* A, double* pfaff);

/* ZGEMM / DGEMM of BLAS (C = alpha op(A) op(B) + beta C, op = 'N', 'T' or
 * 'C'; column-major with leading dimensions; alpha and beta are complex
 * (2 doubles) for tvap_zgemm and real (1 double) for tvap_dgemm) in the
 * arithmetic the context uses for the path's own products
 * (tvap_set_gemm_mode).  Host or device memory; the call returns when C is
 * written.  In modes 1 and 2 a product with K >= 16 and at least 10^6
 * multiply-adds is emulated on the tensor cores: every row i of op(A) and
 * column j of op(B) gets one power-of-two scale 2^e (2^e <= its largest
 * entry), each entry is rounded to an integer multiple of 2^(e-53) (error
 * <= 2^-54 of the row's or column's largest entry) and written as 8 balanced
 * base-2^7 digits, and the digit pairs of total weight below the 8th are
 * dropped.  With a_i = max_k max(|Re op(A)_ik|, |Im op(A)_ik|) and b_j the
 * same over column j of op(B):
 *   real:    |C_ij - (op(A) op(B))_ij| <= 2^-49 K a_i b_j
 *   complex: |C_ij - (op(A) op(B))_ij| <= 2^-46 K a_i b_j
 * before the final rounding of C_ij to FP64 and the scaling by alpha and
 * beta.  The bound is relative to the largest entries of the row and the
 * column, not to each term: an entry of C much smaller than K a_i b_j keeps
 * fewer correct digits than a FP64 product (error <= ~2^-53 K sum_k |A_ik
 * B_kj|) gives it.  The emulated modes do not carry NaN or infinity
 * through: a non-finite operand gives undefined results.  Mode 0 runs on the
 * FP64 pipe.  Replaces the BLAS calls
 * of the reference (not a reference routine of
 * its own). */
int tvap_zgemm(tvap_ctx* ctx, char transa, char transb, int m, int n, int k, const double* alpha, const double* A,
               int lda, const double* B, int ldb, const double* beta, double* C, int ldc);
int tvap_dgemm(tvap_ctx* ctx, char transa, char transb, int m, int n, int k, const double* alpha, const double* A,
               int lda, const double* B, int ldb, const double* beta, double* C, int ldc);

#ifdef __cplusplus
}
#endif
#endif
