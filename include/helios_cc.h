/*
 * helios_cc.h -- C ABI of the GB300 closed-shell PPP CCSD engine (helios "r-ccsd").
 *
 * Drop-in for the coupled-cluster call of helios. The reference drives CCSD
 * through module globals from getEnergy (src/modules/mod_property.f90:55-338):
 *   setCCParameters('r-ccsd')  -> hx_ccsd_create / hx_ccsd_create_batch
 *   initCC (SCF, MO Fock, integrals, guessCC)        -> hx_ccsd_init
 *   iterationCC(iteration, epsilon, accuracy)        -> hx_ccsd_iterate
 *   energyCC(energy)                                 -> hx_ccsd_energy
 *   iterator(iterationCC, energyCC, ...)             -> hx_ccsd_solve / hx_ccsd_solve_batch
 *   finalizeCC                                       -> hx_ccsd_destroy
 * (src/methods/coupledCluster/mod_cc.f90:82-485, 489-603, 634-650, 820-891,
 *  1916-1952; src/calculation/gIterator.f90:1-210.)
 *
 * Conventions
 *  - Every entry point returns 0 (HX_OK) or a negative code; iteration
 *    outcomes use the iterator's statuses: 1 converged, -1 failed (max
 *    iterations), -2 diverged, -3 stagnated, -4 interrupted. Errors are
 *    <= -100 and hx_last_error() describes the last one. Nothing exits,
 *    aborts or traps.
 *  - Caller buffers are host memory, copied in and out; device memory belongs
 *    to the handle. One handle per host thread; it owns one CUDA stream.
 *  - Energies are in eV, coordinates in Angstrom, fields in eV/Angstrom.
 *  - Amplitudes cross the ABI in the reference's Fortran layout: t1(o, v) and
 *    t2(o, o, v, v), column-major, virtual indices counted from the first
 *    virtual orbital (t1(i, a) of the reference is t1[i + o*(a-o-1)] with
 *    1-based i, a).
 */
#ifndef HELIOS_CC_H
#define HELIOS_CC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HX_OK 0
#define HX_CONVERGED 1
#define HX_FAILED_MAXITER (-1)
#define HX_DIVERGED (-2)
#define HX_STAGNATED (-3)
#define HX_INTERRUPTED (-4)
#define HX_ERR_ARG (-100)
#define HX_ERR_CUDA (-101)
#define HX_ERR_NOMEM (-102)
#define HX_ERR_STATE (-103)
#define HX_ERR_SCF (-104)
#define HX_ERR_KERNEL (-105)
#define HX_ERR_UNSUPPORTED (-106)

#define HX_COULOMB_OHNO_KLOPMAN 0
#define HX_COULOMB_MATAGA_NISHIMOTO 1
#define HX_COULOMB_HUBBARD 2

#define HX_BOND_SINGLE 0
#define HX_BOND_DOUBLE 1
#define HX_BOND_NONSET (-1)

#define HX_PRECISION_FP64 0
#define HX_PRECISION_MIXED 1
#define HX_PRECISION_EXACT 2   /* every iteration on the 7-slice tensor-core GEMM that emulates FP64 */

/* One molecule block of a helios input (src/input/readMoleculeInformation.f90:20-117). */
typedef struct hx_ppp_model {
    int32_t n_sites;
    const double *coords;      /* n_sites x 3, Angstrom (re-centred by the engine) */
    const double *alpha;       /* site energies, eV */
    const double *gamma;       /* one-centre repulsions, eV */
    const int32_t *nels;       /* pi electrons donated per site */
    int32_t n_bonds;
    const int32_t *bond_i;     /* 0-based site indices */
    const int32_t *bond_j;
    const double *beta;        /* resonance integrals, eV */
    const int32_t *bond_kind;  /* HX_BOND_SINGLE / HX_BOND_DOUBLE / HX_BOND_NONSET */
} hx_ppp_model;

/* The input keywords of the path (src/input/definebd.f90), with helios's
 * defaults filled in by hx_cc_params_default. */
typedef struct hx_cc_params {
    int32_t coulomb;              /* parametrization:coulomb-integrals (ohno-klopman) */
    double bond_alternation;      /* parametrization:bond-alternation (0) */
    double field[3];              /* field:along-x/y/z, or p*polariz:derive-step (0) */
    int32_t scf_maxiter;          /* scf:max-iterations (400) */
    double scf_eps;               /* scf:accuracy, as 10^-value (1e-12) */
    double scf_step;              /* scf:iter-step (0.05) */
    int32_t projection_type;      /* coupled-cluster:projection-type 1 or 2 (= "2-1", default) */
    int32_t cc_maxiter;           /* coupled-cluster:max-iterations (2000) */
    double cc_eps;                /* coupled-cluster:accuracy, as 10^-value (1e-12) */
    double t1_step, t2_step;      /* coupled-cluster:t1-step, t2-step (1, 1) */
    int32_t diis_enabled;         /* coupled-cluster:diis-enabled (1) */
    int32_t diis_steps;           /* coupled-cluster:diis-steps (20, range 2..50) */
    int32_t check_divergence;     /* iteration:enable-divergence-check (1) */
    double divergence_threshold;  /* iteration:divergence-threshold, as 10^value (1e3) */
    int32_t check_stagnation;     /* iteration:enable-stagnation-check (1) */
    double stagnation_threshold;  /* iteration:stagnation-threshold, percent (60) */
    int32_t stagnation_after;     /* iteration:stagnation-check-after (200) */
    int32_t precision;            /* HX_PRECISION_FP64 (default), HX_PRECISION_MIXED or HX_PRECISION_EXACT */
    int32_t guess;                /* 0 reference guess (guessCC), 1 learned guess */
    double mixed_switch;          /* mixed precision: residual at which a molecule moves from
                                     3-slice to 4-slice tensor-core iterations (1e-3); 4-slice
                                     run to 1e-3 mixed_switch, then 5-slice; any of them hands
                                     over to the check iterations below 0.1 eps */
    int32_t mixed_patience;       /* mixed precision: iterations without a new lowest residual
                                     after which a molecule moves on to the next phase (3) */
    int32_t mixed_check;          /* mixed precision: the iterations that may declare
                                     convergence: 0 = 7-slice tensor-core contractions that
                                     emulate FP64 (default), 1 = FP64 on the CUDA cores */
    int32_t tile_tuning;          /* mixed precision, tensor-core tile shapes per (precision
                                     mode, contraction group, size class): 0 = from the tile
                                     table (hx_tile_table_load), the default shape where it
                                     has no entry (default); 1 = the same, but a missing entry
                                     is found by timing every candidate on this handle's own
                                     contractions when it is created, and added to the table;
                                     2 = the default shapes */
    int32_t tile_force;           /* >= 0: candidate tile_force of every precision mode (the
                                     last one where a mode has fewer); -1 (default): as
                                     tile_tuning says */
} hx_cc_params;

typedef struct hx_ccsd hx_ccsd;

/* Fill p with helios's defaults. */
void hx_cc_params_default(hx_cc_params *p);

/* setCCParameters('r-ccsd') (mod_cc.f90:82-485; r-ccsd branch :415-428): build
 * the PPP Hamiltonian of one molecule and allocate the device state. */
int hx_ccsd_create(const hx_ppp_model *m, const hx_cc_params *p, hx_ccsd **out);

/* The same for n molecules solved together (one batched launch per step). */
int hx_ccsd_create_batch(const hx_ppp_model *ms, int32_t n, const hx_cc_params *p, hx_ccsd **out);

/* initCC r-ccsd (mod_cc.f90:489-603, :538-558, guessCC :634-650): RHF SCF,
 * MO Fock, reference energy, integrals and the starting amplitudes. An SCF
 * that does not converge returns HX_ERR_SCF; in a batch such a molecule is
 * left out instead (hx_ccsd_solve_batch reports HX_ERR_SCF as its status)
 * and the call fails only if no SCF converged. */
int hx_ccsd_init(hx_ccsd *h);

/* Replace molecule mol's amplitudes (reference layout, see above). This call
 * and hx_ccsd_get_amplitudes stage the arrays in a pinned host buffer the
 * handle keeps (o*v + (o*v)^2 doubles of the largest molecule asked for, freed
 * by hx_ccsd_destroy; pageable memory if pinning fails). */
int hx_ccsd_set_guess(hx_ccsd *h, int32_t mol, const double *t1, const double *t2);

/* ---- Learned T2 guess (no counterpart in the reference; it replaces the
 * MP2-like guessCC amplitudes when hx_cc_params.guess = 1). The network is
 * 8 -> 256 -> 256 -> 256 -> 1 with SiLU, bf16 weights in layers 2 and 3,
 * FP32 accumulation; its parameters are one float32 blob of
 * hx_mlp_nparam() values: W1[256x8] b1 W2[256x256] b2 W3[256x256] b3 w4[256]
 * b4 x_shift[8] x_scale[8] y_scale. Per amplitude (ia) <= (jb) it reads
 * x = (guess, e_i, e_j, e_a, e_b, (ia|jb), (ib|ja), 8/N) and predicts
 * t2 - guess; both t2 entries of the pair receive guess + prediction. */
int hx_mlp_nparam(void);

/* Install (params != NULL, copied) or remove (NULL) the network used by
 * hx_ccsd_init when guess = 1. */
int hx_ccsd_set_model(hx_ccsd *h, const float *params);

/* Training rows of a solved molecule: for n canonical pair indices rows[k]
 * (index r of the pair (p, q), p <= q, in row-major order of the upper
 * triangle of the (ia) x (jb) matrix, p = i*v + a) the 8 inputs X[k][8] and
 * the target T[k] = t2(current) - guess. */
int hx_ccsd_training_rows(hx_ccsd *h, int32_t mol, int32_t n, const int64_t *rows, float *X, float *T);

/* Network on n input rows X[n][8] (host arrays): Y[n] = predictions
 * (tcgen05 inference kernel). */
int hx_mlp_predict(const float *params, const float *X, int64_t n, float *Y);

/* Mean-squared-error loss (in units of y_scale^2) and its gradient with
 * respect to every blob entry (0 for the fixed normalisation constants) on
 * n rows, computed on the GPU by the training kernels. */
int hx_mlp_grad(const float *params, const float *X, const float *T, int32_t n, float *loss, float *grad);

/* Train the network on the GPU: Adam (cosine-decayed learning rate lr) over
 * `epochs` passes of shuffled mini-batches of `batch` rows; params is updated
 * in place and epoch_loss[e] (if not NULL) receives each epoch's mean loss.
 * The 256-wide products of each step run on the BF16 tensor cores with FP32
 * accumulation (weights, activations and the loss gradients entering them
 * rounded to bf16); the weight gradients are summed with split-K atomics, so
 * two runs differ in the last bits. */
int hx_mlp_train(float *params, const float *X, const float *T, int64_t n, int32_t epochs, int32_t batch, float lr,
                 uint64_t seed, float *epoch_loss);

/* iterationCC (mod_cc.f90:820-891) for every active molecule: residuals,
 * Jacobi step, DIIS. acc[0] = max|d1|, acc[1] = max|d2| of molecule 0
 * (acc[2..4] = -1, as the reference fills them). The contractions run on the
 * 7-slice tensor-core GEMM for HX_PRECISION_EXACT handles and on the FP64
 * CUDA cores otherwise (the mixed-precision ladder is hx_ccsd_solve's). */
int hx_ccsd_iterate(hx_ccsd *h, int32_t iteration, double eps, double acc[5]);

/* energyCC r-ccsd (mod_cc.f90:1916-1952) of molecule 0: e[0] total,
 * e[1] reference energy, e[2] singles part, e[3] doubles part, e[4] 0. */
int hx_ccsd_energy(hx_ccsd *h, double e[5]);

/* iterator(iterationCC, energyCC, maxiter, eps) (gIterator.f90:1-210) for
 * molecule 0; *status gets the iterator status (1, -1, -2, -3, -4). */
int hx_ccsd_solve(hx_ccsd *h, int32_t maxiter, double eps, int32_t *status, int32_t *iters,
                  double e[5]);

/* The iterator for every molecule of a batch; arrays have n entries (e: n x 5). */
int hx_ccsd_solve_batch(hx_ccsd *h, int32_t *status, int32_t *iters, double *e);

/* Amplitudes of molecule mol in the reference layout (t1: o*v, t2: o*o*v*v). */
int hx_ccsd_get_amplitudes(hx_ccsd *h, int32_t mol, double *t1, double *t2);

/* SCF results of molecule mol: C (N x N, column p = MO p, row-major [site][MO]),
 * orbital energies (N), MO Fock (N x N row-major); scf[0..3] = E_total, E_el,
 * E_nuc, last accuracy; scf_status[0..1] = status, iterations. Any pointer may
 * be NULL. */
int hx_ccsd_get_scf(hx_ccsd *h, int32_t mol, double *C, double *eps, double *fmo, double scf[4],
                    int32_t scf_status[2]);

/* Per-iteration record of molecule mol's last solve: for each iteration
 * k < cap, out[5k..5k+4] = max|d1|, max|d2|, E_total, seconds since the start
 * of the solve, phase of the iteration (0 FP64 CUDA cores; 1, 2, 3, 4: seven-
 * (FP64 emulated), five-, four- and three-slice tensor-core contractions).
 * Returns the number of iterations recorded. */
int hx_ccsd_trace(hx_ccsd *h, int32_t mol, double *out, int32_t cap);

/* r-ccsd(t): the (T) triples correction of molecule mol from its amplitudes
 * after a solve (the reference computes it in the spin-orbital basis,
 * mod_cc.f90:2028-2111; this is the same quantity in spatial orbitals).
 * e[0] = (T) = E[4] + E[5] in the textbook sign convention, e[1] = E[4]
 * (connected triples), e[2] = E[5] (disconnected), e[3] = the reference's
 * triples term c1 + c2 + c3, which is -(T): its c1 multiplies amp^2 by
 * D = F_aa + F_bb + F_cc - F_ii - F_jj - F_kk > 0, and c3 (a term in F_kc)
 * vanishes for canonical RHF orbitals. The triples i <= j <= k are taken in
 * slabs on the 7-slice (FP64-emulating) tensor-core GEMM; the call allocates
 * O(o v^3) doubles plus one slab (at most about 24 GB) and returns
 * HX_ERR_NOMEM when not even one slab fits. */
int hx_ccsd_triples(hx_ccsd *h, int32_t mol, double e[4]);

/* Engine utility with no counterpart in the reference: device timing.
 * out[0] = ms of the last hx_ccsd_init (SCF, integrals, guess), out[1] = ms
 * of the last solve, both from CUDA events on the handle's stream;
 * out[2..5] = launches, ms, algorithmic flops (2*M*N*K) and tensor-core
 * flops issued by the tcgen05 GEMM since profiling was switched on;
 * out[6] = device bytes held by the handle; out[7] = kernels the library
 * launched (all handles) since profiling was last switched on. profile = 1 switches per-launch
 * GEMM timing on (and clears the totals), 0 off, -1 leaves it. */
int hx_ccsd_timing(hx_ccsd *h, double out[8], int32_t profile);

/* Sizes of molecule mol: dims[0..3] = N, o, v, electrons. */
int hx_ccsd_dims(hx_ccsd *h, int32_t mol, int32_t dims[4]);

/* Request a cooperative stop (the reference's stop-iteration / SIGUSR1); safe
 * from any thread. The running solve ends with status -4 after the current
 * iteration. */
void hx_ccsd_cancel(hx_ccsd *h);

/* finalizeCC: free the device state. */
void hx_ccsd_destroy(hx_ccsd *h);

/* Engine utility with no counterpart in the reference: C = A B^T for
 * row-major FP64 host matrices (A: M x K, B: N x K, C: M x N) on the engine's
 * FP64 CUDA-core GEMM (precision 0) or its exact-slice tcgen05 GEMM with
 * 3 slices (precision 1, about 2^-24 of the row maxima), 5 slices (precision
 * 2, about 2^-35), 4 slices (precision 3, about 2^-32) or 7 slices
 * (precision 4: FP64 emulated, as accurate as the FP64 product); the launch
 * is repeated reps times after one warm-up and
 * *ms (if not NULL) receives the mean device time per launch. */
int hx_gemm(const double *A, const double *B, double *C, int32_t M, int32_t N, int32_t K, int32_t precision,
            int32_t reps, double *ms);
/* hx_gemm on tile candidate `variant` (0 .. hx_tile_variants(mode) - 1) of
 * the tensor-core precision's mode, -1 for the default; no counterpart in the
 * reference (it measures the candidates the tile autotuner chooses from).
 * Every candidate forms the same sums. */
int hx_gemm_tile(const double *A, const double *B, double *C, int32_t M, int32_t N, int32_t K, int32_t precision,
                 int32_t variant, int32_t reps, double *ms);

/* Allocation-free variant of hx_gemm; it has no counterpart in the
 * reference. For callers that cannot allocate device memory at call time: a
 * host that has handed the device's memory to its own pool allocator (so
 * cudaMalloc would fail), or code that must not stall work on other streams
 * (cudaFree synchronises the whole device). C = A B^T for row-major FP64
 * matrices already in DEVICE memory
 * (A: M x K, B: N x K, C: M x N), always on the tcgen05 exact-slice GEMM
 * (precision 1: 3 slices, 2: 5 slices; FP64 is rejected). It calls no
 * allocator: the operand slices, row exponents, error word and descriptors
 * live in one static device array of about 5.3 MB, whose address is looked
 * up once per device (cudaGetSymbolAddress) on the first call; make that
 * first call before any stream capture. The address is kept for the life of
 * the library, so a device reset (cudaDeviceReset) while the library is
 * loaded is not supported. Dimensions above HX_NOALLOC_MAX_DIM return
 * HX_ERR_ARG. C is zeroed and accumulated on `stream` (a cudaStream_t;
 * NULL = the legacy default stream), and the call returns after the stream
 * has synchronised: it reads the kernel's error word back, so a call on a
 * stream that is being captured returns HX_ERR_ARG and leaves the capture
 * untouched. Results equal hx_gemm's bit for bit wherever hx_gemm uses the
 * tensor cores (M*N*K >= 1e4). The scratch is shared: calls that overlap in
 * time, on any streams or host threads, race and corrupt each other's
 * results. */
#define HX_NOALLOC_MAX_DIM 512
int hx_gemm_noalloc(const double *A, const double *B, double *C, int32_t M, int32_t N, int32_t K,
                    int32_t precision, void *stream);

/* ---- Tensor-core tile autotuner (no counterpart in the reference). Every
 * precision mode of the exact-slice GEMM has a few candidate tile widths
 * (hx_tile_variants); they form the same sums in the same order and differ
 * in speed only. The process-wide tile table maps (mode, contraction group,
 * size class N, size class work) to a candidate: entries of 5 int32 values.
 * hx_tile_table copies up to cap entries and returns how many there are;
 * hx_tile_table_load merges n entries (a table measured on the GB300 ships
 * with the Python front end). */
int hx_tile_table(int32_t *entries, int32_t cap);
int hx_tile_table_load(const int32_t *entries, int32_t n);
/* Output tile widths (BN) of mode's candidates (mode 0..3: 3, 4, 5, 7
 * slices); returns their number. */
int hx_tile_variants(int32_t mode, int32_t *bn, int32_t cap);
/* The candidate each (mode, group) of a mixed-precision handle runs,
 * var[mode * groups + group]; *tune_ms (if not NULL) = milliseconds its
 * creation spent timing candidates. Returns 4 * groups (0 for FP64 handles). */
int hx_ccsd_tile_choices(hx_ccsd *h, int32_t *var, int32_t cap, double *tune_ms);

/* Copy the message of the last error (thread-local) into buf; returns its length. */
int hx_last_error(char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* HELIOS_CC_H */
