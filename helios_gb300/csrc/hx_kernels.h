// Host-side launchers of the engine's kernels.
#pragma once
#include "hx_plan.h"

long long hx_tgemm_f64_prepare(TgemmDesc *descs, int n);
cudaError_t hx_tgemm_f64_launch(const TgemmDesc *d_descs, int n, long long total_tiles,
                                const int *d_active, cudaStream_t s);

cudaError_t hx_scf_launch(const ScfMol *d_mols, int nmol, int nmax, const ScfParams &p, double *d_gpart,
                          cudaStream_t s);

cudaError_t hx_ew_dress_init(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s);
cudaError_t hx_ew_dress_fock(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s);
cudaError_t hx_ew_zdo_products(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s);
cudaError_t hx_ew_gamma_scale(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s);
cudaError_t hx_ew_fock_blocks(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s);
cudaError_t hx_ew_c_combine(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s);
cudaError_t hx_ew_setup(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s);
cudaError_t hx_ew_setup2(const CCMol *m, const int *act, const HxSched &S, int guess, cudaStream_t s);
// pair-unit kernels: dynamic shared memory for kernel 0 (make_u), 1 (step and
// push), 2 (amplitudes and energy); the attribute is raised once to the largest
size_t hx_unit_smem(const int *o, const int *v, int nmol, int kernel);
cudaError_t hx_unit_kernels_init(size_t smem_max);
cudaError_t hx_ew_make_u(const CCMol *m, const int *act, const HxSched &S, size_t smem, cudaStream_t s);
cudaError_t hx_tail(const CCMol *m, const DiisMol *h, const int *act, const HxSched &S, const size_t smem[2],
                    double s1, double s2, int proj, int use_diis, const double *gate, double *part, cudaStream_t s);
cudaError_t hx_energy(const CCMol *m, const DiisMol *h, const int *act, const HxSched &S, size_t smem, double *part,
                      cudaStream_t s);

// (T) triples (hx_triples.cu): ZDO pair products of the occupied and virtual
// orbitals; the energy partials of a slab of triples (i, j, k) for one i, the
// pairs (j, k) listed in `pairs`, and their ordered sum (out[0] = E[4],
// out[1] = E[5] of the slab, each triple weighted by its permutations).
cudaError_t hx_triples_pairs(const double *C, int N, int o, double *Bvv0, double *Boo0, cudaStream_t s);
cudaError_t hx_triples_energy(const double *W, const int2 *pairs, int npairs, int i, const double *t1,
                              const double *gov, const double *Fmo, int N, int o, double *part, double *out,
                              cudaStream_t s);

// Device-side iterator (hx_control.cu): record the solve's start time; after an
// iteration apply the stop rules and the phase ladder, write the next
// iteration's masks (act_ph may be NULL for FP64 handles) and count the
// molecules still running (remaining) and per next phase (occ[5]); in a
// captured iteration, set the conditional node of each entry of hs from the
// count of its phase (entries with phase < 0 are skipped), clear occ and add
// one to runs[p] for every phase p that runs.
struct PhaseCondition {
    cudaGraphConditionalHandle handle;
    int phase, pad_;
};
cudaError_t hx_control_start(unsigned long long *d_t0, cudaStream_t s);
cudaError_t hx_control(const CCMol *mols, const DiisMol *diis, CtlMol *ctl, const CtlParams &P, const volatile int *cancel_flag,
                       const unsigned long long *t0, int *active, int *act_ph, double *gate, double *trace,
                       int *remaining, int *occ, cudaStream_t s);
cudaError_t hx_phase_conditions(int *occ, const PhaseCondition *hs, int n, int *runs, cudaStream_t s);
// Last node of a solve's loop body: keep looping while molecules run, at most cap times.
cudaError_t hx_loop_condition(const int *remaining, cudaGraphConditionalHandle loop, int *count, int cap, cudaStream_t s);
