// Per-molecule device views shared by the kernels and the host plan.
#pragma once
#include <vector>
#include "hx_common.cuh"

#define HX_SCF_GRID_MAX 152    // CTAs of the cooperative SCF (global partials are sized for it)
#define HX_MAX_DIIS 50         // largest coupled-cluster:diis-steps (definebd.f90: range 2..50)

struct ScfParams {
    int maxiter;
    double eps, step, divergence, stag_pct;
    int stag_after, check_div, check_stag;
};

// One molecule's SCF state in device memory (row-major N x N matrices).
struct ScfMol {
    int N, nocc;
    const double *core, *G, *huckel;
    const double *D0, *V0;          // optional warm start (density and basis)
    double *F, *D, *V, *E, *A, *W1, *W2, *Fmo;
    double *out;                    // [0] E_total [1] E_el [2] E_nuc [3] last accuracy
    int *status;                    // [0] status [1] iterations
};

// One molecule's CCSD state. Pair layout: X[i][a][j][b] for o x v x o x v
// tensors, i.e. a (o*v) x (o*v) matrix over excitations (ia) with the
// reference's order (i outer, a inner). Site-basis factors are [site][...].
struct CCMol {
    int N, o, v;
    int pad_;
    // constants of the molecule (after SCF)
    const double *Cmo, *G, *h, *Fmo;      // N x N
    double *Bov0, *GBov0;                 // [N][o*v]  C_mu,k C_mu,c and G . it
    double *gov, *Lov;                    // pair: (kc|ld), 2(kc|ld)-(kd|lc)
    double *D1, *D2;                      // denominators F_ii-F_aa, F_ii+F_jj-F_aa-F_bb
    // amplitudes and residuals
    double *t1, *t2, *r1, *r2, *u;
    // T1-dressed factors
    double *X, *Y, *Pm, *H2, *W1, *Fd;    // N x N
    double *Bia, *GBia;                   // [N][o*v]  X_mu,a Y_mu,i (index i*v+a)
    double *Boo, *GBoo;                   // [N][o*o]  X_mu,k Y_mu,i (index k*o+i)
    double *Bvv, *GBvv;                   // [N][v*v]  X_mu,a Y_mu,c (index a*v+c)
    // contraction scratch
    double *T1s, *Ts, *Z, *Woo;           // ladder: o*v*o*N, o*N*o*N, Ts X: o*N*o*N, o^4
    double *Vvv;                          // MO-basis ladder integrals (ac|bd)~ [(a c)][(b d)], v^4
                                          // (small molecules in mixed precision; else null)
    double *Cint, *Cp, *Dint, *X2;        // o^2 v^2 each
    double *Fvv2, *Foo2;                  // v*v, o*o
    double *U, *UG, *Vs;                  // [o*v][N], [o*v][N], [o][N]
    // results of the iteration (device): [0] max|d1| [1] max|d2| [2] E_total
    // [3] E_ref [4] 2 sum F t1 [5] doubles part
    double *res;
    double eref;
};

// DIIS history of one molecule: nd slots of the amplitude vector (t1, t2) and
// of the error vector (d1, 3*Omega2 or d2), used as a ring (slot = count % nd).
// A vector holds what the reference's packed vectors hold, the singles and the
// pairs (ia) <= (jb), blocked: t1 (o*v), then the v x v blocks [a][b] of the
// occupied pairs i <= j in row-major order of that triangle, so
// L = o*v + v*v*o(o+1)/2 (a diagonal block i = j carries both (ia,ib) and
// (ib,ia), which are equal). gram is nd x nd in slot order; coef holds
// HX_MAX_DIIS+2 doubles: the mixing coefficients by slot, then how many
// vectors to mix (1: none, take the newest) and the newest slot.
struct DiisMol {
    double *Ht, *He, *gram, *coef;
    int *count;
    int nd;
    long long L;
};

// One grouped tensor-GEMM launch of the plan (descriptors on host and device).
struct Group {
    std::vector<TgemmDesc> h;
    TgemmDesc *d = nullptr;
    long long tiles = 0;
};

// ---------------------------------------------------------------- schedules
// Launches over a batch give every molecule blocks in proportion to its work
// (prefix sums of blocks per molecule, `start[nmol + 1]`), so molecules of 8
// and of 160 sites finish together. Element-wise kinds cover HX_EW_CHUNK
// elements per block; the pair-unit kinds cover one unit: the singles, or a
// group of v x v pair blocks (i, j) of about HX_UNIT_ELEMS elements.
#define HX_EW_CHUNK 2048
#define HX_UNIT_ELEMS 1024
#define HX_PART_STRIDE (2 + HX_MAX_DIIS)   // partials per unit: two maxima or sums, then DIIS dots

enum { SK_NN, SK_ZDO, SK_PAIR, SK_ONON, SK_FOCK, SK_SETUP, SK_UP, SK_FULL, SK_COUNT };

struct HxSched {
    const int *start[SK_COUNT];    // device: first block of each molecule, then the total
    long long blocks[SK_COUNT];    // host: the total
    int nmol;
    int vmax;                      // largest v of the batch (tile size of the pair-unit kernels)
};

__host__ __device__ inline int hx_unit_blocks(int v)   // v x v blocks per pair unit (1..64)
{
    const int g = HX_UNIT_ELEMS / (v * v);
    return g < 1 ? 1 : (g > 64 ? 64 : g);
}
// doubles of shared memory one pair-unit tile takes ([block][a][b], rows of v + 1)
__host__ __device__ inline long long hx_unit_tile(int o, int v)
{
    const long long t = (long long)hx_unit_blocks(v) * v * (v + 1);
    return t > (long long)o * v ? t : (long long)o * v;      // the singles unit stages o*v values
}
// units of a molecule: the singles unit, then the upper-triangle (i <= j)
// blocks (SK_UP) or all o*o blocks (SK_FULL) in groups of hx_unit_blocks(v)
__host__ __device__ inline long long hx_units(int o, int v, bool upper)
{
    const long long nb = upper ? (long long)o * (o + 1) / 2 : (long long)o * o;
    const int g = hx_unit_blocks(v);
    return 1 + (nb + g - 1) / g;
}

// ---------------------------------------------------------------- device-side iterator
// The state of the iterator (gIterator.f90:88-210) and of the mixed-precision
// phase ladder of one molecule, kept on the device so that a solve runs
// without a host round trip per iteration (k_control, hx_control.cu).
struct CtlMol {
    int iteration, successful, status, active, phase, stall, fp_returns, ntrace;
    long long dcount;                  // DIIS pushes so far
    double current, best, fin_scale;
    double ph_end[5];                  // residual at which each phase ended (0 not ended, -1 purged)
    signed char slot_phase[HX_MAX_DIIS];   // phase that produced each DIIS slot (-1 empty or purged)
};

struct CtlParams {
    int nmol, maxiter, mixed, check_ph, patience, max_returns, diis_enabled;
    int check_div, check_stag, stag_after, trace_cap;
    double eps, mixed_switch, mid_span, high_margin, purge, div_thr, stag_thr;
};
