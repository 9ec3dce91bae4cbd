// The iterator on the device: after every iteration one thread per molecule
// applies the stop rules of gIterator.f90:88-210 (converged, diverged,
// stagnated, maximum iterations, stop request) and, in mixed precision, the
// phase ladder (3-, 4-, 5-slice tensor-core iterations handing over to the
// FP64-accurate check), the DIIS gate and the purge of vectors made in a
// finished cheaper phase. It writes the launch masks of the next iteration,
// counts the molecules that run each phase next and those still running, and
// appends the molecule's trace record, so the host replays a captured
// iteration and only reads the running count every few iterations.
#include "hx_common.cuh"
#include "hx_plan.h"
#include "hx_kernels.h"

namespace {
enum { PH_FP64 = 0, PH_EXACT = 1, PH_HIGH = 2, PH_MID = 3, PH_LOW = 4, PH_COUNT = 5 };

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// the stop rules of the generic iterator (gIterator.f90:88-210)
__device__ int rules_update(CtlMol &c, double acc, const CtlParams &P, bool cancel)
{
    ++c.iteration;
    const double previous = c.current;
    c.current = acc;
    if (c.current < previous) ++c.successful;
    if (cancel) return HX_INTERRUPTED;
    if (c.current < P.eps) return HX_CONVERGED;
    if (!(c.current == c.current)) return HX_DIVERGED;
    if (P.check_div && c.current > P.div_thr) return HX_DIVERGED;
    if (c.iteration + 1 > P.maxiter) return HX_FAILED_MAXITER;
    if (P.check_stag && c.iteration > P.stag_after && 100.0 * c.successful / c.iteration <= P.stag_thr)
        return HX_STAGNATED;
    return 0;
}

__global__ void k_control(const CCMol *__restrict__ mols, const DiisMol *__restrict__ diis, CtlMol *__restrict__ ctl,
                          CtlParams P, const volatile int *cancel_flag, const unsigned long long *__restrict__ t0,
                          int *__restrict__ active, int *__restrict__ act_ph, double *__restrict__ gate,
                          double *__restrict__ trace, int *__restrict__ remaining, int *__restrict__ occ)
{
    const int mi = blockIdx.x * blockDim.x + threadIdx.x;
    if (mi >= P.nmol) return;
    CtlMol c = ctl[mi];
    if (!c.active) return;
    const double *r = mols[mi].res;
    const double a = fmax(r[0], r[1]);
    const int ph = c.phase;
    const bool cancel = *cancel_flag != 0;
    if (c.ntrace < P.trace_cap) {
        double *t = trace + ((long long)mi * P.trace_cap + c.ntrace) * 5;
        t[0] = r[0]; t[1] = r[1]; t[2] = r[2];
        t[3] = (double)(gtimer() - *t0) * 1e-9;
        t[4] = (double)ph;
        ++c.ntrace;
    }
    const DiisMol &h = diis[mi];
    const int nd = h.nd;
    if (P.diis_enabled && a >= gate[mi]) {          // the step pushed (t, error) into the ring
        c.slot_phase[c.dcount % nd] = (signed char)ph;
        ++c.dcount;
    }
    if (P.mixed) {
        // vectors of a finished cheaper phase leave the extrapolation once the
        // residual is below purge x the level at which that phase ended: their
        // Gram row and column are cleared and the diagonal made huge
        const int valid = (int)(c.dcount < nd ? c.dcount : nd);
        for (int p2 = PH_HIGH; p2 < PH_COUNT; ++p2) {
            if (!(c.ph_end[p2] > 0.0) || !(a < P.purge * c.ph_end[p2])) continue;
            for (int k = 0; k < valid; ++k) {
                if (c.slot_phase[k] != p2) continue;
                for (int q = 0; q < nd; ++q) h.gram[k * nd + q] = h.gram[q * nd + k] = 0.0;
                h.gram[k * nd + k] = 1e100;
                c.slot_phase[k] = -1;
            }
            c.ph_end[p2] = -1.0;
        }
    }
    if (ph >= PH_HIGH && !cancel) {
        // tensor-core phases never claim convergence: they hand over
        if (a < c.best) { c.best = a; c.stall = 0; } else ++c.stall;
        const double fin = P.high_margin * c.fin_scale * P.eps;
        const double below = ph == PH_LOW ? P.mixed_switch : ph == PH_MID ? P.mid_span * P.mixed_switch : 0.0;
        const bool stalled = c.stall >= P.patience;
        int next = ph;
        if (a < fin) next = P.check_ph;
        else if (a < below || stalled) next = ph == PH_HIGH ? P.check_ph : ph - 1;
        const int s = rules_update(c, next != ph ? fmax(a, P.eps * 2) : a, P, false);
        if (s == HX_DIVERGED || s == HX_STAGNATED || s == HX_FAILED_MAXITER) {
            c.status = s;
            c.active = 0;
        } else if (next != ph) {
            c.phase = next;
            c.stall = 0;
            c.best = 1e300;
            c.ph_end[ph] = a;
            // HIGH stalled above its hand-over target: the check phase iterates on
            if (ph == PH_HIGH && a >= fin) c.fp_returns = P.max_returns;
            if (stalled && a >= fin && ph != PH_HIGH) {              // LOW or MID: restart DIIS
                h.count[0] = 0;
                c.dcount = 0;
                for (int k = 0; k < HX_MAX_DIIS; ++k) c.slot_phase[k] = -1;
                for (int k = 0; k < PH_COUNT; ++k) c.ph_end[k] = 0.0;
            }
        }
    } else {
        const int s = rules_update(c, a, P, cancel);
        if (s != 0) {
            c.status = s;
            c.active = 0;
        } else if (P.mixed && c.fp_returns < P.max_returns) {
            // the check did not confirm convergence: more 5-slice iterations to a
            // 10x tighter target, then check again
            c.phase = PH_HIGH;
            c.fin_scale *= 0.1;
            ++c.fp_returns;
            c.stall = 0;
            c.best = 1e300;
        } else if (P.mixed && ph == PH_EXACT) {
            if (a < c.best) { c.best = a; c.stall = 0; }
            else if (++c.stall >= P.patience) { c.phase = PH_FP64; c.stall = 0; }
        }
    }
    if (!c.active) atomicSub(remaining, 1);
    else atomicAdd(&occ[c.phase], 1);                 // the next iteration runs this phase
    gate[mi] = (P.mixed && c.phase >= PH_HIGH) ? P.high_margin * c.fin_scale * P.eps : P.eps;
    active[mi] = c.active;
    if (act_ph)
        for (int p = 0; p < PH_COUNT; ++p) act_ph[p * P.nmol + mi] = c.active && c.phase == p;
    ctl[mi] = c;
}

__global__ void k_control_start(unsigned long long *t0) { *t0 = gtimer(); }

// First node of a captured iteration: each phase's conditional body runs only
// if some molecule is in that phase (counted by the last iteration's
// k_control); the counts start again from zero, and runs[p] counts the
// iterations in which phase p ran.
// (one handle per conditional node; entries with phase < 0 are unused)
__global__ void k_phase_conditions(int *occ, const PhaseCondition *hs, int n, int *runs)
{
    unsigned int on[5];
    for (int p = 0; p < 5; ++p) { on[p] = occ[p] > 0 ? 1u : 0u; occ[p] = 0; runs[p] += (int)on[p]; }
    for (int k = 0; k < n; ++k)
        if (hs[k].phase >= 0) cudaGraphSetConditional(hs[k].handle, on[hs[k].phase]);
}

// Last node of the loop body: run the body again while a molecule is still
// running, and never more than cap times (count is cleared before the launch).
__global__ void k_loop_condition(const int *remaining, cudaGraphConditionalHandle loop, int *count, int cap)
{
    const int n = ++*count;
    cudaGraphSetConditional(loop, (*remaining > 0 && n < cap) ? 1u : 0u);
}
}  // namespace

cudaError_t hx_loop_condition(const int *remaining, cudaGraphConditionalHandle loop, int *count, int cap, cudaStream_t s)
{
    k_loop_condition<<<1, 1, 0, s>>>(remaining, loop, count, cap);
    hx_count_launches(1);
    return cudaGetLastError();
}

cudaError_t hx_control_start(unsigned long long *d_t0, cudaStream_t s)
{
    k_control_start<<<1, 1, 0, s>>>(d_t0);
    hx_count_launches(1);
    return cudaGetLastError();
}

cudaError_t hx_phase_conditions(int *occ, const PhaseCondition *hs, int n, int *runs, cudaStream_t s)
{
    k_phase_conditions<<<1, 1, 0, s>>>(occ, hs, n, runs);
    hx_count_launches(1);
    return cudaGetLastError();
}

cudaError_t hx_control(const CCMol *mols, const DiisMol *diis, CtlMol *ctl, const CtlParams &P, const volatile int *cancel_flag,
                       const unsigned long long *t0, int *active, int *act_ph, double *gate, double *trace,
                       int *remaining, int *occ, cudaStream_t s)
{
    k_control<<<(P.nmol + 63) / 64, 64, 0, s>>>(mols, diis, ctl, P, cancel_flag, t0, active, act_ph, gate, trace,
                                                remaining, occ);
    hx_count_launches(1);
    return cudaGetLastError();
}
