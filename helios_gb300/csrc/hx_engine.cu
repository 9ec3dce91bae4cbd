// Host side of the engine: PPP model, device state, the contraction plan of one
// CCSD iteration, the iterator, and the C ABI of include/helios_cc.h.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/helios_cc.h"
#include "hx_kernels.h"
#include "hx_layout.h"
#include "hx_mlp.h"
#include "hx_tc.h"

cudaError_t hx_mlp_sample(const CCMol *d_mols, int mol, const long long *d_rows, int n, float *dX, float *dT,
                          cudaStream_t s);

// ---------------------------------------------------------------- errors
static thread_local char g_err[1024];
static std::atomic<long long> g_launches{0};

void hx_count_launches(int n) { g_launches.fetch_add(n); }

void hx_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

#define HX_TRY(expr)                                  \
    do {                                              \
        int rc_ = (expr);                             \
        if (rc_ < 0) return rc_;                      \
    } while (0)

#define HX_CU(call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            hx_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return HX_ERR_CUDA;                                                              \
        }                                                                                    \
    } while (0)

// ---------------------------------------------------------------- PPP model
// src/modules/mod_helios.f90:42-43
static const double kBohr = 0.52917721067, kHartree = 27.21138602;

struct HostModel {
    int N = 0, nel = 0;
    std::vector<double> coords, G, core, huckel;
};

// readMoleculeInformation.f90:20-159 + gamma :216-264 + perturbate
// (mod_helios.f90:577-601) with the diagonal field of setCore/applyField.
static int build_model(const hx_ppp_model *m, const hx_cc_params *p, HostModel &out)
{
    const int n = m->n_sites;
    if (n < 2 || n > HX_MAX_MOL_N) {
        hx_set_error("n_sites=%d outside 2..%d", n, HX_MAX_MOL_N);
        return HX_ERR_ARG;
    }
    if (!m->coords || !m->alpha || !m->gamma || !m->nels || (m->n_bonds > 0 && (!m->bond_i || !m->bond_j || !m->beta))) {
        hx_set_error("model with NULL arrays");
        return HX_ERR_ARG;
    }
    out.N = n;
    out.nel = 0;
    for (int i = 0; i < n; ++i) out.nel += m->nels[i];
    if (out.nel % 2 || out.nel <= 0 || out.nel >= 2 * n) {
        hx_set_error("closed-shell r-ccsd needs an even electron count in 2..2N-2 (got %d for N=%d)", out.nel, n);
        return HX_ERR_ARG;
    }
    out.coords.assign(m->coords, m->coords + 3 * n);
    double cen[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) cen[k] += out.coords[3 * i + k];
    for (int k = 0; k < 3; ++k) cen[k] /= n;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) out.coords[3 * i + k] -= cen[k];
    const double tr = 1.0 / (kBohr * kHartree);
    out.G.assign((size_t)n * n, 0.0);
    for (int a = 0; a < n; ++a)
        for (int b = a; b < n; ++b) {
            double d2 = 0;
            for (int k = 0; k < 3; ++k) {
                double x = out.coords[3 * a + k] - out.coords[3 * b + k];
                d2 += x * x;
            }
            double r = std::sqrt(d2), med = (m->gamma[a] + m->gamma[b]) / 2.0, g = 0.0;
            if (p->coulomb == HX_COULOMB_OHNO_KLOPMAN) g = med / std::sqrt(1.0 + (tr * med * r) * (tr * med * r));
            else if (p->coulomb == HX_COULOMB_MATAGA_NISHIMOTO) g = med / (1.0 + tr * med * r);
            else if (p->coulomb == HX_COULOMB_HUBBARD) g = (a == b) ? m->gamma[a] : 0.0;
            else { hx_set_error("unknown coulomb type %d", p->coulomb); return HX_ERR_ARG; }
            out.G[(size_t)a * n + b] = out.G[(size_t)b * n + a] = g;
        }
    std::vector<double> connect((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) connect[(size_t)i * n + i] = m->alpha[i];
    for (int k = 0; k < m->n_bonds; ++k) {
        int i = m->bond_i[k], j = m->bond_j[k];
        if (i < 0 || j < 0 || i >= n || j >= n) { hx_set_error("bond %d joins invalid sites", k); return HX_ERR_ARG; }
        connect[(size_t)i * n + j] = connect[(size_t)j * n + i] = m->beta[k];
    }
    if (p->bond_alternation != 0.0) {
        for (int k = 0; k < m->n_bonds; ++k) {
            int i = m->bond_i[k], j = m->bond_j[k];
            int kind = m->bond_kind ? m->bond_kind[k] : HX_BOND_NONSET;
            if (kind == HX_BOND_NONSET) break;   // the reference leaves the rest unscaled
            double f = (kind == HX_BOND_DOUBLE) ? 1.0 + p->bond_alternation : 1.0 - p->bond_alternation;
            connect[(size_t)i * n + j] = connect[(size_t)j * n + i] = m->beta[k] * f;
        }
    }
    out.core = connect;
    for (int k = 0; k < n; ++k) {
        double s = 0;
        for (int l = 0; l < n; ++l)
            if (l != k) s += m->nels[l] * out.G[(size_t)k * n + l];
        out.core[(size_t)k * n + k] -= s;
    }
    out.huckel = connect;
    for (int mu = 0; mu < n; ++mu) {
        double pert = 0;
        for (int k = 0; k < 3; ++k) pert += p->field[k] * out.coords[3 * mu + k];
        out.core[(size_t)mu * n + mu] += pert;
        out.huckel[(size_t)mu * n + mu] += pert;
    }
    return HX_OK;
}

// ---------------------------------------------------------------- arena
struct Arena {
    size_t used = 0;
    char *base = nullptr;
    // first pass counts (base == nullptr), second pass hands out pointers
    template <class T> T *take(size_t count)
    {
        size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
        T *p = base ? reinterpret_cast<T *>(base + used) : nullptr;
        used += bytes;
        return p;
    }
};

// ---------------------------------------------------------------- iterator rules
struct Rules {   // gIterator.f90:88-210
    int iteration = 0, successful = 1;
    double current = 0.0;
    int update(double acc, const hx_cc_params &p, int maxiter, double eps, bool cancel)
    {
        ++iteration;
        double previous = current;
        current = acc;
        if (current < previous) ++successful;
        if (cancel) return HX_INTERRUPTED;
        if (current < eps) return HX_CONVERGED;
        if (!(current == current)) return HX_DIVERGED;
        if (p.check_divergence && current > p.divergence_threshold) return HX_DIVERGED;
        if (iteration + 1 > maxiter) return HX_FAILED_MAXITER;
        if (p.check_stagnation && iteration > p.stagnation_after &&
            100.0 * successful / iteration <= p.stagnation_threshold) return HX_STAGNATED;
        return 0;
    }
};

enum { PH_FP64 = 0, PH_EXACT = 1, PH_HIGH = 2, PH_MID = 3, PH_LOW = 4, PH_COUNT = 5 };
// tensor-core mode (tc::run_group) of a phase: LOW 0, MID 1, HIGH 2, EXACT 3
static inline int tc_mode(int ph) { return PH_LOW - ph; }

struct hx_ccsd {
    hx_cc_params p{};
    int nmol = 0;
    std::vector<HostModel> models;
    std::vector<int> N, o, v;
    cudaStream_t st = nullptr;
    char *arena = nullptr;
    size_t arena_bytes = 0;
    // device views
    std::vector<ScfMol> scf;
    std::vector<CCMol> cc;
    std::vector<DiisMol> diis;
    ScfMol *d_scf = nullptr;
    CCMol *d_cc = nullptr;
    DiisMol *d_diis = nullptr;
    int *d_active = nullptr;
    std::vector<int> active;
    double *d_gate = nullptr;            // per molecule: residual below which the DIIS step is skipped
    std::vector<double> gate;
    double gate_eps = 0.0;               // convergence target the gates were made for
    double *d_part = nullptr;
    double *d_res = nullptr;             // nmol x 8 iteration results (inside the arena)
    HxSched sched{};                     // balanced launch schedules of the batch (hx_plan.h)
    int *d_sched = nullptr;
    size_t unit_smem[3] = {0, 0, 0};     // dynamic shared memory of the pair-unit kernels
    std::vector<Group> plan;             // GEMM groups of one iteration (in order)
    std::vector<Group> setup_groups;
    long long maxw_oNoN = 0;
    bool initialized = false;
    std::atomic<int> cancel{0};
    // per molecule host results
    std::vector<double> res;             // nmol x 6
    std::vector<Rules> rules;
    std::vector<int> status;
    std::vector<int> scf_failed;         // batches: molecules whose SCF did not converge are left out
    tc::Engine *tce = nullptr;           // tensor-core backend (mixed precision)
    mlp::Model *model = nullptr;         // learned T2 guess (guess = 1)
    // mixed precision: per-molecule phase (PH_LOW / PH_MID / PH_HIGH / PH_EXACT
    // tensor-core iterations, PH_FP64 CUDA-core FP64) and one launch mask per phase
    std::vector<int> phase, stall;
    std::vector<double> best;
    std::vector<double> fin_scale;       // mixed: tightening of the hand-over target after a failed FP64 check
    std::vector<int> fp_returns;          // mixed: checks that sent a molecule back to 5-slice iterations
    // host mirror of each molecule's DIIS ring: pushes so far and the phase
    // that produced each slot (-1 empty or purged); residual at which each
    // phase ended (0 = not ended, -1 = its vectors purged)
    std::vector<long long> dcount;
    std::vector<std::vector<int>> slot_phase;
    std::vector<std::array<double, PH_COUNT>> ph_end;
    int *d_act_ph[PH_COUNT] = {};        // one launch mask per phase, contiguous ([phase][molecule])
    // device-side iterator of solve_all (hx_control.cu)
    CtlMol *d_ctl = nullptr;
    double *d_trace = nullptr;           // [molecule][trace_cap][5]
    int trace_cap = 0;
    int *d_remaining = nullptr, *d_occ = nullptr, *d_loops = nullptr;   // one block: [0], [2..6], [7],
    int *d_runs = nullptr;                                              // [8..12] iterations per phase
    long long phase_nodes[5] = {};       // kernels captured in each phase's conditional bodies
    int *d_cancel = nullptr;             // device address of h_pinned[8] (mapped host memory)
    unsigned long long *d_t0 = nullptr;
    double *h_amp = nullptr;             // pinned staging of hx_ccsd_set_guess / hx_ccsd_get_amplitudes
    size_t h_amp_elems = 0;
    int *h_pinned = nullptr;             // pinned, mapped: [0..7] mirror of that block ([0] molecules
                                         // still running, [2..6] per phase next), [8] the stop request
                                         // (read by the device)
    bool device_ctl = false;             // solve_all: the device decides phases and masks
    bool capturing = false;              // iteration_body is being captured: phases become conditional nodes
    bool profiling = false;              // per-launch GEMM timing: iterations are launched one by one
    cudaStream_t st2 = nullptr;          // captures the bodies of the conditional nodes
    // conditional handles of a captured iteration, one per conditional node
    // (a plan group's launches of one phase), made as the nodes are captured
    std::vector<PhaseCondition> cond;
    PhaseCondition *d_cond = nullptr;    // room for one per (plan group, phase)
    std::vector<std::vector<std::array<double, 5>>> trace;
    // device time of the last hx_ccsd_init and solve (events on st)
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float init_ms = 0.f, solve_ms = 0.f;
    double prof[4] = {0, 0, 0, 0};
};

// ---------------------------------------------------------------- plan helpers
static TgemmDesc tg(const double *A, const double *B, double *C, int batch, int M, int N, int K, int Mi,
                    int Ni, int Ki, std::initializer_list<long long> a, std::initializer_list<long long> b,
                    std::initializer_list<long long> c, double alpha, double beta, int mol)
{
    TgemmDesc d;
    memset(&d, 0, sizeof(d));
    d.A = A; d.B = B; d.C = C;
    d.batch = batch; d.M = M; d.N = N; d.K = K; d.Mi = Mi; d.Ni = Ni; d.Ki = Ki;
    std::copy(a.begin(), a.end(), d.a);
    std::copy(b.begin(), b.end(), d.b);
    std::copy(c.begin(), c.end(), d.c);
    d.alpha = alpha; d.beta = beta; d.mol = mol;
    return d;
}

// Operands that stay fixed between hx_ccsd_init calls: the tensor-core
// backend slices them once per initialisation.
static void mark_constants(hx_ccsd *h)
{
    for (auto &g : h->plan)
        for (auto &d : g.h) {
            const CCMol &m = h->cc[d.mol];
            auto fixed = [&](const double *p) {
                const double *lo[] = {m.Cmo, m.G, m.gov, m.Lov, m.Bov0, m.GBov0};
                const size_t n[] = {(size_t)m.N * m.N, (size_t)m.N * m.N, (size_t)m.o * m.v * m.o * m.v,
                                    (size_t)m.o * m.v * m.o * m.v, (size_t)m.N * m.o * m.v, (size_t)m.N * m.o * m.v};
                for (int k = 0; k < 6; ++k)
                    if (p >= lo[k] && p < lo[k] + n[k]) return 1;
                return 0;
            };
            d.a_const = fixed(d.A);
            d.b_const = fixed(d.B);
        }
}

static int upload_group(Group &g)
{
    g.tiles = hx_tgemm_f64_prepare(g.h.data(), (int)g.h.size());
    if (g.h.empty()) return HX_OK;
    HX_CU(cudaMalloc(&g.d, sizeof(TgemmDesc) * g.h.size()));
    HX_CU(cudaMemcpy(g.d, g.h.data(), sizeof(TgemmDesc) * g.h.size(), cudaMemcpyHostToDevice));
    return HX_OK;
}

// While an iteration is captured: a conditional (if) node on phase ph's
// condition is added to the capture, and body(s2) is captured into its graph.
template <class F>
static int with_condition(hx_ccsd *h, int ph, F body)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t nd = 0;
    HX_CU(cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, &deps, &edges, &nd));
    alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)] = {};   // (no default constructor)
    cudaGraphNodeParams &np = *reinterpret_cast<cudaGraphNodeParams *>(raw);
    np.type = cudaGraphNodeTypeConditional;
    PhaseCondition pc;
    memset(&pc, 0, sizeof(pc));
    pc.phase = ph;
    HX_CU(cudaGraphConditionalHandleCreate(&pc.handle, g, 0, 0));
    if (h->cond.size() >= h->plan.size() * PH_COUNT) { hx_set_error("too many conditional nodes"); return HX_ERR_STATE; }
    h->cond.push_back(pc);
    np.conditional.handle = pc.handle;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    HX_CU(cudaGraphAddNode(&node, g, deps, edges, nd, &np));
    HX_CU(cudaStreamUpdateCaptureDependencies(h->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    HX_CU(cudaStreamBeginCaptureToGraph(h->st2, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal));
    const long long before = g_launches.load();
    const cudaError_t e = body(h->st2);
    h->phase_nodes[ph] += g_launches.load() - before;
    cudaGraph_t out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(h->st2, &out);
    HX_CU(e);
    HX_CU(e2);
    return HX_OK;
}

// Each molecule runs the group in its current phase: the tensor-core modes
// on tcgen05, FP64 on the CUDA-core kernel; one launch per phase in use, with
// that phase's mask (every launch skips the molecules that are not its own).
static int run_group(hx_ccsd *h, Group &g)
{
    if (g.tiles == 0) return HX_OK;
    if (h->tce) {
        int n[PH_COUNT] = {};
        for (int mi = 0; mi < h->nmol; ++mi)
            if (h->active[mi]) ++n[h->phase[mi]];
        if (h->device_ctl && h->capturing) {
            // each phase's launches become the body of a conditional node that
            // runs only when some molecule is in that phase this iteration
            for (int ph = 0; ph < PH_COUNT; ++ph)
                HX_TRY(with_condition(h, ph, [&](cudaStream_t s2) {
                    if (ph == PH_FP64) return hx_tgemm_f64_launch(g.d, (int)g.h.size(), g.tiles, h->d_act_ph[PH_FP64], s2);
                    return tc::run_group(h->tce, g.h.data(), (int)g.h.size(), h->d_act_ph[ph], s2, tc_mode(ph));
                }));
            return HX_OK;
        }
        if (h->device_ctl)                       // the phases the device counted for this iteration
            for (int ph = 0; ph < PH_COUNT; ++ph) n[ph] = h->h_pinned[2 + ph];
        for (int ph = PH_LOW; ph >= PH_EXACT; --ph) {
            if (!n[ph]) continue;
            cudaError_t e = tc::run_group(h->tce, g.h.data(), (int)g.h.size(), h->d_act_ph[ph], h->st, tc_mode(ph));
            if (e != cudaSuccess) { hx_set_error("tensor-core group: %s", cudaGetErrorString(e)); return HX_ERR_CUDA; }
        }
        if (n[PH_FP64]) HX_CU(hx_tgemm_f64_launch(g.d, (int)g.h.size(), g.tiles, h->d_act_ph[PH_FP64], h->st));
        return HX_OK;
    }
    HX_CU(hx_tgemm_f64_launch(g.d, (int)g.h.size(), g.tiles, h->d_active, h->st));
    return HX_OK;
}

// Mixed precision: a tensor-core phase hands over to FP64 once its residual
// is below kHighMargin * eps (times the molecule's fin_scale).
static const double kHighMargin = 0.1;
// A tensor-core phase keeps the DIIS extrapolation down to its hand-over
// target: below eps, plain steps (the reference's converged case) throw the
// residual back up by several times and the phase wanders for tens of
// iterations before it reaches kHighMargin * eps.
static double diis_gate(const hx_ccsd *h, int mi)
{
    if (h->tce && h->phase[mi] >= PH_HIGH) return kHighMargin * h->fin_scale[mi] * h->gate_eps;
    return h->gate_eps;
}

// The phase of iterations driven from the host (hx_ccsd_iterate) and the one a
// handle returns to after a solve: the 7-slice phase for HX_PRECISION_EXACT
// (every iteration of such a handle is one), FP64 otherwise (the mixed ladder
// belongs to hx_ccsd_solve).
static int idle_phase(const hx_ccsd *h)
{
    return h->p.precision == HX_PRECISION_EXACT ? PH_EXACT : PH_FP64;
}

static int upload_masks(hx_ccsd *h)
{
    for (int mi = 0; mi < h->nmol; ++mi) h->gate[mi] = diis_gate(h, mi);
    HX_CU(cudaMemcpyAsync(h->d_gate, h->gate.data(), sizeof(double) * h->nmol, cudaMemcpyHostToDevice, h->st));
    std::vector<int> m((size_t)PH_COUNT * h->nmol);
    for (int ph = 0; ph < PH_COUNT; ++ph)
        for (int mi = 0; mi < h->nmol; ++mi) m[(size_t)ph * h->nmol + mi] = h->active[mi] && h->phase[mi] == ph;
    HX_CU(cudaMemcpyAsync(h->d_active, h->active.data(), sizeof(int) * h->nmol, cudaMemcpyHostToDevice, h->st));
    if (h->d_act_ph[0])
        for (int ph = 0; ph < PH_COUNT; ++ph)
            HX_CU(cudaMemcpyAsync(h->d_act_ph[ph], &m[(size_t)ph * h->nmol], sizeof(int) * h->nmol,
                                  cudaMemcpyHostToDevice, h->st));
    // the masks and gates are pageable host vectors: wait so they may change
    HX_CU(cudaStreamSynchronize(h->st));
    return HX_OK;
}

// The particle-particle ladder and the t2 part of the hole-hole intermediate
// go through the site basis (four and two GEMMs of K = v or N: o^2 (v^2 N +
// v N^2) flops instead of o^2 v^4). For small molecules on the tensor cores
// those GEMMs are single k-block tiles that the MMAs barely use, so up to
// kMoLadderMaxV virtual orbitals the mixed path builds (ac|bd)~ (v^2 x v^2 x
// N) and does both terms as two deep GEMMs in the MO basis (o^2 x v^2 x v^2
// and o^2 x o^2 x v^2): more flops, far fewer and fuller tiles. FP64
// iterations keep the site basis, which has the fewest flops.
static const int kMoLadderMaxV = 32;
static bool mo_ladder(const hx_ccsd *h, int mi)
{
    return h->p.precision != HX_PRECISION_FP64 && h->v[mi] <= kMoLadderMaxV;
}

// Descriptors of every contraction of one iteration, for every molecule.
// Index conventions are spelled out in hx_plan.h; each block cites the term
// of the T1-dressed closed-shell CCSD equations it evaluates.
static void build_plan(hx_ccsd *h)
{
    enum { G_DRESS_XY, G_DRESS_P, G_FD1, G_FD2, G_GB, G_LEAD, G_LAD_A, G_LAD_B, G_LAD_D, G_LAD_E, G_W_D,
           G_W_E, G_W_INT, G_HH, G_CINT1, G_CINT2, G_CTERM, G_DINT1, G_DINT2, G_DINT3, G_DTERM, G_FVOO,
           G_E1, G_E2, G_S1, G_S_UG, G_S_V, G_S_R1, G_COUNT };
    h->plan.assign(G_COUNT, Group());
    auto &P = h->plan;
    for (int mi = 0; mi < h->nmol; ++mi) {
        const CCMol &m = h->cc[mi];
        const int N = m.N, o = m.o, v = m.v, ov = o * v;
        const double *Cmo = m.Cmo, *G = m.G;
        // T1 dressing: X = [Co | Cv - Co t1], Y = [Co + Cv t1^T | Cv]
        P[G_DRESS_XY].h.push_back(tg(Cmo, m.t1, m.X + o, 1, N, v, o, N, v, o, {0, N, 0, 1, 0}, {0, 1, 0, v, 0}, {0, N, 0, 1, 0}, -1.0, 1.0, mi));
        P[G_DRESS_XY].h.push_back(tg(Cmo + o, m.t1, m.Y, 1, N, o, v, N, o, v, {0, N, 0, 1, 0}, {0, v, 0, 1, 0}, {0, N, 0, 1, 0}, 1.0, 1.0, mi));
        // Pm = Yo Xo^T (dressed half density)
        P[G_DRESS_P].h.push_back(tg(m.Y, m.X, m.Pm, 1, N, N, o, N, N, o, {0, N, 0, 1, 0}, {0, N, 0, 1, 0}, {0, N, 0, 1, 0}, 1.0, 0.0, mi));
        // Fd = X^T H2 Y
        P[G_FD1].h.push_back(tg(m.H2, m.Y, m.W1, 1, N, N, N, N, N, N, {0, N, 0, 1, 0}, {0, 1, 0, N, 0}, {0, N, 0, 1, 0}, 1.0, 0.0, mi));
        P[G_FD2].h.push_back(tg(m.X, m.W1, m.Fd, 1, N, N, N, N, N, N, {0, 1, 0, N, 0}, {0, 1, 0, N, 0}, {0, N, 0, 1, 0}, 1.0, 0.0, mi));
        // G . B for the dressed ZDO products
        P[G_GB].h.push_back(tg(G, m.Bia, m.GBia, 1, N, ov, N, N, ov, N, {0, N, 0, 1, 0}, {0, 1, 0, ov, 0}, {0, ov, 0, 1, 0}, 1.0, 0.0, mi));
        P[G_GB].h.push_back(tg(G, m.Boo, m.GBoo, 1, N, o * o, N, N, o * o, N, {0, N, 0, 1, 0}, {0, 1, 0, o * o, 0}, {0, o * o, 0, 1, 0}, 1.0, 0.0, mi));
        P[G_GB].h.push_back(tg(G, m.Bvv, m.GBvv, 1, N, v * v, N, N, v * v, N, {0, N, 0, 1, 0}, {0, 1, 0, v * v, 0}, {0, v * v, 0, 1, 0}, 1.0, 0.0, mi));
        // leading term (ai|bj)~ -> r2 (initialises r2)
        P[G_LEAD].h.push_back(tg(m.Bia, m.GBia, m.r2, 1, ov, ov, N, ov, ov, N, {0, 1, 0, ov, 0}, {0, 1, 0, ov, 0}, {0, ov, 0, 1, 0}, 1.0, 0.0, mi));
        // particle-particle ladder through the site basis:
        //   sum_cd (ac|bd)~ t_ij^cd = sum_mu,nu X_mu,a X_nu,b G_mu,nu [sum_cd C_mu,c C_nu,d t_ij^cd]
        const long long vv = (long long)v * v, vov = (long long)v * ov;
        if (mo_ladder(h, mi)) {
            // (ac|bd)~ = sum_mu Bvv[mu][ac] GBvv[mu][bd]; r2_ij^ab += sum_cd (ac|bd)~ t_ij^cd
            P[G_LAD_A].h.push_back(tg(m.Bvv, m.GBvv, m.Vvv, 1, (int)vv, (int)vv, N, (int)vv, (int)vv, N, {0, 1, 0, vv, 0}, {0, 1, 0, vv, 0}, {0, vv, 0, 1, 0}, 1.0, 0.0, mi));
            P[G_LAD_E].h.push_back(tg(m.t2, m.Vvv, m.r2, 1, o * o, (int)vv, (int)vv, o, v, v, {vov, v, ov, 1, 0}, {vv * v, v, vv, 1, 0}, {vov, v, ov, 1, 0}, 1.0, 1.0, mi));
            // W_klij = sum_cd (kc|ld) t_ij^cd into Woo[i][k][j][l] ((ki|lj)~ is added below)
            P[G_W_E].h.push_back(tg(m.gov, m.t2, m.Woo, 1, o * o, o * o, (int)vv, o, o, v, {(long long)v * ov, v, ov, 1, 0}, {vov, v, ov, 1, 0}, {(long long)o * o, 1, (long long)o * o * o, o, 0}, 1.0, 0.0, mi));
        } else {
            P[G_LAD_A].h.push_back(tg(m.t2, Cmo + o, m.T1s, 1, o * v * o, N, v, o * v * o, N, v, {0, v, 0, 1, 0}, {0, N, 0, 1, 0}, {0, N, 0, 1, 0}, 1.0, 0.0, mi));
            P[G_LAD_B].h.push_back(tg(Cmo + o, m.T1s, m.Ts, o, N, o * N, v, N, o * N, v, {0, N, 0, 1, 0}, {0, 1, 0, (long long)o * N, (long long)v * o * N}, {0, (long long)o * N, 0, 1, (long long)N * o * N}, 1.0, 0.0, mi));
            //   Z = Ts X: its virtual columns (X_v = Cv - Co t1) close the ladder, its
            //   occupied ones (X_o = Co exactly: the dressing leaves them) feed the
            //   hole-hole intermediate below -- one product, one slicing of Ts
            P[G_LAD_D].h.push_back(tg(m.Ts, m.X, m.Z, 1, o * N * o, N, N, o * N * o, N, N, {0, N, 0, 1, 0}, {0, 1, 0, N, 0}, {0, N, 0, 1, 0}, 1.0, 0.0, mi));
            P[G_LAD_E].h.push_back(tg(m.X + o, m.Z + o, m.r2, o, v, ov, N, v, v, N, {0, 1, 0, N, 0}, {N, 1, 0, (long long)o * N, (long long)N * o * N}, {0, ov, v, 1, (long long)v * ov}, 1.0, 1.0, mi));
            // hole-hole ladder: W_klij = (ki|lj)~ + sum_cd t_ij^cd (kc|ld), the latter through the site basis
            //   (G_W_D stays empty: Z's occupied columns are the former Zo = Ts Co)
            P[G_W_E].h.push_back(tg(Cmo, m.Z, m.Woo, o, o, o * o, N, o, o, N, {0, 1, 0, N, 0}, {N, 1, 0, (long long)o * N, (long long)N * o * N}, {0, o * o, o, 1, (long long)o * o * o}, 1.0, 0.0, mi));
        }
        P[G_W_INT].h.push_back(tg(m.Boo, m.GBoo, m.Woo, 1, o * o, o * o, N, o, o, N, {o, 1, 0, o * o, 0}, {o, 1, 0, o * o, 0}, {(long long)o * o, (long long)o * o * o, 1, o, 0}, 1.0, 1.0, mi));
        P[G_HH].h.push_back(tg(m.Woo, m.t2, m.r2, 1, o * o, v * v, o * o, o, v, o, {(long long)o * o * o, o, (long long)o * o, 1, 0}, {ov, 1, (long long)v * ov, v, 0}, {(long long)v * ov, v, ov, 1, 0}, 1.0, 1.0, mi));
        // C: Cint_kiac = (ki|ac)~ - 1/2 sum_ld t_li^ad (kd|lc);  C_ij^ab = -sum_kc t_kj^bc Cint_kiac
        P[G_CINT1].h.push_back(tg(m.Boo, m.GBvv, m.Cint, 1, o * o, v * v, N, o * o, v * v, N, {0, 1, 0, o * o, 0}, {0, 1, 0, v * v, 0}, {0, v * v, 0, 1, 0}, 1.0, 0.0, mi));
        P[G_CINT2].h.push_back(tg(m.t2, m.gov, m.Cint, 1, ov, ov, ov, v, v, v, {v, ov, (long long)v * ov, 1, 0}, {(long long)v * ov, 1, v, ov, 0}, {(long long)v * v, v, (long long)ov * v, 1, 0}, -0.5, 1.0, mi));
        P[G_CTERM].h.push_back(tg(m.Cint, m.t2, m.Cp, 1, ov, ov, ov, v, v, v, {(long long)v * v, v, (long long)ov * v, 1, 0}, {v, ov, (long long)v * ov, 1, 0}, {(long long)v * ov, ov, v, 1, 0}, -1.0, 0.0, mi));
        // D: Dint_aikc = L_aikc + 1/2 sum_ld u_il^ad L_ldkc;  D_ij^ab = 1/2 sum_kc u_jk^bc Dint_aikc
        P[G_DINT1].h.push_back(tg(m.Bia, m.GBov0, m.Dint, 1, ov, ov, N, ov, ov, N, {0, 1, 0, ov, 0}, {0, 1, 0, ov, 0}, {0, ov, 0, 1, 0}, 2.0, 0.0, mi));
        P[G_DINT2].h.push_back(tg(m.Bvv, m.GBoo, m.Dint, 1, v * v, o * o, N, v, o, N, {v, 1, 0, v * v, 0}, {o, 1, 0, o * o, 0}, {ov, 1, v, (long long)v * ov, 0}, -1.0, 1.0, mi));
        P[G_DINT3].h.push_back(tg(m.u, m.Lov, m.Dint, 1, ov, ov, ov, ov, ov, ov, {0, ov, 0, 1, 0}, {0, ov, 0, 1, 0}, {0, ov, 0, 1, 0}, 0.5, 1.0, mi));
        P[G_DTERM].h.push_back(tg(m.Dint, m.u, m.X2, 1, ov, ov, ov, ov, ov, ov, {0, ov, 0, 1, 0}, {0, ov, 0, 1, 0}, {0, ov, 0, 1, 0}, 0.5, 1.0, mi));
        // E: F'_bc = F~_bc - sum_kld u_kl^bd (ld|kc);  F'_kj = F~_kj + sum_lcd u_lj^cd (kd|lc)
        P[G_FVOO].h.push_back(tg(m.u, m.gov, m.Fvv2, 1, v, v, o * ov, v, v, ov, {0, ov, (long long)v * ov, 1, 0}, {0, ov, (long long)v * ov, 1, 0}, {0, v, 0, 1, 0}, -1.0, 1.0, mi));
        P[G_FVOO].h.push_back(tg(m.gov, m.u, m.Foo2, 1, o, o, v * ov, o, o, ov, {0, (long long)v * ov, ov, 1, 0}, {0, (long long)v * ov, ov, 1, 0}, {0, o, 0, 1, 0}, 1.0, 1.0, mi));
        //    E_ij^ab = sum_c t_ij^ac F'_bc - sum_k t_ik^ab F'_kj
        P[G_E1].h.push_back(tg(m.t2, m.Fvv2, m.X2, 1, o * v * o, v, v, o * v * o, v, v, {0, v, 0, 1, 0}, {0, v, 0, 1, 0}, {0, v, 0, 1, 0}, 1.0, 1.0, mi));
        //    (one GEMM per molecule: N runs over (ia, b), so C rows are contiguous in b)
        P[G_E2].h.push_back(tg(m.Foo2, m.t2, m.X2, 1, o, ov * v, o, o, v, o, {0, 1, 0, o, 0}, {ov, 1, 0, v, 0}, {0, v, ov, 1, 0}, -1.0, 1.0, mi));
        // singles: r1 = F~_ai + sum_kc u_ik^ac F~_kc + sum_kcd u_ki^cd (ad|kc)~ - sum_klc u_kl^ac (ki|lc)~
        P[G_S1].h.push_back(tg(m.u, m.Fd + o, m.r1, 1, ov, 1, ov, ov, 1, v, {0, ov, v, 1, 0}, {0, 0, N, 1, 0}, {0, 1, 0, 0, 0}, 1.0, 1.0, mi));
        P[G_S1].h.push_back(tg(m.u, m.Bov0, m.U, 1, ov, N, ov, ov, N, ov, {0, ov, 0, 1, 0}, {0, ov, 0, 1, 0}, {0, N, 0, 1, 0}, 1.0, 0.0, mi));
        P[G_S_UG].h.push_back(tg(m.U, G, m.UG, 1, ov, N, N, ov, N, N, {0, N, 0, 1, 0}, {0, N, 0, 1, 0}, {0, N, 0, 1, 0}, 1.0, 0.0, mi));
        P[G_S_V].h.push_back(tg(m.UG, m.Y + o, m.Vs, N, o, 1, v, o, 1, v, {0, (long long)v * N, 0, N, 1}, {0, 0, 0, 1, N}, {0, N, 0, 0, 1}, 1.0, 0.0, mi));
        P[G_S_R1].h.push_back(tg(m.Vs, m.X + o, m.r1, 1, o, v, N, o, v, N, {0, N, 0, 1, 0}, {0, 1, 0, N, 0}, {0, v, 0, 1, 0}, 1.0, 1.0, mi));
        P[G_S_R1].h.push_back(tg(m.Boo, m.UG, m.r1, 1, o, v, o * N, o, v, N, {0, 1, o, (long long)o * o, 0}, {0, N, (long long)v * N, 1, 0}, {0, v, 0, 1, 0}, -1.0, 1.0, mi));
    }
    // Note G_S_R1 holds two GEMMs into r1: they run in one launch on disjoint
    // tiles of the same output, so they must not overlap -> keep separate groups.
    Group extra;
    extra.h.assign(P[G_S_R1].h.begin() + 0, P[G_S_R1].h.end());
    P[G_S_R1].h.clear();
    Group g1, g2;
    for (size_t k = 0; k < extra.h.size(); ++k) (k % 2 == 0 ? g1 : g2).h.push_back(extra.h[k]);
    P[G_S_R1] = g1;
    P.push_back(g2);
}

// ---------------------------------------------------------------- allocation
static int allocate(hx_ccsd *h)
{
    const int nd = h->p.diis_enabled ? h->p.diis_steps : 0;
    for (int pass = 0; pass < 2; ++pass) {
        Arena A;
        A.base = pass ? h->arena : nullptr;
        h->scf.assign(h->nmol, ScfMol());
        h->cc.assign(h->nmol, CCMol());
        h->diis.assign(h->nmol, DiisMol());
        for (int mi = 0; mi < h->nmol; ++mi) {
            const int N = h->N[mi], o = h->o[mi], v = h->v[mi];
            const size_t nn = (size_t)N * N, ov = (size_t)o * v, pr = ov * ov;
            ScfMol &s = h->scf[mi];
            s.N = N; s.nocc = o;
            s.core = A.take<double>(nn); s.G = A.take<double>(nn); s.huckel = A.take<double>(nn);
            s.D0 = nullptr; s.V0 = nullptr;
            s.F = A.take<double>(nn); s.D = A.take<double>(nn); s.V = A.take<double>(nn); s.E = A.take<double>(N);
            s.A = A.take<double>(nn); s.W1 = A.take<double>(nn); s.W2 = A.take<double>(nn); s.Fmo = A.take<double>(nn);
            s.out = A.take<double>(4); s.status = A.take<int>(2);
            CCMol &m = h->cc[mi];
            m.N = N; m.o = o; m.v = v;
            m.Cmo = s.V; m.G = s.G; m.h = s.core; m.Fmo = s.Fmo;
            m.Bov0 = A.take<double>(N * ov); m.GBov0 = A.take<double>(N * ov);
            m.gov = A.take<double>(pr); m.Lov = A.take<double>(pr);
            m.D1 = A.take<double>(ov); m.D2 = A.take<double>(pr);
            m.t1 = A.take<double>(ov); m.t2 = A.take<double>(pr);
            m.r1 = A.take<double>(ov); m.r2 = A.take<double>(pr); m.u = A.take<double>(pr);
            m.X = A.take<double>(nn); m.Y = A.take<double>(nn); m.Pm = A.take<double>(nn);
            m.H2 = A.take<double>(nn); m.W1 = A.take<double>(nn); m.Fd = A.take<double>(nn);
            m.Bia = A.take<double>(N * ov); m.GBia = A.take<double>(N * ov);
            m.Boo = A.take<double>((size_t)N * o * o); m.GBoo = A.take<double>((size_t)N * o * o);
            m.Bvv = A.take<double>((size_t)N * v * v); m.GBvv = A.take<double>((size_t)N * v * v);
            m.T1s = A.take<double>((size_t)o * v * o * N); m.Ts = A.take<double>((size_t)o * N * o * N);
            m.Z = A.take<double>((size_t)o * N * o * N);
            m.Woo = A.take<double>((size_t)o * o * o * o);
            m.Vvv = mo_ladder(h, mi) ? A.take<double>((size_t)v * v * v * v) : nullptr;
            m.Cint = A.take<double>(pr); m.Cp = A.take<double>(pr); m.Dint = A.take<double>(pr); m.X2 = A.take<double>(pr);
            m.Fvv2 = A.take<double>((size_t)v * v); m.Foo2 = A.take<double>((size_t)o * o);
            m.U = A.take<double>(ov * N); m.UG = A.take<double>(ov * N); m.Vs = A.take<double>((size_t)o * N);
            DiisMol &d = h->diis[mi];
            d.nd = nd > 0 ? nd : 1;
            d.L = (long long)(ov + (size_t)v * v * o * (o + 1) / 2);   // singles + canonical pair blocks
            d.Ht = nd ? A.take<double>((size_t)nd * d.L) : nullptr;
            d.He = nd ? A.take<double>((size_t)nd * d.L) : nullptr;
            d.gram = A.take<double>((size_t)HX_MAX_DIIS * HX_MAX_DIIS);
            d.coef = A.take<double>(HX_MAX_DIIS + 2);
            d.count = A.take<int>(1);
            h->maxw_oNoN = std::max<long long>(h->maxw_oNoN, (long long)(ov + pr + N * ov));
        }
        double *resblock = A.take<double>((size_t)8 * h->nmol);
        for (int mi = 0; mi < h->nmol; ++mi) h->cc[mi].res = resblock ? resblock + 8 * mi : nullptr;
        h->d_res = resblock;
        if (pass == 0) {
            h->arena_bytes = A.used;
            cudaError_t e = cudaMalloc(&h->arena, A.used);
            if (e != cudaSuccess) {
                hx_set_error("cudaMalloc(%zu bytes) for the molecule state: %s", A.used, cudaGetErrorString(e));
                return HX_ERR_NOMEM;
            }
            HX_CU(cudaMemsetAsync(h->arena, 0, A.used, h->st));
        }
    }
    HX_CU(cudaMalloc(&h->d_scf, sizeof(ScfMol) * h->nmol));
    HX_CU(cudaMalloc(&h->d_cc, sizeof(CCMol) * h->nmol));
    HX_CU(cudaMalloc(&h->d_diis, sizeof(DiisMol) * h->nmol));
    HX_CU(cudaMalloc(&h->d_active, sizeof(int) * h->nmol));
    // balanced schedules: blocks per molecule in proportion to its work
    {
        const int n = h->nmol;
        std::vector<int> st((size_t)SK_COUNT * (n + 1));
        h->sched.nmol = n;
        h->sched.vmax = 0;
        for (int k = 0; k < SK_COUNT; ++k) {
            long long acc = 0;
            for (int mi = 0; mi < n; ++mi) {
                const long long N = h->N[mi], o = h->o[mi], v = h->v[mi], ov = o * v;
                long long work = 0;
                switch (k) {
                case SK_NN: work = N * N; break;
                case SK_ZDO: work = N * (ov + o * o + v * v); break;
                case SK_PAIR: work = ov * ov; break;
                case SK_ONON: work = o * N * o * N; break;
                case SK_FOCK: work = ov + v * v + o * o; break;
                case SK_SETUP: work = ov + ov * ov + N * ov; break;
                }
                st[(size_t)k * (n + 1) + mi] = (int)acc;
                if (k == SK_UP) acc += hx_units((int)o, (int)v, true);
                else if (k == SK_FULL) acc += hx_units((int)o, (int)v, false);
                else acc += (work + HX_EW_CHUNK - 1) / HX_EW_CHUNK;
                if (acc > INT32_MAX / 2) { hx_set_error("batch too large for one launch"); return HX_ERR_ARG; }
                h->sched.vmax = std::max(h->sched.vmax, (int)v);
            }
            st[(size_t)k * (n + 1) + n] = (int)acc;
            h->sched.blocks[k] = acc;
        }
        HX_CU(cudaMalloc(&h->d_sched, sizeof(int) * st.size()));
        HX_CU(cudaMemcpy(h->d_sched, st.data(), sizeof(int) * st.size(), cudaMemcpyHostToDevice));
        for (int k = 0; k < SK_COUNT; ++k) h->sched.start[k] = h->d_sched + (size_t)k * (n + 1);
        for (int kk = 0; kk < 3; ++kk) h->unit_smem[kk] = hx_unit_smem(h->o.data(), h->v.data(), n, kk);
        const size_t mx = std::max(h->unit_smem[0], std::max(h->unit_smem[1], h->unit_smem[2]));
        if (mx > 227 * 1024) { hx_set_error("pair units need %zu bytes of shared memory", mx); return HX_ERR_ARG; }
        HX_CU(hx_unit_kernels_init(mx));
    }
    HX_CU(cudaMalloc(&h->d_part, sizeof(double) * std::max<size_t>((size_t)h->sched.blocks[SK_UP] * HX_PART_STRIDE,
                                                                   2 * HX_SCF_GRID_MAX)));
    HX_CU(cudaMalloc(&h->d_act_ph[0], sizeof(int) * PH_COUNT * h->nmol));
    for (int ph = 1; ph < PH_COUNT; ++ph) h->d_act_ph[ph] = h->d_act_ph[0] + (size_t)ph * h->nmol;
    HX_CU(cudaMalloc(&h->d_ctl, sizeof(CtlMol) * h->nmol));
    HX_CU(cudaMalloc(&h->d_remaining, 16 * sizeof(int)));
    h->d_occ = h->d_remaining + 2;
    h->d_loops = h->d_remaining + 7;
    h->d_runs = h->d_remaining + 8;
    HX_CU(cudaMalloc(&h->d_t0, sizeof(unsigned long long)));
    HX_CU(cudaHostAlloc((void **)&h->h_pinned, 16 * sizeof(int), cudaHostAllocMapped));
    memset(h->h_pinned, 0, 16 * sizeof(int));
    {
        int *dp = nullptr;
        HX_CU(cudaHostGetDevicePointer((void **)&dp, h->h_pinned, 0));
        h->d_cancel = dp + 8;
    }
    HX_CU(cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking));
    HX_CU(cudaMalloc(&h->d_gate, sizeof(double) * h->nmol));
    h->gate.assign(h->nmol, 0.0);
    h->active.assign(h->nmol, 1);
    h->scf_failed.assign(h->nmol, 0);
    h->phase.assign(h->nmol, idle_phase(h));
    h->dcount.assign(h->nmol, 0);
    h->slot_phase.assign(h->nmol, {});
    h->ph_end.assign(h->nmol, {});
    h->stall.assign(h->nmol, 0);
    h->best.assign(h->nmol, 1e300);
    h->fin_scale.assign(h->nmol, 1.0);
    h->fp_returns.assign(h->nmol, 0);
    h->trace.assign(h->nmol, {});
    h->res.assign((size_t)h->nmol * 8, 0.0);
    h->status.assign(h->nmol, 0);
    h->rules.assign(h->nmol, Rules());
    return HX_OK;
}

static int upload_views(hx_ccsd *h)
{
    HX_CU(cudaMemcpyAsync(h->d_scf, h->scf.data(), sizeof(ScfMol) * h->nmol, cudaMemcpyHostToDevice, h->st));
    HX_CU(cudaMemcpyAsync(h->d_cc, h->cc.data(), sizeof(CCMol) * h->nmol, cudaMemcpyHostToDevice, h->st));
    HX_CU(cudaMemcpyAsync(h->d_diis, h->diis.data(), sizeof(DiisMol) * h->nmol, cudaMemcpyHostToDevice, h->st));
    HX_CU(cudaMemcpyAsync(h->d_active, h->active.data(), sizeof(int) * h->nmol, cudaMemcpyHostToDevice, h->st));
    return HX_OK;
}

// ---------------------------------------------------------------- C ABI
extern "C" {

void hx_cc_params_default(hx_cc_params *p)
{
    memset(p, 0, sizeof(*p));
    p->coulomb = HX_COULOMB_OHNO_KLOPMAN;
    p->bond_alternation = 0.0;
    p->scf_maxiter = 400;
    p->scf_eps = 1e-12;
    p->scf_step = 0.05;
    p->projection_type = 2;
    p->cc_maxiter = 2000;
    p->cc_eps = 1e-12;
    p->t1_step = 1.0;
    p->t2_step = 1.0;
    p->diis_enabled = 1;
    p->diis_steps = 20;
    p->check_divergence = 1;
    p->divergence_threshold = 1e3;
    p->check_stagnation = 1;
    p->stagnation_threshold = 60.0;
    p->stagnation_after = 200;
    p->precision = HX_PRECISION_FP64;
    p->guess = 0;
    p->mixed_switch = 1e-3;
    p->mixed_patience = 3;
    p->mixed_check = 0;
    p->tile_tuning = 0;
    p->tile_force = -1;
}

int hx_ccsd_create_batch(const hx_ppp_model *ms, int32_t n, const hx_cc_params *p, hx_ccsd **out)
{
    if (!ms || !p || !out || n <= 0) { hx_set_error("hx_ccsd_create_batch: bad arguments"); return HX_ERR_ARG; }
    *out = nullptr;
    if (p->projection_type != 1 && p->projection_type != 2) { hx_set_error("projection-type must be 1 or 2"); return HX_ERR_ARG; }
    if (p->diis_enabled && (p->diis_steps < 2 || p->diis_steps > HX_MAX_DIIS)) { hx_set_error("diis-steps outside 2..%d", HX_MAX_DIIS); return HX_ERR_ARG; }
    if (p->precision != HX_PRECISION_FP64 && p->precision != HX_PRECISION_MIXED && p->precision != HX_PRECISION_EXACT) {
        hx_set_error("unknown precision mode");
        return HX_ERR_ARG;
    }
    if (p->mixed_check != 0 && p->mixed_check != 1) { hx_set_error("mixed_check must be 0 (7-slice emulated FP64) or 1 (FP64)"); return HX_ERR_ARG; }
    if (p->tile_tuning < 0 || p->tile_tuning > 2 || p->tile_force < -1) { hx_set_error("tile_tuning must be 0, 1 or 2 and tile_force >= -1"); return HX_ERR_ARG; }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { hx_set_error("no CUDA device"); return HX_ERR_CUDA; }
    hx_ccsd *h = new hx_ccsd();
    h->p = *p;
    h->nmol = n;
    h->models.resize(n);
    for (int i = 0; i < n; ++i) {
        int rc = build_model(&ms[i], p, h->models[i]);
        if (rc < 0) { delete h; return rc; }
        h->N.push_back(h->models[i].N);
        h->o.push_back(h->models[i].nel / 2);
        h->v.push_back(h->models[i].N - h->models[i].nel / 2);
    }
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
        hx_set_error("cudaStreamCreate failed"); delete h; return HX_ERR_CUDA;
    }
    int rc = allocate(h);
    if (rc < 0) { hx_ccsd_destroy(h); return rc; }
    for (int mi = 0; mi < n; ++mi) {
        const HostModel &M = h->models[mi];
        size_t bytes = sizeof(double) * M.N * M.N;
        if (cudaMemcpyAsync((void *)h->scf[mi].core, M.core.data(), bytes, cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
            cudaMemcpyAsync((void *)h->scf[mi].G, M.G.data(), bytes, cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
            cudaMemcpyAsync((void *)h->scf[mi].huckel, M.huckel.data(), bytes, cudaMemcpyHostToDevice, h->st) != cudaSuccess) {
            hx_set_error("upload of the PPP model failed"); hx_ccsd_destroy(h); return HX_ERR_CUDA;
        }
    }
    rc = upload_views(h);
    if (rc < 0) { hx_ccsd_destroy(h); return rc; }
    build_plan(h);
    mark_constants(h);
    for (auto &g : h->plan) {
        rc = upload_group(g);
        if (rc < 0) { hx_ccsd_destroy(h); return rc; }
    }
    if (p->precision != HX_PRECISION_FP64) {
        rc = tc::create(&h->tce, h->plan, h->st, p->tile_tuning, p->tile_force);
        if (rc < 0) { hx_ccsd_destroy(h); return rc; }
    }
    if (cudaStreamSynchronize(h->st) != cudaSuccess) { hx_set_error("set-up failed"); hx_ccsd_destroy(h); return HX_ERR_CUDA; }
    *out = h;
    return HX_OK;
}

int hx_ccsd_create(const hx_ppp_model *m, const hx_cc_params *p, hx_ccsd **out)
{
    return hx_ccsd_create_batch(m, 1, p, out);
}

static int cc_setup(hx_ccsd *h, int guess)
{
    // Bov0, D1, D2; then G.Bov0, gov = Bov0^T G Bov0; then Lov and the guess
    HX_CU(hx_ew_setup(h->d_cc, h->d_active, h->sched, h->st));
    Group g1, g2;
    for (int mi = 0; mi < h->nmol; ++mi) {
        const CCMol &m = h->cc[mi];
        const int N = m.N, ov = m.o * m.v;
        g1.h.push_back(tg(m.G, m.Bov0, m.GBov0, 1, N, ov, N, N, ov, N, {0, N, 0, 1, 0}, {0, 1, 0, ov, 0}, {0, ov, 0, 1, 0}, 1.0, 0.0, mi));
        g2.h.push_back(tg(m.Bov0, m.GBov0, m.gov, 1, ov, ov, N, ov, ov, N, {0, 1, 0, ov, 0}, {0, 1, 0, ov, 0}, {0, ov, 0, 1, 0}, 1.0, 0.0, mi));
    }
    HX_TRY(upload_group(g1));
    HX_TRY(upload_group(g2));
    HX_CU(hx_tgemm_f64_launch(g1.d, (int)g1.h.size(), g1.tiles, h->d_active, h->st));
    HX_CU(hx_tgemm_f64_launch(g2.d, (int)g2.h.size(), g2.tiles, h->d_active, h->st));
    HX_CU(hx_ew_setup2(h->d_cc, h->d_active, h->sched, guess, h->st));
    HX_CU(cudaStreamSynchronize(h->st));
    cudaFree(g1.d);
    cudaFree(g2.d);
    return HX_OK;
}

// Learned T2 guess: after the reference guess, t2 <- guess + network
// prediction on every canonical pair of every molecule (inference on the
// tensor cores, features from the device state).
static int apply_learned_guess(hx_ccsd *h)
{
    if (!h->model) {
        hx_set_error("guess = 1 (learned) but no model was given (hx_ccsd_set_model)");
        return HX_ERR_STATE;
    }
    for (int mi = 0; mi < h->nmol; ++mi) {
        if (h->scf_failed[mi]) continue;
        const long long ov = (long long)h->o[mi] * h->v[mi];
        HX_CU(h->model->apply(h->d_cc, mi, ov * (ov + 1) / 2, h->st));
    }
    HX_CU(cudaStreamSynchronize(h->st));
    if (int w = h->model->error_word()) {
        hx_set_error("learned guess: a tensor-core wait timed out (code %d)", w);
        return HX_ERR_KERNEL;
    }
    return HX_OK;
}

static void diis_mirror_reset(hx_ccsd *h, int mi);

int hx_ccsd_init(hx_ccsd *h)
{
    if (!h) { hx_set_error("NULL handle"); return HX_ERR_ARG; }
    ScfParams sp;
    sp.maxiter = h->p.scf_maxiter;
    sp.eps = h->p.scf_eps;
    sp.step = h->p.scf_step;
    sp.divergence = h->p.divergence_threshold;
    sp.stag_pct = h->p.stagnation_threshold;
    sp.stag_after = h->p.stagnation_after;
    sp.check_div = h->p.check_divergence;
    sp.check_stag = h->p.check_stagnation;
    int nmax = 0;
    for (int mi = 0; mi < h->nmol; ++mi) nmax = std::max(nmax, h->N[mi]);
    if (!h->ev[0]) for (int k = 0; k < 4; ++k) HX_CU(cudaEventCreate(&h->ev[k]));
    HX_CU(cudaEventRecord(h->ev[0], h->st));
    HX_CU(hx_scf_launch(h->d_scf, h->nmol, nmax, sp, h->d_part, h->st));
    std::vector<double> out(4);
    std::vector<int> st(2);
    HX_CU(cudaStreamSynchronize(h->st));
    // one molecule: an SCF that does not converge is an error (as in the
    // reference); in a batch the molecule is left out with status HX_ERR_SCF
    int failed = 0;
    for (int mi = 0; mi < h->nmol; ++mi) {
        HX_CU(cudaMemcpy(out.data(), h->scf[mi].out, sizeof(double) * 4, cudaMemcpyDeviceToHost));
        HX_CU(cudaMemcpy(st.data(), h->scf[mi].status, sizeof(int) * 2, cudaMemcpyDeviceToHost));
        h->scf_failed[mi] = st[0] != HX_CONVERGED;
        if (h->scf_failed[mi]) {
            hx_set_error("SCF of molecule %d ended with status %d after %d iterations (accuracy %.3e)", mi, st[0], st[1], out[3]);
            if (h->nmol == 1) return HX_ERR_SCF;
            ++failed;
        }
        h->cc[mi].eref = out[0];
        h->active[mi] = !h->scf_failed[mi];
    }
    if (failed == h->nmol) return HX_ERR_SCF;
    HX_TRY(upload_masks(h));
    HX_TRY(upload_views(h));
    HX_TRY(cc_setup(h, 1));
    if (h->p.guess == 1) HX_TRY(apply_learned_guess(h));
    if (h->tce) tc::invalidate(h->tce);          // new orbitals: re-slice the constant operands
    for (int mi = 0; mi < h->nmol; ++mi) {
        h->rules[mi] = Rules();
        h->status[mi] = h->scf_failed[mi] ? HX_ERR_SCF : 0;
        h->active[mi] = !h->scf_failed[mi];
    }
    for (int mi = 0; mi < h->nmol; ++mi) {
        HX_CU(cudaMemsetAsync(h->diis[mi].count, 0, sizeof(int), h->st));
        diis_mirror_reset(h, mi);
    }
    HX_TRY(upload_views(h));
    HX_CU(cudaEventRecord(h->ev[1], h->st));
    HX_TRY(upload_masks(h));
    cudaEventElapsedTime(&h->init_ms, h->ev[0], h->ev[1]);
    h->initialized = true;
    return HX_OK;
}

// One iterationCC for every active molecule (no host synchronisation).
static int iteration_body(hx_ccsd *h, double eps)
{
    if (!h->device_ctl && eps != h->gate_eps) { h->gate_eps = eps; HX_TRY(upload_masks(h)); }
    auto &P = h->plan;
    int k = 0;
    HX_CU(hx_ew_dress_init(h->d_cc, h->d_active, h->sched, h->st));
    HX_TRY(run_group(h, P[k++]));                                    // dress X, Y
    HX_TRY(run_group(h, P[k++]));                                    // Pm
    HX_CU(hx_ew_dress_fock(h->d_cc, h->d_active, h->sched, h->st));
    HX_TRY(run_group(h, P[k++]));                                    // W1 = H2 Y
    HX_TRY(run_group(h, P[k++]));                                    // Fd = X^T W1
    HX_CU(hx_ew_zdo_products(h->d_cc, h->d_active, h->sched, h->st));
    HX_TRY(run_group(h, P[k++]));                                    // G B
    HX_CU(hx_ew_make_u(h->d_cc, h->d_active, h->sched, h->unit_smem[0], h->st));
    HX_CU(hx_ew_fock_blocks(h->d_cc, h->d_active, h->sched, h->st));
    HX_TRY(run_group(h, P[k++]));                                    // lead
    HX_TRY(run_group(h, P[k++]));                                    // lad_a
    HX_TRY(run_group(h, P[k++]));                                    // lad_b
    HX_CU(hx_ew_gamma_scale(h->d_cc, h->d_active, h->sched, h->st));
    HX_TRY(run_group(h, P[k++]));                                    // lad_d
    HX_TRY(run_group(h, P[k++]));                                    // lad_e
    HX_TRY(run_group(h, P[k++]));                                    // w_d
    HX_TRY(run_group(h, P[k++]));                                    // w_e
    HX_TRY(run_group(h, P[k++]));                                    // w_int
    HX_TRY(run_group(h, P[k++]));                                    // hh
    HX_TRY(run_group(h, P[k++]));                                    // cint1
    HX_TRY(run_group(h, P[k++]));                                    // cint2
    HX_TRY(run_group(h, P[k++]));                                    // cterm
    HX_CU(hx_ew_c_combine(h->d_cc, h->d_active, h->sched, h->st));
    HX_TRY(run_group(h, P[k++]));                                    // dint1
    HX_TRY(run_group(h, P[k++]));                                    // dint2
    HX_TRY(run_group(h, P[k++]));                                    // dint3
    HX_TRY(run_group(h, P[k++]));                                    // dterm
    HX_TRY(run_group(h, P[k++]));                                    // F'vv, F'oo
    HX_TRY(run_group(h, P[k++]));                                    // e1
    HX_TRY(run_group(h, P[k++]));                                    // e2
    // (r2 += X2 + X2 pair-transposed is part of the step below)
    HX_TRY(run_group(h, P[k++]));                                    // singles: u F, U
    HX_TRY(run_group(h, P[k++]));                                    // UG
    HX_TRY(run_group(h, P[k++]));                                    // Vs
    HX_TRY(run_group(h, P[k++]));                                    // r1 += Vs Xv
    HX_TRY(run_group(h, P[k++]));                                    // r1 -= Boo UG
    const int use_diis = h->p.diis_enabled ? 1 : 0;
    HX_CU(hx_tail(h->d_cc, h->d_diis, h->d_active, h->sched, h->unit_smem + 1, h->p.t1_step, h->p.t2_step,
                  h->p.projection_type, use_diis, h->d_gate, h->d_part, h->st));
    return HX_OK;
}

static int fetch_results(hx_ccsd *h)
{
    HX_CU(cudaMemcpyAsync(h->res.data(), h->d_res, sizeof(double) * 8 * h->nmol, cudaMemcpyDeviceToHost, h->st));
    HX_CU(cudaStreamSynchronize(h->st));
    return HX_OK;
}

int hx_ccsd_iterate(hx_ccsd *h, int32_t iteration, double eps, double acc[5])
{
    if (!h || !h->initialized) { hx_set_error("hx_ccsd_iterate before hx_ccsd_init"); return HX_ERR_STATE; }
    (void)iteration;
    HX_TRY(iteration_body(h, eps));
    HX_TRY(fetch_results(h));
    if (acc) {
        acc[0] = h->res[0]; acc[1] = h->res[1];
        acc[2] = acc[3] = acc[4] = -1.0;
    }
    return HX_OK;
}

int hx_ccsd_energy(hx_ccsd *h, double e[5])
{
    if (!h || !h->initialized) { hx_set_error("hx_ccsd_energy before hx_ccsd_init"); return HX_ERR_STATE; }
    HX_CU(hx_energy(h->d_cc, h->d_diis, nullptr, h->sched, h->unit_smem[2], h->d_part, h->st));
    HX_TRY(fetch_results(h));
    if (e) { e[0] = h->res[2]; e[1] = h->res[3]; e[2] = h->res[4]; e[3] = h->res[5]; e[4] = 0.0; }
    return HX_OK;
}

static void diis_mirror_reset(hx_ccsd *h, int mi)
{
    h->dcount[mi] = 0;
    h->slot_phase[mi].assign((size_t)h->diis[mi].nd, -1);
    h->ph_end[mi] = {};
}

// Mixed precision keeps the DIIS history across a precision switch (a plain
// "2-1" step is unstable, so a restart costs iterations), but a vector made
// in a cheaper phase carries that phase's error. Once the residual has fallen
// to kPurge of the level at which that phase ended, its vectors are taken out
// of the extrapolation: their Gram row and column are cleared and the
// diagonal made huge, so their DIIS coefficients vanish; the slots are
// reused by later pushes as usual.
static const double kPurge = 0.1;


// The iterator (gIterator.f90:88-210) over every active molecule. In mixed
// precision a molecule walks down a ladder of phases:
//   LOW   3-slice tensor-core contractions (about 2^-24 of the operands' row
//         maxima) until the residual falls below mixed_switch;
//   MID   4-slice (about 2^-32) until it falls below kMidSpan * mixed_switch;
//   HIGH  5-slice (about 2^-35) until it falls below kHighMargin * eps;
//   check the iteration that may declare convergence: EXACT, 7-slice
//         contractions that emulate FP64 ones (mixed_check = 0), or plain
//         CUDA-core FP64 (mixed_check = 1). Convergence is declared only
//         here, so the final residual and energy carry FP64 accuracy (the
//         defect correction). A check that does not confirm convergence
//         sends the molecule back to 5-slice iterations with a 10x tighter
//         hand-over target (at most kMaxFp64Returns times); after that the
//         check phase iterates on, and EXACT iterations that stop improving
//         for mixed_patience iterations hand over to CUDA-core FP64.
// A tensor-core phase hands over to the check below kHighMargin * eps (the
// iteration is not monotone, and one more 5-slice iteration costs less than
// a check whose residual lands just above eps). A phase switches while its
// own error is still about 1 % of the residual, so the DIIS history is kept;
// a phase that stops improving for mixed_patience iterations hands over early
// and the DIIS history restarts (its error vectors are then too noisy to mix
// with more accurate ones).
static const double kMidSpan = 1e-3;
static const int kMaxFp64Returns = 3;

// The iterator runs on the device (k_control, after every iteration). The
// host uploads each molecule's iterator state and builds one CUDA graph for
// the whole solve: a conditional while node whose body is one captured
// iteration -- a node that sets each phase's condition from the number of
// molecules in that phase, every contraction group with one conditional node
// per phase (its launches masked per molecule), the element-wise kernels, the
// tail, k_control, and a node that continues the loop while a molecule is
// still running (at most maxiter + 8 times, so the loop always ends). The
// host launches it once and waits. A stop request (hx_ccsd_cancel) is a word
// of mapped host memory that k_control reads every iteration. With per-launch
// GEMM timing on (hx_ccsd_timing) the iterations are launched one by one
// instead (the timing events belong to the host's launches), each with the
// phases the device counted for it.
static int solve_all(hx_ccsd *h, int maxiter, double eps)
{
    const bool mixed = h->tce != nullptr;
    const int n = h->nmol;
    int remaining = 0;
    std::vector<CtlMol> c(n);
    for (int mi = 0; mi < n; ++mi) {
        remaining += h->active[mi];
        // HX_PRECISION_EXACT: every iteration is a 7-slice (FP64-emulating) check iteration
        h->phase[mi] = !mixed ? PH_FP64 : h->p.precision == HX_PRECISION_EXACT ? PH_EXACT : PH_LOW;
        h->fin_scale[mi] = 1.0;                  // (the first iteration's DIIS gates)
        CtlMol &x = c[mi];
        memset(&x, 0, sizeof(x));
        x.iteration = h->rules[mi].iteration;
        x.successful = h->rules[mi].successful;
        x.current = h->rules[mi].current;
        x.status = h->status[mi];
        x.active = h->active[mi];
        x.phase = h->phase[mi];
        x.best = 1e300;
        x.fin_scale = 1.0;
        if (mixed && h->p.precision == HX_PRECISION_EXACT) x.fp_returns = kMaxFp64Returns;   // never back to 5 slices
        x.dcount = h->dcount[mi];
        for (int k = 0; k < HX_MAX_DIIS; ++k)
            x.slot_phase[k] = (signed char)(k < (int)h->slot_phase[mi].size() ? h->slot_phase[mi][k] : -1);
        for (int k = 0; k < PH_COUNT; ++k) x.ph_end[k] = h->ph_end[mi][k];
        h->trace[mi].clear();
    }
    h->gate_eps = eps;
    HX_TRY(upload_masks(h));
    const int cap = (int)std::min<long long>((long long)maxiter + 1, 10000);
    if (cap > h->trace_cap) {
        cudaFree(h->d_trace);
        h->d_trace = nullptr;
        h->trace_cap = 0;
        HX_CU(cudaMalloc(&h->d_trace, sizeof(double) * 5 * (size_t)cap * n));
        h->trace_cap = cap;
    }
    CtlParams P;
    memset(&P, 0, sizeof(P));
    P.nmol = n; P.maxiter = maxiter; P.mixed = mixed; P.check_ph = h->p.mixed_check == 1 ? PH_FP64 : PH_EXACT;
    P.patience = h->p.mixed_patience; P.max_returns = kMaxFp64Returns; P.diis_enabled = h->p.diis_enabled;
    P.check_div = h->p.check_divergence; P.check_stag = h->p.check_stagnation; P.stag_after = h->p.stagnation_after;
    P.trace_cap = h->trace_cap; P.eps = eps; P.mixed_switch = h->p.mixed_switch; P.mid_span = kMidSpan;
    P.high_margin = kHighMargin; P.purge = kPurge; P.div_thr = h->p.divergence_threshold;
    P.stag_thr = h->p.stagnation_threshold;
    HX_CU(cudaMemcpyAsync(h->d_ctl, c.data(), sizeof(CtlMol) * n, cudaMemcpyHostToDevice, h->st));
    h->h_pinned[0] = remaining;
    h->h_pinned[1] = 0;
    reinterpret_cast<volatile int *>(h->h_pinned)[8] = 0;
    for (int ph = 0; ph < PH_COUNT; ++ph) h->h_pinned[2 + ph] = 0;
    for (int mi = 0; mi < n; ++mi)
        if (h->active[mi]) ++h->h_pinned[2 + h->phase[mi]];
    HX_CU(cudaMemcpyAsync(h->d_remaining, h->h_pinned, 8 * sizeof(int), cudaMemcpyHostToDevice, h->st));
    if (h->tce) HX_CU(tc::prepare_fixed(h->tce, h->st));
    h->cancel.store(0);
    HX_CU(cudaMemsetAsync(h->d_loops, 0, 6 * sizeof(int), h->st));      // the loop count and runs[5]
    HX_CU(cudaEventRecord(h->ev[2], h->st));
    HX_CU(hx_control_start(h->d_t0, h->st));
    auto control = [&]() {
        return hx_control(h->d_cc, h->d_diis, h->d_ctl, P, h->d_cancel, h->d_t0, h->d_active,
                          mixed ? h->d_act_ph[0] : nullptr, h->d_gate, h->d_trace, h->d_remaining, h->d_occ, h->st);
    };
    h->device_ctl = true;
    const bool graph = !h->profiling;
    cudaGraphExec_t exec = nullptr;
    long long nodes = 0;
    int rc = HX_OK;
    if (graph) {
        const long long before = g_launches.load();
        // one graph for the whole solve: a while node whose body is one
        // iteration (the phase-condition node, every group with one conditional
        // node per phase, the tail, k_control, then the loop condition)
        cudaGraph_t gr = nullptr;
        const char *step = "cudaGraphCreate";
        cudaError_t ce = cudaGraphCreate(&gr, 0);
        const int ncond = (int)(h->plan.size() * PH_COUNT);
        h->cond.clear();
        for (int ph = 0; ph < PH_COUNT; ++ph) h->phase_nodes[ph] = 0;
        if (ce == cudaSuccess && mixed && !h->d_cond) {
            step = "cudaMalloc";
            ce = cudaMalloc(&h->d_cond, sizeof(PhaseCondition) * ncond);
        }
        cudaGraphConditionalHandle loop = 0;
        cudaGraph_t body = nullptr;
        if (ce == cudaSuccess) {
            step = "the loop's conditional handle";
            ce = cudaGraphConditionalHandleCreate(&loop, gr, 1, cudaGraphCondAssignDefault);
        }
        if (ce == cudaSuccess) {
            step = "the while node";
            alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)] = {};
            cudaGraphNodeParams &np = *reinterpret_cast<cudaGraphNodeParams *>(raw);
            np.type = cudaGraphNodeTypeConditional;
            np.conditional.handle = loop;
            np.conditional.type = cudaGraphCondTypeWhile;
            np.conditional.size = 1;
            cudaGraphNode_t wnode;
            ce = cudaGraphAddNode(&wnode, gr, nullptr, nullptr, 0, &np);
            if (ce == cudaSuccess) body = np.conditional.phGraph_out[0];
        }
        if (ce == cudaSuccess) {
            step = "cudaStreamBeginCaptureToGraph";
            ce = cudaStreamBeginCaptureToGraph(h->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if (ce == cudaSuccess) {
                if (mixed) {
                    step = "the phase-condition kernel";
                    ce = hx_phase_conditions(h->d_occ, h->d_cond, ncond, h->d_runs, h->st);
                }
                h->capturing = true;
                if (ce == cudaSuccess) rc = iteration_body(h, eps);
                h->capturing = false;
                if (ce == cudaSuccess && rc == HX_OK) { step = "the control kernel"; ce = control(); }
                if (ce == cudaSuccess && rc == HX_OK) {
                    step = "the loop-condition kernel";
                    ce = hx_loop_condition(h->d_remaining, loop, h->d_loops, maxiter + 8, h->st);
                }
                cudaGraph_t out = nullptr;
                const cudaError_t ce2 = cudaStreamEndCapture(h->st, &out);
                if (ce == cudaSuccess && ce2 != cudaSuccess) { step = "cudaStreamEndCapture"; ce = ce2; }
            }
        }
        if (rc == HX_OK && ce == cudaSuccess && mixed) {
            // the handles the capture made, read by the first node at run time
            step = "cudaMemcpy of the conditional handles";
            std::vector<PhaseCondition> all(ncond);
            memset(all.data(), 0, sizeof(PhaseCondition) * ncond);
            for (int k = 0; k < ncond; ++k) all[k].phase = k < (int)h->cond.size() ? h->cond[k].phase : -1;
            for (size_t k = 0; k < h->cond.size(); ++k) all[k].handle = h->cond[k].handle;
            ce = cudaMemcpy(h->d_cond, all.data(), sizeof(PhaseCondition) * ncond, cudaMemcpyHostToDevice);
        }
        if (rc == HX_OK && ce == cudaSuccess) { step = "cudaGraphInstantiate"; ce = cudaGraphInstantiate(&exec, gr, 0); }
        if (gr) cudaGraphDestroy(gr);
        nodes = g_launches.load() - before;
        g_launches.fetch_sub(nodes);                 // captured, not run: counted per replay below
        if (rc == HX_OK && ce != cudaSuccess) {
            hx_set_error("capturing the iteration (%s): %s", step, cudaGetErrorString(ce));
            rc = HX_ERR_CUDA;
        }
    }
    long long launched = 0;
    if (graph && rc == HX_OK) {
        // the whole solve is one launch; the host waits for it
        cudaError_t ce = cudaGraphLaunch(exec, h->st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->st);
        if (ce != cudaSuccess) { hx_set_error("solve graph: %s", cudaGetErrorString(ce)); rc = HX_ERR_CUDA; }
        // kernels run: every iteration's unconditional ones, and each phase's
        // bodies in the iterations that phase ran
        int lr[6] = {0, 0, 0, 0, 0, 0};
        if (rc == HX_OK && cudaMemcpy(lr, h->d_loops, sizeof(lr), cudaMemcpyDeviceToHost) == cudaSuccess) {
            long long cond_nodes = 0, run = 0;
            for (int ph = 0; ph < PH_COUNT; ++ph) { cond_nodes += h->phase_nodes[ph]; run += h->phase_nodes[ph] * lr[1 + ph]; }
            hx_count_launches((int)((nodes - cond_nodes) * lr[0] + run));
        }
        const int loops = lr[0];
        if (rc == HX_OK && h->tce) {
            tc::collect(h->tce, h->prof);
            if (tc::error_word(h->tce) != 0) {
                hx_set_error("a tensor-core kernel timed out waiting (code %d)", tc::error_word(h->tce));
                rc = HX_ERR_KERNEL;
            }
        }
        if (rc == HX_OK && loops >= maxiter + 8) {
            hx_set_error("the device iterator did not stop after %d iterations", loops);
            rc = HX_ERR_STATE;
        }
    }
    while (!graph && rc == HX_OK) {
        // launched one by one: the phases counted at the last read run
        // (h_pinned[2..6]); the device counts the next ones from zero
        if (cudaMemsetAsync(h->d_occ, 0, PH_COUNT * sizeof(int), h->st) != cudaSuccess) {
            hx_set_error("solve: cudaMemsetAsync failed");
            rc = HX_ERR_CUDA;
        }
        if (rc == HX_OK) rc = iteration_body(h, eps);
        if (rc == HX_OK && control() != cudaSuccess) { hx_set_error("iterator kernel launch failed"); rc = HX_ERR_CUDA; }
        ++launched;
        if (rc != HX_OK) break;
        cudaError_t ce = cudaMemcpyAsync(h->h_pinned, h->d_remaining, 8 * sizeof(int), cudaMemcpyDeviceToHost, h->st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->st);
        if (ce != cudaSuccess) { hx_set_error("solve: %s", cudaGetErrorString(ce)); rc = HX_ERR_CUDA; break; }
        if (h->tce) {
            tc::collect(h->tce, h->prof);
            if (tc::error_word(h->tce) != 0) {
                hx_set_error("a tensor-core kernel timed out waiting (code %d)", tc::error_word(h->tce));
                rc = HX_ERR_KERNEL;
                break;
            }
        }
        if (h->h_pinned[0] <= 0) break;
        if (launched > (long long)maxiter + 8) {
            hx_set_error("the device iterator did not stop after %lld iterations", launched);
            rc = HX_ERR_STATE;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    h->device_ctl = false;
    if (rc < 0) { cudaStreamSynchronize(h->st); return rc; }
    HX_CU(cudaEventRecord(h->ev[3], h->st));
    HX_CU(cudaEventSynchronize(h->ev[3]));
    cudaEventElapsedTime(&h->solve_ms, h->ev[2], h->ev[3]);
    // the iterator's state and traces back to the host mirrors
    HX_CU(cudaMemcpy(c.data(), h->d_ctl, sizeof(CtlMol) * n, cudaMemcpyDeviceToHost));
    int maxnt = 0;
    for (int mi = 0; mi < n; ++mi) maxnt = std::max(maxnt, c[mi].ntrace);
    std::vector<double> tr((size_t)n * maxnt * 5);
    if (maxnt > 0)
        HX_CU(cudaMemcpy2D(tr.data(), sizeof(double) * 5 * maxnt, h->d_trace, sizeof(double) * 5 * h->trace_cap,
                           sizeof(double) * 5 * maxnt, n, cudaMemcpyDeviceToHost));
    for (int mi = 0; mi < n; ++mi) {
        const CtlMol &x = c[mi];
        h->rules[mi].iteration = x.iteration;
        h->rules[mi].successful = x.successful;
        h->rules[mi].current = x.current;
        h->status[mi] = x.status;
        h->dcount[mi] = x.dcount;
        for (int k = 0; k < (int)h->slot_phase[mi].size(); ++k) h->slot_phase[mi][k] = k < HX_MAX_DIIS ? x.slot_phase[k] : -1;
        for (int k = 0; k < PH_COUNT; ++k) h->ph_end[mi][k] = x.ph_end[k];
        for (int t = 0; t < x.ntrace; ++t) {
            const double *row = &tr[((size_t)mi * maxnt + t) * 5];
            h->trace[mi].push_back({row[0], row[1], row[2], row[3], row[4]});
        }
    }
    HX_TRY(fetch_results(h));
    if (h->tce) tc::collect(h->tce, h->prof);
    // keep every molecule addressable for getters / energy after the solve
    for (int mi = 0; mi < n; ++mi) { h->active[mi] = !h->scf_failed[mi]; h->phase[mi] = idle_phase(h); }
    HX_TRY(upload_masks(h));
    return HX_OK;
}

int hx_ccsd_trace(hx_ccsd *h, int32_t mol, double *out, int32_t cap)
{
    if (!h || mol < 0 || mol >= h->nmol) { hx_set_error("bad handle or molecule index"); return HX_ERR_ARG; }
    const auto &t = h->trace[mol];
    int n = (int)t.size();
    for (int k = 0; k < n && k < cap && out; ++k)
        for (int c = 0; c < 5; ++c) out[5 * k + c] = t[k][c];
    return n;
}

int hx_ccsd_solve(hx_ccsd *h, int32_t maxiter, double eps, int32_t *status, int32_t *iters, double e[5])
{
    if (!h || !h->initialized) { hx_set_error("hx_ccsd_solve before hx_ccsd_init"); return HX_ERR_STATE; }
    HX_TRY(solve_all(h, maxiter, eps));
    if (status) *status = h->status[0];
    if (iters) *iters = h->rules[0].iteration;
    if (e) { e[0] = h->res[2]; e[1] = h->res[3]; e[2] = h->res[4]; e[3] = h->res[5]; e[4] = 0.0; }
    return HX_OK;
}

int hx_ccsd_solve_batch(hx_ccsd *h, int32_t *status, int32_t *iters, double *e)
{
    if (!h || !h->initialized) { hx_set_error("hx_ccsd_solve_batch before hx_ccsd_init"); return HX_ERR_STATE; }
    HX_TRY(solve_all(h, h->p.cc_maxiter, h->p.cc_eps));
    for (int mi = 0; mi < h->nmol; ++mi) {
        if (status) status[mi] = h->status[mi];
        if (iters) iters[mi] = h->rules[mi].iteration;
        if (e) for (int k = 0; k < 4; ++k) e[mi * 5 + k] = h->res[(size_t)mi * 8 + 2 + k];
        if (e) e[mi * 5 + 4] = 0.0;
    }
    return HX_OK;
}

// Pinned host staging for the amplitude transfers, grown to the largest
// molecule asked for (pageable memory would go through the driver's bounce
// buffer and fault its pages in on every call); NULL if it cannot be pinned.
static double *amp_stage(hx_ccsd *h, size_t elems)
{
    if (elems > h->h_amp_elems) {
        if (h->h_amp) cudaFreeHost(h->h_amp);
        h->h_amp = nullptr;
        h->h_amp_elems = 0;
        if (cudaMallocHost(&h->h_amp, sizeof(double) * elems) != cudaSuccess) {
            cudaGetLastError();
            h->h_amp = nullptr;
            return nullptr;
        }
        h->h_amp_elems = elems;
    }
    return h->h_amp;
}

int hx_ccsd_get_amplitudes(hx_ccsd *h, int32_t mol, double *t1, double *t2)
{
    if (!h || mol < 0 || mol >= h->nmol) { hx_set_error("bad handle or molecule index"); return HX_ERR_ARG; }
    const int o = h->o[mol], v = h->v[mol];
    const size_t ov = (size_t)o * v;
    std::vector<double> pageable;
    double *buf = amp_stage(h, ov + ov * ov);
    if (!buf) { pageable.resize(ov + ov * ov); buf = pageable.data(); }
    HX_CU(cudaMemcpyAsync(buf, h->cc[mol].t1, sizeof(double) * ov, cudaMemcpyDeviceToHost, h->st));
    HX_CU(cudaMemcpyAsync(buf + ov, h->cc[mol].t2, sizeof(double) * ov * ov, cudaMemcpyDeviceToHost, h->st));
    HX_CU(cudaStreamSynchronize(h->st));
    if (t1) hx::t1_from_engine(buf, t1, o, v);
    if (t2) hx::t2_from_engine(buf + ov, t2, o, v);
    return HX_OK;
}

int hx_ccsd_set_guess(hx_ccsd *h, int32_t mol, const double *t1, const double *t2)
{
    if (!h || !h->initialized || mol < 0 || mol >= h->nmol || !t1 || !t2) { hx_set_error("hx_ccsd_set_guess: bad arguments or state"); return HX_ERR_ARG; }
    const int o = h->o[mol], v = h->v[mol];
    const size_t ov = (size_t)o * v;
    std::vector<double> pageable;
    double *buf = amp_stage(h, ov + ov * ov);
    if (!buf) { pageable.resize(ov + ov * ov); buf = pageable.data(); }
    hx::t1_to_engine(t1, buf, o, v);
    hx::t2_to_engine(t2, buf + ov, o, v);
    HX_CU(cudaMemcpyAsync(h->cc[mol].t1, buf, sizeof(double) * ov, cudaMemcpyHostToDevice, h->st));
    HX_CU(cudaMemcpyAsync(h->cc[mol].t2, buf + ov, sizeof(double) * ov * ov, cudaMemcpyHostToDevice, h->st));
    HX_CU(cudaMemsetAsync(h->diis[mol].count, 0, sizeof(int), h->st));
    diis_mirror_reset(h, mol);
    HX_CU(cudaStreamSynchronize(h->st));
    h->rules[mol] = Rules();
    return HX_OK;
}

int hx_ccsd_get_scf(hx_ccsd *h, int32_t mol, double *C, double *eps, double *fmo, double scf[4], int32_t scf_status[2])
{
    if (!h || mol < 0 || mol >= h->nmol) { hx_set_error("bad handle or molecule index"); return HX_ERR_ARG; }
    const ScfMol &s = h->scf[mol];
    const size_t nn = (size_t)s.N * s.N;
    if (C) HX_CU(cudaMemcpyAsync(C, s.V, sizeof(double) * nn, cudaMemcpyDeviceToHost, h->st));
    if (eps) HX_CU(cudaMemcpyAsync(eps, s.E, sizeof(double) * s.N, cudaMemcpyDeviceToHost, h->st));
    if (fmo) HX_CU(cudaMemcpyAsync(fmo, s.Fmo, sizeof(double) * nn, cudaMemcpyDeviceToHost, h->st));
    if (scf) HX_CU(cudaMemcpyAsync(scf, s.out, sizeof(double) * 4, cudaMemcpyDeviceToHost, h->st));
    if (scf_status) HX_CU(cudaMemcpyAsync(scf_status, s.status, sizeof(int) * 2, cudaMemcpyDeviceToHost, h->st));
    HX_CU(cudaStreamSynchronize(h->st));
    return HX_OK;
}

int hx_ccsd_dims(hx_ccsd *h, int32_t mol, int32_t dims[4])
{
    if (!h || mol < 0 || mol >= h->nmol || !dims) { hx_set_error("bad arguments"); return HX_ERR_ARG; }
    dims[0] = h->N[mol]; dims[1] = h->o[mol]; dims[2] = h->v[mol]; dims[3] = h->models[mol].nel;
    return HX_OK;
}

int hx_ccsd_timing(hx_ccsd *h, double out[8], int32_t profile)
{
    if (!h) { hx_set_error("NULL handle"); return HX_ERR_ARG; }
    if (profile >= 0) {
        if (h->tce) tc::set_profile(h->tce, profile != 0);
        h->profiling = profile != 0;
        if (profile) { for (int k = 0; k < 4; ++k) h->prof[k] = 0.0; g_launches.store(0); }
    }
    if (out) {
        out[0] = h->init_ms;
        out[1] = h->solve_ms;
        if (h->tce) tc::collect(h->tce, h->prof);
        for (int k = 0; k < 4; ++k) out[2 + k] = h->prof[k];
        out[6] = (double)h->arena_bytes;
        out[7] = (double)g_launches.load();
    }
    return HX_OK;
}

void hx_ccsd_cancel(hx_ccsd *h)
{
    if (!h) return;
    h->cancel.store(1);
    // a running solve's control kernel reads this mapped word every iteration
    if (h->h_pinned) reinterpret_cast<volatile int *>(h->h_pinned)[8] = 1;
}

int hx_ccsd_set_model(hx_ccsd *h, const float *params)
{
    if (!h) { hx_set_error("NULL handle"); return HX_ERR_ARG; }
    if (!params) {
        if (h->model) { h->model->release(); delete h->model; h->model = nullptr; }
        return HX_OK;
    }
    if (!h->model) h->model = new mlp::Model();
    return h->model->load(params);
}

int hx_ccsd_training_rows(hx_ccsd *h, int32_t mol, int32_t n, const int64_t *rows, float *X, float *T)
{
    if (!h || !h->initialized || mol < 0 || mol >= h->nmol || n <= 0 || !rows || !X || !T) {
        hx_set_error("hx_ccsd_training_rows: bad arguments or state");
        return HX_ERR_ARG;
    }
    const long long ov = (long long)h->o[mol] * h->v[mol], npairs = ov * (ov + 1) / 2;
    for (int k = 0; k < n; ++k)
        if (rows[k] < 0 || rows[k] >= npairs) { hx_set_error("hx_ccsd_training_rows: row %d out of range", k); return HX_ERR_ARG; }
    long long *dr = nullptr;
    float *dX = nullptr, *dT = nullptr;
    int rc = HX_OK;
    if (cudaMalloc(&dr, sizeof(long long) * n) != cudaSuccess || cudaMalloc(&dX, sizeof(float) * 8 * n) != cudaSuccess ||
        cudaMalloc(&dT, sizeof(float) * n) != cudaSuccess) {
        hx_set_error("hx_ccsd_training_rows: allocation failed");
        rc = HX_ERR_NOMEM;
    }
    cudaError_t e = cudaSuccess;
    if (rc == HX_OK) e = cudaMemcpyAsync(dr, rows, sizeof(long long) * n, cudaMemcpyHostToDevice, h->st);
    if (rc == HX_OK && e == cudaSuccess) e = hx_mlp_sample(h->d_cc, mol, dr, n, dX, dT, h->st);
    if (rc == HX_OK && e == cudaSuccess) e = cudaMemcpyAsync(X, dX, sizeof(float) * 8 * n, cudaMemcpyDeviceToHost, h->st);
    if (rc == HX_OK && e == cudaSuccess) e = cudaMemcpyAsync(T, dT, sizeof(float) * n, cudaMemcpyDeviceToHost, h->st);
    if (rc == HX_OK && e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (rc == HX_OK && e != cudaSuccess) { hx_set_error("hx_ccsd_training_rows: %s", cudaGetErrorString(e)); rc = HX_ERR_CUDA; }
    cudaFree(dr);
    cudaFree(dX);
    cudaFree(dT);
    return rc;
}

void hx_ccsd_destroy(hx_ccsd *h)
{
    if (!h) return;
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->tce) tc::destroy(h->tce);
    if (h->model) { h->model->release(); delete h->model; }
    for (int k = 0; k < 4; ++k) if (h->ev[k]) cudaEventDestroy(h->ev[k]);
    for (auto &g : h->plan) if (g.d) cudaFree(g.d);
    cudaFree(h->arena);
    cudaFree(h->d_scf);
    cudaFree(h->d_cc);
    cudaFree(h->d_diis);
    cudaFree(h->d_active);
    cudaFree(h->d_act_ph[0]);
    cudaFree(h->d_ctl);
    cudaFree(h->d_cond);
    cudaFree(h->d_trace);
    cudaFree(h->d_remaining);
    cudaFree(h->d_t0);
    if (h->h_pinned) cudaFreeHost(h->h_pinned);
    if (h->h_amp) cudaFreeHost(h->h_amp);
    if (h->st2) cudaStreamDestroy(h->st2);
    cudaFree(h->d_gate);
    cudaFree(h->d_part);
    cudaFree(h->d_sched);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
}

// (T) of molecule mol from its current amplitudes (hx_triples.cu has the
// formulas), over the occupied triples i <= j <= k. The integrals come from
// the site basis: I1[i][a][b][d] = (ai|bd) = (G C_ai)^T C_bd and J[k][c][j][l]
// = (ck|jl) = C_ck^T G C_jl, FP64 GEMMs once per call. The triples are taken
// in slabs (one i, a range of j, every k >= j), each within a byte budget
// (a few GB whatever the molecule): for a slab W_ijk^abc is formed directly as
// the six pair permutations of X, twelve GEMMs of (v^2 x v x v) and
// (v^2 x v x o) per (i, j), batched over k, on the 7-slice tensor-core GEMM
// (an emulated FP64 product, as accurate as the FP64 one), then the energy
// kernel sums the slab's triples. Memory is O(o v^3) for the integrals plus
// the slab, not O(o^3 v^3).
namespace {
// one of the twelve permutation terms for a fixed (i, j): batch over k = j .. o-1
TgemmDesc triples_term(int t, const CCMol &m, const double *I1, const double *J, double *Wj, int i, int j)
{
    const int o = m.o, v = m.v, nk = o - j, M = v * v;
    const long long vvv = (long long)v * v * v, vov = (long long)v * o * v, voo = (long long)v * o * o;
    const long long vv = (long long)v * v, ov = (long long)o * v, oo = (long long)o * o;
    const double *T2 = m.t2;
    // output W[k - j][a][b][c]: C strides (m outer, m inner, n outer, n inner, batch)
    // Where A does not depend on k (P1, P2, P3, P5) k joins the columns, n = (k - j, x),
    // so the large operand is sliced once; P4 and P6 keep k as a batch index.
    const int NK = nk * v;
    switch (t) {
    // P1 = X(ia, jb, kc): m = (a, b), n = (k, c)
    case 0: return tg(I1 + i * vvv, T2 + j * vov + j * v, Wj, 1, M, NK, v, v, v, v, {vv, v, 0, 1, 0}, {vov, ov, 0, 1, 0}, {vv, v, vvv, 1, 0}, 1.0, 0.0, 0);
    case 1: return tg(T2 + i * vov, J + j * voo + j * o, Wj, 1, M, NK, o, v, v, o, {ov, 1, 0, v, 0}, {voo, oo, 0, 1, 0}, {vv, v, vvv, 1, 0}, -1.0, 1.0, 0);
    // P2 = X(ia, kc, jb): m = (a, c), n = (k, b)
    case 2: return tg(I1 + i * vvv, T2 + j * vov + j * v, Wj, 1, M, NK, v, v, v, v, {vv, v, 0, 1, 0}, {v, ov, 0, 1, 0}, {vv, 1, vvv, v, 0}, 1.0, 1.0, 0);
    case 3: return tg(T2 + i * vov, J + j * voo + j * o, Wj, 1, M, NK, o, v, v, o, {ov, 1, 0, v, 0}, {o, oo, 0, 1, 0}, {vv, 1, vvv, v, 0}, -1.0, 1.0, 0);
    // P3 = X(jb, ia, kc): m = (b, a), n = (k, c)
    case 4: return tg(I1 + j * vvv, T2 + j * vov + i * v, Wj, 1, M, NK, v, v, v, v, {vv, v, 0, 1, 0}, {vov, ov, 0, 1, 0}, {v, vv, vvv, 1, 0}, 1.0, 1.0, 0);
    case 5: return tg(T2 + j * vov, J + j * voo + i * o, Wj, 1, M, NK, o, v, v, o, {ov, 1, 0, v, 0}, {voo, oo, 0, 1, 0}, {v, vv, vvv, 1, 0}, -1.0, 1.0, 0);
    // P4 = X(kc, ia, jb): m = (c, a), n = b, batch k
    case 6: return tg(I1 + j * vvv, T2 + j * vov + i * v, Wj, nk, M, v, v, v, v, v, {vv, v, 0, 1, vvv}, {0, ov, 0, 1, 0}, {1, vv, 0, v, vvv}, 1.0, 1.0, 0);
    case 7: return tg(T2 + j * vov, J + j * voo + i * o, Wj, nk, M, v, o, v, v, o, {ov, 1, 0, v, vov}, {0, oo, 0, 1, 0}, {1, vv, 0, v, vvv}, -1.0, 1.0, 0);
    // P5 = X(jb, kc, ia): m = (b, c), n = (k, a)
    case 8: return tg(I1 + j * vvv, T2 + i * vov + j * v, Wj, 1, M, NK, v, v, v, v, {vv, v, 0, 1, 0}, {v, ov, 0, 1, 0}, {v, 1, vvv, vv, 0}, 1.0, 1.0, 0);
    case 9: return tg(T2 + j * vov, J + i * voo + j * o, Wj, 1, M, NK, o, v, v, o, {ov, 1, 0, v, 0}, {o, oo, 0, 1, 0}, {v, 1, vvv, vv, 0}, -1.0, 1.0, 0);
    // P6 = X(kc, jb, ia): m = (c, b), n = a, batch k
    case 10: return tg(I1 + j * vvv, T2 + i * vov + j * v, Wj, nk, M, v, v, v, v, v, {vv, v, 0, 1, vvv}, {0, ov, 0, 1, 0}, {1, v, 0, vv, vvv}, 1.0, 1.0, 0);
    default: return tg(T2 + j * vov, J + i * voo + j * o, Wj, nk, M, v, o, v, v, o, {ov, 1, 0, v, vov}, {0, oo, 0, 1, 0}, {1, v, 0, vv, vvv}, -1.0, 1.0, 0);
    }
}
}  // namespace

int hx_ccsd_triples(hx_ccsd *h, int32_t mol, double e[4])
{
    if (!h || !h->initialized) { hx_set_error("hx_ccsd_triples before hx_ccsd_init"); return HX_ERR_STATE; }
    if (mol < 0 || mol >= h->nmol) { hx_set_error("hx_ccsd_triples: molecule %d of %d", mol, h->nmol); return HX_ERR_ARG; }
    if (h->scf_failed[mol]) { hx_set_error("hx_ccsd_triples: the SCF of molecule %d did not converge", mol); return HX_ERR_SCF; }
    const CCMol &m = h->cc[mol];
    const int N = m.N, o = m.o, v = m.v;
    const long long ov = (long long)o * v, vvv = (long long)v * v * v;
    const size_t nI1 = (size_t)ov * v * v, nJ = (size_t)ov * o * o;
    const size_t nBvv = (size_t)N * v * v, nBoo = (size_t)N * o * o;
    // slab budget: W (v^3 doubles per triple) plus the 7-slice bf16 copies of the
    // operands a k-batched term (P4, P6) slices per triple (14 B per element of a
    // v^2 x K tile, K padded to 64)
    const double per_pair = 8.0 * vvv + 14.0 * ((v * v + 127) / 128 * 128) * (double)((v + 63) / 64 * 64);
    size_t fre = 0, tot = 0;
    HX_CU(cudaMemGetInfo(&fre, &tot));
    const double fixed_bytes = 8.0 * (nI1 + nJ + nBvv + 2 * nBoo);
    const double budget = std::min(24e9, 0.5 * ((double)fre - fixed_bytes));
    const long long max_pairs = (long long)(budget / per_pair);
    if (max_pairs < o) {
        hx_set_error("hx_ccsd_triples: N = %d needs about %.1f GB of device memory for one slab of triples, "
                     "%.1f GB are free", N, (fixed_bytes + o * per_pair) / 1e9, fre / 1e9);
        return HX_ERR_NOMEM;
    }
    // slabs: (i, j0, j1) with sum_{j0 <= j < j1} (o - j) <= max_pairs
    struct Slab { int i, j0, j1; long long pairs; };
    std::vector<Slab> slabs;
    long long maxp = 0;
    for (int i = 0; i < o; ++i)
        for (int j0 = i; j0 < o;) {
            int j1 = j0;
            long long p = 0;
            while (j1 < o && p + (o - j1) <= max_pairs) { p += o - j1; ++j1; }
            slabs.push_back({i, j0, j1, p});
            maxp = std::max(maxp, p);
            j0 = j1;
        }
    const size_t nW = (size_t)maxp * vvv;
    const size_t elems = nI1 + nJ + nBvv + 2 * nBoo + nW + 2 * (size_t)maxp + 2 * slabs.size();
    double *buf = nullptr;
    int2 *d_pairs = nullptr;
    HX_CU(cudaMalloc(&buf, elems * sizeof(double)));
    if (cudaMalloc(&d_pairs, sizeof(int2) * (size_t)maxp) != cudaSuccess) {
        cudaFree(buf);
        hx_set_error("hx_ccsd_triples: allocation failed");
        return HX_ERR_NOMEM;
    }
    double *I1 = buf, *J = I1 + nI1, *Bvv0 = J + nJ, *Boo0 = Bvv0 + nBvv, *GBoo0 = Boo0 + nBoo, *W = GBoo0 + nBoo,
           *part = W + nW, *out = part + 2 * maxp;
    std::vector<Group> gs(3);
    const long long oo = (long long)o * o, vv = (long long)v * v;
    gs[0].h.push_back(tg(m.G, Boo0, GBoo0, 1, N, (int)oo, N, N, (int)oo, N, {0, N, 0, 1, 0}, {0, 1, 0, oo, 0}, {0, oo, 0, 1, 0}, 1.0, 0.0, mol));
    gs[1].h.push_back(tg(m.Bov0, GBoo0, J, 1, (int)ov, (int)oo, N, (int)ov, (int)oo, N, {0, 1, 0, ov, 0}, {0, 1, 0, oo, 0}, {0, oo, 0, 1, 0}, 1.0, 0.0, mol));
    gs[2].h.push_back(tg(m.GBov0, Bvv0, I1, 1, (int)ov, (int)vv, N, (int)ov, (int)vv, N, {0, 1, 0, ov, 0}, {0, 1, 0, vv, 0}, {0, vv, 0, 1, 0}, 1.0, 0.0, mol));
    int rc = HX_OK;
    cudaError_t ce = hx_triples_pairs(m.Cmo, N, o, Bvv0, Boo0, h->st);
    for (auto &g : gs) {
        if (ce != cudaSuccess || rc != HX_OK) break;
        rc = upload_group(g);
        if (rc == HX_OK) ce = hx_tgemm_f64_launch(g.d, (int)g.h.size(), g.tiles, nullptr, h->st);
    }
    std::vector<int2> pairs;
    for (size_t si = 0; si < slabs.size() && rc == HX_OK && ce == cudaSuccess; ++si) {
        const Slab &sl = slabs[si];
        std::vector<Group> plan(12);
        pairs.clear();
        for (int j = sl.j0; j < sl.j1; ++j) {
            double *Wj = W + (long long)pairs.size() * vvv;
            for (int t = 0; t < 12; ++t) plan[t].h.push_back(triples_term(t, m, I1, J, Wj, sl.i, j));
            for (int k = j; k < o; ++k) pairs.push_back(make_int2(j, k));
        }
        tc::Engine *te = nullptr;
        rc = tc::create(&te, plan, h->st, 2, 0, 3);      // the 7-slice (emulated FP64) mode only
        for (int t = 0; t < 12 && rc == HX_OK && ce == cudaSuccess; ++t)
            ce = tc::run_group(te, plan[t].h.data(), (int)plan[t].h.size(), nullptr, h->st, 3);
        if (rc == HX_OK && ce == cudaSuccess)
            ce = cudaMemcpyAsync(d_pairs, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice, h->st);
        if (rc == HX_OK && ce == cudaSuccess)
            ce = hx_triples_energy(W, d_pairs, (int)pairs.size(), sl.i, m.t1, m.gov, m.Fmo, N, o, part, out + 2 * si,
                                   h->st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->st);   // the pair list is pageable host memory
        if (rc == HX_OK && ce == cudaSuccess && te && tc::error_word(te)) {
            hx_set_error("hx_ccsd_triples: a tensor-core wait timed out");
            rc = HX_ERR_KERNEL;
        }
        tc::destroy(te);
    }
    std::vector<double> r(2 * slabs.size(), 0.0);
    if (ce == cudaSuccess && rc == HX_OK)
        ce = cudaMemcpyAsync(r.data(), out, sizeof(double) * r.size(), cudaMemcpyDeviceToHost, h->st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->st);
    for (auto &g : gs) if (g.d) cudaFree(g.d);
    cudaFree(buf);
    cudaFree(d_pairs);
    if (rc != HX_OK) return rc;
    if (ce != cudaSuccess) { hx_set_error("hx_ccsd_triples: %s", cudaGetErrorString(ce)); return HX_ERR_CUDA; }
    double e4 = 0.0, e5 = 0.0;
    for (size_t si = 0; si < slabs.size(); ++si) { e4 += r[2 * si]; e5 += r[2 * si + 1]; }
    if (e) {
        e[0] = e4 + e5;          // (T) = E[4] + E[5] (spin-orbital textbook sign)
        e[1] = e4;
        e[2] = e5;
        e[3] = -(e4 + e5);       // the reference's triples term c1 + c2 (+ c3 = 0 for canonical RHF)
    }
    return HX_OK;
}

// C = A B^T for row-major FP64 host matrices, on the engine's FP64 or
// tensor-core GEMM; reps > 1 repeats the launch and reports the mean time.
int hx_gemm(const double *A, const double *B, double *C, int32_t M, int32_t N, int32_t K, int32_t precision,
            int32_t reps, double *ms)
{
    return hx_gemm_tile(A, B, C, M, N, K, precision, -1, reps, ms);
}

// The same with tile candidate `variant` of the precision's mode (-1: the default).
int hx_gemm_tile(const double *A, const double *B, double *C, int32_t M, int32_t N, int32_t K, int32_t precision,
                 int32_t variant, int32_t reps, double *ms)
{
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || reps < 1 || precision < 0 || precision > 4 || variant < -1) {
        hx_set_error("hx_gemm: bad arguments");
        return HX_ERR_ARG;
    }
    if (variant >= 0 && precision > 0) {
        int32_t bn[8];
        const int mode = precision == 2 ? 2 : precision == 3 ? 1 : precision == 4 ? 3 : 0;
        if (variant >= hx_tile_variants(mode, bn, 8)) {
            hx_set_error("hx_gemm_tile: precision %d has no tile candidate %d", precision, variant);
            return HX_ERR_ARG;
        }
    }
    cudaStream_t st;
    HX_CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    double *dA = nullptr, *dB = nullptr, *dC = nullptr;
    int *dact = nullptr;
    int rc = HX_OK;
    tc::Engine *te = nullptr;
    std::vector<Group> plan(1);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto fail = [&](int code) { rc = code; };
    if (cudaMalloc(&dA, sizeof(double) * (size_t)M * K) != cudaSuccess ||
        cudaMalloc(&dB, sizeof(double) * (size_t)N * K) != cudaSuccess ||
        cudaMalloc(&dC, sizeof(double) * (size_t)M * N) != cudaSuccess || cudaMalloc(&dact, sizeof(int)) != cudaSuccess) {
        hx_set_error("hx_gemm: device allocation failed");
        fail(HX_ERR_NOMEM);
    }
    if (rc == HX_OK) {
        int one = 1;
        cudaMemcpy(dA, A, sizeof(double) * (size_t)M * K, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B, sizeof(double) * (size_t)N * K, cudaMemcpyHostToDevice);
        cudaMemcpy(dact, &one, sizeof(int), cudaMemcpyHostToDevice);
        // accumulate into a zeroed C (beta = 1) so that long-K problems use split-K as in the plan
        cudaMemset(dC, 0, sizeof(double) * (size_t)M * N);
        plan[0].h.push_back(tg(dA, dB, dC, 1, M, N, K, M, N, K, {0, K, 0, 1, 0}, {0, K, 0, 1, 0}, {0, N, 0, 1, 0}, 1.0, 1.0, 0));
        rc = upload_group(plan[0]);
    }
    if (rc == HX_OK && precision != HX_PRECISION_FP64) rc = tc::create(&te, plan, st, 2, variant);
    if (rc == HX_OK) {
        auto launch = [&]() -> cudaError_t {
            if (te) return tc::run_group(te, plan[0].h.data(), 1, dact, st,
                                         precision == 2 ? 2 : precision == 3 ? 1 : precision == 4 ? 3 : 0);
            return hx_tgemm_f64_launch(plan[0].d, 1, plan[0].tiles, dact, st);
        };
        cudaError_t ce = launch();               // warm-up
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps && ce == cudaSuccess; ++r) ce = launch();
        cudaEventRecord(e1, st);
        // C now holds (reps + 1) A B^T: one clean product for the caller
        if (ce == cudaSuccess) ce = cudaMemsetAsync(dC, 0, sizeof(double) * (size_t)M * N, st);
        if (ce == cudaSuccess) ce = launch();
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) { hx_set_error("hx_gemm: %s", cudaGetErrorString(ce)); rc = HX_ERR_CUDA; }
        if (rc == HX_OK && te && tc::error_word(te)) { hx_set_error("hx_gemm: tensor-core wait timed out"); rc = HX_ERR_KERNEL; }
        if (rc == HX_OK) {
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            if (ms) *ms = t / reps;
            cudaMemcpy(C, dC, sizeof(double) * (size_t)M * N, cudaMemcpyDeviceToHost);
        }
    }
    if (te) tc::destroy(te);
    if (plan[0].d) cudaFree(plan[0].d);
    cudaFree(dA); cudaFree(dB); cudaFree(dC); cudaFree(dact);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    return rc;
}

int hx_last_error(char *buf, size_t len)
{
    size_t n = strlen(g_err);
    if (buf && len) {
        size_t c = n < len - 1 ? n : len - 1;
        memcpy(buf, g_err, c);
        buf[c] = 0;
    }
    return (int)n;
}

}  // extern "C"

// ---------------------------------------------------------------- tile autotuner
extern "C" int hx_tile_table(int32_t *entries, int32_t cap) { return tc::table_get(entries, cap); }

extern "C" int hx_tile_table_load(const int32_t *entries, int32_t n)
{
    if (n < 0 || (n > 0 && !entries)) { hx_set_error("hx_tile_table_load: bad arguments"); return HX_ERR_ARG; }
    return tc::table_load(entries, n);
}

extern "C" int hx_tile_variants(int32_t mode, int32_t *bn, int32_t cap)
{
    const int n = tc::variants(mode, bn, cap);
    if (n < 0) hx_set_error("hx_tile_variants: mode %d outside 0..3", mode);
    return n;
}

extern "C" int hx_ccsd_tile_choices(hx_ccsd *h, int32_t *var, int32_t cap, double *tune_ms)
{
    if (!h) { hx_set_error("NULL handle"); return HX_ERR_ARG; }
    if (tune_ms) *tune_ms = tc::tune_ms(h->tce);
    return h->tce ? tc::choices(h->tce, var, cap) : 0;
}
