// PPP-RHF on the GPU in FP64: one CTA per molecule runs the whole SCF.
//
// Iteration of helios's SCF (src/methods/mod_scf.f90:106-136):
//   Fmin = (F R - R F) R,  R = 2D - 1          (prepareFmin :446-494)
//   accuracy = max|Fmin|
//   D -= (iter-step) Fmin;  F = fock(D)        (prepareFockian :417-442)
//   diagonalise F; D = aufbau(V); F = fock(D)
// with the generic iterator's stop rules (src/calculation/gIterator.f90:88-210).
// The guess diagonalises huckelCore (guessSCF :351-386) unless a density is given.
//
// Diagonalisation is a cyclic two-sided Jacobi method with the round-robin
// (circle) ordering, so the N/2 rotations of a round are disjoint and run in
// parallel. It works on A = V^T F V in the current orbital basis (warm start:
// the basis of the previous iteration already nearly diagonalises F) and
// accumulates the rotations into V. Eigenpairs are then sorted ascending, as
// the reference's tred4 returns them (src/modules/mod_math.f90:31-230).
//
// The SCF body is written once over an execution context: a batch runs one
// CTA per molecule (BlockCtx, barriers are __syncthreads); a single large
// molecule runs on a cooperative grid (GridCtx, barriers are grid syncs) so
// that every Jacobi round and every N^3 product is spread over many SMs.
#include <algorithm>
#include <cooperative_groups.h>
#include "hx_common.cuh"
#include "hx_plan.h"

namespace {
namespace cg = cooperative_groups;
constexpr int NT = 512;

// ---- execution contexts -------------------------------------------------
struct BlockCtx {
    int tid, nt;
    double *sh;          // >= 33 doubles of shared scratch
    __device__ BlockCtx(double *s) : tid(threadIdx.x), nt(blockDim.x), sh(s) {}
    __device__ void sync() { __syncthreads(); }
    __device__ double reduce(double v, bool mx)
    {
        for (int o = 16; o > 0; o >>= 1) {
            double w = __shfl_xor_sync(0xffffffffu, v, o);
            v = mx ? fmax(v, w) : v + w;
        }
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        __syncthreads();
        if (lane == 0) sh[wid] = v;
        __syncthreads();
        if (wid == 0) {
            v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) {
                double w = __shfl_xor_sync(0xffffffffu, v, o);
                v = mx ? fmax(v, w) : v + w;
            }
            if (lane == 0) sh[32] = v;
        }
        __syncthreads();
        double r = sh[32];
        __syncthreads();
        return r;
    }
};

struct GridCtx {
    int tid, nt;
    double *sh;          // shared scratch of this CTA
    double *gpart;       // 2 x gridDim.x global partials
    int parity;
    __device__ GridCtx(double *s, double *gp)
        : tid(blockIdx.x * blockDim.x + threadIdx.x), nt(gridDim.x * blockDim.x), sh(s), gpart(gp), parity(0) {}
    __device__ void sync() { cg::this_grid().sync(); }
    __device__ double reduce(double v, bool mx)
    {
        BlockCtx b(sh);
        v = b.reduce(v, mx);
        double *p = gpart + parity * gridDim.x;
        parity ^= 1;
        if (threadIdx.x == 0) p[blockIdx.x] = v;
        sync();
        double r = mx ? 0.0 : 0.0;
        for (unsigned k = 0; k < gridDim.x; ++k) r = mx ? fmax(r, p[k]) : r + p[k];
        return r;   // the same ordered sum in every thread
    }
};

// C = op(A) op(B) for N x N row-major matrices (ta/tb: use the transpose).
template <class Ctx>
__device__ void mm(Ctx &c, double *C, const double *A, const double *B, int n, bool ta, bool tb, int kmax)
{
    for (int e = c.tid; e < n * n; e += c.nt) {
        int i = e / n, j = e % n;
        double s = 0.0;
        for (int k = 0; k < kmax; ++k) {
            double a = ta ? A[k * n + i] : A[i * n + k];
            double b = tb ? B[j * n + k] : B[k * n + j];
            s = fma(a, b, s);
        }
        C[e] = s;
    }
    c.sync();
}

// F = core - G o D + 2 diag(G diag D)
template <class Ctx>
__device__ void fock(Ctx &c, double *F, const double *core, const double *G, const double *D, int n)
{
    for (int e = c.tid; e < n * n; e += c.nt) {
        int i = e / n, j = e % n;
        double f = core[e] - G[e] * D[e];
        if (i == j) {
            double s = 0.0;
            for (int l = 0; l < n; ++l) s += G[i * n + l] * D[l * n + l];
            f += 2.0 * s;
        }
        F[e] = f;
    }
    c.sync();
}

// D = sum_{i<nocc} V[:,i] V[:,i]^T
template <class Ctx>
__device__ void density(Ctx &c, double *D, const double *V, int n, int nocc)
{
    for (int e = c.tid; e < n * n; e += c.nt) {
        int mu = e / n, nu = e % n;
        double s = 0.0;
        for (int i = 0; i < nocc; ++i) s = fma(V[mu * n + i], V[nu * n + i], s);
        D[e] = s;
    }
    c.sync();
}

// Jacobi eigen-decomposition of symmetric A (n x n, destroyed: its diagonal
// ends as the eigenvalues); rotations accumulate into V. W is n x n scratch.
// pp/pq/pc/ps are shared arrays of the CTA: every CTA derives the rotations
// of a round itself from the same matrix entries, so a round needs only the
// two barriers between its column and row passes.
template <class Ctx>
__device__ int jacobi(Ctx &c, double *A, double *V, double *E, double *W, int n, int *pp, int *pq, double *pc,
                      double *ps)
{
    const int np = n + (n & 1);
    int sweeps = 0;
    for (; sweeps < 40; ++sweeps) {
        double off = 0.0, tot = 0.0;
        for (int e = c.tid; e < n * n; e += c.nt) {
            double a = A[e] * A[e];
            tot += a;
            if (e / n != e % n) off += a;
        }
        off = c.reduce(off, false);
        tot = c.reduce(tot, false);
        if (off <= 1e-30 * tot || off < 1e-300) break;
        for (int r = 0; r < np - 1; ++r) {
            for (int k = threadIdx.x; k < np / 2; k += blockDim.x) {
                int x = k, y = np - 1 - k;
                int p = (x == 0) ? 0 : 1 + (x - 1 + r) % (np - 1);
                int q = 1 + (y - 1 + r) % (np - 1);
                if (p > q) { int t = p; p = q; q = t; }
                double cc = 1.0, s = 0.0;
                if (q < n) {
                    double apq = A[p * n + q];
                    if (fabs(apq) > 1e-300) {
                        double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                        double t;
                        if (fabs(theta) > 1e150) t = 0.5 / theta;
                        else t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        cc = 1.0 / sqrt(t * t + 1.0);
                        s = t * cc;
                    }
                } else {
                    p = -1;   // bye for odd n
                }
                pp[k] = p; pq[k] = q; pc[k] = cc; ps[k] = s;
            }
            // every CTA has read the pair entries before any column is rotated
            c.sync();
            // columns of A and V: X <- X J
            for (int e = c.tid; e < (np / 2) * n; e += c.nt) {
                int k = e / n, row = e % n, p = pp[k], q = pq[k];
                if (p < 0 || ps[k] == 0.0) continue;
                double cs = pc[k], s = ps[k];
                double akp = A[row * n + p], akq = A[row * n + q];
                A[row * n + p] = cs * akp - s * akq;
                A[row * n + q] = s * akp + cs * akq;
                double vkp = V[row * n + p], vkq = V[row * n + q];
                V[row * n + p] = cs * vkp - s * vkq;
                V[row * n + q] = s * vkp + cs * vkq;
            }
            c.sync();
            // rows of A: A <- J^T A
            for (int e = c.tid; e < (np / 2) * n; e += c.nt) {
                int k = e / n, col = e % n, p = pp[k], q = pq[k];
                if (p < 0 || ps[k] == 0.0) continue;
                double cs = pc[k], s = ps[k];
                double apk = A[p * n + col], aqk = A[q * n + col];
                A[p * n + col] = cs * apk - s * aqk;
                A[q * n + col] = s * apk + cs * aqk;
            }
            c.sync();
        }
    }
    // sort ascending: rank each eigenvalue, permute V's columns through W
    for (int e = c.tid; e < n * n; e += c.nt) {
        int row = e / n, p = e % n;
        double ep = A[p * n + p];
        int rank = 0;
        for (int q = 0; q < n; ++q) {
            double eq = A[q * n + q];
            rank += (eq < ep) || (eq == ep && q < p);
        }
        W[row * n + rank] = V[row * n + p];
        if (row == 0) E[rank] = ep;
    }
    c.sync();
    for (int e = c.tid; e < n * n; e += c.nt) V[e] = W[e];
    c.sync();
    return sweeps;
}

template <class Ctx>
__device__ void scf_body(Ctx &c, const ScfMol &m, const ScfParams &prm, int *pp, int *pq, double *pc, double *ps)
{
    const int n = m.N, no = m.nocc, nn = n * n;
    double *F = m.F, *D = m.D, *V = m.V, *A = m.A, *W1 = m.W1, *W2 = m.W2;

    // guess
    if (m.D0) {
        for (int e = c.tid; e < nn; e += c.nt) D[e] = m.D0[e];
        for (int e = c.tid; e < nn; e += c.nt) V[e] = m.V0 ? m.V0[e] : (e / n == e % n);
        c.sync();
    } else {
        for (int e = c.tid; e < nn; e += c.nt) {
            A[e] = m.huckel[e];
            V[e] = (e / n == e % n) ? 1.0 : 0.0;
        }
        c.sync();
        jacobi(c, A, V, m.E, W1, n, pp, pq, pc, ps);
        density(c, D, V, n, no);
    }
    fock(c, F, m.core, m.G, D, n);

    int iteration = 0, successful = 1, status = 0;
    double current = 0.0;
    for (;;) {
        ++iteration;
        // W1 = F R, R = 2D - 1
        for (int e = c.tid; e < nn; e += c.nt) W2[e] = 2.0 * D[e] - (e / n == e % n);
        c.sync();
        mm(c, W1, F, W2, n, false, false, n);
        // A = W1 - W1^T  (F R - R F, both symmetric)
        for (int e = c.tid; e < nn; e += c.nt) A[e] = W1[e] - W1[(e % n) * n + e / n];
        c.sync();
        mm(c, W1, A, W2, n, false, false, n);           // Fmin
        double acc = 0.0;
        for (int e = c.tid; e < nn; e += c.nt) acc = fmax(acc, fabs(W1[e]));
        acc = c.reduce(acc, true);
        for (int e = c.tid; e < nn; e += c.nt) D[e] -= prm.step * W1[e];
        c.sync();
        fock(c, F, m.core, m.G, D, n);
        // diagonalise F in the current basis: A = V^T F V
        mm(c, W1, F, V, n, false, false, n);
        mm(c, A, V, W1, n, true, false, n);
        jacobi(c, A, V, m.E, W1, n, pp, pq, pc, ps);
        density(c, D, V, n, no);
        fock(c, F, m.core, m.G, D, n);

        double previous = current;
        current = acc;
        if (current < previous) ++successful;
        if (!(current == current)) { status = HX_DIVERGED; break; }   // NaN
        if (current < prm.eps) { status = HX_CONVERGED; break; }
        if (prm.check_div && current > prm.divergence) { status = HX_DIVERGED; break; }
        if (iteration + 1 > prm.maxiter) { status = HX_FAILED_MAXITER; break; }
        if (prm.check_stag && iteration > prm.stag_after &&
            100.0 * successful / iteration <= prm.stag_pct) { status = HX_STAGNATED; break; }
    }
    // energy: Eel = sum D (core + F), Enuc = sum_{mu<nu} G   (energySCF :166-200)
    double eel = 0.0, enuc = 0.0;
    for (int e = c.tid; e < nn; e += c.nt) {
        eel += D[e] * (m.core[e] + F[e]);
        if (e / n < e % n) enuc += m.G[e];
    }
    eel = c.reduce(eel, false);
    enuc = c.reduce(enuc, false);
    if (c.tid == 0) {
        m.out[0] = eel + enuc;
        m.out[1] = eel;
        m.out[2] = enuc;
        m.out[3] = current;
        m.status[0] = status;
        m.status[1] = iteration;
    }
    // MO Fock (prepareFock('spatial'), mod_cc.f90:2336-2396): Fmo = V^T F V
    mm(c, W1, F, V, n, false, false, n);
    mm(c, m.Fmo, V, W1, n, true, false, n);
}

__global__ void __launch_bounds__(NT) scf_kernel(const ScfMol *__restrict__ mols, ScfParams prm)
{
    __shared__ double sh[40];
    __shared__ int pp[HX_MAX_MOL_N / 2], pq[HX_MAX_MOL_N / 2];
    __shared__ double pc[HX_MAX_MOL_N / 2], ps[HX_MAX_MOL_N / 2];
    const ScfMol m = mols[blockIdx.x];
    BlockCtx c(sh);
    scf_body(c, m, prm, pp, pq, pc, ps);
}

__global__ void __launch_bounds__(256) scf_grid_kernel(const ScfMol *__restrict__ mols, ScfParams prm, double *gpart)
{
    __shared__ double sh[40];
    __shared__ int pp[HX_MAX_MOL_N / 2], pq[HX_MAX_MOL_N / 2];
    __shared__ double pc[HX_MAX_MOL_N / 2], ps[HX_MAX_MOL_N / 2];
    const ScfMol m = mols[0];
    GridCtx c(sh, gpart);
    scf_body(c, m, prm, pp, pq, pc, ps);
}
}  // namespace

// One molecule of more than 64 sites runs on a cooperative grid (one CTA per
// Jacobi pair, at most one per SM); batches run one CTA per molecule.
cudaError_t hx_scf_launch(const ScfMol *d_mols, int nmol, int nmax, const ScfParams &p, double *d_gpart,
                          cudaStream_t s)
{
    if (nmol == 1 && nmax > 64 && d_gpart) {
        int dev = 0, nsm = 0, per_sm = 0, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, scf_grid_kernel, 256, 0);
        int grid = std::min(nmax / 2, nsm * std::max(per_sm, 1));
        grid = std::min(grid, HX_SCF_GRID_MAX);
        if (coop && per_sm > 0 && grid >= 2) {
            ScfParams pc = p;
            const ScfMol *pm = d_mols;
            double *gp = d_gpart;
            void *args[] = {(void *)&pm, (void *)&pc, (void *)&gp};
            hx_count_launches(1);
            return cudaLaunchCooperativeKernel((void *)scf_grid_kernel, dim3(grid), dim3(256), args, 0, s);
        }
    }
    scf_kernel<<<nmol, NT, 0, s>>>(d_mols, p);
    hx_count_launches(1);
    return cudaGetLastError();
}
